"""Seeded synthetic planetesimal disks and run parameters.

The disk sampler follows GPLUM's SolidDisk::createInitialCondition
(src/disk.h:89-171): semimajor axes from a surface density
Sigma ~ a^-p, random angles, Kepler's equation for the eccentric anomaly,
and the orbital-element -> position/velocity map of src/kepler.h:77-93.
Eccentricities and inclinations are Rayleigh-distributed with the requested
rms (in reduced Hill radii h = (m / 3 M_sun)^(1/3)); GPLUM's own generator
draws half-normal magnitudes with the same rms.  Units: G = M_sun = 1, AU,
time in yr / 2 pi.  Every draw comes from numpy's PCG64 with the given seed.
"""
from dataclasses import dataclass, asdict
import numpy as np

L_CGS = 14959787070000.0
M_CGS = 1.9884e33


def density_code_units(g_per_cm3):
    """Bulk density in M_sun / AU^3 (GPLUM's `dens = 2.CGS`)."""
    return g_per_cm3 * L_CGS**3 / M_CGS


@dataclass
class P3TParams:
    """FPGrav static parameters (src/particle.h:917-961 defaults overridden
    by the run's parameter.dat).  Defaults are the CPU-runnable 3000-body
    disk: dt_tree 2^-7, r_out = 3 r_Hill, r_in = 0.1 r_out."""
    eps2: float = 0.0
    eps2_sun: float = 0.0
    m_sun: float = 1.0
    dt_tree: float = 2.0**-7
    dt_min: float = 2.0**-30
    eta: float = 0.02
    eta_0: float = 0.002
    eta_sun: float = 0.02
    eta_sun0: float = 0.002
    alpha2: float = 1.0
    gamma: float = 0.1
    R_cut0: float = 3.0
    R_cut1: float = 0.0
    R_search0: float = 1.1
    R_search1: float = 6.0
    R_search2: float = 1.1
    R_search3: float = 2.0
    r_cut_min: float = 0.0
    r_cut_max: float = 0.0
    p_cut: float = 0.0
    dens: float = density_code_units(2.0)
    # tree
    theta: float = 0.5
    n_leaf_limit: int = 8
    n_group_limit: int = 64

    def vector(self):
        """The 21-double parameter block of the C interfaces."""
        return np.array([self.eps2, self.eps2_sun, self.m_sun, self.dt_tree, self.dt_min,
                         self.eta, self.eta_0, self.eta_sun, self.eta_sun0, self.alpha2,
                         self.gamma, self.R_cut0, self.R_cut1, self.R_search0, self.R_search1,
                         self.R_search2, self.R_search3, self.r_cut_min, self.r_cut_max,
                         self.p_cut, self.dens], dtype=np.float64)

    def as_dict(self):
        return asdict(self)


def _solve_kepler(l, e):
    u = l + e * np.sin(l)
    for _ in range(30):
        du = (u - e * np.sin(u) - l) / (1.0 - e * np.cos(u))
        u = u - du
    return u


def make_disk(n, m, a_in, a_out, p=1.5, ecc_hill=2.0, inc_hill=1.0, seed=0, m_sun=1.0,
              dens=density_code_units(2.0), f=1.0, a=None):
    """Returns dict(id, mass, r_planet, f, pos, vel) for n equal-mass bodies
    (semimajor axes drawn from the annulus, or the given array `a`)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = (m / (3.0 * m_sun)) ** (1.0 / 3.0)
    # dN/da ~ a Sigma ~ a^(1-p): inverse CDF in a^(2-p)
    q = 2.0 - p
    u = rng.random(n)
    if a is not None:
        a = np.asarray(a, np.float64)
    elif abs(q) < 1e-12:
        a = a_in * (a_out / a_in) ** u
    else:
        a = (a_in**q + u * (a_out**q - a_in**q)) ** (1.0 / q)
    # Rayleigh with rms r: scale r / sqrt(2)
    ecc = rng.rayleigh(ecc_hill * h / np.sqrt(2.0), n)
    inc = rng.rayleigh(inc_hill * h / np.sqrt(2.0), n)
    l = 2 * np.pi * rng.random(n)
    omg = 2 * np.pi * rng.random(n)
    OMG = 2 * np.pi * rng.random(n)
    uu = _solve_kepler(l, ecc)
    nmean = np.sqrt(m_sun / a**3)
    P = np.stack([np.cos(omg) * np.cos(OMG) - np.sin(omg) * np.sin(OMG) * np.cos(inc),
                  np.cos(omg) * np.sin(OMG) + np.sin(omg) * np.cos(OMG) * np.cos(inc),
                  np.sin(omg) * np.sin(inc)], axis=1)
    Q = np.stack([-np.sin(omg) * np.cos(OMG) - np.cos(omg) * np.sin(OMG) * np.cos(inc),
                  -np.sin(omg) * np.sin(OMG) + np.cos(omg) * np.cos(OMG) * np.cos(inc),
                  np.cos(omg) * np.sin(inc)], axis=1)
    cu, su = np.cos(uu), np.sin(uu)
    esq = np.sqrt(1.0 - ecc * ecc)
    pos = a[:, None] * ((cu - ecc)[:, None] * P + (esq * su)[:, None] * Q)
    rinv = 1.0 / np.sqrt(np.sum(pos * pos, axis=1))
    vel = (a * a * nmean * rinv)[:, None] * (-su[:, None] * P + (esq * cu)[:, None] * Q)
    mass = np.full(n, m)
    r_planet = (0.75 * mass / (np.pi * dens)) ** (1.0 / 3.0)
    return dict(id=np.arange(n, dtype=np.int64), mass=mass, r_planet=r_planet,
                f=np.full(n, f), pos=np.ascontiguousarray(pos), vel=np.ascontiguousarray(vel))


# The five workloads (disk model, sizes).  Names say what they are.
def disk_3000():
    """3000 bodies, m = 1e-9, 0.95-1.05 AU, rms e = 2 h, rms i = h."""
    return make_disk(3000, 1e-9, 0.95, 1.05, ecc_hill=2.0, inc_hill=1.0, seed=1)


def disk_1m_soft(n=1048576, seed=2):
    """Soft-force workload: n bodies, m = 1e-10, 0.5-1.5 AU."""
    return make_disk(n, 1e-10, 0.5, 1.5, ecc_hill=2.0, inc_hill=1.0, seed=seed)


def disk_1m_hard(n=1048576, seed=3, m_at_1m=7e-11):
    """Hard-part workload: the 0.95-1.05 AU disk model at n bodies, rms e = 6 h,
    rms i = 3 h.  The body mass (7e-11 at n = 1,048,576; scaled as n^-1.5 for
    smaller n, which keeps the mean neighbour count) puts the neighbour graph
    just below percolation: tens of thousands of clusters of 2 to ~300 bodies
    with a power-law tail.  (At m = 1e-9 the annulus percolates into a single
    cluster at this n.)"""
    m = m_at_1m * (1048576.0 / n) ** 1.5
    return make_disk(n, m, 0.95, 1.05, ecc_hill=6.0, inc_hill=3.0, seed=seed)


def disk_1m_embryos(n=1048576, seed=4, m=1e-10, m_embryo=3.0e-7, a_embryo=(0.7, 0.9, 1.1, 1.3)):
    """Embryo workload: n planetesimals of m = 1e-10 in 0.5-1.5 AU with the
    hard-part disk's random velocities (rms e = 6 h, rms i = 3 h), plus four
    embryos of 0.1 Earth mass (3e-7 M_sun) at 0.7, 0.9, 1.1 and 1.3 AU (rms
    e = 2 h, rms i = h of their own mass).  The embryos carry the last ids."""
    d = make_disk(n, m, 0.5, 1.5, ecc_hill=6.0, inc_hill=3.0, seed=seed)
    e = make_disk(len(a_embryo), m_embryo, 0.5, 1.5, ecc_hill=2.0, inc_hill=1.0, seed=seed + 1000,
                  a=np.array(a_embryo))
    out = {k: np.concatenate([d[k], e[k]]) for k in ("mass", "r_planet", "f", "pos", "vel")}
    out["id"] = np.arange(n + len(a_embryo), dtype=np.int64)
    out["pos"] = np.ascontiguousarray(out["pos"])
    out["vel"] = np.ascontiguousarray(out["vel"])
    return out


def disk_8m(n=8388608, seed=5):
    """Large disk: n planetesimals of m = 1.25e-11 in 0.3-3 AU, rms e = 4 h,
    rms i = 2 h."""
    return make_disk(n, 1.25e-11, 0.3, 3.0, ecc_hill=4.0, inc_hill=2.0, seed=seed)
