"""Record layouts that cross the P3T boundary, as numpy dtypes.

They are byte-identical to GPLUM's FDPS classes (src/particle.h of GPLUM):

* ``EPI_DTYPE``  -- EPIGrav, 48 B (src/particle.h:93-141)
* ``EPJ_DTYPE``  -- EPJGrav, 112 B (src/particle.h:149-170)
* ``SPJ_DTYPE``  -- FDPS SPJQuadrupole, 80 B (mass, pos, symmetric quad)
* ``FORCE_DTYPE`` -- ForceGrav, 32 B (src/particle.h:16-86)
* ``FPGRAV_DTYPE`` -- FPGrav, 344 B (src/particle.h:93-170,404-500; the build
  with individual cutoffs, quadrupole moments and collisions), the element of
  GPLUM's ParticleSystem<FPGrav> and of its binary restart file
"""
import numpy as np

INT32_MAX = 2**31 - 1

EPI_DTYPE = np.dtype([("id_local", "<i4"), ("myrank", "<i4"), ("pos", "<f8", 3),
                      ("r_out", "<f8"), ("r_search", "<f8")])
EPJ_DTYPE = np.dtype([("id_local", "<i4"), ("myrank", "<i4"), ("pos", "<f8", 3),
                      ("r_out", "<f8"), ("r_search", "<f8"), ("id", "<i8"), ("mass", "<f8"),
                      ("vel", "<f8", 3), ("acc_d", "<f8", 3)])
SPJ_DTYPE = np.dtype([("mass", "<f8"), ("pos", "<f8", 3), ("xx", "<f8"), ("yy", "<f8"),
                      ("zz", "<f8"), ("xy", "<f8"), ("xz", "<f8"), ("yz", "<f8")])
FORCE_DTYPE = np.dtype([("acc", "<f4", 3), ("phi", "<f4"), ("number", "<i4"), ("rank", "<i4"),
                        ("id_max", "<i4"), ("id_min", "<i4")])

FPGRAV_DTYPE = np.dtype([("id_local", "<i4"), ("myrank", "<i4"), ("pos", "<f8", 3),
                         ("r_out", "<f8"), ("r_search", "<f8"), ("id", "<i8"), ("mass", "<f8"),
                         ("vel", "<f8", 3), ("acc_d", "<f8", 3), ("acc", "<f8", 3), ("acc_s", "<f8", 3),
                         ("jerk_d", "<f8", 3), ("jerk_s", "<f8", 3), ("acc_gd", "<f8", 3), ("phi", "<f8"),
                         ("phi_d", "<f8"), ("phi_s", "<f8"), ("v_disp", "<f8"), ("r_out_inv", "<f8"),
                         ("time", "<f8"), ("dt", "<f8"), ("acc0", "<f8"), ("r_planet", "<f8"), ("f", "<f8"),
                         ("number", "<i4"), ("rank", "<i4"), ("id_max", "<i4"), ("id_min", "<i4"),
                         ("id_cluster", "<i8"), ("n_cluster", "<i4"), ("in_domain", "u1"), ("is_sent", "u1"),
                         ("is_dead", "u1"), ("is_merged", "u1")])

assert EPI_DTYPE.itemsize == 48
assert EPJ_DTYPE.itemsize == 112
assert SPJ_DTYPE.itemsize == 80
assert FORCE_DTYPE.itemsize == 32
assert FPGRAV_DTYPE.itemsize == 344 and FPGRAV_DTYPE.fields["id_cluster"][1] == 328


def cleared_forces(n):
    """ForceGrav records after ForceGrav::clear (src/particle.h:81-85)."""
    f = np.zeros(n, FORCE_DTYPE)
    f["id_max"] = -1
    f["id_min"] = INT32_MAX
    return f
