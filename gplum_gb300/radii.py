"""Individual cut-off and search radii (host input preparation).

Restates GPLUM's setCutoffRadii for the individual-cutoff build
(src/particle.h:1319-1457 calcRandomVel, :713-733 setROutRSearch,
:653-699 getSemimajorAxis2 / getRHill) with numpy: the random velocity
v_disp is the rms deviation from circular Keplerian speed in 32 radial
bins, Gaussian-smoothed across bins; then
    r_out    = clip(max(R_cut0 a^-p_cut r_Hill, R_cut1 v_disp dt_tree), r_cut_min, r_cut_max)
    r_search = R_search0 r_out + R_search1 v_disp dt_tree.
"""
import numpy as np


def random_velocity(pos, vel, m_sun=1.0, nbin=32):
    r2 = pos[:, 0] ** 2 + pos[:, 1] ** 2
    ri = np.sqrt(r2)
    r_max = np.sqrt(r2.max()) * 1.01
    r_min = np.sqrt(r2.min()) * 0.99
    dr = (r_max - r_min) / nbin
    drinv = 1.0 / dr
    b = ((ri - r_min) * drinv).astype(np.int64)
    b[b == nbin] = nbin - 1
    vk = np.stack([-pos[:, 1] / ri, pos[:, 0] / ri, np.zeros_like(ri)], axis=1) * np.sqrt(m_sun / ri)[:, None]
    vr = vel - vk
    v2 = (vr * vr).sum(1)
    vsum = np.bincount(b, weights=v2, minlength=nbin)
    cnt = np.bincount(b, minlength=nbin)
    vd = np.where(cnt > 0, np.sqrt(vsum / np.maximum(cnt, 1)), 0.0)
    centers = r_min + (np.arange(nbin) + 0.5) * dr
    out = np.empty(len(ri))
    for s in range(0, len(ri), 1 << 18):
        ddr = centers[None, :] - ri[s:s + (1 << 18), None]
        ex = np.exp(-ddr * ddr * drinv * drinv)
        out[s:s + (1 << 18)] = (ex * vd[None, :]).sum(1) / (ex * (cnt > 0)[None, :]).sum(1)
    return out


def cutoff_radii(pos, vel, mass, params):
    """Returns (r_out, r_search, v_disp)."""
    P = params
    v_disp = random_velocity(pos, vel, P.m_sun)
    r = np.sqrt((pos * pos).sum(1))
    rv = (pos * vel).sum(1)
    ax = 1.0 / (2.0 / r - (vel * vel).sum(1) / P.m_sun)
    ecc = np.sqrt((1.0 - r / ax) ** 2 + rv * rv / (P.m_sun * ax))
    ax = np.where(ecc < 0.6, ax, r)
    r_hill = np.power(mass / (3.0 * P.m_sun), 1.0 / 3.0) * ax
    r_out = np.maximum(P.R_cut0 * np.power(ax, -P.p_cut) * r_hill, P.R_cut1 * v_disp * P.dt_tree)
    r_out = np.maximum(r_out, P.r_cut_min)
    if P.r_cut_max > 0.0:
        r_out = np.minimum(P.r_cut_max, r_out)
    r_search = P.R_search0 * r_out + P.R_search1 * v_disp * P.dt_tree
    return r_out, r_search, v_disp
