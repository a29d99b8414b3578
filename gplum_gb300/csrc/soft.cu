// Fused EP-EP + EP-SP soft-force kernels for sm_103a.
//
// One CTA of 128 threads per i-group.  The group's i-particles sit in
// registers; its EPJ list, then its SPJ list, are gathered tile by tile
// (128 entries) into shared memory, where each entry is shifted to the
// group origin once (FP64 subtraction, then the FP32 rounding the functor
// applies) and then reused by every i of the group.
//
// Work split per CTA, by group size ni (uniform per CTA; the thresholds are
// SoftArgs::t_ipt2/t_s1/t_s2, set by the autotuner, defaults shown):
//   ni > 128 : 2 i per thread           ni in (64,128] : 1 i per thread
//   ni in (32,64] : two sub-blocks of 64 threads, each taking half of every
//   j tile      ni <= 32 : four sub-blocks of 32 threads, a quarter each.
// Sub-block partial sums are combined in a fixed order, so results do not
// depend on scheduling.
//
// Mixed kernel (reference functors src/gravity_kernel.hpp:25-121 and
// 138-238 of GPLUM, PIKG specs src/gravity_kernel_epep.pikg and
// src/gravity_kernel_epsp.pikg):
//   * displacements: FP64 relative to epi[0], rounded to FP32 (as the functor);
//     for EP-EP the rounding residue is kept as a second FP32 term and added
//     back for the force arithmetic, so near pairs keep ~1e-7 relative
//     precision in r however far they sit from the group origin;
//   * neighbour screen: r2_real = ((rx*rx + ry*ry) + rz*rz) + eps2 in FP32
//     with every product and sum rounded separately (no FMA), compared with
//     max(rs2_i, rs2_j) -- bit-identical to the functor, so neighbour counts,
//     rank sums and id_min/id_max match exactly;
//   * forces: FP32 with rsqrt + one Newton step, FMA allowed; partial sums of
//     32 pairs are folded into an error-free (TwoSum) FP32 hi/lo pair, so the
//     accumulation error does not grow with the list length.
// FP64 kernel: the same formulas with every quantity in double, plain
// 1/sqrt -- the "plain FP64" form used as the accuracy and speed baseline.
//
// Optional candidate emission: every screen hit (j != i) appends j's particle
// index to the i's row of a [n x cap] candidate table; the device-side
// cutoff correction and neighbour search read it instead of a tree query.
#include "p3t_common.cuh"
#include "p3t_soft.cuh"

namespace p3t {

constexpr int SB = 128;  // threads per CTA
constexpr int TJ = 128;  // list entries per shared-memory tile
constexpr int CHUNK = 32;  // pairs per FP32 partial sum before folding

__device__ __forceinline__ void fold(float &hi, float &lo, float v) {
    const float s = hi + v;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (v - bb);
    hi = s;
    lo += err;
}

// --------------------------------------------------------------------------
// mixed precision
template <int S, int IPT, bool EMIT>
__device__ __forceinline__ void group_mixed(const SoftArgs &A, int g, int ib, int ni, float4 *sa, float4 *sb,
                                            float4 *sc, int *sidx, int *scnt, float *redf, int *redi) {
    // i-particles [ib, ib + ni) of group g (ni <= 2 * SB); the origin is the
    // group's first i-particle, as in the functor
    constexpr int W = SB / S;
    const int tid = threadIdx.x;
    const int sub = tid / W, lane = tid % W;
    const int i0 = A.i_off[g];
    const int j0 = A.j_off[g], nj = A.j_off[g + 1] - j0;
    const int s0 = A.s_off[g], ns = A.s_off[g + 1] - s0;
    const float eps2 = A.eps2;

    int p_first = A.i_idx[i0];
    if ((unsigned)p_first >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p_first = 0; }
    const double ox = A.iptcl[p_first].x, oy = A.iptcl[p_first].y, oz = A.iptcl[p_first].z;

    float xi[IPT], yi[IPT], zi[IPT], xl[IPT], yl[IPT], zl[IPT], ro2i[IPT], rs2i[IPT];
    int idi[IPT], rki[IPT], pid[IPT], li[IPT];
    bool vi[IPT];
    float ahx[IPT], alx[IPT], ahy[IPT], aly[IPT], ahz[IPT], alz[IPT], ahp[IPT], alp[IPT];
    int ngb[IPT], rk[IPT], idmax[IPT], idmin[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        li[k] = lane + k * W;
        vi[k] = li[k] < ni;
        int p = vi[k] ? A.i_idx[i0 + ib + li[k]] : p_first;
        if ((unsigned)p >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; vi[k] = false; }
        pid[k] = p;
        const SoftPtcl r = A.iptcl[p];
        const double dx = r.x - ox, dy = r.y - oy, dz = r.z - oz;
        xi[k] = __double2float_rn(dx);
        yi[k] = __double2float_rn(dy);
        zi[k] = __double2float_rn(dz);
        xl[k] = __double2float_rn(dx - (double)xi[k]);
        yl[k] = __double2float_rn(dy - (double)yi[k]);
        zl[k] = __double2float_rn(dz - (double)zi[k]);
        ro2i[k] = r.ro2;
        rs2i[k] = r.rs2;
        idi[k] = r.id_local;
        rki[k] = r.rank;
        ahx[k] = alx[k] = ahy[k] = aly[k] = ahz[k] = alz[k] = ahp[k] = alp[k] = 0.f;
        ngb[k] = 0; rk[k] = 0; idmax[k] = -1; idmin[k] = INT32_MAX_;
    }
    if (EMIT) {
        for (int t = tid; t < ni; t += SB) scnt[t] = 0;
    }
    // Screen prefilter.  The force's r^2 (residue-corrected displacement, FMA)
    // differs from the screen's exact r^2 by FP32 rounding (< 6e-7 relative)
    // and by the residues, |delta| <= 1.06e-7 (2 L + r_s) for a pair inside
    // the search radius r_s, L the group's largest local coordinate.  With
    // L <= 2e4 r_s,min the force's r^2 stays below 1.01 r_s^2 for every pair
    // the exact screen accepts, so skipping pairs above that is exact.
    bool pre_ok;
    {
        float L = 0.f, rmin2 = 3.0e38f;
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (vi[k]) {
                L = fmaxf(L, fmaxf(fabsf(xi[k]), fmaxf(fabsf(yi[k]), fabsf(zi[k]))));
                rmin2 = fminf(rmin2, rs2i[k]);
            }
        pre_ok = __syncthreads_and(L * L <= 4.0e8f * rmin2) != 0;
    }

    // ---- EP-EP ----
    for (int base = 0; base < nj; base += TJ) {
        const int nt = min(TJ, nj - base);
        __syncthreads();
        if (tid < nt) {
            int p = A.j_idx[j0 + base + tid];
            if ((unsigned)p >= (unsigned)A.n_ptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; }
            const SoftPtcl r = A.ptcl[p];
            const double dx = r.x - ox, dy = r.y - oy, dz = r.z - oz;
            const float hx = __double2float_rn(dx), hy = __double2float_rn(dy), hz = __double2float_rn(dz);
            sa[tid] = make_float4(hx, hy, hz, r.m);
            sb[tid] = make_float4(r.ro2, r.rs2, __int_as_float(r.id_local), __int_as_float(r.rank));
            sc[tid] = make_float4(__double2float_rn(dx - (double)hx), __double2float_rn(dy - (double)hy),
                                  __double2float_rn(dz - (double)hz), 0.f);
            if (EMIT) sidx[tid] = p;
        }
        __syncthreads();
        const int jb = sub * (TJ / S), je = min(jb + TJ / S, nt);
        for (int c0 = jb; c0 < je; c0 += CHUNK) {
            const int c1 = min(c0 + CHUNK, je);
            float tx[IPT], ty[IPT], tz[IPT], tp[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) tx[k] = ty[k] = tz[k] = tp[k] = 0.f;
#pragma unroll 4
            for (int jj = c0; jj < c1; jj++) {
                const float4 a = sa[jj];
                const float4 b = sb[jj];
                const float4 c = sc[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    // the functor's FP32 displacement (screen) ...
                    const float hx = xi[k] - a.x, hy = yi[k] - a.y, hz = zi[k] - a.z;
                    // ... and the same displacement with the low parts restored (force)
                    const float rx = hx + (xl[k] - c.x), ry = hy + (yl[k] - c.y), rz = hz + (zl[k] - c.z);
                    const float r2f = fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, eps2)));
                    const float r2 = fmaxf(r2f, fmaxf(ro2i[k], b.x));
                    float ri = rsqrtf(r2);
                    ri = ri * fmaf(-0.5f * r2, ri * ri, 1.5f);
                    const float mr = a.w * ri;
                    const float mr3 = mr * (ri * ri);
                    tx[k] = fmaf(mr3, rx, tx[k]);
                    ty[k] = fmaf(mr3, ry, ty[k]);
                    tz[k] = fmaf(mr3, rz, tz[k]);
                    tp[k] += mr;
                    // the exact screen only where the force's r^2 is within 1 % of
                    // the search radius (pre_ok: proven to miss no neighbour)
                    const float rs2 = fmaxf(rs2i[k], b.y);
                    if (pre_ok && !(r2f < 1.01f * rs2)) continue;
                    const float r2r =
                        __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(hx, hx), __fmul_rn(hy, hy)), __fmul_rn(hz, hz)), eps2);
                    if (r2r < rs2) {
                        const int idj = __float_as_int(b.z), rkj = __float_as_int(b.w);
                        if ((idi[k] != idj || rki[k] != rkj) && vi[k]) {
                            ngb[k] += 1;
                            rk[k] += abs(rki[k] - rkj);
                            idmax[k] = max(idmax[k], idj);
                            idmin[k] = min(idmin[k], idj);
                            if (EMIT) {
                                const int slot = atomicAdd(&scnt[li[k]], 1);
                                if (slot < A.cand_cap)
                                    A.cand[(size_t)pid[k] * A.cand_cap + slot] = sidx[jj];
                                else
                                    atomicOr(A.status, ST_CAND_OVERFLOW);
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                fold(ahx[k], alx[k], tx[k]);
                fold(ahy[k], aly[k], ty[k]);
                fold(ahz[k], alz[k], tz[k]);
                fold(ahp[k], alp[k], tp[k]);
            }
        }
    }

    // ---- EP-SP (quadrupole) ----
    for (int base = 0; base < ns; base += TJ) {
        const int nt = min(TJ, ns - base);
        __syncthreads();
        if (tid < nt) {
            int q = A.s_idx[s0 + base + tid];
            if ((unsigned)q >= (unsigned)A.n_spj) { atomicOr(A.status, ST_BAD_INDEX); q = 0; }
            const SPJRec &r = A.spj[q];
            const float qxx = (float)r.xx, qyy = (float)r.yy, qzz = (float)r.zz;
            const float qxy = (float)r.xy, qyz = (float)r.yz, qzx = (float)r.xz;
            const float tr = A.trace_mode ? (float)(r.xx + r.yy + r.zz) : (float)(r.xx + r.yy + r.xx);
            sa[tid] = make_float4(__double2float_rn(r.pos[0] - ox), __double2float_rn(r.pos[1] - oy),
                                  __double2float_rn(r.pos[2] - oz), (float)r.mass);
            sb[tid] = make_float4(3.0f * qxx - tr, 3.0f * qyy - tr, 3.0f * qzz - tr, -(eps2 * tr));
            sc[tid] = make_float4(3.0f * qxy, 3.0f * qyz, 3.0f * qzx, 0.f);
        }
        __syncthreads();
        const int jb = sub * (TJ / S), je = min(jb + TJ / S, nt);
        for (int c0 = jb; c0 < je; c0 += CHUNK) {
            const int c1 = min(c0 + CHUNK, je);
            float tx[IPT], ty[IPT], tz[IPT], tp[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) tx[k] = ty[k] = tz[k] = tp[k] = 0.f;
#pragma unroll 2
            for (int jj = c0; jj < c1; jj++) {
                const float4 a = sa[jj];
                const float4 q1 = sb[jj];
                const float4 q2 = sc[jj];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const float rx = a.x - xi[k], ry = a.y - yi[k], rz = a.z - zi[k];
                    const float r2 = fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, eps2)));
                    // rsqrt without the Newton step: its 2-ulp error is far below the
                    // quadrupole truncation of a far cell
                    const float ri = rsqrtf(r2);
                    const float r2i = ri * ri;
                    const float r3i = r2i * ri;
                    const float r4i = r2i * r2i;
                    const float r5i = r2i * r3i;
                    const float qrx = fmaf(q1.x, rx, fmaf(q2.x, ry, q2.z * rz));
                    const float qry = fmaf(q1.y, ry, fmaf(q2.y, rz, q2.x * rx));
                    const float qrz = fmaf(q1.z, rz, fmaf(q2.z, rx, q2.y * ry));
                    const float rqr = fmaf(qrx, rx, fmaf(qry, ry, fmaf(qrz, rz, q1.w)));
                    const float rqr4 = rqr * r4i;
                    const float meff = fmaf(0.5f, rqr4, a.w);
                    const float meff3 = fmaf(2.5f, rqr4, a.w) * r3i;
                    tx[k] = fmaf(r5i, qrx, fmaf(-meff3, rx, tx[k]));
                    ty[k] = fmaf(r5i, qry, fmaf(-meff3, ry, ty[k]));
                    tz[k] = fmaf(r5i, qrz, fmaf(-meff3, rz, tz[k]));
                    tp[k] = fmaf(meff, ri, tp[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                fold(ahx[k], alx[k], tx[k]);
                fold(ahy[k], aly[k], ty[k]);
                fold(ahz[k], alz[k], tz[k]);
                fold(ahp[k], alp[k], tp[k]);
            }
        }
    }

    // ---- combine sub-blocks in a fixed order and write ForceGrav ----
    if (S > 1) {
        __syncthreads();
        float *f = redf + tid * 8;
        f[0] = ahx[0]; f[1] = alx[0]; f[2] = ahy[0]; f[3] = aly[0];
        f[4] = ahz[0]; f[5] = alz[0]; f[6] = ahp[0]; f[7] = alp[0];
        int *q = redi + tid * 4;
        q[0] = ngb[0]; q[1] = rk[0]; q[2] = idmax[0]; q[3] = idmin[0];
        __syncthreads();
        if (sub == 0) {
            for (int s = 1; s < S; s++) {
                const float *h = redf + (tid + s * W) * 8;
                const int *c = redi + (tid + s * W) * 4;
                fold(ahx[0], alx[0], h[0]); alx[0] += h[1];
                fold(ahy[0], aly[0], h[2]); aly[0] += h[3];
                fold(ahz[0], alz[0], h[4]); alz[0] += h[5];
                fold(ahp[0], alp[0], h[6]); alp[0] += h[7];
                ngb[0] += c[0]; rk[0] += c[1];
                idmax[0] = max(idmax[0], c[2]); idmin[0] = min(idmin[0], c[3]);
            }
        }
    }
    if (sub == 0) {
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            if (!vi[k]) continue;
            ForceRec &o = A.force[pid[k]];
            ForceRec r;
            if (A.accumulate) {
                r = o;
            } else {
                r.acc[0] = r.acc[1] = r.acc[2] = r.phi = 0.f;
                r.number = 0; r.rank = 0; r.id_max = -1; r.id_min = INT32_MAX_;
            }
            r.acc[0] -= ahx[k] + alx[k];
            r.acc[1] -= ahy[k] + aly[k];
            r.acc[2] -= ahz[k] + alz[k];
            r.phi -= ahp[k] + alp[k];
            r.number += ngb[k];
            r.rank += rk[k];
            r.id_max = max(idmax[k], r.id_max);
            r.id_min = min(idmin[k], r.id_min);
            o = r;
        }
    }
}

template <bool EMIT>
__global__ void __launch_bounds__(SB, 4) soft_mixed_kernel(SoftArgs A) {
    __shared__ float4 sa[TJ], sb[TJ], sc[TJ];
    __shared__ int sidx[EMIT ? TJ : 1];
    __shared__ int scnt[EMIT ? 2 * SB : 1];
    __shared__ float redf[SB * 8];
    __shared__ int redi[SB * 4];
    const int g = A.group_order ? A.group_order[blockIdx.x] : blockIdx.x;
    const int ni_all = A.i_off[g + 1] - A.i_off[g];
    // groups above 2 * SB members (not produced by a tree with
    // n_group_limit <= 256) run as consecutive chunks over the same lists
    for (int ib = 0; ib < ni_all; ib += 2 * SB) {
        const int ni = min(2 * SB, ni_all - ib);
        if (ni > A.t_ipt2)
            group_mixed<1, 2, EMIT>(A, g, ib, ni, sa, sb, sc, sidx, scnt, redf, redi);
        else if (ni > A.t_s1)
            group_mixed<1, 1, EMIT>(A, g, ib, ni, sa, sb, sc, sidx, scnt, redf, redi);
        else if (ni > A.t_s2)
            group_mixed<2, 1, EMIT>(A, g, ib, ni, sa, sb, sc, sidx, scnt, redf, redi);
        else
            group_mixed<4, 1, EMIT>(A, g, ib, ni, sa, sb, sc, sidx, scnt, redf, redi);
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// plain FP64
template <int S, int IPT, bool EMIT>
__device__ __forceinline__ void group_f64(const SoftArgs &A, int g, int ib, int ni, D4 *da, D4 *db, D4 *dc,
                                          int2 *dids, int *sidx, int *scnt, double *redd, int *redi) {
    constexpr int W = SB / S;
    const int tid = threadIdx.x;
    const int sub = tid / W, lane = tid % W;
    const int i0 = A.i_off[g];
    const int j0 = A.j_off[g], nj = A.j_off[g + 1] - j0;
    const int s0 = A.s_off[g], ns = A.s_off[g + 1] - s0;
    const double eps2 = A.eps2_d;

    double xi[IPT], yi[IPT], zi[IPT], roi[IPT], rsi[IPT];
    int idi[IPT], rki[IPT], pid[IPT], li[IPT];
    bool vi[IPT];
    double ax[IPT], ay[IPT], az[IPT], ap[IPT];
    int ngb[IPT], rk[IPT], idmax[IPT], idmin[IPT];
    const int p_first = A.i_idx[i0];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        li[k] = lane + k * W;
        vi[k] = li[k] < ni;
        int p = vi[k] ? A.i_idx[i0 + ib + li[k]] : p_first;
        if ((unsigned)p >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; vi[k] = false; }
        pid[k] = p;
        xi[k] = A.iptcl[p].x; yi[k] = A.iptcl[p].y; zi[k] = A.iptcl[p].z;
        roi[k] = A.i_r_out[p]; rsi[k] = A.i_r_search[p];
        idi[k] = A.iptcl[p].id_local; rki[k] = A.iptcl[p].rank;
        ax[k] = ay[k] = az[k] = ap[k] = 0.;
        ngb[k] = 0; rk[k] = 0; idmax[k] = -1; idmin[k] = INT32_MAX_;
    }
    if (EMIT)
        for (int t = tid; t < ni; t += SB) scnt[t] = 0;

    for (int base = 0; base < nj; base += TJ) {
        const int nt = min(TJ, nj - base);
        __syncthreads();
        if (tid < nt) {
            int p = A.j_idx[j0 + base + tid];
            if ((unsigned)p >= (unsigned)A.n_ptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; }
            const SoftPtcl &r = A.ptcl[p];
            da[tid] = D4c(r.x, r.y, r.z, A.mass[p]);
            db[tid] = D4c(A.r_out[p], A.r_search[p], 0., 0.);
            dids[tid] = make_int2(r.id_local, r.rank);
            if (EMIT) sidx[tid] = p;
        }
        __syncthreads();
        const int jb = sub * (TJ / S), je = min(jb + TJ / S, nt);
        for (int jj = jb; jj < je; jj++) {
            const D4 a = da[jj];
            const D4 b = db[jj];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                const double rx = xi[k] - a.x, ry = yi[k] - a.y, rz = zi[k] - a.z;
                const double ro = fmax(roi[k], b.x), rs = fmax(rsi[k], b.y);
                const double r2r = rx * rx + ry * ry + rz * rz + eps2;
                const double r2 = fmax(r2r, ro * ro);
                const double ri = 1.0 / sqrt(r2);
                const double mr = a.w * ri;
                const double mr3 = mr * ri * ri;
                ax[k] += mr3 * rx;
                ay[k] += mr3 * ry;
                az[k] += mr3 * rz;
                ap[k] += mr;
                if (r2r < rs * rs * 1.0201) {
                    const int idj = dids[jj].x, rkj = dids[jj].y;
                    if ((idi[k] != idj || rki[k] != rkj) && vi[k]) {
                        ngb[k] += 1;
                        rk[k] += abs(rki[k] - rkj);
                        idmax[k] = max(idmax[k], idj);
                        idmin[k] = min(idmin[k], idj);
                        if (EMIT) {
                            const int slot = atomicAdd(&scnt[li[k]], 1);
                            if (slot < A.cand_cap)
                                A.cand[(size_t)pid[k] * A.cand_cap + slot] = sidx[jj];
                            else
                                atomicOr(A.status, ST_CAND_OVERFLOW);
                        }
                    }
                }
            }
        }
    }
    for (int base = 0; base < ns; base += TJ) {
        const int nt = min(TJ, ns - base);
        __syncthreads();
        if (tid < nt) {
            int q = A.s_idx[s0 + base + tid];
            if ((unsigned)q >= (unsigned)A.n_spj) { atomicOr(A.status, ST_BAD_INDEX); q = 0; }
            const SPJRec &r = A.spj[q];
            const double tr = A.trace_mode ? r.xx + r.yy + r.zz : r.xx + r.yy + r.xx;
            da[tid] = D4c(r.pos[0], r.pos[1], r.pos[2], r.mass);
            db[tid] = D4c(3. * r.xx - tr, 3. * r.yy - tr, 3. * r.zz - tr, -(eps2 * tr));
            dc[tid] = D4c(3. * r.xy, 3. * r.yz, 3. * r.xz, 0.);
        }
        __syncthreads();
        const int jb = sub * (TJ / S), je = min(jb + TJ / S, nt);
        for (int jj = jb; jj < je; jj++) {
            const D4 a = da[jj], q1 = db[jj], q2 = dc[jj];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                const double rx = a.x - xi[k], ry = a.y - yi[k], rz = a.z - zi[k];
                const double r2 = rx * rx + ry * ry + rz * rz + eps2;
                const double ri = 1.0 / sqrt(r2);
                const double r2i = ri * ri, r3i = r2i * ri, r4i = r2i * r2i, r5i = r2i * r3i;
                const double qrx = q1.x * rx + q2.x * ry + q2.z * rz;
                const double qry = q1.y * ry + q2.y * rz + q2.x * rx;
                const double qrz = q1.z * rz + q2.z * rx + q2.y * ry;
                const double rqr = q1.w + qrx * rx + qry * ry + qrz * rz;
                const double rqr4 = rqr * r4i;
                const double meff = a.w + 0.5 * rqr4;
                const double meff3 = (a.w + 2.5 * rqr4) * r3i;
                ax[k] += r5i * qrx - meff3 * rx;
                ay[k] += r5i * qry - meff3 * ry;
                az[k] += r5i * qrz - meff3 * rz;
                ap[k] += meff * ri;
            }
        }
    }
    if (S > 1) {
        __syncthreads();
        double *f = redd + tid * 4;
        f[0] = ax[0]; f[1] = ay[0]; f[2] = az[0]; f[3] = ap[0];
        int *q = redi + tid * 4;
        q[0] = ngb[0]; q[1] = rk[0]; q[2] = idmax[0]; q[3] = idmin[0];
        __syncthreads();
        if (sub == 0) {
            for (int s = 1; s < S; s++) {
                const double *h = redd + (tid + s * W) * 4;
                const int *c = redi + (tid + s * W) * 4;
                ax[0] += h[0]; ay[0] += h[1]; az[0] += h[2]; ap[0] += h[3];
                ngb[0] += c[0]; rk[0] += c[1];
                idmax[0] = max(idmax[0], c[2]); idmin[0] = min(idmin[0], c[3]);
            }
        }
    }
    if (sub == 0) {
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            if (!vi[k]) continue;
            D4 &o4 = A.acc64[pid[k]];
            D4 r4 = A.accumulate ? o4 : D4c(0., 0., 0., 0.);
            r4.x -= ax[k]; r4.y -= ay[k]; r4.z -= az[k]; r4.w -= ap[k];
            o4 = r4;
            ForceRec &o = A.force[pid[k]];
            ForceRec r;
            if (A.accumulate) {
                r = o;
            } else {
                r.number = 0; r.rank = 0; r.id_max = -1; r.id_min = INT32_MAX_;
            }
            r.acc[0] = (float)r4.x; r.acc[1] = (float)r4.y; r.acc[2] = (float)r4.z; r.phi = (float)r4.w;
            r.number += ngb[k];
            r.rank += rk[k];
            r.id_max = max(idmax[k], r.id_max);
            r.id_min = min(idmin[k], r.id_min);
            o = r;
        }
    }
}

template <bool EMIT>
__global__ void __launch_bounds__(SB, 2) soft_f64_kernel(SoftArgs A) {
    __shared__ D4 da[TJ], db[TJ], dc[TJ];
    __shared__ int2 dids[TJ];
    __shared__ int sidx[EMIT ? TJ : 1];
    __shared__ int scnt[EMIT ? 2 * SB : 1];
    __shared__ double redd[SB * 4];
    __shared__ int redi[SB * 4];
    const int g = A.group_order ? A.group_order[blockIdx.x] : blockIdx.x;
    const int ni_all = A.i_off[g + 1] - A.i_off[g];
    for (int ib = 0; ib < ni_all; ib += 2 * SB) {
        const int ni = min(2 * SB, ni_all - ib);
        if (ni > A.t_ipt2)
            group_f64<1, 2, EMIT>(A, g, ib, ni, da, db, dc, dids, sidx, scnt, redd, redi);
        else if (ni > A.t_s1)
            group_f64<1, 1, EMIT>(A, g, ib, ni, da, db, dc, dids, sidx, scnt, redd, redi);
        else if (ni > A.t_s2)
            group_f64<2, 1, EMIT>(A, g, ib, ni, da, db, dc, dids, sidx, scnt, redd, redi);
        else
            group_f64<4, 1, EMIT>(A, g, ib, ni, da, db, dc, dids, sidx, scnt, redd, redi);
        __syncthreads();
    }
}

// --------------------------------------------------------------------------
// EPJGrav records -> SoftPtcl (+ FP64 side arrays for the FP64 form)
__global__ void pack_epj_kernel(const EPJRec *__restrict__ in, int n, SoftPtcl *out, double *mass, double *r_out,
                                double *r_search) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const EPJRec &e = in[i];
    SoftPtcl r;
    r.x = e.pos[0];
    r.y = e.pos[1];
    r.z = e.pos[2];
    r.m = (float)e.mass;
    const float ro = (float)e.r_out, rs = (float)e.r_search;
    r.ro2 = __fmul_rn(ro, ro);
    r.rs2 = __fmul_rn(__fmul_rn(rs, rs), 1.0201f);
    r.id_local = e.id_local;
    r.rank = e.myrank;
    r.pad = 0;
    out[i] = r;
    mass[i] = e.mass;
    r_out[i] = e.r_out;
    r_search[i] = e.r_search;
}

__global__ void pack_epi_kernel(const EPIRec *__restrict__ in, int n, SoftPtcl *out, double *r_out, double *r_search) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const EPIRec &e = in[i];
    SoftPtcl r;
    r.x = e.pos[0];
    r.y = e.pos[1];
    r.z = e.pos[2];
    r.m = 0.f;
    const float ro = (float)e.r_out, rs = (float)e.r_search;
    r.ro2 = __fmul_rn(ro, ro);
    r.rs2 = __fmul_rn(__fmul_rn(rs, rs), 1.0201f);
    r.id_local = e.id_local;
    r.rank = e.myrank;
    r.pad = 0;
    out[i] = r;
    r_out[i] = e.r_out;
    r_search[i] = e.r_search;
}

__global__ void iota_kernel(int *out, int n, int base) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = base + i;
}

cudaError_t launch_pack_epi(const EPIRec *in, int n, SoftPtcl *out, double *r_out, double *r_search, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    pack_epi_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, out, r_out, r_search);
    return cudaGetLastError();
}

cudaError_t launch_iota(int *out, int n, int base, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(out, n, base);
    return cudaGetLastError();
}

cudaError_t launch_pack_epj(const EPJRec *in, int n, SoftPtcl *out, double *mass, double *r_out, double *r_search,
                            cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    pack_epj_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, out, mass, r_out, r_search);
    return cudaGetLastError();
}

cudaError_t launch_soft(const SoftArgs &Ain, int precision, bool emit, cudaStream_t st) {
    SoftArgs A = Ain;
    if (A.n_group <= 0) return cudaSuccess;
    if (A.t_ipt2 <= 0 && A.t_s1 <= 0 && A.t_s2 <= 0) {
        A.t_ipt2 = 128;
        A.t_s1 = 64;
        A.t_s2 = 32;
    }
    if (precision == 0) {
        if (emit)
            soft_mixed_kernel<true><<<A.n_group, SB, 0, st>>>(A);
        else
            soft_mixed_kernel<false><<<A.n_group, SB, 0, st>>>(A);
    } else {
        if (emit)
            soft_f64_kernel<true><<<A.n_group, SB, 0, st>>>(A);
        else
            soft_f64_kernel<false><<<A.n_group, SB, 0, st>>>(A);
    }
    return cudaGetLastError();
}

}  // namespace p3t
