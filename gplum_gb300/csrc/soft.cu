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
//   ni > 128 : 2 consecutive i per thread   ni in (64,128] : 1 i per thread
//   (t_ipt2 = 256: one i per thread throughout, groups above 128 in chunks)
//   ni in (32,64] : two sub-blocks of 64 threads, each taking half of every
//   j tile      ni <= 32 : four sub-blocks of 32 threads, a quarter each.
// Sub-block partial sums are combined in a fixed order, so results do not
// depend on scheduling.  Warps whose i-slots all lie past ni skip the pair
// loops, so the issue slots spent follow ni in steps of 32 i-slots.
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
#include <mutex>

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
//
// Packed pairs: every FP32 operation of the pair loops acts on two list
// entries at once (float2 through fma.rn.f32x2 / add.rn.f32x2 /
// mul.rn.f32x2, one issue slot for two lanes' worth of FP32 work).  A tile
// is staged pair-interleaved -- entries 2q and 2q+1 side by side in each
// float4 -- so one shared-memory load yields ready packed operands.  The
// tile's j coordinates (and, for superparticles, the quadrupole terms) are
// stored negated, so every difference is an addition and the superparticle
// terms come out with the force's sign; each product and sum is the exact
// negation of the unnegated one.  A tile is padded with massless entries
// 1e18 away, which contribute exact zeros; the pair loops run over the
// entries rounded up to a multiple of 16.
//
// Displacements.  EP-EP: from the two-float splits (SoftSplit),
// r = (xh_i - xh_j) + (xl_i - xl_j) in FP32: the first difference rounds
// relative to r itself and the split carries x to ~2^-48, so r keeps ~1e-7
// relative precision however far the pair sits from the group origin.
// EP-SP: relative to the group origin (the functor's epi[0]), each side's
// local coordinate rounded from its split, rn((xh - oxh) + (xl - oxl)).
// No FP64 arithmetic in the staging except the functor's own local
// coordinates of the j-particles, which the exact neighbour screen needs.
//
// Neighbour screen: inside the loop a pair only sets a bit when the force's
// r^2 lies below 1.01 max(r_s,i^2, r_s,j^2) (precomputed per i and per j as
// 1.01 r_s^2: x -> rn(1.01 x) is monotone, so the max commutes); after each
// chunk of 32 entries the flagged pairs alone are re-screened exactly, in
// list order, with the functor's FP32 arithmetic on its own rounded local
// coordinates rn(x - x_epi[0]).
constexpr int TM = 128;     // list entries per mixed-form tile
constexpr int TP = TM / 2;  // entry pairs per tile

struct MixedTile {
    // EP-EP: a = -(xh0,xh1,yh0,yh1) b = (-zh0,-zh1,m0,m1)
    //        c = -(xl0,xl1,yl0,yl1) d = (-zl0,-zl1,ro2_0,ro2_1) e = (t0,t1) t = 1.01 rs2_j
    // EP-SP: a = -(x0,x1,y0,y1) local  b = (-z0,-z1,m0,m1)
    //        c = -(q'xx, q'yy)         d = (-q'zz, -mtr)   f = -(3qxy, 3qyz)  e = -(3qzx)
    float4 a[TP], b[TP], c[TP], d[TP], f[TP];
    float2 e[TP];
    float4 r[TM];  // EP-EP exact screen: the functor's local (x, y, z) and rs2
    int2 q[TM];    // EP-EP (id_local, rank)
    int idx[TM];   // EP-EP particle index of each entry (candidate emission)
};

__device__ __forceinline__ float rsqrt_ftz(float x) {
    // MUFU reciprocal square root; every argument here is a normal positive float
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float2 rsqrt2(float2 v) { return make_float2(rsqrt_ftz(v.x), rsqrt_ftz(v.y)); }
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }
__device__ __forceinline__ void put2(float4 *arr, int t, int comp, float v) {
    // entry t's value of packed component comp (0: .x/.y, 1: .z/.w)
    reinterpret_cast<float *>(arr)[4 * (t >> 1) + 2 * comp + (t & 1)] = v;
}

template <int S, int IPT, bool EMIT, int UNR>
__device__ __forceinline__ void group_mixed(const SoftArgs &A, int g, int ib, int ni, MixedTile &T, float4 *sI,
                                            int4 *sQ, int *scnt, float *redf, int *redi) {
    // i-particles [ib, ib + ni) of group g (ni <= 2 * SB); the origin is the
    // group's first i-particle, as in the functor
    constexpr int W = SB / S;
    const int tid = threadIdx.x;
    const int sub = tid / W, lane = tid % W;
    const int i0 = A.i_off[g];
    const int j0 = A.j_off[g], nj = A.j_off[g + 1] - j0;
    const int s0 = A.s_off[g], ns = A.s_off[g + 1] - s0;
    const float eps2 = A.eps2;
    const float2 eps2_2 = dup2(eps2);

    int p_first = A.i_idx[i0];
    if ((unsigned)p_first >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p_first = 0; }
    const double ox = A.iptcl[p_first].x, oy = A.iptcl[p_first].y, oz = A.iptcl[p_first].z;
    const SoftSplit o = A.isplit[p_first];

    // per i, in registers: split position (EP-EP force), r_out^2 and the
    // flag threshold; in shared memory (sI, sQ, one slot per thread and i;
    // read only by the exact screen and the final write): the functor's local
    // coordinates, rs2, id_local, rank, the particle index
    float xh[IPT], yh[IPT], zh[IPT], xl[IPT], yl[IPT], zl[IPT], xf[IPT], yf[IPT], zf[IPT];
    float ro2i[IPT], thi[IPT];
    int li[IPT];
    bool vi[IPT];
    float ahx[IPT], alx[IPT], ahy[IPT], aly[IPT], ahz[IPT], alz[IPT], ahp[IPT], alp[IPT];
    int ngb[IPT], rk[IPT], idmax[IPT], idmin[IPT];
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        li[k] = lane * IPT + k;
        vi[k] = li[k] < ni;
        int p = vi[k] ? A.i_idx[i0 + ib + li[k]] : p_first;
        if ((unsigned)p >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; vi[k] = false; }
        const SoftPtcl r = A.iptcl[p];
        const SoftSplit sp = A.isplit[p];
        xf[k] = __double2float_rn(r.x - ox);
        yf[k] = __double2float_rn(r.y - oy);
        zf[k] = __double2float_rn(r.z - oz);
        sI[tid * IPT + k] = make_float4(xf[k], yf[k], zf[k], r.rs2);
        sQ[tid * IPT + k] = make_int4(r.id_local, r.rank, p, 0);
        xh[k] = sp.xh; yh[k] = sp.yh; zh[k] = sp.zh;
        xl[k] = sp.xl; yl[k] = sp.yl; zl[k] = sp.zl;
        ro2i[k] = r.ro2;
        ahx[k] = alx[k] = ahy[k] = aly[k] = ahz[k] = alz[k] = ahp[k] = alp[k] = 0.f;
        ngb[k] = 0; rk[k] = 0; idmax[k] = -1; idmin[k] = INT32_MAX_;
    }
    // a warp whose i-slots all lie past the group skips the pair loops (it
    // still stages tiles and meets every barrier)
    const bool wact = (lane & ~31) * IPT < ni;
    if (EMIT) {
        for (int t = tid; t < ni; t += SB) scnt[t] = 0;
    }
    // Screen prefilter.  The force's r^2 (split displacement, FMA) is within
    // 5e-7 relative of the exact r^2; the functor's differs from the exact one
    // by its rounding of the local coordinates, |delta| <= 1.06e-7 (2 L + r_s)
    // per component for a pair inside the search radius r_s, L the group's
    // largest local coordinate.  With L <= 2e4 r_s,min the force's r^2 stays
    // below 1.01 r_s^2 for every pair the exact screen accepts, so leaving
    // pairs above that unflagged is exact; otherwise every pair is flagged.
    {
        float L = 0.f, rmin2 = 3.0e38f;
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (vi[k]) {
                L = fmaxf(L, fmaxf(fabsf(xf[k]), fmaxf(fabsf(yf[k]), fabsf(zf[k]))));
                rmin2 = fminf(rmin2, sI[tid * IPT + k].w);
            }
        const bool pre_ok = __syncthreads_and(L * L <= 4.0e8f * rmin2) != 0;
#pragma unroll
        for (int k = 0; k < IPT; k++) thi[k] = pre_ok ? 1.01f * sI[tid * IPT + k].w : 3.0e38f;
    }
    const float2 c15 = dup2(1.5f), cm05 = dup2(-0.5f);

    // ---- EP-EP ----
    for (int base = 0; base < nj; base += TM) {
        const int nt = min(TM, nj - base);
        __syncthreads();
        for (int t = tid; t < TM; t += SB) {
            if (t < nt) {
                int p = A.j_idx[j0 + base + t];
                if ((unsigned)p >= (unsigned)A.n_ptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; }
                const SoftSplit sp = A.jsplit[p];
                const SoftPtcl &r = A.ptcl[p];
                const double x = r.x, y = r.y, z = r.z;
                const float rs2 = r.rs2;
                const int id = r.id_local, rank = r.rank;
                put2(T.a, t, 0, -sp.xh); put2(T.a, t, 1, -sp.yh);
                put2(T.b, t, 0, -sp.zh); put2(T.b, t, 1, sp.m);
                put2(T.c, t, 0, -sp.xl); put2(T.c, t, 1, -sp.yl);
                put2(T.d, t, 0, -sp.zl); put2(T.d, t, 1, sp.ro2);
                reinterpret_cast<float *>(T.e)[t] = 1.01f * rs2;
                T.r[t] = make_float4(__double2float_rn(x - ox), __double2float_rn(y - oy), __double2float_rn(z - oz),
                                     rs2);
                T.q[t] = make_int2(id, rank);
                if (EMIT) T.idx[t] = p;
            } else {  // padding: massless, far away, never flagged
                put2(T.a, t, 0, -1.0e18f); put2(T.a, t, 1, -1.0e18f);
                put2(T.b, t, 0, -1.0e18f); put2(T.b, t, 1, 0.f);
                put2(T.c, t, 0, 0.f); put2(T.c, t, 1, 0.f);
                put2(T.d, t, 0, 0.f); put2(T.d, t, 1, 0.f);
                reinterpret_cast<float *>(T.e)[t] = 0.f;
                T.r[t] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
                T.q[t] = make_int2(-1, -1);
            }
        }
        __syncthreads();
        // this sub-block's share of the tile, in chunks of 32 entries (the last
        // one of a list may be 16)
        const int jb = sub * (TM / S);
        const int je = wact ? min(jb + TM / S, (nt + 15) & ~15) : jb;
        for (int c0 = jb; c0 < je; c0 += CHUNK) {
            const int nq = min(CHUNK, je - c0) >> 1;  // entry pairs in this chunk: 16, or 8 at a list's end
            float2 tx[IPT], ty[IPT], tz[IPT], tp[IPT];
            unsigned nm[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                tx[k] = ty[k] = tz[k] = tp[k] = dup2(0.f);
                nm[k] = 0u;
            }
#pragma unroll UNR
            for (int q = 0; q < nq; q++) {
                const int pq = (c0 >> 1) + q;
                const float4 a = T.a[pq], b = T.b[pq], c = T.c[pq], d = T.d[pq];
                const float2 e = T.e[pq];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    const float2 rx = __fadd2_rn(__fadd2_rn(dup2(xh[k]), lo2(a)), __fadd2_rn(dup2(xl[k]), lo2(c)));
                    const float2 ry = __fadd2_rn(__fadd2_rn(dup2(yh[k]), hi2(a)), __fadd2_rn(dup2(yl[k]), hi2(c)));
                    const float2 rz = __fadd2_rn(__fadd2_rn(dup2(zh[k]), lo2(b)), __fadd2_rn(dup2(zl[k]), lo2(d)));
                    const float2 r2f = __ffma2_rn(rx, rx, __ffma2_rn(ry, ry, __ffma2_rn(rz, rz, eps2_2)));
                    const float2 r2 = make_float2(fmaxf(r2f.x, fmaxf(ro2i[k], d.z)), fmaxf(r2f.y, fmaxf(ro2i[k], d.w)));
                    float2 ri = rsqrt2(r2);
                    ri = __fmul2_rn(ri, __ffma2_rn(__fmul2_rn(cm05, r2), __fmul2_rn(ri, ri), c15));
                    const float2 mr = __fmul2_rn(hi2(b), ri);
                    const float2 mr3 = __fmul2_rn(mr, __fmul2_rn(ri, ri));
                    tx[k] = __ffma2_rn(mr3, rx, tx[k]);
                    ty[k] = __ffma2_rn(mr3, ry, ty[k]);
                    tz[k] = __ffma2_rn(mr3, rz, tz[k]);
                    tp[k] = __fadd2_rn(tp[k], mr);
                    if (r2f.x < fmaxf(thi[k], e.x)) nm[k] |= 1u << (2 * q);
                    if (r2f.y < fmaxf(thi[k], e.y)) nm[k] |= 2u << (2 * q);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                fold(ahx[k], alx[k], tx[k].x + tx[k].y);
                fold(ahy[k], aly[k], ty[k].x + ty[k].y);
                fold(ahz[k], alz[k], tz[k].x + tz[k].y);
                fold(ahp[k], alp[k], tp[k].x + tp[k].y);
                // exact screen of the flagged pairs, in list order
                unsigned m = vi[k] ? nm[k] : 0u;
                if (m) {
                    const float4 me = sI[tid * IPT + k];
                    const int4 mq = sQ[tid * IPT + k];
                    do {
                    const int jj = c0 + __ffs(m) - 1;
                    m &= m - 1;
                    const float4 rr = T.r[jj];
                    const float hx = __fsub_rn(me.x, rr.x);
                    const float hy = __fsub_rn(me.y, rr.y);
                    const float hz = __fsub_rn(me.z, rr.z);
                    const float r2r =
                        __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(hx, hx), __fmul_rn(hy, hy)), __fmul_rn(hz, hz)), eps2);
                    if (r2r < fmaxf(me.w, rr.w)) {
                        const int2 qq = T.q[jj];
                        const int idj = qq.x, rkj = qq.y;
                        if (mq.x != idj || mq.y != rkj) {
                            ngb[k] += 1;
                            rk[k] += abs(mq.y - rkj);
                            idmax[k] = max(idmax[k], idj);
                            idmin[k] = min(idmin[k], idj);
                            if (EMIT) {
                                const int slot = atomicAdd(&scnt[li[k]], 1);
                                if (slot < A.cand_cap)
                                    A.cand[(size_t)mq.z * A.cand_cap + slot] = T.idx[jj];
                                else
                                    atomicOr(A.status, ST_CAND_OVERFLOW);
                            }
                        }
                    }
                    } while (m);
                }
            }
        }
    }

    // ---- EP-SP (quadrupole) ----
    // origin-relative FP32 coordinates of the i-particles
#pragma unroll
    for (int k = 0; k < IPT; k++) {
        xf[k] = __fadd_rn(__fsub_rn(xh[k], o.xh), __fsub_rn(xl[k], o.xl));
        yf[k] = __fadd_rn(__fsub_rn(yh[k], o.yh), __fsub_rn(yl[k], o.yl));
        zf[k] = __fadd_rn(__fsub_rn(zh[k], o.zh), __fsub_rn(zl[k], o.zl));
    }
    const float2 c05 = dup2(-0.5f), c25 = dup2(-2.5f);
    for (int base = 0; base < ns; base += TM) {
        const int nt = min(TM, ns - base);
        __syncthreads();
        for (int t = tid; t < TM; t += SB) {
            if (t < nt) {
                int q = A.s_idx[s0 + base + t];
                if ((unsigned)q >= (unsigned)A.n_spj) { atomicOr(A.status, ST_BAD_INDEX); q = 0; }
                const float4 *rp = reinterpret_cast<const float4 *>(A.spjp + q);
                const float4 p0 = rp[0], p1 = rp[1], p2 = rp[2], p3 = rp[3];
                // -(local coordinate) = (oxh - xh) + (oxl - xl)
                put2(T.a, t, 0, __fadd_rn(__fsub_rn(o.xh, p0.x), __fsub_rn(o.xl, p1.x)));
                put2(T.a, t, 1, __fadd_rn(__fsub_rn(o.yh, p0.y), __fsub_rn(o.yl, p1.y)));
                put2(T.b, t, 0, __fadd_rn(__fsub_rn(o.zh, p0.z), __fsub_rn(o.zl, p1.z)));
                put2(T.b, t, 1, p0.w);
                put2(T.c, t, 0, p2.x);
                put2(T.c, t, 1, p2.y);
                put2(T.d, t, 0, p2.z);
                put2(T.d, t, 1, p1.w);
                put2(T.f, t, 0, p2.w);
                put2(T.f, t, 1, p3.x);
                reinterpret_cast<float *>(T.e)[t] = p3.y;
            } else {  // padding: massless, far away
                put2(T.a, t, 0, -1.0e18f); put2(T.a, t, 1, -1.0e18f);
                put2(T.b, t, 0, -1.0e18f); put2(T.b, t, 1, 0.f);
                put2(T.c, t, 0, 0.f); put2(T.c, t, 1, 0.f);
                put2(T.d, t, 0, 0.f); put2(T.d, t, 1, 0.f);
                put2(T.f, t, 0, 0.f); put2(T.f, t, 1, 0.f);
                reinterpret_cast<float *>(T.e)[t] = 0.f;
            }
        }
        __syncthreads();
        const int jb = sub * (TM / S);
        const int je = wact ? min(jb + TM / S, (nt + 15) & ~15) : jb;
        for (int c0 = jb; c0 < je; c0 += CHUNK) {
            const int nq = min(CHUNK, je - c0) >> 1;  // entry pairs in this chunk: 16, or 8 at a list's end
            float2 tx[IPT], ty[IPT], tz[IPT], tp[IPT];
#pragma unroll
            for (int k = 0; k < IPT; k++) tx[k] = ty[k] = tz[k] = tp[k] = dup2(0.f);
#pragma unroll 4
            for (int q = 0; q < nq; q++) {
                const int pq = (c0 >> 1) + q;
                const float4 a = T.a[pq], b = T.b[pq], c = T.c[pq], d = T.d[pq], f = T.f[pq];
                const float2 e = T.e[pq];
#pragma unroll
                for (int k = 0; k < IPT; k++) {
                    // r' = x_i - x_j (the negated displacement); with the tile's
                    // negated quadrupole, qr = -Q'r' and nrqr = -(mtr + r'Q'r')
                    const float2 rx = __fadd2_rn(dup2(xf[k]), lo2(a));
                    const float2 ry = __fadd2_rn(dup2(yf[k]), hi2(a));
                    const float2 rz = __fadd2_rn(dup2(zf[k]), lo2(b));
                    const float2 r2 = __ffma2_rn(rx, rx, __ffma2_rn(ry, ry, __ffma2_rn(rz, rz, eps2_2)));
                    // rsqrt without the Newton step: its 2-ulp error is far below the
                    // quadrupole truncation of a far cell
                    const float2 ri = rsqrt2(r2);
                    const float2 r2i = __fmul2_rn(ri, ri);
                    const float2 r3i = __fmul2_rn(r2i, ri);
                    const float2 r4i = __fmul2_rn(r2i, r2i);
                    const float2 r5i = __fmul2_rn(r2i, r3i);
                    const float2 qrx = __ffma2_rn(lo2(c), rx, __ffma2_rn(lo2(f), ry, __fmul2_rn(e, rz)));
                    const float2 qry = __ffma2_rn(hi2(c), ry, __ffma2_rn(hi2(f), rz, __fmul2_rn(lo2(f), rx)));
                    const float2 qrz = __ffma2_rn(lo2(d), rz, __ffma2_rn(e, rx, __fmul2_rn(hi2(f), ry)));
                    const float2 nrqr = __ffma2_rn(qrx, rx, __ffma2_rn(qry, ry, __ffma2_rn(qrz, rz, hi2(d))));
                    const float2 nrqr4 = __fmul2_rn(nrqr, r4i);
                    const float2 meff = __ffma2_rn(c05, nrqr4, hi2(b));
                    const float2 meff3 = __fmul2_rn(__ffma2_rn(c25, nrqr4, hi2(b)), r3i);
                    // acc_i += r5i Q'r - meff3 r  with r = -r'
                    tx[k] = __ffma2_rn(r5i, qrx, __ffma2_rn(meff3, rx, tx[k]));
                    ty[k] = __ffma2_rn(r5i, qry, __ffma2_rn(meff3, ry, ty[k]));
                    tz[k] = __ffma2_rn(r5i, qrz, __ffma2_rn(meff3, rz, tz[k]));
                    tp[k] = __ffma2_rn(meff, ri, tp[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; k++) {
                fold(ahx[k], alx[k], tx[k].x + tx[k].y);
                fold(ahy[k], aly[k], ty[k].x + ty[k].y);
                fold(ahz[k], alz[k], tz[k].x + tz[k].y);
                fold(ahp[k], alp[k], tp[k].x + tp[k].y);
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
            ForceRec &o = A.force[sQ[tid * IPT + k].z];
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

// One i-particle per thread throughout (groups above SB members run as
// chunks of SB over the same lists): the packed pair loops keep two list
// entries in flight per thread, and the register budget this leaves allows
// OCC resident CTAs per SM (the autotuner picks 4, 5 or 6).
template <bool EMIT, int OCC>
__global__ void __launch_bounds__(SB, OCC) soft_mixed_kernel(SoftArgs A) {
    __shared__ MixedTile T;
    __shared__ float4 sI[SB];
    __shared__ int4 sQ[SB];
    __shared__ int scnt[EMIT ? SB : 1];
    __shared__ float redf[SB * 8];
    __shared__ int redi[SB * 4];
    const int g = A.group_order ? A.group_order[blockIdx.x] : blockIdx.x;
    const int ni_all = A.i_off[g + 1] - A.i_off[g];
    // EP-EP unroll depth: as deep as the register budget holds without spills
    constexpr int UNR = OCC <= 4 ? 8 : 2;
    for (int ib = 0; ib < ni_all; ib += SB) {
        const int ni = min(SB, ni_all - ib);
        if (ni > A.t_s1)
            group_mixed<1, 1, EMIT, UNR>(A, g, ib, ni, T, sI, sQ, scnt, redf, redi);
        else if (ni > A.t_s2)
            group_mixed<2, 1, EMIT, UNR>(A, g, ib, ni, T, sI, sQ, scnt, redf, redi);
        else
            group_mixed<4, 1, EMIT, UNR>(A, g, ib, ni, T, sI, sQ, scnt, redf, redi);
        __syncthreads();
    }
}

// the mixed kernel's staging: pipelined (1) or gather-then-compute (0, the
// default: at 1M bodies 1.046 ms per pass against 1.062 pipelined -- with six
// CTAs per SM the gather's latency is already hidden, and the FMA pipe, not
// the staging, bounds the pass)
int g_soft_pipe = 0;

// --------------------------------------------------------------------------
// mixed precision, pipelined staging
//
// The same arithmetic, in the same order, as group_mixed with one i per
// thread; only the staging of the tiles differs.  There the CTA gathered a
// tile (global loads, FP64 shifts, shared stores), met a barrier, computed it
// and met a second barrier, so the gather's latency stood between every two
// tiles.  Here the EP-EP tiles and then the EP-SP tiles form one sequence: a
// thread copies the records of its entry of tile t + 2 into a raw staging
// slot with cp.async while the CTA computes tile t, and converts tile t + 1
// from the raw slot into the second tile buffer at the start of tile t's
// turn -- one barrier per tile, the global latency behind a tile of pair
// work.  A thread reads back only the raw slot it copied itself.
struct __align__(16) RawEntry {
    float4 v[5];  // EP-EP: SoftSplit (v[0..1]), SoftPtcl (v[2..4]); EP-SP: SpjPack (v[0..3])
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

struct PipeSmem {
    MixedTile T[2];
    RawEntry raw[TM];  // also the sub-block reduction's space at the end of a group
    float4 sI[SB];
    int4 sQ[SB];
};

// list entry e of tile t (EP-EP tiles first): its record copies started;
// returns the particle / superparticle index, -1 for padding
__device__ __forceinline__ int pipe_issue(const SoftArgs &A, int t, int Tep, int j0, int nj, int s0, int ns, int e,
                                          RawEntry &R) {
    if (t < Tep) {
        const int k = t * TM + e;
        if (k >= nj) return -1;
        int p = A.j_idx[j0 + k];
        if ((unsigned)p >= (unsigned)A.n_ptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; }
        const float4 *sp = reinterpret_cast<const float4 *>(A.jsplit + p);
        const float4 *rp = reinterpret_cast<const float4 *>(A.ptcl + p);
        cp_async16(&R.v[0], sp);
        cp_async16(&R.v[1], sp + 1);
        cp_async16(&R.v[2], rp);
        cp_async16(&R.v[3], rp + 1);
        cp_async16(&R.v[4], rp + 2);
        return p;
    }
    const int k = (t - Tep) * TM + e;
    if (k >= ns) return -1;
    int q = A.s_idx[s0 + k];
    if ((unsigned)q >= (unsigned)A.n_spj) { atomicOr(A.status, ST_BAD_INDEX); q = 0; }
    const float4 *qp = reinterpret_cast<const float4 *>(A.spjp + q);
    cp_async16(&R.v[0], qp);
    cp_async16(&R.v[1], qp + 1);
    cp_async16(&R.v[2], qp + 2);
    cp_async16(&R.v[3], qp + 3);
    return q;
}

// entry e of tile t from its raw slot into tile buffer T (group_mixed's staging arithmetic)
template <bool EMIT>
__device__ __forceinline__ void pipe_convert(int t, int Tep, int e, int p, const RawEntry &R, MixedTile &T, double ox,
                                             double oy, double oz, const SoftSplit &o) {
    if (t < Tep) {
        if (p >= 0) {
            const SoftSplit &sp = *reinterpret_cast<const SoftSplit *>(&R.v[0]);
            const SoftPtcl &r = *reinterpret_cast<const SoftPtcl *>(&R.v[2]);
            const double x = r.x, y = r.y, z = r.z;
            const float rs2 = r.rs2;
            put2(T.a, e, 0, -sp.xh); put2(T.a, e, 1, -sp.yh);
            put2(T.b, e, 0, -sp.zh); put2(T.b, e, 1, sp.m);
            put2(T.c, e, 0, -sp.xl); put2(T.c, e, 1, -sp.yl);
            put2(T.d, e, 0, -sp.zl); put2(T.d, e, 1, sp.ro2);
            reinterpret_cast<float *>(T.e)[e] = 1.01f * rs2;
            T.r[e] = make_float4(__double2float_rn(x - ox), __double2float_rn(y - oy), __double2float_rn(z - oz), rs2);
            T.q[e] = make_int2(r.id_local, r.rank);
            if (EMIT) T.idx[e] = p;
        } else {  // padding: massless, far away, never flagged
            put2(T.a, e, 0, -1.0e18f); put2(T.a, e, 1, -1.0e18f);
            put2(T.b, e, 0, -1.0e18f); put2(T.b, e, 1, 0.f);
            put2(T.c, e, 0, 0.f); put2(T.c, e, 1, 0.f);
            put2(T.d, e, 0, 0.f); put2(T.d, e, 1, 0.f);
            reinterpret_cast<float *>(T.e)[e] = 0.f;
            T.r[e] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
            T.q[e] = make_int2(-1, -1);
        }
        return;
    }
    if (p >= 0) {
        const float4 p0 = R.v[0], p1 = R.v[1], p2 = R.v[2], p3 = R.v[3];
        put2(T.a, e, 0, __fadd_rn(__fsub_rn(o.xh, p0.x), __fsub_rn(o.xl, p1.x)));
        put2(T.a, e, 1, __fadd_rn(__fsub_rn(o.yh, p0.y), __fsub_rn(o.yl, p1.y)));
        put2(T.b, e, 0, __fadd_rn(__fsub_rn(o.zh, p0.z), __fsub_rn(o.zl, p1.z)));
        put2(T.b, e, 1, p0.w);
        put2(T.c, e, 0, p2.x);
        put2(T.c, e, 1, p2.y);
        put2(T.d, e, 0, p2.z);
        put2(T.d, e, 1, p1.w);
        put2(T.f, e, 0, p2.w);
        put2(T.f, e, 1, p3.x);
        reinterpret_cast<float *>(T.e)[e] = p3.y;
    } else {  // padding: massless, far away
        put2(T.a, e, 0, -1.0e18f); put2(T.a, e, 1, -1.0e18f);
        put2(T.b, e, 0, -1.0e18f); put2(T.b, e, 1, 0.f);
        put2(T.c, e, 0, 0.f); put2(T.c, e, 1, 0.f);
        put2(T.d, e, 0, 0.f); put2(T.d, e, 1, 0.f);
        put2(T.f, e, 0, 0.f); put2(T.f, e, 1, 0.f);
        reinterpret_cast<float *>(T.e)[e] = 0.f;
    }
}

template <int S, bool EMIT, int UNR>
__device__ __forceinline__ void group_mixed_pipe(const SoftArgs &A, int g, int ib, int ni, PipeSmem &M, int *scnt) {
    constexpr int W = SB / S;
    const int tid = threadIdx.x;
    const int sub = tid / W, lane = tid % W;
    const int i0 = A.i_off[g];
    const int j0 = A.j_off[g], nj = A.j_off[g + 1] - j0;
    const int s0 = A.s_off[g], ns = A.s_off[g + 1] - s0;
    const float eps2 = A.eps2;
    const float2 eps2_2 = dup2(eps2);

    int p_first = A.i_idx[i0];
    if ((unsigned)p_first >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p_first = 0; }
    const double ox = A.iptcl[p_first].x, oy = A.iptcl[p_first].y, oz = A.iptcl[p_first].z;
    const SoftSplit o = A.isplit[p_first];

    // the i-particle of this thread (group_mixed with IPT = 1)
    float xh, yh, zh, xl, yl, zl, xf, yf, zf, ro2i, thi;
    const int li = lane;
    bool vi = li < ni;
    float ahx = 0.f, alx = 0.f, ahy = 0.f, aly = 0.f, ahz = 0.f, alz = 0.f, ahp = 0.f, alp = 0.f;
    int ngb = 0, rk = 0, idmax = -1, idmin = INT32_MAX_;
    {
        int p = vi ? A.i_idx[i0 + ib + li] : p_first;
        if ((unsigned)p >= (unsigned)A.n_iptcl) { atomicOr(A.status, ST_BAD_INDEX); p = 0; vi = false; }
        const SoftPtcl r = A.iptcl[p];
        const SoftSplit sp = A.isplit[p];
        xf = __double2float_rn(r.x - ox);
        yf = __double2float_rn(r.y - oy);
        zf = __double2float_rn(r.z - oz);
        M.sI[tid] = make_float4(xf, yf, zf, r.rs2);
        M.sQ[tid] = make_int4(r.id_local, r.rank, p, 0);
        xh = sp.xh; yh = sp.yh; zh = sp.zh;
        xl = sp.xl; yl = sp.yl; zl = sp.zl;
        ro2i = r.ro2;
    }
    const bool wact = (lane & ~31) < ni;
    if (EMIT) {
        for (int t = tid; t < ni; t += SB) scnt[t] = 0;
    }
    {
        float L = 0.f, rmin2 = 3.0e38f;
        if (vi) {
            L = fmaxf(fabsf(xf), fmaxf(fabsf(yf), fabsf(zf)));
            rmin2 = M.sI[tid].w;
        }
        const bool pre_ok = __syncthreads_and(L * L <= 4.0e8f * rmin2) != 0;
        thi = pre_ok ? 1.01f * M.sI[tid].w : 3.0e38f;
    }
    const float2 c15 = dup2(1.5f), cm05 = dup2(-0.5f);
    const float2 c05 = dup2(-0.5f), c25 = dup2(-2.5f);

    const int Tep = (nj + TM - 1) / TM, Tn = Tep + (ns + TM - 1) / TM;
    RawEntry &R = M.raw[tid];
    int pn = -1;
    if (Tn > 0) {
        pn = pipe_issue(A, 0, Tep, j0, nj, s0, ns, tid, R);
        cp_async_commit();
        cp_async_wait_all();
        pipe_convert<EMIT>(0, Tep, tid, pn, R, M.T[0], ox, oy, oz, o);
    }
    if (Tn > 1) {
        pn = pipe_issue(A, 1, Tep, j0, nj, s0, ns, tid, R);
        cp_async_commit();
    }
    __syncthreads();
    for (int t = 0; t < Tn; t++) {
        const int cur = t & 1;
        if (t + 1 < Tn) {
            cp_async_wait_all();
            pipe_convert<EMIT>(t + 1, Tep, tid, pn, R, M.T[cur ^ 1], ox, oy, oz, o);
        }
        if (t + 2 < Tn) {
            pn = pipe_issue(A, t + 2, Tep, j0, nj, s0, ns, tid, R);
            cp_async_commit();
        }
        const MixedTile &T = M.T[cur];
        const int jb = sub * (TM / S);
        if (t < Tep) {
            // ---- EP-EP ----
            const int nt = min(TM, nj - t * TM);
            const int je = wact ? min(jb + TM / S, (nt + 15) & ~15) : jb;
            for (int c0 = jb; c0 < je; c0 += CHUNK) {
                const int nq = min(CHUNK, je - c0) >> 1;
                float2 tx = dup2(0.f), ty = dup2(0.f), tz = dup2(0.f), tp = dup2(0.f);
                unsigned nm = 0u;
#pragma unroll UNR
                for (int q = 0; q < nq; q++) {
                    const int pq = (c0 >> 1) + q;
                    const float4 a = T.a[pq], b = T.b[pq], c = T.c[pq], d = T.d[pq];
                    const float2 e = T.e[pq];
                    const float2 rx = __fadd2_rn(__fadd2_rn(dup2(xh), lo2(a)), __fadd2_rn(dup2(xl), lo2(c)));
                    const float2 ry = __fadd2_rn(__fadd2_rn(dup2(yh), hi2(a)), __fadd2_rn(dup2(yl), hi2(c)));
                    const float2 rz = __fadd2_rn(__fadd2_rn(dup2(zh), lo2(b)), __fadd2_rn(dup2(zl), lo2(d)));
                    const float2 r2f = __ffma2_rn(rx, rx, __ffma2_rn(ry, ry, __ffma2_rn(rz, rz, eps2_2)));
                    const float2 r2 = make_float2(fmaxf(r2f.x, fmaxf(ro2i, d.z)), fmaxf(r2f.y, fmaxf(ro2i, d.w)));
                    float2 ri = rsqrt2(r2);
                    ri = __fmul2_rn(ri, __ffma2_rn(__fmul2_rn(cm05, r2), __fmul2_rn(ri, ri), c15));
                    const float2 mr = __fmul2_rn(hi2(b), ri);
                    const float2 mr3 = __fmul2_rn(mr, __fmul2_rn(ri, ri));
                    tx = __ffma2_rn(mr3, rx, tx);
                    ty = __ffma2_rn(mr3, ry, ty);
                    tz = __ffma2_rn(mr3, rz, tz);
                    tp = __fadd2_rn(tp, mr);
                    if (r2f.x < fmaxf(thi, e.x)) nm |= 1u << (2 * q);
                    if (r2f.y < fmaxf(thi, e.y)) nm |= 2u << (2 * q);
                }
                fold(ahx, alx, tx.x + tx.y);
                fold(ahy, aly, ty.x + ty.y);
                fold(ahz, alz, tz.x + tz.y);
                fold(ahp, alp, tp.x + tp.y);
                unsigned m = vi ? nm : 0u;
                if (m) {
                    const float4 me = M.sI[tid];
                    const int4 mq = M.sQ[tid];
                    do {
                        const int jj = c0 + __ffs(m) - 1;
                        m &= m - 1;
                        const float4 rr = T.r[jj];
                        const float hx = __fsub_rn(me.x, rr.x);
                        const float hy = __fsub_rn(me.y, rr.y);
                        const float hz = __fsub_rn(me.z, rr.z);
                        const float r2r =
                            __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(hx, hx), __fmul_rn(hy, hy)), __fmul_rn(hz, hz)), eps2);
                        if (r2r < fmaxf(me.w, rr.w)) {
                            const int2 qq = T.q[jj];
                            const int idj = qq.x, rkj = qq.y;
                            if (mq.x != idj || mq.y != rkj) {
                                ngb += 1;
                                rk += abs(mq.y - rkj);
                                idmax = max(idmax, idj);
                                idmin = min(idmin, idj);
                                if (EMIT) {
                                    const int slot = atomicAdd(&scnt[li], 1);
                                    if (slot < A.cand_cap)
                                        A.cand[(size_t)mq.z * A.cand_cap + slot] = T.idx[jj];
                                    else
                                        atomicOr(A.status, ST_CAND_OVERFLOW);
                                }
                            }
                        }
                    } while (m);
                }
            }
        } else {
            // ---- EP-SP (quadrupole) ----
            if (t == Tep) {  // origin-relative FP32 coordinates of the i-particle
                xf = __fadd_rn(__fsub_rn(xh, o.xh), __fsub_rn(xl, o.xl));
                yf = __fadd_rn(__fsub_rn(yh, o.yh), __fsub_rn(yl, o.yl));
                zf = __fadd_rn(__fsub_rn(zh, o.zh), __fsub_rn(zl, o.zl));
            }
            const int nt = min(TM, ns - (t - Tep) * TM);
            const int je = wact ? min(jb + TM / S, (nt + 15) & ~15) : jb;
            for (int c0 = jb; c0 < je; c0 += CHUNK) {
                const int nq = min(CHUNK, je - c0) >> 1;
                float2 tx = dup2(0.f), ty = dup2(0.f), tz = dup2(0.f), tp = dup2(0.f);
#pragma unroll 4
                for (int q = 0; q < nq; q++) {
                    const int pq = (c0 >> 1) + q;
                    const float4 a = T.a[pq], b = T.b[pq], c = T.c[pq], d = T.d[pq], f = T.f[pq];
                    const float2 e = T.e[pq];
                    const float2 rx = __fadd2_rn(dup2(xf), lo2(a));
                    const float2 ry = __fadd2_rn(dup2(yf), hi2(a));
                    const float2 rz = __fadd2_rn(dup2(zf), lo2(b));
                    const float2 r2 = __ffma2_rn(rx, rx, __ffma2_rn(ry, ry, __ffma2_rn(rz, rz, eps2_2)));
                    const float2 ri = rsqrt2(r2);
                    const float2 r2i = __fmul2_rn(ri, ri);
                    const float2 r3i = __fmul2_rn(r2i, ri);
                    const float2 r4i = __fmul2_rn(r2i, r2i);
                    const float2 r5i = __fmul2_rn(r2i, r3i);
                    const float2 qrx = __ffma2_rn(lo2(c), rx, __ffma2_rn(lo2(f), ry, __fmul2_rn(e, rz)));
                    const float2 qry = __ffma2_rn(hi2(c), ry, __ffma2_rn(hi2(f), rz, __fmul2_rn(lo2(f), rx)));
                    const float2 qrz = __ffma2_rn(lo2(d), rz, __ffma2_rn(e, rx, __fmul2_rn(hi2(f), ry)));
                    const float2 nrqr = __ffma2_rn(qrx, rx, __ffma2_rn(qry, ry, __ffma2_rn(qrz, rz, hi2(d))));
                    const float2 nrqr4 = __fmul2_rn(nrqr, r4i);
                    const float2 meff = __ffma2_rn(c05, nrqr4, hi2(b));
                    const float2 meff3 = __fmul2_rn(__ffma2_rn(c25, nrqr4, hi2(b)), r3i);
                    tx = __ffma2_rn(r5i, qrx, __ffma2_rn(meff3, rx, tx));
                    ty = __ffma2_rn(r5i, qry, __ffma2_rn(meff3, ry, ty));
                    tz = __ffma2_rn(r5i, qrz, __ffma2_rn(meff3, rz, tz));
                    tp = __ffma2_rn(meff, ri, tp);
                }
                fold(ahx, alx, tx.x + tx.y);
                fold(ahy, aly, ty.x + ty.y);
                fold(ahz, alz, tz.x + tz.y);
                fold(ahp, alp, tp.x + tp.y);
            }
        }
        __syncthreads();
    }
    // ---- combine sub-blocks in a fixed order and write ForceGrav ----
    if (S > 1) {
        float *redf = reinterpret_cast<float *>(M.raw);
        int *redi = reinterpret_cast<int *>(redf + SB * 8);
        float *f = redf + tid * 8;
        f[0] = ahx; f[1] = alx; f[2] = ahy; f[3] = aly;
        f[4] = ahz; f[5] = alz; f[6] = ahp; f[7] = alp;
        int *q = redi + tid * 4;
        q[0] = ngb; q[1] = rk; q[2] = idmax; q[3] = idmin;
        __syncthreads();
        if (sub == 0) {
            for (int s2 = 1; s2 < S; s2++) {
                const float *h = redf + (tid + s2 * W) * 8;
                const int *c = redi + (tid + s2 * W) * 4;
                fold(ahx, alx, h[0]); alx += h[1];
                fold(ahy, aly, h[2]); aly += h[3];
                fold(ahz, alz, h[4]); alz += h[5];
                fold(ahp, alp, h[6]); alp += h[7];
                ngb += c[0]; rk += c[1];
                idmax = max(idmax, c[2]); idmin = min(idmin, c[3]);
            }
        }
    }
    if (sub == 0 && vi) {
        ForceRec &orec = A.force[M.sQ[tid].z];
        ForceRec r;
        if (A.accumulate) {
            r = orec;
        } else {
            r.acc[0] = r.acc[1] = r.acc[2] = r.phi = 0.f;
            r.number = 0; r.rank = 0; r.id_max = -1; r.id_min = INT32_MAX_;
        }
        r.acc[0] -= ahx + alx;
        r.acc[1] -= ahy + aly;
        r.acc[2] -= ahz + alz;
        r.phi -= ahp + alp;
        r.number += ngb;
        r.rank += rk;
        r.id_max = max(idmax, r.id_max);
        r.id_min = min(idmin, r.id_min);
        orec = r;
    }
}

template <bool EMIT, int OCC>
__global__ void __launch_bounds__(SB, OCC) soft_mixed_pipe_kernel(SoftArgs A) {
    __shared__ PipeSmem M;
    __shared__ int scnt[EMIT ? SB : 1];
    const int g = A.group_order ? A.group_order[blockIdx.x] : blockIdx.x;
    const int ni_all = A.i_off[g + 1] - A.i_off[g];
    constexpr int UNR = OCC <= 4 ? 8 : 2;
    for (int ib = 0; ib < ni_all; ib += SB) {
        const int ni = min(SB, ni_all - ib);
        if (ni > A.t_s1)
            group_mixed_pipe<1, EMIT, UNR>(A, g, ib, ni, M, scnt);
        else if (ni > A.t_s2)
            group_mixed_pipe<2, EMIT, UNR>(A, g, ib, ni, M, scnt);
        else
            group_mixed_pipe<4, EMIT, UNR>(A, g, ib, ni, M, scnt);
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
        li[k] = lane * IPT + k;
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
    const bool wact = (lane & ~31) * IPT < ni;
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
        const int jb = sub * (TJ / S), je = wact ? min(jb + TJ / S, nt) : jb;
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
        const int jb = sub * (TJ / S), je = wact ? min(jb + TJ / S, nt) : jb;
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
    const int span = A.t_ipt2 >= 2 * SB ? SB : 2 * SB;
    for (int ib = 0; ib < ni_all; ib += span) {
        const int ni = min(span, ni_all - ib);
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
    { P3T_COUNT_LAUNCH(); pack_epi_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, out, r_out, r_search); }
    return cudaGetLastError();
}

cudaError_t launch_iota(int *out, int n, int base, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    { P3T_COUNT_LAUNCH(); iota_kernel<<<(n + 255) / 256, 256, 0, st>>>(out, n, base); }
    return cudaGetLastError();
}

cudaError_t launch_pack_epj(const EPJRec *in, int n, SoftPtcl *out, double *mass, double *r_out, double *r_search,
                            cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    { P3T_COUNT_LAUNCH(); pack_epj_kernel<<<(n + 255) / 256, 256, 0, st>>>(in, n, out, mass, r_out, r_search); }
    return cudaGetLastError();
}

// Mixed-form preprocessing: per-particle splits and packed superparticles.
__global__ void split_kernel(const SoftPtcl *__restrict__ p, int n, SoftSplit *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SoftPtcl r = p[i];
    SoftSplit s;
    s.xh = __double2float_rn(r.x);
    s.yh = __double2float_rn(r.y);
    s.zh = __double2float_rn(r.z);
    s.xl = __double2float_rn(r.x - (double)s.xh);
    s.yl = __double2float_rn(r.y - (double)s.yh);
    s.zl = __double2float_rn(r.z - (double)s.zh);
    s.m = r.m;
    s.ro2 = r.ro2;
    out[i] = s;
}

__global__ void spj_pack_kernel(const SPJRec *__restrict__ in, int n, float eps2, int trace_mode, SpjPack *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const SPJRec &r = in[i];
    SpjPack s;
    s.xh = __double2float_rn(r.pos[0]);
    s.yh = __double2float_rn(r.pos[1]);
    s.zh = __double2float_rn(r.pos[2]);
    s.xl = __double2float_rn(r.pos[0] - (double)s.xh);
    s.yl = __double2float_rn(r.pos[1] - (double)s.yh);
    s.zl = __double2float_rn(r.pos[2] - (double)s.zh);
    s.m = (float)r.mass;
    const float qxx = (float)r.xx, qyy = (float)r.yy, qzz = (float)r.zz;
    const float tr = trace_mode ? (float)(r.xx + r.yy + r.zz) : (float)(r.xx + r.yy + r.xx);
    s.nmtr = eps2 * tr;
    s.nqxx = -(3.0f * qxx - tr);
    s.nqyy = -(3.0f * qyy - tr);
    s.nqzz = -(3.0f * qzz - tr);
    s.nqxy = -(3.0f * (float)r.xy);
    s.nqyz = -(3.0f * (float)r.yz);
    s.nqzx = -(3.0f * (float)r.xz);
    s.pad0 = s.pad1 = 0.f;
    out[i] = s;
}

namespace {

// launch_soft's own scratch for callers that pass none: per device, grown
// stream-ordered on the launching stream
struct MixedScratch {
    SoftSplit *isplit = nullptr, *jsplit = nullptr;
    size_t icap = 0, jcap = 0;
    SpjPack *spj = nullptr;
    size_t scap = 0;
};
constexpr int MAX_DEV = 64;
MixedScratch g_mixed[MAX_DEV];
std::mutex g_mixed_mu;

template <class T>
cudaError_t grow(T **p, size_t *cap, size_t n, cudaStream_t st) {
    if (n <= *cap) return cudaSuccess;
    if (*p) {
        cudaError_t e = cudaFreeAsync(*p, st);
        if (e != cudaSuccess) return e;
        *p = nullptr;
        *cap = 0;
    }
    const size_t want = n + n / 4 + 1024;
    cudaError_t e = cudaMallocAsync((void **)p, want * sizeof(T), st);
    if (e != cudaSuccess) return e;
    *cap = want;
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_soft(const SoftArgs &Ain, int precision, bool emit, cudaStream_t st) {
    SoftArgs A = Ain;
    if (A.n_group <= 0) return cudaSuccess;
    if (A.t_ipt2 <= 0 && A.t_s1 <= 0 && A.t_s2 <= 0) {
        A.t_ipt2 = 128;
        A.t_s1 = 64;
        A.t_s2 = 32;
    }
    if (precision == 0) {
        const bool same = A.iptcl == A.ptcl;
        if (!A.jsplit || !A.spjp || (!same && !A.isplit)) {
            int dev = 0;
            cudaError_t e = cudaGetDevice(&dev);
            if (e != cudaSuccess) return e;
            if (dev < 0 || dev >= MAX_DEV) return cudaErrorInvalidDevice;
            std::lock_guard<std::mutex> lk(g_mixed_mu);
            MixedScratch &m = g_mixed[dev];
            if ((e = grow(&m.jsplit, &m.jcap, (size_t)A.n_ptcl, st)) != cudaSuccess) return e;
            if ((e = grow(&m.spj, &m.scap, (size_t)(A.n_spj > 0 ? A.n_spj : 1), st)) != cudaSuccess) return e;
            if (!same && (e = grow(&m.isplit, &m.icap, (size_t)A.n_iptcl, st)) != cudaSuccess) return e;
            A.jsplit = m.jsplit;
            A.spjp = m.spj;
            A.isplit = m.isplit;
        }
        if (same) A.isplit = A.jsplit;
        if (A.n_ptcl > 0) { P3T_COUNT_LAUNCH(); split_kernel<<<(A.n_ptcl + 255) / 256, 256, 0, st>>>(A.ptcl, A.n_ptcl, A.jsplit); }
        if (!same && A.n_iptcl > 0)
            { P3T_COUNT_LAUNCH(); split_kernel<<<(A.n_iptcl + 255) / 256, 256, 0, st>>>(A.iptcl, A.n_iptcl, A.isplit); }
        if (A.n_spj > 0)
            { P3T_COUNT_LAUNCH(); spj_pack_kernel<<<(A.n_spj + 255) / 256, 256, 0, st>>>(A.spj, A.n_spj, A.eps2, A.trace_mode, A.spjp); }
        const int occ = A.occ ? A.occ : 5;
#define P3T_SOFT_MIXED(OCC)                                                                               \
    do {                                                                                                  \
        P3T_COUNT_LAUNCH();                                                                               \
        if (g_soft_pipe && emit) soft_mixed_pipe_kernel<true, OCC><<<A.n_group, SB, 0, st>>>(A);        \
        else if (g_soft_pipe) soft_mixed_pipe_kernel<false, OCC><<<A.n_group, SB, 0, st>>>(A);          \
        else if (emit) soft_mixed_kernel<true, OCC><<<A.n_group, SB, 0, st>>>(A);                       \
        else soft_mixed_kernel<false, OCC><<<A.n_group, SB, 0, st>>>(A);                                \
    } while (0)
        if (occ == 4)
            P3T_SOFT_MIXED(4);
        else if (occ == 6)
            P3T_SOFT_MIXED(6);
        else
            P3T_SOFT_MIXED(5);
#undef P3T_SOFT_MIXED
    } else {
        if (emit)
            { P3T_COUNT_LAUNCH(); soft_f64_kernel<true><<<A.n_group, SB, 0, st>>>(A); }
        else
            { P3T_COUNT_LAUNCH(); soft_f64_kernel<false><<<A.n_group, SB, 0, st>>>(A); }
    }
    return cudaGetLastError();
}

}  // namespace p3t

extern "C" int p3t_set_soft_pipe(int on) {
    p3t::g_soft_pipe = on ? 1 : 0;
    return 0;
}
