// Lane-dense form of the hard part: one CTA integrates a "bundle" of many
// clusters at once.
//
// FP64 runs at 1/64 of the FP32 rate on this GPU, and a warp instruction
// occupies the FP64 pipe for all 32 lanes whether or not they are active.  A
// warp (or thread) per cluster leaves most lanes idle: a cluster has a few
// active members per block step, and a serial pair loop per member has one
// live partner in several.  Here the CTA keeps up to BCAP members of up to
// bmaxcl(BCAP) clusters in shared memory and advances every cluster by one block
// step per iteration, so each phase runs over the union of the bundle's
// work items:
//   - member phases (predict, correct, time steps) over all members or all
//     active members of all clusters;
//   - pair phases over (target, partner) items: an FP32 distance prefilter
//     (with a per-cluster margin proven below) packs the live pairs into a
//     ring in (target, partner) order; their FP64 terms are computed one pair
//     per thread; the terms are then added to each target's accumulators in
//     partner order, which is the summation order of the reference loop
//     (src/gravity_hard.h:203-367), so the sums are bit-identical;
//   - collision detection over unordered member pairs, FP32 prefilter, FP64
//     R for the survivors and a per-cluster lexicographic (R, pair) minimum.
// Finished clusters leave the bundle and the queue refills it, so the CTA
// stays full until the queue is empty.  The main 256-slot bundle runs one
// thread per slot (bundle_threads: 8 warps, 2 CTAs per SM at 128 registers):
// the member phases are long dependent FP64 chains, and twice the warps of a
// 128-thread bundle keep the FP64 pipe busier (55 % vs 47 % of cycles,
// 10-11 % less time at 1M bodies).  Clusters larger than BCAP_MAIN run
// concurrently in k_hard_wide: alone in a wide bundle of BCAP_WIDE slots, or
// beyond that in the one-cluster-per-CTA form (run_cluster<128>).
//
// The global per-slot arrays (struct Hard) stay the state of record; shared
// memory mirrors the fields that other members read (positions, velocities,
// predicted state, masses, radii, ids, flags) and is refreshed after every
// phase that changes them.
//
// Prefilter margins.  FP32 coordinates are taken relative to the cluster's
// first member, u = fl32(x - ref).  While every stored |x - ref| component
// stays below E (checked at every store; a violation switches the cluster to
// exact FP64 tests for good), a computed FP32 distance exceeds the exact one
// by at most err = 3e-7 E plus 1.6e-7 relative.  A pair whose exact cutoff
// test passes (|dr|^2 r_out_inv^2 <= 1.000001) then has an FP32 value
// <= (1.000001 + err r_out_inv_max)^2 * 1.000001 =: thr_f, and a pair with
// exact R < 1 has FP32 d^2 <= thr_c (r_i + r_j)_32^2 with
// thr_c = (1.000001 + err / (2 min f r_p))^2 * 1.000001 (both rounded up to
// FP32).  Pairs above the thresholds are therefore beyond the cutoff (their
// terms are exact zeros) or have R > 1, so skipping them is exact; pairs below
// them but beyond the cutoff contribute exact +-0 terms to accumulators that
// start at +0, which leaves every sum unchanged.
#pragma once

namespace p3t {

constexpr int BT = 128;      // threads of a bundle (one CTA) unless bundle_threads says otherwise
constexpr int BPT = 4;       // (target, partner) items a thread tests per round of bundle_pairs
constexpr int BCAP_MAIN = 256;  // member slots of a bundle
constexpr int BCAP_WIDE = 512;  // member slots of the wide form (clusters of 257..512 bodies, one at a time)
// clusters in a bundle at once: half its member slots, at most one per thread
__host__ __device__ constexpr int bmaxcl(int cap) { return cap / 2 < 128 ? cap / 2 : 128; }
// threads of a bundle of `cap` member slots: one per slot for the main
// 256-slot form (8 warps; twice the warps per SM of 128 at 2 CTAs per SM,
// for the FP64 dependency chains), 128 for the others
__host__ __device__ constexpr int bundle_threads(int cap) { return cap == 256 ? 256 : (cap == 512 ? 512 : 128); }
constexpr int BSURV = 64;    // colliding-pair candidates kept per block step
constexpr int BCLAIM = 8;    // clusters claimed from the queue at a time

enum : int { CF_COL = 1, CF_FIN = 2, CF_FRESH = 4, CF_EXACT = 8 };
enum : unsigned char { MF_ACT = 1, MF_TGT = 2 };

template <int BCAP>
struct BundleSmem {
    static constexpr int NT = bundle_threads(BCAP);  // threads of the bundle
    // member mirror (pool slot p)
    double pos[3 * BCAP], vel[3 * BCAP], xp[3 * BCAP], vp[3 * BCAP];
    double mass[BCAP], roi[BCAP], fr[BCAP];
    double acc[7 * BCAP];  // force accumulators of the running pair phase
    double term[7 * NT];   // FP64 pair terms of one drain
    long long id[BCAP];
    float pos32[3 * BCAP], xp32[3 * BCAP], roi32[BCAP], fr32[BCAP];
    int gslot[BCAP];
    int pfx[BCAP + 1];
    int ring[(BPT + 1) * NT];  // live pair items: a round's BPT per thread beyond a part drain
    int seg[NT + 1];
    short tgt[BCAP], cl[BCAP], owner[BCAP];
    unsigned char dead[BCAP], merged[BCAP], flag[BCAP];
    // clusters (bundle index k)
    double c_ts[bmaxcl(BCAP)], c_ref[3 * bmaxcl(BCAP)], c_ed[bmaxcl(BCAP)], c_edd[bmaxcl(BCAP)];
    unsigned long long c_key[bmaxcl(BCAP)], c_red[4 * bmaxcl(BCAP)];
    long long c_pb[bmaxcl(BCAP)], c_work[bmaxcl(BCAP)], c_t0[bmaxcl(BCAP)];
    long long c_label[bmaxcl(BCAP)], c_fragn[bmaxcl(BCAP)];  // id_cluster, fragments made (KOMINAMI)
    int c_n0[bmaxcl(BCAP)], c_addn[bmaxcl(BCAP)], c_addg[bmaxcl(BCAP)];  // members at admission; new fragments (count, first slot)
    float c_thrf[bmaxcl(BCAP)], c_thrc[bmaxcl(BCAP)], c_E32[bmaxcl(BCAP)];
    int c_idx[bmaxcl(BCAP)], c_off[bmaxcl(BCAP)], c_n[bmaxcl(BCAP)], c_goff[bmaxcl(BCAP)], c_steps[bmaxcl(BCAP)], c_ncol[bmaxcl(BCAP)];
    int c_flags[bmaxcl(BCAP)], c_imp[bmaxcl(BCAP)], c_tar[bmaxcl(BCAP)];
    // colliding-pair candidates
    double sv_R[BSURV];
    long long sv_p[BSURV];
    int sv_k[BSURV];
    // claimed, not yet admitted clusters
    int pend_c[BCLAIM], pend_n[BCLAIM];
    int ws[NT / 32];
    int used, ncl, fresh_k, fresh_p, n_sv, n_pend, i_pend, exhausted, any, grew, phase;
    long long ph_acc[HP_N], ph_t;  // optional per-phase clock counts (thread 0)
};

// the end of a phase of the bundle loop (after its barrier): thread 0 adds
// the clock cycles since the last mark to the phase's count
#define HP_MARK(id)                                            \
    do {                                                       \
        if (A.phase_cycles && threadIdx.x == 0) {              \
            const long long t_ = clock64();                    \
            B.ph_acc[id] += t_ - B.ph_t;                       \
            B.ph_t = t_;                                       \
        }                                                      \
    } while (0)

__device__ __forceinline__ unsigned long long dbits(double x) {
    return (unsigned long long)__double_as_longlong(x);
}
__device__ __forceinline__ double bitsd(unsigned long long b) { return __longlong_as_double((long long)b); }

// exclusive block-wide prefix sum of v over NT threads; all threads must call
template <int NT>
__device__ __forceinline__ int bscan(int v, int *ws, int &total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    int off = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < NT / 32; k++) {
        const int c = ws[k];
        off += (k < w) ? c : 0;
        tot += c;
    }
    __syncthreads();
    total = tot;
    return off + x - v;
}

// FP32 copy of a position relative to the cluster origin, with the bound check
template <int BCAP>
__device__ __forceinline__ void st32b(BundleSmem<BCAP> &B, float *dst, int p, V3 x, int k) {
    const float u0 = (float)(x.x - B.c_ref[3 * k]), u1 = (float)(x.y - B.c_ref[3 * k + 1]),
                u2 = (float)(x.z - B.c_ref[3 * k + 2]);
    dst[3 * p] = u0;
    dst[3 * p + 1] = u1;
    dst[3 * p + 2] = u2;
    const float E = B.c_E32[k];
    if (!(fabsf(u0) < E && fabsf(u1) < E && fabsf(u2) < E)) atomicOr(&B.c_flags[k], CF_EXACT);
}

// mirror every field of slot p from the state of record (global slot g)
template <int BCAP>
__device__ __forceinline__ void mirror_all(BundleSmem<BCAP> &B, const Hard &H, int p, int g, int k, bool with32) {
    const V3 x = ld3(H.pos, g);
    st3(B.pos, p, x);
    st3(B.vel, p, ld3(H.vel, g));
    st3(B.xp, p, ld3(H.xp, g));
    st3(B.vp, p, ld3(H.vp, g));
    B.mass[p] = H.mass[g];
    B.roi[p] = H.r_out_inv[g];
    const double fr = H.f[g] * H.r_planet[g];
    B.fr[p] = fr;
    B.fr32[p] = (float)fr;
    B.roi32[p] = (float)H.r_out_inv[g];
    B.id[p] = H.id[g];
    B.dead[p] = (unsigned char)H.dead[g];
    B.merged[p] = (unsigned char)H.merged[g];
    B.gslot[p] = g;
    B.cl[p] = (short)k;
    if (with32) {
        st32b(B, B.pos32, p, x, k);
        st32b(B, B.xp32, p, ld3(H.xp, g), k);
    }
}

// ---- pair phases ------------------------------------------------------------
// ordered list of the occupied slots whose flag has `bit`
template <int BCAP>
__device__ int bundle_list(BundleSmem<BCAP> &B, unsigned char bit) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    constexpr int PER = BCAP / BT;
    const int base = threadIdx.x * PER;
    int c = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int p = base + j;
        if (p < B.used && (B.flag[p] & bit)) c++;
    }
    int tot;
    int off = bscan<BT>(c, B.ws, tot);
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int p = base + j;
        if (p < B.used && (B.flag[p] & bit)) B.tgt[off++] = (short)p;
    }
    __syncthreads();
    return tot;
}

// the seven terms (acc_d xyz, jerk_d xyz, -phi_d) of target s from partner t,
// the arithmetic of hard_force for one pair
template <int BCAP>
__device__ __forceinline__ void pair_terms(const Params &P, const BundleSmem<BCAP> &B, int mode, int s, int t, double *o) {
    V3 xi, vi, xj, vj;
    if (mode == 1) { xi = ld3(B.xp, s); vi = ld3(B.vp, s); }
    else { xi = ld3(B.pos, s); vi = ld3(B.vel, s); }
    if (mode == 0) { xj = ld3(B.pos, t); vj = ld3(B.vel, t); }
    else { xj = ld3(B.xp, t); vj = ld3(B.vp, t); }
    const V3 dr = xj - xi;
    double dr2 = dot(dr, dr);
    dr2 += P.eps2;
    const double r_out_inv = dmin(B.roi[s], B.roi[t]);
    const V3 dv = vj - vi;
    const double rij = sqrt(dr2);
    const double rinv = 1. / rij;
    const double r2inv = rinv * rinv;
    const double r3inv = r2inv * rinv;
    const double mj = B.mass[t];
    const double mr3 = mj * r3inv;
    const double alpha = dot(dr, dv) * r2inv;
    double Wc = 0.;
    if (mode == 0) Wc = 1. - cut_W(P, rij, r_out_inv);
    const double Kc = 1. - cut_K(P, rij, r_out_inv);
    const double dKdt = cut_dKdt(P, rij, r_out_inv, alpha);
    const double alpha_c = alpha * Kc;
    const V3 a = mr3 * Kc * dr;
    const V3 j = mr3 * (Kc * dv - (3. * alpha_c + dKdt) * dr);
    o[0] = a.x; o[1] = a.y; o[2] = a.z;
    o[3] = j.x; o[4] = j.y; o[5] = j.z;
    o[6] = (mode == 0) ? -(mj * rinv * Wc) : 0.;
}

// terms of ring[0..m), then in-order addition into the targets' accumulators
template <int BCAP>
__device__ void bundle_drain(const Params &P, BundleSmem<BCAP> &B, const int *ring, int mode, int m) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const int q = threadIdx.x;
    int sq = -1;
    if (q < m) {
        const int e = ring[q];
        sq = e >> 16;
        double o[7];
        pair_terms(P, B, mode, sq, e & 0xffff, o);
#pragma unroll
        for (int c = 0; c < 7; c++) B.term[c * BT + q] = o[c];
    }
    const int head = (q < m) && (q == 0 || (ring[q - 1] >> 16) != sq);
    int nseg;
    const int off = bscan<BT>(head, B.ws, nseg);
    if (head) B.seg[off] = q;
    if (q == 0) B.seg[nseg] = m;
    __syncthreads();
    const int ncomp = (mode == 0) ? 7 : 6;
    for (int it = q; it < ncomp * nseg; it += BT) {
        const int j = it / ncomp, c = it - ncomp * j;
        const int a = B.seg[j], b = B.seg[j + 1];
        const int s = ring[a] >> 16;
        double acc = B.acc[c * BCAP + s];
        for (int k = a; k < b; k++) acc += B.term[c * BT + k];
        B.acc[c * BCAP + s] = acc;
    }
    __syncthreads();
}

// mode 0: full (pos/vel, with phi); 1: predicted i and j; 2: corrected i,
// predicted j -- for the nt targets in B.tgt
template <int BCAP>
__device__ void bundle_pairs(const HardArgs &A, BundleSmem<BCAP> &B, int mode, int nt) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const int tid = threadIdx.x;
    constexpr int PER = BCAP / BT;
    for (int i = tid; i < nt; i += BT) {
        const int s = B.tgt[i];
#pragma unroll
        for (int c = 0; c < 7; c++) B.acc[c * BCAP + s] = 0.;
    }
    // partner-count prefix over the targets
    int total;
    {
        const int base = tid * PER;
        int c = 0;
#pragma unroll
        for (int j = 0; j < PER; j++)
            if (base + j < nt) c += B.c_n[B.cl[B.tgt[base + j]]];
        int off = bscan<BT>(c, B.ws, total);
#pragma unroll
        for (int j = 0; j < PER; j++)
            if (base + j < nt) {
                B.pfx[base + j] = off;
                off += B.c_n[B.cl[B.tgt[base + j]]];
            }
        if (tid == 0) B.pfx[nt] = total;
        __syncthreads();
    }
    const float *xi32 = (mode == 1) ? B.xp32 : B.pos32;
    const float *xj32 = (mode == 0) ? B.pos32 : B.xp32;
    // rounds of BPT consecutive items per thread (the ring stays in (target,
    // partner) order); full drains of BT items as the ring fills
    int ring_n = 0;
    long long n_live = 0;
    for (int base = 0; base < total; base += BPT * BT) {
        const int f0 = base + BPT * tid;
        int e[BPT], nl = 0;
        unsigned lv = 0u;
        if (f0 < total) {
            int lo = 0, hi = nt - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (B.pfx[mid] <= f0) lo = mid;
                else hi = mid - 1;
            }
#pragma unroll
            for (int u = 0; u < BPT; u++) {
                const int f = f0 + u;
                e[u] = 0;
                if (f >= total) continue;
                while (B.pfx[lo + 1] <= f) lo++;
                const int s = B.tgt[lo], k = B.cl[s];
                const int t = B.c_off[k] + (f - B.pfx[lo]);
                int live = 0;
                if (B.id[s] != B.id[t]) {
                    if (!(B.c_flags[k] & CF_EXACT)) {
                        const float rf = fminf(B.roi32[s], B.roi32[t]);
                        live = d2_32(xi32, s, xj32, t) * (rf * rf) <= B.c_thrf[k];
                    } else {
                        const V3 xi = ld3((mode == 1) ? B.xp : B.pos, s);
                        const V3 dr = ld3((mode == 0) ? B.pos : B.xp, t) - xi;
                        double dr2 = dot(dr, dr);
                        dr2 += A.P.eps2;
                        const double r = dmin(B.roi[s], B.roi[t]);
                        live = !(dr2 * r * r > 1.000001);
                    }
                }
                e[u] = (s << 16) | t;
                lv |= (unsigned)live << u;
                nl += live;
            }
        }
        int cnt;
        int off = ring_n + bscan<BT>(nl, B.ws, cnt);
#pragma unroll
        for (int u = 0; u < BPT; u++)
            if ((lv >> u) & 1u) B.ring[off++] = e[u];
        ring_n += cnt;
        n_live += cnt;
        __syncthreads();
        int head = 0;
        while (ring_n - head >= BT) {
            const long long t0 = (A.phase_cycles && tid == 0) ? clock64() : 0;
            bundle_drain(A.P, B, B.ring + head, mode, BT);
            if (A.phase_cycles && tid == 0) B.ph_acc[HP_DRAIN] += clock64() - t0;
            head += BT;
        }
        if (head > 0) {
            // the rest (fewer than BT items, at or beyond BT) to the front
            const int rest = ring_n - head;
            if (tid < rest) B.ring[tid] = B.ring[head + tid];
            ring_n = rest;
            __syncthreads();
        }
    }
    if (ring_n > 0) {
        const long long t0 = (A.phase_cycles && tid == 0) ? clock64() : 0;
        bundle_drain(A.P, B, B.ring, mode, ring_n);
        if (A.phase_cycles && tid == 0) B.ph_acc[HP_DRAIN] += clock64() - t0;
    }
    if (A.live && tid == 0) atomicAdd(&A.live[mode == 0 ? 1 : 0], (unsigned long long)n_live);
}

// sun force and the accumulated pair sums of the targets to the state of
// record, then mergeAccJerk for the merged targets (merge_sel 1: active
// phase, merged alive targets; 2: all merged targets with twins)
template <int BCAP>
__device__ void bundle_finalize(const HardArgs &A, BundleSmem<BCAP> &B, int mode, int nt, int merge_sel) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const Hard &H = A.H;
    for (int i = threadIdx.x; i < nt; i += BT) {
        const int s = B.tgt[i], g = B.gslot[s];
        V3 xi, vi, as, js;
        if (mode == 1) { xi = ld3(B.xp, s); vi = ld3(B.vp, s); }
        else { xi = ld3(B.pos, s); vi = ld3(B.vel, s); }
        if (mode == 0) {
            double phs;
            sun_force(A.P, xi, vi, as, js, &phs);
            H.phi_s[g] = phs;
            H.phi_d[g] = B.acc[6 * BCAP + s];
        } else {
            sun_force(A.P, xi, vi, as, js, nullptr);
        }
        st3(H.acc_s, g, as);
        st3(H.jerk_s, g, js);
        st3(H.acc_d, g, v3(B.acc[s], B.acc[BCAP + s], B.acc[2 * BCAP + s]));
        st3(H.jerk_d, g, v3(B.acc[3 * BCAP + s], B.acc[4 * BCAP + s], B.acc[5 * BCAP + s]));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nt; i += BT) {
        const int s = B.tgt[i], g = B.gslot[s];
        const bool m = (merge_sel == 1) ? (!B.dead[s] && B.merged[s]) : (B.merged[s] && H.tw_head[g] >= 0);
        if (m) merge_acc_jerk(H, g);
    }
    __syncthreads();
}

// ---- collision detection ------------------------------------------------------
// unordered pairs {a, b} of each cluster, balanced over members: member a
// takes b = a + d (mod n) for d = 1..n/2 (the pair at distance n/2 once)
template <int BCAP>
__device__ void bundle_detect(const HardArgs &A, BundleSmem<BCAP> &B, bool second) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    for (int p = threadIdx.x; p < B.used; p += BT) {
        if (B.dead[p]) continue;
        const int k = B.cl[p];
        const int o = B.c_off[k], n = B.c_n[k], a = p - o;
        const bool exact = (B.c_flags[k] & CF_EXACT) != 0;
        const float thr = B.c_thrc[k];
        for (int d = 1; 2 * d <= n; d++) {
            if (2 * d == n && a >= d) break;
            int b = a + d;
            if (b >= n) b -= n;
            const int q = o + b;
            if (B.dead[q]) continue;
            if (!exact) {
                const float rs = B.fr32[p] + B.fr32[q];
                if (d2_32(B.xp32, p, B.xp32, q) > thr * (rs * rs)) continue;
            }
            const int lo = (a < b) ? a : b, hi = (a < b) ? b : a;
            const V3 dr = ld3(B.xp, o + lo) - ld3(B.xp, o + hi);
            const double d2 = dot(dr, dr);
            const double r2 = B.fr[o + lo] + B.fr[o + hi];
            if (d2 > r2 * r2 * 1.000001) continue;
            const double R = sqrt(d2) / r2;
            if (!(R < 1.)) continue;
            const long long pp = (long long)lo * n + hi;
            if (!second) {
                atomicMin(&B.c_key[k], dbits(R));
                const int i = atomicAdd(&B.n_sv, 1);
                if (i < BSURV) {
                    B.sv_k[i] = k;
                    B.sv_R[i] = R;
                    B.sv_p[i] = pp;
                }
            } else if (dbits(R) == B.c_key[k]) {
                atomicMin(&B.c_pb[k], pp);
            }
        }
    }
}

// ---- bundle lifecycle ---------------------------------------------------------------
// warp 0: claim clusters from the queue and admit them while they fit (lane
// 0 decides, the decisions are broadcast so the warp's control flow stays
// uniform).  Phase 0: the heavy clusters (the first n_tier[3] of tier 1:
// predicted long chains of block steps), one at a time and alone in the
// bundle, so their iterations stay short; phase 1: the rest, packed.
template <int BCAP>
__device__ void bundle_refill(const HardArgs &A, BundleSmem<BCAP> &B) {
    const int lane = threadIdx.x & 31;
    const int n_heavy = A.n_tier[3];
    if (threadIdx.x < 32) {
        int lone = 0;
        if (lane == 0 && B.phase == 0) {
            if (B.ncl > 0) {
                lone = 1;  // a heavy cluster is running: nothing joins it
            } else {
                const int q = atomicAdd(&A.queue[2], 1);
                if (q < n_heavy) {
                    const int c = A.order[A.n_tier[0] + q];
                    const int k = B.ncl++;
                    B.c_idx[k] = c;
                    B.c_off[k] = 0;
                    B.c_n[k] = A.cnt[c];
                    B.c_flags[k] = CF_FRESH;
                    B.used = B.c_n[k];
                    lone = 1;
                } else {
                    B.phase = 1;
                }
            }
        }
        lone = __shfl_sync(0xffffffffu, lone, 0);
        __syncwarp();
        for (int guard = 0; !lone && guard < (1 << 20); guard++) {
            int stop = 0, claim = 0;
            if (lane == 0 && B.i_pend >= B.n_pend) {
                if (B.exhausted) stop = 1;
                else claim = 1;
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            claim = __shfl_sync(0xffffffffu, claim, 0);
            if (stop) break;
            if (claim) {
                int q = 0;
                if (lane == 0) q = atomicAdd(&A.queue[1], BCLAIM);
                q = __shfl_sync(0xffffffffu, q, 0);
                const int qi = q + lane;
                const bool ok = lane < BCLAIM && qi < A.n_tier[1] - n_heavy;
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (ok) {
                    const int c = A.order[A.n_tier[0] + n_heavy + qi];
                    B.pend_c[lane] = c;
                    B.pend_n[lane] = A.cnt[c];
                }
                __syncwarp();
                if (lane == 0) {
                    B.n_pend = __popc(m);
                    B.i_pend = 0;
                    if (__popc(m) < BCLAIM) B.exhausted = 1;
                }
                __syncwarp();
                if (m == 0u) break;
            }
            // admit in queue order
            int full = 0;
            if (lane == 0) {
                while (B.i_pend < B.n_pend) {
                    const int c = B.pend_c[B.i_pend], n = B.pend_n[B.i_pend];
                    // with fragmentation, keep room for the fragments of a collision
                    const int room = (A.frag.a_frag > 0.) ? 2 * A.frag.n_frag_max : 0;
                    if (B.used + n + room > BCAP || B.ncl >= bmaxcl(BCAP)) break;
                    const int k = B.ncl++;
                    B.c_idx[k] = c;
                    B.c_off[k] = B.used;
                    B.c_n[k] = n;
                    B.c_flags[k] = CF_FRESH;
                    B.used += n;
                    B.i_pend++;
                }
                full = B.i_pend < B.n_pend;
            }
            full = __shfl_sync(0xffffffffu, full, 0);
            __syncwarp();
            if (full) break;  // the next claimed cluster waits for space
        }
    }
    __syncthreads();
}

// load the fresh clusters (bundle indices fresh_k..ncl-1, slots fresh_p..used-1)
template <int BCAP>
__device__ void bundle_load(const HardArgs &A, BundleSmem<BCAP> &B) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const Hard &H = A.H;
    const int tid = threadIdx.x;
    const int k0 = B.fresh_k, k1 = B.ncl, p0 = B.fresh_p, p1 = B.used;
    for (int k = k0 + tid; k < k1; k += BT) {
        const int c = B.c_idx[k];
        const int goff = A.off[c];
        B.c_goff[k] = goff;
        const V3 r0 = ld3(A.S.pos, A.members[goff]);
        B.c_ref[3 * k] = r0.x; B.c_ref[3 * k + 1] = r0.y; B.c_ref[3 * k + 2] = r0.z;
        B.c_steps[k] = 0; B.c_ncol[k] = 0; B.c_work[k] = 0;
        B.c_label[k] = A.S.id_cluster[A.members[goff]];
        B.c_fragn[k] = 0;
        B.c_n0[k] = B.c_n[k];
        B.c_addn[k] = 0;
        B.c_ed[k] = 0.; B.c_edd[k] = 0.;
        B.c_t0[k] = A.times ? global_ns() : 0;
        B.c_red[4 * k] = 0ULL;                 // max |x - ref| component
        B.c_red[4 * k + 1] = 0ULL;             // max |v| component
        B.c_red[4 * k + 2] = 0ULL;             // max r_out_inv
        B.c_red[4 * k + 3] = dbits(1.e300);    // min f r_planet
    }
    __syncthreads();
    for (int p = p0 + tid; p < p1; p += BT) {
        int lo = k0, hi = k1 - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (B.c_off[mid] <= p) lo = mid;
            else hi = mid - 1;
        }
        const int k = lo, g = B.c_goff[k] + (p - B.c_off[k]), i = A.members[g];
        // FPHard(const FPGrav&), src/particle.h:1096-1116
        st3(H.pos, g, ld3(A.S.pos, i)); st3(H.vel, g, ld3(A.S.vel, i));
        st3(H.acc_s, g, ld3(A.S.acc_s, i)); st3(H.jerk_s, g, ld3(A.S.jerk_s, i));
        st3(H.acc_d, g, ld3(A.S.acc_d, i)); st3(H.jerk_d, g, ld3(A.S.jerk_d, i));
        const V3 z = v3(0., 0., 0.);
        st3(H.x0, g, z); st3(H.v0, g, z); st3(H.a0_s, g, z); st3(H.j0_s, g, z); st3(H.a0_d, g, z);
        st3(H.j0_d, g, z); st3(H.xp, g, z); st3(H.vp, g, z); st3(H.a2_s, g, z); st3(H.a3_s, g, z);
        st3(H.a2_d, g, z); st3(H.a3_d, g, z);
        H.phi_d[g] = A.S.phi_d[i]; H.phi_s[g] = A.S.phi_s[i];
        H.mass[g] = A.S.mass[i]; H.r_planet[g] = A.S.r_planet[i]; H.f[g] = A.S.f[i];
        H.r_out_inv[g] = A.S.r_out_inv[i];
        H.time_c[g] = A.S.time[i]; H.th[g] = 0.; H.dt[g] = A.S.dt[i]; H.acc0[g] = A.S.acc0[i];
        H.id[g] = A.S.id[i];
        H.dead[g] = 0; H.merged[g] = 0;
        H.tw_head[g] = H.tw_tail[g] = H.tw_next[g] = -1;
        mirror_all(B, H, p, g, k, false);
        B.owner[p] = -1;
        B.flag[p] = 0;
        const V3 x = ld3(H.pos, g), v = ld3(H.vel, g);
        const double ext = dmax(fabs(x.x - B.c_ref[3 * k]), dmax(fabs(x.y - B.c_ref[3 * k + 1]),
                                                                  fabs(x.z - B.c_ref[3 * k + 2])));
        const double vm = dmax(fabs(v.x), dmax(fabs(v.y), fabs(v.z)));
        atomicMax(&B.c_red[4 * k], dbits(ext));
        atomicMax(&B.c_red[4 * k + 1], dbits(vm));
        atomicMax(&B.c_red[4 * k + 2], dbits(B.roi[p]));
        atomicMin(&B.c_red[4 * k + 3], dbits(B.fr[p]));
    }
    __syncthreads();
    for (int k = k0 + tid; k < k1; k += BT) {
        // coordinate bound, then the prefilter thresholds (see the header)
        const double E = (bitsd(B.c_red[4 * k]) + 2. * bitsd(B.c_red[4 * k + 1]) * A.t_end) * 1.0001 + 1.e-30;
        const double err = 3.e-7 * E;
        const double rmax = bitsd(B.c_red[4 * k + 2]), frmin = bitsd(B.c_red[4 * k + 3]);
        const double tf = 1.000001 + 1.0001 * err * rmax;
        const double tc = 1.000001 + 1.0001 * err / (2. * frmin);
        B.c_thrf[k] = __double2float_ru(tf * tf * 1.000001);
        B.c_thrc[k] = (frmin > 0.) ? __double2float_ru(tc * tc * 1.000001) : __int_as_float(0x7f800000);
        B.c_E32[k] = __double2float_rd(E);
    }
    __syncthreads();
    for (int p = tid; p < p1; p += BT) {
        if (p < p0) {
            B.flag[p] = 0;
            continue;
        }
        st32b(B, B.pos32, p, ld3(B.pos, p), B.cl[p]);
        B.flag[p] = MF_TGT;
    }
    __syncthreads();
}

// member-parallel loop over the occupied slots
#define FOR_SLOTS(p) for (int p = threadIdx.x; p < B.used; p += BT)
#define FOR_CLUSTERS(k) for (int k = threadIdx.x; k < B.ncl; k += BT)

// A cluster made fragments (KOMINAMI): its member range grows by them, the
// clusters after it move up, and every slot is mirrored again from the
// state of record (fragments are rare; owners are remapped).
template <int BCAP>
__device__ void bundle_grow(const HardArgs &A, BundleSmem<BCAP> &B) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const Hard &H = A.H;
    const int tid = threadIdx.x;
    static_assert(bmaxcl(BCAP) <= BT, "one thread per bundle cluster");
    const int add = (tid < B.ncl) ? B.c_addn[tid] : 0;
    const int nn = (tid < B.ncl) ? B.c_n[tid] + add : 0;
    int tot;
    const int noff = bscan<BT>(nn, B.ws, tot);
    constexpr int PER = BCAP / BT;
    int mv_new[PER], mv_g[PER], mv_k[PER], mv_own[PER];
    int my_old_n = 0, my_addg = 0;
    if (tid < B.ncl) {
        my_old_n = B.c_n[tid];
        my_addg = B.c_addg[tid];
    }
    __syncthreads();
    if (tot > BCAP) {  // no room: the fragments cannot be integrated here
        if (tid == 0) atomicOr(A.status, ST_CLUSTER_TOO_BIG);
        return;
    }
    if (tid < B.ncl) B.c_key[tid] = (unsigned long long)(unsigned)noff;  // new offsets, by cluster
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int p = tid + j * BT;
        mv_new[j] = -1;
        if (p < B.used) {
            const int k = B.cl[p];
            const int no = (int)B.c_key[k];
            mv_new[j] = no + (p - B.c_off[k]);
            mv_g[j] = B.gslot[p];
            mv_k[j] = k;
            mv_own[j] = (B.owner[p] >= 0) ? no + (B.owner[p] - B.c_off[k]) : -1;
        }
    }
    __syncthreads();
    if (tid < B.ncl) {
        B.c_off[tid] = noff;
        B.c_n[tid] = nn;
        // fragments are smaller than the members the prefilter margins were
        // set for: exact FP64 tests for this cluster from here on
        if (add > 0) B.c_flags[tid] |= CF_EXACT;
    }
    if (tid == 0) B.used = tot;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
        if (mv_new[j] < 0) continue;
        mirror_all(B, H, mv_new[j], mv_g[j], mv_k[j], true);
        B.owner[mv_new[j]] = (short)mv_own[j];
    }
    if (tid < B.ncl)
        for (int i = 0; i < add; i++) {
            const int q = noff + my_old_n + i;
            mirror_all(B, H, q, my_addg + i, tid, true);
            B.owner[q] = -1;
        }
    __syncthreads();
}

// one block step of every cluster in the bundle (timeIntegrate_multi body,
// src/hermite.h:224-479)
template <int BCAP>
__device__ void bundle_step(const HardArgs &A, BundleSmem<BCAP> &B) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const Params &P = A.P;
    const Hard &H = A.H;
    // makeActiveList: ts = min over alive members of th + dt
    FOR_CLUSTERS(k) {
        B.c_steps[k]++;
        B.c_key[k] = dbits(1.e10);
    }
    __syncthreads();
    FOR_SLOTS(p) {
        if (B.dead[p]) continue;
        const int g = B.gslot[p];
        atomicMin(&B.c_key[B.cl[p]], dbits(H.th[g] + H.dt[g]));
    }
    __syncthreads();
    FOR_CLUSTERS(k) {
        B.c_ts[k] = bitsd(B.c_key[k]);
        B.c_key[k] = dbits(1.);
        B.c_pb[k] = 0x7fffffffffffffffLL;
    }
    if (threadIdx.x == 0) B.n_sv = 0;
    __syncthreads();
    HP_MARK(HP_TS);
    // predict every member
    FOR_SLOTS(p) {
        const int g = B.gslot[p], k = B.cl[p];
        V3 xp, vp;
        predict(H, g, B.c_ts[k] - H.th[g], xp, vp);
        st3(B.xp, p, xp);
        st3(B.vp, p, vp);
        st32b(B, B.xp32, p, xp, k);
    }
    __syncthreads();
    HP_MARK(HP_PREDICT);
    // collisionDetermination, src/hermite.h:98-196
    bundle_detect(A, B, false);
    __syncthreads();
    if (B.n_sv <= BSURV) {
        for (int i = threadIdx.x; i < B.n_sv; i += BT)
            if (dbits(B.sv_R[i]) == B.c_key[B.sv_k[i]]) atomicMin(&B.c_pb[B.sv_k[i]], B.sv_p[i]);
    } else {
        bundle_detect(A, B, true);
    }
    __syncthreads();
    FOR_CLUSTERS(k) {
        int fl = B.c_flags[k] & ~CF_COL;
        if (B.c_key[k] < dbits(1.)) {
            fl |= CF_COL;
            const int o = B.c_off[k], n = B.c_n[k];
            const int a = (int)(B.c_pb[k] / n), b = (int)(B.c_pb[k] % n);
            if (B.mass[o + a] < B.mass[o + b]) { B.c_imp[k] = o + a; B.c_tar[k] = o + b; }
            else { B.c_imp[k] = o + b; B.c_tar[k] = o + a; }
        }
        B.c_flags[k] = fl;
    }
    __syncthreads();
    HP_MARK(HP_DETECT);
    // the active set (every alive member on a collision) and the twins of
    // active merged members
    FOR_SLOTS(p) {
        const int k = B.cl[p], g = B.gslot[p];
        const bool col = (B.c_flags[k] & CF_COL) != 0;
        if (col) H.dt[g] = B.c_ts[k] - H.th[g];
        unsigned char f = 0;
        if (!B.dead[p] && (col || H.th[g] + H.dt[g] == B.c_ts[k])) {
            f = MF_ACT | MF_TGT;
            atomicAdd((unsigned long long *)&B.c_work[k], (unsigned long long)B.c_n[k]);
        }
        B.flag[p] = f;
    }
    __syncthreads();
    FOR_SLOTS(p) {
        const int ow = B.owner[p];
        if (B.dead[p] && ow >= 0 && (B.flag[ow] & MF_ACT)) B.flag[p] |= MF_TGT;
    }
    __syncthreads();
    const int nt = bundle_list(B, MF_TGT);
    HP_MARK(HP_ACTIVE);
    bundle_pairs(A, B, 1, nt);
    HP_MARK(HP_PAIRS);
    bundle_finalize(A, B, 1, nt, 1);
    HP_MARK(HP_FINAL);
    for (int it = 0; it < 2; it++) {
        // FPHard::correct, one thread per (target, component): correct()'s
        // arithmetic component by component
        for (int i = threadIdx.x; i < 3 * nt; i += BT) {
            const int t = i / 3, d = i - 3 * t;
            const int s = B.tgt[t], g = B.gslot[s], k = B.cl[s];
            const int gd = 3 * g + d;
            // every input first (one round trip to the state of record)
            const double th = H.th[g], as = H.acc_s[gd], a0s = H.a0_s[gd], j0s = H.j0_s[gd], js = H.jerk_s[gd];
            const double ad = H.acc_d[gd], a0d = H.a0_d[gd], j0d = H.j0_d[gd], jd = H.jerk_d[gd];
            const double xp = H.xp[gd], vp = H.vp[gd];
            const double Dt = B.c_ts[k] - th;
            const double Dt2 = Dt * Dt, Di = recip_pow2_or_div(Dt), Di2 = Di * Di, Di3 = Di2 * Di;
            const double Am_s = as - a0s, J0_s = Dt * j0s, J1_s = Dt * js;
            const double A2_s = 3. * Am_s - (J1_s + 2. * J0_s);
            const double A3_s = -2. * Am_s + (J1_s + J0_s);
            H.a2_s[gd] = 2. * Di2 * (A2_s + 3. * A3_s);
            H.a3_s[gd] = 6. * Di3 * A3_s;
            const double Am_d = ad - a0d, J0_d = j0d * Dt, J1_d = jd * Dt;
            const double A2_d = 3. * Am_d - (J1_d + 2. * J0_d);
            const double A3_d = -2. * Am_d + (J1_d + J0_d);
            H.a2_d[gd] = 2. * (A2_d + 3. * A3_d) * Di2;
            H.a3_d[gd] = 6. * A3_d * Di3;
            const double A2 = A2_s + A2_d, A3 = A3_s + A3_d;
            const double x = xp + 1.6666666666666667e-2 * Dt2 * (5. * A2 + 3. * 1.1666666666666667e-3 * A3);
            const double v = vp + 8.3333333333333333e-2 * Dt * (4. * A2 + 3. * A3);
            H.pos[gd] = x;
            H.vel[gd] = v;
            B.pos[3 * s + d] = x;
            B.vel[3 * s + d] = v;
            const float u = (float)(x - B.c_ref[3 * k + d]);
            B.pos32[3 * s + d] = u;
            if (!(fabsf(u) < B.c_E32[k])) atomicOr(&B.c_flags[k], CF_EXACT);
        }
        __syncthreads();
        HP_MARK(HP_CORRECT);
        bundle_pairs(A, B, 2, nt);
        HP_MARK(HP_PAIRS);
        bundle_finalize(A, B, 2, nt, 1);
        HP_MARK(HP_FINAL);
    }
    // time and calcDeltat: the two criteria of a target (planets, sun) in a
    // pair of lanes, exchanged by a shuffle; the even lane goes on with the
    // target's time and dt_hermite's step choice
    for (int base = 0; base < 2 * nt; base += BT) {
        const int i = base + threadIdx.x, t = i >> 1;
        const bool act = i < 2 * nt;
        int s = 0, g = 0, k = 0;
        bool upd = false;
        double crit = 0.;
        if (act) {
            s = B.tgt[t];
            g = B.gslot[s];
            k = B.cl[s];
            upd = !(B.c_flags[k] & CF_COL) && !B.dead[s];
            if (upd) {
                // one code path for both lanes (the inputs chosen by parity)
                const bool sun = (i & 1) != 0;
                crit = dt4th(sun ? P.eta_sun : P.eta, P.alpha2, sun ? 0. : H.acc0[g], ld3(sun ? H.acc_s : H.acc_d, g),
                             ld3(sun ? H.jerk_s : H.jerk_d, g), ld3(sun ? H.a2_s : H.a2_d, g),
                             ld3(sun ? H.a3_s : H.a3_d, g));
            }
        }
        const double other = __shfl_xor_sync(0xffffffffu, crit, 1);
        if (act && !(i & 1)) {
            H.th[g] += B.c_ts[k] - H.th[g];
            if (upd) H.dt[g] = dt_next_hermite(P, H.th[g], H.dt[g], dmin(crit, other));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nt; i += BT) {
        const int s = B.tgt[i], k = B.cl[s];
        if (B.dead[s] && B.owner[s] >= 0 && !(B.c_flags[k] & CF_COL)) H.dt[B.gslot[s]] = H.dt[B.gslot[B.owner[s]]];
    }
    if (threadIdx.x == 0) B.any = 0;
    __syncthreads();
    HP_MARK(HP_DT);
    // collisions: one thread per colliding cluster
    if (threadIdx.x == 0) B.grew = 0;
    __syncthreads();
    FOR_CLUSTERS(k) {
        B.c_addn[k] = 0;
        if (!(B.c_flags[k] & CF_COL)) continue;
        B.any = 1;
        ColRec rec;
        double e1 = 0., e2 = 0.;
        const int o = B.c_off[k], n = B.c_n[k];
        int fs[32];
        FragCtx X{&A, &B.gslot[o], n, B.c_idx[k], B.c_label[k], &B.c_fragn[k], fs};
        const int nf = collide(P, H, B.gslot[B.c_imp[k]], B.gslot[B.c_tar[k]], e1, e2, rec, &X);
        B.c_ed[k] += e1;
        B.c_edd[k] += e2;
        rec.cluster = B.c_idx[k];
        rec.seq = B.c_ncol[k]++;
        rec.n = B.c_n0[k];
        const int slot = atomicAdd(A.n_cols, 1);
        if (slot < A.col_cap) A.cols[slot] = rec;
        else atomicOr(A.status, ST_QUEUE_OVERFLOW);
        if (nf > 0) {
            B.c_addn[k] = nf;
            B.c_addg[k] = fs[0];  // a collision's fragments have consecutive slots
            B.grew = 1;
            for (int i = 0; i < nf; i++) A.frags[fs[i] - A.frag_base].n0 = B.c_n0[k];
        }
        // twin owners (pool slots) from the merge lists
        for (int j = 0; j < n; j++) B.owner[o + j] = -1;
        for (int j = 0; j < n; j++) {
            const int gj = B.gslot[o + j];
            if (!H.merged[gj]) continue;
            for (int t = H.tw_head[gj], gg = 0; t >= 0 && gg < 4096; t = H.tw_next[t], gg++)
                for (int q = 0; q < n; q++)
                    if (B.gslot[o + q] == t) {
                        B.owner[o + q] = (short)(o + j);
                        break;
                    }
        }
    }
    __syncthreads();
    if (B.grew) bundle_grow(A, B);
    __syncthreads();
    if (B.any) {
        FOR_SLOTS(p) {
            const int k = B.cl[p];
            B.flag[p] = 0;
            if (!(B.c_flags[k] & CF_COL)) continue;
            mirror_all(B, H, p, B.gslot[p], k, true);
            B.flag[p] = MF_TGT;
        }
        __syncthreads();
        const int nc = bundle_list(B, MF_TGT);
        bundle_pairs(A, B, 0, nc);
        bundle_finalize(A, B, 0, nc, 2);
        for (int i = threadIdx.x; i < nc; i += BT) {
            const int s = B.tgt[i], g = B.gslot[s];
            if (!B.dead[s])
                H.dt[g] = dt_initial(P, H.th[g], H.dt[g], H.acc0[g], ld3(H.acc_d, g), ld3(H.jerk_d, g),
                                     ld3(H.acc_s, g), ld3(H.jerk_s, g));
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nc; i += BT) {
            const int s = B.tgt[i], g = B.gslot[s];
            if (B.merged[s])
                for (int t = H.tw_head[g], gg = 0; t >= 0 && gg < 4096; t = H.tw_next[t], gg++) H.dt[t] = H.dt[g];
        }
        __syncthreads();
    }
    HP_MARK(HP_COLLIDE);
    // getSystemTime, src/hermite.h:25-35
    FOR_CLUSTERS(k) B.c_key[k] = dbits(1.e10);
    __syncthreads();
    FOR_SLOTS(p) {
        if (!B.dead[p]) atomicMin(&B.c_key[B.cl[p]], dbits(H.th[B.gslot[p]]));
    }
    if (threadIdx.x == 0) B.any = 0;
    __syncthreads();
    FOR_CLUSTERS(k) {
        const double time = bitsd(B.c_key[k]);
        if (time < A.t_end && B.c_steps[k] >= A.max_steps) atomicOr(A.status, ST_ITER_CAP);
        if (!(time < A.t_end) || B.c_steps[k] >= A.max_steps) {
            B.c_flags[k] |= CF_FIN;
            B.any = 1;
        }
    }
    __syncthreads();
    HP_MARK(HP_TIME);
}

// final forces, write-back and removal of the finished clusters
template <int BCAP>
__device__ void bundle_retire(const HardArgs &A, BundleSmem<BCAP> &B) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    const Hard &H = A.H;
    const int tid = threadIdx.x;
    FOR_SLOTS(p) B.flag[p] = (B.c_flags[B.cl[p]] & CF_FIN) ? MF_TGT : 0;
    __syncthreads();
    const int nt = bundle_list(B, MF_TGT);
    bundle_pairs(A, B, 0, nt);
    bundle_finalize(A, B, 0, nt, 2);
    // write back to FPGrav, with resetTime (src/hard.h:768-787)
    for (int i = tid; i < nt; i += BT) {
        const int s = B.tgt[i], g = B.gslot[s], k = B.cl[s];
        if (g >= A.frag_base) {  // a fragment: joins the system after the launch
            A.frags[g - A.frag_base].n_cl = B.c_n[k];
            continue;
        }
        const int idx = A.members[g];
        st3(A.S.pos, idx, ld3(H.pos, g)); st3(A.S.vel, idx, ld3(H.vel, g));
        st3(A.S.acc_s, idx, ld3(H.acc_s, g)); st3(A.S.jerk_s, idx, ld3(H.jerk_s, g));
        st3(A.S.acc_d, idx, ld3(H.acc_d, g)); st3(A.S.jerk_d, idx, ld3(H.jerk_d, g));
        A.S.phi_d[idx] = H.phi_d[g]; A.S.phi_s[idx] = H.phi_s[g];
        A.S.mass[idx] = H.mass[g]; A.S.r_planet[idx] = H.r_planet[g];
        A.S.time[idx] = H.time_c[g] + H.th[g]; A.S.dt[idx] = H.dt[g];
        A.S.id[idx] = H.id[g];
        A.S.dead[idx] = H.dead[g]; A.S.merged[idx] = H.merged[g];
        A.S.n_cluster[idx] = B.c_n[k];
    }
    FOR_CLUSTERS(k) {
        if (!(B.c_flags[k] & CF_FIN)) continue;
        const int c = B.c_idx[k];
        A.cl_edisp[2 * c] = (B.c_ncol[k] > 0) ? B.c_ed[k] : 0.;
        A.cl_edisp[2 * c + 1] = (B.c_ncol[k] > 0) ? B.c_edd[k] : 0.;
        if (A.cost) {
            A.cost[2 * c] = B.c_steps[k];
            A.cost[2 * c + 1] = B.c_work[k];
        }
        if (A.times) {
            A.times[2 * c] = B.c_t0[k];
            A.times[2 * c + 1] = global_ns();
        }
    }
    __syncthreads();
    // compaction: kept clusters move down, in order
    int keep = 0, nk = 0, nkeep = 0, noff = 0, tot = 0;
    int t_idx = 0, t_n = 0, t_goff = 0, t_steps = 0, t_ncol = 0, t_flags = 0;
    double t_ref0 = 0., t_ref1 = 0., t_ref2 = 0., t_ed = 0., t_edd = 0.;
    long long t_work = 0, t_t0 = 0;
    float t_thrf = 0.f, t_thrc = 0.f, t_E = 0.f;
    long long t_label = 0, t_fragn = 0;
    int t_n0 = 0;
    if (tid < B.ncl) {
        keep = !(B.c_flags[tid] & CF_FIN);
        t_idx = B.c_idx[tid]; t_n = B.c_n[tid]; t_goff = B.c_goff[tid];
        t_steps = B.c_steps[tid]; t_ncol = B.c_ncol[tid]; t_flags = B.c_flags[tid];
        t_ref0 = B.c_ref[3 * tid]; t_ref1 = B.c_ref[3 * tid + 1]; t_ref2 = B.c_ref[3 * tid + 2];
        t_ed = B.c_ed[tid]; t_edd = B.c_edd[tid]; t_work = B.c_work[tid]; t_t0 = B.c_t0[tid];
        t_thrf = B.c_thrf[tid]; t_thrc = B.c_thrc[tid]; t_E = B.c_E32[tid];
        t_label = B.c_label[tid]; t_fragn = B.c_fragn[tid]; t_n0 = B.c_n0[tid];
    }
    static_assert(bmaxcl(BCAP) <= BT, "one thread per bundle cluster");
    nk = bscan<BT>(keep, B.ws, nkeep);
    noff = bscan<BT>(keep ? t_n : 0, B.ws, tot);
    // slots: read the old placement before anything moves
    constexpr int PER = BCAP / BT;
    int mv_new[PER], mv_g[PER], mv_k[PER], mv_own[PER];
    __syncthreads();
    if (keep) {
        // old -> new offset per kept cluster, through c_key (free here)
        B.c_key[tid] = (unsigned long long)(unsigned)noff | ((unsigned long long)(unsigned)nk << 32);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int p = tid + j * BT;
        mv_new[j] = -1;
        if (p < B.used) {
            const int k = B.cl[p];
            if (!(B.c_flags[k] & CF_FIN)) {
                const int no = (int)(B.c_key[k] & 0xffffffffULL), kk = (int)(B.c_key[k] >> 32);
                mv_new[j] = no + (p - B.c_off[k]);
                mv_g[j] = B.gslot[p];
                mv_k[j] = kk;
                mv_own[j] = (B.owner[p] >= 0) ? no + (B.owner[p] - B.c_off[k]) : -1;
            }
        }
    }
    __syncthreads();
    if (keep) {
        B.c_idx[nk] = t_idx; B.c_off[nk] = noff; B.c_n[nk] = t_n; B.c_goff[nk] = t_goff;
        B.c_steps[nk] = t_steps; B.c_ncol[nk] = t_ncol; B.c_flags[nk] = t_flags;
        B.c_ref[3 * nk] = t_ref0; B.c_ref[3 * nk + 1] = t_ref1; B.c_ref[3 * nk + 2] = t_ref2;
        B.c_ed[nk] = t_ed; B.c_edd[nk] = t_edd; B.c_work[nk] = t_work; B.c_t0[nk] = t_t0;
        B.c_thrf[nk] = t_thrf; B.c_thrc[nk] = t_thrc; B.c_E32[nk] = t_E;
        B.c_label[nk] = t_label; B.c_fragn[nk] = t_fragn; B.c_n0[nk] = t_n0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PER; j++) {
        const int p = tid + j * BT;
        if (mv_new[j] >= 0 && mv_new[j] != p) {
            mirror_all(B, H, mv_new[j], mv_g[j], mv_k[j], true);
            B.owner[mv_new[j]] = (short)mv_own[j];
        } else if (mv_new[j] >= 0) {
            B.cl[p] = (short)mv_k[j];
            B.owner[p] = (short)mv_own[j];
        }
    }
    if (tid == 0) {
        B.ncl = nkeep;
        B.used = tot;
    }
    __syncthreads();
}

// The clusters above BCAP_MAIN bodies (the queue's tier 0), concurrently
// with k_hard_bundles: one CTA takes one at a time -- up to BCAP_WIDE bodies
// (fragment room included) as a lone wide bundle, the lane-dense form, larger
// ones in the one-cluster-per-CTA form.  Same arithmetic, bit for bit, as
// every other form.
constexpr int WT = bundle_threads(BCAP_WIDE);  // threads of a wide CTA (it holds its SM)
__global__ void __launch_bounds__(WT, 1) k_hard_wide(HardArgs A) {
    extern __shared__ __align__(16) unsigned char bundle_smem[];
    BundleSmem<BCAP_WIDE> &B = *reinterpret_cast<BundleSmem<BCAP_WIDE> *>(bundle_smem);
    __shared__ double red_d[WT / 32];
    __shared__ long long red_l[WT / 32];
    __shared__ int q_sh;
    const int tid = threadIdx.x;
    Team<WT> tm{tid, red_d, red_l};
    const int room = (A.frag.a_frag > 0.) ? 2 * A.frag.n_frag_max : 0;
    for (int guard = 0; guard < (1 << 30); guard++) {
        if (tid == 0) q_sh = atomicAdd(&A.queue[0], 1);
        __syncthreads();
        const int q = q_sh;
        __syncthreads();
        if (q >= A.n_tier[0]) break;
        const int c = A.order[q];
        const int n = A.cnt[c];
        if (n + room > BCAP_WIDE) {
            run_cluster<WT>(A, c, tm);
            continue;
        }
        if (tid == 0) {
            B.ncl = 1;
            B.c_idx[0] = c;
            B.c_off[0] = 0;
            B.c_n[0] = n;
            B.c_flags[0] = CF_FRESH;
            B.used = n;
            B.fresh_k = 0;
            B.fresh_p = 0;
            B.n_pend = B.i_pend = 0;
            B.exhausted = 1;
            B.phase = 1;
        }
        __syncthreads();
        bundle_load(A, B);
        {
            const int nt = bundle_list(B, MF_TGT);
            bundle_pairs(A, B, 0, nt);
            bundle_finalize(A, B, 0, nt, 2);
        }
        // bundle_step advances the cluster by one block step; it retires when done
        for (int it = 0; it < A.max_steps + 8; it++) {
            bundle_step(A, B);
            if (B.any) bundle_retire(A, B);
            if (B.ncl == 0) break;
        }
        __syncthreads();
    }
}

// one CTA: (without k_hard_wide) the clusters above BCAP one at a time, then
// bundles of BCAP member slots until the queue is empty; OCC CTAs per SM
template <int BCAP, int OCC>
__global__ void __launch_bounds__(bundle_threads(BCAP), OCC) k_hard_bundles(HardArgs A) {
    constexpr int BT = BundleSmem<BCAP>::NT;
    extern __shared__ __align__(16) unsigned char bundle_smem[];
    BundleSmem<BCAP> &B = *reinterpret_cast<BundleSmem<BCAP> *>(bundle_smem);
    __shared__ double red_d[BT / 32];
    __shared__ long long red_l[BT / 32];
    __shared__ int q_sh;
    const int tid = threadIdx.x;
    const long long t_k0 = A.phase_cycles ? clock64() : 0;
    const Team<BT> tm{tid, red_d, red_l};
    if (!A.wide) {
        for (int guard = 0; guard < (1 << 30); guard++) {
            if (tid == 0) q_sh = atomicAdd(&A.queue[0], 1);
            __syncthreads();
            const int q = q_sh;
            __syncthreads();
            if (q >= A.n_tier[0]) break;
            run_cluster<BT>(A, A.order[q], tm);
        }
    }
    // the lone tier: each cluster integrated alone by the whole CTA, the
    // bundle's shared memory holding its state (the predicted longest chains
    // start first, beside bundles on the other CTA slots of the SM)
    if (A.lone_in) {
        LoneSmem<BT> &L = *reinterpret_cast<LoneSmem<BT> *>(bundle_smem);
        for (int guard = 0; guard < (1 << 30); guard++) {
            if (tid == 0) q_sh = atomicAdd(&A.queue[3], 1);
            __syncthreads();
            const int q = q_sh;
            __syncthreads();
            if (q >= A.n_tier[2]) break;
            const int c = A.order[A.n_tier[0] + A.n_tier[1] + q];
            if (A.cnt[c] > LCAP) {  // the lone tier holds at most LCAP members
                if (tid == 0) atomicOr(A.status, ST_CLUSTER_TOO_BIG);
                continue;
            }
            lone_cluster<BT>(A, c, L, tm, red_d);
        }
    }
    if (tid == 0) {
        B.used = 0;
        B.ncl = 0;
        B.n_pend = 0;
        B.i_pend = 0;
        B.exhausted = 0;
        B.phase = 0;
        for (int k = 0; k < HP_N; k++) B.ph_acc[k] = 0;
        B.ph_t = clock64();
        B.ph_acc[HP_LONE] = B.ph_t - t_k0;  // the clusters above the slots, the lone tier
    }
    __syncthreads();
    for (int guard = 0; guard < (1 << 30); guard++) {
        if (tid == 0) {
            B.fresh_k = B.ncl;
            B.fresh_p = B.used;
        }
        __syncthreads();
        bundle_refill(A, B);
        if (B.ncl == 0) break;
        if (B.fresh_k < B.ncl) {
            bundle_load(A, B);
            const int nt = bundle_list(B, MF_TGT);
            bundle_pairs(A, B, 0, nt);
            bundle_finalize(A, B, 0, nt, 2);
        }
        HP_MARK(HP_ADMIT);
        bundle_step(A, B);
        if (B.any) bundle_retire(A, B);
        HP_MARK(HP_RETIRE);
    }
    if (A.phase_cycles && tid == 0)
        for (int k = 0; k < HP_N; k++) atomicAdd(&A.phase_cycles[k], (unsigned long long)B.ph_acc[k]);
}

#undef FOR_SLOTS
#undef FOR_CLUSTERS

}  // namespace p3t
