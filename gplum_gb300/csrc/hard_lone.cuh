// Lone-cluster form of the hard part: the clusters of at most LCAP members
// that the learned cost model predicts to take the longest chains of block
// steps, each integrated alone by one CTA whose shared memory holds the whole
// cluster -- either a 256-thread CTA of the bundle kernel (first, before it
// packs bundles), or a 128-thread CTA of k_hard_lone holding a whole SM.
//
// Such a cluster's time is its chain of block steps, and a block step is a
// chain of FP64 operations: a warp's FP64 instruction occupies its issue slot
// for 64 cycles whatever its active lanes (so instruction-level parallelism
// inside one thread buys nothing), and the SM's FP64 unit takes one warp
// instruction per ~19 cycles from all warps together.  So the chain shortens
// only when independent parts of it sit in different lanes or warps:
//   - predictor and corrector: one thread per (member, component);
//   - pair terms: one thread per (target, partner) pair (terms are then added
//     to each target in partner order, the order of src/gravity_hard.h:203-367);
//   - the sun force of the targets in the last warp, beside the pair terms;
//   - the two time-step criteria (planets, sun; src/particle.h:1276-1314) of a
//     member in two threads.
// Every value is computed by the same operations in the same order as the
// team form (run_cluster) and the bundle form, so results are bit-identical;
// the state lives in shared memory (no global round trips) and each phase is
// one CTA barrier.  k_hard_lone's shared memory request is large enough that
// no bundle CTA shares its SM, so its warps have the FP64 unit to themselves.
//
// Collisions are rare: a block step that detects one goes, as of its start,
// to the global state of record, the team form's loop (cluster_loop,
// one_step) integrates that block step, and the lone form reloads the result
// -- dead members, merged targets and their twins included -- and goes on.
#pragma once

namespace p3t {

constexpr int LONE_T = 128;  // threads of a k_hard_lone CTA
constexpr int LCAP = 64;     // members of a lone cluster at most
constexpr int LRING = 256;   // live pair items per drain
// k_hard_lone's shared memory request: large enough that no bundle CTA fits
// beside it on its SM, so its warps have the FP64 unit to themselves
constexpr int LONE_EXCL_SMEM = 132 * 1024;

// the state of one lone cluster, for a CTA of NT threads (the last warp
// computes the sun force beside the pair terms)
template <int NT>
struct LoneSmem {
    // member state: component d of member m at [d][m]
    double pos[3][LCAP], vel[3][LCAP], acc_s[3][LCAP], jerk_s[3][LCAP], acc_d[3][LCAP], jerk_d[3][LCAP];
    double a0_s[3][LCAP], j0_s[3][LCAP], a0_d[3][LCAP], j0_d[3][LCAP], xp[3][LCAP], vp[3][LCAP];
    double a2_s[3][LCAP], a3_s[3][LCAP], a2_d[3][LCAP], a3_d[3][LCAP];
    double mass[LCAP], roi[LCAP], fr[LCAP], th[LCAP], dt[LCAP], acc0[LCAP], phi_d[LCAP], phi_s[LCAP];
    double rp[LCAP], fa[LCAP];  // r_planet and f (fr = f r_planet)
    double dtq[2][LCAP];  // the planets' and the sun's dt4th of each active member
    double term[7][LRING];
    float pos32[3][LCAP], xp32[3][LCAP], roi32[LCAP], fr32[LCAP];
    long long id[LCAP];
    int tgt[LCAP];        // targets of the running pass: the active members ascending, then their twins
    // after a collision: dead members, merged targets and their twins (the
    // team form's tw_* links as member indices, -1 for none)
    int dead[LCAP], merged[LCAP], tw_head[LCAP], tw_tail[LCAP], tw_next[LCAP];
    int ring[LRING + NT];
    int seg[LRING + 1];
    int ws[NT / 32];
    double ts;
    int n_tgt, n_act;  // targets, of which the first n_act are active members
    int any_merged;
};

// exclusive block-wide prefix of v over the NT threads; all threads call
template <int NT>
__device__ __forceinline__ int lscan(int v, int *ws, int &total) {
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

__device__ __forceinline__ V3 lv(const double (*a)[LCAP], int m) { return v3(a[0][m], a[1][m], a[2][m]); }
__device__ __forceinline__ void lst(double (*a)[LCAP], int m, V3 v) {
    a[0][m] = v.x;
    a[1][m] = v.y;
    a[2][m] = v.z;
}
__device__ __forceinline__ void lst32(float (*a)[LCAP], int m, V3 x, const Pre &pre) {
    a[0][m] = (float)(x.x - pre.ref[0]);
    a[1][m] = (float)(x.y - pre.ref[1]);
    a[2][m] = (float)(x.z - pre.ref[2]);
}
__device__ __forceinline__ float ld2_32(const float (*a)[LCAP], int s, const float (*b)[LCAP], int t) {
    const float dx = a[0][s] - b[0][t], dy = a[1][s] - b[1][t], dz = a[2][s] - b[2][t];
    return dx * dx + dy * dy + dz * dz;
}

// the terms of target s from partner t (hard_force's arithmetic for one pair)
template <int NT>
__device__ __forceinline__ void lone_terms(const Params &P, const LoneSmem<NT> &L, int mode, int s, int t, double *o) {
    const V3 xi = (mode == 1) ? lv(L.xp, s) : lv(L.pos, s);
    const V3 vi = (mode == 1) ? lv(L.vp, s) : lv(L.vel, s);
    const V3 dr = ((mode == 0) ? lv(L.pos, t) : lv(L.xp, t)) - xi;
    double dr2 = dot(dr, dr);
    dr2 += P.eps2;
    const double r_out_inv = dmin(L.roi[s], L.roi[t]);
    const V3 dv = ((mode == 0) ? lv(L.vel, t) : lv(L.vp, t)) - vi;
    const double rij = sqrt(dr2);
    const double rinv = 1. / rij;
    const double r2inv = rinv * rinv;
    const double r3inv = r2inv * rinv;
    const double mj = L.mass[t];
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
    o[6] = mj * rinv * Wc;
}

// the sun force of every target (src/gravity_hard.h:5-111), by the sun warp
template <int NT>
__device__ void lone_sun(const Params &P, LoneSmem<NT> &L, int mode) {
    for (int t = threadIdx.x & 31; t < L.n_tgt; t += 32) {
        const int s = L.tgt[t];
        const V3 xi = (mode == 1) ? lv(L.xp, s) : lv(L.pos, s);
        const V3 vi = (mode == 1) ? lv(L.vp, s) : lv(L.vel, s);
        V3 as, js;
        double phs;
        sun_force(P, xi, vi, as, js, mode == 0 ? &phs : nullptr);
        if (mode == 0) L.phi_s[s] = phs;
        lst(L.acc_s, s, as);
        lst(L.jerk_s, s, js);
    }
}

// terms of ring[0..m) by the threads outside the sun warp (which computes the
// targets' sun force meanwhile when `sun` is set), then in-order addition into
// the targets' sums
template <int NT>
__device__ void lone_drain(const Params &P, LoneSmem<NT> &L, int mode, int m, bool sun) {
    constexpr int NW = NT - 32;  // term threads
    const int tid = threadIdx.x;
    if (tid < NW) {
        for (int q = tid; q < m; q += NW) {
            const int e = L.ring[q];
            double o[7];
            lone_terms(P, L, mode, L.tgt[e >> 16], e & 0xffff, o);
#pragma unroll
            for (int c = 0; c < 7; c++) L.term[c][q] = o[c];
        }
    } else if (sun) {
        lone_sun(P, L, mode);
    }
    // segments of equal target (the ring is in (target, partner) order)
    int nseg = 0;
    {
        int head[2] = {0, 0};
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const int q = 2 * tid + r;  // consecutive items per thread: heads come out in ring order
            head[r] = (q < m) && (q == 0 || (L.ring[q - 1] >> 16) != (L.ring[q] >> 16));
        }
        const int off = lscan<NT>(head[0] + head[1], L.ws, nseg);
        if (head[0]) L.seg[off] = 2 * tid;
        if (head[1]) L.seg[off + head[0]] = 2 * tid + 1;
        if (tid == 0) L.seg[nseg] = m;
    }
    __syncthreads();
    const int ncomp = (mode == 0) ? 7 : 6;
    for (int it = tid; it < ncomp * nseg; it += NT) {
        const int j = it / ncomp, c = it - ncomp * j;
        const int a = L.seg[j], b = L.seg[j + 1];
        const int s = L.tgt[L.ring[a] >> 16];
        double acc = (c < 3) ? L.acc_d[c][s] : (c < 6 ? L.jerk_d[c - 3][s] : L.phi_d[s]);
        if (c < 6)
            for (int k = a; k < b; k++) acc += L.term[c][k];
        else
            for (int k = a; k < b; k++) acc -= L.term[c][k];
        if (c < 3) L.acc_d[c][s] = acc;
        else if (c < 6) L.jerk_d[c - 3][s] = acc;
        else L.phi_d[s] = acc;
    }
    __syncthreads();
}

// one force pass over the targets L.tgt[0..L.n_tgt): mode 0 full (pos/vel,
// with phi), 1 predicted i and j, 2 corrected i and predicted j
template <int NT>
__device__ void lone_pass(const HardArgs &A, LoneSmem<NT> &L, int n, int mode, const Pre &pre) {
    const Params &P = A.P;
    const int tid = threadIdx.x, nt = L.n_tgt;
    for (int it = tid; it < 7 * nt; it += NT) {
        const int t = it / 7, c = it - 7 * t, s = L.tgt[t];
        if (c < 3) L.acc_d[c][s] = 0.;
        else if (c < 6) L.jerk_d[c - 3][s] = 0.;
        else if (mode == 0) L.phi_d[s] = 0.;
    }
    __syncthreads();
    bool sun = true;  // the sun force still to do (with the first drain)
    const float(*xi32)[LCAP] = (mode == 1) ? L.xp32 : L.pos32;
    const float(*xj32)[LCAP] = (mode == 0) ? L.pos32 : L.xp32;
    const double(*XJ)[LCAP] = (mode == 0) ? L.pos : L.xp;
    const int total = nt * n;
    int ring_n = 0;
    for (int base = 0; base < total; base += NT) {
        const int f = base + tid;
        int live = 0, e = 0;
        if (f < total) {
            const int ti = f / n, t = f - ti * n, s = L.tgt[ti];
            // hard_force's tests: same body, FP32 prefilter, exact cutoff
            if (L.id[s] != L.id[t]) {
                bool keep = true;
                if (pre.on) {
                    const float rf = fminf(L.roi32[s], L.roi32[t]);
                    keep = !(ld2_32(xi32, s, xj32, t) * (rf * rf) > 4.0f);
                }
                if (keep) {
                    const V3 xi = (mode == 1) ? lv(L.xp, s) : lv(L.pos, s);
                    const V3 dr = lv(XJ, t) - xi;
                    double dr2 = dot(dr, dr);
                    dr2 += P.eps2;
                    const double r_out_inv = dmin(L.roi[s], L.roi[t]);
                    live = !(dr2 * r_out_inv * r_out_inv > 1.000001);
                }
            }
            e = (ti << 16) | t;
        }
        int cnt;
        const int off = lscan<NT>(live, L.ws, cnt);
        if (live) L.ring[ring_n + off] = e;
        ring_n += cnt;
        __syncthreads();
        if (ring_n >= LRING) {
            lone_drain(P, L, mode, LRING, sun);
            sun = false;
            const int rest = ring_n - LRING;
            if (tid < rest) L.ring[tid] = L.ring[LRING + tid];
            ring_n = rest;
            __syncthreads();
        }
    }
    if (ring_n > 0) {
        lone_drain(P, L, mode, ring_n, sun);
    } else if (sun) {
        if ((tid >> 5) == NT / 32 - 1) lone_sun(P, L, mode);
        __syncthreads();
    }
}

// FPHard::correct (src/particle.h:1208-1274) of the targets, one thread per
// (target, component); then the FP32 copy of the corrected position
template <int NT>
__device__ void lone_correct(LoneSmem<NT> &L, const Pre &pre) {
    const int nt = L.n_tgt;
    for (int it = threadIdx.x; it < 3 * nt; it += NT) {
        const int t = it / 3, d = it - 3 * t, s = L.tgt[t];
        const double Dt = L.ts - L.th[s];
        const double Dt2 = Dt * Dt, Di = recip_pow2_or_div(Dt), Di2 = Di * Di, Di3 = Di2 * Di;
        const double Am_s = L.acc_s[d][s] - L.a0_s[d][s], J0_s = Dt * L.j0_s[d][s], J1_s = Dt * L.jerk_s[d][s];
        const double A2_s = 3. * Am_s - (J1_s + 2. * J0_s);
        const double A3_s = -2. * Am_s + (J1_s + J0_s);
        L.a2_s[d][s] = 2. * Di2 * (A2_s + 3. * A3_s);
        L.a3_s[d][s] = 6. * Di3 * A3_s;
        const double Am_d = L.acc_d[d][s] - L.a0_d[d][s], J0_d = L.j0_d[d][s] * Dt, J1_d = L.jerk_d[d][s] * Dt;
        const double A2_d = 3. * Am_d - (J1_d + 2. * J0_d);
        const double A3_d = -2. * Am_d + (J1_d + J0_d);
        L.a2_d[d][s] = 2. * (A2_d + 3. * A3_d) * Di2;
        L.a3_d[d][s] = 6. * A3_d * Di3;
        const double A2 = A2_s + A2_d, A3 = A3_s + A3_d;
        const double x = L.xp[d][s] + 1.6666666666666667e-2 * Dt2 * (5. * A2 + 3. * 1.1666666666666667e-3 * A3);
        L.pos[d][s] = x;
        L.vel[d][s] = L.vp[d][s] + 8.3333333333333333e-2 * Dt * (4. * A2 + 3. * A3);
        L.pos32[d][s] = (float)(x - pre.ref[d]);
    }
    __syncthreads();
}

// the block-wide minimum of v
template <int NT>
__device__ __forceinline__ double lmin(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = dmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double m = red[0];
    for (int w = 1; w < NT / 32; w++) m = dmin(m, red[w]);
    return m;
}

// mergeAccJerk (src/hermite.h:36-83) of the merged targets among
// L.tgt[0..cnt): the mass-weighted mean of the target's and its twins'
// planet terms, the merge_acc_jerk arithmetic in the same order.  linked:
// only targets that have twins (the team form's finish), else every merged one.
template <int NT>
__device__ void lone_merge(LoneSmem<NT> &L, int cnt, bool linked) {
    for (int t = threadIdx.x; t < cnt; t += NT) {
        const int s = L.tgt[t];
        if (!L.merged[s] || (linked && L.tw_head[s] < 0)) continue;
        V3 a = L.mass[s] * lv(L.acc_d, s), j = L.mass[s] * lv(L.jerk_d, s);
        double m = L.mass[s];
        for (int k = L.tw_head[s], g = 0; k >= 0 && g < LCAP; k = L.tw_next[k], g++) {
            addto(a, L.mass[k] * lv(L.acc_d, k));
            addto(j, L.mass[k] * lv(L.jerk_d, k));
            m += L.mass[k];
        }
        const double mi = 1. / m;
        a = a * mi;
        j = j * mi;
        lst(L.acc_d, s, a);
        lst(L.jerk_d, s, j);
        for (int k = L.tw_head[s], g = 0; k >= 0 && g < LCAP; k = L.tw_next[k], g++) {
            lst(L.acc_d, k, a);
            lst(L.jerk_d, k, j);
        }
    }
    __syncthreads();
}

// the cluster's state to the hard-part state of record (slots o..o+n-1),
// as of a block step's start
template <int NT>
__device__ void lone_store(const HardArgs &A, int c, const LoneSmem<NT> &L, const Pre &pre) {
    const Hard &H = A.H;
    const int o = A.off[c], n = A.cnt[c];
    auto glob = [o](int k) { return k >= 0 ? o + k : -1; };
    for (int m = threadIdx.x; m < n; m += NT) {
        const int g = o + m, i = A.members[g];
        st3(H.pos, g, lv(L.pos, m)); st3(H.vel, g, lv(L.vel, m));
        st3(H.acc_s, g, lv(L.acc_s, m)); st3(H.jerk_s, g, lv(L.jerk_s, m));
        st3(H.acc_d, g, lv(L.acc_d, m)); st3(H.jerk_d, g, lv(L.jerk_d, m));
        const V3 z = v3(0., 0., 0.);
        st3(H.x0, g, z); st3(H.v0, g, z); st3(H.a0_s, g, z); st3(H.j0_s, g, z); st3(H.a0_d, g, z);
        st3(H.j0_d, g, z); st3(H.xp, g, z); st3(H.vp, g, z); st3(H.a2_s, g, z); st3(H.a3_s, g, z);
        st3(H.a2_d, g, z); st3(H.a3_d, g, z);
        H.phi_d[g] = L.phi_d[m]; H.phi_s[g] = L.phi_s[m];
        H.mass[g] = L.mass[m]; H.r_planet[g] = L.rp[m]; H.f[g] = L.fa[m];
        H.r_out_inv[g] = L.roi[m];
        H.time_c[g] = A.S.time[i]; H.th[g] = L.th[m]; H.dt[g] = L.dt[m]; H.acc0[g] = L.acc0[m];
        H.id[g] = L.id[m];
        H.dead[g] = L.dead[m]; H.merged[g] = L.merged[m];
        H.tw_head[g] = glob(L.tw_head[m]); H.tw_tail[g] = glob(L.tw_tail[m]); H.tw_next[g] = glob(L.tw_next[m]);
        st32(H.pos32, g, lv(L.pos, m), pre);
        H.roi32[g] = L.roi32[m];
        H.fr32[g] = L.fr32[m];
    }
    __syncthreads();
}

// the state of record back into shared memory, after the team form's loop
// integrated a block step with a collision
template <int NT>
__device__ void lone_reload(const HardArgs &A, int c, LoneSmem<NT> &L, const Pre &pre) {
    const Hard &H = A.H;
    const int o = A.off[c], n = A.cnt[c];
    auto loc = [o](int g) { return g >= 0 ? g - o : -1; };
    if (threadIdx.x == 0) L.any_merged = 0;
    __syncthreads();
    for (int m = threadIdx.x; m < n; m += NT) {
        const int g = o + m;
        lst(L.pos, m, ld3(H.pos, g)); lst(L.vel, m, ld3(H.vel, g));
        lst(L.acc_s, m, ld3(H.acc_s, g)); lst(L.jerk_s, m, ld3(H.jerk_s, g));
        lst(L.acc_d, m, ld3(H.acc_d, g)); lst(L.jerk_d, m, ld3(H.jerk_d, g));
        L.phi_d[m] = H.phi_d[g]; L.phi_s[m] = H.phi_s[g];
        L.mass[m] = H.mass[g]; L.rp[m] = H.r_planet[g]; L.fa[m] = H.f[g];
        L.fr[m] = H.f[g] * H.r_planet[g];
        L.th[m] = H.th[g]; L.dt[m] = H.dt[g]; L.acc0[m] = H.acc0[g];
        L.id[m] = H.id[g];
        L.dead[m] = H.dead[g]; L.merged[m] = H.merged[g];
        L.tw_head[m] = loc(H.tw_head[g]); L.tw_tail[m] = loc(H.tw_tail[g]); L.tw_next[m] = loc(H.tw_next[g]);
        lst32(L.pos32, m, lv(L.pos, m), pre);
        L.fr32[m] = H.fr32[g];
        if (L.merged[m]) L.any_merged = 1;
    }
    __syncthreads();
}

// timeIntegrate_multi (src/hermite.h:224-479) of cluster c by one CTA
template <int NT>
__device__ void lone_cluster(const HardArgs &A, int c, LoneSmem<NT> &L, const Team<NT> &tm, double *red_d) {
    const Params &P = A.P;
    const int tid = threadIdx.x;
    const int o = A.off[c], n = A.cnt[c];
    ClusterRun run;
    run.t_start = (A.times && tid == 0) ? global_ns() : 0;
    // FPHard(const FPGrav&), src/particle.h:1096-1116
    for (int m = tid; m < n; m += NT) {
        const int i = A.members[o + m];
        lst(L.pos, m, ld3(A.S.pos, i));
        lst(L.vel, m, ld3(A.S.vel, i));
        lst(L.acc_s, m, ld3(A.S.acc_s, i));
        lst(L.jerk_s, m, ld3(A.S.jerk_s, i));
        lst(L.acc_d, m, ld3(A.S.acc_d, i));
        lst(L.jerk_d, m, ld3(A.S.jerk_d, i));
        L.phi_d[m] = A.S.phi_d[i];
        L.phi_s[m] = A.S.phi_s[i];
        L.mass[m] = A.S.mass[i];
        L.roi[m] = A.S.r_out_inv[i];
        L.rp[m] = A.S.r_planet[i];
        L.fa[m] = A.S.f[i];
        L.fr[m] = A.S.f[i] * A.S.r_planet[i];
        L.dead[m] = 0; L.merged[m] = 0;
        L.tw_head[m] = L.tw_tail[m] = L.tw_next[m] = -1;
        L.th[m] = 0.;
        L.dt[m] = A.S.dt[i];
        L.acc0[m] = A.S.acc0[i];
        L.id[m] = A.S.id[i];
    }
    // the team form's FP32 prefilter (cluster_load)
    Pre pre;
    {
        const V3 r0 = ld3(A.S.pos, A.members[o]);
        pre.ref[0] = r0.x; pre.ref[1] = r0.y; pre.ref[2] = r0.z;
        double ext = 0., rmin = 1.e300;
        for (int m = tid; m < n; m += NT) {
            const int i = A.members[o + m];
            const V3 d = ld3(A.S.pos, i) - r0;
            ext = dmax(ext, dmax(fabs(d.x), dmax(fabs(d.y), fabs(d.z))));
            rmin = dmin(rmin, dmin(2. * A.S.f[i] * A.S.r_planet[i], 1. / A.S.r_out_inv[i]));
            lst32(L.pos32, m, ld3(A.S.pos, i), pre);
            L.roi32[m] = (float)A.S.r_out_inv[i];
            L.fr32[m] = (float)(A.S.f[i] * A.S.r_planet[i]);
        }
        ext = -lmin<NT>(-ext, red_d);
        rmin = lmin<NT>(rmin, red_d);
        pre.on = (ext + 0.05) * 1e-6 < 0.25 * rmin;
    }
    for (int m = tid; m < n; m += NT) L.tgt[m] = m;
    if (tid == 0) {
        L.n_tgt = n;
        L.any_merged = 0;
    }
    __syncthreads();
    lone_pass(A, L, n, 0, pre);
    double time = 0.;
    int steps = 0;
    long long work = 0;
    while (time < A.t_end) {
        if (++steps > A.max_steps) {
            if (tid == 0) atomicOr(A.status, ST_ITER_CAP);
            break;
        }
        // makeActiveList, src/hermite.h:4-24
        double tsm = 1.e10;
        for (int m = tid; m < n; m += NT)
            if (!L.dead[m]) tsm = dmin(tsm, L.th[m] + L.dt[m]);
        const double ts = lmin<NT>(tsm, red_d);
        if (tid == 0) L.ts = ts;
        // predict every member, one thread per (member, component)
        for (int it = tid; it < 3 * n; it += NT) {
            const int d = it / n, m = it - d * n;
            const double Dt = ts - L.th[m];
            const double as = L.acc_s[d][m], js = L.jerk_s[d][m], ad = L.acc_d[d][m], jd = L.jerk_d[d][m];
            L.a0_s[d][m] = as; L.j0_s[d][m] = js; L.a0_d[d][m] = ad; L.j0_d[d][m] = jd;
            const double a = as + ad, j = js + jd;
            const double x = L.pos[d][m] + Dt * (L.vel[d][m] + Dt * (0.5 * a + 1.6666666666666667e-1 * Dt * j));
            L.xp[d][m] = x;
            L.vp[d][m] = L.vel[d][m] + Dt * (a + Dt * 0.5 * j);
            L.xp32[d][m] = (float)(x - pre.ref[d]);
        }
        __syncthreads();
        // collisionDetermination, src/hermite.h:98-196: unordered pairs (a < b)
        // stand for both ordered ones (equal R; the smaller index a n + b)
        double Rb = 1.;
        long long pb = 0x7fffffffffffffffLL;
        for (int a = 0; a + 1 < n; a++)
            for (int b = a + 1 + tid; b < n; b += NT) {
                if (L.dead[a] || L.dead[b]) continue;
                if (pre.on) {
                    const float rs = L.fr32[a] + L.fr32[b];
                    if (ld2_32(L.xp32, a, L.xp32, b) > 4.0f * rs * rs) continue;
                }
                const V3 dr = lv(L.xp, a) - lv(L.xp, b);
                const double d2 = dot(dr, dr);
                const double r2 = L.fr[a] + L.fr[b];
                if (d2 > r2 * r2 * 1.000001) continue;
                const double R = sqrt(d2) / r2;
                const long long p = (long long)a * n + b;
                if (R < Rb || (R == Rb && R < 1. && p < pb)) { Rb = R; pb = p; }
            }
        tm.argmin(Rb, pb);
        if (Rb < 1.) {
            // a collision: the team form integrates this block step from its
            // start (the same prediction, the same collision), then the lone
            // form goes on from the state it leaves
            lone_store(A, c, L, pre);
            run.time = time;
            run.steps = steps - 1;
            run.work = work;
            cluster_loop<NT>(A, c, tm, pre, run, true);
            time = run.time;
            steps = run.steps;
            work = run.work;
            lone_reload(A, c, L, pre);
            continue;
        }
        // the active set, ascending member order (alive members only), then
        // the twins of the merged ones, which move with their target
        {
            int f[2], tot;
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int m = 2 * tid + r;
                f[r] = (m < n) && !L.dead[m] && (L.th[m] + L.dt[m] == ts);
            }
            int off = lscan<NT>(f[0] + f[1], L.ws, tot);
            if (f[0]) L.tgt[off++] = 2 * tid;
            if (f[1]) L.tgt[off] = 2 * tid + 1;
            if (tid == 0) {
                L.n_tgt = tot;
                L.n_act = tot;
            }
            __syncthreads();
            work += (long long)(f[0] + f[1]) * n;
            if (L.any_merged) {
                if (tid == 0) {
                    int k = tot;
                    for (int t = 0; t < tot; t++) {
                        const int s = L.tgt[t];
                        if (L.merged[s])
                            for (int x = L.tw_head[s], g = 0; x >= 0 && g < LCAP && k < LCAP; x = L.tw_next[x], g++)
                                L.tgt[k++] = x;
                    }
                    L.n_tgt = k;
                }
                __syncthreads();
            }
        }
        const int na = L.n_act;
        lone_pass(A, L, n, 1, pre);
        if (L.any_merged) lone_merge(L, na, false);
        for (int it2 = 0; it2 < 2; it2++) {
            lone_correct(L, pre);
            lone_pass(A, L, n, 2, pre);
            if (L.any_merged) lone_merge(L, na, false);
        }
        // time and calcDeltat: the two criteria of a member in two threads
        const int nt = L.n_tgt;
        for (int it = tid; it < 2 * na; it += NT) {
            const int t = it >> 1, q = it & 1, s = L.tgt[t];
            // one code path for both criteria (the inputs chosen by q): lanes
            // of a warp that took two paths would run them one after the other
            const bool sun = q != 0;
            L.dtq[q][t] = dt4th(sun ? P.eta_sun : P.eta, P.alpha2, sun ? 0. : L.acc0[s], lv(sun ? L.acc_s : L.acc_d, s),
                                lv(sun ? L.jerk_s : L.jerk_d, s), lv(sun ? L.a2_s : L.a2_d, s),
                                lv(sun ? L.a3_s : L.a3_d, s));
        }
        __syncthreads();
        for (int t = tid; t < nt; t += NT) {
            const int s = L.tgt[t];
            const double tc = ts - L.th[s];
            L.th[s] += tc;
            if (t >= na) continue;  // a twin: its target's dt below
            // dt_hermite with the criteria above
            const double dtc = L.dt[s];
            double dt_next = dmin(2. * dtc, 0.5 * P.dt_tree);
            const double dt_1 = dmin(L.dtq[0][t], L.dtq[1][t]);
            const double tt = L.th[s];
            double rem = rem_pow2(tt, dt_next);
            for (int k = 0; rem != 0.0 && k < 1100; k++) {
                dt_next *= 0.5;
                rem = rem_pow2(tt, dt_next);
            }
            for (int k = 0; dt_1 < dt_next && 0.5 * dtc < dt_next && k < 1100; k++) dt_next *= 0.5;
            if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
            L.dt[s] = dt_next;
        }
        __syncthreads();
        if (L.any_merged) {
            for (int t = tid; t < na; t += NT) {
                const int s = L.tgt[t];
                if (L.merged[s])
                    for (int x = L.tw_head[s], g = 0; x >= 0 && g < LCAP; x = L.tw_next[x], g++) L.dt[x] = L.dt[s];
            }
            __syncthreads();
        }
        // getSystemTime, src/hermite.h:25-35
        double tmin = 1.e10;
        for (int m = tid; m < n; m += NT)
            if (!L.dead[m]) tmin = dmin(tmin, L.th[m]);
        time = lmin<NT>(tmin, red_d);
    }
    // last full force, write-back with resetTime (src/hard.h:768-787), logs
    for (int m = tid; m < n; m += NT) L.tgt[m] = m;
    if (tid == 0) L.n_tgt = n;
    __syncthreads();
    lone_pass(A, L, n, 0, pre);
    if (L.any_merged) lone_merge(L, n, true);
    for (int m = tid; m < n; m += NT) {
        const int i = A.members[o + m];
        st3(A.S.pos, i, lv(L.pos, m)); st3(A.S.vel, i, lv(L.vel, m));
        st3(A.S.acc_s, i, lv(L.acc_s, m)); st3(A.S.jerk_s, i, lv(L.jerk_s, m));
        st3(A.S.acc_d, i, lv(L.acc_d, m)); st3(A.S.jerk_d, i, lv(L.jerk_d, m));
        A.S.phi_d[i] = L.phi_d[m]; A.S.phi_s[i] = L.phi_s[m];
        A.S.mass[i] = L.mass[m]; A.S.r_planet[i] = L.rp[m];
        A.S.time[i] = A.S.time[i] + L.th[m];
        A.S.dt[i] = L.dt[m];
        A.S.id[i] = L.id[m];
        A.S.dead[i] = L.dead[m]; A.S.merged[i] = L.merged[m];
        A.S.n_cluster[i] = n;
    }
    if (A.cost) atomicAdd((unsigned long long *)&A.cost[2 * c + 1], (unsigned long long)work);
    if (tid == 0) {
        A.cl_edisp[2 * c] = (run.n_col > 0) ? run.ed : 0.;
        A.cl_edisp[2 * c + 1] = (run.n_col > 0) ? run.edd : 0.;
        if (A.cost) A.cost[2 * c] = steps;
        if (A.times) {
            A.times[2 * c] = run.t_start;
            A.times[2 * c + 1] = global_ns();
        }
    }
    __syncthreads();
}

// The lone clusters (tier 2 of the bundle form's queue) one after another
// per CTA, on a stream of their own beside k_hard_bundles.
__global__ void __launch_bounds__(LONE_T, 1) k_hard_lone(HardArgs A) {
    extern __shared__ __align__(16) unsigned char lone_smem[];
    LoneSmem<LONE_T> &L = *reinterpret_cast<LoneSmem<LONE_T> *>(lone_smem);
    __shared__ double red_d[LONE_T / 32];
    __shared__ long long red_l[LONE_T / 32];
    __shared__ int q_sh;
    const int tid = threadIdx.x;
    Team<LONE_T> tm{tid, red_d, red_l};
    for (int guard = 0; guard < (1 << 30); guard++) {
        if (tid == 0) q_sh = atomicAdd(&A.queue[3], 1);
        __syncthreads();
        const int q = q_sh;
        __syncthreads();
        if (q >= A.n_tier[2]) break;
        const int c = A.order[A.n_tier[0] + A.n_tier[1] + q];
        if (A.cnt[c] > LCAP) {  // the lone tier holds at most LONE_NMAX members
            if (tid == 0) atomicOr(A.status, ST_CLUSTER_TOO_BIG);
            continue;
        }
        lone_cluster(A, c, L, tm, red_d);
    }
}

}  // namespace p3t
