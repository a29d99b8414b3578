// Device-resident P3T step: particle state, the FP64 cutoff correction and
// neighbour search, cluster labelling and lists, kicks, energy, merging and
// cut-off radii.  Compiled with -fmad=false (see p3t_phys.cuh).
#include <cmath>
#include <cstdio>
#include <type_traits>
#include <cstring>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_engine.cuh"
#include "p3t_phys.cuh"
#include "p3t_soft.cuh"

namespace p3t {

Engine g_eng;

// ---------------------------------------------------------------------------
// small device helpers
__global__ void k_fill_i32(int32_t *p, int n, int32_t v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void k_fill_i64(int64_t *p, int n, int64_t v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}
__global__ void k_iota(int32_t *p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}
inline int nb(int n, int t = 256) { return (n + t - 1) / t; }

// Exclusive scan of int32 (block-level Hillis-Steele in shared memory, then
// block sums scanned recursively).
__global__ void k_scan_block(const int32_t *in, int32_t *out, int32_t *bsum, int n) {
    __shared__ int32_t s[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int32_t v = (i < n) ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        int32_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}
__global__ void k_scan_add(int32_t *out, const int32_t *bscan, int n) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) out[i] += bscan[blockIdx.x];
}

int Engine::scan(const int32_t *in, int32_t *out, int n, int32_t *total) {
    if (n <= 0) {
        if (total) *total = 0;
        return 0;
    }
    // levels of block sums live in scan_tmp
    std::vector<int> sizes;
    int m = n;
    size_t need = 0;
    while (true) {
        const int blocks = (m + 1023) / 1024;
        sizes.push_back(m);
        need += (size_t)blocks * 2;
        if (blocks <= 1) break;
        m = blocks;
    }
    int r = scan_tmp.reserve(need + 2);
    if (r) return r;
    // recursive scan
    struct Lvl { const int32_t *in; int32_t *out; int32_t *bsum; int n; };
    std::vector<Lvl> lv;
    int32_t *tmp = scan_tmp.p;
    const int32_t *cur_in = in;
    int32_t *cur_out = out;
    int cn = n;
    while (true) {
        const int blocks = (cn + 1023) / 1024;
        int32_t *bsum = tmp;
        int32_t *bscan = tmp + blocks;
        tmp += 2 * blocks;
        lv.push_back({cur_in, cur_out, bsum, cn});
        { P3T_COUNT_LAUNCH(); k_scan_block<<<blocks, 1024, 0, c->stream>>>(cur_in, cur_out, bsum, cn); }
        if (blocks <= 1) break;
        cur_in = bsum;
        cur_out = bscan;
        cn = blocks;
    }
    for (int L = (int)lv.size() - 2; L >= 0; L--) {
        const int blocks = (lv[L].n + 1023) / 1024;
        { P3T_COUNT_LAUNCH(); k_scan_add<<<blocks, 1024, 0, c->stream>>>(lv[L].out, lv[L + 1].out, lv[L].n); }
    }
    if (total) {
        // total = out[n-1] + in[n-1]
        int32_t a = 0, b = 0;
        if (n > 0) {
            cudaMemcpyAsync(&a, out + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
            cudaMemcpyAsync(&b, in + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        }
        r = cuda_status(cudaStreamSynchronize(c->stream));
        if (r) return r;
        *total = a + b;
    }
    return cuda_status(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// state -> soft-kernel particle records
__global__ void k_pack_state(State S, SoftPtcl *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    SoftPtcl r;
    r.x = S.pos[3 * i];
    r.y = S.pos[3 * i + 1];
    r.z = S.pos[3 * i + 2];
    r.m = (float)S.mass[i];
    const float ro = (float)S.r_out[i], rs = (float)S.r_search[i];
    r.ro2 = __fmul_rn(ro, ro);
    r.rs2 = __fmul_rn(__fmul_rn(rs, rs), 1.0201f);
    r.id_local = i;
    r.rank = 0;
    r.pad = 0;
    out[i] = r;
}

// ---------------------------------------------------------------------------
// cutoff correction + neighbour search, src/gravity_soft.h:75-528
struct CorrOut {
    V3 acc, acc_d, jerk;
    double phi, phi_d, acc0;
    int number;
    int64_t idc;
};

// correctForceLong / correctForceLongInitial (src/gravity_soft.h:245-528) in
// three passes, so that the FP64 pair arithmetic runs lane-dense: a warp
// instruction of the FP64 pipe costs the pipe all 32 lanes whatever the
// mask, and bodies have from 0 to dozens of candidates.
//   1. per body: its candidates (the soft kernel's screen hits) in ascending
//      index order, invalid and same-id entries dropped, appended to a pair
//      list (a block of consecutive slots per body);
//   2. per pair: the pair's terms (corr_pair's arithmetic, unchanged);
//   3. per body: the terms folded in candidate order -- the order of
//      GPLUM's loop -- then the write-back (and, initially, the sun force
//      and the first time step).
// Results are bit-identical to one thread walking its candidates.
struct PairTerms {
    V3 acc, acc_d, jerk;
    double phi, phi_d, acc0;
    int flags;  // 1: neighbour, 2: inside r_out
};

// the next smallest candidate of body i above `last` (lists are short; -1: none)
__device__ __forceinline__ int next_cand(const int32_t *__restrict__ cand, int i, int cap, int kc, int last) {
    int best = 0x7fffffff;
    for (int u = 0; u < kc; u++) {
        const int c = cand[(size_t)i * cap + u];
        if (c > last && c < best) best = c;
    }
    return best == 0x7fffffff ? -1 : best;
}

// pass 1: per body, the usable candidates in ascending index order -- counted
// (fill = false) or written to the body's slots of the pair list (fill = true)
template <bool FILL>
__global__ void k_corr_list(State S, const ForceRec *__restrict__ F, const int32_t *__restrict__ cand, int cap,
                            int32_t *pair_n, const int32_t *__restrict__ pair_base, int32_t *pair_i, int32_t *pair_j,
                            int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int k = F[i].number;
    const int64_t id_i = S.id[i];
    const int kc = min(k, cap);
    if (!FILL && k > cap) atomicOr(status, ST_CAND_OVERFLOW);
    const int base = FILL ? pair_base[i] : 0;
    int m = 0, last = -1;
    for (int t = 0; t < kc; t++) {
        const int j = next_cand(cand, i, cap, kc, last);
        if (j < 0) break;
        last = j;
        if ((unsigned)j >= (unsigned)S.n) {
            if (!FILL) atomicOr(status, ST_BAD_INDEX);
            continue;
        }
        if (S.id[j] == id_i) continue;
        if (FILL) {
            pair_i[base + m] = i;
            pair_j[base + m] = j;
        }
        m++;
    }
    if (!FILL) pair_n[i] = m;
}

// corr_pair's arithmetic for one pair (src/gravity_soft.h:75-242), terms out
template <bool INITIAL>
__global__ void __launch_bounds__(128) k_corr_pairs(State S, Params P, int np, const int32_t *__restrict__ pair_i,
                                                    const int32_t *__restrict__ pair_j, PairTerms *out) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        const int i = pair_i[q], j = pair_j[q];
        PairTerms o;
        o.flags = 0;
        const V3 pos_i = ld3(S.pos, i), vel_i = ld3(S.vel, i), accd_i = ld3(S.acc_d, i);
        const double mj = S.mass[j];
        const double r_out = dmax(S.r_out[i], S.r_out[j]);
        const double r_out_inv = dmin(S.r_out_inv[i], S.r_out_inv[j]);
        const double r_search = dmax(S.r_search[i], S.r_search[j]);
        const V3 dr = ld3(S.pos, j) - pos_i;
        double dr2 = dot(dr, dr);
        dr2 += P.eps2;
        const double rij = sqrt(dr2);
        const V3 dv = ld3(S.vel, j) - vel_i;
        const V3 da = ld3(S.acc_d, j) - accd_i;
        const double drdv = dot(dr, dv);
        const double dv2 = dot(dv, dv);
        const double da2 = dot(da, da);
        const double t_min = dmin(dmax(-drdv / sqrt(dv2), 0.), P.dt_tree);
        const double dr2_min = dmin(dr2, dr2 + 2. * drdv * t_min + dv2 * t_min * t_min);
        const double r_crit = P.R_search2 * r_out;
        const double v_crit_a = P.R_search3 * 0.5 * P.dt_tree;
        if (dr2_min < r_crit * r_crit || dv2 < v_crit_a * v_crit_a * da2 || (INITIAL && da2 == 0.)) {
            if (rij < r_search) {
                // NeighborList::addNeighbor, src/neighbor.h:635-670
                o.flags |= 1;
                o.acc0 = r_out * r_out / mj;
            }
        }
        if (rij < r_out) {
            o.flags |= 2;
            const double rinv = 1. / rij;
            const double r2inv = rinv * rinv;
            const double r3inv = rinv * r2inv;
            const double W = cut_W(P, rij, r_out_inv);
            const double K = cut_K(P, rij, r_out_inv);
            const double r_min = dmin(rinv, r_out_inv);
            o.phi = mj * (rinv * W - r_min);
            o.acc = mj * (r3inv * K - r_min * r_min * r_min) * dr;
            if (INITIAL) {
                const double alpha = drdv * r2inv;
                const double dKdt = cut_dKdt(P, rij, r_out_inv, alpha);
                const double alpha_c = alpha * (1. - K);
                o.phi_d = mj * rinv * (1. - W);
                o.acc_d = mj * r3inv * (1. - K) * dr;
                o.jerk = mj * r3inv * ((1. - K) * dv - (3. * alpha_c + dKdt) * dr);
            }
        }
        out[q] = o;
    }
}

template <bool INITIAL>
__global__ void __launch_bounds__(128, 4) k_correct(State S, Params P, const ForceRec *__restrict__ F, int cap,
                                                    const int32_t *__restrict__ pair_base,
                                                    const int32_t *__restrict__ pair_n,
                                                    const int32_t *__restrict__ pair_j,
                                                    const PairTerms *__restrict__ terms, int32_t *counters,
                                                    int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const ForceRec fr = F[i];
    const V3 pos_i = ld3(S.pos, i), vel_i = ld3(S.vel, i), accd_i = ld3(S.acc_d, i);
    const double m_i = S.mass[i], roi_i = S.r_out_inv[i];
    const int64_t id_i = S.id[i];
    V3 acc_s = ld3(S.acc_s, i), jerk_s = ld3(S.jerk_s, i);
    if (INITIAL) {
        double phs;
        sun_force(P, pos_i, vel_i, acc_s, jerk_s, &phs);
        st3(S.acc_s, i, acc_s);
        st3(S.jerk_s, i, jerk_s);
        S.phi_s[i] = phs;
    }
    CorrOut o;
    o.acc = o.acc_d = o.jerk = v3(0., 0., 0.);
    o.phi = o.phi_d = o.acc0 = 0.;
    o.number = 0;
    o.idc = id_i;
    o.phi += m_i * roi_i;
    const int base = pair_base[i], m = pair_n[i];
    for (int t = 0; t < m; t++) {
        const PairTerms &q = terms[base + t];
        if (q.flags & 1) {
            const int j = pair_j[base + t];
            if (o.number < cap) S.nbr[(size_t)i * cap + o.number] = j;
            o.number++;
            o.idc = (S.id[j] < o.idc) ? S.id[j] : o.idc;
            o.acc0 += q.acc0;
        }
        if (q.flags & 2) {
            o.phi -= q.phi;
            addto(o.acc, q.acc);
            if (INITIAL) {
                o.phi_d -= q.phi_d;
                addto(o.acc_d, q.acc_d);
                addto(o.jerk, q.jerk);
            }
        }
    }
    if (o.number > cap) atomicOr(status, ST_CAND_OVERFLOW);
    // write back (FPGrav::copyFromForce then the corrections)
    st3(S.acc, i, v3((double)fr.acc[0], (double)fr.acc[1], (double)fr.acc[2]) + o.acc);
    S.phi[i] = (double)fr.phi + o.phi;
    S.acc0[i] = (o.acc0 > 0.) ? o.number / o.acc0 : 0.;
    S.number[i] = o.number;
    S.rank[i] = fr.rank;
    S.id_max[i] = fr.id_max;
    S.id_min[i] = fr.id_min;
    S.id_cluster[i] = o.idc;
    S.nbr_n[i] = min(o.number, cap);
    if (o.number) {
        atomicAdd(&counters[0], o.number);
        atomicAdd(&counters[1], 1);
    }
    if (INITIAL) {
        st3(S.acc_d_new, i, o.acc_d);
        S.phi_d[i] = o.phi_d;
        st3(S.jerk_d, i, o.jerk);
        // calcDeltatInitial reads the pre-pass acc_d (src/gravity_soft.h:388-391,510)
        S.dt[i] = dt_initial(P, S.time[i], S.dt[i], S.acc0[i], accd_i, o.jerk, acc_s, jerk_s);
    }
}

__global__ void k_copy3(double *dst, const double *src, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * n) dst[i] = src[i];
}

// NeighborList::pair_list (src/neighbor.h:635-670): the local pairs (i, j),
// i < j, j a neighbour of i, by i and then in neighbour-list order.
__global__ void k_pair_count(State S, int cap, int32_t *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int m = S.nbr_n[i];
    int c = 0;
    for (int t = 0; t < m; t++) c += (i < S.nbr[(size_t)i * cap + t]) ? 1 : 0;
    cnt[i] = c;
}
__global__ void k_pair_fill(State S, int cap, const int32_t *base, int32_t *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int m = S.nbr_n[i];
    int k = base[i];
    for (int t = 0; t < m; t++) {
        const int j = S.nbr[(size_t)i * cap + t];
        if (i < j) {
            out[2 * k] = i;
            out[2 * k + 1] = j;
            k++;
        }
    }
}

// ---------------------------------------------------------------------------
// cluster labelling, src/neighbor.h:800-839: connected components of the
// local pairs (i < j, j a neighbour of i), each labelled with the minimum
// id_cluster of its members.  Union-find with hooking to the smaller index.
__device__ __forceinline__ int uf_find(const int32_t *lab, int x) {
    for (int k = 0; k < 1 << 20; k++) {
        const int p = lab[x];
        if (p == x) return x;
        x = p;
    }
    return x;
}
__global__ void k_union(State S, int cap, int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int m = S.nbr_n[i];
    for (int t = 0; t < m; t++) {
        const int j = S.nbr[(size_t)i * cap + t];
        if (!(i < j)) continue;
        int a = i, b = j;
        int tries = 0;
        while (true) {
            a = uf_find(S.label, a);
            b = uf_find(S.label, b);
            if (a == b) break;
            if (a > b) { int t2 = a; a = b; b = t2; }
            const int old = atomicCAS(&S.label[b], b, a);
            if (old == b) break;
            if (++tries > (1 << 20)) { atomicOr(status, ST_ITER_CAP); break; }
        }
    }
}
__global__ void k_compress(State S, int64_t *cmin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int r = uf_find(S.label, i);
    S.label[i] = r;
    atomicMin((unsigned long long *)&cmin[r], (unsigned long long)S.id_cluster[i]);
}
__global__ void k_apply_label(State S, const int64_t *cmin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    S.id_cluster[i] = cmin[S.label[i]];
}

// ---------------------------------------------------------------------------
// cluster lists, src/hard.h:321-438: members are the particles with
// neighbours, grouped by component, clusters ordered by their smallest
// member index, members in ascending index order.
__global__ void k_head(State S, int32_t *head) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    if (S.number[i] > 0) atomicMin(&head[S.label[i]], i);
}
__global__ void k_head_flag(State S, const int32_t *head, int32_t *flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    flag[i] = (S.number[i] > 0 && head[S.label[i]] == i) ? 1 : 0;
}
__global__ void k_member_count(State S, const int32_t *head, const int32_t *cidx, int32_t *cl_of, int32_t *cnt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    if (S.number[i] > 0) {
        const int c = cidx[head[S.label[i]]];
        cl_of[i] = c;
        atomicAdd(&cnt[c], 1);
    } else {
        cl_of[i] = -1;
    }
}
__global__ void k_member_fill(State S, const int32_t *cl_of, const int32_t *off, int32_t *fill, int32_t *members) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const int c = cl_of[i];
    if (c < 0) return;
    const int s = atomicAdd(&fill[c], 1);
    members[off[c] + s] = i;
}
// one warp per cluster: rank members by index
__global__ void k_member_sort(int nc, const int32_t *off, const int32_t *cnt, const int32_t *in, int32_t *out) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= nc) return;
    const int o = off[w], m = cnt[w];
    for (int a = lane; a < m; a += 32) {
        const int v = in[o + a];
        int r = 0;
        for (int b = 0; b < m; b++) r += (in[o + b] < v);
        out[o + r] = v;
    }
}

// ---------------------------------------------------------------------------
// kicks, energy
__global__ void k_kick(State S, double half_dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const V3 v = ld3(S.vel, i), a = ld3(S.acc, i);
    st3(S.vel, i, v + half_dt * a);
}
// Energy::calcEnergy, src/energy.h:29-63, per-block partial sums in a fixed
// order, then one ordered pass over the blocks.
__global__ void k_energy_partial(State S, double *part) {
    __shared__ double s[4][256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ek = 0., es = 0., ep = 0., ed = 0.;
    if (i < S.n) {
        const double m = S.mass[i];
        const V3 v = ld3(S.vel, i);
        ek = dot(m * v, v);
        es = m * S.phi_s[i];
        ep = m * S.phi[i];
        ed = m * S.phi_d[i];
    }
    s[0][threadIdx.x] = ek; s[1][threadIdx.x] = es; s[2][threadIdx.x] = ep; s[3][threadIdx.x] = ed;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int q = 0; q < 4; q++) s[q][threadIdx.x] += s[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[4 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}
// one block of 256: each thread sums a contiguous run of block partials in
// order, then a fixed tree over the threads (deterministic)
__global__ void k_energy_final(const double *part, int nblk, double *out) {
    __shared__ double s[4][256];
    const int t = threadIdx.x, per = (nblk + 255) / 256;
    double q[4] = {0., 0., 0., 0.};
    for (int b = t * per; b < min(nblk, (t + 1) * per); b++)
        for (int k = 0; k < 4; k++) q[k] += part[4 * b + k];
    for (int k = 0; k < 4; k++) s[k][t] = q[k];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (t < h)
            for (int k = 0; k < 4; k++) s[k][t] += s[k][t + h];
        __syncthreads();
    }
    if (t) return;
    const double ek = 0.5 * s[0][0], es = s[1][0], ep = 0.5 * s[2][0], ed = 0.5 * s[3][0];
    out[1] = ek; out[2] = es; out[3] = ep; out[4] = ed;
    out[0] = ek + es + (ep + ed);
}

// ---------------------------------------------------------------------------
// cut-off radii, src/particle.h:713-733,1319-1457 (individual cutoff)
__global__ void k_rminmax(State S, double *mm) {
    __shared__ double smax[256], smin[256];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double r2 = 0., r2m = -1.7976931348623157e308;
    if (i < S.n) {
        const double x = S.pos[3 * i], y = S.pos[3 * i + 1];
        r2 = x * x + y * y;
        r2m = -r2;
    }
    smax[threadIdx.x] = r2;
    smin[threadIdx.x] = r2m;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            smax[threadIdx.x] = dmax(smax[threadIdx.x], smax[threadIdx.x + h]);
            smin[threadIdx.x] = dmax(smin[threadIdx.x], smin[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // non-negative doubles order like their bit patterns: mm[0] = max r^2,
        // mm[1] = min r^2 (src/particle.h:1324-1333 keeps it as max of -r^2)
        atomicMax((unsigned long long *)&mm[0], (unsigned long long)__double_as_longlong(smax[0]));
        atomicMin((unsigned long long *)&mm[1], (unsigned long long)__double_as_longlong(-smin[0]));
    }
}
constexpr int NBIN = 32;
constexpr int VD_T = 96;
constexpr int VD_BLOCKS_PER_SM = 6;
__global__ void k_vdisp_partial(State S, double r_min, double drinv, double m_sun, double *part, int *cntp) {
    __shared__ double sv[NBIN][VD_T];
    __shared__ int sc[NBIN][VD_T];
    for (int b = 0; b < NBIN; b++) { sv[b][threadIdx.x] = 0.; sc[b][threadIdx.x] = 0; }
    const int per = (S.n + gridDim.x - 1) / gridDim.x;
    const int beg = blockIdx.x * per, end = min(S.n, beg + per);
    for (int i = beg + threadIdx.x; i < end; i += blockDim.x) {
        const V3 pos = ld3(S.pos, i);
        const double ri = sqrt(pos.x * pos.x + pos.y * pos.y);
        int b = (int)((ri - r_min) * drinv);
        if (b == NBIN) b = NBIN - 1;
        b = max(0, min(NBIN - 1, b));
        V3 vk = v3(-pos.y / ri, pos.x / ri, 0.);
        vk = vk * sqrt(m_sun / sqrt(pos.x * pos.x + pos.y * pos.y));
        const V3 vr = ld3(S.vel, i) - vk;
        sv[b][threadIdx.x] += dot(vr, vr);
        sc[b][threadIdx.x] += 1;
    }
    __syncthreads();
    if (threadIdx.x < NBIN) {
        double s = 0.;
        int c = 0;
        for (int t = 0; t < VD_T; t++) { s += sv[threadIdx.x][t]; c += sc[threadIdx.x][t]; }
        part[blockIdx.x * NBIN + threadIdx.x] = s;
        cntp[blockIdx.x * NBIN + threadIdx.x] = c;
    }
}
// the bins' sums over the partials: 32 slices of the partials per bin, then
// the slices in order (one block of 32 x 32 threads)
__global__ void k_vdisp_bins(const double *part, const int *cntp, int nblk, double *vd, int *cnt) {
    __shared__ double ss[32][NBIN + 1];
    __shared__ int sn[32][NBIN + 1];
    const int b = threadIdx.x & (NBIN - 1), sl = threadIdx.x / NBIN;
    double s = 0.;
    int c = 0;
    for (int k = sl; k < nblk; k += 32) { s += part[k * NBIN + b]; c += cntp[k * NBIN + b]; }
    ss[sl][b] = s;
    sn[sl][b] = c;
    __syncthreads();
    if (sl) return;
    s = 0.;
    c = 0;
    for (int k = 0; k < 32; k++) { s += ss[k][b]; c += sn[k][b]; }
    vd[b] = (c > 0) ? sqrt(s / c) : 0.;
    cnt[b] = c;
}
// The Gaussian weights w_b = exp(-t_b^2), t_b = (r_min + (b + 1/2) dr - r) / dr
// (src/particle.h:1443-1456): by the bin-by-bin FP64 exp for the RB bins on
// either side of the body's own, in FP32 beyond (their weights are below
// exp(-(RB + 1/2)^2) ~ 1e-13 of the nearest, so FP32's 1e-6 relative error
// there stays below 1e-19 of the sums); the sums come out within a few ulp
// of the bin-by-bin FP64 arithmetic at a third of its FP64 work.
constexpr int RB = 5;
__global__ void k_radii(State S, Params P, double r_min, double dr, double drinv, const double *vd, const int *cnt) {
    __shared__ double s_vd[NBIN], s_on[NBIN];
    __shared__ float s_vdf[NBIN], s_onf[NBIN];
    if (threadIdx.x < NBIN) {
        s_vd[threadIdx.x] = vd[threadIdx.x];
        s_on[threadIdx.x] = (cnt[threadIdx.x] > 0) ? 1. : 0.;
        s_vdf[threadIdx.x] = (float)vd[threadIdx.x];
        s_onf[threadIdx.x] = (cnt[threadIdx.x] > 0) ? 1.f : 0.f;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const V3 pos = ld3(S.pos, i), vel = ld3(S.vel, i);
    const double r2 = pos.x * pos.x + pos.y * pos.y;
    const double rc = sqrt(r2);
    const double x = (rc - r_min) * drinv;
    const int b0 = max(0, min(NBIN - 1, (int)floor(x)));
    const int lo = max(0, b0 - RB), hi = min(NBIN - 1, b0 + RB);
    double vs = 0., ws = 0.;
    for (int b = lo; b <= hi; b++) {
        const double ddr = r_min + (b + 0.5) * dr - rc;
        const double ex = exp(-ddr * ddr * drinv * drinv);
        vs += s_vd[b] * ex;
        ws += s_on[b] * ex;
    }
    const float xf = (float)x;
    float vsf = 0.f, wsf = 0.f;
    for (int b = 0; b < NBIN; b++) {
        if (b >= lo && b <= hi) continue;
        const float t = ((float)b + 0.5f) - xf;
        const float w = expf(-t * t);
        vsf += s_vdf[b] * w;
        wsf += s_onf[b] * w;
    }
    vs += (double)vsf;
    ws += (double)wsf;
    const double v_disp = vs / ws;
    S.v_disp[i] = v_disp;
    const double r = sqrt(dot(pos, pos));
    const double rv = dot(pos, vel);
    double ax = 1.0 / (2.0 / r - dot(vel, vel) / P.m_sun);
    const double ecccosu = 1. - r / ax;
    const double eccsinu2 = rv * rv / (P.m_sun * ax);
    if (!(sqrt(ecccosu * ecccosu + eccsinu2) < 0.6)) ax = r;
    // the cube root GPLUM takes as pow(x, 1/3.), by cbrt (within 1 ulp of it,
    // at a sixth of its cost)
    const double rHill = cbrt(S.mass[i] / (3. * P.m_sun)) * ax;
    // pow(ax, -0) is 1 for every ax
    const double fac = (P.p_cut == 0.) ? 1. : pow(ax, -P.p_cut);
    const double r_out_i = dmax(P.R_cut0 * fac * rHill, P.R_cut1 * v_disp * P.dt_tree);
    double ro = dmax(r_out_i, P.r_cut_min);
    if (P.r_cut_max > 0.) ro = dmin(P.r_cut_max, ro);
    S.r_out[i] = ro;
    S.r_out_inv[i] = 1. / ro;
    S.r_search[i] = P.R_search0 * ro + P.R_search1 * v_disp * P.dt_tree;
}

// ---------------------------------------------------------------------------
// MergeParticle, src/func.h:160-207: targets fold in their dead twins (same
// id; twins share the target's cluster or are fragments made by the last
// hard part), twins leave the system (order-preserving).
__global__ void k_merge_targets(State S, const int32_t *cl_of, const int32_t *off, const int32_t *cnt,
                                const int32_t *members, int32_t *keep, double *e_t, int32_t *tflag, int frag_lo,
                                int frag_hi, const int32_t *frag_cl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    e_t[i] = 0.;
    tflag[i] = 0;
    if (!(S.merged[i] && !S.dead[i])) return;
    tflag[i] = 1;
    // twins: the cluster's members (ascending index), then the fragments the
    // hard part appended (higher indices, ascending)
    const int c = (i < frag_lo) ? cl_of[i] : (i < frag_hi ? frag_cl[i - frag_lo] : -1);
    double e = 0.;
    const int nm = (c >= 0) ? cnt[c] : 0;
    for (int t = 0; t < nm + (frag_hi - frag_lo); t++) {
        const int j = (t < nm) ? members[off[c] + t] : frag_lo + (t - nm);
        if (S.id[j] == S.id[i] && i != j) {
            const double mi = S.mass[i], mj = S.mass[j];
            const V3 vrel = ld3(S.vel, j) - ld3(S.vel, i);
            S.mass[i] += mj;
            st3(S.vel, i, (mi * ld3(S.vel, i) + mj * ld3(S.vel, j)) / (mi + mj));
            S.phi[i] = (mi * S.phi[i] + mj * S.phi[j]) / (mi + mj);
            S.phi_d[i] = (mi * S.phi_d[i] + mj * S.phi_d[j]) / (mi + mj);
            e -= dot(0.5 * mi * mj / (mi + mj) * vrel, vrel);
            keep[j] = 0;
        }
    }
    S.merged[i] = 0;
    e_t[i] = e;
}
// sum of e_t over the targets in ascending index order (the order of the
// reference's loop); the targets are first gathered by a scan
__global__ void k_gather_targets(const double *e_t, const int32_t *tflag, const int32_t *tpos, int n, double *tl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && tflag[i]) tl[tpos[i]] = e_t[i];
}
__global__ void k_sum_ordered(const double *v, int n, double *out) {
    if (threadIdx.x || blockIdx.x) return;
    double s = 0.;
    for (int i = 0; i < n; i++) s += v[i];
    *out = s;
}
// every field of the state in one pass: field f (words 32-bit words per
// body) gathers its kept bodies into tmp + off[f], then the compacted runs go
// back in a second pass
constexpr int CF_MAX = 32;
struct CompactSet {
    uint32_t *p[CF_MAX];
    int words[CF_MAX];
    long long off[CF_MAX];  // in words
    int nf;
};
__global__ void k_compact_gather(CompactSet C, const int32_t *keep, const int32_t *pos, int n, uint32_t *tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !keep[i]) return;
    const long long d = pos[i];
    for (int f = 0; f < C.nf; f++) {
        const int w = C.words[f];
        const uint32_t *src = C.p[f] + (long long)i * w;
        uint32_t *dst = tmp + C.off[f] + d * w;
        for (int k = 0; k < w; k++) dst[k] = src[k];
    }
}
// blockIdx.y: the field; its first nk bodies' words from the gathered run
__global__ void k_compact_back(CompactSet C, int nk, const uint32_t *tmp) {
    const int f = blockIdx.y;
    const long long nw = (long long)nk * C.words[f];
    uint32_t *dst = C.p[f];
    const uint32_t *src = tmp + C.off[f];
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nw; j += (long long)gridDim.x * blockDim.x)
        dst[j] = src[j];
}

// ---------------------------------------------------------------------------
// Engine host methods
template <class T>
static int alloc_field(T **p, size_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    return cuda_status(cudaMalloc(p, std::max<size_t>(n, 1) * sizeof(T)));
}

int Engine::ensure(int n) {
    if (!c) {
        c = ctx_get(0);
        if (!c) return -(int)cudaErrorNoDevice;
    }
    if (n <= S.cap && S.nbr && cand_cap_alloc == c->cand_cap) return 0;
    const int cap = std::max(n, S.cap);
    int r = 0;
    State &s = S;
    for (double **f : {&s.mass, &s.r_planet, &s.f, &s.phi, &s.phi_d, &s.phi_s, &s.r_out, &s.r_out_inv, &s.r_search,
                       &s.v_disp, &s.time, &s.dt, &s.acc0})
        if (n > s.cap && (r = alloc_field(f, cap))) return r;
    for (double **f : {&s.pos, &s.vel, &s.acc, &s.acc_d, &s.jerk_d, &s.acc_s, &s.jerk_s, &s.acc_d_new})
        if (n > s.cap && (r = alloc_field(f, 3 * (size_t)cap))) return r;
    for (int64_t **f : {&s.id, &s.id_cluster})
        if (n > s.cap && (r = alloc_field(f, cap))) return r;
    for (int32_t **f : {&s.number, &s.rank, &s.id_max, &s.id_min, &s.n_cluster, &s.dead, &s.merged, &s.nbr_n, &s.label})
        if (n > s.cap && (r = alloc_field(f, cap))) return r;
    if ((r = alloc_field(&s.nbr, (size_t)cap * c->cand_cap))) return r;
    cand_cap_alloc = c->cand_cap;
    s.cap = cap;
    return 0;
}

__global__ void k_max_number(const ForceRec *__restrict__ F, int n, int *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int v = i < n ? F[i].number : 0;
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(out, v);
}

int soft_run_state() {
    Context *c = g_eng.c ? g_eng.c : ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    for (int attempt = 0;; attempt++) {
        int r = p3t_soft_run(1);
        if (r) return r;
        const int st = read_status(c);
        if (st == 0) return 0;
        if (st != ST_CAND_OVERFLOW || attempt >= 3) return st;
        // widest row needed: the largest screen-hit count of this pass
        if ((r = g_eng.counters.reserve(4))) return r;
        int32_t *mx = g_eng.counters.p + 2;
        cudaMemsetAsync(mx, 0, sizeof(int32_t), c->stream);
        const int n = c->res_n;
        { P3T_COUNT_LAUNCH(); k_max_number<<<(n + 255) / 256, 256, 0, c->stream>>>(c->res.force.p, n, mx); }
        int h = 0;
        if ((r = d2h(c, &h, mx, sizeof(int)))) return r;
        int cap = c->cand_cap;
        while (cap < h) cap *= 2;
        if (cap == c->cand_cap || cap > (1 << 16)) return st;
        c->cand_cap = cap;
        if (g_eng.S.cap > 0 && (r = g_eng.ensure(g_eng.S.n))) return r;
    }
}

// Capacity for n bodies keeping the first S.n of every field (new
// particles from fragmentation).
int Engine::grow(int n) {
    if (n <= S.cap) return 0;
    const int cap = n + n / 8 + 1024;
    int r = 0;
    if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    auto move = [&](auto **f, size_t w) -> int {
        using T = std::remove_pointer_t<std::remove_pointer_t<decltype(f)>>;
        T *np = nullptr;
        int rr = cuda_status(cudaMalloc(&np, std::max<size_t>((size_t)cap * w, 1) * sizeof(T)));
        if (rr) return rr;
        if (*f && S.n > 0) cudaMemcpy(np, *f, (size_t)S.n * w * sizeof(T), cudaMemcpyDeviceToDevice);
        if (*f) cudaFree(*f);
        *f = np;
        return 0;
    };
    State &s = S;
    for (double **f : {&s.mass, &s.r_planet, &s.f, &s.phi, &s.phi_d, &s.phi_s, &s.r_out, &s.r_out_inv, &s.r_search,
                       &s.v_disp, &s.time, &s.dt, &s.acc0})
        if ((r = move(f, 1))) return r;
    for (double **f : {&s.pos, &s.vel, &s.acc, &s.acc_d, &s.jerk_d, &s.acc_s, &s.jerk_s, &s.acc_d_new})
        if ((r = move(f, 3))) return r;
    for (int64_t **f : {&s.id, &s.id_cluster})
        if ((r = move(f, 1))) return r;
    for (int32_t **f : {&s.number, &s.rank, &s.id_max, &s.id_min, &s.n_cluster, &s.dead, &s.merged, &s.nbr_n, &s.label})
        if ((r = move(f, 1))) return r;
    if ((r = alloc_field(&s.nbr, (size_t)cap * c->cand_cap))) return r;
    s.cap = cap;
    return 0;
}

Params Engine::params() const {
    Params P;
    const double *p = c->params;
    P.eps2 = p[0]; P.eps2_sun = p[1]; P.m_sun = p[2]; P.dt_tree = p[3]; P.dt_min = p[4];
    P.eta = p[5]; P.eta_0 = p[6]; P.eta_sun = p[7]; P.eta_sun0 = p[8]; P.alpha2 = p[9];
    P.gamma = p[10]; P.R_cut0 = p[11]; P.R_cut1 = p[12]; P.R_search0 = p[13]; P.R_search1 = p[14];
    P.R_search2 = p[15]; P.R_search3 = p[16]; P.r_cut_min = p[17]; P.r_cut_max = p[18]; P.p_cut = p[19];
    P.dens = p[20];
    // FPGrav::setGamma, src/particle.h:619-633 (host libm)
    const double g = P.gamma;
    P.g_1_inv = 1. / (g - 1.);
    const double g2 = g * g;
    const double gi3 = P.g_1_inv * P.g_1_inv * P.g_1_inv;
    P.g_1_inv7 = gi3 * gi3 * P.g_1_inv;
    P.w_y = 7. / 3. * ((((((g - 9.) * g + 45.) * g - 60. * std::log(g)) * g - 45.) * g + 9.) * g - 1.) * P.g_1_inv7;
    P.f1 = (-10. / 3. + 14. * (g + 1.) - 21. * ((g + 3.) * g + 1.) + 35. / 3. * (((g + 9.) * g + 9.) * g + 1.) -
            70. * ((g + 3.) * g + 1.) * g + 210. * (g + 1.) * g2 + (((g - 7.) * g + 21.) * g - 35.) * g2 * g2) *
           P.g_1_inv7;
    return P;
}

int Engine::load(int n, const long long *id, const double *mass, const double *r_planet, const double *f,
                 const double *pos, const double *vel) {
    int r = ensure(n);
    if (r) return r;
    S.n = n;
    if ((r = h2d(c, S.id, id, n * sizeof(int64_t))) || (r = h2d(c, S.mass, mass, n * sizeof(double))) ||
        (r = h2d(c, S.r_planet, r_planet, n * sizeof(double))) || (r = h2d(c, S.f, f, n * sizeof(double))) ||
        (r = h2d(c, S.pos, pos, 3 * n * sizeof(double))) || (r = h2d(c, S.vel, vel, 3 * n * sizeof(double))))
        return r;
    // start-up reset, src/main_p3t.cpp:291-303
    for (double *p : {S.acc, S.acc_d, S.jerk_d, S.acc_s, S.jerk_s})
        cudaMemsetAsync(p, 0, 3 * (size_t)n * sizeof(double), c->stream);
    for (double *p : {S.phi, S.phi_d, S.phi_s, S.time, S.dt, S.acc0, S.v_disp, S.r_out, S.r_out_inv, S.r_search})
        cudaMemsetAsync(p, 0, (size_t)n * sizeof(double), c->stream);
    for (int32_t *p : {S.number, S.rank, S.n_cluster, S.dead, S.merged, S.nbr_n})
        cudaMemsetAsync(p, 0, (size_t)n * sizeof(int32_t), c->stream);
    { P3T_COUNT_LAUNCH(); k_fill_i32<<<nb(n), 256, 0, c->stream>>>(S.id_max, n, -1); }
    { P3T_COUNT_LAUNCH(); k_fill_i32<<<nb(n), 256, 0, c->stream>>>(S.id_min, n, INT32_MAX_); }
    cudaMemcpyAsync(S.id_cluster, S.id, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, c->stream);
    n_clusters = 0;
    frag_lo = frag_hi = n;
    id_next = 0;
    for (int i = 0; i < n; i++)
        if (i == 0 || id[i] + 1 > id_next) id_next = id[i] + 1;
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int Engine::pack_soft() {
    DevSet &d = c->res;
    int r = 0;
    if ((r = d.ptcl.reserve(S.n)) || (r = d.force.reserve(S.n)) || (r = d.acc64.reserve(S.n)) ||
        (r = d.mass.reserve(S.n)) || (r = d.r_out.reserve(S.n)) || (r = d.r_search.reserve(S.n)))
        return r;
    { P3T_COUNT_LAUNCH(); k_pack_state<<<nb(S.n), 256, 0, c->stream>>>(S, d.ptcl.p); }
    cudaMemcpyAsync(d.mass.p, S.mass, S.n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(d.r_out.p, S.r_out, S.n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(d.r_search.p, S.r_search, S.n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
    c->res_n = S.n;
    return cuda_status(cudaGetLastError());
}

int Engine::correct(int initial) {
    const Params P = params();
    int r = ensure(S.n);
    if (r) return r;
    // the candidate table of a soft pass over this state must exist
    if (!c->res.cand.p || !c->res.force.p || c->res_n != S.n) return ST_BAD_INDEX;
    if ((r = counters.reserve(4)) || (r = pair_n.reserve(S.n)) || (r = pair_base.reserve(S.n))) return r;
    cudaMemsetAsync(counters.p, 0, 4 * sizeof(int32_t), c->stream);
    const int cap = c->cand_cap;
    const ForceRec *F = c->res.force.p;
    const int32_t *cand = c->res.cand.p;
    { P3T_COUNT_LAUNCH(); k_corr_list<false><<<nb(S.n, 128), 128, 0, c->stream>>>(S, F, cand, cap, pair_n.p, nullptr, nullptr, nullptr,
                                                            c->status); }
    int32_t np = 0;
    if ((r = scan(pair_n.p, pair_base.p, S.n, &np))) return r;
    if ((r = pair_i.reserve(np)) || (r = pair_j.reserve(np)) || (r = pair_terms.reserve(np))) return r;
    { P3T_COUNT_LAUNCH(); k_corr_list<true><<<nb(S.n, 128), 128, 0, c->stream>>>(S, F, cand, cap, nullptr, pair_base.p, pair_i.p,
                                                           pair_j.p, c->status); }
    if (np > 0) {
        if (initial)
            { P3T_COUNT_LAUNCH(); k_corr_pairs<true><<<nb(np, 128), 128, 0, c->stream>>>(S, P, np, pair_i.p, pair_j.p, pair_terms.p); }
        else
            { P3T_COUNT_LAUNCH(); k_corr_pairs<false><<<nb(np, 128), 128, 0, c->stream>>>(S, P, np, pair_i.p, pair_j.p, pair_terms.p); }
    }
    if (initial)
        { P3T_COUNT_LAUNCH(); k_correct<true><<<nb(S.n, 128), 128, 0, c->stream>>>(S, P, F, cap, pair_base.p, pair_n.p, pair_j.p,
                                                             pair_terms.p, counters.p, c->status); }
    else
        { P3T_COUNT_LAUNCH(); k_correct<false><<<nb(S.n, 128), 128, 0, c->stream>>>(S, P, F, cap, pair_base.p, pair_n.p, pair_j.p,
                                                              pair_terms.p, counters.p, c->status); }
    if (initial) { P3T_COUNT_LAUNCH(); k_copy3<<<nb(3 * S.n), 256, 0, c->stream>>>(S.acc_d, S.acc_d_new, S.n); }
    return cuda_status(cudaGetLastError());
}

int Engine::cluster() {
    int r = cmin.reserve(S.n);
    if (r) return r;
    { P3T_COUNT_LAUNCH(); k_iota<<<nb(S.n), 256, 0, c->stream>>>(S.label, S.n); }
    { P3T_COUNT_LAUNCH(); k_fill_i64<<<nb(S.n), 256, 0, c->stream>>>(cmin.p, S.n, (int64_t)0x7fffffffffffffffLL); }
    { P3T_COUNT_LAUNCH(); k_union<<<nb(S.n), 256, 0, c->stream>>>(S, c->cand_cap, c->status); }
    { P3T_COUNT_LAUNCH(); k_compress<<<nb(S.n), 256, 0, c->stream>>>(S, cmin.p); }
    { P3T_COUNT_LAUNCH(); k_apply_label<<<nb(S.n), 256, 0, c->stream>>>(S, cmin.p); }
    return cuda_status(cudaGetLastError());
}

int Engine::make_list() {
    const int n = S.n;
    int r = 0;
    if ((r = head.reserve(n)) || (r = flag.reserve(n)) || (r = cidx.reserve(n)) || (r = cl_of.reserve(n)) ||
        (r = cl_cnt.reserve(n + 1)) || (r = cl_off.reserve(n + 1)) || (r = cl_fill.reserve(n + 1)) ||
        (r = members_tmp.reserve(n)) || (r = members.reserve(n)))
        return r;
    { P3T_COUNT_LAUNCH(); k_fill_i32<<<nb(n), 256, 0, c->stream>>>(head.p, n, 0x7fffffff); }
    { P3T_COUNT_LAUNCH(); k_head<<<nb(n), 256, 0, c->stream>>>(S, head.p); }
    { P3T_COUNT_LAUNCH(); k_head_flag<<<nb(n), 256, 0, c->stream>>>(S, head.p, flag.p); }
    int32_t nc = 0;
    if ((r = scan(flag.p, cidx.p, n, &nc))) return r;
    n_clusters = nc;
    cudaMemsetAsync(cl_cnt.p, 0, (nc + 1) * sizeof(int32_t), c->stream);
    cudaMemsetAsync(cl_fill.p, 0, (nc + 1) * sizeof(int32_t), c->stream);
    { P3T_COUNT_LAUNCH(); k_member_count<<<nb(n), 256, 0, c->stream>>>(S, head.p, cidx.p, cl_of.p, cl_cnt.p); }
    int32_t nm = 0;
    if (nc > 0 && (r = scan(cl_cnt.p, cl_off.p, nc, &nm))) return r;
    n_members = nm;
    { P3T_COUNT_LAUNCH(); k_member_fill<<<nb(n), 256, 0, c->stream>>>(S, cl_of.p, cl_off.p, cl_fill.p, members_tmp.p); }
    if (nc > 0) { P3T_COUNT_LAUNCH(); k_member_sort<<<nb(nc * 32), 256, 0, c->stream>>>(nc, cl_off.p, cl_cnt.p, members_tmp.p, members.p); }
    return cuda_status(cudaGetLastError());
}

int Engine::kick() {
    { P3T_COUNT_LAUNCH(); k_kick<<<nb(S.n), 256, 0, c->stream>>>(S, 0.5 * c->params[3]); }
    return cuda_status(cudaGetLastError());
}

int Engine::energy(double *out5) {
    const int blocks = nb(S.n);
    int r = 0;
    if ((r = epart.reserve(4 * (size_t)blocks + 8))) return r;
    { P3T_COUNT_LAUNCH(); k_energy_partial<<<blocks, 256, 0, c->stream>>>(S, epart.p); }
    { P3T_COUNT_LAUNCH(); k_energy_final<<<1, 256, 0, c->stream>>>(epart.p, blocks, epart.p + 4 * blocks); }
    cudaMemcpyAsync(out5, epart.p + 4 * blocks, 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int Engine::cutoff_radii() {
    const Params P = params();
    int r = 0;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int nblk = sms * VD_BLOCKS_PER_SM;
    if ((r = epart.reserve(2 + 2 * NBIN + (size_t)nblk * NBIN)) || (r = icnt.reserve(NBIN + (size_t)nblk * NBIN)))
        return r;
    double *mm = epart.p, *vd = epart.p + 2, *part = epart.p + 2 + 2 * NBIN;
    int *cnt = icnt.p, *cntp = icnt.p + NBIN;
    const double init[2] = {0., 1.7976931348623157e308};
    cudaMemcpyAsync(mm, init, 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    { P3T_COUNT_LAUNCH(); k_rminmax<<<nb(S.n), 256, 0, c->stream>>>(S, mm); }
    double h[2];
    cudaMemcpyAsync(h, mm, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    // src/particle.h:1324-1339 (r_min tracked as max of -r^2)
    const double r_max = std::sqrt(h[0]) * 1.01;
    const double r_min = std::sqrt(h[1]) * 0.99;
    const double dr = (r_max - r_min) / NBIN, drinv = 1. / dr;
    { P3T_COUNT_LAUNCH(); k_vdisp_partial<<<nblk, VD_T, 0, c->stream>>>(S, r_min, drinv, P.m_sun, part, cntp); }
    { P3T_COUNT_LAUNCH(); k_vdisp_bins<<<1, 32 * NBIN, 0, c->stream>>>(part, cntp, nblk, vd, cnt); }
    { P3T_COUNT_LAUNCH(); k_radii<<<nb(S.n), 256, 0, c->stream>>>(S, P, r_min, dr, drinv, vd, cnt); }
    return cuda_status(cudaGetLastError());
}

int Engine::merge(double *edisp) {
    const int n = S.n;
    int r = 0;
    if ((r = keep.reserve(n)) || (r = kpos.reserve(n)) || (r = et.reserve(2 * (size_t)n + 1)) ||
        (r = tflag.reserve(n)) || (r = tpos.reserve(n)))
        return r;
    { P3T_COUNT_LAUNCH(); k_fill_i32<<<nb(n), 256, 0, c->stream>>>(keep.p, n, 1); }
    { P3T_COUNT_LAUNCH(); k_merge_targets<<<nb(n), 256, 0, c->stream>>>(S, cl_of.p, cl_off.p, cl_cnt.p, members.p, keep.p, et.p,
                                                    tflag.p, frag_lo, frag_hi, frag_cl.p); }
    int32_t nt = 0;
    if ((r = scan(tflag.p, tpos.p, n, &nt))) return r;
    double *tl = et.p + n;
    { P3T_COUNT_LAUNCH(); k_gather_targets<<<nb(n), 256, 0, c->stream>>>(et.p, tflag.p, tpos.p, n, tl); }
    { P3T_COUNT_LAUNCH(); k_sum_ordered<<<1, 32, 0, c->stream>>>(tl, nt, et.p + 2 * (size_t)n); }
    double e = 0.;
    cudaMemcpyAsync(&e, et.p + 2 * (size_t)n, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    int32_t nk = 0;
    if ((r = scan(keep.p, kpos.p, n, &nk))) return r;  // synchronizes
    *edisp = e;
    frag_lo = frag_hi = n;
    if (nk == n) return 0;
    return compact(n, nk);
}

// order-preserving compaction of every field to the bodies with keep = 1
// (kpos: their new positions, nk: how many)
int Engine::compact(int n, int nk) {
    int r = 0;
    CompactSet C{};
    long long words = 0;
    auto add = [&](void *p, int w) {
        C.p[C.nf] = (uint32_t *)p;
        C.words[C.nf] = w;
        C.off[C.nf] = words;
        words += (long long)n * w;
        C.nf++;
    };
    for (double *f : {S.mass, S.r_planet, S.f, S.phi, S.phi_d, S.phi_s, S.r_out, S.r_out_inv, S.r_search, S.v_disp,
                      S.time, S.dt, S.acc0})
        add(f, 2);
    for (double *f : {S.pos, S.vel, S.acc, S.acc_d, S.jerk_d, S.acc_s, S.jerk_s}) add(f, 6);
    for (int64_t *f : {S.id, S.id_cluster}) add(f, 2);
    for (int32_t *f : {S.number, S.rank, S.id_max, S.id_min, S.n_cluster, S.dead, S.merged}) add(f, 1);
    if ((r = compact_tmp.reserve((size_t)words * sizeof(uint32_t)))) return r;
    uint32_t *tmp = (uint32_t *)compact_tmp.p;
    { P3T_COUNT_LAUNCH(); k_compact_gather<<<nb(n), 256, 0, c->stream>>>(C, keep.p, kpos.p, n, tmp); }
    if (nk > 0) { P3T_COUNT_LAUNCH(); k_compact_back<<<dim3(std::max(1, std::min(nb(nk), 1024)), C.nf), 256, 0, c->stream>>>(C, nk, tmp); }
    if ((r = cuda_status(cudaGetLastError()))) return r;
    S.n = nk;
    n_clusters = 0;
    frag_lo = frag_hi = nk;
    return cuda_status(cudaStreamSynchronize(c->stream));
}

// removeParticlesOutOfBoundary, src/func.h:209-355
__global__ void k_remove_flag(State S, double rmax2, double rmin2, int32_t *keep, int32_t *gone) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= S.n) return;
    const V3 x = ld3(S.pos, i);
    const double pos2 = dot(x, x);
    const int out = (pos2 > rmax2 || pos2 < rmin2) ? 1 : 0;
    keep[i] = 1 - out;
    gone[i] = out;
}
__global__ void k_remove_list(const int32_t *gone, const int32_t *gpos, int n, int32_t *list) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && gone[i]) list[gpos[i]] = i;
}
// the energy the removed bodies take with them, in list (index) order
__global__ void k_remove_energy(State S, Params P, const int32_t *list, int nr, double *out) {
    if (threadIdx.x || blockIdx.x) return;
    double e = 0.;
    for (int a = 0; a < nr; a++) {
        const int i = list[a];
        const double massi = S.mass[i];
        const V3 veli = ld3(S.vel, i);
        e -= dot(0.5 * massi * veli, veli);
        e -= massi * S.phi_s[i];
        e -= massi * S.phi_d[i];
        e -= massi * S.phi[i];
        for (int b = 0; b < a; b++) {
            const int j = list[b];
            if (S.id[i] != S.id[j]) {
                const V3 dr = ld3(S.pos, i) - ld3(S.pos, j);
                const double rinv = 1. / sqrt(dot(dr, dr) + P.eps2);
                e += -massi * S.mass[j] * rinv;
            }
        }
    }
    *out = e;
}

int Engine::remove(double r_max, double r_min, double *edisp, int *n_removed) {
    const int n = S.n;
    int r = 0;
    if ((r = keep.reserve(n)) || (r = kpos.reserve(n)) || (r = tflag.reserve(n)) || (r = tpos.reserve(n)) ||
        (r = et.reserve(2)))
        return r;
    { P3T_COUNT_LAUNCH(); k_remove_flag<<<nb(n), 256, 0, c->stream>>>(S, r_max * r_max, r_min * r_min, keep.p, tflag.p); }
    int32_t nr = 0;
    if ((r = scan(tflag.p, tpos.p, n, &nr))) return r;
    *n_removed = nr;
    *edisp = 0.;
    if (nr == 0) return 0;
    if ((r = members_tmp.reserve(std::max(n, nr)))) return r;
    { P3T_COUNT_LAUNCH(); k_remove_list<<<nb(n), 256, 0, c->stream>>>(tflag.p, tpos.p, n, members_tmp.p); }
    { P3T_COUNT_LAUNCH(); k_remove_energy<<<1, 32, 0, c->stream>>>(S, params(), members_tmp.p, nr, et.p); }
    if ((r = d2h(c, edisp, et.p, sizeof(double)))) return r;
    int32_t nk = 0;
    if ((r = scan(keep.p, kpos.p, n, &nk))) return r;
    return compact(n, nk);
}

}  // namespace p3t

using namespace p3t;

extern "C" {

// Device-to-device copy of every state field (and the cluster lists) into a
// backup, and back: lets a caller time or retry a phase on the same state.
static State g_backup;
static int g_backup_n = -1;
int p3t_state_snapshot(int restore) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    State &S = E.S;
    if (!restore) {
        if (g_backup.cap < S.cap) {
            // allocate the backup with the state's capacity
            State b;
            b.cap = S.cap;
            auto al = [&](auto **p, size_t n) -> int {
                return cuda_status(cudaMalloc((void **)p, std::max<size_t>(n, 1) * sizeof(**p)));
            };
            int r = 0;
            for (double **f : {&b.mass, &b.r_planet, &b.f, &b.phi, &b.phi_d, &b.phi_s, &b.r_out, &b.r_out_inv,
                               &b.r_search, &b.v_disp, &b.time, &b.dt, &b.acc0})
                if ((r = al(f, S.cap))) return r;
            for (double **f : {&b.pos, &b.vel, &b.acc, &b.acc_d, &b.jerk_d, &b.acc_s, &b.jerk_s})
                if ((r = al(f, 3 * (size_t)S.cap))) return r;
            for (int64_t **f : {&b.id, &b.id_cluster})
                if ((r = al(f, S.cap))) return r;
            for (int32_t **f : {&b.number, &b.rank, &b.id_max, &b.id_min, &b.n_cluster, &b.dead, &b.merged})
                if ((r = al(f, S.cap))) return r;
            g_backup = b;
        }
        g_backup_n = S.n;
    } else if (g_backup_n != S.n) {
        return ST_BAD_INDEX;
    }
    State &src = restore ? g_backup : S;
    State &dst = restore ? S : g_backup;
    const size_t n = S.n;
    cudaStream_t st = E.c->stream;
    auto cp = [&](void *d, const void *s2, size_t b) { cudaMemcpyAsync(d, s2, b, cudaMemcpyDeviceToDevice, st); };
    cp(dst.mass, src.mass, n * 8); cp(dst.r_planet, src.r_planet, n * 8); cp(dst.f, src.f, n * 8);
    cp(dst.phi, src.phi, n * 8); cp(dst.phi_d, src.phi_d, n * 8); cp(dst.phi_s, src.phi_s, n * 8);
    cp(dst.r_out, src.r_out, n * 8); cp(dst.r_out_inv, src.r_out_inv, n * 8); cp(dst.r_search, src.r_search, n * 8);
    cp(dst.v_disp, src.v_disp, n * 8); cp(dst.time, src.time, n * 8); cp(dst.dt, src.dt, n * 8);
    cp(dst.acc0, src.acc0, n * 8);
    cp(dst.pos, src.pos, n * 24); cp(dst.vel, src.vel, n * 24); cp(dst.acc, src.acc, n * 24);
    cp(dst.acc_d, src.acc_d, n * 24); cp(dst.jerk_d, src.jerk_d, n * 24); cp(dst.acc_s, src.acc_s, n * 24);
    cp(dst.jerk_s, src.jerk_s, n * 24);
    cp(dst.id, src.id, n * 8); cp(dst.id_cluster, src.id_cluster, n * 8);
    cp(dst.number, src.number, n * 4); cp(dst.rank, src.rank, n * 4); cp(dst.id_max, src.id_max, n * 4);
    cp(dst.id_min, src.id_min, n * 4); cp(dst.n_cluster, src.n_cluster, n * 4); cp(dst.dead, src.dead, n * 4);
    cp(dst.merged, src.merged, n * 4);
    return cuda_status(cudaStreamSynchronize(st));
}

int p3t_state_load(int n, const long long *id, const double *mass, const double *r_planet, const double *f,
                   const double *pos, const double *vel) {
    if (n < 0) return ST_BAD_INDEX;
    return g_eng.load(n, id, mass, r_planet, f, pos, vel);
}

int p3t_state_n(void) { return g_eng.S.n; }

// field codes: see include/gplum_p3t.h
static void *field_ptr(int field, int *width, int *kind) {
    State &S = g_eng.S;
    *width = 1;
    *kind = 0;  // 0 double, 1 int64, 2 int32
    switch (field) {
        case 0: *width = 3; return S.pos;
        case 1: *width = 3; return S.vel;
        case 2: *width = 3; return S.acc;
        case 3: *width = 3; return S.acc_d;
        case 4: *width = 3; return S.jerk_d;
        case 5: *width = 3; return S.acc_s;
        case 6: *width = 3; return S.jerk_s;
        case 10: return S.phi;
        case 11: return S.phi_d;
        case 12: return S.phi_s;
        case 13: return S.mass;
        case 14: return S.r_out;
        case 15: return S.r_search;
        case 16: return S.dt;
        case 17: return S.acc0;
        case 18: return S.time;
        case 19: return S.r_planet;
        case 20: return S.v_disp;
        case 21: return S.r_out_inv;
        case 22: return S.f;
        case 100: *kind = 1; return S.id;
        case 101: *kind = 1; return S.id_cluster;
        case 102: *kind = 2; return S.number;
        case 103: *kind = 2; return S.n_cluster;
        case 104: *kind = 2; return S.dead;
        case 105: *kind = 2; return S.merged;
        case 106: *kind = 2; return S.rank;
        case 107: *kind = 2; return S.id_min;
        case 108: *kind = 2; return S.id_max;
        default: return nullptr;
    }
}
static size_t kind_size(int kind) { return kind == 0 ? 8 : (kind == 1 ? 8 : 4); }

int p3t_state_get(int field, void *out) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    int w, kind;
    void *p = field_ptr(field, &w, &kind);
    if (!p) return ST_BAD_INDEX;
    const size_t b = (size_t)g_eng.S.n * w * kind_size(kind);
    int r = cuda_status(cudaMemcpyAsync(out, p, b, cudaMemcpyDeviceToHost, c->stream));
    if (r) return r;
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int p3t_state_set(int field, const void *in) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    int w, kind;
    void *p = field_ptr(field, &w, &kind);
    if (!p) return ST_BAD_INDEX;
    return h2d(c, p, in, (size_t)g_eng.S.n * w * kind_size(kind));
}

int p3t_set_cutoff_radii(void) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    return g_eng.cutoff_radii();
}

int p3t_set_r_planet(void) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    // FPGrav::setRPlanet, src/particle.h:757-759 (host: one pow per body)
    const int n = g_eng.S.n;
    std::vector<double> m(n), rp(n);
    int r = d2h(g_eng.c, m.data(), g_eng.S.mass, n * sizeof(double));
    if (r) return r;
    for (int i = 0; i < n; i++) rp[i] = std::pow(0.75 * m[i] / (3.14159265358979323846 * c->params[20]), 1. / 3.);
    return h2d(c, g_eng.S.r_planet, rp.data(), n * sizeof(double));
}

int p3t_state_soft(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                   const int *s_off, const int *s_idx, const void *spj, int n_spj) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    int r = g_eng.pack_soft();
    if (r) return r;
    if ((r = p3t_upload_lists(n_group, i_off, i_idx, j_off, j_idx, s_off, s_idx, spj, n_spj))) return r;
    return soft_run_state();
}

int p3t_correct(int initial) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    int r = g_eng.correct(initial);
    if (r) return r;
    return read_status(g_eng.c);
}

int p3t_correct_and_search(int initial) { return p3t_correct(initial); }

int p3t_remove_out_of_boundary(double r_max, double r_min, double *edisp) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    int nr = 0;
    int r = g_eng.remove(r_max, r_min, edisp, &nr);
    if (r > 0) return P3T_COUNT_STATUS(r);
    return r ? r : nr;
}

int p3t_neighbor_counts(int *ngb_tot, int *with_ngb) {
    Context *c = ctx_get(0);
    if (!c || !g_eng.counters.p) return -(int)cudaErrorNoDevice;
    int h[2];
    int r = d2h(g_eng.c, h, g_eng.counters.p, 2 * sizeof(int));
    *ngb_tot = h[0];
    *with_ngb = h[1];
    return r;
}

int p3t_neighbor_list(int i, int *out, int cap) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    if (i < 0 || i >= g_eng.S.n) return -1;
    int m = 0;
    d2h(g_eng.c, &m, g_eng.S.nbr_n + i, sizeof(int));
    m = std::min(m, cap);
    if (m > 0) d2h(g_eng.c, out, g_eng.S.nbr + (size_t)i * c->cand_cap, m * sizeof(int));
    return m;
}

int p3t_neighbor_pairs(int *out, long long cap) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    if (cap < 0 || (cap > 0 && !out)) return -(int)cudaErrorInvalidValue;
    const int n = E.S.n;
    int r = 0;
    if ((r = E.tflag.reserve(n)) || (r = E.tpos.reserve(n))) return r;
    { P3T_COUNT_LAUNCH(); k_pair_count<<<nb(n), 256, 0, E.c->stream>>>(E.S, E.c->cand_cap, E.tflag.p); }
    int32_t np = 0;
    if ((r = E.scan(E.tflag.p, E.tpos.p, n, &np))) return r;
    if (cap >= np && np > 0) {
        if ((r = E.members_tmp.reserve(2 * (size_t)np))) return r;
        { P3T_COUNT_LAUNCH(); k_pair_fill<<<nb(n), 256, 0, E.c->stream>>>(E.S, E.c->cand_cap, E.tpos.p, E.members_tmp.p); }
        if ((r = cuda_status(cudaGetLastError())) ||
            (r = d2h(E.c, out, E.members_tmp.p, 2 * (size_t)np * sizeof(int32_t))))
            return r;
    }
    return np;
}

int p3t_cluster_label(void) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    int r = g_eng.cluster();
    if (r) return r;
    if ((r = g_eng.make_list())) return r;
    return read_status(g_eng.c);
}

int p3t_cluster_lists(int *n_clusters, int *off, int *members) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    *n_clusters = g_eng.n_clusters;
    if (off) {
        d2h(g_eng.c, off, g_eng.cl_off.p, g_eng.n_clusters * sizeof(int));
        off[g_eng.n_clusters] = g_eng.n_members;
    }
    if (members && g_eng.n_members)
        d2h(g_eng.c, members, g_eng.members.p, g_eng.n_members * sizeof(int));
    return cuda_status(cudaGetLastError());
}

int p3t_kick(void) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    return g_eng.kick();
}

int p3t_energy(double *out5) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    return g_eng.energy(out5);
}

int p3t_merge(double *edisp) {
    if (!g_eng.c) return -(int)cudaErrorNoDevice;
    return g_eng.merge(edisp);
}

}  // extern "C"
