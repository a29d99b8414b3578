// Device octree and interaction lists for the soft force.
//
// The caller side of the soft-force path, on the device: the contract of the
// host builder (csrc/tree.cpp, include/p3t_tree.h; in GPLUM, FDPS's
// TreeForForce with LONG_SYMMETRY search and quadrupole moments, called at
// src/main_p3t.cpp:344-355,581-587,672-676):
//   * 63-bit Morton keys on the root cube (side = 1.0001 x the largest
//     extent, anchored at the bodies' lower corner with margin
//     (side - extent)/2 on every axis), bodies in key order (ties by index);
//   * a node splits into one child per occupied octant while it holds more
//     than min(n_leaf_limit, n_group_limit) bodies (21 levels at most);
//   * i-groups are the highest nodes with at most n_group_limit bodies (or
//     leaves), in Morton order;
//   * a cell is opened when its search box (bodies +- 1.1 r_search) overlaps
//     the group's body box, or the group's search box overlaps the cell's
//     body box, or size^2 > theta^2 d^2 (d: cell centre of mass to the
//     group's body box); opened leaves give EPJ entries, unopened cells SPJ
//     entries (quadrupole about the centre of mass).
// Steps: bounding box (two-stage reduction); keys; a stable LSD radix sort of
// (key, index) in 8 passes of 8 bits; the tree one level at a time (a scan of
// "a new 3-bit digit starts here" over the sorted keys gives the children,
// contiguous, in level order); moments and boxes bottom-up (leaves sum their
// bodies in key order, as the host builder; inner nodes combine children by
// the parallel-axis rule); groups; and the walks, split into (group, node of
// the upper three levels) tasks taken in pre-order, each walking its subtree
// with the host builder's stack discipline (count, then fill), so the
// concatenated lists equal the host builder's entry for entry (SPJ entries
// name the same cells; node numbers are in level order here).  By default the
// walk is breadth first instead, one CTA per group over an order-keeping
// frontier (k_walk_bfs), giving the same lists; the task walk is its
// fallback.  The lists go straight into the resident soft-force buffers.  Compiled with -fmad=false so the box and
// opening arithmetic rounds as the host builder's (-ffp-contract=off).
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_engine.cuh"

namespace p3t {

struct TNode {
    double ilo[3], ihi[3], olo[3], ohi[3];  // body box, search box (bodies +- 1.1 r_search)
    double com[3], size;
    int first, count, child0, nchild;
};

// FP32 copy of the walk's fields (rounded to nearest), for the ternary
// opening test below
struct TNodeF {
    float ilo[3], ihi[3], olo[3], ohi[3], com[3], size;
    int first, count, child0, nchild;
};

constexpr int RADIX_TILE = 4096;  // keys per radix block (256 threads x 16)
constexpr int WALK_STACK = 256;

// ---- bounding box and keys ------------------------------------------------------
__global__ void k_bbox_partial(const double *pos, int n, double *part) {
    __shared__ double s[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int d = 0; d < 3; d++) {
            lo[d] = fmin(lo[d], pos[3 * i + d]);
            hi[d] = fmax(hi[d], pos[3 * i + d]);
        }
    for (int d = 0; d < 3; d++) {
        s[d][threadIdx.x] = lo[d];
        s[3 + d][threadIdx.x] = hi[d];
    }
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int d = 0; d < 3; d++) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + o]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

// root cube as the host builder: out = {base.xyz, size, scale} (one block of
// 256); anchored at the lower corner, so a thin axis is not cut at coarse levels
__global__ void k_bbox_root(const double *part, int nblk, double *out) {
    __shared__ double s[6][256];
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int b = threadIdx.x; b < nblk; b += 256)
        for (int d = 0; d < 3; d++) {
            lo[d] = fmin(lo[d], part[6 * b + d]);
            hi[d] = fmax(hi[d], part[6 * b + 3 + d]);
        }
    for (int d = 0; d < 3; d++) {
        s[d][threadIdx.x] = lo[d];
        s[3 + d][threadIdx.x] = hi[d];
    }
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int d = 0; d < 3; d++) {
                s[d][threadIdx.x] = fmin(s[d][threadIdx.x], s[d][threadIdx.x + o]);
                s[3 + d][threadIdx.x] = fmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + o]);
            }
        __syncthreads();
    }
    if (threadIdx.x) return;
    double ext = 0.;
    for (int d = 0; d < 3; d++) ext = fmax(ext, s[3 + d][0] - s[d][0]);
    const double size = ext * 1.0001 + 1e-300;
    for (int d = 0; d < 3; d++) out[d] = s[d][0] - 0.5 * (size - ext);
    out[3] = size;
    out[4] = double(1 << 21) / size;
}

__device__ __forceinline__ unsigned long long spread21(unsigned long long v) {
    v &= 0x1fffffULL;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

__global__ void k_keys(const double *pos, int n, const double *root, unsigned long long *key, int *idx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned long long c[3];
    for (int d = 0; d < 3; d++) {
        const double u = (pos[3 * i + d] - root[d]) * root[4];
        long long v = (long long)u;
        v = v < 0 ? 0 : (v > (1 << 21) - 1 ? (1 << 21) - 1 : v);
        c[d] = (unsigned long long)v;
    }
    key[i] = (spread21(c[0]) << 2) | (spread21(c[1]) << 1) | spread21(c[2]);
    idx[i] = i;
}

// ---- stable LSD radix sort of (key, index) -----------------------------------------
__global__ void __launch_bounds__(256) k_radix_hist(const unsigned long long *key, int n, int shift, int nblk,
                                                    int *hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * RADIX_TILE;
    for (int j = threadIdx.x; j < RADIX_TILE; j += 256) {
        const int k = base + j;
        if (k < n) atomicAdd(&h[(key[k] >> shift) & 255], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];  // digit-major
}

// scatter of one tile in 16 rounds of 256 keys; within a round, keys with the
// same digit keep their order (warp match + per-warp counts)
__global__ void __launch_bounds__(256) k_radix_scatter(const unsigned long long *key, const int *idx, int n,
                                                       int shift, int nblk, const int *offs,
                                                       unsigned long long *key_out, int *idx_out) {
    __shared__ int cnt[8][256];
    __shared__ int run[256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int j = 0; j < 8; j++) cnt[j][tid] = 0;
    run[tid] = offs[tid * nblk + blockIdx.x];
    __syncthreads();
    const int base = blockIdx.x * RADIX_TILE;
    for (int r = 0; r < RADIX_TILE / 256; r++) {
        const int k = base + r * 256 + tid;
        const bool valid = k < n;
        unsigned long long kv = 0;
        int iv = 0, d = 256;
        if (valid) {
            kv = key[k];
            iv = idx[k];
            d = (int)((kv >> shift) & 255);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) cnt[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int off = run[d] + rank;
            for (int ww = 0; ww < w; ww++) off += cnt[ww][d];
            key_out[off] = kv;
            idx_out[off] = iv;
        }
        __syncthreads();
        int add = 0;
        for (int ww = 0; ww < 8; ww++) {
            add += cnt[ww][tid];
            cnt[ww][tid] = 0;
        }
        run[tid] += add;
        __syncthreads();
    }
}

// ---- tree, one level at a time -------------------------------------------------------
__global__ void k_root_node(TNode *nd, int *parent, const double *root, int n, int limit, int *enode) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k == 0) {
        nd[0].first = 0;
        nd[0].count = n;
        nd[0].child0 = -1;
        nd[0].nchild = 0;
        nd[0].size = root[3];
        parent[0] = -1;
    }
    if (k < n) enode[k] = (n > limit) ? 0 : -1;
}

__global__ void k_lvl_heads(const unsigned long long *key, const int *enode, const TNode *nd, int n, int shift,
                            int *head) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int p = enode[k];
    int h = 0;
    if (p >= 0) h = (k == nd[p].first) || (((key[k] >> shift) & 7ULL) != ((key[k - 1] >> shift) & 7ULL));
    head[k] = h;
}

__global__ void k_lvl_make(const int *enode, const int *head, const int *hs, int n, int base, TNode *nd,
                           int *parent, int *enode_next) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int p = enode[k];
    if (p < 0) {
        enode_next[k] = -1;
        return;
    }
    const int c = base + hs[k] + head[k] - 1;
    enode_next[k] = c;
    if (head[k]) {
        nd[c].first = k;
        nd[c].size = nd[p].size * 0.5;
        nd[c].child0 = -1;
        nd[c].nchild = 0;
        parent[c] = p;
        if (k == nd[p].first) nd[p].child0 = c;
    }
}

__global__ void k_lvl_count(int base, int m, TNode *nd, const int *parent) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const int c = base + t, p = parent[c];
    const int end = (t + 1 < m && parent[c + 1] == p) ? nd[c + 1].first : nd[p].first + nd[p].count;
    nd[c].count = end - nd[c].first;
    if (nd[p].child0 == c) {
        int j = 1;
        while (t + j < m && parent[c + j] == p && j < 8) j++;
        nd[p].nchild = j;
    }
}

__global__ void k_lvl_split(int n, int level, int limit, const TNode *nd, int *enode) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int c = enode[k];
    if (c >= 0 && !(nd[c].count > limit && level < 21)) enode[k] = -1;
}

// ---- moments and boxes, bottom-up -------------------------------------------------------
constexpr int LEAF_B = 8;  // bodies of a leaf loaded at once (leaves hold at most n_leaf_limit = 8)
// Node c's moments and boxes: a leaf sums its bodies in key order (the host
// builder's sums), an inner node combines its children in child order by the
// parallel-axis rule.  Children are read through L2 (ld.cg): they may have
// been written by other CTAs of the same launch.
__device__ void node_moments(int c, TNode *nd, SPJRec *spj, const int *order, const double *pos, const double *mass,
                             const double *rs) {
    TNode &N = nd[c];
    const int nchild = __ldcg(&N.nchild), child0 = __ldcg(&N.child0);
    double m = 0., cx = 0., cy = 0., cz = 0., q[6] = {0., 0., 0., 0., 0., 0.};
    double ilo[3] = {1e300, 1e300, 1e300}, ihi[3] = {-1e300, -1e300, -1e300};
    double olo[3] = {1e300, 1e300, 1e300}, ohi[3] = {-1e300, -1e300, -1e300};
    if (nchild == 0) {
        const int first = N.first, count = N.count;
        // in blocks of LEAF_B bodies, every load of a block issued before its
        // sums (the sums stay in key order)
        for (int k0 = first; k0 < first + count; k0 += LEAF_B) {
            int pb[LEAF_B];
#pragma unroll
            for (int u = 0; u < LEAF_B; u++) pb[u] = (k0 + u < first + count) ? order[k0 + u] : -1;
#pragma unroll
            for (int u = 0; u < LEAF_B; u++) {
                const int p = pb[u];
                if (p < 0) break;
                const double x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2], mp = mass[p];
                m += mp;
                cx += mp * x;
                cy += mp * y;
                cz += mp * z;
                const double r = 1.1 * rs[p];
                const double v[3] = {x, y, z};
                for (int d = 0; d < 3; d++) {
                    ilo[d] = fmin(ilo[d], v[d] - 0.);
                    ihi[d] = fmax(ihi[d], v[d] + 0.);
                    olo[d] = fmin(olo[d], v[d] - r);
                    ohi[d] = fmax(ohi[d], v[d] + r);
                }
            }
        }
        if (m != 0.) {
            cx /= m;
            cy /= m;
            cz /= m;
        }
        for (int k0 = first; k0 < first + count; k0 += LEAF_B) {
            int pb[LEAF_B];
#pragma unroll
            for (int u = 0; u < LEAF_B; u++) pb[u] = (k0 + u < first + count) ? order[k0 + u] : -1;
#pragma unroll
            for (int u = 0; u < LEAF_B; u++) {
                const int p = pb[u];
                if (p < 0) break;
                const double dx = pos[3 * p] - cx, dy = pos[3 * p + 1] - cy, dz = pos[3 * p + 2] - cz, mp = mass[p];
                q[0] += mp * dx * dx; q[1] += mp * dy * dy; q[2] += mp * dz * dz;
                q[3] += mp * dx * dy; q[4] += mp * dx * dz; q[5] += mp * dy * dz;
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (j >= nchild) break;
            const int ch = child0 + j;
            const double mc = __ldcg(&spj[ch].mass);
            m += mc;
            cx += mc * __ldcg(&spj[ch].pos[0]);
            cy += mc * __ldcg(&spj[ch].pos[1]);
            cz += mc * __ldcg(&spj[ch].pos[2]);
            for (int d = 0; d < 3; d++) {
                ilo[d] = fmin(ilo[d], __ldcg(&nd[ch].ilo[d]));
                ihi[d] = fmax(ihi[d], __ldcg(&nd[ch].ihi[d]));
                olo[d] = fmin(olo[d], __ldcg(&nd[ch].olo[d]));
                ohi[d] = fmax(ohi[d], __ldcg(&nd[ch].ohi[d]));
            }
        }
        if (m != 0.) {
            cx /= m;
            cy /= m;
            cz /= m;
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (j >= nchild) break;
            const SPJRec *S = spj + child0 + j;
            const double mc = __ldcg(&S->mass);
            const double dx = __ldcg(&S->pos[0]) - cx, dy = __ldcg(&S->pos[1]) - cy, dz = __ldcg(&S->pos[2]) - cz;
            q[0] += __ldcg(&S->xx) + mc * dx * dx; q[1] += __ldcg(&S->yy) + mc * dy * dy;
            q[2] += __ldcg(&S->zz) + mc * dz * dz;
            q[3] += __ldcg(&S->xy) + mc * dx * dy; q[4] += __ldcg(&S->xz) + mc * dx * dz;
            q[5] += __ldcg(&S->yz) + mc * dy * dz;
        }
    }
    for (int d = 0; d < 3; d++) {
        N.ilo[d] = ilo[d];
        N.ihi[d] = ihi[d];
        N.olo[d] = olo[d];
        N.ohi[d] = ohi[d];
    }
    N.com[0] = cx;
    N.com[1] = cy;
    N.com[2] = cz;
    SPJRec &S = spj[c];
    S.mass = m;
    S.pos[0] = cx;
    S.pos[1] = cy;
    S.pos[2] = cz;
    S.xx = q[0]; S.yy = q[1]; S.zz = q[2]; S.xy = q[3]; S.xz = q[4]; S.yz = q[5];
}

// one level (nodes lo..hi-1) per launch, deepest level first
__global__ void k_moments(int lo, int hi, TNode *nd, SPJRec *spj, const int *order, const double *pos,
                          const double *mass, const double *rs) {
    const int c = lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= hi) return;
    node_moments(c, nd, spj, order, pos, mass, rs);
}

// Moments in lane-dense launches: every leaf at once from a compacted list
// (their body sums are the bulk of the FP64 work), then the inner nodes one
// level at a time, deepest first.  A launch over all nodes of a level, or one
// climbing thread per finished child, left most lanes of the FP64 pipe's warp
// instructions idle (ncu: 23 % lane efficiency for the climbing form).
__global__ void k_leaf_flag(int nn, const TNode *nd, int *flag) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nn) flag[c] = nd[c].nchild == 0;
}
// leaves to the front of `list` (ascending), inner nodes to the back in
// ascending node order (so each level's inner nodes are one run; inner node c
// sits at nn - 1 - (c - pos[c]) counted from the back); count = leaves
__global__ void k_leaf_list(int nn, const int *flag, const int *pos, int *list, int *count) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nn) return;
    if (flag[c]) list[pos[c]] = c;
    else list[nn - 1 - (c - pos[c])] = c;
    if (c == nn - 1) *count = pos[c] + flag[c];
}
__global__ void k_moments_leaves(const int *list, const int *count, TNode *nd, SPJRec *spj, const int *order,
                                 const double *pos, const double *mass, const double *rs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= *count) return;
    node_moments(list[t], nd, spj, order, pos, mass, rs);
}
// the inner nodes of level [lo, hi): their run in the back of `list` (from
// the leaf-position scan: inner nodes below c number c - lpos[c])
__global__ void k_moments_inner(int lo, int hi, int nn, const int *list, const int *lpos, const int *flag, TNode *nd,
                                SPJRec *spj, const int *order, const double *pos, const double *mass, const double *rs) {
    const int a = lo - lpos[lo];                                 // inner nodes before the level
    const int b = (hi < nn) ? hi - lpos[hi] : nn - (lpos[nn - 1] + flag[nn - 1]);  // ... and up to its end
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (a + t >= b) return;
    node_moments(list[nn - 1 - (a + t)], nd, spj, order, pos, mass, rs);
}

// ---- groups ---------------------------------------------------------------------------------
__global__ void k_group_mark(int nn, const TNode *nd, const int *parent, int ngl, int *gmark) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nn) return;
    const TNode &N = nd[c];
    const bool cand = N.count <= ngl || N.nchild == 0;
    const bool top = (c == 0) || nd[parent[c]].count > ngl;
    if (cand && top) gmark[N.first] = c + 1;
}

__global__ void k_group_flag(const int *gmark, int n, int *flag) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) flag[k] = gmark[k] > 0;
}

__global__ void k_group_fill(const int *gmark, const int *gpos, int n, int ng, int *gnode, int *i_off) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n && gmark[k] > 0) {
        gnode[gpos[k]] = gmark[k] - 1;
        i_off[gpos[k]] = k;
    }
    if (k == 0) i_off[ng] = n;
}

// ---- walk --------------------------------------------------------------------------------------
__device__ __forceinline__ bool box_overlap(const double *alo, const double *ahi, const double *blo,
                                            const double *bhi) {
    for (int d = 0; d < 3; d++)
        if (ahi[d] < blo[d] || bhi[d] < alo[d]) return false;
    return true;
}

__device__ __forceinline__ double box_dist2(const double *lo, const double *hi, const double *x) {
    double s = 0.;
    for (int d = 0; d < 3; d++) {
        double e = 0.;
        if (x[d] < lo[d]) e = lo[d] - x[d];
        else if (x[d] > hi[d]) e = x[d] - hi[d];
        s += e * e;
    }
    return s;
}

// The walk split into tasks: pair (group g, top node t) for each of the
// ntop nodes of the upper `depth` levels, taken in the tree's pre-order.  The
// open test of every pair goes first (k_walk_open); then a pair is reached
// when all its top-node ancestors are open for g, and it contributes: an SPJ
// entry (reached, not open), its bodies (reached, open leaf), nothing
// (reached, open, above the split depth: its children are pairs of their
// own), or the depth-first walk of its subtree (reached, open, at the split
// depth).  Pairs in (group, pre-order) order concatenate to the single walk's
// output, entry for entry.
__device__ __forceinline__ bool cell_open(const TNode &C, const double *gilo, const double *gihi,
                                          const double *golo, const double *gohi, double theta2) {
    const bool near = box_overlap(C.olo, C.ohi, gilo, gihi) || box_overlap(golo, gohi, C.ilo, C.ihi);
    return near || (C.size * C.size > theta2 * box_dist2(gilo, gihi, C.com));
}

__global__ void k_node_f32(const TNode *nd, int nn, TNodeF *nf) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nn) return;
    const TNode &N = nd[c];
    TNodeF F;
    for (int d = 0; d < 3; d++) {
        F.ilo[d] = (float)N.ilo[d];
        F.ihi[d] = (float)N.ihi[d];
        F.olo[d] = (float)N.olo[d];
        F.ohi[d] = (float)N.ohi[d];
        F.com[d] = (float)N.com[d];
    }
    F.size = (float)N.size;
    F.first = N.first;
    F.count = N.count;
    F.child0 = N.child0;
    F.nchild = N.nchild;
    nf[c] = F;
}

// Ternary comparisons on FP32 copies of doubles (each within 2^-24 relative
// of its double): +1 when a < b certainly holds for the doubles, -1 when
// a >= b certainly holds, 0 when the copies cannot tell.  b - a differs from
// the FP32 difference of the copies by less than 1.8e-7 (|a| + |b|) (two
// conversions and one rounded subtraction); the margin is 2.5e-7.
__device__ __forceinline__ int lt3(float a, float b) {
    const float d = b - a, e = 2.5e-7f * (fabsf(a) + fabsf(b)) + 1e-30f;
    return d > e ? 1 : (d < -e ? -1 : 0);
}
// box overlap (no dimension separated): +1 yes, -1 no, 0 unknown
__device__ __forceinline__ int overlap3(const float *alo, const float *ahi, const float *blo, const float *bhi) {
    int res = 1;
    for (int d = 0; d < 3; d++) {
        const int s1 = lt3(ahi[d], blo[d]), s2 = lt3(bhi[d], alo[d]);
        if (s1 == 1 || s2 == 1) return -1;  // separated for sure
        if (s1 == 0 || s2 == 0) res = 0;
    }
    return res;
}
// The cell test of the host builder on the FP32 copies: +1 open, -1 closed,
// 0 unknown.  The distance from the group box carries an absolute error
// below E_d = 2.5e-7 (|x| + |lo or hi|) per dimension, so d^2 is within
// B = sum(2 |e_d| E_d + E_d^2) + 4e-7 d^2; sizes and theta^2 carry 2e-7
// relative, covered by the 4e-7 factors.
__device__ __forceinline__ int open3(const TNodeF &C, const float *gilo, const float *gihi, const float *golo,
                                     const float *gohi, float theta2) {
    const int a = overlap3(C.olo, C.ohi, gilo, gihi);
    if (a == 1) return 1;
    const int b = overlap3(golo, gohi, C.ilo, C.ihi);
    if (b == 1) return 1;
    if (a == 0 || b == 0) return 0;
    float d2 = 0.f, bnd = 0.f;
    for (int d = 0; d < 3; d++) {
        const float x = C.com[d];
        float e = 0.f, E = 0.f;
        if (x < gilo[d]) {
            e = gilo[d] - x;
            E = 2.5e-7f * (fabsf(x) + fabsf(gilo[d]));
        } else if (x > gihi[d]) {
            e = x - gihi[d];
            E = 2.5e-7f * (fabsf(x) + fabsf(gihi[d]));
        } else {
            E = 2.5e-7f * (fabsf(x) + fmaxf(fabsf(gilo[d]), fabsf(gihi[d])));
        }
        d2 += e * e;
        bnd += 2.f * e * E + E * E;
    }
    bnd += 4e-7f * d2 + 1e-37f;
    const float s2 = C.size * C.size;
    if (s2 * (1.f - 4e-7f) > theta2 * (d2 + bnd) * (1.f + 4e-7f)) return 1;
    if (s2 * (1.f + 4e-7f) < theta2 * fmaxf(d2 - bnd, 0.f) * (1.f - 4e-7f)) return -1;
    return 0;
}

__global__ void k_walk_open(const TNode *nd, const TNodeF *nf, const int *gnode, int ng, const int *top, int ntop,
                            double theta2, float theta2f, unsigned char *ostat) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (long long)ng * ntop) return;
    const int g = (int)(p / ntop), t = (int)(p - (long long)g * ntop);
    const TNodeF &G = nf[gnode[g]];
    int o = open3(nf[top[t]], G.ilo, G.ihi, G.olo, G.ohi, theta2f);
    if (o == 0) {
        const TNode &Gd = nd[gnode[g]];
        o = cell_open(nd[top[t]], Gd.ilo, Gd.ihi, Gd.olo, Gd.ohi, theta2) ? 1 : -1;
    }
    ostat[p] = o > 0 ? 1 : 0;
}

// Class of each pair and its entry counts: not reached or an open node above
// the split depth (no entries), unopened (one SPJ entry), open leaf (its
// bodies), open node at the split depth (a subtree task, counted later).
// fill == 1 writes the entries of the first three kinds.
__global__ void k_walk_class(const TNode *nd, const int *top, const int *top_anc, const int *top_lvl, long long np,
                             int ntop, int depth, const unsigned char *ostat, const int *order, int fill, int *jc,
                             int *sc, int *task_flag, const int *jo, const int *so, int *j_idx, int *s_idx) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const int g = (int)(p / ntop), t = (int)(p - (long long)g * ntop);
    const unsigned char *os = ostat + (long long)g * ntop;
    bool reached = true;
    for (int a = 0; a < depth; a++) {
        const int ta = top_anc[t * depth + a];
        if (ta >= 0 && !os[ta]) reached = false;
    }
    int nj = 0, ns = 0, task = 0;
    const int c = top[t];
    if (reached) {
        const TNode &C = nd[c];
        if (!os[t]) {
            if (fill) s_idx[so[p]] = c;
            ns = 1;
        } else if (C.nchild == 0) {
            if (fill)
                for (int k = 0; k < C.count; k++) j_idx[jo[p] + k] = order[C.first + k];
            nj = C.count;
        } else if (top_lvl[t] == depth) {
            task = 1;
        }
    }
    if (!fill) {
        jc[p] = nj;
        sc[p] = ns;
        task_flag[p] = task;
    }
}

// the subtree walks of the compacted tasks (pair indices), one per thread;
// the opening test runs on the FP32 copies and falls back to the doubles
// only when the copies cannot decide
__global__ void k_walk_tasks(const TNode *nd, const TNodeF *nf, const int *gnode, const int *top, int ntop,
                             const int *tasks, int ntask, double theta2, float theta2f, const int *order, int fill,
                             int *jc, int *sc, const int *jo, const int *so, int *j_idx, int *s_idx, int *status) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ntask) return;
    const long long p = tasks[q];
    const int g = (int)(p / ntop), t = (int)(p - (long long)g * ntop);
    const int gn = gnode[g];
    float fil[3], fih[3], fol[3], foh[3];
    {
        const TNodeF &G = nf[gn];
        for (int d = 0; d < 3; d++) {
            fil[d] = G.ilo[d];
            fih[d] = G.ihi[d];
            fol[d] = G.olo[d];
            foh[d] = G.ohi[d];
        }
    }
    const TNodeF &C = nf[top[t]];
    int stack[WALK_STACK];
    int sp = 0;
    for (int ch = C.nchild - 1; ch >= 0; ch--) stack[sp++] = C.child0 + ch;
    int nj = 0, ns = 0;
    const int jbase = fill ? jo[p] : 0, sbase = fill ? so[p] : 0;
    for (int guard = 0; sp > 0 && guard < (1 << 26); guard++) {
        const int c = stack[--sp];
        const TNodeF &Q = nf[c];
        int o = open3(Q, fil, fih, fol, foh, theta2f);
        if (o == 0) {
            const TNode &Gd = nd[gn];
            o = cell_open(nd[c], Gd.ilo, Gd.ihi, Gd.olo, Gd.ohi, theta2) ? 1 : -1;
        }
        if (o < 0) {
            if (fill) s_idx[sbase + ns] = c;
            ns++;
        } else if (Q.nchild == 0) {
            if (fill)
                for (int k = 0; k < Q.count; k++) j_idx[jbase + nj + k] = order[Q.first + k];
            nj += Q.count;
        } else {
            if (sp + Q.nchild > WALK_STACK) {
                atomicOr(status, ST_QUEUE_OVERFLOW);
                break;
            }
            for (int ch = Q.nchild - 1; ch >= 0; ch--) stack[sp++] = Q.child0 + ch;
        }
    }
    if (!fill) {
        jc[p] = nj;
        sc[p] = ns;
    }
}

// ---- the walk as one CTA per group, breadth first --------------------------------------------
// The host builder's depth-first walk emits, in visiting order, one SPJ entry
// per unopened cell and the bodies of every opened leaf.  The same sequence
// comes out of a breadth-first sweep that keeps a frontier of items in that
// order: each round replaces every still-untested cell by its outcome -- an
// unopened cell or an opened leaf stays as a final item, an opened inner cell
// gives way to its children in child order -- so that after the last round
// the frontier is the depth-first output sequence.  All the CTA's threads
// test the frontier's cells at once (the subtree walks of one thread each
// ran at ~3 active lanes per instruction).  Items: node << 2 | kind.
constexpr int BFS_T = 128;
constexpr int BFS_CAP = 4096;  // frontier items per group (more: the group takes the task walk)
enum : int { FI_PEND = 0, FI_SPJ = 1, FI_EPJ = 2 };

// exclusive block-wide prefix of v over BFS_T threads (all threads call)
__device__ __forceinline__ int bfs_scan(int v, int *ws, int &total) {
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
    for (int k = 0; k < BFS_T / 32; k++) {
        const int c = ws[k];
        off += (k < w) ? c : 0;
        tot += c;
    }
    __syncthreads();
    total = tot;
    return off + x - v;
}

// count pass: the final frontier of group g (blockIdx.x) into store[off[g] ..
// off[g] + len[g]) and its EPJ / SPJ entry counts; a frontier above cap (<= BFS_CAP)
// items or a full store sets *overflow (the lists then come from the task walk)
__global__ void __launch_bounds__(BFS_T) k_walk_bfs(const TNode *nd, const TNodeF *nf, const int *gnode, int ng,
                                                    double theta2, float theta2f, int *jc, int *sc, int *len,
                                                    long long *off, int *store, unsigned long long *cursor,
                                                    long long store_cap, int *overflow, int cap) {
    __shared__ int buf[2][BFS_CAP];
    __shared__ int ws[BFS_T / 32];
    __shared__ long long s_base;
    const int g = blockIdx.x, tid = threadIdx.x;
    if (g >= ng) return;
    const int gn = gnode[g];
    float fil[3], fih[3], fol[3], foh[3];
    {
        const TNodeF &G = nf[gn];
        for (int d = 0; d < 3; d++) {
            fil[d] = G.ilo[d];
            fih[d] = G.ihi[d];
            fol[d] = G.olo[d];
            foh[d] = G.ohi[d];
        }
    }
    if (tid == 0) buf[0][0] = (0 << 2) | FI_PEND;  // the root
    __syncthreads();
    int cur = 0, n = 1;
    bool over = false, pend = true;
    for (int round = 0; pend && round < 64; round++) {
        int run = 0, grown = 0;
        for (int base = 0; base < n; base += BFS_T) {
            const int q = base + tid;
            int item = 0, cnt = 0, kind = FI_SPJ, nch = 0, c0 = 0;
            if (q < n) {
                item = buf[cur][q];
                kind = item & 3;
                cnt = 1;
                if (kind == FI_PEND) {
                    const int c = item >> 2;
                    const TNodeF &Q = nf[c];
                    int o = open3(Q, fil, fih, fol, foh, theta2f);
                    if (o == 0) {
                        const TNode &Gd = nd[gn];
                        o = cell_open(nd[c], Gd.ilo, Gd.ihi, Gd.olo, Gd.ohi, theta2) ? 1 : -1;
                    }
                    if (o < 0) {
                        kind = FI_SPJ;
                    } else if (Q.nchild == 0) {
                        kind = FI_EPJ;
                    } else {
                        nch = Q.nchild;
                        c0 = Q.child0;
                        cnt = nch;
                    }
                    item = (c << 2) | kind;
                }
            }
            int tot = 0;
            const int o = run + bfs_scan(cnt, ws, tot);
            if (q < n && o + cnt <= cap) {
                if (nch) {
                    for (int k = 0; k < nch; k++) buf[cur ^ 1][o + k] = ((c0 + k) << 2) | FI_PEND;
                } else {
                    buf[cur ^ 1][o] = item;
                }
            }
            grown += __syncthreads_or(nch > 0);
            run += tot;
        }
        if (run > cap) {
            over = true;
            break;
        }
        cur ^= 1;
        n = run;
        pend = grown > 0;
        __syncthreads();
    }
    if (pend && !over) over = true;  // deeper than 64 rounds
    if (!over) {
        int nj = 0, ns = 0;
        for (int q = tid; q < n; q += BFS_T) {
            const int it = buf[cur][q];
            if ((it & 3) == FI_EPJ) nj += nf[it >> 2].count;
            else ns += 1;
        }
        int tj = 0, ts = 0;
        bfs_scan(nj, ws, tj);
        bfs_scan(ns, ws, ts);
        if (tid == 0) {
            const long long b = (long long)atomicAdd(cursor, (unsigned long long)n);
            s_base = b;
            if (b + n > store_cap) atomicOr(overflow, 1);
            jc[g] = tj;
            sc[g] = ts;
            len[g] = n;
            off[g] = b;
        }
        __syncthreads();
        const long long b = s_base;
        if (b + n <= store_cap)
            for (int q = tid; q < n; q += BFS_T) store[b + q] = buf[cur][q];
    } else if (tid == 0) {
        atomicOr(overflow, 1);
        jc[g] = 0;
        sc[g] = 0;
        len[g] = 0;
        off[g] = 0;
    }
}

// fill pass: group g's entries from its stored frontier, in frontier order
__global__ void __launch_bounds__(BFS_T) k_walk_bfs_fill(const TNodeF *nf, int ng, const int *len, const long long *off,
                                                         const int *store, const int *order, const int *j_off,
                                                         const int *s_off, int *j_idx, int *s_idx) {
    __shared__ int ws[BFS_T / 32];
    const int g = blockIdx.x, tid = threadIdx.x;
    if (g >= ng) return;
    const int n = len[g];
    const int *fr = store + off[g];
    int jrun = j_off[g], srun = s_off[g];
    for (int base = 0; base < n; base += BFS_T) {
        const int q = base + tid;
        int it = 0, nj = 0, ns = 0, first = 0;
        if (q < n) {
            it = fr[q];
            if ((it & 3) == FI_EPJ) {
                const TNodeF &Q = nf[it >> 2];
                nj = Q.count;
                first = Q.first;
            } else {
                ns = 1;
            }
        }
        int tj = 0, ts = 0;
        const int oj = jrun + bfs_scan(nj, ws, tj);
        const int os = srun + bfs_scan(ns, ws, ts);
        for (int k = 0; k < nj; k++) j_idx[oj + k] = order[first + k];
        if (ns) s_idx[os] = it >> 2;
        jrun += tj;
        srun += ts;
    }
}

__global__ void k_task_list(const int *flag, const int *pos, long long np, int *tasks) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np && flag[p]) tasks[pos[p]] = (int)p;
}

// per-group list offsets from the per-pair offsets
__global__ void k_walk_group_off(const int *jo, const int *so, int ng, int ntop, int nj, int ns, int *j_off,
                                 int *s_off) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > ng) return;
    j_off[g] = (g < ng) ? jo[(long long)g * ntop] : nj;
    s_off[g] = (g < ng) ? so[(long long)g * ntop] : ns;
}

// launch order of the soft kernel: largest groups first (key: weight desc, group asc)
__global__ void k_group_weight(int ng, const int *i_off, const int *j_off, const int *s_off,
                               unsigned long long *key, int *idx) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const long long ni = i_off[g + 1] - i_off[g];
    const long long nj = (j_off[g + 1] - j_off[g]) + 2LL * (s_off[g + 1] - s_off[g]);
    const long long w = ((ni + 31) / 32) * 32 * nj;
    const unsigned long long wc = (unsigned long long)(w < (1LL << 43) ? w : (1LL << 43) - 1);
    key[g] = (((1ULL << 43) - 1 - wc) << 20) | (unsigned long long)g;
    idx[g] = g;
}

// ---- host side ----------------------------------------------------------------------------------
struct DTree {
    DevBuf<double> part, root;
    DevBuf<unsigned long long> key, key2;
    DevBuf<int> idx, idx2, hist, hoff, head, hs, enode, enode2, parent, gmark, gflag, gpos, gnode;
    DevBuf<TNode> nd;
    DevBuf<TNodeF> nf;
    DevBuf<int> top, pc, tasks;
    DevBuf<unsigned char> ostat;
    DevBuf<int> bjc, bsc, blen, bstore, bover;  // breadth-first walk
    DevBuf<int> arrived;                        // leaf flags, positions and list of the moments
    DevBuf<long long> boff;
    DevBuf<unsigned long long> bcur;
    long long bstore_cap = 1LL << 24;
    size_t node_cap = 0;
    std::vector<int> level_start;
    int n_nodes = 0, n_groups = 0;
};
static DTree g_dt;
static int g_walk_depth = 3;  // levels above the walk's task split
static int g_walk_bfs = 1;    // walk form: breadth first per group (1) or subtree tasks (0)
static int g_walk_last = -1;  // the form the last build's lists came from
static int g_walk_cap = BFS_CAP;  // frontier items a group's CTA may hold (lower: more groups take the task walk)
static int g_moments_up = 1;  // moments: leaves in one launch, then inner nodes per level (1); all nodes per level (0)

// (key, idx) sorted in place by key, stably (8 passes of 8 bits over `bits`)
static int radix_sort(Context *c, DTree &T, unsigned long long *&key, int *&idx, unsigned long long *&key2,
                      int *&idx2, int n, int bits) {
    const int nblk = (n + RADIX_TILE - 1) / RADIX_TILE;
    int r = 0;
    if ((r = T.hist.reserve(256 * (size_t)nblk)) || (r = T.hoff.reserve(256 * (size_t)nblk + 1))) return r;
    for (int shift = 0; shift < bits; shift += 8) {
        { P3T_COUNT_LAUNCH(); k_radix_hist<<<nblk, 256, 0, c->stream>>>(key, n, shift, nblk, T.hist.p); }
        if ((r = g_eng.scan(T.hist.p, T.hoff.p, 256 * nblk, nullptr))) return r;  // stream-ordered, no host wait
        { P3T_COUNT_LAUNCH(); k_radix_scatter<<<nblk, 256, 0, c->stream>>>(key, idx, n, shift, nblk, T.hoff.p, key2, idx2); }
        std::swap(key, key2);
        std::swap(idx, idx2);
    }
    return cuda_status(cudaGetLastError());
}

// node storage that keeps its contents when it grows
static int grow_nodes(Context *c, DTree &T, size_t need) {
    if (need <= T.node_cap) return 0;
    const size_t cap = std::max(need, T.node_cap * 2);
    TNode *np = nullptr;
    int *pp = nullptr;
    int r = cuda_status(cudaMalloc(&np, cap * sizeof(TNode)));
    if (r) return r;
    if ((r = cuda_status(cudaMalloc(&pp, cap * sizeof(int))))) {
        cudaFree(np);
        return r;
    }
    if (T.node_cap) {
        cudaMemcpyAsync(np, T.nd.p, T.node_cap * sizeof(TNode), cudaMemcpyDeviceToDevice, c->stream);
        cudaMemcpyAsync(pp, T.parent.p, T.node_cap * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
        cudaStreamSynchronize(c->stream);
    }
    T.nd.release();
    T.parent.release();
    T.nd.p = np;
    T.nd.cap = cap * sizeof(TNode);
    T.parent.p = pp;
    T.parent.cap = cap * sizeof(int);
    T.node_cap = cap;
    return 0;
}

static inline int nblocks(long long n, int t = 256) { return (int)std::max<long long>(1, (n + t - 1) / t); }

// Builds the tree of the state's bodies and writes the group lists and the
// SPJ array into the resident soft-force set.
static int device_tree(Context *c, double theta, int n_leaf_limit, int n_group_limit) {
    Engine &E = g_eng;
    DTree &T = g_dt;
    DevSet &d = c->res;
    const int n = E.S.n;
    if (n <= 0 || theta <= 0. || n_leaf_limit < 1 || n_group_limit < 1) return ST_BAD_INDEX;
    const int limit = std::min(n_leaf_limit, n_group_limit);
    int r = 0;
    const int pb = std::min(1024, nblocks(n));
    if ((r = T.part.reserve(6 * (size_t)pb)) || (r = T.root.reserve(8)) || (r = T.key.reserve(n)) ||
        (r = T.key2.reserve(n)) || (r = T.idx.reserve(n)) || (r = T.idx2.reserve(n)) || (r = T.head.reserve(n)) ||
        (r = T.hs.reserve(n)) || (r = T.enode.reserve(n)) || (r = T.enode2.reserve(n)) ||
        (r = T.gmark.reserve(n)) || (r = T.gflag.reserve(n)) || (r = T.gpos.reserve(n)))
        return r;
    // 1. root cube, keys, sort
    { P3T_COUNT_LAUNCH(); k_bbox_partial<<<pb, 256, 0, c->stream>>>(E.S.pos, n, T.part.p); }
    { P3T_COUNT_LAUNCH(); k_bbox_root<<<1, 256, 0, c->stream>>>(T.part.p, pb, T.root.p); }
    { P3T_COUNT_LAUNCH(); k_keys<<<nblocks(n), 256, 0, c->stream>>>(E.S.pos, n, T.root.p, T.key.p, T.idx.p); }
    unsigned long long *key = T.key.p, *key2 = T.key2.p;
    int *idx = T.idx.p, *idx2 = T.idx2.p;
    if ((r = radix_sort(c, T, key, idx, key2, idx2, n, 64))) return r;  // 8 passes: back in T.key / T.idx
    // 2. levels
    if ((r = grow_nodes(c, T, (size_t)n / 4 + 1024))) return r;
    { P3T_COUNT_LAUNCH(); k_root_node<<<nblocks(n), 256, 0, c->stream>>>(T.nd.p, T.parent.p, T.root.p, n, limit, T.enode.p); }
    T.level_start.assign(1, 0);
    int base = 1;
    int *en = T.enode.p, *en2 = T.enode2.p;
    for (int level = 0; level < 21; level++) {
        { P3T_COUNT_LAUNCH(); k_lvl_heads<<<nblocks(n), 256, 0, c->stream>>>(key, en, T.nd.p, n, 3 * (20 - level), T.head.p); }
        int m = 0;
        if ((r = E.scan(T.head.p, T.hs.p, n, &m))) return r;
        if (m == 0) break;
        if ((r = grow_nodes(c, T, (size_t)base + m))) return r;
        T.level_start.push_back(base);
        { P3T_COUNT_LAUNCH(); k_lvl_make<<<nblocks(n), 256, 0, c->stream>>>(en, T.head.p, T.hs.p, n, base, T.nd.p, T.parent.p, en2); }
        { P3T_COUNT_LAUNCH(); k_lvl_count<<<nblocks(m), 256, 0, c->stream>>>(base, m, T.nd.p, T.parent.p); }
        { P3T_COUNT_LAUNCH(); k_lvl_split<<<nblocks(n), 256, 0, c->stream>>>(n, level + 1, limit, T.nd.p, en2); }
        std::swap(en, en2);
        base += m;
    }
    T.level_start.push_back(base);
    T.n_nodes = base;
    if ((r = d.spj.reserve(base))) return r;
    // 3. moments, bottom-up in one launch (or one launch per level, deepest first)
    if (g_moments_up) {
        if ((r = T.arrived.reserve(3 * (size_t)base + 1))) return r;
        int *flag = T.arrived.p, *lpos = T.arrived.p + base, *list = T.arrived.p + 2 * base, *cnt = list + base;
        { P3T_COUNT_LAUNCH(); k_leaf_flag<<<nblocks(base), 256, 0, c->stream>>>(base, T.nd.p, flag); }
        if ((r = E.scan(flag, lpos, base, nullptr))) return r;
        { P3T_COUNT_LAUNCH(); k_leaf_list<<<nblocks(base), 256, 0, c->stream>>>(base, flag, lpos, list, cnt); }
        { P3T_COUNT_LAUNCH(); k_moments_leaves<<<nblocks(base, 128), 128, 0, c->stream>>>(list, cnt, T.nd.p, d.spj.p, idx,
                                                                                      E.S.pos, E.S.mass,
                                                                                      E.S.r_search); }
        for (int L = (int)T.level_start.size() - 2; L >= 0; L--) {
            const int lo = T.level_start[L], hi = T.level_start[L + 1];
            { P3T_COUNT_LAUNCH(); k_moments_inner<<<nblocks(hi - lo, 128), 128, 0, c->stream>>>(lo, hi, base, list, lpos, flag,
                                                                                           T.nd.p, d.spj.p, idx,
                                                                                           E.S.pos, E.S.mass,
                                                                                           E.S.r_search); }
        }
    } else {
        for (int L = (int)T.level_start.size() - 2; L >= 0; L--) {
            const int lo = T.level_start[L], hi = T.level_start[L + 1];
            { P3T_COUNT_LAUNCH(); k_moments<<<nblocks(hi - lo, 128), 128, 0, c->stream>>>(lo, hi, T.nd.p, d.spj.p, idx, E.S.pos, E.S.mass,
                                                                    E.S.r_search); }
        }
    }
    // 4. groups in Morton order
    cudaMemsetAsync(T.gmark.p, 0, n * sizeof(int), c->stream);
    { P3T_COUNT_LAUNCH(); k_group_mark<<<nblocks(base), 256, 0, c->stream>>>(base, T.nd.p, T.parent.p, n_group_limit, T.gmark.p); }
    { P3T_COUNT_LAUNCH(); k_group_flag<<<nblocks(n), 256, 0, c->stream>>>(T.gmark.p, n, T.gflag.p); }
    int ng = 0;
    if ((r = E.scan(T.gflag.p, T.gpos.p, n, &ng))) return r;
    T.n_groups = ng;
    if ((r = T.gnode.reserve(ng + 1)) || (r = d.i_off.reserve(ng + 1)) || (r = d.j_off.reserve(ng + 1)) ||
        (r = d.s_off.reserve(ng + 1)) || (r = d.i_idx.reserve(n)))
        return r;
    { P3T_COUNT_LAUNCH(); k_group_fill<<<nblocks(n), 256, 0, c->stream>>>(T.gmark.p, T.gpos.p, n, ng, T.gnode.p, d.i_off.p); }
    cudaMemcpyAsync(d.i_idx.p, idx, n * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    // 5. walks: breadth first, one CTA per group; if a frontier outgrows its
    // CTA (or the frontier store), the task walk below
    if ((r = T.nf.reserve(T.n_nodes))) return r;
    { P3T_COUNT_LAUNCH(); k_node_f32<<<nblocks(T.n_nodes), 256, 0, c->stream>>>(T.nd.p, T.n_nodes, T.nf.p); }
    bool walked = false;
    if (g_walk_bfs && ng > 0) {
        if ((r = T.bjc.reserve(ng)) || (r = T.bsc.reserve(ng)) || (r = T.blen.reserve(ng)) ||
            (r = T.boff.reserve(ng)) || (r = T.bover.reserve(1)) || (r = T.bcur.reserve(1)) ||
            (r = T.bstore.reserve((size_t)T.bstore_cap)))
            return r;
        cudaMemsetAsync(T.bover.p, 0, sizeof(int), c->stream);
        cudaMemsetAsync(T.bcur.p, 0, sizeof(unsigned long long), c->stream);
        { P3T_COUNT_LAUNCH(); k_walk_bfs<<<ng, BFS_T, 0, c->stream>>>(T.nd.p, T.nf.p, T.gnode.p, ng, theta * theta,
                                                                  (float)(theta * theta), T.bjc.p, T.bsc.p, T.blen.p,
                                                                  T.boff.p, T.bstore.p, T.bcur.p, T.bstore_cap,
                                                                  T.bover.p, g_walk_cap); }
        int over = 0;
        unsigned long long used = 0;
        int nj = 0, ns = 0;
        if ((r = E.scan(T.bjc.p, d.j_off.p, ng, &nj)) || (r = E.scan(T.bsc.p, d.s_off.p, ng, &ns)) ||
            (r = d2h(c, &over, T.bover.p, sizeof(int))) || (r = d2h(c, &used, T.bcur.p, sizeof(used))))
            return r;
        if (!over) {
            if ((r = h2d(c, d.j_off.p + ng, &nj, sizeof(int))) || (r = h2d(c, d.s_off.p + ng, &ns, sizeof(int))) ||
                (r = d.j_idx.reserve(nj)) || (r = d.s_idx.reserve(ns)))
                return r;
            { P3T_COUNT_LAUNCH(); k_walk_bfs_fill<<<ng, BFS_T, 0, c->stream>>>(T.nf.p, ng, T.blen.p, T.boff.p, T.bstore.p,
                                                                           idx, d.j_off.p, d.s_off.p, d.j_idx.p,
                                                                           d.s_idx.p); }
            walked = true;
        } else if ((long long)used > T.bstore_cap) {
            T.bstore_cap = (long long)(used + used / 4);  // room for the next build
        }
    }
    g_walk_last = walked ? 1 : 0;
    // the task walk: the top levels in pre-order (host, from the node table),
    // then (group, top node) pairs: open tests, counts, offsets, entries
    if (!walked) {
        const int nlev = (int)T.level_start.size() - 1;
        const int depth = std::min(g_walk_depth, nlev - 1);
        const int ntop_nodes = T.level_start[depth + 1];
        std::vector<TNode> tn(ntop_nodes);
        if ((r = d2h(c, tn.data(), T.nd.p, ntop_nodes * sizeof(TNode)))) return r;
        std::vector<int> top, anc, lvl;
        std::vector<int> path;
        std::vector<int> pos_of(ntop_nodes, -1);
        // pre-order from the root, levels 0..depth
        std::vector<std::pair<int, int>> st{{0, 0}};
        std::vector<int> par_top(ntop_nodes, -1);
        while (!st.empty()) {
            const int nd_id = st.back().first, L = st.back().second;
            st.pop_back();
            pos_of[nd_id] = (int)top.size();
            top.push_back(nd_id);
            lvl.push_back(L);
            if (L < depth)
                for (int ch = tn[nd_id].nchild - 1; ch >= 0; ch--) {
                    par_top[tn[nd_id].child0 + ch] = nd_id;
                    st.push_back({tn[nd_id].child0 + ch, L + 1});
                }
        }
        const int ntop = (int)top.size();
        anc.assign((size_t)ntop * std::max(depth, 1), -1);
        for (int t = 0; t < ntop; t++) {
            int a = par_top[top[t]], k = 0;
            while (a >= 0 && k < depth) {
                anc[(size_t)t * depth + k++] = pos_of[a];
                a = par_top[a];
            }
        }
        const long long np = (long long)ng * ntop;
        if (np > 2000000000LL) return ST_QUEUE_OVERFLOW;
        if ((r = T.top.reserve(3 * (size_t)ntop + (size_t)ntop * std::max(depth, 1))) ||
            (r = T.ostat.reserve(np)) || (r = T.pc.reserve(6 * np + 6)))
            return r;
        int *top_d = T.top.p, *lvl_d = T.top.p + ntop, *anc_d = T.top.p + 2 * ntop;
        if ((r = h2d(c, top_d, top.data(), ntop * sizeof(int))) || (r = h2d(c, lvl_d, lvl.data(), ntop * sizeof(int))) ||
            (r = h2d(c, anc_d, anc.data(), anc.size() * sizeof(int))))
            return r;
        int *jc = T.pc.p, *sc = T.pc.p + np, *jo = T.pc.p + 2 * np, *so = T.pc.p + 3 * np;
        int *tflag = T.pc.p + 4 * np, *tpos = T.pc.p + 5 * np;
        const int wb = (int)std::min<long long>((np + 127) / 128, 1LL << 30);
        const float th2f = (float)(theta * theta);
        { P3T_COUNT_LAUNCH(); k_walk_open<<<wb, 128, 0, c->stream>>>(T.nd.p, T.nf.p, T.gnode.p, ng, top_d, ntop, theta * theta, th2f,
                                               T.ostat.p); }
        { P3T_COUNT_LAUNCH(); k_walk_class<<<wb, 128, 0, c->stream>>>(T.nd.p, top_d, anc_d, lvl_d, np, ntop, depth, T.ostat.p, idx, 0, jc,
                                                sc, tflag, nullptr, nullptr, nullptr, nullptr); }
        int ntask = 0;
        if ((r = E.scan(tflag, tpos, (int)np, &ntask)) || (r = T.tasks.reserve(ntask + 1))) return r;
        { P3T_COUNT_LAUNCH(); k_task_list<<<wb, 128, 0, c->stream>>>(tflag, tpos, np, T.tasks.p); }
        { P3T_COUNT_LAUNCH(); k_walk_tasks<<<nblocks(ntask, 128), 128, 0, c->stream>>>(T.nd.p, T.nf.p, T.gnode.p, top_d, ntop, T.tasks.p,
                                                                 ntask, theta * theta, th2f, idx, 0, jc, sc, nullptr,
                                                                 nullptr, nullptr, nullptr, c->status); }
        int nj = 0, ns = 0;
        if ((r = E.scan(jc, jo, (int)np, &nj)) || (r = E.scan(sc, so, (int)np, &ns))) return r;
        { P3T_COUNT_LAUNCH(); k_walk_group_off<<<nblocks(ng + 1), 256, 0, c->stream>>>(jo, so, ng, ntop, nj, ns, d.j_off.p, d.s_off.p); }
        if ((r = d.j_idx.reserve(nj)) || (r = d.s_idx.reserve(ns))) return r;
        { P3T_COUNT_LAUNCH(); k_walk_class<<<wb, 128, 0, c->stream>>>(T.nd.p, top_d, anc_d, lvl_d, np, ntop, depth, T.ostat.p, idx, 1, jc,
                                                sc, tflag, jo, so, d.j_idx.p, d.s_idx.p); }
        { P3T_COUNT_LAUNCH(); k_walk_tasks<<<nblocks(ntask, 128), 128, 0, c->stream>>>(T.nd.p, T.nf.p, T.gnode.p, top_d, ntop, T.tasks.p,
                                                                 ntask, theta * theta, th2f, idx, 1, jc, sc, jo, so,
                                                                 d.j_idx.p, d.s_idx.p, c->status); }
    }
    // 6. the soft kernel's launch order (the bodies' key buffers and the
    // group-scan scratch are free by now)
    if ((r = d.order.reserve(ng))) return r;
    if (ng > 0) {
        unsigned long long *k1 = T.key.p, *k2 = T.key2.p;
        int *i1 = T.gflag.p, *i2 = T.head.p;
        { P3T_COUNT_LAUNCH(); k_group_weight<<<nblocks(ng), 256, 0, c->stream>>>(ng, d.i_off.p, d.j_off.p, d.s_off.p, k1, i1); }
        if ((r = radix_sort(c, T, k1, i1, k2, i2, ng, 64))) return r;
        cudaMemcpyAsync(d.order.p, i1, ng * sizeof(int), cudaMemcpyDeviceToDevice, c->stream);
    }
    d.order_valid = true;
    c->res_groups = ng;
    c->res_spj = base;
    c->res_n = n;
    return cuda_status(cudaGetLastError());
}

}  // namespace p3t

using namespace p3t;

extern "C" {

int p3t_set_walk(int form) {
    if (form < 0 || form > 3) return -(int)cudaErrorInvalidValue;
    g_walk_bfs = form & 1;
    g_moments_up = (form >> 1) ^ 1;
    return 0;
}

int p3t_walk_last(void) { return g_walk_last; }

int p3t_set_walk_limits(int frontier_cap, long long store_items) {
    if (frontier_cap < 1 || frontier_cap > BFS_CAP || store_items < 0) return -(int)cudaErrorInvalidValue;
    g_walk_cap = frontier_cap;
    if (store_items > 0) g_dt.bstore_cap = store_items;
    return 0;
}

int p3t_state_tree(double theta, int n_leaf_limit, int n_group_limit) {
    Context *c = ctx_get(0);
    if (!c || !g_eng.c) return -(int)cudaErrorNoDevice;
    int r = g_eng.pack_soft();
    if (r) return r;
    if ((r = device_tree(c, theta, n_leaf_limit, n_group_limit))) return r;
    return read_status(c);
}

int p3t_state_tree_soft(double theta, int n_leaf_limit, int n_group_limit) {
    int r = p3t_state_tree(theta, n_leaf_limit, n_group_limit);
    if (r) return r;
    return soft_run_state();
}

int p3t_tree_lists_counts(long long *counts) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    const int ng = c->res_groups;
    counts[0] = ng;
    counts[1] = c->res_n;
    int nj = 0, ns = 0;
    if (ng > 0) {
        int r = d2h(c, &nj, c->res.j_off.p + ng, sizeof(int));
        if (r || (r = d2h(c, &ns, c->res.s_off.p + ng, sizeof(int)))) return r;
    }
    counts[2] = nj;
    counts[3] = ns;
    counts[4] = c->res_spj;
    return 0;
}

int p3t_tree_lists_get(int *i_off, int *i_idx, int *j_off, int *j_idx, int *s_off, int *s_idx, void *spj) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    long long k[5];
    int r = p3t_tree_lists_counts(k);
    if (r) return r;
    DevSet &d = c->res;
    const int ng = (int)k[0];
    if ((r = d2h(c, i_off, d.i_off.p, (ng + 1) * sizeof(int))) || (r = d2h(c, j_off, d.j_off.p, (ng + 1) * sizeof(int))) ||
        (r = d2h(c, s_off, d.s_off.p, (ng + 1) * sizeof(int))) || (r = d2h(c, i_idx, d.i_idx.p, k[1] * sizeof(int))) ||
        (r = d2h(c, j_idx, d.j_idx.p, k[2] * sizeof(int))) || (r = d2h(c, s_idx, d.s_idx.p, k[3] * sizeof(int))))
        return r;
    if (spj && (r = d2h(c, spj, d.spj.p, k[4] * sizeof(SPJRec)))) return r;
    return 0;
}

}  // extern "C"
