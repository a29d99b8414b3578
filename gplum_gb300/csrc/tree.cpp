// Host-side Barnes-Hut octree and interaction-list builder.
//
// This is the caller side of the soft-force path: in GPLUM the lists come
// from FDPS's TreeForForce (LONG_SYMMETRY search mode, quadrupole moments,
// MAKE_LIST, called at src/main_p3t.cpp:344-355,581-587 of GPLUM).  FDPS is
// not part of the GPLUM tree, so this file builds lists with the same
// contract, and the same lists feed both the device kernels and the CPU
// checkers:
//   * particles are grouped into i-groups of at most n_group_limit members
//     (tree cells, members in Morton order);
//   * a particle j enters a group's EPJ list whenever its distance to some
//     member i can be below max(1.1 r_search_i, 1.1 r_search_j) (the
//     symmetric search rule, with the 1.1 SAFTY_FACTOR of
//     src/particle.h:6,119-125); every other cell that passes the opening
//     test enters as a quadrupole superparticle (SPJ);
//   * the opening test is size/d < theta, d the distance from the cell's
//     centre of mass to the group's bounding box.
// Quadrupoles are raw second moments about the centre of mass.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/p3t_tree.h"

namespace {

struct Box {
    double lo[3], hi[3];
    void reset() {
        for (int d = 0; d < 3; d++) { lo[d] = 1e300; hi[d] = -1e300; }
    }
    void add(const double *x, double r) {
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], x[d] - r);
            hi[d] = std::max(hi[d], x[d] + r);
        }
    }
    void merge(const Box &b) {
        for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], b.lo[d]); hi[d] = std::max(hi[d], b.hi[d]); }
    }
    bool overlaps(const Box &b) const {
        for (int d = 0; d < 3; d++)
            if (hi[d] < b.lo[d] || b.hi[d] < lo[d]) return false;
        return true;
    }
    double dist2(const double *x) const {
        double s = 0.;
        for (int d = 0; d < 3; d++) {
            double e = 0.;
            if (x[d] < lo[d]) e = lo[d] - x[d];
            else if (x[d] > hi[d]) e = x[d] - hi[d];
            s += e * e;
        }
        return s;
    }
};

struct Node {
    int first, count;      // range in the Morton-sorted order
    int child0, nchild;    // children are contiguous node ids
    double size;           // cube side length
    double mass, com[3], quad[6];  // quad: xx yy zz xy xz yz
    Box inner, outer;      // bbox of positions / of positions +- 1.1 r_search
};

inline uint64_t spread21(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

}  // namespace

struct P3TTree {
    int n = 0;
    std::vector<int> order;  // Morton order -> particle index
    std::vector<uint64_t> key;
    std::vector<Node> nodes;
    std::vector<int> groups;  // node ids of i-groups
    // exported lists
    std::vector<int> i_off, i_idx, j_off, j_idx, s_off, s_idx;
    int status = 0;
};

static void build_node(P3TTree &t, int id, int level, const double *pos, const double *mass,
                       const double *rs, int n_leaf_limit) {
    Node &nd = t.nodes[id];
    // moments and boxes from the member particles
    nd.mass = 0.;
    for (int d = 0; d < 3; d++) nd.com[d] = 0.;
    nd.inner.reset();
    nd.outer.reset();
    for (int k = nd.first; k < nd.first + nd.count; k++) {
        int p = t.order[k];
        nd.mass += mass[p];
        for (int d = 0; d < 3; d++) nd.com[d] += mass[p] * pos[3 * p + d];
        nd.inner.add(&pos[3 * p], 0.);
        nd.outer.add(&pos[3 * p], 1.1 * rs[p]);
    }
    if (nd.mass != 0.)
        for (int d = 0; d < 3; d++) nd.com[d] /= nd.mass;
    for (int q = 0; q < 6; q++) nd.quad[q] = 0.;
    for (int k = nd.first; k < nd.first + nd.count; k++) {
        int p = t.order[k];
        double dx = pos[3 * p] - nd.com[0], dy = pos[3 * p + 1] - nd.com[1], dz = pos[3 * p + 2] - nd.com[2];
        double m = mass[p];
        nd.quad[0] += m * dx * dx; nd.quad[1] += m * dy * dy; nd.quad[2] += m * dz * dz;
        nd.quad[3] += m * dx * dy; nd.quad[4] += m * dx * dz; nd.quad[5] += m * dy * dz;
    }
    nd.child0 = -1;
    nd.nchild = 0;
    if (nd.count <= n_leaf_limit || level >= 21) return;
    // split by the next 3 Morton bits
    const int shift = 3 * (20 - level);
    int starts[9];
    int k = nd.first;
    const int end = nd.first + nd.count;
    for (int oct = 0; oct < 8; oct++) {
        starts[oct] = k;
        while (k < end && (int)((t.key[k] >> shift) & 7) == oct) k++;
    }
    starts[8] = end;
    int nch = 0;
    for (int oct = 0; oct < 8; oct++)
        if (starts[oct + 1] > starts[oct]) nch++;
    const int c0 = (int)t.nodes.size();
    t.nodes.resize(t.nodes.size() + nch);
    int c = c0;
    for (int oct = 0; oct < 8; oct++) {
        if (starts[oct + 1] == starts[oct]) continue;
        Node &ch = t.nodes[c];
        ch.first = starts[oct];
        ch.count = starts[oct + 1] - starts[oct];
        ch.size = t.nodes[id].size * 0.5;
        c++;
    }
    t.nodes[id].child0 = c0;
    t.nodes[id].nchild = nch;
    for (int i = 0; i < nch; i++) build_node(t, c0 + i, level + 1, pos, mass, rs, n_leaf_limit);
}

static void collect_groups(P3TTree &t, int id, int n_group_limit) {
    const Node &nd = t.nodes[id];
    if (nd.count <= n_group_limit || nd.nchild == 0) {
        t.groups.push_back(id);
        return;
    }
    for (int c = 0; c < nd.nchild; c++) collect_groups(t, nd.child0 + c, n_group_limit);
}

extern "C" {

P3TTree *p3t_tree_build(int n, const double *pos, const double *mass, const double *r_search,
                        double theta, int n_leaf_limit, int n_group_limit) {
    P3TTree *t = new P3TTree();
    t->n = n;
    if (n <= 0 || theta <= 0. || n_leaf_limit < 1 || n_group_limit < 1) {
        t->status = 1;
        return t;
    }
    // root cube
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], pos[3 * i + d]);
            hi[d] = std::max(hi[d], pos[3 * i + d]);
        }
    double ext = 0.;
    for (int d = 0; d < 3; d++) ext = std::max(ext, hi[d] - lo[d]);
    const double size = ext * 1.0001 + 1e-300;
    // the cube is anchored at the bodies' lower corner (margin (size - ext)/2
    // on every axis): along the widest axis this centres the bodies, and a
    // thin axis (a disk's normal) is not cut through the bodies until the
    // cells are thinner than the bodies' extent along it -- a cut near the
    // mid-plane at a coarse level would leave sparse, wide groups on one side
    double base[3];
    for (int d = 0; d < 3; d++) base[d] = lo[d] - 0.5 * (size - ext);
    // Morton keys and sort
    std::vector<std::pair<uint64_t, int>> kv(n);
    const double scale = double(1 << 21) / size;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        uint64_t c[3];
        for (int d = 0; d < 3; d++) {
            double u = (pos[3 * i + d] - base[d]) * scale;
            int64_t v = (int64_t)u;
            v = std::max<int64_t>(0, std::min<int64_t>((1 << 21) - 1, v));
            c[d] = (uint64_t)v;
        }
        kv[i] = {(spread21(c[0]) << 2) | (spread21(c[1]) << 1) | spread21(c[2]), i};
    }
    std::sort(kv.begin(), kv.end());
    t->order.resize(n);
    t->key.resize(n);
    for (int i = 0; i < n; i++) { t->key[i] = kv[i].first; t->order[i] = kv[i].second; }
    kv.clear();
    kv.shrink_to_fit();
    // tree
    t->nodes.reserve(2 * (size_t)n / std::max(1, n_leaf_limit) + 64);
    t->nodes.resize(1);
    t->nodes[0].first = 0;
    t->nodes[0].count = n;
    t->nodes[0].size = size;
    // leaves never exceed the group limit, so every group is a cell of at most
    // n_group_limit particles (except exactly coincident positions)
    build_node(*t, 0, 0, pos, mass, r_search, std::min(n_leaf_limit, n_group_limit));
    collect_groups(*t, 0, n_group_limit);

    // interaction lists, one walk per group
    const int ng = (int)t->groups.size();
    std::vector<std::vector<int>> jl(ng), sl(ng);
    const double theta2 = theta * theta;
#pragma omp parallel for schedule(dynamic, 4)
    for (int g = 0; g < ng; g++) {
        const Node &gn = t->nodes[t->groups[g]];
        const Box &gin = gn.inner, &gout = gn.outer;
        std::vector<int> stack;
        stack.reserve(256);
        stack.push_back(0);
        std::vector<int> &J = jl[g], &S = sl[g];
        while (!stack.empty()) {
            int c = stack.back();
            stack.pop_back();
            const Node &cn = t->nodes[c];
            bool near = cn.outer.overlaps(gin) || gout.overlaps(cn.inner);
            bool open = near || (cn.size * cn.size > theta2 * gin.dist2(cn.com));
            if (!open) {
                S.push_back(c);
            } else if (cn.nchild == 0) {
                for (int k = cn.first; k < cn.first + cn.count; k++) J.push_back(t->order[k]);
            } else {
                for (int ch = cn.nchild - 1; ch >= 0; ch--) stack.push_back(cn.child0 + ch);
            }
        }
    }
    // CSR export
    long long tot_i = 0, tot_j = 0, tot_s = 0;
    for (int g = 0; g < ng; g++) {
        tot_i += t->nodes[t->groups[g]].count;
        tot_j += (long long)jl[g].size();
        tot_s += (long long)sl[g].size();
    }
    if (tot_j > 2147483647LL || tot_s > 2147483647LL) {
        t->status = 2;
        return t;
    }
    t->i_off.resize(ng + 1);
    t->j_off.resize(ng + 1);
    t->s_off.resize(ng + 1);
    t->i_off[0] = t->j_off[0] = t->s_off[0] = 0;
    for (int g = 0; g < ng; g++) {
        t->i_off[g + 1] = t->i_off[g] + t->nodes[t->groups[g]].count;
        t->j_off[g + 1] = t->j_off[g] + (int)jl[g].size();
        t->s_off[g + 1] = t->s_off[g] + (int)sl[g].size();
    }
    t->i_idx.resize(tot_i);
    t->j_idx.resize(tot_j);
    t->s_idx.resize(tot_s);
#pragma omp parallel for schedule(static)
    for (int g = 0; g < ng; g++) {
        const Node &gn = t->nodes[t->groups[g]];
        for (int k = 0; k < gn.count; k++) t->i_idx[t->i_off[g] + k] = t->order[gn.first + k];
        std::copy(jl[g].begin(), jl[g].end(), t->j_idx.begin() + t->j_off[g]);
        std::copy(sl[g].begin(), sl[g].end(), t->s_idx.begin() + t->s_off[g]);
    }
    return t;
}

int p3t_tree_status(const P3TTree *t) { return t ? t->status : 1; }

// counts[0] groups, [1] i entries, [2] EPJ entries, [3] SPJ entries, [4] tree nodes
void p3t_tree_counts(const P3TTree *t, long long *counts) {
    counts[0] = (long long)t->groups.size();
    counts[1] = (long long)t->i_idx.size();
    counts[2] = (long long)t->j_idx.size();
    counts[3] = (long long)t->s_idx.size();
    counts[4] = (long long)t->nodes.size();
}

// Copies the lists out.  spj receives one SPJQuadrupole record per tree node
// (mass, pos.xyz, quad.xx yy zz xy xz yz = 10 doubles, the 80-byte FDPS
// superparticle layout); SPJ list entries index that array.
void p3t_tree_export(const P3TTree *t, int *i_off, int *i_idx, int *j_off, int *j_idx, int *s_off,
                     int *s_idx, double *spj) {
    std::memcpy(i_off, t->i_off.data(), t->i_off.size() * sizeof(int));
    std::memcpy(j_off, t->j_off.data(), t->j_off.size() * sizeof(int));
    std::memcpy(s_off, t->s_off.data(), t->s_off.size() * sizeof(int));
    std::memcpy(i_idx, t->i_idx.data(), t->i_idx.size() * sizeof(int));
    std::memcpy(j_idx, t->j_idx.data(), t->j_idx.size() * sizeof(int));
    std::memcpy(s_idx, t->s_idx.data(), t->s_idx.size() * sizeof(int));
    if (spj) {
        for (size_t c = 0; c < t->nodes.size(); c++) {
            const Node &nd = t->nodes[c];
            double *o = spj + 10 * c;
            o[0] = nd.mass;
            o[1] = nd.com[0]; o[2] = nd.com[1]; o[3] = nd.com[2];
            for (int q = 0; q < 6; q++) o[4 + q] = nd.quad[q];
        }
    }
}

void p3t_tree_free(P3TTree *t) { delete t; }

}  // extern "C"
