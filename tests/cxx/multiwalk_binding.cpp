// The FDPS-side binding of the library's multiwalk pair, as a GPLUM build
// adds it: the functor call of src/main_p3t.cpp:351-355 becomes
// calcForceAllAndWriteBackMultiWalk(DispatchP3T, RetrieveP3T, ...), whose two
// callbacks forward FDPS's per-walk arrays to p3t_soft_dispatch /
// p3t_soft_retrieve.
//
// Compiled two ways by tests/test_binding_cxx.py:
//   -DGPLUM_TYPES: against GPLUM's own record classes (its particle.h over
//     the single-rank PS shim of oracle/ref_shim), where the reference tree
//     is present -- the static_asserts below then prove that EPIGrav,
//     EPJGrav, MySPJQuadrupole and ForceGrav have the layouts the C ABI
//     reads and writes;
//   default: against the library's C structs of the same layout, linked with
//     the library and run on the GPU: main() drives the callbacks the way
//     FDPS drives a multiwalk force (groups in batches of n_walk_limit walks,
//     each walk its i-group's EPI records and its EPJ and SPJ lists) and
//     writes every body's ForceGrav record.
//
//   multiwalk_binding IN OUT N_WALK_LIMIT
// IN: int64 {n, n_group, n_spj}, double params[21], EPJGrav[n], SPJ[n_spj],
//     int32 i_off[n_group+1], i_idx[...], j_off[n_group+1], j_idx[...],
//     s_off[n_group+1], s_idx[...]
// OUT: ForceGrav[n] in particle order.
#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gplum_p3t.h"

#ifdef GPLUM_TYPES
#include <iostream>
#include <fstream>
#include <stdlib.h>
#include <map>
#define USE_RE_SEARCH_NEIGHBOR
#define PIKG_USE_FDPS_VECTOR
#include <particle_simulator.hpp>
constexpr PS::F64 MY_PI = 3.14159265358979323846L;
constexpr PS::F64 L_MKS = 149597870700;
constexpr PS::F64 L_CGS = 14959787070000;
constexpr PS::F64 M_MKS = 1.9884e30;
constexpr PS::F64 M_CGS = 1.9884e33;
constexpr PS::F64 T_MKS = 365.25 * 24. * 60. * 60. / (2. * MY_PI);
constexpr PS::F64 T_CGS = 365.25 * 24. * 60. * 60. / (2. * MY_PI);
constexpr PS::S64 S32_MAX = (1LL << 31);
#include "mathfunc.h"
#include "kepler.h"
#include "particle.h"
using EPI_t = EPIGrav;
using EPJ_t = EPJGrav;
using SPJ_t = MySPJQuadrupole;
using Force_t = ForceGrav;
// the layouts the C ABI assumes, member by member
static_assert(sizeof(EPI_t) == sizeof(p3t_epi_t) && sizeof(EPJ_t) == sizeof(p3t_epj_t) &&
                  sizeof(SPJ_t) == sizeof(p3t_spj_t) && sizeof(Force_t) == sizeof(p3t_force_t),
              "record sizes");
static_assert(offsetof(EPI_t, id_local) == offsetof(p3t_epi_t, id_local) &&
                  offsetof(EPI_t, myrank) == offsetof(p3t_epi_t, myrank) &&
                  offsetof(EPI_t, pos) == offsetof(p3t_epi_t, pos) &&
                  offsetof(EPI_t, r_out) == offsetof(p3t_epi_t, r_out) &&
                  offsetof(EPI_t, r_search) == offsetof(p3t_epi_t, r_search),
              "EPIGrav members");
static_assert(offsetof(EPJ_t, pos) == offsetof(p3t_epj_t, pos) && offsetof(EPJ_t, r_out) == offsetof(p3t_epj_t, r_out) &&
                  offsetof(EPJ_t, r_search) == offsetof(p3t_epj_t, r_search) &&
                  offsetof(EPJ_t, id) == offsetof(p3t_epj_t, id) && offsetof(EPJ_t, mass) == offsetof(p3t_epj_t, mass) &&
                  offsetof(EPJ_t, vel) == offsetof(p3t_epj_t, vel) &&
                  offsetof(EPJ_t, acc_d) == offsetof(p3t_epj_t, acc_d),
              "EPJGrav members");
static_assert(offsetof(SPJ_t, mass) == offsetof(p3t_spj_t, mass) && offsetof(SPJ_t, pos) == offsetof(p3t_spj_t, pos) &&
                  offsetof(SPJ_t, quad) == offsetof(p3t_spj_t, xx),
              "SPJQuadrupole members");
static_assert(offsetof(Force_t, acc) == offsetof(p3t_force_t, acc) && offsetof(Force_t, phi) == offsetof(p3t_force_t, phi) &&
                  offsetof(Force_t, neighbor) == offsetof(p3t_force_t, number) && sizeof(NeighborInfo) == 16,
              "ForceGrav members");
#else
namespace PS {
typedef int S32;
}
using EPI_t = p3t_epi_t;
using EPJ_t = p3t_epj_t;
using SPJ_t = p3t_spj_t;
using Force_t = p3t_force_t;
#endif

// ---- the binding ----------------------------------
static PS::S32 DispatchP3T(const PS::S32 tag, const PS::S32 n_walk, const EPI_t *epi[], const PS::S32 n_epi[],
                           const EPJ_t *epj[], const PS::S32 n_epj[], const SPJ_t *spj[], const PS::S32 n_spj[]) {
    return p3t_soft_dispatch(tag, n_walk, (const void **)epi, n_epi, (const void **)epj, n_epj, (const void **)spj,
                             n_spj);
}
static PS::S32 RetrieveP3T(const PS::S32 tag, const PS::S32 n_walk, const PS::S32 ni[], Force_t *force[]) {
    return p3t_soft_retrieve(tag, n_walk, ni, (void **)force);
}

#ifndef GPLUM_TYPES
// ---- a stand-in for FDPS's multiwalk driver ------------------------------------
template <class T>
static bool rd(FILE *f, T *p, size_t n) {
    return std::fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s IN OUT N_WALK_LIMIT\n", argv[0]);
        return 2;
    }
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    long long hdr[3];
    double params[21];
    if (!rd(in, hdr, 3) || !rd(in, params, 21)) return 2;
    const int n = (int)hdr[0], ng = (int)hdr[1], ns = (int)hdr[2];
    std::vector<EPJ_t> epj(n);
    std::vector<SPJ_t> spj(ns);
    std::vector<int> i_off(ng + 1), j_off(ng + 1), s_off(ng + 1);
    if (!rd(in, epj.data(), n) || !rd(in, spj.data(), ns) || !rd(in, i_off.data(), ng + 1)) return 2;
    std::vector<int> i_idx(i_off[ng]);
    if (!rd(in, i_idx.data(), i_idx.size()) || !rd(in, j_off.data(), ng + 1)) return 2;
    std::vector<int> j_idx(j_off[ng]);
    if (!rd(in, j_idx.data(), j_idx.size()) || !rd(in, s_off.data(), ng + 1)) return 2;
    std::vector<int> s_idx(s_off[ng]);
    if (!rd(in, s_idx.data(), s_idx.size())) return 2;
    std::fclose(in);
    int r = p3t_init(0);
    if (r || (r = p3t_set_params(params))) {
        std::fprintf(stderr, "init failed: %d\n", r);
        return 1;
    }
    const int n_walk_limit = std::atoi(argv[3]);
    std::vector<Force_t> out(n);
    // per group, the arrays FDPS hands to a walk: EPI copies of the i-group
    // (EPIGrav::copyFromFP), EPJ and SPJ lists gathered by index
    std::vector<std::vector<EPI_t>> wi(ng);
    std::vector<std::vector<EPJ_t>> wj(ng);
    std::vector<std::vector<SPJ_t>> ws(ng);
    for (int g = 0; g < ng; g++) {
        for (int k = i_off[g]; k < i_off[g + 1]; k++) {
            EPI_t e;
            std::memcpy(&e, &epj[i_idx[k]], sizeof(EPI_t));  // EPJGrav starts with the EPIGrav members
            wi[g].push_back(e);
        }
        for (int k = j_off[g]; k < j_off[g + 1]; k++) wj[g].push_back(epj[j_idx[k]]);
        for (int k = s_off[g]; k < s_off[g + 1]; k++) ws[g].push_back(spj[s_idx[k]]);
    }
    for (int g0 = 0; g0 < ng; g0 += n_walk_limit) {
        const int nw = std::min(n_walk_limit, ng - g0);
        std::vector<const EPI_t *> pi(nw);
        std::vector<const EPJ_t *> pj(nw);
        std::vector<const SPJ_t *> ps(nw);
        std::vector<PS::S32> ni(nw), nj(nw), nsp(nw);
        for (int w = 0; w < nw; w++) {
            const int g = g0 + w;
            pi[w] = wi[g].data(); ni[w] = (PS::S32)wi[g].size();
            pj[w] = wj[g].data(); nj[w] = (PS::S32)wj[g].size();
            ps[w] = ws[g].data(); nsp[w] = (PS::S32)ws[g].size();
        }
        const int tag = (g0 / n_walk_limit) % 2;
        if ((r = DispatchP3T(tag, nw, pi.data(), ni.data(), pj.data(), nj.data(), ps.data(), nsp.data()))) {
            std::fprintf(stderr, "dispatch failed: %d\n", r);
            return 1;
        }
        std::vector<std::vector<Force_t>> fw(nw);
        std::vector<Force_t *> pf(nw);
        for (int w = 0; w < nw; w++) {
            fw[w].resize(std::max(1, ni[w]));
            pf[w] = fw[w].data();
        }
        if ((r = RetrieveP3T(tag, nw, ni.data(), pf.data()))) {
            std::fprintf(stderr, "retrieve failed: %d\n", r);
            return 1;
        }
        for (int w = 0; w < nw; w++) {
            const int g = g0 + w;
            for (int k = 0; k < ni[w]; k++) out[i_idx[i_off[g] + k]] = fw[w][k];
        }
    }
    FILE *o = std::fopen(argv[2], "wb");
    if (!o || std::fwrite(out.data(), sizeof(Force_t), n, o) != (size_t)n) return 2;
    std::fclose(o);
    return 0;
}
#endif
