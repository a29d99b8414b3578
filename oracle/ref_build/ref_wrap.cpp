// Reference build of GPLUM's hot path: GPLUM's own headers, compiled
// unchanged from the reference source tree against the single-rank PS shim in
// ../ref_shim, behind a small extern "C" surface used only by tests and by the
// golden-fixture generator.  TEST INFRASTRUCTURE ONLY: nothing in the product
// links or loads this file's output.
//
// The prelude mirrors src/main_p3t.cpp:1-63 of GPLUM (same system headers,
// macros, constants, type aliases and include order) so that the headers see
// exactly the environment they are written for.  One consequence: the C++
// <stdlib.h> brings the floating-point overloads of abs() into the global
// namespace, so the unqualified abs() of src/kepler.h:23 is the double one.
#include <iostream>
#include <fstream>
#include <vector>
#include <algorithm>
#include <stdlib.h>
#include <unistd.h>
#include <sys/stat.h>
#include <map>
#include <dirent.h>
#include <ctime>
#include <cstring>

#define USE_RE_SEARCH_NEIGHBOR
#define PIKG_USE_FDPS_VECTOR

#include <particle_simulator.hpp>
#include "../ngb_grid.h"

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
using Moment_t = MyMomentQuadrupole;
using Force_t = ForceGrav;
using FP_t = FPGrav;
using FPH_t = FPHard;

#include "energy.h"
#include "neighbor.h"
#include "gravity_hard.h"
#include "gravity_soft.h"
#include "collisionA.h"
#include "collisionB.h"
#include "hermite.h"
#include "hard.h"
#include "gravity_kernel.hpp"
#include "disk.h"
#include "read.h"
#include "time.h"
#include "func.h"

static_assert(sizeof(EPI_t) == 48, "EPIGrav layout");
static_assert(sizeof(EPJ_t) == 112, "EPJGrav layout");
static_assert(sizeof(SPJ_t) == 80, "SPJQuadrupole layout");
static_assert(sizeof(Force_t) == 32, "ForceGrav layout");

// ---------------------------------------------------------------------------
// Single-rank particle system and neighbour query (FDPS stand-ins).
template <class T>
struct RefSystem {
    std::vector<T> v;
    PS::S32 getNumberOfParticleLocal() const { return (PS::S32)v.size(); }
    PS::S32 getNumberOfParticleGlobal() const { return (PS::S32)v.size(); }
    T &operator[](PS::S32 i) { return v[i]; }
    const T &operator[](PS::S32 i) const { return v[i]; }
    // order-preserving removal
    void removeParticle(const PS::S32 *idx, PS::S32 n) {
        std::vector<char> dead(v.size(), 0);
        for (PS::S32 k = 0; k < n; k++) dead[idx[k]] = 1;
        size_t w = 0;
        for (size_t r = 0; r < v.size(); r++)
            if (!dead[r]) v[w++] = v[r];
        v.resize(w);
    }
};

// Neighbour query over the current particle set: every EPJ whose distance to
// the query particle is below max(getRSearch_i, getRSearch_j) (the symmetric
// LONG_SYMMETRY rule), in ascending particle index (oracle/ngb_grid.h).
struct RefNgbTree {
    std::vector<EPJ_t> epj;
    NgbGrid grid;
    std::vector<int> cand;
    std::vector<std::vector<EPJ_t>> out;

    void build(RefSystem<FP_t> &pp) {
        const PS::S32 n = pp.getNumberOfParticleLocal();
        epj.resize(n);
        for (PS::S32 i = 0; i < n; i++) epj[i].copyFromFP(pp[i]);
        grid.build(n, [&](int i, double &x, double &y, double &z) {
            x = epj[i].pos.x; y = epj[i].pos.y; z = epj[i].pos.z;
        }, [&](int i) { return (double)epj[i].getRSearch(); });
        out.assign(1, {});
    }
    template <class Tp>
    PS::S32 getNeighborListOneParticle(const Tp &p, EPJ_t *&next) {
        std::vector<EPJ_t> &o = out[0];
        o.clear();
        // the query particle is one of the particles the tree was built on
        // (setIDLocalAndMyrank ran before the correction); found by position
        // otherwise
        int i = (int)p.id_local;
        if (i < 0 || i >= (int)epj.size() || !(epj[i].pos == p.pos)) {
            i = -1;
            for (int k = 0; k < (int)epj.size() && i < 0; k++)
                if (epj[k].pos == p.pos && epj[k].id == p.id) i = k;
            if (i < 0) PS::Abort(-1);
        }
        grid.query(i, cand, [&](int j) {
            PS::F64vec d = epj[j].pos - p.pos;
            PS::F64 r = std::max(p.getRSearch(), epj[j].getRSearch());
            return d * d < r * r;
        });
        for (int j : cand) o.push_back(epj[j]);
        next = o.data();
        return (PS::S32)o.size();
    }
};

static RefSystem<FP_t> g_pp;
static NeighborList *g_nlist = nullptr;
static HardSystem g_hard;
static RefNgbTree g_tree;
static PS::S32 g_n_ngb_tot = 0, g_n_with_ngb = 0;

extern "C" {

// --- parameters -----------------------------------------------------------
// p[ 0] eps2      p[ 1] eps2_sun  p[ 2] m_sun     p[ 3] dt_tree   p[ 4] dt_min
// p[ 5] eta       p[ 6] eta_0     p[ 7] eta_sun   p[ 8] eta_sun0  p[ 9] alpha2
// p[10] gamma     p[11] R_cut0    p[12] R_cut1    p[13] R_search0 p[14] R_search1
// p[15] R_search2 p[16] R_search3 p[17] r_cut_min p[18] r_cut_max p[19] p_cut
// p[20] dens
void ref_set_params(const double *p) {
    FP_t::eps2 = p[0];
    FP_t::eps2_sun = p[1];
    FP_t::m_sun = p[2];
    FP_t::dt_tree = p[3];
    FP_t::dt_min = p[4];
    FP_t::eta = p[5];
    FP_t::eta_0 = p[6];
    FP_t::eta_sun = p[7];
    FP_t::eta_sun0 = p[8];
    FP_t::alpha2 = p[9];
    FP_t::setGamma(p[10]);
    FP_t::R_cut0 = p[11];
    FP_t::R_cut1 = p[12];
    FP_t::R_search0 = p[13];
    FP_t::R_search1 = p[14];
    FP_t::R_search2 = p[15];
    FP_t::R_search3 = p[16];
    FP_t::r_cut_min = p[17];
    FP_t::r_cut_max = p[18];
    FP_t::p_cut = p[19];
    FP_t::dens = p[20];
}

void ref_get_gamma_consts(double *out) {
    out[0] = FP_t::gamma;
    out[1] = FP_t::g_1_inv;
    out[2] = FP_t::g_1_inv7;
    out[3] = FP_t::w_y;
    out[4] = FP_t::f1;
}

// --- soft functors, called exactly as FDPS calls them -----------------------
void ref_epep(const void *epi, int ni, const void *epj, int nj, void *force) {
    calcForceEPEPWithSearch()((const EPI_t *)epi, ni, (const EPJ_t *)epj, nj, (Force_t *)force);
}
void ref_epsp(const void *epi, int ni, const void *spj, int nj, void *force) {
    calcForceEPSP()((const EPI_t *)epi, ni, (const SPJ_t *)spj, nj, (Force_t *)force);
}
void ref_force_clear(void *force, int n) {
    Force_t *f = (Force_t *)force;
    for (int i = 0; i < n; i++) f[i].clear();
}

// --- cutoff functions ----------------------------------------------------------
double ref_cutoff_W(double rij, double r_out_inv) { return cutoff_W(rij, r_out_inv); }
double ref_cutoff_K(double rij, double r_out_inv) { return cutoff_K(rij, r_out_inv); }
double ref_cutoff_dKdt(double rij, double r_out_inv, double alpha) {
    return cutoff_dKdt(rij, r_out_inv, alpha);
}

// --- Kepler ------------------------------------------------------------------
double ref_solve_kepler(double l, double ecc) { return solveKeplerEq(l, ecc); }

// --- particle state -------------------------------------------------------------
void ref_load(int n, const long long *id, const double *mass, const double *r_planet,
              const double *f, const double *pos, const double *vel) {
    g_pp.v.assign(n, FP_t());
    for (int i = 0; i < n; i++) {
        FP_t &p = g_pp.v[i];
        std::memset((void *)&p, 0, sizeof(FP_t));
        p.id = id[i];
        p.mass = mass[i];
        p.r_planet = r_planet[i];
        p.f = f[i];
        p.pos = PS::F64vec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p.vel = PS::F64vec(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p.neighbor.clear();
        p.time = 0.;
        p.dt = 0.;
        p.id_cluster = p.id;
        p.n_cluster = 1;
        p.inDomain = true;
        p.isSent = false;
        p.isDead = false;
        p.isMerged = false;
    }
    if (!g_nlist) g_nlist = new NeighborList();
    g_hard.initialize();
}

int ref_n() { return g_pp.getNumberOfParticleLocal(); }

// Field export.  Which field each code names is fixed by the test harness.
void ref_get_f64(int field, double *out) {
    const int n = ref_n();
    for (int i = 0; i < n; i++) {
        const FP_t &p = g_pp.v[i];
        switch (field) {
            case 0: out[3*i] = p.pos.x; out[3*i+1] = p.pos.y; out[3*i+2] = p.pos.z; break;
            case 1: out[3*i] = p.vel.x; out[3*i+1] = p.vel.y; out[3*i+2] = p.vel.z; break;
            case 2: out[3*i] = p.acc.x; out[3*i+1] = p.acc.y; out[3*i+2] = p.acc.z; break;
            case 3: out[3*i] = p.acc_d.x; out[3*i+1] = p.acc_d.y; out[3*i+2] = p.acc_d.z; break;
            case 4: out[3*i] = p.jerk_d.x; out[3*i+1] = p.jerk_d.y; out[3*i+2] = p.jerk_d.z; break;
            case 5: out[3*i] = p.acc_s.x; out[3*i+1] = p.acc_s.y; out[3*i+2] = p.acc_s.z; break;
            case 6: out[3*i] = p.jerk_s.x; out[3*i+1] = p.jerk_s.y; out[3*i+2] = p.jerk_s.z; break;
            case 10: out[i] = p.phi; break;
            case 11: out[i] = p.phi_d; break;
            case 12: out[i] = p.phi_s; break;
            case 13: out[i] = p.mass; break;
            case 14: out[i] = p.r_out; break;
            case 15: out[i] = p.r_search; break;
            case 16: out[i] = p.dt; break;
            case 17: out[i] = p.acc0; break;
            case 18: out[i] = p.time; break;
            case 19: out[i] = p.r_planet; break;
            case 20: out[i] = p.v_disp; break;
            case 21: out[i] = p.r_out_inv; break;
            case 22: out[i] = p.f; break;
            default: break;
        }
    }
}
void ref_get_i64(int field, long long *out) {
    const int n = ref_n();
    for (int i = 0; i < n; i++) {
        const FP_t &p = g_pp.v[i];
        switch (field) {
            case 0: out[i] = p.id; break;
            case 1: out[i] = p.id_cluster; break;
            case 2: out[i] = p.neighbor.number; break;
            case 3: out[i] = p.n_cluster; break;
            case 4: out[i] = p.isDead; break;
            case 5: out[i] = p.isMerged; break;
            case 6: out[i] = p.neighbor.rank; break;
            case 7: out[i] = p.neighbor.id_min; break;
            case 8: out[i] = p.neighbor.id_max; break;
            default: break;
        }
    }
}
void ref_set_f64(int field, const double *in) {
    const int n = ref_n();
    for (int i = 0; i < n; i++) {
        FP_t &p = g_pp.v[i];
        switch (field) {
            case 0: p.pos = PS::F64vec(in[3*i], in[3*i+1], in[3*i+2]); break;
            case 1: p.vel = PS::F64vec(in[3*i], in[3*i+1], in[3*i+2]); break;
            case 3: p.acc_d = PS::F64vec(in[3*i], in[3*i+1], in[3*i+2]); break;
            case 14: p.r_out = in[i]; break;
            case 15: p.r_search = in[i]; break;
            case 21: p.r_out_inv = in[i]; break;
            default: break;
        }
    }
}

// GPLUM's snapshot writers on the reference system's bodies: FileHeader
// (src/energy.h:65-127) then FPGrav::writeAscii / writeBinary
// (src/particle.h:845-876) of every body in order -- the single-process
// behaviour of FDPS's writeParticleAscii / writeParticleBinary, which
// makeSnap / makeSnapTmp call (src/func.h:53-80).  e_init / e_now: the seven
// Energy fields in declaration order.
int ref_write_snapshot(const char *path, int binary, double time, int id_next, const double *e_init,
                       const double *e_now) {
    Energy a, b;
    double *fa[7] = {&a.etot, &a.ekin, &a.ephi_sun, &a.ephi_planet, &a.ephi, &a.ephi_d, &a.edisp};
    double *fb[7] = {&b.etot, &b.ekin, &b.ephi_sun, &b.ephi_planet, &b.ephi, &b.ephi_d, &b.edisp};
    for (int k = 0; k < 7; k++) {
        *fa[k] = e_init[k];
        *fb[k] = e_now[k];
    }
    FileHeader h(ref_n(), id_next, time, a, b);
    FILE *fp = std::fopen(path, binary ? "wb" : "w");
    if (!fp) return -1;
    if (binary) {
        h.writeBinary(fp);
        for (int i = 0; i < ref_n(); i++) g_pp[i].writeBinary(fp);
    } else {
        h.writeAscii(fp);
        for (int i = 0; i < ref_n(); i++) g_pp[i].writeAscii(fp);
    }
    std::fclose(fp);
    return 0;
}
// sizeof(FPGrav), sizeof(FileHeader) and the byte offsets of FPGrav's members
// in GPLUM's compiled class
void ref_fpgrav_layout(long long *out) {
    FP_t p;
    const char *b = (const char *)&p;
    long long v[] = {(long long)sizeof(FP_t), (long long)sizeof(FileHeader),
                     (long long)((const char *)&p.id_local - b), (long long)((const char *)&p.myrank - b),
                     (long long)((const char *)&p.pos - b), (long long)((const char *)&p.r_out - b),
                     (long long)((const char *)&p.r_search - b), (long long)((const char *)&p.id - b),
                     (long long)((const char *)&p.mass - b), (long long)((const char *)&p.vel - b),
                     (long long)((const char *)&p.acc_d - b), (long long)((const char *)&p.acc - b),
                     (long long)((const char *)&p.acc_s - b), (long long)((const char *)&p.jerk_d - b),
                     (long long)((const char *)&p.jerk_s - b), (long long)((const char *)&p.acc_gd - b),
                     (long long)((const char *)&p.phi - b), (long long)((const char *)&p.phi_d - b),
                     (long long)((const char *)&p.phi_s - b), (long long)((const char *)&p.v_disp - b),
                     (long long)((const char *)&p.r_out_inv - b), (long long)((const char *)&p.time - b),
                     (long long)((const char *)&p.dt - b), (long long)((const char *)&p.acc0 - b),
                     (long long)((const char *)&p.r_planet - b), (long long)((const char *)&p.f - b),
                     (long long)((const char *)&p.neighbor - b), (long long)((const char *)&p.id_cluster - b),
                     (long long)((const char *)&p.n_cluster - b), (long long)((const char *)&p.inDomain - b),
                     (long long)((const char *)&p.isSent - b), (long long)((const char *)&p.isDead - b),
                     (long long)((const char *)&p.isMerged - b)};
    for (size_t k = 0; k < sizeof v / sizeof v[0]; k++) out[k] = v[k];
}

// setIDLocalAndMyrank (src/func.h:135-149) followed by setCutoffRadii
// (src/particle.h:1528-1543).
void ref_set_id_local() {
    for (int i = 0; i < ref_n(); i++) {
        g_pp[i].id_local = i;
        g_pp[i].myrank = 0;
        g_pp[i].inDomain = true;
        g_pp[i].isSent = false;
    }
}
void ref_set_cutoff_radii() { setCutoffRadii(g_pp); }
void ref_set_r_planet() { for (int i = 0; i < ref_n(); i++) g_pp[i].setRPlanet(); }

// Soft force over caller-supplied interaction lists.  Group g owns i-particles
// i_idx[i_off[g] .. i_off[g+1]), EPJ particle indices j_idx[j_off[g] ..], and
// superparticles spj[s_idx[s_off[g] ..]] (spj is an array of SPJQuadrupole).
// Forces are cleared, both functors accumulate, then copyFromForce
// (src/particle.h:761-766) writes them back.
void ref_soft_force(int n_group, const int *i_off, const int *i_idx, const int *j_off,
                    const int *j_idx, const int *s_off, const int *s_idx, const void *spj_all) {
    const SPJ_t *spj_arr = (const SPJ_t *)spj_all;
#pragma omp parallel for schedule(dynamic, 1)
    for (int g = 0; g < n_group; g++) {
        const int ni = i_off[g + 1] - i_off[g];
        const int nj = j_off[g + 1] - j_off[g];
        const int ns = s_off[g + 1] - s_off[g];
        std::vector<EPI_t> epi(ni);
        std::vector<EPJ_t> epj(nj);
        std::vector<SPJ_t> spj(ns);
        std::vector<Force_t> force(ni);
        for (int k = 0; k < ni; k++) { epi[k].copyFromFP(g_pp[i_idx[i_off[g] + k]]); force[k].clear(); }
        for (int k = 0; k < nj; k++) epj[k].copyFromFP(g_pp[j_idx[j_off[g] + k]]);
        for (int k = 0; k < ns; k++) spj[k] = spj_arr[s_idx[s_off[g] + k]];
        calcForceEPEPWithSearch()(epi.data(), ni, epj.data(), nj, force.data());
        calcForceEPSP()(epi.data(), ni, spj.data(), ns, force.data());
        for (int k = 0; k < ni; k++) g_pp[i_idx[i_off[g] + k]].copyFromForce(force[k]);
    }
}

// correctForceLong / correctForceLongInitial (src/gravity_soft.h:245-528).
void ref_correct(int initial) {
    g_tree.build(g_pp);
    if (initial)
        correctForceLongInitial(g_pp, g_tree, *g_nlist, g_n_ngb_tot, g_n_with_ngb);
    else
        correctForceLong(g_pp, g_tree, *g_nlist, g_n_ngb_tot, g_n_with_ngb);
}
int ref_n_ngb_tot() { return g_n_ngb_tot; }
int ref_n_with_ngb() { return g_n_with_ngb; }
int ref_n_pairs() { return (int)g_nlist->pair_list.size(); }
void ref_get_pairs(int *out) {
    for (size_t k = 0; k < g_nlist->pair_list.size(); k++) {
        out[2 * k] = g_nlist->pair_list[k].first;
        out[2 * k + 1] = g_nlist->pair_list[k].second;
    }
}
int ref_n_list_size(int i) { return (int)g_nlist->n_list[i].size(); }
void ref_n_list(int i, long long *out) {
    for (size_t k = 0; k < g_nlist->n_list[i].size(); k++) out[k] = g_nlist->n_list[i][k].id;
}

// cluster labelling (src/neighbor.h:800-839), with the single-rank exchange
// loop of src/main_p3t.cpp:472-487.
void ref_cluster() {
    g_nlist->createConnectedRankList();
    g_nlist->resizeExDataBuffer();
    g_nlist->createNeighborCluster(g_pp);
    g_nlist->inputExData(g_pp);
    g_nlist->selectSendRecvParticle(g_pp);
}

// velKick (src/gravity_soft.h:5-12)
void ref_kick() { velKick(g_pp); }

// makeList + timeIntegrate (src/hard.h:321-829).  Returns the number of
// collisions; collision pairs (impactor id, target id) go to col_out.
int ref_hard(int istep, long long *col_out, int col_cap, double *edisp_out) {
    static ExParticleSystem<FP_t> ex;
    ex.initialize();
    ex.resize(0, 0);
    g_hard.clear();
    g_hard.reserve_hard(2 * (g_n_with_ngb + 1));
    int n_in = g_hard.makeList(g_pp, ex);
    int n_out = g_hard.timeIntegrate(g_pp, ex, g_nlist->n_list, istep);
    if (n_in != n_out) return -1;
    int nc = (int)g_hard.collision_list.size();
    for (int k = 0; k < nc && k < col_cap; k++) {
        col_out[2 * k] = g_hard.collision_list[k].id_imp;
        col_out[2 * k + 1] = g_hard.collision_list[k].id_tar;
    }
    edisp_out[0] = g_hard.getEnergyDissipationGlobal();
    edisp_out[1] = g_hard.getHardEnergyDissipationGlobal();
    return nc;
}
// per-collision energy changes {edisp, edisp_d} in collision-list order
void ref_col_edisp(int k, double *out) {
    out[0] = g_hard.collision_list[k].edisp;
    out[1] = g_hard.collision_list[k].edisp_d;
}
int ref_n_cluster() { return g_hard.getNumberOfClusterLocal(); }
int ref_n_isolated() { return g_hard.getNumberOfIsolatedParticleLocal(); }
// the figure GPLUM logs as the largest cluster (src/hard.h:143-149, as written)
int ref_largest_cluster() { return g_hard.getNumberOfParticleInLargestClusterLocal(); }

// energy (src/energy.h:29-63): out = {etot, ekin, ephi_sun, ephi, ephi_d}
void ref_energy(double *out) {
    Energy e;
    e.calcEnergy(g_pp);
    out[0] = e.etot;
    out[1] = e.ekin;
    out[2] = e.ephi_sun;
    out[3] = e.ephi;
    out[4] = e.ephi_d;
}

// MergeParticle (src/func.h:160-207): folds dead twins into their targets.
void ref_merge(int n_col, double *edisp) { MergeParticle(g_pp, n_col, *edisp); }
// removeParticlesOutOfBoundary (src/func.h:209-355); its report goes nowhere
int ref_remove(double r_max, double r_min, double *edisp) {
    std::ofstream sink("/dev/null");
    return removeParticlesOutOfBoundary(g_pp, *edisp, r_max, r_min, sink);
}

}  // extern "C"

// One collision in isolation, for pinning the fragmentation model: a cluster
// of n FPHard records (26 doubles each, layout of oracle/harness.py
// UNIT_FIELDS), its merge list as (target, twin) pairs in insertion order,
// and the colliding pair; runs Collision::inputPair, collisionOutcome,
// setParticle, calcEnergyDissipation and setNeighbors (src/collisionA.h,
// src/collisionB.h; KOMINAMI when built with it, drand48 seeded by the
// caller through ref_srand48), then clears the impactor's merged flag as the
// Hermite loop does.  Writes the n + n_frag records, the energy
// changes {edisp, edisp_d} and the fragment counter; returns n_frag.
extern "C" void ref_srand48(long seed) { srand48(seed); }
extern "C" void ref_set_frag(double a_frag, int n_frag, double m_min) {
#ifdef KOMINAMI
    Collision::a_frag = a_frag;
    Collision::N_frag = n_frag;
#else
    (void)a_frag;
    (void)n_frag;
#endif
    Collision0::m_min = m_min;
}
// Collision0::write2File of each unit collision, appended to this file when set
static std::string g_col_file;
extern "C" void ref_set_collision_file(const char *path) { g_col_file = path ? path : ""; }

extern "C" int ref_collide_unit(int n, const double *in, int n_tw, const int *tw, int imp, int tar,
                                long long *id_next, double *out, int cap, double *edisp) {
    std::vector<FPHard> pp(n);
    for (int i = 0; i < n; i++) {
        const double *r = in + 26 * i;
        FPHard &p = pp[i];
        p.pos = PS::F64vec(r[0], r[1], r[2]);
        p.vel = PS::F64vec(r[3], r[4], r[5]);
        p.mass = r[6]; p.r_planet = r[7]; p.f = r[8]; p.r_out = r[9]; p.r_out_inv = r[10];
        p.r_search = r[11]; p.v_disp = r[12]; p.time = r[13]; p.time_c = r[14]; p.dt = r[15];
        p.phi = r[16]; p.phi_d = r[17]; p.phi_s = r[18]; p.acc0 = r[19];
        p.id = (PS::S64)r[20]; p.id_cluster = (PS::S64)r[21]; p.neighbor.number = (PS::S32)r[22];
        p.isDead = r[23] != 0.; p.isMerged = r[24] != 0.;
    }
    std::multimap<PS::S32, PS::S32> merge_list;
    for (int k = 0; k < n_tw; k++) merge_list.insert(std::make_pair(tw[2 * k], tw[2 * k + 1]));
    Collision col;
    std::vector<FPHard> pfrag;
    col.inputPair(pp, merge_list, std::make_pair(imp, tar));
    PS::S64 idn = *id_next;
    const int nf = col.collisionOutcome(pfrag);
    col.setParticle(pp, pfrag, merge_list, idn);
    edisp[0] = col.calcEnergyDissipation(pp, merge_list);
    edisp[1] = col.getHardEnergyDissipation();
    col.setNeighbors(pp);
    if (!g_col_file.empty()) {
        std::ofstream f(g_col_file, std::ios::app);
        col.write2File(f);
    }
    // the merge-list bookkeeping that follows in src/hermite.h:413-423
    if (col.flag_merge && pp[imp].isMerged) pp[imp].isMerged = false;
    *id_next = idn;
    for (int i = 0; i < (int)pp.size() && i < cap; i++) {
        double *r = out + 26 * i;
        const FPHard &p = pp[i];
        r[0] = p.pos.x; r[1] = p.pos.y; r[2] = p.pos.z; r[3] = p.vel.x; r[4] = p.vel.y; r[5] = p.vel.z;
        r[6] = p.mass; r[7] = p.r_planet; r[8] = p.f; r[9] = p.r_out; r[10] = p.r_out_inv;
        r[11] = p.r_search; r[12] = p.v_disp; r[13] = p.time; r[14] = p.time_c; r[15] = p.dt;
        r[16] = p.phi; r[17] = p.phi_d; r[18] = p.phi_s; r[19] = p.acc0;
        r[20] = (double)p.id; r[21] = (double)p.id_cluster; r[22] = p.neighbor.number;
        r[23] = p.isDead; r[24] = p.isMerged; r[25] = 0.;
    }
    return nf;
}
