// CPU restatement of GPLUM's P3T hot path.  TEST INFRASTRUCTURE ONLY: the
// checker for tests/, __graft_entry__.smoke() and the CPU baseline of
// bench.py.  Nothing in the product links or loads it.
//
// Every function restates one reference function (file:line cited beside it)
// with the same formulas and the same order of floating-point operations, so
// that, compiled without FMA contraction, it rounds exactly as the reference
// does.  Sums over lists run in list order.  The extern "C" surface mirrors
// oracle/ref_build/ref_wrap.cpp with the prefix orc_.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <limits>
#include <map>
#include <numeric>
#include <vector>

#include <omp.h>

#include "ngb_grid.h"
#include "p3t_oracle.h"

namespace {

// std::min / std::max semantics, NaN behaviour included
template <class T> inline T lo_of(T a, T b) { return (b < a) ? b : a; }
template <class T> inline T hi_of(T a, T b) { return (a < b) ? b : a; }

struct V3 {
    double x, y, z;
};
inline V3 v3(double a, double b, double c) { return V3{a, b, c}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 &operator+=(V3 &a, V3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
inline V3 &operator-=(V3 &a, V3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
const V3 ZERO = {0., 0., 0.};

// --- record layouts crossing the boundary (FDPS classes of GPLUM) ---------
struct EPI {  // src/particle.h:93-141
    int32_t id_local, myrank;
    double pos[3];
    double r_out, r_search;
};
struct EPJ {  // src/particle.h:149-170
    int32_t id_local, myrank;
    double pos[3];
    double r_out, r_search;
    int64_t id;
    double mass, vel[3], acc_d[3];
};
struct SPJ {  // FDPS SPJQuadrupole
    double mass, pos[3], xx, yy, zz, xy, xz, yz;
};
struct FORCE {  // src/particle.h:16-86
    float acc[3], phi;
    int32_t number, rank, id_max, id_min;
};
static_assert(sizeof(EPI) == 48, "EPI");
static_assert(sizeof(EPJ) == 112, "EPJ");
static_assert(sizeof(SPJ) == 80, "SPJ");
static_assert(sizeof(FORCE) == 32, "FORCE");

// --- run parameters (FPGrav statics, src/particle.h:917-961) ---------------
struct Params {
    double eps2 = 0., eps2_sun = 0., m_sun = 1., dt_tree = 1. / 32., dt_min = 1. / 8192.;
    double eta = 0.01, eta_0 = 0.001, eta_sun = 0.01, eta_sun0 = 0.001, alpha2 = 1.;
    double gamma = 0.5, g_1_inv = -2., g_1_inv7 = -128., w_y = 0., f1 = 0.;
    double R_cut0 = 2., R_cut1 = 8., R_search0 = 1., R_search1 = 4., R_search2 = 1., R_search3 = 4.;
    double r_cut_min = 0., r_cut_max = 0., p_cut = 0., dens = 5.049667e6;
};
Params P;

// FPGrav::setGamma, src/particle.h:619-633
void set_gamma(double g) {
    P.gamma = g;
    P.g_1_inv = 1. / (g - 1.);
    const double g2 = g * g;
    const double gi3 = P.g_1_inv * P.g_1_inv * P.g_1_inv;
    P.g_1_inv7 = gi3 * gi3 * P.g_1_inv;
    P.w_y = 7. / 3. * ((((((g - 9.) * g + 45.) * g - 60. * std::log(g)) * g - 45.) * g + 9.) * g - 1.) *
            P.g_1_inv7;
    P.f1 = (-10. / 3. + 14. * (g + 1.) - 21. * ((g + 3.) * g + 1.) + 35. / 3. * (((g + 9.) * g + 9.) * g + 1.) -
            70. * ((g + 3.) * g + 1.) * g + 210. * (g + 1.) * g2 + (((g - 7.) * g + 21.) * g - 35.) * g2 * g2) *
           P.g_1_inv7;
}

// --- cutoff functions, src/cutfunc.h:4-66 ----------------------------------
double cut_f(double y) {  // cutoff_f
    const double g = P.gamma, g2 = g * g;
    return (((((((-10. / 3. * y + 14. * (g + 1.)) * y - 21. * ((g + 3.) * g + 1.)) * y +
                35. / 3. * (((g + 9.) * g + 9.) * g + 1.)) * y - 70. * ((g + 3.) * g + 1.) * g) * y +
              210. * (g + 1.) * g2) * y - 140. * g2 * g * std::log(y)) * y +
            (((g - 7.) * g + 21.) * g - 35.) * g2 * g2) * P.g_1_inv7;
}
double cut_W(double rij, double r_out_inv) {  // cutoff_W
    const double y = rij * r_out_inv;
    if (1.0 <= y) return 1.0;
    if (y <= P.gamma) return y * P.w_y;
    return cut_f(y) + y * (1. - P.f1);
}
double cut_Kx(double x) {  // cutoff_K(x)
    if (x < 0.) return 0.;
    if (x >= 1.) return 1.;
    const double x2 = x * x;
    return (((-20. * x + 70.) * x - 84.) * x + 35.) * x2 * x2;
}
double cut_dKdr(double x, double r_out_inv) {  // cutoff_dKdr
    const double x_1 = x - 1.;
    return (x < 0. || x >= 1.) ? 0. : (140. * x * x * x * x_1 * x_1 * x_1 * r_out_inv * P.g_1_inv);
}
double cut_K(double rij, double r_out_inv) {  // cutoff_K(rij, r_out_inv)
    return cut_Kx((P.gamma - rij * r_out_inv) * P.g_1_inv);
}
double cut_dKdt(double rij, double r_out_inv, double alpha) {  // cutoff_dKdt
    const double x = (P.gamma - rij * r_out_inv) * P.g_1_inv;
    return alpha * rij * cut_dKdr(x, r_out_inv);
}
double cut_W2(double dr2, double a, double b) { return cut_W(std::sqrt(dr2), lo_of(a, b)); }

// --- soft functors ------------------------------------------------------------
// EP-EP with neighbour screen, src/gravity_kernel.hpp:25-121 (default,
// non-PIKG build).  FP64 displacement from epi[0], then FP32 arithmetic.
void epep_f32(const EPI *epi, int ni, const EPJ *epj, int nj, FORCE *force) {
    const float eps2 = (float)P.eps2;
    std::vector<float> jx(nj), jy(nj), jz(nj), jm(nj), jro(nj), jrs(nj);
    std::vector<int32_t> jid(nj), jrk(nj);
    const double *o = epi[0].pos;
    for (int j = 0; j < nj; j++) {
        jx[j] = (float)(epj[j].pos[0] - o[0]);
        jy[j] = (float)(epj[j].pos[1] - o[1]);
        jz[j] = (float)(epj[j].pos[2] - o[2]);
        jm[j] = (float)epj[j].mass;
        jro[j] = (float)epj[j].r_out;
        jrs[j] = (float)epj[j].r_search;
        jid[j] = epj[j].id_local;
        jrk[j] = epj[j].myrank;
    }
    for (int i = 0; i < ni; i++) {
        float ax = 0.f, ay = 0.f, az = 0.f, pot = 0.f;
        int32_t ngb = 0, rk = 0, idmax = -1, idmin = INT_MAX;
        const float xi = (float)(epi[i].pos[0] - o[0]);
        const float yi = (float)(epi[i].pos[1] - o[1]);
        const float zi = (float)(epi[i].pos[2] - o[2]);
        const float roi = (float)epi[i].r_out, rsi = (float)epi[i].r_search;
        const int32_t idi = epi[i].id_local, rki = epi[i].myrank;
        for (int j = 0; j < nj; j++) {
            const float rx = xi - jx[j], ry = yi - jy[j], rz = zi - jz[j];
            const float ro = hi_of(roi, jro[j]);
            const float rs = hi_of(rsi, jrs[j]);
            const float ro2 = ro * ro;
            const float rs2 = rs * rs * 1.0201f;
            const float r2_real = rx * rx + ry * ry + rz * rz + eps2;
            const float r2 = hi_of(r2_real, ro2);
            float rinv = (float)(1.0f / ::sqrt((double)r2));  // ::sqrt is the double overload, as in the functor
            const float t = 3.0f - r2 * (rinv * rinv);
            rinv *= (t * 0.5f);
            const float r2inv = rinv * rinv;
            const float p = rinv * jm[j];
            ax += p * r2inv * rx;
            ay += p * r2inv * ry;
            az += p * r2inv * rz;
            pot += p;
            if (r2_real < rs2 && (idi != jid[j] || rki != jrk[j])) {
                ngb += 1;
                rk += std::abs(rki - jrk[j]);
                idmax = hi_of(idmax, jid[j]);
                idmin = lo_of(idmin, jid[j]);
            }
        }
        force[i].acc[0] -= ax;
        force[i].acc[1] -= ay;
        force[i].acc[2] -= az;
        force[i].phi -= pot;
        force[i].number += ngb;
        force[i].rank += rk;
        force[i].id_max = hi_of(idmax, force[i].id_max);
        force[i].id_min = lo_of(idmin, force[i].id_min);
    }
}

// EP-SP quadrupole, src/gravity_kernel.hpp:138-238.  trace_mode 0 keeps the
// default build's trace xx+yy+xx (src/gravity_kernel.hpp:177); 1 uses the
// PIKG spec's xx+yy+zz (src/gravity_kernel_epsp.pikg:75).
void epsp_f32(const EPI *epi, int ni, const SPJ *spj, int nj, FORCE *force, int trace_mode) {
    const float eps2 = (float)P.eps2;
    std::vector<float> jx(nj), jy(nj), jz(nj), jm(nj), qxx(nj), qyy(nj), qzz(nj), qxy(nj), qyz(nj),
        qzx(nj), tr(nj);
    const double *o = epi[0].pos;
    for (int j = 0; j < nj; j++) {
        jx[j] = (float)(spj[j].pos[0] - o[0]);
        jy[j] = (float)(spj[j].pos[1] - o[1]);
        jz[j] = (float)(spj[j].pos[2] - o[2]);
        jm[j] = (float)spj[j].mass;
        qxx[j] = (float)spj[j].xx;
        qyy[j] = (float)spj[j].yy;
        qzz[j] = (float)spj[j].zz;
        qxy[j] = (float)spj[j].xy;
        qyz[j] = (float)spj[j].yz;
        qzx[j] = (float)spj[j].xz;
        tr[j] = trace_mode ? (float)(spj[j].xx + spj[j].yy + spj[j].zz)
                           : (float)(spj[j].xx + spj[j].yy + spj[j].xx);
    }
    for (int i = 0; i < ni; i++) {
        const float xi = (float)(epi[i].pos[0] - o[0]);
        const float yi = (float)(epi[i].pos[1] - o[1]);
        const float zi = (float)(epi[i].pos[2] - o[2]);
        float ax = 0.f, ay = 0.f, az = 0.f, pot = 0.f;
        for (int j = 0; j < nj; j++) {
            const float rx = jx[j] - xi, ry = jy[j] - yi, rz = jz[j] - zi;
            const float r2 = rx * rx + ry * ry + rz * rz + eps2;
            float rinv = (float)(1.0f / ::sqrt((double)r2));  // ::sqrt is the double overload, as in the functor
            const float t = 3.0f - r2 * (rinv * rinv);
            rinv *= (t * 0.5f);
            const float r2inv = rinv * rinv;
            const float r3inv = r2inv * rinv;
            const float r4inv = r2inv * r2inv;
            const float r5inv = r2inv * r3inv;
            const float sxx = 3.0f * qxx[j] - tr[j];
            const float syy = 3.0f * qyy[j] - tr[j];
            const float szz = 3.0f * qzz[j] - tr[j];
            const float sxy = 3.0f * qxy[j];
            const float syz = 3.0f * qyz[j];
            const float szx = 3.0f * qzx[j];
            const float mtr = -(eps2 * tr[j]);
            const float qrx = sxx * rx + sxy * ry + szx * rz;
            const float qry = syy * ry + syz * rz + sxy * rx;
            const float qrz = szz * rz + szx * rx + syz * ry;
            const float rqr = mtr + qrx * rx + qry * ry + qrz * rz;
            const float rqr_r4 = rqr * r4inv;
            const float meff = jm[j] + 0.5f * rqr_r4;
            const float meff3 = (jm[j] + 2.5f * rqr_r4) * r3inv;
            ax += r5inv * qrx - meff3 * rx;
            ay += r5inv * qry - meff3 * ry;
            az += r5inv * qrz - meff3 * rz;
            pot += meff * rinv;
        }
        force[i].acc[0] -= ax;
        force[i].acc[1] -= ay;
        force[i].acc[2] -= az;
        force[i].phi -= pot;
    }
}

// FP64 restatements: the same formulas with every quantity in double and an
// exact 1/sqrt (no Newton step needed).  acc4 = {ax, ay, az, phi}.
void epep_f64(const EPI *epi, int ni, const EPJ *epj, int nj, double *acc4, int *ngb4) {
    for (int i = 0; i < ni; i++) {
        double ax = 0., ay = 0., az = 0., pot = 0.;
        int32_t ngb = 0, rk = 0, idmax = -1, idmin = INT_MAX;
        for (int j = 0; j < nj; j++) {
            const double rx = epi[i].pos[0] - epj[j].pos[0];
            const double ry = epi[i].pos[1] - epj[j].pos[1];
            const double rz = epi[i].pos[2] - epj[j].pos[2];
            const double ro = hi_of(epi[i].r_out, epj[j].r_out);
            const double rs = hi_of(epi[i].r_search, epj[j].r_search);
            const double r2_real = rx * rx + ry * ry + rz * rz + P.eps2;
            const double r2 = hi_of(r2_real, ro * ro);
            const double rinv = 1.0 / std::sqrt(r2);
            const double p = rinv * epj[j].mass;
            ax += p * rinv * rinv * rx;
            ay += p * rinv * rinv * ry;
            az += p * rinv * rinv * rz;
            pot += p;
            if (r2_real < rs * rs * 1.0201 && (epi[i].id_local != epj[j].id_local || epi[i].myrank != epj[j].myrank)) {
                ngb += 1;
                rk += std::abs(epi[i].myrank - epj[j].myrank);
                idmax = hi_of(idmax, epj[j].id_local);
                idmin = lo_of(idmin, epj[j].id_local);
            }
        }
        acc4[4 * i + 0] -= ax;
        acc4[4 * i + 1] -= ay;
        acc4[4 * i + 2] -= az;
        acc4[4 * i + 3] -= pot;
        if (ngb4) {
            ngb4[4 * i + 0] += ngb;
            ngb4[4 * i + 1] += rk;
            ngb4[4 * i + 2] = hi_of(idmax, ngb4[4 * i + 2]);
            ngb4[4 * i + 3] = lo_of(idmin, ngb4[4 * i + 3]);
        }
    }
}

void epsp_f64(const EPI *epi, int ni, const SPJ *spj, int nj, double *acc4, int trace_mode) {
    for (int i = 0; i < ni; i++) {
        double ax = 0., ay = 0., az = 0., pot = 0.;
        for (int j = 0; j < nj; j++) {
            const double rx = spj[j].pos[0] - epi[i].pos[0];
            const double ry = spj[j].pos[1] - epi[i].pos[1];
            const double rz = spj[j].pos[2] - epi[i].pos[2];
            const double tr = trace_mode ? spj[j].xx + spj[j].yy + spj[j].zz : spj[j].xx + spj[j].yy + spj[j].xx;
            const double r2 = rx * rx + ry * ry + rz * rz + P.eps2;
            const double rinv = 1.0 / std::sqrt(r2);
            const double r2inv = rinv * rinv, r3inv = r2inv * rinv, r4inv = r2inv * r2inv, r5inv = r2inv * r3inv;
            const double sxx = 3. * spj[j].xx - tr, syy = 3. * spj[j].yy - tr, szz = 3. * spj[j].zz - tr;
            const double sxy = 3. * spj[j].xy, syz = 3. * spj[j].yz, szx = 3. * spj[j].xz;
            const double mtr = -(P.eps2 * tr);
            const double qrx = sxx * rx + sxy * ry + szx * rz;
            const double qry = syy * ry + syz * rz + sxy * rx;
            const double qrz = szz * rz + szx * rx + syz * ry;
            const double rqr = mtr + qrx * rx + qry * ry + qrz * rz;
            const double rqr_r4 = rqr * r4inv;
            const double meff = spj[j].mass + 0.5 * rqr_r4;
            const double meff3 = (spj[j].mass + 2.5 * rqr_r4) * r3inv;
            ax += r5inv * qrx - meff3 * rx;
            ay += r5inv * qry - meff3 * ry;
            az += r5inv * qrz - meff3 * rz;
            pot += meff * rinv;
        }
        acc4[4 * i + 0] -= ax;
        acc4[4 * i + 1] -= ay;
        acc4[4 * i + 2] -= az;
        acc4[4 * i + 3] -= pot;
    }
}

// --- particle state (FPGrav / FPHard fields the path touches) ---------------
struct Ptcl {
    int64_t id;
    double mass, r_planet, f;
    V3 pos, vel, acc, acc_d, jerk_d, acc_s, jerk_s;
    double phi, phi_d, phi_s;
    double r_out, r_out_inv, r_search, v_disp;
    double time, dt, acc0;
    int32_t number, rank, id_max, id_min;  // NeighborInfo
    int64_t id_cluster;
    int32_t n_cluster;
    bool dead, merged;
    int32_t id_local;
};

struct HPtcl : Ptcl {  // FPHard additions, src/particle.h:970-997
    V3 x0, v0, a0_s, j0_s, a0_d, j0_d, xp, vp, a2_s, a3_s, a2_d, a3_d;
    double time_c;
};

std::vector<Ptcl> S;                          // the particle system
std::vector<std::vector<int64_t>> NLIST;      // neighbour ids per particle
std::vector<std::pair<int, int>> PAIRS;       // local pairs i<j
int N_NGB_TOT = 0, N_WITH_NGB = 0, N_CLUSTER = 0, N_ISO = 0;

// dt criteria, src/particle.h:345-383
double dt2nd(double eta, double alpha2, double acc0, V3 acc, V3 jerk) {
    const double Acc2 = dot(acc, acc) + alpha2 * acc0 * acc0;
    const double Jerk2 = dot(jerk, jerk);
    return (Jerk2 > 0.) ? eta * std::sqrt(Acc2 / Jerk2) : std::numeric_limits<double>::max();
}
double dt4th(double eta, double alpha2, double acc0, V3 acc, V3 jerk, V3 snap, V3 crac) {
    const double Acc = std::sqrt(dot(acc, acc) + alpha2 * acc0 * acc0);
    const double Jerk2 = dot(jerk, jerk);
    const double Jerk = std::sqrt(Jerk2);
    const double Snap2 = dot(snap, snap);
    const double Snap = std::sqrt(Snap2);
    const double Crac = std::sqrt(dot(crac, crac));
    return (Jerk > 0.) ? eta * std::sqrt((Acc * Snap + Jerk2) / (Jerk * Crac + Snap2))
                       : std::numeric_limits<double>::max();
}

// FPGrav::calcDeltatInitial, src/particle.h:886-914
void dt_initial(Ptcl &p) {
    double dt_next = 0.5 * P.dt_tree;
    const double dt_1 = lo_of(dt2nd(P.eta_0, P.alpha2, p.acc0, p.acc_d, p.jerk_d),
                              dt2nd(P.eta_sun0, P.alpha2, 0., p.acc_s, p.jerk_s));
    double rem = std::fmod(p.time, dt_next);
    while (rem != 0.0) {
        dt_next *= 0.5;
        rem = std::fmod(p.time, dt_next);
    }
    if (p.dt > 0.)
        while (2. * p.dt < dt_next) dt_next *= 0.5;
    while (dt_1 < dt_next) dt_next *= 0.5;
    if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
    p.dt = dt_next;
}

// FPHard::calcDeltat, src/particle.h:1276-1314
void dt_hermite(HPtcl &p) {
    double dt_next = lo_of(2. * p.dt, 0.5 * P.dt_tree);
    const double dt_1 = lo_of(dt4th(P.eta, P.alpha2, p.acc0, p.acc_d, p.jerk_d, p.a2_d, p.a3_d),
                              dt4th(P.eta_sun, P.alpha2, 0., p.acc_s, p.jerk_s, p.a2_s, p.a3_s));
    double rem = std::fmod(p.time, dt_next);
    while (rem != 0.0) {
        dt_next *= 0.5;
        rem = std::fmod(p.time, dt_next);
    }
    while (dt_1 < dt_next && 0.5 * p.dt < dt_next) dt_next *= 0.5;
    if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
    p.dt = dt_next;
}

// calcStarGravity on (x, v), src/gravity_hard.h:5-111
void sun_force(V3 x, V3 v, V3 &acc_s, V3 &jerk_s, double *phi_s) {
    const V3 dr = v3(-x.x, -x.y, -x.z), dv = v3(-v.x, -v.y, -v.z);
    const double r2inv = 1. / (dot(dr, dr) + P.eps2_sun);
    const double rinv = std::sqrt(r2inv);
    const double r3inv = rinv * r2inv;
    const double mr3 = P.m_sun * r3inv;
    const double alpha = dot(dr, dv) * r2inv;
    if (phi_s) *phi_s = -P.m_sun * rinv;
    acc_s = mr3 * dr;
    jerk_s = mr3 * (dv - 3. * alpha * dr);
}

// FPHard::predict / correct, src/particle.h:1183-1274
void predict(HPtcl &p, double Dt) {
    p.x0 = p.pos; p.v0 = p.vel; p.a0_s = p.acc_s; p.j0_s = p.jerk_s; p.j0_d = p.jerk_d; p.a0_d = p.acc_d;
    const V3 a = p.acc_s + p.acc_d, j = p.jerk_s + p.jerk_d;
    p.xp = p.pos + Dt * (p.vel + Dt * (0.5 * a + 1.6666666666666667e-1 * Dt * j));
    p.vp = p.vel + Dt * (a + Dt * 0.5 * j);
}
void correct(HPtcl &p, double Dt) {
    const double Dt2 = Dt * Dt, Di = 1. / Dt, Di2 = Di * Di, Di3 = Di2 * Di;
    const V3 Am_s = p.acc_s - p.a0_s, J0_s = Dt * p.j0_s, J1_s = Dt * p.jerk_s;
    const V3 A2_s = 3. * Am_s - (J1_s + 2. * J0_s);
    const V3 A3_s = -2. * Am_s + (J1_s + J0_s);
    p.a2_s = 2. * Di2 * (A2_s + 3. * A3_s);
    p.a3_s = 6. * Di3 * A3_s;
    const V3 Am_d = p.acc_d - p.a0_d, J0_d = p.j0_d * Dt, J1_d = p.jerk_d * Dt;
    const V3 A2_d = 3. * Am_d - (J1_d + 2. * J0_d);
    const V3 A3_d = -2. * Am_d + (J1_d + J0_d);
    p.a2_d = 2. * (A2_d + 3. * A3_d) * Di2;
    p.a3_d = 6. * A3_d * Di3;
    const V3 A2 = A2_s + A2_d, A3 = A3_s + A3_d;
    p.pos = p.xp + 1.6666666666666667e-2 * Dt2 * (5. * A2 + 3. * 1.1666666666666667e-3 * A3);
    p.vel = p.vp + 8.3333333333333333e-2 * Dt * (4. * A2 + 3. * A3);
}

// Hard pair sums over a cluster, src/gravity_hard.h:203-367.  mode 0: full
// (pos/vel of both, with phi_d); 1: predicted i and j; 2: corrected i,
// predicted j.
void hard_force(HPtcl &pi, const std::vector<HPtcl> &c, int mode) {
    V3 xi, vi;
    if (mode == 0) {
        sun_force(pi.pos, pi.vel, pi.acc_s, pi.jerk_s, &pi.phi_s);
        pi.phi_d = 0.;
        xi = pi.pos; vi = pi.vel;
    } else if (mode == 1) {
        sun_force(pi.xp, pi.vp, pi.acc_s, pi.jerk_s, nullptr);
        xi = pi.xp; vi = pi.vp;
    } else {
        sun_force(pi.pos, pi.vel, pi.acc_s, pi.jerk_s, nullptr);
        xi = pi.pos; vi = pi.vel;
    }
    pi.acc_d = ZERO;
    pi.jerk_d = ZERO;
    for (const HPtcl &pj : c) {
        if (pi.id == pj.id) continue;
        const V3 xj = (mode == 0) ? pj.pos : pj.xp;
        const V3 vj = (mode == 0) ? pj.vel : pj.vp;
        const V3 dr = xj - xi;
        double dr2 = dot(dr, dr);
        dr2 += P.eps2;
        const V3 dv = vj - vi;
        const double rij = std::sqrt(dr2);
        const double rinv = 1. / rij;
        const double r2inv = rinv * rinv;
        const double r3inv = r2inv * rinv;
        const double roi = lo_of(pi.r_out_inv, pj.r_out_inv);
        const double mr3 = pj.mass * r3inv;
        const double alpha = dot(dr, dv) * r2inv;
        double Wc = 0.;
        if (mode == 0) Wc = 1. - cut_W(rij, roi);
        const double Kc = 1. - cut_K(rij, roi);
        const double dKdt = cut_dKdt(rij, roi, alpha);
        const double alpha_c = alpha * Kc;
        if (mode == 0) pi.phi_d -= pj.mass * rinv * Wc;
        pi.acc_d += mr3 * Kc * dr;
        pi.jerk_d += mr3 * (Kc * dv - (3. * alpha_c + dKdt) * dr);
    }
}

// mergeAccJerk, src/hermite.h:36-83 (twins of target t)
void merge_acc_jerk(std::vector<HPtcl> &c, int t, const std::vector<int> &tw) {
    V3 a = c[t].mass * c[t].acc_d, j = c[t].mass * c[t].jerk_d;
    double m = c[t].mass;
    for (int k : tw) {
        a += c[k].mass * c[k].acc_d;
        j += c[k].mass * c[k].jerk_d;
        m += c[k].mass;
    }
    const double mi = 1. / m;
    a = a * mi;
    j = j * mi;
    c[t].acc_d = a; c[t].jerk_d = j;
    for (int k : tw) { c[k].acc_d = a; c[k].jerk_d = j; }
}

struct ColRec {
    int64_t id_imp, id_tar;
    double time;
    double edisp, edisp_d;
    int n_frag;       // fragments made by this collision
    int64_t id_frag;  // temporary id of its first fragment (the others count down)
    // the collision-file record (Collision0::write2File, src/collisionA.h:122-148)
    double mass_imp, mass_tar, mass_frag;
    V3 pos_imp, pos_tar, vel_imp, vel_tar;
    double dpos_g_rel, dvel_g_rel;
};
std::vector<ColRec> COLS;
ColRec LAST_UNIT;  // the record of the last orc_collide_unit
double EDISP = 0., EDISP_D = 0.;

// KOMINAMI fragmentation (src/collisionB.h:7-93; m_min src/collisionA.h:57,152).
// a_frag = 0 gives no fragments, the perfect accretion of Collision0.
double A_FRAG = 0.0;
int N_FRAG = 10;
double M_MIN = 9.426627927538057e-12;
// Fragment-circle phase: GPLUM draws drand48() (src/collisionA.h:727), whose
// sequence depends on the order OpenMP threads reach their collisions.  Mode
// 0 (default) draws from a counter-based generator keyed by (tree step,
// impactor id, target id, seed), the same on every device; mode 1 calls
// drand48() in the reference's processing order, for pinning against it.
int FRAG_RNG = 0;
uint64_t FRAG_SEED = 0;
int CUR_STEP = 0;
int64_t ID_NEXT = 0;  // next particle id (src/main_p3t.cpp:233,295-305)
constexpr double MY_PI = 3.14159265358979323846;  // src/main_p3t.cpp:25

uint64_t mix64(uint64_t z) {  // splitmix64 finaliser
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
double frag_uniform(int64_t id_imp, int64_t id_tar) {
    if (FRAG_RNG == 1) return drand48();
    uint64_t h = mix64(FRAG_SEED ^ 0x5851f42d4c957f2dULL);
    h = mix64(h ^ (uint64_t)(int64_t)CUR_STEP);
    h = mix64(h ^ (uint64_t)id_imp);
    h = mix64(h ^ (uint64_t)id_tar);
    return (double)(h >> 11) * 0x1.0p-53;
}

// One collision: Collision0::inputPair (src/collisionA.h:156-213), the
// KOMINAMI collisionOutcome with setFragmentCircle (src/collisionB.h:43-93,
// src/collisionA.h:708-742), Collision0::setParticle, calcEnergyDissipation
// and setNeighbors (src/collisionA.h:220-706).  Fragments are appended to the
// cluster c (their temporary ids count down from -(128 id_cluster + id_next
// + 1)); id_next is the cluster's fragment counter (src/hermite.h:243).
// Returns the number of fragments.
int collide(std::vector<HPtcl> &c, std::map<int, std::vector<int>> &twins, int imp, int tar,
            double &edisp, double &edisp_d, ColRec &rec, int64_t &id_next) {
    const std::vector<int> tw_imp = twins.count(imp) ? twins[imp] : std::vector<int>();
    const std::vector<int> tw_tar = twins.count(tar) ? twins[tar] : std::vector<int>();
    rec.id_imp = c[imp].id;
    rec.id_tar = c[tar].id;
    rec.time = c[imp].time_c + c[imp].time;
    const V3 pos_imp = c[imp].pos, pos_tar = c[tar].pos, vel_imp = c[imp].vel, vel_tar = c[tar].vel;
    double m_imp = c[imp].mass, m_tar = c[tar].mass;
    if (c[imp].merged)
        for (int k : tw_imp) m_imp += c[k].mass;
    if (c[tar].merged)
        for (int k : tw_tar) m_tar += c[k].mass;
    const double r_planet_tar = c[tar].r_planet, f_imp = c[imp].f, f_tar = c[tar].f;
    const V3 pos_g = (m_imp * pos_imp + m_tar * pos_tar) / (m_imp + m_tar);
    const V3 vel_g = (m_imp * vel_imp + m_tar * vel_tar) / (m_imp + m_tar);
    // collisionOutcome (KOMINAMI)
    int n_frag = (int)std::floor(A_FRAG * m_imp / M_MIN);
    if (n_frag < 2) n_frag = 0;
    if (n_frag > N_FRAG) n_frag = N_FRAG;
    const double mass_frag = n_frag ? (A_FRAG * m_imp) : 0.;
    const double mass_rem = m_imp + m_tar - mass_frag;
    V3 masspos = ZERO, massvel = ZERO;
    std::vector<HPtcl> F;
    if (n_frag) {
        const V3 ximp = pos_imp - pos_tar, vimp = vel_imp - vel_tar;
        const double f_frag = f_imp;
        const double r_planet_frag = std::pow(0.75 * mass_frag / n_frag / (MY_PI * P.dens), 1. / 3.);
        const double r_planet_rem = std::pow(mass_rem / m_tar, 1. / 3.) * r_planet_tar;
        const double r_frag = 2. * std::max(f_tar, f_frag) * (r_planet_frag + r_planet_rem);
        const double r2_frag = r_frag * r_frag + P.eps2;
        const double r_frag_inv = std::sqrt(1. / r2_frag);
        const double v_frag = 1.05 * std::sqrt(2. * mass_rem * r_frag_inv);
        const double m_f = mass_frag / n_frag;
        // setFragmentCircle
        V3 e0 = ximp;
        V3 e1 = vimp - (dot(vimp, ximp) / dot(ximp, ximp)) * ximp;
        e0 = e0 / std::sqrt(dot(e0, e0));
        e1 = e1 / std::sqrt(dot(e1, e1));
        const double theta0 = 2. * M_PI * frag_uniform(rec.id_imp, rec.id_tar);
        for (int i = 0; i < n_frag; i++) {
            HPtcl h;
            std::memset((void *)&h, 0, sizeof(HPtcl));
            h.mass = m_f;
            const double theta = theta0 + 2. * M_PI * i / n_frag;
            h.pos = pos_g + r_frag * (std::cos(theta) * e0 + std::sin(theta) * e1);
            h.vel = vel_g + v_frag * (std::cos(theta) * e0 + std::sin(theta) * e1);
            masspos += h.mass * h.pos;
            massvel += h.mass * h.vel;
            F.push_back(h);
        }
    }
    const V3 pos_new = (m_imp * pos_imp + m_tar * pos_tar - masspos) / mass_rem;
    const V3 vel_new = (m_imp * vel_imp + m_tar * vel_tar - massvel) / mass_rem;
    {
        // the record: masses and states before the collision, and
        // Collision0::setParticle's centre of mass after it -- fragments in
        // creation order, then remnant and target (src/collisionA.h:232-234,
        // 288-291,344-348) -- against pos_g / vel_g (src/collisionA.h:205-206)
        double mass_tot = 0.;
        for (int i = 0; i < n_frag; i++) mass_tot += F[i].mass;
        const V3 mp = masspos + ((m_imp - mass_frag) * pos_new + m_tar * pos_new);
        const V3 mv = massvel + ((m_imp - mass_frag) * vel_new + m_tar * vel_new);
        mass_tot += m_imp - mass_frag + m_tar;
        const V3 dpos_g = mp / mass_tot - pos_g, dvel_g = mv / mass_tot - vel_g;
        rec.mass_imp = m_imp;
        rec.mass_tar = m_tar;
        rec.mass_frag = mass_frag;
        rec.pos_imp = pos_imp;
        rec.pos_tar = pos_tar;
        rec.vel_imp = vel_imp;
        rec.vel_tar = vel_tar;
        rec.dpos_g_rel = std::sqrt(dot(dpos_g, dpos_g) / dot(pos_g, pos_g));
        rec.dvel_g_rel = std::sqrt(dot(dvel_g, dvel_g) / dot(vel_g, vel_g));
    }
    // setParticle (flag_merge)
    c[imp].r_planet = 0.;
    c[tar].r_planet *= std::pow(mass_rem / m_tar, 1. / 3.);
    c[imp].mass -= mass_frag;
    c[imp].id = c[tar].id;
    c[imp].dead = true;
    for (int k : tw_imp) { c[k].id = c[tar].id; c[k].dead = true; }
    c[tar].merged = true;
    const int id_c_frag = n_frag ? (int)c.size() : 0;
    const int64_t id_frag = n_frag ? (-(128 * c[imp].id_cluster + id_next + 1)) : 0;
    for (int i = 0; i < n_frag; i++) {
        HPtcl &h = F[i];
        h.r_planet = std::pow(0.75 * h.mass / (MY_PI * P.dens), 1. / 3.);  // setRPlanet
        h.f = c[imp].f;
        h.r_out = c[imp].r_out;
        h.r_out_inv = c[imp].r_out_inv;
        h.r_search = c[imp].r_search;
        h.v_disp = c[imp].v_disp;
        h.time = c[imp].time;
        h.time_c = c[imp].time_c;
        h.dt = c[imp].dt;
        h.phi = c[imp].phi;
        h.phi_d = c[imp].phi_d;
        h.phi_s = c[imp].phi_s;
        // GPLUM leaves acc0 of a fragment unset (FPHard() does not initialise
        // it); the reference build showed a denormal there, whose square --
        // the only way acc0 enters calcDeltatInitial -- is 0
        h.acc0 = 0.;
        h.id = id_frag - i;
        h.id_cluster = c[imp].id_cluster;
        h.dead = false;
        h.merged = false;
        h.number = c[imp].number;  // setNeighbors
        h.rank = 0; h.id_max = -1; h.id_min = INT_MAX;
        id_next++;
    }
    c.insert(c.end(), F.begin(), F.end());
    c[imp].pos = pos_new; c[imp].vel = vel_new;
    for (int k : tw_imp) { c[k].pos = pos_new; c[k].vel = vel_new; }
    c[tar].pos = pos_new; c[tar].vel = vel_new;
    for (int k : tw_tar) { c[k].pos = pos_new; c[k].vel = vel_new; }
    // calcEnergyDissipation
    const double m_i = c[imp].mass + mass_frag;
    double e_kin = 0.;
    // (scalar * v) . v, the evaluation order of "s * v * v" with FDPS vectors
    V3 vr = vel_imp - vel_tar;
    e_kin -= dot(0.5 * m_imp * m_tar / (m_imp + m_tar) * vr, vr);
    vr = vel_new - vel_g;
    e_kin += dot(0.5 * (m_imp - mass_frag) * vr, vr);
    vr = vel_new - vel_g;
    e_kin += dot(0.5 * m_tar * vr, vr);
    for (int i = 0; i < n_frag; i++) {
        const HPtcl &h = c[id_c_frag + i];
        vr = h.vel - vel_g;
        e_kin += dot(0.5 * h.mass * vr, vr);
    }
    double e_int = 0., e_int_d = 0.;
    V3 dr = pos_imp - pos_tar;
    double dr2 = dot(dr, dr) + P.eps2;
    double rinv = std::sqrt(1. / dr2), rinv_new;
    double dphi = m_i * rinv;
    e_int += c[tar].mass * dphi;
    e_int_d += c[tar].mass * dphi * (1. - cut_W2(dr2, c[imp].r_out_inv, c[tar].r_out_inv));
    for (int k : tw_tar) {
        e_int += c[k].mass * dphi;
        e_int_d += c[k].mass * dphi * (1. - cut_W2(dr2, c[imp].r_out_inv, c[k].r_out_inv));
    }
    for (int ki : tw_imp) {
        dphi = c[ki].mass * rinv;
        e_int += c[tar].mass * dphi;
        e_int_d += c[tar].mass * dphi * (1. - cut_W2(dr2, c[ki].r_out_inv, c[tar].r_out_inv));
        for (int kj : tw_tar) {
            e_int += c[kj].mass * dphi;
            e_int_d += c[kj].mass * dphi * (1. - cut_W2(dr2, c[ki].r_out_inv, c[kj].r_out_inv));
        }
    }
    for (int i = 0; i < n_frag; i++) {
        const int f0 = id_c_frag + i;
        dr = c[f0].pos - c[imp].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv_new = std::sqrt(1. / dr2);
        dphi = -c[f0].mass * rinv_new;
        e_int += c[imp].mass * dphi;
        e_int_d += c[imp].mass * dphi * (1. - cut_W2(dr2, c[imp].r_out_inv, c[f0].r_out_inv));
        for (int k : tw_imp) {
            e_int += c[k].mass * dphi;
            e_int_d += c[k].mass * dphi * (1. - cut_W2(dr2, c[k].r_out_inv, c[f0].r_out_inv));
        }
        dr = c[f0].pos - c[tar].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv_new = std::sqrt(1. / dr2);
        dphi = -c[f0].mass * rinv_new;
        e_int += c[tar].mass * dphi;
        e_int_d += c[tar].mass * dphi * (1. - cut_W2(dr2, c[tar].r_out_inv, c[f0].r_out_inv));
        for (int k : tw_tar) {
            e_int += c[k].mass * dphi;
            e_int_d += c[k].mass * dphi * (1. - cut_W2(dr2, c[k].r_out_inv, c[f0].r_out_inv));
        }
        for (int j = 0; j < i; j++) {
            const int f1 = id_c_frag + j;
            dr = c[f0].pos - c[f1].pos;
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = std::sqrt(1. / dr2);
            dphi = -c[f0].mass * c[f1].mass * rinv_new;
            e_int += dphi;
            e_int_d += dphi * (1. - cut_W2(dr2, c[f0].r_out_inv, c[f1].r_out_inv));
        }
    }
    for (int i = 0; i < id_c_frag; i++) {
        if (c[i].id == c[imp].id || c[i].id == c[tar].id) continue;
        const double m_nei = c[i].mass;
        dr = pos_imp - c[i].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv = std::sqrt(1. / dr2);
        dr = c[imp].pos - c[i].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv_new = std::sqrt(1. / dr2);
        dphi = m_nei * (rinv - rinv_new);
        e_int += m_nei * (m_i * rinv - c[imp].mass * rinv_new);
        e_int_d += m_nei * (m_i * rinv - c[imp].mass * rinv_new) *
                   (1. - cut_W2(dr2, c[imp].r_out_inv, c[i].r_out_inv));
        for (int k : tw_imp) {
            e_int += c[k].mass * dphi;
            e_int_d += c[k].mass * dphi * (1. - cut_W2(dr2, c[k].r_out_inv, c[i].r_out_inv));
        }
        for (int j = 0; j < n_frag; j++) {
            const int fj = id_c_frag + j;
            dr = c[fj].pos - c[i].pos;
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = std::sqrt(1. / dr2);
            dphi = -m_nei * c[fj].mass * rinv_new;
            e_int += dphi;
            e_int_d += dphi * (1. - cut_W2(dr2, c[fj].r_out_inv, c[i].r_out_inv));
        }
        dr = pos_tar - c[i].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv = std::sqrt(1. / dr2);
        dr = c[tar].pos - c[i].pos;
        dr2 = dot(dr, dr) + P.eps2;
        rinv_new = std::sqrt(1. / dr2);
        dphi = m_nei * (rinv - rinv_new);
        e_int += c[tar].mass * dphi;
        e_int_d += c[tar].mass * dphi * (1. - cut_W2(dr2, c[tar].r_out_inv, c[i].r_out_inv));
        for (int k : tw_tar) {
            e_int += c[k].mass * dphi;
            e_int_d += c[k].mass * dphi * (1. - cut_W2(dr2, c[k].r_out_inv, c[i].r_out_inv));
        }
    }
    double e_sun = 0.;
    e_sun += m_imp / std::sqrt(dot(pos_imp, pos_imp) + P.eps2) + m_tar / std::sqrt(dot(pos_tar, pos_tar) + P.eps2);
    e_sun -= m_tar * std::sqrt(1. / (dot(c[tar].pos, c[tar].pos) + P.eps2));
    e_sun -= (m_imp - mass_frag) * std::sqrt(1. / (dot(c[imp].pos, c[imp].pos) + P.eps2));
    for (int i = 0; i < n_frag; i++) {
        const HPtcl &h = c[id_c_frag + i];
        e_sun -= h.mass * std::sqrt(1. / (dot(h.pos, h.pos) + P.eps2));
    }
    e_sun *= P.m_sun;
    edisp = e_kin + e_int + e_sun;
    edisp_d = e_kin + e_int_d + e_sun;
    if (getenv("ORC_DEBUG_COL")) fprintf(stderr, "ORC DEkin: %.15e DEint: %.15e DEint_hard: %.15e DEsun: %.15e\n", e_kin, e_int, e_int_d, e_sun);
    rec.n_frag = n_frag;
    rec.id_frag = id_frag;
    // merge_list update, src/hermite.h:413-423
    std::vector<int> &t = twins[tar];
    t.push_back(imp);
    if (c[imp].merged) {
        for (int k : tw_imp) t.push_back(k);
        twins.erase(imp);
        c[imp].merged = false;
    }
    return n_frag;
}

// timeIntegrate_multi, src/hermite.h:224-479 (perfect accretion)
void integrate_cluster(std::vector<HPtcl> &c, double t_end, int &n_col, double &edisp, double &edisp_d,
                       std::vector<ColRec> &cols) {
    std::map<int, std::vector<int>> twins;  // target -> dead twins, insertion order
    n_col = 0;
    edisp = edisp_d = 0.;
    int64_t id_next = 0;  // fragments made in this cluster
    int n = (int)c.size();
    for (int i = 0; i < n; i++) hard_force(c[i], c, 0);
    for (int i = 0; i < n; i++) c[i].dead = c[i].merged = false;
    double time = 0.;
    std::vector<int> act;
    while (time < t_end) {
        // makeActiveList, src/hermite.h:4-24
        double ts = 1.e10;
        act.clear();
        for (int i = 0; i < n; i++) {
            if (c[i].dead) continue;
            const double ti = c[i].time + c[i].dt;
            if (ts > ti) { ts = ti; act.clear(); act.push_back(i); }
            else if (ts == ti) act.push_back(i);
        }
        for (int i = 0; i < n; i++) {
            c[i].xp = ZERO; c[i].vp = ZERO;
            predict(c[i], ts - c[i].time);
        }
        // collisionDetermination, src/hermite.h:98-196
        double Rmin = 1.;
        int col = 0, imp = -1, tar = -1;
        for (int i = 0; i < n; i++) {
            if (c[i].dead) continue;
            for (int j = 0; j < n; j++) {
                if (i == j || c[j].dead) continue;
                const V3 dr = c[i].xp - c[j].xp;
                const double r1 = std::sqrt(dot(dr, dr));
                const double r2 = c[i].f * c[i].r_planet + c[j].f * c[j].r_planet;
                const double R = r1 / r2;
                if (R < Rmin) {
                    Rmin = R;
                    if (c[i].mass < c[j].mass) { imp = i; tar = j; }
                    else { imp = j; tar = i; }
                    col = 1;
                }
            }
        }
        if (col) {
            act.clear();
            for (int i = 0; i < n; i++) {
                c[i].dt = ts - c[i].time;
                if (c[i].dead) continue;
                act.push_back(i);
            }
        }
        for (int a : act) {
            static const std::vector<int> none;
            const std::vector<int> &tw = (c[a].merged && twins.count(a)) ? twins[a] : none;
            hard_force(c[a], c, 1);
            if (c[a].merged) {
                for (int k : tw) hard_force(c[k], c, 1);
                merge_acc_jerk(c, a, tw);
            }
            const double tc = ts - c[a].time;
            for (int it = 0; it < 2; it++) {
                correct(c[a], tc);
                if (c[a].merged)
                    for (int k : tw) correct(c[k], tc);
                hard_force(c[a], c, 2);
                if (c[a].merged) {
                    for (int k : tw) hard_force(c[k], c, 2);
                    merge_acc_jerk(c, a, tw);
                }
            }
            c[a].time += tc;
            if (c[a].merged)
                for (int k : tw) c[k].time += tc;
            if (!col) {
                dt_hermite(c[a]);
                if (c[a].merged)
                    for (int k : tw) c[k].dt = c[a].dt;
            }
        }
        if (col) {
            double e1 = 0., e2 = 0.;
            ColRec rec;
            collide(c, twins, imp, tar, e1, e2, rec, id_next);
            n = (int)c.size();
            rec.edisp = e1;
            rec.edisp_d = e2;
            edisp += e1;
            edisp_d += e2;
            cols.push_back(rec);
            n_col++;
            for (int i = 0; i < n; i++) hard_force(c[i], c, 0);
            for (auto &kv : twins) merge_acc_jerk(c, kv.first, kv.second);
            for (int i = 0; i < n; i++) {
                if (!c[i].dead) dt_initial(c[i]);
                if (c[i].merged && twins.count(i))
                    for (int k : twins[i]) c[k].dt = c[i].dt;
            }
        }
        // getSystemTime, src/hermite.h:25-35
        double tmin = 1.e10;
        for (int i = 0; i < n; i++)
            if (!c[i].dead && tmin > c[i].time) tmin = c[i].time;
        time = tmin;
    }
    for (int i = 0; i < n; i++) hard_force(c[i], c, 0);
    if (n_col > 0)
        for (auto &kv : twins) merge_acc_jerk(c, kv.first, kv.second);
}

// timeIntegrate_isolated, src/hermite.h:734-785
void integrate_isolated(HPtcl &p, double t_end) {
    sun_force(p.pos, p.vel, p.acc_s, p.jerk_s, &p.phi_s);
    while (p.time < t_end) {
        predict(p, p.dt);
        p.acc_d = ZERO;
        p.jerk_d = ZERO;
        sun_force(p.xp, p.vp, p.acc_s, p.jerk_s, nullptr);
        for (int it = 0; it < 2; it++) {
            correct(p, p.dt);
            sun_force(p.pos, p.vel, p.acc_s, p.jerk_s, nullptr);
        }
        p.time += p.dt;
        dt_hermite(p);
    }
    p.phi_s = 0.;
    p.phi_d = 0.;
    sun_force(p.pos, p.vel, p.acc_s, p.jerk_s, &p.phi_s);
}

// Kepler drift, src/kepler.h:3-93 and src/hermite.h:787-815
double kepler_eq(double u, double e) { return u - e * std::sin(u); }
int KEPLER_ABS_INT = 0;  // how the reference's unqualified abs() resolved
double solve_kepler(double l, double e) {
    const double e2 = e * e, e3 = e2 * e, e4 = e2 * e2, e5 = e3 * e2, e6 = e3 * e3;
    double u = l + (e - e3 / 8. + e5 / 192.) * std::sin(l) + (e2 / 2. - e4 / 6. + e6 / 48.) * std::sin(2. * l) +
               (3. * e3 / 8. - 27. * e5 / 128.) * std::sin(3. * l) + (e4 / 3. - 4. * e6 / 15.) * std::sin(4. * l) +
               125. * e5 / 384. * std::sin(5. * l) + 27. * e6 / 80. * std::sin(6. * l);
    const double res = kepler_eq(u, e) - l;
    const double ares = KEPLER_ABS_INT ? (double)std::abs((int)res) : std::fabs(res);
    if (ares > 1.e-15) {
        double u0;
        int loop = 0;
        do {
            u0 = u;
            const double s = std::sin(u0), co = std::cos(u0);
            u = u0 - ((u0 - e * s - l) / (1. - e * co));
            loop++;
        } while (std::fabs(u - u0) > 1.e-15 && loop < 10);
    }
    return u;
}
void kepler_drift(Ptcl &p, double t0, double t1) {
    const double mu = P.m_sun;
    const double r2 = dot(p.pos, p.pos), r = std::sqrt(r2), rinv = 1. / r;
    const double v2 = dot(p.vel, p.vel), rv = dot(p.pos, p.vel);
    const double ax = 1.0 / (2.0 * rinv - v2 / mu);
    const double ecccosu = 1. - r / ax;
    const double eccsinu = rv / std::sqrt(mu * ax);
    const double ecc = std::sqrt(ecccosu * ecccosu + eccsinu * eccsinu);
    const double n = std::sqrt(mu / (ax * ax * ax));
    double u, cosu, sinu;
    if (ecc != 0) {
        u = std::atan2(eccsinu, ecccosu);
        cosu = ecccosu / ecc;
        sinu = eccsinu / ecc;
    } else {
        u = 0.; cosu = 1.; sinu = 0.;
    }
    const double aninv = std::sqrt(ax / mu);
    const double ecc_sq = std::sqrt(1. - ecc * ecc);
    const V3 PP = rinv * cosu * p.pos - aninv * sinu * p.vel;
    const V3 QQ = (rinv * sinu * p.pos + aninv * (cosu - ecc) * p.vel) / ecc_sq;
    double l = kepler_eq(u, ecc);
    l += n * (t1 - t0);
    u = solve_kepler(l, ecc);
    const double cu = std::cos(u), su = std::sin(u);
    const double esq = std::sqrt(1. - ecc * ecc);
    p.pos = ax * ((cu - ecc) * PP + esq * su * QQ);
    const double ri = std::sqrt(1. / dot(p.pos, p.pos));
    p.vel = ax * ax * n * ri * (-su * PP + esq * cu * QQ);
    p.time += (t1 - t0);
    p.phi_d = 0.;
    p.acc_d = ZERO;
    p.jerk_d = ZERO;
    sun_force(p.pos, p.vel, p.acc_s, p.jerk_s, &p.phi_s);
    dt_initial(p);
}
double eccentricity(const Ptcl &p) {  // FPGrav::getEccentricity, src/particle.h:668-681
    const double r = std::sqrt(dot(p.pos, p.pos));
    const double rv = dot(p.pos, p.vel);
    const double ax = 1.0 / (2.0 / r - dot(p.vel, p.vel) / P.m_sun);
    const double ecccosu = 1. - r / ax;
    const double eccsinu2 = rv * rv / (P.m_sun * ax);
    return std::sqrt(ecccosu * ecccosu + eccsinu2);
}

// --- correction + neighbour search, src/gravity_soft.h:75-528 -------------
// Candidates of the correction: every j with |x_j - x_i| < max(1.1 r_search_i,
// 1.1 r_search_j) (getRSearch, src/particle.h:119-125), ascending index.
struct Grid {
    NgbGrid g;
    void build() {
        g.build((int)S.size(), [](int i, double &x, double &y, double &z) {
            x = S[i].pos.x; y = S[i].pos.y; z = S[i].pos.z;
        }, [](int i) { return 1.1 * S[i].r_search; });
    }
    void query(int i, std::vector<int> &out) const {
        const Ptcl &p = S[i];
        g.query(i, out, [&](int j) {
            const V3 d = S[j].pos - p.pos;
            const double r = std::max(1.1 * p.r_search, 1.1 * S[j].r_search);
            return dot(d, d) < r * r;
        });
    }
};

struct CorrAcc {
    V3 acc = ZERO, acc_d = ZERO, jerk = ZERO;
    double phi = 0., phi_d = 0., acc0 = 0.;
};

// correctForceBetween2Particles(Initial), src/gravity_soft.h:75-242.  The
// neighbour test reads acc_d from acc_d_old (the pre-pass values).
void corr_pair(int i, int j, bool initial, const std::vector<V3> &acc_d_old, CorrAcc &a,
               std::vector<int64_t> &nl, std::vector<std::pair<int, int>> &pairs) {
    Ptcl &pi = S[i];
    const Ptcl &pj = S[j];
    const double r_out = hi_of(pi.r_out, pj.r_out);
    const double r_out_inv = lo_of(pi.r_out_inv, pj.r_out_inv);
    const double r_search = hi_of(pi.r_search, pj.r_search);
    if (pj.id == pi.id) {
        a.phi += pj.mass * r_out_inv;
        return;
    }
    const V3 dr = pj.pos - pi.pos;
    double dr2 = dot(dr, dr);
    dr2 += P.eps2;
    const double rij = std::sqrt(dr2);
    const V3 dv = pj.vel - pi.vel;
    const V3 da = acc_d_old[j] - acc_d_old[i];
    const double drdv = dot(dr, dv);
    const double dv2 = dot(dv, dv);
    const double da2 = dot(da, da);
    const double t_min = lo_of(hi_of(-drdv / std::sqrt(dv2), 0.), P.dt_tree);
    const double dr2_min = lo_of(dr2, dr2 + 2. * drdv * t_min + dv2 * t_min * t_min);
    const double r_crit = P.R_search2 * r_out;
    const double v_crit_a = P.R_search3 * 0.5 * P.dt_tree;
    if (dr2_min < r_crit * r_crit || dv2 < v_crit_a * v_crit_a * da2 || (initial && da2 == 0.)) {
        if (rij < r_search) {
            // NeighborList::addNeighbor, src/neighbor.h:635-670
            nl.push_back(pj.id);
            pi.number++;
            pi.id_cluster = lo_of(pi.id_cluster, pj.id);
            if (i < pj.id_local) pairs.push_back({i, pj.id_local});
            a.acc0 += r_out * r_out / pj.mass;
        }
    }
    if (rij < r_out) {
        const double rinv = 1. / rij;
        const double r2inv = rinv * rinv;
        const double r3inv = rinv * r2inv;
        const double W = cut_W(rij, r_out_inv);
        const double K = cut_K(rij, r_out_inv);
        const double r_min = lo_of(rinv, r_out_inv);
        a.phi -= pj.mass * (rinv * W - r_min);
        a.acc += pj.mass * (r3inv * K - r_min * r_min * r_min) * dr;
        if (initial) {
            const double alpha = drdv * r2inv;
            const double dKdt = cut_dKdt(rij, r_out_inv, alpha);
            const double alpha_c = alpha * (1. - K);
            a.phi_d -= pj.mass * rinv * (1. - W);
            a.acc_d += pj.mass * r3inv * (1. - K) * dr;
            a.jerk += pj.mass * r3inv * ((1. - K) * dv - (3. * alpha_c + dKdt) * dr);
        }
    }
}

// correctForceLong / correctForceLongInitial, src/gravity_soft.h:245-528.
// Candidate sets: kernel count <= 2 -> the kernel's id_min / id_max; more ->
// the grid query (a superset of every pair the test can accept).
void correct_all(bool initial) {
    const int n = (int)S.size();
    Grid grid;
    grid.build();
    std::vector<V3> acc_d_old(n);
    for (int i = 0; i < n; i++) acc_d_old[i] = S[i].acc_d;
    NLIST.assign(n, {});
    std::vector<std::vector<std::pair<int, int>>> pp(n);
    std::vector<V3> acc_d_new(n);
    int ngb_tot = 0, with_ngb = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : ngb_tot, with_ngb)
    for (int i = 0; i < n; i++) {
        Ptcl &p = S[i];
        if (initial) sun_force(p.pos, p.vel, p.acc_s, p.jerk_s, &p.phi_s);
        CorrAcc a;
        const int k = p.number;
        p.number = 0;
        p.id_cluster = p.id;
        a.phi += p.mass * p.r_out_inv;
        if (k > 0) {
            if (k > 2 || p.rank != 0) {
                std::vector<int> cand;
                grid.query(i, cand);
                for (int j : cand) {
                    if (S[j].id == p.id) continue;
                    corr_pair(i, j, initial, acc_d_old, a, NLIST[i], pp[i]);
                }
            } else {
                for (int q = 0; q < k; q++) {
                    const int j = (q == 0) ? p.id_min : p.id_max;
                    corr_pair(i, j, initial, acc_d_old, a, NLIST[i], pp[i]);
                }
            }
        }
        if (p.number) {
            ngb_tot += p.number;
            with_ngb++;
        }
        p.acc += a.acc;
        p.phi += a.phi;
        p.acc0 = (a.acc0 > 0.) ? p.number / a.acc0 : 0.;
        if (initial) {
            acc_d_new[i] = a.acc_d;
            p.phi_d = a.phi_d;
            p.jerk_d = a.jerk;
            dt_initial(p);  // reads the pre-pass acc_d, as the reference does
        }
    }
    if (initial)
        for (int i = 0; i < n; i++) S[i].acc_d = acc_d_new[i];
    PAIRS.clear();
    for (int i = 0; i < n; i++) PAIRS.insert(PAIRS.end(), pp[i].begin(), pp[i].end());
    N_NGB_TOT = ngb_tot;
    N_WITH_NGB = with_ngb;
}

// NeighborList::createNeighborCluster, src/neighbor.h:800-839: every
// connected component of PAIRS takes the minimum of its members' id_cluster.
int find_root(std::vector<int> &par, int x) {
    while (par[x] != x) { par[x] = par[par[x]]; x = par[x]; }
    return x;
}
void cluster_all() {
    const int n = (int)S.size();
    std::vector<int> par(n);
    std::iota(par.begin(), par.end(), 0);
    for (auto &pr : PAIRS) {
        int a = find_root(par, pr.first), b = find_root(par, pr.second);
        if (a != b) par[std::max(a, b)] = std::min(a, b);
    }
    std::vector<int64_t> cmin(n, std::numeric_limits<int64_t>::max());
    for (int i = 0; i < n; i++) {
        int r = find_root(par, i);
        cmin[r] = std::min(cmin[r], S[i].id_cluster);
    }
    for (int i = 0; i < n; i++) S[i].id_cluster = cmin[find_root(par, i)];
}

HPtcl to_hard(const Ptcl &p) {  // FPHard(const FPGrav&), src/particle.h:1096-1116
    HPtcl h;
    static_cast<Ptcl &>(h) = p;
    h.x0 = h.v0 = h.a0_s = h.j0_s = h.a0_d = h.j0_d = h.xp = h.vp = ZERO;
    h.a2_s = h.a3_s = h.a2_d = h.a3_d = ZERO;
    h.time_c = p.time;
    h.time = 0;
    return h;
}

// HardSystem::makeList + timeIntegrate, src/hard.h:321-829
int hard_all(int istep) {
    const int n = (int)S.size();
    std::vector<std::pair<int64_t, int>> keys;
    int niso = 0;
    for (int i = 0; i < n; i++) {
        if (S[i].number) keys.push_back({S[i].id_cluster, i});
        else niso++;
    }
    std::stable_sort(keys.begin(), keys.end(),
                     [](const std::pair<int64_t, int> &a, const std::pair<int64_t, int> &b) { return a.first < b.first; });
    std::vector<std::vector<int>> clusters;
    for (size_t k = 0; k < keys.size(); k++) {
        if (k == 0 || keys[k].first != keys[k - 1].first) clusters.push_back({});
        clusters.back().push_back(keys[k].second);
    }
    N_CLUSTER = (int)clusters.size();
    N_ISO = niso;
    COLS.clear();
    EDISP = EDISP_D = 0.;
    CUR_STEP = istep;
    int done = 0;
    // clusters of 64 or more members first, then the rest, each in cluster
    // order (src/hard.h:562-575,583,700-701)
    std::vector<int> order;
    for (int pass = 0; pass < 2; pass++)
        for (int k = 0; k < (int)clusters.size(); k++)
            if ((clusters[k].size() >= 64) == (pass == 0)) order.push_back(k);
    // clusters are independent: integrate them in parallel, then fold the
    // per-cluster results in the reference's order
    const int ncl = (int)order.size();
    std::vector<std::vector<ColRec>> ccols(ncl);
    std::vector<double> ce1(ncl, 0.), ce2(ncl, 0.);
    std::vector<int> cnc(ncl, 0);
    std::vector<std::vector<Ptcl>> cfrag(ncl);  // fragments of each cluster, in creation order
    // (drand48 fragment phases follow the reference's sequential order)
#pragma omp parallel for schedule(dynamic, 2) if (FRAG_RNG == 0)
    for (int q = 0; q < ncl; q++) {
        auto &cl = clusters[order[q]];
        std::vector<HPtcl> c;
        for (int i : cl) c.push_back(to_hard(S[i]));
        integrate_cluster(c, P.dt_tree, cnc[q], ce1[q], ce2[q], ccols[q]);
        for (size_t k = 0; k < c.size(); k++) {
            c[k].n_cluster = (int)c.size();
            c[k].time = c[k].time_c + c[k].time;  // resetTime
            c[k].time_c = 0.;
            if (k < cl.size()) S[cl[k]] = static_cast<Ptcl &>(c[k]);
            else cfrag[q].push_back(static_cast<Ptcl &>(c[k]));
        }
    }
    for (int q = 0; q < ncl; q++) {
        if (cnc[q] > 0) { EDISP += ce1[q]; EDISP_D += ce2[q]; }
        COLS.insert(COLS.end(), ccols[q].begin(), ccols[q].end());
        done += (int)clusters[order[q]].size();
    }
    // rewriteFragmentID + addFragment2ParticleSystem (src/hard.h:832-943):
    // new ids in collision-list order, then the fragments join the system in
    // cluster order; dead members that merged into a fragment take its new id
    {
        std::map<int64_t, int64_t> o2n;
        for (const ColRec &r : COLS)
            for (int j = 0; j < r.n_frag; j++) o2n[r.id_frag - j] = ID_NEXT++;
        // the records carry the final ids (Collision0::setNewFragmentID)
        for (ColRec &r : COLS) {
            if (r.id_imp < 0) r.id_imp = o2n.at(r.id_imp);
            if (r.id_tar < 0) r.id_tar = o2n.at(r.id_tar);
            if (r.n_frag) r.id_frag = o2n.at(r.id_frag);
        }
        for (int q = 0; q < ncl; q++) {
            const auto &cl = clusters[order[q]];
            for (Ptcl h : cfrag[q]) {
                const int64_t old = h.id, nid = (old < 0) ? o2n.at(old) : old;
                if (h.merged)
                    for (int i : cl)
                        if (S[i].id == old) S[i].id = nid;
                h.id = nid;
                S.push_back(h);
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
        if (S[i].number) continue;
        if (eccentricity(S[i]) < 0.8 && P.eps2_sun == 0.) {
            kepler_drift(S[i], (istep - 1) * P.dt_tree, istep * P.dt_tree);
        } else {
            HPtcl h = to_hard(S[i]);
            integrate_isolated(h, P.dt_tree);
            h.time = h.time_c + h.time;
            h.time_c = 0.;
            S[i] = static_cast<Ptcl &>(h);
        }
        S[i].n_cluster = 1;
    }
    return (int)COLS.size();
}

// FPGrav::setROutRSearch, calcRandomVel, setCutoffRadii,
// src/particle.h:713-733,1319-1457,1528-1543
void set_cutoff_radii() {
    const int n = (int)S.size();
    double r_max = 0., r_min = -std::numeric_limits<double>::max();
    for (int i = 0; i < n; i++) {
        const double r2 = S[i].pos.x * S[i].pos.x + S[i].pos.y * S[i].pos.y;
        r_max = std::max(r_max, r2);
        r_min = std::max(r_min, -r2);
    }
    r_max = std::sqrt(r_max) * 1.01;
    r_min = std::sqrt(-r_min) * 0.99;
    const int NB = 32;
    const double dr = (r_max - r_min) / NB, drinv = 1. / dr;
    double vd[NB];
    int np[NB];
    for (int b = 0; b < NB; b++) { vd[b] = 0.; np[b] = 0; }
    for (int i = 0; i < n; i++) {
        const V3 pos = S[i].pos;
        const double ri = std::sqrt(pos.x * pos.x + pos.y * pos.y);
        int b = (int)((ri - r_min) * drinv);
        if (b == NB) b = NB - 1;
        V3 vk = v3(-pos.y / ri, pos.x / ri, 0.);
        vk = vk * std::sqrt(P.m_sun / std::sqrt(pos.x * pos.x + pos.y * pos.y));
        const V3 vr = S[i].vel - vk;
        vd[b] += dot(vr, vr);
        np[b]++;
    }
    for (int b = 0; b < NB; b++) vd[b] = (np[b] > 0) ? std::sqrt(vd[b] / np[b]) : 0.;
    for (int i = 0; i < n; i++) {
        const double r2 = S[i].pos.x * S[i].pos.x + S[i].pos.y * S[i].pos.y;
        double vsum = 0., wsum = 0.;
        for (int b = 0; b < NB; b++) {
            const double ddr = r_min + (b + 0.5) * dr - std::sqrt(r2);
            const double ex = std::exp(-ddr * ddr * drinv * drinv);
            vsum += vd[b] * ex;
            wsum += (np[b] > 0) ? ex : 0.;
        }
        S[i].v_disp = vsum / wsum;
    }
    for (int i = 0; i < n; i++) {
        Ptcl &p = S[i];
        // getRHill with getSemimajorAxis2, src/particle.h:653-699
        double ax;
        {
            const double r = std::sqrt(dot(p.pos, p.pos));
            const double rv = dot(p.pos, p.vel);
            ax = 1.0 / (2.0 / r - dot(p.vel, p.vel) / P.m_sun);
            const double ecccosu = 1. - r / ax;
            const double eccsinu2 = rv * rv / (P.m_sun * ax);
            const double ecc = std::sqrt(ecccosu * ecccosu + eccsinu2);
            if (!(ecc < 0.6)) ax = r;
        }
        const double rHill = std::pow(p.mass / (3. * P.m_sun), 1. / 3.) * ax;
        const double r_out_i = hi_of(P.R_cut0 * std::pow(ax, -P.p_cut) * rHill, P.R_cut1 * p.v_disp * P.dt_tree);
        p.r_out = hi_of(r_out_i, P.r_cut_min);
        if (P.r_cut_max > 0.) p.r_out = lo_of(P.r_cut_max, p.r_out);
        p.r_out_inv = 1. / p.r_out;
        p.r_search = P.R_search0 * p.r_out + P.R_search1 * p.v_disp * P.dt_tree;
    }
}

}  // namespace

extern "C" {

void orc_epep_f32(const void *epi, int ni, const void *epj, int nj, void *force) {
    epep_f32((const EPI *)epi, ni, (const EPJ *)epj, nj, (FORCE *)force);
}
void orc_epsp_f32(const void *epi, int ni, const void *spj, int nj, void *force, int trace_mode) {
    epsp_f32((const EPI *)epi, ni, (const SPJ *)spj, nj, (FORCE *)force, trace_mode);
}
void orc_epep_f64(const void *epi, int ni, const void *epj, int nj, double *acc, int *ngb) {
    epep_f64((const EPI *)epi, ni, (const EPJ *)epj, nj, acc, ngb);
}
void orc_epsp_f64(const void *epi, int ni, const void *spj, int nj, double *acc, int trace_mode) {
    epsp_f64((const EPI *)epi, ni, (const SPJ *)spj, nj, acc, trace_mode);
}

// Batched soft force over CSR lists (same list format as p3t_tree_export):
// mode 0 = F32 functors into FORCE records, 1 = FP64 restatement into
// acc4/ngb4.  Particle data come as FDPS records: epi_all[n] (EPIGrav) and
// epj_all[n] (EPJGrav); spj_all is the SPJ record array.
void orc_soft_lists(int mode, int trace_mode, int n_group, const int *i_off, const int *i_idx, const int *j_off,
                    const int *j_idx, const int *s_off, const int *s_idx, const void *epi_all,
                    const void *epj_all, const void *spj_all, void *force_out, double *acc4, int *ngb4,
                    int nthreads) {
    const EPI *EI = (const EPI *)epi_all;
    const EPJ *EJ = (const EPJ *)epj_all;
    const SPJ *SJ = (const SPJ *)spj_all;
    FORCE *F = (FORCE *)force_out;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int g = 0; g < n_group; g++) {
        const int ni = i_off[g + 1] - i_off[g], nj = j_off[g + 1] - j_off[g], ns = s_off[g + 1] - s_off[g];
        std::vector<EPI> ei(ni);
        std::vector<EPJ> ej(nj);
        std::vector<SPJ> sj(ns);
        for (int k = 0; k < ni; k++) ei[k] = EI[i_idx[i_off[g] + k]];
        for (int k = 0; k < nj; k++) ej[k] = EJ[j_idx[j_off[g] + k]];
        for (int k = 0; k < ns; k++) sj[k] = SJ[s_idx[s_off[g] + k]];
        if (mode == 0) {
            std::vector<FORCE> f(ni);
            for (int k = 0; k < ni; k++) {
                f[k] = FORCE{{0.f, 0.f, 0.f}, 0.f, 0, 0, -1, INT_MAX};
            }
            epep_f32(ei.data(), ni, ej.data(), nj, f.data());
            epsp_f32(ei.data(), ni, sj.data(), ns, f.data(), trace_mode);
            for (int k = 0; k < ni; k++) F[i_idx[i_off[g] + k]] = f[k];
        } else {
            std::vector<double> a(4 * ni, 0.);
            std::vector<int> q(4 * ni);
            for (int k = 0; k < ni; k++) { q[4 * k] = 0; q[4 * k + 1] = 0; q[4 * k + 2] = -1; q[4 * k + 3] = INT_MAX; }
            epep_f64(ei.data(), ni, ej.data(), nj, a.data(), q.data());
            epsp_f64(ei.data(), ni, sj.data(), ns, a.data(), trace_mode);
            for (int k = 0; k < ni; k++) {
                const int p = i_idx[i_off[g] + k];
                for (int c = 0; c < 4; c++) acc4[4 * p + c] = a[4 * k + c];
                if (ngb4)
                    for (int c = 0; c < 4; c++) ngb4[4 * p + c] = q[4 * k + c];
            }
        }
    }
}

// --- state API mirroring ref_wrap.cpp ------------------------------------------
void orc_set_params(const double *p) {
    P.eps2 = p[0]; P.eps2_sun = p[1]; P.m_sun = p[2]; P.dt_tree = p[3]; P.dt_min = p[4];
    P.eta = p[5]; P.eta_0 = p[6]; P.eta_sun = p[7]; P.eta_sun0 = p[8]; P.alpha2 = p[9];
    set_gamma(p[10]);
    P.R_cut0 = p[11]; P.R_cut1 = p[12]; P.R_search0 = p[13]; P.R_search1 = p[14];
    P.R_search2 = p[15]; P.R_search3 = p[16]; P.r_cut_min = p[17]; P.r_cut_max = p[18];
    P.p_cut = p[19]; P.dens = p[20];
}
void orc_get_gamma_consts(double *out) {
    out[0] = P.gamma; out[1] = P.g_1_inv; out[2] = P.g_1_inv7; out[3] = P.w_y; out[4] = P.f1;
}
void orc_set_kepler_abs_int(int v) { KEPLER_ABS_INT = v; }
double orc_cutoff_W(double rij, double r_out_inv) { return cut_W(rij, r_out_inv); }
double orc_cutoff_K(double rij, double r_out_inv) { return cut_K(rij, r_out_inv); }
double orc_cutoff_dKdt(double rij, double r_out_inv, double alpha) { return cut_dKdt(rij, r_out_inv, alpha); }
double orc_solve_kepler(double l, double ecc) { return solve_kepler(l, ecc); }

void orc_load(int n, const long long *id, const double *mass, const double *r_planet, const double *f,
              const double *pos, const double *vel) {
    S.assign(n, Ptcl());
    for (int i = 0; i < n; i++) {
        Ptcl &p = S[i];
        std::memset((void *)&p, 0, sizeof(Ptcl));
        p.id = id[i];
        p.mass = mass[i];
        p.r_planet = r_planet[i];
        p.f = f[i];
        p.pos = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p.vel = v3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        p.number = 0; p.rank = 0; p.id_max = -1; p.id_min = INT_MAX;
        p.id_cluster = p.id;
        p.n_cluster = 1;
        if (i == 0 || p.id + 1 > ID_NEXT) ID_NEXT = p.id + 1;
    }
}
// GPLUM's FPGrav record (src/particle.h:93-170,404-500; the build with
// individual cutoffs, quadrupole moments and collisions): 344 bytes.
struct FPGravRec {
    int32_t id_local, myrank;
    double pos[3], r_out, r_search;
    int64_t id;
    double mass, vel[3], acc_d[3], acc[3], acc_s[3], jerk_d[3], jerk_s[3], acc_gd[3];
    double phi, phi_d, phi_s, v_disp, r_out_inv, time, dt, acc0, r_planet, f;
    int32_t number, rank, id_max, id_min;
    int64_t id_cluster;
    int32_t n_cluster;
    uint8_t in_domain, is_sent, is_dead, is_merged;
};
static_assert(sizeof(FPGravRec) == 344, "FPGrav record");

// The whole state from FPGrav records (every field the step carries); the
// neighbour lists of the last correction are kept.  id_next < 0: unchanged.
void orc_put_fpgrav(int n, const void *records, long long id_next) {
    const FPGravRec *r = (const FPGravRec *)records;
    S.assign(n, Ptcl());
    for (int i = 0; i < n; i++) {
        Ptcl &p = S[i];
        const FPGravRec &q = r[i];
        std::memset((void *)&p, 0, sizeof(Ptcl));
        p.id = q.id;
        p.mass = q.mass;
        p.r_planet = q.r_planet;
        p.f = q.f;
        p.pos = v3(q.pos[0], q.pos[1], q.pos[2]);
        p.vel = v3(q.vel[0], q.vel[1], q.vel[2]);
        p.acc = v3(q.acc[0], q.acc[1], q.acc[2]);
        p.acc_d = v3(q.acc_d[0], q.acc_d[1], q.acc_d[2]);
        p.jerk_d = v3(q.jerk_d[0], q.jerk_d[1], q.jerk_d[2]);
        p.acc_s = v3(q.acc_s[0], q.acc_s[1], q.acc_s[2]);
        p.jerk_s = v3(q.jerk_s[0], q.jerk_s[1], q.jerk_s[2]);
        p.phi = q.phi; p.phi_d = q.phi_d; p.phi_s = q.phi_s;
        p.r_out = q.r_out; p.r_out_inv = q.r_out_inv; p.r_search = q.r_search; p.v_disp = q.v_disp;
        p.time = q.time; p.dt = q.dt; p.acc0 = q.acc0;
        p.number = q.number; p.rank = q.rank; p.id_max = q.id_max; p.id_min = q.id_min;
        p.id_cluster = q.id_cluster;
        p.n_cluster = q.n_cluster;
        p.dead = q.is_dead != 0;
        p.merged = q.is_merged != 0;
        p.id_local = i;
    }
    if (id_next >= 0) ID_NEXT = id_next;
}
int orc_n() { return (int)S.size(); }

void orc_get_f64(int field, double *out) {
    const int n = (int)S.size();
    for (int i = 0; i < n; i++) {
        const Ptcl &p = S[i];
        const V3 *v = nullptr;
        switch (field) {
            case 0: v = &p.pos; break;
            case 1: v = &p.vel; break;
            case 2: v = &p.acc; break;
            case 3: v = &p.acc_d; break;
            case 4: v = &p.jerk_d; break;
            case 5: v = &p.acc_s; break;
            case 6: v = &p.jerk_s; break;
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
        if (v) { out[3 * i] = v->x; out[3 * i + 1] = v->y; out[3 * i + 2] = v->z; }
    }
}
void orc_get_i64(int field, long long *out) {
    const int n = (int)S.size();
    for (int i = 0; i < n; i++) {
        const Ptcl &p = S[i];
        switch (field) {
            case 0: out[i] = p.id; break;
            case 1: out[i] = p.id_cluster; break;
            case 2: out[i] = p.number; break;
            case 3: out[i] = p.n_cluster; break;
            case 4: out[i] = p.dead; break;
            case 5: out[i] = p.merged; break;
            case 6: out[i] = p.rank; break;
            case 7: out[i] = p.id_min; break;
            case 8: out[i] = p.id_max; break;
            default: break;
        }
    }
}
void orc_set_f64(int field, const double *in) {
    const int n = (int)S.size();
    for (int i = 0; i < n; i++) {
        Ptcl &p = S[i];
        switch (field) {
            case 0: p.pos = v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
            case 1: p.vel = v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
            case 3: p.acc_d = v3(in[3 * i], in[3 * i + 1], in[3 * i + 2]); break;
            case 14: p.r_out = in[i]; break;
            case 15: p.r_search = in[i]; break;
            case 21: p.r_out_inv = in[i]; break;
            default: break;
        }
    }
}
void orc_set_id_local() {
    for (int i = 0; i < (int)S.size(); i++) S[i].id_local = i;
}
void orc_set_cutoff_radii() { set_cutoff_radii(); }
void orc_set_r_planet() {
    for (Ptcl &p : S) p.r_planet = std::pow(0.75 * p.mass / (3.14159265358979323846 * P.dens), 1. / 3.);
}

// Export the EPI/EPJ records of the current state (FPGrav -> EPIGrav/EPJGrav
// copyFromFP, src/particle.h:127-169).
void orc_export_ep(void *epi_out, void *epj_out) {
    EPI *ei = (EPI *)epi_out;
    EPJ *ej = (EPJ *)epj_out;
    for (int i = 0; i < (int)S.size(); i++) {
        const Ptcl &p = S[i];
        EPI a;
        a.id_local = p.id_local; a.myrank = 0;
        a.pos[0] = p.pos.x; a.pos[1] = p.pos.y; a.pos[2] = p.pos.z;
        a.r_out = p.r_out; a.r_search = p.r_search;
        if (ei) ei[i] = a;
        if (ej) {
            EPJ b;
            std::memcpy((void *)&b, &a, sizeof(EPI));
            b.id = p.id; b.mass = p.mass;
            b.vel[0] = p.vel.x; b.vel[1] = p.vel.y; b.vel[2] = p.vel.z;
            b.acc_d[0] = p.acc_d.x; b.acc_d[1] = p.acc_d.y; b.acc_d[2] = p.acc_d.z;
            ej[i] = b;
        }
    }
}

// Soft force on the current state with caller-supplied lists, then
// FPGrav::copyFromForce (src/particle.h:761-766).
void orc_soft_force(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                    const int *s_off, const int *s_idx, const void *spj_all) {
    const int n = (int)S.size();
    std::vector<EPI> ei(n);
    std::vector<EPJ> ej(n);
    std::vector<FORCE> f(n);
    orc_export_ep(ei.data(), ej.data());
    orc_soft_lists(0, 0, n_group, i_off, i_idx, j_off, j_idx, s_off, s_idx, ei.data(), ej.data(), spj_all,
                   f.data(), nullptr, nullptr, omp_get_max_threads());
    for (int i = 0; i < n; i++) {
        S[i].acc = v3(f[i].acc[0], f[i].acc[1], f[i].acc[2]);
        S[i].phi = f[i].phi;
        S[i].number = f[i].number; S[i].rank = f[i].rank; S[i].id_max = f[i].id_max; S[i].id_min = f[i].id_min;
    }
}
// Overwrite the kernel outputs (acc, phi, neighbour info) from FORCE records.
void orc_set_force(const void *force) {
    const FORCE *f = (const FORCE *)force;
    for (int i = 0; i < (int)S.size(); i++) {
        S[i].acc = v3(f[i].acc[0], f[i].acc[1], f[i].acc[2]);
        S[i].phi = f[i].phi;
        S[i].number = f[i].number; S[i].rank = f[i].rank; S[i].id_max = f[i].id_max; S[i].id_min = f[i].id_min;
    }
}

void orc_correct(int initial) { correct_all(initial != 0); }
int orc_n_ngb_tot() { return N_NGB_TOT; }
int orc_n_with_ngb() { return N_WITH_NGB; }
int orc_n_pairs() { return (int)PAIRS.size(); }
void orc_get_pairs(int *out) {
    for (size_t k = 0; k < PAIRS.size(); k++) { out[2 * k] = PAIRS[k].first; out[2 * k + 1] = PAIRS[k].second; }
}
int orc_n_list_size(int i) { return (int)NLIST[i].size(); }
void orc_n_list(int i, long long *out) {
    for (size_t k = 0; k < NLIST[i].size(); k++) out[k] = NLIST[i][k];
}
void orc_cluster() { cluster_all(); }
// KOMINAMI fragmentation parameters (a_frag = 0: perfect accretion) and the
// fragment-phase generator (0 keyed, 1 drand48 seeded here)
void orc_set_frag(double a_frag, int n_frag, double m_min, int rng_mode, unsigned long long seed) {
    A_FRAG = a_frag;
    N_FRAG = n_frag;
    M_MIN = m_min;
    FRAG_RNG = rng_mode;
    FRAG_SEED = seed;
    if (rng_mode == 1) srand48((long)seed);
}
long long orc_id_next() { return ID_NEXT; }
// One collision in isolation (the counterpart of ref_collide_unit in
// oracle/ref_build/ref_wrap.cpp; record layout UNIT_FIELDS of harness.py).
int orc_collide_unit(int n, const double *in, int n_tw, const int *tw, int imp, int tar, long long *id_next,
                     double *out, int cap, double *edisp) {
    std::vector<HPtcl> c(n);
    for (int i = 0; i < n; i++) {
        const double *r = in + 26 * i;
        HPtcl &p = c[i];
        std::memset((void *)&p, 0, sizeof(HPtcl));
        p.pos = v3(r[0], r[1], r[2]);
        p.vel = v3(r[3], r[4], r[5]);
        p.mass = r[6]; p.r_planet = r[7]; p.f = r[8]; p.r_out = r[9]; p.r_out_inv = r[10];
        p.r_search = r[11]; p.v_disp = r[12]; p.time = r[13]; p.time_c = r[14]; p.dt = r[15];
        p.phi = r[16]; p.phi_d = r[17]; p.phi_s = r[18]; p.acc0 = r[19];
        p.id = (int64_t)r[20]; p.id_cluster = (int64_t)r[21]; p.number = (int32_t)r[22];
        p.dead = r[23] != 0.; p.merged = r[24] != 0.;
    }
    std::map<int, std::vector<int>> twins;
    for (int k = 0; k < n_tw; k++) twins[tw[2 * k]].push_back(tw[2 * k + 1]);
    ColRec rec;
    double e1 = 0., e2 = 0.;
    int64_t idn = *id_next;
    const int nf = collide(c, twins, imp, tar, e1, e2, rec, idn);
    LAST_UNIT = rec;
    *id_next = idn;
    edisp[0] = e1;
    edisp[1] = e2;
    for (int i = 0; i < (int)c.size() && i < cap; i++) {
        double *r = out + 26 * i;
        const HPtcl &p = c[i];
        r[0] = p.pos.x; r[1] = p.pos.y; r[2] = p.pos.z; r[3] = p.vel.x; r[4] = p.vel.y; r[5] = p.vel.z;
        r[6] = p.mass; r[7] = p.r_planet; r[8] = p.f; r[9] = p.r_out; r[10] = p.r_out_inv;
        r[11] = p.r_search; r[12] = p.v_disp; r[13] = p.time; r[14] = p.time_c; r[15] = p.dt;
        r[16] = p.phi; r[17] = p.phi_d; r[18] = p.phi_s; r[19] = p.acc0;
        r[20] = (double)p.id; r[21] = (double)p.id_cluster; r[22] = p.number;
        r[23] = p.dead; r[24] = p.merged; r[25] = 0.;
    }
    return nf;
}
void orc_kick() {
    for (Ptcl &p : S) p.vel += 0.5 * P.dt_tree * p.acc;
}
int orc_hard(int istep, long long *col_out, int col_cap, double *edisp_out) {
    const int nc = hard_all(istep);
    for (int k = 0; k < nc && k < col_cap; k++) { col_out[2 * k] = COLS[k].id_imp; col_out[2 * k + 1] = COLS[k].id_tar; }
    edisp_out[0] = EDISP;
    edisp_out[1] = EDISP_D;
    return nc;
}
// record k of the last hard part: time id_imp id_tar n_frag id_frag mass_imp
// mass_tar mass_frag pos_imp(3) pos_tar(3) vel_imp(3) vel_tar(3) flag
// dpos_g_rel dvel_g_rel (25 doubles)
static void put_record(const ColRec &r, double *o) {
    o[0] = r.time; o[1] = (double)r.id_imp; o[2] = (double)r.id_tar; o[3] = r.n_frag;
    o[4] = r.n_frag ? (double)r.id_frag : 0.;
    o[5] = r.mass_imp; o[6] = r.mass_tar; o[7] = r.mass_frag;
    const V3 v[4] = {r.pos_imp, r.pos_tar, r.vel_imp, r.vel_tar};
    for (int q = 0; q < 4; q++) { o[8 + 3 * q] = v[q].x; o[9 + 3 * q] = v[q].y; o[10 + 3 * q] = v[q].z; }
    o[20] = 1.;  // flag_merge
    o[21] = r.dpos_g_rel; o[22] = r.dvel_g_rel; o[23] = o[24] = 0.;
}
void orc_col_record(int k, double *out) { put_record(COLS[k], out); }
void orc_last_unit_record(double *out) { put_record(LAST_UNIT, out); }
void orc_col_edisp(int k, double *out) {
    out[0] = COLS[k].edisp;
    out[1] = COLS[k].edisp_d;
}
int orc_n_cluster() { return N_CLUSTER; }
int orc_n_isolated() { return N_ISO; }
void orc_energy(double *out) {  // Energy::calcEnergy, src/energy.h:29-63
    double ek = 0., es = 0., ep = 0., ed = 0.;
    for (const Ptcl &p : S) {
        const V3 mv = p.mass * p.vel;
        ek += dot(mv, p.vel);
        es += p.mass * p.phi_s;
        ep += p.mass * p.phi;
        ed += p.mass * p.phi_d;
    }
    ek *= 0.5; ep *= 0.5; ed *= 0.5;
    out[1] = ek; out[2] = es; out[3] = ep; out[4] = ed;
    out[0] = ek + es + (ep + ed);
}
// removeParticlesOutOfBoundary, src/func.h:209-355: bodies with |x|^2 above
// r_max^2 or below r_min^2 leave; their kinetic and potential energies and
// their mutual potential go to the dissipated energy (list in index order,
// the single-thread order of the reference's critical section).
int orc_remove(double r_max, double r_min, double *edisp) {
    const double rmax2 = r_max * r_max, rmin2 = r_min * r_min;
    std::vector<int> rl;
    for (int i = 0; i < (int)S.size(); i++) {
        const double pos2 = dot(S[i].pos, S[i].pos);
        if (pos2 > rmax2 || pos2 < rmin2) rl.push_back(i);
    }
    double e = 0.;
    for (size_t i = 0; i < rl.size(); i++) {
        const Ptcl &a = S[rl[i]];
        const double massi = a.mass;
        const V3 veli = a.vel;
        e -= dot(0.5 * massi * veli, veli);
        e -= massi * a.phi_s;
        e -= massi * a.phi_d;
        e -= massi * a.phi;
        for (size_t j = 0; j < i; j++) {
            const Ptcl &b = S[rl[j]];
            if (a.id != b.id) {
                const V3 dr = a.pos - b.pos;
                const double rinv = 1. / std::sqrt(dot(dr, dr) + P.eps2);
                e += -massi * b.mass * rinv;
            }
        }
    }
    if (!rl.empty()) {
        std::vector<char> gone(S.size(), 0);
        for (int i : rl) gone[i] = 1;
        size_t w = 0;
        for (size_t r = 0; r < S.size(); r++)
            if (!gone[r]) S[w++] = S[r];
        S.resize(w);
    }
    *edisp += e;
    return (int)rl.size();
}
// MergeParticle, src/func.h:160-207 (order-preserving removal)
void orc_merge(int n_col, double *edisp) {
    (void)n_col;
    const int n = (int)S.size();
    std::vector<char> gone(n, 0);
    double e = 0.;
    for (int i = 0; i < n; i++) {
        if (S[i].merged && !S[i].dead) {
            for (int j = 0; j < n; j++) {
                if (S[j].id == S[i].id && i != j) {
                    const double mi = S[i].mass, mj = S[j].mass;
                    const V3 vrel = S[j].vel - S[i].vel;
                    S[i].mass += mj;
                    S[i].vel = (mi * S[i].vel + mj * S[j].vel) / (mi + mj);
                    S[i].phi = (mi * S[i].phi + mj * S[j].phi) / (mi + mj);
                    S[i].phi_d = (mi * S[i].phi_d + mj * S[j].phi_d) / (mi + mj);
                    e -= dot(0.5 * mi * mj / (mi + mj) * vrel, vrel);
                    gone[j] = 1;
                }
            }
            S[i].merged = false;
        }
    }
    *edisp += e;
    size_t w = 0;
    for (int r = 0; r < n; r++)
        if (!gone[r]) S[w++] = S[r];
    S.resize(w);
}

}  // extern "C"
