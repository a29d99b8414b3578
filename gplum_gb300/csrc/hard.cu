// Hard part of the P3T step on the device: every neighbour cluster of the
// step in one persistent launch, one warp per cluster taken from a device
// work queue, 4th-order block-timestep Hermite with collision detection and
// perfect accretion (src/hermite.h:224-479, src/hard.h:554-829,
// src/collisionA.h:86-706 of GPLUM); isolated bodies take the Kepler drift
// or the sun-only Hermite (src/hermite.h:734-815, src/kepler.h).
// Compiled with -fmad=false (see p3t_phys.cuh).
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_engine.cuh"
#include "p3t_phys.cuh"

namespace p3t {

constexpr int MAX_BLOCK_STEPS = 1 << 20;  // per cluster and tree step
// phases of the bundle form's loop, for its optional clock counts (the order
// of p3t_hard_phase_cycles)
enum : int {
    HP_LONE, HP_ADMIT, HP_TS, HP_PREDICT, HP_DETECT, HP_ACTIVE, HP_PAIRS, HP_FINAL, HP_CORRECT, HP_DT, HP_COLLIDE,
    HP_TIME, HP_RETIRE, HP_DRAIN, HP_N
};

// Per-member working copy of one cluster (FPHard fields), indexed by the
// member's slot in the cluster lists.
struct Hard {
    double *pos, *vel, *acc_s, *jerk_s, *acc_d, *jerk_d;
    double *x0, *v0, *a0_s, *j0_s, *a0_d, *j0_d, *xp, *vp, *a2_s, *a3_s, *a2_d, *a3_d;
    double *phi_d, *phi_s, *mass, *r_planet, *f, *r_out_inv, *th, *dt, *acc0, *time_c;
    int64_t *id;
    int32_t *dead, *merged, *tw_head, *tw_tail, *tw_next;
    // FP32 copies of corrected and predicted positions relative to the
    // cluster's first member, of r_out_inv and of f * r_planet: a cheap
    // distance prefilter
    float *pos32, *xp32, *roi32, *fr32;
};

// Per-cluster prefilter state (uniform across the team).
struct Pre {
    bool on;          // prefilter proven safe for this cluster
    double ref[3];    // origin of the FP32 coordinates
};
__device__ __forceinline__ void st32(float *p, int s, V3 x, const Pre &pre) {
    p[3 * s] = (float)(x.x - pre.ref[0]);
    p[3 * s + 1] = (float)(x.y - pre.ref[1]);
    p[3 * s + 2] = (float)(x.z - pre.ref[2]);
}
__device__ __forceinline__ float d2_32(const float *a, int s, const float *b, int t) {
    const float dx = a[3 * s] - b[3 * t], dy = a[3 * s + 1] - b[3 * t + 1], dz = a[3 * s + 2] - b[3 * t + 2];
    return dx * dx + dy * dy + dz * dz;
}

struct ColRec {
    int64_t id_imp, id_tar;
    double time, edisp, edisp_d;
    int32_t cluster, seq, n;  // cluster index, collision number within it, cluster size
    int32_t n_frag, frag0;    // fragments made (KOMINAMI) and the first one's fragment index
    int64_t id_frag;          // temporary id of the first fragment (the others count down)
    // the collision-file record (Collision0::write2File, src/collisionA.h:122-148):
    // masses (twins included) and states before the collision, and the
    // relative shifts of the centre of mass, |pos_g_new - pos_g| / |pos_g| etc.
    double mass_imp, mass_tar, mass_frag;
    double pos_imp[3], pos_tar[3], vel_imp[3], vel_tar[3];
    double dpos_g_rel, dvel_g_rel;
};

// One fragment (KOMINAMI), in creation order within its cluster: the FPGrav
// fields the hard part does not carry, copied from the impactor
// (src/collisionA.h:293-316), and where its hard state lives.
struct FragRec {
    int32_t cluster, seq, gslot, n_cl;  // cluster, creation number in it, hard slot, final cluster size
    double r_out, r_search, v_disp, phi;
    int32_t number, n0;  // impactor's neighbour count (setNeighbors); its cluster's size at admission
    int64_t id_cluster;
};

// KOMINAMI fragmentation (src/collisionB.h:7-93); a_frag = 0 turns it off
struct FragParams {
    double a_frag, m_min;
    int n_frag_max, istep;
    unsigned long long seed;
};

struct HardArgs {
    State S;
    Params P;
    Hard H;
    const int32_t *off, *cnt, *members, *order;
    int n_clusters;
    const int *n_tier;   // [3] clusters per tier, in `order` (device)
    int32_t *queue;      // [3] tier queue heads
    long long *cost;     // optional [2 * n_clusters]: block steps, pair sweeps
    long long *times;    // optional [2 * n_clusters]: start, end (global timer, ns)
    double *cl_edisp;  // [2 * n_clusters]
    ColRec *cols;
    int32_t *n_cols;
    int col_cap;
    int *status;
    double t_end;
    FragParams frag;
    FragRec *frags;      // [frag_cap] fragments of this launch
    int32_t *n_frags;    // fragments made so far
    int frag_base, frag_cap;  // hard slots frag_base + k hold fragment k
    int wide;                 // bundle form: clusters above BCAP_MAIN in k_hard_wide (1) or run_cluster (0)
    int max_steps;            // block steps a cluster may take in one tree step (ST_ITER_CAP beyond)
    int lone_in;              // bundle form: the lone tier runs in the bundle CTAs (1) or in k_hard_lone (0)
    unsigned long long *phase_cycles;  // optional [HP_N]: clock cycles per phase of the bundle loop, all CTAs
    unsigned long long *live; // optional [2]: pair terms evaluated (predicted/corrected, full), bundle form
};

// ---- FPHard::predict / correct / calcDeltat, src/particle.h:1183-1314 ----
// the predicted position and velocity also come back to the caller (no
// reload of what was just stored)
__device__ __forceinline__ void predict(const Hard &H, int s, double Dt, V3 &xp, V3 &vp) {
    const V3 pos = ld3(H.pos, s), vel = ld3(H.vel, s), as = ld3(H.acc_s, s), js = ld3(H.jerk_s, s),
             ad = ld3(H.acc_d, s), jd = ld3(H.jerk_d, s);
    // FPHard's x0 and v0 (the step's start) are never read here: not stored
    st3(H.a0_s, s, as); st3(H.j0_s, s, js); st3(H.j0_d, s, jd);
    st3(H.a0_d, s, ad);
    const V3 a = as + ad, j = js + jd;
    xp = pos + Dt * (vel + Dt * (0.5 * a + 1.6666666666666667e-1 * Dt * j));
    vp = vel + Dt * (a + Dt * 0.5 * j);
    st3(H.xp, s, xp);
    st3(H.vp, s, vp);
}
__device__ __forceinline__ void predict(const Hard &H, int s, double Dt) {
    V3 xp, vp;
    predict(H, s, Dt, xp, vp);
}
__device__ __forceinline__ void correct(const Hard &H, int s, double Dt) {
    const double Dt2 = Dt * Dt, Di = recip_pow2_or_div(Dt), Di2 = Di * Di, Di3 = Di2 * Di;
    const V3 Am_s = ld3(H.acc_s, s) - ld3(H.a0_s, s), J0_s = Dt * ld3(H.j0_s, s), J1_s = Dt * ld3(H.jerk_s, s);
    const V3 A2_s = 3. * Am_s - (J1_s + 2. * J0_s);
    const V3 A3_s = -2. * Am_s + (J1_s + J0_s);
    st3(H.a2_s, s, 2. * Di2 * (A2_s + 3. * A3_s));
    st3(H.a3_s, s, 6. * Di3 * A3_s);
    const V3 Am_d = ld3(H.acc_d, s) - ld3(H.a0_d, s), J0_d = ld3(H.j0_d, s) * Dt, J1_d = ld3(H.jerk_d, s) * Dt;
    const V3 A2_d = 3. * Am_d - (J1_d + 2. * J0_d);
    const V3 A3_d = -2. * Am_d + (J1_d + J0_d);
    st3(H.a2_d, s, 2. * (A2_d + 3. * A3_d) * Di2);
    st3(H.a3_d, s, 6. * A3_d * Di3);
    const V3 A2 = A2_s + A2_d, A3 = A3_s + A3_d;
    st3(H.pos, s, ld3(H.xp, s) + 1.6666666666666667e-2 * Dt2 * (5. * A2 + 3. * 1.1666666666666667e-3 * A3));
    st3(H.vel, s, ld3(H.vp, s) + 8.3333333333333333e-2 * Dt * (4. * A2 + 3. * A3));
}
// the next time step from the current one, the member's time and dt_1, the
// smaller of its two criteria (the rest of FPHard::calcDeltat)
__device__ __forceinline__ double dt_next_hermite(const Params &P, double time, double dt, double dt_1) {
    double dt_next = dmin(2. * dt, 0.5 * P.dt_tree);
    double rem = rem_pow2(time, dt_next);
    for (int k = 0; rem != 0.0 && k < 1100; k++) {
        dt_next *= 0.5;
        rem = rem_pow2(time, dt_next);
    }
    for (int k = 0; dt_1 < dt_next && 0.5 * dt < dt_next && k < 1100; k++) dt_next *= 0.5;
    if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
    return dt_next;
}
__device__ __forceinline__ void dt_hermite(const Params &P, const Hard &H, int s) {
    const double dt_1 = dmin(dt4th(P.eta, P.alpha2, H.acc0[s], ld3(H.acc_d, s), ld3(H.jerk_d, s), ld3(H.a2_d, s),
                                   ld3(H.a3_d, s)),
                             dt4th(P.eta_sun, P.alpha2, 0., ld3(H.acc_s, s), ld3(H.jerk_s, s), ld3(H.a2_s, s),
                                   ld3(H.a3_s, s)));
    H.dt[s] = dt_next_hermite(P, H.th[s], H.dt[s], dt_1);
}

// ---- pair sums over a cluster, src/gravity_hard.h:203-367 -------------------
// mode 0: full (pos/vel, with phi); 1: predicted i and j; 2: corrected i, predicted j
//
// Pairs at rij >= r_out (here: dr2 * r_out_inv^2 > 1 + 1e-6, a margin far
// above rounding) have K = W = 1 and dK/dr = 0 exactly, so their terms are
// exact zeros; they are skipped after the distance test, which leaves every
// sum bit-identical (the accumulators start at +0 and never become -0).
//
// With the FP32 prefilter on, a pair is first tested on the FP32 relative
// coordinates: it is skipped when its FP32 distance exceeds twice the cutoff
// radius, which the prefilter's safety condition (run_cluster) guarantees is
// beyond the cutoff in exact arithmetic too.
__device__ void hard_force(const Params &P, const Hard &H, int o, int n, int s, int mode, const Pre &pre) {
    V3 xi, vi, as, js;
    if (mode == 0) {
        xi = ld3(H.pos, s); vi = ld3(H.vel, s);
        double phs;
        sun_force(P, xi, vi, as, js, &phs);
        H.phi_s[s] = phs;
    } else if (mode == 1) {
        xi = ld3(H.xp, s); vi = ld3(H.vp, s);
        sun_force(P, xi, vi, as, js, nullptr);
    } else {
        xi = ld3(H.pos, s); vi = ld3(H.vel, s);
        sun_force(P, xi, vi, as, js, nullptr);
    }
    st3(H.acc_s, s, as);
    st3(H.jerk_s, s, js);
    V3 ad = v3(0., 0., 0.), jd = v3(0., 0., 0.);
    double phd = 0.;
    const int64_t idi = H.id[s];
    const double roi = H.r_out_inv[s];
    const double *X = (mode == 0) ? H.pos : H.xp;
    const float *xi32 = (mode == 1) ? H.xp32 : H.pos32;
    const float *xj32 = (mode == 0) ? H.pos32 : H.xp32;
    const float roi32 = H.roi32[s];
    for (int k = 0; k < n; k++) {
        const int t = o + k;
        if (idi == H.id[t]) continue;
        if (pre.on) {
            const float rf = fminf(roi32, H.roi32[t]);
            if (d2_32(xi32, s, xj32, t) * (rf * rf) > 4.0f) continue;
        }
        const V3 dr = ld3(X, t) - xi;
        double dr2 = dot(dr, dr);
        dr2 += P.eps2;
        const double r_out_inv = dmin(roi, H.r_out_inv[t]);
        if (dr2 * r_out_inv * r_out_inv > 1.000001) continue;
        const V3 vj = (mode == 0) ? ld3(H.vel, t) : ld3(H.vp, t);
        const V3 dv = vj - vi;
        const double rij = sqrt(dr2);
        const double rinv = 1. / rij;
        const double r2inv = rinv * rinv;
        const double r3inv = r2inv * rinv;
        const double mj = H.mass[t];
        const double mr3 = mj * r3inv;
        const double alpha = dot(dr, dv) * r2inv;
        double Wc = 0.;
        if (mode == 0) Wc = 1. - cut_W(P, rij, r_out_inv);
        const double Kc = 1. - cut_K(P, rij, r_out_inv);
        const double dKdt = cut_dKdt(P, rij, r_out_inv, alpha);
        const double alpha_c = alpha * Kc;
        if (mode == 0) phd -= mj * rinv * Wc;
        addto(ad, mr3 * Kc * dr);
        addto(jd, mr3 * (Kc * dv - (3. * alpha_c + dKdt) * dr));
    }
    if (mode == 0) H.phi_d[s] = phd;
    st3(H.acc_d, s, ad);
    st3(H.jerk_d, s, jd);
}

// mergeAccJerk for target t, src/hermite.h:36-83 (twins in insertion order)
__device__ void merge_acc_jerk(const Hard &H, int t) {
    V3 a = H.mass[t] * ld3(H.acc_d, t), j = H.mass[t] * ld3(H.jerk_d, t);
    double m = H.mass[t];
    for (int k = H.tw_head[t], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        addto(a, H.mass[k] * ld3(H.acc_d, k));
        addto(j, H.mass[k] * ld3(H.jerk_d, k));
        m += H.mass[k];
    }
    const double mi = 1. / m;
    a = a * mi;
    j = j * mi;
    st3(H.acc_d, t, a);
    st3(H.jerk_d, t, j);
    for (int k = H.tw_head[t], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        st3(H.acc_d, k, a);
        st3(H.jerk_d, k, j);
    }
}

__device__ __forceinline__ double cut_W2(const Params &P, double dr2, double a, double b) {
    return cut_W(P, sqrt(dr2), dmin(a, b));
}

// The fragment-circle phase: a counter-based draw keyed by (tree step,
// impactor id, target id, seed) -- GPLUM draws drand48() from OpenMP threads
// (src/collisionA.h:727), whose order is not reproducible; the oracle uses
// the same keyed draw.  splitmix64 finaliser, 53-bit uniform in [0, 1).
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double frag_uniform(const FragParams &F, long long id_imp, long long id_tar) {
    unsigned long long h = mix64(F.seed ^ 0x5851f42d4c957f2dULL);
    h = mix64(h ^ (unsigned long long)(long long)F.istep);
    h = mix64(h ^ (unsigned long long)id_imp);
    h = mix64(h ^ (unsigned long long)id_tar);
    return (double)(h >> 11) * 0x1.0p-53;
}

// Where one cluster's fragments go and what they inherit (bundle form only).
struct FragCtx {
    const HardArgs *A;
    const int *mem;      // hard slots of the cluster's members, in member order
    int n;               // members (earlier fragments included)
    int cluster;
    long long label;     // the cluster's id_cluster
    long long *id_next;  // fragments made in this cluster so far (src/hermite.h:243)
    int *out_slots;      // [n_frag_max]: hard slots of the new fragments
};

// Collision0::inputPair, the KOMINAMI collisionOutcome with setFragmentCircle
// (src/collisionB.h:43-93, src/collisionA.h:708-742), Collision0::setParticle,
// calcEnergyDissipation and setNeighbors (src/collisionA.h:86-706) with the
// merge-list update (src/hermite.h:395-423).  One lane.  Without a fragment
// context (or with a_frag = 0) this is perfect accretion.  Returns the
// number of fragments, whose hard slots are written to X->out_slots.
__device__ int collide(const Params &P, const Hard &H, int imp, int tar, double &edisp, double &edisp_d,
                       ColRec &rec, const FragCtx *X) {
    rec.id_imp = H.id[imp];
    rec.id_tar = H.id[tar];
    rec.time = H.time_c[imp] + H.th[imp];
    rec.n_frag = 0;
    rec.frag0 = -1;
    rec.id_frag = 0;
    const V3 pos_imp = ld3(H.pos, imp), pos_tar = ld3(H.pos, tar), vel_imp = ld3(H.vel, imp),
             vel_tar = ld3(H.vel, tar);
    double m_imp = H.mass[imp], m_tar = H.mass[tar];
    if (H.merged[imp])
        for (int k = H.tw_head[imp], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) m_imp += H.mass[k];
    if (H.merged[tar])
        for (int k = H.tw_head[tar], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) m_tar += H.mass[k];
    const double r_planet_tar = H.r_planet[tar], f_imp = H.f[imp], f_tar = H.f[tar];
    const V3 vel_g = (m_imp * vel_imp + m_tar * vel_tar) / (m_imp + m_tar);
    const V3 pos_g = (m_imp * pos_imp + m_tar * pos_tar) / (m_imp + m_tar);
    // collisionOutcome (KOMINAMI)
    int n_frag = 0;
    const FragParams *F = X ? &X->A->frag : nullptr;
    if (F && F->a_frag > 0.) {
        n_frag = (int)floor(F->a_frag * m_imp / F->m_min);
        if (n_frag < 2) n_frag = 0;
        if (n_frag > F->n_frag_max) n_frag = F->n_frag_max;
    }
    const double mass_frag = n_frag ? (F->a_frag * m_imp) : 0.;
    const double mass_rem = m_imp + m_tar - mass_frag;
    V3 masspos = v3(0., 0., 0.), massvel = v3(0., 0., 0.);
    int f0 = 0;
    if (n_frag && !X->mem) {  // the one-cluster-per-CTA form does not place fragments
        atomicOr(X->A->status, ST_CLUSTER_TOO_BIG);
        n_frag = 0;
    }
    if (n_frag) {
        f0 = atomicAdd(X->A->n_frags, n_frag);
        if (f0 + n_frag > X->A->frag_cap) {
            atomicOr(X->A->status, ST_QUEUE_OVERFLOW);
            n_frag = 0;
        }
    }
    const double mass_frag_k = n_frag ? mass_frag : 0.;
    const double mass_rem_k = n_frag ? mass_rem : m_imp + m_tar - 0.;
    if (n_frag) {
        const V3 ximp = pos_imp - pos_tar, vimp = vel_imp - vel_tar;
        const double f_frag = f_imp;
        const double r_planet_frag = pow(0.75 * mass_frag / n_frag / (3.14159265358979323846 * P.dens), 1. / 3.);
        const double r_planet_rem = pow(mass_rem / m_tar, 1. / 3.) * r_planet_tar;
        const double r_frag = 2. * dmax(f_tar, f_frag) * (r_planet_frag + r_planet_rem);
        const double r2_frag = r_frag * r_frag + P.eps2;
        const double r_frag_inv = sqrt(1. / r2_frag);
        const double v_frag = 1.05 * sqrt(2. * mass_rem * r_frag_inv);
        const double m_f = mass_frag / n_frag;
        // setFragmentCircle
        V3 e0 = ximp;
        V3 e1 = vimp - (dot(vimp, ximp) / dot(ximp, ximp)) * ximp;
        e0 = e0 / sqrt(dot(e0, e0));
        e1 = e1 / sqrt(dot(e1, e1));
        const double theta0 = 2. * 3.14159265358979323846 * frag_uniform(*F, rec.id_imp, rec.id_tar);
        for (int i = 0; i < n_frag; i++) {
            const int gf = X->A->frag_base + f0 + i;
            const double theta = theta0 + 2. * 3.14159265358979323846 * i / n_frag;
            const double ct = cos(theta), st = sin(theta);
            const V3 fp = pos_g + r_frag * (ct * e0 + st * e1);
            const V3 fv = vel_g + v_frag * (ct * e0 + st * e1);
            H.mass[gf] = m_f;
            st3(H.pos, gf, fp);
            st3(H.vel, gf, fv);
            // (the predicted state is rebuilt before it is next read; starting
            // it at the position keeps the bundle's coordinate bound)
            st3(H.xp, gf, fp);
            st3(H.vp, gf, fv);
            masspos = masspos + m_f * fp;
            massvel = massvel + m_f * fv;
        }
    }
    const V3 pos_new = (m_imp * pos_imp + m_tar * pos_tar - masspos) / mass_rem_k;
    const V3 vel_new = (m_imp * vel_imp + m_tar * vel_tar - massvel) / mass_rem_k;
    {
        // the record: Collision0::setParticle's centre of mass after the
        // collision -- fragments (in creation order), then the remnant and the
        // target (src/collisionA.h:232-234,288-291,344-348)
        double mass_tot = 0.;
        for (int i = 0; i < n_frag; i++) mass_tot += mass_frag / n_frag;
        const V3 mp = masspos + ((m_imp - mass_frag_k) * pos_new + m_tar * pos_new);
        const V3 mv = massvel + ((m_imp - mass_frag_k) * vel_new + m_tar * vel_new);
        mass_tot += m_imp - mass_frag_k + m_tar;
        const V3 dpos_g = mp / mass_tot - pos_g, dvel_g = mv / mass_tot - vel_g;
        rec.mass_imp = m_imp;
        rec.mass_tar = m_tar;
        rec.mass_frag = mass_frag_k;
        rec.pos_imp[0] = pos_imp.x; rec.pos_imp[1] = pos_imp.y; rec.pos_imp[2] = pos_imp.z;
        rec.pos_tar[0] = pos_tar.x; rec.pos_tar[1] = pos_tar.y; rec.pos_tar[2] = pos_tar.z;
        rec.vel_imp[0] = vel_imp.x; rec.vel_imp[1] = vel_imp.y; rec.vel_imp[2] = vel_imp.z;
        rec.vel_tar[0] = vel_tar.x; rec.vel_tar[1] = vel_tar.y; rec.vel_tar[2] = vel_tar.z;
        rec.dpos_g_rel = sqrt(dot(dpos_g, dpos_g) / dot(pos_g, pos_g));
        rec.dvel_g_rel = sqrt(dot(dvel_g, dvel_g) / dot(vel_g, vel_g));
    }
    // setParticle (flag_merge)
    H.r_planet[imp] = 0.;
    H.r_planet[tar] *= pow(mass_rem_k / m_tar, 1. / 3.);
    H.mass[imp] -= mass_frag_k;
    H.id[imp] = H.id[tar];
    H.dead[imp] = 1;
    for (int k = H.tw_head[imp], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        H.id[k] = H.id[tar];
        H.dead[k] = 1;
    }
    H.merged[tar] = 1;
    long long id_frag = 0;
    if (n_frag) {
        id_frag = -(128LL * X->label + *X->id_next + 1);
        // the impactor's FPGrav fields the hard part does not carry
        double ro = 0., rs = 0., vd = 0., phi = 0.;
        int num = 0;
        if (imp < X->A->frag_base) {
            const int si = X->A->members[imp];
            ro = X->A->S.r_out[si];
            rs = X->A->S.r_search[si];
            vd = X->A->S.v_disp[si];
            phi = X->A->S.phi[si];
            num = X->A->S.number[si];
        } else {
            const FragRec &R = X->A->frags[imp - X->A->frag_base];
            ro = R.r_out;
            rs = R.r_search;
            vd = R.v_disp;
            phi = R.phi;
            num = R.number;
        }
        for (int i = 0; i < n_frag; i++) {
            const int gf = X->A->frag_base + f0 + i;
            H.r_planet[gf] = pow(0.75 * H.mass[gf] / (3.14159265358979323846 * P.dens), 1. / 3.);  // setRPlanet
            H.f[gf] = H.f[imp];
            H.r_out_inv[gf] = H.r_out_inv[imp];
            H.time_c[gf] = H.time_c[imp];
            H.th[gf] = H.th[imp];
            H.dt[gf] = H.dt[imp];
            H.phi_d[gf] = H.phi_d[imp];
            H.phi_s[gf] = H.phi_s[imp];
            H.acc0[gf] = 0.;  // unset by GPLUM (FPHard()); it enters the time step only squared
            H.id[gf] = id_frag - i;
            H.dead[gf] = 0;
            H.merged[gf] = 0;
            H.tw_head[gf] = H.tw_tail[gf] = H.tw_next[gf] = -1;
            const V3 z = v3(0., 0., 0.);
            st3(H.acc_s, gf, z); st3(H.jerk_s, gf, z); st3(H.acc_d, gf, z); st3(H.jerk_d, gf, z);
            st3(H.x0, gf, z); st3(H.v0, gf, z); st3(H.a0_s, gf, z); st3(H.j0_s, gf, z); st3(H.a0_d, gf, z);
            st3(H.j0_d, gf, z); st3(H.a2_s, gf, z); st3(H.a3_s, gf, z);
            st3(H.a2_d, gf, z); st3(H.a3_d, gf, z);
            FragRec &R = X->A->frags[f0 + i];
            R.cluster = X->cluster;
            R.seq = (int)*X->id_next;
            R.gslot = gf;
            R.n_cl = 0;
            R.r_out = ro;
            R.r_search = rs;
            R.v_disp = vd;
            R.phi = phi;
            R.number = num;  // setNeighbors
            R.n0 = 0;
            R.id_cluster = X->label;
            X->out_slots[i] = gf;
            (*X->id_next)++;
        }
        rec.n_frag = n_frag;
        rec.frag0 = f0;
        rec.id_frag = id_frag;
    }
    st3(H.pos, imp, pos_new); st3(H.vel, imp, vel_new);
    for (int k = H.tw_head[imp], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        st3(H.pos, k, pos_new); st3(H.vel, k, vel_new);
    }
    st3(H.pos, tar, pos_new); st3(H.vel, tar, vel_new);
    for (int k = H.tw_head[tar], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        st3(H.pos, k, pos_new); st3(H.vel, k, vel_new);
    }
    // calcEnergyDissipation
    const double m_i = H.mass[imp] + mass_frag_k;
    double e_kin = 0.;
    V3 vr = vel_imp - vel_tar;
    e_kin -= dot(0.5 * m_imp * m_tar / (m_imp + m_tar) * vr, vr);
    vr = vel_new - vel_g;
    e_kin += dot(0.5 * (m_imp - mass_frag_k) * vr, vr);
    vr = vel_new - vel_g;
    e_kin += dot(0.5 * m_tar * vr, vr);
    for (int i = 0; i < n_frag; i++) {
        const int gf = X->A->frag_base + f0 + i;
        vr = ld3(H.vel, gf) - vel_g;
        e_kin += dot(0.5 * H.mass[gf] * vr, vr);
    }
    double e_int = 0., e_int_d = 0.;
    V3 dr = pos_imp - pos_tar;
    double dr2 = dot(dr, dr) + P.eps2;
    double rinv = sqrt(1. / dr2), rinv_new;
    double dphi = m_i * rinv;
    e_int += H.mass[tar] * dphi;
    e_int_d += H.mass[tar] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[imp], H.r_out_inv[tar]));
    for (int k = H.tw_head[tar], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
        e_int += H.mass[k] * dphi;
        e_int_d += H.mass[k] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[imp], H.r_out_inv[k]));
    }
    for (int ki = H.tw_head[imp], g = 0; ki >= 0 && g < 4096; ki = H.tw_next[ki], g++) {
        dphi = H.mass[ki] * rinv;
        e_int += H.mass[tar] * dphi;
        e_int_d += H.mass[tar] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[ki], H.r_out_inv[tar]));
        for (int kj = H.tw_head[tar], h = 0; kj >= 0 && h < 4096; kj = H.tw_next[kj], h++) {
            e_int += H.mass[kj] * dphi;
            e_int_d += H.mass[kj] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[ki], H.r_out_inv[kj]));
        }
    }
    if (n_frag) {
        const int fb = X->A->frag_base + f0;
        for (int i = 0; i < n_frag; i++) {
            const int a = fb + i;
            dr = ld3(H.pos, a) - ld3(H.pos, imp);
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = sqrt(1. / dr2);
            dphi = -H.mass[a] * rinv_new;
            e_int += H.mass[imp] * dphi;
            e_int_d += H.mass[imp] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[imp], H.r_out_inv[a]));
            for (int k = H.tw_head[imp], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
                e_int += H.mass[k] * dphi;
                e_int_d += H.mass[k] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[k], H.r_out_inv[a]));
            }
            dr = ld3(H.pos, a) - ld3(H.pos, tar);
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = sqrt(1. / dr2);
            dphi = -H.mass[a] * rinv_new;
            e_int += H.mass[tar] * dphi;
            e_int_d += H.mass[tar] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[tar], H.r_out_inv[a]));
            for (int k = H.tw_head[tar], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
                e_int += H.mass[k] * dphi;
                e_int_d += H.mass[k] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[k], H.r_out_inv[a]));
            }
            for (int j = 0; j < i; j++) {
                const int b = fb + j;
                dr = ld3(H.pos, a) - ld3(H.pos, b);
                dr2 = dot(dr, dr) + P.eps2;
                rinv_new = sqrt(1. / dr2);
                dphi = -H.mass[a] * H.mass[b] * rinv_new;
                e_int += dphi;
                e_int_d += dphi * (1. - cut_W2(P, dr2, H.r_out_inv[a], H.r_out_inv[b]));
            }
        }
        // the other members of the cluster, before the new fragments
        for (int q = 0; q < X->n; q++) {
            const int i = X->mem[q];
            if (H.id[i] == H.id[imp] || H.id[i] == H.id[tar]) continue;
            const double m_nei = H.mass[i];
            dr = pos_imp - ld3(H.pos, i);
            dr2 = dot(dr, dr) + P.eps2;
            rinv = sqrt(1. / dr2);
            dr = ld3(H.pos, imp) - ld3(H.pos, i);
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = sqrt(1. / dr2);
            dphi = m_nei * (rinv - rinv_new);
            e_int += m_nei * (m_i * rinv - H.mass[imp] * rinv_new);
            e_int_d += m_nei * (m_i * rinv - H.mass[imp] * rinv_new) *
                       (1. - cut_W2(P, dr2, H.r_out_inv[imp], H.r_out_inv[i]));
            for (int k = H.tw_head[imp], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
                e_int += H.mass[k] * dphi;
                e_int_d += H.mass[k] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[k], H.r_out_inv[i]));
            }
            for (int j = 0; j < n_frag; j++) {
                const int b = fb + j;
                dr = ld3(H.pos, b) - ld3(H.pos, i);
                dr2 = dot(dr, dr) + P.eps2;
                rinv_new = sqrt(1. / dr2);
                dphi = -m_nei * H.mass[b] * rinv_new;
                e_int += dphi;
                e_int_d += dphi * (1. - cut_W2(P, dr2, H.r_out_inv[b], H.r_out_inv[i]));
            }
            dr = pos_tar - ld3(H.pos, i);
            dr2 = dot(dr, dr) + P.eps2;
            rinv = sqrt(1. / dr2);
            dr = ld3(H.pos, tar) - ld3(H.pos, i);
            dr2 = dot(dr, dr) + P.eps2;
            rinv_new = sqrt(1. / dr2);
            dphi = m_nei * (rinv - rinv_new);
            e_int += H.mass[tar] * dphi;
            e_int_d += H.mass[tar] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[tar], H.r_out_inv[i]));
            for (int k = H.tw_head[tar], g = 0; k >= 0 && g < 4096; k = H.tw_next[k], g++) {
                e_int += H.mass[k] * dphi;
                e_int_d += H.mass[k] * dphi * (1. - cut_W2(P, dr2, H.r_out_inv[k], H.r_out_inv[i]));
            }
        }
    }
    double e_sun = 0.;
    e_sun += m_imp / sqrt(dot(pos_imp, pos_imp) + P.eps2) + m_tar / sqrt(dot(pos_tar, pos_tar) + P.eps2);
    const V3 pt = ld3(H.pos, tar), pi = ld3(H.pos, imp);
    e_sun -= m_tar * sqrt(1. / (dot(pt, pt) + P.eps2));
    e_sun -= (m_imp - mass_frag_k) * sqrt(1. / (dot(pi, pi) + P.eps2));
    for (int i = 0; i < n_frag; i++) {
        const V3 fp = ld3(H.pos, X->A->frag_base + f0 + i);
        e_sun -= H.mass[X->A->frag_base + f0 + i] * sqrt(1. / (dot(fp, fp) + P.eps2));
    }
    e_sun *= P.m_sun;
    edisp = e_kin + e_int + e_sun;
    edisp_d = e_kin + e_int_d + e_sun;
    rec.edisp = edisp;
    rec.edisp_d = edisp_d;
    // merge list: imp, then imp's twins, join tar's list
    auto append = [&](int k) {
        H.tw_next[k] = -1;
        if (H.tw_head[tar] < 0) H.tw_head[tar] = k;
        else H.tw_next[H.tw_tail[tar]] = k;
        H.tw_tail[tar] = k;
    };
    const int imp_first = H.tw_head[imp];
    const bool imp_merged = H.merged[imp] != 0;
    append(imp);
    if (imp_merged) {
        for (int k = imp_first, g = 0; k >= 0 && g < 4096; g++) {
            const int nx = H.tw_next[k];
            append(k);
            k = nx;
        }
        H.tw_head[imp] = H.tw_tail[imp] = -1;
        H.merged[imp] = 0;
    }
    return n_frag;
}

// ---- teams: one thread, one warp or one CTA integrates one cluster ----------
template <int TEAM>
struct Team {
    int rank;
    double *red_d;      // shared scratch (CTA teams)
    long long *red_l;
    __device__ __forceinline__ void sync() const {
        if constexpr (TEAM == 32) __syncwarp();
        else if constexpr (TEAM > 32) __syncthreads();
    }
    __device__ __forceinline__ double min(double v) const {
        if constexpr (TEAM == 1) {
            return v;
        } else {
            for (int o = 16; o > 0; o >>= 1) v = dmin(v, __shfl_xor_sync(0xffffffffu, v, o));
            if constexpr (TEAM == 32) {
                return v;
            } else {
                __syncthreads();
                if ((rank & 31) == 0) red_d[rank >> 5] = v;
                __syncthreads();
                double m = red_d[0];
                for (int w = 1; w < TEAM / 32; w++) m = dmin(m, red_d[w]);
                __syncthreads();
                return m;
            }
        }
    }
    // lexicographic min of (R, p)
    __device__ __forceinline__ void argmin(double &R, long long &p) const {
        if constexpr (TEAM > 1) {
            for (int sh = 16; sh > 0; sh >>= 1) {
                const double R2 = __shfl_xor_sync(0xffffffffu, R, sh);
                const long long p2 = __shfl_xor_sync(0xffffffffu, p, sh);
                if (R2 < R || (R2 == R && p2 < p)) { R = R2; p = p2; }
            }
            if constexpr (TEAM > 32) {
                __syncthreads();
                if ((rank & 31) == 0) { red_d[rank >> 5] = R; red_l[rank >> 5] = p; }
                __syncthreads();
                R = red_d[0];
                p = red_l[0];
                for (int w = 1; w < TEAM / 32; w++)
                    if (red_d[w] < R || (red_d[w] == R && red_l[w] < p)) { R = red_d[w]; p = red_l[w]; }
                __syncthreads();
            }
        }
    }
};

__device__ __forceinline__ long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return (long long)t;
}

// Progress of one cluster's integration (uniform across the team except
// `work`, which each team member counts for its own members).
struct ClusterRun {
    double time = 0.;
    int steps = 0, n_col = 0;
    double ed = 0., edd = 0.;
    long long work = 0;
    long long t_start = 0;
};

// timeIntegrate_multi, src/hermite.h:224-479, for cluster c by a team, in
// three parts: load (FPHard from FPGrav, the prefilter, the first full
// force), the block-step loop from run.time on, and the finish (last full
// force, write-back, logs).  The lone-cluster form (hard_lone.cuh) runs its
// own block steps and hands each block step that has a collision to
// cluster_loop (one_step).
template <int TEAM>
__device__ void cluster_load(const HardArgs &A, int c, const Team<TEAM> &tm, Pre &pre) {
    const Params &P = A.P;
    const Hard &H = A.H;
    const int rank = tm.rank;
    const int o = A.off[c], n = A.cnt[c];
    // FPHard(const FPGrav&), src/particle.h:1096-1116
    for (int k = rank; k < n; k += TEAM) {
        const int s = o + k, i = A.members[s];
        st3(H.pos, s, ld3(A.S.pos, i)); st3(H.vel, s, ld3(A.S.vel, i));
        st3(H.acc_s, s, ld3(A.S.acc_s, i)); st3(H.jerk_s, s, ld3(A.S.jerk_s, i));
        st3(H.acc_d, s, ld3(A.S.acc_d, i)); st3(H.jerk_d, s, ld3(A.S.jerk_d, i));
        const V3 z = v3(0., 0., 0.);
        st3(H.x0, s, z); st3(H.v0, s, z); st3(H.a0_s, s, z); st3(H.j0_s, s, z); st3(H.a0_d, s, z);
        st3(H.j0_d, s, z); st3(H.xp, s, z); st3(H.vp, s, z); st3(H.a2_s, s, z); st3(H.a3_s, s, z);
        st3(H.a2_d, s, z); st3(H.a3_d, s, z);
        H.phi_d[s] = A.S.phi_d[i]; H.phi_s[s] = A.S.phi_s[i];
        H.mass[s] = A.S.mass[i]; H.r_planet[s] = A.S.r_planet[i]; H.f[s] = A.S.f[i];
        H.r_out_inv[s] = A.S.r_out_inv[i];
        H.time_c[s] = A.S.time[i]; H.th[s] = 0.; H.dt[s] = A.S.dt[i]; H.acc0[s] = A.S.acc0[i];
        H.id[s] = A.S.id[i];
        H.dead[s] = 0; H.merged[s] = 0;
        H.tw_head[s] = H.tw_tail[s] = H.tw_next[s] = -1;
    }
    // FP32 prefilter: coordinates relative to the first member.  Their
    // distance errors stay below 3.2e-7 (D + motion) with D the cluster's
    // extent; the prefilter only skips pairs beyond twice a cutoff radius, so
    // it is exact whenever that error bound is below a quarter of the
    // smallest radius it is compared with (1e-6 (D + 0.05 AU) below).
    {
        const V3 r0 = ld3(A.S.pos, A.members[o]);
        pre.ref[0] = r0.x; pre.ref[1] = r0.y; pre.ref[2] = r0.z;
        double ext = 0., rmin = 1.e300;
        for (int k = rank; k < n; k += TEAM) {
            const int s = o + k;
            const V3 d = ld3(H.pos, s) - r0;
            ext = dmax(ext, dmax(fabs(d.x), dmax(fabs(d.y), fabs(d.z))));
            rmin = dmin(rmin, dmin(2. * H.f[s] * H.r_planet[s], 1. / H.r_out_inv[s]));
            st32(H.pos32, s, ld3(H.pos, s), pre);
            H.roi32[s] = (float)H.r_out_inv[s];
            H.fr32[s] = (float)(H.f[s] * H.r_planet[s]);
        }
        ext = -tm.min(-ext);
        rmin = tm.min(rmin);
        pre.on = (ext + 0.05) * 1e-6 < 0.25 * rmin;
    }
    tm.sync();
    for (int k = rank; k < n; k += TEAM) hard_force(P, H, o, n, o + k, 0, pre);
    tm.sync();
}

template <int TEAM>
__device__ void cluster_loop(const HardArgs &A, int c, const Team<TEAM> &tm, const Pre &pre, ClusterRun &run,
                             bool one_step = false) {
    const Params &P = A.P;
    const Hard &H = A.H;
    const int rank = tm.rank;
    const int o = A.off[c], n = A.cnt[c];
    int n_col = run.n_col;
    double ed = run.ed, edd = run.edd;
    double time = run.time;
    int steps = run.steps;
    long long work = run.work;
    while (time < A.t_end) {
        if (++steps > A.max_steps) {
            if (rank == 0) atomicOr(A.status, ST_ITER_CAP);
            break;
        }
        // makeActiveList, src/hermite.h:4-24
        double ts = 1.e10;
        for (int k = rank; k < n; k += TEAM) {
            const int s = o + k;
            if (!H.dead[s]) ts = dmin(ts, H.th[s] + H.dt[s]);
        }
        ts = tm.min(ts);
        for (int k = rank; k < n; k += TEAM) {
            const int s = o + k;
            st3(H.xp, s, v3(0., 0., 0.));
            st3(H.vp, s, v3(0., 0., 0.));
            predict(H, s, ts - H.th[s]);
            st32(H.xp32, s, ld3(H.xp, s), pre);
        }
        tm.sync();
        // collisionDetermination, src/hermite.h:98-196: the first ordered pair
        // (i, j) with the smallest R < 1.  Pairs with |dr|^2 above the squared
        // radius sum (1e-6 margin) have R > 1 and are skipped after the
        // distance test.
        double Rb = 1.;
        long long pb = 0x7fffffffffffffffLL;
        for (int a = rank; a < n; a += TEAM) {
            const int si = o + a;
            if (H.dead[si]) continue;
            const V3 xi = ld3(H.xp, si);
            const double ri = H.f[si] * H.r_planet[si];
            const float ri32 = H.fr32[si];
            for (int b = 0; b < n; b++) {
                const int sj = o + b;
                if (a == b || H.dead[sj]) continue;
                if (pre.on) {
                    const float rs = ri32 + H.fr32[sj];
                    if (d2_32(H.xp32, si, H.xp32, sj) > 4.0f * rs * rs) continue;
                }
                const V3 dr = xi - ld3(H.xp, sj);
                const double d2 = dot(dr, dr);
                const double r2 = ri + H.f[sj] * H.r_planet[sj];
                if (d2 > r2 * r2 * 1.000001) continue;
                const double r1 = sqrt(d2);
                const double R = r1 / r2;
                const long long p = (long long)a * n + b;
                if (R < Rb || (R == Rb && R < 1. && p < pb)) { Rb = R; pb = p; }
            }
        }
        tm.argmin(Rb, pb);
        const bool col = Rb < 1.;
        int imp = -1, tar = -1;
        if (col) {
            const int a = (int)(pb / n), b = (int)(pb % n);
            if (H.mass[o + a] < H.mass[o + b]) { imp = o + a; tar = o + b; }
            else { imp = o + b; tar = o + a; }
            for (int k = rank; k < n; k += TEAM) H.dt[o + k] = ts - H.th[o + k];
        }
        tm.sync();
        // correct the active set (all alive on a collision)
        for (int k = rank; k < n; k += TEAM) {
            const int s = o + k;
            if (H.dead[s]) continue;
            if (!col && H.th[s] + H.dt[s] != ts) continue;
            work += n;
            hard_force(P, H, o, n, s, 1, pre);
            if (H.merged[s]) {
                for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++)
                    hard_force(P, H, o, n, t, 1, pre);
                merge_acc_jerk(H, s);
            }
            const double tc = ts - H.th[s];
            for (int it = 0; it < 2; it++) {
                correct(H, s, tc);
                st32(H.pos32, s, ld3(H.pos, s), pre);
                if (H.merged[s])
                    for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++) {
                        correct(H, t, tc);
                        st32(H.pos32, t, ld3(H.pos, t), pre);
                    }
                hard_force(P, H, o, n, s, 2, pre);
                if (H.merged[s]) {
                    for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++)
                        hard_force(P, H, o, n, t, 2, pre);
                    merge_acc_jerk(H, s);
                }
            }
            H.th[s] += tc;
            if (H.merged[s])
                for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++) H.th[t] += tc;
            if (!col) {
                dt_hermite(P, H, s);
                if (H.merged[s])
                    for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++) H.dt[t] = H.dt[s];
            }
        }
        tm.sync();
        if (col) {
            if (rank == 0) {
                ColRec rec;
                double e1 = 0., e2 = 0.;
                FragCtx X{&A, nullptr, 0, c, 0, nullptr, nullptr};
                collide(P, H, imp, tar, e1, e2, rec, A.frag.a_frag > 0. ? &X : nullptr);
                ed += e1;
                edd += e2;
                rec.cluster = c;
                rec.seq = n_col;
                rec.n = n;
                const int slot = atomicAdd(A.n_cols, 1);
                if (slot < A.col_cap) A.cols[slot] = rec;
                else atomicOr(A.status, ST_QUEUE_OVERFLOW);
            }
            n_col++;
            tm.sync();
            for (int k = rank; k < n; k += TEAM) {
                st32(H.pos32, o + k, ld3(H.pos, o + k), pre);
                H.fr32[o + k] = (float)(H.f[o + k] * H.r_planet[o + k]);
            }
            tm.sync();
            for (int k = rank; k < n; k += TEAM) hard_force(P, H, o, n, o + k, 0, pre);
            tm.sync();
            for (int k = rank; k < n; k += TEAM)
                if (H.merged[o + k] && H.tw_head[o + k] >= 0) merge_acc_jerk(H, o + k);
            tm.sync();
            for (int k = rank; k < n; k += TEAM) {
                const int s = o + k;
                if (!H.dead[s])
                    H.dt[s] = dt_initial(P, H.th[s], H.dt[s], H.acc0[s], ld3(H.acc_d, s), ld3(H.jerk_d, s),
                                         ld3(H.acc_s, s), ld3(H.jerk_s, s));
            }
            tm.sync();
            for (int k = rank; k < n; k += TEAM) {
                const int s = o + k;
                if (H.merged[s])
                    for (int t = H.tw_head[s], g = 0; t >= 0 && g < 4096; t = H.tw_next[t], g++) H.dt[t] = H.dt[s];
            }
            tm.sync();
        }
        // getSystemTime, src/hermite.h:25-35
        double tmin = 1.e10;
        for (int k = rank; k < n; k += TEAM)
            if (!H.dead[o + k]) tmin = dmin(tmin, H.th[o + k]);
        time = tm.min(tmin);
        if (one_step) break;
    }
    run.n_col = n_col;
    run.ed = ed;
    run.edd = edd;
    run.time = time;
    run.steps = steps;
    run.work = work;
}

template <int TEAM>
__device__ void cluster_finish(const HardArgs &A, int c, const Team<TEAM> &tm, const Pre &pre, const ClusterRun &run) {
    const Params &P = A.P;
    const Hard &H = A.H;
    const int rank = tm.rank;
    const int o = A.off[c], n = A.cnt[c];
    const int n_col = run.n_col;
    tm.sync();
    for (int k = rank; k < n; k += TEAM) hard_force(P, H, o, n, o + k, 0, pre);
    tm.sync();
    if (n_col > 0)
        for (int k = rank; k < n; k += TEAM)
            if (H.merged[o + k] && H.tw_head[o + k] >= 0) merge_acc_jerk(H, o + k);
    tm.sync();
    // write back to FPGrav, with resetTime (src/hard.h:768-787)
    for (int k = rank; k < n; k += TEAM) {
        const int s = o + k, i = A.members[s];
        st3(A.S.pos, i, ld3(H.pos, s)); st3(A.S.vel, i, ld3(H.vel, s));
        st3(A.S.acc_s, i, ld3(H.acc_s, s)); st3(A.S.jerk_s, i, ld3(H.jerk_s, s));
        st3(A.S.acc_d, i, ld3(H.acc_d, s)); st3(A.S.jerk_d, i, ld3(H.jerk_d, s));
        A.S.phi_d[i] = H.phi_d[s]; A.S.phi_s[i] = H.phi_s[s];
        A.S.mass[i] = H.mass[s]; A.S.r_planet[i] = H.r_planet[s];
        A.S.time[i] = H.time_c[s] + H.th[s]; A.S.dt[i] = H.dt[s];
        A.S.id[i] = H.id[s];
        A.S.dead[i] = H.dead[s]; A.S.merged[i] = H.merged[s];
        A.S.n_cluster[i] = n;
    }
    // per-cluster cost log: block steps and active-body x member pair sweeps
    if (A.cost) atomicAdd((unsigned long long *)&A.cost[2 * c + 1], (unsigned long long)run.work);
    if (rank == 0) {
        A.cl_edisp[2 * c] = (n_col > 0) ? run.ed : 0.;
        A.cl_edisp[2 * c + 1] = (n_col > 0) ? run.edd : 0.;
        if (A.cost) A.cost[2 * c] = run.steps;
        if (A.times) {
            A.times[2 * c] = run.t_start;
            A.times[2 * c + 1] = global_ns();
        }
    }
    tm.sync();
}

template <int TEAM>
__device__ void run_cluster(const HardArgs &A, int c, const Team<TEAM> &tm) {
    ClusterRun run;
    run.t_start = (A.times && tm.rank == 0) ? global_ns() : 0;
    Pre pre;
    cluster_load(A, c, tm, pre);
    cluster_loop(A, c, tm, pre, run);
    cluster_finish(A, c, tm, pre, run);
}

// One persistent launch: clusters of >= cta_min members one per CTA, then
// clusters of >= warp_min members one per warp, then the rest one per thread.
// Each tier takes its clusters from its own queue in the order given
// (largest or costliest first).
__global__ void __launch_bounds__(128, 2) k_hard_clusters(HardArgs A) {
    __shared__ double red_d[4];
    __shared__ long long red_l[4];
    __shared__ int q_sh;
    const int tid = threadIdx.x, lane = tid & 31;
    // tier 1: CTA per cluster
    {
        Team<128> tm{tid, red_d, red_l};
        for (int guard = 0; guard < (1 << 30); guard++) {
            if (tid == 0) q_sh = atomicAdd(&A.queue[0], 1);
            __syncthreads();
            const int q = q_sh;
            __syncthreads();
            if (q >= A.n_tier[0]) break;
            run_cluster<128>(A, A.order[q], tm);
        }
    }
    // tier 2: warp per cluster
    {
        Team<32> tm{lane, nullptr, nullptr};
        for (int guard = 0; guard < (1 << 30); guard++) {
            int q = 0;
            if (lane == 0) q = atomicAdd(&A.queue[1], 1);
            q = __shfl_sync(0xffffffffu, q, 0);
            if (q >= A.n_tier[1]) break;
            run_cluster<32>(A, A.order[A.n_tier[0] + q], tm);
        }
    }
    // tier 3: thread per cluster, a warp takes 32 clusters at a time
    {
        Team<1> tm{0, nullptr, nullptr};
        for (int guard = 0; guard < (1 << 30); guard++) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&A.queue[2], 32);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= A.n_tier[2]) break;
            const int q = base + lane;
            if (q < A.n_tier[2]) run_cluster<1>(A, A.order[A.n_tier[0] + A.n_tier[1] + q], tm);
            __syncwarp();
        }
    }
}

}  // namespace p3t

#include "hard_lone.cuh"
#include "hard_bundle.cuh"

namespace p3t {

// ---- isolated bodies ----------------------------------------------------------
__device__ __forceinline__ double kepler_eq(double u, double e) { return u - e * sin(u); }
__device__ double solve_kepler(double l, double e) {  // src/kepler.h:5-38
    const double e2 = e * e, e3 = e2 * e, e4 = e2 * e2, e5 = e3 * e2, e6 = e3 * e3;
    double u = l + (e - e3 / 8. + e5 / 192.) * sin(l) + (e2 / 2. - e4 / 6. + e6 / 48.) * sin(2. * l) +
               (3. * e3 / 8. - 27. * e5 / 128.) * sin(3. * l) + (e4 / 3. - 4. * e6 / 15.) * sin(4. * l) +
               125. * e5 / 384. * sin(5. * l) + 27. * e6 / 80. * sin(6. * l);
    if (fabs(kepler_eq(u, e) - l) > 1.e-15) {
        double u0;
        int loop = 0;
        do {
            u0 = u;
            const double s = sin(u0), co = cos(u0);
            u = u0 - ((u0 - e * s - l) / (1. - e * co));
            loop++;
        } while (fabs(u - u0) > 1.e-15 && loop < 10);
    }
    return u;
}

struct IsoArgs {
    State S;
    Params P;
    double t0, t1;
    int *status;
    const int32_t *list, *count;  // the isolated bodies and how many
};

// the bodies outside every cluster (no neighbour), ascending: the drift's
// threads take one each, every lane busy (a launch over all bodies left
// nine lanes in ten idle on a disk whose bodies are mostly in clusters)
__global__ void k_iso_flag(const int32_t *number, int n, int32_t *flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = number[i] == 0;
}
__global__ void k_iso_list(const int32_t *flag, const int32_t *pos, int n, int32_t *list, int32_t *count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (flag[i]) list[pos[i]] = i;
    if (i == n - 1) *count = pos[i] + flag[i];
}

__device__ void isolated_body(const IsoArgs &A, int i);
// grid-stride over the list: the grid is sized from the host's count of
// bodies outside the clusters, the device's count is the one obeyed
__global__ void k_isolated(IsoArgs A) {
    const int n_iso = *A.count;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_iso; t += gridDim.x * blockDim.x)
        isolated_body(A, A.list[t]);
}
__device__ void isolated_body(const IsoArgs &A, int i) {
    const State &S = A.S;
    const Params &P = A.P;
    V3 pos = ld3(S.pos, i), vel = ld3(S.vel, i);
    // getEccentricity, src/particle.h:668-681
    double ecc;
    {
        const double r = sqrt(dot(pos, pos));
        const double rv = dot(pos, vel);
        const double ax = 1.0 / (2.0 / r - dot(vel, vel) / P.m_sun);
        const double ecccosu = 1. - r / ax;
        const double eccsinu2 = rv * rv / (P.m_sun * ax);
        ecc = sqrt(ecccosu * ecccosu + eccsinu2);
    }
    V3 as, js;
    double phs;
    if (ecc < 0.8 && P.eps2_sun == 0.) {
        // timeIntegrateKepler_isolated, src/hermite.h:787-815
        const double mu = P.m_sun;
        const double r2 = dot(pos, pos), r = sqrt(r2), rinv = 1. / r;
        const double v2 = dot(vel, vel), rv = dot(pos, vel);
        const double ax = 1.0 / (2.0 * rinv - v2 / mu);
        const double ecccosu = 1. - r / ax;
        const double eccsinu = rv / sqrt(mu * ax);
        const double e = sqrt(ecccosu * ecccosu + eccsinu * eccsinu);
        const double nm = sqrt(mu / (ax * ax * ax));
        double u, cosu, sinu;
        if (e != 0) { u = atan2(eccsinu, ecccosu); cosu = ecccosu / e; sinu = eccsinu / e; }
        else { u = 0.; cosu = 1.; sinu = 0.; }
        const double aninv = sqrt(ax / mu);
        const double ecc_sq = sqrt(1. - e * e);
        const V3 PP = rinv * cosu * pos - aninv * sinu * vel;
        const V3 QQ = (rinv * sinu * pos + aninv * (cosu - e) * vel) / ecc_sq;
        double l = kepler_eq(u, e);
        l += nm * (A.t1 - A.t0);
        u = solve_kepler(l, e);
        const double cu = cos(u), su = sin(u);
        const double esq = sqrt(1. - e * e);
        pos = ax * ((cu - e) * PP + esq * su * QQ);
        const double ri = sqrt(1. / dot(pos, pos));
        vel = ax * ax * nm * ri * (-su * PP + esq * cu * QQ);
        st3(S.pos, i, pos);
        st3(S.vel, i, vel);
        S.time[i] += (A.t1 - A.t0);
        S.phi_d[i] = 0.;
        st3(S.acc_d, i, v3(0., 0., 0.));
        st3(S.jerk_d, i, v3(0., 0., 0.));
        sun_force(P, pos, vel, as, js, &phs);
        st3(S.acc_s, i, as);
        st3(S.jerk_s, i, js);
        S.phi_s[i] = phs;
        S.dt[i] = dt_initial(P, S.time[i], S.dt[i], S.acc0[i], v3(0., 0., 0.), v3(0., 0., 0.), as, js);
    } else {
        // timeIntegrate_isolated, src/hermite.h:734-785, on a one-member Hard
        // view of this body's state arrays
        const double time_c = S.time[i];
        double th = 0., dt = S.dt[i];
        const double acc0 = S.acc0[i];
        V3 ad = v3(0., 0., 0.), jd = v3(0., 0., 0.);
        V3 a0s, j0s, a0d, j0d, xp, vp, a2s, a3s, a2d, a3d;
        sun_force(P, pos, vel, as, js, &phs);
        ad = ld3(S.acc_d, i);
        jd = ld3(S.jerk_d, i);
        int steps = 0;
        while (th < A.t1 - A.t0) {
            if (++steps > MAX_BLOCK_STEPS) { atomicOr(A.status, ST_ITER_CAP); break; }
            // predict
            a0s = as; j0s = js; j0d = jd; a0d = ad;
            {
                const V3 a = as + ad, j = js + jd;
                xp = pos + dt * (vel + dt * (0.5 * a + 1.6666666666666667e-1 * dt * j));
                vp = vel + dt * (a + dt * 0.5 * j);
            }
            ad = v3(0., 0., 0.);
            jd = v3(0., 0., 0.);
            sun_force(P, xp, vp, as, js, nullptr);
            for (int it = 0; it < 2; it++) {
                const double Dt = dt, Dt2 = Dt * Dt, Di = recip_pow2_or_div(Dt), Di2 = Di * Di, Di3 = Di2 * Di;
                const V3 Am_s = as - a0s, J0_s = Dt * j0s, J1_s = Dt * js;
                const V3 A2_s = 3. * Am_s - (J1_s + 2. * J0_s);
                const V3 A3_s = -2. * Am_s + (J1_s + J0_s);
                a2s = 2. * Di2 * (A2_s + 3. * A3_s);
                a3s = 6. * Di3 * A3_s;
                const V3 Am_d = ad - a0d, J0_d = j0d * Dt, J1_d = jd * Dt;
                const V3 A2_d = 3. * Am_d - (J1_d + 2. * J0_d);
                const V3 A3_d = -2. * Am_d + (J1_d + J0_d);
                a2d = 2. * (A2_d + 3. * A3_d) * Di2;
                a3d = 6. * A3_d * Di3;
                const V3 A2 = A2_s + A2_d, A3 = A3_s + A3_d;
                pos = xp + 1.6666666666666667e-2 * Dt2 * (5. * A2 + 3. * 1.1666666666666667e-3 * A3);
                vel = vp + 8.3333333333333333e-2 * Dt * (4. * A2 + 3. * A3);
                sun_force(P, pos, vel, as, js, nullptr);
            }
            th += dt;
            // calcDeltat
            double dt_next = dmin(2. * dt, 0.5 * P.dt_tree);
            const double dt_1 = dmin(dt4th(P.eta, P.alpha2, acc0, ad, jd, a2d, a3d),
                                     dt4th(P.eta_sun, P.alpha2, 0., as, js, a2s, a3s));
            double rem = rem_pow2(th, dt_next);
            for (int k = 0; rem != 0.0 && k < 1100; k++) { dt_next *= 0.5; rem = rem_pow2(th, dt_next); }
            for (int k = 0; dt_1 < dt_next && 0.5 * dt < dt_next && k < 1100; k++) dt_next *= 0.5;
            if (dt_next < 2. * P.dt_min) dt_next = P.dt_min;
            dt = dt_next;
        }
        sun_force(P, pos, vel, as, js, &phs);
        st3(S.pos, i, pos);
        st3(S.vel, i, vel);
        st3(S.acc_s, i, as);
        st3(S.jerk_s, i, js);
        st3(S.acc_d, i, ad);
        st3(S.jerk_d, i, jd);
        S.phi_s[i] = phs;
        S.phi_d[i] = 0.;
        S.time[i] = time_c + th;
        S.dt[i] = dt;
    }
    S.n_cluster[i] = 1;
}


// ---- work-queue order ------------------------------------------------------------
// A counting sort of the clusters by (tier, priority bucket): bins ascend with
// the tier and descend with the priority.  The order within a bin is
// arbitrary; no result depends on the order, only the makespan does.
constexpr int ORDER_NB = 4096;

__global__ void k_order_bins(const int32_t *cnt, const float *prio, int nc, int mode, int main_cap, int warp_min, int cta_min,
                             float pmin, float pscale, int heavy_key, int lone_key, int lone_nmax, int32_t *bin,
                             int32_t *hist, int32_t *n_heavy) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nc) return;
    const int n = cnt[k];
    int key = n < ORDER_NB - 1 ? n : ORDER_NB - 1;
    if (prio) {
        const float v = (prio[k] - pmin) * pscale;
        key = (v >= 0.f) ? (v < (float)(ORDER_NB - 1) ? (int)v : ORDER_NB - 1) : 0;  // NaN -> 0
    }
    // bundle form: tier 0 above the bundle's slots, tier 2 the lone form
    // (predicted longest chains of at most lone_nmax members), tier 1 the rest
    const int tier = (mode == 0) ? (n > main_cap ? 0 : ((key >= lone_key && n <= lone_nmax) ? 2 : 1))
                                 : (n >= cta_min ? 0 : (n >= warp_min ? 1 : 2));
    const int b = tier * ORDER_NB + (ORDER_NB - 1 - key);
    bin[k] = b;
    atomicAdd(&hist[b], 1);
    // bundle form: the other clusters predicted to take long chains of block
    // steps run alone in a bundle CTA first (they head tier 1, the order
    // being by prediction)
    if (mode == 0 && tier == 1 && key >= heavy_key) atomicAdd(n_heavy, 1);
}

// exclusive offsets of the 3 x ORDER_NB bins (one block of 1024) and the
// clusters per tier
__global__ void k_order_scan(int32_t *hist, int32_t *n_tier) {
    constexpr int NBIN = 3 * ORDER_NB, PER = NBIN / 1024;
    __shared__ int ws[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int loc[PER], sum = 0;
#pragma unroll
    for (int j = 0; j < PER; j++) {
        loc[j] = hist[tid * PER + j];
        sum += loc[j];
    }
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    if (w == 0) {
        int v = ws[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        ws[lane] = v;  // inclusive
    }
    __syncthreads();
    int off = x - sum + (w > 0 ? ws[w - 1] : 0);
    const int total = ws[31];
#pragma unroll
    for (int j = 0; j < PER; j++) {
        hist[tid * PER + j] = off;
        off += loc[j];
    }
    __syncthreads();
    if (tid == 0) {
        n_tier[0] = hist[ORDER_NB];
        n_tier[1] = hist[2 * ORDER_NB] - hist[ORDER_NB];
        n_tier[2] = total - hist[2 * ORDER_NB];
    }
}

__global__ void k_order_scatter(const int32_t *bin, int nc, int32_t *offs, int32_t *order) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nc) return;
    order[atomicAdd(&offs[bin[k]], 1)] = k;
}

// ---- host side ------------------------------------------------------------------
struct HardBufs {
    DevBuf<double> d;
    DevBuf<int64_t> id;
    DevBuf<int32_t> i32, order, queue, n_cols;
    DevBuf<double> cl_edisp;
    DevBuf<ColRec> cols;
    DevBuf<long long> cost, times;
    DevBuf<float> f32, prio;
    DevBuf<int32_t> bin, hist, ntier;
    DevBuf<FragRec> frags;
    DevBuf<int32_t> n_frags, fgslot, fidx;
    DevBuf<long long> fmap;
    DevBuf<unsigned long long> live;  // [2] pair terms evaluated by the last launch
    DevBuf<unsigned long long> phase;  // [HP_N] clock cycles per bundle phase (when profiled)
    DevBuf<int32_t> iso;               // isolated bodies: flags, positions, list, count
    Hard H;
    int cap = 0;
    int reserve(int m) {
        if (m <= cap && d.p) return 0;
        const int mm = std::max(m, 1);
        int r = 0;
        const int nvec = 18, nsc = 10;
        if ((r = d.reserve((size_t)mm * (3 * nvec + nsc))) || (r = id.reserve(mm)) || (r = i32.reserve((size_t)mm * 5)) ||
            (r = f32.reserve((size_t)mm * 8)))
            return r;
        H.pos32 = f32.p;
        H.xp32 = f32.p + 3 * (size_t)mm;
        H.roi32 = f32.p + 6 * (size_t)mm;
        H.fr32 = f32.p + 7 * (size_t)mm;
        double *p = d.p;
        double **vecs[nvec] = {&H.pos, &H.vel, &H.acc_s, &H.jerk_s, &H.acc_d, &H.jerk_d, &H.x0, &H.v0, &H.a0_s,
                               &H.j0_s, &H.a0_d, &H.j0_d, &H.xp, &H.vp, &H.a2_s, &H.a3_s, &H.a2_d, &H.a3_d};
        for (int k = 0; k < nvec; k++) { *vecs[k] = p; p += 3 * (size_t)mm; }
        double **scs[nsc] = {&H.phi_d, &H.phi_s, &H.mass, &H.r_planet, &H.f, &H.r_out_inv, &H.th, &H.dt, &H.acc0,
                             &H.time_c};
        for (int k = 0; k < nsc; k++) { *scs[k] = p; p += mm; }
        H.id = id.p;
        int32_t *q = i32.p;
        H.dead = q; q += mm;
        H.merged = q; q += mm;
        H.tw_head = q; q += mm;
        H.tw_tail = q; q += mm;
        H.tw_next = q;
        cap = mm;
        return 0;
    }
};
static HardBufs g_hb;
static std::vector<ColRec> g_cols;
static double g_edisp[2] = {0., 0.};
static int g_warp_min = 8, g_cta_min = 64;
static int g_hard_mode = 0;  // 0: bundles, 1: thread/warp/CTA tiers
static float g_heavy = 6.75f;  // predicted log2(1 + block steps) from which a cluster runs alone (0: never)
static int g_wide = 1;        // clusters above the bundle capacity: wide lone bundles (1) or one per CTA (0)
static int g_bcap = 256, g_bocc = 2;  // bundle member slots and CTAs per SM (256/2, 128/3, 128/4)
static FragParams g_frag = {0., 9.426627927538057e-12, 10, 0, 0ULL};  // off (a_frag = 0)
static int g_frag_cap = 0;  // fragment slots of the current launch
static int g_max_steps = MAX_BLOCK_STEPS;  // block-step cap per cluster and tree step
// lone form: clusters predicted to take at least 2^g_lone - 1 block steps (0:
// off), on g_lone_ctas CTAs of their own (0: in the bundle CTAs)
static int g_hard_profile = 0;  // per-phase clock counts of the bundle loop
static float g_lone = 0.f;
static int g_lone_ctas = 0;
// events around the last cluster launch (k_hard_bundles / k_hard_clusters) on
// the library stream, and whether they hold a launch
static cudaEvent_t g_ev_launch[2] = {nullptr, nullptr};
static bool g_launch_timed = false;
static int g_last_nc = 0;  // clusters of the last launch (its cost log and sizes stay valid until the next)

// Sums over the last launch's clusters: {sum of active x member pair sweeps,
// sum of n (n - 1) x block steps, sum of sweeps / n (active members over block
// steps), largest block-step count, sum of n x block steps (predictions)};
// one block.
__global__ void k_cost_sums(const long long *__restrict__ cost, const int32_t *__restrict__ cnt, int nc,
                            double *out) {
    __shared__ double s0[512], s1[512], s2[512], s3[512], s4[512];
    double a = 0., b = 0., d = 0., m = 0., e = 0.;
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const double st = (double)cost[2 * c], w = (double)cost[2 * c + 1], n = (double)max(cnt[c], 1);
        a += w;
        b += n * (n - 1.) * st;
        d += w / n;
        m = fmax(m, st);
        e += n * st;
    }
    s0[threadIdx.x] = a; s1[threadIdx.x] = b; s2[threadIdx.x] = d; s3[threadIdx.x] = m; s4[threadIdx.x] = e;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s0[threadIdx.x] += s0[threadIdx.x + o];
            s1[threadIdx.x] += s1[threadIdx.x + o];
            s2[threadIdx.x] += s2[threadIdx.x + o];
            s3[threadIdx.x] = fmax(s3[threadIdx.x], s3[threadIdx.x + o]);
            s4[threadIdx.x] += s4[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s0[0]; out[1] = s1[0]; out[2] = s2[0]; out[3] = s3[0]; out[4] = s4[0];
    }
}

// Fragments made by a launch join the particle system (addFragment2ParticleSystem,
// src/hard.h:858-943): the r-th new body is the fragment in hard slot
// gslot[r] (record fidx[r]); temporary (negative) ids map through
// old[k] -> new[k].
__device__ __forceinline__ long long frag_new_id(long long id, const long long *map, int nmap) {
    if (id >= 0) return id;
    for (int k = 0; k < nmap; k++)
        if (map[2 * k] == id) return map[2 * k + 1];
    return id;
}
__global__ void k_frag_append(State S, Hard H, const FragRec *fr, const int32_t *gslot, const int32_t *fidx, int nf,
                              int n0, const long long *map, int nmap, int32_t *frag_cl) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nf) return;
    const int g = gslot[r], i = n0 + r;
    const FragRec &R = fr[fidx[r]];
    st3(S.pos, i, ld3(H.pos, g));
    st3(S.vel, i, ld3(H.vel, g));
    st3(S.acc, i, v3(0., 0., 0.));
    st3(S.acc_d, i, ld3(H.acc_d, g));
    st3(S.jerk_d, i, ld3(H.jerk_d, g));
    st3(S.acc_s, i, ld3(H.acc_s, g));
    st3(S.jerk_s, i, ld3(H.jerk_s, g));
    S.phi[i] = R.phi;
    S.phi_d[i] = H.phi_d[g];
    S.phi_s[i] = H.phi_s[g];
    S.mass[i] = H.mass[g];
    S.r_planet[i] = H.r_planet[g];
    S.f[i] = H.f[g];
    S.r_out[i] = R.r_out;
    S.r_out_inv[i] = H.r_out_inv[g];
    S.r_search[i] = R.r_search;
    S.v_disp[i] = R.v_disp;
    S.time[i] = H.time_c[g] + H.th[g];  // resetTime
    S.dt[i] = H.dt[g];
    S.acc0[i] = H.acc0[g];
    S.number[i] = R.number;
    S.rank[i] = 0;
    S.id_max[i] = -1;
    S.id_min[i] = 2147483647;
    S.n_cluster[i] = R.n_cl;
    S.nbr_n[i] = 0;
    S.dead[i] = H.dead[g];
    S.merged[i] = H.merged[g];
    S.id[i] = frag_new_id(H.id[g], map, nmap);
    S.id_cluster[i] = R.id_cluster;
    frag_cl[r] = R.cluster;
}
// dead members that merged into a fragment carry its temporary id
__global__ void k_frag_ids(State S, int n, const long long *map, int nmap) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && S.id[i] < 0) S.id[i] = frag_new_id(S.id[i], map, nmap);
}
static std::vector<float> g_prio;

}  // namespace p3t

using namespace p3t;

extern "C" {

int p3t_set_hard_tiers(int warp_min, int cta_min) {
    if (warp_min < 1 || cta_min < warp_min) return ST_BAD_INDEX;
    g_warp_min = warp_min;
    g_cta_min = cta_min;
    return 0;
}

int p3t_set_fragmentation(double a_frag, int n_frag, double m_min, unsigned long long seed) {
    if (a_frag < 0. || n_frag < 0 || n_frag > 32 || !(m_min > 0.)) return ST_BAD_INDEX;
    g_frag.a_frag = a_frag;
    g_frag.n_frag_max = n_frag;
    g_frag.m_min = m_min;
    g_frag.seed = seed;
    return 0;
}

long long p3t_id_next(void) { return g_eng.id_next; }

int p3t_set_hard_heavy(float log2_steps) {
    if (!(log2_steps >= 0.f)) return ST_BAD_INDEX;
    g_heavy = log2_steps;
    return 0;
}

int p3t_set_hard_bundle(int member_slots, int ctas_per_sm) {
    const bool ok = (member_slots == 256 && ctas_per_sm == 2) || (member_slots == 128 && (ctas_per_sm == 3 || ctas_per_sm == 4));
    if (!ok) return ST_BAD_INDEX;
    g_bcap = member_slots;
    g_bocc = ctas_per_sm;
    return 0;
}

int p3t_set_hard_wide(int on) {
    if (on != 0 && on != 1) return ST_BAD_INDEX;
    g_wide = on;
    return 0;
}

int p3t_set_hard_mode(int mode) {
    if (mode != 0 && mode != 1) return ST_BAD_INDEX;
    g_hard_mode = mode;
    return 0;
}

int p3t_set_cluster_priority(const float *prio, int n) {
    if (n != g_eng.n_clusters || n < 0) return ST_BAD_INDEX;
    g_prio.assign(prio, prio + n);
    return 0;
}

int p3t_hard_costs(long long *out, int n) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    if (n != g_eng.n_clusters || !g_hb.cost.p) return ST_BAD_INDEX;
    return d2h(c, out, g_hb.cost.p, 2 * (size_t)n * sizeof(long long));
}

int p3t_hard_times(long long *out, int n) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    if (n != g_eng.n_clusters || !g_hb.times.p) return ST_BAD_INDEX;
    return d2h(c, out, g_hb.times.p, 2 * (size_t)n * sizeof(long long));
}

// Stage 1 of the hard part: buffers and the work-queue order (device only,
// queued on the library stream).
static int g_enqueued = -1;  // cluster count of the enqueued lists

int p3t_hard_enqueue(void) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    Context *c = E.c;
    HardBufs &B = g_hb;
    const int nc = E.n_clusters;
    int r = 0;
    if (g_frag.a_frag > 0. && g_hard_mode != 0) return ST_BAD_INDEX;  // fragments need the bundle form
    g_frag_cap = (g_frag.a_frag > 0.) ? std::max(1024, g_frag.n_frag_max * 4096) : 0;
    if ((r = B.reserve(E.n_members + g_frag_cap)) || (r = B.order.reserve(nc)) || (r = B.queue.reserve(4)) ||
        (r = B.n_cols.reserve(1)) || (r = B.cl_edisp.reserve(2 * (size_t)nc + 2)) ||
        (r = B.cols.reserve(4096)) || (r = B.frags.reserve(g_frag_cap + 1)) || (r = B.n_frags.reserve(1)) ||
        (r = B.live.reserve(2)))
        return r;
    cudaMemsetAsync(B.n_frags.p, 0, sizeof(int32_t), c->stream);
    cudaMemsetAsync(B.live.p, 0, 2 * sizeof(unsigned long long), c->stream);
    if (g_hard_profile) {
        if ((r = B.phase.reserve(HP_N))) return r;
        cudaMemsetAsync(B.phase.p, 0, HP_N * sizeof(unsigned long long), c->stream);
    }
    // schedule, on the device: clusters binned by tier (bundle mode: above
    // the bundle capacity first; tier mode: CTA >= g_cta_min > warp >=
    // g_warp_min > thread), then by priority (the caller's, the learned cost
    // model's, else the size), highest first
    if ((r = B.bin.reserve(nc + 1)) || (r = B.hist.reserve(3 * ORDER_NB)) || (r = B.ntier.reserve(4))) return r;
    cudaMemsetAsync(B.hist.p, 0, 3 * ORDER_NB * sizeof(int32_t), c->stream);
    cudaMemsetAsync(B.ntier.p, 0, 4 * sizeof(int32_t), c->stream);
    if (nc > 0) {
        const float *prio = nullptr;
        float pmin = 0.f, pscale = 1.f;
        if ((int)g_prio.size() == nc) {
            if ((r = B.prio.reserve(nc)) || (r = h2d(c, B.prio.p, g_prio.data(), nc * sizeof(float)))) return r;
            const auto mm = std::minmax_element(g_prio.begin(), g_prio.end());
            pmin = *mm.first;
            pscale = (*mm.second > *mm.first) ? (ORDER_NB - 1) / (*mm.second - *mm.first) : 0.f;
            prio = B.prio.p;
        } else {
            prio = sched_priority(c, nc, &pmin, &pscale);
        }
        // heavy clusters: learned prediction of log2(1 + block steps) >= g_heavy;
        // lone ones: >= g_lone (the lone form is perfect accretion only)
        int heavy_key = 2147483647, lone_key = 2147483647;
        if (prio && (int)g_prio.size() != nc && g_heavy > 0.f)
            heavy_key = std::min(ORDER_NB - 1, (int)((g_heavy - pmin) * pscale));
        if (prio && (int)g_prio.size() != nc && g_lone > 0.f && g_frag.a_frag <= 0. && g_hard_mode == 0)
            lone_key = std::max(0, std::min(ORDER_NB - 1, (int)((g_lone - pmin) * pscale)));
        { P3T_COUNT_LAUNCH(); k_order_bins<<<(nc + 255) / 256, 256, 0, c->stream>>>(E.cl_cnt.p, prio, nc, g_hard_mode, g_bcap, g_warp_min, g_cta_min,
                                                              pmin, pscale, heavy_key, lone_key, LCAP, B.bin.p,
                                                              B.hist.p, B.ntier.p + 3); }
        { P3T_COUNT_LAUNCH(); k_order_scan<<<1, 1024, 0, c->stream>>>(B.hist.p, B.ntier.p); }
        { P3T_COUNT_LAUNCH(); k_order_scatter<<<(nc + 255) / 256, 256, 0, c->stream>>>(B.bin.p, nc, B.hist.p, B.order.p); }
        if ((r = cuda_status(cudaGetLastError()))) return r;
    }
    g_prio.clear();
    if ((r = B.cost.reserve(2 * (size_t)nc + 2)) || (r = B.times.reserve(2 * (size_t)nc + 2))) return r;
    cudaMemsetAsync(B.cost.p, 0, (2 * (size_t)nc + 2) * sizeof(long long), c->stream);
    cudaMemsetAsync(B.queue.p, 0, 4 * sizeof(int32_t), c->stream);
    cudaMemsetAsync(B.n_cols.p, 0, sizeof(int32_t), c->stream);
    g_enqueued = nc;
    return cuda_status(cudaGetLastError());
}

// Stage 2: the persistent cluster launch and the isolated-body drift of tree
// step istep (queued, no host synchronisation).
int p3t_hard_integrate(int istep) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    Context *c = E.c;
    HardBufs &B = g_hb;
    const int nc = E.n_clusters;
    if (g_enqueued != nc) return ST_BAD_INDEX;
    g_enqueued = -1;
    g_launch_timed = false;
    g_last_nc = nc;
    int r = 0;
    const Params P = E.params();
    // The isolated bodies' drift (k_isolated) touches only bodies outside
    // every cluster, so it runs beside the cluster launch, queued after it on
    // a stream of the lowest priority: its blocks take the SMs the cluster
    // launch leaves in its tail, and the library stream waits for both.  Its
    // blocks reserve ISO_SMEM of shared memory they do not use, so none lands
    // beside a lone-form CTA (whose FP64 chain it would slow).
    static cudaStream_t s_iso = nullptr;
    static cudaEvent_t ev_iso_ready = nullptr, ev_iso_done = nullptr;
    constexpr int ISO_SMEM = 96 * 1024;
    if (!s_iso) {
        int lo = 0, hi = 0;
        if ((r = cuda_status(cudaDeviceGetStreamPriorityRange(&lo, &hi))) ||
            (r = cuda_status(cudaStreamCreateWithPriority(&s_iso, cudaStreamNonBlocking, lo))) ||
            (r = cuda_status(cudaEventCreateWithFlags(&ev_iso_ready, cudaEventDisableTiming))) ||
            (r = cuda_status(cudaEventCreateWithFlags(&ev_iso_done, cudaEventDisableTiming))) ||
            (r = cuda_status(cudaFuncSetAttribute(k_isolated, cudaFuncAttributeMaxDynamicSharedMemorySize, ISO_SMEM))))
            return r;
    }
    if (E.S.n > 0) {
        const int n = E.S.n;
        if ((r = g_hb.iso.reserve(3 * (size_t)n + 1))) return r;
        int32_t *flag = g_hb.iso.p, *pos = flag + n, *list = pos + n;
        { P3T_COUNT_LAUNCH(); k_iso_flag<<<(n + 255) / 256, 256, 0, c->stream>>>(E.S.number, n, flag); }
        if ((r = E.scan(flag, pos, n, nullptr))) return r;
        { P3T_COUNT_LAUNCH(); k_iso_list<<<(n + 255) / 256, 256, 0, c->stream>>>(flag, pos, n, list, list + n); }
        if ((r = cuda_status(cudaEventRecord(ev_iso_ready, c->stream)))) return r;
    }
    if (nc > 0) {
        HardArgs A{};
        A.S = E.S;
        A.P = P;
        A.H = B.H;
        A.off = E.cl_off.p;
        A.cnt = E.cl_cnt.p;
        A.members = E.members.p;
        A.order = B.order.p;
        A.n_clusters = nc;
        A.n_tier = B.ntier.p;
        A.queue = B.queue.p;
        A.cost = B.cost.p;
        A.times = B.times.p;
        A.cl_edisp = B.cl_edisp.p;
        A.cols = B.cols.p;
        A.n_cols = B.n_cols.p;
        A.col_cap = 4096;
        A.status = c->status;
        A.t_end = P.dt_tree;
        A.frag = g_frag;
        A.frag.istep = istep;
        A.frags = B.frags.p;
        A.n_frags = B.n_frags.p;
        A.frag_base = E.n_members;
        A.frag_cap = g_frag_cap;
        A.wide = g_wide;
        A.max_steps = g_max_steps;
        A.live = B.live.p;
        A.phase_cycles = g_hard_profile ? B.phase.p : nullptr;
        if (!g_ev_launch[0] && ((r = cuda_status(cudaEventCreate(&g_ev_launch[0]))) ||
                                (r = cuda_status(cudaEventCreate(&g_ev_launch[1])))))
            return r;
        g_launch_timed = false;
        int sms = 152;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        if (g_hard_mode == 0) {
            static bool attr = false;
            static cudaStream_t s_wide = nullptr, s_lone = nullptr;
            static cudaEvent_t ev_done = nullptr, ev_lone = nullptr;
            const int smem_w = (int)sizeof(BundleSmem<BCAP_WIDE>);
            static_assert(sizeof(BundleSmem<BCAP_WIDE>) <= 200 * 1024, "the wide bundle fits an SM");
            static_assert(sizeof(LoneSmem<bundle_threads(256)>) <= sizeof(BundleSmem<256>) &&
                              sizeof(LoneSmem<BT>) <= 200 * 1024 && sizeof(LoneSmem<LONE_T>) <= LONE_EXCL_SMEM,
                          "lone state fits the shared memory it borrows");
            // the lone tier in the bundle CTAs: k_hard_lone with no CTAs of its own
            const bool lone = g_lone > 0.f && g_frag.a_frag <= 0.;
            A.lone_in = (lone && g_lone_ctas == 0) ? 1 : 0;
            int smem = g_bcap == 128 ? (int)sizeof(BundleSmem<128>) : (int)sizeof(BundleSmem<256>);
            if (A.lone_in && g_bcap == 128) smem = std::max(smem, (int)sizeof(LoneSmem<BT>));
            if (!attr) {
                if ((r = cuda_status(cudaFuncSetAttribute(k_hard_bundles<256, 2>,
                                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)sizeof(BundleSmem<256>)))) ||
                    (r = cuda_status(cudaFuncSetAttribute(
                         k_hard_bundles<128, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)std::max(sizeof(BundleSmem<128>), sizeof(LoneSmem<BT>))))) ||
                    (r = cuda_status(cudaFuncSetAttribute(
                         k_hard_bundles<128, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)std::max(sizeof(BundleSmem<128>), sizeof(LoneSmem<BT>))))) ||
                    (r = cuda_status(cudaFuncSetAttribute(k_hard_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          smem_w))) ||
                    (r = cuda_status(cudaFuncSetAttribute(k_hard_lone, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          LONE_EXCL_SMEM))) ||
                    (r = cuda_status(cudaStreamCreateWithPriority(&s_lone, cudaStreamNonBlocking, -1000))) ||
                    (r = cuda_status(cudaEventCreateWithFlags(&ev_lone, cudaEventDisableTiming))) ||
                    (r = cuda_status(cudaStreamCreateWithPriority(&s_wide, cudaStreamNonBlocking, -1000))) ||
                    (r = cuda_status(cudaEventCreateWithFlags(&ev_done, cudaEventDisableTiming))))
                    return r;
                attr = true;
            }
            // the lone clusters (with CTAs of their own) and the clusters above
            // BCAP_MAIN bodies on streams of their own, started first so that
            // they hold SMs from the beginning (no launch when there are none)
            bool lone_k = lone && g_lone_ctas > 0;
            if ((r = cuda_status(cudaEventRecord(g_ev_launch[0], c->stream)))) return r;
            // The wide and lone CTAs must hold their SMs before the persistent
            // bundle CTAs fill every SM (with a cross-stream event the bundle
            // kernel was dispatched first): the queue is complete when the
            // library stream has drained; its tier sizes then give the wide
            // grid, and both kernels are submitted before the bundle kernel
            // with no dependency left to resolve.
            int wide_ctas = 0;
            if (A.wide || lone_k) {
                int nt[3] = {0, 0, 0};
                if ((r = d2h(c, nt, B.ntier.p, sizeof(nt)))) return r;  // synchronizes the stream
                wide_ctas = A.wide ? std::min(nt[0], std::max(1, sms / 16)) : 0;
                if (nt[2] == 0) lone_k = false;
            }
            if (lone_k) {
                { P3T_COUNT_LAUNCH(); k_hard_lone<<<g_lone_ctas, LONE_T, LONE_EXCL_SMEM, s_lone>>>(A); }
                if ((r = cuda_status(cudaGetLastError())) || (r = cuda_status(cudaEventRecord(ev_lone, s_lone))))
                    return r;
            }
            if (wide_ctas > 0) {
                { P3T_COUNT_LAUNCH(); k_hard_wide<<<wide_ctas, WT, smem_w, s_wide>>>(A); }
                if ((r = cuda_status(cudaGetLastError()))) return r;
            }
            // persistent: g_bocc CTAs per SM (fewer when there are few clusters)
            const int blocks = std::max(1, std::min(sms * g_bocc, (nc + 3) / 4));
            if (g_bcap == 256)
                { P3T_COUNT_LAUNCH(); k_hard_bundles<256, 2><<<blocks, bundle_threads(256), smem, c->stream>>>(A); }
            else if (g_bocc == 3)
                { P3T_COUNT_LAUNCH(); k_hard_bundles<128, 3><<<blocks, BT, smem, c->stream>>>(A); }
            else
                { P3T_COUNT_LAUNCH(); k_hard_bundles<128, 4><<<blocks, BT, smem, c->stream>>>(A); }
            if ((r = cuda_status(cudaGetLastError()))) return r;
            if (wide_ctas > 0 && ((r = cuda_status(cudaEventRecord(ev_done, s_wide))) ||
                                  (r = cuda_status(cudaStreamWaitEvent(c->stream, ev_done, 0)))))
                return r;
            if (lone_k && (r = cuda_status(cudaStreamWaitEvent(c->stream, ev_lone, 0)))) return r;
            // the launch's time spans all three forms
            if ((r = cuda_status(cudaEventRecord(g_ev_launch[1], c->stream)))) return r;
            g_launch_timed = true;
        } else {
            const int blocks = std::max(1, std::min(sms * 2, (nc + 3) / 4));
            if ((r = cuda_status(cudaEventRecord(g_ev_launch[0], c->stream)))) return r;
            { P3T_COUNT_LAUNCH(); k_hard_clusters<<<blocks, 128, 0, c->stream>>>(A); }
            if ((r = cuda_status(cudaEventRecord(g_ev_launch[1], c->stream)))) return r;
            g_launch_timed = true;
        }
        if ((r = cuda_status(cudaGetLastError()))) return r;
    }
    if (E.S.n > 0) {
        IsoArgs I;
        I.S = E.S;
        I.P = P;
        I.t0 = (istep - 1) * P.dt_tree;
        I.t1 = istep * P.dt_tree;
        I.status = c->status;
        I.list = g_hb.iso.p + 2 * (size_t)E.S.n;
        I.count = I.list + E.S.n;
        // the bodies outside the clusters: n - members (the device count checks it)
        const int n_iso = std::max(1, E.S.n - E.n_members);
        if ((r = cuda_status(cudaStreamWaitEvent(s_iso, ev_iso_ready, 0)))) return r;
        { P3T_COUNT_LAUNCH(); k_isolated<<<(n_iso + 127) / 128, 128, ISO_SMEM, s_iso>>>(I); }
        if ((r = cuda_status(cudaGetLastError())) || (r = cuda_status(cudaEventRecord(ev_iso_done, s_iso))) ||
            (r = cuda_status(cudaStreamWaitEvent(c->stream, ev_iso_done, 0))))
            return r;
    }
    return cuda_status(cudaGetLastError());
}

// Stage 3: wait for the launch, then the collision list in the reference's
// order and the dissipated energy; returns the number of collisions.
int p3t_hard_fetch(int col_cap, long long *col_pairs, double *edisp) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    Context *c = E.c;
    HardBufs &B = g_hb;
    int r = 0;
    int ncol = 0;
    if ((r = d2h(c, &ncol, B.n_cols.p, sizeof(int)))) return r;
    ncol = std::min(ncol, 4096);
    g_cols.resize(ncol);
    if (ncol && (r = d2h(c, g_cols.data(), B.cols.p, ncol * sizeof(ColRec))))
        return r;
    // collision-list order of the reference: clusters of 64+ members first,
    // each group in cluster order, collisions in time order within a cluster
    std::stable_sort(g_cols.begin(), g_cols.end(), [&](const ColRec &a, const ColRec &b) {
        const bool la = a.n >= 64, lb = b.n >= 64;
        if (la != lb) return la;
        if (a.cluster != b.cluster) return a.cluster < b.cluster;
        return a.seq < b.seq;
    });
    for (int k = 0; k < ncol && k < col_cap; k++) {
        col_pairs[2 * k] = g_cols[k].id_imp;
        col_pairs[2 * k + 1] = g_cols[k].id_tar;
    }
    // dissipated energy in the reference's order (src/hard.h:562-583,700-765):
    // per cluster the sum of its collisions in time order, then over clusters
    // of 64+ members in cluster order, then the rest in cluster order.  Clusters
    // without a collision add exact zeros, so only the listed ones are summed.
    g_edisp[0] = g_edisp[1] = 0.;
    for (int k = 0; k < ncol;) {
        double e = 0., ed = 0.;
        int j = k;
        for (; j < ncol && g_cols[j].cluster == g_cols[k].cluster; j++) {
            e += g_cols[j].edisp;
            ed += g_cols[j].edisp_d;
        }
        g_edisp[0] += e;
        g_edisp[1] += ed;
        k = j;
    }
    edisp[0] = g_edisp[0];
    edisp[1] = g_edisp[1];
    // fragments join the system (rewriteFragmentID + addFragment2ParticleSystem,
    // src/hard.h:832-943): ids in collision-list order, bodies in cluster
    // order (clusters of 64+ members first), fragments in creation order
    int nfr = 0;
    if (g_frag_cap > 0 && (r = d2h(c, &nfr, B.n_frags.p, sizeof(int)))) return r;
    nfr = std::min(nfr, g_frag_cap);
    if (nfr > 0) {
        std::vector<FragRec> fr(nfr);
        if ((r = d2h(c, fr.data(), B.frags.p, nfr * sizeof(FragRec)))) return r;
        std::vector<long long> map;
        for (const ColRec &cr : g_cols)
            for (int j = 0; j < cr.n_frag; j++) {
                map.push_back(cr.id_frag - j);
                map.push_back(E.id_next++);
            }
        // the collision records carry the final ids (Collision0::setNewFragmentID,
        // src/collisionA.h:116-120, applied before the records are written)
        auto remap = [&](long long v) {
            if (v >= 0) return v;
            for (size_t k = 0; k + 1 < map.size(); k += 2)
                if (map[k] == v) return map[k + 1];
            return v;
        };
        for (ColRec &cr : g_cols) {
            cr.id_imp = remap(cr.id_imp);
            cr.id_tar = remap(cr.id_tar);
            if (cr.n_frag) cr.id_frag = remap(cr.id_frag);
        }
        std::vector<int> ord(nfr);
        for (int k = 0; k < nfr; k++) ord[k] = k;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) {
            const bool la = fr[a].n0 >= 64, lb = fr[b].n0 >= 64;
            if (la != lb) return la;
            if (fr[a].cluster != fr[b].cluster) return fr[a].cluster < fr[b].cluster;
            return fr[a].seq < fr[b].seq;
        });
        std::vector<int> gs(nfr);
        for (int k = 0; k < nfr; k++) gs[k] = fr[ord[k]].gslot;
        const int n0 = E.S.n, nmap = (int)map.size() / 2;
        if ((r = E.grow(n0 + nfr)) || (r = B.fgslot.reserve(nfr)) || (r = B.fidx.reserve(nfr)) ||
            (r = B.fmap.reserve(map.size() + 2)) || (r = E.frag_cl.reserve(nfr)))
            return r;
        if ((r = h2d(c, B.fgslot.p, gs.data(), nfr * sizeof(int))) || (r = h2d(c, B.fidx.p, ord.data(), nfr * sizeof(int))) ||
            (map.size() && (r = h2d(c, B.fmap.p, map.data(), map.size() * sizeof(long long)))))
            return r;
        { P3T_COUNT_LAUNCH(); k_frag_append<<<(nfr + 127) / 128, 128, 0, c->stream>>>(E.S, B.H, B.frags.p, B.fgslot.p, B.fidx.p, nfr, n0,
                                                                B.fmap.p, nmap, E.frag_cl.p); }
        { P3T_COUNT_LAUNCH(); k_frag_ids<<<(n0 + 255) / 256, 256, 0, c->stream>>>(E.S, n0, B.fmap.p, nmap); }
        if ((r = cuda_status(cudaGetLastError()))) return r;
        E.S.n = n0 + nfr;
        E.frag_lo = n0;
        E.frag_hi = n0 + nfr;
        if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    }
    int st = read_status(c);
    if (st) return P3T_COUNT_STATUS(st);
    return ncol;
}

int p3t_collision_records(int cap, p3t_collision_t *out) {
    const int n = (int)g_cols.size();
    if (cap < 0 || (cap > 0 && !out)) return P3T_IO_BAD_ARGUMENT;
    for (int k = 0; k < n && k < cap; k++) {
        const ColRec &c = g_cols[k];
        p3t_collision_t &o = out[k];
        o.time = c.time;
        o.id_imp = c.id_imp;
        o.id_tar = c.id_tar;
        o.n_frag = c.n_frag;
        o.id_frag = c.n_frag ? c.id_frag : 0;
        o.mass_imp = c.mass_imp;
        o.mass_tar = c.mass_tar;
        o.mass_frag = c.mass_frag;
        for (int d = 0; d < 3; d++) {
            o.pos_imp[d] = c.pos_imp[d];
            o.pos_tar[d] = c.pos_tar[d];
            o.vel_imp[d] = c.vel_imp[d];
            o.vel_tar[d] = c.vel_tar[d];
        }
        o.flag = 1;  // flag_merge: both outcomes of this build merge (src/collisionA.h:101, collisionB.h:90)
        o.dpos_g_rel = c.dpos_g_rel;
        o.dvel_g_rel = c.dvel_g_rel;
    }
    return n;
}

int p3t_collisions_write(const char *path, int append) {
    const int n = (int)g_cols.size();
    std::vector<p3t_collision_t> v(n);
    const int r = p3t_collision_records(n, v.data());
    if (r < 0) return r;
    return p3t_collisions_write_host(path, append, n, v.data());
}

int p3t_hard(int istep, int col_cap, long long *col_pairs, double *edisp) {
    int r = p3t_hard_enqueue();
    if (r || (r = p3t_hard_integrate(istep))) return r > 0 ? P3T_COUNT_STATUS(r) : r;
    return p3t_hard_fetch(col_cap, col_pairs, edisp);
}

int p3t_set_hard_lone(float log2_steps, int ctas) {
    if (ctas < 0 || ctas > 4096 || !(log2_steps >= 0.f)) return -(int)cudaErrorInvalidValue;
    g_lone = log2_steps;
    g_lone_ctas = ctas;
    return 0;
}

int p3t_set_hard_profile(int on) {
    g_hard_profile = on ? 1 : 0;
    return 0;
}

int p3t_hard_phase_cycles(unsigned long long *out, int n) {
    if (!out || n < HP_N) return -(int)cudaErrorInvalidValue;
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    if (!g_hard_profile || !g_hb.phase.p) {
        for (int k = 0; k < HP_N; k++) out[k] = 0;
        return 0;
    }
    return d2h(c, out, g_hb.phase.p, HP_N * sizeof(unsigned long long));
}

int p3t_set_hard_step_cap(int max_block_steps) {
    if (max_block_steps < 1 || max_block_steps > MAX_BLOCK_STEPS) return -(int)cudaErrorInvalidValue;
    g_max_steps = max_block_steps;
    return 0;
}

int p3t_hard_launch_stats(double *launch_ms, long long *pairs3, double *sums5) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    int r = 0;
    if (launch_ms) {
        float ms = 0.f;
        if (g_launch_timed && (r = cuda_status(cudaEventSynchronize(g_ev_launch[1])))) return r;
        if (g_launch_timed && (r = cuda_status(cudaEventElapsedTime(&ms, g_ev_launch[0], g_ev_launch[1])))) return r;
        *launch_ms = g_launch_timed ? (double)ms : 0.;
    }
    if (pairs3) {
        unsigned long long v[2] = {0ULL, 0ULL};
        if (g_hb.live.p && (r = d2h(E.c, v, g_hb.live.p, sizeof(v)))) return r;
        pairs3[0] = (long long)v[0];
        pairs3[1] = (long long)v[1];
        pairs3[2] = (g_hard_mode == 0) ? 1 : 0;  // counted by the bundle form only
    }
    if (sums5) {
        double h[5] = {0., 0., 0., 0., 0.};
        if (g_last_nc > 0 && g_hb.cost.p && E.cl_cnt.p) {
            static DevBuf<double> buf;
            if ((r = buf.reserve(5))) return r;
            { P3T_COUNT_LAUNCH(); k_cost_sums<<<1, 512, 0, E.c->stream>>>(g_hb.cost.p, E.cl_cnt.p, g_last_nc, buf.p); }
            if ((r = cuda_status(cudaGetLastError())) || (r = d2h(E.c, h, buf.p, sizeof h))) return r;
        }
        for (int k = 0; k < 5; k++) sums5[k] = h[k];
    }
    return 0;
}

}  // extern "C"
