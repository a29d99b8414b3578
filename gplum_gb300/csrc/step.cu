// The whole P3T tree step as one native call, and the exchange of GPLUM's
// FPGrav particle records with the device state.
//
// p3t_startup / p3t_tree_step run the phases of GPLUM's main loop
// (src/main_p3t.cpp:289-364 start-up, :423-717 one step) in order on the
// HBM-resident state, on the library stream, with the host taking only the
// decisions that loop takes (collisions, removals, the periodic re-force).
// Every phase boundary is marked by a CUDA event, so the step's device time
// and its phase split come from the GPU's own clock (p3t_step_phases_ms).
//
// p3t_state_put_fpgrav / p3t_state_get_fpgrav move a host array of 344-byte
// FPGrav records (GPLUM's ParticleSystem<FPGrav>) to and from the
// structure-of-arrays state in one copy each way: the records cross the host
// link as one block, and a kernel unpacks (packs) them through shared memory
// with coalesced 8-byte loads and stores.
#include <algorithm>
#include <cstring>

#include "../../include/gplum_p3t.h"
#include "p3t_engine.cuh"
#include "p3t_fpgrav.h"

namespace p3t {
namespace {

constexpr int REC_T = 64;                                  // records per CTA of the pack kernels
constexpr int REC_W = (int)sizeof(FPGravRecord) / 8;       // 43 eight-byte words per record

// records [b*REC_T, ...) of `in` into shared memory, 8-byte words, coalesced
__device__ void stage_in(const unsigned long long *__restrict__ in, unsigned long long *sm, int n) {
    const int r0 = blockIdx.x * REC_T;
    const int nr = min(REC_T, n - r0);
    const unsigned long long *src = in + (size_t)r0 * REC_W;
    for (int w = threadIdx.x; w < nr * REC_W; w += blockDim.x) sm[w] = src[w];
}

__global__ void __launch_bounds__(REC_T) k_fp_unpack(const unsigned long long *__restrict__ in, int n, State S) {
    __shared__ unsigned long long sm[REC_T * REC_W];
    stage_in(in, sm, n);
    __syncthreads();
    const int i = blockIdx.x * REC_T + threadIdx.x;
    if (i >= n) return;
    const FPGravRecord &r = *reinterpret_cast<const FPGravRecord *>(sm + threadIdx.x * REC_W);
    for (int d = 0; d < 3; d++) {
        S.pos[3 * i + d] = r.pos[d];
        S.vel[3 * i + d] = r.vel[d];
        S.acc[3 * i + d] = r.acc[d];
        S.acc_d[3 * i + d] = r.acc_d[d];
        S.jerk_d[3 * i + d] = r.jerk_d[d];
        S.acc_s[3 * i + d] = r.acc_s[d];
        S.jerk_s[3 * i + d] = r.jerk_s[d];
    }
    S.r_out[i] = r.r_out;
    S.r_search[i] = r.r_search;
    S.id[i] = r.id;
    S.mass[i] = r.mass;
    S.phi[i] = r.phi;
    S.phi_d[i] = r.phi_d;
    S.phi_s[i] = r.phi_s;
    S.v_disp[i] = r.v_disp;
    S.r_out_inv[i] = r.r_out_inv;
    S.time[i] = r.time;
    S.dt[i] = r.dt;
    S.acc0[i] = r.acc0;
    S.r_planet[i] = r.r_planet;
    S.f[i] = r.f;
    S.number[i] = r.number;
    S.rank[i] = r.rank;
    S.id_max[i] = r.id_max;
    S.id_min[i] = r.id_min;
    S.id_cluster[i] = r.id_cluster;
    S.n_cluster[i] = r.n_cluster;
    S.dead[i] = r.is_dead;
    S.merged[i] = r.is_merged;
}

__global__ void __launch_bounds__(REC_T) k_fp_pack(State S, int n, unsigned long long *__restrict__ out) {
    __shared__ unsigned long long sm[REC_T * REC_W];
    const int i = blockIdx.x * REC_T + threadIdx.x;
    if (i < n) {
        FPGravRecord &r = *reinterpret_cast<FPGravRecord *>(sm + threadIdx.x * REC_W);
        r.id_local = i;  // setIDLocalAndMyrank (src/func.h:135-149), one rank
        r.myrank = 0;
        for (int d = 0; d < 3; d++) {
            r.pos[d] = S.pos[3 * i + d];
            r.vel[d] = S.vel[3 * i + d];
            r.acc[d] = S.acc[3 * i + d];
            r.acc_d[d] = S.acc_d[3 * i + d];
            r.jerk_d[d] = S.jerk_d[3 * i + d];
            r.acc_s[d] = S.acc_s[3 * i + d];
            r.jerk_s[d] = S.jerk_s[3 * i + d];
            r.acc_gd[d] = 0.;
        }
        r.r_out = S.r_out[i];
        r.r_search = S.r_search[i];
        r.id = S.id[i];
        r.mass = S.mass[i];
        r.phi = S.phi[i];
        r.phi_d = S.phi_d[i];
        r.phi_s = S.phi_s[i];
        r.v_disp = S.v_disp[i];
        r.r_out_inv = S.r_out_inv[i];
        r.time = S.time[i];
        r.dt = S.dt[i];
        r.acc0 = S.acc0[i];
        r.r_planet = S.r_planet[i];
        r.f = S.f[i];
        r.number = S.number[i];
        r.rank = S.rank[i];
        r.id_max = S.id_max[i];
        r.id_min = S.id_min[i];
        r.id_cluster = S.id_cluster[i];
        r.n_cluster = S.n_cluster[i];
        r.in_domain = 1;
        r.is_sent = 0;
        r.is_dead = (uint8_t)(S.dead[i] != 0);
        r.is_merged = (uint8_t)(S.merged[i] != 0);
    }
    __syncthreads();
    const int r0 = blockIdx.x * REC_T;
    const int nr = min(REC_T, n - r0);
    unsigned long long *dst = out + (size_t)r0 * REC_W;
    for (int w = threadIdx.x; w < nr * REC_W; w += blockDim.x) dst[w] = sm[w];
}

// loop parameters of the last p3t_startup, the step's phase events
struct StepCtx {
    p3t_loop_params_t lp{0.5, 8, 256, 1024, 40., 0.1};
    bool have_lp = false;
    cudaEvent_t ev[P3T_STEP_PHASES + 1] = {};
    bool ev_ok = false;
    bool timed = false;
    DevBuf<unsigned long long> fp;  // staging of FPGrav records
};
StepCtx g_step;

int events_init(Context *c) {
    (void)c;
    if (g_step.ev_ok) return 0;
    for (auto &e : g_step.ev) {
        const int r = cuda_status(cudaEventCreate(&e));
        if (r) return r;
    }
    g_step.ev_ok = true;
    return 0;
}

int mark(Context *c, int k) { return cuda_status(cudaEventRecord(g_step.ev[k], c->stream)); }

}  // namespace
}  // namespace p3t

using namespace p3t;

extern "C" {

int p3t_startup(const p3t_loop_params_t *lp, double *energy5) {
    Engine &E = g_eng;
    if (!E.c && !(E.c = ctx_get(0))) return -(int)cudaErrorNoDevice;
    if (lp) {
        if (!(lp->theta >= 0.) || lp->n_leaf_limit < 1 || lp->n_group_limit < 1 || lp->reset_step < 1)
            return -(int)cudaErrorInvalidValue;
        g_step.lp = *lp;
    }
    g_step.have_lp = true;
    const p3t_loop_params_t &L = g_step.lp;
    int r = 0;
    if ((r = p3t_set_cutoff_radii())) return r;
    // src/main_p3t.cpp:344-364: two passes of the soft force and
    // correctForceLongInitial (USE_RE_SEARCH_NEIGHBOR)
    for (int pass = 0; pass < 2; pass++) {
        if ((r = p3t_state_tree_soft(L.theta, L.n_leaf_limit, L.n_group_limit))) return r;
        if ((r = p3t_correct(1))) return r;
    }
    double e[5];
    if ((r = p3t_energy(e))) return r;
    if (energy5) std::memcpy(energy5, e, sizeof e);
    return 0;
}

int p3t_tree_step(int istep, p3t_step_result_t *out) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    if (!g_step.have_lp) return -(int)cudaErrorInvalidValue;  // p3t_startup first
    Context *c = E.c;
    const p3t_loop_params_t &L = g_step.lp;
    p3t_step_result_t res;
    std::memset(&res, 0, sizeof res);
    int r = 0;
    if ((r = events_init(c))) return r;
    g_step.timed = false;
    static long long cols_buf[2 * 4096];
    double ed_hard[2] = {0., 0.};
    // 1st velocity kick (src/main_p3t.cpp:446)
    if ((r = mark(c, P3T_PH_KICK1)) || (r = p3t_kick())) return r;
    // createNeighborCluster + makeList (:474-481, :523-524)
    if ((r = mark(c, P3T_PH_CLUSTER)) || (r = p3t_cluster_label())) return r;
    res.n_clusters = E.n_clusters;
    res.n_isolated = E.S.n - E.n_members;
    // timeIntegrate + collisions (:525-540)
    if ((r = mark(c, P3T_PH_HARD))) return r;
    const int ncol = p3t_hard(istep, 4096, cols_buf, ed_hard);
    if (ncol < 0) return P3T_STATUS_BITS(ncol) ? P3T_STATUS_BITS(ncol) : ncol;
    res.n_col = ncol;
    res.edisp_hard[0] = ed_hard[0];
    res.edisp_hard[1] = ed_hard[1];
    double edisp = ed_hard[0];
    // soft force on the new positions and correctForceLong (:583-593)
    if ((r = mark(c, P3T_PH_SOFT)) ||
        (r = p3t_state_tree_soft(L.theta, L.n_leaf_limit, L.n_group_limit)))
        return r;
    if ((r = mark(c, P3T_PH_CORRECT)) || (r = p3t_correct(0))) return r;
    // 2nd velocity kick and the energy (:611-625)
    if ((r = mark(c, P3T_PH_KICK2)) || (r = p3t_kick())) return r;
    if ((r = mark(c, P3T_PH_ENERGY)) || (r = p3t_energy(res.energy))) return r;
    // MergeParticle (:636-638)
    if ((r = mark(c, P3T_PH_MERGE))) return r;
    if (ncol > 0) {
        double em = 0.;
        if ((r = p3t_merge(&em))) return r;
        edisp += em;
    }
    // removeParticlesOutOfBoundary (:641)
    if ((r = mark(c, P3T_PH_REMOVE))) return r;
    double erem = 0.;
    const int nrem = p3t_remove_out_of_boundary(L.r_max, L.r_min, &erem);
    if (nrem < 0) return P3T_STATUS_BITS(nrem) ? P3T_STATUS_BITS(nrem) : nrem;
    res.n_removed = nrem;
    edisp += erem;
    // re-force after collisions, removals and every reset_step (:646-710)
    if ((r = mark(c, P3T_PH_REFORCE))) return r;
    if (ncol > 0 || nrem > 0 || istep % L.reset_step == L.reset_step - 1) {
        res.reforced = 1;
        if ((r = p3t_set_cutoff_radii()) || (r = p3t_state_tree_soft(L.theta, L.n_leaf_limit, L.n_group_limit)) ||
            (r = p3t_correct(1)) || (r = p3t_energy(res.energy)))
            return r;
    }
    if ((r = mark(c, P3T_STEP_PHASES)) || (r = cuda_status(cudaEventSynchronize(g_step.ev[P3T_STEP_PHASES]))))
        return r;
    g_step.timed = true;
    res.edisp = edisp;
    res.n_body = E.S.n;
    if (out) *out = res;
    return 0;
}

int p3t_step_phases_ms(float *ms) {
    if (!ms) return -(int)cudaErrorInvalidValue;
    if (!g_step.timed) return -(int)cudaErrorNotReady;
    for (int k = 0; k < P3T_STEP_PHASES; k++) {
        const int r = cuda_status(cudaEventElapsedTime(&ms[k], g_step.ev[k], g_step.ev[k + 1]));
        if (r) return r;
    }
    return 0;
}

int p3t_state_put_fpgrav(int n, const void *records, long long id_next) {
    Engine &E = g_eng;
    if (n < 0 || (n > 0 && !records)) return -(int)cudaErrorInvalidValue;
    int r = E.ensure(n);
    if (r) return r;
    Context *c = E.c;
    if ((r = g_step.fp.reserve((size_t)n * REC_W))) return r;
    if ((r = h2d(c, g_step.fp.p, records, (size_t)n * sizeof(FPGravRecord)))) return r;
    E.S.n = n;
    if (n > 0) { P3T_COUNT_LAUNCH(); k_fp_unpack<<<(n + REC_T - 1) / REC_T, REC_T, 0, c->stream>>>(g_step.fp.p, n, E.S); }
    if ((r = cuda_status(cudaGetLastError()))) return r;
    if (id_next > E.id_next) E.id_next = id_next;
    E.frag_lo = E.frag_hi = n;
    return 0;
}

int p3t_state_get_fpgrav(void *records, int cap) {
    Engine &E = g_eng;
    if (!E.c) return -(int)cudaErrorNoDevice;
    const int n = E.S.n;
    if (cap < n || (n > 0 && !records)) return -(int)cudaErrorInvalidValue;
    Context *c = E.c;
    int r = 0;
    if ((r = g_step.fp.reserve((size_t)n * REC_W))) return r;
    if (n > 0) { P3T_COUNT_LAUNCH(); k_fp_pack<<<(n + REC_T - 1) / REC_T, REC_T, 0, c->stream>>>(E.S, n, g_step.fp.p); }
    if ((r = cuda_status(cudaGetLastError()))) return r;
    if ((r = d2h(c, records, g_step.fp.p, (size_t)n * sizeof(FPGravRecord)))) return r;
    return n;
}

}  // extern "C"
