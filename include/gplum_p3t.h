/* GB300 (sm_103a) P3T hot path of GPLUM behind a C ABI.
 *
 * Plain C types only: record pointers, counts, status codes.  All functions
 * return 0 on success, a negative value for a CUDA runtime error (-code), or
 * a positive bit set reported by a kernel:
 *   1 neighbour-candidate table overflow   2 list index out of range
 *   4 iteration cap reached                8 queue / pair buffer overflow
 *   16 cluster larger than the hard kernel's capacity
 * Entry points that return a count (p3t_hard, p3t_hard_fetch,
 * p3t_remove_out_of_boundary) report kernel status bits as
 * P3T_COUNT_STATUS(bits) = -(65536 + bits), below every CUDA and file error
 * code; P3T_STATUS_BITS(r) gives the bits back (0 for any other value).
 * There is no CPU fallback: without a usable CUDA device every compute entry
 * point returns a negative status.
 *
 * Record layouts (byte-identical to GPLUM's FDPS classes, src/particle.h):
 *   EPIGrav  48 B {int32 id_local, myrank; double pos[3], r_out, r_search}
 *   EPJGrav 112 B EPIGrav + {int64 id; double mass, vel[3], acc_d[3]}
 *   SPJQuad  80 B {double mass, pos[3], xx, yy, zz, xy, xz, yz}
 *   ForceGrav 32 B {float acc[3], phi; int32 number, rank, id_max, id_min}
 *
 * The library holds one process-wide context bound to one GPU; the calls
 * are meant to come from one host thread, as GPLUM's driver makes them.
 */
#ifndef GPLUM_P3T_H
#define GPLUM_P3T_H

/* The records as C structs (the layouts above, no padding): a C caller can
 * use these; GPLUM passes its own classes, which have the same layout. */
typedef struct {
    int id_local, myrank;
    double pos[3], r_out, r_search;
} p3t_epi_t;
typedef struct {
    int id_local, myrank;
    double pos[3], r_out, r_search;
    long long id;
    double mass, vel[3], acc_d[3];
} p3t_epj_t;
typedef struct {
    double mass, pos[3], xx, yy, zz, xy, xz, yz;
} p3t_spj_t;
typedef struct {
    float acc[3], phi;
    int number, rank, id_max, id_min;
} p3t_force_t;
#ifdef __cplusplus
static_assert(sizeof(p3t_epi_t) == 48 && sizeof(p3t_epj_t) == 112 && sizeof(p3t_spj_t) == 80 &&
                  sizeof(p3t_force_t) == 32,
              "record layouts");
#endif

#define P3T_COUNT_STATUS(bits) (-(65536 + (bits)))
#define P3T_STATUS_BITS(r) ((r) <= -65536 ? -(r)-65536 : 0)

#ifdef __cplusplus
extern "C" {
#endif

/* ---- context ------------------------------------------------------------------
 * p3t_init replaces nothing in GPLUM (FDPS owns no GPU); it selects the device
 * and creates the library stream.  Every other entry point calls it with
 * device 0 on first use. */
int p3t_init(int device);
int p3t_finalize(void);
/* FPGrav static parameters (src/particle.h:417-479), 21 doubles:
 * eps2, eps2_sun, m_sun, dt_tree, dt_min, eta, eta_0, eta_sun, eta_sun0,
 * alpha2, gamma, R_cut0, R_cut1, R_search0, R_search1, R_search2, R_search3,
 * r_cut_min, r_cut_max, p_cut, dens  (FPGrav::readParameter, :500-542). */
int p3t_set_params(const double *params21);
/* precision 0 = mixed FP32/FP64 (default), 1 = plain FP64 form.
 * trace_mode 0 = the default build's quadrupole trace xx+yy+xx
 * (src/gravity_kernel.hpp:177), 1 = xx+yy+zz (src/gravity_kernel_epsp.pikg:75).
 * cand_cap = neighbour-candidate slots per particle for the device-side
 * correction (default 64). */
int p3t_set_options(int precision, int trace_mode, int cand_cap);
/* Work split of the soft kernel by i-group size ni: ni > t_ipt2 two
 * i-particles per thread (FP64 form; the mixed form runs groups above 128
 * members as chunks of 128), > t_s1 one per thread, > t_s2 the j lists split
 * two ways, else four (0 <= t_s2 <= 32 <= ..., t_s2 <= t_s1 <= 64,
 * t_s1 <= t_ipt2 <= 128, or t_ipt2 = 256: one i-particle per thread
 * throughout, groups above 128 in chunks; defaults 128, 64, 32).  Set by the autotuner
 * (gplum_gb300/autotune.py); forces agree to rounding across settings, the
 * neighbour fields bit for bit. */
int p3t_set_soft_tiles(int t_ipt2, int t_s1, int t_s2);
/* Register budget of the mixed soft kernel, as resident CTAs of 128 threads
 * per SM it is compiled for: 4, 5 (default) or 6.  Set by the autotuner;
 * results do not depend on it. */
int p3t_set_soft_occupancy(int ctas_per_sm);
/* Staging of the mixed soft kernel's tiles: 1 pipelined -- each thread
 * copies the records of its entry two tiles ahead with cp.async and converts
 * the next tile into a second buffer while the CTA computes the current one,
 * one barrier per tile; 0 (default, 1.5 % faster at 1M bodies) gather,
 * barrier, compute, barrier.  Bit-identical results.  No counterpart in
 * GPLUM's interface. */
int p3t_set_soft_pipe(int on);
/* The library's CUDA stream (cudaStream_t) for callers that order their own
 * work or timing events after the library's launches. */
void *p3t_stream(void);
int p3t_synchronize(void);

/* ---- FDPS functor surface --------------------------------------------------------
 * Single-group, synchronous calls with the exact argument list and
 * accumulate-into semantics of GPLUM's functors:
 *   calcForceEPEPWithSearch::operator()  src/gravity_kernel.hpp:25-121
 *   calcForceEPSP::operator()            src/gravity_kernel.hpp:138-238 */
int p3t_epep(const void *epi, int ni, const void *epj, int nj, void *force);
int p3t_epsp(const void *epi, int ni, const void *spj, int nj, void *force);

/* ---- FDPS multiwalk pair ----------------------------------------------------------
 * Drop-in dispatch/retrieve for
 *   tree.calcForceAllAndWriteBackMultiWalk(p3t_soft_dispatch, p3t_soft_retrieve,
 *                                          tag, system, dinfo, n_walk_limit, true)
 * replacing the functor pair of src/main_p3t.cpp:351-355,583-587,672-676.
 * One dispatch carries n_walk i-groups with their EPJ and SPJ lists (EP-EP
 * and EP-SP in one launch); the matching retrieve writes each group's
 * ForceGrav records as ForceGrav::clear followed by both functors.  Up to 8
 * tags may be in flight. */
int p3t_soft_dispatch(int tag, int n_walk, const void **epi, const int *n_epi, const void **epj,
                      const int *n_epj, const void **spj, const int *n_spj);
int p3t_soft_retrieve(int tag, int n_walk, const int *n_epi, void **force);
/* Index form (FDPS calcForceAllAndWriteBackMultiWalkIndex): the EPJ and SPJ
 * arrays travel once per call when send_flag is non-zero, and each walk
 * names its list entries by index into them. */
int p3t_soft_dispatch_index(int tag, int n_walk, const void **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const int **id_spj, const int *n_spj, const void *epj,
                            int n_epj_tot, const void *spj, int n_spj_tot, int send_flag);

/* ---- device-resident soft force ---------------------------------------------------
 * The GB300-native form of the same computation: particles and lists stay in
 * HBM and the kernel reads them by index.  Lists are the CSR output of
 * p3t_tree_export (include/p3t_tree.h); particle k's EPJGrav record is
 * epj[k] and its id_local must be k. */
int p3t_upload_particles(int n, const void *epj);
int p3t_upload_lists(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                     const int *s_off, const int *s_idx, const void *spj, int n_spj);
/* Enqueues the fused EP-EP + EP-SP kernel on the library stream (no host
 * sync); ForceGrav records start cleared.  emit_candidates != 0 also fills
 * the neighbour-candidate table used by p3t_correct. */
int p3t_soft_run(int emit_candidates);
/* Copies ForceGrav records (particle order) to the host; synchronizes. */
int p3t_download_forces(void *force, int n);
/* Status bits accumulated by kernels since the last call; clears them. */
int p3t_status(void);
/* Host buffers in, host ForceGrav records out, in one call (upload, kernel,
 * download). */
int p3t_soft_force_host(int n, const void *epj, int n_group, const int *i_off, const int *i_idx,
                        const int *j_off, const int *j_idx, const int *s_off, const int *s_idx,
                        const void *spj, int n_spj, void *force);

/* ---- device-resident P3T step ----------------------------------------------------
 * The particle system lives in HBM (the FPGrav fields the step touches);
 * each call below is one phase of GPLUM's tree step (src/main_p3t.cpp:423-717)
 * on that state.  Field codes of p3t_state_get / p3t_state_set:
 *   double[n][3]: 0 pos, 1 vel, 2 acc (soft), 3 acc_d, 4 jerk_d, 5 acc_s, 6 jerk_s
 *   double[n]:   10 phi, 11 phi_d, 12 phi_s, 13 mass, 14 r_out, 15 r_search,
 *                16 dt, 17 acc0, 18 time, 19 r_planet, 20 v_disp, 21 r_out_inv, 22 f
 *   int64[n]:   100 id, 101 id_cluster
 *   int32[n]:   102 neighbor.number, 103 n_cluster, 104 isDead, 105 isMerged,
 *               106 neighbor.rank, 107 neighbor.id_min, 108 neighbor.id_max */
/* Loads n bodies and applies the start-up reset (src/main_p3t.cpp:291-303). */
int p3t_state_load(int n, const long long *id, const double *mass, const double *r_planet, const double *f,
                   const double *pos, const double *vel);
int p3t_state_n(void);
int p3t_state_get(int field, void *out);
int p3t_state_set(int field, const void *in);
/* restore = 0: copy every state field to a device backup; restore = 1:
 * copy the backup back (same body count).  Lets a caller time or retry a
 * phase on one state (tier autotuning, cost logging).  No counterpart in
 * GPLUM. */
int p3t_state_snapshot(int restore);
/* setCutoffRadii (src/particle.h:1528-1543) on the device. */
int p3t_set_cutoff_radii(void);
/* FPGrav::setRPlanet for every body (src/particle.h:757-759). */
int p3t_set_r_planet(void);
/* Soft force of the state over caller-supplied lists (the
 * calcForceAllAndWriteBack pass of src/main_p3t.cpp:583-587), with the
 * neighbour-candidate table filled for p3t_correct. */
int p3t_state_soft(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                   const int *s_off, const int *s_idx, const void *spj, int n_spj);
/* The same step with the lists built on the device from the state's own
 * positions, masses and search radii (no host round trip): the octree and
 * interaction lists of include/p3t_tree.h's builder (FDPS's TreeForForce as
 * GPLUM drives it, src/main_p3t.cpp:344-355,581-587,672-676), written into
 * the resident soft-force buffers.  p3t_state_tree builds only;
 * p3t_state_tree_soft builds and runs the soft force (with candidates). */
int p3t_state_tree(double theta, int n_leaf_limit, int n_group_limit);
int p3t_state_tree_soft(double theta, int n_leaf_limit, int n_group_limit);
/* The resident lists (from p3t_state_tree or an upload): counts[0..4] =
 * groups, i entries, EPJ entries, SPJ entries, SPJ records; then the CSR
 * arrays and the SPJ records (80-byte SPJQuadrupole each) in the layout of
 * include/p3t_tree.h. */
int p3t_tree_lists_counts(long long *counts);
int p3t_tree_lists_get(int *i_off, int *i_idx, int *j_off, int *j_idx, int *s_off, int *s_idx, void *spj);
/* correctForceLong (initial = 0) / correctForceLongInitial (initial = 1),
 * src/gravity_soft.h:245-528: FP64 cutoff correction, exact neighbour test,
 * neighbour lists, acc0 (and for initial: sun force, acc_d, jerk_d, phi_d,
 * first dt). */
int p3t_correct(int initial);
/* The same call under the name of the hot-path contract: correctForceLong /
 * correctForceLongInitial with the neighbour search (src/gravity_soft.h:245-528). */
int p3t_correct_and_search(int initial);
int p3t_neighbor_counts(int *n_ngb_tot, int *n_with_ngb);
/* Neighbour local indices of body i (returns their count, at most cap). */
int p3t_neighbor_list(int i, int *out, int cap);
/* NeighborList::pair_list (src/neighbor.h:635-670) of the last correction:
 * the local pairs (i, j), i < j, j a neighbour of i, ordered by i and then
 * by neighbour-list order (ascending j), as int[2] each.  Returns the pair
 * count; the pairs are written when cap >= that count. */
int p3t_neighbor_pairs(int *out, long long cap);
/* NeighborList::createNeighborCluster (src/neighbor.h:800-839) followed by
 * HardSystem::makeList (src/hard.h:321-438). */
int p3t_cluster_label(void);
/* off has n_clusters + 1 entries, members sum(cluster sizes). */
int p3t_cluster_lists(int *n_clusters, int *off, int *members);
/* HardSystem::timeIntegrate (src/hard.h:554-829): every cluster in one
 * persistent launch plus the isolated-body drift.  Returns the number of
 * collisions (>= 0) and writes (impactor id, target id) pairs and the
 * dissipated energy {total, hard part}; a negative value is an error. */
int p3t_hard(int istep, int col_cap, long long *col_pairs, double *edisp);
/* p3t_hard in three stages (HardSystem::makeList / timeIntegrate / the
 * collision records, src/hard.h:321-438,554-829): enqueue orders the
 * clusters of the last p3t_cluster_label into the work queue and integrate
 * queues the launches for tree step istep, both without waiting (except that
 * integrate waits for the queue's tier sizes before it submits the wide form
 * and the lone form's own kernel, so that their CTAs take SMs before the
 * persistent bundle CTAs); fetch waits and returns the collision count with
 * the pairs and the dissipated energy as p3t_hard does. */
int p3t_hard_enqueue(void);
int p3t_hard_integrate(int istep);
int p3t_hard_fetch(int col_cap, long long *col_pairs, double *edisp);
/* Size tiers of the hard launch: clusters of >= cta_min members run one per
 * CTA, of >= warp_min one per warp, smaller ones one per thread (defaults
 * 8 and 64; GPLUM's own cutoff between its parallel and serial cluster
 * loops is 64, src/hard.h:562).  No counterpart in GPLUM's interface. */
int p3t_set_hard_tiers(int warp_min, int cta_min);
/* Execution form of the hard launch: 0 (default) bundles -- each CTA holds
 * the members of many clusters in shared memory and advances them together,
 * so FP64 work is spread over all lanes; clusters above the bundle capacity
 * (256 members) run one per CTA.  1: the size tiers of p3t_set_hard_tiers.
 * Both give identical results.  No counterpart in GPLUM's interface. */
int p3t_set_hard_mode(int mode);
/* Bundle form with the learned order: clusters whose predicted
 * log2(1 + block steps) is at least log2_steps run first, each alone in a
 * bundle CTA, so the longest chains of block steps do not wait on a full
 * bundle (default 6.75, about 110 block steps; set by the autotuner from
 * whole runs; 0 turns it off).  Results do not depend on it. */
int p3t_set_hard_heavy(float log2_steps);
/* Bundle form: the clusters above the bundle's member slots run in a second,
 * concurrent launch as lone bundles of up to 512 slots, one per CTA of 512
 * threads holding its SM, submitted before the bundle kernel (1, default), or
 * one cluster per CTA inside the main launch (0).  Results are bit-identical;
 * set by the autotuner. */
int p3t_set_hard_wide(int on);
/* Bundle form: member slots per bundle and resident CTAs per SM -- 256/2
 * (default), 128/3 or 128/4 (clusters above the slot count go to the wide
 * or one-per-CTA form).  Results are bit-identical; set by the autotuner. */
int p3t_set_hard_bundle(int member_slots, int ctas_per_sm);
/* Bundle form with the learned order: clusters whose predicted
 * log2(1 + block steps) is at least log2_steps and that have at most 64
 * members run in the lone form -- each integrated alone by one CTA that holds
 * the whole cluster in shared memory for all its block steps, with the
 * independent parts of a block step (members x components, target x partner
 * pair terms, the sun force, the two time-step criteria) spread over the
 * CTA's threads -- which shortens a block step's chain of FP64 operations
 * (the longest chains of block steps set the launch's span).  ctas = 0: the
 * lone clusters run first in the bundle kernel's own CTAs (256 threads, beside
 * bundles on the SM's other CTA slot); ctas > 0: in a kernel of that many
 * 128-thread CTAs of their own, each holding a whole SM.  Perfect accretion
 * only (with fragmentation the clusters stay in the bundles); a block step
 * with a collision runs in the one-cluster-per-CTA form's loop and the lone
 * form goes on from its result.  log2_steps = 0:
 * off (the default).  Results are bit-identical.  ctas in [0, 4096].  No
 * counterpart in GPLUM's interface. */
int p3t_set_hard_lone(float log2_steps, int ctas);
/* Device tree forms.  Bit 0, the walk of the interaction lists: 1 (default)
 * breadth first, one CTA per group, every thread testing cells of the
 * group's frontier; 0 the subtree tasks of one thread each.  Both emit the
 * host builder's depth-first lists entry for entry (a group whose frontier
 * outgrows its CTA takes the task walk).  Bit 1, the moments: 0 (default)
 * every leaf in one launch over a compacted leaf list, then the inner nodes
 * one level at a time; 1 all nodes one level at a time; the same values.  No
 * counterpart in GPLUM's interface. */
int p3t_set_walk(int form);
/* Per-phase clock counts of the bundle form's loop (off by default; on, each
 * CTA's thread 0 reads the SM clock at the barriers that end the phases):
 * p3t_hard_phase_cycles writes, summed over the CTAs of the last launch, the
 * cycles of: 0 clusters above the slots and the lone tier, 1 admission
 * (claim, load, first force), 2 block time, 3 prediction, 4 collision
 * detection, 5 active set, 6 pair terms, 7 their sums, 8 correction, 9 time
 * steps, 10 collisions, 11 system time, 12 retirement, 13 of which (in
 * 1, 6, 12) the pair-term drains; n >= 14.  No
 * counterpart in GPLUM's interface (its CALC_WTIME timers are per call). */
int p3t_set_hard_profile(int on);
int p3t_hard_phase_cycles(unsigned long long *out, int n);
/* The walk form the last device tree's lists came from (1 breadth first, 0
 * tasks), -1 before the first build. */
int p3t_walk_last(void);
/* Limits of the breadth-first walk: frontier items a group's CTA may hold
 * (1..4096, default 4096) and items of the store that keeps the groups'
 * final frontiers between the count and fill passes (0: unchanged; it grows
 * by itself after an overflow).  A build that exceeds either takes the task
 * walk for its lists (same lists).  For tests of that fallback. */
int p3t_set_walk_limits(int frontier_cap, long long store_items);
/* KOMINAMI fragmentation of the collision outcome (src/collisionB.h:7-93;
 * Collision::a_frag, N_frag, Collision0::m_min of parameter.dat).  a_frag = 0
 * (the default) is perfect accretion.  A collision makes
 * n = min(N_frag, floor(a_frag m_imp / m_min)) fragments (none if n < 2) of
 * total mass a_frag m_imp on a circle around the merged pair; they join the
 * particle system after the hard launch with new ids (id_next onwards) in
 * the reference's order.  GPLUM draws the circle's phase from drand48 in
 * OpenMP order; here it is a counter-based draw keyed by (tree step,
 * impactor id, target id, seed).  Needs the bundle form of the hard launch
 * (p3t_set_hard_mode(0)); clusters above its capacity cannot fragment (status
 * bit 16). */
int p3t_set_fragmentation(double a_frag, int n_frag, double m_min, unsigned long long seed);
/* The next particle id the system will hand out (src/main_p3t.cpp:233). */
long long p3t_id_next(void);

/* ---- learned work-queue order (no counterpart in GPLUM) ------------------
 * A 4-32-32-1 FP32 MLP (tanh) predicts log2(1 + block steps) of each cluster
 * from four features: log2 n, log2 min |dr|/r_out over neighbour pairs,
 * log2(1e-6 + max |dv| dt_tree / r_out), log2(dt_tree / min member dt).
 * Parameters: W1[32][4], b1[32], W2[32][32], b2[32], w3[32], b3 (1249
 * floats); norm: feature mean[4], feature scale[4], target mean, target
 * scale (inputs enter as (x - mean) * scale, the output leaves as
 * out / scale + mean).  The order never changes any result. */
#define P3T_MLP_PARAMS 1249
#define P3T_MLP_NORM 10
/* Install / read the model (host arrays). */
int p3t_mlp_set(const float *params, const float *norm);
int p3t_mlp_get(float *params, float *norm);
/* Forget the model (the next p3t_mlp_train starts from fresh weights). */
int p3t_mlp_reset(void);
/* Predictions for n raw feature rows (host arrays [n][4] -> [n]). */
int p3t_mlp_predict(const float *x, int n, float *out);
/* Loss 0.5 mean((f(x) - y)^2) of the standardised target and its gradient
 * with respect to the parameters (host arrays), under the installed model. */
int p3t_mlp_loss_grad(const float *x, const float *y, int n, float *loss, float *grad);
/* Minibatch Adam on the device; without an installed model the weights
 * start from a seeded uniform draw and the standardisation is fitted to the
 * data.  loss_per_epoch[epochs] may be NULL. */
int p3t_mlp_train(const float *x, const float *y, int n, int epochs, int batch, float lr, unsigned long long seed,
                  float *loss_per_epoch);
/* Features of the current clusters (after p3t_cluster_label), [n][4]. */
int p3t_cluster_features(float *out, int n);
/* 0: size order (default); 1: the installed model's order (size order
 * while no model is installed). */
int p3t_set_schedule(int mode);
/* Optional priority of each cluster of the current lists (n = cluster
 * count, higher first within its tier) for the next p3t_hard; without it
 * clusters go largest first.  Ordering never changes results. */
int p3t_set_cluster_priority(const float *prio, int n);
/* Per-cluster cost of the last p3t_hard: {block steps, active-body x member
 * pair sweeps} for each cluster, in cluster-list order. */
int p3t_hard_costs(long long *out, int n);
/* Per-cluster timeline of the last p3t_hard: {start, end} of each cluster's
 * integration on the device's global timer (ns), in cluster-list order. */
int p3t_hard_times(long long *out, int n);
/* velKick, src/gravity_soft.h:5-12. */
int p3t_kick(void);
/* Energy::calcEnergy, src/energy.h:29-63: {etot, ekin, ephi_sun, ephi, ephi_d}. */
int p3t_energy(double *out5);
/* MergeParticle, src/func.h:160-207 (order-preserving removal of the merged
 * twins); adds the dissipated energy to *edisp. */
int p3t_merge(double *edisp);
/* removeParticlesOutOfBoundary, src/func.h:209-355: bodies with |x| above
 * r_max or below r_min leave the system (order-preserving); *edisp receives
 * the energy they take with them.  Returns how many left. */
int p3t_remove_out_of_boundary(double r_max, double r_min, double *edisp);

/* ---- the whole tree step -------------------------------------------------------
 * GPLUM's main loop (src/main_p3t.cpp:289-364 start-up, :423-717 one step)
 * on the device-resident state, each call running its phases in the loop's
 * order: kick, createNeighborCluster + makeList, HardSystem::timeIntegrate
 * with the collisions, the soft force and correctForceLong, kick,
 * Energy::calcEnergy, MergeParticle, removeParticlesOutOfBoundary and, after
 * a collision or removal or every reset_step steps, setCutoffRadii + soft
 * force + correctForceLongInitial + energy.  The hard launch follows
 * p3t_set_hard_mode / p3t_set_schedule; the soft force p3t_set_options.
 * There is no single counterpart in GPLUM: these replace its loop body for
 * a driver that keeps the particles on the device. */
typedef struct {
    double theta;                    /* tree opening angle (parameter.dat theta) */
    int n_leaf_limit, n_group_limit; /* FDPS tree limits (parameter.dat) */
    int reset_step;                  /* re-force every reset_step steps (parameter.dat reset_step) */
    double r_max, r_min;             /* removal boundaries (parameter.dat r_max, r_min) */
} p3t_loop_params_t;
typedef struct {
    int n_col;           /* collisions of the step (pairs: p3t_collision_records) */
    int n_removed;       /* bodies removed outside [r_min, r_max] */
    int n_body;          /* bodies after the step */
    int reforced;        /* 1 if the re-force pass ran */
    int n_clusters;      /* neighbour clusters of the hard part (HardSystem's count) */
    int n_isolated;      /* bodies without neighbours (Kepler drift or sun-only Hermite) */
    double energy[5];    /* Energy::calcEnergy after the step: etot, ekin, ephi_sun, ephi, ephi_d */
    double edisp;        /* energy dissipated in the step: collisions, merges, removals */
    double edisp_hard[2];/* of which the hard part's collisions {total, hard part} */
} p3t_step_result_t;
/* phases of p3t_step_phases_ms, in step order */
enum {
    P3T_PH_KICK1, P3T_PH_CLUSTER, P3T_PH_HARD, P3T_PH_SOFT, P3T_PH_CORRECT, P3T_PH_KICK2, P3T_PH_ENERGY,
    P3T_PH_MERGE, P3T_PH_REMOVE, P3T_PH_REFORCE, P3T_STEP_PHASES
};
/* Start-up after p3t_state_load (and p3t_set_r_planet where the radii come
 * from the masses): cutoff radii, then two passes of soft force +
 * correctForceLongInitial; energy5 (may be NULL) receives the initial
 * energy.  lp (NULL: keep the last, initially theta 0.5, 8, 256, 1024, 40,
 * 0.1) sets the loop parameters for the steps that follow. */
int p3t_startup(const p3t_loop_params_t *lp, double *energy5);
/* Tree step istep (1, 2, ...): returns 0 or a status (kernel bits
 * positive, CUDA errors negative) and fills *out (may be NULL). */
int p3t_tree_step(int istep, p3t_step_result_t *out);
/* Device time (ms) of each phase of the last p3t_tree_step, from CUDA events
 * on the library stream: P3T_STEP_PHASES floats; their sum is the step. */
int p3t_step_phases_ms(float *ms);
/* The state to and from a host array of GPLUM FPGrav records (344 bytes
 * each, ParticleSystem<FPGrav>'s element; src/particle.h:93-170,404-500),
 * one copy each way.  put replaces the state's bodies and every field the
 * step carries (no start-up reset; the neighbour lists of the last
 * correction stay with the library, so a caller that changes the body set
 * runs p3t_startup again); id_next (< 0: unchanged) raises the next
 * particle id.  get writes n records (cap >= n) and returns n. */
int p3t_state_put_fpgrav(int n, const void *records, long long id_next);
int p3t_state_get_fpgrav(void *records, int cap);
/* Block steps one cluster may take in one tree step (default and maximum
 * 1048576); a cluster that reaches it stops there and the launch reports
 * status bit 4.  No counterpart in GPLUM. */
int p3t_set_hard_step_cap(int max_block_steps);
/* The last hard launch: device time (ms) of the cluster kernel from CUDA
 * events around it on the library stream; pairs3 = {pair terms evaluated in
 * the predicted/corrected passes, in full-force passes, 1 if the launch
 * counted them (bundle form) else 0}; sums5 = over its clusters {sum of
 * active x member pair sweeps, sum of n (n - 1) x block steps, sum of active
 * members over block steps, largest block-step count, sum of n x block steps
 * (member predictions)}.  Valid until the next hard call (merges and removals
 * in between do not change them).  Any pointer may be NULL. */
int p3t_hard_launch_stats(double *launch_ms, long long *pairs3, double *sums5);

/* ---- soft force without allocation ---------------------------------------------
 * No counterpart in GPLUM.  For callers that cannot allocate device memory
 * (their device memory comes from another runtime's arena or pool, or their
 * process may not call cudaMalloc): the same fused EP-EP + EP-SP soft force
 * as p3t_soft_force_host, mixed precision, on buffers the caller provides.
 * epj (n EPJGrav records, id_local = index), the CSR lists, spj (n_spj
 * SPJQuadrupole records) and force (n ForceGrav records, overwritten as
 * ForceGrav::clear followed by both functors) are device-accessible
 * pointers; stream is a cudaStream_t (0 for the default stream); the call
 * returns after the stream has finished its work.  The library allocates
 * nothing for it: its only scratch is static per-device arrays of
 * P3T_NOALLOC_MAX_BODIES packed bodies and their FP32 position splits
 * (5 MiB), P3T_NOALLOC_MAX_SPJ packed superparticles (4 MiB), held by every
 * GPU that loads the library until the process exits, and a status word.
 * n above P3T_NOALLOC_MAX_BODIES or n_spj above P3T_NOALLOC_MAX_SPJ is
 * rejected with -cudaErrorInvalidValue and a message on stderr, and so are
 * null buffers.  The first call on a device looks up the static arrays'
 * device addresses.  Every call waits for its stream (it reads the status
 * word back), so it cannot be made on a stream under CUDA-graph capture.  The
 * offsets are checked on the device before any list is read (each starts at
 * 0 and never decreases; i_off[n_group] <= n): a violation returns status 2
 * and runs no force kernel; out-of-range list entries are clamped and also
 * return 2.  All calls share the scratch: calls that overlap on the GPU race
 * and must be serialised by the caller.  The launch shape is the one
 * p3t_set_soft_tiles / p3t_set_soft_occupancy set. */
#define P3T_NOALLOC_MAX_BODIES 65536
#define P3T_NOALLOC_MAX_SPJ 65536
int p3t_soft_force_noalloc(int n, const void *epj, int n_group, const int *i_off, const int *i_idx,
                           const int *j_off, const int *j_idx, const int *s_off, const int *s_idx,
                           const void *spj, int n_spj, double eps2, int trace_mode, void *force,
                           void *stream);

/* ---- snapshots (GPLUM's output and restart files) --------------------------------
 * snapNNNNNN.dat (ASCII, makeSnap src/func.h:53-66) and snap_tmp.dat
 * (binary, makeSnapTmp src/func.h:68-80): a FileHeader (src/energy.h:65-127)
 * then every body -- FPGrav::writeAscii / writeBinary, src/particle.h:829-876
 * -- in order, byte for byte as GPLUM writes them (the binary body record is
 * GPLUM's 344-byte FPGrav of the build with individual cutoffs, quadrupole
 * moments and collisions).  Energies are GPLUM's Energy fields in order:
 * etot, ekin, ephi_sun, ephi_planet, ephi, ephi_d, edisp (the ASCII header
 * carries etot, ekin, ephi_sun, ephi_planet and edisp). */
typedef struct {
    int n_body;
    int id_next;
    double time;
    double e_init[7];
    double e_now[7];
} p3t_file_header_t;
/* Host arrays of n bodies (pos, vel and the *_d / *_s vectors: 3 per body).
 * Writing needs id, mass, pos, vel (and r_planet, f for ASCII); other null
 * pointers write GPLUM's defaults.  Reading fills the non-null arrays. */
typedef struct {
    long long *id;
    double *mass, *r_planet, *f;
    double *pos, *vel;
    double *acc, *acc_d, *jerk_d, *acc_s, *jerk_s;
    double *phi, *phi_d, *phi_s, *r_out, *r_search, *r_out_inv, *v_disp, *time, *dt, *acc0;
    long long *id_cluster;
    int *number, *rank, *id_max, *id_min, *n_cluster, *dead, *merged;
} p3t_bodies_t;
#define P3T_IO_ERROR (-1001)        /* the file could not be opened, written or closed */
#define P3T_IO_FORMAT (-1002)       /* the file is not in the expected format */
#define P3T_IO_BAD_ARGUMENT (-1003) /* a null pointer or too small capacity */
/* The file from host arrays (n bodies; header->n_body is set to n).  No GPU. */
int p3t_snapshot_write_host(const char *path, int binary, const p3t_file_header_t *header, int n,
                            const p3t_bodies_t *bodies);
/* Reads a file's header and, with cap >= its body count, its bodies; returns
 * the body count.  An ASCII file may lack the header line (GPLUM's initial
 * conditions).  No GPU. */
int p3t_snapshot_read_host(const char *path, int binary, p3t_file_header_t *header, int cap,
                           const p3t_bodies_t *bodies);
/* The device state's bodies to a file.  async = 1: the device-to-host copies
 * are queued on the library stream (ordered before later phases) and the file
 * is formatted and written by a host thread while the next phases run;
 * p3t_snapshot_wait() joins it and returns its status.  A new write first
 * waits for the previous one. */
int p3t_snapshot_write(const char *path, int binary, const p3t_file_header_t *header, int async);
int p3t_snapshot_wait(void);
/* Loads a file into the device state (GPLUM's start-up read,
 * src/main_p3t.cpp:238-305): every body's time set to header time, neighbour
 * counts, cluster sizes and merge/dead flags cleared; a binary file restores
 * every FPGrav field the step carries.  The next id continues from
 * max(header id_next - 1, largest id) + 1.  Returns the body count. */
int p3t_snapshot_read(const char *path, int binary, p3t_file_header_t *header);

/* ---- collision records (collisionNNNNNN.dat) ---------------------------------------
 * One line per collision of a tree step, Collision0::write2File
 * (src/collisionA.h:122-148): time, impactor and target ids, fragment count
 * and first fragment id (final ids, src/hard.h:838-855), masses (twins
 * included) and states before the collision, the flag word, and the
 * relative shifts of the centre of mass |pos_g_new - pos_g| / |pos_g| and
 * |vel_g_new - vel_g| / |vel_g|. */
typedef struct {
    double time;
    long long id_imp, id_tar;
    int n_frag;
    long long id_frag;
    double mass_imp, mass_tar, mass_frag;
    double pos_imp[3], pos_tar[3], vel_imp[3], vel_tar[3];
    int flag;
    double dpos_g_rel, dvel_g_rel;
} p3t_collision_t;
/* Appends (append = 1) or writes n records in GPLUM's format.  No GPU. */
int p3t_collisions_write_host(const char *path, int append, int n, const p3t_collision_t *records);
/* The records of the last p3t_hard / p3t_hard_fetch, in collision-list
 * order: copies up to cap of them, returns how many there are. */
int p3t_collision_records(int cap, p3t_collision_t *out);
/* The last hard call's records to a collision file (append = 1: add to it). */
int p3t_collisions_write(const char *path, int append);

/* ---- measurement -------------------------------------------------------------
 * FMA throughput of this GPU (TFLOP/s, FMA = 2 flops), FP32 (fp64 = 0),
 * FP64 (fp64 = 1) or packed FP32 pairs (fp64 = 2, fma.rn.f32x2): the roofline denominators of the soft (FP32-pipe) and
 * hard (FP64-pipe) kernels.  No counterpart in GPLUM. */
int p3t_probe_fma_peak(int fp64, double *tflops);
/* Kernel launches the library has made since it was loaded (every launch
 * site counts; the peak probe above excepted).  No counterpart in GPLUM. */
unsigned long long p3t_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
