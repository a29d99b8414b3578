/* GB300 (sm_103a) P3T hot path of GPLUM behind a C ABI.
 *
 * Plain C types only: record pointers, counts, status codes.  All functions
 * return 0 on success, a negative value for a CUDA runtime error (-code), or
 * a positive bit set reported by a kernel:
 *   1 neighbour-candidate table overflow   2 list index out of range
 *   4 iteration cap reached                8 queue / pair buffer overflow
 *   16 cluster larger than the hard kernel's capacity
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

/* ---- measurement -------------------------------------------------------------
 * FMA throughput of this GPU (TFLOP/s, FMA = 2 flops), FP32 (fp64 = 0) or
 * FP64 (fp64 = 1): the roofline denominators of the soft (FP32-pipe) and
 * hard (FP64-pipe) kernels.  No counterpart in GPLUM. */
int p3t_probe_fma_peak(int fp64, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
