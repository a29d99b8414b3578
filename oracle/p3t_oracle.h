/* CPU restatement of GPLUM's P3T hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * Used by tests/ (as the checker), by __graft_entry__.smoke() and by the CPU
 * baseline legs of bench.py.  The product never links or loads it.
 *
 * The extern "C" surface mirrors oracle/ref_build/ref_wrap.cpp (prefix orc_
 * instead of ref_) so that the same harness drives both; the restatement is
 * pinned against the reference build by tests/test_oracle_pin.py and by the
 * committed fixtures in tests/golden/.
 *
 * Record layouts shared with the device path (FDPS classes of GPLUM):
 *   EPIGrav  48 B  {int id_local, myrank; double pos[3], r_out, r_search}
 *   EPJGrav 112 B  EPIGrav + {long long id; double mass, vel[3], acc_d[3]}
 *   SPJQuad  80 B  {double mass, pos[3], xx, yy, zz, xy, xz, yz}
 *   ForceGrav 32 B {float acc[3], phi; int number, rank, id_max, id_min}
 */
#ifndef P3T_ORACLE_H
#define P3T_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* soft functors (src/gravity_kernel.hpp:25-121, 138-238) */
void orc_epep_f32(const void *epi, int ni, const void *epj, int nj, void *force);
void orc_epsp_f32(const void *epi, int ni, const void *spj, int nj, void *force, int trace_mode);
/* FP64 restatement: acc/phi accumulate into double acc[4*ni] (x,y,z,phi), the
 * neighbour fields into int ngb[4*ni] (number, rank, id_max, id_min). */
void orc_epep_f64(const void *epi, int ni, const void *epj, int nj, double *acc, int *ngb);
void orc_epsp_f64(const void *epi, int ni, const void *spj, int nj, double *acc, int trace_mode);

#ifdef __cplusplus
}
#endif
#endif
