// Soft-force kernel interface (device side of p3t_soft_* in include/gplum_p3t.h).
#pragma once
#include "p3t_common.cuh"

namespace p3t {

// Mixed form, per particle: the FP32 two-float split of the FP64 position
// (xh = rn(x), xl = rn(x - xh); xh + xl carries x to ~2^-48 relative) with
// the mass and squared r_out, so the pair loops form displacements from FP32
// data alone.
struct __align__(16) SoftSplit {
    float xh, yh, zh, m, xl, yl, zl, ro2;
};
static_assert(sizeof(SoftSplit) == 32, "SoftSplit");
// Mixed form, per superparticle: the split position, the mass, and the
// quadrupole terms the pair loop uses, negated: -(3Q - tr I) and
// eps^2 tr (= -mtr), tr as trace_mode selects.
struct __align__(16) SpjPack {
    float xh, yh, zh, m, xl, yl, zl, nmtr;
    float nqxx, nqyy, nqzz, nqxy, nqyz, nqzx, pad0, pad1;
};
static_assert(sizeof(SpjPack) == 64, "SpjPack");

struct SoftArgs {
    // CSR lists (see include/p3t_tree.h)
    const int *i_off, *i_idx, *j_off, *j_idx, *s_off, *s_idx;
    const int *group_order;  // optional launch order of groups (nullptr = 0..n_group-1)
    int n_group;
    // particles and superparticles: i_idx indexes iptcl, j_idx indexes ptcl
    // (the same array in the device-resident form)
    const SoftPtcl *iptcl;
    const double *i_r_out, *i_r_search;     // FP64 copies (FP64 form)
    int n_iptcl;
    const SoftPtcl *ptcl;
    const double *mass, *r_out, *r_search;  // FP64 copies (FP64 form)
    int n_ptcl;
    const SPJRec *spj;
    int n_spj;
    // parameters
    float eps2;
    double eps2_d;
    int trace_mode;  // 0: xx+yy+xx (default GPLUM build), 1: xx+yy+zz (PIKG spec)
    int accumulate;  // 1: add into existing ForceGrav records, 0: overwrite
    // outputs
    ForceRec *force;  // indexed like iptcl
    D4 *acc64;   // FP64 form only: {ax, ay, az, phi}, indexed like iptcl
    int *cand;        // optional [n_iptcl x cand_cap] table of j indices
    int cand_cap;
    int *status;
    // work split of an i-group of ni members over the CTA's 128 threads:
    // ni > t_ipt2: 2 i per thread (FP64 form only); > t_s1: 1 i per thread; > t_s2: the j list
    // split 2 ways; else 4 ways (0 <= t_s2 <= 32, t_s2 <= t_s1 <= 64,
    // t_s1 <= t_ipt2 <= 128 or t_ipt2 = 256: never 2 i per thread, groups
    // above 128 in chunks of 128; 0 = the defaults 128, 64, 32)
    int t_ipt2, t_s1, t_s2;
    // mixed form: resident CTAs per SM the kernel is compiled for (4, 5 or 6;
    // 0 = 5), i.e. its register budget
    int occ;
    // mixed form scratch, filled by launch_soft before the pair kernel:
    // [n_iptcl], [n_ptcl] and [n_spj] records.  nullptr = launch_soft's own
    // per-device buffers (stream-ordered, grown on demand).
    SoftSplit *isplit, *jsplit;
    SpjPack *spjp;
};

// The soft launch shape last set through p3t_set_soft_tiles /
// p3t_set_soft_occupancy: {t_ipt2, t_s1, t_s2, occ}, process-wide, for entry
// points that run without the library context (p3t_soft_force_noalloc).
extern int g_soft_shape[4];

cudaError_t launch_pack_epj(const EPJRec *in, int n, SoftPtcl *out, double *mass, double *r_out, double *r_search,
                            cudaStream_t st);
cudaError_t launch_pack_epi(const EPIRec *in, int n, SoftPtcl *out, double *r_out, double *r_search, cudaStream_t st);
cudaError_t launch_iota(int *out, int n, int base, cudaStream_t st);
cudaError_t launch_soft(const SoftArgs &A, int precision, bool emit, cudaStream_t st);

}  // namespace p3t
