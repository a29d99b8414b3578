// Shared device-side definitions of the P3T path.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace p3t {

// --- host/device record layouts (byte-identical to GPLUM's FDPS classes) ---
struct EPIRec {  // EPIGrav, src/particle.h:93-141 (48 B)
    int32_t id_local, myrank;
    double pos[3];
    double r_out, r_search;
};
struct EPJRec {  // EPJGrav, src/particle.h:149-170 (112 B)
    int32_t id_local, myrank;
    double pos[3];
    double r_out, r_search;
    int64_t id;
    double mass, vel[3], acc_d[3];
};
struct SPJRec {  // FDPS SPJQuadrupole (80 B)
    double mass, pos[3], xx, yy, zz, xy, xz, yz;
};
struct ForceRec {  // ForceGrav, src/particle.h:16-86 (32 B)
    float acc[3], phi;
    int32_t number, rank, id_max, id_min;
};
static_assert(sizeof(EPIRec) == 48, "EPIGrav layout");
static_assert(sizeof(EPJRec) == 112, "EPJGrav layout");
static_assert(sizeof(SPJRec) == 80, "SPJQuadrupole layout");
static_assert(sizeof(ForceRec) == 32, "ForceGrav layout");

// Per-particle record the soft kernel gathers (48 B, 16-byte aligned): the
// FP64 position plus the FP32 quantities the functor uses, with the squared
// radii precomputed exactly as the functor rounds them:
//   ro2 = (float)r_out^2, rs2 = ((float)r_search^2) * 1.0201f.
// max(a,b)^2 rounds to max(a^2, b^2) for non-negative a, b, so the per-pair
// max of these equals the functor's per-pair square of the max.
struct __align__(16) SoftPtcl {
    double x, y, z;
    float m, ro2, rs2;
    int32_t id_local;
    int32_t rank;
    int32_t pad;
};
static_assert(sizeof(SoftPtcl) == 48, "SoftPtcl");

// status bits written by kernels (0 = ok)
enum : int {
    ST_OK = 0,
    ST_CAND_OVERFLOW = 1,   // a particle had more screen hits than candidate slots
    ST_BAD_INDEX = 2,       // a list entry pointed outside its array
    ST_ITER_CAP = 4,        // an iterative loop hit its cap
    ST_QUEUE_OVERFLOW = 8,  // a work queue or pair buffer overflowed
    ST_CLUSTER_TOO_BIG = 16 // a cluster exceeded the hard kernel's capacity
};

constexpr int INT32_MAX_ = 2147483647;

// Host-side count of the library's kernel launches (p3t_launch_count): every
// <<<...>>> launch site of the library is preceded by P3T_COUNT_LAUNCH().
extern unsigned long long g_launch_count;
#define P3T_COUNT_LAUNCH() ((void)__atomic_fetch_add(&::p3t::g_launch_count, 1ULL, __ATOMIC_RELAXED))

// 4 doubles, 16-byte aligned (the FP64 form's {ax, ay, az, phi} record)
struct __align__(16) D4 {
    double x, y, z, w;
};
__host__ __device__ inline D4 D4c(double x, double y, double z, double w) { return D4{x, y, z, w}; }

}  // namespace p3t
