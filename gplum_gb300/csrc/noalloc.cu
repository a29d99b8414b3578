// Soft force for callers that cannot allocate device memory.
//
// Some hosts of this library run it inside a runtime that owns every device
// allocation (a memory arena or pool handed out by another framework, or a
// sandboxed process in which cudaMalloc is not permitted).  Those callers can
// pass device buffers they already have, but they cannot let the library call
// cudaMalloc/cudaFree.  p3t_soft_force_noalloc serves them: the caller passes
// the body records, the interaction lists, the superparticles and the output
// buffer (all device-accessible), and the only scratch the computation needs
// -- the packed body records the soft kernel gathers, their FP32 splits, the
// packed superparticles, and one status word -- lives in file-scope static
// device arrays.
//
// Those arrays exist once per GPU that loads this library and stay allocated
// until the process exits (P3T_NOALLOC_MAX_BODIES x 80 B = 5 MiB,
// P3T_NOALLOC_MAX_SPJ x 64 B = 4 MiB, plus one status word).  Their device addresses are looked up once per device, on
// that device's first call (cudaGetSymbolAddress with the device current).
// A call waits for its stream (it reads the status word back to the host), so
// it cannot be made on a stream that is being captured into a CUDA graph.
// Every call shares the arrays: calls that overlap on the GPU (different
// streams, or several host threads) race on them and must be serialised by
// the caller.  The caller's CSR offsets are checked on the device before any
// list is read through them (status bit 2); list entries out of range are
// clamped by the kernel and reported the same way.
#include <cstdio>
#include <mutex>

#include "../../include/gplum_p3t.h"
#include "p3t_common.cuh"
#include "p3t_soft.cuh"

namespace {

static __device__ __align__(256) p3t::SoftPtcl g_noalloc_bodies[P3T_NOALLOC_MAX_BODIES];
static __device__ __align__(256) p3t::SoftSplit g_noalloc_split[P3T_NOALLOC_MAX_BODIES];
static __device__ __align__(256) p3t::SpjPack g_noalloc_spj[P3T_NOALLOC_MAX_SPJ];
static __device__ __align__(256) int g_noalloc_status[1];

struct DeviceScratch {
    bool ready = false;
    p3t::SoftPtcl *bodies = nullptr;
    p3t::SoftSplit *split = nullptr;
    p3t::SpjPack *spj = nullptr;
    int *status = nullptr;
};
constexpr int MAX_DEVICES = 64;
DeviceScratch g_scratch[MAX_DEVICES];
std::mutex g_scratch_mu;

// Device addresses of the static arrays for the current device.  The array
// names are host-side stand-ins: only these looked-up addresses may be
// passed to kernels.
int scratch_for_current_device(DeviceScratch **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return -(int)e;
    if (dev < 0 || dev >= MAX_DEVICES) return -(int)cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    DeviceScratch &s = g_scratch[dev];
    if (!s.ready) {
        e = cudaGetSymbolAddress((void **)&s.bodies, g_noalloc_bodies);
        if (e != cudaSuccess) return -(int)e;
        e = cudaGetSymbolAddress((void **)&s.split, g_noalloc_split);
        if (e != cudaSuccess) return -(int)e;
        e = cudaGetSymbolAddress((void **)&s.spj, g_noalloc_spj);
        if (e != cudaSuccess) return -(int)e;
        e = cudaGetSymbolAddress((void **)&s.status, g_noalloc_status);
        if (e != cudaSuccess) return -(int)e;
        s.ready = true;
    }
    *out = &s;
    return 0;
}

// EPJGrav records -> the soft kernel's packed bodies (the same packing as the
// allocating path: FP64 position, FP32 mass, squared radii rounded as the
// functor rounds them)
__global__ void k_noalloc_pack(const p3t::EPJRec *__restrict__ in, int n, p3t::SoftPtcl *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const p3t::EPJRec &e = in[i];
    p3t::SoftPtcl r;
    r.x = e.pos[0];
    r.y = e.pos[1];
    r.z = e.pos[2];
    r.m = (float)e.mass;
    const float ro = (float)e.r_out, rs = (float)e.r_search;
    r.ro2 = __fmul_rn(ro, ro);
    r.rs2 = __fmul_rn(__fmul_rn(rs, rs), 1.0201f);
    r.id_local = e.id_local;
    r.rank = e.myrank;
    r.pad = 0;
    out[i] = r;
}

// The caller's CSR offsets, checked on the device before any list is read:
// each starts at 0 and never decreases, and the i lists hold at most n
// entries.  A violation sets status bit 2 (list index out of range).
__global__ void k_noalloc_check(const int *__restrict__ i_off, const int *__restrict__ j_off,
                                const int *__restrict__ s_off, int n_group, int n, int *status) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g > n_group) return;
    bool bad = false;
    if (g == 0) bad = i_off[0] != 0 || j_off[0] != 0 || s_off[0] != 0;
    else bad = i_off[g] < i_off[g - 1] || j_off[g] < j_off[g - 1] || s_off[g] < s_off[g - 1];
    if (g == n_group) bad = bad || i_off[g] > n;
    if (bad) atomicOr(status, p3t::ST_BAD_INDEX);
}

}  // namespace

extern "C" int p3t_soft_force_noalloc(int n, const void *epj, int n_group, const int *i_off, const int *i_idx,
                                      const int *j_off, const int *j_idx, const int *s_off, const int *s_idx,
                                      const void *spj, int n_spj, double eps2, int trace_mode, void *force,
                                      void *stream) {
    if (n < 0 || n > P3T_NOALLOC_MAX_BODIES) {
        std::fprintf(stderr,
                     "[gplum_p3t] p3t_soft_force_noalloc: %d bodies exceed the static scratch of %d bodies; "
                     "use p3t_soft_force_host or the resident path for larger systems\n",
                     n, P3T_NOALLOC_MAX_BODIES);
        return -(int)cudaErrorInvalidValue;
    }
    if (n_spj > P3T_NOALLOC_MAX_SPJ) {
        std::fprintf(stderr,
                     "[gplum_p3t] p3t_soft_force_noalloc: %d superparticles exceed the static scratch of %d; "
                     "use p3t_soft_force_host or the resident path for larger systems\n",
                     n_spj, P3T_NOALLOC_MAX_SPJ);
        return -(int)cudaErrorInvalidValue;
    }
    if (n_group < 0 || n_spj < 0 || (trace_mode != 0 && trace_mode != 1)) return -(int)cudaErrorInvalidValue;
    if (n == 0 || n_group == 0) return 0;
    // every buffer the kernels will read or write must be there
    if (!epj || !force || !i_off || !i_idx || !j_off || !j_idx || !s_off || !s_idx || (n_spj > 0 && !spj))
        return -(int)cudaErrorInvalidValue;
    DeviceScratch *s = nullptr;
    int r = scratch_for_current_device(&s);
    if (r) return r;
    cudaStream_t st = (cudaStream_t)stream;
    // the status word keeps the previous call's value: clear it
    cudaError_t e = cudaMemsetAsync(s->status, 0, sizeof(int), st);
    if (e != cudaSuccess) return -(int)e;
    // the offsets first: no list is read through a malformed one
    { P3T_COUNT_LAUNCH(); k_noalloc_check<<<(n_group + 256) / 256, 256, 0, st>>>(i_off, j_off, s_off, n_group, n, s->status); }
    if ((e = cudaGetLastError()) != cudaSuccess) return -(int)e;
    {
        int h = 0;
        if ((e = cudaMemcpyAsync(&h, s->status, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return -(int)e;
        if (h) return h;
    }
    { P3T_COUNT_LAUNCH(); k_noalloc_pack<<<(n + 255) / 256, 256, 0, st>>>((const p3t::EPJRec *)epj, n, s->bodies); }
    if ((e = cudaGetLastError()) != cudaSuccess) return -(int)e;
    p3t::SoftArgs A{};
    A.i_off = i_off;
    A.i_idx = i_idx;
    A.j_off = j_off;
    A.j_idx = j_idx;
    A.s_off = s_off;
    A.s_idx = s_idx;
    A.group_order = nullptr;
    A.n_group = n_group;
    A.iptcl = s->bodies;
    A.n_iptcl = n;
    A.ptcl = s->bodies;
    A.n_ptcl = n;
    A.spj = (const p3t::SPJRec *)spj;
    A.n_spj = n_spj;
    A.eps2 = (float)eps2;
    A.eps2_d = eps2;
    A.trace_mode = trace_mode;
    A.accumulate = 0;
    A.force = (p3t::ForceRec *)force;
    A.acc64 = nullptr;
    A.cand = nullptr;
    A.cand_cap = 0;
    A.status = s->status;
    A.jsplit = s->split;
    A.isplit = s->split;
    A.spjp = s->spj;
    // the launch shape the setters chose (the same as the allocating path's)
    A.t_ipt2 = p3t::g_soft_shape[0];
    A.t_s1 = p3t::g_soft_shape[1];
    A.t_s2 = p3t::g_soft_shape[2];
    A.occ = p3t::g_soft_shape[3];
    if ((e = launch_soft(A, 0, false, st)) != cudaSuccess) return -(int)e;
    int h = 0;
    if ((e = cudaMemcpyAsync(&h, s->status, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return -(int)e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return -(int)e;
    return h;
}
