// C ABI of the P3T soft-force path (declarations and contracts in
// include/gplum_p3t.h).  One process-wide context bound to one GPU.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_common.cuh"
#include "p3t_soft.cuh"

namespace p3t {

Context *g_ctx = nullptr;
static std::mutex g_mu;

int cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return 0;
    std::fprintf(stderr, "[gplum_p3t] CUDA error %d: %s\n", (int)e, cudaGetErrorString(e));
    return -(int)e;
}

Context *ctx_get(int device) {
    if (g_ctx) return g_ctx;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_ctx) return g_ctx;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0) return nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    Context *c = new Context();
    c->device = device;
    // the library stream one step below the highest priority: the hard
    // part's side launches that must hold SMs from the start (the lone form)
    // take the highest, so the CTA dispatcher places theirs before the
    // persistent bundle CTAs; work queued beside it at the lowest (the
    // isolated bodies' drift) only takes SMs the step's own launches leave free
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    const int prio = (prio_hi < prio_lo) ? prio_hi + 1 : prio_hi;
    if (cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio) != cudaSuccess) {
        delete c;
        return nullptr;
    }
    if (cudaMalloc(&c->status, sizeof(int)) != cudaSuccess) {
        delete c;
        return nullptr;
    }
    cudaMemsetAsync(c->status, 0, sizeof(int), c->stream);
    // default parameters: FPGrav defaults, src/particle.h:917-961
    const double def[21] = {0., 0., 1., 1. / 32., 1. / 8192., 0.01, 0.001, 0.01, 0.001, 1.,
                            0.5, 2., 8., 1., 4., 1., 4., 0., 0., 0., 5.049667e6};
    std::memcpy(c->params, def, sizeof(def));
    g_ctx = c;
    return c;
}

int grow_raw(void **p, size_t *cap, size_t bytes) {
    if (bytes <= *cap) return 0;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    size_t nb = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMalloc(p, nb);
    if (e != cudaSuccess) return cuda_status(e);
    *cap = nb;
    return 0;
}

int grow_host(void **p, size_t *cap, size_t bytes) {
    if (bytes <= *cap) return 0;
    if (*p) cudaFreeHost(*p);
    *p = nullptr;
    *cap = 0;
    size_t nb = bytes + bytes / 4 + 256;
    cudaError_t e = cudaMallocHost(p, nb);
    if (e != cudaSuccess) return cuda_status(e);
    *cap = nb;
    return 0;
}

int check_csr(int n_group, const int *off) {
    if (n_group < 0) return ST_BAD_INDEX;
    if (n_group == 0) return (off && off[0] != 0) ? ST_BAD_INDEX : 0;
    if (!off || off[0] != 0) return ST_BAD_INDEX;
    for (int g = 0; g < n_group; g++)
        if (off[g + 1] < off[g]) return ST_BAD_INDEX;
    return 0;
}

int check_lists(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                const int *s_off, const int *s_idx, const void *spj, int n_spj) {
    int r = 0;
    if (n_spj < 0 || (n_spj > 0 && !spj)) return ST_BAD_INDEX;
    if ((r = check_csr(n_group, i_off)) || (r = check_csr(n_group, j_off)) || (r = check_csr(n_group, s_off)))
        return r;
    if (n_group == 0) return 0;
    if ((i_off[n_group] > 0 && !i_idx) || (j_off[n_group] > 0 && !j_idx) || (s_off[n_group] > 0 && !s_idx))
        return ST_BAD_INDEX;
    return 0;
}

int read_status(Context *c) {
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_status(e);
    if (h) cudaMemsetAsync(c->status, 0, sizeof(int), c->stream);
    return h;
}

bool is_pinned(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Host->device uploads issued as one batch: pinned sources are copied by the
// DMA engine directly, pageable ones are first gathered into the context's
// pinned staging buffer.  flush() waits for the copies, so the caller's and
// the staging buffers may be reused afterwards.
struct Uploader {
    Context *c;
    struct Item { void *dst; const void *src; size_t bytes; bool pinned; };
    std::vector<Item> items;
    explicit Uploader(Context *cc) : c(cc) {}
    void add(void *dst, const void *src, size_t bytes) {
        if (bytes) items.push_back({dst, src, bytes, is_pinned(src)});
    }
    // queues the copies; returns once they are on the stream (the caller's
    // pinned sources and the staging buffer must stay untouched until the
    // stream has run them)
    int issue() {
        size_t stage = 0;
        for (auto &it : items)
            if (!it.pinned) stage += (it.bytes + 255) / 256 * 256;
        int r = grow_host(&c->h_stage, &c->h_stage_cap, stage);
        if (r) return r;
        char *h = (char *)c->h_stage;
        for (auto &it : items) {
            const void *src = it.src;
            if (!it.pinned) {
                std::memcpy(h, it.src, it.bytes);
                src = h;
                h += (it.bytes + 255) / 256 * 256;
            }
            r = cuda_status(cudaMemcpyAsync(it.dst, src, it.bytes, cudaMemcpyHostToDevice, c->stream));
            if (r) return r;
        }
        items.clear();
        return 0;
    }
    int flush() {
        size_t stage = 0;
        for (auto &it : items)
            if (!it.pinned) stage += (it.bytes + 255) / 256 * 256;
        int r = grow_host(&c->h_stage, &c->h_stage_cap, stage);
        if (r) return r;
        char *h = (char *)c->h_stage;
        for (auto &it : items) {
            const void *src = it.src;
            if (!it.pinned) {
                std::memcpy(h, it.src, it.bytes);
                src = h;
                h += (it.bytes + 255) / 256 * 256;
            }
            r = cuda_status(cudaMemcpyAsync(it.dst, src, it.bytes, cudaMemcpyHostToDevice, c->stream));
            if (r) return r;
        }
        items.clear();
        return cuda_status(cudaStreamSynchronize(c->stream));
    }
};

int d2h(Context *c, void *dst, const void *src, size_t bytes) {
    if (bytes == 0) return 0;
    int r = cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
    if (r) return r;
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int h2d(Context *c, void *dst, const void *src, size_t bytes) {
    Uploader u(c);
    u.add(dst, src, bytes);
    return u.flush();
}

// Builds SoftArgs over a set of device buffers.
SoftArgs make_args(Context *c, DevSet &d, int n_group, int n_ptcl, int n_spj, bool accumulate) {
    SoftArgs A;
    std::memset(&A, 0, sizeof(A));
    A.i_off = d.i_off.p; A.i_idx = d.i_idx.p; A.j_off = d.j_off.p; A.j_idx = d.j_idx.p;
    A.s_off = d.s_off.p; A.s_idx = d.s_idx.p;
    A.group_order = d.order_valid ? d.order.p : nullptr;
    A.n_group = n_group;
    A.ptcl = d.ptcl.p; A.mass = d.mass.p; A.r_out = d.r_out.p; A.r_search = d.r_search.p;
    A.n_ptcl = n_ptcl;
    A.iptcl = d.ptcl.p; A.i_r_out = d.r_out.p; A.i_r_search = d.r_search.p;
    A.n_iptcl = n_ptcl;
    A.spj = d.spj.p; A.n_spj = n_spj;
    A.eps2 = (float)c->params[0];
    A.eps2_d = c->params[0];
    A.trace_mode = c->trace_mode;
    A.accumulate = accumulate ? 1 : 0;
    A.force = d.force.p;
    A.acc64 = d.acc64.p;
    A.cand = d.cand.p;
    A.cand_cap = c->cand_cap;
    A.status = c->status;
    A.t_ipt2 = c->tiles[0];
    A.t_s1 = c->tiles[1];
    A.t_s2 = c->tiles[2];
    A.occ = c->soft_occ;
    return A;
}

// Launch order: largest groups first (less tail imbalance).
// launch order of the groups: most pair work first (i-slots in whole warps x
// list entries, a superparticle counted twice)
static void group_order_host(int n_group, const int *i_off_h, const int *j_off_h, const int *s_off_h, int *ord) {
    std::vector<std::pair<long long, int>> w(n_group);
    for (int g = 0; g < n_group; g++) {
        const long long ni = i_off_h[g + 1] - i_off_h[g];
        const long long nj = (j_off_h[g + 1] - j_off_h[g]) + 2LL * (s_off_h[g + 1] - s_off_h[g]);
        w[g] = {-(((ni + 31) / 32) * 32 * nj), g};
    }
    std::sort(w.begin(), w.end());
    for (int g = 0; g < n_group; g++) ord[g] = w[g].second;
}

int set_group_order(Context *c, DevSet &d, int n_group, const int *i_off_h, const int *j_off_h,
                           const int *s_off_h) {
    std::vector<int> ord(n_group);
    group_order_host(n_group, i_off_h, j_off_h, s_off_h, ord.data());
    int r = d.order.reserve((size_t)n_group);
    if (r) return r;
    r = cuda_status(cudaMemcpyAsync(d.order.p, ord.data(), n_group * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    if (r) return r;
    r = cuda_status(cudaStreamSynchronize(c->stream));  // ord is a host temporary
    d.order_valid = (r == 0);
    return r;
}

}  // namespace p3t

using namespace p3t;

#define CTX_OR_FAIL(c)                    \
    Context *c = ctx_get(0);              \
    if (!c) return -(int)cudaErrorNoDevice;

namespace p3t {
unsigned long long g_launch_count = 0;
int g_soft_shape[4] = {128, 64, 32, 5};
}

extern "C" {

unsigned long long p3t_launch_count(void) { return __atomic_load_n(&p3t::g_launch_count, __ATOMIC_RELAXED); }

int p3t_init(int device) {
    Context *c = ctx_get(device);
    return c ? 0 : -(int)cudaErrorNoDevice;
}

int p3t_finalize(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ctx) return 0;
    Context *c = g_ctx;
    cudaStreamSynchronize(c->stream);
    c->release();
    cudaFree(c->status);
    cudaStreamDestroy(c->stream);
    delete c;
    g_ctx = nullptr;
    return 0;
}

int p3t_set_params(const double *params21) {
    CTX_OR_FAIL(c);
    std::memcpy(c->params, params21, 21 * sizeof(double));
    c->params_version++;
    return 0;
}

int p3t_set_soft_tiles(int t_ipt2, int t_s1, int t_s2) {
    CTX_OR_FAIL(c);
    if (t_s2 < 0 || t_s2 > 32 || t_s1 < t_s2 || t_s1 > 64 || t_ipt2 < t_s1 || (t_ipt2 > 128 && t_ipt2 != 256))
        return ST_BAD_INDEX;
    c->tiles[0] = g_soft_shape[0] = t_ipt2;
    c->tiles[1] = g_soft_shape[1] = t_s1;
    c->tiles[2] = g_soft_shape[2] = t_s2;
    return 0;
}

int p3t_set_soft_occupancy(int ctas_per_sm) {
    CTX_OR_FAIL(c);
    if (ctas_per_sm < 4 || ctas_per_sm > 6) return ST_BAD_INDEX;
    c->soft_occ = g_soft_shape[3] = ctas_per_sm;
    return 0;
}

int p3t_set_options(int precision, int trace_mode, int cand_cap) {
    CTX_OR_FAIL(c);
    if (precision < 0 || precision > 1 || trace_mode < 0 || trace_mode > 1 || cand_cap < 1) return ST_BAD_INDEX;
    c->precision = precision;
    c->trace_mode = trace_mode;
    c->cand_cap = cand_cap;
    return 0;
}

void *p3t_stream(void) {
    Context *c = ctx_get(0);
    return c ? (void *)c->stream : nullptr;
}

int p3t_synchronize(void) {
    CTX_OR_FAIL(c);
    return cuda_status(cudaStreamSynchronize(c->stream));
}

int p3t_status(void) {
    CTX_OR_FAIL(c);
    return read_status(c);
}

// ---- device-resident soft force ---------------------------------------------
int p3t_upload_particles(int n, const void *epj) {
    if (n < 0 || (n > 0 && !epj)) return ST_BAD_INDEX;
    CTX_OR_FAIL(c);
    DevSet &d = c->res;
    int r = 0;
    if ((r = d.epj_stage.reserve(n)) || (r = d.ptcl.reserve(n)) || (r = d.mass.reserve(n)) ||
        (r = d.r_out.reserve(n)) || (r = d.r_search.reserve(n)) || (r = d.force.reserve(n)) ||
        (r = d.acc64.reserve(n)))
        return r;
    if ((r = h2d(c, d.epj_stage.p, epj, (size_t)n * sizeof(EPJRec)))) return r;
    r = cuda_status(launch_pack_epj(d.epj_stage.p, n, d.ptcl.p, d.mass.p, d.r_out.p, d.r_search.p, c->stream));
    if (r) return r;
    c->res_n = n;
    return 0;
}

int p3t_upload_lists(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                     const int *s_off, const int *s_idx, const void *spj, int n_spj) {
    if (const int e = check_lists(n_group, i_off, i_idx, j_off, j_idx, s_off, s_idx, spj, n_spj)) return e;
    CTX_OR_FAIL(c);
    DevSet &d = c->res;
    const long long ni = n_group ? i_off[n_group] : 0, nj = n_group ? j_off[n_group] : 0,
                    ns = n_group ? s_off[n_group] : 0;
    int r = 0;
    if ((r = d.i_off.reserve(n_group + 1)) || (r = d.j_off.reserve(n_group + 1)) || (r = d.s_off.reserve(n_group + 1)) ||
        (r = d.i_idx.reserve(ni)) || (r = d.j_idx.reserve(nj)) || (r = d.s_idx.reserve(ns)) ||
        (r = d.spj.reserve(n_spj)))
        return r;
    Uploader u(c);
    u.add(d.i_off.p, i_off, (n_group + 1) * sizeof(int));
    u.add(d.j_off.p, j_off, (n_group + 1) * sizeof(int));
    u.add(d.s_off.p, s_off, (n_group + 1) * sizeof(int));
    u.add(d.i_idx.p, i_idx, ni * sizeof(int));
    u.add(d.j_idx.p, j_idx, nj * sizeof(int));
    u.add(d.s_idx.p, s_idx, ns * sizeof(int));
    u.add(d.spj.p, spj, (size_t)n_spj * sizeof(SPJRec));
    if ((r = u.flush())) return r;
    c->res_groups = n_group;
    c->res_spj = n_spj;
    d.order_valid = false;
    return set_group_order(c, d, n_group, i_off, j_off, s_off);
}

int p3t_soft_run(int emit_candidates) {
    CTX_OR_FAIL(c);
    DevSet &d = c->res;
    int r = 0;
    if (emit_candidates && (r = d.cand.reserve((size_t)c->res_n * c->cand_cap))) return r;
    SoftArgs A = make_args(c, d, c->res_groups, c->res_n, c->res_spj, false);
    if (!emit_candidates) A.cand = nullptr;
    return cuda_status(launch_soft(A, c->precision, emit_candidates != 0, c->stream));
}

int p3t_download_forces(void *force, int n) {
    CTX_OR_FAIL(c);
    if (n > c->res_n || n < 0) return ST_BAD_INDEX;
    int r = grow_host(&c->h_out, &c->h_out_cap, (size_t)n * sizeof(ForceRec));
    if (r) return r;
    if (is_pinned(force)) {
        r = cuda_status(cudaMemcpyAsync(force, c->res.force.p, (size_t)n * sizeof(ForceRec), cudaMemcpyDeviceToHost,
                                        c->stream));
        if (r) return r;
        r = cuda_status(cudaStreamSynchronize(c->stream));
        if (r) return r;
    } else {
        r = cuda_status(cudaMemcpyAsync(c->h_out, c->res.force.p, (size_t)n * sizeof(ForceRec),
                                        cudaMemcpyDeviceToHost, c->stream));
        if (r) return r;
        r = cuda_status(cudaStreamSynchronize(c->stream));
        if (r) return r;
        std::memcpy(force, c->h_out, (size_t)n * sizeof(ForceRec));
    }
    return read_status(c);
}

// One call, host buffers in and out, with a single wait: every upload is
// queued at once (pinned sources go straight to the copy engine), the group
// launch order is computed on the host while they run, then the kernels and
// the force download follow on the stream.
int p3t_soft_force_host(int n, const void *epj, int n_group, const int *i_off, const int *i_idx, const int *j_off,
                        const int *j_idx, const int *s_off, const int *s_idx, const void *spj, int n_spj,
                        void *force) {
    if (n < 0 || (n > 0 && (!epj || !force))) return ST_BAD_INDEX;
    if (const int e = check_lists(n_group, i_off, i_idx, j_off, j_idx, s_off, s_idx, spj, n_spj)) return e;
    CTX_OR_FAIL(c);
    DevSet &d = c->res;
    const long long ni = n_group ? i_off[n_group] : 0, nj = n_group ? j_off[n_group] : 0,
                    ns = n_group ? s_off[n_group] : 0;
    int r = 0;
    if ((r = d.epj_stage.reserve(n)) || (r = d.ptcl.reserve(n)) || (r = d.mass.reserve(n)) ||
        (r = d.r_out.reserve(n)) || (r = d.r_search.reserve(n)) || (r = d.force.reserve(n)) ||
        (r = d.acc64.reserve(n)) || (r = d.i_off.reserve(n_group + 1)) || (r = d.j_off.reserve(n_group + 1)) ||
        (r = d.s_off.reserve(n_group + 1)) || (r = d.i_idx.reserve(ni)) || (r = d.j_idx.reserve(nj)) ||
        (r = d.s_idx.reserve(ns)) || (r = d.spj.reserve(n_spj)) || (r = d.order.reserve((size_t)n_group)) ||
        (r = grow_host(&c->h_order, &c->h_order_cap, (size_t)n_group * sizeof(int) + 4)))
        return r;
    Uploader u(c);
    u.add(d.epj_stage.p, epj, (size_t)n * sizeof(EPJRec));
    u.add(d.i_off.p, i_off, (n_group + 1) * sizeof(int));
    u.add(d.j_off.p, j_off, (n_group + 1) * sizeof(int));
    u.add(d.s_off.p, s_off, (n_group + 1) * sizeof(int));
    u.add(d.i_idx.p, i_idx, ni * sizeof(int));
    u.add(d.j_idx.p, j_idx, nj * sizeof(int));
    u.add(d.s_idx.p, s_idx, ns * sizeof(int));
    u.add(d.spj.p, spj, (size_t)n_spj * sizeof(SPJRec));
    // an early return leaves no copy of this call running (the caller's
    // buffers and the staging and order buffers are reused afterwards)
    auto fail = [&](int e) {
        cudaStreamSynchronize(c->stream);
        return e;
    };
    if ((r = u.issue())) return fail(r);
    if ((r = cuda_status(launch_pack_epj(d.epj_stage.p, n, d.ptcl.p, d.mass.p, d.r_out.p, d.r_search.p, c->stream))))
        return fail(r);
    c->res_n = n;
    c->res_groups = n_group;
    c->res_spj = n_spj;
    if (n_group > 0) {
        // h_order is free: every call ends with a wait on the stream
        group_order_host(n_group, i_off, j_off, s_off, (int *)c->h_order);
        if ((r = cuda_status(cudaMemcpyAsync(d.order.p, c->h_order, n_group * sizeof(int), cudaMemcpyHostToDevice,
                                             c->stream))))
            return fail(r);
    }
    d.order_valid = true;
    if ((r = p3t_soft_run(0))) return fail(r);
    return p3t_download_forces(force, n);
}

}  // extern "C"
