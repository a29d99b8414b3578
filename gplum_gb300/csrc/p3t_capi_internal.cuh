// Library context shared by the C-ABI translation units.
#pragma once
#include <algorithm>
#include <cstddef>
#include <cuda_runtime.h>

#include "p3t_common.cuh"

namespace p3t {

int cuda_status(cudaError_t e);
int grow_raw(void **p, size_t *cap, size_t bytes);
int grow_host(void **p, size_t *cap, size_t bytes);

// Grow-only device array.
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;  // bytes
    int reserve(size_t n) { return grow_raw((void **)&p, &cap, std::max<size_t>(n, 1) * sizeof(T)); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// One set of device buffers for a soft-force problem.
struct DevSet {
    DevBuf<EPJRec> epj_stage;
    DevBuf<EPIRec> epi_stage;
    DevBuf<SoftPtcl> iptcl;
    DevBuf<double> i_r_out, i_r_search;
    DevBuf<SoftPtcl> ptcl;
    DevBuf<double> mass, r_out, r_search;
    DevBuf<SPJRec> spj;
    DevBuf<int> i_off, i_idx, j_off, j_idx, s_off, s_idx, order;
    DevBuf<ForceRec> force;
    DevBuf<D4> acc64;
    DevBuf<int> cand;
    bool order_valid = false;
    void release() {
        epj_stage.release(); epi_stage.release(); iptcl.release(); i_r_out.release(); i_r_search.release(); ptcl.release(); mass.release(); r_out.release();
        r_search.release(); spj.release(); i_off.release(); i_idx.release(); j_off.release(); j_idx.release();
        s_off.release(); s_idx.release(); order.release(); force.release(); acc64.release(); cand.release();
    }
};

constexpr int MAX_TAGS = 8;

// State of one in-flight multiwalk dispatch.
struct WalkSlot {
    DevSet d;
    void *h_in = nullptr;
    size_t h_in_cap = 0;
    void *h_out = nullptr;
    size_t h_out_cap = 0;
    cudaEvent_t done = nullptr;
    int n_i = 0;
    bool busy = false;
    int status = 0;
};

struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int *status = nullptr;  // device status bits
    double params[21];
    int params_version = 0;
    int precision = 0;
    int trace_mode = 0;
    int cand_cap = 64;
    int tiles[3] = {128, 64, 32};  // soft-kernel work split (SoftArgs::t_ipt2, t_s1, t_s2)
    int soft_occ = 5;              // mixed soft kernel: resident CTAs per SM (SoftArgs::occ)
    // resident problem
    DevSet res;
    int res_n = 0, res_groups = 0, res_spj = 0;
    // index-form multiwalk: EPJ/SPJ arrays resident across dispatches
    DevSet idx;
    int idx_nj = 0, idx_ns = 0;
    // pinned staging
    void *h_stage = nullptr;
    size_t h_stage_cap = 0;
    void *h_out = nullptr;
    size_t h_out_cap = 0;
    void *h_order = nullptr;  // group launch order on its way to the device
    size_t h_order_cap = 0;
    WalkSlot walk[MAX_TAGS];

    void release() {
        res.release();
        idx.release();
        if (h_stage) cudaFreeHost(h_stage);
        if (h_out) cudaFreeHost(h_out);
        if (h_order) cudaFreeHost(h_order);
        h_stage = h_out = h_order = nullptr;
        h_stage_cap = h_out_cap = h_order_cap = 0;
        for (auto &w : walk) {
            w.d.release();
            if (w.h_in) cudaFreeHost(w.h_in);
            if (w.h_out) cudaFreeHost(w.h_out);
            if (w.done) cudaEventDestroy(w.done);
            w = WalkSlot();
        }
    }
};

extern Context *g_ctx;
Context *ctx_get(int device);
int read_status(Context *c);
// Host checks of caller lists before any copy or kernel: CSR offsets start at
// 0 and never decrease; index arrays and records are present where the
// offsets say there are entries.  ST_BAD_INDEX otherwise.  (GPLUM trusts
// FDPS's lists; a C caller here can hand any pointer.)
int check_csr(int n_group, const int *off);
int check_lists(int n_group, const int *i_off, const int *i_idx, const int *j_off, const int *j_idx,
                const int *s_off, const int *s_idx, const void *spj, int n_spj);
// Async host->device copy; pinned sources go straight to the DMA engine,
// pageable ones through the context's pinned staging buffer.
int h2d(Context *c, void *dst, const void *src, size_t bytes);
// Device -> host copy ordered after the work queued on the library's
// stream (a non-blocking stream, which plain cudaMemcpy does not wait for).
int d2h(Context *c, void *dst, const void *src, size_t bytes);

struct SoftArgs;
SoftArgs make_args(Context *c, DevSet &d, int n_group, int n_ptcl, int n_spj, bool accumulate);
int set_group_order(Context *c, DevSet &d, int n_group, const int *i_off_h, const int *j_off_h, const int *s_off_h);
bool is_pinned(const void *p);

}  // namespace p3t
