// FDPS-facing entry points of the soft force: the single-group functor
// calls and the multiwalk dispatch/retrieve pair (pointer and index forms).
// They stage FDPS's per-walk arrays into the same device layout the
// resident path uses and launch the same kernels.
#include <cstring>
#include <vector>

#include "../../include/gplum_p3t.h"
#include "p3t_capi_internal.cuh"
#include "p3t_common.cuh"
#include "p3t_soft.cuh"

using namespace p3t;

namespace {

DevSet g_fun;  // buffers of the single-group functor calls

int set_offsets(Context *c, DevSet &d, int n_group, const std::vector<int> &io, const std::vector<int> &jo,
                const std::vector<int> &so) {
    int r = 0;
    if ((r = d.i_off.reserve(n_group + 1)) || (r = d.j_off.reserve(n_group + 1)) || (r = d.s_off.reserve(n_group + 1)))
        return r;
    if ((r = h2d(c, d.i_off.p, io.data(), io.size() * sizeof(int)))) return r;
    if ((r = h2d(c, d.j_off.p, jo.data(), jo.size() * sizeof(int)))) return r;
    return h2d(c, d.s_off.p, so.data(), so.size() * sizeof(int));
}

// Functor call: one group, accumulate into the caller's ForceGrav records.
int functor_call(const void *epi, int ni, const void *epj, int nj, const void *spj, int ns, void *force) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    if (ni <= 0) return 0;
    if (!epi || !force || nj < 0 || ns < 0 || (nj > 0 && !epj) || (ns > 0 && !spj)) return ST_BAD_INDEX;
    DevSet &d = g_fun;
    int r = 0;
    if ((r = d.epi_stage.reserve(ni)) || (r = d.iptcl.reserve(ni)) || (r = d.i_r_out.reserve(ni)) ||
        (r = d.i_r_search.reserve(ni)) || (r = d.epj_stage.reserve(nj)) || (r = d.ptcl.reserve(nj)) ||
        (r = d.mass.reserve(nj)) || (r = d.r_out.reserve(nj)) || (r = d.r_search.reserve(nj)) ||
        (r = d.spj.reserve(ns)) || (r = d.i_idx.reserve(ni)) || (r = d.j_idx.reserve(nj)) ||
        (r = d.s_idx.reserve(ns)) || (r = d.force.reserve(ni)) || (r = d.acc64.reserve(ni)))
        return r;
    if ((r = h2d(c, d.epi_stage.p, epi, (size_t)ni * sizeof(EPIRec)))) return r;
    if (nj && (r = h2d(c, d.epj_stage.p, epj, (size_t)nj * sizeof(EPJRec)))) return r;
    if (ns && (r = h2d(c, d.spj.p, spj, (size_t)ns * sizeof(SPJRec)))) return r;
    if ((r = h2d(c, d.force.p, force, (size_t)ni * sizeof(ForceRec)))) return r;
    std::vector<int> io = {0, ni}, jo = {0, nj}, so = {0, ns};
    if ((r = set_offsets(c, d, 1, io, jo, so))) return r;
    if ((r = cuda_status(launch_pack_epi((const EPIRec *)d.epi_stage.p, ni, d.iptcl.p, d.i_r_out.p, d.i_r_search.p,
                                         c->stream))))
        return r;
    if ((r = cuda_status(launch_pack_epj(d.epj_stage.p, nj, d.ptcl.p, d.mass.p, d.r_out.p, d.r_search.p, c->stream))))
        return r;
    if ((r = cuda_status(launch_iota(d.i_idx.p, ni, 0, c->stream))) ||
        (r = cuda_status(launch_iota(d.j_idx.p, nj, 0, c->stream))) ||
        (r = cuda_status(launch_iota(d.s_idx.p, ns, 0, c->stream))))
        return r;
    d.order_valid = false;
    SoftArgs A = make_args(c, d, 1, nj, ns, true);
    A.iptcl = d.iptcl.p; A.i_r_out = d.i_r_out.p; A.i_r_search = d.i_r_search.p; A.n_iptcl = ni;
    A.cand = nullptr;
    if (c->precision == 1) {
        // FP64 form accumulates in double: seed it from the caller's records
        std::vector<D4> seed(ni);
        const ForceRec *f = (const ForceRec *)force;
        for (int k = 0; k < ni; k++) seed[k] = D4c(f[k].acc[0], f[k].acc[1], f[k].acc[2], f[k].phi);
        if ((r = h2d(c, d.acc64.p, seed.data(), ni * sizeof(D4)))) return r;
    }
    if ((r = cuda_status(launch_soft(A, c->precision, false, c->stream)))) return r;
    if ((r = cuda_status(cudaMemcpyAsync(force, d.force.p, (size_t)ni * sizeof(ForceRec), cudaMemcpyDeviceToHost,
                                         c->stream))))
        return r;
    if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    return read_status(c);
}

WalkSlot *slot_for(Context *c, int tag) {
    if (tag < 0) return nullptr;
    WalkSlot &w = c->walk[tag % MAX_TAGS];
    if (!w.done && cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    return &w;
}

// Per-walk counts of a dispatch: non-negative, with a record pointer where a
// count is positive, and totals that fit the int offsets.
int check_walks(int n_walk, const int *cnt, const void *const *ptr) {
    if (n_walk < 0 || (n_walk > 0 && !cnt)) return ST_BAD_INDEX;
    long long tot = 0;
    for (int k = 0; k < n_walk; k++) {
        if (cnt[k] < 0 || (cnt[k] > 0 && (!ptr || !ptr[k]))) return ST_BAD_INDEX;
        tot += cnt[k];
    }
    return tot > 2147483647LL ? ST_BAD_INDEX : 0;
}

// Common tail of both dispatch forms: kernel, download, event.
int launch_walks(Context *c, WalkSlot &w, int n_walk, int n_i, const SoftPtcl *jptcl, const double *jmass,
                 const double *jro, const double *jrs, int n_j, const SPJRec *spj, int n_s) {
    DevSet &d = w.d;
    int r = 0;
    if ((r = d.force.reserve(n_i)) || (r = d.acc64.reserve(n_i))) return r;
    d.order_valid = false;
    SoftArgs A = make_args(c, d, n_walk, n_j, n_s, false);
    A.ptcl = jptcl; A.mass = jmass; A.r_out = jro; A.r_search = jrs; A.n_ptcl = n_j;
    A.spj = spj; A.n_spj = n_s;
    A.iptcl = d.iptcl.p; A.i_r_out = d.i_r_out.p; A.i_r_search = d.i_r_search.p; A.n_iptcl = n_i;
    A.cand = nullptr;
    if ((r = cuda_status(launch_soft(A, c->precision, false, c->stream)))) return r;
    if ((r = grow_host(&w.h_out, &w.h_out_cap, (size_t)n_i * sizeof(ForceRec)))) return r;
    if ((r = cuda_status(cudaMemcpyAsync(w.h_out, d.force.p, (size_t)n_i * sizeof(ForceRec), cudaMemcpyDeviceToHost,
                                         c->stream))))
        return r;
    if ((r = cuda_status(cudaEventRecord(w.done, c->stream)))) return r;
    w.n_i = n_i;
    w.busy = true;
    return 0;
}

// Gathers the walks' EPI records into slot staging and onto the device.
int stage_epi(Context *c, WalkSlot &w, int n_walk, const void **epi, const int *n_epi, int &n_i) {
    n_i = 0;
    for (int k = 0; k < n_walk; k++) n_i += n_epi[k];
    DevSet &d = w.d;
    int r = 0;
    if ((r = d.epi_stage.reserve(n_i)) || (r = d.iptcl.reserve(n_i)) || (r = d.i_r_out.reserve(n_i)) ||
        (r = d.i_r_search.reserve(n_i)) || (r = d.i_idx.reserve(n_i)))
        return r;
    if ((r = grow_host(&w.h_in, &w.h_in_cap, (size_t)n_i * sizeof(EPIRec)))) return r;
    char *h = (char *)w.h_in;
    for (int k = 0; k < n_walk; k++) {
        std::memcpy(h, epi[k], (size_t)n_epi[k] * sizeof(EPIRec));
        h += (size_t)n_epi[k] * sizeof(EPIRec);
    }
    if ((r = cuda_status(cudaMemcpyAsync(d.epi_stage.p, w.h_in, (size_t)n_i * sizeof(EPIRec), cudaMemcpyHostToDevice,
                                         c->stream))))
        return r;
    if ((r = cuda_status(launch_pack_epi(d.epi_stage.p, n_i, d.iptcl.p, d.i_r_out.p, d.i_r_search.p, c->stream))))
        return r;
    return cuda_status(launch_iota(d.i_idx.p, n_i, 0, c->stream));
}

}  // namespace

extern "C" {

int p3t_epep(const void *epi, int ni, const void *epj, int nj, void *force) {
    return functor_call(epi, ni, epj, nj, nullptr, 0, force);
}

int p3t_epsp(const void *epi, int ni, const void *spj, int nj, void *force) {
    return functor_call(epi, ni, nullptr, 0, spj, nj, force);
}

int p3t_soft_dispatch(int tag, int n_walk, const void **epi, const int *n_epi, const void **epj, const int *n_epj,
                      const void **spj, const int *n_spj) {
    int e = 0;
    if ((e = check_walks(n_walk, n_epi, epi)) || (e = check_walks(n_walk, n_epj, epj)) ||
        (e = check_walks(n_walk, n_spj, spj)))
        return e;
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    WalkSlot *ws = slot_for(c, tag);
    if (!ws || n_walk < 0) return ST_BAD_INDEX;
    WalkSlot &w = *ws;
    if (w.busy) cudaEventSynchronize(w.done);  // a retrieve was skipped: the slot is reused in order
    if (w.busy) w.busy = false;
    int r = 0, n_i = 0;
    // wait for any earlier use of this slot's pinned buffers
    if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    if ((r = stage_epi(c, w, n_walk, epi, n_epi, n_i))) return r;
    int n_j = 0, n_s = 0;
    std::vector<int> io(n_walk + 1), jo(n_walk + 1), so(n_walk + 1);
    io[0] = jo[0] = so[0] = 0;
    for (int k = 0; k < n_walk; k++) {
        io[k + 1] = io[k] + n_epi[k];
        jo[k + 1] = jo[k] + n_epj[k];
        so[k + 1] = so[k] + n_spj[k];
    }
    n_j = jo[n_walk];
    n_s = so[n_walk];
    DevSet &d = w.d;
    if ((r = d.epj_stage.reserve(n_j)) || (r = d.ptcl.reserve(n_j)) || (r = d.mass.reserve(n_j)) ||
        (r = d.r_out.reserve(n_j)) || (r = d.r_search.reserve(n_j)) || (r = d.spj.reserve(n_s)) ||
        (r = d.j_idx.reserve(n_j)) || (r = d.s_idx.reserve(n_s)))
        return r;
    // EPJ and SPJ records of every walk, concatenated (pageable sources are
    // staged by h2d)
    {
        std::vector<char> cat((size_t)n_j * sizeof(EPJRec) + (size_t)n_s * sizeof(SPJRec));
        char *h = cat.data();
        for (int k = 0; k < n_walk; k++) {
            std::memcpy(h, epj[k], (size_t)n_epj[k] * sizeof(EPJRec));
            h += (size_t)n_epj[k] * sizeof(EPJRec);
        }
        char *hs = h;
        for (int k = 0; k < n_walk; k++) {
            std::memcpy(h, spj[k], (size_t)n_spj[k] * sizeof(SPJRec));
            h += (size_t)n_spj[k] * sizeof(SPJRec);
        }
        if (n_j && (r = h2d(c, d.epj_stage.p, cat.data(), (size_t)n_j * sizeof(EPJRec)))) return r;
        if (n_s && (r = h2d(c, d.spj.p, hs, (size_t)n_s * sizeof(SPJRec)))) return r;
    }
    if ((r = set_offsets(c, d, n_walk, io, jo, so))) return r;
    if ((r = cuda_status(launch_pack_epj(d.epj_stage.p, n_j, d.ptcl.p, d.mass.p, d.r_out.p, d.r_search.p, c->stream))) ||
        (r = cuda_status(launch_iota(d.j_idx.p, n_j, 0, c->stream))) ||
        (r = cuda_status(launch_iota(d.s_idx.p, n_s, 0, c->stream))))
        return r;
    return launch_walks(c, w, n_walk, n_i, d.ptcl.p, d.mass.p, d.r_out.p, d.r_search.p, n_j, d.spj.p, n_s);
}

int p3t_soft_dispatch_index(int tag, int n_walk, const void **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const int **id_spj, const int *n_spj, const void *epj, int n_epj_tot,
                            const void *spj, int n_spj_tot, int send_flag) {
    int e = 0;
    if ((e = check_walks(n_walk, n_epi, epi)) || (e = check_walks(n_walk, n_epj, (const void *const *)id_epj)) ||
        (e = check_walks(n_walk, n_spj, (const void *const *)id_spj)))
        return e;
    if (send_flag && (n_epj_tot < 0 || n_spj_tot < 0 || (n_epj_tot > 0 && !epj) || (n_spj_tot > 0 && !spj)))
        return ST_BAD_INDEX;
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    WalkSlot *ws = slot_for(c, tag);
    if (!ws || n_walk < 0) return ST_BAD_INDEX;
    WalkSlot &w = *ws;
    int r = 0;
    if ((r = cuda_status(cudaStreamSynchronize(c->stream)))) return r;
    w.busy = false;
    DevSet &x = c->idx;
    if (send_flag) {
        if ((r = x.epj_stage.reserve(n_epj_tot)) || (r = x.ptcl.reserve(n_epj_tot)) || (r = x.mass.reserve(n_epj_tot)) ||
            (r = x.r_out.reserve(n_epj_tot)) || (r = x.r_search.reserve(n_epj_tot)) || (r = x.spj.reserve(n_spj_tot)))
            return r;
        if (n_epj_tot && (r = h2d(c, x.epj_stage.p, epj, (size_t)n_epj_tot * sizeof(EPJRec)))) return r;
        if (n_spj_tot && (r = h2d(c, x.spj.p, spj, (size_t)n_spj_tot * sizeof(SPJRec)))) return r;
        if ((r = cuda_status(launch_pack_epj(x.epj_stage.p, n_epj_tot, x.ptcl.p, x.mass.p, x.r_out.p, x.r_search.p,
                                             c->stream))))
            return r;
        c->idx_nj = n_epj_tot;
        c->idx_ns = n_spj_tot;
    }
    int n_i = 0;
    if ((r = stage_epi(c, w, n_walk, epi, n_epi, n_i))) return r;
    std::vector<int> io(n_walk + 1), jo(n_walk + 1), so(n_walk + 1);
    io[0] = jo[0] = so[0] = 0;
    for (int k = 0; k < n_walk; k++) {
        io[k + 1] = io[k] + n_epi[k];
        jo[k + 1] = jo[k] + n_epj[k];
        so[k + 1] = so[k] + n_spj[k];
    }
    DevSet &d = w.d;
    if ((r = d.j_idx.reserve(jo[n_walk])) || (r = d.s_idx.reserve(so[n_walk]))) return r;
    {
        std::vector<int> jl(jo[n_walk]), sl(so[n_walk]);
        for (int k = 0; k < n_walk; k++) {
            if (n_epj[k]) std::memcpy(jl.data() + jo[k], id_epj[k], n_epj[k] * sizeof(int));
            if (n_spj[k]) std::memcpy(sl.data() + so[k], id_spj[k], n_spj[k] * sizeof(int));
        }
        if (!jl.empty() && (r = h2d(c, d.j_idx.p, jl.data(), jl.size() * sizeof(int)))) return r;
        if (!sl.empty() && (r = h2d(c, d.s_idx.p, sl.data(), sl.size() * sizeof(int)))) return r;
    }
    if ((r = set_offsets(c, d, n_walk, io, jo, so))) return r;
    return launch_walks(c, w, n_walk, n_i, x.ptcl.p, x.mass.p, x.r_out.p, x.r_search.p, c->idx_nj, x.spj.p,
                        c->idx_ns);
}

int p3t_soft_retrieve(int tag, int n_walk, const int *n_epi, void **force) {
    Context *c = ctx_get(0);
    if (!c) return -(int)cudaErrorNoDevice;
    WalkSlot *ws = slot_for(c, tag);
    if (!ws || !ws->busy) return ST_BAD_INDEX;
    WalkSlot &w = *ws;
    int r = cuda_status(cudaEventSynchronize(w.done));
    w.busy = false;
    if (r) return r;
    const ForceRec *h = (const ForceRec *)w.h_out;
    int off = 0;
    for (int k = 0; k < n_walk; k++) {
        if (off + n_epi[k] > w.n_i) return ST_BAD_INDEX;
        std::memcpy(force[k], h + off, (size_t)n_epi[k] * sizeof(ForceRec));
        off += n_epi[k];
    }
    return read_status(c);
}

}  // extern "C"
