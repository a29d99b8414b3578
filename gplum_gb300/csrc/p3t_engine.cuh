// Device-resident P3T step engine (one per process, bound to the library's
// context and stream).
#pragma once
#include "p3t_capi_internal.cuh"
#include "p3t_state.cuh"

namespace p3t {

struct Engine {
    Context *c = nullptr;
    State S;
    int cand_cap_alloc = 0;
    int n_clusters = 0, n_members = 0;
    DevBuf<int32_t> counters, head, flag, cidx, cl_of, cl_cnt, cl_off, cl_fill, members_tmp, members, keep, kpos,
        scan_tmp, tflag, tpos;
    DevBuf<int64_t> cmin;
    DevBuf<double> epart, et;
    DevBuf<int> icnt;
    // correction pair list: per body its count and first slot; per pair (i, j) and terms
    DevBuf<int32_t> pair_n, pair_base, pair_i, pair_j;
    DevBuf<struct PairTerms> pair_terms;
    DevBuf<char> compact_tmp;
    // KOMINAMI fragments appended by the last hard part: particles
    // [frag_lo, frag_hi) with their clusters in frag_cl
    DevBuf<int32_t> frag_cl;
    int frag_lo = 0, frag_hi = 0;
    long long id_next = 0;  // next particle id (src/main_p3t.cpp:233,295-305)

    int ensure(int n);
    int grow(int n);  // capacity for n bodies, keeping the state
    Params params() const;
    int load(int n, const long long *id, const double *mass, const double *r_planet, const double *f,
             const double *pos, const double *vel);
    int pack_soft();
    int correct(int initial);
    int cluster();
    int make_list();
    int kick();
    int energy(double *out5);
    int cutoff_radii();
    int merge(double *edisp);
    int remove(double r_max, double r_min, double *edisp, int *n_removed);
    int compact(int n, int nk);
    int scan(const int32_t *in, int32_t *out, int n, int32_t *total);
};

extern Engine g_eng;

// Soft pass with candidate emission over the engine's resident state and
// lists.  When a particle had more screen hits than the candidate table's
// width, the width grows to the next power of two above the largest count
// and the pass runs again (a few embryos among planetesimals have hundreds
// of candidates; the table starts at 64).
int soft_run_state();

// Device priorities (higher first) of the current clusters from the learned
// cost model, with the scale that maps them to the order's bins, or nullptr
// when the size order applies (sched.cu).
const float *sched_priority(Context *c, int nc, float *pmin, float *pscale);

}  // namespace p3t
