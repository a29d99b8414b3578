// Fixed-radius neighbour query shared by the two CPU checkers.  TEST
// INFRASTRUCTURE ONLY.
//
// Stand-in for FDPS's TreeForForce::getNeighborListOneParticle, which GPLUM
// calls from correctForceLong[Initial] (src/gravity_soft.h:297,439) with the
// symmetric LONG_SYMMETRY rule: every particle j with
// |x_j - x_i|^2 < max(rq_i, rq_j)^2, rq the particle's search radius.  FDPS
// is absent from the reference tree, so both checkers use this query and
// return its candidates in ascending particle index (the order in which the
// device pass folds its terms).
//
// Linear in N: a uniform grid of cell size h over every particle whose rq is
// at most h, stored as particle indices sorted by a 63-bit cell key (no cap on
// the number of cells); a query scans, per (z, y) row of its cell box, one
// contiguous key range found by binary search.  h is the largest rq among the
// "normal" particles; the few with a much larger radius (rq above 4 x the
// median, at most 64 of them, e.g. embryos among planetesimals) are kept in
// a short list every query tests directly, and their own queries scan a wider
// cell box.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

struct NgbGrid {
    double h = 1., x0[3] = {0., 0., 0.};
    int64_t nc[3] = {1, 1, 1};
    std::vector<uint64_t> key;  // cell keys of the gridded particles, ascending
    std::vector<int> idx;       // their particle indices, in key order
    std::vector<int> wide;      // particles outside the grid (large rq), ascending
    std::vector<double> px, py, pz, rq;

    static constexpr int BITS = 21;
    uint64_t key_of(int64_t cx, int64_t cy, int64_t cz) const {
        return ((uint64_t)cz << (2 * BITS)) | ((uint64_t)cy << BITS) | (uint64_t)cx;
    }
    int64_t cell(double x, int d) const {
        const double c = std::floor((x - x0[d]) / h);
        if (!(c > 0.)) return 0;
        return std::min<int64_t>(nc[d] - 1, (int64_t)c);
    }

    // n particles, positions (x[i], y[i], z[i]) and search radii r[i]
    template <class Pos, class Rad>
    void build(int n, Pos pos, Rad rad) {
        px.resize(n); py.resize(n); pz.resize(n); rq.resize(n);
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = 0; i < n; i++) {
            pos(i, px[i], py[i], pz[i]);
            rq[i] = rad(i);
            const double x[3] = {px[i], py[i], pz[i]};
            for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], x[d]); hi[d] = std::max(hi[d], x[d]); }
        }
        wide.clear();
        key.clear();
        idx.clear();
        if (n == 0) return;
        // threshold between gridded and wide particles
        std::vector<double> s(rq);
        std::nth_element(s.begin(), s.begin() + n / 2, s.end());
        double thr = 4. * s[n / 2];
        if (n > 64) {
            std::nth_element(s.begin(), s.begin() + (n - 65), s.end());
            thr = std::max(thr, s[n - 65]);  // at most 64 wide particles
        }
        h = 0.;
        for (int i = 0; i < n; i++)
            if (rq[i] <= thr) h = std::max(h, rq[i]);
            else wide.push_back(i);
        h = std::max(h, 1e-12);
        for (int d = 0; d < 3; d++) {
            x0[d] = lo[d];
            // keep every coordinate inside the key's BITS bits
            h = std::max(h, (hi[d] - lo[d]) / (double)((1 << BITS) - 2));
        }
        for (int d = 0; d < 3; d++) nc[d] = (int64_t)std::floor((hi[d] - lo[d]) / h) + 1;
        std::vector<std::pair<uint64_t, int>> kv;
        kv.reserve(n);
        for (int i = 0; i < n; i++)
            if (rq[i] <= thr) kv.push_back({key_of(cell(px[i], 0), cell(py[i], 1), cell(pz[i], 2)), i});
        std::sort(kv.begin(), kv.end());
        key.resize(kv.size());
        idx.resize(kv.size());
        for (size_t k = 0; k < kv.size(); k++) {
            key[k] = kv[k].first;
            idx[k] = kv[k].second;
        }
    }

    // indices j (i itself included) for which accept(j) holds, among every
    // particle that can lie within max(rq_i, rq_j) of i; ascending order
    template <class Accept>
    void query(int i, std::vector<int> &out, Accept accept) const {
        out.clear();
        // gridded particles have rq_j <= h; pad the box for rounding
        const double R = std::max(rq[i], h) * (1. + 1e-9);
        const int64_t cx0 = cell(px[i] - R, 0), cx1 = cell(px[i] + R, 0);
        const int64_t cy0 = cell(py[i] - R, 1), cy1 = cell(py[i] + R, 1);
        const int64_t cz0 = cell(pz[i] - R, 2), cz1 = cell(pz[i] + R, 2);
        for (int64_t cz = cz0; cz <= cz1; cz++)
            for (int64_t cy = cy0; cy <= cy1; cy++) {
                const uint64_t k1 = key_of(cx1, cy, cz);
                size_t k = std::lower_bound(key.begin(), key.end(), key_of(cx0, cy, cz)) - key.begin();
                for (; k < key.size() && key[k] <= k1; k++)
                    if (accept(idx[k])) out.push_back(idx[k]);
            }
        for (int j : wide)
            if (accept(j)) out.push_back(j);
        std::sort(out.begin(), out.end());
    }
};
