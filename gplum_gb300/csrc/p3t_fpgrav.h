// GPLUM's FPGrav particle record as it lies in memory (EPIGrav, EPJGrav and
// FPGrav members in declaration order, src/particle.h:93-170,404-500, for the
// build with individual cutoffs, quadrupole moments and collisions): 344
// bytes, no padding.  It is the body record of the binary restart file
// snap_tmp.dat (src/particle.h:862-876) and the element of GPLUM's
// ParticleSystem<FPGrav>, so a host caller can hand its particle array to the
// library as is.
#pragma once
#include <cstddef>
#include <cstdint>

namespace p3t {

struct FPGravRecord {
    int32_t id_local, myrank;
    double pos[3];
    double r_out, r_search;
    int64_t id;
    double mass;
    double vel[3], acc_d[3];
    double acc[3], acc_s[3], jerk_d[3], jerk_s[3], acc_gd[3];
    double phi, phi_d, phi_s;
    double v_disp, r_out_inv;
    double time, dt, acc0;
    double r_planet, f;
    int32_t number, rank, id_max, id_min;  // NeighborInfo
    int64_t id_cluster;
    int32_t n_cluster;
    uint8_t in_domain, is_sent, is_dead, is_merged;
};
static_assert(sizeof(FPGravRecord) == 344, "FPGrav record");
static_assert(offsetof(FPGravRecord, pos) == 8 && offsetof(FPGravRecord, id) == 48 &&
                  offsetof(FPGravRecord, acc) == 112 && offsetof(FPGravRecord, phi) == 232 &&
                  offsetof(FPGravRecord, r_planet) == 296 && offsetof(FPGravRecord, number) == 312 &&
                  offsetof(FPGravRecord, id_cluster) == 328 && offsetof(FPGravRecord, in_domain) == 340,
              "FPGrav offsets");

}  // namespace p3t
