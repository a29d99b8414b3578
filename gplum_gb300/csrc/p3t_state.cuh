// Device-resident particle state of the P3T step (the FPGrav fields the hot
// path reads and writes, src/particle.h:404-500 of GPLUM), kept as
// structure-of-arrays in HBM.  Vectors are n x 3 doubles.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "p3t_common.cuh"

namespace p3t {

// FPGrav statics in the order of the 21-double parameter block
struct Params {
    double eps2, eps2_sun, m_sun, dt_tree, dt_min, eta, eta_0, eta_sun, eta_sun0, alpha2;
    double gamma, R_cut0, R_cut1, R_search0, R_search1, R_search2, R_search3, r_cut_min, r_cut_max, p_cut, dens;
    // derived (FPGrav::setGamma, src/particle.h:619-633)
    double g_1_inv, g_1_inv7, w_y, f1;
};

struct State {
    int n = 0, cap = 0;
    int64_t *id = nullptr, *id_cluster = nullptr;
    double *mass = nullptr, *r_planet = nullptr, *f = nullptr;
    double *pos = nullptr, *vel = nullptr, *acc = nullptr, *acc_d = nullptr, *jerk_d = nullptr, *acc_s = nullptr,
           *jerk_s = nullptr;
    double *phi = nullptr, *phi_d = nullptr, *phi_s = nullptr;
    double *r_out = nullptr, *r_out_inv = nullptr, *r_search = nullptr, *v_disp = nullptr;
    double *time = nullptr, *dt = nullptr, *acc0 = nullptr;
    int32_t *number = nullptr, *rank = nullptr, *id_max = nullptr, *id_min = nullptr, *n_cluster = nullptr;
    int32_t *dead = nullptr, *merged = nullptr;
    // scratch of the step
    double *acc_d_new = nullptr;     // correctForceLongInitial keeps the pre-pass acc_d
    int32_t *nbr = nullptr;          // [n x cand_cap] neighbour local indices
    int32_t *nbr_n = nullptr;        // neighbours per particle (== number)
    int32_t *label = nullptr;        // union-find parent / component root
};

}  // namespace p3t
