/* Host-side octree and interaction-list builder for the P3T soft force.
 *
 * Replaces the list-building half of FDPS TreeForForce as GPLUM drives it:
 *   tree_grav.initialize(n_tot, theta, n_leaf_limit, n_group_limit)      src/main_p3t.cpp:344-346
 *   tree_grav.calcForceAllAndWriteBack(EPEP, EPSP, ..., PS::MAKE_LIST)   src/main_p3t.cpp:351-355,583-587,672-676
 * with SEARCH_MODE_LONG_SYMMETRY (src/main_p3t.cpp:65-69) and quadrupole
 * superparticles (src/main_p3t.cpp:40-46).  The lists it returns are the
 * input of p3t_soft_dispatch_index (gplum_p3t.h).
 *
 * Layouts: pos is n x 3 doubles; the SPJ array is one FDPS SPJQuadrupole
 * record per tree node: {mass, pos.x, pos.y, pos.z, quad.xx, quad.yy,
 * quad.zz, quad.xy, quad.xz, quad.yz} (80 bytes).  Lists are CSR:
 * group g owns i_idx[i_off[g]..i_off[g+1]) (particle indices, Morton order),
 * j_idx[j_off[g]..j_off[g+1]) (particle indices) and
 * s_idx[s_off[g]..s_off[g+1]) (SPJ record indices).
 */
#ifndef P3T_TREE_H
#define P3T_TREE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct P3TTree P3TTree;

/* Builds the tree and all group lists.  r_search is GPLUM's per-particle
 * search radius (FPGrav::r_search); the 1.1 safety factor of
 * EPIGrav::getRSearch (src/particle.h:119-125) is applied inside. */
P3TTree *p3t_tree_build(int n, const double *pos, const double *mass, const double *r_search,
                        double theta, int n_leaf_limit, int n_group_limit);
/* 0 ok, 1 bad arguments, 2 list too long for 32-bit offsets */
int p3t_tree_status(const P3TTree *t);
/* counts[0..4] = groups, i entries, EPJ entries, SPJ entries, tree nodes */
void p3t_tree_counts(const P3TTree *t, long long *counts);
void p3t_tree_export(const P3TTree *t, int *i_off, int *i_idx, int *j_off, int *j_idx, int *s_off,
                     int *s_idx, double *spj);
void p3t_tree_free(P3TTree *t);

#ifdef __cplusplus
}
#endif
#endif
