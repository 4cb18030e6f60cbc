/*
 * fest_oracle.h - CPU restatement (FP64, plain C) of FEST-3D's explicit
 * residual-and-update path.  TEST INFRASTRUCTURE ONLY: the parity tests,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the
 * checker.  Nothing in the product links or calls it.
 *
 * Every routine follows one reference procedure loop by loop, with the
 * reference's expression order (the parity build uses -ffp-contract=off so
 * no FMA contraction changes the rounding).  The block object plays the role
 * of the reference's module-level arrays (face_interpolant, gradients,
 * viscosity, global_sst, wall_dist, update, scheme, time).
 */
#ifndef FEST_ORACLE_H
#define FEST_ORACLE_H
#include "../include/fest_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fo_block fo_block;

/* array ids for fo_ptr / fo_size */
enum {
  FO_QP = 0, FO_TEMP, FO_NODES, FO_CELLS, FO_IFACES, FO_JFACES, FO_KFACES,
  FO_XL, FO_XR, FO_YL, FO_YR, FO_ZL, FO_ZR, FO_PDIF,
  FO_F, FO_G, FO_H, FO_RES,
  FO_GX, FO_GY, FO_GZ, FO_MU, FO_MUT, FO_F1, FO_DIST,
  FO_DT, FO_USTORE, FO_RSTORE,
  FO_NARRAYS
};

fo_block *fo_create(const fest_extent *d, const fest_flow *flow,
                    const fest_scheme *scheme, const fest_bc *bc);
void fo_destroy(fo_block *b);
double *fo_ptr(fo_block *b, int id);
long fo_size(const fo_block *b, int id);
int fo_n_grad(const fo_block *b);
/* OpenMP threads used by the loops (1 = serial); returns previous value */
int fo_set_threads(int n);

/* geometry: ghost_grid (grid.f90:137) + setup_geometry (geometry.f90:548) */
void fo_setup_geometry(fo_block *b);
/* wall distance (wall_dist.f90:84-131) */
void fo_find_wall_dist(fo_block *b, const double *wall_xyz, int n_wall);

/* boundary conditions */
void fo_apply_interface(fo_block **blocks, int nblocks);          /* interface1.f90:496 */
int  fo_populate_ghost_primitive(fo_block *b, int current_iter);  /* bc_primitive.f90:55 */

/* residual pieces */
void fo_compute_temperature(fo_block *b);                         /* update.f90:170 */
int  fo_compute_face_interpolant(fo_block *b);                    /* face_interpolant.f90:79 */
void fo_reconstruct_boundary_state(fo_block *b);                  /* boundary_state_reconstruction.f90:28 */
int  fo_compute_fluxes(fo_block *b);                              /* scheme.f90:68 */
int  fo_evaluate_all_gradients(fo_block *b);                      /* gradients.f90:276 */
int  fo_calculate_viscosity(fo_block *b);                         /* viscosity.f90:52 */
int  fo_compute_viscous_fluxes(fo_block *b);                      /* viscous.f90:55 */
void fo_compute_residue(fo_block *b);                             /* scheme.f90:111 */
void fo_add_source_term_residue(fo_block *b);                     /* source.f90:94 */
void fo_compute_time_step(fo_block *b, double CFL);               /* time.f90:291 */
/* update_with(...,'conservative',TF,SF,TU,Rn,un) (update.f90:228-491);
 * use_store != 0 passes R_store/U_store as Rn/un */
int  fo_update_with(fo_block *b, double TF, double SF, int TU, int use_store);

/* drivers over a set of blocks (the MPI ranks of the reference) */
int fo_get_total_conservative_residue(fo_block **blocks, int nb, int current_iter);
int fo_get_next_solution(fo_block **blocks, int nb, int current_iter, double CFL);
/* one iteration of the reference's implicit integrator (update.f90:215-218,
 * LU-SGS of lusgs.f90:186-1196), laminar and k-omega SST blocks
 * (FEST_ERR_ARG otherwise): kept to replay the reference's own implicit
 * test runs */
int fo_lusgs_next_solution(fo_block **blocks, int nb, int current_iter, double CFL);
int fo_plusgs_next_solution(fo_block **blocks, int nb, int current_iter, double CFL);
/* res_abs[0..n_var] (resnorm.f90:171-225) */
void fo_find_resnorm(fo_block **blocks, int nb, double *res_abs);

#ifdef __cplusplus
}
#endif
#endif
