/*
 * fest_gpu.h - C ABI of the GB300 (sm_103a) explicit residual-and-update path
 * of the FEST-3D structured finite-volume solver.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns an int status (FEST_OK == 0).  Host arrays use exactly the
 * Fortran column-major shapes of the reference, including lower bounds, so
 * a Fortran caller passes c_loc() of its own arrays unchanged:
 *
 *   qp      (-2:imx+2,-2:jmx+2,-2:kmx+2,1:n_var)         double
 *   Temp, mu, mu_t, sst_F1, dist  (-2:imx+2,-2:jmx+2,-2:kmx+2)
 *   cells   (-2:imx+2,-2:jmx+2,-2:kmx+2) of {volume,cx,cy,cz}   (AoS, 32 B)
 *   Ifaces  (-2:imx+3,-2:jmx+2,-2:kmx+2) of {A,nx,ny,nz}        (AoS, 32 B)
 *   Jfaces  (-2:imx+2,-2:jmx+3,-2:kmx+2) of {A,nx,ny,nz}
 *   Kfaces  (-2:imx+2,-2:jmx+2,-2:kmx+3) of {A,nx,ny,nz}
 *   nodes   (-2:imx+3,-2:jmx+3,-2:kmx+3) of {x,y,z}
 *   x_qp_left/right (0:imx+1,1:jmx-1,1:kmx-1,1:n_var), y_* and z_* alike
 *   F (1:imx,1:jmx-1,1:kmx-1,n_var), G (1:imx-1,1:jmx,1:kmx-1,n_var),
 *   H (1:imx-1,1:jmx-1,1:kmx,n_var), residue (1:imx-1,1:jmx-1,1:kmx-1,n_var)
 *   gradqp_x/y/z (0:imx,0:jmx,0:kmx,1:n_grad)   n_grad = 4 laminar, 6 SST
 *   delta_t (1:imx-1,1:jmx-1,1:kmx-1)
 *
 * imx, jmx, kmx are NODE counts (vartypes.f90:21-26): a block has
 * (imx-1)(jmx-1)(kmx-1) interior cells and 3 ghost layers per side.
 *
 * Ownership: the caller owns host arrays; a handle owns device copies of
 * the state, metrics and every module-level array of the reference
 * (face states, gradients, viscosities, fluxes, residue, time step).
 * No host pointer is retained past a call.  A handle is synchronous on its
 * own CUDA stream and must not be used from two threads at once; distinct
 * handles are independent.
 *
 * Module entry points take nullable host pointers: a non-NULL input is
 * uploaded before the kernel runs, a non-NULL output is downloaded after
 * it; NULL means "use / keep the device-resident copy in the handle".
 */
#ifndef FEST_GPU_H
#define FEST_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference aborts through Fatal_error, error.h:1) */
#define FEST_OK                  0
#define FEST_ERR_ARG             1  /* bad argument / unsupported option       */
#define FEST_ERR_CUDA            2  /* a CUDA runtime call failed              */
#define FEST_ERR_NAN             3  /* NaN in a flux/gradient/state (ausm.f90:195) */
#define FEST_ERR_NEGATIVE_STATE  4  /* rho<0 or p<0 after update (update.f90:448) */
#define FEST_ERR_TIMEOUT         5  /* a bounded device wait gave up           */
#define FEST_ERR_NOMEM           6  /* device allocation failed                */
#define FEST_ERR_NO_DEVICE       7  /* no CUDA device visible                  */
#define FEST_ERR_SCRATCH         8  /* request exceeds a fixed scratch area    */

/* ---- scheme selectors (schemetype, vartypes.f90:197-232) ---------------- */
enum { FEST_FLUX_AUSM = 0, FEST_FLUX_AUSMP = 1, FEST_FLUX_AUSMUP = 2,
       FEST_FLUX_SLAU = 3, FEST_FLUX_LDFSS0 = 4, FEST_FLUX_VAN_LEER = 5 };
enum { FEST_INTERP_NONE = 0, FEST_INTERP_MUSCL = 1, FEST_INTERP_PPM = 2,
       FEST_INTERP_WENO = 3, FEST_INTERP_WENO_NM = 4 };
/* FEST_TIME_IMPLICIT: the reference's "implicit" (update.f90:215-218), one
 * residual and time step, then the LU-SGS update of lusgs.f90:134-1196
 * (laminar and k-omega SST, FP64, module path; batches of blocks too).
 * FEST_TIME_PLUSGS: its "plusgs" (update.f90:219-222), the same with the
 * low-Mach preconditioned update of plusgs.f90:139-1431. */
enum { FEST_TIME_NONE = 0, FEST_TIME_RK2 = 1, FEST_TIME_RK4 = 2,
       FEST_TIME_TVDRK2 = 3, FEST_TIME_TVDRK3 = 4, FEST_TIME_IMPLICIT = 5,
       FEST_TIME_PLUSGS = 6 };
/* FEST_TURB_SA: the Spalart-Allmaras model ('sa', n_var = 6, the sixth
 * variable tv; viscosity.f90:149-213, viscous.f90:570-656,
 * source.f90:845-983, update.f90:405-420,474-475), FP64 module path
 * (fest_get_next_solution, fest_step with the explicit integrators) */
/* FEST_TURB_KKL: the k-kL model ('kkl', n_var = 7: k and kL;
 * viscosity.f90:469-533, viscous.f90:450-567, source.f90:607-832,
 * update.f90:399-404), FP64 module path as SA */
enum { FEST_TURB_NONE = 0, FEST_TURB_SST = 1, FEST_TURB_SST2003 = 2, FEST_TURB_SA = 3, FEST_TURB_KKL = 4 };
enum { FEST_MU_CONSTANT = 0, FEST_MU_SUTHERLAND = 1 };
/* transition model (schemetype%transition): FEST_TRANSITION_BC, the
 * algebraic 'bc' intermittency on the production of SA ('saBC',
 * source.f90:985-1194) or k-omega SST (source.f90:467-604); FP64 module
 * path, explicit integrators (and LU-SGS/PLU-SGS for SST-BC).
 * FEST_TRANSITION_LCTM2015: Menter's 2015 one-equation intermittency model
 * on k-omega SST (n_var = 8, the eighth variable the intermittency;
 * source.f90:273-465, viscous.f90:658-749, viscosity.f90:265-280, CC.f90,
 * lusgs.f90:2263-2700, plusgs.f90:2130-2624), FP64 module path, explicit
 * integrators, LU-SGS and PLU-SGS */
enum { FEST_TRANSITION_NONE = 0, FEST_TRANSITION_BC = 1, FEST_TRANSITION_LCTM2015 = 2 };
/* MUSCL limiter: the reference hard-codes Koren's alpha family
 * (muscl.f90:151,176); van Albada (muscl.f90:178, commented out there) is an
 * extension selectable here. */
enum { FEST_LIMITER_KOREN = 0, FEST_LIMITER_VAN_ALBADA = 1 };
/* arithmetic of the hot path */
enum { FEST_FP64 = 0, FEST_MIXED = 1 };

/* boundary condition ids (bc_primitive.f90:160-206, bc.f90:27-32) */
enum { FEST_BC_SUPERSONIC_INLET = -1, FEST_BC_SUPERSONIC_OUTLET = -2,
       FEST_BC_SUBSONIC_INLET = -3, FEST_BC_SUBSONIC_OUTLET = -4,
       FEST_BC_WALL = -5, FEST_BC_SLIP_WALL = -6, FEST_BC_POLE = -7,
       FEST_BC_FAR_FIELD = -8, FEST_BC_PERIODIC_SINGLE = -9,
       FEST_BC_INTERFACE = -10, FEST_BC_TOTAL_PRESSURE = -11 };

typedef struct {            /* extent, vartypes.f90:21-26 */
  int imx, jmx, kmx, n_var;
} fest_extent;

typedef struct {            /* flowtype, vartypes.f90:235-286 */
  double density_inf, x_speed_inf, y_speed_inf, z_speed_inf, pressure_inf;
  double tk_inf, tw_inf;
  double vel_mag, MInf;     /* derived by init_infinity_values, state.f90:87-88 */
  double gm, R_gas, mu_ref, T_ref, Sutherland_temp, Pr, tPr;
  int mu_variation;         /* FEST_MU_* */
  int reserved;
  double tv_inf;            /* Spalart-Allmaras free-stream tv (state.f90:106-109) */
  double tkl_inf;           /* k-kL free-stream kL (state.f90:101-103) */
  double tu_inf;            /* free-stream turbulence intensity, percent (flow%tu_inf) */
  double tgm_inf;           /* LCTM2015 free-stream intermittency (state.f90:261-265) */
} fest_flow;

typedef struct {            /* schemetype, vartypes.f90:197-232 */
  int scheme_name;          /* FEST_FLUX_* */
  int interpolant;          /* FEST_INTERP_* */
  int time_stepping_method; /* 'l' (local) or 'g' (global) */
  int time_step_accuracy;   /* FEST_TIME_* */
  double global_time_step;  /* used by 'g' when > 0 (time.f90:275) */
  int ilimiter_switch, jlimiter_switch, klimiter_switch;
  int itlimiter_switch, jtlimiter_switch, ktlimiter_switch;
  int iPB_switch, jPB_switch, kPB_switch;
  int turbulence;           /* FEST_TURB_* */
  int accur;                /* higher-order ghost switch (bc.f90:48-50) */
  int limiter;              /* FEST_LIMITER_* */
  int transition;           /* FEST_TRANSITION_* */
} fest_scheme;

typedef struct {            /* boundarytype, vartypes.f90:289-367 */
  int id[6];                /* imin,imax,jmin,jmax,kmin,kmax */
  /* interface partner of a face whose id is -10 (or >= 0): the ghost layer
   * l of this face receives interior layer l of face partner_face[f] of
   * block partner_block[f] (interface1.f90:96-700), at the tangential
   * position partner_orient[f] maps it to.  A handle stepped on its own
   * pairs only with itself (partner_block == block_id); pairs between
   * blocks are exchanged inside a batch.  A face paired with itself
   * reproduces what MPI_SENDRECV to the own rank does in the reference (a
   * mirror). */
  int partner_block[6];
  int partner_face[6];
  double fixed_density[6], fixed_pressure[6];
  double fixed_x_speed[6], fixed_y_speed[6], fixed_z_speed[6];
  double fixed_tk[6], fixed_tw[6];
  double fixed_wall_temperature[6];
  double fixed_Tpressure[6], fixed_Ttemperature[6];
  /* this block's number in its case (the reference's process_id): a face
   * whose partner_block equals it pairs with this same block; any other
   * partner_block names another handle of a batch (fest_batch_create),
   * matched by that handle's block_id.  Default 0. */
  int block_id;
  /* orientation of each interface face relative to its partner face, from
   * the face's line of the reference's mapping file (mapping.f90:64-236,
   * interface1.f90:96-464): bit 0 set when the partner's range along this
   * face's first tangential direction runs backwards (s > e), bit 1 the
   * same for the second direction, bit 2 the dir_switch column (the two
   * tangential directions swapped).  Tangential directions: (j, k) on i
   * faces, (i, k) on j faces, (i, j) on k faces.  Default 0 (aligned). */
  int partner_orient[6];
  /* fixed tv of each face for Spalart-Allmaras blocks (read_bc.f90:112-115) */
  double fixed_tv[6];
  /* fixed kL of each face for k-kL blocks (read_bc.f90) */
  double fixed_tkl[6];
  /* fixed intermittency of each face for LCTM2015 blocks (bc%fixed_tgm) */
  double fixed_tgm[6];
} fest_bc;

typedef struct fest_handle fest_handle;

/* ---- lifetime ---------------------------------------------------------- */
/* setup_scheme/setup_bc/setup_gradients/setup_viscosity/setup_update of the
 * reference (scheme.f90:29, bc.f90:18, gradients.f90:94, viscosity.f90:553,
 * update.f90:92) in one call.  Allocates every device array of the block. */
int fest_create(const fest_extent *dims, const fest_flow *flow,
                const fest_scheme *scheme, const fest_bc *bc,
                fest_handle **out);
int fest_destroy(fest_handle *h);
/* FEST_FP64 (default) or FEST_MIXED for fest_step */
int fest_set_precision(fest_handle *h, int precision);
/* last device-side error word (FEST_ERR_*), cleared by the call */
int fest_last_device_error(fest_handle *h);
/* number of kernels this handle has launched so far */
long long fest_kernel_launches(const fest_handle *h);

/* ---- geometry (grid.f90:137-236 ghost_grid, geometry.f90:548-580) ------ */
/* nodes: interior nodes (1:imx,1:jmx,1:kmx) filled, ghosts extrapolated
 * here.  Outputs (nullable) receive the metrics; they also stay on device. */
int fest_setup_geometry(fest_handle *h, double *nodes, double *cells,
                        double *Ifaces, double *Jfaces, double *Kfaces);
/* upload metrics computed elsewhere (e.g. by the Fortran setup_geometry) */
int fest_set_metrics(fest_handle *h, const double *cells, const double *Ifaces,
                     const double *Jfaces, const double *Kfaces);
/* wall distance (wall_dist.f90:84-131): min node distance to the given wall
 * node list, averaged to cells.  dist (nullable) receives the result. */
int fest_find_wall_dist(fest_handle *h, const double *wall_xyz, int n_wall,
                        double *dist);
int fest_set_wall_dist(fest_handle *h, const double *dist);

/* ---- state ------------------------------------------------------------- */
int fest_upload_state(fest_handle *h, const double *qp);
int fest_download_state(fest_handle *h, double *qp);
/* The state for a checkpoint (replaces the qp that solver.f90:186 hands to
 * dump_solution.f90:27-52 checkpoint) while stepping goes on.
 * fest_snapshot_begin enqueues a device copy of the current padded state
 * after the work already on the handle's stream, and that copy's transfer
 * into qp (the padded shape of fest_download_state) on a copy stream of the
 * handle's own; it returns without waiting.  Steps enqueued afterwards
 * (fest_step_async, fest_batch_step_async) run while the transfer travels,
 * provided qp is pinned host memory (cudaHostAlloc / cudaMallocHost;
 * pageable memory makes the call wait for the transfer).  qp must not be
 * read before fest_snapshot_wait returns, which blocks until the transfer
 * is complete and returns the device error word as it stood when the state
 * was copied (FEST_OK, or the failed step's FEST_ERR_*; the word itself is
 * left for fest_last_device_error).  One snapshot at a time: a second
 * begin before the wait returns FEST_ERR_ARG; a wait with none pending
 * returns FEST_OK. */
int fest_snapshot_begin(fest_handle *h, double *qp);
int fest_snapshot_wait(fest_handle *h);

/* ---- module arrays held by the handle -----------------------------------
 * The reference keeps these as module variables (face_interpolant.f90:17-22,
 * gradients.f90:17-19, viscosity.f90:41-44, global_sst.f90:25,
 * wall_dist.f90, time.f90, scheme.f90:29-63); a drop-in shim reads and writes
 * them through these two calls.  Sizes are in doubles. */
enum { FEST_ARR_QP = 0, FEST_ARR_TEMP, FEST_ARR_CELLS, FEST_ARR_IFACES,
       FEST_ARR_JFACES, FEST_ARR_KFACES, FEST_ARR_NODES,
       FEST_ARR_X_QP_LEFT, FEST_ARR_X_QP_RIGHT, FEST_ARR_Y_QP_LEFT,
       FEST_ARR_Y_QP_RIGHT, FEST_ARR_Z_QP_LEFT, FEST_ARR_Z_QP_RIGHT,
       FEST_ARR_F, FEST_ARR_G, FEST_ARR_H, FEST_ARR_RESIDUE,
       FEST_ARR_GRADQP_X, FEST_ARR_GRADQP_Y, FEST_ARR_GRADQP_Z,
       FEST_ARR_MU, FEST_ARR_MU_T, FEST_ARR_SST_F1, FEST_ARR_DIST,
       FEST_ARR_DELTA_T, FEST_ARR_COUNT };
long long fest_array_size(const fest_handle *h, int which);
int fest_set_array(fest_handle *h, int which, const double *host);
int fest_get_array(fest_handle *h, int which, double *host);

/* ---- module-level entry points (drop-ins for the Fortran procedures) --- */
/* apply_interface (interface1.f90:96) + populate_ghost_primitive
 * (bc_primitive.f90:55): ghost layers of qp for every face, then the 0.33
 * corner averaging (bc_primitive.f90:209-224). */
int fest_populate_ghost_primitive(fest_handle *h, double *qp, int current_iter);
/* Temp = p/(R rho) over the padded block (update.f90:170) */
int fest_compute_temperature(fest_handle *h, const double *qp, double *Temp);
/* compute_face_interpolant (face_interpolant.f90:79) */
int fest_compute_face_interpolant(fest_handle *h, const double *qp,
                                  double *x_qp_left, double *x_qp_right,
                                  double *y_qp_left, double *y_qp_right,
                                  double *z_qp_left, double *z_qp_right);
/* reconstruct_boundary_state (boundary_state_reconstruction.f90:28); the
 * face-state arrays are in/out (nullable: device-resident ones) */
int fest_reconstruct_boundary_state(fest_handle *h, const double *qp,
                                    double *x_qp_left, double *x_qp_right,
                                    double *y_qp_left, double *y_qp_right,
                                    double *z_qp_left, double *z_qp_right);
/* compute_fluxes (scheme.f90:68) from the face states held in the handle */
int fest_compute_fluxes(fest_handle *h, double *F, double *G, double *H);
/* evaluate_all_gradients (gradients.f90:276) incl. apply_gradient_bc */
int fest_evaluate_all_gradients(fest_handle *h, const double *qp,
                                const double *Temp, double *gradqp_x,
                                double *gradqp_y, double *gradqp_z);
/* calculate_viscosity (viscosity.f90:52): mu, mu_t and sst_F1 */
int fest_calculate_viscosity(fest_handle *h, const double *qp, double *mu,
                             double *mu_t, double *sst_F1);
/* compute_viscous_fluxes (viscous.f90:55): adds into F, G, H (in/out) */
int fest_compute_viscous_fluxes(fest_handle *h, const double *qp, double *F,
                                double *G, double *H);
/* compute_residue (scheme.f90:111) */
int fest_compute_residue(fest_handle *h, const double *F, const double *G,
                         const double *H, double *residue);
/* add_source_term_residue (source.f90:94): residue in/out */
int fest_add_source_term_residue(fest_handle *h, const double *qp,
                                 double *residue);
/* compute_time_step (time.f90:291), using the face states of the handle */
int fest_compute_time_step(fest_handle *h, const double *qp, double CFL,
                           double *delta_t);
/* get_total_conservative_Residue (update.f90:495): all of the above in the
 * reference's order on the resident state; outputs nullable */
int fest_get_total_conservative_residue(fest_handle *h, double *qp,
                                        int current_iter, double *residue);
/* get_next_solution (update.f90:129): one iteration of the configured
 * integrator on the resident state.  qp (nullable) is uploaded before and
 * downloaded after; residue/delta_t (nullable) receive the last stage's. */
int fest_get_next_solution(fest_handle *h, double *qp, int current_iter,
                           double CFL, double *residue, double *delta_t);
/* find_resnorm (resnorm.f90:62): res_abs[0..n_var] from the last residue
 * and fluxes; res_abs[0] is |net mass flux| (resnorm.f90:190-198),
 * res_abs[l] = sqrt(sum R_l^2) / scale_l (resnorm.f90:171-176, 221). */
int fest_find_resnorm(fest_handle *h, double *res_abs);

/* ---- fused fast path ----------------------------------------------------- */
/* n_iters iterations starting at iteration number first_iter, state kept on
 * device, in the precision chosen by fest_set_precision.  In FEST_MIXED the
 * stencil arithmetic runs in FP32 and the primitive state, the metrics and
 * the norm stay FP64.  res_abs (nullable) receives the last norm. */
int fest_step(fest_handle *h, int n_iters, int first_iter, double CFL,
              double *res_abs);

/* fest_step on a host state: qp (the padded host array, as
 * fest_upload_state takes it) goes to the device, n_iters iterations run,
 * and the state comes back into qp, with one synchronisation for the
 * whole call: get_next_solution (update.f90:129-226) n_iters times on the
 * caller's array.  Pinned, mapped host arrays move over the host link by
 * a copy kernel.  res_abs (nullable) receives the last norm. */
int fest_step_host(fest_handle *h, double *qp, int n_iters, int first_iter, double CFL,
                   double *res_abs);
/* fest_step_host on the interior cells only: q is a dense
 * (imx-1)(jmx-1)(kmx-1) x n_var array (i fastest, the cell-centred
 * solution without ghost layers, as the reference's output files hold
 * it).  The ghost cells stay the handle's own: every BC refills them from
 * the interior at each stage, and the fix() layers written in iterations
 * 1-2 persist on the device as they do in the reference's qp.  Pinned,
 * mapped arrays are read and written by the GPU over the host link. */
int fest_step_host_interior(fest_handle *h, double *q, int n_iters, int first_iter, double CFL,
                            double *res_abs);

/* enqueue fest_step's work on the handle's stream and return at once;
 * errors surface at the next synchronous call (fest_last_device_error) */
int fest_step_async(fest_handle *h, int n_iters, int first_iter, double CFL);
/* run the handle's work on a caller-owned CUDA stream (cudaStream_t passed
 * as void*); NULL restores the handle's own stream */
int fest_set_stream(fest_handle *h, void *cuda_stream);
/* time every fused stage-sweep launch with CUDA events on the handle's
 * stream (enable != 0 starts and clears the record); read the launch count
 * and their summed device time */
int fest_profile(fest_handle *h, int enable);
int fest_profile_read(fest_handle *h, long long *launches, double *total_ms);
/* device time (CUDA events on the handle's stream) of the kernels of the
 * last fest_step, fest_step_host, fest_get_total_conservative_residue or
 * fest_residual_vjp call: from after its host inputs arrived to before its
 * outputs left */
int fest_last_kernel_ms(fest_handle *h, double *ms);

/* ---- batches ------------------------------------------------------------- */
/* No counterpart in the reference (its blocks advance one MPI rank each,
 * exchanging interface ghosts with MPI_SENDRECV, interface1.f90:96-464).
 * The blocks of a multiblock case advanced together, stage by stage, each
 * interface face's ghost layers copied on the device from its partner
 * block's interior (fest_bc.partner_block names the partner's block_id,
 * partner_orient its orientation).  All handles must use one precision and
 * the fused path's schemes with one integrator.  FEST_MIXED batches (one
 * reconstruction, flux scheme and physics) run one ghost launch and one
 * sweep launch per RK stage for every block from iteration 3 on; FP64
 * batches launch each block's own sweep.  Geometry and state are set
 * through the handles as usual.  fest_batch_create moves every handle onto
 * the first handle's current stream and fest_batch_destroy gives each its
 * own stream back: destroy the batch before any of its handles.  Each
 * handle still answers fest_find_resnorm, fest_download_state etc. for its
 * block; a handle with partners in other blocks steps only in its batch
 * (its own step and residual entry points return FEST_ERR_ARG). */
typedef struct fest_batch fest_batch;
int fest_batch_create(fest_handle *const *blocks, int n_blocks, fest_batch **out);
int fest_batch_destroy(fest_batch *b);
/* n_iters iterations of every block from iteration number first_iter;
 * _async returns after enqueueing on the batch's stream */
int fest_batch_step(fest_batch *b, int n_iters, int first_iter, double CFL);
int fest_batch_step_async(fest_batch *b, int n_iters, int first_iter, double CFL);

/* ---- adjoint ------------------------------------------------------------- */
/* No counterpart in the reference.  Reverse-mode product with the
 * transposed Jacobian of the residual that fest_get_total_conservative_residue
 * computes at this iteration: dq = (dR/dq)^T lambda, q the interior primitive
 * state (ghost cells follow it through the BCs of the iteration), lambda in
 * the residue layout, dq in the qp layout (ghost entries zero).  qp
 * (nullable: the device state) is uploaded and its ghosts filled first.
 * FP64.  Inviscid, laminar and k-omega SST blocks of the fused-path kind
 * (n_var 5, or 7 with SST; >= 4 interior cells per direction, no -9 face,
 * no pressure switch, adiabatic -5 walls; viscous: no interface ids >= 0;
 * SST: viscous, and no far-field (-8), total-pressure (-11) or interface
 * faces, whose k and omega ghosts depend on the fill's last column), the
 * viscous terms with the temperature p/(rho R) of the state; FEST_ERR_ARG
 * otherwise. */
int fest_residual_vjp(fest_handle *h, const double *qp, int current_iter,
                      const double *lambda, double *dq);
/* No counterpart in the reference.  The same product with respect to the
 * grid nodes: dnodes = (dR/dnodes)^T lambda + (dfaces/dnodes)^T faces_bar,
 * through the face metrics of the fluxes and of the BCs (tangency normals,
 * Riemann normals), for laminar blocks also through the face records,
 * volumes and centres that the Green-Gauss gradients, their BCs and the
 * viscous fluxes read, then the face vectors, the cell volumes and centres
 * and the ghost-node extrapolation (grid.f90:137-236, geometry.f90).
 * dnodes in the nodes layout (interior nodes carry the result, ghost nodes
 * zero); lambda and the three face-layout adjoints *_bar (an objective's
 * explicit metric dependence) are nullable; dq (nullable) receives
 * fest_residual_vjp's result.  Same restrictions as fest_residual_vjp,
 * inviscid and laminar blocks only (SST wall distances depend on the nodes
 * too), and no WENO_NM (volume weights). */
int fest_residual_vjp_nodes(fest_handle *h, const double *qp, int current_iter,
                            const double *lambda, const double *Ifaces_bar,
                            const double *Jfaces_bar, const double *Kfaces_bar,
                            double *dq, double *dnodes);
/* No counterpart in the reference.  Adjoint of the steady residual at the
 * device state (a converged primal, local time steps at CFL): solves
 * (dR/dq)^T psi = -dJ/dq for psi (residue layout) as the fixed point
 * phi = G^T phi + dJ/dq, G the handle's integrator map (forward Euler or
 * TVD-RK3) linearised at the primal fixed point, built from stages
 * S = I - P dR/dq with P = (dt/V) dq/dU; it converges where that primal
 * iteration does.  dJdq in the qp layout (interior entries used).
 * Stops after max_iters or when the RMS update has dropped by tol;
 * n_done, drop (nullable) report the iterations and that drop.  Then
 * dJ/dalpha = dJ/dalpha|_q + psi . dR/dalpha for any parameter alpha.
 * Blocks fest_residual_vjp supports, local time steps, forward Euler or
 * TVD-RK3; for k-omega SST blocks P maps k and omega through U/rho and the
 * update's point-implicit destruction factors (update.f90:395-398). */
int fest_adjoint_solve(fest_handle *h, const double *dJdq, double CFL,
                       int max_iters, double tol, double *psi, int *n_done,
                       double *drop);

/* ---- measurement ---------------------------------------------------------- */
/* No counterpart in the reference.  The arithmetic roof of the current
 * device, measured with event-timed dependent FMA chains on every SM: kind 0
 * FP64, 1 FP32; *tflops in TFLOP/s (two per fused multiply-add).  The FP64
 * sweeps are bound by it on this hardware. */
int fest_measure_peak(int kind, double *tflops);

/* ---- allocation-free norm ------------------------------------------------ */
/* No counterpart in the reference.  find_resnorm (resnorm.f90:62) without a
 * handle, on caller-owned DEVICE arrays: residue in the FEST_ARR_RESIDUE
 * layout, F/G/H in the FEST_ARR_F/G/H layouts (only variable 1, the mass
 * flux, is read); res_abs (host, n_var+1) as fest_find_resnorm returns it.
 * For callers that cannot allocate device memory where they need the norm
 * (memory held by their own pool, or an asynchronous loop that a
 * cudaMalloc/cudaFree pair would synchronise).  It allocates nothing: its
 * scratch is a fixed 32 KiB area per device, so n_var may be at most 7
 * (FEST_ERR_SCRATCH otherwise); n_var must be 5 (Euler, laminar) or 7
 * (k-omega SST, scaled by tk_inf and tw_inf), FEST_ERR_ARG otherwise.  Calls that overlap in time on one device
 * race on that area and must be serialised by the caller.  The first call
 * on each device (with that device current) does the setup.  Runs on
 * cuda_stream (NULL: the legacy default stream) and returns after
 * synchronising it, so no call can be stream-captured: a call on a
 * capturing stream returns FEST_ERR_ARG and leaves the capture intact. */
int fest_find_resnorm_noalloc(const fest_extent *ext, const fest_flow *flow,
                              const double *residue, const double *F,
                              const double *G, const double *H,
                              double *res_abs, void *cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* FEST_GPU_H */
