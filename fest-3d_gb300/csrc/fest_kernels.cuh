// fest_kernels.cuh - host-side launchers of the module kernels (FP64, the
// reference's structure: one kernel per Fortran procedure, module arrays
// materialised in HBM).
#pragma once
#include "fest_common.cuh"

namespace fest {

// device arrays of one block, all in the reference's Fortran layouts
struct DevBlock {
  double *qp, *Temp, *cells, *faces[3], *nodes;
  double *fsL[3], *fsR[3];  // x/y/z_qp_left/right
  double *flux[3];          // F, G, H
  double *res, *grad[3], *mu, *mut, *F1, *dist, *dt, *Ustore, *Rstore;
  double *red;              // reduction scratch (kRedSlots doubles)
  int *err;                 // device error word
  float *qp32;              // FP32 mirror of qp kept by the mixed fused path (else null)
  int qp32_pitch;           // its row pitch (imx+5 rounded up to a multiple of 4)
};

// index in the FP32 state mirror of padded cell c (a pidx) of variable l:
// the mirror has the padded layout of qp with rows padded to `pitch` so
// that TMA tiles can address it (row strides a multiple of 16 bytes)
__host__ __device__ __forceinline__ long long mirror_index(const Dims& d, int pitch, long long c, int l) {
  const int ci = (int)c;  // P * n_var < 2^31 on the fused path
  return (long long)(ci % d.ni) + (long long)pitch * (ci / d.ni + (long long)d.nj * d.nk * l);
}
constexpr int kRedSlots = 1 << 16;

// the vorticity and strain magnitudes of add_sst_source_lctm2015
// (source.f90:347-362) and of lusgs.f90:2445-2460, from the cell gradients
__device__ __forceinline__ void lctm_vort_strain(const DevBlock& b, long long og, long long NG, double& vort,
                                                 double& strain) {
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  const double wa = G(1, 3) - G(2, 2), wb = G(2, 1) - G(0, 3), wc = G(0, 2) - G(1, 1);
  vort = ::sqrt(((wa * wa) + (wb * wb) + (wc * wc)));
  const double sa = G(1, 3) + G(2, 2), sb = G(2, 1) + G(0, 3), sc = G(0, 2) + G(1, 1);
  strain = ::sqrt((sa * sa) + (sb * sb) + (sc * sc) + 2 * (G(0, 1) * G(0, 1)) + 2 * (G(1, 2) * G(1, 2)) +
                2 * (G(2, 3) * G(2, 3)));
}

// the onset terms shared by the source and the implicit update:
// Fturb = ::exp(-(RT/2)^4) and max(min(Rev/(2.2 Re_theta), 2) -
// max(1 - (RT/3.5)^3, 0), 0) (source.f90:433-440, lusgs.f90:2463-2470)
__device__ __forceinline__ void lctm_onset(double Rev, double RT, double Re_theta, double& Fturb, double& Fonset) {
  const double h = 0.5 * RT, h2 = h * h;
  Fturb = ::exp(-(h2 * h2));
  const double Fonset2 = fmin2(Rev / (2.2 * Re_theta), 2.0);
  const double t3 = RT / 3.5;
  const double Fonset3 = fmax2(1.0 - (t3 * t3) * t3, 0.0);
  Fonset = fmax2(Fonset2 - Fonset3, 0.0);
}


// a block as seen by the interface exchange of another block
struct BlockRef {
  DevBlock b;
  Dims d;
};

struct Launcher {
  cudaStream_t s;
  long long* count;  // kernels launched through this launcher
};

// ghost cells: interface exchange + populate_ghost_primitive + corners
// d_table: device array of every block a face of this block may pair with
void launch_ghosts(const Params& p, const DevBlock& b, const BlockRef* d_table, int iter,
                   const Launcher& L, bool corners = true);
bool ghosts_need_sequential(const Params& p);
// true when no face's BC reads beyond the block's interior cells (the
// faces may then fill their ghosts concurrently, in any buffer)
bool ghost_depth_ok(const Params& p, bool stencil_only = false);
void launch_temperature(const Params& p, const DevBlock& b, const Launcher& L);
// mode 0: compute_face_interpolant only; 1: + reconstruct_boundary_state;
// 2: reconstruct_boundary_state alone on the held face states
void launch_face_states(const Params& p, const DevBlock& b, int mode, const Launcher& L);
void launch_fluxes(const Params& p, const DevBlock& b, const Launcher& L);
void launch_gradients(const Params& p, const DevBlock& b, const Launcher& L);
void launch_viscosity(const Params& p, const DevBlock& b, const Launcher& L);
void launch_viscous_fluxes(const Params& p, const DevBlock& b, const Launcher& L);
void launch_residue(const Params& p, const DevBlock& b, bool with_source, const Launcher& L);
void launch_source(const Params& p, const DevBlock& b, const Launcher& L);
void launch_time_step(const Params& p, const DevBlock& b, double CFL, const Launcher& L);
void launch_update(const Params& p, const DevBlock& b, double TF, double SF, int TU, int use_store,
                   const Launcher& L);
void launch_blend(const Params& p, const DevBlock& b, double a, double c, const Launcher& L);
// res_abs partials of this block: out[0] mass imbalance, out[l] sum R_l^2
void launch_resnorm(const Params& p, const DevBlock& b, double* d_out, const Launcher& L);
// the LU-SGS update of the implicit integrator (fest_lusgs.cu) on the
// residue and time step held by b; scratch: lusgs_scratch_doubles doubles
long long lusgs_scratch_doubles(const Dims& d);
void launch_lusgs(const Params& p, const DevBlock& b, double* scratch, const Launcher& L);
void launch_geometry(const Params& p, const DevBlock& b, const Launcher& L);
void launch_wall_dist(const Params& p, const DevBlock& b, const double* d_wall, int n_wall,
                      double* d_node_dist, const Launcher& L);
// adjoint of the residual (inviscid or laminar): bar (padded qp layout) =
// (dR/dq)^T lam (residue layout), ghost cells filled for iteration iter
// beforehand and, for laminar blocks, the temperature, gradients and
// viscosity of the state computed (launch_viscous_prep)
bool vjp_supported(const Params& p);
// bar_faces (null, or three face-layout arrays, zeroed by the caller) also
// receive (dR/dfaces)^T lam; bar_grad: 12 doubles per interior cell of work
// space for laminar blocks
// face_work: vjp_face_work_doubles(d) doubles of work space (the flux
// transposes of one direction's faces)
// bar_cells (laminar blocks with bar_faces: 4 doubles per padded cell,
// zeroed by the caller) receives (dR/dcells)^T lam, the cell volumes' and
// centres' share of the viscous terms
void launch_residual_vjp(const Params& p, const DevBlock& b, int iter, const double* lam,
                         double* bar, const Launcher& L, double* const* bar_faces, double* bar_grad,
                         double* face_work, double* bar_cells = nullptr);
long long vjp_face_work_doubles(const Dims& d);
// the bar_grad work space: 12 doubles per interior cell (laminar), or the
// SST's gradient, eddy-viscosity and F1 adjoints
long long vjp_grad_work_doubles(const Dims& d, bool sst);
// nodes-layout bar_nodes = (dfaces/dnodes)^T bar_faces + (dcells/dnodes)^T
// bar_cells (nullable), through the face vectors, the cell volumes and
// centres, and the ghost-node extrapolation (interior nodes carry the result)
void launch_geometry_vjp(const Params& p, const DevBlock& b, double* const* bar_faces, double* bar_nodes,
                         const Launcher& L, const double* bar_cells = nullptr);
// work arrays of the fixed-point adjoint: phi, dJ, a, b, c, bar in the qp
// layout, mu in the residue layout, sq one double
struct AdjointWork {
  double *phi, *dJ, *a, *b, *c, *bar, *mu, *sq;
  double* grad;  // 12 per interior cell (laminar blocks)
  double* face;  // vjp_face_work_doubles
};
// one step phi <- G^T phi + dJ/dq (G the integrator's map linearised at the
// fixed point: forward Euler or TVD-RK3); sq += |change of phi|^2
void launch_adjoint_iteration(const Params& p, const DevBlock& b, AdjointWork& w, const Launcher& L);
// psi = -P^T H phi (residue layout), the adjoint of the residual
void launch_adjoint_psi(const Params& p, const DevBlock& b, AdjointWork& w, double* psi,
                        const Launcher& L);

}  // namespace fest
