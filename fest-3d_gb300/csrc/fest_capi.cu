// fest_capi.cu - the extern "C" boundary: handle lifetime, host<->device
// movement of the reference's Fortran-layout arrays, and the module-level
// and integrator entry points built from the module kernels.
#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fest_fused.cuh"
#include "fest_kernels.cuh"

using namespace fest;

struct fest_handle {
  Params p;
  fest_extent ext;
  fest_flow flow;
  fest_scheme sc;
  fest_bc bc;
  cudaStream_t s = nullptr;      // stream in use
  cudaStream_t own = nullptr;    // the handle's own stream
  DevBlock d{};
  BlockRef* d_table = nullptr;
  double* d_resnorm = nullptr;
  double* d_nodedist = nullptr;
  double* d_wall = nullptr;
  int n_wall_cap = 0;
  int precision = FEST_FP64;
  long long launches = 0;
  FusedState* fused = nullptr;
  double* d_vjp_bar = nullptr;  // adjoint work arrays, allocated on first use
  double* d_vjp_lam = nullptr;
  double* d_vjp_grad = nullptr;  // viscous adjoint work (vjp_grad_work_doubles)
  double* d_vjp_face = nullptr;  // adjoint: one direction's face flux transposes
  double* d_lu = nullptr;        // LU-SGS work arrays, allocated on first use
  double* d_stage = nullptr;     // interior-cell staging for pageable host arrays
  int* h_err = nullptr;          // pinned host copy of the device error word
  // state snapshot for the output writers (fest_snapshot_begin): the
  // device copy, its error word, the copy stream and its two events
  double* d_snap = nullptr;
  int* h_snap_err = nullptr;
  cudaStream_t snap_s = nullptr;
  cudaEvent_t snap_ev[2] = {nullptr, nullptr};
  bool snap_busy = false;
  // events around the device work of the last timed call (after its inputs
  // arrived, before its outputs leave): fest_last_kernel_ms
  cudaEvent_t kev[2] = {nullptr, nullptr};
  std::vector<void*> allocs;
  Launcher L() { return Launcher{s, &launches}; }
};

namespace {

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return FEST_OK;
  if (e == cudaErrorMemoryAllocation) return FEST_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FEST_ERR_NO_DEVICE;
  return FEST_ERR_CUDA;
}

#define CK(x)                                  \
  do {                                         \
    cudaError_t e_ = (x);                      \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

#define RET(x)                \
  do {                        \
    int r_ = (x);             \
    if (r_) return r_;        \
  } while (0)

int dalloc(fest_handle* h, double** p, long long n) {
  if (n <= 0) n = 1;
  CK(cudaMalloc((void**)p, sizeof(double) * (size_t)n));
  h->allocs.push_back(*p);
  CK(cudaMemsetAsync(*p, 0, sizeof(double) * (size_t)n, h->s));
  return FEST_OK;
}

struct Sizes {
  long long qp, pad, cells, faces[3], nodes, fs[3], fl[3], res, grad, dt;
};
Sizes sizes_of(const Dims& d, int n_grad) {
  Sizes z;
  z.pad = d.P;
  z.qp = d.P * d.nv;
  z.cells = 4 * d.P;
  for (int dir = 0; dir < 3; ++dir) {
    z.faces[dir] = 4 * nfaces(d, dir);
    z.fs[dir] = fsdim(d, dir).N * d.nv;
    z.fl[dir] = fldim(d, dir).N * d.nv;
  }
  z.nodes = 3LL * (d.imx + 6) * (d.jmx + 6) * (d.kmx + 6);
  z.res = ncells(d) * d.nv;
  z.grad = ngrad(d) * n_grad;
  z.dt = ncells(d);
  return z;
}

// Whole arrays cross the host link by the copy engines (cudaMemcpyAsync):
// on this part they move pinned host memory at the link's rate (about
// 200 GB/s each way, measured against SM copy kernels of every width and
// grid, which reach the same or slightly less).
int up(fest_handle* h, double* dst, const double* src, long long n) {
  if (!src) return FEST_OK;
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, h->s));
  return FEST_OK;
}
int down(fest_handle* h, double* dst, const double* src, long long n) {
  if (!dst) return FEST_OK;
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->s));
  return FEST_OK;
}

// the device address of a pinned, mapped host array, or null
const void* mapped_alias(const void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// interior cells (1..imx-1, 1..jmx-1, 1..kmx-1) of the padded state and a
// dense (imx-1)(jmx-1)(kmx-1) x n_var array, i fastest: to_padded scatters
// the dense array into the state, else gathers from it.  Either side may
// be a pinned, mapped host array, which the threads then read or write
// over the link directly.
__global__ void k_interior_copy(Dims d, const double* __restrict__ src, double* __restrict__ dst, int to_padded) {
  const long long nc = ncells(d), n = nc * d.nv;
  const long long st = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += st) {
    const long long l = t / nc, c = t % nc;
    const int i = 1 + (int)(c % (d.imx - 1));
    const long long r = c / (d.imx - 1);
    const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
    const long long pp = pidx(d, i, j, k) + d.P * l;
    if (to_padded) dst[pp] = src[t];
    else dst[t] = src[pp];
  }
}
int interior_copy(fest_handle* h, const double* src, double* dst, int to_padded) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_interior_copy<<<sms * 4, 256, 0, h->s>>>(h->p.d, src, dst, to_padded);
  ++h->launches;
  CK(cudaGetLastError());
  return FEST_OK;
}
// a device-readable copy of a host interior array: the array itself when it
// is pinned and mapped, else the staging buffer after a copy
int interior_source(fest_handle* h, const double* host, const double** src) {
  const long long n = ncells(h->p.d) * h->p.d.nv;
  if (const void* a = mapped_alias(host)) {
    *src = static_cast<const double*>(a);
    return FEST_OK;
  }
  if (!h->d_stage) RET(dalloc(h, &h->d_stage, n));
  CK(cudaMemcpyAsync(h->d_stage, host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, h->s));
  *src = h->d_stage;
  return FEST_OK;
}
// the padded device state's interior cells -> a host interior array
int down_interior(fest_handle* h, double* host, const double* qdev) {
  const long long n = ncells(h->p.d) * h->p.d.nv;
  if (const void* a = mapped_alias(host))
    return interior_copy(h, qdev, static_cast<double*>(const_cast<void*>(a)), 0);
  if (!h->d_stage) RET(dalloc(h, &h->d_stage, n));
  RET(interior_copy(h, qdev, h->d_stage, 0));
  CK(cudaMemcpyAsync(host, h->d_stage, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, h->s));
  return FEST_OK;
}

// wait for the stream; report CUDA errors, then the device error word
int finish(fest_handle* h) {
  CK(cudaGetLastError());
  int err = 0;
  if (h->h_err) {  // the error word rides on the stream: one synchronisation
    CK(cudaMemcpyAsync(h->h_err, h->d.err, sizeof(int), cudaMemcpyDeviceToHost, h->s));
    CK(cudaStreamSynchronize(h->s));
    err = *h->h_err;
  } else {
    CK(cudaStreamSynchronize(h->s));
    CK(cudaMemcpy(&err, h->d.err, sizeof(int), cudaMemcpyDeviceToHost));
  }
  if (err) {
    CK(cudaMemset(h->d.err, 0, sizeof(int)));
    return err;
  }
  return FEST_OK;
}


bool valid_id(int id) { return id >= -11 && id <= -1 ? true : id >= 0; }

void fill_params(fest_handle* h) {
  Params& p = h->p;
  memset(&p, 0, sizeof(p));
  const fest_extent& e = h->ext;
  p.d.imx = e.imx; p.d.jmx = e.jmx; p.d.kmx = e.kmx; p.d.nv = e.n_var;
  p.d.ni = e.imx + 5; p.d.nj = e.jmx + 5; p.d.nk = e.kmx + 5;
  p.d.P = (long long)p.d.ni * p.d.nj * p.d.nk;
  const fest_flow& f = h->flow;
  p.gm = f.gm; p.R = f.R_gas; p.mu_ref = f.mu_ref; p.T_ref = f.T_ref; p.S = f.Sutherland_temp;
  p.Pr = f.Pr; p.tPr = f.tPr; p.MInf = f.MInf; p.p_inf = f.pressure_inf; p.rho_inf = f.density_inf;
  p.u_inf = f.x_speed_inf; p.v_inf = f.y_speed_inf; p.w_inf = f.z_speed_inf;
  p.mu_var = f.mu_variation;
  const fest_scheme& s = h->sc;
  p.flux = s.scheme_name; p.interp = s.interpolant; p.limiter = s.limiter; p.turb = s.turbulence;
  p.tstep = s.time_stepping_method; p.gdt = s.global_time_step;
  p.integ = s.time_step_accuracy;
  p.lam[0] = s.ilimiter_switch; p.lam[1] = s.jlimiter_switch; p.lam[2] = s.klimiter_switch;
  p.tlim[0] = s.itlimiter_switch; p.tlim[1] = s.jtlimiter_switch; p.tlim[2] = s.ktlimiter_switch;
  p.pb[0] = s.iPB_switch; p.pb[1] = s.jPB_switch; p.pb[2] = s.kPB_switch;
  // get_n_grad (gradients.f90:229-258)
  p.n_grad = s.turbulence == FEST_TURB_NONE ? 4 : s.turbulence == FEST_TURB_SA ? 5 : 6;
  if (s.transition == FEST_TRANSITION_LCTM2015) p.n_grad += 1;  // gradients.f90:260-265
  p.sa_cv1_3 = pow(7.1, 3.0);
  p.kkl_c025 = pow(0.09, 0.25);
  p.kkl_c075 = pow(0.09, 0.75);
  // the free-stream Reynolds number per unit length (state.f90:89) and
  // the 'bc' model's constants of it and of Tu (source.f90:576-581)
  p.transition = s.transition;
  if (s.transition == FEST_TRANSITION_BC) {
    const double Re = f.density_inf * f.vel_mag * 1.0 / f.mu_ref;
    p.bc_nu_cr = 5.0 / Re;
    p.bc_re_theta_t = (803.73 * (pow((f.tu_inf + 0.6067), (-1.027))));
  }
  // setup_bc (bc.f90:48-50)
  p.c2 = 1 + s.accur; p.c3 = 0.5 * s.accur; p.c1 = p.c2 - p.c3;
  const fest_bc& b = h->bc;
  // ppm_flag (boundary_state_reconstruction.f90:45-47)
  p.ppm_flag = (s.interpolant == FEST_INTERP_PPM || s.interpolant == FEST_INTERP_WENO ||
                s.interpolant == FEST_INTERP_WENO_NM);
  p.self_block = 0;
  for (int i = 0; i < 6; ++i) {
    p.id[i] = b.id[i];
    if (b.id[i] == -7) p.ppm_flag = 1;
    // a pair with this same block resolves to entry 0 of the handle's own
    // block table; pairs with other blocks resolve inside a batch
    p.part_block[i] = b.partner_block[i] == b.block_id ? 0 : -1;
    p.part_face[i] = b.partner_face[i];
    p.part_orient[i] = b.partner_orient[i];
    p.fix_rho[i] = b.fixed_density[i]; p.fix_p[i] = b.fixed_pressure[i];
    p.fix_u[i] = b.fixed_x_speed[i]; p.fix_v[i] = b.fixed_y_speed[i]; p.fix_w[i] = b.fixed_z_speed[i];
    p.fix_tk[i] = b.fixed_tk[i]; p.fix_tw[i] = b.fixed_tw[i]; p.fix_tv[i] = b.fixed_tv[i];
    p.fix_tkl[i] = b.fixed_tkl[i]; p.fix_tgm[i] = b.fixed_tgm[i];
    p.Tw[i] = b.fixed_wall_temperature[i]; p.Tp[i] = b.fixed_Tpressure[i];
  }
  params_f32(p);
}

double* arr_ptr(fest_handle* h, int which) {
  DevBlock& d = h->d;
  switch (which) {
    case FEST_ARR_QP: return d.qp;
    case FEST_ARR_TEMP: return d.Temp;
    case FEST_ARR_CELLS: return d.cells;
    case FEST_ARR_IFACES: return d.faces[0];
    case FEST_ARR_JFACES: return d.faces[1];
    case FEST_ARR_KFACES: return d.faces[2];
    case FEST_ARR_NODES: return d.nodes;
    case FEST_ARR_X_QP_LEFT: return d.fsL[0];
    case FEST_ARR_X_QP_RIGHT: return d.fsR[0];
    case FEST_ARR_Y_QP_LEFT: return d.fsL[1];
    case FEST_ARR_Y_QP_RIGHT: return d.fsR[1];
    case FEST_ARR_Z_QP_LEFT: return d.fsL[2];
    case FEST_ARR_Z_QP_RIGHT: return d.fsR[2];
    case FEST_ARR_F: return d.flux[0];
    case FEST_ARR_G: return d.flux[1];
    case FEST_ARR_H: return d.flux[2];
    case FEST_ARR_RESIDUE: return d.res;
    case FEST_ARR_GRADQP_X: return d.grad[0];
    case FEST_ARR_GRADQP_Y: return d.grad[1];
    case FEST_ARR_GRADQP_Z: return d.grad[2];
    case FEST_ARR_MU: return d.mu;
    case FEST_ARR_MU_T: return d.mut;
    case FEST_ARR_SST_F1: return d.F1;
    case FEST_ARR_DIST: return d.dist;
    case FEST_ARR_DELTA_T: return d.dt;
    default: return nullptr;
  }
}

long long arr_size(const fest_handle* h, int which) {
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  switch (which) {
    case FEST_ARR_QP: return z.qp;
    case FEST_ARR_TEMP: case FEST_ARR_MU: case FEST_ARR_MU_T: case FEST_ARR_SST_F1:
    case FEST_ARR_DIST: return z.pad;
    case FEST_ARR_CELLS: return z.cells;
    case FEST_ARR_IFACES: return z.faces[0];
    case FEST_ARR_JFACES: return z.faces[1];
    case FEST_ARR_KFACES: return z.faces[2];
    case FEST_ARR_NODES: return z.nodes;
    case FEST_ARR_X_QP_LEFT: case FEST_ARR_X_QP_RIGHT: return z.fs[0];
    case FEST_ARR_Y_QP_LEFT: case FEST_ARR_Y_QP_RIGHT: return z.fs[1];
    case FEST_ARR_Z_QP_LEFT: case FEST_ARR_Z_QP_RIGHT: return z.fs[2];
    case FEST_ARR_F: return z.fl[0];
    case FEST_ARR_G: return z.fl[1];
    case FEST_ARR_H: return z.fl[2];
    case FEST_ARR_RESIDUE: return z.res;
    case FEST_ARR_GRADQP_X: case FEST_ARR_GRADQP_Y: case FEST_ARR_GRADQP_Z: return z.grad;
    case FEST_ARR_DELTA_T: return z.dt;
    default: return 0;
  }
}

// mark the start (0) or end (1) of a call's device work on the handle's stream
void kmark(fest_handle* h, int which) {
  if (h->kev[which]) cudaEventRecord(h->kev[which], h->s);
}

// a handle whose interface faces pair with other blocks fills its ghosts
// only inside a batch (fest_batch_create resolves the partners)
bool needs_batch(const fest_handle* h) {
  for (int f = 0; f < 6; ++f)
    if ((h->p.id[f] == -10 || h->p.id[f] >= 0) && h->p.part_block[f] < 0) return true;
  return false;
}

// the fused path may hold the current state in one of its own buffers:
// bring it back to the handle's qp before a module entry point reads it
int sync_fused(fest_handle* h) {
  if (h->fused) RET(fused_export_state(h->fused, h->d.qp, h->s));
  return FEST_OK;
}

__global__ void k_fill(double* x, long long n, double v) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] = v;
}

// get_total_conservative_Residue (update.f90:495-547) on the resident state;
// p and tab: the block's parameters and the block table its interface
// faces read (a batch's, whose part_block indices p holds)
int residual_module(fest_handle* h, int iter, const Params& p, const BlockRef* tab) {
  Launcher L = h->L();
  launch_ghosts(p, h->d, tab, iter, L);
  launch_face_states(p, h->d, 1, L);
  launch_fluxes(p, h->d, L);
  if (p.mu_ref != 0.0) {
    launch_gradients(p, h->d, L);
    launch_viscosity(p, h->d, L);
    launch_viscous_fluxes(p, h->d, L);
  }
  launch_residue(p, h->d, true, L);
  return FEST_OK;
}
int residual_fp64(fest_handle* h, int iter) { return residual_module(h, iter, h->p, h->d_table); }

// update_with_lusgs (lusgs.f90:134-183) on the residue and time step held
int lusgs_update(fest_handle* h, const Params& p) {
  if (!h->d_lu) RET(dalloc(h, &h->d_lu, lusgs_scratch_doubles(p.d)));
  launch_lusgs(p, h->d, h->d_lu, h->L());
  return FEST_OK;
}

// get_next_solution (update.f90:129-226) on the resident state, FP64
int next_solution_fp64(fest_handle* h, int it, double CFL) {
  const Params& p = h->p;
  Launcher L = h->L();
  const Dims& d = p.d;
  launch_temperature(p, h->d, L);
  auto store = [&]() {
    CK(cudaMemcpyAsync(h->d.Ustore, h->d.qp, sizeof(double) * d.P * d.nv, cudaMemcpyDeviceToDevice, h->s));
    return FEST_OK;
  };
  auto zeroR = [&]() {
    CK(cudaMemsetAsync(h->d.Rstore, 0, sizeof(double) * ncells(d) * d.nv, h->s));
    return FEST_OK;
  };
  switch (h->sc.time_step_accuracy) {
    case FEST_TIME_NONE:
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      launch_update(p, h->d, 1., 1., 0, 0, L);
      break;
    case FEST_TIME_RK4:
      RET(zeroR()); RET(store());
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      launch_update(p, h->d, 0.5, 1., 0, 1, L);
      residual_fp64(h, it); launch_update(p, h->d, 0.5, 2., 0, 1, L);
      residual_fp64(h, it); launch_update(p, h->d, 1.0, 2., 0, 1, L);
      residual_fp64(h, it); launch_update(p, h->d, 1. / 6., 1., 1, 1, L);
      break;
    case FEST_TIME_RK2:
      RET(zeroR()); RET(store());
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      launch_update(p, h->d, 0.5, 1., 0, 1, L);
      residual_fp64(h, it); launch_update(p, h->d, 0.5, 1., 1, 1, L);
      break;
    case FEST_TIME_TVDRK3:
      RET(store());
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      launch_update(p, h->d, 1.0, 1., 0, 0, L);
      residual_fp64(h, it); launch_update(p, h->d, 1.0, 1., 0, 0, L);
      launch_blend(p, h->d, 0.75, 0.25, L);
      residual_fp64(h, it); launch_update(p, h->d, 1.0, 1., 0, 0, L);
      launch_blend(p, h->d, 1. / 3., 2. / 3., L);
      break;
    case FEST_TIME_TVDRK2:
      RET(store());
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      launch_update(p, h->d, 1.0, 1., 0, 0, L);
      residual_fp64(h, it); launch_update(p, h->d, 1.0, 1., 0, 0, L);
      launch_blend(p, h->d, 0.5, 0.5, L);
      break;
    case FEST_TIME_PLUSGS:    // update.f90:219-222
    case FEST_TIME_IMPLICIT:  // update.f90:215-218
      residual_fp64(h, it);
      launch_time_step(p, h->d, CFL, L);
      RET(lusgs_update(h, p));
      break;
    default:
      return FEST_ERR_ARG;
  }
  return FEST_OK;
}

}  // namespace

// ============================================================================
extern "C" {

int fest_create(const fest_extent* dims, const fest_flow* flow, const fest_scheme* scheme,
                const fest_bc* bc, fest_handle** out) {
  if (!dims || !flow || !scheme || !bc || !out) return FEST_ERR_ARG;
  *out = nullptr;
  if (dims->imx < 2 || dims->jmx < 2 || dims->kmx < 2) return FEST_ERR_ARG;
  // set_n_var_value (state.f90:280-305)
  int nv_need = scheme->turbulence == FEST_TURB_NONE ? 5 : scheme->turbulence == FEST_TURB_SA ? 6 : 7;
  if (scheme->transition == FEST_TRANSITION_LCTM2015) nv_need += 1;  // state.f90:308-318
  if (dims->n_var != nv_need) return FEST_ERR_ARG;
  if (scheme->scheme_name < 0 || scheme->scheme_name > 5) return FEST_ERR_ARG;
  if (scheme->interpolant < 0 || scheme->interpolant > 4) return FEST_ERR_ARG;
  if (scheme->turbulence < 0 || scheme->turbulence > FEST_TURB_KKL) return FEST_ERR_ARG;
  // the implicit integrators' Spalart-Allmaras and k-kL branches are not built
  if ((scheme->turbulence == FEST_TURB_SA || scheme->turbulence == FEST_TURB_KKL) &&
      (scheme->time_step_accuracy == FEST_TIME_IMPLICIT || scheme->time_step_accuracy == FEST_TIME_PLUSGS))
    return FEST_ERR_ARG;
  if (scheme->time_step_accuracy < 0 || scheme->time_step_accuracy > FEST_TIME_PLUSGS) return FEST_ERR_ARG;
  // the 'bc' transition model replaces the SA or SST source only
  // (source.f90:124-143; the implicit integrators update SST-BC as SST,
  // lusgs.f90:161-164); lctm2015 is not built
  if (scheme->transition < FEST_TRANSITION_NONE || scheme->transition > FEST_TRANSITION_LCTM2015) return FEST_ERR_ARG;
  if (scheme->transition == FEST_TRANSITION_BC &&
      (scheme->turbulence == FEST_TURB_NONE || scheme->turbulence == FEST_TURB_KKL || flow->mu_ref <= 0.0))
    return FEST_ERR_ARG;
  // LCTM2015 sits on k-omega SST (source.f90:134-143)
  if (scheme->transition == FEST_TRANSITION_LCTM2015 &&
      (!(scheme->turbulence == FEST_TURB_SST || scheme->turbulence == FEST_TURB_SST2003) || flow->mu_ref <= 0.0))
    return FEST_ERR_ARG;
  if (scheme->time_stepping_method != 'l' && scheme->time_stepping_method != 'g') return FEST_ERR_ARG;
  for (int f = 0; f < 6; ++f) {
    if (!valid_id(bc->id[f])) return FEST_ERR_ARG;
    if (bc->id[f] == -10 || bc->id[f] >= 0) {
      if (bc->partner_block[f] < 0 || bc->partner_face[f] < 0 || bc->partner_face[f] > 5 ||
          bc->partner_orient[f] < 0 || bc->partner_orient[f] > 7)
        return FEST_ERR_ARG;
      // the exchange copies interior layers 1..3 of the partner face
      int n = f / 2 == 0 ? dims->imx : f / 2 == 1 ? dims->jmx : dims->kmx;
      if (n - 1 < 3) return FEST_ERR_ARG;
      if (bc->partner_block[f] != bc->block_id) continue;  // another block: checked by the batch
      int pf = bc->partner_face[f];
      int na = (f / 2 == 0 ? dims->jmx : dims->imx), nb = (f / 2 == 2 ? dims->jmx : dims->kmx);
      int pa = (pf / 2 == 0 ? dims->jmx : dims->imx), pb = (pf / 2 == 2 ? dims->jmx : dims->kmx);
      if (bc->partner_orient[f] & 4) std::swap(pa, pb);
      if (na != pa || nb != pb) return FEST_ERR_ARG;
      int pn = pf / 2 == 0 ? dims->imx : pf / 2 == 1 ? dims->jmx : dims->kmx;
      if (pn - 1 < 3) return FEST_ERR_ARG;
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return FEST_ERR_NO_DEVICE;
  fest_handle* h = new fest_handle();
  h->ext = *dims;
  h->flow = *flow;
  h->sc = *scheme;
  h->bc = *bc;
  fill_params(h);
  int rc = FEST_OK;
  if (cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return FEST_ERR_CUDA;
  }
  h->own = h->s;
  if (cudaEventCreate(&h->kev[0]) != cudaSuccess || cudaEventCreate(&h->kev[1]) != cudaSuccess) {
    h->kev[0] = h->kev[1] = nullptr;
    cudaGetLastError();
  }
  const Dims& d = h->p.d;
  Sizes z = sizes_of(d, h->p.n_grad);
  DevBlock& b = h->d;
  auto A = [&](double** p, long long n) {
    if (rc == FEST_OK) rc = dalloc(h, p, n);
  };
  A(&b.qp, z.qp); A(&b.Temp, z.pad); A(&b.cells, z.cells); A(&b.nodes, z.nodes);
  for (int dir = 0; dir < 3; ++dir) {
    A(&b.faces[dir], z.faces[dir]);
    A(&b.fsL[dir], z.fs[dir]);
    A(&b.fsR[dir], z.fs[dir]);
    A(&b.flux[dir], z.fl[dir]);
    A(&b.grad[dir], z.grad);
  }
  A(&b.res, z.res); A(&b.mu, z.pad); A(&b.mut, z.pad); A(&b.F1, z.pad); A(&b.dist, z.pad);
  A(&b.dt, z.dt); A(&b.Ustore, z.qp); A(&b.Rstore, z.res); A(&b.red, kRedSlots);
  A(&h->d_resnorm, 16);
  if (rc == FEST_OK) {
    if (cudaMalloc((void**)&b.err, sizeof(int)) != cudaSuccess) rc = FEST_ERR_NOMEM;
    else {
      h->allocs.push_back(b.err);
      cudaMemsetAsync(b.err, 0, sizeof(int), h->s);
    }
    // pinned host word for the error check (without it finish() reads the
    // device word synchronously)
    if (cudaMallocHost((void**)&h->h_err, sizeof(int)) != cudaSuccess) {
      h->h_err = nullptr;
      cudaGetLastError();
    }
  }
  if (rc == FEST_OK) {
    // setup_viscosity: mu = mu_ref everywhere (viscosity.f90:562-566)
    k_fill<<<(unsigned)((z.pad + 255) / 256), 256, 0, h->s>>>(b.mu, z.pad, flow->mu_ref);
    ++h->launches;
    BlockRef self{b, d};
    if (cudaMalloc((void**)&h->d_table, sizeof(BlockRef)) != cudaSuccess) rc = FEST_ERR_NOMEM;
    else {
      h->allocs.push_back(h->d_table);
      cudaMemcpyAsync(h->d_table, &self, sizeof(BlockRef), cudaMemcpyHostToDevice, h->s);
    }
  }
  if (rc == FEST_OK) rc = finish(h);
  if (rc != FEST_OK) {
    fest_destroy(h);
    return rc;
  }
  *out = h;
  return FEST_OK;
}

int fest_destroy(fest_handle* h) {
  if (!h) return FEST_OK;
  if (h->s) cudaStreamSynchronize(h->s);
  cudaGetLastError();  // nothing of this handle's may linger for the next call
  if (h->snap_busy) cudaEventSynchronize(h->snap_ev[1]);
  if (h->snap_s) cudaStreamSynchronize(h->snap_s);
  cudaGetLastError();
  if (h->fused) fused_destroy(h->fused);
  for (void* p : h->allocs) cudaFree(p);
  if (h->own) cudaStreamDestroy(h->own);
  if (h->snap_s) cudaStreamDestroy(h->snap_s);
  if (h->h_err) cudaFreeHost(h->h_err);
  if (h->h_snap_err) cudaFreeHost(h->h_snap_err);
  for (cudaEvent_t e : h->snap_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : h->kev)
    if (e) cudaEventDestroy(e);
  delete h;
  return FEST_OK;
}

int fest_set_precision(fest_handle* h, int precision) {
  if (!h || (precision != FEST_FP64 && precision != FEST_MIXED)) return FEST_ERR_ARG;
  h->precision = precision;
  return FEST_OK;
}

int fest_last_device_error(fest_handle* h) {
  if (!h) return FEST_ERR_ARG;
  return finish(h);
}

long long fest_kernel_launches(const fest_handle* h) { return h ? h->launches : 0; }

long long fest_array_size(const fest_handle* h, int which) { return h ? arr_size(h, which) : 0; }

int fest_set_array(fest_handle* h, int which, const double* host) {
  if (!h || !host) return FEST_ERR_ARG;
  RET(sync_fused(h));
  double* d = arr_ptr(h, which);
  if (!d) return FEST_ERR_ARG;
  RET(up(h, d, host, arr_size(h, which)));
  return finish(h);
}

int fest_get_array(fest_handle* h, int which, double* host) {
  if (!h || !host) return FEST_ERR_ARG;
  RET(sync_fused(h));
  double* d = arr_ptr(h, which);
  if (!d) return FEST_ERR_ARG;
  RET(down(h, host, d, arr_size(h, which)));
  return finish(h);
}

// the fused path keeps FP32 copies of the metrics: new metrics retire it
// (its state goes back to qp first; it is rebuilt at the next fest_step)
static int drop_fused(fest_handle* h) {
  if (!h->fused) return FEST_OK;
  RET(sync_fused(h));
  CK(cudaStreamSynchronize(h->s));
  fused_destroy(h->fused);
  h->fused = nullptr;
  return FEST_OK;
}

int fest_setup_geometry(fest_handle* h, double* nodes, double* cells, double* Ifaces,
                        double* Jfaces, double* Kfaces) {
  if (!h || !nodes) return FEST_ERR_ARG;
  RET(drop_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.nodes, nodes, z.nodes));
  launch_geometry(h->p, h->d, h->L());
  RET(down(h, nodes, h->d.nodes, z.nodes));
  RET(down(h, cells, h->d.cells, z.cells));
  RET(down(h, Ifaces, h->d.faces[0], z.faces[0]));
  RET(down(h, Jfaces, h->d.faces[1], z.faces[1]));
  RET(down(h, Kfaces, h->d.faces[2], z.faces[2]));
  return finish(h);
}

int fest_set_metrics(fest_handle* h, const double* cells, const double* Ifaces,
                     const double* Jfaces, const double* Kfaces) {
  if (!h) return FEST_ERR_ARG;
  RET(drop_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.cells, cells, z.cells));
  RET(up(h, h->d.faces[0], Ifaces, z.faces[0]));
  RET(up(h, h->d.faces[1], Jfaces, z.faces[1]));
  RET(up(h, h->d.faces[2], Kfaces, z.faces[2]));
  return finish(h);
}

int fest_find_wall_dist(fest_handle* h, const double* wall_xyz, int n_wall, double* dist) {
  if (!h || !wall_xyz || n_wall <= 0) return FEST_ERR_ARG;
  RET(drop_fused(h));  // the SST sweep keeps an FP32 copy of the distances
  const Dims& d = h->p.d;
  if (n_wall > h->n_wall_cap) {
    if (h->d_wall) cudaFree(h->d_wall);
    CK(cudaMalloc((void**)&h->d_wall, sizeof(double) * 3 * (size_t)n_wall));
    h->n_wall_cap = n_wall;
  }
  if (!h->d_nodedist) RET(dalloc(h, &h->d_nodedist, (long long)(d.imx + 6) * (d.jmx + 6) * (d.kmx + 6)));
  RET(up(h, h->d_wall, wall_xyz, 3LL * n_wall));
  launch_wall_dist(h->p, h->d, h->d_wall, n_wall, h->d_nodedist, h->L());
  RET(down(h, dist, h->d.dist, d.P));
  int rc = finish(h);
  cudaFree(h->d_wall);
  h->d_wall = nullptr;
  h->n_wall_cap = 0;
  return rc;
}

int fest_set_wall_dist(fest_handle* h, const double* dist) {
  if (!h || !dist) return FEST_ERR_ARG;
  RET(drop_fused(h));
  RET(up(h, h->d.dist, dist, h->p.d.P));
  return finish(h);
}

int fest_upload_state(fest_handle* h, const double* qp) {
  if (!h || !qp) return FEST_ERR_ARG;
  RET(up(h, h->d.qp, qp, h->p.d.P * h->p.d.nv));
  if (h->fused) fused_invalidate(h->fused);
  return finish(h);
}

int fest_download_state(fest_handle* h, double* qp) {
  if (!h || !qp) return FEST_ERR_ARG;
  // reading leaves the fused path's buffers as they are (no re-seeding at
  // the next step)
  const double* cur = fused_current_state(h->fused);
  RET(down(h, qp, cur ? cur : h->d.qp, h->p.d.P * h->p.d.nv));
  return finish(h);
}

// checkpoint (dump_solution.f90:27-52) without stopping the stepping: the
// current state is copied on the device, in stream order after the work
// already enqueued, and the copy crosses the link on a stream of its own,
// so that steps enqueued after this call run while it travels.  The error
// word is copied beside the state: a snapshot of a failed step says so.
int fest_snapshot_begin(fest_handle* h, double* qp_host) {
  if (!h || !qp_host || h->snap_busy) return FEST_ERR_ARG;
  const long long n = h->p.d.P * h->p.d.nv;
  // the copy stream, its events and the pinned error word, made once (a
  // part that failed is made again at the next call)
  if (!h->snap_s) CK(cudaStreamCreateWithFlags(&h->snap_s, cudaStreamNonBlocking));
  for (cudaEvent_t& e : h->snap_ev)
    if (!e) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  if (!h->h_snap_err) CK(cudaMallocHost((void**)&h->h_snap_err, sizeof(int)));
  if (!h->d_snap) RET(dalloc(h, &h->d_snap, n + 1));
  const double* cur = fused_current_state(h->fused);
  CK(cudaMemcpyAsync(h->d_snap, cur ? cur : h->d.qp, sizeof(double) * (size_t)n,
                     cudaMemcpyDeviceToDevice, h->s));
  CK(cudaMemcpyAsync(h->d_snap + n, h->d.err, sizeof(int), cudaMemcpyDeviceToDevice, h->s));
  CK(cudaEventRecord(h->snap_ev[0], h->s));
  CK(cudaStreamWaitEvent(h->snap_s, h->snap_ev[0], 0));
  CK(cudaMemcpyAsync(qp_host, h->d_snap, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost,
                     h->snap_s));
  CK(cudaMemcpyAsync(h->h_snap_err, h->d_snap + n, sizeof(int), cudaMemcpyDeviceToHost,
                     h->snap_s));
  CK(cudaEventRecord(h->snap_ev[1], h->snap_s));
  h->snap_busy = true;
  return FEST_OK;
}

int fest_snapshot_wait(fest_handle* h) {
  if (!h) return FEST_ERR_ARG;
  if (!h->snap_busy) return FEST_OK;
  h->snap_busy = false;
  CK(cudaEventSynchronize(h->snap_ev[1]));
  return *h->h_snap_err;
}

int fest_populate_ghost_primitive(fest_handle* h, double* qp, int current_iter) {
  if (!h || needs_batch(h)) return FEST_ERR_ARG;
  RET(sync_fused(h));
  long long n = h->p.d.P * h->p.d.nv;
  RET(up(h, h->d.qp, qp, n));
  launch_ghosts(h->p, h->d, h->d_table, current_iter, h->L());
  RET(down(h, qp, h->d.qp, n));
  return finish(h);
}

int fest_compute_temperature(fest_handle* h, const double* qp, double* Temp) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  RET(up(h, h->d.qp, qp, h->p.d.P * h->p.d.nv));
  launch_temperature(h->p, h->d, h->L());
  RET(down(h, Temp, h->d.Temp, h->p.d.P));
  return finish(h);
}

static int face_state_call(fest_handle* h, const double* qp, double* xl, double* xr, double* yl,
                           double* yr, double* zl, double* zr, int mode) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  double* hs[6] = {xl, xr, yl, yr, zl, zr};
  if (mode == 2)
    for (int m = 0; m < 6; ++m) RET(up(h, m % 2 ? h->d.fsR[m / 2] : h->d.fsL[m / 2], hs[m], z.fs[m / 2]));
  launch_face_states(h->p, h->d, mode, h->L());
  for (int m = 0; m < 6; ++m) RET(down(h, hs[m], m % 2 ? h->d.fsR[m / 2] : h->d.fsL[m / 2], z.fs[m / 2]));
  return finish(h);
}

int fest_compute_face_interpolant(fest_handle* h, const double* qp, double* xl, double* xr,
                                  double* yl, double* yr, double* zl, double* zr) {
  return face_state_call(h, qp, xl, xr, yl, yr, zl, zr, 0);
}

int fest_reconstruct_boundary_state(fest_handle* h, const double* qp, double* xl, double* xr,
                                    double* yl, double* yr, double* zl, double* zr) {
  return face_state_call(h, qp, xl, xr, yl, yr, zl, zr, 2);
}

int fest_compute_fluxes(fest_handle* h, double* F, double* G, double* H) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  launch_fluxes(h->p, h->d, h->L());
  RET(down(h, F, h->d.flux[0], z.fl[0]));
  RET(down(h, G, h->d.flux[1], z.fl[1]));
  RET(down(h, H, h->d.flux[2], z.fl[2]));
  return finish(h);
}

int fest_evaluate_all_gradients(fest_handle* h, const double* qp, const double* Temp,
                                double* gx, double* gy, double* gz) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  RET(up(h, h->d.Temp, Temp, z.pad));
  launch_gradients(h->p, h->d, h->L());
  RET(down(h, gx, h->d.grad[0], z.grad));
  RET(down(h, gy, h->d.grad[1], z.grad));
  RET(down(h, gz, h->d.grad[2], z.grad));
  return finish(h);
}

int fest_calculate_viscosity(fest_handle* h, const double* qp, double* mu, double* mu_t,
                             double* sst_F1) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  launch_viscosity(h->p, h->d, h->L());
  RET(down(h, mu, h->d.mu, z.pad));
  RET(down(h, mu_t, h->d.mut, z.pad));
  RET(down(h, sst_F1, h->d.F1, z.pad));
  return finish(h);
}

int fest_compute_viscous_fluxes(fest_handle* h, const double* qp, double* F, double* G, double* H) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  RET(up(h, h->d.flux[0], F, z.fl[0]));
  RET(up(h, h->d.flux[1], G, z.fl[1]));
  RET(up(h, h->d.flux[2], H, z.fl[2]));
  launch_viscous_fluxes(h->p, h->d, h->L());
  RET(down(h, F, h->d.flux[0], z.fl[0]));
  RET(down(h, G, h->d.flux[1], z.fl[1]));
  RET(down(h, H, h->d.flux[2], z.fl[2]));
  return finish(h);
}

int fest_compute_residue(fest_handle* h, const double* F, const double* G, const double* H,
                         double* residue) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.flux[0], F, z.fl[0]));
  RET(up(h, h->d.flux[1], G, z.fl[1]));
  RET(up(h, h->d.flux[2], H, z.fl[2]));
  launch_residue(h->p, h->d, false, h->L());
  RET(down(h, residue, h->d.res, z.res));
  return finish(h);
}

int fest_add_source_term_residue(fest_handle* h, const double* qp, double* residue) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  RET(up(h, h->d.res, residue, z.res));
  launch_source(h->p, h->d, h->L());
  RET(down(h, residue, h->d.res, z.res));
  return finish(h);
}

int fest_compute_time_step(fest_handle* h, const double* qp, double CFL, double* delta_t) {
  if (!h) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  launch_time_step(h->p, h->d, CFL, h->L());
  RET(down(h, delta_t, h->d.dt, z.dt));
  return finish(h);
}

int fest_get_total_conservative_residue(fest_handle* h, double* qp, int current_iter,
                                        double* residue) {
  if (!h || needs_batch(h)) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  kmark(h, 0);
  RET(residual_fp64(h, current_iter));
  kmark(h, 1);
  RET(down(h, qp, h->d.qp, z.qp));
  RET(down(h, residue, h->d.res, z.res));
  return finish(h);
}

// laminar blocks: the primal's temperature, gradients (with their BCs) and
// viscosity at the resident state, which the residual's VJP reads
static int viscous_prep(fest_handle* h) {
  if (h->p.mu_ref == 0.0) return FEST_OK;
  if (!h->d_vjp_grad)
    RET(dalloc(h, &h->d_vjp_grad, vjp_grad_work_doubles(h->p.d, h->p.turb != FEST_TURB_NONE)));
  launch_temperature(h->p, h->d, h->L());
  launch_gradients(h->p, h->d, h->L());
  launch_viscosity(h->p, h->d, h->L());
  return FEST_OK;
}

int fest_residual_vjp(fest_handle* h, const double* qp, int current_iter, const double* lambda,
                      double* dq) {
  if (!h || !lambda || !dq) return FEST_ERR_ARG;
  if (!vjp_supported(h->p) || needs_batch(h)) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  if (!h->d_vjp_bar) RET(dalloc(h, &h->d_vjp_bar, z.qp));
  if (!h->d_vjp_lam) RET(dalloc(h, &h->d_vjp_lam, z.res));
  if (!h->d_vjp_face) RET(dalloc(h, &h->d_vjp_face, vjp_face_work_doubles(h->p.d)));
  if (qp) RET(up(h, h->d.qp, qp, z.qp));
  RET(up(h, h->d_vjp_lam, lambda, z.res));
  kmark(h, 0);
  launch_ghosts(h->p, h->d, h->d_table, current_iter, h->L());
  RET(viscous_prep(h));
  launch_residual_vjp(h->p, h->d, current_iter, h->d_vjp_lam, h->d_vjp_bar, h->L(), nullptr, h->d_vjp_grad,
                      h->d_vjp_face);
  kmark(h, 1);
  RET(down(h, dq, h->d_vjp_bar, z.qp));
  return finish(h);
}

int fest_residual_vjp_nodes(fest_handle* h, const double* qp, int current_iter, const double* lambda,
                            const double* Ifaces_bar, const double* Jfaces_bar,
                            const double* Kfaces_bar, double* dq, double* dnodes) {
  if (!h || !dnodes || needs_batch(h)) return FEST_ERR_ARG;
  // metric adjoints of inviscid and laminar residuals (SST: the wall
  // distances depend on the nodes too)
  if (!vjp_supported(h->p) || h->p.interp == FEST_INTERP_WENO_NM || h->p.turb != FEST_TURB_NONE)
    return FEST_ERR_ARG;
  const bool visc = h->p.mu_ref != 0.0;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  if (!h->d_vjp_bar) RET(dalloc(h, &h->d_vjp_bar, z.qp));
  if (!h->d_vjp_lam) RET(dalloc(h, &h->d_vjp_lam, z.res));
  if (!h->d_vjp_face) RET(dalloc(h, &h->d_vjp_face, vjp_face_work_doubles(h->p.d)));
  // the handle keeps the gradient work array (viscous_prep would allocate
  // it among this call's own temporaries otherwise)
  if (visc && !h->d_vjp_grad) RET(dalloc(h, &h->d_vjp_grad, vjp_grad_work_doubles(h->p.d, false)));
  const size_t n0 = h->allocs.size();
  double *bf[3] = {nullptr, nullptr, nullptr}, *bn = nullptr, *bc = nullptr;
  int rc = FEST_OK;
  for (int dir = 0; dir < 3 && !rc; ++dir) rc = dalloc(h, &bf[dir], z.faces[dir]);
  if (!rc) rc = dalloc(h, &bn, z.nodes);
  if (!rc && visc) rc = dalloc(h, &bc, z.cells);
  const double* fin[3] = {Ifaces_bar, Jfaces_bar, Kfaces_bar};
  for (int dir = 0; dir < 3 && !rc; ++dir)
    if (fin[dir]) rc = up(h, bf[dir], fin[dir], z.faces[dir]);
  if (!rc && qp) rc = up(h, h->d.qp, qp, z.qp);
  if (!rc && lambda) rc = up(h, h->d_vjp_lam, lambda, z.res);
  else if (!rc) rc = cuda_status(cudaMemsetAsync(h->d_vjp_lam, 0, sizeof(double) * z.res, h->s));
  if (!rc) {
    launch_ghosts(h->p, h->d, h->d_table, current_iter, h->L());
    rc = viscous_prep(h);
  }
  if (!rc) {
    launch_residual_vjp(h->p, h->d, current_iter, h->d_vjp_lam, h->d_vjp_bar, h->L(), bf, h->d_vjp_grad,
                        h->d_vjp_face, bc);
    launch_geometry_vjp(h->p, h->d, bf, bn, h->L(), bc);
    rc = down(h, dnodes, bn, z.nodes);
  }
  if (!rc && dq) rc = down(h, dq, h->d_vjp_bar, z.qp);
  if (!rc) rc = finish(h);
  cudaStreamSynchronize(h->s);
  while (h->allocs.size() > n0) {
    cudaFree(h->allocs.back());
    h->allocs.pop_back();
  }
  return rc;
}

int fest_adjoint_solve(fest_handle* h, const double* dJdq, double CFL, int max_iters, double tol,
                       double* psi, int* n_done, double* drop) {
  if (!h || !dJdq || max_iters < 0) return FEST_ERR_ARG;
  if (!vjp_supported(h->p) || h->p.tstep != 'l' || needs_batch(h)) return FEST_ERR_ARG;
  if (h->p.integ != FEST_TIME_NONE && h->p.integ != FEST_TIME_TVDRK3) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  if (!h->d_vjp_bar) RET(dalloc(h, &h->d_vjp_bar, z.qp));
  if (!h->d_vjp_lam) RET(dalloc(h, &h->d_vjp_lam, z.res));
  // the handle keeps this one: allocated before the solve's own work arrays,
  // which release() frees
  if (h->p.mu_ref != 0.0 && !h->d_vjp_grad)
    RET(dalloc(h, &h->d_vjp_grad, vjp_grad_work_doubles(h->p.d, h->p.turb != FEST_TURB_NONE)));
  if (!h->d_vjp_face) RET(dalloc(h, &h->d_vjp_face, vjp_face_work_doubles(h->p.d)));
  AdjointWork w{};
  w.bar = h->d_vjp_bar;
  w.mu = h->d_vjp_lam;
  w.face = h->d_vjp_face;
  const size_t n0 = h->allocs.size();
  int rc = FEST_OK;
  for (double** x : {&w.phi, &w.dJ, &w.a, &w.b, &w.c})
    if (!rc) rc = dalloc(h, x, z.qp);
  if (!rc) rc = dalloc(h, &w.sq, 1);
  auto release = [&]() {  // the work arrays are the allocations made here
    cudaStreamSynchronize(h->s);
    while (h->allocs.size() > n0) {
      cudaFree(h->allocs.back());
      h->allocs.pop_back();
    }
  };
  if (!rc) rc = up(h, w.dJ, dJdq, z.qp);
  // the frozen primal: ghost cells, face states, (laminar) temperature,
  // gradients and viscosity, and the local time step
  if (!rc) rc = residual_fp64(h, 3);
  if (!rc) rc = viscous_prep(h);
  w.grad = h->d_vjp_grad;
  if (!rc) launch_time_step(h->p, h->d, CFL, h->L());
  Launcher L = h->L();
  double first = -1.0, last = 0.0;
  int it = 0;
  while (!rc && it < max_iters) {
    const int chunk = std::min(20, max_iters - it);
    cudaMemsetAsync(w.sq, 0, sizeof(double), h->s);
    for (int n = 0; n < chunk; ++n) launch_adjoint_iteration(h->p, h->d, w, L);
    it += chunk;
    double s2 = 0.0;
    rc = down(h, &s2, w.sq, 1);
    if (!rc) rc = finish(h);
    if (rc) break;
    last = sqrt(s2 / chunk);
    if (first < 0.0) first = last;
    if (!(last == last)) { rc = FEST_ERR_NAN; break; }
    if (first > 0.0 && last <= tol * first) break;
  }
  if (!rc && psi) {
    launch_adjoint_psi(h->p, h->d, w, w.mu, L);
    rc = down(h, psi, w.mu, z.res);
    if (!rc) rc = finish(h);
  }
  if (n_done) *n_done = it;
  if (drop) *drop = first > 0.0 ? last / first : 0.0;
  release();
  return rc;
}

int fest_get_next_solution(fest_handle* h, double* qp, int current_iter, double CFL,
                           double* residue, double* delta_t) {
  if (!h || needs_batch(h)) return FEST_ERR_ARG;
  RET(sync_fused(h));
  Sizes z = sizes_of(h->p.d, h->p.n_grad);
  RET(up(h, h->d.qp, qp, z.qp));
  RET(next_solution_fp64(h, current_iter, CFL));
  RET(down(h, qp, h->d.qp, z.qp));
  RET(down(h, residue, h->d.res, z.res));
  RET(down(h, delta_t, h->d.dt, z.dt));
  return finish(h);
}

// setup_scale (resnorm.f90:128-169) and assemble (resnorm.f90:211-225)
// from the device sums of find_resnorm
static void resnorm_assemble(const fest_handle* h, const double* sums, double* res_abs) {
  const fest_flow& f = h->flow;
  double sc[NVMOD + 1];
  sc[0] = 1.;
  sc[1] = f.density_inf * f.vel_mag;
  sc[2] = sc[3] = sc[4] = f.density_inf * f.vel_mag * f.vel_mag;
  sc[5] = (0.5 * f.density_inf * (f.vel_mag * f.vel_mag * f.vel_mag) +
           ((f.gm / (f.gm - 1.)) * f.pressure_inf));
  // resnorm.f90:155-163: the sixth variable's scale is tv_inf's for SA
  sc[6] = f.density_inf * f.vel_mag * (h->sc.turbulence == FEST_TURB_SA ? f.tv_inf : f.tk_inf);
  sc[7] = f.density_inf * f.vel_mag * (h->sc.turbulence == FEST_TURB_KKL ? f.tkl_inf : f.tw_inf);
  // setup_scale (resnorm.f90:128-167) sets no scale for LCTM2015's
  // intermittency: its norm is taken unscaled
  sc[8] = 1.0;
  res_abs[0] = fabs(sums[0] / sc[0]);
  for (int l = 1; l <= h->p.d.nv; ++l) res_abs[l] = sqrt(sums[l] / (sc[l] * sc[l]));
}

int fest_find_resnorm(fest_handle* h, double* res_abs) {
  if (!h || !res_abs) return FEST_ERR_ARG;
  launch_resnorm(h->p, h->d, h->d_resnorm, h->L());
  double sums[NVMOD + 1];
  RET(down(h, sums, h->d_resnorm, h->p.d.nv + 1));
  RET(finish(h));
  resnorm_assemble(h, sums, res_abs);
  return FEST_OK;
}

static int step_enqueue(fest_handle* h, int n_iters, int first_iter, double CFL) {
  if (!h || n_iters < 0 || needs_batch(h)) return FEST_ERR_ARG;
  if (fused_supported(h->p, h->precision)) {
    if (!h->fused) RET(fused_create(h->p, h->d, h->d_table, h->s, &h->fused));
    return fused_run(h->fused, h->p, h->d, h->precision, n_iters, first_iter, CFL, h->s,
                     &h->launches);
  }
  if (h->precision == FEST_MIXED) return FEST_ERR_ARG;  // mixed needs the fused sweep
  RET(sync_fused(h));
  for (int n = 0; n < n_iters; ++n) RET(next_solution_fp64(h, first_iter + n, CFL));
  return FEST_OK;
}

int fest_step(fest_handle* h, int n_iters, int first_iter, double CFL, double* res_abs) {
  if (h) kmark(h, 0);
  RET(step_enqueue(h, n_iters, first_iter, CFL));
  kmark(h, 1);
  if (res_abs) return fest_find_resnorm(h, res_abs);
  return finish(h);
}

int fest_step_async(fest_handle* h, int n_iters, int first_iter, double CFL) {
  return step_enqueue(h, n_iters, first_iter, CFL);
}

int fest_step_host_interior(fest_handle* h, double* q, int n_iters, int first_iter, double CFL,
                            double* res_abs) {
  if (!h || !q || n_iters < 0 || needs_batch(h)) return FEST_ERR_ARG;
  // the interior goes into the state the next step reads, whose ghost
  // cells (the persistent fix() layers among them) are the handle's own:
  // the fused path's current buffer and FP32 mirror in place, or, before
  // the fused path has a state, the primary state
  const double* src = nullptr;
  RET(interior_source(h, q, &src));
  if (!(h->fused && fused_import_interior(h->fused, src, h->s, &h->launches) == FEST_OK)) {
    RET(sync_fused(h));
    RET(interior_copy(h, src, h->d.qp, 1));
    if (h->fused) fused_invalidate(h->fused);
  }
  kmark(h, 0);
  RET(step_enqueue(h, n_iters, first_iter, CFL));
  double sums[NVMOD + 1];
  if (res_abs) {
    launch_resnorm(h->p, h->d, h->d_resnorm, h->L());
    RET(down(h, sums, h->d_resnorm, h->p.d.nv + 1));
  }
  kmark(h, 1);
  const double* cur = fused_current_state(h->fused);
  RET(down_interior(h, q, cur ? cur : h->d.qp));
  RET(finish(h));
  if (res_abs) resnorm_assemble(h, sums, res_abs);
  return FEST_OK;
}

int fest_step_host(fest_handle* h, double* qp, int n_iters, int first_iter, double CFL, double* res_abs) {
  if (!h || !qp || n_iters < 0 || needs_batch(h)) return FEST_ERR_ARG;
  const long long n = h->p.d.P * h->p.d.nv;
  RET(up(h, h->d.qp, qp, n));
  if (h->fused) fused_invalidate(h->fused);
  kmark(h, 0);
  RET(step_enqueue(h, n_iters, first_iter, CFL));
  double sums[NVMOD + 1];
  if (res_abs) {
    launch_resnorm(h->p, h->d, h->d_resnorm, h->L());
    RET(down(h, sums, h->d_resnorm, h->p.d.nv + 1));
  }
  kmark(h, 1);
  const double* cur = fused_current_state(h->fused);
  RET(down(h, qp, cur ? cur : h->d.qp, n));
  RET(finish(h));
  if (res_abs) resnorm_assemble(h, sums, res_abs);
  return FEST_OK;
}

struct fest_batch {
  std::vector<fest_handle*> h;
  std::vector<cudaStream_t> prev;  // each handle's stream before the batch
  FusedBatch* fb = nullptr;
  // implicit batches (module path): the blocks' parameters with batch
  // indices for their partners, and the table of every block's state
  bool implicit = false;
  std::vector<Params> p;
  BlockRef* d_tab = nullptr;
};

int fest_batch_create(fest_handle* const* blocks, int n_blocks, fest_batch** out) {
  if (!out) return FEST_ERR_ARG;
  *out = nullptr;
  if (!blocks || n_blocks < 1) return FEST_ERR_ARG;
  fest_handle* h0 = blocks[0];
  if (!h0) return FEST_ERR_ARG;
  const int prec = h0->precision;
  const int integ0 = h0->sc.time_step_accuracy;
  const bool implicit = integ0 == FEST_TIME_IMPLICIT || integ0 == FEST_TIME_PLUSGS;
  for (int n = 0; n < n_blocks; ++n) {
    fest_handle* h = blocks[n];
    if (!h || h->precision != prec) return FEST_ERR_ARG;
    if (implicit) {  // LU-SGS: FP64 module path, every block implicit
      if (prec != FEST_FP64 || h->sc.time_step_accuracy != integ0) return FEST_ERR_ARG;
    } else if (!fused_supported(h->p, prec)) {
      return FEST_ERR_ARG;
    }
  }
  // interface partners as batch indices: the block itself, or the one
  // other handle whose block_id is the face's partner_block
  std::vector<Params> p(n_blocks);
  for (int n = 0; n < n_blocks; ++n) {
    const fest_handle* h = blocks[n];
    p[n] = h->p;
    p[n].self_block = n;
    for (int f = 0; f < 6; ++f) {
      if (!(h->bc.id[f] == -10 || h->bc.id[f] >= 0)) continue;
      const int pb = h->bc.partner_block[f];
      if (pb == h->bc.block_id) {
        p[n].part_block[f] = n;
        continue;
      }
      int m = -1;
      for (int k = 0; k < n_blocks; ++k)
        if (k != n && blocks[k]->bc.block_id == pb) {
          if (m >= 0) return FEST_ERR_ARG;  // two blocks with that number
          m = k;
        }
      if (m < 0) return FEST_ERR_ARG;
      // the partner face has this face's columns (swapped with dir_switch)
      // and the three interior layers the exchange copies
      int na, nb, pa, pc;
      face_columns(h->p.d, f, na, nb);
      const int pf = h->bc.partner_face[f];
      face_columns(blocks[m]->p.d, pf, pa, pc);
      if (h->bc.partner_orient[f] & 4) std::swap(pa, pc);
      if (na != pa || nb != pc || extent_of(blocks[m]->p.d, pf / 2) - 1 < 3) return FEST_ERR_ARG;
      p[n].part_block[f] = m;
    }
  }
  std::vector<FusedState*> f;
  std::vector<DevBlock> d;
  fest_batch* b = new fest_batch();
  int rc = FEST_OK;
  for (int n = 0; n < n_blocks && !rc; ++n) {
    fest_handle* h = blocks[n];
    // one stream for the whole batch: the first block's current one
    rc = cuda_status(cudaStreamSynchronize(h->s));
    b->h.push_back(h);
    b->prev.push_back(h->s);
    h->s = h0->s;
    if (!implicit && !rc && !h->fused) rc = fused_create(h->p, h->d, h->d_table, h->s, &h->fused);
    f.push_back(h->fused);
    d.push_back(h->d);
  }
  if (!rc && implicit) {
    b->implicit = true;
    b->p = p;
    std::vector<BlockRef> t(n_blocks);
    for (int n = 0; n < n_blocks; ++n) t[n] = BlockRef{d[n], p[n].d};
    if (cudaMalloc((void**)&b->d_tab, sizeof(BlockRef) * n_blocks) != cudaSuccess) rc = FEST_ERR_NOMEM;
    else rc = cuda_status(cudaMemcpy(b->d_tab, t.data(), sizeof(BlockRef) * n_blocks, cudaMemcpyHostToDevice));
  } else if (!rc) {
    rc = fused_batch_create(f, p, d, prec, &b->fb);
  }
  if (rc) {
    fest_batch_destroy(b);
    return rc;
  }
  *out = b;
  return FEST_OK;
}

int fest_batch_destroy(fest_batch* b) {
  if (!b) return FEST_OK;
  if (!b->h.empty()) cudaStreamSynchronize(b->h[0]->s);
  fused_batch_destroy(b->fb);
  if (b->d_tab) cudaFree(b->d_tab);
  for (size_t n = 0; n < b->h.size(); ++n) b->h[n]->s = b->prev[n];  // handles get their streams back
  delete b;
  return FEST_OK;
}

int fest_batch_step_async(fest_batch* b, int n_iters, int first_iter, double CFL) {
  if (!b || n_iters < 0) return FEST_ERR_ARG;
  fest_handle* h0 = b->h[0];
  for (fest_handle* h : b->h)
    if (h->s != h0->s || h->precision != h0->precision) return FEST_ERR_ARG;
  if (b->implicit) {
    // the blocks in lockstep: every residual (whose ghost fills read the
    // other blocks' states) before any block's LU-SGS update changes its own
    const size_t nb = b->h.size();
    for (int n = 0; n < n_iters; ++n) {
      const int it = first_iter + n;
      for (size_t m = 0; m < nb; ++m) RET(sync_fused(b->h[m]));
      for (size_t m = 0; m < nb; ++m) launch_temperature(b->p[m], b->h[m]->d, b->h[m]->L());
      for (size_t m = 0; m < nb; ++m) {
        RET(residual_module(b->h[m], it, b->p[m], b->d_tab));
        launch_time_step(b->p[m], b->h[m]->d, CFL, b->h[m]->L());
      }
      for (size_t m = 0; m < nb; ++m) RET(lusgs_update(b->h[m], b->p[m]));
    }
    return FEST_OK;
  }
  return fused_batch_run(b->fb, n_iters, first_iter, CFL, h0->s, &h0->launches);
}

int fest_batch_step(fest_batch* b, int n_iters, int first_iter, double CFL) {
  RET(fest_batch_step_async(b, n_iters, first_iter, CFL));
  for (fest_handle* h : b->h) RET(finish(h));
  return FEST_OK;
}

int fest_set_stream(fest_handle* h, void* stream) {
  if (!h) return FEST_ERR_ARG;
  CK(cudaStreamSynchronize(h->s));
  h->s = stream ? (cudaStream_t)stream : h->own;
  return FEST_OK;
}

int fest_profile(fest_handle* h, int enable) {
  if (!h || needs_batch(h)) return FEST_ERR_ARG;
  if (!h->fused && fused_supported(h->p, h->precision))
    RET(fused_create(h->p, h->d, h->d_table, h->s, &h->fused));
  fused_profile(h->fused, enable != 0);
  return FEST_OK;
}

int fest_profile_read(fest_handle* h, long long* launches, double* total_ms) {
  if (!h || !h->fused) return FEST_ERR_ARG;
  return fused_profile_read(h->fused, launches, total_ms);
}

int fest_last_kernel_ms(fest_handle* h, double* ms) {
  if (!h || !ms || !h->kev[0] || !h->kev[1]) return FEST_ERR_ARG;
  CK(cudaEventSynchronize(h->kev[1]));
  float t = 0.f;
  CK(cudaEventElapsedTime(&t, h->kev[0], h->kev[1]));
  *ms = t;
  return FEST_OK;
}

}  // extern "C"
