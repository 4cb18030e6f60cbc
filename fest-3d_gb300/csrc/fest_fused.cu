// fest_fused.cu - fused RK-stage sweep for inviscid blocks.
//
// One kernel per RK stage does, for a tile of cells, what the reference
// spreads over compute_face_interpolant, reconstruct_boundary_state,
// compute_fluxes, compute_residue, compute_time_step (stage 1) and
// update_with (update.f90:129-547): nothing between the state read and the
// state write touches HBM except the metrics.
//
// Tile: a CTA of 32x8 threads covers 30 interior cells in i (lanes 1..30,
// lanes 0/31 are the i-halo) by 6 in j (warps 1..6, warps 0/7 the j-halo)
// and marches along k.  A 5-plane ring in shared memory holds the stencil
// (planes k-2..k+2, 36x12 cells each, converted to the arithmetic type on
// load).  i-face fluxes are exchanged with warp shuffles, j-face fluxes
// through shared memory, k-face fluxes stay in registers across the march.
//
// T = float  (FEST_MIXED): reconstruction, flux, residual and the update's
//             increments in FP32; the state stays FP64 and is advanced by
//             adding an FP64 increment (delta form), metrics are read FP64.
// T = double (FEST_FP64): the reference's arithmetic, update_with verbatim.
#include <algorithm>
#include <vector>

#include "fest_fused.cuh"

namespace fest {

namespace {

constexpr int TX = 32, TY = 8;        // threads per CTA
constexpr int IX = TX - 2, IY = TY - 2;  // interior cells per CTA
constexpr int SW = TX + 4, SH = TY + 4;  // stencil plane extents (halo 2)
constexpr int NRING = 5;

struct StageArgs {
  const double* qin;    // stencil state (padded, ghosts filled)
  double* qout;         // output state (interior written)
  const double* qbase;  // state the update starts from (qin, or U_store for RK2/4)
  const double* qU;     // blend source (U_store) when bA != 0
  double bA, bB;        // out = bA*U + bB*updated (TVD-RK blends)
  double TF, SF;        // update_with time/store factors
  int TU, use_rn;       // RK2/RK4 residual accumulation
  double* Rn;           // accumulator (interior, nv)
  double* dt;           // local time step (interior)
  int compute_dt;
  double CFL;
  double* res_out;      // nullable: FP64 residual of this stage (interior)
  double* mflux[3];     // nullable: boundary mass fluxes (F,G,H var 1)
  const double* faces[3];
  const double* cells;
  int* err;
};

template <typename T> struct SmemLine {
  const T* p;   // element of normal coordinate c0
  int c0, stride;
  __device__ __forceinline__ T operator()(int c) const { return p[(c - c0) * stride]; }
};
template <typename T> struct RingLine {
  const T* ring;  // ring + var/row/col offset; plane c lives in slot (c+2)%5
  int plane_stride;
  __device__ __forceinline__ T operator()(int c) const { return ring[((c + 2) % NRING) * plane_stride]; }
};
struct VolLine {
  const double* p;  // cells + 4*pidx(cell at normal coordinate 0)
  long long stride;
  int n;            // extent along the line: coordinates clamp to [-2, n+2]
  __device__ __forceinline__ double operator()(int c) const {
    c = c < -2 ? -2 : (c > n + 2 ? n + 2 : c);
    return p[4 * c * stride];
  }
};
template <typename T> struct VolLineT {
  VolLine v;
  __device__ __forceinline__ T operator()(int c) const { return (T)v(c); }
};

template <typename T>
__device__ __forceinline__ void load_face(const double* faces, long long idx, T& A, T& nx, T& ny, T& nz) {
  const double2* f2 = reinterpret_cast<const double2*>(faces + 4 * idx);
  double2 a = __ldg(f2), b = __ldg(f2 + 1);
  A = (T)a.x; nx = (T)a.y; ny = (T)b.x; nz = (T)b.y;
}

// sound-speed term of compute_local_time_step (time.f90:167-231) for a face
template <typename T>
__device__ __forceinline__ T lambda_face(T gm, const T* L, const T* R, T A, T nx, T ny, T nz, T u,
                                         T v, T w) {
  T c = T(0.5) * (sqrt(gm * L[4] / L[0]) + sqrt(gm * R[4] / R[0]));
  return A * (fabs((u * nx) + (v * ny) + (w * nz)) + c);
}

// ---- the update of one cell -------------------------------------------------
// FP64: update_with(...,'conservative',...) (update.f90:367-485) verbatim.
__device__ __forceinline__ bool update_cell(const Params& p, const StageArgs& a, long long c0,
                                            long long ci, const double* R_in, double dtc,
                                            double vol) {
  const long long P = p.d.P, N = ncells(p.d);
  const double gm = p.gm;
  double R[5], u1[5], u2[5];
#pragma unroll
  for (int l = 0; l < 5; ++l) R[l] = R_in[l];
  u1[0] = a.qbase[c0];
#pragma unroll
  for (int l = 1; l < 5; ++l) u1[l] = a.qbase[c0 + P * l] * u1[0];
  double s1 = u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3];
  u1[4] = (u1[4] / (gm - 1.) + 0.5 * s1) / u1[0];
  if (a.use_rn) {
#pragma unroll
    for (int l = 0; l < 5; ++l) {
      double rn = a.Rn[ci + N * l] + a.SF * R[l];
      a.Rn[ci + N * l] = rn;
      if (a.TU) R[l] = rn;
    }
  }
  const double fac = (a.TF * dtc / vol);
#pragma unroll
  for (int l = 0; l < 5; ++l) u2[l] = u1[l] - R[l] * fac;
#pragma unroll
  for (int l = 1; l < 5; ++l) u2[l] = u2[l] / u2[0];
  double s2 = u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3];
  u2[4] = (gm - 1.) * u2[0] * (u2[4] - (0.5 * s2));
  bool bad = (u2[0] < 0.) || (u2[4] < 0.);
#pragma unroll
  for (int l = 0; l < 5; ++l) bad |= (u2[l] != u2[l]);
  if (bad) return false;
#pragma unroll
  for (int l = 0; l < 5; ++l) {
    double v = u2[l];
    if (a.bA != 0.0) v = a.bA * a.qU[c0 + P * l] + a.bB * v;
    a.qout[c0 + P * l] = v;
  }
  return true;
}

// FP32 arithmetic, FP64 accumulation: the conservative increment
// dU = R*TF*dt/V is turned into primitive increments exactly (no
// linearisation) in FP32 and added to the FP64 state.
__device__ __forceinline__ bool update_cell(const Params& p, const StageArgs& a, long long c0,
                                            long long ci, const float* R_in, float dtc, float vol) {
  const long long P = p.d.P, N = ncells(p.d);
  const float gm1 = (float)(p.gm - 1.0);
  float R[5];
#pragma unroll
  for (int l = 0; l < 5; ++l) R[l] = R_in[l];
  if (a.use_rn) {
#pragma unroll
    for (int l = 0; l < 5; ++l) {
      double rn = a.Rn[ci + N * l] + a.SF * (double)R[l];
      a.Rn[ci + N * l] = rn;
      if (a.TU) R[l] = (float)rn;
    }
  }
  double b64[5];
#pragma unroll
  for (int l = 0; l < 5; ++l) b64[l] = a.qbase[c0 + P * l];
  const float rho = (float)b64[0], u = (float)b64[1], v = (float)b64[2], w = (float)b64[3];
  const float fac = (float)a.TF * dtc / vol;
  const float dr = R[0] * fac, dmx = R[1] * fac, dmy = R[2] * fac, dmz = R[3] * fac, dE = R[4] * fac;
  const float r2 = rho - dr;
  const float ir2 = 1.0f / r2;
  const float du = (u * dr - dmx) * ir2, dv = (v * dr - dmy) * ir2, dw = (w * dr - dmz) * ir2;
  const float u2 = u + du, v2 = v + dv, w2 = w + dw;
  const float dp = gm1 * (-dE + 0.5f * dr * (u2 * u2 + v2 * v2 + w2 * w2) -
                          0.5f * rho * (2.0f * (u * du + v * dv + w * dw) + du * du + dv * dv + dw * dw));
  double out[5] = {b64[0] - (double)dr, b64[1] + (double)du, b64[2] + (double)dv, b64[3] + (double)dw,
                   b64[4] + (double)dp};
  bool bad = (out[0] < 0.) || (out[4] < 0.);
#pragma unroll
  for (int l = 0; l < 5; ++l) bad |= (out[l] != out[l]);
  if (bad) return false;
#pragma unroll
  for (int l = 0; l < 5; ++l) {
    double val = out[l];
    if (a.bA != 0.0) val = a.bA * a.qU[c0 + P * l] + a.bB * val;
    a.qout[c0 + P * l] = val;
  }
  return true;
}

template <typename T>
__global__ void __launch_bounds__(TX* TY) k_stage(Params p, StageArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int NV = 5;
  T* ring = reinterpret_cast<T*>(smem_raw);               // [NRING][NV][SH][SW]
  T* xch = ring + NRING * NV * SH * SW;                   // [NV][TY][TX] j-face left states
  T* gfl = xch + NV * TY * TX;                            // [NV][TY][TX] j-face fluxes
  T* lam = gfl + NV * TY * TX;                            // [TY][TX]    j-face dt terms
  const Dims& d = p.d;
  const int lane = threadIdx.x, w = threadIdx.y, tid = w * TX + lane;
  const int ib = 1 + IX * blockIdx.x, jb = 1 + IY * blockIdx.y;
  const int i = ib - 1 + lane, j = jb - 1 + w;
  const int i0 = ib - 3, j0 = jb - 3;  // stencil plane origin (col 0, row 0)
  const bool in_i = lane >= 1 && lane <= IX && i <= d.imx - 1;
  const bool in_j = w >= 1 && w <= IY && j <= d.jmx - 1;
  const int plane = NV * SH * SW;
  const T gm = (T)p.gm;
  const bool thin = d.kmx == 2;

  // clamp to the padded block so halo lanes past the edge stay finite
  auto clampi = [&](int x, int hi) { return x < -2 ? -2 : (x > hi + 2 ? hi + 2 : x); };

  auto load_plane = [&](int k) {
    T* dst = ring + ((k + 2) % NRING) * plane;
    for (int e = tid; e < NV * SH * SW; e += TX * TY) {
      int l = e / (SH * SW), rem = e - l * (SH * SW), r = rem / SW, c = rem - r * SW;
      int gi = clampi(i0 + c, d.imx), gj = clampi(j0 + r, d.jmx);
      dst[e] = (T)__ldg(a.qin + pidx(d, gi, gj, k) + d.P * l);
    }
  };

  // per-thread march state for cell (i, j, k-1)
  T Lp_prev[NV], H_prev[NV], dF_prev[NV], dG_prev[NV];
  T lamk_prev = 0, lami_lo_prev = 0, lami_hi_prev = 0, lamj_lo_prev = 0, lamj_hi_prev = 0;
#pragma unroll
  for (int l = 0; l < NV; ++l) { Lp_prev[l] = 0; H_prev[l] = 0; dF_prev[l] = 0; dG_prev[l] = 0; }

  const long long sj = d.ni, sk = (long long)d.ni * d.nj;
  for (int kl = -2; kl <= d.kmx + 2; ++kl) {
    __syncthreads();
    load_plane(kl);
    __syncthreads();
    const int k = kl - 2;  // plane processed now
    if (k < 0) continue;
    const bool kin = k >= 1 && k <= d.kmx - 1;
    T dF[NV], dG[NV];
#pragma unroll
    for (int l = 0; l < NV; ++l) { dF[l] = T(0); dG[l] = T(0); }
    T lami_lo = 0, lami_hi = 0, lamj_lo = 0, lamj_hi = 0;
    const int r = w + 2;               // own row in the stencil plane
    const int cc = lane + 2;           // own column
    const T* own = ring + ((k + 2) % NRING) * plane + r * SW + cc;  // var 0 of own cell
    T qc[NV];
#pragma unroll
    for (int l = 0; l < NV; ++l) qc[l] = own[l * SH * SW];
    // ---------------- i-faces (warp shuffles) ----------------
    if (kin && in_j) {  // warp-uniform
      T Rm[NV], Lp[NV];
      const T* rowp = ring + ((k + 2) % NRING) * plane + r * SW;
      const long long cbase = pidx(d, 0, clampi(j, d.jmx), k);
      VolLineT<T> vol{VolLine{a.cells + 4 * cbase, 1, d.imx}};
      SmemLine<T> pres{rowp + 4 * SH * SW + cc, i, 1};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        SmemLine<T> q{rowp + l * SH * SW + cc, i, 1};
        recon_cell<T>(p, 0, i, l + 1, q, pres, vol, Rm[l], Lp[l]);
      }
      T L[NV], F[NV];
#pragma unroll
      for (int l = 0; l < NV; ++l) L[l] = __shfl_up_sync(0xffffffffu, Lp[l], 1);
      T A, nx, ny, nz;
      load_face<T>(a.faces[0], fidx(d, 0, clampi(i, d.imx), clampi(j, d.jmx), k), A, nx, ny, nz);
      face_flux<T>(p, L, Rm, A, nx, ny, nz, (T)wall_mask(p, 0, i), F);
      if (a.compute_dt) lami_lo = lambda_face<T>(gm, L, Rm, A, nx, ny, nz, qc[1], qc[2], qc[3]);
      lami_hi = __shfl_down_sync(0xffffffffu, lami_lo, 1);
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        T Fh = __shfl_down_sync(0xffffffffu, F[l], 1);
        dF[l] = Fh - F[l];
      }
      if (a.mflux[0] && in_j && (i == 1 || i == d.imx) && lane >= 1)
        a.mflux[0][flidx(fldim(d, 0), i, j, k)] = (double)F[0];
    }
    // ---------------- j-faces (shared memory) ----------------
    if (kin) {
      T Rm[NV], Lp[NV];
      const T* colp = ring + ((k + 2) % NRING) * plane + cc;
      const long long cbase = pidx(d, clampi(i, d.imx), 0, k);
      VolLineT<T> vol{VolLine{a.cells + 4 * cbase, sj, d.jmx}};
      SmemLine<T> pres{colp + 4 * SH * SW + r * SW, j, SW};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        SmemLine<T> q{colp + l * SH * SW + r * SW, j, SW};
        recon_cell<T>(p, 1, j, l + 1, q, pres, vol, Rm[l], Lp[l]);
      }
#pragma unroll
      for (int l = 0; l < NV; ++l) xch[(l * TY + w) * TX + lane] = Lp[l];
      __syncthreads();
      T F[NV];
#pragma unroll
      for (int l = 0; l < NV; ++l) F[l] = T(0);
      if (w >= 1) {
        T L[NV];
#pragma unroll
        for (int l = 0; l < NV; ++l) L[l] = xch[(l * TY + w - 1) * TX + lane];
        T A, nx, ny, nz;
        load_face<T>(a.faces[1], fidx(d, 1, clampi(i, d.imx), clampi(j, d.jmx), k), A, nx, ny, nz);
        face_flux<T>(p, L, Rm, A, nx, ny, nz, (T)wall_mask(p, 1, j), F);
#pragma unroll
        for (int l = 0; l < NV; ++l) gfl[(l * TY + w) * TX + lane] = F[l];
        if (a.compute_dt) {
          lamj_lo = lambda_face<T>(gm, L, Rm, A, nx, ny, nz, qc[1], qc[2], qc[3]);
          lam[w * TX + lane] = lamj_lo;
        }
        if (a.mflux[1] && in_i && (j == 1 || j == d.jmx))
          a.mflux[1][flidx(fldim(d, 1), i, j, k)] = (double)F[0];
      }
      __syncthreads();
      if (w <= TY - 2) {
#pragma unroll
        for (int l = 0; l < NV; ++l) dG[l] = gfl[(l * TY + w + 1) * TX + lane] - F[l];
        if (a.compute_dt) lamj_hi = lam[(w + 1) * TX + lane];
      }
    } else {
      __syncthreads();
      __syncthreads();
    }
    // ---------------- k-faces (registers, marching) ----------------
    if (in_i && in_j) {
      T Rm[NV], Lp[NV];
      const T* cp = ring + r * SW + cc;
      const long long cbase = pidx(d, i, j, 0);
      VolLineT<T> vol{VolLine{a.cells + 4 * cbase, sk, d.kmx}};
      RingLine<T> pres{cp + 4 * SH * SW, plane};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        RingLine<T> q{cp + l * SH * SW, plane};
        recon_cell<T>(p, 2, k, l + 1, q, pres, vol, Rm[l], Lp[l]);
      }
      T H[NV];
      T lamk = 0;
      if (k >= 1) {
        T A, nx, ny, nz;
        load_face<T>(a.faces[2], fidx(d, 2, i, j, k), A, nx, ny, nz);
        if (thin) {
#pragma unroll
          for (int l = 0; l < NV; ++l) H[l] = T(0);
        } else {
          face_flux<T>(p, Lp_prev, Rm, A, nx, ny, nz, (T)wall_mask(p, 2, k), H);
        }
        if (a.compute_dt) lamk = lambda_face<T>(gm, Lp_prev, Rm, A, nx, ny, nz, qc[1], qc[2], qc[3]);
        if (a.mflux[2] && (k == 1 || k == d.kmx)) a.mflux[2][flidx(fldim(d, 2), i, j, k)] = (double)H[0];
        if (k >= 2) {
          // cell (i, j, k-1) is complete: residual (scheme.f90:133-135)
          const int kc = k - 1;
          const long long c0 = pidx(d, i, j, kc), ci = cidx(d, i, j, kc);
          T R[NV];
#pragma unroll
          for (int l = 0; l < NV; ++l) R[l] = (dF_prev[l] + dG_prev[l]) + (H[l] - H_prev[l]);
          const T vol_c = (T)a.cells[4 * c0];
          T dtc;
          if (a.compute_dt) {
            T s = lami_lo_prev + lamj_lo_prev + lamk_prev + lami_hi_prev + lamj_hi_prev + lamk;
            dtc = (T(1) / s) * vol_c * (T)a.CFL;
            a.dt[ci] = (double)dtc;
          } else {
            dtc = (T)a.dt[ci];
          }
          if (a.res_out)
#pragma unroll
            for (int l = 0; l < NV; ++l) a.res_out[ci + ncells(d) * l] = (double)R[l];
          if (!update_cell(p, a, c0, ci, R, dtc, vol_c)) raise_error(a.err, FEST_ERR_NEGATIVE_STATE);
        }
      }
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        Lp_prev[l] = Lp[l];
        if (k >= 1) H_prev[l] = H[l];
        if (kin) { dF_prev[l] = dF[l]; dG_prev[l] = dG[l]; }
      }
      if (k >= 1) lamk_prev = lamk;
      if (kin) {
        lami_lo_prev = lami_lo; lami_hi_prev = lami_hi;
        lamj_lo_prev = lamj_lo; lamj_hi_prev = lamj_hi;
      }
    }
  }
}

// TVD blends of the reference run over the whole padded block
// (update.f90:203-206), ghosts included; the blended ghosts matter where
// BCs stop rewriting them (fix() after iteration 2).  Non-interior cells:
// q = a*Us + b*X with Us the state before the iteration's BCs and X the last
// stage's input (its ghosts as that stage's BCs left them).
__global__ void k_ghost_blend(Dims d, double* q, const double* Us, const double* X, double a, double b) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.P * d.nv) return;
  long long c = t % d.P;
  int i = (int)(c % d.ni) - 2;
  long long r = c / d.ni;
  int j = (int)(r % d.nj) - 2, k = (int)(r / d.nj) - 2;
  bool interior = i >= 1 && i <= d.imx - 1 && j >= 1 && j <= d.jmx - 1 && k >= 1 && k <= d.kmx - 1;
  if (!interior) q[t] = a * Us[t] + b * X[t];
}

template <typename T> size_t stage_smem() {
  return sizeof(T) * ((size_t)NRING * 5 * SH * SW + 2 * 5 * TY * TX + TY * TX);
}

}  // namespace

struct FusedState {
  Dims d;
  double* Q[3] = {nullptr, nullptr, nullptr};  // Q[0] is the handle's qp
  double* Us = nullptr;  // state at the start of a TVD iteration (<= 2)
  BlockRef* table[3] = {nullptr, nullptr, nullptr};
  int cur = 0;       // buffer holding the current state
  bool seeded = false;
  std::vector<void*> allocs;
  bool profiling = false;
  std::vector<cudaEvent_t> ev;  // start/end pairs of profiled launches
  size_t nev = 0;               // events in use
};

bool fused_supported(const Params& p, int precision) {
  (void)precision;
  // ping-pong buffers keep each stage's ghosts in its own input buffer; BC
  // sets that read another face's ghosts (thin blocks, -9, two Riemann
  // faces) need the in-place module path
  return p.mu_ref == 0.0 && p.turb == FEST_TURB_NONE && p.d.nv == 5 && p.tstep == 'l' &&
         !ghosts_need_sequential(p);
}

int fused_create(const Params& p, const DevBlock& b, const BlockRef* table, cudaStream_t s,
                 FusedState** out) {
  (void)table;
  *out = nullptr;
  if (!fused_supported(p, FEST_MIXED)) return FEST_ERR_ARG;
  FusedState* f = new FusedState();
  f->d = p.d;
  f->Q[0] = b.qp;
  size_t bytes = sizeof(double) * (size_t)p.d.P * p.d.nv;
  for (int n = 1; n < 3; ++n) {
    if (cudaMalloc((void**)&f->Q[n], bytes) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
    f->allocs.push_back(f->Q[n]);
  }
  if (p.integ == FEST_TIME_TVDRK2 || p.integ == FEST_TIME_TVDRK3) {
    if (cudaMalloc((void**)&f->Us, bytes) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
    f->allocs.push_back(f->Us);
  }
  for (int n = 0; n < 3; ++n) {
    BlockRef ref{b, p.d};
    ref.b.qp = f->Q[n];
    if (cudaMalloc((void**)&f->table[n], sizeof(BlockRef)) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
    f->allocs.push_back(f->table[n]);
    cudaMemcpyAsync(f->table[n], &ref, sizeof(BlockRef), cudaMemcpyHostToDevice, s);
  }
  cudaFuncSetAttribute(k_stage<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_smem<float>());
  cudaFuncSetAttribute(k_stage<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)stage_smem<double>());
  *out = f;
  return FEST_OK;
}

void fused_destroy(FusedState* f) {
  if (!f) return;
  for (cudaEvent_t e : f->ev) cudaEventDestroy(e);
  for (void* x : f->allocs) cudaFree(x);
  delete f;
}

void fused_invalidate(FusedState* f) {
  if (f) { f->cur = 0; f->seeded = false; }
}

// copy the full padded state of buffer `from` into the others so ghost
// values that the BCs write only early (fix() at iter<=2) exist everywhere
static void seed(FusedState* f, cudaStream_t s) {
  size_t bytes = sizeof(double) * (size_t)f->d.P * f->d.nv;
  for (int n = 0; n < 3; ++n)
    if (n != f->cur) cudaMemcpyAsync(f->Q[n], f->Q[f->cur], bytes, cudaMemcpyDeviceToDevice, s);
  f->seeded = true;
}

static void stage(FusedState* f, const Params& p, const DevBlock& b, int prec, int in, int out,
                  int base, double bA, double bB, double TF, double SF, int TU, int use_rn,
                  int compute_dt, double CFL, int iter, bool last, cudaStream_t s, long long* cnt) {
  DevBlock bb = b;
  bb.qp = f->Q[in];
  Launcher L{s, cnt};
  launch_ghosts(p, bb, f->table[in], iter, L);
  StageArgs a;
  a.qin = f->Q[in];
  a.qout = f->Q[out];
  a.qbase = f->Q[base];
  a.qU = f->Q[f->cur];
  a.bA = bA; a.bB = bB; a.TF = TF; a.SF = SF; a.TU = TU; a.use_rn = use_rn;
  a.Rn = b.Rstore; a.dt = b.dt; a.compute_dt = compute_dt; a.CFL = CFL;
  a.res_out = last ? b.res : nullptr;
  for (int dir = 0; dir < 3; ++dir) {
    a.mflux[dir] = last ? b.flux[dir] : nullptr;
    a.faces[dir] = b.faces[dir];
  }
  a.cells = b.cells;
  a.err = b.err;
  dim3 grid((p.d.imx - 1 + IX - 1) / IX, (p.d.jmx - 1 + IY - 1) / IY);
  dim3 blk(TX, TY);
  if (f->profiling) {
    if (f->nev + 2 > f->ev.size())
      for (int n = 0; n < 256; ++n) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        f->ev.push_back(e);
      }
    cudaEventRecord(f->ev[f->nev], s);
  }
  if (prec == FEST_MIXED) k_stage<float><<<grid, blk, stage_smem<float>(), s>>>(p, a);
  else k_stage<double><<<grid, blk, stage_smem<double>(), s>>>(p, a);
  if (f->profiling) {
    cudaEventRecord(f->ev[f->nev + 1], s);
    f->nev += 2;
  }
  ++*cnt;
}

int fused_run(FusedState* f, const Params& p, const DevBlock& b, int prec, int n_iters,
              int first_iter, double CFL, cudaStream_t s, long long* cnt) {
  if (!f) return FEST_ERR_ARG;
  if (!f->seeded) seed(f, s);
  for (int n = 0; n < n_iters; ++n) {
    const int it = first_iter + n;
    const bool lastit = (n == n_iters - 1);
    const int U = f->cur, A = (U + 1) % 3, B = (U + 2) % 3;
    if (it <= 2) {
      // fix() ghosts are written only while current_iter <= 2
      // (bc_primitive.f90:236,318,366) and persist afterwards: every
      // buffer that later serves as a stage input must receive them
      for (int n = 0; n < 3; ++n) {
        if (n == U) continue;
        DevBlock bb = b;
        bb.qp = f->Q[n];
        launch_ghosts(p, bb, f->table[n], it, Launcher{s, cnt});
      }
    }
    const size_t bytes = sizeof(double) * (size_t)p.d.P * p.d.nv;
    const bool tvd_early = it <= 2 && (p.integ == FEST_TIME_TVDRK2 || p.integ == FEST_TIME_TVDRK3);
    if (tvd_early) cudaMemcpyAsync(f->Us, f->Q[U], bytes, cudaMemcpyDeviceToDevice, s);
    switch (p.integ) {
      case FEST_TIME_NONE:
        stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, lastit, s, cnt);
        f->cur = A;
        break;
      case FEST_TIME_TVDRK2:
        stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, false, s, cnt);
        stage(f, p, b, prec, A, U, A, 0.5, 0.5, 1., 1., 0, 0, 0, CFL, it, lastit, s, cnt);
        if (tvd_early) {
          long long n = p.d.P * p.d.nv;
          k_ghost_blend<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Q[U], f->Us, f->Q[A], 0.5, 0.5);
          ++*cnt;
        }
        break;
      case FEST_TIME_TVDRK3:
        stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, false, s, cnt);
        stage(f, p, b, prec, A, B, A, 0.75, 0.25, 1., 1., 0, 0, 0, CFL, it, false, s, cnt);
        stage(f, p, b, prec, B, U, B, 1. / 3., 2. / 3., 1., 1., 0, 0, 0, CFL, it, lastit, s, cnt);
        if (tvd_early) {
          long long n = p.d.P * p.d.nv;
          k_ghost_blend<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Q[U], f->Us, f->Q[B], 1. / 3., 2. / 3.);
          ++*cnt;
        }
        break;
      case FEST_TIME_RK2:
        cudaMemsetAsync(b.Rstore, 0, sizeof(double) * ncells(p.d) * p.d.nv, s);
        stage(f, p, b, prec, U, A, U, 0, 1, 0.5, 1., 0, 1, 1, CFL, it, false, s, cnt);
        stage(f, p, b, prec, A, U, U, 0, 1, 0.5, 1., 1, 1, 0, CFL, it, lastit, s, cnt);
        break;
      case FEST_TIME_RK4:
        cudaMemsetAsync(b.Rstore, 0, sizeof(double) * ncells(p.d) * p.d.nv, s);
        stage(f, p, b, prec, U, A, U, 0, 1, 0.5, 1., 0, 1, 1, CFL, it, false, s, cnt);
        stage(f, p, b, prec, A, B, U, 0, 1, 0.5, 2., 0, 1, 0, CFL, it, false, s, cnt);
        stage(f, p, b, prec, B, A, U, 0, 1, 1.0, 2., 0, 1, 0, CFL, it, false, s, cnt);
        stage(f, p, b, prec, A, U, U, 0, 1, 1. / 6., 1., 1, 1, 0, CFL, it, lastit, s, cnt);
        break;
      default:
        return FEST_ERR_ARG;
    }
    // the blended ghosts must persist in every buffer once fix() stops
    if (tvd_early)
      for (int n = 0; n < 3; ++n)
        if (n != f->cur) cudaMemcpyAsync(f->Q[n], f->Q[f->cur], bytes, cudaMemcpyDeviceToDevice, s);
  }
  return FEST_OK;
}

int fused_export_state(FusedState* f, double* qp, cudaStream_t s) {
  if (!f) return FEST_ERR_ARG;
  if (f->Q[f->cur] != qp) {
    cudaMemcpyAsync(qp, f->Q[f->cur], sizeof(double) * (size_t)f->d.P * f->d.nv,
                    cudaMemcpyDeviceToDevice, s);
    f->cur = 0;
    f->seeded = false;
  }
  return FEST_OK;
}

void fused_profile(FusedState* f, bool enable) {
  if (!f) return;
  f->profiling = enable;
  if (enable) f->nev = 0;
}

int fused_profile_read(FusedState* f, long long* launches, double* total_ms) {
  if (!f) return FEST_ERR_ARG;
  double t = 0.0;
  for (size_t n = 0; n + 1 < f->nev; n += 2) {
    float ms = 0.f;
    if (cudaEventSynchronize(f->ev[n + 1]) != cudaSuccess) return FEST_ERR_CUDA;
    cudaEventElapsedTime(&ms, f->ev[n], f->ev[n + 1]);
    t += ms;
  }
  if (launches) *launches = (long long)(f->nev / 2);
  if (total_ms) *total_ms = t;
  return FEST_OK;
}

int fused_export_residual(FusedState* f, const DevBlock&, cudaStream_t) { return f ? FEST_OK : FEST_ERR_ARG; }

}  // namespace fest
