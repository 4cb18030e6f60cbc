// fest_stage.cuh - the fused RK-stage sweep kernel, templated on the
// arithmetic type, the reconstruction and the flux scheme; instantiated per
// reconstruction in fest_stage_<method>.cu.
//
// One kernel per RK stage does, for a tile of cells, what the reference
// spreads over compute_face_interpolant, reconstruct_boundary_state,
// compute_fluxes, compute_residue, compute_time_step (stage 1) and
// update_with (update.f90:129-547): between the state read and the state
// write nothing touches HBM except the metrics.
//
// Tile: a CTA of 32x8 threads covers 30 interior cells in i (lanes 1..30,
// lanes 0/31 are the i-halo) by 6 in j (warps 1..6, warps 0/7 the j-halo)
// and marches along k over a chunk of interior planes (several chunks per
// column when the block is small, so every SM gets work).  A ring of
// stencil planes in shared memory holds planes k-2..k+2 (12 rows x 36
// columns x 5 variables each).  In FP32 the planes arrive by TMA
// (cp.async.bulk.tensor from the FP32 state mirror, one 4-D box per plane,
// completion on an mbarrier per ring slot, one plane prefetched ahead of
// the march); in FP64 the threads load and store them.  i-face fluxes travel
// by warp shuffles, j-face fluxes through shared memory, k-face fluxes stay
// in registers across the march.
//
// T = float  (FEST_MIXED): reconstruction, flux, residual and the update's
//             increments in FP32; the state stays FP64 and is advanced by
//             adding an FP64 increment (delta form); metrics are read FP64.
// T = double (FEST_FP64): the reference's arithmetic, update_with verbatim.
#pragma once
#include <cuda.h>  // CUtensorMap

#include "fest_common.cuh"

namespace fest {

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
  int k_chunk;          // interior k planes per CTA (gridDim.z chunks)
  // FP32 mirrors read by the mixed sweep (T = float); unused in FP64
  const float* qin32;   // stencil state (interior from the previous stage, ghosts from the fill)
  float* qout32;        // mirror of qout (interior written)
  const float4* faces32[3];  // {A,nx,ny,nz} per face
  const float* vol32;   // cell volumes (padded)
  int mpitch;           // row pitch of the state mirror (imx+5 rounded up to 4)
};

// one block of a batched stage launch (device memory, 64-byte aligned for
// the tensor map)
struct BatchEntry {
  CUtensorMap tm;  // the block's stencil mirror (FP32)
  Params p;
  StageArgs a;
  int cta0;        // first CTA of this block in the batched grid
  int tx, ty;      // tiles in i and j; k-chunks = CTAs / (tx*ty)
};

namespace stage {

constexpr int TX = 32, TY = 8;        // threads per CTA
constexpr int IX = TX - 2, IY = TY - 2;  // interior cells per CTA
constexpr int SW = TX + 4, SH = TY + 4;  // stencil plane extents (halo 2)
// ring geometry per arithmetic type: FP32 rows are 40 wide so that the TMA
// box can start on a 16-byte boundary (the tile origin 30*bx is 2 mod 4 for
// odd bx; the box starts 0 or 2 columns early), 6 slots for one plane of
// prefetch; FP64 keeps 36-wide rows and 5 slots
template <typename T> struct RingGeom;
template <> struct RingGeom<float> { static constexpr int W = 40, N = 6; };
template <> struct RingGeom<double> { static constexpr int W = 36, N = 5; };



template <typename T> struct SmemLine {
  const T* p;   // element of normal coordinate c0
  int c0, stride;
  __device__ __forceinline__ T operator()(int c) const { return p[(c - c0) * stride]; }
};
template <typename T> struct RingLine {
  const T* ring;  // ring + var/row/col offset; plane c lives in slot (c-base)%N
  int plane_stride, base;
  __device__ __forceinline__ T operator()(int c) const {
    return ring[((c - base) % RingGeom<T>::N) * plane_stride];
  }
};

// ---- TMA and mbarrier (PTX) -------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// one 4-D tile (x, y, z, w) of the tensor map into shared memory; the
// mbarrier expects its bytes
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* tm, int x, int y, int z,
                                            int w, uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}
// wait for phase `parity` of the barrier, giving up after ~2^31 cycles
// (about a second): returns false then
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > (1ll << 31)) return false;
  }
}
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

__device__ __forceinline__ void load_face(const StageArgs& a, int dir, long long idx, double& A,
                                          double& nx, double& ny, double& nz) {
  const double2* f2 = reinterpret_cast<const double2*>(a.faces[dir] + 4 * idx);
  double2 u = __ldg(f2), v = __ldg(f2 + 1);
  A = u.x; nx = u.y; ny = v.x; nz = v.y;
}
__device__ __forceinline__ void load_face(const StageArgs& a, int dir, long long idx, float& A,
                                          float& nx, float& ny, float& nz) {
  const float4 u = __ldg(a.faces32[dir] + idx);
  A = u.x; nx = u.y; ny = u.z; nz = u.w;
}
// cell volume along a line: AoS cells (FP64) or the FP32 mirror
struct VolLine32 {
  const float* p;  // vol32 + pidx(cell at normal coordinate 0)
  long long stride;
  int n;
  __device__ __forceinline__ float operator()(int c) const {
    c = c < -2 ? -2 : (c > n + 2 ? n + 2 : c);
    return p[c * stride];
  }
};
__device__ __forceinline__ VolLineT<double> vol_line(const StageArgs& a, double, long long base,
                                                     long long stride, int n) {
  return VolLineT<double>{VolLine{a.cells + 4 * base, stride, n}};
}
__device__ __forceinline__ VolLine32 vol_line(const StageArgs& a, float, long long base,
                                              long long stride, int n) {
  return VolLine32{a.vol32 + base, stride, n};
}
__device__ __forceinline__ double cell_vol(const StageArgs& a, double, long long c0) { return a.cells[4 * c0]; }
__device__ __forceinline__ float cell_vol(const StageArgs& a, float, long long c0) { return a.vol32[c0]; }
__device__ __forceinline__ const double* stencil_src(const StageArgs& a, double) { return a.qin; }
__device__ __forceinline__ const float* stencil_src(const StageArgs& a, float) { return a.qin32; }

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
                                            double vol, const double*, long long) {
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
                                            long long ci, const float* R_in, float dtc, float vol,
                                            const float* qc, long long m0) {
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
  const long long mvar = (long long)a.mpitch * p.d.nj * p.d.nk;  // mirror variable stride
  // FP32 copies of the base state: the stencil's own cell when the update
  // starts from the stencil state (bit-identical to converting b64)
  const bool own = a.qbase == a.qin;
  const float rho = own ? qc[0] : (float)b64[0], u = own ? qc[1] : (float)b64[1],
              v = own ? qc[2] : (float)b64[2], w = own ? qc[3] : (float)b64[3];
  const float fac = (float)a.TF * dtc / vol;
  const float dr = R[0] * fac, dmx = R[1] * fac, dmy = R[2] * fac, dmz = R[3] * fac, dE = R[4] * fac;
  const float r2 = rho - dr;
  const float ir2 = 1.0f / r2;
  const float du = (u * dr - dmx) * ir2, dv = (v * dr - dmy) * ir2, dw = (w * dr - dmz) * ir2;
  const float u2 = u + du, v2 = v + dv, w2 = w + dw;
  const float dp = gm1 * (-dE + 0.5f * dr * (u2 * u2 + v2 * v2 + w2 * w2) -
                          0.5f * rho * (2.0f * (u * du + v * dv + w * dw) + du * du + dv * dv + dw * dw));
  // negative or NaN density/pressure after the update (update.f90:448),
  // judged in FP32 (a NaN anywhere in the increments reaches rn or pn)
  const float p0 = own ? qc[4] : (float)b64[4];
  const float rn = rho - dr, pn = p0 + dp;
  if (!(rn >= 0.0f) || !(pn >= 0.0f) || du != du || dv != dv || dw != dw) return false;
  const double out[5] = {b64[0] - (double)dr, b64[1] + (double)du, b64[2] + (double)dv,
                         b64[3] + (double)dw, b64[4] + (double)dp};
#pragma unroll
  for (int l = 0; l < 5; ++l) {
    double val = out[l];
    if (a.bA != 0.0) val = a.bA * a.qU[c0 + P * l] + a.bB * val;
    a.qout[c0 + P * l] = val;
    a.qout32[m0 + mvar * l] = (float)val;
  }
  return true;
}

// The sweep of one CTA: tile (bx, by) of the block, k-chunk bz.  The
// single-block kernel passes its block indices; the batched kernel maps its
// CTA to a block of the batch and a tile of that block.
template <typename T, int INTERP, int FLUX>
__device__ __forceinline__ void stage_body(const Params& p, const StageArgs& a, const CUtensorMap* tmp,
                                           int bx, int by, int bz) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr int NV = 5;
  constexpr int RW = RingGeom<T>::W, NR = RingGeom<T>::N;
  constexpr bool kTma = sizeof(T) == 4;
  T* ring = reinterpret_cast<T*>(smem_raw);               // [NR][NV][SH][RW]
  T* xch = ring + NR * NV * SH * RW;                      // [NV][TY][TX] j-face left states
  T* gfl = xch + NV * TY * TX;                            // [NV][TY][TX] j-face fluxes
  T* lam = gfl + NV * TY * TX;                            // [TY][TX]    j-face dt terms
  uint64_t* bars = reinterpret_cast<uint64_t*>(lam + TY * TX);  // [NR] ring-slot barriers
  __shared__ int abort_flag;
  const Dims& d = p.d;
  const int lane = threadIdx.x, w = threadIdx.y, tid = w * TX + lane;
  const int ib = 1 + IX * bx, jb = 1 + IY * by;
  const int i = ib - 1 + lane, j = jb - 1 + w;
  const int i0 = ib - 3, j0 = jb - 3;  // stencil plane origin (col 0, row 0)
  const bool in_i = lane >= 1 && lane <= IX && i <= d.imx - 1;
  const bool in_j = w >= 1 && w <= IY && j <= d.jmx - 1;
  const int plane = NV * SH * RW;
  const T gm = (T)p.gm;
  // FP32: the TMA box starts ox columns left of the tile's stencil origin
  const int ox = kTma ? ((IX * bx) & 3) : 0;
  const bool thin = d.kmx == 2;

  // clamp to the padded block so halo lanes past the edge stay finite
  auto clampi = [&](int x, int hi) { return x < -2 ? -2 : (x > hi + 2 ? hi + 2 : x); };

  const int k0 = 1 + a.k_chunk * bz;
  const int k1 = min(k0 + a.k_chunk - 1, d.kmx - 1);
  const int base = k0 - 3;                 // first plane of the chunk's march
  const int nplanes = (k1 + 3) - base + 1;
  auto slot = [&](int c) { return (c - base) % NR; };

  // FP64: per-thread load offsets of the stencil plane (plane k adds (k+2)*ni*nj)
  constexpr int NLOAD = kTma ? 1 : (NV * SH * SW + TX * TY - 1) / (TX * TY);
  int off[NLOAD];
  if constexpr (!kTma) {
#pragma unroll
    for (int m = 0; m < NLOAD; ++m) {
      int e = tid + m * TX * TY;
      if (e >= NV * SH * SW) e = NV * SH * SW - 1;
      int l = e / (SH * SW), rem = e - l * (SH * SW), r = rem / SW, c = rem - r * SW;
      int gi = clampi(i0 + c, d.imx), gj = clampi(j0 + r, d.jmx);
      off[m] = (int)(pidx(d, gi, gj, -2) + d.P * l);
    }
  }
  const int plane_stride = d.ni * d.nj;
  const T* qsrc = stencil_src(a, T(0));
  auto load_plane = [&](int k) {  // FP64 path
    T* dst = ring + slot(k) * plane;
    const T* src = qsrc + (long long)(k + 2) * plane_stride;
#pragma unroll
    for (int m = 0; m < NLOAD; ++m) {
      int e = tid + m * TX * TY;
      if (e < NV * SH * SW) dst[e] = __ldg(src + off[m]);
    }
  };
  // FP32 path: plane c of the mirror -> ring slot, box (40 x 12 x 1 x 5)
  // at array coordinates (30*bx - ox, 6*by, c+2, 0); columns or rows past
  // the array are zero-filled and feed only discarded halo lanes
  constexpr uint32_t kPlaneBytes = (uint32_t)(NV * SH * RW * sizeof(T));
  auto issue = [&](int c) {
    fence_proxy_async();  // earlier generic reads of the slot come first
    tma_load_4d(ring + slot(c) * plane, tmp, IX * bx - ox, IY * by, c + 2, 0,
                bars + slot(c), kPlaneBytes);
  };
  if constexpr (kTma) {
    if (tid == 0) {
      abort_flag = 0;
      for (int n = 0; n < NR; ++n) mbar_init(bars + n, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (tid == 0)
      for (int n = 0; n < NR && n < nplanes; ++n) issue(base + n);
  }

  // per-thread march state for cell (i, j, k-1)
  T Lp_prev[NV], H_prev[NV], dF_prev[NV], dG_prev[NV];
  T lamk_prev = 0, lami_lo_prev = 0, lami_hi_prev = 0, lamj_lo_prev = 0, lamj_hi_prev = 0;
#pragma unroll
  for (int l = 0; l < NV; ++l) { Lp_prev[l] = 0; H_prev[l] = 0; dF_prev[l] = 0; dG_prev[l] = 0; }

  const long long sj = d.ni, sk = (long long)d.ni * d.nj;
  for (int n = 0; n < nplanes; ++n) {
    const int kl = base + n;  // plane arriving now
    __syncthreads();
    if constexpr (kTma) {
      if (abort_flag) return;  // uniform: read after the barrier
      // the slot of plane n+1 last held plane n+1-NR, read up to iteration n-1
      if (tid == 0 && n + 1 >= NR && n + 1 < nplanes) issue(kl + 1);
      if (!mbar_wait(bars + slot(kl), (uint32_t)((n / NR) & 1))) {
        raise_error(a.err, FEST_ERR_TIMEOUT);
        abort_flag = 1;
      }
    } else {
      load_plane(kl);
      __syncthreads();
    }
    const int k = kl - 2;  // plane processed now
    if (k < k0 - 1) continue;
    const bool kin = k >= k0 && k <= k1;
    T dF[NV], dG[NV];
#pragma unroll
    for (int l = 0; l < NV; ++l) { dF[l] = T(0); dG[l] = T(0); }
    T lami_lo = 0, lami_hi = 0, lamj_lo = 0, lamj_hi = 0;
    const int r = w + 2;               // own row in the stencil plane
    const int cc = lane + 2 + ox;      // own column
    const T* own = ring + slot(k) * plane + r * RW + cc;  // var 0 of own cell
    T qc[NV];
#pragma unroll
    for (int l = 0; l < NV; ++l) qc[l] = own[l * SH * RW];
    // ---------------- i-faces (warp shuffles) ----------------
    if (kin && in_j) {  // warp-uniform
      T Rm[NV], Lp[NV];
      const T* rowp = ring + slot(k) * plane + r * RW;
      const auto vol = vol_line(a, T(0), pidx(d, 0, clampi(j, d.jmx), k), 1, d.imx);
      SmemLine<T> pres{rowp + 4 * SH * RW + cc, i, 1};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        SmemLine<T> q{rowp + l * SH * RW + cc, i, 1};
        recon_cell<T, INTERP>(p, 0, i, l + 1, q, pres, vol, Rm[l], Lp[l]);
      }
      T L[NV], F[NV];
#pragma unroll
      for (int l = 0; l < NV; ++l) L[l] = __shfl_up_sync(0xffffffffu, Lp[l], 1);
      T A, nx, ny, nz;
      load_face(a, 0, fidx(d, 0, clampi(i, d.imx), clampi(j, d.jmx), k), A, nx, ny, nz);
      face_flux<T, FLUX>(p, L, Rm, A, nx, ny, nz, (T)wall_mask(p, 0, i), F);
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
      const T* colp = ring + slot(k) * plane + cc;
      const auto vol = vol_line(a, T(0), pidx(d, clampi(i, d.imx), 0, k), sj, d.jmx);
      SmemLine<T> pres{colp + 4 * SH * RW + r * RW, j, RW};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        SmemLine<T> q{colp + l * SH * RW + r * RW, j, RW};
        recon_cell<T, INTERP>(p, 1, j, l + 1, q, pres, vol, Rm[l], Lp[l]);
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
        load_face(a, 1, fidx(d, 1, clampi(i, d.imx), clampi(j, d.jmx), k), A, nx, ny, nz);
        face_flux<T, FLUX>(p, L, Rm, A, nx, ny, nz, (T)wall_mask(p, 1, j), F);
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
      const T* cp = ring + r * RW + cc;
      const auto vol = vol_line(a, T(0), pidx(d, i, j, 0), sk, d.kmx);
      RingLine<T> pres{cp + 4 * SH * RW, plane, base};
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        RingLine<T> q{cp + l * SH * RW, plane, base};
        recon_cell<T, INTERP>(p, 2, k, l + 1, q, pres, vol, Rm[l], Lp[l]);
      }
      T H[NV];
      T lamk = 0;
      if (k >= k0) {
        T A, nx, ny, nz;
        load_face(a, 2, fidx(d, 2, i, j, k), A, nx, ny, nz);
        if (thin) {
#pragma unroll
          for (int l = 0; l < NV; ++l) H[l] = T(0);
        } else {
          face_flux<T, FLUX>(p, Lp_prev, Rm, A, nx, ny, nz, (T)wall_mask(p, 2, k), H);
        }
        if (a.compute_dt) lamk = lambda_face<T>(gm, Lp_prev, Rm, A, nx, ny, nz, qc[1], qc[2], qc[3]);
        if (a.mflux[2] && (k == 1 || k == d.kmx)) a.mflux[2][flidx(fldim(d, 2), i, j, k)] = (double)H[0];
        if (k >= k0 + 1) {
          // cell (i, j, k-1) is complete: residual (scheme.f90:133-135)
          const int kc = k - 1;
          const long long c0 = pidx(d, i, j, kc), ci = cidx(d, i, j, kc);
          T R[NV];
#pragma unroll
          for (int l = 0; l < NV; ++l) R[l] = (dF_prev[l] + dG_prev[l]) + (H[l] - H_prev[l]);
          const T vol_c = cell_vol(a, T(0), c0);
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
          // the finished cell's own stencil values (plane k-1 of the ring)
          T qo[5];
          const T* own1 = ring + slot(kc) * plane + r * RW + cc;
#pragma unroll
          for (int l = 0; l < 5; ++l) qo[l] = own1[l * SH * RW];
          const long long m0 = (long long)(i + 2) + (long long)a.mpitch * ((j + 2) + (long long)d.nj * (kc + 2));
          if (!update_cell(p, a, c0, ci, R, dtc, vol_c, qo, m0))
            raise_error(a.err, FEST_ERR_NEGATIVE_STATE);
        }
      }
#pragma unroll
      for (int l = 0; l < NV; ++l) {
        Lp_prev[l] = Lp[l];
        if (k >= k0) H_prev[l] = H[l];
        if (kin) { dF_prev[l] = dF[l]; dG_prev[l] = dG[l]; }
      }
      if (k >= k0) lamk_prev = lamk;
      if (kin) {
        lami_lo_prev = lami_lo; lami_hi_prev = lami_hi;
        lamj_lo_prev = lamj_lo; lamj_hi_prev = lamj_hi;
      }
    }
  }
}

// MB: CTAs per SM the registers are budgeted for (FP32: 2 = 115 registers,
// no spills, fewer instructions; 3 = 80 registers, more warps to hide
// latency on large blocks; the tuner picks per block)
template <typename T, int INTERP, int FLUX, int MB>
__global__ void __launch_bounds__(TX* TY, MB)
    k_stage(Params p, StageArgs a, const __grid_constant__ CUtensorMap tm) {
  stage_body<T, INTERP, FLUX>(p, a, &tm, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One launch for every block of a batch: block b owns CTAs
// [cta0, cta0 + tx*ty*nz) of the 1-D grid.
template <typename T, int INTERP, int FLUX>
__global__ void __launch_bounds__(TX* TY, sizeof(T) == 4 ? 3 : 1)
    k_stage_batch(const BatchEntry* e, int nb) {
  __shared__ Params sp;
  __shared__ StageArgs sa;
  __shared__ int sb;
  const int tid = threadIdx.y * TX + threadIdx.x;
  if (tid == 0) {
    int lo = 0, hi = nb - 1;  // last entry with cta0 <= blockIdx.x
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (e[mid].cta0 <= (int)blockIdx.x) lo = mid;
      else hi = mid - 1;
    }
    sb = lo;
  }
  __syncthreads();
  const BatchEntry& E = e[sb];
  {
    const int* src = reinterpret_cast<const int*>(&E.p);
    int* dst = reinterpret_cast<int*>(&sp);
    for (int n = tid; n < (int)(sizeof(Params) / 4); n += TX * TY) dst[n] = src[n];
    src = reinterpret_cast<const int*>(&E.a);
    dst = reinterpret_cast<int*>(&sa);
    for (int n = tid; n < (int)(sizeof(StageArgs) / 4); n += TX * TY) dst[n] = src[n];
  }
  __syncthreads();
  const int local = (int)blockIdx.x - E.cta0;
  stage_body<T, INTERP, FLUX>(sp, sa, &E.tm, local % E.tx, (local / E.tx) % E.ty, local / (E.tx * E.ty));
}

template <typename T> inline size_t stage_smem() {
  return sizeof(T) * ((size_t)RingGeom<T>::N * 5 * SH * RingGeom<T>::W + 2 * 5 * TY * TX + TY * TX) +
         sizeof(uint64_t) * RingGeom<T>::N + 16;
}


}  // namespace stage

// one host launcher per reconstruction (fest_stage_<method>.cu)
#define FEST_STAGE_LAUNCHER(name)                                                         \
  int name(int prec, int flux, int occ, dim3 grid, cudaStream_t s, const Params& p, const StageArgs& a, \
           const CUtensorMap& tm)
FEST_STAGE_LAUNCHER(launch_stage_none);
FEST_STAGE_LAUNCHER(launch_stage_muscl);
FEST_STAGE_LAUNCHER(launch_stage_ppm);
FEST_STAGE_LAUNCHER(launch_stage_weno);
FEST_STAGE_LAUNCHER(launch_stage_weno_nm);
// batched: every block of the batch in one launch of `ctas` CTAs
#define FEST_BATCH_LAUNCHER(name) \
  int name(int prec, int flux, int ctas, cudaStream_t s, const BatchEntry* e, int nb)
FEST_BATCH_LAUNCHER(launch_batch_none);
FEST_BATCH_LAUNCHER(launch_batch_muscl);
FEST_BATCH_LAUNCHER(launch_batch_ppm);
FEST_BATCH_LAUNCHER(launch_batch_weno);
FEST_BATCH_LAUNCHER(launch_batch_weno_nm);

template <int INTERP>
int launch_stage_t(int prec, int flux, int occ, dim3 grid, cudaStream_t s, const Params& p,
                   const StageArgs& a, const CUtensorMap& tm) {
  using namespace stage;
  const dim3 blk(TX, TY);
  static bool attrs = false;
#define FEST_SET(T, F, MB)                                                                     \
  cudaFuncSetAttribute(k_stage<T, INTERP, F, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)stage_smem<T>())
  if (!attrs) {
    FEST_SET(float, 0, 2); FEST_SET(float, 1, 2); FEST_SET(float, 2, 2);
    FEST_SET(float, 3, 2); FEST_SET(float, 4, 2); FEST_SET(float, 5, 2);
    FEST_SET(float, 0, 3); FEST_SET(float, 1, 3); FEST_SET(float, 2, 3);
    FEST_SET(float, 3, 3); FEST_SET(float, 4, 3); FEST_SET(float, 5, 3);
    FEST_SET(double, 0, 1); FEST_SET(double, 1, 1); FEST_SET(double, 2, 1);
    FEST_SET(double, 3, 1); FEST_SET(double, 4, 1); FEST_SET(double, 5, 1);
    attrs = true;
  }
#undef FEST_SET
#define FEST_GO(T, F, MB) k_stage<T, INTERP, F, MB><<<grid, blk, stage_smem<T>(), s>>>(p, a, tm)
#define FEST_FLUXES(T, MB)                 \
  switch (flux) {                          \
    case 0: FEST_GO(T, 0, MB); break;      \
    case 1: FEST_GO(T, 1, MB); break;      \
    case 2: FEST_GO(T, 2, MB); break;      \
    case 3: FEST_GO(T, 3, MB); break;      \
    case 4: FEST_GO(T, 4, MB); break;      \
    case 5: FEST_GO(T, 5, MB); break;      \
    default: return FEST_ERR_ARG;          \
  }
  if (prec == FEST_MIXED) {
    if (occ >= 3) { FEST_FLUXES(float, 3) }
    else { FEST_FLUXES(float, 2) }
  } else {
    FEST_FLUXES(double, 1)
  }
#undef FEST_FLUXES
#undef FEST_GO
  return FEST_OK;
}

template <int INTERP>
int launch_batch_t(int prec, int flux, int ctas, cudaStream_t s, const BatchEntry* e, int nb) {
  using namespace stage;
  const dim3 blk(TX, TY);
  static bool attrs = false;
#define FEST_SET(T, F)                                                                           \
  cudaFuncSetAttribute(k_stage_batch<T, INTERP, F>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)stage_smem<T>())
  if (!attrs) {
    FEST_SET(float, 0); FEST_SET(float, 1); FEST_SET(float, 2);
    FEST_SET(float, 3); FEST_SET(float, 4); FEST_SET(float, 5);
    attrs = true;
  }
#undef FEST_SET
  if (prec != FEST_MIXED) return FEST_ERR_ARG;  // batches run the FP32 sweep
#define FEST_GO(F) k_stage_batch<float, INTERP, F><<<ctas, blk, stage_smem<float>(), s>>>(e, nb)
  switch (flux) {
    case 0: FEST_GO(0); break;
    case 1: FEST_GO(1); break;
    case 2: FEST_GO(2); break;
    case 3: FEST_GO(3); break;
    case 4: FEST_GO(4); break;
    case 5: FEST_GO(5); break;
    default: return FEST_ERR_ARG;
  }
#undef FEST_GO
  return FEST_OK;
}

}  // namespace fest
