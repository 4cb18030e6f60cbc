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
#include "fest_convert.cuh"

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
  const float4* cells32;  // {volume, cx, cy, cz} (FP32, padded layout): viscous sweeps
  const float* dist32;    // wall distance (FP32, padded layout): SST sweeps
  // FP64 viscous sweeps: the temperature of the iteration's start (padded;
  // the reference's gradients use it, update.f90:170) and the wall distance
  const double* Temp;
  const double* dist;
  float f_TF, f_CFL, f_bB;  // FP32 copies of TF, CFL and bB
  int blend;              // bA != 0
  // FP32 sweeps after iteration 2: faces (bit f) whose ghost layer 1 the
  // sweep computes in shared memory from the staged interior cells, and
  // k-interfaces (bit 0: kmin, bit 1: kmax) whose ghost planes the TMA
  // fetches from the partner face's interior planes
  int ring_ghosts;
  int kper;
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

// Face states of NV variables of one cell along a line: WENO5 in the FP32
// sweep two variables per instruction stream (weno_pair), every other
// method and FP64 one variable at a time (recon_cell); the boundary
// overrides of the cells next to a boundary face follow per variable.
// ROLL keeps the loop over the variables rolled (instruction-cache size).
template <typename T, int INTERP, int NV, bool ROLL, class MakeLine, class Lpres, class Lvol>
__device__ __forceinline__ void recon_vars(const Params& p, int dir, int c, const MakeLine& line, const Lpres& pres,
                                           const Lvol& vol, T* Rm, T* Lp) {
  if constexpr (sizeof(T) == 4 && INTERP == FEST_INTERP_WENO) {
    const bool nb = near_boundary(p, dir, c);
    if constexpr (ROLL) {
#pragma unroll 1
      for (int l = 0; l < NV; l += 2) {
        const int l2 = l + 1 < NV ? l + 1 : l;
        const auto qa = line(l), qb = line(l2);
        float2 rm, lp;
        weno_pair(qa, qb, c, rm, lp);
        Rm[l] = rm.x; Lp[l] = lp.x; Rm[l2] = rm.y; Lp[l2] = lp.y;
        if (nb) {
          boundary_override<T, INTERP>(p, dir, c, l + 1, qa, Rm[l], Lp[l]);
          if (l2 != l) boundary_override<T, INTERP>(p, dir, c, l2 + 1, qb, Rm[l2], Lp[l2]);
        }
      }
    } else {
#pragma unroll
      for (int l = 0; l < NV; l += 2) {
        const int l2 = l + 1 < NV ? l + 1 : l;
        const auto qa = line(l), qb = line(l2);
        float2 rm, lp;
        weno_pair(qa, qb, c, rm, lp);
        Rm[l] = rm.x; Lp[l] = lp.x; Rm[l2] = rm.y; Lp[l2] = lp.y;
        if (nb) {
          boundary_override<T, INTERP>(p, dir, c, l + 1, qa, Rm[l], Lp[l]);
          if (l2 != l) boundary_override<T, INTERP>(p, dir, c, l2 + 1, qb, Rm[l2], Lp[l2]);
        }
      }
    }
  } else if constexpr (ROLL) {
#pragma unroll 1
    for (int l = 0; l < NV; ++l) recon_cell<T, INTERP>(p, dir, c, l + 1, line(l), pres, vol, Rm[l], Lp[l]);
  } else {
#pragma unroll
    for (int l = 0; l < NV; ++l) recon_cell<T, INTERP>(p, dir, c, l + 1, line(l), pres, vol, Rm[l], Lp[l]);
  }
}

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

// ---- FP32 <-> FP64 conversions (integer arithmetic, fest_convert.cuh) -------
__device__ __forceinline__ double to_f64(float x) { return f2d(x); }
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ float from_f64(double x, float) { return d2f(x); }
__device__ __forceinline__ double from_f64(double x, double) { return x; }

// ---- the update of one cell -------------------------------------------------
// FP64: update_with(...,'conservative',...) (update.f90:367-485) verbatim;
// SST (NV = 7): the point-implicit destruction (update.f90:395-398, F1 the
// cell's blending function, omega of the stage's input state) and k, omega
// written only where they stay non-negative (update.f90:479-480).
template <int NV>
__device__ __forceinline__ bool update_cell(const Params& p, const StageArgs& a, long long c0,
                                            long long ci, const double* R_in, double dtc,
                                            double vol, const double*, long long, double F1) {
  const long long P = p.d.P, N = ncells(p.d);
  const double gm = p.gm;
  double R[NV], u1[NV], u2[NV];
#pragma unroll
  for (int l = 0; l < NV; ++l) R[l] = R_in[l];
  u1[0] = a.qbase[c0];
#pragma unroll
  for (int l = 1; l < NV; ++l) u1[l] = a.qbase[c0 + P * l] * u1[0];
  double s1 = u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3];
  u1[4] = (u1[4] / (gm - 1.) + 0.5 * s1) / u1[0];
  if constexpr (NV == 7) {
    const double beta = 0.075 * F1 + (1. - F1) * 0.0828;
    const double wv = a.qin[c0 + 6 * P];
    R[5] = R[5] / (1 + (beta * wv * dtc));
    R[6] = R[6] / (1 + (2 * beta * wv * dtc));
  }
  if (a.use_rn) {
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      double rn = a.Rn[ci + N * l] + a.SF * R[l];
      a.Rn[ci + N * l] = rn;
      if (a.TU) R[l] = rn;
    }
  }
  const double fac = (a.TF * dtc / vol);
#pragma unroll
  for (int l = 0; l < NV; ++l) u2[l] = u1[l] - R[l] * fac;
#pragma unroll
  for (int l = 1; l < NV; ++l) u2[l] = u2[l] / u2[0];
  double s2 = u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3];
  u2[4] = (gm - 1.) * u2[0] * (u2[4] - (0.5 * s2));
  bool bad = (u2[0] < 0.) || (u2[4] < 0.);
#pragma unroll
  for (int l = 0; l < NV; ++l) bad |= (u2[l] != u2[l]);
  if (bad) return false;
#pragma unroll
  for (int l = 0; l < NV; ++l) {
    double v = u2[l];
    if (l >= 5 && v < 0.) v = a.qin[c0 + P * l];  // k, omega that would turn negative keep the stage input
    if (a.blend) v = a.bA * a.qU[c0 + P * l] + a.bB * v;
    a.qout[c0 + P * l] = v;
  }
  return true;
}

// FP32 arithmetic, FP64 accumulation: the conservative increment
// dU = R*TF*dt/V is turned into primitive increments exactly (no
// linearisation) in FP32 and added to the FP64 state.  SST (NV = 7): the
// point-implicit destruction of update.f90:395-398 divides the k and omega
// residuals first (F1: the cell's blending function), and k, omega are
// written only where they stay non-negative (update.f90:479-480).
template <int NV>
__device__ __forceinline__ bool update_cell_f32(const Params& p, const StageArgs& a, long long c0,
                                                long long ci, const float* R_in, float dtc, float vol,
                                                const float* qc, long long m0, float F1) {
  const long long P = p.d.P, N = ncells(p.d);
  const float gm1 = p.f_gm1;
  float R[NV];
#pragma unroll
  for (int l = 0; l < NV; ++l) R[l] = R_in[l];
  if constexpr (NV == 7) {
    const float beta = 0.075f * F1 + (1.0f - F1) * 0.0828f;
    const float wv = qc[6];  // omega of the stage's input state
    R[5] = R[5] / (1.0f + (beta * wv * dtc));
    R[6] = R[6] / (1.0f + (2.0f * beta * wv * dtc));
  }
  if (a.use_rn) {
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      double rn = fma(a.SF, f2d(R[l]), a.Rn[ci + N * l]);
      a.Rn[ci + N * l] = rn;
      if (a.TU) R[l] = d2f(rn);
    }
  }
  double b64[NV];
#pragma unroll
  for (int l = 0; l < NV; ++l) b64[l] = a.qbase[c0 + P * l];
  const long long mvar = (long long)a.mpitch * p.d.nj * p.d.nk;  // mirror variable stride
  // FP32 copies of the base state: the stencil's own cell when the update
  // starts from the stencil state (bit-identical to converting b64)
  const bool own = a.qbase == a.qin;
  const float rho = own ? qc[0] : d2f(b64[0]), u = own ? qc[1] : d2f(b64[1]),
              v = own ? qc[2] : d2f(b64[2]), w = own ? qc[3] : d2f(b64[3]);
  const float fac = a.f_TF * dtc / vol;
  const float dr = R[0] * fac, dmx = R[1] * fac, dmy = R[2] * fac, dmz = R[3] * fac, dE = R[4] * fac;
  const float r2 = rho - dr;
  const float ir2 = 1.0f / r2;
  const float du = (u * dr - dmx) * ir2, dv = (v * dr - dmy) * ir2, dw = (w * dr - dmz) * ir2;
  const float u2 = u + du, v2 = v + dv, w2 = w + dw;
  const float dp = gm1 * (-dE + 0.5f * dr * (u2 * u2 + v2 * v2 + w2 * w2) -
                          0.5f * rho * (2.0f * (u * du + v * dv + w * dw) + du * du + dv * dv + dw * dw));
  // negative or NaN density/pressure after the update (update.f90:448),
  // decided in FP32 (a NaN anywhere in the increments reaches rn or pn)
  const float p0 = own ? qc[4] : d2f(b64[4]);
  const float rn = rho - dr, pn = p0 + dp;
  if (!(rn >= 0.0f) || !(pn >= 0.0f) || du != du || dv != dv || dw != dw) return false;
  // new state = base + increment; the TVD blends bA*U + bB*(base + inc)
  // as two FMAs, fma(bB, base, fma(bA, U, bB*inc))
  float inc[NV];
  inc[0] = -dr; inc[1] = du; inc[2] = dv; inc[3] = dw; inc[4] = dp;
  bool keep[NV];
#pragma unroll
  for (int l = 0; l < NV; ++l) keep[l] = false;
  if constexpr (NV == 7) {
    const float tk = own ? qc[5] : d2f(b64[5]), tw = own ? qc[6] : d2f(b64[6]);
    const float dk = (tk * dr - R[5] * fac) * ir2, dom = (tw * dr - R[6] * fac) * ir2;
    if (dk != dk || dom != dom) return false;
    inc[5] = dk;
    inc[6] = dom;
    keep[5] = b64[5] + f2d(dk) < 0.0;
    keep[6] = b64[6] + f2d(dom) < 0.0;
  }
  const float bBf = a.f_bB;
#pragma unroll
  for (int l = 0; l < NV; ++l) {
    double val;
    if (keep[l]) {
      val = a.qin[c0 + P * l];  // k, omega that would turn negative keep the stage input
      if (a.blend) val = fma(a.bA, a.qU[c0 + P * l], a.bB * val);
    } else if (a.blend) {
      val = fma(a.bB, b64[l], fma(a.bA, a.qU[c0 + P * l], f2d(bBf * inc[l])));
    } else {
      val = b64[l] + f2d(inc[l]);
    }
    a.qout[c0 + P * l] = val;
    a.qout32[m0 + mvar * l] = d2f(val);
  }
  return true;
}


// ---- viscous and SST terms of the sweep -------------------------------------
// Templated on the arithmetic type: FP32 in the mixed sweep (fast division
// and square root), FP64 in the FP64 sweep with the reference's operations.
// Face and cell records: {A,nx,ny,nz} and {volume,cx,cy,cz}, float4 (FP32
// copies) or D4 (the FP64 arrays).
struct D4 {
  double x, y, z, w;
};
template <typename T> struct Rec4;
template <> struct Rec4<float> { using type = float4; };
template <> struct Rec4<double> { using type = D4; };
template <typename T> using R4 = typename Rec4<T>::type;
__device__ __forceinline__ float4 mk4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
__device__ __forceinline__ D4 mk4(double a, double b, double c, double d) { return D4{a, b, c, d}; }
__device__ __forceinline__ float4 ld_face4(const StageArgs& a, int dir, long long idx, float) {
  return __ldg(a.faces32[dir] + idx);
}
__device__ __forceinline__ D4 ld_face4(const StageArgs& a, int dir, long long idx, double) {
  const double2* f2 = reinterpret_cast<const double2*>(a.faces[dir] + 4 * idx);
  const double2 u = __ldg(f2), v = __ldg(f2 + 1);
  return D4{u.x, u.y, v.x, v.y};
}
__device__ __forceinline__ float4 ld_cell4(const StageArgs& a, long long idx, float) { return __ldg(a.cells32 + idx); }
__device__ __forceinline__ D4 ld_cell4(const StageArgs& a, long long idx, double) {
  const double2* c2 = reinterpret_cast<const double2*>(a.cells + 4 * idx);
  const double2 u = __ldg(c2), v = __ldg(c2 + 1);
  return D4{u.x, u.y, v.x, v.y};
}
__device__ __forceinline__ float ld_dist(const StageArgs& a, long long idx, float) { return __ldg(a.dist32 + idx); }
__device__ __forceinline__ double ld_dist(const StageArgs& a, long long idx, double) { return __ldg(a.dist + idx); }
__device__ __forceinline__ float ex_tanh(float x) { return tanhf(x); }
__device__ __forceinline__ double ex_tanh(double x) { return tanh(x); }
__device__ __forceinline__ float ex_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double ex_pow(double x, double y) { return pow(x, y); }

template <typename T> struct ViscCell {
  T u, v, w, rho;  // primitive velocity, density
  T Tm;            // temperature p/(rho R) of the stage's state (viscosity, flux)
  T Tg;            // temperature the gradients use (FP64: the iteration's start)
  T k, om;         // SST: turbulent kinetic energy, specific dissipation
};
// Tg: the temperature of the gradient sums, or a negative value for the
// stage's own (FP32 sweep)
template <bool TURB, typename T>
__device__ __forceinline__ ViscCell<T> visc_cell(const T* q, int vs, T R, T Tg) {
  ViscCell<T> c;
  c.rho = q[0];
  c.u = q[vs];
  c.v = q[2 * vs];
  c.w = q[3 * vs];
  c.Tm = dv(q[4 * vs], c.rho * R);
  c.Tg = Tg < T(0) ? c.Tm : Tg;
  if constexpr (TURB) {
    c.k = q[5 * vs];
    c.om = q[6 * vs];
  } else {
    c.k = T(0);
    c.om = T(0);
  }
  return c;
}
// gradient variable l of a cell: u, v, w, T (+ k, omega for SST), the
// reference's gradient order (gradients.f90:276-482); gvar for the gradient
// sums, fvar for the differences of the viscous face correction
template <typename T> __device__ __forceinline__ T gvar(const ViscCell<T>& c, int l) {
  return l == 0 ? c.u : l == 1 ? c.v : l == 2 ? c.w : l == 3 ? c.Tg : l == 4 ? c.k : c.om;
}
template <typename T> __device__ __forceinline__ T fvar(const ViscCell<T>& c, int l) {
  return l == 3 ? c.Tm : gvar(c, l);
}
// dynamic viscosity at a cell: constant mu_ref, or Sutherland's law from the
// cell temperature (viscosity.f90:109-136)
__device__ __forceinline__ float visc_mu(const Params& p, float T) {
  const float mu_ref = p.f_mu_ref;
  if (p.mu_var != FEST_MU_SUTHERLAND) return mu_ref;
  const float Tr = p.f_T_ref, S = p.f_S;
  const float t = dv(T, Tr);
  return mu_ref * (t * sq(t)) * dv(Tr + S, T + S);
}
__device__ __forceinline__ double visc_mu(const Params& p, double T) {
  if (p.mu_var != FEST_MU_SUTHERLAND) return p.mu_ref;
  return p.mu_ref * (pow(T / p.T_ref, 1.5)) * ((p.T_ref + p.S) / (T + p.S));
}
// Green-Gauss gradient of the NGV gradient variables at a cell
// (gradients.f90:276-482): grad = sum over faces of +-(phi_nb + phi_c) n A
// / (2V), low faces of i, j, k first; z components zero on a single-plane
// block.  nb[0..5] = i-1, j-1, k-1, i+1, j+1, k+1; f[0..5] the matching
// faces; G[3*l + component].
template <int NGV, typename T>
__device__ __forceinline__ void visc_gg(const ViscCell<T>& c, const ViscCell<T>* nb, const R4<T>* f, T vol,
                                        bool thin, T* G) {
  const T iv2 = dv(T(1), T(2) * vol);
#pragma unroll
  for (int l = 0; l < NGV; ++l) {
    const T vc = gvar(c, l);
    T vn[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) vn[m] = gvar(nb[m], l);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
      T g = T(0);
      if (!(thin && comp == 2)) {
        const T n0 = comp == 0 ? f[0].y : comp == 1 ? f[0].z : f[0].w;
        const T n1 = comp == 0 ? f[1].y : comp == 1 ? f[1].z : f[1].w;
        const T n2 = comp == 0 ? f[2].y : comp == 1 ? f[2].z : f[2].w;
        const T n3 = comp == 0 ? f[3].y : comp == 1 ? f[3].z : f[3].w;
        const T n4 = comp == 0 ? f[4].y : comp == 1 ? f[4].z : f[4].w;
        const T n5 = comp == 0 ? f[5].y : comp == 1 ? f[5].z : f[5].w;
        T s = -((vn[0] + vc) * n0 * f[0].x);
        s = s - (vn[1] + vc) * n1 * f[1].x;
        s = s - (vn[2] + vc) * n2 * f[2].x;
        s = s + (vn[3] + vc) * n3 * f[3].x;
        s = s + (vn[4] + vc) * n4 * f[4].x;
        s = s + (vn[5] + vc) * n5 * f[5].x;
        if constexpr (sizeof(T) == 8) g = s / (T(2) * vol);
        else g = s * iv2;
      }
      G[3 * l + comp] = g;
    }
  }
}
// gradient of a ghost cell from its interior neighbour (apply_gradient_bc,
// gradients.f90:486-676): normal jump over the boundary face, adiabatic
// walls flip the temperature gradient, plus the interior tangential part
template <int NGV, typename T>
__device__ __forceinline__ void visc_gbc(const Params& p, int f, const T* GI, const ViscCell<T>& cI,
                                         const ViscCell<T>& cG, T volI, R4<T> fc, T* GG) {
  const T sig = (f % 2) ? T(-1) : T(1);
  T ccx, ccy, ccz;
  if constexpr (sizeof(T) == 8) {
    ccx = fc.x * fc.y / volI; ccy = fc.x * fc.z / volI; ccz = fc.x * fc.w / volI;
  } else {
    const T av = dv(fc.x, volI);
    ccx = av * fc.y; ccy = av * fc.z; ccz = av * fc.w;
  }
#pragma unroll
  for (int l = 0; l < NGV; ++l) {
    const T diff = gvar(cI, l) - gvar(cG, l);
    GG[3 * l + 0] = sig * diff * ccx;
    GG[3 * l + 1] = sig * diff * ccy;
    GG[3 * l + 2] = sig * diff * ccz;
  }
  const double Tw = p.Tw[f];
  if (p.id[f] == -5 && Tw < 1.0 && Tw >= 0.0) {
    GG[9] = -GI[9]; GG[10] = -GI[10]; GG[11] = -GI[11];
  }
#pragma unroll
  for (int l = 0; l < NGV; ++l) {
    const T gx = GI[3 * l], gy = GI[3 * l + 1], gz = GI[3 * l + 2];
    const T dot = (gx * fc.y) + (gy * fc.z) + (gz * fc.w);
    GG[3 * l + 0] = GG[3 * l + 0] + (gx - dot * fc.y);
    GG[3 * l + 1] = GG[3 * l + 1] + (gy - dot * fc.z);
    GG[3 * l + 2] = GG[3 * l + 2] + (gz - dot * fc.w);
  }
}
// Viscous flux of a face between cells L and R (viscous.f90:144-325):
// face gradient = mean of the cell gradients, corrected along the
// centre-to-centre vector; Fv holds the terms that the reference subtracts
// from F(2:5) (and, for SST, from F(6:7)).  SST (viscous.f90:328-447): eddy
// viscosity added to the stresses and the heat flux, the -2/3 rho k normal
// stress and the k and omega diffusion with F1-blended sigmas, all skipped
// on the k faces of a single-plane block (sst_face false).
template <bool TURB = false, typename T>
__device__ __forceinline__ void visc_flux(const Params& p, const T* GL, const T* GR, const ViscCell<T>& L,
                                          const ViscCell<T>& Rc, R4<T> cL, R4<T> cR, T muL, T muR, T mutL,
                                          T mutR, T F1L, T F1R, R4<T> fc, bool sst_face, T* Fv) {
  constexpr int NGV = TURB ? 6 : 4;
  T G[3][NGV];
#pragma unroll
  for (int comp = 0; comp < 3; ++comp)
#pragma unroll
    for (int l = 0; l < NGV; ++l) G[comp][l] = T(0.5) * (GL[3 * l + comp] + GR[3 * l + comp]);
  const T dx = cR.y - cL.y, dy = cR.z - cL.z, dz = cR.w - cL.w;
  const T dLR = sq(dx * dx + dy * dy + dz * dz);
#pragma unroll
  for (int l = 0; l < NGV; ++l) {
    const T del = fvar(Rc, l) - fvar(L, l);
    if constexpr (sizeof(T) == 8) {
      const T nc = (del - (G[0][l] * dx + G[1][l] * dy + G[2][l] * dz)) / dLR;
      G[0][l] = G[0][l] + (nc * dx / dLR);
      G[1][l] = G[1][l] + (nc * dy / dLR);
      G[2][l] = G[2][l] + (nc * dz / dLR);
    } else {
      const T idLR = dv(T(1), dLR);
      const T nc = (del - (G[0][l] * dx + G[1][l] * dy + G[2][l] * dz)) * idLR;
      G[0][l] = G[0][l] + (nc * dx * idLR);
      G[1][l] = G[1][l] + (nc * dy * idLR);
      G[2][l] = G[2][l] + (nc * dz * idLR);
    }
  }
  const T mu_f = T(0.5) * (muL + muR);
  const T mut_f = TURB ? T(0.5) * (mutL + mutR) : T(0);
  const T tm = TURB ? mu_f + mut_f : mu_f;
  const T div3 = dvc(G[0][0] + G[1][1] + G[2][2], T(3));
  const T Txx = T(2) * tm * (G[0][0] - div3), Tyy = T(2) * tm * (G[1][1] - div3),
          Tzz = T(2) * tm * (G[2][2] - div3);
  const T Txy = tm * (G[0][1] + G[1][0]), Txz = tm * (G[0][2] + G[2][0]), Tyz = tm * (G[1][2] + G[2][1]);
  const T gm = pv<T>(p.gm, p.f_gm), Rg = pv<T>(p.R, p.f_R);
  const T kd = TURB ? dv(mu_f, pv<T>(p.Pr, p.f_Pr)) + dv(mut_f, pv<T>(p.tPr, p.f_tPr)) : dv(tm, pv<T>(p.Pr, p.f_Pr));
  const T Kh = sizeof(T) == 8 ? kd * gm * Rg / (gm - T(1)) : kd * gm * Rg * dv(T(1), gm - T(1));
  const T Qx = Kh * G[0][3], Qy = Kh * G[1][3], Qz = Kh * G[2][3];
  const T uf = T(0.5) * (L.u + Rc.u), vf = T(0.5) * (L.v + Rc.v), wf = T(0.5) * (L.w + Rc.w);
  const T A = fc.x, nx = fc.y, ny = fc.z, nz = fc.w;
  Fv[0] = (Txx * nx + Txy * ny + Txz * nz) * A;
  Fv[1] = (Txy * nx + Tyy * ny + Tyz * nz) * A;
  Fv[2] = (Txz * nx + Tyz * ny + Tzz * nz) * A;
  Fv[3] = A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) + ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
               ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz));
  if constexpr (TURB) {
    Fv[4] = T(0);
    Fv[5] = T(0);
    if (sst_face) {
      const T F1f = T(0.5) * (F1L + F1R);
      const T skf = T(0.85) * F1f + T(1.0) * (T(1) - F1f);
      const T swf = T(0.5) * F1f + T(0.856) * (T(1) - F1f);
      const T rhof = T(0.5) * (L.rho + Rc.rho), tkf = T(0.5) * (L.k + Rc.k);
      const T Tk = dvc(T(-2) * rhof * tkf, T(3));
      const T dk = G[0][4] * nx + G[1][4] * ny + G[2][4] * nz;
      const T dw = G[0][5] * nx + G[1][5] * ny + G[2][5] * nz;
      Fv[0] += Tk * nx * A;
      Fv[1] += Tk * ny * A;
      Fv[2] += Tk * nz * A;
      const T kdiff = A * ((mu_f + skf * mut_f) * dk);
      Fv[3] += kdiff;
      Fv[4] = kdiff;
      Fv[5] = A * ((mu_f + swf * mut_f) * dw);
    }
  }
}
// viscous time-step term of a face (add_viscous_time, time.f90:366-448;
// add_turbulent_time, time.f90:450-531, with mu_t): A mu/(rho |(c_L -
// c_R).n|) with mu and rho of the face's high-side cell
template <typename T>
__device__ __forceinline__ T visc_lambda(R4<T> fc, R4<T> cL, R4<T> cR, T muR, T rhoR) {
  const T d = fabs(((cL.y - cR.y) * fc.y) + ((cL.z - cR.z) * fc.z) + ((cL.w - cR.w) * fc.w));
  if constexpr (sizeof(T) == 8) return fc.x * (muR / (rhoR * d));
  else return fc.x * dv(muR, rhoR * d);
}

// SST quantities of a cell (viscosity.f90:52-546, source.f90:158-270): eddy
// viscosity, blending function F1, cross-diffusion CD (clamped) and the
// vorticity magnitude.  G: the cell's gradients of u, v, w, T, k, omega.
template <typename T> struct SstCell {
  T mut, F1, CD, vort;
};
template <typename T>
__device__ __forceinline__ SstCell<T> sst_cell(const Params& p, const ViscCell<T>& c, T mu, T dd, const T* G) {
  const T bstar = T(0.09), a1 = T(0.31), sw2 = T(0.856);
  const bool s2003 = p.turb == FEST_TURB_SST2003;
  SstCell<T> s;
  const T var1 = dv(sq(c.k), bstar * c.om * dd);
  const T var2 = dv(T(500) * dv(mu, c.rho), (dd * dd) * c.om);
  const T arg2 = fmax2(T(2) * var1, var2);
  const T F2 = ex_tanh(arg2 * arg2);
  const T NUM = c.rho * a1 * c.k;
  // G(component, variable) of the reference = G[3*(variable-1) + component]
  const T wx = G[7] - G[5], wy = G[2] - G[6], wz = G[3] - G[1];
  s.vort = sq(wx * wx + wy * wy + wz * wz);
  T DENOM;
  if (s2003) {
    const T sxx = G[0], syy = G[4], szz = G[8];
    const T syz = G[7] + G[5], szx = G[2] + G[6], sxy = G[3] + G[1];
    const T SijSij = (T(2) * (sxx * sxx)) + (T(2) * (syy * syy)) + (T(2) * (szz * szz)) + syz * syz +
                     szx * szx + sxy * sxy;
    DENOM = fmax2(fmax2(a1 * c.om, sq(SijSij) * F2), T(1.0e-10));
  } else {
    DENOM = fmax2(fmax2(a1 * c.om, s.vort * F2), T(1.0e-20));
  }
  s.mut = dv(NUM, DENOM);
  T CD = dv(T(2) * c.rho * sw2 * (G[12] * G[15] + G[13] * G[16] + G[14] * G[17]), c.om);
  s.CD = fmax2(CD, s2003 ? T(1.0e-10) : T(1.0e-20));
  const T right = dv(T(4) * (c.rho * sw2 * c.k), s.CD * (dd * dd));
  const T arg1 = fmin2(fmax2(var1, var2), right);
  const T a2 = arg1 * arg1;
  s.F1 = ex_tanh(a2 * a2);
  return s;
}
// SST source of an interior cell (add_sst_source, source.f90:158-270):
// production limited by 20 (sst) or 10 (sst2003) times the destruction;
// the residual of k and omega loses Sk, Sw
template <typename T>
__device__ __forceinline__ void sst_source(const Params& p, const ViscCell<T>& c, const SstCell<T>& s, const T* G,
                                           T vol, T& Sk, T& Sw) {
  constexpr double kBeta1 = 0.075, kBeta2 = 0.0828, kBstar = 0.09, kSw1 = 0.5, kSw2 = 0.856, kKap = 0.41;
  // gamma_{1,2} = beta_{1,2}/beta* - sigma_w{1,2} kappa^2 / sqrt(beta*), sqrt(0.09) = 0.3
  constexpr T kG1 = (T)((kBeta1 / kBstar) - ((kSw1 * (kKap * kKap)) / 0.3));
  constexpr T kG2 = (T)((kBeta2 / kBstar) - ((kSw2 * (kKap * kKap)) / 0.3));
  const bool s2003 = p.turb == FEST_TURB_SST2003;
  const T lim = s2003 ? T(10) : T(20);
  const T gama1 = s2003 ? T(5.0 / 9.0) : kG1, gama2 = s2003 ? T(0.44) : kG2;
  const T F1 = s.F1;
  const T gama = gama1 * F1 + gama2 * (T(1) - F1);
  const T beta = (T)kBeta1 * F1 + (T)kBeta2 * (T(1) - F1);
  const T Dk = (T)kBstar * c.rho * c.om * c.k;
  const T Dw = beta * c.rho * (c.om * c.om);
  const T divergence = G[0] + G[4] + G[8];
  T Pk = s.mut * (s.vort * s.vort) - ((T(2) / T(3)) * c.rho * c.k * divergence);
  Pk = fmin2(Pk, lim * Dk);
  const T Pw = dv(c.rho * gama, s.mut) * Pk;
  Sk = (Pk - Dk) * vol;
  Sw = (Pw - Dw + (T(1) - F1) * s.CD) * vol;
}
// eddy viscosity and F1 of a ghost cell next to a boundary face with a
// negative id: faces -1..-9 copy the interior values, the wall negating
// mu_t (viscosity.f90:287-340); other faces keep what calculate_viscosity
// computed there from the ghost's own state and boundary gradient
template <typename T>
__device__ __forceinline__ void sst_ghost(const Params& p, int f, const ViscCell<T>& cG, T muG, const T* GG,
                                          T ddG, T mutI, T F1I, T& mutG, T& F1G) {
  const int id = p.id[f];
  if (id <= -1 && id >= -9) {
    mutG = id == -5 ? -mutI : mutI;
    F1G = F1I;
  } else {
    const SstCell<T> s = sst_cell(p, cG, muG, ddG, GG);
    mutG = s.mut;
    F1G = s.F1;
  }
}

// ---- ghost layer 1 of a boundary face in FP32 -------------------------------
// Riemann-invariant ghost state (bc_primitive.f90:1237-1776 for -11, the
// far-field form for -8) from the interior cell's primitive values; fc: the
// boundary face record (normals of low faces flipped to point outwards).
// Returns the boundary normal velocity.  Fast FP32 division, square root
// and power, as everywhere in the mixed sweep.
__device__ __forceinline__ float riemann_ghost_f32(const Params& p, int f, float4 fc, float uu, float vv, float ww,
                                                   float pI, float rI, float& rg, float& ug, float& vg, float& wg,
                                                   float& pg) {
  const bool tp = p.id[f] == -11;
  const float gm = p.f_gm;
  const float sg = (f % 2 == 0) ? -1.f : 1.f;
  const float nx = sg * fc.y, ny = sg * fc.z, nz = sg * fc.w;
  const float uinf = p.f_u_inf, vinf = p.f_v_inf, winf = p.f_w_inf;
  const float pinf = p.f_p_inf, rinf = p.f_rho_inf;
  const float cexp = sq(dv(gm * pI, rI)), cinf = sq(dv(gm * pinf, rinf));
  const float Unexp = uu * nx + vv * ny + ww * nz, Uninf = uinf * nx + vinf * ny + winf * nz;
  const float Rinf = Uninf - dv(2.f * cinf, gm - 1.f), Rexp = Unexp + dv(2.f * cexp, gm - 1.f);
  const float Unb = 0.5f * (Rexp + Rinf), Cb = 0.25f * (gm - 1.f) * (Rexp - Rinf);
  rg = 0.f;
  pg = 0.f;
  if (Unb > 0.f) {
    const float vd = Unb - Unexp;
    ug = uu + vd * nx; vg = vv + vd * ny; wg = ww + vd * nz;
    if (!tp) {
      const float sv = dv(pI, __powf(rI, gm));
      rg = __powf(dv(Cb * Cb, gm * sv), dv(1.f, gm - 1.f));
      pg = dv(rg * Cb * Cb, gm);
    }
  } else {
    const float vd = Unb - Uninf;
    ug = uinf + vd * nx; vg = vinf + vd * ny; wg = winf + vd * nz;
    if (!tp) {
      const float sv = dv(pinf, __powf(rinf, gm));
      rg = __powf(dv(Cb * Cb, gm * sv), dv(1.f, gm - 1.f));
      pg = dv(rg * Cb * Cb, gm);
    }
  }
  if (tp) {
    const float Mb = dv(sq(ug * ug + vg * vg + wg * wg), Cb);
    pg = dv(p.f_Tp[f], __powf((1.f + 0.5f * (gm - 1.f) * Mb * Mb), dv(gm, gm - 1.f)));
    rg = dv(gm * pg, Cb * Cb);
  }
  return Unb;
}

// Ghost layer 1 of face f at one column from its interior layers 1 and 2:
// the face procedures of the FP32 ghost fill (bc_primitive.f90:160-206,
// copy_bc.f90, FT_bc.f90:15-107, bc_primitive.f90:392-402,564-643,
// 1237-1945) at layer 1, after iteration 2 (no fix() writes).  G, I1, I2
// address variable 0, variables vs apart.  fn: the face's own record, fr:
// the I-face record at the same index (flow tangency's normals,
// FT_bc.f90:67-69), dd1: the interior cell's wall distance (SST walls).
// Faces -8/-11 with SST (k, omega follow the face's last column) are not
// handled here.
template <int NV>
__device__ __forceinline__ void ghost_layer1(const Params& p, int f, float* G, const float* I1, const float* I2,
                                             int vs, float4 fn, float4 fr, float dd1) {
  const float c1 = p.f_c1, c2 = p.f_c2, c3 = p.f_c3;
  const float gm = p.f_gm, R = p.f_R;
  auto symm = [&](int l) { G[l * vs] = dv(c2 * I1[l * vs] - c3 * I2[l * vs], c1); };
  switch (p.id[f]) {
    case -2:
    case -7:
#pragma unroll
      for (int l = 0; l < NV; ++l) G[l * vs] = I1[l * vs];
      break;
    case -3: G[4 * vs] = I1[4 * vs]; break;
    case -4:
#pragma unroll
      for (int l = 0; l < 4; ++l) G[l * vs] = I1[l * vs];
      if constexpr (NV == 7) { G[5 * vs] = I1[5 * vs]; G[6 * vs] = I1[6 * vs]; }
      break;
    case -5: {
      symm(4);
      const float Tw = p.f_Tw[f];
      if (Tw < 0.f) {
        const float pp = I1[4 * vs], rho = I1[0];
        const float stag = dv(pp, R * rho) * (1.f + dv(0.5f * (gm - 1.f) * gm * pp, rho));
        G[0] = dv(G[4 * vs], R * stag);
      } else if (Tw > 1.f) {
        const float Ti = dv(I1[4 * vs], R * I1[0]);
        G[0] = dv(G[4 * vs], R * (2.f * Tw - Ti));
      } else {
        symm(0);
      }
      G[vs] = -I1[vs]; G[2 * vs] = -I1[2 * vs]; G[3 * vs] = -I1[3 * vs];
      if constexpr (NV == 7) {
        G[5 * vs] = -I1[5 * vs];
        const float Tf = 0.5f * ((G[4 * vs] / G[0]) + (I1[4 * vs] / I1[0])) / R;
        const float Tr = p.f_T_ref, S = p.f_S;
        const float mu = p.f_mu_ref * powf(Tf / Tr, 1.5f) * ((Tr + S) / (Tf + S));
        const float rho = 0.5f * (G[0] + I1[0]);
        const float dd = 2.f * dd1;
        G[6 * vs] = 120.f * mu / (rho * 0.075f * (dd * dd)) - I1[6 * vs];
      }
    } break;
    case -6: {
      symm(0); symm(4);
      if constexpr (NV == 7) { symm(5); symm(6); }
      const float uu = I1[vs], vv = I1[2 * vs], ww = I1[3 * vs];
      const float dot = uu * fn.y + vv * fn.z + ww * fn.w;
      G[vs] = uu - (2.f * dot * fr.y);
      G[2 * vs] = vv - (2.f * dot * fr.z);
      G[3 * vs] = ww - (2.f * dot * fr.w);
    } break;
    case -8:
    case -11: {
      float rg, ug, vg, wg, pg;
      riemann_ghost_f32(p, f, fn, I1[vs], I1[2 * vs], I1[3 * vs], I1[4 * vs], I1[0], rg, ug, vg, wg, pg);
      G[0] = rg; G[vs] = ug; G[2 * vs] = vg; G[3 * vs] = wg; G[4 * vs] = pg;
    } break;
    default: break;  // -1: fix() only
  }
}

// The sweep of one CTA: tile (bx, by) of the block, k-chunk bz.  The
// single-block kernel passes its block indices; the batched kernel maps its
// CTA to a block of the batch and a tile of that block.
// VISC adds the laminar viscous terms, TURB (with VISC) the k-omega SST
// model: seven variables, six gradient variables, eddy viscosity and F1 per
// cell, the SST face terms, source and time-step terms and the update's
// point-implicit destruction.
template <typename T, int INTERP, int FLUX, bool VISC = false, bool TURB = false>
__device__ __forceinline__ void stage_body(const Params& p, const StageArgs& a, const CUtensorMap* tmp,
                                           int bx, int by, int bz) {
  static_assert(!TURB || VISC, "the SST terms come with the viscous terms");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  constexpr int NV = TURB ? 7 : 5;
  constexpr int NGV = TURB ? 6 : 4, NGC = 3 * NGV;  // gradient variables, gradient floats per cell
  constexpr int NXV = VISC ? NGC + (TURB ? 4 : 1) : 0;  // viscous j-exchange floats per thread
  constexpr int RW = RingGeom<T>::W, NR = RingGeom<T>::N;
  constexpr bool kTma = sizeof(T) == 4;
  T* ring = reinterpret_cast<T*>(smem_raw);               // [NR][NV][SH][RW]
  T* xch = ring + NR * NV * SH * RW;                      // [NV][TY][TX] j-face left states
  T* gfl = xch + NV * TY * TX;                            // [NV][TY][TX] j-face fluxes
  T* lam = gfl + NV * TY * TX;                            // [TY][TX]    j-face dt terms
  // viscous: [NGC][TY][TX] cell gradients, [TY][TX] viscous j-face dt
  // terms; SST: [TY][TX] each of mu_t, F1 and turbulent j-face dt terms
  T* gxch = lam + TY * TX;
  T* lamv = gxch + NGC * TY * TX;
  T* mutx = lamv + TY * TX;
  T* f1x = mutx + TY * TX;
  T* lamt = f1x + TY * TX;
  uint64_t* bars = reinterpret_cast<uint64_t*>(lam + TY * TX + NXV * TY * TX);  // [NR]
  __shared__ int abort_flag;
  const Dims& d = p.d;
  const int lane = threadIdx.x, w = threadIdx.y, tid = w * TX + lane;
  const int ib = 1 + IX * bx, jb = 1 + IY * by;
  const int i = ib - 1 + lane, j = jb - 1 + w;
  const int i0 = ib - 3, j0 = jb - 3;  // stencil plane origin (col 0, row 0)
  const bool in_i = lane >= 1 && lane <= IX && i <= d.imx - 1;
  const bool in_j = w >= 1 && w <= IY && j <= d.jmx - 1;
  const int plane = NV * SH * RW;
  const T gm = pv<T>(p.gm, p.f_gm);
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
  // FP32 path: plane c of the mirror -> ring slot, box (40 x 12 x 1 x NV)
  // at array coordinates (30*bx - ox, 6*by, c+2, 0); columns or rows past
  // the array are zero-filled and feed only discarded halo lanes
  constexpr uint32_t kPlaneBytes = (uint32_t)(NV * SH * RW * sizeof(T));
  auto issue = [&](int c) {
    fence_proxy_async();  // earlier generic accesses of the slot come first
    // k-interfaces: ghost plane 1-L <- partner plane kmx-L, kmx+L-1 <- L
    int src = c;
    if ((a.kper & 1) && c <= 0) src = c + d.kmx - 1;
    else if ((a.kper & 2) && c >= d.kmx) src = c - d.kmx + 1;
    tma_load_4d(ring + slot(c) * plane, tmp, IX * bx - ox, IY * by, src + 2, 0,
                bars + slot(c), kPlaneBytes);
  };
  // in-ring ghost layer 1 of the faces in a.ring_ghosts (FP32 sweep): ring
  // column of array index i = i - (ib-3) + ox, ring row of j = j - (jb-3)
  const int rgm = kTma ? a.ring_ghosts : 0;
  const int col_ilo = 3 - ib + ox, col_ihi = d.imx - ib + 3 + ox;
  const int row_jlo = 3 - jb, row_jhi = d.jmx - jb + 3;
  const bool g_ilo = (rgm & 1) && col_ilo >= 0, g_ihi = (rgm & 2) && col_ihi < RW;
  const bool g_jlo = (rgm & 4) && row_jlo >= 0, g_jhi = (rgm & 8) && row_jhi < SH;
  const bool g_ij = g_ilo || g_ihi || g_jlo || g_jhi;
  // In-ring i/j ghost tasks, done by the halo warps 0 and TY-1 (idle while
  // the interior warps do the k faces): q = 0..RW-1 the j-face ghost of
  // ring column q (the low face; the high one too, second, in a block of
  // at most IY interior rows), q = RW..RW+2*SH-1 the i-face ghost of a ring
  // row (low face, then high).  Per task: ring offset, face record (own
  // face, I-face) and wall-distance indices at k = 0 (32-bit: the fused
  // path takes blocks with P*n_var < 2^31).
  const int VS = SH * RW;  // variable stride in a ring plane
  const int gq = w == 0 ? lane : (w == TY - 1 ? TX + lane : -1);
  auto ghost_task = [&](int q, bool second, int& face, int& off, int& fn, int& fr, int& dd) -> bool {
    if (q < RW) {
      const bool hi = second || !g_jlo;
      const int ii = q + ib - 3 - ox;
      if (!(hi ? g_jhi : g_jlo) || ii < 1 || ii > d.imx - 1) return false;
      face = 2 + hi;
      off = (hi ? row_jhi : row_jlo) * RW + q;
      fn = (int)fidx(d, 1, ii, hi ? d.jmx : 1, 0);
      fr = (int)fidx(d, 0, ii, hi ? d.jmx : 1, 0);
      dd = (int)pidx(d, ii, hi ? d.jmx - 1 : 1, 0);
      return true;
    }
    const int r2 = q - RW, hi = r2 >= SH, r = r2 - hi * SH, jj = jb - 3 + r;
    if (r2 >= 2 * SH || !(hi ? g_ihi : g_ilo) || jj < 1 || jj > d.jmx - 1) return false;
    face = hi;
    off = r * RW + (hi ? col_ihi : col_ilo);
    fn = fr = (int)fidx(d, 0, hi ? d.imx : 1, jj, 0);
    dd = (int)pidx(d, hi ? d.imx - 1 : 1, jj, 0);
    return true;
  };
  int gt_face = -1, gt_off = 0, gt_fn = 0, gt_fr = 0, gt_dd = 0;
  bool gt_second = false;
  if (g_ij && gq >= 0) {
    if (!ghost_task(gq, false, gt_face, gt_off, gt_fn, gt_fr, gt_dd)) gt_face = -1;
    gt_second = gq < RW && g_jlo && g_jhi;
  }
  // k strides of the I-face, J-face and cell arrays
  const int sI = d.nj * (d.ni + 1), sJ = (d.nj + 1) * d.ni, sC = d.ni * d.nj;
  // apply this thread's tasks to plane kp (fn0/fr0/dd0: the first task's
  // records on that plane)
  auto ij_ghosts = [&](int kp, float4 fn0, float4 fr0, float dd0) {
    float* P = reinterpret_cast<float*>(ring) + slot(kp) * plane;
    auto apply = [&](int face, int off, float4 fn, float4 fr, float dd) {
      float* G = P + off;
      const int st = face == 0 ? 1 : (face == 1 ? -1 : (face == 2 ? RW : -RW));  // inwards
      ghost_layer1<NV>(p, face, G, G + st, G + 2 * st, VS, fn, fr, dd);
    };
    if (gt_face >= 0) apply(gt_face, gt_off, fn0, fr0, dd0);
    if (gt_second) {
      int face, off, fn, fr, dd;
      if (ghost_task(gq, true, face, off, fn, fr, dd)) {
        const float4 fnv = __ldg(a.faces32[1] + (fn + sJ * kp)), frv = __ldg(a.faces32[0] + (fr + sI * kp));
        float ddv = 0.f;
        if constexpr (TURB) ddv = __ldg(a.dist32 + (dd + sC * kp));
        apply(face, off, fnv, frv, ddv);
      }
    }
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
  // viscous march state: raw gradient of cell (i, j, k-1), viscous dt terms
  T Gprev[VISC ? NGC : 1];
#pragma unroll
  for (int m = 0; m < (VISC ? NGC : 1); ++m) Gprev[m] = T(0);
  T lvk_prev = 0, lvi_lo_prev = 0, lvi_hi_prev = 0, lvj_lo_prev = 0, lvj_hi_prev = 0;
  // SST march state: mu_t, F1 and source of cell (i, j, k-1), turbulent dt terms
  T mut_prev = 0, F1_prev = 0, Sk_prev = 0, Sw_prev = 0;
  T ltk_prev = 0, lti_lo_prev = 0, lti_hi_prev = 0, ltj_lo_prev = 0, ltj_hi_prev = 0;
  const T Rg = pv<T>(p.R, p.f_R);
  // the temperature of a cell's gradient sums: FP64 reads the iteration's
  // start (a.Temp), FP32 takes its stage's own (a negative value)
  auto tgrad = [&](int ii, int jj, int kk) -> T {
    if constexpr (sizeof(T) == 8) return __ldg(a.Temp + pidx(d, clampi(ii, d.imx), clampi(jj, d.jmx), kk));
    else return T(-1);
  };

  const long long sj = d.ni, sk = (long long)d.ni * d.nj;
  for (int n = 0; n < nplanes; ++n) {
    const int kl = base + n;  // plane arriving now
    __syncthreads();
    // ghost tasks on plane kl (FP32): face records fetched while it is in flight
    const bool gij_now = (gt_face >= 0 || gt_second) && kl >= 1 && kl <= d.kmx - 1;
    float4 g_fn = make_float4(0.f, 0.f, 0.f, 0.f), g_fr = g_fn;
    float g_dd = 0.f;
    if (gt_face >= 0 && gij_now) {
      g_fn = __ldg(a.faces32[gt_face / 2] + (gt_fn + (gt_face < 2 ? sI : sJ) * kl));
      g_fr = gt_face < 2 ? g_fn : __ldg(a.faces32[0] + (gt_fr + sI * kl));
      if constexpr (TURB) g_dd = __ldg(a.dist32 + (gt_dd + sC * kl));
    }
    if constexpr (kTma) {
      if (abort_flag) return;  // uniform: read after the barrier
      // the slot of plane n+1 last held plane n+1-NR, read up to iteration n-1
      if (tid == 0 && n + 1 >= NR && n + 1 < nplanes) issue(kl + 1);
      if (!mbar_wait(bars + slot(kl), (uint32_t)((n / NR) & 1))) {
        raise_error(a.err, FEST_ERR_TIMEOUT);
        abort_flag = 1;
      }
      if (rgm) {
        float* ringf = reinterpret_cast<float*>(ring);
        // k ghost planes: read in this very step, so computed by all
        // threads and published by a barrier (uniform over the CTA)
        const bool fix_klo = (rgm & 16) && kl == 2 && base <= 0;  // plane 0 from planes 1, 2
        const bool fix_khi = (rgm & 32) && kl == d.kmx;           // plane kmx from kmx-1, kmx-2
        if (fix_klo || fix_khi) {
          auto fix_kplane = [&](int f, int kg, int ka, int kb) {
            float* G0 = ringf + slot(kg) * plane;
            const float* A1 = ringf + slot(ka) * plane;
            const float* A2 = ringf + slot(kb) * plane;
            const int fk = f == 4 ? 1 : d.kmx;
            for (int e = tid; e < SH * RW; e += TX * TY) {
              const int r = e / RW, c = e - r * RW;
              const int ii = c + ib - 3 - ox, jj = jb - 3 + r;
              if (ii < 1 || ii > d.imx - 1 || jj < 1 || jj > d.jmx - 1) continue;
              const float4 fn = __ldg(a.faces32[2] + fidx(d, 2, ii, jj, fk));
              const float4 fr = __ldg(a.faces32[0] + fidx(d, 0, ii, jj, fk));
              float dd1 = 0.f;
              if constexpr (TURB) dd1 = __ldg(a.dist32 + pidx(d, ii, jj, ka));
              ghost_layer1<NV>(p, f, G0 + e, A1 + e, A2 + e, VS, fn, fr, dd1);
            }
          };
          if (fix_klo) fix_kplane(4, 0, 1, 2);
          if (fix_khi) {
            if (fix_klo) __syncthreads();  // a single interior plane: kmin's ghosts first
            fix_kplane(5, d.kmx, d.kmx - 1, d.kmx - 2);
          }
          __syncthreads();
        }
      }
    } else {
      load_plane(kl);
      __syncthreads();
    }
    const int k = kl - 2;  // plane processed now
    // i/j ghost cells of plane kl are first read two steps later, as the
    // own plane's i/j stencils (this step reads plane kl at interior
    // columns only): the halo warps make them at the end of the step, or
    // now when the step has nothing else to do
    if (k < k0 - 1) {
      if (gij_now) ij_ghosts(kl, g_fn, g_fr, g_dd);
      continue;
    }
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
    // viscous: this cell's values, centre, viscosity and raw Green-Gauss
    // gradient (every thread, halo included); SST: its mu_t, F1 and source
    ViscCell<T> Vc{};
    R4<T> cown = mk4(T(1), T(0), T(0), T(0));
    T muc = T(0), Gc[VISC ? NGC : 1];
    T lvi_lo = 0, lvi_hi = 0, lvj_lo = 0, lvj_hi = 0;
    SstCell<T> Sc{T(0), T(0), T(0), T(0)};
    T ddc = T(1), Skc = T(0), Swc = T(0);
    T lti_lo = 0, lti_hi = 0, ltj_lo = 0, ltj_hi = 0;
    const int ci_ = clampi(i, d.imx), cj_ = clampi(j, d.jmx);
    if constexpr (VISC) {
      const T* o = own;
      Vc = visc_cell<TURB>(o, VS, Rg, tgrad(i, j, k));
      ViscCell<T> nb[6];
      nb[0] = visc_cell<TURB>(o - 1, VS, Rg, tgrad(i - 1, j, k));
      nb[1] = visc_cell<TURB>(o - RW, VS, Rg, tgrad(i, j - 1, k));
      nb[2] = visc_cell<TURB>(ring + slot(k - 1) * plane + r * RW + cc, VS, Rg, tgrad(i, j, k - 1));
      nb[3] = visc_cell<TURB>(o + 1, VS, Rg, tgrad(i + 1, j, k));
      nb[4] = visc_cell<TURB>(o + RW, VS, Rg, tgrad(i, j + 1, k));
      nb[5] = visc_cell<TURB>(ring + slot(k + 1) * plane + r * RW + cc, VS, Rg, tgrad(i, j, k + 1));
      const int ci1 = clampi(i + 1, d.imx + 1), cj1 = clampi(j + 1, d.jmx + 1);
      R4<T> fgg[6];
      fgg[0] = ld_face4(a, 0, fidx(d, 0, ci_, cj_, k), T(0));
      fgg[1] = ld_face4(a, 1, fidx(d, 1, ci_, cj_, k), T(0));
      fgg[2] = ld_face4(a, 2, fidx(d, 2, ci_, cj_, k), T(0));
      fgg[3] = ld_face4(a, 0, fidx(d, 0, ci1, cj_, k), T(0));
      fgg[4] = ld_face4(a, 1, fidx(d, 1, ci_, cj1, k), T(0));
      fgg[5] = ld_face4(a, 2, fidx(d, 2, ci_, cj_, k + 1), T(0));
      cown = ld_cell4(a, pidx(d, ci_, cj_, k), T(0));
      visc_gg<NGV>(Vc, nb, fgg, cown.x, thin, Gc);
      muc = visc_mu(p, Vc.Tm);
      if constexpr (TURB) {
        ddc = ld_dist(a, pidx(d, ci_, cj_, k), T(0));
        Sc = sst_cell(p, Vc, muc, ddc, Gc);
        if (kin && in_i && in_j) sst_source(p, Vc, Sc, Gc, cown.x, Skc, Swc);
      }
    }
    // ---------------- i-faces (warp shuffles) ----------------
    if (kin && in_j) {  // warp-uniform
      T Rm[NV], Lp[NV];
      const T* rowp = ring + slot(k) * plane + r * RW;
      const auto vol = vol_line(a, T(0), pidx(d, 0, clampi(j, d.jmx), k), 1, d.imx);
      SmemLine<T> pres{rowp + 4 * SH * RW + cc, i, 1};
      // not unrolled: the sweep's code outgrows the instruction cache
      // (stalls on instruction fetch were the largest before this)
      auto iline = [&](int l) { return SmemLine<T>{rowp + l * SH * RW + cc, i, 1}; };
      recon_vars<T, INTERP, NV, !(sizeof(T) == 4 && INTERP == FEST_INTERP_WENO)>(p, 0, i, iline, pres, vol, Rm, Lp);
      T L[NV], F[NV];
#pragma unroll
      for (int l = 0; l < NV; ++l) L[l] = __shfl_up_sync(0xffffffffu, Lp[l], 1);
      T A, nx, ny, nz;
      load_face(a, 0, fidx(d, 0, clampi(i, d.imx), clampi(j, d.jmx), k), A, nx, ny, nz);
      face_flux<T, FLUX>(p, L, Rm, A, nx, ny, nz, (T)wall_mask(p, 0, i), F);
      if (a.compute_dt) lami_lo = lambda_face<T>(gm, L, Rm, A, nx, ny, nz, qc[1], qc[2], qc[3]);
      lami_hi = __shfl_down_sync(0xffffffffu, lami_lo, 1);
      if constexpr (VISC) {  // viscous flux of the low i-face (cells i-1, i)
        T Gl[NGC], GL[NGC], GR[NGC], Fv[TURB ? 6 : 4];
#pragma unroll
        for (int m = 0; m < NGC; ++m) Gl[m] = __shfl_up_sync(0xffffffffu, Gc[m], 1);
#pragma unroll
        for (int m = 0; m < NGC; ++m) { GL[m] = Gl[m]; GR[m] = Gc[m]; }
        const ViscCell<T> VL = visc_cell<TURB>(own - 1, VS, Rg, tgrad(i - 1, j, k));
        const R4<T> cL = ld_cell4(a, pidx(d, clampi(i - 1, d.imx), cj_, k), T(0));
        const R4<T> fc = mk4(A, nx, ny, nz);
        const T muL = visc_mu(p, VL.Tm);
        T mutL = T(0), F1L = T(0), mutR = Sc.mut, F1R = Sc.F1;
        if constexpr (TURB) {
          mutL = __shfl_up_sync(0xffffffffu, Sc.mut, 1);
          F1L = __shfl_up_sync(0xffffffffu, Sc.F1, 1);
        }
        const T mutLi = mutL, F1Li = F1L;
        if (i - 1 == 0 && p.id[0] < 0) {
          visc_gbc<NGV>(p, 0, Gc, Vc, VL, cown.x, fc, GL);
          if constexpr (TURB)
            sst_ghost(p, 0, VL, muL, GL, ld_dist(a, pidx(d, clampi(i - 1, d.imx), cj_, k), T(0)), Sc.mut,
                      Sc.F1, mutL, F1L);
        }
        if (i == d.imx && p.id[1] < 0) {
          visc_gbc<NGV>(p, 1, Gl, VL, Vc, cL.x, fc, GR);
          if constexpr (TURB) sst_ghost(p, 1, Vc, muc, GR, ddc, mutLi, F1Li, mutR, F1R);
        }
        visc_flux<TURB>(p, GL, GR, VL, Vc, cL, cown, muL, muc, mutL, mutR, F1L, F1R, fc, true, Fv);
#pragma unroll
        for (int l = 0; l < 4; ++l) F[1 + l] -= Fv[l];
        if constexpr (TURB) { F[5] -= Fv[4]; F[6] -= Fv[5]; }
        if (a.compute_dt) {
          lvi_lo = visc_lambda(fc, cL, cown, muc, Vc.rho);
          if constexpr (TURB) lti_lo = visc_lambda(fc, cL, cown, mutR, Vc.rho);
        }
        lvi_hi = __shfl_down_sync(0xffffffffu, lvi_lo, 1);
        if constexpr (TURB) lti_hi = __shfl_down_sync(0xffffffffu, lti_lo, 1);
      }
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
      auto jline = [&](int l) { return SmemLine<T>{colp + l * SH * RW + r * RW, j, RW}; };
      recon_vars<T, INTERP, NV, !(sizeof(T) == 4 && INTERP == FEST_INTERP_WENO)>(p, 1, j, jline, pres, vol, Rm, Lp);
#pragma unroll
      for (int l = 0; l < NV; ++l) xch[(l * TY + w) * TX + lane] = Lp[l];
      if constexpr (VISC) {
#pragma unroll
        for (int m = 0; m < NGC; ++m) gxch[(m * TY + w) * TX + lane] = Gc[m];
        if constexpr (TURB) {
          mutx[w * TX + lane] = Sc.mut;
          f1x[w * TX + lane] = Sc.F1;
        }
      }
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
        if constexpr (VISC) {  // viscous flux of the low j-face (cells j-1, j)
          T Gd[NGC], GL[NGC], GR[NGC], Fv[TURB ? 6 : 4];
#pragma unroll
          for (int m = 0; m < NGC; ++m) Gd[m] = gxch[(m * TY + w - 1) * TX + lane];
          const ViscCell<T> VD = visc_cell<TURB>(own - RW, VS, Rg, tgrad(i, j - 1, k));
          const R4<T> cD = ld_cell4(a, pidx(d, ci_, clampi(j - 1, d.jmx), k), T(0));
          const R4<T> fc = mk4(A, nx, ny, nz);
          const T muD = visc_mu(p, VD.Tm);
          T mutD = T(0), F1D = T(0), mutR = Sc.mut, F1R = Sc.F1;
          if constexpr (TURB) {
            mutD = mutx[(w - 1) * TX + lane];
            F1D = f1x[(w - 1) * TX + lane];
          }
          const T mutDi = mutD, F1Di = F1D;
#pragma unroll
          for (int m = 0; m < NGC; ++m) { GL[m] = Gd[m]; GR[m] = Gc[m]; }
          if (j - 1 == 0 && p.id[2] < 0) {
            visc_gbc<NGV>(p, 2, Gc, Vc, VD, cown.x, fc, GL);
            if constexpr (TURB)
              sst_ghost(p, 2, VD, muD, GL, ld_dist(a, pidx(d, ci_, clampi(j - 1, d.jmx), k), T(0)), Sc.mut,
                        Sc.F1, mutD, F1D);
          }
          if (j == d.jmx && p.id[3] < 0) {
            visc_gbc<NGV>(p, 3, Gd, VD, Vc, cD.x, fc, GR);
            if constexpr (TURB) sst_ghost(p, 3, Vc, muc, GR, ddc, mutDi, F1Di, mutR, F1R);
          }
          visc_flux<TURB>(p, GL, GR, VD, Vc, cD, cown, muD, muc, mutD, mutR, F1D, F1R, fc, true, Fv);
#pragma unroll
          for (int l = 0; l < 4; ++l) F[1 + l] -= Fv[l];
          if constexpr (TURB) { F[5] -= Fv[4]; F[6] -= Fv[5]; }
          if (a.compute_dt) {
            lvj_lo = visc_lambda(fc, cD, cown, muc, Vc.rho);
            lamv[w * TX + lane] = lvj_lo;
            if constexpr (TURB) {
              ltj_lo = visc_lambda(fc, cD, cown, mutR, Vc.rho);
              lamt[w * TX + lane] = ltj_lo;
            }
          }
        }
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
        if constexpr (VISC)
          if (a.compute_dt) {
            lvj_hi = lamv[(w + 1) * TX + lane];
            if constexpr (TURB) ltj_hi = lamt[(w + 1) * TX + lane];
          }
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
      auto kline = [&](int l) { return RingLine<T>{cp + l * SH * RW, plane, base}; };
      recon_vars<T, INTERP, NV, false>(p, 2, k, kline, pres, vol, Rm, Lp);
      T H[NV];
      T lamk = 0;
      T lvk = 0, ltk = 0;
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
        if constexpr (VISC) {  // viscous flux of the low k-face (cells k-1, k)
          T GL[NGC], GR[NGC], Fv[TURB ? 6 : 4];
          const ViscCell<T> VK = visc_cell<TURB>(ring + slot(k - 1) * plane + r * RW + cc, VS, Rg, tgrad(i, j, k - 1));
          const R4<T> cK = ld_cell4(a, pidx(d, i, j, k - 1), T(0));
          const R4<T> fc = mk4(A, nx, ny, nz);
          const T muK = visc_mu(p, VK.Tm);
          T mutK = mut_prev, F1K = F1_prev, mutR = Sc.mut, F1R = Sc.F1;
#pragma unroll
          for (int m = 0; m < NGC; ++m) { GL[m] = Gprev[m]; GR[m] = Gc[m]; }
          if (k - 1 == 0 && p.id[4] < 0) {
            visc_gbc<NGV>(p, 4, Gc, Vc, VK, cown.x, fc, GL);
            if constexpr (TURB)
              sst_ghost(p, 4, VK, muK, GL, ld_dist(a, pidx(d, i, j, k - 1), T(0)), Sc.mut, Sc.F1, mutK, F1K);
          }
          if (k == d.kmx && p.id[5] < 0) {
            visc_gbc<NGV>(p, 5, Gprev, VK, Vc, cK.x, fc, GR);
            if constexpr (TURB) sst_ghost(p, 5, Vc, muc, GR, ddc, mut_prev, F1_prev, mutR, F1R);
          }
          visc_flux<TURB>(p, GL, GR, VK, Vc, cK, cown, muK, muc, mutK, mutR, F1K, F1R, fc, !thin, Fv);
#pragma unroll
          for (int l = 0; l < 4; ++l) H[1 + l] -= Fv[l];
          if constexpr (TURB) { H[5] -= Fv[4]; H[6] -= Fv[5]; }
          if (a.compute_dt) {
            lvk = visc_lambda(fc, cK, cown, muc, Vc.rho);
            if constexpr (TURB) ltk = visc_lambda(fc, cK, cown, mutR, Vc.rho);
          }
        }
        if (a.mflux[2] && (k == 1 || k == d.kmx)) a.mflux[2][flidx(fldim(d, 2), i, j, k)] = (double)H[0];
        if (k >= k0 + 1) {
          // cell (i, j, k-1) is complete: residual (scheme.f90:133-135)
          const int kc = k - 1;
          const long long c0 = pidx(d, i, j, kc), ci = cidx(d, i, j, kc);
          T R[NV];
#pragma unroll
          for (int l = 0; l < NV; ++l) R[l] = (dF_prev[l] + dG_prev[l]) + (H[l] - H_prev[l]);
          if constexpr (TURB) {  // add_sst_source (source.f90:265-266)
            R[5] = R[5] - Sk_prev;
            R[6] = R[6] - Sw_prev;
          }
          const T vol_c = cell_vol(a, T(0), c0);
          T dtc;
          if (a.compute_dt) {
            T s = lami_lo_prev + lamj_lo_prev + lamk_prev + lami_hi_prev + lamj_hi_prev + lamk;
            dtc = (T(1) / s) * vol_c * pv<T>(a.CFL, a.f_CFL);
            if constexpr (VISC) {  // add_viscous_time (time.f90:366-448)
              const T cfl = pv<T>(a.CFL, a.f_CFL);
              T sv = lvi_lo_prev + lvj_lo_prev + lvk_prev + lvi_hi_prev + lvj_hi_prev + lvk;
              sv = pv<T>(p.gm, p.f_gm) * sv / pv<T>(p.Pr, p.f_Pr);
              sv = T(2) / (sv + (T(2) * cfl * vol_c / dtc));
              dtc = cfl * (sv * vol_c);
            }
            if constexpr (TURB) {  // add_turbulent_time (time.f90:450-531)
              const T cfl = pv<T>(a.CFL, a.f_CFL);
              T st = lti_lo_prev + ltj_lo_prev + ltk_prev + lti_hi_prev + ltj_hi_prev + ltk;
              st = pv<T>(p.gm, p.f_gm) * st / pv<T>(p.tPr, p.f_tPr);
              st = T(2) / (st + (T(2) * cfl * vol_c / dtc));
              dtc = cfl * (st * vol_c);
            }
            a.dt[ci] = to_f64(dtc);
          } else {
            dtc = from_f64(a.dt[ci], T(0));
          }
          if (a.res_out)
#pragma unroll
            for (int l = 0; l < NV; ++l) a.res_out[ci + ncells(d) * l] = to_f64(R[l]);
          // the finished cell's own stencil values (plane k-1 of the ring)
          T qo[NV];
          const T* own1 = ring + slot(kc) * plane + r * RW + cc;
#pragma unroll
          for (int l = 0; l < NV; ++l) qo[l] = own1[l * SH * RW];
          const long long m0 = (long long)(i + 2) + (long long)a.mpitch * ((j + 2) + (long long)d.nj * (kc + 2));
          bool ok;
          if constexpr (kTma) ok = update_cell_f32<NV>(p, a, c0, ci, R, dtc, vol_c, qo, m0, F1_prev);
          else ok = update_cell<NV>(p, a, c0, ci, R, dtc, vol_c, qo, m0, F1_prev);
          if (!ok) raise_error(a.err, FEST_ERR_NEGATIVE_STATE);
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
      if constexpr (VISC) {
#pragma unroll
        for (int m = 0; m < NGC; ++m) Gprev[m] = Gc[m];
        if (k >= k0) lvk_prev = lvk;
        if (kin) {
          lvi_lo_prev = lvi_lo; lvi_hi_prev = lvi_hi;
          lvj_lo_prev = lvj_lo; lvj_hi_prev = lvj_hi;
        }
      }
      if constexpr (TURB) {
        mut_prev = Sc.mut;
        F1_prev = Sc.F1;
        Sk_prev = Skc;
        Sw_prev = Swc;
        if (k >= k0) ltk_prev = ltk;
        if (kin) {
          lti_lo_prev = lti_lo; lti_hi_prev = lti_hi;
          ltj_lo_prev = ltj_lo; ltj_hi_prev = ltj_hi;
        }
      }
    }
    if (gij_now) ij_ghosts(kl, g_fn, g_fr, g_dd);  // halo warps, published by the next barrier
  }
}

// MB: CTAs per SM the registers are budgeted for (FP32: 2 = 115 registers,
// no spills, fewer instructions; 3 = 80 registers, more warps to hide
// latency on large blocks; the tuner picks per block)
template <typename T, int INTERP, int FLUX, int MB, bool VISC = false, bool TURB = false>
__global__ void __launch_bounds__(TX* TY, MB)
    k_stage(Params p, StageArgs a, const __grid_constant__ CUtensorMap tm) {
  stage_body<T, INTERP, FLUX, VISC, TURB>(p, a, &tm, blockIdx.x, blockIdx.y, blockIdx.z);
}

// One launch for every block of a batch: block b owns CTAs
// [cta0, cta0 + tx*ty*nz) of the 1-D grid.
template <typename T, int INTERP, int FLUX, bool VISC = false, bool TURB = false>
__global__ void __launch_bounds__(TX* TY, TURB ? 1 : (VISC ? 2 : (sizeof(T) == 4 ? 3 : 1)))
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
  stage_body<T, INTERP, FLUX, VISC, TURB>(sp, sa, &E.tm, local % E.tx, (local / E.tx) % E.ty,
                                         local / (E.tx * E.ty));
}

template <typename T, bool VISC = false, bool TURB = false> inline size_t stage_smem() {
  constexpr size_t NV = TURB ? 7 : 5, NXV = VISC ? (TURB ? 18 + 4 : 12 + 1) : 0;
  return sizeof(T) * ((size_t)RingGeom<T>::N * NV * SH * RingGeom<T>::W + 2 * NV * TY * TX + TY * TX) +
         sizeof(T) * NXV * TY * TX + sizeof(uint64_t) * RingGeom<T>::N + 16;
}


}  // namespace stage

// one host launcher per reconstruction (fest_stage_<method>.cu)
#define FEST_STAGE_LAUNCHER(name)                                                         \
  int name(int prec, int flux, int occ, dim3 grid, cudaStream_t s, const Params& p, const StageArgs& a, \
           const CUtensorMap& tm)
// the FP64 viscous and SST sweeps (fest_stage_<method>_visc64.cu, _sst64.cu)
FEST_STAGE_LAUNCHER(launch_stage_none_visc64);
FEST_STAGE_LAUNCHER(launch_stage_muscl_visc64);
FEST_STAGE_LAUNCHER(launch_stage_ppm_visc64);
FEST_STAGE_LAUNCHER(launch_stage_weno_visc64);
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_visc64);
FEST_STAGE_LAUNCHER(launch_stage_none_sst64);
FEST_STAGE_LAUNCHER(launch_stage_muscl_sst64);
FEST_STAGE_LAUNCHER(launch_stage_ppm_sst64);
FEST_STAGE_LAUNCHER(launch_stage_weno_sst64);
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_sst64);
// the SST FP32 sweeps (fest_stage_<method>_sst.cu)
FEST_STAGE_LAUNCHER(launch_stage_none_sst);
FEST_STAGE_LAUNCHER(launch_stage_muscl_sst);
FEST_STAGE_LAUNCHER(launch_stage_ppm_sst);
FEST_STAGE_LAUNCHER(launch_stage_weno_sst);
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_sst);
// the laminar-viscous FP32 sweeps (fest_stage_<method>_visc.cu)
FEST_STAGE_LAUNCHER(launch_stage_none_visc);
FEST_STAGE_LAUNCHER(launch_stage_muscl_visc);
FEST_STAGE_LAUNCHER(launch_stage_ppm_visc);
FEST_STAGE_LAUNCHER(launch_stage_weno_visc);
FEST_STAGE_LAUNCHER(launch_stage_weno_nm_visc);
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
FEST_BATCH_LAUNCHER(launch_batch_none_sst);
FEST_BATCH_LAUNCHER(launch_batch_muscl_sst);
FEST_BATCH_LAUNCHER(launch_batch_ppm_sst);
FEST_BATCH_LAUNCHER(launch_batch_weno_sst);
FEST_BATCH_LAUNCHER(launch_batch_weno_nm_sst);
FEST_BATCH_LAUNCHER(launch_batch_none_visc);
FEST_BATCH_LAUNCHER(launch_batch_muscl_visc);
FEST_BATCH_LAUNCHER(launch_batch_ppm_visc);
FEST_BATCH_LAUNCHER(launch_batch_weno_visc);
FEST_BATCH_LAUNCHER(launch_batch_weno_nm_visc);

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

// the laminar-viscous sweep: FP32 with one register budget (1 CTA of 256
// threads per 64K registers would waste the SM, so MB = 2 with what
// spills); FP64 one CTA per SM
template <int INTERP, typename T = float>
int launch_stage_visc_t(int flux, dim3 grid, cudaStream_t s, const Params& p, const StageArgs& a,
                        const CUtensorMap& tm) {
  using namespace stage;
  constexpr int MB = sizeof(T) == 4 ? 2 : 1;
  const dim3 blk(TX, TY);
  static bool attrs = false;
  const size_t smem = stage_smem<T, true>();
#define FEST_SET(F) \
  cudaFuncSetAttribute(k_stage<T, INTERP, F, MB, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
  if (!attrs) {
    FEST_SET(0); FEST_SET(1); FEST_SET(2); FEST_SET(3); FEST_SET(4); FEST_SET(5);
    attrs = true;
  }
#undef FEST_SET
#define FEST_GO(F) k_stage<T, INTERP, F, MB, true><<<grid, blk, smem, s>>>(p, a, tm)
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

// the SST sweep: seven variables and the SST exchange need ~118 KB (FP32)
// or ~197 KB (FP64) of shared memory, so one CTA per SM with the whole
// register file
template <int INTERP, typename T = float>
int launch_stage_sst_t(int flux, dim3 grid, cudaStream_t s, const Params& p, const StageArgs& a,
                       const CUtensorMap& tm) {
  using namespace stage;
  const dim3 blk(TX, TY);
  static bool attrs = false;
  const size_t smem = stage_smem<T, true, true>();
#define FEST_SET(F)                                                                                      \
  cudaFuncSetAttribute(k_stage<T, INTERP, F, 1, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)smem)
  if (!attrs) {
    FEST_SET(0); FEST_SET(1); FEST_SET(2); FEST_SET(3); FEST_SET(4); FEST_SET(5);
    attrs = true;
  }
#undef FEST_SET
#define FEST_GO(F) k_stage<T, INTERP, F, 1, true, true><<<grid, blk, smem, s>>>(p, a, tm)
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

template <int INTERP>
int launch_batch_sst_t(int flux, int ctas, cudaStream_t s, const BatchEntry* e, int nb) {
  using namespace stage;
  const dim3 blk(TX, TY);
  static bool attrs = false;
  const size_t smem = stage_smem<float, true, true>();
#define FEST_SET(F)                                                                                          \
  cudaFuncSetAttribute(k_stage_batch<float, INTERP, F, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                       (int)smem)
  if (!attrs) {
    FEST_SET(0); FEST_SET(1); FEST_SET(2); FEST_SET(3); FEST_SET(4); FEST_SET(5);
    attrs = true;
  }
#undef FEST_SET
#define FEST_GO(F) k_stage_batch<float, INTERP, F, true, true><<<ctas, blk, smem, s>>>(e, nb)
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

template <int INTERP>
int launch_batch_visc_t(int flux, int ctas, cudaStream_t s, const BatchEntry* e, int nb) {
  using namespace stage;
  const dim3 blk(TX, TY);
  static bool attrs = false;
  const size_t smem = stage_smem<float, true>();
#define FEST_SET(F) \
  cudaFuncSetAttribute(k_stage_batch<float, INTERP, F, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
  if (!attrs) {
    FEST_SET(0); FEST_SET(1); FEST_SET(2); FEST_SET(3); FEST_SET(4); FEST_SET(5);
    attrs = true;
  }
#undef FEST_SET
#define FEST_GO(F) k_stage_batch<float, INTERP, F, true><<<ctas, blk, smem, s>>>(e, nb)
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
