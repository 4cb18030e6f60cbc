// fest_common.cuh - device-side parameter block, index maps and the pointwise
// numerics of FEST-3D's explicit path (reconstruction, boundary-face
// override, convective fluxes), templated on the arithmetic type so the FP64
// module kernels and the FP32 fused sweep share one implementation.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fest_gpu.h"

namespace fest {

constexpr int NVMAX = 7;
// the module kernels' bound: LCTM2015 adds the intermittency as an eighth
// variable on the module path only (the fused sweep and the VJP keep NVMAX)
constexpr int NVMOD = 8;

struct Dims {
  int imx, jmx, kmx, nv;  // node counts (vartypes.f90:21-26) and n_var
  int ni, nj, nk;          // padded cell extents imx+5 ...
  long long P;             // padded cells per variable
};

// Everything a kernel needs from flowtype/schemetype/boundarytype, by value.
struct Params {
  Dims d;
  double gm, R, mu_ref, T_ref, S, Pr, tPr, MInf, p_inf, rho_inf, u_inf, v_inf, w_inf;
  int flux, interp, limiter, turb, mu_var, ppm_flag, n_grad, tstep;
  double gdt;  // schemetype%global_time_step
  int integ;   // schemetype%time_step_accuracy (FEST_TIME_*)
  int lam[3], tlim[3], pb[3];
  int id[6];
  // interface partners: block (index into the ghost fill's block table,
  // -1 while unresolved), face, orientation (bit 0/1: first/second
  // tangential direction reversed, bit 2: swapped); self_block: this
  // block's own index in that table
  int part_block[6], part_face[6], part_orient[6];
  int self_block;
  double c1, c2, c3;
  double fix_rho[6], fix_p[6], fix_u[6], fix_v[6], fix_w[6], fix_tk[6], fix_tw[6], fix_tv[6], fix_tkl[6], fix_tgm[6];
  // Spalart-Allmaras: cv1**3, folded on the host to the correctly rounded
  // power as the reference's compiler folds its parameter
  double sa_cv1_3;
  // k-kL: cmu**0.25 and cmu**0.75, folded on the host likewise
  double kkl_c025, kkl_c075;
  // the 'bc' transition model (FEST_TRANSITION_*): its critical eddy
  // viscosity 5/Re and transition Reynolds number 803.73 (Tu + 0.6067)**-1.027,
  // both uniform, taken on the host
  int transition;
  double bc_nu_cr, bc_re_theta_t;
  double Tw[6], Tp[6];
  // FP32 copies of the constants the FP32 sweep uses (rounded on the host,
  // so the device does no FP64 conversions for them)
  float f_gm, f_gm1, f_R, f_MInf, f_p_inf, f_rho_inf, f_u_inf, f_v_inf, f_w_inf;
  float f_mu_ref, f_T_ref, f_S, f_Pr, f_tPr, f_c1, f_c2, f_c3;
  float f_Tw[6], f_Tp[6];
};

// fill the FP32 copies in a Params from its FP64 fields
inline void params_f32(Params& p) {
  p.f_gm = (float)p.gm; p.f_gm1 = (float)(p.gm - 1.0); p.f_R = (float)p.R; p.f_MInf = (float)p.MInf;
  p.f_p_inf = (float)p.p_inf; p.f_rho_inf = (float)p.rho_inf;
  p.f_u_inf = (float)p.u_inf; p.f_v_inf = (float)p.v_inf; p.f_w_inf = (float)p.w_inf;
  p.f_mu_ref = (float)p.mu_ref; p.f_T_ref = (float)p.T_ref; p.f_S = (float)p.S;
  p.f_Pr = (float)p.Pr; p.f_tPr = (float)p.tPr;
  p.f_c1 = (float)p.c1; p.f_c2 = (float)p.c2; p.f_c3 = (float)p.c3;
  for (int f = 0; f < 6; ++f) { p.f_Tw[f] = (float)p.Tw[f]; p.f_Tp[f] = (float)p.Tp[f]; }
}

// a Params constant in the arithmetic type T: the FP64 field (FP64 and dual
// numbers), or its FP32 copy
template <typename T> __host__ __device__ __forceinline__ T pv(double d, float) { return T(d); }
template <> __host__ __device__ __forceinline__ float pv<float>(double, float f) { return f; }

// ---- index maps (Fortran column-major, lower bounds as in the reference) ----
__host__ __device__ __forceinline__ long long pidx(const Dims& d, int i, int j, int k) {
  return ((long long)(k + 2) * d.nj + (j + 2)) * d.ni + (i + 2);
}
// faces of direction dir: (-2:imx+2+f0, -2:jmx+2+f1, -2:kmx+2+f2)
__host__ __device__ __forceinline__ long long fidx(const Dims& d, int dir, int i, int j, int k) {
  int n0 = d.ni + (dir == 0), n1 = d.nj + (dir == 1);
  return ((long long)(k + 2) * n1 + (j + 2)) * n0 + (i + 2);
}
__host__ __device__ __forceinline__ long long nfaces(const Dims& d, int dir) {
  return (long long)(d.ni + (dir == 0)) * (d.nj + (dir == 1)) * (d.nk + (dir == 2));
}
// face-state arrays x_qp_left etc: (1-f0:imx-1+2f0, 1-f1:..., 1-f2:...)
struct FSDim { int lo0, lo1, lo2, n0, n1, n2; long long N; };
__host__ __device__ __forceinline__ FSDim fsdim(const Dims& d, int dir) {
  FSDim s;
  int f0 = dir == 0, f1 = dir == 1, f2 = dir == 2;
  s.lo0 = 1 - f0; s.lo1 = 1 - f1; s.lo2 = 1 - f2;
  s.n0 = d.imx - 1 + 3 * f0; s.n1 = d.jmx - 1 + 3 * f1; s.n2 = d.kmx - 1 + 3 * f2;
  s.N = (long long)s.n0 * s.n1 * s.n2;
  return s;
}
__host__ __device__ __forceinline__ long long fsidx(const FSDim& s, int i, int j, int k) {
  return ((long long)(k - s.lo2) * s.n1 + (j - s.lo1)) * s.n0 + (i - s.lo0);
}
// flux arrays F/G/H: (1:imx-1+f0, 1:jmx-1+f1, 1:kmx-1+f2)
struct FlDim { int n0, n1, n2; long long N; };
__host__ __device__ __forceinline__ FlDim fldim(const Dims& d, int dir) {
  FlDim s;
  s.n0 = d.imx - 1 + (dir == 0); s.n1 = d.jmx - 1 + (dir == 1); s.n2 = d.kmx - 1 + (dir == 2);
  s.N = (long long)s.n0 * s.n1 * s.n2;
  return s;
}
__host__ __device__ __forceinline__ long long flidx(const FlDim& s, int i, int j, int k) {
  return ((long long)(k - 1) * s.n1 + (j - 1)) * s.n0 + (i - 1);
}
// interior cell arrays (residue, delta_t): (1:imx-1, 1:jmx-1, 1:kmx-1)
__host__ __device__ __forceinline__ long long ncells(const Dims& d) {
  return (long long)(d.imx - 1) * (d.jmx - 1) * (d.kmx - 1);
}
__host__ __device__ __forceinline__ long long cidx(const Dims& d, int i, int j, int k) {
  return ((long long)(k - 1) * (d.jmx - 1) + (j - 1)) * (d.imx - 1) + (i - 1);
}
// gradient arrays: (0:imx, 0:jmx, 0:kmx)
__host__ __device__ __forceinline__ long long ngrad(const Dims& d) {
  return (long long)(d.imx + 1) * (d.jmx + 1) * (d.kmx + 1);
}
__host__ __device__ __forceinline__ long long gidx(const Dims& d, int i, int j, int k) {
  return ((long long)k * (d.jmx + 1) + j) * (d.imx + 1) + i;
}
__host__ __device__ __forceinline__ int extent_of(const Dims& d, int dir) {
  return dir == 0 ? d.imx : dir == 1 ? d.jmx : d.kmx;
}
__host__ __device__ __forceinline__ long long pstride(const Dims& d, int dir) {
  return dir == 0 ? 1 : dir == 1 ? (long long)d.ni : (long long)d.ni * d.nj;
}

// Tangential position (pa, pb) on the partner face of ghost column (ta, tb)
// of an interface face with na x nb interior columns: the receive loops of
// apply_interface (interface1.f90:96-464) over the index ranges of
// change_map_to_particular_range (mapping.f90:159-236).  orient bit 0/1
// reverses the first/second tangential direction, bit 2 swaps them.
__host__ __device__ __forceinline__ void interface_map(int orient, int na, int nb, int ta, int tb, int& pa,
                                                       int& pb) {
  const int a = (orient & 1) ? na - ta : ta - 1;
  const int b = (orient & 2) ? nb - tb : tb - 1;
  if (orient & 4) { pa = 1 + b; pb = 1 + a; }
  else { pa = 1 + a; pb = 1 + b; }
}
// interior columns of face f (its two tangential extents)
__host__ __device__ __forceinline__ void face_columns(const Dims& d, int f, int& na, int& nb) {
  na = (f / 2 == 0 ? d.jmx : d.imx) - 1;
  nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
}

// ---- Fortran intrinsics with the reference's semantics ----------------------
template <typename T> __device__ __forceinline__ T fsign1(T m) { return copysign(T(1), m); }
template <typename T> __device__ __forceinline__ T fmax2(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T fmin2(T a, T b) { return a < b ? a : b; }
// max(0, 1-floor(|M|)) (ausm.f90:70): 1 subsonic, 0 otherwise
template <typename T> __device__ __forceinline__ T subsonic(T m) {
  T v = T(1) - floor(fabs(m));
  return v > T(0) ? v : T(0);
}

// ---- arithmetic policy ---------------------------------------------------------
// FP64 keeps IEEE division and square root (the reference's arithmetic).
// The FP32 path of FEST_MIXED uses the hardware approximations: a reciprocal
// based divide (2 ulp), x*rsqrt(x) for the square root (negative -> NaN, as
// IEEE), and a multiplication by the folded reciprocal for constant divisors.
__device__ __forceinline__ double dv(double a, double b) { return a / b; }
__device__ __forceinline__ float dv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double dvc(double a, double c) { return a / c; }
__device__ __forceinline__ float dvc(float a, float c) { return a * (1.0f / c); }
__device__ __forceinline__ double sq(double x) { return sqrt(x); }
__device__ __forceinline__ float sq(float x) { return x == 0.0f ? 0.0f : x * rsqrtf(x); }

// ---- per-cell reconstruction along a line -----------------------------------
// A Line gives the cell values of one variable along direction dir through a
// fixed (tangential) position: q(c) is the cell at normal coordinate c.
template <typename T, typename S> struct Line {
  const S* base;  // cell at normal coordinate 0
  long long stride;
  __device__ __forceinline__ T operator()(int c) const { return (T)base[c * stride]; }
};

template <typename T> __device__ __forceinline__ T limiter_fn(T r, int lim) {
  if (lim == FEST_LIMITER_VAN_ALBADA) return dv(((r * r) + r), ((r * r) + T(1)));
  const T alpha = T(2) / T(3);  // Koren alpha family, muscl.f90:151,176
  return fmax2(T(0), fmin2(fmin2(T(2) * r, alpha * (r - T(1)) + T(1)), T(2)));
}

// MUSCL kappa=1/3 (muscl.f90:115-200) for cell c: Rm = state at its low face,
// Lp = state at its high face.
template <typename T, class Lq>
__device__ __forceinline__ void muscl_cell(const Lq& q, int c, T sw, int lim, T& Rm, T& Lp) {
  const T kappa = T(1) / T(3), eps = T(1e-14);
  T qc = q(c);
  T fd = q(c + 1) - qc;
  T bd = qc - q(c - 1);
  T r = dv(fd, bd + copysign(eps, bd));
  T psi1 = limiter_fn(r, lim);
  r = dv(bd, fd + copysign(eps, fd));
  T psi2 = limiter_fn(r, lim);
  psi1 = (T(1) - (T(1) - psi1) * sw);
  psi2 = (T(1) - (T(1) - psi2) * sw);
  Lp = qc + T(0.25) * (((T(1) - kappa) * psi1 * bd) + ((T(1) + kappa) * psi2 * fd));
  Rm = qc - T(0.25) * (((T(1) + kappa) * psi1 * bd) + ((T(1) - kappa) * psi2 * fd));
}

// boundary-face MUSCL without eps, limiter max(0,min(2r,(2+r)/3,2))
// (boundary_state_reconstruction.f90:101-117)
template <typename T, class Lq>
__device__ __forceinline__ void muscl_noeps_cell(const Lq& q, int c, T sw, T& Rm, T& Lp) {
  const T kappa = T(1) / T(3);
  T qc = q(c);
  T fd = q(c + 1) - qc;
  T bd = qc - q(c - 1);
  T r = dv(fd, bd);
  T psi1 = fmax2(T(0), fmin2(fmin2(T(2) * r, dvc((T(2) + r), T(3))), T(2)));
  psi1 = (T(1) - (T(1) - psi1) * sw);
  r = dv(bd, fd);
  T psi2 = fmax2(T(0), fmin2(fmin2(T(2) * r, dvc((T(2) + r), T(3))), T(2)));
  psi2 = (T(1) - (T(1) - psi2) * sw);
  // 0/0 (flat data) leaves psi undefined in the reference; any finite psi
  // multiplies a zero difference there
  if (psi1 != psi1) psi1 = T(2);
  if (psi2 != psi2) psi2 = T(2);
  Lp = qc + T(0.25) * (((T(1) - kappa) * psi1 * bd) + ((T(1) + kappa) * psi2 * fd));
  Rm = qc - T(0.25) * (((T(1) + kappa) * psi1 * bd) + ((T(1) - kappa) * psi2 * fd));
}

// WENO5-JS (weno.f90:59-87)
template <typename T, class Lq>
__device__ __forceinline__ void weno_cell(const Lq& q, int c, T& Rm, T& Lp) {
  const T eps = T(1e-6);
  const T g0 = T(1) / T(10), g1 = T(6) / T(10), g2 = T(3) / T(10);
  T um2 = q(c - 2), um1 = q(c - 1), u0 = q(c), up1 = q(c + 1), up2 = q(c + 2);
  T t1, t2, B0, B1, B2;
  t1 = um2 - T(2) * um1 + u0; t2 = um2 - T(4) * um1 + T(3) * u0;
  B0 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = um1 - T(2) * u0 + up1; t2 = um1 - up1;
  B1 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = u0 - T(2) * up1 + up2; t2 = T(3) * u0 - T(4) * up1 + up2;
  B2 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  T e0 = eps + B0, e1 = eps + B1, e2 = eps + B2;
  T w0 = dv(g0, (e0 * e0)), w1 = dv(g1, (e1 * e1)), w2 = dv(g2, (e2 * e2));
  T P0 = dvc((T(2) * um2 - T(7) * um1 + T(11) * u0), T(6));
  T P1 = dvc((-T(1) * um1 + T(5) * u0 + T(2) * up1), T(6));
  T P2 = dvc((T(2) * u0 + T(5) * up1 - T(1) * up2), T(6));
  Lp = dv((w0 * P0 + w1 * P1 + w2 * P2), (w0 + w1 + w2));
  P0 = dvc((T(2) * up2 - T(7) * up1 + T(11) * u0), T(6));
  P1 = dvc((-T(1) * up1 + T(5) * u0 + T(2) * um1), T(6));
  P2 = dvc((T(2) * u0 + T(5) * um1 - T(1) * um2), T(6));
  w0 = dv(g0, (e2 * e2)); w1 = dv(g1, (e1 * e1)); w2 = dv(g2, (e0 * e0));
  Rm = dv((w0 * P0 + w1 * P1 + w2 * P2), (w0 + w1 + w2));
}

// ---- packed FP32 pairs -------------------------------------------------------
// Blackwell executes two FP32 adds, multiplies or FMAs in one instruction
// (FADD2/FMUL2/FFMA2 on float2): the FP32 sweep reconstructs two variables
// per instruction stream.  Same rounding per element as the scalar forms.
__device__ __forceinline__ float2 pk(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 pmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 prcp(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }

// WENO5-JS (weno.f90:59-87) of two variables at once: qa, qb are their
// lines.  The weights' reciprocals 1/(eps+B_k)^2 serve both faces, and the
// 1/6 of the candidate-stencil estimates moves into the normalisation.
template <class Lq>
__device__ __forceinline__ void weno_pair(const Lq& qa, const Lq& qb, int c, float2& Rm, float2& Lp) {
  const float2 um2 = make_float2(qa(c - 2), qb(c - 2)), um1 = make_float2(qa(c - 1), qb(c - 1)),
               u0 = make_float2(qa(c), qb(c)), up1 = make_float2(qa(c + 1), qb(c + 1)),
               up2 = make_float2(qa(c + 2), qb(c + 2));
  const float2 k1312 = pk(13.0f / 12.0f), k14 = pk(0.25f), eps = pk(1e-6f);
  float2 t1, t2;
  t1 = padd(psub(um2, padd(um1, um1)), u0);
  t2 = pfma(pk(3.0f), u0, pfma(pk(-4.0f), um1, um2));
  const float2 B0 = pfma(k1312, pmul(t1, t1), pmul(k14, pmul(t2, t2)));
  t1 = padd(psub(um1, padd(u0, u0)), up1);
  t2 = psub(um1, up1);
  const float2 B1 = pfma(k1312, pmul(t1, t1), pmul(k14, pmul(t2, t2)));
  t1 = padd(psub(u0, padd(up1, up1)), up2);
  t2 = padd(pfma(pk(-4.0f), up1, pmul(pk(3.0f), u0)), up2);
  const float2 B2 = pfma(k1312, pmul(t1, t1), pmul(k14, pmul(t2, t2)));
  float2 e = padd(eps, B0);
  const float2 r0 = prcp(pmul(e, e));
  e = padd(eps, B1);
  const float2 r1 = prcp(pmul(e, e));
  e = padd(eps, B2);
  const float2 r2 = prcp(pmul(e, e));
  const float2 w1 = pmul(pk(0.6f), r1);
  // high face: linear weights 0.1, 0.6, 0.3 on stencils (c-2..c), (c-1..c+1), (c..c+2)
  float2 w0 = pmul(pk(0.1f), r0), w2 = pmul(pk(0.3f), r2);
  float2 P0 = pfma(pk(11.0f), u0, pfma(pk(-7.0f), um1, padd(um2, um2)));
  float2 P1 = psub(pfma(pk(2.0f), up1, pmul(pk(5.0f), u0)), um1);
  float2 P2 = psub(pfma(pk(5.0f), up1, padd(u0, u0)), up2);
  float2 num = pfma(w2, P2, pfma(w1, P1, pmul(w0, P0)));
  float2 den = pmul(pk(6.0f), padd(padd(w0, w1), w2));
  Lp = pmul(num, prcp(den));
  // low face: the mirrored stencils, weights 0.1 on (c..c+2), 0.3 on (c-2..c)
  w0 = pmul(pk(0.1f), r2);
  w2 = pmul(pk(0.3f), r0);
  P0 = pfma(pk(11.0f), u0, pfma(pk(-7.0f), up1, padd(up2, up2)));
  P1 = psub(pfma(pk(2.0f), um1, pmul(pk(5.0f), u0)), up1);
  P2 = psub(pfma(pk(5.0f), um1, padd(u0, u0)), um2);
  num = pfma(w2, P2, pfma(w1, P1, pmul(w0, P0)));
  den = pmul(pk(6.0f), padd(padd(w0, w1), w2));
  Rm = pmul(num, prcp(den));
}

// WENO on non-uniform cells (weno_NM.f90:82-116); v(c) are cell volumes
template <typename T, class Lq, class Lv>
__device__ __forceinline__ void weno_nm_cell(const Lq& q, const Lv& v, int c, T& Rm, T& Lp) {
  const T eps = T(1e-6);
  const T g0 = T(1) / T(10), g1 = T(6) / T(10), g2 = T(3) / T(10);
  T um2 = q(c - 2), um1 = q(c - 1), u0 = q(c), up1 = q(c + 1), up2 = q(c + 2);
  T vm2 = v(c - 2), vm1 = v(c - 1), v0 = v(c), vp1 = v(c + 1), vp2 = v(c + 2);
  T a12 = dv(vp2, (vp1 + vp2)), a01 = dv(vp1, (v0 + vp1)), a10 = dv(v0, (vm1 + v0)),
    a21 = dv(vm1, (vm2 + vm1));
  T U01 = (T(1) - a01) * u0 + a01 * up1;
  T U12 = (T(1) - a12) * up1 + a12 * up2;
  T U10 = (T(1) - a10) * um1 + a10 * u0;
  T U21 = (T(1) - a21) * um2 + a21 * um1;
  T U00 = um1 + (T(1) - a21) * (um1 - um2);
  T U11 = up1 + a12 * (up1 - up2);
  T t1, t2, B0, B1, B2, P0, P1, P2, e;
  P0 = dvc((T(6) * u0 - T(1) * U10 - T(2) * U00), T(3));
  P1 = dvc((-T(1) * U10 + T(2) * u0 + T(2) * U01), T(3));
  P2 = dvc((T(2) * U01 + T(2) * up1 - T(1) * U12), T(3));
  t1 = T(2) * U10 - T(2) * U00; t2 = T(4) * u0 - T(2) * U10 - T(2) * U00;
  B0 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = T(2) * U10 - T(4) * u0 + T(2) * U01; t2 = -T(2) * U10 + T(2) * U01;
  B1 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = T(2) * U01 - T(4) * up1 + T(2) * U12; t2 = -T(6) * U01 + T(8) * up1 - T(2) * U12;
  B2 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  T w0, w1, w2;
  e = eps + B0; w0 = dv(g0, (e * e));
  e = eps + B1; w1 = dv(g1, (e * e));
  e = eps + B2; w2 = dv(g2, (e * e));
  Lp = dv((w0 * P0 + w1 * P1 + w2 * P2), (w0 + w1 + w2));
  P0 = dvc((T(6) * u0 - T(1) * U01 - T(2) * U11), T(3));
  P1 = dvc((-T(1) * U01 + T(2) * u0 + T(2) * U10), T(3));
  P2 = dvc((T(2) * U10 + T(2) * um1 - T(1) * U21), T(3));
  t1 = T(2) * U01 - T(2) * U11; t2 = T(4) * u0 - T(2) * U01 - T(2) * U11;
  B0 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = T(2) * U01 - T(4) * u0 + T(2) * U10; t2 = -T(2) * U01 + T(2) * U10;
  B1 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  t1 = T(2) * U10 - T(4) * um1 + T(2) * U21; t2 = -T(6) * U10 + T(8) * um1 - T(2) * U21;
  B2 = (T(13) / T(12)) * (t1 * t1) + (T(1) / T(4)) * (t2 * t2);
  e = eps + B0; w0 = dv(g0, (e * e));
  e = eps + B1; w1 = dv(g1, (e * e));
  e = eps + B2; w2 = dv(g2, (e * e));
  Rm = dv((w0 * P0 + w1 * P1 + w2 * P2), (w0 + w1 + w2));
}

// PPM face estimate (ppm.f90:47-49) and extremum removal (ppm.f90:86-101)
template <typename T, class Lq> __device__ __forceinline__ T ppm_estimate(const Lq& q, int f) {
  return dvc((T(7) * (q(f) + q(f - 1)) - (q(f + 1) + q(f - 2))), T(12));
}
template <typename T, class Lq>
__device__ __forceinline__ void ppm_cell(const Lq& q, int c, bool lim, T& Rm, T& Lp) {
  Rm = ppm_estimate<T>(q, c);
  Lp = ppm_estimate<T>(q, c + 1);
  if (!lim) return;
  T qc = q(c);
  if ((Lp - qc) * (qc - Rm) <= T(0)) {
    Lp = qc;
    Rm = qc;
  } else {
    T dqrl = Lp - Rm;
    T dq6 = T(6) * (qc - T(0.5) * (Lp + Rm));
    if (dqrl * dq6 > dqrl * dqrl) Rm = T(3) * qc - T(2) * Lp;
    else if (-dqrl * dqrl > dqrl * dq6) Lp = T(3) * qc - T(2) * Rm;
  }
}

// pressure-based switch factor of cell c (muscl.f90:182-201): interior cells
// 1..n-1 from |p(c+1)-p(c-1)|, cells 0 and n copy their neighbour
template <typename T, class Lp_>
__device__ __forceinline__ T pdif_cell(const Lp_& p, int c, int n, T p_inf) {
  int cc = c < 1 ? 1 : (c > n - 1 ? n - 1 : c);
  T pd2 = fabs(p(cc + 1) - p(cc - 1));
  return T(1) - dv(pd2, (pd2 + p_inf));
}

// One cell's two face-side states for variable l along direction dir: the
// interior reconstruction of compute_face_interpolant with the optional
// pressure switch (face_interpolant.f90:79-105).
// INTERP >= 0 fixes the method at compile time (the fused sweeps); -1 reads
// it from the parameter block (the module kernels).
template <typename T, int INTERP = -1, class Lq, class Lpres, class Lvol>
__device__ __forceinline__ void recon_interior(const Params& p, int dir, int c, int l, const Lq& q,
                                               const Lpres& pres, const Lvol& vol, T& Rm, T& Lp) {
  int n = extent_of(p.d, dir);
  T sw = T((l >= 6) ? p.tlim[dir] : p.lam[dir]);
  const int interp = INTERP >= 0 ? INTERP : p.interp;
  switch (interp) {
    case FEST_INTERP_NONE: Rm = q(c); Lp = q(c); break;
    case FEST_INTERP_MUSCL: muscl_cell<T>(q, c, sw, p.limiter, Rm, Lp); break;
    case FEST_INTERP_PPM: ppm_cell<T>(q, c, p.lam[dir] == 1, Rm, Lp); break;
    case FEST_INTERP_WENO: weno_cell<T>(q, c, Rm, Lp); break;
    default: weno_nm_cell<T>(q, vol, c, Rm, Lp); break;
  }
  if ((interp == FEST_INTERP_MUSCL || interp == FEST_INTERP_PPM) && p.pb[dir] == 1) {
    T qc = q(c);
    T pd = pdif_cell<T>(pres, c, n, pv<T>(p.p_inf, p.f_p_inf));
    if (c <= n - 1) Lp = qc + (pd * (Lp - qc));
    if (c >= 1) Rm = qc - (pd * (qc - Rm));
  }
}

// reconstruct_boundary_state (boundary_state_reconstruction.f90:28-412) for
// cell c: overrides applied in the reference's order, imin-type writes
// first and imax-type writes last, so thin blocks resolve the same way.
template <typename T, int INTERP = -1, class Lq>
__device__ __forceinline__ void boundary_override(const Params& p, int dir, int c, int l,
                                                  const Lq& q, T& Rm, T& Lp) {
  if ((INTERP >= 0 ? INTERP : p.interp) == FEST_INTERP_NONE) return;
  int n = extent_of(p.d, dir);
  T sw = T((l >= 6) ? p.tlim[dir] : p.lam[dir]);
  int idmin = p.id[2 * dir], idmax = p.id[2 * dir + 1];
  if (idmin < 0 && idmin != -10) {
    if (p.ppm_flag && c == 1) muscl_noeps_cell<T>(q, 1, sw, Rm, Lp);
    bool ff = (idmin == -8 || idmin == -9);
    if (c == 0) Lp = ff ? q(0) : T(0.5) * (q(0) + q(1));
    if (c == 1 && ff) Rm = q(0);
  }
  if (idmax < 0 && idmax != -10) {
    if (p.ppm_flag && c == n - 1) muscl_noeps_cell<T>(q, n - 1, sw, Rm, Lp);
    bool ff = (idmax == -8 || idmax == -9);
    if (c == n) Rm = ff ? q(n) : T(0.5) * (q(n - 1) + q(n));
    if (c == n - 1 && ff) Lp = q(n);
  }
}
// true when boundary_override may change cell c's states
__device__ __forceinline__ bool near_boundary(const Params& p, int dir, int c) {
  int n = extent_of(p.d, dir);
  return c <= 1 || c >= n - 1;
}

template <typename T, int INTERP = -1, class Lq, class Lpres, class Lvol>
__device__ __forceinline__ void recon_cell(const Params& p, int dir, int c, int l, const Lq& q,
                                           const Lpres& pres, const Lvol& vol, T& Rm, T& Lp) {
  recon_interior<T, INTERP>(p, dir, c, l, q, pres, vol, Rm, Lp);
  if (near_boundary(p, dir, c)) boundary_override<T, INTERP>(p, dir, c, l, q, Rm, Lp);
}

// ---- convective fluxes: one face, all variables -----------------------------
// ausm.f90:59-151, van_leer.f90:59-145, ldfss0.f90:59-160
template <typename T, int NVL = NVMAX>
__device__ __forceinline__ void flux_ausm_family(int kind, int nv, T gm, const T* qL, const T* qR,
                                                 T A, T nx, T ny, T nz, T mask, T* Fo) {
  T c = T(0.5) * (sq(dv(gm * qL[4], qL[0])) + sq(dv(gm * qR[4], qR[0])));
  T ic = dv(T(1), c);
  T ML = (qL[1] * nx + qL[2] * ny + qL[3] * nz) * ic;
  T ap = T(0.5) * (T(1) + fsign1(ML));
  T bL = -subsonic(ML);
  T t = T(1) + ML;
  T Mp = T(0.25) * (t * t);
  T Dp = T(0.25) * (t * t) * (T(2) - ML);
  T cp = (ap * (T(1) + bL) * ML) - bL * Mp;
  T sDp = (ap * (T(1) + bL)) - (bL * Dp);
  T MR = (qR[1] * nx + qR[2] * ny + qR[3] * nz) * ic;
  T am = T(0.5) * (T(1) - fsign1(MR));
  T bR = -subsonic(MR);
  t = T(1) - MR;
  T Mm = -T(0.25) * (t * t);
  T Dm = T(0.25) * (t * t) * (T(2) + MR);
  T cm = (am * (T(1) + bR) * MR) - bR * Mm;
  T sDm = (am * (T(1) + bR)) - (bR * Dm);
  if (kind == FEST_FLUX_AUSM) {
    T tc = cp + cm;
    cp = fmax2(T(0), tc);
    cm = fmin2(T(0), tc);
  } else if (kind == FEST_FLUX_LDFSS0) {
    T s = sq((ML * ML + MR * MR) * T(0.5)) - T(1);
    T Ml = T(0.25) * bL * bR * (s * s);
    T Mpl = Ml * (T(1) - dv((qL[4] - qR[4]), (T(2) * qL[0] * (c * c))));
    T Mml = Ml * (T(1) - dv((qL[4] - qR[4]), (T(2) * qR[0] * (c * c))));
    cp = cp - Mpl;
    cm = cm + Mml;
  }
  T g1 = dv(gm, (gm - T(1)));
  T Fp0 = qL[0] * c * cp * mask;
  T Fm0 = qR[0] * c * cm * mask;
  T hL = (T(0.5) * (qL[1] * qL[1] + qL[2] * qL[2] + qL[3] * qL[3])) + dv(g1 * qL[4], qL[0]);
  T hR = (T(0.5) * (qR[1] * qR[1] + qR[2] * qR[2] + qR[3] * qR[3])) + dv(g1 * qR[4], qR[0]);
  Fo[0] = Fp0 * A + Fm0 * A;
  Fo[1] = ((Fp0 * qL[1]) + (sDp * qL[4] * nx)) * A + ((Fm0 * qR[1]) + (sDm * qR[4] * nx)) * A;
  Fo[2] = ((Fp0 * qL[2]) + (sDp * qL[4] * ny)) * A + ((Fm0 * qR[2]) + (sDm * qR[4] * ny)) * A;
  Fo[3] = ((Fp0 * qL[3]) + (sDp * qL[4] * nz)) * A + ((Fm0 * qR[3]) + (sDm * qR[4] * nz)) * A;
  Fo[4] = (Fp0 * hL) * A + (Fm0 * hR) * A;
#pragma unroll
  for (int l = 5; l < NVL; ++l)
    if (l < nv) Fo[l] = (Fp0 * qL[l]) * A + (Fm0 * qR[l]) * A;
}

// slau.f90:85-196, ausmP.f90:88-192, ausmUP.f90:92-210
template <typename T, int NVL = NVMAX>
__device__ __forceinline__ void flux_mass_family(int kind, int nv, T gm, T MInf, const T* qL,
                                                 const T* qR, T A, T nx, T ny, T nz, T mask,
                                                 T* Fo) {
  T rL = qL[0], uL = qL[1], vL = qL[2], wL = qL[3], pL = qL[4];
  T rR = qR[0], uR = qR[1], vR = qR[2], wR = qR[3], pR = qR[4];
  T g1 = dv(gm, (gm - T(1)));
  T HL = (T(0.5) * (uL * uL + vL * vL + wL * wL)) + dv(g1 * pL, rL);
  T HR = (T(0.5) * (uR * uR + vR * vR + wR * wR)) + dv(g1 * pR, rR);
  T VnL = uL * nx + vL * ny + wL * nz;
  T VnR = uR * nx + vR * ny + wR * nz;
  T mass, pbar;
  if (kind == FEST_FLUX_SLAU) {
    T C = T(0.5) * (sq(dv(gm * pL, rL)) + sq(dv(gm * pR, rR)));
    T iC = dv(T(1), C);
    T ML = VnL * iC, MR = VnR * iC;
    T aL = fmax2(T(0), T(1) - floor(fabs(ML)));
    T aR = fmax2(T(0), T(1) - floor(fabs(MR)));
    T betaL = (T(1) - aL) * T(0.5) * (T(1) + fsign1(ML)) +
              (aL) * T(0.25) * (T(2) - ML) * ((ML + T(1)) * (ML + T(1)));
    T betaR = (T(1) - aR) * T(0.5) * (T(1) - fsign1(MR)) +
              (aR) * T(0.25) * (T(2) + MR) * ((MR - T(1)) * (MR - T(1)));
    T vt = sq(T(0.5) * ((uL * uL) + (vL * vL) + (wL * wL) + (uR * uR) + (vR * vR) + (wR * wR)));
    T Mcap = fmin2(T(1), vt * iC);
    T Xi = (T(1) - Mcap) * (T(1) - Mcap);
    T Vnabs = dv((rL * fabs(VnL) + rR * fabs(VnR)), (rL + rR));
    T fnG = -fmax2(fmin2(ML, T(0)), T(-1)) * fmin2(fmax2(MR, T(0)), T(1));
    pbar = T(0.5) * ((pL + pR) + (betaL - betaR) * (pL - pR) +
                     (T(1) - Xi) * (betaL + betaR - T(1)) * (pL + pR));
    T VnabsL = (T(1) - fnG) * Vnabs + fnG * fabs(VnL);
    T VnabsR = (T(1) - fnG) * Vnabs + fnG * fabs(VnR);
    mass = T(0.5) * ((rL * (VnL + VnabsL) + rR * (VnR - VnabsR)) - (Xi * (pR - pL) * iC));
  } else {
    T cs = sq(dv(T(2) * (gm - T(1)) * (T(0.5) * (HL + HR)), (gm + T(1))));
    T cL, cR;
    if (kind == FEST_FLUX_AUSMP) {
      cL = dv(cs * cs, (fmax2(cs, fabs(VnL))));
      cR = dv(cs * cs, (fmax2(cs, fabs(VnR))));
    } else {
      cL = dv(cs * cs, (fmax2(cs, VnL)));
      cR = dv(cs * cs, (fmax2(cs, -VnR)));
    }
    T C = fmin2(cL, cR);
    T iC = dv(T(1), C);
    T ML = VnL * iC, MR = VnR * iC;
    T Mb = T(0), fna = T(0), alfa = T(0.1875);
    if (kind == FEST_FLUX_AUSMUP) {
      Mb = sq(dv(T(0.5) * ((VnL * VnL) + (VnR * VnR)), (C * C)));
      T Mo = sq(fmin2(T(1), fmax2(Mb * Mb, MInf * MInf)));
      fna = Mo * (T(2) - Mo);
      alfa = dvc(T(3) * (T(-4) + (T(5) * fna * fna)), T(16));
    }
    T aL = subsonic(ML), aR = subsonic(MR);
    T t = T(1) + ML;
    T FmL = (T(0.5) * (T(1) + fsign1(ML)) * (T(1) - aL) * ML) + aL * T(0.25) * (t * t);
    T betaL = (T(0.5) * (T(1) + fsign1(ML)) * (T(1) - aL)) + aL * T(0.25) * (t * t) * (T(2) - ML);
    t = T(1) - MR;
    T FmR = (T(0.5) * (T(1) - fsign1(MR)) * (T(1) - aR) * MR) - aR * T(0.25) * (t * t);
    T betaR = (T(0.5) * (T(1) - fsign1(MR)) * (T(1) - aR)) + aR * T(0.25) * (t * t) * (T(2) + MR);
    t = ML * ML - T(1);
    FmL = FmL + aL * T(0.125) * (t * t);
    betaL = betaL + aL * alfa * (t * t) * ML;
    t = MR * MR - T(1);
    FmR = FmR - aR * T(0.125) * (t * t);
    betaR = betaR - aR * alfa * (t * t) * MR;
    T Mface = FmL + FmR;
    pbar = betaL * pL + betaR * pR;
    if (kind == FEST_FLUX_AUSMUP) {
      const T Kp = T(0.25), Ku = T(0.75), sigma = T(1);
      T Pu = -Ku * betaL * betaR * (rL + rR) * fna * C * (VnR - VnL);
      T Mp = dv(-T(2) * Kp * fmax2(T(1) - (sigma * Mb * Mb), T(0)) * (pR - pL),
                (fna * (rL + rR) * C * C));
      Mface = FmL + FmR + Mp;
      pbar = betaL * pL + betaR * pR + Pu;
    }
    mass = (Mface > T(0)) ? Mface * C * rL : Mface * C * rR;
  }
  mass = mass * mask;
  T Fp0 = T(0.5) * (mass + fabs(mass));
  T Fm0 = T(0.5) * (mass - fabs(mass));
  Fo[0] = (Fp0 + Fm0) * A;
  Fo[1] = ((Fp0 * uL + Fm0 * uR) + (pbar * nx)) * A;
  Fo[2] = ((Fp0 * vL + Fm0 * vR) + (pbar * ny)) * A;
  Fo[3] = ((Fp0 * wL + Fm0 * wR) + (pbar * nz)) * A;
  Fo[4] = (Fp0 * HL + Fm0 * HR) * A;
#pragma unroll
  for (int l = 5; l < NVL; ++l)
    if (l < nv) Fo[l] = (Fp0 * qL[l] + Fm0 * qR[l]) * A;
}

// FLUX >= 0 fixes the scheme at compile time (the fused sweeps)
template <typename T, int FLUX = -1, int NVL = NVMAX>
__device__ __forceinline__ void face_flux(const Params& p, const T* qL, const T* qR, T A, T nx,
                                          T ny, T nz, T mask, T* Fo) {
  const int kind = FLUX >= 0 ? FLUX : p.flux;
  if (kind == FEST_FLUX_AUSM || kind == FEST_FLUX_VAN_LEER || kind == FEST_FLUX_LDFSS0)
    flux_ausm_family<T, NVL>(kind, p.d.nv, pv<T>(p.gm, p.f_gm), qL, qR, A, nx, ny, nz, mask, Fo);
  else
    flux_mass_family<T, NVL>(kind, p.d.nv, pv<T>(p.gm, p.f_gm), pv<T>(p.MInf, p.f_MInf), qL, qR, A, nx, ny, nz, mask,
                        Fo);
}

// wall mass-flux mask of a face (bc.f90:57-66): 0 at the first/last face of a
// direction whose boundary id is -5, -6 or -7
__device__ __forceinline__ int wall_mask(const Params& p, int dir, int f) {
  int n = extent_of(p.d, dir);
  int idlo = p.id[2 * dir], idhi = p.id[2 * dir + 1];
  bool wlo = (idlo == -5 || idlo == -6 || idlo == -7);
  bool whi = (idhi == -5 || idhi == -6 || idhi == -7);
  return ((f == 1 && wlo) || (f == n && whi)) ? 0 : 1;
}

// bc_primitive.f90:209-224: the edge and corner ghosts as the mean (0.33
// times the sum) of their three neighbours, in the reference's order: the
// i-lines of the j/k edges, the k-lines of the i/j edges, the corners.  The
// j-lines of the i/k edges are left as they are.  One CTA; q(i, j, k, l)
// returns the cell of variable l (1-based).
template <typename T, class Q>
__device__ void corner_average(const Dims& d, const Q& q) {
  const int imx = d.imx, jmx = d.jmx, kmx = d.kmx, nv = d.nv;
  const T c = T(0.33);
  const int tid = threadIdx.x;
  const int ni = imx + 5, nk = kmx + 5;
  for (int s = 0; s < 4; ++s) {
    for (int t = tid; t < ni * nv; t += blockDim.x) {
      const int i = -2 + t % ni, l = 1 + t / ni;
      switch (s) {
        case 0: q(i, 0, 0, l) = c * (q(i, 1, 1, l) + q(i, 0, 1, l) + q(i, 1, 0, l)); break;
        case 1: q(i, 0, kmx, l) = c * (q(i, 1, kmx - 1, l) + q(i, 0, kmx - 1, l) + q(i, 1, kmx, l)); break;
        case 2: q(i, jmx, 0, l) = c * (q(i, jmx - 1, 1, l) + q(i, jmx, 1, l) + q(i, jmx - 1, 0, l)); break;
        default:
          q(i, jmx, kmx, l) = c * (q(i, jmx - 1, kmx - 1, l) + q(i, jmx, kmx - 1, l) + q(i, jmx - 1, kmx, l));
      }
    }
    __syncthreads();
  }
  for (int s = 0; s < 4; ++s) {
    for (int t = tid; t < nk * nv; t += blockDim.x) {
      const int k = -2 + t % nk, l = 1 + t / nk;
      switch (s) {
        case 0: q(imx, 0, k, l) = c * (q(imx - 1, 1, k, l) + q(imx - 1, 0, k, l) + q(imx, 1, k, l)); break;
        case 1: q(0, 0, k, l) = c * (q(1, 1, k, l) + q(1, 0, k, l) + q(0, 1, k, l)); break;
        case 2: q(0, jmx, k, l) = c * (q(1, jmx - 1, k, l) + q(1, jmx, k, l) + q(0, jmx - 1, k, l)); break;
        default:
          q(imx, jmx, k, l) = c * (q(imx - 1, jmx - 1, k, l) + q(imx - 1, jmx, k, l) + q(imx, jmx - 1, k, l));
      }
    }
    __syncthreads();
  }
  for (int l = 1 + tid; l <= nv; l += blockDim.x) {
    q(0, 0, 0, l) = c * (q(1, 0, 0, l) + q(0, 1, 0, l) + q(0, 0, 1, l));
    q(imx, 0, 0, l) = c * (q(imx - 1, 0, 0, l) + q(imx, 1, 0, l) + q(imx, 0, 1, l));
    q(0, jmx, 0, l) = c * (q(1, jmx, 0, l) + q(0, jmx - 1, 0, l) + q(0, jmx, 1, l));
    q(0, 0, kmx, l) = c * (q(1, 0, kmx, l) + q(0, 1, kmx, l) + q(0, 0, kmx - 1, l));
    q(imx, jmx, 0, l) = c * (q(imx - 1, jmx, 0, l) + q(imx, jmx - 1, 0, l) + q(imx, jmx, 1, l));
    q(imx, 0, kmx, l) = c * (q(imx - 1, 0, kmx, l) + q(imx, 1, kmx, l) + q(imx, 0, kmx - 1, l));
    q(0, jmx, kmx, l) = c * (q(1, jmx, kmx, l) + q(0, jmx - 1, kmx, l) + q(0, jmx, kmx - 1, l));
    q(imx, jmx, kmx, l) = c * (q(imx - 1, jmx, kmx, l) + q(imx, jmx - 1, kmx, l) + q(imx, jmx, kmx - 1, l));
  }
}
// An interface face carries no gradient BC (apply_gradient_bc treats the
// negative ids only): the viscous terms take its ghost cells' own
// Green-Gauss gradient, whose neighbours include the averaged edge ghosts.
// Viscous blocks with such a face need the edge averaging on the fused path.
__host__ __device__ __forceinline__ bool needs_edge_ghosts(const Params& p) {
  if (p.mu_ref == 0.0) return false;
  for (int f = 0; f < 6; ++f)
    if (p.id[f] >= 0) return true;
  return false;
}

// device error word: first error wins, later ones keep it
__device__ __forceinline__ void raise_error(int* err, int code) { atomicCAS(err, 0, code); }

}  // namespace fest
