// fest_dual.cuh - forward-mode dual numbers for the local Jacobians of the
// residual's building blocks (reconstruction of one face state, the flux of
// one face, the Riemann ghost state of one boundary column).
//
// The adjoint (fest_adjoint.cu) runs in reverse order - face fluxes, then
// face states, then ghost cells, then interior cells - and at each step
// needs the transposed Jacobian of a small function with at most 10 inputs.
// Instantiating the primal's own templated device code on Dual<T, N>
// gives those Jacobians exactly (every branch, limiter and switch as the
// primal took it), so the adjoint cannot drift from the primal it
// differentiates.  A non-differentiable point (a limiter kink, |x| at 0,
// floor) takes the one-sided derivative of the branch the primal took.
#pragma once
#include "fest_common.cuh"

namespace fest {

template <typename T, int N> struct Dual {
  T v;
  T d[N];
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(double x) : v(T(x)) {
#pragma unroll
    for (int n = 0; n < N; ++n) d[n] = T(0);
  }
  // value x with derivative 1 along input `seed` (none when seed < 0)
  __device__ __forceinline__ static Dual var(T x, int seed) {
    Dual r(0.0);
    r.v = x;
    if (seed >= 0 && seed < N) r.d[seed] = T(1);
    return r;
  }
  __device__ __forceinline__ static Dual cst(T x) {
    Dual r(0.0);
    r.v = x;
    return r;
  }
};

#define FEST_DUAL template <typename T, int N> __device__ __forceinline__

FEST_DUAL Dual<T, N> operator+(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] + b.d[n];
  return r;
}
FEST_DUAL Dual<T, N> operator-(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] - b.d[n];
  return r;
}
FEST_DUAL Dual<T, N> operator-(const Dual<T, N>& a) {
  Dual<T, N> r;
  r.v = -a.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = -a.d[n];
  return r;
}
FEST_DUAL Dual<T, N> operator*(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] * b.v + a.v * b.d[n];
  return r;
}
FEST_DUAL Dual<T, N> operator/(const Dual<T, N>& a, const Dual<T, N>& b) {
  Dual<T, N> r;
  r.v = a.v / b.v;
  const T ib = T(1) / b.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = (a.d[n] - r.v * b.d[n]) * ib;
  return r;
}
FEST_DUAL bool operator<(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v < b.v; }
FEST_DUAL bool operator>(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v > b.v; }
FEST_DUAL bool operator<=(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v <= b.v; }
FEST_DUAL bool operator>=(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v >= b.v; }
FEST_DUAL bool operator==(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v == b.v; }
FEST_DUAL bool operator!=(const Dual<T, N>& a, const Dual<T, N>& b) { return a.v != b.v; }

FEST_DUAL Dual<T, N> sqrt(const Dual<T, N>& a) {
  Dual<T, N> r;
  r.v = ::sqrt(a.v);
  const T h = r.v > T(0) ? T(0.5) / r.v : T(0);
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] * h;
  return r;
}
FEST_DUAL Dual<T, N> fabs(const Dual<T, N>& a) { return a.v < T(0) ? -a : a; }
FEST_DUAL Dual<T, N> tanh(const Dual<T, N>& a) {
  Dual<T, N> r;
  r.v = ::tanh(a.v);
  const T g = T(1) - r.v * r.v;
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] * g;
  return r;
}
FEST_DUAL Dual<T, N> floor(const Dual<T, N>& a) { return Dual<T, N>::cst(::floor(a.v)); }
FEST_DUAL Dual<T, N> copysign(const Dual<T, N>& a, const Dual<T, N>& b) {
  return (signbit(a.v) == signbit(b.v)) ? a : -a;
}
FEST_DUAL Dual<T, N> pow(const Dual<T, N>& a, const Dual<T, N>& b) {  // b constant
  Dual<T, N> r;
  r.v = ::pow(a.v, b.v);
  const T g = b.v * ::pow(a.v, b.v - T(1));
#pragma unroll
  for (int n = 0; n < N; ++n) r.d[n] = a.d[n] * g;
  return r;
}
// the arithmetic policy of the primal, on duals
FEST_DUAL Dual<T, N> dv(const Dual<T, N>& a, const Dual<T, N>& b) { return a / b; }
FEST_DUAL Dual<T, N> dvc(const Dual<T, N>& a, const Dual<T, N>& c) { return a / c; }
FEST_DUAL Dual<T, N> sq(const Dual<T, N>& a) { return sqrt(a); }

#undef FEST_DUAL

// Ghost layer 1 of a Riemann-invariant boundary (far field -8 when tp is
// false, total pressure -11 when true; bc_primitive.f90:645-1234,
// 1237-1776) from interior layer 1 `in` (rho,u,v,w,p) and the outward unit
// normal (nx,ny,nz) of the boundary face.  Used by the adjoint (on duals)
// and by the FP32 mirror ghost fill.
template <typename T>
__device__ __forceinline__ void riemann_ghost(const Params& p, int f, bool tp, T nx, T ny, T nz,
                                              const T* in, T* g) {
  const T gm = T(p.gm);
  const T uinf = T(p.u_inf), vinf = T(p.v_inf), winf = T(p.w_inf);
  const T pinf = T(p.p_inf), rinf = T(p.rho_inf);
  const T uu = in[1], vv = in[2], ww = in[3], pI = in[4], rI = in[0];
  const T cexp = sqrt(gm * pI / rI), cinf = sqrt(gm * pinf / rinf);
  const T Unexp = uu * nx + vv * ny + ww * nz, Uninf = uinf * nx + vinf * ny + winf * nz;
  const T Rinf = Uninf - T(2) * cinf / (gm - T(1)), Rexp = Unexp + T(2) * cexp / (gm - T(1));
  const T Unb = T(0.5) * (Rexp + Rinf), Cb = T(0.25) * (gm - T(1)) * (Rexp - Rinf);
  T ug, vg, wg, rg = T(0), pg = T(0);
  if (Unb > T(0)) {
    const T vd = Unb - Unexp;
    ug = uu + vd * nx; vg = vv + vd * ny; wg = ww + vd * nz;
    if (!tp) {
      const T sv = pI / pow(rI, gm);
      rg = pow(Cb * Cb / (gm * sv), T(1) / (gm - T(1)));
      pg = rg * Cb * Cb / gm;
    }
  } else {
    const T vd = Unb - Uninf;
    ug = uinf + vd * nx; vg = vinf + vd * ny; wg = winf + vd * nz;
    if (!tp) {
      const T sv = pinf / pow(rinf, gm);
      rg = pow(Cb * Cb / (gm * sv), T(1) / (gm - T(1)));
      pg = rg * Cb * Cb / gm;
    }
  }
  if (tp) {
    const T Mb = sqrt(ug * ug + vg * vg + wg * wg) / Cb;
    pg = T(p.Tp[f]) / pow((T(1) + T(0.5) * (gm - T(1)) * Mb * Mb), gm / (gm - T(1)));
    rg = gm * pg / (Cb * Cb);
  }
  g[0] = rg; g[1] = ug; g[2] = vg; g[3] = wg; g[4] = pg;
}

}  // namespace fest
