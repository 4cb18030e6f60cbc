// fest_adjoint.cu - reverse-mode product with the transposed Jacobian of the
// inviscid residual: dq = (dR/dq)^T lambda, R as get_total_conservative_Residue
// computes it (update.f90:495-547: ghost cells, face states, fluxes, residue)
// and q the interior primitive state.  No counterpart in the reference.
//
// Reverse order of the primal:
//   residue  R(c) = sum over the faces of c of +-F(face)   (scheme.f90:133-135)
//     -> every face's flux receives mu = lambda(left cell) - lambda(right cell)
//   flux     F = F(qL, qR) (one of the six schemes)
//     -> qL, qR receive (dF/dqL)^T mu, (dF/dqR)^T mu
//   face states qL = Lp(left cell), qR = Rm(right cell) (reconstruction with
//   its boundary overrides)
//     -> the up-to-5 cells of each stencil receive their share
//   ghost cells (the BC of each face at this iteration)
//     -> the interior cells they were computed from
// The local Jacobians come from the primal's own templated device code run
// on dual numbers (fest_dual.cuh).  Face contributions meet in cells by FP64
// atomic adds.
#include <algorithm>

#include "fest_dual.cuh"
#include "fest_kernels.cuh"

namespace fest {

namespace {

constexpr int TPB_ADJ = 128;

template <typename T, int N> struct DualLine {
  const double* base;  // variable l, cell at normal coordinate 0
  long long stride;
  int center;  // seeds the N cells center - N/2 .. center + N/2
  __device__ __forceinline__ Dual<T, N> operator()(int c) const {
    return Dual<T, N>::var((T)base[c * stride], c - center + N / 2);
  }
};
template <typename T, int N> struct ConstLine {
  const double* base;
  long long stride;
  __device__ __forceinline__ Dual<T, N> operator()(int c) const {
    return Dual<T, N>::cst((T)base[c * stride]);
  }
};
template <typename T, int N> struct VolConst {
  const double* p;  // cells + 4*pidx(cell at normal coordinate 0)
  long long stride;
  int n;
  __device__ __forceinline__ Dual<T, N> operator()(int c) const {
    c = c < -2 ? -2 : (c > n + 2 ? n + 2 : c);
    return Dual<T, N>::cst((T)p[4 * c * stride]);
  }
};

// the same lines in plain arithmetic (the face-state values)
template <typename T> struct ValLine {
  const double* base;
  long long stride;
  __device__ __forceinline__ T operator()(int c) const { return (T)base[c * stride]; }
};
template <typename T> struct VolVal {
  const double* p;
  long long stride;
  int n;
  __device__ __forceinline__ T operator()(int c) const {
    c = c < -2 ? -2 : (c > n + 2 ? n + 2 : c);
    return (T)p[4 * c * stride];
  }
};

__device__ __forceinline__ void cell_of(int dir, int c, int ta, int tb, int& i, int& j, int& k) {
  if (dir == 0) { i = c; j = ta; k = tb; }
  else if (dir == 1) { i = ta; j = c; k = tb; }
  else { i = ta; j = tb; k = c; }
}

// Reverse mode of the SLAU flux (slau.f90:85-196, flux_mass_family):
// bx = mu^T dF/d(qL, qR) in one backward sweep over the forward values,
// about four times the flux's own arithmetic where the ten forward
// directions of Dual<T, 10> cost about twenty.  The derivative conventions
// at the kinks are the dual numbers' (fest_dual.cuh): fabs takes the sign
// of its argument (+1 at 0), fmax2/fmin2 the branch they return, floor
// and copysign none, sqrt 1/(2 sqrt(x)) (0 at 0).  NV = 5, or 7 with k and
// omega carried by the mass flux; bx[0..NV-1] left, bx[NV..2NV-1] right.
template <typename T, int NV>
__device__ __forceinline__ void slau_vjp(T gm, const T* qL, const T* qR, T A, T nx, T ny, T nz, T mask,
                                         const T* mu, T* bx) {
  const T rL = qL[0], uL = qL[1], vL = qL[2], wL = qL[3], pL = qL[4];
  const T rR = qR[0], uR = qR[1], vR = qR[2], wR = qR[3], pR = qR[4];
  // forward, as flux_mass_family computes it
  const T g1 = gm / (gm - T(1));
  const T HL = (T(0.5) * (uL * uL + vL * vL + wL * wL)) + (g1 * pL) / rL;
  const T HR = (T(0.5) * (uR * uR + vR * vR + wR * wR)) + (g1 * pR) / rR;
  const T VnL = uL * nx + vL * ny + wL * nz;
  const T VnR = uR * nx + vR * ny + wR * nz;
  const T cL2 = (gm * pL) / rL, cR2 = (gm * pR) / rR;
  const T sL = ::sqrt(cL2), sR = ::sqrt(cR2);
  const T C = T(0.5) * (sL + sR);
  const T iC = T(1) / C;
  const T ML = VnL * iC, MR = VnR * iC;
  const T aL = fmax2(T(0), T(1) - ::floor(::fabs(ML)));
  const T aR = fmax2(T(0), T(1) - ::floor(::fabs(MR)));
  const T betaL = (T(1) - aL) * T(0.5) * (T(1) + fsign1(ML)) +
                  (aL) * T(0.25) * (T(2) - ML) * ((ML + T(1)) * (ML + T(1)));
  const T betaR = (T(1) - aR) * T(0.5) * (T(1) - fsign1(MR)) +
                  (aR) * T(0.25) * (T(2) + MR) * ((MR - T(1)) * (MR - T(1)));
  const T S2 = T(0.5) * ((uL * uL) + (vL * vL) + (wL * wL) + (uR * uR) + (vR * vR) + (wR * wR));
  const T vt = ::sqrt(S2);
  const T x = vt * iC;
  const bool capped = T(1) < x;  // fmin2(1, x) returns the constant
  const T Mcap = capped ? T(1) : x;
  const T Xi = (T(1) - Mcap) * (T(1) - Mcap);
  const T aVL = ::fabs(VnL), aVR = ::fabs(VnR);
  const T sgL = VnL < T(0) ? T(-1) : T(1), sgR = VnR < T(0) ? T(-1) : T(1);
  const T Nv = rL * aVL + rR * aVR, Dv = rL + rR;
  const T Vnabs = Nv / Dv;
  const bool a1 = ML < T(0);                // fmin2(ML, 0) returns ML
  const T fa1 = a1 ? ML : T(0);
  const bool a2 = fa1 > T(-1);              // fmax2(., -1) returns it
  const T fa = a2 ? fa1 : T(-1);
  const bool b1 = MR > T(0);                // fmax2(MR, 0) returns MR
  const T fb1 = b1 ? MR : T(0);
  const bool b2 = fb1 < T(1);               // fmin2(., 1) returns it
  const T fb = b2 ? fb1 : T(1);
  const T fnG = -fa * fb;
  const T pbar = T(0.5) * ((pL + pR) + (betaL - betaR) * (pL - pR) +
                           (T(1) - Xi) * (betaL + betaR - T(1)) * (pL + pR));
  const T VnabsL = (T(1) - fnG) * Vnabs + fnG * aVL;
  const T VnabsR = (T(1) - fnG) * Vnabs + fnG * aVR;
  const T mass0 = T(0.5) * ((rL * (VnL + VnabsL) + rR * (VnR - VnabsR)) - (Xi * (pR - pL) * iC));
  const T mass = mass0 * mask;
  const T Fp0 = T(0.5) * (mass + ::fabs(mass)), Fm0 = T(0.5) * (mass - ::fabs(mass));
  // backward
  const T m0 = mu[0] * A, m1 = mu[1] * A, m2 = mu[2] * A, m3 = mu[3] * A, m4 = mu[4] * A;
  T b_rL = T(0), b_uL = m1 * Fp0, b_vL = m2 * Fp0, b_wL = m3 * Fp0, b_pL = T(0);
  T b_rR = T(0), b_uR = m1 * Fm0, b_vR = m2 * Fm0, b_wR = m3 * Fm0, b_pR = T(0);
  const T b_HL = m4 * Fp0, b_HR = m4 * Fm0;
  T b_Fp0 = m0 + m1 * uL + m2 * vL + m3 * wL + m4 * HL;
  T b_Fm0 = m0 + m1 * uR + m2 * vR + m3 * wR + m4 * HR;
#pragma unroll
  for (int l = 5; l < NV; ++l) {  // Fo[l] = (Fp0 qL[l] + Fm0 qR[l]) A
    b_Fp0 += mu[l] * A * qL[l];
    b_Fm0 += mu[l] * A * qR[l];
    bx[l] = mu[l] * A * Fp0;
    bx[NV + l] = mu[l] * A * Fm0;
  }
  const T b_pbar = m1 * nx + m2 * ny + m3 * nz;
  const T sm = mass < T(0) ? T(-1) : T(1);
  const T b_mass0 = (b_Fp0 * T(0.5) * (T(1) + sm) + b_Fm0 * T(0.5) * (T(1) - sm)) * mask;
  // mass0
  const T hm = T(0.5) * b_mass0;
  b_rL += hm * (VnL + VnabsL);
  b_rR += hm * (VnR - VnabsR);
  T b_VnL = hm * rL, b_VnR = hm * rR;
  const T b_VnabsL = hm * rL, b_VnabsR = -hm * rR;
  T b_Xi = -hm * (pR - pL) * iC;
  b_pR += -hm * Xi * iC;
  b_pL += hm * Xi * iC;
  T b_iC = -hm * Xi * (pR - pL);
  // VnabsL, VnabsR
  const T b_fnG = b_VnabsL * (aVL - Vnabs) + b_VnabsR * (aVR - Vnabs);
  const T b_Vnabs = (b_VnabsL + b_VnabsR) * (T(1) - fnG);
  b_VnL += b_VnabsL * fnG * sgL;
  b_VnR += b_VnabsR * fnG * sgR;
  // pbar
  const T hp = T(0.5) * b_pbar;
  const T cc = (T(1) - Xi) * (betaL + betaR - T(1));
  b_pL += hp * (T(1) + (betaL - betaR) + cc);
  b_pR += hp * (T(1) - (betaL - betaR) + cc);
  const T b_betaL = hp * ((pL - pR) + (T(1) - Xi) * (pL + pR));
  const T b_betaR = hp * (-(pL - pR) + (T(1) - Xi) * (pL + pR));
  b_Xi += -hp * (betaL + betaR - T(1)) * (pL + pR);
  // fnG = -fa * fb
  T b_ML = T(0), b_MR = T(0);
  if (a1 && a2) b_ML += -b_fnG * fb;
  if (b1 && b2) b_MR += -b_fnG * fa;
  // Vnabs = Nv / Dv
  const T b_Nv = b_Vnabs / Dv, b_Dv = -b_Vnabs * Vnabs / Dv;
  b_rL += b_Nv * aVL + b_Dv;
  b_rR += b_Nv * aVR + b_Dv;
  b_VnL += b_Nv * rL * sgL;
  b_VnR += b_Nv * rR * sgR;
  // Xi, Mcap = x = vt iC
  const T b_Mcap = -T(2) * (T(1) - Mcap) * b_Xi;
  if (!capped) {
    const T hv = vt > T(0) ? b_Mcap * iC * (T(0.5) / vt) : T(0);  // through S2
    b_iC += b_Mcap * vt;
    b_uL += hv * uL; b_vL += hv * vL; b_wL += hv * wL;
    b_uR += hv * uR; b_vR += hv * vR; b_wR += hv * wR;
  }
  // betaL, betaR (aL, aR piecewise constant)
  b_ML += b_betaL * aL * T(0.25) * (-((ML + T(1)) * (ML + T(1))) + (T(2) - ML) * T(2) * (ML + T(1)));
  b_MR += b_betaR * aR * T(0.25) * (((MR - T(1)) * (MR - T(1))) + (T(2) + MR) * T(2) * (MR - T(1)));
  // ML = VnL iC, MR = VnR iC
  b_VnL += b_ML * iC;
  b_VnR += b_MR * iC;
  b_iC += b_ML * VnL + b_MR * VnR;
  // iC = 1 / C, C = (sL + sR) / 2
  const T b_C = -b_iC * iC * iC;
  const T b_cL2 = sL > T(0) ? T(0.5) * b_C * (T(0.5) / sL) : T(0);
  const T b_cR2 = sR > T(0) ? T(0.5) * b_C * (T(0.5) / sR) : T(0);
  b_pL += b_cL2 * gm / rL;
  b_rL += -b_cL2 * cL2 / rL;
  b_pR += b_cR2 * gm / rR;
  b_rR += -b_cR2 * cR2 / rR;
  // HL, HR
  b_uL += b_HL * uL; b_vL += b_HL * vL; b_wL += b_HL * wL;
  b_pL += b_HL * g1 / rL;
  b_rL += -b_HL * (g1 * pL) / (rL * rL);
  b_uR += b_HR * uR; b_vR += b_HR * vR; b_wR += b_HR * wR;
  b_pR += b_HR * g1 / rR;
  b_rR += -b_HR * (g1 * pR) / (rR * rR);
  // VnL, VnR
  b_uL += b_VnL * nx; b_vL += b_VnL * ny; b_wL += b_VnL * nz;
  b_uR += b_VnR * nx; b_vR += b_VnR * ny; b_wR += b_VnR * nz;
  bx[0] = b_rL; bx[1] = b_uL; bx[2] = b_vL; bx[3] = b_wL; bx[4] = b_pL;
  bx[NV + 0] = b_rR; bx[NV + 1] = b_uR; bx[NV + 2] = b_vR; bx[NV + 3] = b_wR; bx[NV + 4] = b_pR;
}

// faces of direction dir: faces 1..n along dir at the interior tangential
// positions, face t at c = 1 + t % n, (ta, tb) from t / n
__device__ __forceinline__ void face_of(const Dims& d, int dir, long long t, int& c, int& ta, int& tb) {
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1;
  c = 1 + (int)(t % n);
  const long long r = t / n;
  ta = 1 + (int)(r % na);
  tb = 1 + (int)(r / na);
}

// the cells 0..n of the line (ta, tb) along dir, whose reconstructions
// give the states of faces 1..n: cell c's low side is face c's right
// state, its high side face c+1's left state.  Face c of the line is entry
// (c - 1) + n r of a face array (face_of), r = (ta - 1) + na (tb - 1).
__device__ __forceinline__ void cell_line_of(const Dims& d, int dir, long long t, int& c, long long& r,
                                             int& ta, int& tb) {
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1;
  c = (int)(t % (n + 1));
  r = t / (n + 1);
  ta = 1 + (int)(r % na);
  tb = 1 + (int)(r / na);
}

// one thread per (cell, variable) of cells 0..n: the cell's reconstruction
// of that variable in plain arithmetic, its low side stored as face c's
// right state w[(NV + l) nf + f] and its high side as face c+1's left state
// w[l nf + f]
template <typename T, int NV>
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_states(Params p, DevBlock b, double* w, int dir) {
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long nf = (long long)n * na * nb, ncl = (long long)(n + 1) * na * nb;
  const long long tl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= NV * ncl) return;
  const int l = (int)(tl / ncl);
  int c, ta, tb, i, j, k;
  long long r;
  cell_line_of(d, dir, tl - l * ncl, c, r, ta, tb);
  cell_of(dir, 0, ta, tb, i, j, k);
  const long long P = d.P, st = pstride(d, dir), c0 = pidx(d, i, j, k);
  VolVal<T> vol{b.cells + 4 * c0, st, n};
  ValLine<T> pres{b.qp + c0 + P * 4, st};
  ValLine<T> q{b.qp + c0 + P * l, st};
  T Rm, Lp;
  recon_cell<T>(p, dir, c, l + 1, q, pres, vol, Rm, Lp);
  if (c >= 1) w[(NV + l) * nf + (c - 1) + n * r] = (double)Rm;
  if (c <= n - 1) w[l * nf + c + n * r] = (double)Lp;
}

// one thread per face of direction dir: mu = lambda(left) - lambda(right)
// transposed through the flux onto the 2 NV face-state values (read from
// the work array k_vjp_states filled, overwritten in place by the
// transposes, bx[m * nf + t]); and, when bar_face is given, onto the face
// record.  Reverse mode for SLAU, forward duals over the 2 NV values
// otherwise.
template <typename T, bool SLAU, int NV>
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_flux(Params p, DevBlock b, const double* lam, double* bxo,
                                                      double* bar_face, int dir) {
  using D10 = Dual<T, 2 * NV>;
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long nf = (long long)n * na * nb;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nf) return;
  int c, ta, tb;
  face_of(d, dir, t, c, ta, tb);
  const long long N = ncells(d);
  // mu = lambda(left) - lambda(right); ghost cells carry no residual
  T mu[NV];
  int i, j, k;
#pragma unroll
  for (int l = 0; l < NV; ++l) mu[l] = T(0);
  if (c - 1 >= 1) {
    cell_of(dir, c - 1, ta, tb, i, j, k);
#pragma unroll
    for (int l = 0; l < NV; ++l) mu[l] += (T)lam[cidx(d, i, j, k) + N * l];
  }
  if (c <= n - 1) {
    cell_of(dir, c, ta, tb, i, j, k);
#pragma unroll
    for (int l = 0; l < NV; ++l) mu[l] -= (T)lam[cidx(d, i, j, k) + N * l];
  }
  bool any = false;
#pragma unroll
  for (int l = 0; l < NV; ++l) any |= mu[l] != T(0);
  if (!any) {
#pragma unroll
    for (int m = 0; m < 2 * NV; ++m) bxo[m * nf + t] = 0.0;
    return;
  }
  // the face states' values (k_vjp_states)
  cell_of(dir, 0, ta, tb, i, j, k);
  T qL[NV], qR[NV];
#pragma unroll
  for (int l = 0; l < NV; ++l) {
    qL[l] = (T)bxo[l * nf + t];
    qR[l] = (T)bxo[(NV + l) * nf + t];
  }
  const long long fi = fidx(d, dir, i + (dir == 0 ? c : 0), j + (dir == 1 ? c : 0), k + (dir == 2 ? c : 0));
  const double* fc = b.faces[dir] + 4 * fi;
  const T mask_v = (T)wall_mask(p, dir, c);
  T bx[2 * NV];
  if constexpr (SLAU) {
    slau_vjp<T, NV>((T)p.gm, qL, qR, (T)fc[0], (T)fc[1], (T)fc[2], (T)fc[3], mask_v, mu, bx);
  } else {
    D10 xl[NVMAX], xr[NVMAX], Fo[NVMAX];
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      xl[l] = D10::var(qL[l], l);
      xr[l] = D10::var(qR[l], NV + l);
    }
    const D10 A = D10::cst((T)fc[0]), nx = D10::cst((T)fc[1]), ny = D10::cst((T)fc[2]),
              nz = D10::cst((T)fc[3]);
    face_flux<D10>(p, xl, xr, A, nx, ny, nz, D10::cst(mask_v), Fo);
#pragma unroll
    for (int m = 0; m < 2 * NV; ++m) {
      T s = T(0);
#pragma unroll
      for (int l = 0; l < NV; ++l) s += mu[l] * Fo[l].d[m];
      bx[m] = s;
    }
  }
#pragma unroll
  for (int m = 0; m < 2 * NV; ++m) bxo[m * nf + t] = (double)bx[m];
  // face metrics {A, nx, ny, nz} (the flux at fixed face states)
  if (bar_face) {
    using D4 = Dual<T, 4>;
    D4 xl[NVMAX], xr[NVMAX], Fo[NVMAX];
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      xl[l] = D4::cst(qL[l]);
      xr[l] = D4::cst(qR[l]);
    }
    face_flux<D4>(p, xl, xr, D4::var((T)fc[0], 0), D4::var((T)fc[1], 1), D4::var((T)fc[2], 2),
                  D4::var((T)fc[3], 3), D4::cst(mask_v), Fo);
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      T s = T(0);
#pragma unroll
      for (int l = 0; l < NV; ++l) s += mu[l] * Fo[l].d[m];
      if (s != T(0)) atomicAdd(bar_face + 4 * fi + m, (double)s);
    }
  }
}

// one thread per (cell, variable) of cells 0..n: the cell's two face
// states of that variable (its low side, face c's right state; its high
// side, face c+1's left state) differentiated with respect to its W-cell
// stencil (W = 5 for PPM and the WENOs, 3 for MUSCL and first order, which
// read no further, boundary overrides included) by forward duals, times
// the flux transposes of k_vjp_flux; the W targets c-W/2..c+W/2 are summed
// in registers before one atomic add each
template <typename T, int NV, int W>
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_recon(Params p, DevBlock b, const double* bxi, double* bar,
                                                       int dir) {
  using D5 = Dual<T, W>;
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long nf = (long long)n * na * nb, ncl = (long long)(n + 1) * na * nb;
  const long long tl = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tl >= NV * ncl) return;
  const int l = (int)(tl / ncl);
  int c, ta, tb, i, j, k;
  long long r;
  cell_line_of(d, dir, tl - l * ncl, c, r, ta, tb);
  const T br = c >= 1 ? (T)bxi[(NV + l) * nf + (c - 1) + n * r] : T(0);
  const T bl = c <= n - 1 ? (T)bxi[l * nf + c + n * r] : T(0);
  if (bl == T(0) && br == T(0)) return;
  cell_of(dir, 0, ta, tb, i, j, k);
  const long long P = d.P, st = pstride(d, dir), c0 = pidx(d, i, j, k);
  VolConst<T, W> vol{b.cells + 4 * c0, st, n};
  ConstLine<T, W> pres{b.qp + c0 + P * 4, st};
  D5 Rm, Lp;
  DualLine<T, W> qa{b.qp + c0 + P * l, st, c};
  recon_cell<D5>(p, dir, c, l + 1, qa, pres, vol, Rm, Lp);
#pragma unroll
  for (int s = 0; s < W; ++s) {
    const T a = br * Rm.d[s] + bl * Lp.d[s];
    if (a != T(0)) atomicAdd(bar + c0 + (c - W / 2 + s) * st + P * l, (double)a);
  }
}

// ---- laminar viscous terms (gradients.f90, viscosity.f90, viscous.f90) -----
// The viscous flux of a face (viscous.f90:144-325, laminar: mu_t = 0) as a
// function of its 21 inputs x: the mean of the two cells' gradients
// x[4c+l] (component c, variable l of u, v, w, T), the left and right cells'
// u, v, w, T (x[12..15], x[16..19]) and the face viscosity x[20]; the
// geometry enters as constants.  Returns the four terms the reference
// subtracts from F(2:5).
template <typename D>
__device__ __forceinline__ void visc_flux_d(const Params& p, const D* x, const double* C0, const double* C1,
                                            const double* fc, D* Fv) {
  D G[3][4];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int l = 0; l < 4; ++l) G[c][l] = x[4 * c + l];
  const double dx0 = C1[1] - C0[1], dy0 = C1[2] - C0[2], dz0 = C1[3] - C0[3];
  const D delx(dx0), dely(dy0), delz(dz0), dLR(::sqrt(dx0 * dx0 + dy0 * dy0 + dz0 * dz0));
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const D del = x[16 + l] - x[12 + l];
    const D nc = (del - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
    G[0][l] = G[0][l] + (nc * delx / dLR);
    G[1][l] = G[1][l] + (nc * dely / dLR);
    G[2][l] = G[2][l] + (nc * delz / dLR);
  }
  const D two(2.), three(3.), half(0.5);
  const D tm = x[20];
  const D dudx = G[0][0], dudy = G[1][0], dudz = G[2][0];
  const D dvdx = G[0][1], dvdy = G[1][1], dvdz = G[2][1];
  const D dwdx = G[0][2], dwdy = G[1][2], dwdz = G[2][2];
  const D Txx = two * tm * (dudx - ((dudx + dvdy + dwdz) / three));
  const D Tyy = two * tm * (dvdy - ((dudx + dvdy + dwdz) / three));
  const D Tzz = two * tm * (dwdz - ((dudx + dvdy + dwdz) / three));
  const D Txy = tm * (dvdx + dudy), Txz = tm * (dwdx + dudz), Tyz = tm * (dwdy + dvdz);
  const D Kh = (tm / D(p.Pr)) * D(p.gm) * D(p.R) / D(p.gm - 1);
  const D Qx = Kh * G[0][3], Qy = Kh * G[1][3], Qz = Kh * G[2][3];
  const D A(fc[0]), nx(fc[1]), ny(fc[2]), nz(fc[3]);
  const D uf = half * (x[12] + x[16]), vf = half * (x[13] + x[17]), wf = half * (x[14] + x[18]);
  Fv[0] = (Txx * nx + Txy * ny + Txz * nz) * A;
  Fv[1] = (Txy * nx + Tyy * ny + Tyz * nz) * A;
  Fv[2] = (Txz * nx + Tyz * ny + Tzz * nz) * A;
  Fv[3] = A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) + ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
               ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz));
}

// visc_flux_d's arithmetic as a function of the face's geometry instead:
// g[0..3] the face record {A, nx, ny, nz}, g[4..6] and g[7..9] the left
// and right cells' centres; x: the values of visc_flux_d's 21 inputs.
template <typename D>
__device__ __forceinline__ void visc_flux_geo_d(const Params& p, const double* x, const D* g, D* Fv) {
  D G[3][4];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int l = 0; l < 4; ++l) G[c][l] = D(x[4 * c + l]);
  const D delx = g[7] - g[4], dely = g[8] - g[5], delz = g[9] - g[6];
  const D dLR = sqrt(delx * delx + dely * dely + delz * delz);
#pragma unroll
  for (int l = 0; l < 4; ++l) {
    const D del = D(x[16 + l]) - D(x[12 + l]);
    const D nc = (del - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
    G[0][l] = G[0][l] + (nc * delx / dLR);
    G[1][l] = G[1][l] + (nc * dely / dLR);
    G[2][l] = G[2][l] + (nc * delz / dLR);
  }
  const D two(2.), three(3.), half(0.5);
  const D tm(x[20]);
  const D dudx = G[0][0], dudy = G[1][0], dudz = G[2][0];
  const D dvdx = G[0][1], dvdy = G[1][1], dvdz = G[2][1];
  const D dwdx = G[0][2], dwdy = G[1][2], dwdz = G[2][2];
  const D Txx = two * tm * (dudx - ((dudx + dvdy + dwdz) / three));
  const D Tyy = two * tm * (dvdy - ((dudx + dvdy + dwdz) / three));
  const D Tzz = two * tm * (dwdz - ((dudx + dvdy + dwdz) / three));
  const D Txy = tm * (dvdx + dudy), Txz = tm * (dwdx + dudz), Tyz = tm * (dwdy + dvdz);
  const D Kh = (tm / D(p.Pr)) * D(p.gm) * D(p.R) / D(p.gm - 1);
  const D Qx = Kh * G[0][3], Qy = Kh * G[1][3], Qz = Kh * G[2][3];
  const D A = g[0], nx = g[1], ny = g[2], nz = g[3];
  const D uf = half * (D(x[12]) + D(x[16])), vf = half * (D(x[13]) + D(x[17])), wf = half * (D(x[14]) + D(x[18]));
  Fv[0] = (Txx * nx + Txy * ny + Txz * nz) * A;
  Fv[1] = (Txy * nx + Tyy * ny + Tyz * nz) * A;
  Fv[2] = (Txz * nx + Tyz * ny + Tzz * nz) * A;
  Fv[3] = A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) + ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
               ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz));
}

// d mu / d T of calculate_viscosity (viscosity.f90:109-136; constant mu: 0)
__device__ __forceinline__ double dmu_dT(const Params& p, double T) {
  if (p.mu_var != FEST_MU_SUTHERLAND) return 0.0;
  const double mu = p.mu_ref * (::pow(T / p.T_ref, 1.5)) * ((p.T_ref + p.S) / (T + p.S));
  return mu * (1.5 / T - 1.0 / (T + p.S));
}

// adjoints of a cell's u, v, w, T into its primitive state (T = p/(rho R),
// the temperature of update.f90:170 at this state)
__device__ __forceinline__ void give_uvwT(const Params& p, const DevBlock& b, double* bar, long long c,
                                          const double* g) {
  const long long P = p.d.P;
  const double rho = b.qp[c], pr = b.qp[c + 4 * P];
  if (g[0] != 0.0) atomicAdd(bar + c + P, g[0]);
  if (g[1] != 0.0) atomicAdd(bar + c + 2 * P, g[1]);
  if (g[2] != 0.0) atomicAdd(bar + c + 3 * P, g[2]);
  if (g[3] != 0.0) {
    atomicAdd(bar + c + 4 * P, g[3] / (rho * p.R));
    atomicAdd(bar + c, -g[3] * pr / (rho * rho * p.R));
  }
}

// one thread per face of direction dir: the transposed viscous flux onto
// mu = lambda(left) - lambda(right) (the flux enters the residual with a
// minus sign).  Gradient adjoints go to barG (interior cells, 12 per cell
// as [component][variable]); a ghost cell's gradient is its face's
// gradient BC (gradients.f90:486-676) of the interior cell, transposed here.
// With bar_face and bar_cells (metric adjoints, nullable) it also adds the
// flux's derivatives with respect to the face record and the two cells'
// centres, and those of a ghost gradient's BC with respect to the boundary
// face record and the interior cell's volume.
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_viscous(Params p, DevBlock b, const double* lam, double* bar,
                                                         double* barG, int dir, double* bar_face,
                                                         double* bar_cells) {
  using D = Dual<double, 21>;
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * na * nb) return;
  const int c = 1 + (int)(t % n);
  const long long r = t / n;
  const int ta = 1 + (int)(r % na), tb = 1 + (int)(r / na);
  const long long P = d.P, N = ncells(d), NG = ngrad(d);
  double mu[4] = {0, 0, 0, 0};
  int i, j, k;
  if (c - 1 >= 1) {
    cell_of(dir, c - 1, ta, tb, i, j, k);
    for (int l = 0; l < 4; ++l) mu[l] += lam[cidx(d, i, j, k) + N * (l + 1)];
  }
  if (c <= n - 1) {
    cell_of(dir, c, ta, tb, i, j, k);
    for (int l = 0; l < 4; ++l) mu[l] -= lam[cidx(d, i, j, k) + N * (l + 1)];
  }
  if (mu[0] == 0.0 && mu[1] == 0.0 && mu[2] == 0.0 && mu[3] == 0.0) return;
  int il, jl, kl, ir, jr, kr;
  cell_of(dir, c - 1, ta, tb, il, jl, kl);
  cell_of(dir, c, ta, tb, ir, jr, kr);
  const long long cL = pidx(d, il, jl, kl), cR = pidx(d, ir, jr, kr);
  const long long gL = gidx(d, il, jl, kl), gR = gidx(d, ir, jr, kr);
  D x[21], Fv[4];
#pragma unroll
  for (int cc = 0; cc < 3; ++cc)
#pragma unroll
    for (int l = 0; l < 4; ++l)
      x[4 * cc + l] = D::var(0.5 * (b.grad[cc][gL + NG * l] + b.grad[cc][gR + NG * l]), 4 * cc + l);
  const double TL = b.qp[cL + 4 * P] / (b.qp[cL] * p.R), TR = b.qp[cR + 4 * P] / (b.qp[cR] * p.R);
  for (int l = 0; l < 3; ++l) {
    x[12 + l] = D::var(b.qp[cL + P * (l + 1)], 12 + l);
    x[16 + l] = D::var(b.qp[cR + P * (l + 1)], 16 + l);
  }
  x[15] = D::var(TL, 15);
  x[19] = D::var(TR, 19);
  x[20] = D::var(0.5 * (b.mu[cL] + b.mu[cR]), 20);
  const long long fi = fidx(d, dir, ir, jr, kr);
  visc_flux_d<D>(p, x, b.cells + 4 * cL, b.cells + 4 * cR, b.faces[dir] + 4 * fi, Fv);
  double bx[21];
#pragma unroll
  for (int m = 0; m < 21; ++m) {
    double s = 0.0;
#pragma unroll
    for (int l = 0; l < 4; ++l) s -= mu[l] * Fv[l].d[m];
    bx[m] = s;
  }
  if (bar_face) {
    // the same flux as a function of the face record and the cell centres
    using DG = Dual<double, 10>;
    double xv[21];
#pragma unroll
    for (int m = 0; m < 21; ++m) xv[m] = x[m].v;
    const double* fc0 = b.faces[dir] + 4 * fi;
    const double* CL = b.cells + 4 * cL + 1;
    const double* CR = b.cells + 4 * cR + 1;
    DG g[10], Fg[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) g[m] = DG::var(fc0[m], m);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      g[4 + m] = DG::var(CL[m], 4 + m);
      g[7 + m] = DG::var(CR[m], 7 + m);
    }
    visc_flux_geo_d<DG>(p, xv, g, Fg);
    double bg[10];
#pragma unroll
    for (int m = 0; m < 10; ++m) {
      double s = 0.0;
#pragma unroll
      for (int l = 0; l < 4; ++l) s -= mu[l] * Fg[l].d[m];
      bg[m] = s;
    }
    for (int m = 0; m < 4; ++m) atomicAdd(bar_face + 4 * fi + m, bg[m]);
    for (int m = 0; m < 3; ++m) {
      atomicAdd(bar_cells + 4 * cL + 1 + m, bg[4 + m]);
      atomicAdd(bar_cells + 4 * cR + 1 + m, bg[7 + m]);
    }
  }
  // cell values and the face viscosity
  double gLv[4] = {bx[12], bx[13], bx[14], bx[15]}, gRv[4] = {bx[16], bx[17], bx[18], bx[19]};
  gLv[3] += 0.5 * bx[20] * dmu_dT(p, TL);
  gRv[3] += 0.5 * bx[20] * dmu_dT(p, TR);
  // gradients: half of the mean to each side; ghost sides through the BC
  double gG[2][12];
#pragma unroll
  for (int m = 0; m < 12; ++m) gG[0][m] = gG[1][m] = 0.5 * bx[m];
  for (int side = 0; side < 2; ++side) {
    const bool ghost = side == 0 ? (c == 1 && p.id[2 * dir] < 0) : (c == n && p.id[2 * dir + 1] < 0);
    double* gv = side == 0 ? gLv : gRv;
    if (!ghost) {
      const int ci = side == 0 ? (int)cidx(d, il, jl, kl) : (int)cidx(d, ir, jr, kr);
      for (int m = 0; m < 12; ++m)
        if (gG[side][m] != 0.0) atomicAdd(barG + (long long)ci * 12 + m, gG[side][m]);
      continue;
    }
    // G_ghost = jump(cI - cG) + tangential(G_I) (adiabatic walls: -G_I for T)
    const int f = 2 * dir + side;  // the low face has the ghost on the left
    const double* fc = b.faces[dir] + 4 * fi;
    const double nx = fc[1], ny = fc[2], nz = fc[3];
    const long long cI = side == 0 ? cR : cL;
    const double vI = b.cells[4 * cI];
    const double cc3[3] = {fc[0] * nx / vI, fc[0] * ny / vI, fc[0] * nz / vI};
    const double nn[3] = {nx, ny, nz};
    const double sig = side ? -1.0 : 1.0;
    const bool adiab = p.id[f] == -5 && (p.Tw[f] < 1. && p.Tw[f] >= 0.);
    double gI[12], jI[4], jG[4];
    for (int l = 0; l < 4; ++l) {
      double dot = 0.0;
      for (int q = 0; q < 3; ++q) dot += gG[side][4 * q + l] * nn[q];
      for (int q = 0; q < 3; ++q) gI[4 * q + l] = gG[side][4 * q + l] - nn[q] * dot;
      double s = 0.0;
      for (int q = 0; q < 3; ++q) s += gG[side][4 * q + l] * cc3[q];
      jI[l] = sig * s;
      jG[l] = -sig * s;
    }
    if (adiab) {
      for (int q = 0; q < 3; ++q) gI[4 * q + 3] -= gG[side][4 * q + 3];
      jI[3] = 0.0;
      jG[3] = 0.0;
    }
    if (bar_face) {
      // G_ghost(l) = sig (phi_I - phi_G) A n / V_I + G_I - n (G_I . n), the
      // T row of an adiabatic wall -n (G_I . n) (gradients.f90:486-676):
      // derivatives with respect to A, n and V_I
      const long long gIc = side == 0 ? gR : gL;
      const long long cG = side == 0 ? cL : cR;
      const double A = fc[0];
      const double TI = b.qp[cI + 4 * P] / (b.qp[cI] * p.R), TG = b.qp[cG + 4 * P] / (b.qp[cG] * p.R);
      double bA = 0.0, bn[3] = {0.0, 0.0, 0.0}, bV = 0.0;
      for (int l = 0; l < 4; ++l) {
        double GI[3], gb[3];
        for (int q = 0; q < 3; ++q) {
          GI[q] = b.grad[q][gIc + NG * l];
          gb[q] = gG[side][4 * q + l];
        }
        const double GIn = GI[0] * nn[0] + GI[1] * nn[1] + GI[2] * nn[2];
        const double gbn = gb[0] * nn[0] + gb[1] * nn[1] + gb[2] * nn[2];
        for (int q = 0; q < 3; ++q) bn[q] -= gb[q] * GIn + gbn * GI[q];
        if (adiab && l == 3) continue;
        const double diff = l == 3 ? TI - TG : b.qp[cI + P * (l + 1)] - b.qp[cG + P * (l + 1)];
        const double sd = sig * diff / vI;
        bA += sd * gbn;
        for (int q = 0; q < 3; ++q) bn[q] += sd * A * gb[q];
        bV -= sd * A * gbn / vI;
      }
      double* bfc = bar_face + 4 * fi;
      atomicAdd(bfc, bA);
      for (int q = 0; q < 3; ++q) atomicAdd(bfc + 1 + q, bn[q]);
      atomicAdd(bar_cells + 4 * cI, bV);
    }
    const int ci = side == 0 ? (int)cidx(d, ir, jr, kr) : (int)cidx(d, il, jl, kl);
    for (int m = 0; m < 12; ++m)
      if (gI[m] != 0.0) atomicAdd(barG + (long long)ci * 12 + m, gI[m]);
    double* gInt = side == 0 ? gRv : gLv;  // the interior cell's u, v, w, T
    for (int l = 0; l < 4; ++l) {
      gInt[l] += jI[l];
      gv[l] += jG[l];
    }
  }
  give_uvwT(p, b, bar, cL, gLv);
  give_uvwT(p, b, bar, cR, gRv);
}

// one thread per interior cell: its gradient adjoint through the
// Green-Gauss sum (gradients.f90:405-482) onto u, v, w, T of the cell and
// its six neighbours
// With bar_faces and bar_cells (nullable) it also adds the sum's
// derivatives with respect to the six face records and the cell's volume.
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_grad(Params p, DevBlock b, const double* barG, double* bar,
                                                      double* bf0, double* bf1, double* bf2,
                                                      double* bar_cells) {
  const Dims& d = p.d;
  const long long N = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int i = 1 + (int)(t % (d.imx - 1));
  const long long r = t / (d.imx - 1);
  const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
  const double* g = barG + t * 12;  // [component][variable]
  bool any = false;
  for (int m = 0; m < 12; ++m) any |= g[m] != 0.0;
  if (!any) return;
  const int ncomp = d.kmx > 2 ? 3 : 2;
  const long long c0 = pidx(d, i, j, k);
  const double vol2 = 2 * b.cells[4 * c0];
  // faces i, j, k (low, sign -1) and i+1, j+1, k+1 (high, +1) with their neighbours
  const double* fr[6] = {b.faces[0] + 4 * fidx(d, 0, i, j, k), b.faces[1] + 4 * fidx(d, 1, i, j, k),
                         b.faces[2] + 4 * fidx(d, 2, i, j, k), b.faces[0] + 4 * fidx(d, 0, i + 1, j, k),
                         b.faces[1] + 4 * fidx(d, 1, i, j + 1, k), b.faces[2] + 4 * fidx(d, 2, i, j, k + 1)};
  const long long nbc[6] = {pidx(d, i - 1, j, k), pidx(d, i, j - 1, k), pidx(d, i, j, k - 1),
                            pidx(d, i + 1, j, k), pidx(d, i, j + 1, k), pidx(d, i, j, k + 1)};
  double own[4] = {0, 0, 0, 0};
  for (int f = 0; f < 6; ++f) {
    const double sg = f < 3 ? -1.0 : 1.0;
    double gn[4];
    for (int l = 0; l < 4; ++l) {
      double s = 0.0;
      for (int q = 0; q < ncomp; ++q) s += g[4 * q + l] * fr[f][1 + q];
      gn[l] = sg * s * fr[f][0] / vol2;
      own[l] += gn[l];
    }
    give_uvwT(p, b, bar, nbc[f], gn);
  }
  give_uvwT(p, b, bar, c0, own);
  if (!bf0) return;
  // grad(q, l) = sum_f sg (phi_nb + phi_c)(l) n_q A / (2 V): face records and V
  auto phi = [&](long long c, int l) {
    return l == 3 ? b.qp[c + 4 * d.P] / (b.qp[c] * p.R) : b.qp[c + d.P * (l + 1)];
  };
  double* bfs[3] = {bf0, bf1, bf2};
  const long long fix[6] = {fidx(d, 0, i, j, k), fidx(d, 1, i, j, k), fidx(d, 2, i, j, k),
                            fidx(d, 0, i + 1, j, k), fidx(d, 1, i, j + 1, k), fidx(d, 2, i, j, k + 1)};
  double pc[4];
  for (int l = 0; l < 4; ++l) pc[l] = phi(c0, l);
  for (int f = 0; f < 6; ++f) {
    const double sg = f < 3 ? -1.0 : 1.0;
    double bA = 0.0, bn[3] = {0.0, 0.0, 0.0};
    for (int l = 0; l < 4; ++l) {
      const double w = sg * (phi(nbc[f], l) + pc[l]) / vol2;
      for (int q = 0; q < ncomp; ++q) {
        bA += g[4 * q + l] * w * fr[f][1 + q];
        bn[q] += g[4 * q + l] * w * fr[f][0];
      }
    }
    double* o = bfs[f % 3] + 4 * fix[f];
    atomicAdd(o, bA);
    for (int q = 0; q < ncomp; ++q) atomicAdd(o + 1 + q, bn[q]);
  }
  const long long og = gidx(d, i, j, k), NG = ngrad(d);
  double bV = 0.0;
  for (int l = 0; l < 4; ++l)
    for (int q = 0; q < ncomp; ++q) bV -= g[4 * q + l] * b.grad[q][og + NG * l];
  atomicAdd(bar_cells + 4 * c0, bV / b.cells[4 * c0]);
}

// ghost (layer L) / interior (layer m) cell of face f at (ta, tb)
__device__ __forceinline__ long long gcell_p(const Dims& d, int f, int L, int ta, int tb) {
  switch (f) {
    case 0: return pidx(d, 1 - L, ta, tb);
    case 1: return pidx(d, d.imx + L - 1, ta, tb);
    case 2: return pidx(d, ta, 1 - L, tb);
    case 3: return pidx(d, ta, d.jmx + L - 1, tb);
    case 4: return pidx(d, ta, tb, 1 - L);
    default: return pidx(d, ta, tb, d.kmx + L - 1);
  }
}
__device__ __forceinline__ long long icell_p(const Dims& d, int f, int m, int ta, int tb) {
  switch (f) {
    case 0: return pidx(d, m, ta, tb);
    case 1: return pidx(d, d.imx - m, ta, tb);
    case 2: return pidx(d, ta, m, tb);
    case 3: return pidx(d, ta, d.jmx - m, tb);
    case 4: return pidx(d, ta, tb, m);
    default: return pidx(d, ta, tb, d.kmx - m);
  }
}

// ---- k-omega SST terms (viscous.f90:144-447, viscosity.f90:215-546,
// source.f90:158-270, gradients.f90:276-676) ---------------------------------
// Gradients here are 18 per cell, G[3 l + c] for variable l of u, v, w, T,
// k, omega and component c, over the gradient range (0:imx, 0:jmx, 0:kmx).

constexpr double kSstA1 = 0.31, kSstBstar = 0.09, kSstBeta1 = 0.075, kSstBeta2 = 0.0828,
                 kSstSigK1 = 0.85, kSstSigK2 = 1.0, kSstSigW1 = 0.5, kSstSigW2 = 0.856, kSstKappa = 0.41;

// The face's viscous flux with the SST terms as a function of its 35
// inputs: x[0..17] the mean of the two cells' gradients, x[18..23] and
// x[24..29] the left and right cells' u, v, w, T, k, omega, x[30], x[31]
// their densities, x[32..34] the face's mean laminar viscosity, eddy
// viscosity and F1.  Fv: the six terms the reference subtracts from
// F(2:7) (momentum, energy, k, omega).
template <typename D>
__device__ __forceinline__ void visc_flux_sst_d(const Params& p, const D* x, const double* C0, const double* C1,
                                                const double* fc, D* Fv) {
  D G[3][6];
#pragma unroll
  for (int l = 0; l < 6; ++l)
#pragma unroll
    for (int c = 0; c < 3; ++c) G[c][l] = x[3 * l + c];
  const double dx0 = C1[1] - C0[1], dy0 = C1[2] - C0[2], dz0 = C1[3] - C0[3];
  const D delx(dx0), dely(dy0), delz(dz0), dLR(::sqrt(dx0 * dx0 + dy0 * dy0 + dz0 * dz0));
#pragma unroll
  for (int l = 0; l < 6; ++l) {
    const D del = x[24 + l] - x[18 + l];
    const D nc = (del - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
    G[0][l] = G[0][l] + (nc * delx / dLR);
    G[1][l] = G[1][l] + (nc * dely / dLR);
    G[2][l] = G[2][l] + (nc * delz / dLR);
  }
  const D mu_f = x[32], mut_f = x[33], F1 = x[34];
  const D tm = mu_f + mut_f;
  const D two(2.), three(3.), half(0.5);
  const D dudx = G[0][0], dudy = G[1][0], dudz = G[2][0];
  const D dvdx = G[0][1], dvdy = G[1][1], dvdz = G[2][1];
  const D dwdx = G[0][2], dwdy = G[1][2], dwdz = G[2][2];
  const D Txx = two * tm * (dudx - ((dudx + dvdy + dwdz) / three));
  const D Tyy = two * tm * (dvdy - ((dudx + dvdy + dwdz) / three));
  const D Tzz = two * tm * (dwdz - ((dudx + dvdy + dwdz) / three));
  const D Txy = tm * (dvdx + dudy), Txz = tm * (dwdx + dudz), Tyz = tm * (dwdy + dvdz);
  const D Kh = (mu_f / D(p.Pr) + mut_f / D(p.tPr)) * D(p.gm) * D(p.R) / D(p.gm - 1);
  const D Qx = Kh * G[0][3], Qy = Kh * G[1][3], Qz = Kh * G[2][3];
  const D A(fc[0]), nx(fc[1]), ny(fc[2]), nz(fc[3]);
  const D uf = half * (x[18] + x[24]), vf = half * (x[19] + x[25]), wf = half * (x[20] + x[26]);
  // viscous.f90:328-447
  const D skf = D(kSstSigK1) * F1 + D(kSstSigK2) * (D(1.) - F1);
  const D swf = D(kSstSigW1) * F1 + D(kSstSigW2) * (D(1.) - F1);
  const D rhof = half * (x[30] + x[31]), tkf = half * (x[22] + x[28]);
  const D Tk = D(-2.0) * rhof * tkf / D(3.0);
  const D dk = G[0][4] * nx + G[1][4] * ny + G[2][4] * nz;
  const D dw = G[0][5] * nx + G[1][5] * ny + G[2][5] * nz;
  const D kdiff = A * ((mu_f + skf * mut_f) * dk);
  Fv[0] = (Txx * nx + Txy * ny + Txz * nz) * A + Tk * nx * A;
  Fv[1] = (Txy * nx + Tyy * ny + Tyz * nz) * A + Tk * ny * A;
  Fv[2] = (Txz * nx + Tyz * ny + Tzz * nz) * A + Tk * nz * A;
  Fv[3] = A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) + ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
               ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz)) + kdiff;
  Fv[4] = kdiff;
  Fv[5] = A * ((mu_f + swf * mut_f) * dw);
}

// adjoints of a cell's u, v, w, T, k, omega and rho into its primitive state
__device__ __forceinline__ void give_sst(const Params& p, const DevBlock& b, double* bar, long long c,
                                         const double* g, double grho) {
  give_uvwT(p, b, bar, c, g);
  const long long P = p.d.P;
  if (g[4] != 0.0) atomicAdd(bar + c + 5 * P, g[4]);
  if (g[5] != 0.0) atomicAdd(bar + c + 6 * P, g[5]);
  if (grho != 0.0) atomicAdd(bar + c, grho);
}

// one thread per face of direction dir (the SST block's laminar and SST
// viscous terms together): the transposed flux onto the mean gradient
// (half to each cell's gradient adjoint barG, ghost cells included), the
// cells' u, v, w, T, k, omega, rho, the laminar viscosity (through
// Sutherland's law onto T) and the eddy viscosity and F1 (half to each
// cell's barMut, barF1)
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_viscous_sst(Params p, DevBlock b, const double* lam, double* bar,
                                                             double* barG, double* barMut, double* barF1, int dir) {
  // the 35 input directions in five passes of seven (duals of 35 would
  // not fit in registers)
  using D = Dual<double, 7>;
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * na * nb) return;
  int c, ta, tb;
  face_of(d, dir, t, c, ta, tb);
  const long long P = d.P, N = ncells(d), NG = ngrad(d);
  double mu[6] = {0, 0, 0, 0, 0, 0};
  int i, j, k;
  if (c - 1 >= 1) {
    cell_of(dir, c - 1, ta, tb, i, j, k);
    for (int l = 0; l < 6; ++l) mu[l] += lam[cidx(d, i, j, k) + N * (l + 1)];
  }
  if (c <= n - 1) {
    cell_of(dir, c, ta, tb, i, j, k);
    for (int l = 0; l < 6; ++l) mu[l] -= lam[cidx(d, i, j, k) + N * (l + 1)];
  }
  bool any = false;
  for (int l = 0; l < 6; ++l) any |= mu[l] != 0.0;
  if (!any) return;
  int il, jl, kl, ir, jr, kr;
  cell_of(dir, c - 1, ta, tb, il, jl, kl);
  cell_of(dir, c, ta, tb, ir, jr, kr);
  const long long cL = pidx(d, il, jl, kl), cR = pidx(d, ir, jr, kr);
  const long long gL = gidx(d, il, jl, kl), gR = gidx(d, ir, jr, kr);
  const double* q = b.qp;
  const double TL = q[cL + 4 * P] / (q[cL] * p.R), TR = q[cR + 4 * P] / (q[cR] * p.R);
  double xv[35];
  for (int l = 0; l < 6; ++l)
    for (int cc = 0; cc < 3; ++cc) xv[3 * l + cc] = 0.5 * (b.grad[cc][gL + NG * l] + b.grad[cc][gR + NG * l]);
  {
    const double vL[6] = {q[cL + P], q[cL + 2 * P], q[cL + 3 * P], TL, q[cL + 5 * P], q[cL + 6 * P]};
    const double vR[6] = {q[cR + P], q[cR + 2 * P], q[cR + 3 * P], TR, q[cR + 5 * P], q[cR + 6 * P]};
    for (int l = 0; l < 6; ++l) {
      xv[18 + l] = vL[l];
      xv[24 + l] = vR[l];
    }
  }
  xv[30] = q[cL];
  xv[31] = q[cR];
  xv[32] = 0.5 * (b.mu[cL] + b.mu[cR]);
  xv[33] = 0.5 * (b.mut[cL] + b.mut[cR]);
  xv[34] = 0.5 * (b.F1[cL] + b.F1[cR]);
  const long long fi = fidx(d, dir, ir, jr, kr);
  double bx[35];
#pragma unroll 1
  for (int g0 = 0; g0 < 35; g0 += 7) {
    D x[35], Fv[6];
    for (int m = 0; m < 35; ++m) x[m] = D::var(xv[m], m - g0);  // seeds g0..g0+6 only
    visc_flux_sst_d<D>(p, x, b.cells + 4 * cL, b.cells + 4 * cR, b.faces[dir] + 4 * fi, Fv);
    for (int m = 0; m < 7; ++m) {
      double s = 0.0;
      for (int l = 0; l < 6; ++l) s -= mu[l] * Fv[l].d[m];
      bx[g0 + m] = s;
    }
  }
  for (int m = 0; m < 18; ++m)
    if (bx[m] != 0.0) {
      atomicAdd(barG + gL * 18 + m, 0.5 * bx[m]);
      atomicAdd(barG + gR * 18 + m, 0.5 * bx[m]);
    }
  double gl[6], gr[6];
  for (int l = 0; l < 6; ++l) {
    gl[l] = bx[18 + l];
    gr[l] = bx[24 + l];
  }
  gl[3] += 0.5 * bx[32] * dmu_dT(p, TL);
  gr[3] += 0.5 * bx[32] * dmu_dT(p, TR);
  give_sst(p, b, bar, cL, gl, bx[30]);
  give_sst(p, b, bar, cR, gr, bx[31]);
  if (bx[33] != 0.0) {
    atomicAdd(barMut + cL, 0.5 * bx[33]);
    atomicAdd(barMut + cR, 0.5 * bx[33]);
  }
  if (bx[34] != 0.0) {
    atomicAdd(barF1 + cL, 0.5 * bx[34]);
    atomicAdd(barF1 + cR, 0.5 * bx[34]);
  }
}

// eddy viscosity and F1 of a cell (viscosity.f90:215-546) and, for an
// interior cell, its SST source (source.f90:158-270), on duals over
// (rho, k, omega, T, G[18]); the laminar viscosity from T
template <typename D>
__device__ __forceinline__ void sst_cell_d(const Params& p, const D* x, double dd, double vol, bool source,
                                           D& mut, D& F1, D& Sk, D& Sw) {
  const bool s2003 = p.turb == FEST_TURB_SST2003;
  const D rho = x[0], tk = x[1], tw = x[2], T = x[3];
  const D* G = x + 4;
  D mu;
  if (p.mu_var == FEST_MU_SUTHERLAND)
    mu = D(p.mu_ref) * pow(T / D(p.T_ref), D(1.5)) * ((D(p.T_ref) + D(p.S)) / (T + D(p.S)));
  else
    mu = D(p.mu_ref);
  const D d1(dd);
  const D var1 = sqrt(tk) / (D(kSstBstar) * tw * d1);
  const D var2 = D(500.) * (mu / rho) / ((d1 * d1) * tw);
  const D arg2 = fmax2(D(2.) * var1, var2);
  const D F = tanh(arg2 * arg2);
  const D NUM = rho * D(kSstA1) * tk;
  // G(component, variable) = G[3 (variable - 1) + component]
  const D wx = G[7] - G[5], wy = G[2] - G[6], wz = G[3] - G[1];
  const D vort = sqrt(wx * wx + wy * wy + wz * wz);
  D DENOM;
  if (s2003) {
    const D sxx = G[0], syy = G[4], szz = G[8];
    const D syz = G[7] + G[5], szx = G[2] + G[6], sxy = G[3] + G[1];
    const D SijSij = (D(2.) * (sxx * sxx)) + (D(2.) * (syy * syy)) + (D(2.) * (szz * szz)) + syz * syz + szx * szx +
                     sxy * sxy;
    DENOM = fmax2(fmax2(D(kSstA1) * tw, sqrt(SijSij) * F), D(1.0e-10));
  } else {
    DENOM = fmax2(fmax2(D(kSstA1) * tw, vort * F), D(1.e-20));
  }
  mut = NUM / DENOM;
  D CD = D(2.) * rho * D(kSstSigW2) * (G[12] * G[15] + G[13] * G[16] + G[14] * G[17]) / tw;
  CD = fmax2(CD, D(s2003 ? 1.0e-10 : 1e-20));
  const D right = D(4.) * (rho * D(kSstSigW2) * tk) / (CD * (d1 * d1));
  const D arg1 = fmin2(fmax2(var1, var2), right);
  const D a2 = arg1 * arg1;
  F1 = tanh(a2 * a2);
  if (!source) return;
  const double lim = s2003 ? 10.0 : 20.0;
  const double g1 = s2003 ? 5.0 / 9.0 : (kSstBeta1 / kSstBstar) - ((kSstSigW1 * (kSstKappa * kSstKappa)) / ::sqrt(kSstBstar));
  const double g2 = s2003 ? 0.44 : (kSstBeta2 / kSstBstar) - ((kSstSigW2 * (kSstKappa * kSstKappa)) / ::sqrt(kSstBstar));
  const D gama = D(g1) * F1 + D(g2) * (D(1.) - F1);
  const D beta = D(kSstBeta1) * F1 + D(kSstBeta2) * (D(1.) - F1);
  const D Dk = D(kSstBstar) * rho * tw * tk;
  const D Dw = beta * rho * (tw * tw);
  const D divergence = G[0] + G[4] + G[8];
  D Pk = mut * (vort * vort) - ((D(2.0) / D(3.0)) * rho * tk * divergence);
  Pk = fmin2(Pk, D(lim) * Dk);
  const D Pw = (rho * gama / mut) * Pk;
  const D lamda = (D(1.) - F1) * CD;
  Sk = (Pk - Dk) * D(vol);
  Sw = (Pw - Dw + lamda) * D(vol);
}

// the face id whose layer-1 ghost cell (i, j, k) of the gradient range is,
// or -1 (interior, edge or corner)
__device__ __forceinline__ int ghost_face_of(const Dims& d, int i, int j, int k) {
  const int oi = (i == 0) + (i == d.imx), oj = (j == 0) + (j == d.jmx), ok = (k == 0) + (k == d.kmx);
  if (oi + oj + ok != 1) return -1;
  if (oi) return i == 0 ? 0 : 1;
  if (oj) return j == 0 ? 2 : 3;
  return k == 0 ? 4 : 5;
}

// ghost layer-1 eddy viscosity and F1 of faces -1..-9 are copies of the
// interior cell's (the wall negating mu_t, viscosity.f90:287-340): their
// adjoints move into the interior cell's
__global__ void k_vjp_mut_ghost(Params p, double* barMut, double* barF1) {
  const int f = blockIdx.z;
  const Dims& d = p.d;
  const int id = p.id[f];
  if (!(id <= -1 && id >= -9)) return;
  const int dir = f / 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)(t / na);
  const long long g = gcell_p(d, f, 1, ta, tb), in = icell_p(d, f, 1, ta, tb);
  const double bm = barMut[g], bf = barF1[g];
  barMut[g] = 0.0;
  barF1[g] = 0.0;
  if (bm != 0.0) atomicAdd(barMut + in, id == -5 ? -bm : bm);
  if (bf != 0.0) atomicAdd(barF1 + in, bf);
}

// one thread per cell of the gradient range whose eddy viscosity and F1
// come from its own state (interior cells, and the layer-1 ghost cells of
// faces other than -1..-9): the transposed mu_t, F1 and (interior) source
// onto its rho, k, omega, p and its gradient (barG)
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_sst_cell(Params p, DevBlock b, const double* lam, double* bar,
                                                          double* barG, const double* barMut,
                                                          const double* barF1) {
  using D = Dual<double, 22>;
  const Dims& d = p.d;
  const long long NG = ngrad(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= NG) return;
  const int i = (int)(t % (d.imx + 1));
  const long long r = t / (d.imx + 1);
  const int j = (int)(r % (d.jmx + 1)), k = (int)(r / (d.jmx + 1));
  const bool interior = i >= 1 && i <= d.imx - 1 && j >= 1 && j <= d.jmx - 1 && k >= 1 && k <= d.kmx - 1;
  if (!interior) {
    const int f = ghost_face_of(d, i, j, k);
    if (f < 0 || (p.id[f] <= -1 && p.id[f] >= -9)) return;
  }
  const long long c0 = pidx(d, i, j, k), P = d.P;
  const double wm = barMut[c0], wf = barF1[c0];
  double wk = 0.0, ww = 0.0;
  if (interior) {
    const long long ci = cidx(d, i, j, k), N = ncells(d);
    wk = -lam[ci + 5 * N];  // the residual of k loses Sk, that of omega Sw
    ww = -lam[ci + 6 * N];
  }
  if (wm == 0.0 && wf == 0.0 && wk == 0.0 && ww == 0.0) return;
  const double* q = b.qp;
  const double rho = q[c0], pr = q[c0 + 4 * P];
  const double T = pr / (rho * p.R);
  D x[22];
  x[0] = D::var(rho, 0);
  x[1] = D::var(q[c0 + 5 * P], 1);
  x[2] = D::var(q[c0 + 6 * P], 2);
  x[3] = D::var(T, 3);
  for (int l = 0; l < 6; ++l)
    for (int cc = 0; cc < 3; ++cc) x[4 + 3 * l + cc] = D::var(b.grad[cc][t + NG * l], 4 + 3 * l + cc);
  D mut, F1, Sk, Sw;
  sst_cell_d<D>(p, x, b.dist[c0], b.cells[4 * c0], interior, mut, F1, Sk, Sw);
  double bx[22];
  for (int m = 0; m < 22; ++m) {
    double s = wm * mut.d[m] + wf * F1.d[m];
    if (interior) s += wk * Sk.d[m] + ww * Sw.d[m];
    bx[m] = s;
  }
  for (int m = 0; m < 18; ++m)
    if (bx[4 + m] != 0.0) atomicAdd(barG + t * 18 + m, bx[4 + m]);
  // T = p / (rho R)
  const double grho = bx[0] - bx[3] * pr / (rho * rho * p.R), gp = bx[3] / (rho * p.R);
  if (grho != 0.0) atomicAdd(bar + c0, grho);
  if (gp != 0.0) atomicAdd(bar + c0 + 4 * P, gp);
  if (bx[1] != 0.0) atomicAdd(bar + c0 + 5 * P, bx[1]);
  if (bx[2] != 0.0) atomicAdd(bar + c0 + 6 * P, bx[2]);
}

// a layer-1 ghost cell's gradient of a face with a negative id
// (apply_gradient_bc, gradients.f90:486-676) is the jump over the face
// sigma (v_I - v_G) A n / V_I plus the interior gradient's tangential part
// (adiabatic walls: minus the interior temperature gradient in place of
// its jump); transposed onto the interior gradient and the two cells'
// variables.  One thread per ghost column.
__global__ void k_vjp_grad_bc(Params p, DevBlock b, double* barG, double* bar) {
  const int f = blockIdx.z;
  const Dims& d = p.d;
  const int id = p.id[f];
  if (!(id < 0)) return;
  const int dir = f / 2, hi = f % 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)(t / na);
  const int n = extent_of(d, dir);
  int gi, gj, gk, ii, ij, ik;
  const int cg = hi ? n : 0, ci = hi ? n - 1 : 1;
  if (dir == 0) { gi = cg; gj = ta; gk = tb; ii = ci; ij = ta; ik = tb; }
  else if (dir == 1) { gi = ta; gj = cg; gk = tb; ii = ta; ij = ci; ik = tb; }
  else { gi = ta; gj = tb; gk = cg; ii = ta; ij = tb; ik = ci; }
  const long long og = gidx(d, gi, gj, gk), oi = gidx(d, ii, ij, ik);
  double a[18];
  bool any = false;
  for (int m = 0; m < 18; ++m) {
    a[m] = barG[og * 18 + m];
    barG[og * 18 + m] = 0.0;
    any |= a[m] != 0.0;
  }
  if (!any) return;
  const int fcn = hi ? n : 1;
  const double* fc = b.faces[dir] + 4 * fidx(d, dir, dir == 0 ? fcn : ta, dir == 1 ? fcn : (dir == 0 ? ta : tb),
                                             dir == 2 ? fcn : tb);
  const double nx = fc[1], ny = fc[2], nz = fc[3];
  const long long cI = pidx(d, ii, ij, ik), cG = pidx(d, gi, gj, gk);
  const double vI = b.cells[4 * cI];
  const double cc3[3] = {fc[0] * nx / vI, fc[0] * ny / vI, fc[0] * nz / vI};
  const double nn[3] = {nx, ny, nz};
  const double sig = hi ? -1.0 : 1.0;
  const bool adiab = id == -5 && (p.Tw[f] < 1. && p.Tw[f] >= 0.);
  double gI[6] = {0, 0, 0, 0, 0, 0}, gG[6] = {0, 0, 0, 0, 0, 0};
  for (int l = 0; l < 6; ++l) {
    double dot = 0.0, s = 0.0;
    for (int q = 0; q < 3; ++q) {
      dot += a[3 * l + q] * nn[q];
      s += a[3 * l + q] * cc3[q];
    }
    for (int q = 0; q < 3; ++q) {
      double g = a[3 * l + q] - nn[q] * dot;           // the tangential part
      if (adiab && l == 3) g -= a[3 * l + q];          // minus the interior T gradient
      if (g != 0.0) atomicAdd(barG + oi * 18 + 3 * l + q, g);
    }
    if (!(adiab && l == 3)) {
      gI[l] = sig * s;
      gG[l] = -sig * s;
    }
  }
  give_sst(p, b, bar, cI, gI, 0.0);
  give_sst(p, b, bar, cG, gG, 0.0);
}

// one thread per interior cell: its gradient adjoint (18 values, barG)
// through the Green-Gauss sum (gradients.f90:405-482) onto u, v, w, T, k,
// omega of the cell and its six neighbours
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_grad_sst(Params p, DevBlock b, const double* barG, double* bar) {
  const Dims& d = p.d;
  const long long N = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int i = 1 + (int)(t % (d.imx - 1));
  const long long r = t / (d.imx - 1);
  const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
  const double* g = barG + gidx(d, i, j, k) * 18;  // [variable][component]
  bool any = false;
  for (int m = 0; m < 18; ++m) any |= g[m] != 0.0;
  if (!any) return;
  const int ncomp = d.kmx > 2 ? 3 : 2;
  const long long c0 = pidx(d, i, j, k);
  const double vol2 = 2 * b.cells[4 * c0];
  const double* fr[6] = {b.faces[0] + 4 * fidx(d, 0, i, j, k), b.faces[1] + 4 * fidx(d, 1, i, j, k),
                         b.faces[2] + 4 * fidx(d, 2, i, j, k), b.faces[0] + 4 * fidx(d, 0, i + 1, j, k),
                         b.faces[1] + 4 * fidx(d, 1, i, j + 1, k), b.faces[2] + 4 * fidx(d, 2, i, j, k + 1)};
  const long long nbc[6] = {pidx(d, i - 1, j, k), pidx(d, i, j - 1, k), pidx(d, i, j, k - 1),
                            pidx(d, i + 1, j, k), pidx(d, i, j + 1, k), pidx(d, i, j, k + 1)};
  double own[6] = {0, 0, 0, 0, 0, 0};
  for (int f = 0; f < 6; ++f) {
    const double sg = f < 3 ? -1.0 : 1.0;
    double gn[6];
    for (int l = 0; l < 6; ++l) {
      double s = 0.0;
      for (int q = 0; q < ncomp; ++q) s += g[3 * l + q] * fr[f][1 + q];
      gn[l] = sg * s * fr[f][0] / vol2;
      own[l] += gn[l];
    }
    give_sst(p, b, bar, nbc[f], gn, 0.0);
  }
  give_sst(p, b, bar, c0, own, 0.0);
}

// the ghost cells' adjoints flow back into the interior cells the BC of
// their face computed them from (bc_primitive.f90:160-206 and the
// procedures it calls, at iteration iter); the ghost entries end at zero
template <typename T>
__global__ void __launch_bounds__(TPB_ADJ) k_vjp_ghosts(Params p, DevBlock b, double* bar, int iter,
                                                        double* bf0, double* bf1, double* bf2) {
  double* bfd[3] = {bf0, bf1, bf2};  // face-metric adjoints (null: not wanted)
  const Dims& d = p.d;
  const int f = blockIdx.z, dir = f / 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)(t / na);
  const long long P = d.P;
  const int id = p.id[f];
  auto take = [&](int L, int l) -> double {  // read and clear a ghost adjoint
    double* g = bar + gcell_p(d, f, L, ta, tb) + P * l;
    const double v = *g;
    *g = 0.0;
    return v;
  };
  auto give = [&](int m, int l, double v) {
    if (v != 0.0) atomicAdd(bar + icell_p(d, f, m, ta, tb) + P * l, v);
  };
  auto flat = [&](int l) { give(1, l, take(1, l) + take(2, l) + take(3, l)); };
  auto symm = [&](int l) {
    for (int L = 1; L <= 3; ++L) {
      const double g = take(L, l);
      give(L, l, p.c2 / p.c1 * g);
      give(L + 1, l, -p.c3 / p.c1 * g);
    }
  };
  auto anti = [&](int l) { for (int L = 1; L <= 3; ++L) give(L, l, -take(L, l)); };
  auto none = [&](int l) { for (int L = 1; L <= 3; ++L) take(L, l); };  // constant ghosts
  int fi, fj, fk;
  {
    const int c = (f % 2 == 0) ? 1 : extent_of(d, dir);
    if (dir == 0) { fi = c; fj = ta; fk = tb; }
    else if (dir == 1) { fi = ta; fj = c; fk = tb; }
    else { fi = ta; fj = tb; fk = c; }
  }
  const int nv = d.nv;  // 5, or 7 with k and omega (bc_primitive.f90:160-206)
  switch (id) {
    case -1: for (int l = 0; l < nv; ++l) none(l); break;
    case -2:
    case -7: for (int l = 0; l < nv; ++l) flat(l); break;
    case -3: for (int l = 0; l < 4; ++l) none(l); flat(4); for (int l = 5; l < nv; ++l) none(l); break;
    case -4: for (int l = 0; l < 4; ++l) flat(l); none(4); for (int l = 5; l < nv; ++l) flat(l); break;
    case -5:  // adiabatic wall (the host admits Tw in [0,1] only)
      if (nv == 7) {
        // set_omega_at_wall (bc_primitive.f90:564-643), last in the fill:
        // omega_G(L) = 120 mu(Tf) / (rho_f beta1 (2 d_1)^2) - omega_I(L),
        // Tf and rho_f the means over ghost and interior layer 1 (whose
        // ghost values the wall's own copies made, so their adjoints go to
        // the ghost entries the copies below then move inwards)
        const long long g1 = gcell_p(d, f, 1, ta, tb), i1 = icell_p(d, f, 1, ta, tb);
        const double rg = b.qp[g1], pg = b.qp[g1 + 4 * P], ri = b.qp[i1], pi = b.qp[i1 + 4 * P];
        const double Tf = 0.5 * ((pg / rg) + (pi / ri)) / p.R;
        const double Tr = p.T_ref, S = p.S;
        const double mu = p.mu_ref * ::pow(Tf / Tr, 1.5) * ((Tr + S) / (Tf + S));
        const double dmu = mu * (1.5 / Tf - 1.0 / (Tf + S));
        const double rf = 0.5 * (rg + ri), dd = 2 * b.dist[i1];
        const double W = 120 * mu / (rf * kSstBeta1 * (dd * dd));
        double gT = 0.0, gR = 0.0;
        for (int L = 1; L <= 3; ++L) {
          const double a = take(L, 6);
          give(L, 6, -a);
          gT += a * W * dmu / mu;
          gR += -a * W / rf;
        }
        // Tf = (pg/rg + pi/ri) / (2 R), rho_f = (rg + ri) / 2
        bar[g1 + 4 * P] += gT * 0.5 / (rg * p.R);
        bar[g1] += -gT * 0.5 * pg / (rg * rg * p.R) + 0.5 * gR;
        give(1, 4, gT * 0.5 / (ri * p.R));
        give(1, 0, -gT * 0.5 * pi / (ri * ri * p.R) + 0.5 * gR);
        anti(5);
      }
      symm(4); symm(0); anti(1); anti(2); anti(3);
      break;
    case -6: {  // slip wall: g = u - 2 (u.fn) fr  ->  bar_u += g_bar - 2 fn (fr.g_bar)
      for (int l = 5; l < nv; ++l) symm(l);
      symm(0); symm(4);
      const long long in_n = fidx(d, dir, fi, fj, fk), in_r = fidx(d, 0, fi, fj, fk);
      const double* fn = b.faces[dir] + 4 * in_n;
      const double* fr = b.faces[0] + 4 * in_r;
      double bn[3] = {0, 0, 0}, br[3] = {0, 0, 0};
      for (int L = 1; L <= 3; ++L) {
        const double gu = take(L, 1), gv = take(L, 2), gw = take(L, 3);
        const double s = fr[1] * gu + fr[2] * gv + fr[3] * gw;
        give(L, 1, gu - 2.0 * fn[1] * s);
        give(L, 2, gv - 2.0 * fn[2] * s);
        give(L, 3, gw - 2.0 * fn[3] * s);
        if (bf0) {  // g = u - 2 (u.fn) fr
          const long long in = icell_p(d, f, L, ta, tb);
          const double u[3] = {b.qp[in + P], b.qp[in + 2 * P], b.qp[in + 3 * P]};
          const double un = u[0] * fn[1] + u[1] * fn[2] + u[2] * fn[3];
          for (int m = 0; m < 3; ++m) {
            bn[m] += -2.0 * u[m] * s;
            br[m] += -2.0 * un * (m == 0 ? gu : m == 1 ? gv : gw);
          }
        }
      }
      if (bf0)
        for (int m = 0; m < 3; ++m) {
          if (bn[m] != 0.0) atomicAdd(bfd[dir] + 4 * in_n + 1 + m, bn[m]);
          if (br[m] != 0.0) atomicAdd(bf0 + 4 * in_r + 1 + m, br[m]);
        }
    } break;
    case -8:
    case -11: {  // all three layers = riemann_ghost(interior layer 1)
      using D8 = Dual<T, 8>;  // interior layer 1 (5) and the face normal (3)
      double gs[5];
      for (int l = 0; l < 5; ++l) gs[l] = take(1, l) + take(2, l) + take(3, l);
      const long long fnx = fidx(d, dir, fi, fj, fk);
      const double* fc = b.faces[dir] + 4 * fnx;
      const double sg = (f % 2 == 0) ? -1.0 : 1.0;
      const long long in1 = icell_p(d, f, 1, ta, tb);
      D8 in[5], g[5];
      for (int l = 0; l < 5; ++l) in[l] = D8::var((T)b.qp[in1 + P * l], l);
      riemann_ghost<D8>(p, f, id == -11, D8::var((T)(sg * fc[1]), 5), D8::var((T)(sg * fc[2]), 6),
                        D8::var((T)(sg * fc[3]), 7), in, g);
      for (int m = 0; m < 8; ++m) {
        double s = 0.0;
        for (int l = 0; l < 5; ++l) s += gs[l] * (double)g[l].d[m];
        if (m < 5) give(1, m, s);
        else if (bf0 && s != 0.0) atomicAdd(bfd[dir] + 4 * fnx + 1 + (m - 5), sg * s);
      }
    } break;
    default:
      if (id == -10 || id >= 0) {  // ghost L <- layer L of the partner face (same block)
        const int pf = p.part_face[f];
        int na, nb, pa, pb;
        face_columns(d, f, na, nb);
        interface_map(p.part_orient[f], na, nb, ta, tb, pa, pb);
        for (int l = 0; l < nv; ++l)
          for (int L = 1; L <= 3; ++L) {
            const double g = take(L, l);
            if (g != 0.0) atomicAdd(bar + icell_p(d, pf, L, pa, pb) + P * l, g);
          }
      } else {
        for (int l = 0; l < nv; ++l) none(l);
      }
  }
}

unsigned nblocks(long long n) { return (unsigned)((n + TPB_ADJ - 1) / TPB_ADJ); }

// mu = P^T phi with P = (dt/V) dq/dU, the local-time-step preconditioner of
// the forward-Euler update (update.f90:431) mapping a conservative residual
// to a primitive increment; dq/dU of q = (rho,u,v,w,p), U = (rho,rho u,
// rho v, rho w, E)
__global__ void k_adj_precond(Params p, DevBlock b, const double* phi, double* mu) {
  const Dims& d = p.d;
  const long long N = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N) return;
  const int i = 1 + (int)(t % (d.imx - 1));
  const long long r = t / (d.imx - 1);
  const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
  const long long c = pidx(d, i, j, k), ci = cidx(d, i, j, k), P = d.P;
  const double rho = b.qp[c], u = b.qp[c + P], v = b.qp[c + 2 * P], w = b.qp[c + 3 * P];
  const double g1 = p.gm - 1.0;
  const double f0 = phi[c], fu = phi[c + P], fv = phi[c + 2 * P], fw = phi[c + 3 * P], fp = phi[c + 4 * P];
  const double s = b.dt[ci] / b.cells[4 * c];
  double m0 = f0 - (u * fu + v * fv + w * fw) / rho + 0.5 * g1 * (u * u + v * v + w * w) * fp;
  if (d.nv == 7) {
    // k = U6/rho, omega = U7/rho (no k in the energy, update.f90:377-386),
    // and the point-implicit destruction that divides R6, R7 by
    // 1 + beta omega dt and 1 + 2 beta omega dt (update.f90:395-398; its
    // derivatives carry a factor R, zero at the fixed point)
    const double tk = b.qp[c + 5 * P], tw = b.qp[c + 6 * P];
    const double fk = phi[c + 5 * P], fo = phi[c + 6 * P];
    const double F1 = b.F1[c], dt = b.dt[ci];
    const double beta = 0.075 * F1 + (1. - F1) * 0.0828;
    m0 -= (tk * fk + tw * fo) / rho;
    mu[ci + 5 * N] = s * (fk / rho) / (1 + (beta * tw * dt));
    mu[ci + 6 * N] = s * (fo / rho) / (1 + (2 * beta * tw * dt));
  }
  mu[ci] = s * m0;
  mu[ci + N] = s * (fu / rho - g1 * u * fp);
  mu[ci + 2 * N] = s * (fv / rho - g1 * v * fp);
  mu[ci + 3 * N] = s * (fw / rho - g1 * w * fp);
  mu[ci + 4 * N] = s * (g1 * fp);
}

// out = c0 x0 + c1 x1 + c2 x2 + c3 x3 on interior cells (null x: term
// absent); with sq, also sum |out - x0|^2
__global__ void k_adj_combine(Dims d, double* out, double c0, const double* x0, double c1,
                              const double* x1, double c2, const double* x2, double c3,
                              const double* x3, double* sq) {
  __shared__ double red[TPB_ADJ];
  const long long N = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (t < N) {
    const int i = 1 + (int)(t % (d.imx - 1));
    const long long r = t / (d.imx - 1);
    const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
    const long long c = pidx(d, i, j, k);
    for (int l = 0; l < d.nv; ++l) {
      const long long e = c + d.P * l;
      double v = c0 * x0[e];
      if (x1) v += c1 * x1[e];
      if (x2) v += c2 * x2[e];
      if (x3) v += c3 * x3[e];
      if (sq) acc += (v - x0[e]) * (v - x0[e]);
      out[e] = v;
    }
  }
  if (!sq) return;
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0 && red[0] != 0.0) atomicAdd(sq, red[0]);
}

__global__ void k_adj_psi(Dims d, const double* mu, double* psi) {  // psi = -mu
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ncells(d) * d.nv) psi[t] = -mu[t];
}

}  // namespace

long long vjp_grad_work_doubles(const Dims& d, bool sst) {
  return sst ? 18 * ngrad(d) + 2 * d.P : 12 * ncells(d);
}

bool vjp_supported(const Params& p) {
  // no model or k-omega SST (the other models have no residual VJP)
  if (p.turb != FEST_TURB_NONE && p.turb != FEST_TURB_SST && p.turb != FEST_TURB_SST2003) return false;
  if (p.transition != FEST_TRANSITION_NONE) return false;
  const bool sst = p.turb != FEST_TURB_NONE;
  if (p.d.nv != (sst ? 7 : 5)) return false;
  if (sst) {
    // k-omega SST: viscous, and faces whose k and omega ghosts the
    // transpose knows (no far-field or total-pressure faces, whose ghosts
    // depend on the last column of the fill, and no block interfaces)
    if (p.mu_ref == 0.0) return false;
    for (int f = 0; f < 6; ++f)
      if (p.id[f] == -8 || p.id[f] == -11 || p.id[f] >= 0) return false;
  }
  if (p.pb[0] || p.pb[1] || p.pb[2]) return false;  // pressure switch couples variables
  if (ghosts_need_sequential(p) || p.d.kmx == 2) return false;
  for (int f = 0; f < 6; ++f) {
    const int id = p.id[f];
    if (id == -9) return false;
    if (id == -5 && (p.Tw[f] < 0.0 || p.Tw[f] > 1.0)) return false;
    if (p.mu_ref != 0.0 && id >= 0) return false;  // a raw ghost gradient would reach past the ghosts
  }
  return true;
}

// S^T v = v - (dR/dq)^T (P^T v): the transpose of one forward-Euler stage
// linearised at the fixed point
static void apply_ST(const Params& p, const DevBlock& b, const double* v, double* out, AdjointWork& w,
                     const Launcher& L) {
  const long long N = ncells(p.d);
  k_adj_precond<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p, b, v, w.mu);
  launch_residual_vjp(p, b, 3, w.mu, w.bar, L, nullptr, w.grad, w.face);
  k_adj_combine<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p.d, out, 1.0, v, -1.0, w.bar, 0.0, nullptr, 0.0,
                                                 nullptr, nullptr);
  *L.count += 2;
}

// One step phi <- G^T phi + dJ/dq of the transposed integrator map
// linearised at the fixed point (S = I - P dR/dq):
//   forward Euler  G = S
//   TVD-RK3        G = I/3 + S/2 + S^3/6  (update.f90:196-206 blends)
void launch_adjoint_iteration(const Params& p, const DevBlock& b, AdjointWork& w, const Launcher& L) {
  const long long N = ncells(p.d);
  if (p.integ == FEST_TIME_TVDRK3) {
    apply_ST(p, b, w.phi, w.a, w, L);
    apply_ST(p, b, w.a, w.b, w, L);
    apply_ST(p, b, w.b, w.c, w, L);
    k_adj_combine<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p.d, w.phi, 1.0 / 3.0, w.phi, 0.5, w.a, 1.0 / 6.0,
                                                   w.c, 1.0, w.dJ, w.sq);
  } else {
    apply_ST(p, b, w.phi, w.a, w, L);
    k_adj_combine<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p.d, w.phi, 0.0, w.phi, 1.0, w.a, 1.0, w.dJ, 0.0,
                                                   nullptr, w.sq);
  }
  ++*L.count;
}

// psi = -P^T H phi with H = I (forward Euler) or 2/3 I + S^T/6 + (S^T)^2/6
// (TVD-RK3), so that (dR/dq)^T psi = -dJ/dq at the fixed point of phi
void launch_adjoint_psi(const Params& p, const DevBlock& b, AdjointWork& w, double* psi,
                        const Launcher& L) {
  const long long N = ncells(p.d);
  const double* h = w.phi;
  if (p.integ == FEST_TIME_TVDRK3) {
    apply_ST(p, b, w.phi, w.a, w, L);
    apply_ST(p, b, w.a, w.b, w, L);
    k_adj_combine<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p.d, w.c, 2.0 / 3.0, w.phi, 1.0 / 6.0, w.a,
                                                   1.0 / 6.0, w.b, 0.0, nullptr, nullptr);
    ++*L.count;
    h = w.c;
  }
  k_adj_precond<<<nblocks(N), TPB_ADJ, 0, L.s>>>(p, b, h, w.mu);
  k_adj_psi<<<nblocks(N * p.d.nv), TPB_ADJ, 0, L.s>>>(p.d, w.mu, psi);
  *L.count += 2;
}

long long vjp_face_work_doubles(const Dims& d) {
  long long m = 0;
  for (int dir = 0; dir < 3; ++dir)
    m = std::max<long long>(m, (long long)extent_of(d, dir) * ((dir == 0 ? d.jmx : d.imx) - 1) *
                                   ((dir == 2 ? d.jmx : d.kmx) - 1));
  return 2 * NVMAX * m;
}

void launch_residual_vjp(const Params& p, const DevBlock& b, int iter, const double* lam,
                         double* bar, const Launcher& L, double* const* bar_faces, double* bar_grad,
                         double* face_work, double* bar_cells) {
  const Dims& d = p.d;
  const bool visc = p.mu_ref != 0.0, sst = p.turb != FEST_TURB_NONE;
  cudaMemsetAsync(bar, 0, sizeof(double) * (size_t)d.P * d.nv, L.s);
  if (visc) cudaMemsetAsync(bar_grad, 0, sizeof(double) * (size_t)vjp_grad_work_doubles(d, sst), L.s);
  // MUSCL and first-order states read cells c-1..c+1 only
  const bool narrow = p.interp == FEST_INTERP_MUSCL || p.interp == FEST_INTERP_NONE;
  // SST: gradient adjoints over the gradient range, then mu_t and F1
  double* barG = bar_grad;
  double* barMut = sst ? bar_grad + 18 * ngrad(d) : nullptr;
  double* barF1 = sst ? barMut + d.P : nullptr;
  for (int dir = 0; dir < 3; ++dir) {
    const int n = extent_of(d, dir);
    const long long nf = (long long)n * ((dir == 0 ? d.jmx : d.imx) - 1) * ((dir == 2 ? d.jmx : d.kmx) - 1);
    // cells 0..n of every line: the per-(cell, variable) kernels
    const long long ncl = nf / n * (n + 1);
    double* bf = bar_faces ? bar_faces[dir] : nullptr;
    if (d.nv == 7) {
      k_vjp_states<double, 7><<<nblocks(7 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, dir);
      if (p.flux == FEST_FLUX_SLAU)
        k_vjp_flux<double, true, 7><<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, face_work, bf, dir);
      else
        k_vjp_flux<double, false, 7><<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, face_work, bf, dir);
      if (narrow)
        k_vjp_recon<double, 7, 3><<<nblocks(7 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, bar, dir);
      else
        k_vjp_recon<double, 7, 5><<<nblocks(7 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, bar, dir);
    } else {
      k_vjp_states<double, 5><<<nblocks(5 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, dir);
      if (p.flux == FEST_FLUX_SLAU)
        k_vjp_flux<double, true, 5><<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, face_work, bf, dir);
      else
        k_vjp_flux<double, false, 5><<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, face_work, bf, dir);
      if (narrow)
        k_vjp_recon<double, 5, 3><<<nblocks(5 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, bar, dir);
      else
        k_vjp_recon<double, 5, 5><<<nblocks(5 * ncl), TPB_ADJ, 0, L.s>>>(p, b, face_work, bar, dir);
    }
    *L.count += 3;
    if (sst) {
      k_vjp_viscous_sst<<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, bar, barG, barMut, barF1, dir);
      ++*L.count;
    } else if (visc) {
      k_vjp_viscous<<<nblocks(nf), TPB_ADJ, 0, L.s>>>(p, b, lam, bar, bar_grad, dir,
                                                       bar_cells ? bf : nullptr, bar_cells);
      ++*L.count;
    }
  }
  long long wcol = 0;  // the largest face's columns
  for (int dir = 0; dir < 3; ++dir)
    wcol = std::max<long long>(wcol, (long long)((dir == 0 ? d.jmx : d.imx) - 1) *
                                         ((dir == 2 ? d.jmx : d.kmx) - 1));
  if (sst) {
    // mu_t, F1 copies of ghost cells -> the interior cells' own; then every
    // cell whose mu_t and F1 come from its own state (with its source);
    // ghost gradients -> interior gradients; Green-Gauss -> the state
    k_vjp_mut_ghost<<<dim3(nblocks(wcol), 1, 6), TPB_ADJ, 0, L.s>>>(p, barMut, barF1);
    k_vjp_sst_cell<<<nblocks(ngrad(d)), TPB_ADJ, 0, L.s>>>(p, b, lam, bar, barG, barMut, barF1);
    k_vjp_grad_bc<<<dim3(nblocks(wcol), 1, 6), TPB_ADJ, 0, L.s>>>(p, b, barG, bar);
    k_vjp_grad_sst<<<nblocks(ncells(d)), TPB_ADJ, 0, L.s>>>(p, b, barG, bar);
    *L.count += 4;
  } else if (visc) {
    const bool geo = bar_cells && bar_faces;
    k_vjp_grad<<<nblocks(ncells(d)), TPB_ADJ, 0, L.s>>>(p, b, bar_grad, bar, geo ? bar_faces[0] : nullptr,
                                                        geo ? bar_faces[1] : nullptr,
                                                        geo ? bar_faces[2] : nullptr, bar_cells);
    ++*L.count;
  }
  long long wmax = 0;
  for (int dir = 0; dir < 3; ++dir)
    wmax = std::max<long long>(wmax, (long long)((dir == 0 ? d.jmx : d.imx) - 1) *
                                         ((dir == 2 ? d.jmx : d.kmx) - 1));
  k_vjp_ghosts<double><<<dim3(nblocks(wmax), 1, 6), TPB_ADJ, 0, L.s>>>(
      p, b, bar, iter, bar_faces ? bar_faces[0] : nullptr, bar_faces ? bar_faces[1] : nullptr,
      bar_faces ? bar_faces[2] : nullptr);
  ++*L.count;
}

namespace {

__device__ __forceinline__ long long node_i(const Dims& d, int i, int j, int k) {
  return 3 * (((long long)(k + 2) * (d.jmx + 6) + (j + 2)) * (d.imx + 6) + (i + 2));
}

// transpose of the face records {A, n} = {|S|, S/|S|}, S = (d1 x d2)/2 with
// the diagonals of the face (geometry.f90, as k_face_vectors)
__global__ void k_vjp_face_vectors(Dims d, const double* nd, const double* faces, const double* bar_face,
                                   double* bar_nodes, int dir) {
  const int ni = d.imx + 5 + (dir == 0), nj = d.jmx + 5 + (dir == 1), nk = d.kmx + 5 + (dir == 2);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * nk) return;
  const int i = -2 + (int)(t % ni);
  const long long r = t / ni;
  const int j = -2 + (int)(r % nj), k = -2 + (int)(r / nj);
  const long long fi = fidx(d, dir, i, j, k);
  const double* g = bar_face + 4 * fi;
  if (g[0] == 0.0 && g[1] == 0.0 && g[2] == 0.0 && g[3] == 0.0) return;
  long long a1, a0, b1, b0;
  if (dir == 0) { a1 = node_i(d, i, j + 1, k + 1); a0 = node_i(d, i, j, k); b1 = node_i(d, i, j, k + 1); b0 = node_i(d, i, j + 1, k); }
  else if (dir == 1) { a1 = node_i(d, i + 1, j, k + 1); a0 = node_i(d, i, j, k); b1 = node_i(d, i + 1, j, k); b0 = node_i(d, i, j, k + 1); }
  else { a1 = node_i(d, i + 1, j + 1, k); a0 = node_i(d, i, j, k); b1 = node_i(d, i, j + 1, k); b0 = node_i(d, i + 1, j, k); }
  double d1[3], d2[3];
  for (int c = 0; c < 3; ++c) { d1[c] = nd[a1 + c] - nd[a0 + c]; d2[c] = nd[b1 + c] - nd[b0 + c]; }
  const double* f = faces + 4 * fi;
  const double A = f[0], n[3] = {f[1], f[2], f[3]};
  if (A == 0.0) return;
  // S-bar = A-bar n + (n-bar - n (n . n-bar)) / A
  const double ndot = n[0] * g[1] + n[1] * g[2] + n[2] * g[3];
  double sb[3];
  for (int c = 0; c < 3; ++c) sb[c] = g[0] * n[c] + (g[1 + c] - n[c] * ndot) / A;
  // S = (d1 x d2)/2: d1-bar = (d2 x S-bar)/2, d2-bar = (S-bar x d1)/2
  const double d1b[3] = {0.5 * (d2[1] * sb[2] - d2[2] * sb[1]), 0.5 * (d2[2] * sb[0] - d2[0] * sb[2]),
                         0.5 * (d2[0] * sb[1] - d2[1] * sb[0])};
  const double d2b[3] = {0.5 * (sb[1] * d1[2] - sb[2] * d1[1]), 0.5 * (sb[2] * d1[0] - sb[0] * d1[2]),
                         0.5 * (sb[0] * d1[1] - sb[1] * d1[0])};
  for (int c = 0; c < 3; ++c) {
    atomicAdd(bar_nodes + a1 + c, d1b[c]);
    atomicAdd(bar_nodes + a0 + c, -d1b[c]);
    atomicAdd(bar_nodes + b1 + c, d2b[c]);
    atomicAdd(bar_nodes + b0 + c, -d2b[c]);
  }
}

// transpose of the cell records {volume, cx, cy, cz} (geometry.f90, as
// k_cells): the centre is the mean of the eight nodes; the volume, for the
// cells of the range 0..imx, 0..jmx, 0..kmx, the larger of two sums of five
// tetrahedra, each -(a x b).c/6 with a, b, c its edges from its first
// node, whose derivatives are -(b x c)/6, -(c x a)/6, -(a x b)/6 for the
// other three nodes and minus their sum for the first
__device__ __forceinline__ void tet_vol_grad(const double* p1, const double* p2, const double* p3,
                                             const double* p4, double bv, double* g1, double* g2,
                                             double* g3, double* g4) {
  double a[3], b[3], c[3];
  for (int m = 0; m < 3; ++m) {
    a[m] = p2[m] - p1[m];
    b[m] = p3[m] - p1[m];
    c[m] = p4[m] - p1[m];
  }
  const double s = -bv / 6.0;
  const double ga[3] = {s * (b[1] * c[2] - b[2] * c[1]), s * (b[2] * c[0] - b[0] * c[2]),
                        s * (b[0] * c[1] - b[1] * c[0])};
  const double gb[3] = {s * (c[1] * a[2] - c[2] * a[1]), s * (c[2] * a[0] - c[0] * a[2]),
                        s * (c[0] * a[1] - c[1] * a[0])};
  const double gc[3] = {s * (a[1] * b[2] - a[2] * b[1]), s * (a[2] * b[0] - a[0] * b[2]),
                        s * (a[0] * b[1] - a[1] * b[0])};
  for (int m = 0; m < 3; ++m) {
    g2[m] += ga[m];
    g3[m] += gb[m];
    g4[m] += gc[m];
    g1[m] -= ga[m] + gb[m] + gc[m];
  }
}
__device__ __forceinline__ double tet_vol(const double* p1, const double* p2, const double* p3,
                                          const double* p4) {
  const double v = (p4[0] - p1[0]) * ((p2[1] - p1[1]) * (p3[2] - p1[2]) - (p2[2] - p1[2]) * (p3[1] - p1[1])) +
                   (p4[1] - p1[1]) * ((p2[2] - p1[2]) * (p3[0] - p1[0]) - (p2[0] - p1[0]) * (p3[2] - p1[2])) +
                   (p4[2] - p1[2]) * ((p2[0] - p1[0]) * (p3[1] - p1[1]) - (p2[1] - p1[1]) * (p3[0] - p1[0]));
  return -v / 6.;
}
__global__ void k_vjp_cells(Dims d, const double* nd, const double* bar_cells, double* bar_nodes) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.P) return;
  const int i = -2 + (int)(t % d.ni);
  const long long r = t / d.ni;
  const int j = -2 + (int)(r % d.nj), k = -2 + (int)(r / d.nj);
  const double* bc = bar_cells + 4 * pidx(d, i, j, k);
  if (bc[0] == 0.0 && bc[1] == 0.0 && bc[2] == 0.0 && bc[3] == 0.0) return;
  const long long ni[8] = {node_i(d, i, j, k),         node_i(d, i + 1, j, k),
                           node_i(d, i + 1, j + 1, k), node_i(d, i, j + 1, k),
                           node_i(d, i, j, k + 1),     node_i(d, i + 1, j, k + 1),
                           node_i(d, i + 1, j + 1, k + 1), node_i(d, i, j + 1, k + 1)};
  double g[8][3];
  for (int n = 0; n < 8; ++n)
    for (int m = 0; m < 3; ++m) g[n][m] = 0.125 * bc[1 + m];
  if (bc[0] != 0.0 && i >= 0 && i <= d.imx && j >= 0 && j <= d.jmx && k >= 0 && k <= d.kmx) {
    const double* P[8];
    for (int n = 0; n < 8; ++n) P[n] = nd + ni[n];
    // the two five-tetrahedron sums of k_cells, in its order
    const int T1[5][4] = {{0, 4, 7, 5}, {6, 7, 5, 2}, {7, 3, 0, 2}, {5, 0, 2, 7}, {0, 1, 5, 2}};
    const int T2[5][4] = {{1, 5, 4, 6}, {7, 4, 6, 3}, {4, 0, 1, 3}, {6, 1, 3, 4}, {1, 2, 6, 3}};
    double v1 = 0., v = 0.;
    for (int m = 0; m < 5; ++m) v1 = v1 + tet_vol(P[T1[m][0]], P[T1[m][1]], P[T1[m][2]], P[T1[m][3]]);
    for (int m = 0; m < 5; ++m) v = v + tet_vol(P[T2[m][0]], P[T2[m][1]], P[T2[m][2]], P[T2[m][3]]);
    // vol = fmax2(v, v1) = (v > v1 ? v : v1): the derivative of the sum it took
    const int(*T)[4] = v > v1 ? T2 : T1;
    for (int m = 0; m < 5; ++m)
      tet_vol_grad(P[T[m][0]], P[T[m][1]], P[T[m][2]], P[T[m][3]], bc[0], g[T[m][0]], g[T[m][1]],
                   g[T[m][2]], g[T[m][3]]);
  }
  for (int n = 0; n < 8; ++n)
    for (int m = 0; m < 3; ++m)
      if (g[n][m] != 0.0) atomicAdd(bar_nodes + ni[n] + m, g[n][m]);
}

// transpose of the ghost-node extrapolation of direction dir (grid.f90,
// as k_ghost_nodes): its statements in reverse order
__global__ void k_vjp_ghost_nodes(Dims d, double* bn, int dir) {
  const int n0 = (dir == 0 ? d.jmx : d.imx) + 6, n1 = (dir == 2 ? d.jmx : d.kmx) + 6;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n0 * n1) return;
  const int a = -2 + (int)(t % n0), b = -2 + (int)(t / n0);
  const int n = extent_of(d, dir);
  auto N = [&](int c) -> double* {
    return bn + (dir == 0 ? node_i(d, c, a, b) : dir == 1 ? node_i(d, a, c, b) : node_i(d, a, b, c));
  };
  for (int c = 0; c < 3; ++c) {
    // N(m) = 2 N(m-1) - N(m-2) etc., undone last statement first
    auto back = [&](int dst, int s1, int s2) {  // N(dst) = 2 N(s1) - N(s2)
      const double g = N(dst)[c];
      N(dst)[c] = 0.0;
      N(s1)[c] += 2.0 * g;
      N(s2)[c] -= g;
    };
    back(n + 3, n + 2, n + 1);
    back(n + 2, n + 1, n);
    back(n + 1, n, n - 1);
    back(-2, -1, 0);
    back(-1, 0, 1);
    back(0, 1, 2);
  }
}

}  // namespace

void launch_geometry_vjp(const Params& p, const DevBlock& b, double* const* bar_faces, double* bar_nodes,
                         const Launcher& L, const double* bar_cells) {
  const Dims& d = p.d;
  cudaMemsetAsync(bar_nodes, 0, sizeof(double) * 3 * (size_t)(d.imx + 6) * (d.jmx + 6) * (d.kmx + 6), L.s);
  for (int dir = 0; dir < 3; ++dir) {
    const long long nf = (long long)(d.imx + 5 + (dir == 0)) * (d.jmx + 5 + (dir == 1)) * (d.kmx + 5 + (dir == 2));
    k_vjp_face_vectors<<<nblocks(nf), TPB_ADJ, 0, L.s>>>(d, b.nodes, b.faces[dir], bar_faces[dir], bar_nodes, dir);
    ++*L.count;
  }
  if (bar_cells) {
    k_vjp_cells<<<nblocks(d.P), TPB_ADJ, 0, L.s>>>(d, b.nodes, bar_cells, bar_nodes);
    ++*L.count;
  }
  for (int dir = 2; dir >= 0; --dir) {
    const long long n = (long long)((dir == 0 ? d.jmx : d.imx) + 6) * ((dir == 2 ? d.jmx : d.kmx) + 6);
    k_vjp_ghost_nodes<<<nblocks(n), TPB_ADJ, 0, L.s>>>(d, bar_nodes, dir);
    ++*L.count;
  }
}

}  // namespace fest
