// fest_lusgs.cu - the implicit integrators of the reference: one residual,
// the local time step, then update_with_lusgs (update.f90:215-218,
// lusgs.f90:134-1196) or its low-Mach preconditioned form
// update_with_plusgs (update.f90:219-222, plusgs.f90:139-1431), for laminar
// and k-omega SST blocks, FP64; both also for SST blocks with LCTM2015's
// intermittency (update_lctm2015, lusgs.f90:2263-2700, plusgs.f90:2130-2624).
//
// The reference sweeps the interior cells forward (i fastest, then j, k)
// computing dQ* from the dQ* of each cell's three lower neighbours, then
// backward computing dQ from the dQ of the three upper neighbours.  A cell
// of hyperplane i+j+k = s depends only on cells of plane s-1 (forward) or
// s+1 (backward), so each plane is one launch over all its cells, with the
// per-cell arithmetic of the reference; the result is the sequential
// sweep's.  What does not depend on the sweep (the six faces' spectral
// radii, the diagonal and the fluxes of the unchanged neighbour states) is
// computed for every cell in one launch before the sweeps.
#include "fest_kernels.cuh"

namespace fest {
namespace {

constexpr double kSigK1 = 0.85, kSigK2 = 1.0, kSigW1 = 0.5, kSigW2 = 0.856, kBeta1 = 0.075, kBeta2 = 0.0828,
                 kBstar = 0.09;

// one face seen from the cell being updated: area, outward normal, and the
// means over the two cells of volume, laminar and eddy viscosity and the SST
// blending F1 (lusgs.f90:278-324, 783-835)
struct LuFace {
  double A, nx, ny, nz, vol, mu, mut, F1;
};

// lusgs.f90:491-630 Flux and 1027-1196 SSTFlux: the inviscid flux of the
// neighbour state ql advanced by the conservative change du (k and omega kept
// at ql's values where the advanced ones turn negative), less the thin-layer
// viscous flux between that state and the cell state qr, times the area
template <int N>
__device__ void lu_flux(const Params& p, const double* ql, const double* qr, const double* du, const LuFace& f,
                        double* out) {
  const double gm = p.gm, R = p.R;
  double U[N], W[N];
  U[0] = ql[0];
  U[1] = ql[0] * ql[1];
  U[2] = ql[0] * ql[2];
  U[3] = ql[0] * ql[3];
  U[4] = (ql[4] / (gm - 1.0)) + (0.5 * ql[0] * (ql[1] * ql[1] + ql[2] * ql[2] + ql[3] * ql[3]));
#pragma unroll
  for (int l = 5; l < N; ++l) U[l] = ql[0] * ql[l];
#pragma unroll
  for (int l = 0; l < N; ++l) U[l] = U[l] + du[l];
  W[0] = U[0];
  W[1] = U[1] / U[0];
  W[2] = U[2] / U[0];
  W[3] = U[3] / U[0];
  W[4] = (gm - 1.0) * (U[4] - (0.5 * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / U[0]));
#pragma unroll
  for (int l = 5; l < N; ++l) {
    W[l] = U[l] / U[0];
    if (l < 7) W[l] = W[l] + 0.5 * (1. - copysign(1., W[l])) * (ql[l] - W[l]);
    else W[l] = fmax2(W[l], 0.0);  // the intermittency (lusgs.f90:2783)
  }
  const double nx = f.nx, ny = f.ny, nz = f.nz;
  const double vn = (W[1] * nx) + (W[2] * ny) + (W[3] * nz);
  const double uf = 0.5 * (W[1] + qr[1]), vf = 0.5 * (W[2] + qr[2]), wf = 0.5 * (W[3] + qr[3]);
  out[0] = W[0] * vn;
  out[1] = (W[1] * out[0]) + (W[4] * nx);
  out[2] = (W[2] * out[0]) + (W[4] * ny);
  out[3] = (W[3] * out[0]) + (W[4] * nz);
  const double half_rho_u2 = 0.5 * W[0] * (W[1] * W[1] + W[2] * W[2] + W[3] * W[3]);
  out[4] = (((gm / (gm - 1.0)) * W[4]) + half_rho_u2) * vn;
#pragma unroll
  for (int l = 5; l < N; ++l) out[l] = W[l] * out[0];
  // differences across the face as the only gradient
  const double mu = f.mu + f.mut, s = f.A;
  const double T1 = W[4] / (W[0] * R), T2 = qr[4] / (qr[0] * R);
  const double dT[3] = {(T2 - T1) * nx * s / f.vol, (T2 - T1) * ny * s / f.vol, (T2 - T1) * nz * s / f.vol};
  double g[N - 2][3];  // d(u, v, w[, k, omega])/d(x_d)
#pragma unroll
  for (int c = 0; c < N - 2; ++c) {
    const int v = c < 3 ? 1 + c : 2 + c;
    const double dv = qr[v] - W[v];
    g[c][0] = dv * nx * s / f.vol;
    g[c][1] = dv * ny * s / f.vol;
    g[c][2] = dv * nz * s / f.vol;
  }
  const double tr = g[0][0] + g[1][1] + g[2][2];
  const double txx = 2. * mu * (g[0][0] - tr / 3.0), tyy = 2. * mu * (g[1][1] - tr / 3.0),
               tzz = 2. * mu * (g[2][2] - tr / 3.0);
  const double txy = mu * (g[1][0] + g[0][1]), txz = mu * (g[2][0] + g[0][2]), tyz = mu * (g[2][1] + g[1][2]);
  const double kh = (f.mu / p.Pr + f.mut / p.tPr) * gm * R / (gm - 1.0);
  out[1] = out[1] - (txx * nx + txy * ny + txz * nz);
  out[2] = out[2] - (txy * nx + tyy * ny + tyz * nz);
  out[3] = out[3] - (txz * nx + tyz * ny + tzz * nz);
  out[4] = out[4] - (txx * uf + txy * vf + txz * wf + kh * dT[0]) * nx;
  out[4] = out[4] - (txy * uf + tyy * vf + tyz * wf + kh * dT[1]) * ny;
  out[4] = out[4] - (txz * uf + tyz * vf + tzz * wf + kh * dT[2]) * nz;
  if constexpr (N == 7) {
    const double sk = kSigK1 * f.F1 + kSigK2 * (1.0 - f.F1), sw = kSigW1 * f.F1 + kSigW2 * (1.0 - f.F1);
    // added, as lusgs.f90:1190-1191 has it
    out[5] = out[5] + (f.mu + sk * f.mut) * (g[3][0] * nx + g[3][1] * ny + g[3][2] * nz);
    out[6] = out[6] + (f.mu + sw * f.mut) * (g[4][0] * nx + g[4][1] * ny + g[4][2] * nz);
  }
  if constexpr (N == 8) {  // lctm2015Flux (lusgs.f90:2845-2851)
    const double sk = kSigK1 * f.F1 + kSigK2 * (1.0 - f.F1), sw = kSigW1 * f.F1 + kSigW2 * (1.0 - f.F1);
    out[5] = out[5] + (f.mu + sk * f.mut) * (g[3][0] * nx + g[3][1] * ny + g[3][2] * nz);
    out[6] = out[6] + (f.mu + sw * f.mut) * (g[4][0] * nx + g[4][1] * ny + g[4][2] * nz);
    out[7] = out[7] + (f.mu + f.mut) * (g[5][0] * nx + g[5][1] * ny + g[5][2] * nz);
  }
#pragma unroll
  for (int l = 0; l < N; ++l) out[l] = out[l] * s;
}

// lusgs.f90:633-683 SpectralRadius: convective plus viscous spectral radius
// of the face, times its area; ca, cb the two cell records {vol, centre}
__device__ double lu_radius(const Params& p, const double* qa, const double* qb, const LuFace& f, const double* ca,
                            const double* cb) {
  const double gm = p.gm;
  const double vn = fabs(0.5 * (((qa[1] + qb[1]) * f.nx) + ((qa[2] + qb[2]) * f.ny) + ((qa[3] + qb[3]) * f.nz)));
  const double c = 0.5 * (sqrt(gm * qa[4] / qa[0]) + sqrt(gm * qb[4] / qb[0]));
  const double rho = 0.5 * (qa[0] + qb[0]);
  const double dx = ca[1] - cb[1], dy = ca[2] - cb[2], dz = ca[3] - cb[3];
  const double dist = sqrt(dx * dx + dy * dy + dz * dz);
  const double vis = gm * (f.mu / p.Pr + f.mut / p.tPr) / (rho * dist);
  return (vn + c + vis) * f.A;
}

// plusgs.f90:723-776 SpectralRadius of the preconditioned system: eps is
// the cell's own min(1, max(M^2, Minf^2)), the viscous part twice LU-SGS's
__device__ double plu_radius(const Params& p, const double* qa, const double* qb, const LuFace& f,
                             const double* ca, const double* cb, double eps) {
  const double gm = p.gm;
  const double vn = fabs(0.5 * (((qa[1] + qb[1]) * f.nx) + ((qa[2] + qb[2]) * f.ny) + ((qa[3] + qb[3]) * f.nz)));
  const double c = 0.5 * (sqrt(gm * qa[4] / qa[0]) + sqrt(gm * qb[4] / qb[0]));
  const double rho = 0.5 * (qa[0] + qb[0]);
  const double dx = ca[1] - cb[1], dy = ca[2] - cb[2], dz = ca[3] - cb[3];
  const double dist = sqrt(dx * dx + dy * dy + dz * dz);
  const double vis = 2.0 * gm * (f.mu / p.Pr + f.mut / p.tPr) / (rho * dist);
  return (0.5 * ((1.0 + eps) * vn + sqrt(((eps - 1.0) * (eps - 1.0)) * (vn * vn) + 4 * eps * (c * c))) + vis) * f.A;
}

// plusgs.f90:345-396 and 944-1014: the cell's inverse preconditioner
// P = I - (factor x) c^T with x = (1, u, v, w, H[, k, omega]) and
// c = (|V|^2/2, -u, -v, -w, 1[, -1, 0]); H as the reference has it, with
// 0.5 |V| (not |V|^2)
template <int N>
struct PluP {
  double fx[N], u, v, w, VMag, eps;
  __device__ PluP(const Params& p, const double* q0) {
    const double gm = p.gm, r = q0[0], pr = q0[4];
    u = q0[1];
    v = q0[2];
    w = q0[3];
    VMag = sqrt(u * u + v * v + w * w);
    const double SoundMag = sqrt(gm * pr / r);
    const double M = VMag / SoundMag;
    const double H = (gm * pr / (r * (gm - 1.0))) + 0.5 * (VMag);
    eps = fmin(1.0, fmax(M * M, p.MInf * p.MInf));
    const double factor = (1.0 - eps) * (gm - 1.0) / (SoundMag * SoundMag);
    // plusgs.f90:2338-2355 adds the intermittency to x and a zero to c
    const double x[8] = {1.0, u, v, w, H, N >= 7 ? q0[5 % N] : 0.0, N >= 7 ? q0[6 % N] : 0.0,
                         N == 8 ? q0[7 % N] : 0.0};
#pragma unroll
    for (int i = 0; i < N; ++i) fx[i] = factor * x[i];
  }
  // out = P y, each entry summed over the columns in order
  __device__ void apply(const double* y, double* out) const {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      double s = ((i == 0 ? 1.0 : 0.0) - fx[i] * VMag * VMag / 2.0) * y[0];
      s = s + ((i == 1 ? 1.0 : 0.0) - fx[i] * (-u)) * y[1];
      s = s + ((i == 2 ? 1.0 : 0.0) - fx[i] * (-v)) * y[2];
      s = s + ((i == 3 ? 1.0 : 0.0) - fx[i] * (-w)) * y[3];
      s = s + ((i == 4 ? 1.0 : 0.0) - fx[i] * (1.)) * y[4];
      if constexpr (N >= 7) {
        s = s + ((i == 5 ? 1.0 : 0.0) - fx[i] * (-1.)) * y[5];
        s = s + ((i == 6 ? 1.0 : 0.0) - fx[i] * (0.)) * y[6];
      }
      if constexpr (N == 8) s = s + ((i == 7 ? 1.0 : 0.0) - fx[i] * (0.)) * y[7];
      out[i] = s;
    }
  }
};

struct LuDev {
  double *lam, *D, *Fold;  // per interior cell: 6, n and 6n values
  double *dqs, *dq;        // (0:imx, 0:jmx, 0:kmx, n), zero outside the interior
};

// face s (0..2 low i/j/k, 3..5 high) of cell (i, j, k): the record and the
// neighbour's index
__device__ void lu_face(const Params& p, const DevBlock& b, int i, int j, int k, int s, LuFace& fc, long long& nb) {
  const Dims& d = p.d;
  const int dir = s % 3, hi = s / 3;
  const int oi = dir == 0, oj = dir == 1, ok = dir == 2;
  const int ni = i + (hi ? oi : -oi), nj = j + (hi ? oj : -oj), nk = k + (hi ? ok : -ok);
  const double* f = b.faces[dir] + 4 * fidx(d, dir, i + hi * oi, j + hi * oj, k + hi * ok);
  const double sg = hi ? 1.0 : -1.0;
  const long long c0 = pidx(d, i, j, k);
  nb = pidx(d, ni, nj, nk);
  fc.A = f[0];
  fc.nx = sg * f[1];
  fc.ny = sg * f[2];
  fc.nz = sg * f[3];
  fc.vol = 0.5 * (b.cells[4 * nb] + b.cells[4 * c0]);
  fc.mu = 0.5 * (b.mu[nb] + b.mu[c0]);
  const bool sst = p.turb != FEST_TURB_NONE;
  fc.mut = sst ? 0.5 * (b.mut[nb] + b.mut[c0]) : 0.0;
  fc.F1 = sst ? 0.5 * (b.F1[nb] + b.F1[c0]) : 0.0;
}

__device__ __forceinline__ long long lu_idx(const Dims& d, int i, int j, int k) {
  return ((long long)k * (d.jmx + 1) + j) * (d.imx + 1) + i;
}
__host__ __device__ __forceinline__ long long lu_count(const Dims& d) {
  return (long long)(d.imx + 1) * (d.jmx + 1) * (d.kmx + 1);
}

// everything of a cell that the sweeps do not change
template <int N, bool PLUS>
__global__ void k_lu_prep(Params p, DevBlock b, LuDev u) {
  const Dims& d = p.d;
  const long long nc = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int i = 1 + (int)(t % (d.imx - 1)), j = 1 + (int)((t / (d.imx - 1)) % (d.jmx - 1)),
            k = 1 + (int)(t / ((long long)(d.imx - 1) * (d.jmx - 1)));
  const long long c0 = pidx(d, i, j, k);
  double q0[N];
#pragma unroll
  for (int l = 0; l < N; ++l) q0[l] = b.qp[c0 + d.P * l];
  double sumlam = 0.0, lam[6], eps = 0.0;
  if constexpr (PLUS) eps = PluP<N>(p, q0).eps;
  for (int s = 0; s < 6; ++s) {
    LuFace fc;
    long long nb;
    lu_face(p, b, i, j, k, s, fc, nb);
    double qn[N], zero[N], F[N];
#pragma unroll
    for (int l = 0; l < N; ++l) {
      qn[l] = b.qp[nb + d.P * l];
      zero[l] = 0.0;
    }
    if constexpr (PLUS)
      lam[s] = plu_radius(p, qn, q0, fc, b.cells + 4 * nb, b.cells + 4 * c0, eps);
    else
      lam[s] = lu_radius(p, qn, q0, fc, b.cells + 4 * nb, b.cells + 4 * c0);
    lu_flux<N>(p, qn, q0, zero, fc, F);
#pragma unroll
    for (int l = 0; l < N; ++l) u.Fold[t + nc * (s * N + l)] = F[l];
    u.lam[t + nc * s] = lam[s];
  }
  for (int s = 0; s < 6; ++s) sumlam = sumlam + lam[s];
  const double vol = b.cells[4 * c0];
  double D[N];
#pragma unroll
  for (int l = 0; l < N; ++l) D[l] = (vol / b.dt[t]) + 0.5 * sumlam;
  if constexpr (N >= 7) {  // lusgs.f90:860-862, 2439-2441: the destruction terms of k and omega
    const double f1 = b.F1[c0], beta = f1 * kBeta1 + (1.0 - f1) * kBeta2, w = q0[6];
    D[5] = (D[5] + (kBstar * w) * vol);
    D[6] = (D[6] + 2.0 * beta * w * vol);
  }
  if constexpr (N == 8) {  // lusgs.f90:2443-2475: the intermittency's source, linearised
    double vort, strain;
    lctm_vort_strain(b, gidx(d, i, j, k), ngrad(d), vort, strain);
    const double density = q0[0], dd = b.dist[c0], m = b.mu[c0];
    const double TuL = fmin2(100.0 * sqrt(2.0 * q0[5] / 3.0) / (q0[6] * dd), 100.0);
    const double Re_theta = 100.0 + 1000.0 * exp(-TuL);
    const double Rev = density * dd * dd * strain / m;
    const double RT = density * q0[5] / (m * q0[6]);
    double Fturb, Fonset;
    lctm_onset(Rev, RT, Re_theta, Fturb, Fonset);
    const double Dp = 100 * density * strain * Fonset * (1.0 - 2.0 * q0[7]);
    const double De = 0.06 * vort * Fturb * density * (2.0 * 50.0 * q0[7] - 1.0);
    D[7] = (D[7] + (-Dp + De) * vol);
  }
#pragma unroll
  for (int l = 0; l < N; ++l) u.D[t + nc * l] = D[l];
}

// the cells of hyperplane i+j+k = s: one thread per (j, k), i = s - j - k;
// pass 0 the forward sweep (dQ*), pass 1 the backward one (dQ)
template <int N, bool PLUS>
__global__ void k_lu_plane(Params p, DevBlock b, LuDev u, int pass, int s) {
  const Dims& d = p.d;
  const int nj = d.jmx - 1, nk = d.kmx - 1;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nj * nk) return;
  const int j = 1 + t % nj, k = 1 + t / nj, i = s - j - k;
  if (i < 1 || i > d.imx - 1) return;
  const long long nc = ncells(d), c = cidx(d, i, j, k), c0 = pidx(d, i, j, k), L = lu_count(d);
  double q0[N], acc[N];
#pragma unroll
  for (int l = 0; l < N; ++l) {
    q0[l] = b.qp[c0 + d.P * l];
    acc[l] = 0.0;
  }
  const double* src = pass == 0 ? u.dqs : u.dq;
  for (int dir = 0; dir < 3; ++dir) {
    const int sface = pass == 0 ? dir : 3 + dir;
    LuFace fc;
    long long nb;
    lu_face(p, b, i, j, k, sface, fc, nb);
    const int step = pass ? 1 : -1;
    const int ni = i + (dir == 0 ? step : 0), nj2 = j + (dir == 1 ? step : 0), nk2 = k + (dir == 2 ? step : 0);
    double qn[N], dn[N], fnew[N];
#pragma unroll
    for (int l = 0; l < N; ++l) {
      qn[l] = b.qp[nb + d.P * l];
      dn[l] = src[lu_idx(d, ni, nj2, nk2) + L * l];
    }
    lu_flux<N>(p, qn, q0, dn, fc, fnew);
    const double lam = u.lam[c + nc * sface];
#pragma unroll
    for (int l = 0; l < N; ++l) fnew[l] = fnew[l] - u.Fold[c + nc * (sface * N + l)];
    if constexpr (PLUS) {
      double pf[N];
      PluP<N>(p, q0).apply(fnew, pf);
#pragma unroll
      for (int l = 0; l < N; ++l) fnew[l] = pf[l];
    }
#pragma unroll
    for (int l = 0; l < N; ++l) acc[l] = acc[l] + (fnew[l] - lam * dn[l]);
  }
  double rr[N];
#pragma unroll
  for (int l = 0; l < N; ++l) rr[l] = b.res[c + nc * l];
  if constexpr (PLUS) {
    if (pass == 0) {
      double pr[N];
      PluP<N>(p, q0).apply(rr, pr);
#pragma unroll
      for (int l = 0; l < N; ++l) rr[l] = pr[l];
    }
  }
  const long long o = lu_idx(d, i, j, k);
#pragma unroll
  for (int l = 0; l < N; ++l) {
    const double D = u.D[c + nc * l];
    if (pass == 0)
      u.dqs[o + L * l] = (-rr[l] - 0.5 * acc[l]) / D;
    else
      u.dq[o + L * l] = u.dqs[o + L * l] - 0.5 * acc[l] / D;
  }
}

// U += dQ on the interior cells, back to primitive variables; k and omega
// only where they stay positive (lusgs.f90:455-486, 990-1022)
template <int N>
__global__ void k_lu_apply(Params p, DevBlock b, LuDev u) {
  const Dims& d = p.d;
  const long long nc = ncells(d);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nc) return;
  const int i = 1 + (int)(t % (d.imx - 1)), j = 1 + (int)((t / (d.imx - 1)) % (d.jmx - 1)),
            k = 1 + (int)(t / ((long long)(d.imx - 1) * (d.jmx - 1)));
  const long long c0 = pidx(d, i, j, k), o = lu_idx(d, i, j, k), L = lu_count(d), P = d.P;
  const double gm = p.gm;
  double q[N], U[N];
#pragma unroll
  for (int l = 0; l < N; ++l) q[l] = b.qp[c0 + P * l];
  U[0] = q[0];
  U[1] = q[0] * q[1];
  U[2] = q[0] * q[2];
  U[3] = q[0] * q[3];
  U[4] = (q[4] / (gm - 1.0)) + (0.5 * q[0] * (q[1] * q[1] + q[2] * q[2] + q[3] * q[3]));
#pragma unroll
  for (int l = 5; l < N; ++l) U[l] = q[0] * q[l];
#pragma unroll
  for (int l = 0; l < N; ++l) U[l] = U[l] + u.dq[o + L * l];
  q[0] = U[0];
  q[1] = U[1] / U[0];
  q[2] = U[2] / U[0];
  q[3] = U[3] / U[0];
  q[4] = (gm - 1.0) * (U[4] - (0.5 * (U[1] * U[1] + U[2] * U[2] + U[3] * U[3]) / U[0]));
#pragma unroll
  for (int l = 0; l < 5; ++l) b.qp[c0 + P * l] = q[l];
#pragma unroll
  for (int l = 5; l < N && l < 7; ++l)
    if (U[l] > 0) b.qp[c0 + P * l] = U[l] / U[0];
  if constexpr (N == 8) b.qp[c0 + P * 7] = fmax2(U[7] / U[0], 0.0);  // lusgs.f90:2685-2687
  // a NaN or negative density/pressure (the reference carries it on; the
  // library reports it as update_with does, update.f90:448)
  if (!(q[0] >= 0.0) || !(q[4] >= 0.0)) raise_error(b.err, FEST_ERR_NEGATIVE_STATE);
}

template <int N, bool PLUS>
void lusgs_t(const Params& p, const DevBlock& b, const LuDev& u, const Launcher& L) {
  const Dims& d = p.d;
  const long long nc = ncells(d);
  const unsigned g = (unsigned)((nc + 127) / 128);
  k_lu_prep<N, PLUS><<<g, 128, 0, L.s>>>(p, b, u);
  ++*L.count;
  // dQ* and dQ are zero outside the interior (the layer the sweeps read)
  const size_t bytes = sizeof(double) * (size_t)lu_count(d) * N;
  cudaMemsetAsync(u.dqs, 0, bytes, L.s);
  cudaMemsetAsync(u.dq, 0, bytes, L.s);
  const int nt = (d.jmx - 1) * (d.kmx - 1);
  const unsigned gp = (unsigned)((nt + 63) / 64);  // small CTAs: a plane spreads over the SMs
  const int smax = (d.imx - 1) + (d.jmx - 1) + (d.kmx - 1);
  for (int s = 3; s <= smax; ++s) {
    k_lu_plane<N, PLUS><<<gp, 64, 0, L.s>>>(p, b, u, 0, s);
    ++*L.count;
  }
  for (int s = smax; s >= 3; --s) {
    k_lu_plane<N, PLUS><<<gp, 64, 0, L.s>>>(p, b, u, 1, s);
    ++*L.count;
  }
  k_lu_apply<N><<<g, 128, 0, L.s>>>(p, b, u);
  ++*L.count;
}

}  // namespace

long long lusgs_scratch_doubles(const Dims& d) {
  return ncells(d) * (6 + 7 * (long long)d.nv) + 2 * lu_count(d) * d.nv;
}

void launch_lusgs(const Params& p, const DevBlock& b, double* scratch, const Launcher& L) {
  const Dims& d = p.d;
  const long long nc = ncells(d);
  LuDev u;
  u.lam = scratch;
  u.D = u.lam + 6 * nc;
  u.Fold = u.D + d.nv * nc;
  u.dqs = u.Fold + 6 * d.nv * nc;
  u.dq = u.dqs + lu_count(d) * d.nv;
  const bool plus = p.integ == FEST_TIME_PLUSGS;
  if (d.nv == 8) plus ? lusgs_t<8, true>(p, b, u, L) : lusgs_t<8, false>(p, b, u, L);
  else if (d.nv == 7) plus ? lusgs_t<7, true>(p, b, u, L) : lusgs_t<7, false>(p, b, u, L);
  else plus ? lusgs_t<5, true>(p, b, u, L) : lusgs_t<5, false>(p, b, u, L);
}

}  // namespace fest
