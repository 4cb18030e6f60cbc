// fest_kernels.cu - FP64 module kernels of FEST-3D's explicit path: one kernel
// per reference procedure, reading and writing the reference's module arrays
// in HBM.  Threads map i fastest so every array access is coalesced.
#include "fest_kernels.cuh"

#include <algorithm>

namespace fest {

namespace {

constexpr int TPB = 256;

struct R3 {
  int lo0, lo1, lo2, n0, n1, n2;
  long long N;
};
__host__ __device__ inline R3 r3(int lo0, int hi0, int lo1, int hi1, int lo2, int hi2) {
  R3 r;
  r.lo0 = lo0; r.lo1 = lo1; r.lo2 = lo2;
  r.n0 = hi0 - lo0 + 1; r.n1 = hi1 - lo1 + 1; r.n2 = hi2 - lo2 + 1;
  if (r.n0 < 0) r.n0 = 0;
  if (r.n1 < 0) r.n1 = 0;
  if (r.n2 < 0) r.n2 = 0;
  r.N = (long long)r.n0 * r.n1 * r.n2;
  return r;
}
__device__ __forceinline__ bool decode(const R3& r, int& i, int& j, int& k) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= r.N) return false;
  i = r.lo0 + (int)(t % r.n0);
  t /= r.n0;
  j = r.lo1 + (int)(t % r.n1);
  k = r.lo2 + (int)(t / r.n1);
  return true;
}
inline unsigned nblk(long long n) { return (unsigned)((n + TPB - 1) / TPB); }

// ghost / interior cell of face f, layer L (tangential ta, tb)
__device__ __forceinline__ long long ghost_p(const Dims& d, int f, int L, int ta, int tb) {
  switch (f) {
    case 0: return pidx(d, 1 - L, ta, tb);
    case 1: return pidx(d, d.imx + L - 1, ta, tb);
    case 2: return pidx(d, ta, 1 - L, tb);
    case 3: return pidx(d, ta, d.jmx + L - 1, tb);
    case 4: return pidx(d, ta, tb, 1 - L);
    default: return pidx(d, ta, tb, d.kmx + L - 1);
  }
}
__device__ __forceinline__ long long inner_p(const Dims& d, int f, int m, int ta, int tb) {
  switch (f) {
    case 0: return pidx(d, m, ta, tb);
    case 1: return pidx(d, d.imx - m, ta, tb);
    case 2: return pidx(d, ta, m, tb);
    case 3: return pidx(d, ta, d.jmx - m, tb);
    case 4: return pidx(d, ta, tb, m);
    default: return pidx(d, ta, tb, d.kmx - m);
  }
}
// boundary face (metric) of face f at tangential (ta, tb), in direction dir arrays
__device__ __forceinline__ void bface_ijk(const Dims& d, int f, int ta, int tb, int& i, int& j,
                                          int& k) {
  int c = (f % 2 == 0) ? 1 : extent_of(d, f / 2);
  if (f / 2 == 0) { i = c; j = ta; k = tb; }
  else if (f / 2 == 1) { i = ta; j = c; k = tb; }
  else { i = ta; j = tb; k = c; }
}

enum { CP_ANTI, CP_FLAT, CP_SYMM };

// copy_bc.f90:58-131 for one column of a face
__device__ void copy3_col(const Params& p, double* q, int f, int ta, int tb, int l, int type) {
  double a1, a2, a3;
  int il0, il1, il2;
  if (type == CP_ANTI) { a1 = 1.; a2 = -1.; a3 = 0.; il0 = 1; il1 = 2; il2 = 3; }
  else if (type == CP_FLAT) { a1 = 1.; a2 = 1.; a3 = 0.; il0 = 1; il1 = 1; il2 = 1; }
  else { a1 = p.c1; a2 = p.c2; a3 = p.c3; il0 = 1; il1 = 2; il2 = 3; }
  const long long o = p.d.P * (l - 1);
  int il[3] = {il0, il1, il2};
  for (int L = 1; L <= 3; ++L) {
    long long g = ghost_p(p.d, f, L, ta, tb);
    long long a = inner_p(p.d, f, il[L - 1], ta, tb), b = inner_p(p.d, f, il[L - 1] + 1, ta, tb);
    q[g + o] = (a2 * q[a + o] - a3 * q[b + o]) / a1;
  }
}
__device__ void fix_col(const Params& p, double* q, int f, int ta, int tb, int l, double v) {
  const long long o = p.d.P * (l - 1);
  for (int L = 1; L <= 3; ++L) q[ghost_p(p.d, f, L, ta, tb) + o] = v;
}

// Riemann invariants on ghost layer 1 (far_field / total_pressure); returns Unb
__device__ double riemann_col(const Params& p, const DevBlock& b, int f, int ta, int tb,
                              bool write, bool total_pressure) {
  const Dims& d = p.d;
  double* q = b.qp;
  const long long P = d.P;
  int fi, fj, fk;
  bface_ijk(d, f, ta, tb, fi, fj, fk);
  const double* fc = b.faces[f / 2] + 4 * fidx(d, f / 2, fi, fj, fk);
  double sg = (f % 2 == 0) ? -1.0 : 1.0;
  double nx = sg * fc[1], ny = sg * fc[2], nz = sg * fc[3];
  long long in = inner_p(d, f, 1, ta, tb), g = ghost_p(d, f, 1, ta, tb);
  double u = q[in + P], v = q[in + 2 * P], w = q[in + 3 * P];
  double pI = q[in + 4 * P], rI = q[in];
  double gm = p.gm;
  double cexp = sqrt(gm * pI / rI);
  double cinf = sqrt(gm * p.p_inf / p.rho_inf);
  double Unexp = u * nx + v * ny + w * nz;
  double Uninf = p.u_inf * nx + p.v_inf * ny + p.w_inf * nz;
  double Rinf = Uninf - 2 * cinf / (gm - 1.);
  double Rexp = Unexp + 2 * cexp / (gm - 1.);
  double Unb = 0.5 * (Rexp + Rinf);
  double Cb = 0.25 * (gm - 1.) * (Rexp - Rinf);
  if (!write) return Unb;
  double ug, vg, wg;
  if (Unb > 0.) {
    double vd = Unb - Unexp;
    ug = u + vd * nx; vg = v + vd * ny; wg = w + vd * nz;
    if (!total_pressure) {
      double s = pI / pow(rI, gm);
      double rg = pow(Cb * Cb / (gm * s), 1. / (gm - 1.));
      q[g] = rg;
      q[g + 4 * P] = (rg * Cb * Cb / gm);
    }
  } else {
    double vd = Unb - Uninf;
    ug = p.u_inf + vd * nx; vg = p.v_inf + vd * ny; wg = p.w_inf + vd * nz;
    if (!total_pressure) {
      double s = p.p_inf / pow(p.rho_inf, gm);
      double rg = pow(Cb * Cb / (gm * s), 1. / (gm - 1.));
      q[g] = rg;
      q[g + 4 * P] = (rg * Cb * Cb / gm);
    }
  }
  q[g + P] = ug; q[g + 2 * P] = vg; q[g + 3 * P] = wg;
  if (total_pressure) {
    double Mb = sqrt(ug * ug + vg * vg + wg * wg) / Cb;
    double pg = p.Tp[f] / pow((1 + 0.5 * (gm - 1.) * Mb * Mb), gm / (gm - 1.));
    q[g + 4 * P] = pg;
    q[g] = gm * pg / (Cb * Cb);
  }
  return Unb;
}

// one column (tangential position) of one face: everything the reference's
// BC procedure for that face does at this position, in its order
__device__ void ghost_column(const Params& p, const DevBlock& b, const BlockRef* blocks, int f,
                             int ta, int tb, int iter) {
  const Dims& d = p.d;
  double* q = b.qp;
  const long long P = d.P;
  const bool sst = p.turb == FEST_TURB_SST || p.turb == FEST_TURB_SST2003;
  const bool sa = p.turb == FEST_TURB_SA;  // tv: the sixth variable, treated as k is
  const bool kkl = p.turb == FEST_TURB_KKL;  // k and kL, treated as k is
  // LCTM2015's intermittency: fixed where k is, else a flat copy, at walls
  // too (bc_primitive.f90:258-264, 299-302, 339-345, 384-387, 436-439,
  // 554-557, 715-753)
  const bool lctm = p.transition == FEST_TRANSITION_LCTM2015;
  const int id = p.id[f];
  switch (id) {
    case -1:
      if (iter <= 2) {
        fix_col(p, q, f, ta, tb, 1, p.fix_rho[f]);
        fix_col(p, q, f, ta, tb, 2, p.fix_u[f]);
        fix_col(p, q, f, ta, tb, 3, p.fix_v[f]);
        fix_col(p, q, f, ta, tb, 4, p.fix_w[f]);
        fix_col(p, q, f, ta, tb, 5, p.fix_p[f]);
        if (sst) { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tw[f]); }
        if (sa) fix_col(p, q, f, ta, tb, 6, p.fix_tv[f]);
        if (kkl) { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tkl[f]); }
        if (lctm) fix_col(p, q, f, ta, tb, 8, p.fix_tgm[f]);
      }
      break;
    case -2:
    case -7:
      for (int l = 1; l <= d.nv; ++l) copy3_col(p, q, f, ta, tb, l, CP_FLAT);
      break;
    case -3:
      if (iter <= 2) {
        fix_col(p, q, f, ta, tb, 1, p.fix_rho[f]);
        fix_col(p, q, f, ta, tb, 2, p.fix_u[f]);
        fix_col(p, q, f, ta, tb, 3, p.fix_v[f]);
        fix_col(p, q, f, ta, tb, 4, p.fix_w[f]);
        if (sst) { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tw[f]); }
        if (sa) fix_col(p, q, f, ta, tb, 6, p.fix_tv[f]);
        if (kkl) { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tkl[f]); }
        if (lctm) fix_col(p, q, f, ta, tb, 8, p.fix_tgm[f]);
      }
      copy3_col(p, q, f, ta, tb, 5, CP_FLAT);
      break;
    case -4:
      for (int l = 1; l <= 4; ++l) copy3_col(p, q, f, ta, tb, l, CP_FLAT);
      if (iter <= 2) fix_col(p, q, f, ta, tb, 5, p.fix_p[f]);
      if (sst) { copy3_col(p, q, f, ta, tb, 6, CP_FLAT); copy3_col(p, q, f, ta, tb, 7, CP_FLAT); }
      if (sa) copy3_col(p, q, f, ta, tb, 6, CP_FLAT);
      if (kkl) { copy3_col(p, q, f, ta, tb, 6, CP_FLAT); copy3_col(p, q, f, ta, tb, 7, CP_FLAT); }
      if (lctm) copy3_col(p, q, f, ta, tb, 8, CP_FLAT);
      break;
    case -5: {  // wall (bc_primitive.f90:392-402)
      copy3_col(p, q, f, ta, tb, 5, CP_SYMM);
      double T = p.Tw[f], R = p.R, gm = p.gm;
      if (T < 0.0) {  // temp_based_density (bc_primitive.f90:1778-1945)
        long long i1 = inner_p(d, f, 1, ta, tb);
        double pp = q[i1 + 4 * P], rho = q[i1];
        double stag = (pp / (R * rho)) * (1 + (0.5 * (gm - 1.) * gm * pp / rho));
        for (int L = 1; L <= 3; ++L) {
          long long g = ghost_p(d, f, L, ta, tb);
          q[g] = q[g + 4 * P] / (R * stag);
        }
      } else if (T > 1.0) {
        for (int L = 1; L <= 3; ++L) {
          long long g = ghost_p(d, f, L, ta, tb), in = inner_p(d, f, L, ta, tb);
          double Ti = q[in + 4 * P] / (R * q[in]);
          q[g] = q[g + 4 * P] / (R * (2 * T - Ti));
        }
      } else {
        copy3_col(p, q, f, ta, tb, 1, CP_SYMM);
      }
      copy3_col(p, q, f, ta, tb, 2, CP_ANTI);
      copy3_col(p, q, f, ta, tb, 3, CP_ANTI);
      copy3_col(p, q, f, ta, tb, 4, CP_ANTI);
      if (sa) copy3_col(p, q, f, ta, tb, 6, CP_ANTI);
      if (kkl) { copy3_col(p, q, f, ta, tb, 6, CP_ANTI); copy3_col(p, q, f, ta, tb, 7, CP_ANTI); }
      if (lctm) copy3_col(p, q, f, ta, tb, 8, CP_FLAT);
      if (sst) {
        copy3_col(p, q, f, ta, tb, 6, CP_ANTI);
        // set_omega_at_wall (bc_primitive.f90:564-643)
        long long g0 = ghost_p(d, f, 1, ta, tb), i1 = inner_p(d, f, 1, ta, tb);
        double Tf = 0.5 * ((q[g0 + 4 * P] / q[g0]) + (q[i1 + 4 * P] / q[i1])) / R;
        double mu = p.mu_ref * pow(Tf / p.T_ref, 1.5) * ((p.T_ref + p.S) / (Tf + p.S));
        double rho = 0.5 * (q[g0] + q[i1]);
        double dd = 2 * b.dist[i1];
        for (int L = 1; L <= 3; ++L) {
          long long g = ghost_p(d, f, L, ta, tb), in = inner_p(d, f, L, ta, tb);
          q[g + 6 * P] = 120 * mu / (rho * 0.075 * (dd * dd)) - q[in + 6 * P];
        }
      }
    } break;
    case -6: {  // slip_wall + flow_tangency (FT_bc.f90:15-107)
      copy3_col(p, q, f, ta, tb, 1, CP_SYMM);
      copy3_col(p, q, f, ta, tb, 5, CP_SYMM);
      if (sst) { copy3_col(p, q, f, ta, tb, 6, CP_SYMM); copy3_col(p, q, f, ta, tb, 7, CP_SYMM); }
      if (sa) copy3_col(p, q, f, ta, tb, 6, CP_SYMM);
      if (kkl) { copy3_col(p, q, f, ta, tb, 6, CP_SYMM); copy3_col(p, q, f, ta, tb, 7, CP_SYMM); }
      if (lctm) copy3_col(p, q, f, ta, tb, 8, CP_FLAT);
      int fi, fj, fk;
      bface_ijk(d, f, ta, tb, fi, fj, fk);
      const double* fn = b.faces[f / 2] + 4 * fidx(d, f / 2, fi, fj, fk);
      const double* fr = b.faces[0] + 4 * fidx(d, 0, fi, fj, fk);
      for (int L = 1; L <= 3; ++L) {
        long long g = ghost_p(d, f, L, ta, tb), in = inner_p(d, f, L, ta, tb);
        double u = q[in + P], v = q[in + 2 * P], w = q[in + 3 * P];
        double dot = u * fn[1] + v * fn[2] + w * fn[3];
        q[g + P] = u - (2.0 * dot * fr[1]);
        q[g + 2 * P] = v - (2.0 * dot * fr[2]);
        q[g + 3 * P] = w - (2.0 * dot * fr[3]);
      }
    } break;
    case -8:
    case -11: {
      bool tp = (id == -11);
      riemann_col(p, b, f, ta, tb, true, tp);
      if (sst) {
        int na = (f / 2 == 0 ? d.jmx : d.imx) - 1, nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
        double Ulast = riemann_col(p, b, f, na, nb, false, tp);
        if (Ulast > 0.) { copy3_col(p, q, f, ta, tb, 6, CP_FLAT); copy3_col(p, q, f, ta, tb, 7, CP_FLAT); }
        else { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tw[f]); }
      }
      if (sa) {
        int na = (f / 2 == 0 ? d.jmx : d.imx) - 1, nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
        double Ulast = riemann_col(p, b, f, na, nb, false, tp);
        if (Ulast > 0.) copy3_col(p, q, f, ta, tb, 6, CP_FLAT);
        else fix_col(p, q, f, ta, tb, 6, p.fix_tv[f]);
      }
      if (kkl) {
        int na = (f / 2 == 0 ? d.jmx : d.imx) - 1, nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
        double Ulast = riemann_col(p, b, f, na, nb, false, tp);
        if (Ulast > 0.) { copy3_col(p, q, f, ta, tb, 6, CP_FLAT); copy3_col(p, q, f, ta, tb, 7, CP_FLAT); }
        else { fix_col(p, q, f, ta, tb, 6, p.fix_tk[f]); fix_col(p, q, f, ta, tb, 7, p.fix_tkl[f]); }
      }
      if (lctm) {
        int na = (f / 2 == 0 ? d.jmx : d.imx) - 1, nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
        double Ulast = riemann_col(p, b, f, na, nb, false, tp);
        if (Ulast > 0.) copy3_col(p, q, f, ta, tb, 8, CP_FLAT);
        else fix_col(p, q, f, ta, tb, 8, p.fix_tgm[f]);
      }
    } break;
    default:
      if (id == -10 || id >= 0) {  // interface / periodic exchange (interface1.f90:96-700)
        const BlockRef& pr = blocks[p.part_block[f]];
        const int pf = p.part_face[f];
        int na, nb, pa, pb;
        face_columns(d, f, na, nb);
        interface_map(p.part_orient[f], na, nb, ta, tb, pa, pb);
        for (int l = 1; l <= d.nv; ++l)
          for (int L = 1; L <= 3; ++L)
            q[ghost_p(d, f, L, ta, tb) + P * (l - 1)] =
                pr.b.qp[inner_p(pr.d, pf, L, pa, pb) + pr.d.P * (l - 1)];
      }
      break;
  }
}

__global__ void k_ghosts(Params p, DevBlock b, const BlockRef* blocks, int iter, int fmask) {
  const int f = blockIdx.z;
  if (!((fmask >> f) & 1)) return;
  const Dims& d = p.d;
  const int dir = f / 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  const int wa = na + 6, wb = nb + 6;  // full plane -2..n+3 of each tangential axis
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)wa * wb) return;
  const int ta = -2 + (int)(t % wa), tb = -2 + (int)(t / wa);
  const int id = p.id[f];
  const bool interior = ta >= 1 && ta <= na && tb >= 1 && tb <= nb;
  if (interior && id != -9) ghost_column(p, b, blocks, f, ta, tb, iter);
  if (id == -8 || id == -11 || id == -9) {
    double* q = b.qp;
    for (int l = 1; l <= d.nv; ++l) {
      const long long o = d.P * (l - 1);
      for (int L = 2 - (id == -9); L <= 3; ++L) {
        long long dst, src;
        if (id == -9) {  // periodic_bc (bc_primitive.f90:1948-1978)
          int n = extent_of(d, dir);
          int dc = (f % 2 == 0) ? (-2 + L - 1) : (n + L - 1);
          int sc = (f % 2 == 0) ? (n - 3 + L - 1) : (1 + L - 1);
          if (dir == 0) { dst = pidx(d, dc, ta, tb); src = pidx(d, sc, ta, tb); }
          else if (dir == 1) { dst = pidx(d, ta, dc, tb); src = pidx(d, ta, sc, tb); }
          else { dst = pidx(d, ta, tb, dc); src = pidx(d, ta, tb, sc); }
        } else {
          dst = ghost_p(d, f, L, ta, tb);
          src = ghost_p(d, f, 1, ta, tb);
        }
        q[dst + o] = q[src + o];
      }
    }
  }
  // the mixed fused path reads its stencil from an FP32 mirror: refresh the
  // face ghosts of this column there (edges and corners are never read by
  // an interior update)
  if (b.qp32 && interior && id != -9)
    for (int l = 0; l < d.nv; ++l)
      for (int L = 1; L <= 3; ++L) {
        const long long g = ghost_p(d, f, L, ta, tb);
        b.qp32[mirror_index(d, b.qp32_pitch, g, l)] = (float)b.qp[g + d.P * l];
      }
}

// bc_primitive.f90:209-224 corner/edge averaging, 16 ordered statements
__global__ void k_corners(Params p, double* q) {
  const Dims& d = p.d;
  corner_average<double>(d, [&](int i, int j, int k, int l) -> double& { return q[pidx(d, i, j, k) + d.P * (l - 1)]; });
}

__global__ void k_temperature(Params p, const double* qp, double* T) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.d.P) return;
  T[t] = qp[t + 4 * p.d.P] / (p.R * qp[t]);
}

// compute_face_interpolant (+ reconstruct_boundary_state when override),
// one cell per thread; only_boundary restricts the work to the override
// applied on the arrays already held (the reference's in/out semantics)
__global__ void k_face_states(Params p, DevBlock b, int dir, int override_mode) {
  const Dims& d = p.d;
  const int n = extent_of(d, dir);
  R3 r = dir == 0 ? r3(0, d.imx, 1, d.jmx - 1, 1, d.kmx - 1)
       : dir == 1 ? r3(1, d.imx - 1, 0, d.jmx, 1, d.kmx - 1)
                  : r3(1, d.imx - 1, 1, d.jmx - 1, 0, d.kmx);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const int c = dir == 0 ? i : dir == 1 ? j : k;
  const long long st = pstride(d, dir);
  const int i0 = dir == 0 ? 0 : i, j0 = dir == 1 ? 0 : j, k0 = dir == 2 ? 0 : k;
  const long long base = pidx(d, i0, j0, k0);
  FSDim fs = fsdim(d, dir);
  const long long oR = fsidx(fs, i, j, k);
  const long long oL = fsidx(fs, i + (dir == 0), j + (dir == 1), k + (dir == 2));
  Line<double, double> pres{b.qp + base + 4 * d.P, st};
  Line<double, double> vol{b.cells + 4 * base, 4 * st};
  if (override_mode == 2 && !near_boundary(p, dir, c)) return;
  for (int l = 1; l <= d.nv; ++l) {
    Line<double, double> q{b.qp + base + d.P * (l - 1), st};
    double Rm, Lp;
    if (override_mode == 2) {
      Rm = b.fsR[dir][oR + fs.N * (l - 1)];
      Lp = b.fsL[dir][oL + fs.N * (l - 1)];
    } else {
      recon_interior<double>(p, dir, c, l, q, pres, vol, Rm, Lp);
    }
    if (override_mode >= 1 && near_boundary(p, dir, c)) boundary_override<double>(p, dir, c, l, q, Rm, Lp);
    b.fsR[dir][oR + fs.N * (l - 1)] = Rm;
    b.fsL[dir][oL + fs.N * (l - 1)] = Lp;
  }
  (void)n;
}

// compute_fluxes (scheme.f90:68-109), one face per thread
__global__ void k_fluxes(Params p, DevBlock b, int dir) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1 + (dir == 0), 1, d.jmx - 1 + (dir == 1), 1, d.kmx - 1 + (dir == 2));
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  FSDim fs = fsdim(d, dir);
  FlDim fl = fldim(d, dir);
  const long long o = fsidx(fs, i, j, k);
  double qL[NVMOD], qR[NVMOD], Fo[NVMOD];
#pragma unroll
  for (int l = 0; l < NVMOD; ++l) {
    if (l < d.nv) {
      qL[l] = b.fsL[dir][o + fs.N * l];
      qR[l] = b.fsR[dir][o + fs.N * l];
    }
  }
  const double* fc = b.faces[dir] + 4 * fidx(d, dir, i, j, k);
  const int f = dir == 0 ? i : dir == 1 ? j : k;
  face_flux<double, -1, NVMOD>(p, qL, qR, fc[0], fc[1], fc[2], fc[3], (double)wall_mask(p, dir, f), Fo);
  const long long of = flidx(fl, i, j, k);
  bool bad = false;
#pragma unroll
  for (int l = 0; l < NVMOD; ++l)
    if (l < d.nv) {
      b.flux[dir][of + fl.N * l] = Fo[l];
      bad |= (Fo[l] != Fo[l]);
    }
  if (bad) raise_error(b.err, FEST_ERR_NAN);
}

// gradients.f90:405-482 (Green-Gauss) for all n_grad variables, one cell per thread
__global__ void k_gradients(Params p, DevBlock b) {
  const Dims& d = p.d;
  R3 r = r3(0, d.imx, 0, d.jmx, 0, d.kmx);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const long long c0 = pidx(d, i, j, k);
  const double* fi0 = b.faces[0] + 4 * fidx(d, 0, i, j, k);
  const double* fi1 = b.faces[0] + 4 * fidx(d, 0, i + 1, j, k);
  const double* fj0 = b.faces[1] + 4 * fidx(d, 1, i, j, k);
  const double* fj1 = b.faces[1] + 4 * fidx(d, 1, i, j + 1, k);
  const double* fk0 = b.faces[2] + 4 * fidx(d, 2, i, j, k);
  const double* fk1 = b.faces[2] + 4 * fidx(d, 2, i, j, k + 1);
  const double vol2 = 2 * b.cells[4 * c0];
  const long long sj = d.ni, sk = (long long)d.ni * d.nj;
  const long long og = gidx(d, i, j, k), NG = ngrad(d);
  const int ncomp = d.kmx > 2 ? 3 : 2;
  for (int lg = 1; lg <= p.n_grad; ++lg) {
    // variable: u,v,w from qp(2:4), T from Temp, tk,tw from qp(6:7)
    const double* v = (lg == 4) ? b.Temp : b.qp + d.P * (lg <= 3 ? lg : lg);
    const double vc = v[c0];
    for (int c = 0; c < 3; ++c) {
      double g = 0.0;
      if (c < ncomp) {
        double s = -((v[c0 - 1] + vc) * fi0[1 + c] * fi0[0]);
        s = s - (v[c0 - sj] + vc) * fj0[1 + c] * fj0[0];
        s = s - (v[c0 - sk] + vc) * fk0[1 + c] * fk0[0];
        s = s + (v[c0 + 1] + vc) * fi1[1 + c] * fi1[0];
        s = s + (v[c0 + sj] + vc) * fj1[1 + c] * fj1[0];
        s = s + (v[c0 + sk] + vc) * fk1[1 + c] * fk1[0];
        g = s / vol2;
        if (g != g) raise_error(b.err, FEST_ERR_NAN);
      }
      b.grad[c][og + NG * (lg - 1)] = g;
    }
  }
}

// apply_gradient_bc (gradients.f90:486-676), one boundary cell per thread
__global__ void k_gradient_bc(Params p, DevBlock b) {
  const int f = blockIdx.z;
  const Dims& d = p.d;
  if (!(p.id[f] < 0)) return;
  const int dir = f / 2, hi = f % 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)(t / na);
  int i, j, k;
  bface_ijk(d, f, ta, tb, i, j, k);
  const int il = hi ? 0 : 1, iu = hi ? 1 : 0;
  const int Gi = i - (dir == 0) * il, Gj = j - (dir == 1) * il, Gk = k - (dir == 2) * il;
  const int Ii = i - (dir == 0) * iu, Ij = j - (dir == 1) * iu, Ik = k - (dir == 2) * iu;
  const double* fc = b.faces[dir] + 4 * fidx(d, dir, i, j, k);
  const double nx = fc[1], ny = fc[2], nz = fc[3];
  const long long pI = pidx(d, Ii, Ij, Ik), pG = pidx(d, Gi, Gj, Gk);
  const double vI = b.cells[4 * pI];
  const double cc[3] = {fc[0] * nx / vI, fc[0] * ny / vI, fc[0] * nz / vI};
  const double sig = hi ? -1 : 1;
  const long long gI = gidx(d, Ii, Ij, Ik), gG = gidx(d, Gi, Gj, Gk), NG = ngrad(d);
  const double Tw = p.Tw[f];
  for (int l = 1; l <= p.n_grad; ++l) {
    double diff;
    if (l == 4) diff = b.Temp[pI] - b.Temp[pG];
    else diff = b.qp[pI + d.P * l] - b.qp[pG + d.P * l];
    for (int c = 0; c < 3; ++c) b.grad[c][gG + NG * (l - 1)] = sig * diff * cc[c];
  }
  if (p.id[f] == -5 && (Tw < 1. && Tw >= 0.))
    for (int c = 0; c < 3; ++c) b.grad[c][gG + NG * 3] = -b.grad[c][gI + NG * 3];
  for (int l = 1; l <= p.n_grad; ++l) {
    const long long oI = gI + NG * (l - 1), oG = gG + NG * (l - 1);
    double gx = b.grad[0][oI], gy = b.grad[1][oI], gz = b.grad[2][oI];
    double dot = (gx * nx) + (gy * ny) + (gz * nz);
    b.grad[0][oG] = b.grad[0][oG] + (gx - dot * nx);
    b.grad[1][oG] = b.grad[1][oG] + (gy - dot * ny);
    b.grad[2][oG] = b.grad[2][oG] + (gz - dot * nz);
  }
}

// ---- Spalart-Allmaras (global/global_sa.f90:6-22) -----------------------
constexpr double kSaCb1 = 0.1355, kSaCb2 = 0.6220, kSaCw2 = 0.3, kSaCw3 = 2.0, kSaSigma = 2. / 3.,
                 kSaKappa = 0.41;
__device__ __forceinline__ double sa_cw1() { return (kSaCb1 / (kSaKappa * kSaKappa)) + ((1 + kSaCb2) / kSaSigma); }
// x**6 as gfortran expands an integer power: x2 = x*x, x4 = x2*x2, x4*x2
__device__ __forceinline__ double sa_pow6(double x) {
  const double x2 = x * x, x4 = x2 * x2;
  return x4 * x2;
}
// the wall function fw(r) of source.f90:955-957 and update.f90:416-418
__device__ __forceinline__ double sa_fw(double r) {
  const double g = r + kSaCw2 * (sa_pow6(r) - r);
  return g * pow((1.0 + sa_pow6(kSaCw3)) / (sa_pow6(g) + sa_pow6(kSaCw3)), 1.0 / 6.0);
}
// the cell's vorticity magnitude from its velocity gradients
__device__ __forceinline__ double sa_vort(const DevBlock& b, long long og, long long NG) {
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  const double a = G(1, 3) - G(2, 2), bb = G(2, 1) - G(0, 3), c = G(0, 2) - G(1, 1);
  return sqrt(((a * a) + (bb * bb) + (c * c)));
}

// calculate_viscosity (viscosity.f90:52-546): Sutherland mu, SST mu_t and
// F1, Spalart-Allmaras mu_t
__global__ void k_viscosity(Params p, DevBlock b) {
  const Dims& d = p.d;
  R3 r = r3(0, d.imx, 0, d.jmx, 0, d.kmx);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const long long c0 = pidx(d, i, j, k);
  const double* q = b.qp;
  if (p.mu_ref != 0. && p.mu_var == FEST_MU_SUTHERLAND) {
    double T = q[c0 + 4 * d.P] / (q[c0] * p.R);
    b.mu[c0] = p.mu_ref * (pow(T / p.T_ref, 1.5)) * ((p.T_ref + p.S) / (T + p.S));
  }
  if (p.turb == FEST_TURB_NONE) return;
  if (p.turb == FEST_TURB_KKL) {  // viscosity.f90:469-490
    const double density = q[c0], tk = q[c0 + 5 * d.P], tkl = q[c0 + 6 * d.P];
    double m = p.kkl_c025 * density * tkl / (fmax2(sqrt(tk), 1.e-20));
    if (tkl < 1.e-14 || tk < 1.e-14) m = 0.0;
    b.mut[c0] = m;
    return;
  }
  if (p.turb == FEST_TURB_SA) {  // viscosity.f90:149-160: mu_t = rho tv fv1
    const double tv = q[c0 + 5 * d.P], density = q[c0];
    const double xi = tv * density / b.mu[c0];
    const double x3 = xi * xi * xi;
    const double fv1 = x3 / (x3 + p.sa_cv1_3);
    b.mut[c0] = density * tv * fv1;
    return;
  }
  const double bstar = 0.09, a1 = 0.31, sigma_w2 = 0.856;
  const long long og = gidx(d, i, j, k), NG = ngrad(d);
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  double rho = q[c0], tk = q[c0 + 5 * d.P], tw = q[c0 + 6 * d.P];
  double dd = b.dist[c0];
  double var1 = sqrt(tk) / (bstar * tw * dd);
  double var2 = 500 * (b.mu[c0] / rho) / ((dd * dd) * tw);
  double arg2 = fmax2(2 * var1, var2);
  double F = tanh(arg2 * arg2);
  double NUM = rho * a1 * tk, DENOM;
  bool s2003 = p.turb == FEST_TURB_SST2003;
  if (s2003) {
    double sxx = G(0, 1), syy = G(1, 2), szz = G(2, 3);
    double syz = G(1, 3) + G(2, 2), szx = G(2, 1) + G(0, 3), sxy = G(0, 2) + G(1, 1);
    double SijSij = (2.0 * (sxx * sxx)) + (2.0 * (syy * syy)) + (2.0 * (szz * szz)) + syz * syz +
                    szx * szx + sxy * sxy;
    DENOM = fmax2(fmax2((a1 * tw), sqrt(SijSij) * F), 1.0e-10);
  } else {
    double wx = G(1, 3) - G(2, 2), wy = G(2, 1) - G(0, 3), wz = G(0, 2) - G(1, 1);
    DENOM = fmax2(fmax2((a1 * tw), sqrt(wx * wx + wy * wy + wz * wz) * F), 1.e-20);
  }
  b.mut[c0] = NUM / DENOM;
  double CD = 2 * rho * sigma_w2 * (G(0, 5) * G(0, 6) + G(1, 5) * G(1, 6) + G(2, 5) * G(2, 6)) / tw;
  CD = fmax2(CD, s2003 ? 1.0e-10 : 1e-20);
  double right = 4 * (rho * sigma_w2 * tk) / (CD * (dd * dd));
  double arg1 = fmin2(fmax2(var1, var2), right);
  double a2 = arg1 * arg1;
  double F1 = tanh(a2 * a2);
  if (p.transition == FEST_TRANSITION_LCTM2015) {
    // viscosity.f90:265-280, 390-405: F1 raised to exp(-(var1/120)**8).
    // The reference loop reads density and tk without setting them, so
    // they hold its previous loop's last cell, (imx, jmx, kmx).
    const long long cz = pidx(d, d.imx, d.jmx, d.kmx);
    const double var1 = q[cz] * dd * sqrt(q[cz + 5 * d.P]) / b.mu[c0];
    const double x = var1 / 120, x2 = x * x, x4 = x2 * x2;
    F1 = fmax2(F1, exp(-(x4 * x4)));
  }
  b.F1[c0] = F1;
}

// ghost copies of mu_t / F1 (viscosity.f90:287-340)
__global__ void k_viscosity_ghost(Params p, DevBlock b) {
  const int f = blockIdx.z;
  const Dims& d = p.d;
  const int id = p.id[f];
  if (id == -10 || id >= 0 || id == -11 || id < -9) return;
  if (p.turb == FEST_TURB_KKL && id == -7) return;  // k-kL copies on -1..-4, -6, -8, -9 (viscosity.f90:491-531)
  const double sgn = (id == -5) ? -1.0 : 1.0;
  const int dir = f / 2;
  const int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)(t / na);
  long long g = ghost_p(d, f, 1, ta, tb), in = inner_p(d, f, 1, ta, tb);
  b.mut[g] = sgn < 0 ? -b.mut[in] : b.mut[in];
  b.F1[g] = b.F1[in];
}

// viscous.f90:144-325 laminar (+ viscous.f90:328-447 SST), one face per thread
__global__ void k_viscous(Params p, DevBlock b, int dir) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1 + (dir == 0), 1, d.jmx - 1 + (dir == 1), 1, d.kmx - 1 + (dir == 2));
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const int ii = dir == 0, jj = dir == 1, kk = dir == 2;
  const long long c1 = pidx(d, i, j, k), c0 = pidx(d, i - ii, j - jj, k - kk);
  const long long g1 = gidx(d, i, j, k), g0 = gidx(d, i - ii, j - jj, k - kk), NG = ngrad(d);
  const double* q = b.qp;
  const long long P = d.P;
  double G[3][4];
  for (int c = 0; c < 3; ++c)
    for (int l = 0; l < 4; ++l) G[c][l] = 0.5 * (b.grad[c][g0 + NG * l] + b.grad[c][g1 + NG * l]);
  const double* C1 = b.cells + 4 * c1;
  const double* C0 = b.cells + 4 * c0;
  double delx = C1[1] - C0[1], dely = C1[2] - C0[2], delz = C1[3] - C0[3];
  double dLR = sqrt(delx * delx + dely * dely + delz * delz);
  double TLE = q[c0 + 4 * P] / (q[c0] * p.R), TRE = q[c1 + 4 * P] / (q[c1] * p.R);
  double del[4] = {q[c1 + P] - q[c0 + P], q[c1 + 2 * P] - q[c0 + 2 * P], q[c1 + 3 * P] - q[c0 + 3 * P],
                   TRE - TLE};
  for (int l = 0; l < 4; ++l) {
    double nc = (del[l] - (G[0][l] * delx + G[1][l] * dely + G[2][l] * delz)) / dLR;
    G[0][l] = G[0][l] + (nc * delx / dLR);
    G[1][l] = G[1][l] + (nc * dely / dLR);
    G[2][l] = G[2][l] + (nc * delz / dLR);
  }
  const bool turb = p.turb != FEST_TURB_NONE;
  double mu_f = 0.5 * (b.mu[c0] + b.mu[c1]);
  double mut_f = turb ? 0.5 * (b.mut[c0] + b.mut[c1]) : 0.0;
  double tm = mu_f + mut_f;
  double dudx = G[0][0], dudy = G[1][0], dudz = G[2][0];
  double dvdx = G[0][1], dvdy = G[1][1], dvdz = G[2][1];
  double dwdx = G[0][2], dwdy = G[1][2], dwdz = G[2][2];
  double Txx = 2. * tm * (dudx - ((dudx + dvdy + dwdz) / 3.));
  double Tyy = 2. * tm * (dvdy - ((dudx + dvdy + dwdz) / 3.));
  double Tzz = 2. * tm * (dwdz - ((dudx + dvdy + dwdz) / 3.));
  double Txy = tm * (dvdx + dudy), Txz = tm * (dwdx + dudz), Tyz = tm * (dwdy + dvdz);
  double Kh = (mu_f / p.Pr + mut_f / p.tPr) * p.gm * p.R / (p.gm - 1);
  double Qx = Kh * G[0][3], Qy = Kh * G[1][3], Qz = Kh * G[2][3];
  const double* fc = b.faces[dir] + 4 * fidx(d, dir, i, j, k);
  double A = fc[0], nx = fc[1], ny = fc[2], nz = fc[3];
  double uf = 0.5 * (q[c0 + P] + q[c1 + P]);
  double vf = 0.5 * (q[c0 + 2 * P] + q[c1 + 2 * P]);
  double wf = 0.5 * (q[c0 + 3 * P] + q[c1 + 3 * P]);
  FlDim fl = fldim(d, dir);
  const long long of = flidx(fl, i, j, k);
  double* F = b.flux[dir];
  double F2 = F[of + fl.N] - ((Txx * nx + Txy * ny + Txz * nz) * A);
  double F3 = F[of + 2 * fl.N] - ((Txy * nx + Tyy * ny + Tyz * nz) * A);
  double F4 = F[of + 3 * fl.N] - ((Txz * nx + Tyz * ny + Tzz * nz) * A);
  double F5 = F[of + 4 * fl.N] - (A * (((Txx * uf + Txy * vf + Txz * wf + Qx) * nx) +
                                        ((Txy * uf + Tyy * vf + Tyz * wf + Qy) * ny) +
                                        ((Txz * uf + Tyz * vf + Tzz * wf + Qz) * nz)));
  bool bad = (F2 != F2) || (F3 != F3) || (F4 != F4) || (F5 != F5);
  if (p.turb == FEST_TURB_SA) {
    // compute_viscous_fluxes_sa (viscous.f90:570-656), every direction
    double H[3];
    for (int c = 0; c < 3; ++c) H[c] = 0.5 * (b.grad[c][g0 + NG * 4] + b.grad[c][g1 + NG * 4]);
    const double dtv = q[c1 + 5 * P] - q[c0 + 5 * P];
    const double nc = (dtv - (H[0] * delx + H[1] * dely + H[2] * delz)) / dLR;
    H[0] = H[0] + (nc * delx / dLR);
    H[1] = H[1] + (nc * dely / dLR);
    H[2] = H[2] + (nc * delz / dLR);
    const double rhoface = 0.5 * (q[c0] + q[c1]);
    const double mutv = 0.5 * (q[c0 + 5 * P] + q[c1 + 5 * P]) * rhoface;
    const double F6 = F[of + 5 * fl.N] - (A * ((mu_f + mutv) * (H[0] * nx + H[1] * ny + H[2] * nz))) / kSaSigma;
    F[of + 5 * fl.N] = F6;
    bad |= (F6 != F6);
  }
  if (p.turb == FEST_TURB_KKL) {
    // compute_viscous_fluxes_kkl (viscous.f90:450-567), every direction
    double H[3][2];
    for (int c = 0; c < 3; ++c)
      for (int l = 0; l < 2; ++l) H[c][l] = 0.5 * (b.grad[c][g0 + NG * (4 + l)] + b.grad[c][g1 + NG * (4 + l)]);
    double dl[2] = {q[c1 + 5 * P] - q[c0 + 5 * P], q[c1 + 6 * P] - q[c0 + 6 * P]};
    for (int l = 0; l < 2; ++l) {
      double nc = (dl[l] - (H[0][l] * delx + H[1][l] * dely + H[2][l] * delz)) / dLR;
      H[0][l] = H[0][l] + (nc * delx / dLR);
      H[1][l] = H[1][l] + (nc * dely / dLR);
      H[2][l] = H[2][l] + (nc * delz / dLR);
    }
    const double sigma_k = 1.0, sigma_phi = 1.0;
    const double rhoface = 0.5 * (q[c0] + q[c1]);
    const double tkface = 0.5 * (q[c0 + 5 * P] + q[c1 + 5 * P]);
    const double Tk = -2.0 * rhoface * tkface / 3.0;
    const double dk = H[0][0] * nx + H[1][0] * ny + H[2][0] * nz;
    const double dkl = H[0][1] * nx + H[1][1] * ny + H[2][1] * nz;
    F2 = F2 - (Tk * nx * A);
    F3 = F3 - (Tk * ny * A);
    F4 = F4 - (Tk * nz * A);
    F5 = F5 - (A * ((mu_f + sigma_k * mut_f) * dk));
    const double F6 = F[of + 5 * fl.N] - (A * ((mu_f + sigma_k * mut_f) * dk));
    const double F7 = F[of + 6 * fl.N] - (A * ((mu_f + sigma_phi * mut_f) * dkl));
    F[of + 5 * fl.N] = F6;
    F[of + 6 * fl.N] = F7;
    bad |= (F6 != F6) || (F7 != F7);
  }
  if (turb && p.turb != FEST_TURB_SA && p.turb != FEST_TURB_KKL && !(dir == 2 && d.kmx == 2)) {
    // SST diffusion (viscous.f90:378-444)
    const double sigma_k1 = 0.85, sigma_k2 = 1.0, sigma_w1 = 0.5, sigma_w2 = 0.856;
    double H[3][2];
    for (int c = 0; c < 3; ++c)
      for (int l = 0; l < 2; ++l) H[c][l] = 0.5 * (b.grad[c][g0 + NG * (4 + l)] + b.grad[c][g1 + NG * (4 + l)]);
    double dl[2] = {q[c1 + 5 * P] - q[c0 + 5 * P], q[c1 + 6 * P] - q[c0 + 6 * P]};
    for (int l = 0; l < 2; ++l) {
      double nc = (dl[l] - (H[0][l] * delx + H[1][l] * dely + H[2][l] * delz)) / dLR;
      H[0][l] = H[0][l] + (nc * delx / dLR);
      H[1][l] = H[1][l] + (nc * dely / dLR);
      H[2][l] = H[2][l] + (nc * delz / dLR);
    }
    double F1 = 0.5 * (b.F1[c0] + b.F1[c1]);
    double skf = sigma_k1 * F1 + sigma_k2 * (1.0 - F1);
    double swf = sigma_w1 * F1 + sigma_w2 * (1.0 - F1);
    double rhof = 0.5 * (q[c0] + q[c1]);
    double tkf = 0.5 * (q[c0 + 5 * P] + q[c1 + 5 * P]);
    double Tk = -2.0 * rhof * tkf / 3.0;
    double dk = H[0][0] * nx + H[1][0] * ny + H[2][0] * nz;
    double dw = H[0][1] * nx + H[1][1] * ny + H[2][1] * nz;
    F2 = F2 - (Tk * nx * A);
    F3 = F3 - (Tk * ny * A);
    F4 = F4 - (Tk * nz * A);
    F5 = F5 - (A * ((mu_f + skf * mut_f) * dk));
    double F6 = F[of + 5 * fl.N] - (A * ((mu_f + skf * mut_f) * dk));
    double F7 = F[of + 6 * fl.N] - (A * ((mu_f + swf * mut_f) * dw));
    F[of + 5 * fl.N] = F6;
    F[of + 6 * fl.N] = F7;
    bad |= (F6 != F6) || (F7 != F7);
  }
  if (p.transition == FEST_TRANSITION_LCTM2015 && !(dir == 2 && d.kmx == 2)) {
    // compute_viscous_fluxes_lctm2015 (viscous.f90:658-749): the
    // intermittency diffused with mu + mu_t
    double H[3];
    for (int c = 0; c < 3; ++c) H[c] = 0.5 * (b.grad[c][g0 + NG * 6] + b.grad[c][g1 + NG * 6]);
    const double dg = q[c1 + 7 * P] - q[c0 + 7 * P];
    const double nc = (dg - (H[0] * delx + H[1] * dely + H[2] * delz)) / dLR;
    H[0] = H[0] + (nc * delx / dLR);
    H[1] = H[1] + (nc * dely / dLR);
    H[2] = H[2] + (nc * delz / dLR);
    const double F8 = F[of + 7 * fl.N] - (A * ((mu_f + mut_f) * (H[0] * nx + H[1] * ny + H[2] * nz)));
    F[of + 7 * fl.N] = F8;
    bad |= (F8 != F8);
  }
  F[of + fl.N] = F2;
  F[of + 2 * fl.N] = F3;
  F[of + 3 * fl.N] = F4;
  F[of + 4 * fl.N] = F5;
  if (bad) raise_error(b.err, FEST_ERR_NAN);
}

// compute_residue (scheme.f90:111-141)
__global__ void k_residue(Params p, DevBlock b) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1, 1, d.jmx - 1, 1, d.kmx - 1);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  FlDim fx = fldim(d, 0), fy = fldim(d, 1), fz = fldim(d, 2);
  const long long o = cidx(d, i, j, k), N = ncells(d);
  const long long ox0 = flidx(fx, i, j, k), ox1 = flidx(fx, i + 1, j, k);
  const long long oy0 = flidx(fy, i, j, k), oy1 = flidx(fy, i, j + 1, k);
  const long long oz0 = flidx(fz, i, j, k), oz1 = flidx(fz, i, j, k + 1);
  for (int l = 0; l < d.nv; ++l)
    b.res[o + N * l] = (b.flux[0][ox1 + fx.N * l] - b.flux[0][ox0 + fx.N * l]) +
                       (b.flux[1][oy1 + fy.N * l] - b.flux[1][oy0 + fy.N * l]) +
                       (b.flux[2][oz1 + fz.N * l] - b.flux[2][oz0 + fz.N * l]);
}

// the 'bc' transition model's intermittency (source.f90:571-589 and
// 1159-1170) from the momentum-thickness Reynolds number re_v / 2.193
// against its transition value and the eddy viscosity against its critical
// value
__device__ __forceinline__ double gamma_bc(const Params& p, double re_v, double nu_bc) {
  const double re_theta = re_v / 2.193;
  const double term1 = sqrt(fmax2(re_theta - p.bc_re_theta_t, 0.) / (0.002 * p.bc_re_theta_t));
  const double term2 = sqrt(fmax2(nu_bc - p.bc_nu_cr, 0.0) / p.bc_nu_cr);
  return 1.0 - exp(-(term1 + term2));
}

// add_sa_source (source.f90:845-983): the density gradient from the cell's
// six face sums, whose k faces' normal reads (nx, nx, nx) as the reference
// does (source.f90:913).  With the 'bc' transition model, add_saBC_source
// (source.f90:985-1194): S-hat floored at 1e-10 instead of 0.3 Omega, the
// production scaled by the intermittency and, as there, not by density
__device__ void sa_source(const Params& p, const DevBlock& b, int i, int j, int k) {
  const Dims& d = p.d;
  const long long c0 = pidx(d, i, j, k), og = gidx(d, i, j, k), NG = ngrad(d), P = d.P;
  const double* q = b.qp;
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  const double density = q[c0], tv = q[c0 + 5 * P];
  const long long nb[6] = {pidx(d, i - 1, j, k), pidx(d, i, j - 1, k), pidx(d, i, j, k - 1),
                           pidx(d, i + 1, j, k), pidx(d, i, j + 1, k), pidx(d, i, j, k + 1)};
  const double* fr[6] = {b.faces[0] + 4 * fidx(d, 0, i, j, k), b.faces[1] + 4 * fidx(d, 1, i, j, k),
                         b.faces[2] + 4 * fidx(d, 2, i, j, k), b.faces[0] + 4 * fidx(d, 0, i + 1, j, k),
                         b.faces[1] + 4 * fidx(d, 1, i, j + 1, k), b.faces[2] + 4 * fidx(d, 2, i, j, k + 1)};
  double rf[6], nrm[6][3];
  for (int f = 0; f < 6; ++f) {
    rf[f] = q[nb[f]] + density;
    for (int c = 0; c < 3; ++c) nrm[f][c] = fr[f][f == 2 ? 1 : 1 + c];
  }
  const double vol = b.cells[4 * c0];
  double gr[3];
  for (int c = 0; c < 3; ++c)
    gr[c] = (-(rf[0]) * nrm[0][c] * fr[0][0] - (rf[1]) * nrm[1][c] * fr[1][0] - (rf[2]) * nrm[2][c] * fr[2][0] +
             (rf[3]) * nrm[3][c] * fr[3][0] + (rf[4]) * nrm[4][c] * fr[4][0] + (rf[5]) * nrm[5][c] * fr[5][0]) /
            (2.0 * vol);
  const double vort = sa_vort(b, og, NG);
  const double CD1 = kSaCb2 * ((G(0, 5) * G(0, 5)) + (G(1, 5) * G(1, 5)) + (G(2, 5) * G(2, 5)));
  const double CD2 = ((gr[0] * G(0, 5)) + (gr[1] * G(1, 5)) + (gr[2] * G(2, 5)));
  const double dd = b.dist[c0];
  const double kd = kSaKappa * dd, kd2 = kd * kd;
  const double nu = b.mu[c0] / density;
  const double xi = tv / nu;
  const double x3 = xi * xi * xi;
  const double fv1 = x3 / (x3 + p.sa_cv1_3);
  const double fv2 = 1.0 - xi / (1.0 + (xi * fv1));
  const long long o = cidx(d, i, j, k), N = ncells(d);
  if (p.transition == FEST_TRANSITION_BC) {
    const double u = q[c0 + P], v = q[c0 + 2 * P], w = q[c0 + 3 * P];
    const double vmag = sqrt(u * u + v * v + w * w);
    const double d2 = dd * dd;
    const double inv_k2_d2 = 1.0 / ((kSaKappa * kSaKappa) * d2);
    const double Shat = fmax2(vort + tv * fv2 * inv_k2_d2, 1.0e-10);
    const double inv_Shat = 1.0 / Shat;
    const double nu_bc = (tv * fv1) / (vmag * dd);
    const double re_v = d2 * vort / nu;
    const double Prod = gamma_bc(p, re_v, nu_bc) * kSaCb1 * Shat * tv * vol;
    const double fw = sa_fw(fmin2(tv * inv_Shat * inv_k2_d2, 10.0));
    const double Dest = (sa_cw1() * fw * tv * tv / d2) * (vol);
    const double lam = (density * CD1 / kSaSigma - CD2 * (nu + tv) / kSaSigma) * vol;
    b.res[o + 5 * N] = b.res[o + 5 * N] - (Prod - Dest + lam);
    return;
  }
  const double Scap = fmax2(vort + (tv * fv2 / (kd2)), 0.3 * vort);
  const double rr = fmin2(tv / (Scap * kd2), 10.0);
  const double fw = sa_fw(rr);
  const double td = tv / dd;
  const double D_v = density * sa_cw1() * fw * (td * td);
  const double P_v = density * kSaCb1 * Scap * tv;
  const double lamda = density * CD1 / kSaSigma - CD2 * (nu + tv) / kSaSigma;
  const double S_v = (P_v - D_v + lamda) * vol;
  b.res[o + 5 * N] = b.res[o + 5 * N] - S_v;
}

// add_kkl_source (source.f90:607-832): production by the Reynolds stress,
// the von Karman length from the velocity's second derivatives (Green-Gauss
// sums of the cell gradients over the cell's faces) with its limiters, the
// wall damping
__device__ void kkl_source(const Params& p, const DevBlock& b, int i, int j, int k) {
  const Dims& d = p.d;
  const long long c0 = pidx(d, i, j, k), og = gidx(d, i, j, k), NG = ngrad(d), P = d.P;
  const double* q = b.qp;
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  const double density = q[c0], tk = q[c0 + 5 * P], tkl = q[c0 + 6 * P];
  double S[3][3];
  for (int a = 0; a < 3; ++a)
    for (int c = 0; c < 3; ++c) S[a][c] = 0.5 * (G(c, a + 1) + G(a, c + 1));
  const double delv = G(0, 1) + G(1, 2) + G(2, 3);
  const double mt = b.mut[c0];
  double Pk = 0.;
  for (int a = 0; a < 3; ++a) {
    double T[3];
    for (int c = 0; c < 3; ++c)
      T[c] = a == c ? mt * (2 * S[a][c] - (2.0 / 3.0) * delv) - (2.0 / 3.0) * density * tk : mt * (2 * S[a][c]);
    Pk = Pk + T[0] * G(0, a + 1) + T[1] * G(1, a + 1) + T[2] * G(2, a + 1);
  }
  const double Dk = p.kkl_c075 * density * (pow(tk, 2.5)) / fmax2(tkl, 1.e-20);
  Pk = fmin2(Pk, 20 * Dk);
  const double* fr[6] = {b.faces[0] + 4 * fidx(d, 0, i, j, k), b.faces[1] + 4 * fidx(d, 1, i, j, k),
                         b.faces[2] + 4 * fidx(d, 2, i, j, k), b.faces[0] + 4 * fidx(d, 0, i + 1, j, k),
                         b.faces[1] + 4 * fidx(d, 1, i, j + 1, k), b.faces[2] + 4 * fidx(d, 2, i, j, k + 1)};
  const long long nb[6] = {gidx(d, i - 1, j, k), gidx(d, i, j - 1, k), gidx(d, i, j, k - 1),
                           gidx(d, i + 1, j, k), gidx(d, i, j + 1, k), gidx(d, i, j, k + 1)};
  const double vol2 = 2 * b.cells[4 * c0];
  double lap[3];
  for (int a = 0; a < 3; ++a) {
    double sum = 0.0;
    for (int c = 0; c < 3; ++c) {
      const double* gr = b.grad[c] + NG * a;
      const double gc = gr[og];
      double t = -((gr[nb[0]] + gc) * fr[0][1 + c] * fr[0][0]);
      for (int f = 1; f < 6; ++f) {
        const double v = (gr[nb[f]] + gc) * fr[f][1 + c] * fr[f][0];
        t = f < 3 ? t - v : t + v;
      }
      sum = c == 0 ? t / vol2 : sum + t / vol2;
    }
    lap[a] = sum;
  }
  const double udd = sqrt((lap[0] * lap[0]) + (lap[1] * lap[1]) + (lap[2] * lap[2]));
  double s2 = S[0][0] * S[0][0];
  for (int n = 1; n < 9; ++n) s2 = s2 + S[n / 3][n % 3] * S[n / 3][n % 3];
  const double ud = sqrt(2 * s2);
  const double kap = 0.41;
  double Lvk = kap * fabs(ud / fmax2(udd, 1.e-20));
  const double fp = fmin2(fmax2(Pk / Dk, 0.5), 1.0);
  const double dd = b.dist[c0], m = b.mu[c0];
  Lvk = fmax2(Lvk, tkl / fmax2((tk * 10.0), 1.e-20));
  Lvk = fmin2(Lvk, 1.3 * kap * dd * fp);
  const double eta = density * dd * sqrt(0.3 * tk) / (20 * m);
  const double e2 = eta * eta;
  const double fphi = (1 + 4.7 * eta) / (1 + e2 * e2);
  const double rr = tkl / fmax2(tk * Lvk, 1.e-20);
  const double cphi1 = (1.2 - 0.97 * (rr * rr));
  const double Pkl = cphi1 * tkl * Pk / fmax2(tk, 1.e-20);
  const double Dkl = 0.13 * density * (pow(tk, 1.5));
  const double vol = b.cells[4 * c0];
  const double Sk = (Pk - Dk - 2 * m * tk / (dd * dd)) * vol;
  const double Skl = (Pkl - Dkl - 6 * m * tkl * fphi / (dd * dd)) * vol;
  const long long o = cidx(d, i, j, k), N = ncells(d);
  b.res[o + 5 * N] = b.res[o + 5 * N] - Sk;
  b.res[o + 6 * N] = b.res[o + 6 * N] - Skl;
}

// add_sst_source_lctm2015 (source.f90:273-465): SST's source with the
// production by vorticity times strain scaled by the intermittency, the
// limited extra production, the floored destruction, and the
// intermittency's own source; the pressure-gradient parameter from the
// wall distance's gradient dotted with its unit vector (CC.f90:56-92, the
// six face sums of the distance)
__device__ void lctm_source(const Params& p, const DevBlock& b, int i, int j, int k) {
  const Dims& d = p.d;
  const long long c0 = pidx(d, i, j, k), og = gidx(d, i, j, k), NG = ngrad(d), P = d.P;
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  const double sigma_w1 = 0.5, sigma_w2 = 0.856, beta1 = 0.075, beta2 = 0.0828, bstar = 0.09, kap = 0.41;
  const bool s2003 = p.turb == FEST_TURB_SST2003;
  const int limiter = s2003 ? 10 : 20;
  double gama1 = (beta1 / bstar) - ((sigma_w1 * (kap * kap)) / sqrt(bstar));
  double gama2 = (beta2 / bstar) - ((sigma_w2 * (kap * kap)) / sqrt(bstar));
  if (s2003) { gama1 = 5.0 / 9.0; gama2 = 0.44; }
  const double* q = b.qp;
  const double density = q[c0], tk = q[c0 + 5 * P], tw = q[c0 + 6 * P], gm_ = q[c0 + 7 * P];
  double vort, strain;
  lctm_vort_strain(b, og, NG, vort, strain);
  double CD = 2 * density * sigma_w2 * (G(0, 5) * G(0, 6) + G(1, 5) * G(1, 6) + G(2, 5) * G(2, 6)) / tw;
  CD = fmax2(CD, s2003 ? 1.0e-10 : 1e-20);
  const double F1 = b.F1[c0];
  const double gama = gama1 * F1 + gama2 * (1. - F1);
  const double beta = beta1 * F1 + beta2 * (1. - F1);
  const double D_k = bstar * density * tw * tk;
  const double D_w = beta * density * (tw * tw);
  const double divergence = G(0, 1) + G(1, 2) + G(2, 3);
  const double mt = b.mut[c0], m = b.mu[c0], dd = b.dist[c0];
  double P_k = mt * (vort * strain) - ((2.0 / 3.0) * density * tk * divergence);
  P_k = fmin2(P_k, limiter * D_k);
  const double P_w = (density * gama / mt) * P_k;
  const double lamda = (1. - F1) * CD;
  const long long nb[6] = {pidx(d, i - 1, j, k), pidx(d, i, j - 1, k), pidx(d, i, j, k - 1),
                           pidx(d, i + 1, j, k), pidx(d, i, j + 1, k), pidx(d, i, j, k + 1)};
  const double* fr[6] = {b.faces[0] + 4 * fidx(d, 0, i, j, k), b.faces[1] + 4 * fidx(d, 1, i, j, k),
                         b.faces[2] + 4 * fidx(d, 2, i, j, k), b.faces[0] + 4 * fidx(d, 0, i + 1, j, k),
                         b.faces[1] + 4 * fidx(d, 1, i, j + 1, k), b.faces[2] + 4 * fidx(d, 2, i, j, k + 1)};
  const double vol = b.cells[4 * c0];
  double gd[3];
  for (int c = 0; c < 3; ++c) {
    double s = -((b.dist[nb[0]] + dd) * fr[0][1 + c] * fr[0][0]);
    s = s - (b.dist[nb[1]] + dd) * fr[1][1 + c] * fr[1][0];
    s = s - (b.dist[nb[2]] + dd) * fr[2][1 + c] * fr[2][0];
    s = s + (b.dist[nb[3]] + dd) * fr[3][1 + c] * fr[3][0];
    s = s + (b.dist[nb[4]] + dd) * fr[4][1 + c] * fr[4][0];
    s = s + (b.dist[nb[5]] + dd) * fr[5][1 + c] * fr[5][0];
    gd[c] = s / (2 * vol);
  }
  const double Vn = sqrt(gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2]);
  const double dvdy = gd[0] * (gd[0] / (Vn + 1e-12)) + gd[1] * (gd[1] / (Vn + 1e-12)) + gd[2] * (gd[2] / (Vn + 1e-12));
  double lamd = (-7.57e-3) * (dvdy * dd * dd * density / m) + 0.0128;
  lamd = fmin2(fmax2(lamd, -1.0), 1.0);
  double Fpg = lamd >= 0.0 ? fmin2(1.0 + 14.68 * lamd, 1.5) : fmin2(1.0 - 7.34 * lamd, 3.0);
  Fpg = fmax2(Fpg, 0.0);
  const double TuL = fmin2(100.0 * sqrt(2.0 * tk / 3.0) / (tw * dd), 100.0);
  const double Re_theta = 100.0 + 1000.0 * exp(-TuL * Fpg);
  const double Rev = density * dd * dd * strain / m;
  const double RT = density * tk / (m * tw);
  double Fturb, Fonset;
  lctm_onset(Rev, RT, Re_theta, Fturb, Fonset);
  const double P_gm = 100 * density * strain * gm_ * (1.0 - gm_) * Fonset;
  const double D_gm = 0.06 * density * vort * gm_ * Fturb * ((50.0 * gm_) - 1.0);
  const double Fon_lim = fmin2(fmax2((Rev / (2.2 * 1100.0)) - 1.0, 0.0), 3.0);
  const double Pk_lim = 5 * fmax2(gm_ - 0.2, 0.0) * (1.0 - gm_) * Fon_lim * fmax2(3 * m - mt, 0.0) * strain * vort;
  const double S_k = gm_ * P_k - fmax2(gm_, 0.1) * D_k + Pk_lim;
  const double S_w = P_w - D_w + lamda;
  const double S_gm = P_gm - D_gm;
  const long long o = cidx(d, i, j, k), N = ncells(d);
  b.res[o + 5 * N] = b.res[o + 5 * N] - S_k * vol;
  b.res[o + 6 * N] = b.res[o + 6 * N] - S_w * vol;
  b.res[o + 7 * N] = b.res[o + 7 * N] - S_gm * vol;
}

// add_source_term_residue (source.f90:94-155): add_sa_source (or
// add_saBC_source), add_kkl_source, or add_sst_source (source.f90:158-270;
// or add_sst_bc_source, source.f90:467-604: production mu_t Omega^2 limited
// by 20 D_k, P_w from it before the intermittency scales it, the cross
// diffusion unfloored, the SST constants whatever the variant)
__global__ void k_source(Params p, DevBlock b) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1, 1, d.jmx - 1, 1, d.kmx - 1);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  if (p.turb == FEST_TURB_SA) {
    sa_source(p, b, i, j, k);
    return;
  }
  if (p.turb == FEST_TURB_KKL) {
    kkl_source(p, b, i, j, k);
    return;
  }
  if (p.transition == FEST_TRANSITION_LCTM2015) {
    lctm_source(p, b, i, j, k);
    return;
  }
  const double sigma_w1 = 0.5, sigma_w2 = 0.856, beta1 = 0.075, beta2 = 0.0828, bstar = 0.09,
               kap = 0.41;
  const bool bc = p.transition == FEST_TRANSITION_BC;
  int limiter;
  double gama1, gama2;
  if (p.turb == FEST_TURB_SST2003 && !bc) {
    limiter = 10; gama1 = 5.0 / 9.0; gama2 = 0.44;
  } else {
    limiter = 20;
    gama1 = (beta1 / bstar) - ((sigma_w1 * (kap * kap)) / sqrt(bstar));
    gama2 = (beta2 / bstar) - ((sigma_w2 * (kap * kap)) / sqrt(bstar));
  }
  const double cdmin = limiter == 10 ? 1e-10 : 1e-20;
  const long long c0 = pidx(d, i, j, k), og = gidx(d, i, j, k), NG = ngrad(d);
  auto G = [&](int c, int l) { return b.grad[c][og + NG * (l - 1)]; };
  double rho = b.qp[c0], tk = b.qp[c0 + 5 * d.P], tw = b.qp[c0 + 6 * d.P];
  double a = G(1, 3) - G(2, 2), bb = G(2, 1) - G(0, 3), c = G(0, 2) - G(1, 1);
  double vort = sqrt(((a * a) + (bb * bb) + (c * c)));
  double CD = 2 * rho * sigma_w2 * (G(0, 5) * G(0, 6) + G(1, 5) * G(1, 6) + G(2, 5) * G(2, 6)) / tw;
  if (!bc) CD = fmax2(CD, cdmin);
  double F1 = b.F1[c0];
  double gama = gama1 * F1 + gama2 * (1. - F1);
  double beta = beta1 * F1 + beta2 * (1. - F1);
  double Dk = bstar * rho * tw * tk;
  double Dw = beta * rho * (tw * tw);
  double divergence = G(0, 1) + G(1, 2) + G(2, 3);
  double mt = b.mut[c0];
  double Pk = bc ? mt * (vort * vort) : mt * (vort * vort) - ((2.0 / 3.0) * rho * tk * divergence);
  Pk = fmin2(Pk, limiter * Dk);
  double Pw = (rho * gama / mt) * Pk;
  if (bc) {
    const double u = b.qp[c0 + d.P], v = b.qp[c0 + 2 * d.P], w = b.qp[c0 + 3 * d.P];
    const double vmag = sqrt(u * u + v * v + w * w);
    const double dd = b.dist[c0];
    const double nu_bc = (mt / rho) / (vmag * dd);
    const double re_v = rho * dd * dd * vort / b.mu[c0];
    Pk = gamma_bc(p, re_v, nu_bc) * Pk;
  }
  double Sk = (Pk - Dk) * b.cells[4 * c0];
  double Sw = (Pw - Dw + (1. - F1) * CD) * b.cells[4 * c0];
  const long long o = cidx(d, i, j, k), N = ncells(d);
  b.res[o + 5 * N] = b.res[o + 5 * N] - Sk;
  b.res[o + 6 * N] = b.res[o + 6 * N] - Sw;
}

// compute_local_time_step + add_viscous_time + add_turbulent_time (time.f90)
__global__ void k_time_step(Params p, DevBlock b, double CFL) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1, 1, d.jmx - 1, 1, d.kmx - 1);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const long long c0 = pidx(d, i, j, k), P = d.P;
  const double gm = p.gm;
  const double* q = b.qp;
  double lmx[6], Af[6];
  for (int dir = 0; dir < 3; ++dir) {
    const int di = dir == 0, dj = dir == 1, dk = dir == 2;
    FSDim fs = fsdim(d, dir);
    for (int s = 0; s < 2; ++s) {
      const long long of = fsidx(fs, i + s * di, j + s * dj, k + s * dk);
      const double* L = b.fsL[dir];
      const double* R = b.fsR[dir];
      double cs = 0.5 * (sqrt(gm * L[of + 4 * fs.N] / L[of]) + sqrt(gm * R[of + 4 * fs.N] / R[of]));
      const double* fc = b.faces[dir] + 4 * fidx(d, dir, i + s * di, j + s * dj, k + s * dk);
      const long long cq = c0 + s * pstride(d, dir);
      lmx[3 * s + dir] = fabs((q[cq + P] * fc[1]) + (q[cq + 2 * P] * fc[2]) + (q[cq + 3 * P] * fc[3])) + cs;
      Af[3 * s + dir] = fc[0];
    }
  }
  double sum = (Af[0] * lmx[0]) + (Af[1] * lmx[1]) + (Af[2] * lmx[2]) + (Af[3] * lmx[3]) +
               (Af[4] * lmx[4]) + (Af[5] * lmx[5]);
  const double V = b.cells[4 * c0];
  double dt = (1. / sum) * V * CFL;
  const int nvisc = (p.mu_ref != 0.0) ? ((p.turb != FEST_TURB_NONE) ? 2 : 1) : 0;
  for (int part = 0; part < nvisc; ++part) {
    const double* mu = part == 0 ? b.mu : b.mut;
    const double Pr = part == 0 ? p.Pr : p.tPr;
    const double* cc = b.cells + 4 * c0;
    double lv[6];
    for (int dir = 0; dir < 3; ++dir) {
      const long long st = pstride(d, dir);
      const double* cm = b.cells + 4 * (c0 - st);
      const double* cp = b.cells + 4 * (c0 + st);
      const double* f0 = b.faces[dir] + 4 * fidx(d, dir, i, j, k);
      const double* f1 = b.faces[dir] + 4 * fidx(d, dir, i + (dir == 0), j + (dir == 1), k + (dir == 2));
      lv[dir] = mu[c0] / (q[c0] * fabs(((cm[1] - cc[1]) * f0[1]) + ((cm[2] - cc[2]) * f0[2]) + ((cm[3] - cc[3]) * f0[3])));
      lv[3 + dir] = mu[c0 + st] / (q[c0 + st] * fabs(((cc[1] - cp[1]) * f1[1]) + ((cc[2] - cp[2]) * f1[2]) +
                                                     ((cc[3] - cp[3]) * f1[3])));
    }
    double s = (Af[0] * lv[0]) + (Af[1] * lv[1]) + (Af[2] * lv[2]) + (Af[3] * lv[3]) + (Af[4] * lv[4]) +
               (Af[5] * lv[5]);
    s = gm * s / Pr;
    s = 2. / (s + (2. * CFL * V / dt));
    dt = CFL * (s * V);
  }
  b.dt[cidx(d, i, j, k)] = dt;
}

// min over a block's delta_t (two passes: partial mins then one block)
__global__ void k_min_partial(const double* x, long long n, double* out) {
  __shared__ double sm[TPB];
  double m = 1e308;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    m = fmin(m, x[t]);
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sm[threadIdx.x] = fmin(sm[threadIdx.x], sm[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[blockIdx.x] = sm[0];
}
__global__ void k_fill_min(double* x, long long n, const double* part, int nparts, double gdt) {
  __shared__ double m;
  if (threadIdx.x == 0) {
    double v = 1e308;
    if (gdt > 0) v = gdt;
    else
      for (int i = 0; i < nparts; ++i) v = fmin(v, part[i]);
    m = v;
  }
  __syncthreads();
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
    x[t] = m;
}

// update_with(...,'conservative',...) (update.f90:367-485)
__global__ void k_update(Params p, DevBlock b, double TF, double SF, int TU, int use_store) {
  const Dims& d = p.d;
  R3 r = r3(1, d.imx - 1, 1, d.jmx - 1, 1, d.kmx - 1);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const long long c0 = pidx(d, i, j, k), P = d.P, o = cidx(d, i, j, k), N = ncells(d);
  const double* Qu = use_store ? b.Ustore : b.qp;
  const int nv = d.nv;
  const double gm = p.gm;
  double u1[NVMOD], u2[NVMOD], R[NVMOD];
  u1[0] = Qu[c0];
#pragma unroll
  for (int l = 1; l < NVMOD; ++l)
    if (l < nv) u1[l] = Qu[c0 + P * l] * u1[0];
  double s1 = u1[1] * u1[1] + u1[2] * u1[2] + u1[3] * u1[3];
  u1[4] = (u1[4] / (gm - 1.) + 0.5 * s1) / u1[0];
#pragma unroll
  for (int l = 0; l < NVMOD; ++l)
    if (l < nv) R[l] = b.res[o + N * l];
  const double dtc = b.dt[o];
  const bool sa = p.turb == FEST_TURB_SA;
  if (sa) {
    // update.f90:405-419, xi from the conservative U1(6) and the stage
    // state's density as written there
    const double vort = sa_vort(b, gidx(d, i, j, k), ngrad(d));
    const double dd = b.dist[c0];
    const double kd = kSaKappa * dd, kd2 = kd * kd;
    const double xi = u1[5] * b.qp[c0] / b.mu[c0];
    const double x3 = xi * xi * xi;
    const double fv1 = x3 / (x3 + p.sa_cv1_3);
    const double fv2 = 1.0 - xi / (1 + xi * fv1);
    const double scap = vort + u1[5] * fv2 / (kd2);
    const double rsa = fmin2(u1[5] / (scap * kd2), 10.0);
    const double fw = sa_fw(rsa);
    R[5] = R[5] / (1. + ((-1.0 * u1[0] * kSaCb1 * scap) + (2.0 * u1[0] * sa_cw1() * fw * u1[5] / (dd * dd))) * dtc);
  } else if (p.turb == FEST_TURB_KKL) {
    // update.f90:399-404, with the conservative U1(6), U1(7)
    const double dd = b.dist[c0], m = b.mu[c0];
    const double eta = u1[0] * dd * (sqrt(0.3 * u1[5]) / (20 * m));
    const double e2 = eta * eta;
    const double fphi = (1 + 4.7 * eta) / (1 + e2 * e2);
    R[5] = R[5] / (1. + ((2.5 * ((p.kkl_c075 * sqrt(u1[0]) * (pow(u1[5], 1.5))) / fmax2(u1[6], 1.e-20))) +
                         (2 * m / (dd * dd))) * dtc);
    R[6] = R[6] / (1. + (6 * m * fphi / (dd * dd)) * dtc);
  } else if (p.turb != FEST_TURB_NONE) {
    double F1 = b.F1[c0];
    double beta = 0.075 * F1 + (1. - F1) * 0.0828;
    double w = b.qp[c0 + 6 * P];
    R[5] = R[5] / (1 + (beta * w * dtc));
    R[6] = R[6] / (1 + (2 * beta * w * dtc));
  }
  if (use_store) {
#pragma unroll
    for (int l = 0; l < NVMOD; ++l)
      if (l < nv) {
        double rn = b.Rstore[o + N * l] + SF * R[l];
        b.Rstore[o + N * l] = rn;
        if (TU) R[l] = rn;
      }
  }
  const double fac = (TF * dtc / b.cells[4 * c0]);
#pragma unroll
  for (int l = 0; l < NVMOD; ++l)
    if (l < nv) u2[l] = u1[l] - R[l] * fac;
#pragma unroll
  for (int l = 1; l < NVMOD; ++l)
    if (l < nv) u2[l] = u2[l] / u2[0];
  double s2 = u2[1] * u2[1] + u2[2] * u2[2] + u2[3] * u2[3];
  u2[4] = (gm - 1.) * u2[0] * (u2[4] - (0.5 * s2));
  bool bad = (u2[0] < 0.) || (u2[4] < 0.);
#pragma unroll
  for (int l = 0; l < NVMOD; ++l)
    if (l < nv) bad |= (u2[l] != u2[l]);
  if (bad) {
    raise_error(b.err, FEST_ERR_NEGATIVE_STATE);
    return;
  }
  for (int l = 0; l < 5; ++l) b.qp[c0 + P * l] = u2[l];
  if (sa) {
    b.qp[c0 + 5 * P] = fmax2(u2[5], 1.e-12);  // update.f90:474-475
  } else if (p.turb != FEST_TURB_NONE) {
    if (u2[5] >= 0.) b.qp[c0 + 5 * P] = u2[5];
    if (u2[6] >= 0.) b.qp[c0 + 6 * P] = u2[6];
  }
}

__global__ void k_blend(double* q, const double* u, long long n, double a, double c) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) q[t] = a * u[t] + c * q[t];
}

// resnorm partials (resnorm.f90:171-199): per thread-block sums, FP64
__global__ void k_resnorm_partial(Params p, DevBlock b, double* part, int nparts) {
  const Dims& d = p.d;
  __shared__ double sm[TPB];
  const long long N = ncells(d);
  double acc[NVMOD + 1];
  for (int l = 0; l <= NVMOD; ++l) acc[l] = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < N; t += (long long)gridDim.x * blockDim.x)
    for (int l = 0; l < d.nv; ++l) {
      double v = b.res[t + N * l];
      acc[1 + l] += v * v;
    }
  // mass imbalance through the block's boundary faces (resnorm.f90:190-197)
  FlDim fx = fldim(d, 0), fy = fldim(d, 1), fz = fldim(d, 2);
  const long long nI = (long long)(d.jmx - 1) * (d.kmx - 1), nJ = (long long)(d.imx - 1) * (d.kmx - 1),
                  nK = (long long)(d.imx - 1) * (d.jmx - 1);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nI + nJ + nK;
       t += (long long)gridDim.x * blockDim.x) {
    if (t < nI) {
      int j = 1 + (int)(t % (d.jmx - 1)), k = 1 + (int)(t / (d.jmx - 1));
      acc[0] += b.flux[0][flidx(fx, 1, j, k)] - b.flux[0][flidx(fx, d.imx, j, k)];
    } else if (t < nI + nJ) {
      long long u = t - nI;
      int i = 1 + (int)(u % (d.imx - 1)), k = 1 + (int)(u / (d.imx - 1));
      acc[0] += b.flux[1][flidx(fy, i, 1, k)] - b.flux[1][flidx(fy, i, d.jmx, k)];
    } else {
      long long u = t - nI - nJ;
      int i = 1 + (int)(u % (d.imx - 1)), j = 1 + (int)(u / (d.imx - 1));
      acc[0] += b.flux[2][flidx(fz, i, j, 1)] - b.flux[2][flidx(fz, i, j, d.kmx)];
    }
  }
  for (int l = 0; l <= d.nv; ++l) {
    sm[threadIdx.x] = acc[l];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x + (long long)nparts * l] = sm[0];
    __syncthreads();
  }
}
__global__ void k_resnorm_final(const double* part, int nparts, int nv, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int l = 0; l <= nv; ++l) {
    double s = 0.0;
    for (int i = 0; i < nparts; ++i) s += part[i + (long long)nparts * l];
    out[l] = s;
  }
}

// ---- geometry (grid.f90:137-236, geometry.f90:200-545) ----------------------
__device__ __forceinline__ double* node(const Dims& d, double* nd, int i, int j, int k) {
  return nd + 3 * (((long long)(k + 2) * (d.jmx + 6) + (j + 2)) * (d.imx + 6) + (i + 2));
}
__global__ void k_ghost_nodes(Params p, double* nd, int dir) {
  const Dims& d = p.d;
  const int n0 = (dir == 0 ? d.jmx : d.imx) + 6, n1 = (dir == 2 ? d.jmx : d.kmx) + 6;
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n0 * n1) return;
  const int a = -2 + (int)(t % n0), b = -2 + (int)(t / n0);
  const int n = extent_of(d, dir);
  auto N = [&](int c) -> double* {
    return dir == 0 ? node(d, nd, c, a, b) : dir == 1 ? node(d, nd, a, c, b) : node(d, nd, a, b, c);
  };
  for (int c = 0; c < 3; ++c) {
    N(0)[c] = 2 * N(1)[c] - N(2)[c];
    N(-1)[c] = 2 * N(0)[c] - N(1)[c];
    N(-2)[c] = 2 * N(-1)[c] - N(0)[c];
    N(n + 1)[c] = 2 * N(n)[c] - N(n - 1)[c];
    N(n + 2)[c] = 2 * N(n + 1)[c] - N(n)[c];
    N(n + 3)[c] = 2 * N(n + 2)[c] - N(n + 1)[c];
  }
}
__global__ void k_face_vectors(Params p, double* nd, double* faces, int dir) {
  const Dims& d = p.d;
  R3 r = r3(-2, d.imx + 2 + (dir == 0), -2, d.jmx + 2 + (dir == 1), -2, d.kmx + 2 + (dir == 2));
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const double *a1, *a0, *b1, *b0;
  if (dir == 0) { a1 = node(d, nd, i, j + 1, k + 1); a0 = node(d, nd, i, j, k); b1 = node(d, nd, i, j, k + 1); b0 = node(d, nd, i, j + 1, k); }
  else if (dir == 1) { a1 = node(d, nd, i + 1, j, k + 1); a0 = node(d, nd, i, j, k); b1 = node(d, nd, i + 1, j, k); b0 = node(d, nd, i, j, k + 1); }
  else { a1 = node(d, nd, i + 1, j + 1, k); a0 = node(d, nd, i, j, k); b1 = node(d, nd, i, j + 1, k); b0 = node(d, nd, i + 1, j, k); }
  double d1x = a1[0] - a0[0], d1y = a1[1] - a0[1], d1z = a1[2] - a0[2];
  double d2x = b1[0] - b0[0], d2y = b1[1] - b0[1], d2z = b1[2] - b0[2];
  double nx = 0.5 * (d1y * d2z - d1z * d2y);
  double ny = 0.5 * (d1z * d2x - d1x * d2z);
  double nz = 0.5 * (d1x * d2y - d1y * d2x);
  double A = sqrt(nx * nx + ny * ny + nz * nz);
  const int c = dir == 0 ? i : dir == 1 ? j : k, n = extent_of(d, dir);
  if ((p.id[2 * dir] == -7 && c <= 1) || (p.id[2 * dir + 1] == -7 && c >= n)) A = 0.;
  if (A != 0.) { nx = nx / A; ny = ny / A; nz = nz / A; }
  double* f = faces + 4 * fidx(d, dir, i, j, k);
  f[0] = A; f[1] = nx; f[2] = ny; f[3] = nz;
}
__global__ void k_pole_normals(Params p, double* If) {
  const Dims& d = p.d;
  R3 r = r3(-2, 1, -2, d.jmx + 2, -2, d.kmx + 2);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const double* s = If + 4 * fidx(d, 0, 2, j, k);
  double* f = If + 4 * fidx(d, 0, i, j, k);
  f[1] = s[1];
  f[2] = s[2];
}
__device__ double vol_tet(const double* p1, const double* p2, const double* p3, const double* p4) {
  double v = (p4[0] - p1[0]) * ((p2[1] - p1[1]) * (p3[2] - p1[2]) - (p2[2] - p1[2]) * (p3[1] - p1[1])) +
             (p4[1] - p1[1]) * ((p2[2] - p1[2]) * (p3[0] - p1[0]) - (p2[0] - p1[0]) * (p3[2] - p1[2])) +
             (p4[2] - p1[2]) * ((p2[0] - p1[0]) * (p3[1] - p1[1]) - (p2[1] - p1[1]) * (p3[0] - p1[0]));
  return -v / 6.;
}
__global__ void k_cells(Params p, double* nd, double* cells) {
  const Dims& d = p.d;
  R3 r = r3(-2, d.imx + 2, -2, d.jmx + 2, -2, d.kmx + 2);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const double* P[8] = {node(d, nd, i, j, k),         node(d, nd, i + 1, j, k),
                        node(d, nd, i + 1, j + 1, k), node(d, nd, i, j + 1, k),
                        node(d, nd, i, j, k + 1),     node(d, nd, i + 1, j, k + 1),
                        node(d, nd, i + 1, j + 1, k + 1), node(d, nd, i, j + 1, k + 1)};
  double vol = 1.;
  if (i >= 0 && i <= d.imx && j >= 0 && j <= d.jmx && k >= 0 && k <= d.kmx) {
    double v1 = 0.;
    v1 = v1 + vol_tet(P[0], P[4], P[7], P[5]);
    v1 = v1 + vol_tet(P[6], P[7], P[5], P[2]);
    v1 = v1 + vol_tet(P[7], P[3], P[0], P[2]);
    v1 = v1 + vol_tet(P[5], P[0], P[2], P[7]);
    v1 = v1 + vol_tet(P[0], P[1], P[5], P[2]);
    double v = 0.;
    v = v + vol_tet(P[1], P[5], P[4], P[6]);
    v = v + vol_tet(P[7], P[4], P[6], P[3]);
    v = v + vol_tet(P[4], P[0], P[1], P[3]);
    v = v + vol_tet(P[6], P[1], P[3], P[4]);
    v = v + vol_tet(P[1], P[2], P[6], P[3]);
    vol = fmax2(v, v1);
  }
  double* c = cells + 4 * pidx(d, i, j, k);
  c[0] = vol;
  for (int m = 0; m < 3; ++m) {
    double s = P[0][m] + P[1][m] + P[2][m] + P[6][m] + P[5][m] + P[3][m] + P[7][m] + P[4][m];
    c[1 + m] = 0.125 * s;
  }
}
// wall_dist.f90:96-129: nearest wall node per grid node (wall list tiled in smem)
__global__ void k_node_dist(Params p, const double* nd, const double* w, int nw, double* nd_dist) {
  const Dims& d = p.d;
  __shared__ double sw[3 * TPB];
  const long long Nn = (long long)(d.imx + 6) * (d.jmx + 6) * (d.kmx + 6);
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double x = 0, y = 0, z = 0;
  if (t < Nn) { x = nd[3 * t]; y = nd[3 * t + 1]; z = nd[3 * t + 2]; }
  double m = 1.e+20;
  for (int base = 0; base < nw; base += TPB) {
    int cnt = min(TPB, nw - base);
    __syncthreads();
    if ((int)threadIdx.x < cnt)
      for (int c = 0; c < 3; ++c) sw[3 * threadIdx.x + c] = w[3 * (base + threadIdx.x) + c];
    __syncthreads();
    for (int n = 0; n < cnt; ++n) {
      double dx = sw[3 * n] - x, dy = sw[3 * n + 1] - y, dz = sw[3 * n + 2] - z;
      m = fmin2(m, sqrt(dx * dx + dy * dy + dz * dz));
    }
  }
  if (t < Nn) nd_dist[t] = m;
}
__global__ void k_cell_dist(Params p, const double* nd_dist, double* dist) {
  const Dims& d = p.d;
  R3 r = r3(-2, d.imx + 2, -2, d.jmx + 2, -2, d.kmx + 2);
  int i, j, k;
  if (!decode(r, i, j, k)) return;
  const int n0 = d.imx + 6, n1 = d.jmx + 6;
  auto N = [&](int a, int b, int c) { return nd_dist[((long long)(c + 2) * n1 + (b + 2)) * n0 + (a + 2)]; };
  dist[pidx(d, i, j, k)] = 0.125 * (N(i, j, k) + N(i, j + 1, k) + N(i, j + 1, k + 1) + N(i, j, k + 1) +
                                    N(i + 1, j, k + 1) + N(i + 1, j, k) + N(i + 1, j + 1, k) +
                                    N(i + 1, j + 1, k + 1));
}

}  // namespace

// ============================================================================
bool ghosts_need_sequential(const Params& p) {
  int planes = 0;
  for (int f = 0; f < 6; ++f) {
    if (p.id[f] == -9) return true;
    if (p.id[f] == -8 || p.id[f] == -11) ++planes;
  }
  if (planes > 1) return true;
  // every BC reads at most interior layer 4 from its face; thinner blocks
  // read the opposite face's ghosts and need the reference's face order
  if (p.d.imx - 1 < 4 || p.d.jmx - 1 < 4 || p.d.kmx - 1 < 4) return true;
  return false;
}

bool ghost_depth_ok(const Params& p, bool stencil_only) {
  // interior layers each face's BC reads at an interior column
  // (bc_primitive.f90:160-206): copies 1, symmetric copies and tangency 3
  // (4 with the higher-order ghost term c3), interfaces 3, Riemann 1.
  // stencil_only: only ghost layer 1 of a face with a negative id other
  // than -10 reaches an interior update (the boundary face states are
  // overridden, boundary_state_reconstruction.f90:28-412, and ppm/weno
  // switch to MUSCL on the first interior cell), and symmetric layer 1
  // reads interior layers 1 (and 2 with c3)
  // A single interior layer under such a face (depth 2) is allowed there:
  // the face then reads the opposite face's ghost layer 1, which the mixed
  // path provides in the reference's order (low face from the previous
  // fill, high face after the low one).
  const int symm = stencil_only ? (p.c3 != 0.0 ? 2 : 1) : (p.c3 != 0.0 ? 4 : 3);
  for (int f = 0; f < 6; ++f) {
    const int id = p.id[f];
    int depth;
    switch (id) {
      case -1: depth = 0; break;
      case -2: case -3: case -4: case -7: case -8: case -11: depth = 1; break;
      case -5: case -6: depth = symm; break;
      case -9: return false;
      default: depth = 3;  // interfaces
    }
    const int n = extent_of(p.d, f / 2) - 1;
    if (n < depth && !(stencil_only && depth == 2 && n == 1)) return false;
  }
  return true;
}

void launch_ghosts(const Params& p, const DevBlock& b, const BlockRef* tab, int iter,
                   const Launcher& L, bool corners) {
  const Dims& d = p.d;
  int wmax = 0;
  for (int f = 0; f < 6; ++f) {
    int dir = f / 2;
    int na = (dir == 0 ? d.jmx : d.imx) - 1, nb = (dir == 2 ? d.jmx : d.kmx) - 1;
    wmax = max(wmax, (na + 6) * (nb + 6));
  }
  int mask_if = 0, mask_bc = 0;
  for (int f = 0; f < 6; ++f) {
    if (p.id[f] == -10 || p.id[f] >= 0) mask_if |= 1 << f;
    else mask_bc |= 1 << f;
  }
  dim3 g(nblk(wmax), 1, 6);
  if (ghosts_need_sequential(p)) {
    // apply_interface first (update.f90:534), then each face in order
    if (mask_if) {
      k_ghosts<<<g, TPB, 0, L.s>>>(p, b, tab, iter, mask_if);
      ++*L.count;
    }
    for (int f = 0; f < 6; ++f) {
      if (!((mask_bc >> f) & 1)) continue;
      k_ghosts<<<g, TPB, 0, L.s>>>(p, b, tab, iter, 1 << f);
      ++*L.count;
    }
  } else {
    k_ghosts<<<g, TPB, 0, L.s>>>(p, b, tab, iter, 63);
    ++*L.count;
  }
  if (!corners) return;
  k_corners<<<1, 256, 0, L.s>>>(p, b.qp);
  ++*L.count;
}

void launch_temperature(const Params& p, const DevBlock& b, const Launcher& L) {
  k_temperature<<<nblk(p.d.P), TPB, 0, L.s>>>(p, b.qp, b.Temp);
  ++*L.count;
}

void launch_face_states(const Params& p, const DevBlock& b, int mode, const Launcher& L) {
  const Dims& d = p.d;
  for (int dir = 0; dir < 3; ++dir) {
    long long n = (long long)(d.imx - 1 + 2 * (dir == 0)) * (d.jmx - 1 + 2 * (dir == 1)) *
                  (d.kmx - 1 + 2 * (dir == 2));
    k_face_states<<<nblk(n), TPB, 0, L.s>>>(p, b, dir, mode);
    ++*L.count;
  }
}

void launch_fluxes(const Params& p, const DevBlock& b, const Launcher& L) {
  const Dims& d = p.d;
  for (int dir = 0; dir < 3; ++dir) {
    FlDim fl = fldim(d, dir);
    if (dir == 2 && d.kmx == 2) {
      cudaMemsetAsync(b.flux[2], 0, sizeof(double) * fl.N * d.nv, L.s);
      continue;
    }
    k_fluxes<<<nblk(fl.N), TPB, 0, L.s>>>(p, b, dir);
    ++*L.count;
  }
}

void launch_gradients(const Params& p, const DevBlock& b, const Launcher& L) {
  const Dims& d = p.d;
  k_gradients<<<nblk(ngrad(d)), TPB, 0, L.s>>>(p, b);
  ++*L.count;
  int m = 0;
  for (int f = 0; f < 6; ++f) {
    int dir = f / 2;
    m = max(m, ((dir == 0 ? d.jmx : d.imx) - 1) * ((dir == 2 ? d.jmx : d.kmx) - 1));
  }
  k_gradient_bc<<<dim3(nblk(m), 1, 6), TPB, 0, L.s>>>(p, b);
  ++*L.count;
}

void launch_viscosity(const Params& p, const DevBlock& b, const Launcher& L) {
  const Dims& d = p.d;
  k_viscosity<<<nblk(ngrad(d)), TPB, 0, L.s>>>(p, b);
  ++*L.count;
  if (p.turb != FEST_TURB_NONE) {
    int m = 0;
    for (int f = 0; f < 6; ++f) {
      int dir = f / 2;
      m = max(m, ((dir == 0 ? d.jmx : d.imx) - 1) * ((dir == 2 ? d.jmx : d.kmx) - 1));
    }
    k_viscosity_ghost<<<dim3(nblk(m), 1, 6), TPB, 0, L.s>>>(p, b);
    ++*L.count;
  }
}

void launch_viscous_fluxes(const Params& p, const DevBlock& b, const Launcher& L) {
  for (int dir = 0; dir < 3; ++dir) {
    FlDim fl = fldim(p.d, dir);
    k_viscous<<<nblk(fl.N), TPB, 0, L.s>>>(p, b, dir);
    ++*L.count;
  }
}

void launch_residue(const Params& p, const DevBlock& b, bool with_source, const Launcher& L) {
  k_residue<<<nblk(ncells(p.d)), TPB, 0, L.s>>>(p, b);
  ++*L.count;
  if (with_source) launch_source(p, b, L);
}

void launch_source(const Params& p, const DevBlock& b, const Launcher& L) {
  if (p.turb == FEST_TURB_NONE) return;
  k_source<<<nblk(ncells(p.d)), TPB, 0, L.s>>>(p, b);
  ++*L.count;
}

void launch_time_step(const Params& p, const DevBlock& b, double CFL, const Launcher& L) {
  // compute_time_step (time.f90:291-334): 'l' local, 'g' a fixed global
  // step when given, else the block's minimum local step
  const long long N = ncells(p.d);
  const bool global = p.tstep == 'g';
  int parts = (int)std::min<long long>(1024, (long long)nblk(N));
  if (global && p.gdt > 0) {
    k_fill_min<<<parts, TPB, 0, L.s>>>(b.dt, N, b.red, 0, p.gdt);
    ++*L.count;
    return;
  }
  k_time_step<<<nblk(N), TPB, 0, L.s>>>(p, b, CFL);
  ++*L.count;
  if (global) {
    k_min_partial<<<parts, TPB, 0, L.s>>>(b.dt, N, b.red);
    k_fill_min<<<parts, TPB, 0, L.s>>>(b.dt, N, b.red, parts, -1.0);
    *L.count += 2;
  }
}

void launch_update(const Params& p, const DevBlock& b, double TF, double SF, int TU, int use_store,
                   const Launcher& L) {
  k_update<<<nblk(ncells(p.d)), TPB, 0, L.s>>>(p, b, TF, SF, TU, use_store);
  ++*L.count;
}

void launch_blend(const Params& p, const DevBlock& b, double a, double c, const Launcher& L) {
  long long n = p.d.P * p.d.nv;
  k_blend<<<nblk(n), TPB, 0, L.s>>>(b.qp, b.Ustore, n, a, c);
  ++*L.count;
}

void launch_resnorm(const Params& p, const DevBlock& b, double* d_out, const Launcher& L) {
  int parts = 512;
  k_resnorm_partial<<<parts, TPB, 0, L.s>>>(p, b, b.red, parts);
  k_resnorm_final<<<1, 32, 0, L.s>>>(b.red, parts, p.d.nv, d_out);
  *L.count += 2;
}

void launch_geometry(const Params& p, const DevBlock& b, const Launcher& L) {
  const Dims& d = p.d;
  for (int dir = 0; dir < 3; ++dir) {
    long long n = (long long)((dir == 0 ? d.jmx : d.imx) + 6) * ((dir == 2 ? d.jmx : d.kmx) + 6);
    k_ghost_nodes<<<nblk(n), TPB, 0, L.s>>>(p, b.nodes, dir);
    ++*L.count;
  }
  for (int dir = 0; dir < 3; ++dir) {
    k_face_vectors<<<nblk(nfaces(d, dir)), TPB, 0, L.s>>>(p, b.nodes, b.faces[dir], dir);
    ++*L.count;
  }
  if (p.id[0] == -7) {
    k_pole_normals<<<nblk((long long)4 * (d.jmx + 5) * (d.kmx + 5)), TPB, 0, L.s>>>(p, b.faces[0]);
    ++*L.count;
  }
  k_cells<<<nblk(d.P), TPB, 0, L.s>>>(p, b.nodes, b.cells);
  ++*L.count;
}

void launch_wall_dist(const Params& p, const DevBlock& b, const double* d_wall, int n_wall,
                      double* d_node_dist, const Launcher& L) {
  const Dims& d = p.d;
  long long Nn = (long long)(d.imx + 6) * (d.jmx + 6) * (d.kmx + 6);
  k_node_dist<<<nblk(Nn), TPB, 0, L.s>>>(p, b.nodes, d_wall, n_wall, d_node_dist);
  k_cell_dist<<<nblk(d.P), TPB, 0, L.s>>>(p, d_node_dist, b.dist);
  *L.count += 2;
}

}  // namespace fest
