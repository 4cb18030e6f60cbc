// fest_fused.cu - host side of the fused fast path: ping-pong state buffers,
// per-stage ghost fills, the integrators' stage schedule (update.f90:129-226)
// and the stage-sweep launches (kernels in fest_stage.cuh).
#include <algorithm>
#include <vector>

#include "fest_fused.cuh"
#include "fest_stage.cuh"

namespace fest {

namespace {

using namespace stage;

// TVD blends of the reference run over the whole padded block
// (update.f90:203-206), ghosts included; the blended ghosts matter where
// BCs stop rewriting them (fix() after iteration 2).  Non-interior cells:
// q = a*Us + b*X with Us the state before the iteration's BCs and X the last
// stage's input (its ghosts as that stage's BCs left them).
__global__ void k_ghost_blend(Dims d, double* q, float* q32, int pitch, const double* Us,
                              const double* X, double a, double b) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.P * d.nv) return;
  long long c = t % d.P;
  int i = (int)(c % d.ni) - 2;
  long long r = c / d.ni;
  int j = (int)(r % d.nj) - 2, k = (int)(r / d.nj) - 2;
  bool interior = i >= 1 && i <= d.imx - 1 && j >= 1 && j <= d.jmx - 1 && k >= 1 && k <= d.kmx - 1;
  if (interior) return;
  const double v = a * Us[t] + b * X[t];
  q[t] = v;
  if (q32) q32[mirror_index(d, pitch, c, (int)(t / d.P))] = (float)v;
}

// FP32 mirrors for the mixed sweep: state (whole padded array), face
// records {A,nx,ny,nz} and cell volumes.  Rounding to nearest, as a
// conversion on load would do.
// one row (j, k, variable) of the padded array per block (rows in the x
// dimension of the grid, which has no 65535 limit)
__global__ void k_to_mirror(Dims d, int pitch, const double* src, float* dst) {
  const long long row = blockIdx.x;  // (j + 2) + nj*((k + 2) + nk*l)
  for (int i = threadIdx.x; i < d.ni; i += blockDim.x) dst[row * pitch + i] = (float)src[row * d.ni + i];
}
__global__ void k_faces_to_f32(const double* faces, float4* dst, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double* f = faces + 4 * t;
    dst[t] = make_float4((float)f[0], (float)f[1], (float)f[2], (float)f[3]);
  }
}
__global__ void k_cells_to_f32(const double* cells, float4* dst, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double* c = cells + 4 * t;
    dst[t] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)c[3]);
  }
}
__global__ void k_dist_to_f32(const double* src, float* dst, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = (float)src[t];
}
__global__ void k_vol_to_f32(const double* cells, float* dst, long long n) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    dst[t] = (float)cells[4 * t];
}
// ---- ghost cells on the FP32 mirror (mixed sweep, iterations > 2) ----------
// The same face procedures as the FP64 ghost fill (bc_primitive.f90:160-206,
// copy_bc.f90:58-131, FT_bc.f90:15-107, bc_primitive.f90:1237-1776,
// interface1.f90:496-700), evaluated in FP32 on the mirror that the mixed
// sweep reads.  After iteration 2 no fix() BC writes anything
// (bc_primitive.f90:236,318,366), so only the copy, wall, tangency, Riemann
// and interface procedures remain.  One thread per interior column of a
// face; on the fused path every one of them reads interior cells only
// (blocks have >= 4 interior cells per direction, no -9 faces) and writes
// its own ghost cells, so the faces run concurrently.
struct Mirror {
  float* q;
  int rp, nj, nk;
  long long vs;
  __device__ __forceinline__ float& at(int i, int j, int k, int l) const {
    return q[(i + 2) + (long long)rp * ((j + 2) + (long long)nj * (k + 2)) + vs * l];
  }
};
struct GhostPlan {
  int nf;
  int face[6];
  int na[6];
  long long start[7];
};
// ghost (layer L) and interior (layer m) cell of face f at (ta, tb)
__device__ __forceinline__ void gcell(const Dims& d, int f, int L, int ta, int tb, int& i, int& j, int& k) {
  switch (f) {
    case 0: i = 1 - L; j = ta; k = tb; break;
    case 1: i = d.imx + L - 1; j = ta; k = tb; break;
    case 2: i = ta; j = 1 - L; k = tb; break;
    case 3: i = ta; j = d.jmx + L - 1; k = tb; break;
    case 4: i = ta; j = tb; k = 1 - L; break;
    default: i = ta; j = tb; k = d.kmx + L - 1;
  }
}
__device__ __forceinline__ void icell(const Dims& d, int f, int m, int ta, int tb, int& i, int& j, int& k) {
  switch (f) {
    case 0: i = m; j = ta; k = tb; break;
    case 1: i = d.imx - m; j = ta; k = tb; break;
    case 2: i = ta; j = m; k = tb; break;
    case 3: i = ta; j = d.jmx - m; k = tb; break;
    case 4: i = ta; j = tb; k = m; break;
    default: i = ta; j = tb; k = d.kmx - m;
  }
}

// Riemann-invariant ghost state of column (ta, tb) of face f from its
// interior layer 1; returns the boundary normal velocity Unb
__device__ __forceinline__ float riemann_mirror(const Params& p, const Mirror& M, int f, int ta, int tb,
                                                const float4* Fd, float& rg, float& ug, float& vg, float& wg,
                                                float& pg) {
  const Dims& d = p.d;
  auto I = [&](int m, int l) -> float { int i, j, k; icell(d, f, m, ta, tb, i, j, k); return M.at(i, j, k, l); };
  int fi, fj, fk;
  {
    const int c = (f % 2 == 0) ? 1 : extent_of(d, f / 2);
    if (f / 2 == 0) { fi = c; fj = ta; fk = tb; }
    else if (f / 2 == 1) { fi = ta; fj = c; fk = tb; }
    else { fi = ta; fj = tb; fk = c; }
  }
  const float4 fc = __ldg(Fd + fidx(d, f / 2, fi, fj, fk));
  return riemann_ghost_f32(p, f, fc, I(1, 1), I(1, 2), I(1, 3), I(1, 4), I(1, 0), rg, ug, vg, wg, pg);
}

// dist: the FP64 wall distance (padded), read by the SST wall's omega;
// PM, pd: the mirror and extents of the block an interface face pairs with
// (this block's own for a face paired with the block itself)
__device__ __forceinline__ void ghost_mirror_column(const Params& p, const Mirror& M, int f, int ta, int tb,
                                                    const float4* F0, const float4* F1,
                                                    const float4* F2, const double* dist, const Mirror& PM,
                                                    const Dims& pd) {
  const Dims& d = p.d;
  const int id = p.id[f];
  const bool sst = d.nv == 7;
  auto G = [&](int L, int l) -> float& { int i, j, k; gcell(d, f, L, ta, tb, i, j, k); return M.at(i, j, k, l); };
  auto I = [&](int m, int l) -> float { int i, j, k; icell(d, f, m, ta, tb, i, j, k); return M.at(i, j, k, l); };
  const float c1 = (float)p.c1, c2 = (float)p.c2, c3 = (float)p.c3;
  auto flat = [&](int l) { const float v = I(1, l); for (int L = 1; L <= 3; ++L) G(L, l) = v; };
  auto symm = [&](int l) { for (int L = 1; L <= 3; ++L) G(L, l) = (c2 * I(L, l) - c3 * I(L + 1, l)) / c1; };
  auto anti = [&](int l) { for (int L = 1; L <= 3; ++L) G(L, l) = -I(L, l); };
  const float gm = (float)p.gm, R = (float)p.R;
  // boundary face record of this column
  int fi, fj, fk;
  {
    const int c = (f % 2 == 0) ? 1 : extent_of(d, f / 2);
    if (f / 2 == 0) { fi = c; fj = ta; fk = tb; }
    else if (f / 2 == 1) { fi = ta; fj = c; fk = tb; }
    else { fi = ta; fj = tb; fk = c; }
  }
  const float4* Fd = f / 2 == 0 ? F0 : (f / 2 == 1 ? F1 : F2);
  switch (id) {
    case -1: break;  // supersonic inlet: fix() only
    case -2:
    case -7:
      for (int l = 0; l < d.nv; ++l) flat(l);
      break;
    case -3: flat(4); break;      // subsonic inlet: pressure copied (fix() for the rest)
    case -4:                      // subsonic outlet: rho,u,v,w (and k, omega) copied (fix() for p)
      for (int l = 0; l < 4; ++l) flat(l);
      if (sst) { flat(5); flat(6); }
      break;
    case -5: {  // wall (bc_primitive.f90:392-402)
      symm(4);
      const float Tw = (float)p.Tw[f];
      if (Tw < 0.f) {  // temp_based_density (bc_primitive.f90:1778-1945)
        const float pp = I(1, 4), rho = I(1, 0);
        const float stag = (pp / (R * rho)) * (1.f + (0.5f * (gm - 1.f) * gm * pp / rho));
        for (int L = 1; L <= 3; ++L) G(L, 0) = G(L, 4) / (R * stag);
      } else if (Tw > 1.f) {
        for (int L = 1; L <= 3; ++L) {
          const float Ti = I(L, 4) / (R * I(L, 0));
          G(L, 0) = G(L, 4) / (R * (2.f * Tw - Ti));
        }
      } else {
        symm(0);
      }
      anti(1); anti(2); anti(3);
      if (sst) {
        anti(5);
        // set_omega_at_wall (bc_primitive.f90:564-643): omega from the
        // Sutherland viscosity at the face temperature and twice the first
        // cell's wall distance
        int i1, j1, k1;
        icell(d, f, 1, ta, tb, i1, j1, k1);
        const float Tf = 0.5f * ((G(1, 4) / G(1, 0)) + (I(1, 4) / I(1, 0))) / R;
        const float Tr = (float)p.T_ref, S = (float)p.S;
        const float mu = (float)p.mu_ref * powf(Tf / Tr, 1.5f) * ((Tr + S) / (Tf + S));
        const float rho = 0.5f * (G(1, 0) + I(1, 0));
        const float dd = 2.f * (float)dist[pidx(d, i1, j1, k1)];
        const float om = 120.f * mu / (rho * 0.075f * (dd * dd));
        for (int L = 1; L <= 3; ++L) G(L, 6) = om - I(L, 6);
      }
    } break;
    case -6: {  // slip wall + flow tangency with I-face normals (FT_bc.f90:67-69)
      symm(0); symm(4);
      if (sst) { symm(5); symm(6); }
      const float4 fn = __ldg(Fd + fidx(d, f / 2, fi, fj, fk));
      const float4 fr = __ldg(F0 + fidx(d, 0, fi, fj, fk));
      for (int L = 1; L <= 3; ++L) {
        const float uu = I(L, 1), vv = I(L, 2), ww = I(L, 3);
        const float dot = uu * fn.y + vv * fn.z + ww * fn.w;
        G(L, 1) = uu - (2.f * dot * fr.y);
        G(L, 2) = vv - (2.f * dot * fr.z);
        G(L, 3) = ww - (2.f * dot * fr.w);
      }
    } break;
    case -8:
    case -11: {  // Riemann invariants on layer 1, copied to layers 2-3
      float rg, ug, vg, wg, pg;
      riemann_mirror(p, M, f, ta, tb, Fd, rg, ug, vg, wg, pg);
      for (int L = 1; L <= 3; ++L) {
        G(L, 0) = rg; G(L, 1) = ug; G(L, 2) = vg; G(L, 3) = wg; G(L, 4) = pg;
      }
      if (sst) {
        // k and omega follow the direction of the face's last column
        // (the loop variable the reference tests after its loop)
        const int na = (f / 2 == 0 ? d.jmx : d.imx) - 1, nb = (f / 2 == 2 ? d.jmx : d.kmx) - 1;
        float r2, u2, v2, w2, p2;
        const float Ulast = riemann_mirror(p, M, f, na, nb, Fd, r2, u2, v2, w2, p2);
        if (Ulast > 0.f) {
          flat(5); flat(6);
        } else {
          for (int L = 1; L <= 3; ++L) { G(L, 5) = (float)p.fix_tk[f]; G(L, 6) = (float)p.fix_tw[f]; }
        }
      }
    } break;
    default:
      if (id == -10 || id >= 0) {  // interface: ghost L <- layer L of the partner face
        const int pf = p.part_face[f];
        int na, nb, pa, pb;
        face_columns(d, f, na, nb);
        interface_map(p.part_orient[f], na, nb, ta, tb, pa, pb);
        for (int l = 0; l < d.nv; ++l)
          for (int L = 1; L <= 3; ++L) {
            int i, j, k;
            icell(pd, pf, L, pa, pb, i, j, k);
            G(L, l) = PM.at(i, j, k, l);
          }
      }
  }
}

// tab: the block table of the stage's input buffer (interface partners in
// other blocks of a batch, read through their FP32 mirrors)
__global__ void __launch_bounds__(128) k_ghosts_mirror(Params p, Mirror M, GhostPlan plan,
                                                       const float4* F0, const float4* F1,
                                                       const float4* F2, const double* dist,
                                                       const BlockRef* tab) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= plan.start[plan.nf]) return;
  int n = 0;
  while (t >= plan.start[n + 1]) ++n;
  const long long u = t - plan.start[n];
  const int f = plan.face[n];
  Mirror PM = M;
  Dims pd = p.d;
  if ((p.id[f] == -10 || p.id[f] >= 0) && p.part_block[f] != p.self_block) {
    const BlockRef& r = tab[p.part_block[f]];
    PM = Mirror{r.b.qp32, r.b.qp32_pitch, r.d.nj, r.d.nk, (long long)r.b.qp32_pitch * r.d.nj * r.d.nk};
    pd = r.d;
  }
  ghost_mirror_column(p, M, f, 1 + (int)(u % plan.na[n]), 1 + (int)(u / plan.na[n]), F0, F1, F2, dist, PM, pd);
}

// one (block, face) segment of a batched mirror ghost fill
struct GhostSeg {
  long long start;  // first thread of the segment
  int block, face, na;
  Mirror M;
  const float4* F[3];
  const double* dist;
  Mirror PM;        // the interface partner's mirror (interface faces)
  Dims pd;          // and its extents
};
__global__ void __launch_bounds__(128) k_ghosts_mirror_batch(const Params* ps, const GhostSeg* seg, int nseg,
                                                             long long total) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  int lo = 0, hi = nseg - 1;  // last segment with start <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) / 2;
    if (seg[mid].start <= t) lo = mid;
    else hi = mid - 1;
  }
  const GhostSeg& g = seg[lo];
  const long long u = t - g.start;
  ghost_mirror_column(ps[g.block], g.M, g.face, 1 + (int)(u % g.na), 1 + (int)(u / g.na), g.F[0], g.F[1],
                      g.F[2], g.dist, g.PM, g.pd);
}

// the edge and corner averaging of the reference on an FP32 mirror (one CTA)
__global__ void k_corners_mirror(Dims d, Mirror M) {
  corner_average<float>(d, [&](int i, int j, int k, int l) -> float& { return M.at(i, j, k, l - 1); });
}

// copy ghost layers 1-3 of face f (interior columns, every variable) from
// one mirror (and FP64 buffer, when q is given) to the two others
__global__ void k_ghost_bcast(Dims d, int f, int na, int nb, Mirror src, Mirror d1, Mirror d2, const double* q,
                              double* q1, double* q2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)na * nb * 3 * d.nv) return;
  const int ta = 1 + (int)(t % na), tb = 1 + (int)((t / na) % nb);
  const int L = 1 + (int)((t / ((long long)na * nb)) % 3), l = (int)(t / (3ll * na * nb));
  int i, j, k;
  gcell(d, f, L, ta, tb, i, j, k);
  const float v = src.at(i, j, k, l);
  d1.at(i, j, k, l) = v;
  d2.at(i, j, k, l) = v;
  if (q) {
    const long long c = pidx(d, i, j, k) + d.P * l;
    q1[c] = q[c];
    q2[c] = q[c];
  }
}

unsigned grid_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 152 * 16); }

__device__ __forceinline__ bool is_interior(const Dims& d, long long t) {
  const int i = (int)(t % d.ni) - 2, j = (int)((t / d.ni) % d.nj) - 2, k = (int)(t / ((long long)d.ni * d.nj)) - 2;
  return i >= 1 && i <= d.imx - 1 && j >= 1 && j <= d.jmx - 1 && k >= 1 && k <= d.kmx - 1;
}
// The temperature the reference's gradients use in an iteration
// (update.f90:170: p/(R rho) of its state at the iteration's start): the
// interior from the current buffer q; the ghost cells from G, the ghost
// values the reference's state carries then (the previous iteration's last
// BC fill, TVD-blended like the whole array, update.f90:196-214)
__global__ void k_temp_start(Dims d, double R, const double* q, const double* G, double* Temp) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.P) return;
  const double* s = is_interior(d, t) ? q : G;
  Temp[t] = s[t + 4 * d.P] / (R * s[t]);
}
// the reference's ghost values after an iteration: X, the last stage's
// input with that stage's BC fill, blended with the previous ones by the
// TVD integrators (G = bA G + bB X), taken as they are by the others
__global__ void k_gref(Dims d, double* G, const double* X, double bA, double bB, int blend) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.P * d.nv) return;
  if (is_interior(d, t % d.P)) return;
  G[t] = blend ? bA * G[t] + bB * X[t] : X[t];
}

}  // namespace

struct FusedState {
  Dims d;
  double* Q[3] = {nullptr, nullptr, nullptr};  // Q[0] is the handle's qp
  double* Us = nullptr;  // state at the start of a TVD iteration (<= 2)
  // FP64 viscous sweeps: the ghost values of the reference's state at the
  // iteration's start, for the temperature of its gradients
  double* Gref = nullptr;
  bool gref_valid = false;
  BlockRef* table[3] = {nullptr, nullptr, nullptr};
  int cur = 0;       // buffer holding the current state
  bool seeded = false;
  // mixed sweep: FP32 mirrors of the three state buffers and of the metrics
  float* Q32[3] = {nullptr, nullptr, nullptr};
  float4* F32[3] = {nullptr, nullptr, nullptr};
  float* V32 = nullptr;
  float4* C32 = nullptr;  // {volume, cx, cy, cz} for the viscous sweep
  float* D32 = nullptr;   // wall distance for the SST sweep
  bool visc = false;
  bool turb = false;
  bool mirror_valid = false;  // Q32 interiors match Q
  bool buffers_equal = false;  // Q[0..2] hold the same state (just seeded)
  int kc[2] = {0, 0};         // tuned k-chunk per precision (0: not tuned yet)
  int occ[2] = {1, 2};        // tuned register budget (CTAs per SM) per precision
  int mpitch = 0;             // row pitch of Q32
  long long m_elems = 0;      // floats per Q32 buffer
  CUtensorMap tm[3];          // TMA descriptors of Q32[0..2]
  CUtensorMap tm_none{};      // placeholder for FP64 launches
  // captured iterations (see graph_for)
  struct Graph {
    int prec;
    double CFL;
    bool last;
    int cur;
    cudaGraphExec_t exec;
    int kernels;
  };
  std::vector<Graph> graphs;
  bool use_graphs = true;
  int* tune_err = nullptr;    // error word of the tuning launches
  std::vector<void*> allocs;
  bool profiling = false;
  std::vector<cudaEvent_t> ev;  // start/end pairs of profiled launches
  size_t nev = 0;               // events in use
};

// Directions whose ghost fill depends on the order of the faces: a single
// interior layer under a symmetric face (-5, -6) with the higher-order term
// c3, whose ghost layer 1 then reads the opposite face's ghost layer 1.  The
// reference fills its faces in place, low face first: the low face reads
// the high face's previous fill, the high face the low face's new one.
static int order_dirs(const Params& p) {
  if (p.c3 == 0.0) return 0;
  int m = 0;
  for (int dir = 0; dir < 3; ++dir) {
    if (extent_of(p.d, dir) - 1 != 1) continue;
    for (int s = 0; s < 2; ++s) {
      const int id = p.id[2 * dir + s];
      if (id == -5 || id == -6) m |= 1 << dir;
    }
  }
  return m;
}

static Mirror mirror_of(FusedState* f, int buf) {
  const Dims& d = f->d;
  return Mirror{f->Q32[buf], f->mpitch, d.nj, d.nk, (long long)f->mpitch * d.nj * d.nk};
}

// Faces whose ghosts the FP32 sweep makes itself after iteration 2 (bit f
// of the result: ghost layer 1 from the staged interior cells, the only
// layer an interior update reads for these faces) and k-interfaces served
// by remapped TMA planes (*kper bit 0: kmin, bit 1: kmax).  The rest (i/j
// interfaces, order-dependent directions, SST far-field faces) keep the
// FP32 ghost-fill kernel; -1 faces need nothing after iteration 2.
static int ring_faces(const Params& p, int* kper) {
  const int od = order_dirs(p);
  const bool sst = p.turb != FEST_TURB_NONE;
  int m = 0;
  *kper = 0;
  for (int f = 0; f < 6; ++f) {
    const int id = p.id[f];
    if ((od >> (f / 2)) & 1) continue;
    switch (id) {
      case -2: case -3: case -4: case -5: case -6: case -7: m |= 1 << f; break;
      case -8: case -11: if (!sst) m |= 1 << f; break;
      default:
        if ((id == -10 || id >= 0) && f / 2 == 2 && p.part_face[4] == 5 && p.part_face[5] == 4 &&
            p.part_block[4] == p.self_block && p.part_block[5] == p.self_block && p.part_orient[4] == 0 &&
            p.part_orient[5] == 0)
          *kper |= 1 << (f - 4);
    }
  }
  return m;
}

bool fused_supported(const Params& p, int precision) {
  // ping-pong buffers keep each stage's ghosts in its own input buffer; BC
  // sets that read another face's ghosts (blocks thinner than a BC's read
  // depth, -9) need the in-place module path.  Only ghost layer 1 of a
  // boundary face (and layers 1-3 of an interface) reaches an interior
  // update (ghost_depth_ok with stencil_only); directions whose layer-1 fill
  // depends on the face order are reproduced by the mixed path only.
  // the sweep addresses one plane's stencil with 32-bit offsets
  const bool mixed = precision == FEST_MIXED;
  const bool small_enough = (long long)p.d.P * p.d.nv < (1ll << 31);
  const bool sst = p.turb == FEST_TURB_SST || p.turb == FEST_TURB_SST2003;
  const bool model = p.turb == FEST_TURB_NONE ? p.d.nv == 5
                                               : (sst && p.mu_ref != 0.0 && p.d.nv == 7 &&
                                                  p.transition == FEST_TRANSITION_NONE);
  // the TVD integrators blend ghosts between fills, which order-dependent
  // directions would read; they take the module path
  const bool tvd = p.integ == FEST_TIME_TVDRK2 || p.integ == FEST_TIME_TVDRK3;
  const bool order_ok = mixed ? (order_dirs(p) == 0 || !tvd) : order_dirs(p) == 0;
  // the implicit integrator runs on the module path
  return p.integ <= FEST_TIME_TVDRK3 && model && p.tstep == 'l' && ghost_depth_ok(p, true) && order_ok &&
         small_enough;
}

int fused_create(const Params& p, const DevBlock& b, const BlockRef* table, cudaStream_t s,
                 FusedState** out) {
  (void)table;
  *out = nullptr;
  if (!fused_supported(p, FEST_MIXED)) return FEST_ERR_ARG;
  FusedState* f = new FusedState();
  f->d = p.d;
  f->visc = p.mu_ref != 0.0;
  f->turb = p.turb != FEST_TURB_NONE;
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
  if (p.mu_ref != 0.0) {
    if (cudaMalloc((void**)&f->Gref, bytes) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
    f->allocs.push_back(f->Gref);
  }
  if (cudaMalloc((void**)&f->tune_err, sizeof(int)) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
  f->allocs.push_back(f->tune_err);
  cudaMemsetAsync(f->tune_err, 0, sizeof(int), s);
  for (int n = 0; n < 3; ++n) {
    BlockRef ref{b, p.d};
    ref.b.qp = f->Q[n];
    if (cudaMalloc((void**)&f->table[n], sizeof(BlockRef)) != cudaSuccess) { fused_destroy(f); return FEST_ERR_NOMEM; }
    f->allocs.push_back(f->table[n]);
    cudaMemcpyAsync(f->table[n], &ref, sizeof(BlockRef), cudaMemcpyHostToDevice, s);
  }
  *out = f;
  return FEST_OK;
}

void fused_destroy(FusedState* f) {
  if (!f) return;
  for (cudaEvent_t e : f->ev) cudaEventDestroy(e);
  for (auto& g : f->graphs) cudaGraphExecDestroy(g.exec);
  for (void* x : f->allocs) cudaFree(x);
  delete f;
}

void fused_invalidate(FusedState* f) {
  if (f) { f->cur = 0; f->seeded = false; f->gref_valid = false; }
}

// copy the full padded state of buffer `from` into the others so ghost
// values that the BCs write only early (fix() at iter<=2) exist everywhere
static void seed(FusedState* f, cudaStream_t s) {
  size_t bytes = sizeof(double) * (size_t)f->d.P * f->d.nv;
  for (int n = 0; n < 3; ++n)
    if (n != f->cur) cudaMemcpyAsync(f->Q[n], f->Q[f->cur], bytes, cudaMemcpyDeviceToDevice, s);
  f->seeded = true;
  f->mirror_valid = false;
  f->buffers_equal = true;
}

// allocate and fill the FP32 mirrors the mixed sweep reads (once per
// handle for the metrics; the state mirror whenever it went stale)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 4-D view (i, j, k, variable) of one FP32 state mirror; box = one stencil
// plane of a tile (40 x 12 x 1 x n_var).  Out-of-range elements read as zero.
static int encode_mirror_map(CUtensorMap* tm, float* base, const Dims& d, int pitch) {
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return FEST_ERR_CUDA;
    encode = (EncodeTiledFn)fn;
  }
  const cuuint64_t dims[4] = {(cuuint64_t)d.ni, (cuuint64_t)d.nj, (cuuint64_t)d.nk, (cuuint64_t)d.nv};
  const cuuint64_t strides[3] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * d.nj * 4,
                                 (cuuint64_t)pitch * d.nj * d.nk * 4};
  const cuuint32_t box[4] = {(cuuint32_t)RingGeom<float>::W, (cuuint32_t)SH, 1, (cuuint32_t)d.nv};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? FEST_OK : FEST_ERR_CUDA;
}

static int ensure_mirrors(FusedState* f, const DevBlock& b, cudaStream_t s, long long* cnt) {
  const Dims& d = f->d;
  if (!f->V32) {  // V32 is allocated last: a partial earlier attempt retries
    f->mpitch = (d.ni + 3) & ~3;
    f->m_elems = (long long)f->mpitch * d.nj * d.nk * d.nv;
    for (int m = 0; m < 3; ++m) {
      if (cudaMalloc((void**)&f->Q32[m], sizeof(float) * (size_t)f->m_elems) != cudaSuccess)
        return FEST_ERR_NOMEM;
      f->allocs.push_back(f->Q32[m]);
      int rc = encode_mirror_map(&f->tm[m], f->Q32[m], d, f->mpitch);
      if (rc) return rc;
      const long long nf = nfaces(d, m);
      if (cudaMalloc((void**)&f->F32[m], sizeof(float4) * (size_t)nf) != cudaSuccess) return FEST_ERR_NOMEM;
      f->allocs.push_back(f->F32[m]);
      k_faces_to_f32<<<grid_for(nf), 256, 0, s>>>(b.faces[m], f->F32[m], nf);
      ++*cnt;
    }
    if (cudaMalloc((void**)&f->V32, sizeof(float) * (size_t)d.P) != cudaSuccess) return FEST_ERR_NOMEM;
    f->allocs.push_back(f->V32);
    k_vol_to_f32<<<grid_for(d.P), 256, 0, s>>>(b.cells, f->V32, d.P);
    ++*cnt;
    if (f->visc) {
      if (cudaMalloc((void**)&f->C32, sizeof(float4) * (size_t)d.P) != cudaSuccess) return FEST_ERR_NOMEM;
      f->allocs.push_back(f->C32);
      k_cells_to_f32<<<grid_for(d.P), 256, 0, s>>>(b.cells, f->C32, d.P);
      ++*cnt;
    }
    if (f->turb) {
      if (cudaMalloc((void**)&f->D32, sizeof(float) * (size_t)d.P) != cudaSuccess) return FEST_ERR_NOMEM;
      f->allocs.push_back(f->D32);
      k_dist_to_f32<<<grid_for(d.P), 256, 0, s>>>(b.dist, f->D32, d.P);
      ++*cnt;
    }
    f->mirror_valid = false;
  }
  if (!f->mirror_valid) {
    // whole padded arrays, so that the edge and corner cells the halo lanes
    // read (results discarded) hold finite values
    // (pitch padding columns are outside the tensor map: never read); equal
    // FP64 buffers share one conversion
    const unsigned g = (unsigned)((long long)d.nj * d.nk * d.nv);
    for (int m = 0; m < 3; ++m) {
      if (m > 0 && f->buffers_equal) {
        cudaMemcpyAsync(f->Q32[m], f->Q32[0], sizeof(float) * (size_t)f->m_elems, cudaMemcpyDeviceToDevice, s);
        continue;
      }
      k_to_mirror<<<g, 128, 0, s>>>(d, f->mpitch, f->Q[m], f->Q32[m]);
      ++*cnt;
    }
    f->mirror_valid = true;
  }
  return FEST_OK;
}

static void launch_sweep(const Params& p, int prec, int occ, dim3 grid, cudaStream_t s, const StageArgs& a,
                         const CUtensorMap& tm) {
  if (p.turb != FEST_TURB_NONE) {
    switch (p.interp) {
      case FEST_INTERP_NONE: launch_stage_none_sst(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_MUSCL: launch_stage_muscl_sst(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_PPM: launch_stage_ppm_sst(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_WENO: launch_stage_weno_sst(prec, p.flux, occ, grid, s, p, a, tm); break;
      default: launch_stage_weno_nm_sst(prec, p.flux, occ, grid, s, p, a, tm); break;
    }
    return;
  }
  if (p.mu_ref != 0.0) {
    switch (p.interp) {
      case FEST_INTERP_NONE: launch_stage_none_visc(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_MUSCL: launch_stage_muscl_visc(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_PPM: launch_stage_ppm_visc(prec, p.flux, occ, grid, s, p, a, tm); break;
      case FEST_INTERP_WENO: launch_stage_weno_visc(prec, p.flux, occ, grid, s, p, a, tm); break;
      default: launch_stage_weno_nm_visc(prec, p.flux, occ, grid, s, p, a, tm); break;
    }
    return;
  }
  switch (p.interp) {
    case FEST_INTERP_NONE: launch_stage_none(prec, p.flux, occ, grid, s, p, a, tm); break;
    case FEST_INTERP_MUSCL: launch_stage_muscl(prec, p.flux, occ, grid, s, p, a, tm); break;
    case FEST_INTERP_PPM: launch_stage_ppm(prec, p.flux, occ, grid, s, p, a, tm); break;
    case FEST_INTERP_WENO: launch_stage_weno(prec, p.flux, occ, grid, s, p, a, tm); break;
    default: launch_stage_weno_nm(prec, p.flux, occ, grid, s, p, a, tm); break;
  }
}

// Pick the k-chunk (interior planes per CTA) by timing the sweep itself on
// the current inputs: short chunks give more CTAs, long chunks re-read fewer
// halo planes.  The trial launches write only the stage's output buffers
// (rewritten by the real launch) and a private error word; the RK
// accumulator is left alone.  Chunking does not change any result.
static int tune_chunk(FusedState* f, const Params& p, int prec, StageArgs a, const CUtensorMap& tm,
                      cudaStream_t s, long long* cnt, int* occ_out) {
  const int nk = p.d.kmx - 1;
  const dim3 g0((p.d.imx - 1 + IX - 1) / IX, (p.d.jmx - 1 + IY - 1) / IY, 1);
  a.use_rn = 0; a.TU = 0; a.res_out = nullptr;
  for (int dir = 0; dir < 3; ++dir) a.mflux[dir] = nullptr;
  a.err = f->tune_err;
  const int cand[] = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32, 48, 64, 96, 128};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = nk, best_occ = prec == FEST_MIXED ? 2 : 1;
  float best_ms = 1e30f;
  for (int occ : {2, 3}) {
    // FP64 and the viscous and SST sweeps have one register budget
    if ((prec != FEST_MIXED || p.mu_ref != 0.0) && occ == 3) break;
    int last_chunks = -1;
    for (int kc : cand) {
      if (kc > nk) kc = nk;
      const int chunks = (nk + kc - 1) / kc;
      if (chunks == last_chunks) continue;
      last_chunks = chunks;
      a.k_chunk = (nk + chunks - 1) / chunks;
      dim3 g = g0;
      g.z = chunks;
      launch_sweep(p, prec, occ, g, s, a, tm);  // warm-up
      cudaEventRecord(e0, s);
      for (int r = 0; r < 3; ++r) launch_sweep(p, prec, occ, g, s, a, tm);
      cudaEventRecord(e1, s);
      *cnt += 4;
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess) break;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) { best_ms = ms; best = a.k_chunk; best_occ = occ; }
      if (chunks == 1) break;
    }
  }
  *occ_out = best_occ;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemsetAsync(f->tune_err, 0, sizeof(int), s);
  return best;
}

// the arguments of one stage sweep of block f
static StageArgs stage_args(FusedState* f, const DevBlock& b, bool mixed, int in, int out, int base,
                            double bA, double bB, double TF, double SF, int TU, int use_rn,
                            int compute_dt, double CFL, bool last) {
  StageArgs a;
  a.qin = f->Q[in];
  a.qout = f->Q[out];
  a.qbase = f->Q[base];
  a.qU = f->Q[f->cur];
  a.bA = bA; a.bB = bB; a.TF = TF; a.SF = SF; a.TU = TU; a.use_rn = use_rn;
  a.Rn = b.Rstore; a.dt = b.dt; a.compute_dt = compute_dt; a.CFL = CFL;
  a.f_TF = (float)TF; a.f_CFL = (float)CFL; a.f_bB = (float)bB; a.blend = bA != 0.0;
  a.res_out = last ? b.res : nullptr;
  for (int dir = 0; dir < 3; ++dir) {
    a.mflux[dir] = last ? b.flux[dir] : nullptr;
    a.faces[dir] = b.faces[dir];
  }
  a.cells = b.cells;
  a.err = b.err;
  a.qin32 = mixed ? f->Q32[in] : nullptr;
  a.qout32 = mixed ? f->Q32[out] : nullptr;
  for (int dir = 0; dir < 3; ++dir) a.faces32[dir] = mixed ? f->F32[dir] : nullptr;
  a.vol32 = mixed ? f->V32 : nullptr;
  a.mpitch = f->mpitch;
  a.cells32 = mixed ? f->C32 : nullptr;
  a.dist32 = mixed ? f->D32 : nullptr;
  a.Temp = b.Temp;
  a.dist = b.dist;
  a.ring_ghosts = 0;
  a.kper = 0;
  a.k_chunk = 1;
  return a;
}

// tabs[n]: the block table (this block and its interface partners, each
// with its buffer n) the ghost fill of a stage reading buffer n uses
static void run_stage(FusedState* f, const Params& p, const DevBlock& b, int prec, int in, int out,
                  int base, double bA, double bB, double TF, double SF, int TU, int use_rn,
                  int compute_dt, double CFL, int iter, bool last, BlockRef* const* tabs, cudaStream_t s,
                  long long* cnt) {
  const bool mixed = prec == FEST_MIXED;
  DevBlock bb = b;
  bb.qp = f->Q[in];
  bb.qp32 = mixed ? f->Q32[in] : nullptr;
  bb.qp32_pitch = f->mpitch;
  Launcher L{s, cnt};
  const int od = mixed ? order_dirs(p) : 0;
  int ring = 0, kper = 0;
  if (mixed && iter > 2) {
    // the sweep makes the ghosts of most faces itself; the FP32 ghost fill
    // of the stencil mirror covers the rest (the FP64 ghosts of Q[in] are
    // read by nothing on this path after iteration 2), the high faces of
    // order-dependent directions second
    ring = ring_faces(p, &kper);
    if (needs_edge_ghosts(p)) ring = kper = 0;  // every face's ghosts in the mirror, for the edges
    const int skip = ring | (kper << 4);
    Mirror M = mirror_of(f, in);
    for (int pass = 0; pass < (od ? 2 : 1); ++pass) {
      GhostPlan plan{};
      for (int fc = 0; fc < 6; ++fc) {
        if (p.id[fc] == -1 || ((skip >> fc) & 1)) continue;  // fix() only, or made by the sweep
        const bool second = (fc % 2 == 1) && ((od >> (fc / 2)) & 1);
        if (second != (pass == 1)) continue;
        const int dir = fc / 2;
        const int na = (dir == 0 ? p.d.jmx : p.d.imx) - 1, nb = (dir == 2 ? p.d.jmx : p.d.kmx) - 1;
        plan.face[plan.nf] = fc;
        plan.na[plan.nf] = na;
        plan.start[plan.nf + 1] = plan.start[plan.nf] + (long long)na * nb;
        ++plan.nf;
      }
      const long long work = plan.start[plan.nf];
      if (work > 0) {
        k_ghosts_mirror<<<(unsigned)((work + 127) / 128), 128, 0, s>>>(p, M, plan, f->F32[0], f->F32[1],
                                                                         f->F32[2], b.dist, tabs[in]);
        ++*cnt;
      }
    }
  } else {
    // edge/corner ghosts reach an interior update only through the ghost
    // gradient of an interface face of a viscous block: averaged then
    // (order-dependent blocks are thin, so the faces run one by one)
    launch_ghosts(p, bb, tabs[in], iter, L, needs_edge_ghosts(p));
  }
  if (mixed && needs_edge_ghosts(p)) {
    k_corners_mirror<<<1, 256, 0, s>>>(p.d, mirror_of(f, in));
    ++*cnt;
  }
  // order-dependent directions: the next fill's low face reads this fill's
  // high-face ghosts, in whichever buffer serves as its input
  for (int dir = 0; dir < 3; ++dir) {
    if (!((od >> dir) & 1)) continue;
    const int fc = 2 * dir + 1;
    const int na = (dir == 0 ? p.d.jmx : p.d.imx) - 1, nb = (dir == 2 ? p.d.jmx : p.d.kmx) - 1;
    const long long n = (long long)na * nb * 3 * p.d.nv;
    const int o1 = (in + 1) % 3, o2 = (in + 2) % 3;
    const bool fp64 = iter <= 2;  // the FP64 fill of iterations 1-2 reads the FP64 buffers
    k_ghost_bcast<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        p.d, fc, na, nb, mirror_of(f, in), mirror_of(f, o1), mirror_of(f, o2), fp64 ? f->Q[in] : nullptr,
        f->Q[o1], f->Q[o2]);
    ++*cnt;
  }
  StageArgs a = stage_args(f, b, mixed, in, out, base, bA, bB, TF, SF, TU, use_rn, compute_dt, CFL, last);
  a.ring_ghosts = ring;
  a.kper = kper;
  const CUtensorMap& tm = mixed ? f->tm[in] : f->tm_none;
  const int nk = p.d.kmx - 1;
  int& kc = f->kc[mixed ? 1 : 0];
  int& occ = f->occ[mixed ? 1 : 0];
  if (kc == 0) kc = tune_chunk(f, p, prec, a, tm, s, cnt, &occ);
  a.k_chunk = kc;
  const int chunks = (nk + kc - 1) / kc;
  dim3 grid((p.d.imx - 1 + IX - 1) / IX, (p.d.jmx - 1 + IY - 1) / IY, chunks);
  if (f->profiling) {
    if (f->nev + 2 > f->ev.size())
      for (int n = 0; n < 256; ++n) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        f->ev.push_back(e);
      }
    cudaEventRecord(f->ev[f->nev], s);
  }
  launch_sweep(p, prec, occ, grid, s, a, tm);
  if (f->profiling) {
    cudaEventRecord(f->ev[f->nev + 1], s);
    f->nev += 2;
  }
  ++*cnt;
}

// The stages of one iteration of the integrator (update.f90:129-226) with
// the current state in buffer U: input, output and base buffers, blend and
// update factors.  *zero_rn: RK2/RK4 clear their accumulator first.
struct StageSpec {
  int in, out, base;
  double bA, bB, TF, SF;
  int TU, use_rn, cdt;
  bool last;
};
static int schedule(int integ, int U, bool lastit, StageSpec* st, int* next_cur, bool* zero_rn) {
  const int A = (U + 1) % 3, B = (U + 2) % 3;
  *next_cur = U;
  *zero_rn = false;
  switch (integ) {
    case FEST_TIME_NONE:
      st[0] = {U, A, U, 0, 1, 1., 1., 0, 0, 1, lastit};
      *next_cur = A;
      return 1;
    case FEST_TIME_TVDRK2:
      st[0] = {U, A, U, 0, 1, 1., 1., 0, 0, 1, false};
      st[1] = {A, U, A, 0.5, 0.5, 1., 1., 0, 0, 0, lastit};
      return 2;
    case FEST_TIME_TVDRK3:
      st[0] = {U, A, U, 0, 1, 1., 1., 0, 0, 1, false};
      st[1] = {A, B, A, 0.75, 0.25, 1., 1., 0, 0, 0, false};
      st[2] = {B, U, B, 1. / 3., 2. / 3., 1., 1., 0, 0, 0, lastit};
      return 3;
    case FEST_TIME_RK2:
      *zero_rn = true;
      st[0] = {U, A, U, 0, 1, 0.5, 1., 0, 1, 1, false};
      st[1] = {A, U, U, 0, 1, 0.5, 1., 1, 1, 0, lastit};
      return 2;
    case FEST_TIME_RK4:
      *zero_rn = true;
      st[0] = {U, A, U, 0, 1, 0.5, 1., 0, 1, 1, false};
      st[1] = {A, B, U, 0, 1, 0.5, 2., 0, 1, 0, false};
      st[2] = {B, A, U, 0, 1, 1.0, 2., 0, 1, 0, false};
      st[3] = {A, U, U, 0, 1, 1. / 6., 1., 1, 1, 0, lastit};
      return 4;
    default:
      return 0;
  }
}

// One iteration of the integrator on the stream, in three parts so that
// the blocks of a batch can advance stage by stage together (their ghost
// fills read each other's stage inputs): iter_begin (schedule, fix()
// ghosts of the early iterations, TVD snapshot, accumulator reset), the
// stages (run_stage), iter_end (buffer rotation, TVD ghost blends).
struct IterPlan {
  StageSpec st[4];
  int ns = 0, next = 0;
  bool tvd_early = false;
};
static int iter_begin(FusedState* f, const Params& p, const DevBlock& b, int prec, int it, bool lastit,
                      BlockRef* const* tabs, cudaStream_t s, long long* cnt, IterPlan& ip) {
  const bool mixed = prec == FEST_MIXED;
  const int U = f->cur;
  bool zero_rn = false;
  ip.ns = schedule(p.integ, U, lastit, ip.st, &ip.next, &zero_rn);
  if (ip.ns == 0) return FEST_ERR_ARG;
  if (it <= 2) {
    // fix() ghosts are written only while current_iter <= 2
    // (bc_primitive.f90:236,318,366) and persist afterwards: every
    // buffer that later serves as a stage input must receive them
    for (int n = 0; n < 3; ++n) {
      if (n == U) continue;
      DevBlock bb = b;
      bb.qp = f->Q[n];
      bb.qp32 = mixed ? f->Q32[n] : nullptr;
      bb.qp32_pitch = f->mpitch;
      launch_ghosts(p, bb, tabs[n], it, Launcher{s, cnt}, false);
    }
  }
  if (!mixed && p.mu_ref != 0.0) {
    // the gradients' temperature of this iteration (the FP64 viscous sweep)
    k_temp_start<<<(unsigned)((p.d.P + 255) / 256), 256, 0, s>>>(p.d, p.R, f->Q[U], f->Gref, b.Temp);
    ++*cnt;
  }
  const size_t bytes = sizeof(double) * (size_t)p.d.P * p.d.nv;
  ip.tvd_early = it <= 2 && (p.integ == FEST_TIME_TVDRK2 || p.integ == FEST_TIME_TVDRK3);
  if (ip.tvd_early) cudaMemcpyAsync(f->Us, f->Q[U], bytes, cudaMemcpyDeviceToDevice, s);
  if (zero_rn) cudaMemsetAsync(b.Rstore, 0, sizeof(double) * ncells(p.d) * p.d.nv, s);
  return FEST_OK;
}
static void iter_stage(FusedState* f, const Params& p, const DevBlock& b, int prec, int it, double CFL,
                       const IterPlan& ip, int n, BlockRef* const* tabs, cudaStream_t s, long long* cnt) {
  const StageSpec& z = ip.st[n];
  run_stage(f, p, b, prec, z.in, z.out, z.base, z.bA, z.bB, z.TF, z.SF, z.TU, z.use_rn, z.cdt, CFL, it, z.last,
            tabs, s, cnt);
}
static void iter_end(FusedState* f, const Params& p, int prec, const IterPlan& ip, cudaStream_t s,
                     long long* cnt) {
  const bool mixed = prec == FEST_MIXED;
  const int U = f->cur;
  if (!mixed && p.mu_ref != 0.0) {
    const StageSpec& z = ip.st[ip.ns - 1];
    const long long n = p.d.P * p.d.nv;
    const bool tvd = p.integ == FEST_TIME_TVDRK2 || p.integ == FEST_TIME_TVDRK3;
    k_gref<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Gref, f->Q[z.in], z.bA, z.bB, tvd ? 1 : 0);
    ++*cnt;
  }
  f->cur = ip.next;
  if (ip.tvd_early) {
    // TVD blends run over the ghosts too (update.f90:203-206): the last
    // stage's input X, q = bA*Us + bB*X on non-interior cells
    const size_t bytes = sizeof(double) * (size_t)p.d.P * p.d.nv;
    const StageSpec& z = ip.st[ip.ns - 1];
    long long n = p.d.P * p.d.nv;
    k_ghost_blend<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Q[U], mixed ? f->Q32[U] : nullptr,
                                                             f->mpitch, f->Us, f->Q[z.in], z.bA, z.bB);
    ++*cnt;
    // the blended ghosts must persist in every buffer once fix() stops
    for (int m = 0; m < 3; ++m)
      if (m != f->cur) {
        cudaMemcpyAsync(f->Q[m], f->Q[f->cur], bytes, cudaMemcpyDeviceToDevice, s);
        if (mixed)
          cudaMemcpyAsync(f->Q32[m], f->Q32[f->cur], sizeof(float) * (size_t)f->m_elems,
                          cudaMemcpyDeviceToDevice, s);
      }
  }
}
static int enqueue_iteration(FusedState* f, const Params& p, const DevBlock& b, int prec, int it,
                             bool lastit, double CFL, cudaStream_t s, long long* cnt) {
  IterPlan ip;
  int rc = iter_begin(f, p, b, prec, it, lastit, f->table, s, cnt, ip);
  if (rc) return rc;
  for (int n = 0; n < ip.ns; ++n) iter_stage(f, p, b, prec, it, CFL, ip, n, f->table, s, cnt);
  iter_end(f, p, prec, ip, s, cnt);
  return FEST_OK;
}

// Iterations after the second repeat the same launches with the same
// arguments (fix() BCs and the TVD ghost blends stop), so each distinct
// (precision, CFL, last-iteration flag, current buffer) is captured once as
// a CUDA graph and replayed: one graph launch per iteration instead of one
// launch per kernel.
static int graph_for(FusedState* f, const Params& p, const DevBlock& b, int prec, int it, bool lastit,
                     double CFL, cudaStream_t s, cudaGraphExec_t* out, int* kernels) {
  for (const auto& g : f->graphs)
    if (g.prec == prec && g.CFL == CFL && g.last == lastit && g.cur == f->cur) {
      *out = g.exec;
      *kernels = g.kernels;
      return FEST_OK;
    }
  const int cur0 = f->cur;
  long long n = 0;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return FEST_ERR_CUDA;
  int rc = enqueue_iteration(f, p, b, prec, it, lastit, CFL, s, &n);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &graph);
  f->cur = cur0;  // the capture only recorded the iteration
  if (rc || e != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return rc ? rc : FEST_ERR_CUDA;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return FEST_ERR_CUDA;
  }
  if (f->graphs.size() >= 16) {
    cudaGraphExecDestroy(f->graphs.front().exec);
    f->graphs.erase(f->graphs.begin());
  }
  f->graphs.push_back(FusedState::Graph{prec, CFL, lastit, cur0, exec, (int)n});
  *out = exec;
  *kernels = (int)n;
  return FEST_OK;
}

// the reference's ghost values start as those of the state the run starts
// from (before any graph capture, which would replay the copy)
static void gref_init(FusedState* f, const Params& p, int prec, cudaStream_t s) {
  if (prec != FEST_FP64 || p.mu_ref == 0.0 || f->gref_valid || !f->Gref) return;
  cudaMemcpyAsync(f->Gref, f->Q[f->cur], sizeof(double) * (size_t)p.d.P * p.d.nv, cudaMemcpyDeviceToDevice, s);
  f->gref_valid = true;
}

int fused_run(FusedState* f, const Params& p, const DevBlock& b, int prec, int n_iters,
              int first_iter, double CFL, cudaStream_t s, long long* cnt) {
  if (!f) return FEST_ERR_ARG;
  if (!f->seeded) seed(f, s);
  const bool mixed = prec == FEST_MIXED;
  if (mixed) {
    int rc = ensure_mirrors(f, b, s, cnt);
    if (rc) return rc;
  } else {
    f->mirror_valid = false;  // FP64 stages do not maintain the mirror
  }
  if (n_iters > 0) f->buffers_equal = false;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  gref_init(f, p, prec, s);
  for (int n = 0; n < n_iters; ++n) {
    const int it = first_iter + n;
    const bool lastit = (n == n_iters - 1);
    // graphs once the k-chunk is tuned (tuning synchronises), never inside
    // a caller's own capture, never while stage launches are being timed
    const bool replay = f->use_graphs && it > 2 && f->kc[mixed ? 1 : 0] != 0 && !f->profiling &&
                        cap == cudaStreamCaptureStatusNone;
    if (replay) {
      cudaGraphExec_t exec;
      int kernels = 0;
      if (graph_for(f, p, b, prec, it, lastit, CFL, s, &exec, &kernels) == FEST_OK) {
        if (cudaGraphLaunch(exec, s) != cudaSuccess) return FEST_ERR_CUDA;
        *cnt += kernels;
        if (p.integ == FEST_TIME_NONE) f->cur = (f->cur + 1) % 3;
        continue;
      }
      f->use_graphs = false;  // capture refused: launch directly from now on
    }
    int rc = enqueue_iteration(f, p, b, prec, it, lastit, CFL, s, cnt);
    if (rc) return rc;
  }
  return FEST_OK;
}

const double* fused_current_state(const FusedState* f) { return f && f->seeded ? f->Q[f->cur] : nullptr; }

// dense interior cells -> the FP64 state and (q32 non-null) its mirror,
// converted as the sweep converts the states it writes (d2f: FP32
// subnormals become zero), so that an unchanged state leaves the mirror
// unchanged
__global__ void k_import_interior(Dims d, int pitch, const double* __restrict__ src, double* __restrict__ q64,
                                  float* __restrict__ q32) {
  const long long nc = ncells(d), n = nc * d.nv;
  const long long st = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += st) {
    const long long l = t / nc, c = t % nc;
    const int i = 1 + (int)(c % (d.imx - 1));
    const long long r = c / (d.imx - 1);
    const int j = 1 + (int)(r % (d.jmx - 1)), k = 1 + (int)(r / (d.jmx - 1));
    const long long pp = pidx(d, i, j, k) + d.P * l;
    const double v = src[t];
    q64[pp] = v;
    if (q32) q32[(pp / d.ni) * pitch + pp % d.ni] = d2f(v);
  }
}

int fused_import_interior(FusedState* f, const double* src, cudaStream_t s, long long* cnt) {
  if (!f || !f->seeded) return FEST_ERR_ARG;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* q32 = (f->V32 && f->mirror_valid) ? f->Q32[f->cur] : nullptr;
  k_import_interior<<<sms * 4, 256, 0, s>>>(f->d, f->mpitch, src, f->Q[f->cur], q32);
  ++*cnt;
  f->buffers_equal = false;
  return cudaGetLastError() == cudaSuccess ? FEST_OK : FEST_ERR_CUDA;
}

int fused_export_state(FusedState* f, double* qp, cudaStream_t s) {
  if (!f) return FEST_ERR_ARG;
  if (f->Q[f->cur] != qp)
    cudaMemcpyAsync(qp, f->Q[f->cur], sizeof(double) * (size_t)f->d.P * f->d.nv,
                    cudaMemcpyDeviceToDevice, s);
  // the caller may now change qp: the next fused run starts from it again
  f->cur = 0;
  f->seeded = false;
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


// ---- batches: every block of a multiblock case in one launch per stage ----

struct FusedBatch {
  std::vector<FusedState*> f;
  std::vector<Params> p;  // part_block: batch indices, self_block: the block's own
  std::vector<DevBlock> b;
  int nb = 0, interp = 0, flux = 0, integ = 0, prec = FEST_MIXED;
  // one batched sweep launch per stage (mixed, one kernel for all blocks);
  // otherwise every block's own launches, stage by stage
  bool batched = false;
  BlockRef* tabs[3] = {nullptr, nullptr, nullptr};  // every block with its buffer n (FP64 and FP32)
  bool tabs_ready = false;
  Params* d_params = nullptr;
  int kcap = 0;  // k-chunk cap, tuned on the first batched stage
  struct Table {
    int stage, cur;
    bool last;
    double CFL;
    int kcap;
    BatchEntry* d;
    int ctas;
  };
  std::vector<Table> tables;
  struct GTable {
    int buf;
    GhostSeg* d;
    int nseg;
    long long total;
  };
  std::vector<GTable> gtables;
  struct Graph {
    double CFL;
    bool last;
    int cur;
    cudaGraphExec_t exec;
    int kernels;
  };
  std::vector<Graph> graphs;
  bool use_graphs = true;
};

static int chunk_of(const Params& p, int kcap) { return std::max(1, std::min(p.d.kmx - 1, kcap)); }

// device table of one stage for every block (built once per key)
static FusedBatch::Table* batch_table(FusedBatch* B, int stage, const StageSpec& sp, int cur, double CFL,
                                      int kcap, bool tuning) {
  if (!tuning)
    for (auto& t : B->tables)
      if (t.stage == stage && t.cur == cur && t.last == sp.last && t.CFL == CFL && t.kcap == kcap) return &t;
  std::vector<BatchEntry> h(B->nb);
  int cta = 0;
  for (int n = 0; n < B->nb; ++n) {
    FusedState* f = B->f[n];
    const Params& p = B->p[n];
    BatchEntry& e = h[n];
    e.tm = f->tm[sp.in];
    e.p = p;
    e.a = stage_args(f, B->b[n], true, sp.in, sp.out, sp.base, sp.bA, sp.bB, sp.TF, sp.SF, sp.TU,
                     sp.use_rn, sp.cdt, CFL, sp.last);
    e.a.qU = f->Q[cur];
    e.a.ring_ghosts = ring_faces(p, &e.a.kper);  // batched stages run after iteration 2
    const int kc = chunk_of(p, kcap), nk = p.d.kmx - 1;
    e.a.k_chunk = kc;
    if (tuning) {  // trial launches: private error word, no accumulator, no norms
      e.a.use_rn = 0; e.a.TU = 0; e.a.res_out = nullptr;
      for (int dir = 0; dir < 3; ++dir) e.a.mflux[dir] = nullptr;
      e.a.err = f->tune_err;
    }
    e.tx = (p.d.imx - 1 + IX - 1) / IX;
    e.ty = (p.d.jmx - 1 + IY - 1) / IY;
    e.cta0 = cta;
    cta += e.tx * e.ty * ((nk + kc - 1) / kc);
  }
  FusedBatch::Table t{stage, cur, sp.last, CFL, kcap, nullptr, cta};
  if (cudaMalloc((void**)&t.d, sizeof(BatchEntry) * B->nb) != cudaSuccess) return nullptr;
  if (cudaMemcpy(t.d, h.data(), sizeof(BatchEntry) * B->nb, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(t.d);
    return nullptr;
  }
  if (tuning) {  // the caller frees it
    static thread_local FusedBatch::Table tmp;
    tmp = t;
    return &tmp;
  }
  B->tables.push_back(t);
  return &B->tables.back();
}

static FusedBatch::GTable* batch_ghosts(FusedBatch* B, int buf) {
  for (auto& g : B->gtables)
    if (g.buf == buf) return &g;
  std::vector<GhostSeg> h;
  long long start = 0;
  for (int n = 0; n < B->nb; ++n) {
    FusedState* f = B->f[n];
    const Params& p = B->p[n];
    int kper = 0;
    const int skip = ring_faces(p, &kper) | (kper << 4);
    for (int fc = 0; fc < 6; ++fc) {
      if (p.id[fc] == -1 || ((skip >> fc) & 1)) continue;  // fix() only, or made by the sweep
      const int dir = fc / 2;
      const int na = (dir == 0 ? p.d.jmx : p.d.imx) - 1, nb = (dir == 2 ? p.d.jmx : p.d.kmx) - 1;
      GhostSeg g;
      g.start = start;
      g.block = n;
      g.face = fc;
      g.na = na;
      g.M = Mirror{f->Q32[buf], f->mpitch, p.d.nj, p.d.nk, (long long)f->mpitch * p.d.nj * p.d.nk};
      for (int m = 0; m < 3; ++m) g.F[m] = f->F32[m];
      g.dist = B->b[n].dist;
      g.PM = g.M;
      g.pd = p.d;
      if ((p.id[fc] == -10 || p.id[fc] >= 0) && p.part_block[fc] != n) {  // another block of the batch
        const FusedState* q = B->f[p.part_block[fc]];
        const Dims& qd = B->p[p.part_block[fc]].d;
        g.PM = Mirror{q->Q32[buf], q->mpitch, qd.nj, qd.nk, (long long)q->mpitch * qd.nj * qd.nk};
        g.pd = qd;
      }
      h.push_back(g);
      start += (long long)na * nb;
    }
  }
  FusedBatch::GTable g{buf, nullptr, (int)h.size(), start};
  if (!h.empty()) {
    if (cudaMalloc((void**)&g.d, sizeof(GhostSeg) * h.size()) != cudaSuccess) return nullptr;
    if (cudaMemcpy(g.d, h.data(), sizeof(GhostSeg) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
      return nullptr;
  }
  B->gtables.push_back(g);
  return &B->gtables.back();
}

static int launch_batch(const FusedBatch* B, int ctas, const BatchEntry* e, cudaStream_t s) {
  if (B->p[0].turb != FEST_TURB_NONE) {
    switch (B->interp) {
      case FEST_INTERP_NONE: return launch_batch_none_sst(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_MUSCL: return launch_batch_muscl_sst(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_PPM: return launch_batch_ppm_sst(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_WENO: return launch_batch_weno_sst(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      default: return launch_batch_weno_nm_sst(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    }
  }
  if (B->p[0].mu_ref != 0.0) {
    switch (B->interp) {
      case FEST_INTERP_NONE: return launch_batch_none_visc(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_MUSCL: return launch_batch_muscl_visc(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_PPM: return launch_batch_ppm_visc(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      case FEST_INTERP_WENO: return launch_batch_weno_visc(FEST_MIXED, B->flux, ctas, s, e, B->nb);
      default: return launch_batch_weno_nm_visc(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    }
  }
  switch (B->interp) {
    case FEST_INTERP_NONE: return launch_batch_none(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    case FEST_INTERP_MUSCL: return launch_batch_muscl(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    case FEST_INTERP_PPM: return launch_batch_ppm(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    case FEST_INTERP_WENO: return launch_batch_weno(FEST_MIXED, B->flux, ctas, s, e, B->nb);
    default: return launch_batch_weno_nm(FEST_MIXED, B->flux, ctas, s, e, B->nb);
  }
}

// The project's tile tuner for batches: the k-chunk cap (planes per CTA)
// timed on the first batched stage; short chunks give more CTAs, long ones
// re-read fewer halo planes.  Results do not depend on it.
static int tune_batch(FusedBatch* B, const StageSpec& sp, int cur, double CFL, cudaStream_t s,
                      long long* cnt) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = 64;
  float best_ms = 1e30f;
  for (int cap : {1, 2, 4, 8, 16, 64}) {
    FusedBatch::Table* t = batch_table(B, 0, sp, cur, CFL, cap, true);
    if (!t) break;
    BatchEntry* d = t->d;
    const int ctas = t->ctas;
    launch_batch(B, ctas, d, s);
    cudaEventRecord(e0, s);
    for (int r = 0; r < 3; ++r) launch_batch(B, ctas, d, s);
    cudaEventRecord(e1, s);
    *cnt += 4;
    float ms = 0.f;
    const bool ok = cudaEventSynchronize(e1) == cudaSuccess;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaFree(d);
    if (!ok) break;
    if (ms < best_ms) { best_ms = ms; best = cap; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (FusedState* f : B->f) cudaMemsetAsync(f->tune_err, 0, sizeof(int), s);
  return best;
}

static int batch_iteration(FusedBatch* B, bool lastit, double CFL, cudaStream_t s, long long* cnt) {
  const int U = B->f[0]->cur;
  StageSpec st[4];
  int next = U;
  bool zero_rn = false;
  const int ns = schedule(B->integ, U, lastit, st, &next, &zero_rn);
  if (ns == 0) return FEST_ERR_ARG;
  if (zero_rn)
    for (int n = 0; n < B->nb; ++n)
      cudaMemsetAsync(B->b[n].Rstore, 0, sizeof(double) * ncells(B->p[n].d) * B->p[n].d.nv, s);
  for (int k = 0; k < ns; ++k) {
    FusedBatch::GTable* g = batch_ghosts(B, st[k].in);
    if (!g) return FEST_ERR_NOMEM;
    if (g->total > 0) {
      k_ghosts_mirror_batch<<<(unsigned)((g->total + 127) / 128), 128, 0, s>>>(B->d_params, g->d, g->nseg,
                                                                                g->total);
      ++*cnt;
    }
    FusedBatch::Table* t = batch_table(B, k, st[k], U, CFL, B->kcap, false);
    if (!t) return FEST_ERR_NOMEM;
    int rc = launch_batch(B, t->ctas, t->d, s);
    if (rc) return rc;
    ++*cnt;
  }
  for (FusedState* f : B->f) f->cur = next;
  return FEST_OK;
}

int fused_batch_create(const std::vector<FusedState*>& f, const std::vector<Params>& p,
                       const std::vector<DevBlock>& b, int prec, FusedBatch** out) {
  *out = nullptr;
  if (f.empty() || f.size() != p.size() || f.size() != b.size()) return FEST_ERR_ARG;
  if (prec != FEST_MIXED && prec != FEST_FP64) return FEST_ERR_ARG;
  // the blocks advance stage by stage together: one integrator; a batched
  // mixed sweep also needs one kernel for all (the same reconstruction, flux
  // scheme and physics: Euler, laminar, or SST) and no direction whose
  // ghosts depend on the face order
  bool batched = prec == FEST_MIXED;
  for (size_t n = 0; n < f.size(); ++n) {
    if (!f[n] || !fused_supported(p[n], prec) || p[n].integ != p[0].integ) return FEST_ERR_ARG;
    if (order_dirs(p[n]) || needs_edge_ghosts(p[n]) || p[n].interp != p[0].interp || p[n].flux != p[0].flux ||
        (p[n].mu_ref != 0.0) != (p[0].mu_ref != 0.0) || (p[n].turb != FEST_TURB_NONE) != (p[0].turb != FEST_TURB_NONE))
      batched = false;
  }
  FusedBatch* B = new FusedBatch();
  B->f = f;
  B->p = p;
  B->b = b;
  B->nb = (int)f.size();
  B->interp = p[0].interp;
  B->flux = p[0].flux;
  B->integ = p[0].integ;
  B->prec = prec;
  B->batched = batched;
  bool ok = cudaMalloc((void**)&B->d_params, sizeof(Params) * B->nb) == cudaSuccess &&
            cudaMemcpy(B->d_params, p.data(), sizeof(Params) * B->nb, cudaMemcpyHostToDevice) == cudaSuccess;
  for (int n = 0; n < 3 && ok; ++n) ok = cudaMalloc((void**)&B->tabs[n], sizeof(BlockRef) * B->nb) == cudaSuccess;
  if (!ok) {
    fused_batch_destroy(B);
    return FEST_ERR_NOMEM;
  }
  *out = B;
  return FEST_OK;
}

// the block tables of the three buffers: every block's FP64 buffer and FP32
// mirror n (the mirrors exist once the first run has made them)
static int batch_tables(FusedBatch* B, cudaStream_t s) {
  if (B->tabs_ready) return FEST_OK;
  for (int n = 0; n < 3; ++n) {
    std::vector<BlockRef> t(B->nb);
    for (int m = 0; m < B->nb; ++m) {
      t[m].b = B->b[m];
      t[m].b.qp = B->f[m]->Q[n];
      t[m].b.qp32 = B->f[m]->Q32[n];
      t[m].b.qp32_pitch = B->f[m]->mpitch;
      t[m].d = B->p[m].d;
    }
    if (cudaMemcpyAsync(B->tabs[n], t.data(), sizeof(BlockRef) * B->nb, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return FEST_ERR_CUDA;
  }
  B->tabs_ready = B->prec == FEST_FP64 || B->f[0]->Q32[0] != nullptr;
  return FEST_OK;
}

// one iteration of every block, stage by stage (each block's launches of a
// stage follow the ghost fills that read the other blocks' stage inputs)
static int batch_lockstep(FusedBatch* B, int it, bool lastit, double CFL, cudaStream_t s, long long* cnt) {
  std::vector<IterPlan> ip(B->nb);
  for (int m = 0; m < B->nb; ++m) {
    int rc = iter_begin(B->f[m], B->p[m], B->b[m], B->prec, it, lastit, B->tabs, s, cnt, ip[m]);
    if (rc) return rc;
  }
  for (int k = 0; k < ip[0].ns; ++k)
    for (int m = 0; m < B->nb; ++m) iter_stage(B->f[m], B->p[m], B->b[m], B->prec, it, CFL, ip[m], k, B->tabs, s, cnt);
  for (int m = 0; m < B->nb; ++m) iter_end(B->f[m], B->p[m], B->prec, ip[m], s, cnt);
  return FEST_OK;
}

void fused_batch_destroy(FusedBatch* B) {
  if (!B) return;
  for (auto& g : B->graphs) cudaGraphExecDestroy(g.exec);
  for (auto& t : B->tables) cudaFree(t.d);
  for (auto& g : B->gtables) cudaFree(g.d);
  for (int n = 0; n < 3; ++n) cudaFree(B->tabs[n]);
  cudaFree(B->d_params);
  delete B;
}

int fused_batch_run(FusedBatch* B, int n_iters, int first_iter, double CFL, cudaStream_t s, long long* cnt) {
  if (!B) return FEST_ERR_ARG;
  // every block starts from its own state, in the same buffer
  bool same = true;
  for (FusedState* f : B->f) same = same && f->seeded && f->cur == B->f[0]->cur;
  for (int n = 0; n < B->nb; ++n) {
    FusedState* f = B->f[n];
    if (!same && f->seeded) fused_export_state(f, B->b[n].qp, s);
    if (!f->seeded) seed(f, s);
    if (B->prec == FEST_MIXED) {
      int rc = ensure_mirrors(f, B->b[n], s, cnt);
      if (rc) return rc;
    } else {
      f->mirror_valid = false;  // FP64 stages do not maintain the mirror
    }
    gref_init(f, B->p[n], B->prec, s);
    if (n_iters > 0) f->buffers_equal = false;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &cap);
  if (!B->tabs_ready) {
    if (cap != cudaStreamCaptureStatusNone) return FEST_ERR_ARG;  // the tables copy from the host
    int rc = batch_tables(B, s);
    if (rc) return rc;
  }
  for (int n = 0; n < n_iters; ++n) {
    const int it = first_iter + n;
    const bool lastit = (n == n_iters - 1);
    if (it <= 2 || !B->batched) {
      // the early iterations' special ghost handling, and FP64 batches (no
      // batched FP64 sweep): each block's own launches, stage by stage
      int rc = batch_lockstep(B, it, lastit, CFL, s, cnt);
      if (rc) return rc;
      continue;
    }
    if (B->kcap == 0) {
      if (cap != cudaStreamCaptureStatusNone) return FEST_ERR_ARG;  // tuning synchronises
      StageSpec st[4];
      int next;
      bool z;
      schedule(B->integ, B->f[0]->cur, false, st, &next, &z);
      B->kcap = tune_batch(B, st[0], B->f[0]->cur, CFL, s, cnt);
    }
    {  // device tables of this iteration exist before any capture (they copy from the host)
      StageSpec st[4];
      int next;
      bool z;
      const int ns = schedule(B->integ, B->f[0]->cur, lastit, st, &next, &z);
      for (int k = 0; k < ns; ++k)
        if (!batch_ghosts(B, st[k].in) || !batch_table(B, k, st[k], B->f[0]->cur, CFL, B->kcap, false))
          return FEST_ERR_NOMEM;
    }
    if (B->use_graphs && cap == cudaStreamCaptureStatusNone) {
      cudaGraphExec_t exec = nullptr;
      int kernels = 0;
      const int cur0 = B->f[0]->cur;
      for (const auto& g : B->graphs)
        if (g.CFL == CFL && g.last == lastit && g.cur == cur0) { exec = g.exec; kernels = g.kernels; }
      if (!exec) {
        long long k = 0;
        cudaGraph_t graph = nullptr;
        bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        int rc = ok ? batch_iteration(B, lastit, CFL, s, &k) : FEST_ERR_CUDA;
        if (ok) ok = cudaStreamEndCapture(s, &graph) == cudaSuccess && graph && rc == FEST_OK;
        for (FusedState* f : B->f) f->cur = cur0;
        if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
        if (ok) {
          B->graphs.push_back(FusedBatch::Graph{CFL, lastit, cur0, exec, (int)k});
          kernels = (int)k;
        } else {
          cudaGetLastError();
          B->use_graphs = false;
          exec = nullptr;
        }
      }
      if (exec) {
        if (cudaGraphLaunch(exec, s) != cudaSuccess) return FEST_ERR_CUDA;
        *cnt += kernels;
        if (B->integ == FEST_TIME_NONE)
          for (FusedState* f : B->f) f->cur = (f->cur + 1) % 3;
        continue;
      }
    }
    int rc = batch_iteration(B, lastit, CFL, s, cnt);
    if (rc) return rc;
  }
  return FEST_OK;
}
}  // namespace fest
