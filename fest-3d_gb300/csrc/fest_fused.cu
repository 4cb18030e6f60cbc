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
  // the sweep addresses one plane's stencil with 32-bit offsets
  const bool small_enough = (long long)p.d.P * p.d.nv < (1ll << 31);
  return p.mu_ref == 0.0 && p.turb == FEST_TURB_NONE && p.d.nv == 5 && p.tstep == 'l' &&
         !ghosts_need_sequential(p) && small_enough;
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

static void run_stage(FusedState* f, const Params& p, const DevBlock& b, int prec, int in, int out,
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
  // enough CTAs to give every SM two: split the k-march into chunks
  const int tiles = ((p.d.imx - 1 + IX - 1) / IX) * ((p.d.jmx - 1 + IY - 1) / IY);
  const int nk = p.d.kmx - 1;
  int chunks = std::max(1, std::min(nk, (4 * 152 + tiles - 1) / tiles));
  a.k_chunk = (nk + chunks - 1) / chunks;
  chunks = (nk + a.k_chunk - 1) / a.k_chunk;
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
  switch (p.interp) {
    case FEST_INTERP_NONE: launch_stage_none(prec, p.flux, grid, s, p, a); break;
    case FEST_INTERP_MUSCL: launch_stage_muscl(prec, p.flux, grid, s, p, a); break;
    case FEST_INTERP_PPM: launch_stage_ppm(prec, p.flux, grid, s, p, a); break;
    case FEST_INTERP_WENO: launch_stage_weno(prec, p.flux, grid, s, p, a); break;
    default: launch_stage_weno_nm(prec, p.flux, grid, s, p, a); break;
  }
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
        run_stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, lastit, s, cnt);
        f->cur = A;
        break;
      case FEST_TIME_TVDRK2:
        run_stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, A, U, A, 0.5, 0.5, 1., 1., 0, 0, 0, CFL, it, lastit, s, cnt);
        if (tvd_early) {
          long long n = p.d.P * p.d.nv;
          k_ghost_blend<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Q[U], f->Us, f->Q[A], 0.5, 0.5);
          ++*cnt;
        }
        break;
      case FEST_TIME_TVDRK3:
        run_stage(f, p, b, prec, U, A, U, 0, 1, 1., 1., 0, 0, 1, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, A, B, A, 0.75, 0.25, 1., 1., 0, 0, 0, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, B, U, B, 1. / 3., 2. / 3., 1., 1., 0, 0, 0, CFL, it, lastit, s, cnt);
        if (tvd_early) {
          long long n = p.d.P * p.d.nv;
          k_ghost_blend<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p.d, f->Q[U], f->Us, f->Q[B], 1. / 3., 2. / 3.);
          ++*cnt;
        }
        break;
      case FEST_TIME_RK2:
        cudaMemsetAsync(b.Rstore, 0, sizeof(double) * ncells(p.d) * p.d.nv, s);
        run_stage(f, p, b, prec, U, A, U, 0, 1, 0.5, 1., 0, 1, 1, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, A, U, U, 0, 1, 0.5, 1., 1, 1, 0, CFL, it, lastit, s, cnt);
        break;
      case FEST_TIME_RK4:
        cudaMemsetAsync(b.Rstore, 0, sizeof(double) * ncells(p.d) * p.d.nv, s);
        run_stage(f, p, b, prec, U, A, U, 0, 1, 0.5, 1., 0, 1, 1, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, A, B, U, 0, 1, 0.5, 2., 0, 1, 0, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, B, A, U, 0, 1, 1.0, 2., 0, 1, 0, CFL, it, false, s, cnt);
        run_stage(f, p, b, prec, A, U, U, 0, 1, 1. / 6., 1., 1, 1, 0, CFL, it, lastit, s, cnt);
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
