// fest_noalloc.cu - find_resnorm on caller-owned device arrays, with no
// handle and no device allocation.
//
// Who needs it: a caller that keeps the residual and the boundary fluxes in
// device memory it manages itself (its own kernels, a Fortran driver with
// device arrays, a framework tensor) and cannot or should not allocate at
// the point where it wants the norm.  Typical reasons: the device memory is
// already reserved by the caller's own pool (a caching allocator holding
// nearly all HBM), or the call sits inside an asynchronous time loop where
// an allocate/free pair would synchronise the whole device (cudaFree does).
// fest_find_resnorm needs a handle, and creating one allocates a full block
// state; this entry point needs neither.
//
// Scratch: the per-CTA partial sums, the final sums and an arrival counter
// live in file-scope __device__ arrays (32 KiB + 64 B + 4 B per device),
// whose addresses the host looks up once per device with
// cudaGetSymbolAddress.  The arrival counter must be zero when a launch
// starts: it is zero when the module loads, the first call on a device
// zeroes it again, and the last CTA of every launch puts it back to zero.
// The partial and final sums need no initial value (every launch overwrites
// the slots it reads).
//
// Because the scratch is one fixed area per device, two calls that overlap
// in time on the same device (different streams or host threads without
// ordering between them) race on it and may return wrong norms: callers
// serialise them.  The first call on each device does the setup (symbol
// lookup, counter reset, and the runtime's lazy module load).  No call can
// be part of a stream capture (each one synchronises its stream): a call
// on a capturing stream returns FEST_ERR_ARG.
#include <cmath>
#include <mutex>

#include "fest_common.cuh"

using namespace fest;

namespace {

constexpr int kNaParts = 512;         // CTAs of the reduction (one partial each)
constexpr int kNaThreads = 256;       // threads per CTA
constexpr int kNaSlots = NVMAX + 1;   // mass imbalance + one sum of squares per variable
constexpr int kNaMaxDevices = 64;

// 512 x 8 partial sums (32 KiB), then the 8 final sums
static __device__ __align__(256) double g_resnorm_scratch[kNaParts * kNaSlots + kNaSlots];
// CTAs that have stored their partials in the current launch (must start at 0)
static __device__ __align__(256) unsigned int g_resnorm_arrived;

// One pass: every CTA reduces its share of sum(R_l^2) (resnorm.f90:171-176)
// and of the net boundary mass flux (resnorm.f90:190-198) to one partial per
// quantity; the CTA that arrives last adds the partials in CTA order, so the
// result does not depend on scheduling.  No CTA waits on another.
__global__ void __launch_bounds__(kNaThreads) k_resnorm_noalloc(Dims d, const double* res,
                                                                const double* F, const double* G,
                                                                const double* H, double* scratch,
                                                                unsigned int* arrived) {
  __shared__ double sm[kNaThreads];
  __shared__ bool last;
  const int nv = d.nv;
  double acc[kNaSlots];
  for (int l = 0; l < kNaSlots; ++l) acc[l] = 0.0;
  const long long N = ncells(d);
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (long long t = t0; t < N; t += stride)
    for (int l = 0; l < nv; ++l) {
      const double v = res[t + N * l];
      acc[1 + l] += v * v;
    }
  const FlDim fx = fldim(d, 0), fy = fldim(d, 1), fz = fldim(d, 2);
  const long long nI = (long long)(d.jmx - 1) * (d.kmx - 1), nJ = (long long)(d.imx - 1) * (d.kmx - 1),
                  nK = (long long)(d.imx - 1) * (d.jmx - 1);
  for (long long t = t0; t < nI + nJ + nK; t += stride) {
    if (t < nI) {
      const int j = 1 + (int)(t % (d.jmx - 1)), k = 1 + (int)(t / (d.jmx - 1));
      acc[0] += F[flidx(fx, 1, j, k)] - F[flidx(fx, d.imx, j, k)];
    } else if (t < nI + nJ) {
      const long long u = t - nI;
      const int i = 1 + (int)(u % (d.imx - 1)), k = 1 + (int)(u / (d.imx - 1));
      acc[0] += G[flidx(fy, i, 1, k)] - G[flidx(fy, i, d.jmx, k)];
    } else {
      const long long u = t - nI - nJ;
      const int i = 1 + (int)(u % (d.imx - 1)), j = 1 + (int)(u / (d.imx - 1));
      acc[0] += H[flidx(fz, i, j, 1)] - H[flidx(fz, i, j, d.kmx)];
    }
  }
  const int parts = gridDim.x;
  for (int l = 0; l <= nv; ++l) {
    sm[threadIdx.x] = acc[l];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) scratch[blockIdx.x + (long long)parts * l] = sm[0];
    __syncthreads();
  }
  // publish the partials, then count this CTA in
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(arrived, 1u) == (unsigned int)(parts - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double* sums = scratch + (long long)parts * kNaSlots;
  if (threadIdx.x <= nv) {
    const int l = threadIdx.x;
    double s = 0.0;
    for (int b = 0; b < parts; ++b) s += __ldcg(scratch + b + (long long)parts * l);
    sums[l] = s;
  }
  if (threadIdx.x == 0) atomicExch(arrived, 0u);  // ready for the next launch
}

struct DeviceScratch {
  double* scratch = nullptr;
  unsigned int* arrived = nullptr;
  bool ready = false;
};
DeviceScratch g_dev[kNaMaxDevices];
std::mutex g_setup_mutex;

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return FEST_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FEST_ERR_NO_DEVICE;
  return FEST_ERR_CUDA;
}

}  // namespace

extern "C" int fest_find_resnorm_noalloc(const fest_extent* ext, const fest_flow* flow,
                                         const double* residue, const double* F, const double* G,
                                         const double* H, double* res_abs, void* cuda_stream) {
  if (!ext || !flow || !residue || !F || !G || !H || !res_abs) return FEST_ERR_ARG;
  if (ext->imx < 2 || ext->jmx < 2 || ext->kmx < 2 || ext->n_var < 1) return FEST_ERR_ARG;
  // the fixed scratch holds kNaSlots sums per CTA: n_var + 1 must fit
  if (ext->n_var + 1 > kNaSlots) return FEST_ERR_SCRATCH;
  // the scales below are those of the laminar/Euler (5) and k-omega SST (7)
  // variable sets (resnorm.f90:128-169); other counts (SA's 6, k-kL's 7 with
  // other free-stream scales) are models this library does not build
  if (ext->n_var != 5 && ext->n_var != 7) return FEST_ERR_ARG;
  int dev = -1;
  int rc = status_of(cudaGetDevice(&dev));
  if (rc) return rc;
  if (dev < 0 || dev >= kNaMaxDevices) return FEST_ERR_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  // every call synchronises its stream, which a capture cannot contain: a
  // call on a capturing stream is refused before it touches the capture
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    return FEST_ERR_ARG;
  }
  if (cap != cudaStreamCaptureStatusNone) return FEST_ERR_ARG;
  DeviceScratch& ds = g_dev[dev];
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!ds.ready) {
      // setup, once per device and with that device current
      void* a = nullptr;
      void* b = nullptr;
      if ((rc = status_of(cudaGetSymbolAddress(&a, g_resnorm_scratch)))) return rc;
      if ((rc = status_of(cudaGetSymbolAddress(&b, g_resnorm_arrived)))) return rc;
      if ((rc = status_of(cudaMemsetAsync(b, 0, sizeof(unsigned int), s)))) return rc;
      ds.scratch = (double*)a;
      ds.arrived = (unsigned int*)b;
      ds.ready = true;
    }
  }
  Dims d;
  d.imx = ext->imx; d.jmx = ext->jmx; d.kmx = ext->kmx; d.nv = ext->n_var;
  d.ni = ext->imx + 5; d.nj = ext->jmx + 5; d.nk = ext->kmx + 5;
  d.P = (long long)d.ni * d.nj * d.nk;
  k_resnorm_noalloc<<<kNaParts, kNaThreads, 0, s>>>(d, residue, F, G, H, ds.scratch, ds.arrived);
  if ((rc = status_of(cudaGetLastError()))) return rc;
  double sums[kNaSlots];
  if ((rc = status_of(cudaMemcpyAsync(sums, ds.scratch + kNaParts * kNaSlots,
                                      sizeof(double) * (d.nv + 1), cudaMemcpyDeviceToHost, s))))
    return rc;
  if ((rc = status_of(cudaStreamSynchronize(s)))) return rc;
  // setup_scale (resnorm.f90:128-169) and assemble (resnorm.f90:211-225)
  const fest_flow& f = *flow;
  double sc[kNaSlots];
  sc[0] = 1.;
  sc[1] = f.density_inf * f.vel_mag;
  sc[2] = sc[3] = sc[4] = f.density_inf * f.vel_mag * f.vel_mag;
  sc[5] = (0.5 * f.density_inf * (f.vel_mag * f.vel_mag * f.vel_mag) +
           ((f.gm / (f.gm - 1.)) * f.pressure_inf));
  sc[6] = f.density_inf * f.vel_mag * f.tk_inf;
  sc[7] = f.density_inf * f.vel_mag * f.tw_inf;
  res_abs[0] = std::fabs(sums[0] / sc[0]);
  for (int l = 1; l <= d.nv; ++l) res_abs[l] = std::sqrt(sums[l] / (sc[l] * sc[l]));
  return FEST_OK;
}
