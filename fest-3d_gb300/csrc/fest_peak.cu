// fest_peak.cu - the arithmetic roofs of this GPU, measured: FP64 and FP32
// fused multiply-add throughput of dependent FMA chains (eight per thread,
// every SM filled), event-timed.  The FP64 sweeps are bound by the FP64
// unit, whose rate on this part is a small fraction of the FP32 one; their
// roofline is reported against this number.
#include <cuda_runtime.h>

#include "fest_common.cuh"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T* out, int n, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
int measure(int n, double* tflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return FEST_ERR_CUDA;
  const int blocks = sms * 8, threads = 256;
  T* out = nullptr;
  if (cudaMalloc((void**)&out, sizeof(T) * blocks * threads) != cudaSuccess) return FEST_ERR_NOMEM;
  cudaStream_t s;
  cudaEvent_t e0, e1;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {  // the first launch warms up
    cudaEventRecord(e0, s);
    k_fma_chains<T><<<blocks, threads, 0, s>>>(out, n, T(0.999), T(0.001));
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(out);
  if (e != cudaSuccess) return FEST_ERR_CUDA;
  *tflops = 2.0 * 64.0 * blocks * threads * (double)n / (best * 1e-3) / 1e12;
  return FEST_OK;
}

}  // namespace

extern "C" int fest_measure_peak(int kind, double* tflops) {
  if (!tflops) return FEST_ERR_ARG;
  if (kind == 0) return measure<double>(200, tflops);
  if (kind == 1) return measure<float>(4000, tflops);
  return FEST_ERR_ARG;
}
