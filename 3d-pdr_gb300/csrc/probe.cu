// probe.cu -- peak-rate probes for the roofline denominators the bench reports
// (FP64 and FP32 FMA throughput; the driver measures HBM and bf16 itself).
// Each thread runs 8 independent FMA chains for `iters` iterations; the
// result is written so the chains cannot be removed.
#include "pdr_internal.h"

namespace pdr {
namespace {

template <class T>
__global__ void fma_probe(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <class T>
int probe(double *tflops, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  const int iters = sizeof(T) == 8 ? 2048 : 65536;
  T *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(T) * blocks * threads);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(probe)");
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  fma_probe<T><<<blocks, threads, 0, st>>>(out, iters / 16, T(0.999999), T(1e-7));  // warm-up
  cudaEventRecord(t0, st);
  fma_probe<T><<<blocks, threads, 0, st>>>(out, iters, T(0.999999), T(1e-7));
  cudaEventRecord(t1, st);
  e = cudaEventSynchronize(t1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (e != cudaSuccess) return cuda_fail(e, "probe kernel");
  *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
  return 0;
}

}  // namespace
}  // namespace pdr

extern "C" {
// FMA throughput of the current device in TFLOP/s (2 flops per FMA):
// precision 64 for FP64, 32 for FP32.
int pdr_probe_fma_tflops(int precision, double *tflops, void *stream) {
  if (!tflops || (precision != 32 && precision != 64)) {
    pdr::set_error("pdr_probe_fma_tflops: invalid argument");
    return PDR_E_ARG;
  }
  return precision == 64 ? pdr::probe<double>(tflops, (cudaStream_t)stream)
                         : pdr::probe<float>(tflops, (cudaStream_t)stream);
}
}
