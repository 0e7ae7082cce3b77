// probe.cu -- FP32 FMA throughput probe: the denominator of the rollout kernel's roofline.
#include <cuda_runtime.h>

#include "common.h"

namespace {

// Eight independent FMA chains per thread; 2 FLOP per FMA.
__global__ void fma_probe(float* out, int iters, float a, float b) {
  float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
  float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
      x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
  }
  float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5f) out[blockIdx.x] = s;   // keeps the chains live; never true in practice
}

}  // namespace

extern "C" int spi_probe_fp32_peak(double* flops_per_s) {
  using namespace spi;
  if (!flops_per_s) return set_error(SPI_EINVAL, "null output");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  float* out = nullptr;
  cudaError_t ce = cudaMalloc(&out, 4096 * sizeof(float));
  if (ce != cudaSuccess) return cuda_error(ce, "probe alloc");
  const int threads = 256, blocks = sms * 8, iters = 2048;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  fma_probe<<<blocks, threads>>>(out, iters / 8, 0.999999f, 1e-7f);   // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(t0);
    fma_probe<<<blocks, threads>>>(out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(t1);
    cudaEventSynchronize(t1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (ms < best) best = ms;
  }
  ce = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(out);
  if (ce != cudaSuccess) return cuda_error(ce, "probe");
  const double flops = 2.0 * 8.0 * 16.0 * iters * (double)threads * blocks;
  *flops_per_s = flops / (best * 1e-3);
  return SPI_OK;
}
