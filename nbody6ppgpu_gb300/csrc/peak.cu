// FP32 throughput probe: the denominator of the pair kernel's roofline
// measured on the device it runs on, with the same packed f32x2 FMA
// instruction the pair loop uses.  Each thread runs 8 independent FMA chains
// (enough to cover the pipe latency); every f32x2 FMA is 4 flops.
#include <cuda_runtime.h>

#include "common.cuh"
#include "gpunb.h"

namespace gpunb {

constexpr int PEAK_CHAINS = 8;

__global__ void __launch_bounds__(256) fp32_peak_kernel(int iters, float seed, float *out) {
  f2 a[PEAK_CHAINS];
#pragma unroll
  for (int c = 0; c < PEAK_CHAINS; ++c)
    a[c] = make_float2(seed + threadIdx.x * 1e-7f + c, seed - c);
  const f2 m = make_float2(0.9999999f, 0.9999998f), b = make_float2(1e-7f, 2e-7f);
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
#pragma unroll
      for (int c = 0; c < PEAK_CHAINS; ++c) a[c] = fma2(a[c], m, b);
    }
  }
  f2 s = a[0];
#pragma unroll
  for (int c = 1; c < PEAK_CHAINS; ++c) s = add2(s, a[c]);
  if (s.x == 12345.f && s.y == 54321.f) out[blockIdx.x] = s.x;   // keep the work live
}

}  // namespace gpunb

extern "C" int gpunb_fp32_peak(float *tflops, float *ms) {
  using namespace gpunb;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return GPUNB_E_NO_DEVICE;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * 65536) != cudaSuccess) return GPUNB_E_ALLOC;
  const int blocks = nsm * 8, threads = 256, iters = 1024;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp32_peak_kernel<<<blocks, threads>>>(iters, 1.0f, out);   // warm-up
  cudaEventRecord(e0);
  fp32_peak_kernel<<<blocks, threads>>>(iters, 1.0f, out);
  cudaEventRecord(e1);
  const cudaError_t err = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GPUNB_E_CUDA;
  const double flops = 4.0 * PEAK_CHAINS * 16.0 * iters * (double)blocks * threads;
  if (tflops) *tflops = (float)(flops / (t * 1e-3) / 1e12);
  if (ms) *ms = t;
  return GPUNB_OK;
}
