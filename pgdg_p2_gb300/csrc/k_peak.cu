/*
 * k_peak.cu -- measured FP32 peak of the GPU the library runs on (no
 * reference counterpart; measurement only).
 *
 * The residual, limiter and shifting kernels of the mixed-precision path are
 * bound by the FP32 CUDA cores, not by HBM or the tensor cores, so their
 * roofline denominator is the rate of FP32 fused multiply-adds.  This kernel
 * runs eight independent FFMA chains per thread over every SM (four resident
 * blocks of 256 threads per SM) and the host times it with CUDA events.
 */
#include <cuda_runtime.h>

#include "../../include/pgdg.h"

namespace {

constexpr int CHAINS = 8, UNROLL = 16, THREADS = 256;

__global__ void __launch_bounds__(THREADS) k_ffma_peak(float* out, int iters, float a, float b) {
  float x[CHAINS];
#pragma unroll
  for (int k = 0; k < CHAINS; k++) x[k] = (float)(threadIdx.x + k) * 1e-3f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < UNROLL; u++)
#pragma unroll
      for (int k = 0; k < CHAINS; k++) x[k] = fmaf(x[k], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < CHAINS; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

/* the same chains as packed pairs (FFMA2: two FP32 multiply-adds per instruction) */
__global__ void __launch_bounds__(THREADS) k_ffma2_peak(float* out, int iters, float a, float b) {
  float2 x[CHAINS / 2];
#pragma unroll
  for (int k = 0; k < CHAINS / 2; k++) x[k] = make_float2((float)(threadIdx.x + 2 * k) * 1e-3f, (float)(threadIdx.x + 2 * k + 1) * 1e-3f);
  const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < UNROLL; u++)
#pragma unroll
      for (int k = 0; k < CHAINS / 2; k++) x[k] = __ffma2_rn(x[k], a2, b2);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < CHAINS / 2; k++) s += x[k].x + x[k].y;
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

namespace {
int measure(bool packed, double* tflops, double* ms_out) {
  if (!tflops) return PGDG_EINVAL;
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PGDG_ECUDA;
  const int blocks = nsm * 4;
  float* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc((void**)&out, sizeof(float) * (size_t)blocks * THREADS) != cudaSuccess) return PGDG_ENOMEM;
  int rc = PGDG_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = PGDG_ECUDA;
  const int iters = 4096;
  float ms = 0.f;
  if (rc == PGDG_OK) {
    auto launch = [&](int it) {
      if (packed) k_ffma2_peak<<<blocks, THREADS>>>(out, it, 0.999999f, 1e-6f);
      else k_ffma_peak<<<blocks, THREADS>>>(out, it, 0.999999f, 1e-6f);
    };
    launch(iters / 8); /* warm-up */
    cudaEventRecord(e0);
    launch(iters);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f)
      rc = PGDG_ECUDA;
  }
  if (rc == PGDG_OK) {
    const double flop = 2.0 * CHAINS * UNROLL * (double)iters * (double)blocks * THREADS;
    *tflops = flop / (ms * 1e-3) / 1e12;
    if (ms_out) *ms_out = ms;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  return rc;
}
}  // namespace

extern "C" int pgdg_fp32_peak(double* tflops, double* ms_out) { return measure(false, tflops, ms_out); }
extern "C" int pgdg_fp32_peak_packed(double* tflops, double* ms_out) { return measure(true, tflops, ms_out); }
