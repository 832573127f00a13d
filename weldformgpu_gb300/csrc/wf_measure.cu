// wf_measure.cu — the FP64 arithmetic ceiling the plain form is measured against.
//
// GB300 issues FP64 fused multiply-adds at a small fraction of the FP32 rate,
// so the plain FP64 form of the step is bound by the FP64 pipe, not by HBM.
// wf_fp64_fma_peak() measures that pipe's throughput on the current device:
// every thread runs eight independent chains of dependent FMAs (enough
// independent work per warp to keep the pipe busy), the grid covers every SM
// several times over, and CUDA events time the launch after a warm-up.
#include <cuda_runtime.h>

#include "../../include/weldform_gb300.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(int iters, double a, double b,
                                                        double* __restrict__ sink) {
  double v[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) v[c] = (double)(threadIdx.x + c) * 1.0e-3;
  for (int k = 0; k < iters; k++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) v[c] = fma(v[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += v[c];
  if (s == 1.2345e300) sink[blockIdx.x] = s;   // keeps the chains live; never true
}

}  // namespace

extern "C" int wf_fp64_fma_peak(double* gflops, double* ms_out) {
  if (!gflops) return WF_ERR_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return WF_ERR_CUDA;
  const int blocks = sms * 8;
  const int iters = 4096;
  double* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(double) * blocks) != cudaSuccess) return WF_ERR_ALLOC;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // a and b keep the values bounded (|a| < 1): no overflow or denormals
  k_fp64_fma<<<blocks, kThreads>>>(iters, 0.999999, 1.0e-7, sink);
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; r++) k_fp64_fma<<<blocks, kThreads>>>(iters, 0.999999, 1.0e-7, sink);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) return WF_ERR_CUDA;
  const double flops = 2.0 * kChains * (double)iters * kThreads * blocks * reps;
  *gflops = flops / (ms * 1.0e-3) / 1.0e9;
  if (ms_out) *ms_out = ms / reps;
  return WF_OK;
}
