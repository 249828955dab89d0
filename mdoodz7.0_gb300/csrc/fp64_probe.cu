// fp64_probe.cu -- measured FP64 (DFMA) throughput of the current GPU.
//
// The local rheology update is bound by the FP64 pipe, and the generated peak
// file holds no FP64 figure, so roofline fractions are reported against this
// measured rate: every thread of a full-occupancy grid runs independent chains of
// dependent DFMAs (2 flops each), timed with CUDA events.
#include <cuda_runtime.h>

#include "../../include/mdz_rheo.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dfma(double *out, double a, double b, int iters) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * 1e-3 + c;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 12345.678) out[0] = s;  // keep the chains live
}

}  // namespace

extern "C" int mdz_rheo_measure_fp64_peak(int device, double *tflops) {
  if (!tflops) return MDZ_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dfma, 256, 0);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return MDZ_ECUDA;
  const int blocks = sms * (per_sm > 0 ? per_sm : 1), iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma<<<blocks, 256>>>(out, 0.999999, 1e-7, iters);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(e0);
    k_dfma<<<blocks, 256>>>(out, 0.999999, 1e-7, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return MDZ_ECUDA;
  const double flops = 2.0 * kChains * (double)iters * blocks * 256.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return MDZ_OK;
}
