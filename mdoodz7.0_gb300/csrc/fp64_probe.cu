// fp64_probe.cu -- measurement and self-check helpers.
//
// mdz_rheo_measure_fp64_peak: the local rheology update is bound by the FP64 pipe,
// so roofline fractions are reported against a measured FP64 rate: every thread of a
// full-occupancy grid runs independent chains of dependent DFMAs (2 flops each),
// timed with CUDA events.
// mdz_rheo_math_selftest: the table-driven exp/log of fp64_math.cuh next to CUDA's
// exp/log on the same arguments, for the accuracy tests.
// mdz_rheo_div_selftest: the division by a known divisor of fp64_div.cuh next to CUDA's
// division, for the bit-for-bit test.
// mdz_rheo_quotient_selftest: the output quotient of fp64_div.cuh (two Newton steps on the
// reciprocal estimate), for the accuracy test against IEEE division.
// mdz_rheo_ceil_selftest: the integer-pipe ceil of fp64_bits.cuh next to CUDA's ceil.
// mdz_rheo_dd_selftest: the double-float conversion, exp and log of dd_math.cuh, for the
// accuracy tests.
#include <cuda_runtime.h>

#include "../../include/mdz_rheo.h"
#include "dd_math.cuh"
#include "fp64_div.cuh"
#include "fp64_math.cuh"

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

__global__ void k_math(const double *x, long long n, double *fe, double *ce, double *fl, double *cl) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  fe[i] = mdz::fast_exp(v);
  ce[i] = exp(v);
  fl[i] = mdz::fast_log(v);
  cl[i] = log(v);
}

__global__ void k_div(const double *a, long long n, mdz::Divisor d, double *fast, double *plain) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fast[i] = mdz::div_by(a[i], d);
  plain[i] = a[i] / d.b;
}

__global__ void k_quotient(const double *r, const double *den, long long n, double *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = mdz::quotient(r[i], den[i]);
}

__global__ void k_ceil(const double *q, long long n, int *fast, double *plain) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  fast[i] = mdz::fp64_ceil_int(q[i]);
  plain[i] = ceil(q[i]);
}

// per argument: dd_of_f64(x), dd_exp(dd_of_f64(x)), dd_log_f(x rounded to FP32), as
// (hi, lo) pairs
__global__ void k_dd(const double *x, long long n, float *out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const mdz::f2 a = mdz::dd_of_f64(x[i]);
  const mdz::f2 e = mdz::dd_exp(a);
  const float s = __double2float_rn(x[i]);
  const mdz::f2 l = (s > 1.17549435e-38f && s < 3.4e38f) ? mdz::dd_log_f(s) : mdz::f2{0.0f, 0.0f};
  float *o = out + 6 * i;
  o[0] = a.hi; o[1] = a.lo; o[2] = e.hi; o[3] = e.lo; o[4] = l.hi; o[5] = l.lo;
}

}  // namespace

extern "C" int mdz_rheo_dd_selftest(int device, const double *x, int64_t n, float *out) {
  if (!x || n < 0 || !out) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  const size_t bx = (size_t)n * sizeof(double), bo = (size_t)n * 6 * sizeof(float);
  void *d = nullptr;
  if (cudaMalloc(&d, bx + bo) != cudaSuccess) return MDZ_ENOMEM;
  double *dx = (double *)d;
  float *dout = (float *)((char *)d + bx);
  int rc = MDZ_OK;
  if (cudaMemcpy(dx, x, bx, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK) {
    k_dd<<<(unsigned)((n + 255) / 256), 256>>>(dx, n, dout);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = MDZ_ECUDA;
  }
  if (rc == MDZ_OK && cudaMemcpy(out, dout, bo, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  cudaFree(d);
  return rc;
}

extern "C" int mdz_rheo_quotient_selftest(int device, const double *r, const double *den, int64_t n,
                                          double *out) {
  if (!r || !den || n < 0 || !out) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  const size_t bytes = (size_t)n * sizeof(double);
  double *d = nullptr;
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return MDZ_ENOMEM;
  int rc = MDZ_OK;
  if (cudaMemcpy(d, r, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK && cudaMemcpy(d + n, den, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK) {
    k_quotient<<<(unsigned)((n + 255) / 256), 256>>>(d, d + n, n, d + 2 * n);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = MDZ_ECUDA;
  }
  if (rc == MDZ_OK && cudaMemcpy(out, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  cudaFree(d);
  return rc;
}

extern "C" int mdz_rheo_ceil_selftest(int device, const double *q, int64_t n, int32_t *fast_out, double *cuda_out) {
  if (!q || n < 0 || !fast_out || !cuda_out) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  const size_t bytes = (size_t)n * sizeof(double);
  double *d = nullptr;
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return MDZ_ENOMEM;
  int *di = (int *)(d + 2 * n);
  int rc = MDZ_OK;
  if (cudaMemcpy(d, q, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK) {
    k_ceil<<<(unsigned)((n + 255) / 256), 256>>>(d, n, di, d + n);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = MDZ_ECUDA;
  }
  if (rc == MDZ_OK && cudaMemcpy(fast_out, di, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    rc = MDZ_ECUDA;
  if (rc == MDZ_OK && cudaMemcpy(cuda_out, d + n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  cudaFree(d);
  return rc;
}

extern "C" int mdz_rheo_div_selftest(int device, const double *a, int64_t n, double b, double *fast_out,
                                     double *cuda_out) {
  if (!a || n < 0 || !fast_out || !cuda_out) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  const size_t bytes = (size_t)n * sizeof(double);
  double *d = nullptr;
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return MDZ_ENOMEM;
  int rc = MDZ_OK;
  if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK) {
    k_div<<<(unsigned)((n + 255) / 256), 256>>>(d, n, mdz::make_divisor(b), d + n, d + 2 * n);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = MDZ_ECUDA;
  }
  if (rc == MDZ_OK && cudaMemcpy(fast_out, d + n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK && cudaMemcpy(cuda_out, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  cudaFree(d);
  return rc;
}

extern "C" int mdz_rheo_math_selftest(int device, const double *x, int64_t n, double *fast_exp_out,
                                      double *cuda_exp_out, double *fast_log_out, double *cuda_log_out) {
  if (!x || n < 0 || !fast_exp_out || !cuda_exp_out || !fast_log_out || !cuda_log_out) return MDZ_EINVAL;
  if (n == 0) return MDZ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return MDZ_ECUDA;
  const size_t b = (size_t)n * sizeof(double);
  double *d = nullptr;
  if (cudaMalloc(&d, 5 * b) != cudaSuccess) return MDZ_ENOMEM;
  int rc = MDZ_OK;
  if (cudaMemcpy(d, x, b, cudaMemcpyHostToDevice) != cudaSuccess) rc = MDZ_ECUDA;
  if (rc == MDZ_OK) {
    k_math<<<(unsigned)((n + 255) / 256), 256>>>(d, n, d + n, d + 2 * n, d + 3 * n, d + 4 * n);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = MDZ_ECUDA;
  }
  double *outs[4] = {fast_exp_out, cuda_exp_out, fast_log_out, cuda_log_out};
  for (int k = 0; k < 4 && rc == MDZ_OK; k++)
    if (cudaMemcpy(outs[k], d + (k + 1) * n, b, cudaMemcpyDeviceToHost) != cudaSuccess) rc = MDZ_ECUDA;
  cudaFree(d);
  return rc;
}

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
