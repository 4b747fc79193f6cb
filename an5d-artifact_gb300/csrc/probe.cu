// Measures the FP32/FP64 fused multiply-add throughput of the current device
// (the FP term of the stencil roofline min(HBM*bt/(2*S), P_FP/FPP)).
#include <cuda_runtime.h>

#include "engine_internal.h"

namespace {
template <typename T, int CH>
__global__ void __launch_bounds__(256) fma_probe(T *out, int iters, T a, T b) {
  T x[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) x[c] = (T)(threadIdx.x * 1e-3 + c);
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 16; ++r)
#pragma unroll
      for (int c = 0; c < CH; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += x[c];
  if (s == (T)-1.2345) out[0] = s;  // never true; keeps the chains alive
}

template <typename T>
gbs_status measure(double *gflops) {
  constexpr int CH = 8;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  const int iters = sizeof(T) == 4 ? 4096 : 64;
  T *out = nullptr;
  cudaError_t e = cudaMalloc(&out, sizeof(T));
  if (e != cudaSuccess) return gbs::cuda_fail(e, "cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    fma_probe<T, CH><<<blocks, threads>>>(out, iters, (T)0.9999, (T)1e-4);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return gbs::cuda_fail(e, "fma probe");
  const double flops = 2.0 * CH * 16.0 * iters * (double)blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return GBS_OK;
}
}  // namespace

extern "C" gbs_status gbs_measure_fp_peak(int dtype, double *gflops) {
  if (!gflops) return gbs::fail(GBS_ERR_INVALID, "gflops is NULL");
  if (dtype == GBS_F32) return measure<float>(gflops);
  if (dtype == GBS_F64) return measure<double>(gflops);
  return gbs::fail(GBS_ERR_INVALID, "dtype must be GBS_F32 or GBS_F64");
}

// ---------------------------------------------------------------------------
// Self-test of the constant-divisor division (div_by in gbs_device.cuh)
// against IEEE division: every float input, or `samples` pseudo-random
// double inputs (all bit patterns equally likely) plus the binade edges.
// ---------------------------------------------------------------------------
#include "gbs_device.cuh"

namespace {
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__global__ void div_check_f32(float d, float y, int fast, unsigned long long count, unsigned long long *mism) {
  unsigned long long bad = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    const float x = __uint_as_float((unsigned)i);
    const float a = fast ? gbs::div_by_fast(x, d, y) : gbs::div_by(x, d, y), b = __fdiv_rn(x, d);
    if (__float_as_uint(a) != __float_as_uint(b) && !(isnan(a) && isnan(b))) ++bad;
  }
  if (bad) atomicAdd(mism, bad);
}

__global__ void div_check_f64(double d, double y, unsigned long long count, unsigned long long *mism) {
  unsigned long long bad = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
    unsigned long long bits = mix64(i);
    if (i < 4096) {  // binade edges: mantissa all-zeros / all-ones at every exponent
      const unsigned long long e = (i >> 1) & 0x7ff, s = (i >> 12) & 1;
      bits = (s << 63) | (e << 52) | ((i & 1) ? 0xfffffffffffffull : 0ull);
    }
    const double x = __longlong_as_double((long long)bits);
    const double a = gbs::div_by(x, d, y), b = __ddiv_rn(x, d);
    if (__double_as_longlong(a) != __double_as_longlong(b) && !(isnan(a) && isnan(b))) ++bad;
  }
  if (bad) atomicAdd(mism, bad);
}
}  // namespace

extern "C" gbs_status gbs_check_division(int dtype, double divisor, int checked, long long samples,
                                         long long *mismatches) {
  if (!mismatches) return gbs::fail(GBS_ERR_INVALID, "mismatches is NULL");
  if (divisor == 0.0) return gbs::fail(GBS_ERR_INVALID, "divisor must be nonzero");
  unsigned long long *m = nullptr;
  cudaError_t e = cudaMalloc(&m, sizeof *m);
  if (e != cudaSuccess) return gbs::cuda_fail(e, "cudaMalloc");
  cudaMemset(m, 0, sizeof *m);
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (dtype == GBS_F32) {
    const float d = (float)divisor, y = gbs::div_reciprocal<float>(divisor);
    const unsigned long long count = samples > 0 ? (unsigned long long)samples : (1ull << 32);
    div_check_f32<<<sms * 8, 256>>>(d, y, checked ? 0 : 1, count, m);
  } else if (dtype == GBS_F64) {
    const double y = gbs::div_reciprocal<double>(divisor);
    const unsigned long long count = samples > 0 ? (unsigned long long)samples : (1ull << 28);
    div_check_f64<<<sms * 8, 256>>>(divisor, y, count, m);
  } else {
    cudaFree(m);
    return gbs::fail(GBS_ERR_INVALID, "dtype must be GBS_F32 or GBS_F64");
  }
  unsigned long long h = 0;
  e = cudaMemcpy(&h, m, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(m);
  if (e != cudaSuccess) return gbs::cuda_fail(e, "division self-test");
  *mismatches = (long long)h;
  return GBS_OK;
}
