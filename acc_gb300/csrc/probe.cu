// probe.cu -- FMA-pipe, special-function-unit and L2-atomic throughput
// probes (include/acc_gb300_probe.h).

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/acc_gb300_probe.h"

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_kernel(int iters, T seed, T* sink) {
  T a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = seed + T(threadIdx.x + k);
  const T b = T(0.999999), c = T(1e-7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == T(-12345.678)) *sink = s;  // never true; keeps the chains live
}

// kChains independent chains of one base-2 exponential each (the
// special-function unit's ex2.approx, flushing denormals): a chain's value
// saturates within a few steps, which does not change the unit's rate
__global__ void __launch_bounds__(256) sfu_kernel(int iters, float seed,
                                                  float* sink) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = seed * float(threadIdx.x + k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k)
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(a[k]));
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == -12345.678f) *sink = s;  // never true; keeps the chains live
}

__global__ void __launch_bounds__(256)
    atomic_kernel(double* hist, uint64_t nbins, int iters) {
  uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t h = t * 0x9E3779B97F4A7C15ull;
  for (int i = 0; i < iters; ++i) {
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    atomicAdd(hist + (h % nbins), 1.0);
  }
}

template <typename T>
int fma_peak(int device, int repeats, double* out) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_kernel<T>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  int blocks = sms * per_sm;
  T* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(T)) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = sizeof(T) == 4 ? 20000 : 400;
  double best = 0;
  for (int r = 0; r < repeats + 1; ++r) {
    cudaEventRecord(e0);
    fma_kernel<T><<<blocks, 256>>>(iters, T(1), sink);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * kChains * (double)iters * blocks * 256.0;
    double tf = flops / (ms * 1e-3) / 1e12;
    if (r > 0 && tf > best) best = tf;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  *out = best;
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace

extern "C" int mcv_probe_fma_peak(int device, int precision, int repeats,
                                  double* tflops) {
  if (!tflops || repeats < 1) return 1;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  int rc = precision == 32   ? fma_peak<float>(device, repeats, tflops)
           : precision == 64 ? fma_peak<double>(device, repeats, tflops)
                             : 1;
  cudaSetDevice(prev);
  return rc;
}

extern "C" int mcv_probe_sfu_rate(int device, int repeats,
                                  double* ops_per_s) {
  if (!ops_per_s || repeats < 1) return 1;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sfu_kernel, 256, 0);
  if (per_sm < 1) per_sm = 1;
  const int blocks = sms * per_sm, iters = 4000;
  float* sink = nullptr;
  if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess) {
    cudaSetDevice(prev);
    return 2;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int r = 0; r < repeats + 1; ++r) {
    cudaEventRecord(e0);
    sfu_kernel<<<blocks, 256>>>(iters, 1e-3f, sink);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    const double ops =
        (double)kChains * iters * blocks * 256.0 / (ms * 1e-3);
    if (r > 0 && ops > best) best = ops;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  cudaSetDevice(prev);
  *ops_per_s = best;
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

extern "C" int mcv_probe_atomic_rate(int device, uint64_t nbins, int repeats,
                                     double* ops_per_s) {
  if (!ops_per_s || nbins == 0 || repeats < 1) return 1;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double* hist = nullptr;
  if (cudaMalloc(&hist, nbins * sizeof(double)) != cudaSuccess) {
    cudaSetDevice(prev);
    return 2;
  }
  cudaMemset(hist, 0, nbins * sizeof(double));
  int blocks = sms * 8, iters = 512;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0;
  for (int r = 0; r < repeats + 1; ++r) {
    cudaEventRecord(e0);
    atomic_kernel<<<blocks, 256>>>(hist, nbins, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)blocks * 256.0 * iters / (ms * 1e-3);
    if (r > 0 && ops > best) best = ops;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(hist);
  cudaSetDevice(prev);
  *ops_per_s = best;
  return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
