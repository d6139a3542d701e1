// common.cuh -- neutron state, random streams and math helpers shared by the
// propagation kernels.  Everything is templated on the working precision R
// (float for the fused fast path, double for the plain path).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/acc_gb300.h"

namespace mcv {

// mcni.utils.conversion (the reference reads these from mcni; V2K appears
// in acc/components/optics/guide_baseline.py:16-17).
constexpr double kV2K = 1.58825361e-3;
constexpr double kK2V = 1.0 / kV2K;
constexpr double kSE2V = 437.393377;
constexpr double kVS2E = 5.22703725e-6;
constexpr double kPi = 3.14159265358979323846;

// ------------------------------------------------------------ random streams
// Philox4x32-10 (Salmon et al., SC'11): counter (index lo, index hi, block,
// stream), key (seed lo, seed hi).  Each 128-bit block w0..w3 gives five
// 24-bit integers u (bits 0-23, 24-47, 48-71, 72-95, 96-119 of
// w0 | w1<<32 | w2<<64 | w3<<96) and so five float32-exact uniforms
// u * 2^-24; they are kept in registers and popped by shifting, so no
// local-memory indexing happens.
struct PhiloxStream {
  uint32_t k0, k1, c0, c1, c2, c3;
  uint32_t b0, b1, b2, b3, b4;
  int left;

  __device__ __forceinline__ PhiloxStream(uint64_t seed, uint64_t index,
                                          uint32_t stream)
      : k0((uint32_t)seed), k1((uint32_t)(seed >> 32)), c0((uint32_t)index),
        c1((uint32_t)(index >> 32)), c2(0), c3(stream), b0(0), b1(0), b2(0),
        b3(0), b4(0), left(0) {}

  __device__ __forceinline__ void refill() {
    uint32_t x0 = c0, x1 = c1, x2 = c2, x3 = c3, y0 = k0, y1 = k1;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      if (r) {
        y0 += 0x9E3779B9u;
        y1 += 0xBB67AE85u;
      }
      uint32_t lo0 = 0xD2511F53u * x0, hi0 = __umulhi(0xD2511F53u, x0);
      uint32_t lo1 = 0xCD9E8D57u * x2, hi1 = __umulhi(0xCD9E8D57u, x2);
      uint32_t n0 = hi1 ^ x1 ^ y0, n2 = hi0 ^ x3 ^ y1;
      x0 = n0;
      x1 = lo1;
      x2 = n2;
      x3 = lo0;
    }
    b0 = x0 & 0xFFFFFFu;
    b1 = __funnelshift_r(x0, x1, 24) & 0xFFFFFFu;
    b2 = __funnelshift_r(x1, x2, 16) & 0xFFFFFFu;
    b3 = x2 >> 8;
    b4 = x3 & 0xFFFFFFu;
    left = 5;
    ++c2;
  }

  // the neutron's index (the counter's low words)
  __device__ __forceinline__ uint64_t index() const {
    return (uint64_t)c0 | ((uint64_t)c1 << 32);
  }

  // float32-exact uniform u * 2^-24 in [0, 1)
  __device__ __forceinline__ float next() {
    if (left == 0) refill();
    uint32_t w = b0;
    b0 = b1;
    b1 = b2;
    b2 = b3;
    b3 = b4;
    --left;
    return __uint2float_rz(w) * 5.9604644775390625e-08f;
  }
  // the stream after k more draws, without forming them: whole blocks
  // move the counter, the rest come off a fresh block
  __device__ __forceinline__ void skip(int k) {
    if (k <= 0) return;
    if (k > left) {
      k -= left;
      left = 0;
      c2 += (uint32_t)(k / 5);
      k %= 5;
      if (k == 0) return;
      refill();
    }
    for (; k > 0; --k) next();
  }
  __device__ __forceinline__ int overrun() const { return 0; }
};

// Caller-given uniforms (replay / parity mode); bounded by `n`.
struct InjectedStream {
  const float* p;
  int n, i, bad;
  uint64_t idx;  // the neutron's index
  __device__ __forceinline__ InjectedStream(const float* ptr, int count,
                                            uint64_t index)
      : p(ptr), n(count), i(0), bad(0), idx(index) {}
  __device__ __forceinline__ uint64_t index() const { return idx; }
  __device__ __forceinline__ float next() {
    if (i < n) return p[i++];
    bad = 1;
    return 0.5f;
  }
  __device__ __forceinline__ void skip(int k) {
    if (k <= 0) return;
    if (k > n - i) {
      bad = 1;
      i = n;
    } else {
      i += k;
    }
  }
  __device__ __forceinline__ int overrun() const { return bad; }
};

// ------------------------------------------------------------ time of flight
// FP64 path: a double.  FP32 path: an unevaluated float pair (hi + lo)
// updated with Knuth's TwoSum, which keeps ~48 bits of the accumulated
// time of flight at about one tenth of the cost of a double add on GB300.
template <typename R>
struct Tof;

template <>
struct Tof<double> {
  double t;
  __device__ __forceinline__ void set(double v) { t = v; }
  __device__ __forceinline__ void add(double dt) { t = t + dt; }
  __device__ __forceinline__ double val() const { return t; }
  __device__ __forceinline__ double dval() const { return t; }
};

template <>
struct Tof<float> {
  float hi, lo;
  __device__ __forceinline__ void set(float v) {
    hi = v;
    lo = 0.f;
  }
  __device__ __forceinline__ void add(float dt) {
    float s = __fadd_rn(hi, dt);
    float bp = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(dt, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  __device__ __forceinline__ float val() const { return hi + lo; }
  __device__ __forceinline__ double dval() const {
    return (double)hi + (double)lo;
  }
};

template <typename R>
struct Neutron {
  R x, y, z, vx, vy, vz, sx, sy;
  Tof<R> t;
  R p;
};

// propagate by dt (acc/neutron.py:44-51)
template <typename R>
__device__ __forceinline__ void prop_dt(Neutron<R>& n, R dt) {
  n.x = n.x + n.vx * dt;
  n.y = n.y + n.vy * dt;
  n.z = n.z + n.vz * dt;
  n.t.add(dt);
}

// ------------------------------------------------------------ parameters
template <typename R>
__device__ __forceinline__ R prm(const mcv_component& c, int k);
template <>
__device__ __forceinline__ float prm<float>(const mcv_component& c, int k) {
  return c.fp[k];
}
template <>
__device__ __forceinline__ double prm<double>(const mcv_component& c, int k) {
  return c.dp[k];
}

template <typename R>
__device__ __forceinline__ const R* chain_rot(const mcv_chain& ch, int k);
template <>
__device__ __forceinline__ const float* chain_rot<float>(const mcv_chain& ch,
                                                         int k) {
  return ch.frot[k];
}
template <>
__device__ __forceinline__ const double* chain_rot<double>(const mcv_chain& ch,
                                                           int k) {
  return ch.rot[k];
}
template <typename R>
__device__ __forceinline__ const R* chain_off(const mcv_chain& ch, int k);
template <>
__device__ __forceinline__ const float* chain_off<float>(const mcv_chain& ch,
                                                         int k) {
  return ch.foff[k];
}
template <>
__device__ __forceinline__ const double* chain_off<double>(const mcv_chain& ch,
                                                           int k) {
  return ch.off[k];
}

// ------------------------------------------------------------ math
__device__ __forceinline__ float m_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double m_sqrt(double x) { return sqrt(x); }
// square root of a uniform: the reference applies math.sqrt to the float32
// that xoroshiro128p_uniform_float32 returns (the disc sources,
// source_simple.py:139, SNS_source.py:177, STS_source.py:257), which Numba
// types and evaluates as a float32 square root (correctly rounded); the
// FP64 kernels take the same float32 root of the same 24-bit uniform
__device__ __forceinline__ float m_sqrt_uniform(float u) { return sqrtf(u); }
__device__ __forceinline__ double m_sqrt_uniform(double u) {
  return double(__fsqrt_rn(float(u)));
}
__device__ __forceinline__ float m_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double m_rsqrt(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float m_exp(float x) { return __expf(x); }
__device__ __forceinline__ double m_exp(double x) { return exp(x); }
__device__ __forceinline__ float m_atan2(float y, float x) {
  return atan2f(y, x);
}
__device__ __forceinline__ double m_atan2(double y, double x) {
  return atan2(y, x);
}
__device__ __forceinline__ float m_asin(float x) { return asinf(x); }
__device__ __forceinline__ double m_asin(double x) { return asin(x); }
__device__ __forceinline__ float m_atan(float x) { return atanf(x); }
__device__ __forceinline__ double m_atan(double x) { return atan(x); }
__device__ __forceinline__ float m_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double m_fabs(double x) { return fabs(x); }
__device__ __forceinline__ int m_floori(float x) { return __float2int_rd(x); }
__device__ __forceinline__ int m_floori(double x) {
  return __double2int_rd(x);
}
__device__ __forceinline__ bool m_isnan(float x) { return x != x; }
__device__ __forceinline__ bool m_isnan(double x) { return x != x; }

// sin/cos of 2*pi*u for a uniform u: exact argument reduction in FP32,
// the reference's sin(phi), cos(phi) with phi = u*2*pi in FP64.
// sin and cos of 2 pi u, u in [0, 1): the hardware approximation on
// a = 2 pi (u - 1/2) in [-pi, pi), where its absolute error is below
// 2^-21.4, and sin(2 pi u) = -sin(a), cos(2 pi u) = -cos(a) exactly.  An
// angle drawn from a 24-bit uniform needs no more (the FP32 parity tests
// hold); against sincospif it raised the guide chain's FP32 rate by 2.8%.
__device__ __forceinline__ void m_sincos_2pi(float u, float* s, float* c) {
  const float a = 6.28318530717958647692f * (u - 0.5f);
  float sa, ca;
  __sincosf(a, &sa, &ca);
  *s = -sa;
  *c = -ca;
}
__device__ __forceinline__ void m_sincos_2pi(double u, double* s, double* c) {
  double phi = u * (2 * kPi);
  sincos(phi, s, c);
}

__device__ __forceinline__ int clampi(int i, int n) {
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// ------------------------------------------------------------ device status
struct DevStatus {
  unsigned long long processed;
  unsigned long long bounce_overflow;
  unsigned long long nonfinite;
  unsigned long long bin_oob;
  unsigned long long rng_overrun;
  unsigned long long work_next;  // persistent-launch work queue head
  unsigned long long spare[2];
};

}  // namespace mcv
