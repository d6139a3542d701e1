// track.cuh -- what a kernel does at the points where a neutron's weight
// picks up a parameter-dependent factor, and at tallies.
//
// NoTrack (forward kernels) adds tallies and ignores the weight factors; it
// compiles to nothing else.  GradTrack (the backward replay) follows the
// same neutron -- same Philox counter, same arithmetic -- and accumulates
// d ln p / d theta for the differentiable parameters; at a tally in bin b
// it adds dL/d(sum p)_b * p * d ln p / d theta to the gradient.  Every
// parameter handled here enters only the weight: with the random numbers
// fixed the path does not depend on it, so this is the exact derivative of
// the estimator (the common-random-number derivative).
#pragma once

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "common.cuh"

namespace mcv {

struct Tally {
  double* out;
  uint64_t nbins;
  double down;     // 2^-weight_exp2: the FP32 weight scale divided out
  bool aggregate;  // MCV_COMP_AGGREGATE: warp-aggregated atomics
  double* sm;      // MCV_COMP_SMEM_TALLY: the block's shared-memory copy
};

// The FP32 weight scale of a chain (mcv_chain.weight_exp2, |e| <= 126):
// the source's weight is multiplied by 2^e, tallies and outputs by 2^-e,
// both exact powers of two built from the exponent bits where they are
// used (the chain lives in the constant bank, so nothing stays in a
// register).  The FP64 kernels use 1 and 1.
template <typename R>
__device__ __forceinline__ R weight_up(const mcv_chain& ch) {
  if constexpr (sizeof(R) == 4)
    return __int_as_float((127 + ch.weight_exp2) << 23);
  else
    return R(1);
}
template <typename R>
__device__ __forceinline__ double weight_down(const mcv_chain& ch) {
  if constexpr (sizeof(R) == 4)
    return __longlong_as_double((long long)(1023 - ch.weight_exp2) << 52);
  else
    return 1.0;
}

// Warp-aggregated entry (MCV_COMP_AGGREGATE): the lanes that reach this
// call together (cooperative_groups::coalesced_threads) and hit the same
// bin of the same tally (labeled_partition on the bin's address) first sum
// their count, p and p^2 inside the warp, and the group's first lane makes
// the three atomics.  Not inlined, so that its registers do not weigh on
// the kernels that do not take it.
static __device__ __noinline__ void tally_add_aggregated(double* a,
                                                         uint64_t nbins,
                                                         double p) {
  namespace cg = cooperative_groups;
  const cg::coalesced_group active = cg::coalesced_threads();
  const cg::coalesced_group peers =
      cg::labeled_partition(active, (unsigned long long)(uintptr_t)a);
  const double s1 = cg::reduce(peers, p, cg::plus<double>());
  const double s2 = cg::reduce(peers, p * p, cg::plus<double>());
  if (peers.thread_rank() != 0) return;
  atomicAdd(a, (double)peers.size());
  atomicAdd(a + nbins, s1);
  atomicAdd(a + 2 * nbins, s2);
}

// Lanes of one warp entering the same bin at once make the L2 serialise
// their atomics; from this many on, the entry is warp-aggregated.
constexpr int kHotLanes = 4;

// One entry (1, p, p^2) into bin `bin`: three FP64 atomics into the
// L2-resident histogram.  The lanes that reach the call together first
// check, with one shuffle and one vote, how many of them hit the bin of
// the group's first lane; when kHotLanes or more do (a beam into a few
// bins, a fixed (Q, E) transfer), the warp aggregates its entries before
// the atomics.  Measured on GB300: always aggregating costs 15-35% on
// monitors whose entries spread over many bins, and gains 3.8x on the
// constant-(Q, E) box, whose entries land in one or two bins.
// MCV_COMP_AGGREGATE forces the aggregated path.
__device__ __forceinline__ void tally_add(const Tally& t, uint64_t bin,
                                          double p) {
  if (!t.out) return;
  if (t.sm) {
    // the block's copy in shared memory (MCV_COMP_SMEM_TALLY), added to
    // the tally when the block ends
    atomicAdd(t.sm + bin, 1.0);
    atomicAdd(t.sm + t.nbins + bin, p);
    atomicAdd(t.sm + 2 * t.nbins + bin, p * p);
    return;
  }
  double* a = t.out + bin;
  // the lanes that reach this call together: every lane of the mask runs
  // the straight-line code from here to the vote, so the shuffle and the
  // vote are reached by all of them (coalesced_threads().shfl / ballot do
  // the same with a rank-space bit compaction that measured 7% slower on
  // the thread kernel)
  const unsigned mask = __activemask();
  const unsigned long long mine = (unsigned long long)(uintptr_t)a;
  const unsigned long long lead = __shfl_sync(mask, mine, __ffs(mask) - 1);
  const unsigned same = __ballot_sync(mask, mine == lead);
  if (t.aggregate || __popc(same) >= kHotLanes) {
    tally_add_aggregated(a, t.nbins, p);
    return;
  }
  atomicAdd(a, 1.0);
  atomicAdd(a + t.nbins, p);
  atomicAdd(a + 2 * t.nbins, p * p);
}
__device__ __forceinline__ void tally_add(const Tally& t, uint64_t bin,
                                          float p) {
  // the weight scale is divided out and p^2 formed in double
  tally_add(t, bin, (double)p * t.down);
}

struct NoTrack {
  static constexpr bool kActive = false;
  // per-neutron words the regeneration kernel's tail queue carries
  static constexpr int kQueueWords = 0;
  __device__ __forceinline__ void save(uint32_t*, int, int) const {}
  __device__ __forceinline__ void load(const uint32_t*, int, int) {}
  __device__ __forceinline__ void begin_neutron() {}
  __device__ __forceinline__ void begin_component(const mcv_chain&, int) {}
  template <typename R>
  __device__ __forceinline__ void reflect(R, R, R, R, R, R) {}
  template <typename R>
  __device__ __forceinline__ void atten(R, R) {}
  template <typename R>
  __device__ __forceinline__ void sigma_factor(R) {}
  template <typename R>
  __device__ __forceinline__ void powder_atten(int, R) {}
  template <typename R>
  __device__ __forceinline__ void powder_peak(int, R) {}
  template <typename R>
  __device__ __forceinline__ void sqe(int, int, R, R, double) {}
  template <typename R>
  __device__ __forceinline__ void tally(const Tally& t, uint64_t bin, R p) {
    tally_add(t, bin, p);
  }
};

enum { kGradGuides = 2 };

template <typename R>
struct GradTrack {
  static constexpr bool kActive = true;
  const mcv_grad& g;
  double* powder_x;  // [npeaks+1]: sum over neutrons reaching K peaks
  double* powder_y;  // [npeaks]:   chosen-peak terms
  int cur = 0, gslot = -1, is_hss = 0;
  // per-neutron d ln p / d theta
  R dg[kGradGuides][3];
  R dmu, dsig;
  int sqe_base;
  R sqe_fx, sqe_fy;
  double sqe_invS;  // 1/S can overflow float for tiny S
  int pk1, pk2, peak;
  R pc1, pc2, inv_s;
  // per-thread gradient sums
  double acc_g[kGradGuides][3];
  double acc_mu, acc_sig;

  int hss_comp = -1, sqe_nE = 0;

  // The per-neutron state above, as queue words (FP32): word w of the
  // neutron in `slot` lives at q[w * stride + slot].
  static constexpr int kQueueWords = 19;
  __device__ __forceinline__ void save(uint32_t* q, int stride,
                                       int slot) const {
    const uint32_t w[kQueueWords] = {
        rbits(dg[0][0]), rbits(dg[0][1]), rbits(dg[0][2]),
        rbits(dg[1][0]), rbits(dg[1][1]), rbits(dg[1][2]),
        rbits(dmu),      rbits(dsig),     (uint32_t)sqe_base,
        rbits(sqe_fx),   rbits(sqe_fy),
        (uint32_t)__double2loint(sqe_invS),
        (uint32_t)__double2hiint(sqe_invS),
        (uint32_t)pk1,   (uint32_t)pk2,   (uint32_t)peak,
        rbits(pc1),      rbits(pc2),      rbits(inv_s)};
#pragma unroll
    for (int k = 0; k < kQueueWords; ++k) q[k * stride + slot] = w[k];
  }
  __device__ __forceinline__ void load(const uint32_t* q, int stride,
                                       int slot) {
    uint32_t w[kQueueWords];
#pragma unroll
    for (int k = 0; k < kQueueWords; ++k) w[k] = q[k * stride + slot];
    dg[0][0] = rval(w[0]);
    dg[0][1] = rval(w[1]);
    dg[0][2] = rval(w[2]);
    dg[1][0] = rval(w[3]);
    dg[1][1] = rval(w[4]);
    dg[1][2] = rval(w[5]);
    dmu = rval(w[6]);
    dsig = rval(w[7]);
    sqe_base = (int)w[8];
    sqe_fx = rval(w[9]);
    sqe_fy = rval(w[10]);
    sqe_invS = __hiloint2double((int)w[12], (int)w[11]);
    pk1 = (int)w[13];
    pk2 = (int)w[14];
    peak = (int)w[15];
    pc1 = rval(w[16]);
    pc2 = rval(w[17]);
    inv_s = rval(w[18]);
  }
  // (queue words hold FP32 values: the queue is used by the FP32 kernel)
  static __device__ __forceinline__ uint32_t rbits(R v) {
    return __float_as_uint((float)v);
  }
  static __device__ __forceinline__ R rval(uint32_t w) {
    return R(__uint_as_float(w));
  }

  // the first HSS of the chain is the differentiated sample
  __device__ GradTrack(const mcv_grad& grad, const mcv_chain& ch, double* px,
                       double* py)
      : g(grad), powder_x(px), powder_y(py) {
    for (int c = ch.ncomp - 1; c >= 0; --c)
      if (ch.comp[c].opcode == MCV_OP_HSS) hss_comp = c;
    if (hss_comp >= 0) sqe_nE = ch.comp[hss_comp].ip[5];
#pragma unroll
    for (int s = 0; s < kGradGuides; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) acc_g[s][k] = 0.0;
    acc_mu = acc_sig = 0.0;
    begin_neutron();
  }

  __device__ __forceinline__ void begin_neutron() {
#pragma unroll
    for (int s = 0; s < kGradGuides; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) dg[s][k] = R(0);
    dmu = dsig = R(0);
    sqe_base = -1;
    sqe_fx = sqe_fy = R(0);
    sqe_invS = 0.0;
    pk1 = pk2 = peak = -1;
    pc1 = pc2 = inv_s = R(0);
  }

  // guides count 0, 1 in chain order; more guides are not differentiated
  __device__ __forceinline__ void begin_component(const mcv_chain& ch,
                                                  int c) {
    cur = c;
    int s = 0;
    for (int k = 0; k < c; ++k) s += ch.comp[k].opcode == MCV_OP_GUIDE;
    gslot = (ch.comp[c].opcode == MCV_OP_GUIDE && s < kGradGuides) ? s : -1;
    is_hss = c == hss_comp;
  }

  // d ln R / d(m, alpha, W) of calc_reflectivity (_guide_utils.py:6-23):
  // R = R0 (1 - tanh x)(1 - alpha (Q - Qc)) / 2, x = (Q - m Qc) / W, and
  // d ln(1 - tanh x) / dx = -(1 + tanh x) = -2 / (1 + e^(-2x)).
  __device__ __forceinline__ void reflect(R Q, R R0, R Qc, R alpha, R m,
                                          R W) {
    if (gslot < 0 || !(Q > Qc)) return;
    R x = (Q - m * Qc) / W;
    if (!(x < R(10))) return;
    R one_plus_tanh = R(2) / (R(1) + m_exp(R(-2) * x));
    R da = Q - Qc;
    R s0 = one_plus_tanh * Qc / W, s2 = one_plus_tanh * x / W;
    R s1 = -da / (R(1) - alpha * da);
    if (gslot == 0) {
      dg[0][0] += s0;
      dg[0][1] += s1;
      dg[0][2] += s2;
    } else {
      dg[1][0] += s0;
      dg[1][1] += s1;
      dg[1][2] += s2;
    }
  }
  // attenuation exp(-(mu(v) + sigma) L): d/dmu2200 = -2200 L / v,
  // d/dsigma = -L (a kernel with a constant scattering coefficient)
  __device__ __forceinline__ void atten(R dmu_, R dsig_) {
    if (!is_hss) return;
    dmu += dmu_;
    dsig += dsig_;
  }
  __device__ __forceinline__ void sigma_factor(R sigma) {
    if (is_hss && sigma != R(0)) dsig += R(1) / sigma;
  }
  // powder attenuation: d ln p / d s_j = coef for the K reachable peaks
  __device__ __forceinline__ void powder_atten(int K, R coef) {
    if (!is_hss) return;
    if (pk1 < 0 || pk1 == K) {
      pk1 = K;
      pc1 += coef;
    } else {
      pk2 = K;
      pc2 += coef;
    }
  }
  __device__ __forceinline__ void powder_peak(int j, R s) {
    if (!is_hss) return;
    peak = j;
    inv_s = R(1) / s;
  }
  // bilinear S(Q,E): d ln p / d S_corner = weight_corner / S
  // S: the interpolated table value, unscaled, in double
  __device__ __forceinline__ void sqe(int base, int nE, R fx, R fy, double S) {
    if (!is_hss || !(S > 0.0)) return;
    sqe_base = base;
    sqe_fx = fx;
    sqe_fy = fy;
    sqe_invS = 1.0 / S;
    (void)nE;
  }

  __device__ __forceinline__ void tally(const Tally& t, uint64_t bin, R p) {
    const double* d = g.dout[cur];
    if (!d) return;
    double gb = d[bin];
    if (gb == 0.0) return;
    double gp = gb * ((double)p * t.down);
#pragma unroll
    for (int s = 0; s < kGradGuides; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) acc_g[s][k] += gp * (double)dg[s][k];
    acc_mu += gp * (double)dmu;
    acc_sig += gp * (double)dsig;
    tables(gp);
  }

  __device__ __forceinline__ void tables(double gp) {
    if (hss_comp < 0) return;
    double* dt = g.dtable[hss_comp];
    if (sqe_base >= 0 && dt) {
      double w = gp * sqe_invS;
      double fx = sqe_fx, fy = sqe_fy;
      atomicAdd(dt + sqe_base, w * (1 - fx) * (1 - fy));
      atomicAdd(dt + sqe_base + sqe_nE, w * fx * (1 - fy));
      atomicAdd(dt + sqe_base + 1, w * (1 - fx) * fy);
      atomicAdd(dt + sqe_base + sqe_nE + 1, w * fx * fy);
    }
    if (powder_x) {
      if (pk1 >= 0) atomicAdd(powder_x + pk1, gp * (double)pc1);
      if (pk2 >= 0) atomicAdd(powder_x + pk2, gp * (double)pc2);
      if (peak >= 0) atomicAdd(powder_y + peak, gp * (double)inv_s);
    }
  }

  // warp-reduce the per-thread sums and add them to the gradient arrays
  __device__ void flush(const mcv_chain& ch) {
    int s = 0;
    for (int c = 0; c < ch.ncomp; ++c) {
      int op = ch.comp[c].opcode;
      if (op == MCV_OP_GUIDE) {
        if (s < kGradGuides) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            double v = s == 0 ? acc_g[0][k] : acc_g[1][k];
            for (int o = 16; o > 0; o >>= 1)
              v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0 && g.dparam[c])
              atomicAdd(g.dparam[c] + k, v);
          }
        }
        ++s;
      } else if (c == hss_comp) {
        double v0 = acc_mu, v1 = acc_sig;
        for (int o = 16; o > 0; o >>= 1) {
          v0 += __shfl_down_sync(0xffffffffu, v0, o);
          v1 += __shfl_down_sync(0xffffffffu, v1, o);
        }
        if ((threadIdx.x & 31) == 0 && g.dparam[c]) {
          atomicAdd(g.dparam[c] + 0, v0);
          atomicAdd(g.dparam[c] + 1, v1);
        }
      }
    }
  }
};

}  // namespace mcv
