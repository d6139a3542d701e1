// kernels.cuh -- the propagation kernels and their per-precision launchers.
//
// One thread carries one neutron at a time through the whole chain; the
// grid strides over neutron indices.  The chain description is a
// __grid_constant__ kernel parameter, so component parameters are read from
// the constant bank and every lane of a warp dispatches on the same opcode.
//
// Launchers<R> is instantiated once per precision in its own translation
// unit (launch_fp32.cu, launch_fp64.cu) so that each can be compiled with
// its own floating-point contraction setting.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "components.cuh"
#include "monitors.cuh"
#include "ms.cuh"
#include "sample.cuh"

namespace mcv {

enum { kFlagIdentityRot = MCV_COMP_IDENTITY_ROT,
       kFlagAggregate = MCV_COMP_AGGREGATE,
       kFlagSmemTally = MCV_COMP_SMEM_TALLY };

__host__ __device__ __forceinline__ uint64_t comp_nbins(
    const mcv_component& c) {
  switch (c.opcode) {
    case MCV_OP_PSD_MONITOR:
    case MCV_OP_PSD_MONITOR_4PI:
    case MCV_OP_POSDIV_MONITOR:
    case MCV_OP_IQE_MONITOR:
    case MCV_OP_THETA_TOF_4PI:
    case MCV_OP_CYL_IQE_DETECTOR:
      return (uint64_t)c.ip[0] * (uint64_t)c.ip[1];
    case MCV_OP_WAVELENGTH_MONITOR:
    case MCV_OP_ENERGY_MONITOR:
      return (uint64_t)c.ip[0];
    case MCV_OP_BANKED_DETECTOR:
      return (uint64_t)c.ip[0] * c.ip[1] * c.ip[2] * c.ip[3];
    default:
      return 0;
  }
}

// r' = rot (r - off), v' = rot v  (acc/vec3.py:148-159, acc/neutron.py:18-23)
template <typename R>
__device__ __forceinline__ void apply_transform(Neutron<R>& n,
                                                const mcv_chain& ch, int k) {
  const R* o = chain_off<R>(ch, k);
  R tx = n.x - o[0], ty = n.y - o[1], tz = n.z - o[2];
  if (ch.comp[k].flags & kFlagIdentityRot) {
    n.x = tx;
    n.y = ty;
    n.z = tz;
    return;
  }
  const R* m = chain_rot<R>(ch, k);
  n.x = m[0] * tx + m[1] * ty + m[2] * tz;
  n.y = m[3] * tx + m[4] * ty + m[5] * tz;
  n.z = m[6] * tx + m[7] * ty + m[8] * tz;
  R vx = m[0] * n.vx + m[1] * n.vy + m[2] * n.vz;
  R vy = m[3] * n.vx + m[4] * n.vy + m[5] * n.vz;
  R vz = m[6] * n.vx + m[7] * n.vy + m[8] * n.vz;
  n.vx = vx;
  n.vy = vy;
  n.vz = vz;
}

// One component on one neutron; returns 1 when a guide ran out of bounces.
// kX: the instantiation for chains with the rarer components (SNS source,
// tapered guide, multiple scatterer); the common kernels leave their code
// out so that it weighs on neither their registers nor their instruction
// stream (the host launches the kX kernels for such chains only).
// `smt`: the block's shared-memory tally area (the regeneration kernel's;
// NULL elsewhere), where monitors flagged MCV_COMP_SMEM_TALLY add.
template <typename R, bool kX = false, typename Rng, typename Trk>
__device__ __forceinline__ int run_component(Neutron<R>& n, Rng& rng,
                                             const mcv_component& c,
                                             Trk& trk, const mcv_chain& ch,
                                             double* smt = nullptr) {
  Tally tl{c.tally, comp_nbins(c), weight_down<R>(ch),
           (c.flags & kFlagAggregate) != 0,
           (smt && (c.flags & kFlagSmemTally)) ? smt + c.ip[6] : nullptr};
  switch (c.opcode) {
    case MCV_OP_SOURCE_SIMPLE:
      source_simple<R>(n, rng, c);
      if constexpr (sizeof(R) == 4) n.p *= weight_up<R>(ch);
      return 0;
    case MCV_OP_NEUTRON_STORAGE:
      if constexpr (kX) {
        storage_source<R>(n, rng.index(), c);
        if constexpr (sizeof(R) == 4) n.p *= weight_up<R>(ch);
      }
      return 0;
    case MCV_OP_NEUTRON_TO_STORAGE:
      if constexpr (kX) neutron_to_storage<R>(n, rng.index(), c, tl.down);
      return 0;
    case MCV_OP_SNS_SOURCE:
      if constexpr (kX) {
        sns_source<R>(n, rng, c);
        if constexpr (sizeof(R) == 4) n.p *= weight_up<R>(ch);
      }
      return 0;
    case MCV_OP_GUIDE:
      return guide<R>(n, c, trk);
    case MCV_OP_GUIDE_TAPERING:
      if constexpr (kX) return guide_tapering<R>(n, c);
      return 0;
    case MCV_OP_GUIDE_ANYSHAPE:
      if constexpr (kX) {
        if (c.ip[2] & 1) return guide_anyshape_gravity<R>(n, c);
        return guide_anyshape<R>(n, c);
      }
      return 0;
    case MCV_OP_HSS:
      hss<kX>(n, rng, c, trk);
      return 0;
    case MCV_OP_PSD_MONITOR:
      psd_monitor<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_PSD_MONITOR_4PI:
      psd_monitor_4pi<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_WAVELENGTH_MONITOR:
      wavelength_monitor<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_POSDIV_MONITOR:
      posdiv_monitor<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_IQE_MONITOR:
      iqe_monitor<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_ENERGY_MONITOR:
      energy_monitor<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_THETA_TOF_4PI:
      theta_tof_4pi<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_CYL_IQE_DETECTOR:
      cyl_iqe<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_BANKED_DETECTOR:
      banked<R>(n, c, tl, trk);
      return 0;
    case MCV_OP_SLIT:
      slit_or_beamstop<R>(n, c, false, weight_up<R>(ch));
      return 0;
    case MCV_OP_BEAMSTOP:
      slit_or_beamstop<R>(n, c, true, weight_up<R>(ch));
      return 0;
    default:  // MCV_OP_ARM
      return 0;
  }
}

struct Counters {
  unsigned processed, overflow, nonfinite, overrun;
};

// The components after multiple scatterer `c` on one of its output
// neutrons; returns the index of the last component reached.  Not
// inlined: the scattering tree calls it from several places.
template <typename R, bool kX, typename Rng>
__device__ __noinline__ int ms_downstream(Neutron<R> m, Rng& rng,
                                          const mcv_chain& ch, int c,
                                          Counters& k) {
  NoTrack trk;
  int last = c;
  for (int c2 = c + 1; c2 < ch.ncomp; ++c2) {
    apply_transform<R>(m, ch, c2);
    last = c2;
    k.overflow += run_component<R, kX>(m, rng, ch.comp[c2], trk, ch);
    if (!(m.p > 0)) {
      if (m_isnan(m.p)) k.nonfinite++;
      break;
    }
  }
  return last;
}

// The multiple scatterer's fan-out in the thread kernel: the rest of the
// chain for every output neutron, on the same stream (run_script.py:66-92,
// 245-260); outputs run it as they become final unless a later component
// draws random numbers (ms_downstream_draws), when they wait in `outs` for
// the whole tree as in the reference.  Out of line, so that the tree's
// lists and registers do not weigh on the chains without a multiple
// scatterer that share the kernel.  Returns the last component reached.
template <typename R, typename Rng>
__device__ __noinline__ int ms_fan_out(const Neutron<R>& n, Rng& rng,
                                       const mcv_chain& ch, int c,
                                       Counters& k) {
  const bool hold = ms_downstream_draws(ch, c);
  Neutron<R> outs[MCV_MS_MAX_SCATTERED];
  int nout = 0, last = c;
  auto emit = [&](const Neutron<R>& o) {
    if (hold) outs[nout++] = o;
    else last = ms_downstream<R, true>(o, rng, ch, c, k);
  };
  ms_scatter<R>(ch.comp[c], rng, n, weight_up<R>(ch), emit);
  for (int j = 0; j < nout; ++j)
    last = ms_downstream<R, true>(outs[j], rng, ch, c, k);
  return last;
}

// Whole chain on one neutron (the body of the generated
// process_kernel_no_buffer, acc/run_script.py:182-196).  A neutron leaves
// the chain after a component that leaves its weight not positive.
template <typename R, bool kX = false, typename Rng, typename Trk = NoTrack>
__device__ __forceinline__ int run_chain_one(Neutron<R>& n, Rng& rng,
                                             const mcv_chain& ch,
                                             Counters& k, Trk&& trk = Trk()) {
  // The loop runs over every component for every lane (a dead neutron
  // skips the body) so that c stays warp-uniform: component parameters are
  // then read at uniform constant-bank addresses.
  int last = -1;
  bool alive = true;
  const int nc = ch.ncomp;
  trk.begin_neutron();
  for (int c = 0; c < nc; ++c) {
    if (!alive) continue;
    if (c > 0) apply_transform<R>(n, ch, c);
    last = c;
    trk.begin_component(ch, c);
    if constexpr (kX && !std::decay_t<Trk>::kActive) {
      if (ch.comp[c].opcode == MCV_OP_HMS) {
        last = ms_fan_out<R>(n, rng, ch, c, k);
        alive = false;
        continue;
      }
    }
    k.overflow += run_component<R, kX>(n, rng, ch.comp[c], trk, ch);
    if (!(n.p > 0)) {
      if (m_isnan(n.p)) k.nonfinite++;
      alive = false;
    }
  }
  return last;
}

template <typename R>
__device__ __forceinline__ void zero_neutron(Neutron<R>& n) {
  n.x = n.y = n.z = n.vx = n.vy = n.vz = n.sx = n.sy = n.p = R(0);
  n.t.set(R(0));
}

template <typename R>
__device__ __forceinline__ void store_neutron(const Neutron<R>& n,
                                              double* out, double down) {
  out[0] = n.x;
  out[1] = n.y;
  out[2] = n.z;
  out[3] = n.vx;
  out[4] = n.vy;
  out[5] = n.vz;
  out[6] = n.sx;
  out[7] = n.sy;
  out[8] = n.t.dval();
  out[9] = (double)n.p * down;
}

__device__ __forceinline__ void flush_counters(const Counters& k,
                                               DevStatus* st) {
  unsigned p = __reduce_add_sync(0xffffffffu, k.processed);
  unsigned o = __reduce_add_sync(0xffffffffu, k.overflow);
  unsigned f = __reduce_add_sync(0xffffffffu, k.nonfinite);
  unsigned r = __reduce_add_sync(0xffffffffu, k.overrun);
  if ((threadIdx.x & 31) == 0) {
    if (p) atomicAdd(&st->processed, (unsigned long long)p);
    if (o) atomicAdd(&st->bounce_overflow, (unsigned long long)o);
    if (f) atomicAdd(&st->nonfinite, (unsigned long long)f);
    if (r) atomicAdd(&st->rng_overrun, (unsigned long long)r);
  }
}

constexpr int kMaxThreads = 256;

// MODE 0: Philox; 1: Philox + record; 2: injected uniforms + record.
// kX: the instantiation with the rarer components (run_component).
// kDense: the same kX code held to 4 blocks of 256 threads an SM (64
// registers, some spills), which pays for chains whose time goes into
// sample kernels and the multiple scatterer (latency-bound at 3 blocks)
// and loses for the long guide loops; the host picks (dense_kx_chain).
// The other FP32 kX instantiation is held to 3 blocks (85 registers):
// left free, the compiler takes 128 and 2 blocks, and the segmented, mesh
// and SNS-source chains ran 2-12% slower.
template <typename R, int MODE, bool kX = false, bool kDense = false>
__global__ void __launch_bounds__(
    kMaxThreads, kDense ? 4 : ((kX && sizeof(R) == 4) ? 3 : 0))
    chain_kernel(const __grid_constant__ mcv_chain ch, uint64_t n,
                 uint64_t first, uint64_t seed, const float* __restrict__ uni,
                 int stride, double* __restrict__ out_n,
                 int* __restrict__ out_last, DevStatus* st) {
  Counters k{0, 0, 0, 0};
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += step) {
    Neutron<R> nt;
    zero_neutron(nt);
    int last;
    if constexpr (MODE == 2) {
      InjectedStream rng(uni + i * (uint64_t)stride, stride, first + i);
      last = run_chain_one<R, kX>(nt, rng, ch, k);
      k.overrun += rng.overrun();
    } else {
      PhiloxStream rng(seed, first + i, 0u);
      last = run_chain_one<R, kX>(nt, rng, ch, k);
    }
    k.processed++;
    if constexpr (MODE == 1 || MODE == 2) {
      if (out_n) store_neutron(nt, out_n + i * 10, weight_down<R>(ch));
      if (out_last) out_last[i] = last;
    }
  }
  flush_counters(k, st);
}

// The stream the components after the multiple scatterer see in the tree
// kernel: none of them draws (chains whose later components draw run in the
// thread kernel), and the neutron-storage components read the incident
// neutron's index.  Holding no state, it leaves the lane's Philox stream in
// registers across the out-of-line call below.
struct IndexOnlyStream {
  uint64_t idx;
  __device__ __forceinline__ float next() { return 0.5f; }
  __device__ __forceinline__ void skip(int) {}
  __device__ __forceinline__ int overrun() const { return 0; }
  __device__ __forceinline__ uint64_t index() const { return idx; }
};

// ms_downstream for the tree kernel: the counts to add (x: guide bounce
// overflows, y: non-finite weights) come back by value.
template <typename R>
__device__ __noinline__ uint2 ms_downstream_out(Neutron<R> m, uint64_t index,
                                                const mcv_chain& ch, int c) {
  IndexOnlyStream rng{index};
  Counters k{0, 0, 0, 0};
  ms_downstream<R, true>(m, rng, ch, c, k);
  return make_uint2(k.overflow, k.nonfinite);
}

// ---------------------------------------------------------------------------
// Chains with a multiple scatterer: a warp-synchronous form of the
// scattering tree.
//
// The thread kernel runs each incident neutron's tree (_scatterM ->
// _interactM_path1 -> _interactM1, homogeneous_multiple_scatterer.py:86-256)
// as nested loops on its own lane.  Lanes leave those loops at different
// points (a transfer the neutron cannot make ends its tree early), the warp
// executes the branches one after the other, and each lane's call frames
// and work lists are read and written at different times: on the UN
// benchmark 5 lanes of 32 were active and the per-lane stacks spilled
// gigabytes to DRAM.  Here the same tree is a per-lane state machine: each
// pass of a warp-uniform loop first advances every lane's bookkeeping to its
// next _interactM1 call (or to the end of its tree, emitting the outputs on
// the way), then makes that call on all lanes together and files its two
// outputs.  The warps of a block run each phase together, and when every
// tree of the block has ended the lanes take the next incident neutrons.  Every neutron goes
// through the same operations in the same order, with its own Philox
// stream, as in the thread kernel, so results agree neutron by neutron.
// Used when no component after the scatterer draws random numbers (the
// outputs then run the rest of the chain as they become final,
// ms_downstream_draws).
template <typename R>
struct MsLane {
  Neutron<R> tbs[2][MCV_MS_MAX_SCATTERED];   // _scatterM's work lists
  Neutron<R> ptbs[2][MCV_MS_MAX_SCATTERED];  // _interactM_path1's lists
  // _scatterM: list in use, loop, index, sizes, output count, final index
  int ob, iloop, i, ntbs, s2, out_index, fi, ophase;  // ophase 0 loop, 1 final
  bool full, done;
  // _interactM_path1: active, list in use, loop, index, sizes, outputs,
  // tail index; pphase 0 calls, 1 tail, 2 returned
  bool p_active;
  int pb, pl, pi, pntbs, ps2, pout, ptail, pphase;
};

// the consumer of _scatterM (:214-235) for one _interactM_path1 output;
// `loc`: where the output is (ms_locate), or -1 when not yet located
template <typename R, typename Emit>
__device__ __forceinline__ void ms_take(const mcv_component& c, MsLane<R>& S,
                                        const Neutron<R>& o, R min_prob,
                                        int max_sc, Emit& emit, int loc) {
  if (S.full || S.done) return;
  Neutron<R> s1 = o;
  if (s1.p < min_prob) return;
  if (!(m_sqrt(s1.vx * s1.vx + s1.vy * s1.vy + s1.vz * s1.vz) > R(1.e-6)))
    return;  // is_moving (acc/neutron.py:39-42)
  if (loc < 0) loc = ms_locate<R>(c, s1.x, s1.y, s1.z);
  bool exiting;
  if (loc == kInside) {
    ms_exit_attenuated_inside(c, s1);
    exiting = ms_is_exiting(c, s1);
  } else {
    exiting = ms_is_exiting_at(c, s1, loc);
  }
  if (exiting) {
    emit(s1);
    if (++S.out_index >= max_sc) S.done = true;
    return;
  }
  S.tbs[S.ob ^ 1][S.s2++] = s1;
  if (S.s2 >= max_sc) S.full = true;
}

// Start an incident neutron's tree; false when it is final at once (it
// does not enter the shape: _scatterM emits it unchanged, :203-205).
template <typename R, typename Emit>
__device__ __forceinline__ bool ms_begin(const mcv_component& c, MsLane<R>& S,
                                         const Neutron<R>& n0, Emit& emit) {
  Neutron<R> n = n0;
  if constexpr (sizeof(R) == 4) ms_approach(c, n);
  if (ms_is_exiting(c, n)) {
    emit(n0);
    return false;
  }
  S.tbs[0][0] = n;
  S.ob = 0;
  S.ntbs = 1;
  S.iloop = 0;
  S.i = 0;
  S.s2 = 0;
  S.out_index = 0;
  S.fi = 0;
  S.full = S.done = false;
  S.p_active = false;
  S.ophase = (c.ip[7] & 0xffff) > 0 ? 0 : 1;
  return true;
}

// Advance a lane's tree to its next _interactM1 call (true: the call is on
// S.ptbs[S.pb][S.pi]) or to its end (false), emitting outputs on the way.
template <typename R, typename Emit>
__device__ __forceinline__ bool ms_advance(const mcv_component& c, MsLane<R>& S,
                                        R min_prob, Emit& emit) {
  const int max_sc = c.ip[6], loops = c.ip[7] & 0xffff,
            loops1 = c.ip[7] >> 16;
  for (;;) {
    if (S.p_active) {
      if (S.pphase == 0) {
        if (S.pi < S.pntbs) return true;
        // the end of one _interactM_path1 loop (:163-167)
        S.pb ^= 1;
        S.pntbs = S.ps2;
        S.ps2 = 0;
        S.pi = 0;
        if (S.pntbs == 0 || ++S.pl >= loops1) {
          S.pphase = 1;
          S.ptail = 0;
        }
        continue;
      }
      if (S.pphase == 1 && S.ptail < S.pntbs && S.pout < max_sc &&
          !S.done) {
        // the neutrons still inside after the loops (:168-174)
        ms_take<R>(c, S, S.ptbs[S.pb][S.ptail], min_prob, max_sc, emit, -1);
        ++S.ptail;
        ++S.pout;
        continue;
      }
      // _interactM_path1 returned (:237-240)
      S.p_active = false;
      if (S.done) return false;
      if (S.full) S.i = S.ntbs;
      else ++S.i;
      continue;
    }
    if (S.ophase == 0) {
      if (S.i < S.ntbs) {
        const Neutron<R>& m = S.tbs[S.ob][S.i];
        if (m.p < min_prob) {  // _interactM_path1 returns at once (:130)
          ++S.i;
          continue;
        }
        S.ptbs[0][0] = m;
        S.pb = 0;
        S.pntbs = 1;
        S.ps2 = 0;
        S.pl = 0;
        S.pi = 0;
        S.pout = 0;
        S.pphase = loops1 > 0 ? 0 : 1;
        S.ptail = 0;
        S.p_active = true;
        continue;
      }
      // the end of one _scatterM loop (:241-245)
      S.ob ^= 1;
      S.ntbs = S.s2;
      S.s2 = 0;
      S.i = 0;
      S.full = false;
      if (S.ntbs == 0 || ++S.iloop >= loops) {
        S.ophase = 1;
        S.fi = 0;
      }
      continue;
    }
    // the neutrons still inside after the loops leave with attenuation
    // (:246-255)
    if (S.fi < S.ntbs && S.out_index < max_sc) {
      Neutron<R> m = S.tbs[S.ob][S.fi];
      const R x = m.x, y = m.y, z = m.z;
      ms_propagate_out(c, m);
      const R dx = m.x - x, dy = m.y - y, dz = m.z - z;
      const R dist = m_sqrt(dx * dx + dy * dy + dz * dz);
      const R atten = ms_atten_coeff(m, c);
      m.p *= m_exp(-atten * dist);
      emit(m);
      ++S.out_index;
      ++S.fi;
      continue;
    }
    return false;
  }
}

// File the outputs of the lane's _interactM1 call (:147-162): `t0` the
// transmitted neutron, the scattered one written in place at the next
// list's free entry (S.ptbs[S.pb ^ 1][S.ps2]), which appending it takes.
template <typename R, typename Emit>
__device__ __forceinline__ void ms_file(const mcv_component& c, MsLane<R>& S,
                                        const Neutron<R>& t0, int ns,
                                        R min_prob, Emit& emit) {
  const int max_sc = c.ip[6];
  if (ns > 0) {
    if (!(t0.p < min_prob)) {
      const int loc = ms_locate<R>(c, t0.x, t0.y, t0.z);
      if (loc != kInside) {
        ms_take<R>(c, S, t0, min_prob, max_sc, emit, loc);
        // the rest of the tree of a neutron that has all its outputs is
        // not drawn: nothing after it reads the incident neutron's stream
        if (++S.pout >= max_sc || S.done) {
          S.pphase = 2;
          return;
        }
      } else {
        // a transmitted neutron left inside (it is on the exit surface up
        // to rounding) is appended first, the scattered one after it
        Neutron<R>* nx = S.ptbs[S.pb ^ 1];
        const Neutron<R> s1 = nx[S.ps2];
        nx[S.ps2++] = t0;
        if (S.ps2 >= max_sc) {
          S.pi = S.pntbs;
          return;
        }
        nx[S.ps2] = s1;
      }
    }
    const Neutron<R>& s1 = S.ptbs[S.pb ^ 1][S.ps2];
    if (!(s1.p < min_prob)) {
      const int loc = ms_locate<R>(c, s1.x, s1.y, s1.z);
      if (loc != kInside) {
        ms_take<R>(c, S, s1, min_prob, max_sc, emit, loc);
        if (++S.pout >= max_sc || S.done) {
          S.pphase = 2;
          return;
        }
      } else if (++S.ps2 >= max_sc) {
        S.pi = S.pntbs;
        return;
      }
    }
  }
  ++S.pi;
}

// The warps of a block run each pass's phases (refill and bookkeeping, the
// _interactM1 calls, the filing of their outputs) between block barriers,
// so that they execute the same code at the same time and share the
// instruction cache, and they refill and end together (UN: 4.1e8 n/s
// without the phase barriers, 5.2e8 with them and warp refills, 6.2e8
// with block refills; the hollow cylinder, whose trees are uneven: 8.5e7
// with block refills alone, 1.09e8 with the phase barriers too).
template <typename R>
__global__ void __launch_bounds__(kMaxThreads, 4)
    ms_chain_kernel(const __grid_constant__ mcv_chain ch, uint64_t n,
                    uint64_t first, uint64_t seed, DevStatus* st) {
  constexpr unsigned kFull = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t per = (n + nwarps - 1) / nwarps;
  uint64_t next = warp * per;
  const uint64_t end = next + per < n ? next + per : n;
  int hms = 0;
  while (ch.comp[hms].opcode != MCV_OP_HMS) ++hms;  // the host checked one
  const mcv_component& c = ch.comp[hms];
  const R min_prob = prm<R>(c, 14) * weight_up<R>(ch);
  Counters k{0, 0, 0, 0};
  MsLane<R> S;
  PhiloxStream rng(seed, 0, 0u);
  int state = 0;  // 0 idle, 1 in a tree, 2 no neutrons left
  auto emit = [&](const Neutron<R>& o) {
    const uint2 r = ms_downstream_out<R>(o, rng.index(), ch, hms);
    k.overflow += r.x;
    k.nonfinite += r.y;
  };
  for (;;) {
    // lanes take new neutrons together, once every tree of the block has
    // ended: trees started in the same pass stay in the same phase (the
    // same branches of ms_advance and ms_file) for most of their length,
    // which pays more than the lanes left idle behind the longest tree (UN:
    // 2.8e8 n/s against 1.7e8 when each lane refills as soon as its tree
    // ends).  With warps refilling on their own, the warps of an SM drift
    // apart over a long launch (UN: 5.2e8 n/s at 3e6 neutrons a launch,
    // 4.3e8 at 1e8); refilling a block at once keeps them together (UN
    // 6.2e8 at 1e8; the hollow cylinder 8.5e7 against 6.9e7).
    const bool busy = __syncthreads_or(state == 1);
    const unsigned idle = busy ? 0u : __ballot_sync(kFull, state == 0);
    if (idle) {
      if (state == 0) {
        const uint64_t idx = next + (uint64_t)__popc(idle & below);
        if (idx < end) {
          Neutron<R> nt;
          zero_neutron(nt);
          rng = PhiloxStream(seed, first + idx, 0u);
          NoTrack trk;
          bool alive = true;
          for (int c2 = 0; c2 < hms && alive; ++c2) {
            if (c2 > 0) apply_transform<R>(nt, ch, c2);
            k.overflow += run_component<R, true>(nt, rng, ch.comp[c2], trk,
                                                 ch);
            if (!(nt.p > 0)) {
              if (m_isnan(nt.p)) k.nonfinite++;
              alive = false;
            }
          }
          k.processed++;
          if (alive) {
            if (hms > 0) apply_transform<R>(nt, ch, hms);
            state = ms_begin<R>(c, S, nt, emit) ? 1 : 0;
          }
        } else {
          state = 2;
        }
      }
      next += (uint64_t)__popc(idle);
      if (next > end) next = end;
    }
    if (__syncthreads_and(state == 2)) break;
    bool call = false;
    if (state == 1) {
      call = ms_advance<R>(c, S, min_prob, emit);
      if (!call) state = 0;
    }
    __syncthreads();
    // a call comes with S.ps2 < max_scattered_neutrons: the scattered
    // neutron's entry exists
    Neutron<R> t0;
    int ns = 0;
    if (call)
      ns = ms_interact_m1(c, rng, t0, S.ptbs[S.pb ^ 1][S.ps2],
                          S.ptbs[S.pb][S.pi]);
    __syncthreads();
    if (call) ms_file<R>(c, S, t0, ns, min_prob, emit);
  }
  flush_counters(k, st);
}

// The tail queue of the FP32 regeneration kernel: per warp, a ring of
// kTailCap neutrons that have left the chain's last guide alive, each with
// its position in its Philox stream (20 words, stored word-major so that
// the lanes of a warp touch consecutive banks).
constexpr int kTailWords = 20;
constexpr int kTailCap = 64;
constexpr size_t kTailBytesPerWarp = sizeof(uint32_t) * kTailWords * kTailCap;
// the backward's queue also carries the gradient tracker's state
constexpr size_t kGradTailBytesPerWarp =
    sizeof(uint32_t) * (kTailWords + GradTrack<float>::kQueueWords) * kTailCap;

__device__ __forceinline__ void tail_store(uint32_t* q, int slot,
                                           const Neutron<float>& n,
                                           const PhiloxStream& r) {
  const uint32_t w[kTailWords] = {
      __float_as_uint(n.x),  __float_as_uint(n.y),    __float_as_uint(n.z),
      __float_as_uint(n.vx), __float_as_uint(n.vy),   __float_as_uint(n.vz),
      __float_as_uint(n.sx), __float_as_uint(n.sy),   __float_as_uint(n.t.hi),
      __float_as_uint(n.t.lo), __float_as_uint(n.p),  r.c0,
      r.c1,                  r.c2,                    r.b0,
      r.b1,                  r.b2,                    r.b3,
      r.b4,                  (uint32_t)r.left};
#pragma unroll
  for (int k = 0; k < kTailWords; ++k) q[k * kTailCap + slot] = w[k];
}

__device__ __forceinline__ void tail_load(const uint32_t* q, int slot,
                                          Neutron<float>& n,
                                          PhiloxStream& r) {
  uint32_t w[kTailWords];
#pragma unroll
  for (int k = 0; k < kTailWords; ++k) w[k] = q[k * kTailCap + slot];
  n.x = __uint_as_float(w[0]);
  n.y = __uint_as_float(w[1]);
  n.z = __uint_as_float(w[2]);
  n.vx = __uint_as_float(w[3]);
  n.vy = __uint_as_float(w[4]);
  n.vz = __uint_as_float(w[5]);
  n.sx = __uint_as_float(w[6]);
  n.sy = __uint_as_float(w[7]);
  n.t.hi = __uint_as_float(w[8]);
  n.t.lo = __uint_as_float(w[9]);
  n.p = __uint_as_float(w[10]);
  r.c0 = w[11];
  r.c1 = w[12];
  r.c2 = w[13];
  r.b0 = w[14];
  r.b1 = w[15];
  r.b2 = w[16];
  r.b3 = w[17];
  r.b4 = w[18];
  r.left = (int)w[19];
}

// Path regeneration: the same per-neutron sequence as chain_kernel, but a
// lane whose neutron leaves the chain takes new work at the start of the
// next pass.  A pass sweeps the components in chain order with a
// warp-uniform index k: the lanes whose neutron is at component k run it
// (a guide: its entry), and a lane that gets through moves on to k+1
// within the same sweep.  Then every lane inside a guide, whichever guide,
// makes one bounce in the same instruction stream.  Lanes of a warp stay
// busy while a few neutrons bounce many times, instead of idling until the
// warp's longest path ends; because k is uniform the component parameters
// are read at uniform constant-bank addresses and the opcode dispatch does
// not diverge (only the bounce reads its guide's parameters per lane).
//
// FP32 with shared memory (tail_queue): a neutron that leaves the last
// guide alive is parked in the warp's tail queue and its lane takes new
// work; once the queue holds a neutron for every idle lane (or no new
// neutrons are left), the idle lanes take queued neutrons together, so
// the components after the last guide -- monitors, a sample, a detector,
// which only a few percent of the neutrons reach -- run with the lanes of
// a warp converged.  A full queue leaves the neutron on its lane.
//
// Every neutron is computed with the same functions, in the same order and
// with its own Philox stream, as in chain_kernel, so results agree neutron
// by neutron (up to the compiler's contraction choices).
//
// Shared memory: with kSmem, first `tally_words` doubles of monitor
// tallies (MCV_COMP_SMEM_TALLY: zeroed here, added to the global tallies
// when the block ends), then the tail queues.  Without it (the default
// instantiation) the kernel carries none of that code.
template <typename R, bool kX, typename Trk, bool kSmem = false>
__device__ __forceinline__ void regen_body(const mcv_chain& ch, uint64_t n,
                                           uint64_t first, uint64_t seed,
                                           int tail_queue, int tally_words,
                                           DevStatus* st, Trk& trk) {
  extern __shared__ __align__(16) uint32_t tail_smem[];
  if constexpr (!kSmem) tally_words = 0;
  double* const smt = kSmem ? (double*)tail_smem : nullptr;
  if constexpr (kSmem) {
    for (int i = threadIdx.x; i < tally_words; i += blockDim.x) smt[i] = 0.0;
    __syncthreads();
  }
  constexpr unsigned kFull = 0xffffffffu;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint64_t per = (n + nwarps - 1) / nwarps;
  uint64_t next = warp * per;
  const uint64_t end = next + per < n ? next + per : n;
  Counters k{0, 0, 0, 0};
  Neutron<R> nt;
  zero_neutron(nt);
  PhiloxStream rng(seed, 0, 0u);
  int c = -1;      // component of the lane's neutron; -1 idle, -2 finished
  int inside = 0;  // guide: entered and bouncing
  int nb = 0;      // guide: bounces so far
  const int nc = ch.ncomp;
  int last_guide = -1;
  for (int i = 0; i < nc; ++i)
    if (ch.comp[i].opcode == MCV_OP_GUIDE) last_guide = i;
  // the queue: FP32 only, when something follows the last guide
  bool queue = false;
  if constexpr (sizeof(R) == 4)
    queue = tail_queue && last_guide >= 0 && last_guide + 1 < nc;
  // per slot: the neutron and its stream (kTailWords), then the tracker's
  // per-neutron state
  constexpr int kWords = kTailWords + Trk::kQueueWords;
  uint32_t* q = tail_smem + 2 * tally_words +
                (threadIdx.x >> 5) * (kWords * kTailCap);
  uint32_t* qt = q + kTailWords * kTailCap;
  int qhead = 0, qcount = 0;  // warp-uniform
  for (;;) {
    const bool more = next < end;  // new neutrons left (warp-uniform)
    const unsigned idle = __ballot_sync(kFull, c == -1);
    if (idle) {
      const int nidle = __popc(idle);
      const int rank = __popc(idle & below);
      int npop = 0;
      if (queue && qcount > 0 && (qcount >= nidle || !more))
        npop = qcount < nidle ? qcount : nidle;
      if (c == -1) {
        if (rank < npop) {
          if constexpr (sizeof(R) == 4) {
            tail_load(q, (qhead + rank) % kTailCap, nt, rng);
            trk.load(qt, kTailCap, (qhead + rank) % kTailCap);
          }
          c = last_guide + 1;
          inside = 0;
        } else {
          const uint64_t idx = next + (uint64_t)(rank - npop);
          if (idx < end) {
            zero_neutron(nt);
            rng = PhiloxStream(seed, first + idx, 0u);
            trk.begin_neutron();
            c = 0;
            inside = 0;
          } else {
            c = -2;
          }
        }
      }
      qhead = (qhead + npop) % kTailCap;
      qcount -= npop;
      next += (uint64_t)(nidle - npop);
      if (next > end) next = end;
    }
    if (__all_sync(kFull, c == -2)) break;
    for (int kc = 0; kc < nc; ++kc) {
      if (c != kc || inside) continue;  // inside a guide: bounces below
      const mcv_component& cp = ch.comp[kc];
      trk.begin_component(ch, kc);
      if (cp.opcode == MCV_OP_GUIDE) {
        // the entry here; the bounces below, shared by all guides
        inside = guide_enter<R>(nt, cp);
        nb = 0;
        if (inside) continue;
      } else {
        k.overflow += run_component<R, kX>(nt, rng, cp, trk, ch, smt);
      }
      if (!(nt.p > 0) || kc + 1 >= nc) {
        if (m_isnan(nt.p)) k.nonfinite++;
        c = -1;
        k.processed++;
      } else {
        c = kc + 1;
        apply_transform<R>(nt, ch, kc + 1);
      }
    }
    bool park = false;
    if (inside) {
      // one bounce for every lane inside a guide, whichever guide it is in
      // (that guide's parameters are read per lane)
      bool done = guide_bounce<R>(nt, ch.comp[c], trk);
      if (!done && ++nb >= MCV_MAX_BOUNCES) {
        done = true;
        k.overflow++;
      }
      if (done) {
        inside = 0;
        if (!(nt.p > 0) || c + 1 >= nc) {
          if (m_isnan(nt.p)) k.nonfinite++;
          c = -1;
          k.processed++;
        } else {
          ++c;
          apply_transform<R>(nt, ch, c);
          park = queue && more && c == last_guide + 1;
        }
      }
    }
    if (queue) {
      // park the neutrons that left the last guide, if they all fit
      const unsigned pm = __ballot_sync(kFull, park);
      const int npush = __popc(pm);
      if (npush && qcount + npush <= kTailCap) {
        if (park) {
          if constexpr (sizeof(R) == 4) {
            const int slot = (qhead + qcount + __popc(pm & below)) % kTailCap;
            tail_store(q, slot, nt, rng);
            trk.save(qt, kTailCap, slot);
          }
          c = -1;
        }
        qcount += npush;
      }
      __syncwarp();  // the stores are seen by the lanes that take them
    }
  }
  flush_counters(k, st);
  if constexpr (kSmem) {
    // the block's shared-memory tallies into the global ones
    __syncthreads();
    for (int kc = 0; kc < nc; ++kc) {
      const mcv_component& cp = ch.comp[kc];
      if (!(cp.flags & kFlagSmemTally) || !cp.tally) continue;
      const int m = 3 * (int)comp_nbins(cp);
      const double* src = smt + cp.ip[6];
      for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const double v = src[i];
        if (v != 0.0) atomicAdd(cp.tally + i, v);
      }
    }
  }
}

template <typename R, bool kX = false, bool kSmem = false>
__global__ void __launch_bounds__(kMaxThreads, 4)
    regen_kernel(const __grid_constant__ mcv_chain ch, uint64_t n,
                 uint64_t first, uint64_t seed, int tail_queue,
                 int tally_words, DevStatus* st) {
  NoTrack trk;
  regen_body<R, kX, NoTrack, kSmem>(ch, n, first, seed, tail_queue,
                                    tally_words, st, trk);
}

// The backward replay with the regeneration kernel's structure: the same
// neutrons, lanes and queue as the forward, with the gradient tracker
// (its per-neutron state travels through the tail queue with the neutron).
template <typename R>
__global__ void __launch_bounds__(kMaxThreads)
    grad_regen_kernel(const __grid_constant__ mcv_chain ch,
                      const __grid_constant__ mcv_grad g, uint64_t n,
                      uint64_t first, uint64_t seed, double* powder_x,
                      double* powder_y, int tail_queue, DevStatus* st) {
  GradTrack<R> trk(g, ch, powder_x, powder_y);
  regen_body<R, false>(ch, n, first, seed, tail_queue, 0, st, trk);
  trk.flush(ch);
}

// Backward replay: neutron i of the stream `seed` again, with the gradient
// tracker (track.cuh) in place of the tallies.
template <typename R>
__global__ void __launch_bounds__(kMaxThreads)
    grad_kernel(const __grid_constant__ mcv_chain ch,
                const __grid_constant__ mcv_grad g, uint64_t n,
                uint64_t first, uint64_t seed, double* powder_x,
                double* powder_y, DevStatus* st) {
  Counters k{0, 0, 0, 0};
  GradTrack<R> trk(g, ch, powder_x, powder_y);
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += step) {
    Neutron<R> nt;
    zero_neutron(nt);
    PhiloxStream rng(seed, first + i, 0u);
    run_chain_one<R>(nt, rng, ch, k, trk);
    k.processed++;
  }
  trk.flush(ch);
  flush_counters(k, st);
}

// Buffered mode (ComponentBase.process, ComponentBase.py:79-129): the chain
// applied to a stored neutron array in place; component k draws from
// Philox stream k+1.
template <typename R, bool kX = false>
__global__ void __launch_bounds__(kMaxThreads)
    buffer_kernel(const __grid_constant__ mcv_chain ch, R* __restrict__ buf,
                  uint64_t n, uint64_t first, uint64_t seed, DevStatus* st) {
  Counters k{0, 0, 0, 0};
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += step) {
    R* s = buf + i * 10;
    Neutron<R> nt;
    nt.x = s[0];
    nt.y = s[1];
    nt.z = s[2];
    nt.vx = s[3];
    nt.vy = s[4];
    nt.vz = s[5];
    nt.sx = s[6];
    nt.sy = s[7];
    nt.t.set(s[8]);
    nt.p = s[9] * weight_up<R>(ch);
    for (int c = 0; c < ch.ncomp; ++c) {
      const mcv_component& cp = ch.comp[c];
      const bool source = cp.opcode == MCV_OP_SOURCE_SIMPLE ||
                          cp.opcode == MCV_OP_SNS_SOURCE ||
                          cp.opcode == MCV_OP_NEUTRON_STORAGE;
      if (!source && !(nt.p > 0)) break;
      if (c > 0) apply_transform<R>(nt, ch, c);
      PhiloxStream rng(seed, first + i, (uint32_t)(c + 1));
      NoTrack trk;
      k.overflow += run_component<R, kX>(nt, rng, cp, trk, ch);
    }
    k.processed++;
    s[0] = nt.x;
    s[1] = nt.y;
    s[2] = nt.z;
    s[3] = nt.vx;
    s[4] = nt.vy;
    s[5] = nt.vz;
    s[6] = nt.sx;
    s[7] = nt.sy;
    s[8] = (R)nt.t.dval();
    s[9] = (R)((double)nt.p * weight_down<R>(ch));
  }
  flush_counters(k, st);
}

// Geometry probe: sorted hit times of rays with an HSS shape.
template <typename R>
__global__ void intersect_kernel(const __grid_constant__ mcv_component c,
                                 const double* __restrict__ rays, uint64_t n,
                                 double* __restrict__ out_ts,
                                 int* __restrict__ out_n) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* r = rays + i * 6;
  Hits<R> h = intersect_shape_from<R>(c, (R)r[0], (R)r[1], (R)r[2], (R)r[3],
                                      (R)r[4], (R)r[5]);
  double* o = out_ts + i * MCV_MAX_INTERSECTIONS;
  for (int k = 0; k < MCV_MAX_INTERSECTIONS; ++k)
    o[k] = k < h.n ? (double)h.get(k) : __longlong_as_double(0x7ff8000000000000ll);
  out_n[i] = h.n;
}

// Batched persistent launch over many instrument variants.  Blocks take
// work items of `chunk` neutrons from a device counter (DevStatus::
// work_next); item k belongs to the variant whose cumulative item range
// holds k.  The block stages that variant's chain in shared memory once per
// Copies into dst (a shared-memory mcv_chain) the parts of *src that its
// first ncomp components use: the header, comp[0..ncomp) and the hop
// transforms rot, off, frot, foff [0..ncomp).  The rest of dst is never
// read.  Every region is a multiple of 4 bytes at a 4-byte offset.
__device__ __forceinline__ void stage_chain(unsigned char* dst,
                                            const mcv_chain* src) {
  int nc = src->ncomp;
  nc = nc < 0 ? 0 : (nc > MCV_MAX_COMPONENTS ? MCV_MAX_COMPONENTS : nc);
  const size_t off[6] = {0, offsetof(mcv_chain, comp),
                         offsetof(mcv_chain, rot), offsetof(mcv_chain, off),
                         offsetof(mcv_chain, frot), offsetof(mcv_chain, foff)};
  const size_t len[6] = {offsetof(mcv_chain, comp),
                         nc * sizeof(mcv_component), nc * 9 * sizeof(double),
                         nc * 3 * sizeof(double), nc * 9 * sizeof(float),
                         nc * 3 * sizeof(float)};
  const unsigned char* s = reinterpret_cast<const unsigned char*>(src);
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const uint32_t* a = reinterpret_cast<const uint32_t*>(s + off[r]);
    uint32_t* b = reinterpret_cast<uint32_t*>(dst + off[r]);
    for (int i = threadIdx.x; i < (int)(len[r] / 4); i += blockDim.x)
      b[i] = a[i];
  }
}

// change of variant.  Neutron i of variant v draws from Philox (seeds[v], i).
template <typename R>
__global__ void __launch_bounds__(kMaxThreads)
    batched_kernel(const mcv_chain* __restrict__ variants, int nvar,
                   const uint64_t* __restrict__ counts,
                   const uint64_t* __restrict__ seeds, uint64_t chunk,
                   DevStatus* st) {
  extern __shared__ __align__(16) unsigned char smem[];
  mcv_chain& ch = *reinterpret_cast<mcv_chain*>(smem);
  uint64_t* item_start = reinterpret_cast<uint64_t*>(
      smem + (sizeof(mcv_chain) + 15) / 16 * 16);
  __shared__ uint64_t s_item;
  __shared__ int s_var;
  if (threadIdx.x == 0) {
    uint64_t acc = 0;
    for (int v = 0; v < nvar; ++v) {
      item_start[v] = acc;
      acc += (counts[v] + chunk - 1) / chunk;
    }
    item_start[nvar] = acc;
  }
  __syncthreads();
  const uint64_t total = item_start[nvar];
  int cur = -1;
  Counters k{0, 0, 0, 0};
  for (;;) {
    if (threadIdx.x == 0) {
      uint64_t it = atomicAdd(&st->work_next, 1ull);
      int lo = 0, hi = nvar;  // item_start[lo] <= it < item_start[hi]
      while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (item_start[mid] <= it) lo = mid;
        else hi = mid;
      }
      s_item = it;
      s_var = lo;
    }
    __syncthreads();
    const uint64_t it = s_item;
    const int v = s_var;
    if (it >= total) break;
    if (v != cur) {
      stage_chain(smem, variants + v);
      cur = v;
      __syncthreads();
    }
    const uint64_t a = (it - item_start[v]) * chunk;
    const uint64_t cnt = counts[v];
    const uint64_t b = a + chunk < cnt ? a + chunk : cnt;
    const uint64_t seed = seeds[v];
    for (uint64_t i = a + threadIdx.x; i < b; i += blockDim.x) {
      Neutron<R> nt;
      zero_neutron(nt);
      PhiloxStream rng(seed, i, 0u);
      run_chain_one<R>(nt, rng, ch, k);
      k.processed++;
    }
    __syncthreads();
  }
  flush_counters(k, st);
}

}  // namespace mcv


namespace mcv {

// Host-side launchers of the kernels above for one working precision.
template <typename R>
struct Launchers {
  // x: 0 the common kernels; 1 the chain holds one of the rarer
  // components (kX instantiations); 2 kX with 4 blocks an SM (kDense,
  // FP32 mode 0; other modes and FP64 take 1)
  static int occupancy_chain(int mode, int x, int threads);
  static void chain(int mode, int x, int blocks, int threads,
                    cudaStream_t s, const mcv_chain& ch, uint64_t n,
                    uint64_t first, uint64_t seed, const float* uni,
                    int stride, double* out_n, int* out_last, DevStatus* st);
  // smem: the tail queue's bytes (0 = no queue)
  // smem: the tally area (tally_words doubles) and the tail queue
  static int occupancy_regen(int threads, size_t smem, int tally_words,
                             bool x);
  static void regen(int blocks, int threads, size_t smem, int tally_words,
                    bool x, cudaStream_t s, const mcv_chain& ch, uint64_t n,
                    uint64_t first, uint64_t seed, DevStatus* st);
  static int occupancy_grad_regen(int threads, size_t smem);
  // dynamic shared memory above 48 KB must be allowed per kernel
  static cudaError_t allow_grad_regen_smem(size_t smem);
  static void grad_regen(int blocks, int threads, size_t smem,
                         cudaStream_t s, const mcv_chain& ch,
                         const mcv_grad& g, uint64_t n, uint64_t first,
                         uint64_t seed, double* px, double* py,
                         DevStatus* st);
  static int occupancy_grad(int threads);
  static void grad(int blocks, int threads, cudaStream_t s,
                   const mcv_chain& ch, const mcv_grad& g, uint64_t n,
                   uint64_t first, uint64_t seed, double* px, double* py,
                   DevStatus* st);
  static int occupancy_buffer(int threads, bool x);
  static void buffer(int blocks, int threads, bool x, cudaStream_t s,
                     const mcv_chain& ch, void* buf, uint64_t n,
                     uint64_t first, uint64_t seed, DevStatus* st);
  static int occupancy_ms(int threads);
  static void ms(int blocks, int threads, cudaStream_t s, const mcv_chain& ch,
                 uint64_t n, uint64_t first, uint64_t seed, DevStatus* st);
  static int occupancy_batched(int threads, size_t smem);
  static void batched(int blocks, int threads, size_t smem, cudaStream_t s,
                      const mcv_chain* variants, int nvar,
                      const uint64_t* counts, const uint64_t* seeds,
                      uint64_t chunk, DevStatus* st);
  static void intersect(int blocks, int threads, cudaStream_t s,
                        const mcv_component& c, const double* rays,
                        uint64_t n, double* out_ts, int* out_n);
};

template <typename K>
inline int occupancy_of(K kernel, int threads, size_t smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads,
                                                smem);
  return per_sm < 1 ? 1 : per_sm;
}

// the chain validation of the entry points (engine.cu)
int validate_chain_for(const mcv_chain* ch, mcv_status* st);

// the one kernel that is not per-precision: instantiated in launch_fp64.cu
void powder_finalize(const double* px, const double* py, int npeaks,
                     double* dtable, cudaStream_t s);

#ifdef MCV_DEFINE_LAUNCHERS
template <typename R>
int Launchers<R>::occupancy_chain(int mode, int x, int threads) {
  if constexpr (sizeof(R) == 4) {
    if (x == 2 && mode == 0)
      return occupancy_of(chain_kernel<R, 0, true, true>, threads, 0);
  }
  if (x) {
    if (mode == 0) return occupancy_of(chain_kernel<R, 0, true>, threads, 0);
    if (mode == 1) return occupancy_of(chain_kernel<R, 1, true>, threads, 0);
    return occupancy_of(chain_kernel<R, 2, true>, threads, 0);
  }
  if (mode == 0) return occupancy_of(chain_kernel<R, 0>, threads, 0);
  if (mode == 1) return occupancy_of(chain_kernel<R, 1>, threads, 0);
  return occupancy_of(chain_kernel<R, 2>, threads, 0);
}

template <typename R>
void Launchers<R>::chain(int mode, int x, int blocks, int threads,
                         cudaStream_t s, const mcv_chain& ch, uint64_t n,
                         uint64_t first, uint64_t seed, const float* uni,
                         int stride, double* out_n, int* out_last,
                         DevStatus* st) {
  if constexpr (sizeof(R) == 4) {
    if (x == 2 && mode == 0) {
      chain_kernel<R, 0, true, true><<<blocks, threads, 0, s>>>(
          ch, n, first, seed, uni, stride, out_n, out_last, st);
      return;
    }
  }
#define MCV_CHAIN_LAUNCH(M, X)                                              \
  chain_kernel<R, M, X><<<blocks, threads, 0, s>>>(ch, n, first, seed, uni, \
                                                   stride, out_n, out_last, \
                                                   st)
  if (x) {
    if (mode == 0) MCV_CHAIN_LAUNCH(0, true);
    else if (mode == 1) MCV_CHAIN_LAUNCH(1, true);
    else MCV_CHAIN_LAUNCH(2, true);
  } else {
    if (mode == 0) MCV_CHAIN_LAUNCH(0, false);
    else if (mode == 1) MCV_CHAIN_LAUNCH(1, false);
    else MCV_CHAIN_LAUNCH(2, false);
  }
#undef MCV_CHAIN_LAUNCH
}

// kX chains take no shared-memory tally copies (tally_words is 0 there)
template <typename R>
int Launchers<R>::occupancy_regen(int threads, size_t smem, int tally_words,
                                  bool x) {
  if (x) return occupancy_of(regen_kernel<R, true>, threads, smem);
  return tally_words ? occupancy_of(regen_kernel<R, false, true>, threads,
                                    smem)
                     : occupancy_of(regen_kernel<R, false>, threads, smem);
}

template <typename R>
void Launchers<R>::regen(int blocks, int threads, size_t smem,
                         int tally_words, bool x, cudaStream_t s,
                         const mcv_chain& ch, uint64_t n, uint64_t first,
                         uint64_t seed, DevStatus* st) {
  const int queue = smem > (size_t)tally_words * 8 ? 1 : 0;
  if (x)
    regen_kernel<R, true><<<blocks, threads, smem, s>>>(
        ch, n, first, seed, queue, 0, st);
  else if (tally_words)
    regen_kernel<R, false, true><<<blocks, threads, smem, s>>>(
        ch, n, first, seed, queue, tally_words, st);
  else
    regen_kernel<R, false><<<blocks, threads, smem, s>>>(
        ch, n, first, seed, queue, 0, st);
}

template <typename R>
int Launchers<R>::occupancy_grad_regen(int threads, size_t smem) {
  if (smem > 48 * 1024) allow_grad_regen_smem(smem);
  return occupancy_of(grad_regen_kernel<R>, threads, smem);
}

template <typename R>
cudaError_t Launchers<R>::allow_grad_regen_smem(size_t smem) {
  return cudaFuncSetAttribute(grad_regen_kernel<R>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem);
}

template <typename R>
void Launchers<R>::grad_regen(int blocks, int threads, size_t smem,
                              cudaStream_t s, const mcv_chain& ch,
                              const mcv_grad& g, uint64_t n, uint64_t first,
                              uint64_t seed, double* px, double* py,
                              DevStatus* st) {
  grad_regen_kernel<R><<<blocks, threads, smem, s>>>(
      ch, g, n, first, seed, px, py, smem > 0 ? 1 : 0, st);
}

template <typename R>
int Launchers<R>::occupancy_grad(int threads) {
  return occupancy_of(grad_kernel<R>, threads, 0);
}

template <typename R>
void Launchers<R>::grad(int blocks, int threads, cudaStream_t s,
                        const mcv_chain& ch, const mcv_grad& g, uint64_t n,
                        uint64_t first, uint64_t seed, double* px, double* py,
                        DevStatus* st) {
  grad_kernel<R><<<blocks, threads, 0, s>>>(ch, g, n, first, seed, px, py,
                                            st);
}

template <typename R>
int Launchers<R>::occupancy_buffer(int threads, bool x) {
  return x ? occupancy_of(buffer_kernel<R, true>, threads, 0)
           : occupancy_of(buffer_kernel<R, false>, threads, 0);
}

template <typename R>
void Launchers<R>::buffer(int blocks, int threads, bool x, cudaStream_t s,
                          const mcv_chain& ch, void* buf, uint64_t n,
                          uint64_t first, uint64_t seed, DevStatus* st) {
  if (x)
    buffer_kernel<R, true><<<blocks, threads, 0, s>>>(ch, (R*)buf, n, first,
                                                      seed, st);
  else
    buffer_kernel<R, false><<<blocks, threads, 0, s>>>(ch, (R*)buf, n,
                                                       first, seed, st);
}

template <typename R>
int Launchers<R>::occupancy_ms(int threads) {
  return occupancy_of(ms_chain_kernel<R>, threads, 0);
}

template <typename R>
void Launchers<R>::ms(int blocks, int threads, cudaStream_t s,
                      const mcv_chain& ch, uint64_t n, uint64_t first,
                      uint64_t seed, DevStatus* st) {
  ms_chain_kernel<R><<<blocks, threads, 0, s>>>(ch, n, first, seed, st);
}

template <typename R>
int Launchers<R>::occupancy_batched(int threads, size_t smem) {
  return occupancy_of(batched_kernel<R>, threads, smem);
}

template <typename R>
void Launchers<R>::batched(int blocks, int threads, size_t smem,
                           cudaStream_t s, const mcv_chain* variants,
                           int nvar, const uint64_t* counts,
                           const uint64_t* seeds, uint64_t chunk,
                           DevStatus* st) {
  batched_kernel<R><<<blocks, threads, smem, s>>>(variants, nvar, counts,
                                                  seeds, chunk, st);
}

template <typename R>
void Launchers<R>::intersect(int blocks, int threads, cudaStream_t s,
                             const mcv_component& c, const double* rays,
                             uint64_t n, double* out_ts, int* out_n) {
  intersect_kernel<R><<<blocks, threads, 0, s>>>(c, rays, n, out_ts, out_n);
}
#endif  // MCV_DEFINE_LAUNCHERS

}  // namespace mcv
