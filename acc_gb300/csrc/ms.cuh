// ms.cuh -- the homogeneous multiple scatterer
// (acc/components/samples/homogeneous_multiple_scatterer.py:22-342) and
// the propagation helpers it uses (acc/geometry/propagation.py:11-215).
//
// One incident neutron gives up to max_scattered_neutrons output neutrons
// (transmitted and scattered branches, iterated max_ms_loops x
// max_ms_loops_path1 times).  The work lists are per-thread arrays of
// MCV_MS_MAX_SCATTERED neutrons, as the reference's are per-thread local
// arrays; the outputs go to a callback as they become final, and the
// caller runs the rest of the chain on each.  The FP64
// forms follow the reference's operation order; FP32 takes its hit times
// from the ray's closest approach (intersect_shape_from), and the event
// probability cut is compared in the chain's weight scale.
#pragma once

#include "sample.cuh"

namespace mcv {

// The geometry below is called from many places of the multiple-scattering
// tree, on lanes that are at different places of it: one out-of-line copy
// each (not inlined) keeps the kernel's code small enough for the
// instruction cache, which otherwise dominates its stalls.
template <typename R>
__device__ __noinline__ Hits<R> ms_hits(const mcv_component& c, R x, R y, R z,
                                        R vx, R vy, R vz) {
  return intersect_shape_from<R>(c, x, y, z, vx, vy, vz);
}
template <typename R>
__device__ __noinline__ int ms_locate(const mcv_component& c, R x, R y, R z) {
  return locate_shape<R>(c, x, y, z);
}

// forward_intersect (propagation.py:11-22): the hit times >= 0, in order
template <typename R>
__device__ __forceinline__ Hits<R> forward_hits(const mcv_component& c,
                                                const Neutron<R>& n) {
  Hits<R> h = ms_hits<R>(c, n.x, n.y, n.z, n.vx, n.vy, n.vz);
  int m = h.n;
#pragma unroll
  for (int i = 3; i >= 0; --i)
    if (i < h.n && h.get(i) >= R(0)) m = i;
  Hits<R> f;
  f.n = h.n - m;
  f.t0 = h.get(m < 4 ? m : 3);
  f.t1 = h.get(m + 1 < 4 ? m + 1 : 3);
  f.t2 = h.get(m + 2 < 4 ? m + 2 : 3);
  f.t3 = h.get(m + 3 < 4 ? m + 3 : 3);
  return f;
}

template <typename R>
__device__ __forceinline__ int locate_at(const mcv_component& c,
                                         const Neutron<R>& n, R t) {
  return ms_locate<R>(c, n.x + n.vx * t, n.y + n.vy * t, n.z + n.vz * t);
}

// _is_exiting (propagation.py:24-50) of a neutron at location `loc`
// (ms_locate of its position)
template <typename R>
__device__ __noinline__ bool ms_is_exiting_at(const mcv_component& c,
                                              const Neutron<R>& n, int loc) {
  if (loc == kInside) return false;
  const Hits<R> h = forward_hits(c, n);
  if (h.n == 0) return true;
  if (loc == kOutside) return false;
  R previous = 0;
  for (int it = 0; it < h.n; ++it) {
    const R now = h.get(it), middle = (previous + now) / R(2);
    if (locate_at(c, n, middle) != kOnBorder) return false;
    previous = now;
  }
  return true;
}

template <typename R>
__device__ __forceinline__ bool ms_is_exiting(const mcv_component& c,
                                              const Neutron<R>& n) {
  return ms_is_exiting_at(c, n, ms_locate<R>(c, n.x, n.y, n.z));
}

// _propagate_out (propagation.py:52-59)
template <typename R>
__device__ __forceinline__ void ms_propagate_out(const mcv_component& c,
                                                 Neutron<R>& n) {
  const Hits<R> h = forward_hits(c, n);
  if (h.n == 0) return;
  prop_dt(n, h.get(h.n - 1));
}

// _tof_before_first_exit (propagation.py:154-191); -1 where the reference
// raises (a point outside the shape)
template <typename R>
__device__ __forceinline__ R ms_tof_before_first_exit(const mcv_component& c,
                                                      const Neutron<R>& n) {
  const int loc = ms_locate<R>(c, n.x, n.y, n.z);
  if (loc == kOutside) return R(-1);
  const Hits<R> h = forward_hits(c, n);
  if (h.n == 0) return R(0);
  if (loc == kInside) return h.t0;
  R t = 0;
  for (int i = 0; i < h.n; ++i) {
    const int l1 = locate_at(c, n, h.get(i) / R(2));
    if (l1 == kOutside) return R(0);
    if (l1 == kInside) {
      t = h.get(i);
      break;
    }
  }
  return t;
}

// _propagate_to_next_incident_surface (propagation.py:61-105); a point
// inside the shape (where the reference raises) is left where it is
template <typename R>
__device__ __forceinline__ void ms_to_incident(const mcv_component& c,
                                               Neutron<R>& n) {
  const int loc = ms_locate<R>(c, n.x, n.y, n.z);
  if (loc == kInside) return;
  const Hits<R> h = forward_hits(c, n);
  if (h.n == 0) return;
  R t;
  if (loc == kOutside) {
    t = h.t0;
  } else {
    bool found = false;
    for (int i = 0; i < h.n; ++i) {
      const int l1 = locate_at(c, n, h.get(i) / R(2));
      if (l1 == kInside) return;
      if (l1 == kOutside) {
        t = h.get(i);
        found = true;
        break;
      }
    }
    if (!found) return;
  }
  prop_dt(n, t);
}

// _propagate_to_next_exiting_surface (propagation.py:107-152)
template <typename R>
__device__ __noinline__ void ms_to_exiting(const mcv_component& c,
                                              Neutron<R>& n) {
  const int loc = ms_locate<R>(c, n.x, n.y, n.z);
  R t;
  if (loc == kInside) {
    t = forward_hits(c, n).t0;
  } else {
    if (loc == kOutside) ms_to_incident(c, n);
    const Hits<R> h = forward_hits(c, n);
    bool found = false;
    for (int i = 0; i < h.n; ++i) {
      const int l1 = locate_at(c, n, h.get(i) / R(2));
      if (l1 == kOutside) return;
      if (l1 == kInside) {
        t = h.get(i);
        found = true;
        break;
      }
    }
    if (!found) return;
  }
  prop_dt(n, t);
}

// FP32: an incident neutron arrives in the sample's frame up to metres
// away, and propagating it from there to the shape in float leaves its
// entry point ~1e-7 m off (a float's spacing at 1 m), beyond the on-border
// tolerance of locate: the reference's next steps then see it outside (no
// scattering) or inside.  So it is first moved along its own ray to just
// outside the shape's bounding sphere; the first entry point, the hits and
// the time of flight are those of the original ray.
template <typename R>
__device__ __forceinline__ R shape_bound(const mcv_component& c, int kind,
                                         int base) {
  const R a = prm<R>(c, base), b = prm<R>(c, base + 1),
          d = prm<R>(c, base + 2);
  if (kind == MCV_SHAPE_SPHERE) return a;
  if (kind == MCV_SHAPE_CYLINDER) return m_sqrt(a * a + R(0.25) * b * b);
  return R(0.5) * m_sqrt(a * a + b * b + d * d);
}

template <typename R>
__device__ __forceinline__ void ms_approach(const mcv_component& c,
                                            Neutron<R>& n) {
  R rb = shape_bound<R>(c, c.ip[2], 0);
  if (c.ip[0] != MCV_CSG_PRIMITIVE) {
    const R rb2 = shape_bound<R>(c, c.ip[3], 4);
    rb = rb2 > rb ? rb2 : rb;
  }
  const R v2 = n.vx * n.vx + n.vy * n.vy + n.vz * n.vz;
  const R tc = -(n.x * n.vx + n.y * n.vy + n.z * n.vz) / v2;
  const R tm = tc - R(1.01) * rb / m_sqrt(v2);
  if (tm > R(0)) prop_dt(n, tm);
}

// _calc_atten_coeff (homogeneous_multiple_scatterer.py:67-71)
template <typename R>
__device__ __forceinline__ R ms_atten_coeff(const Neutron<R>& n,
                                            const mcv_component& c) {
  return hss_sigma<R, true>(n, c) + hss_mu<R>(n, c);
}

// _propagate_to_next_exiting_surface_with_attenuation (:73-84)
template <typename R>
__device__ __forceinline__ void ms_exit_attenuated(const mcv_component& c,
                                                   Neutron<R>& n) {
  const R tof = ms_tof_before_first_exit(c, n);
  const R v = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  const R distance = tof * v;
  const R atten = ms_atten_coeff(n, c);
  const R transmission_prob = m_exp(-atten * distance);
  ms_to_exiting(c, n);
  n.p *= transmission_prob;
}

// The same for a neutron inside the shape: _tof_before_first_exit and
// _propagate_to_next_exiting_surface both take the first forward hit of
// the same ray, found once here.
template <typename R>
__device__ __forceinline__ void ms_exit_attenuated_inside(
    const mcv_component& c, Neutron<R>& n) {
  const Hits<R> h = forward_hits(c, n);
  const R tof = h.n == 0 ? R(0) : h.t0;
  const R v = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  const R distance = tof * v;
  const R atten = ms_atten_coeff(n, c);
  const R transmission_prob = m_exp(-atten * distance);
  prop_dt(n, h.t0);
  n.p *= transmission_prob;
}

// _interactM1 (:86-121): the transmitted and the scattered neutron.  The
// absorbed copy (:106-110) is overwritten by the scattered one and the
// kernels' absorb is a no-op (kernels/__init__.py:164-166), so it is not
// formed.  A point left outside the shape (the reference raises) gives no
// output.  For a neutron inside the shape the time to the first exit and
// the transmitted neutron's move come from one forward hit (the two
// reference functions find the same one).  The outputs go to `out0`
// (transmitted) and `out1` (scattered), neither of them `n`.
template <typename R, typename Rng>
__device__ __forceinline__ int ms_interact_m1(const mcv_component& c,
                                              Rng& rng, Neutron<R>& out0,
                                              Neutron<R>& out1,
                                              Neutron<R>& n) {
  const R vx = n.vx, vy = n.vy, vz = n.vz;
  R tof, t_exit;
  if (ms_locate<R>(c, n.x, n.y, n.z) != kInside) {
    ms_to_incident(c, n);
    tof = ms_tof_before_first_exit(c, n);
    t_exit = R(-1);
  } else {
    const Hits<R> h = forward_hits(c, n);
    tof = h.n == 0 ? R(0) : h.t0;
    t_exit = h.t0;
  }
  if (!(tof > R(0))) return 0;
  const R v = m_sqrt(vx * vx + vy * vy + vz * vz);
  const R distance = tof * v;
  const R sigma = hss_sigma<R, true>(n, c);
  const R mu = hss_mu<R>(n, c);
  const R transmission_prob = m_exp(-(mu + sigma) * distance);
  out0 = n;
  if (t_exit >= R(0)) prop_dt(out0, t_exit);
  else ms_to_exiting(c, out0);
  out0.p *= transmission_prob;
  const R rand = rng.next();
  const R x = distance * rand;
  const R prob = distance * m_exp(-(mu + sigma) * x);
  out1 = n;
  out1.p *= prob;
  prop_dt(out1, x / v);
  NoTrack trk;
  hss_kernel<R, true>(out1, rng, c, trk);
  return 2;
}

// _interactM_path1 (:123-177), with its output neutrons handed to
// `emit` in the reference's order instead of collected in a list: the
// work lists are the only per-lane arrays, and they hold the neutrons
// still inside the shape (one a level for the usual shapes).
template <typename R, typename Rng, typename Emit>
__device__ __noinline__ void ms_path1(const mcv_component& c, Rng& rng,
                                         const Neutron<R>& n0, R min_prob,
                                         Emit& emit) {
  const int max_sc = c.ip[6], loops1 = c.ip[7] >> 16;
  if (n0.p < min_prob) return;
  Neutron<R> buf_a[MCV_MS_MAX_SCATTERED], buf_b[MCV_MS_MAX_SCATTERED];
  Neutron<R>* tbs = buf_a;
  Neutron<R>* tbs2 = buf_b;
  int ntbs = 1, out_index = 0;
  tbs[0] = n0;
  for (int iloop = 0; iloop < loops1; ++iloop) {
    int s2 = 0;
    for (int i = 0; i < ntbs; ++i) {
      Neutron<R> sc[2];
      const int ns = ms_interact_m1(c, rng, sc[0], sc[1], tbs[i]);
      for (int j = 0; j < ns; ++j) {
        const Neutron<R>& s1 = sc[j];
        if (s1.p < min_prob) continue;
        if (ms_locate<R>(c, s1.x, s1.y, s1.z) != kInside) {
          emit(s1);
          if (++out_index >= max_sc) return;
          continue;
        }
        tbs2[s2++] = s1;
        if (s2 >= max_sc) break;
      }
      if (s2 >= max_sc) break;
    }
    Neutron<R>* tmp = tbs2;
    tbs2 = tbs;
    tbs = tmp;
    ntbs = s2;
    if (!ntbs) break;
  }
  for (int i = 0; i < ntbs; ++i) {
    if (out_index >= max_sc) break;
    emit(tbs[i]);
    ++out_index;
  }
}

// _scatterM (:196-256): the output neutrons of one incident neutron, each
// handed to `emit` as soon as it is final (in the reference's order).
// `up`: the chain's FP32 weight scale (the probability cut is compared in
// it).  A _interactM_path1 call always runs to its end, so that the draws
// match the reference's (which collects its outputs first): where the
// reference stops reading them (a full work list, the output limit reached)
// the outputs that follow are drawn and dropped.
template <typename R, typename Rng, typename Emit>
__device__ __noinline__ void ms_scatter(const mcv_component& c, Rng& rng,
                                           const Neutron<R>& n0, R up,
                                           Emit& emit) {
  const int max_sc = c.ip[6], loops = c.ip[7] & 0xffff;
  const R min_prob = prm<R>(c, 14) * up;
  Neutron<R> buf_a[MCV_MS_MAX_SCATTERED], buf_b[MCV_MS_MAX_SCATTERED];
  Neutron<R>* tbs = buf_a;
  Neutron<R>* tbs2 = buf_b;
  Neutron<R> n = n0;
  if constexpr (sizeof(R) == 4) ms_approach(c, n);
  if (ms_is_exiting(c, n)) {
    emit(n0);
    return;
  }
  int ntbs = 1, out_index = 0;
  tbs[0] = n;
  for (int iloop = 0; iloop < loops; ++iloop) {
    int s2 = 0;
    bool full = false, done = false;
    auto take = [&](const Neutron<R>& o) {
      if (full || done) return;
      Neutron<R> s1 = o;
      if (s1.p < min_prob) return;
      if (!(m_sqrt(s1.vx * s1.vx + s1.vy * s1.vy + s1.vz * s1.vz) >
            R(1.e-6)))
        return;  // is_moving (acc/neutron.py:39-42)
      if (ms_locate<R>(c, s1.x, s1.y, s1.z) == kInside)
        ms_exit_attenuated(c, s1);
      if (ms_is_exiting(c, s1)) {
        emit(s1);
        if (++out_index >= max_sc) done = true;
        return;
      }
      tbs2[s2++] = s1;
      if (s2 >= max_sc) full = true;
    };
    for (int i = 0; i < ntbs; ++i) {
      ms_path1<R>(c, rng, tbs[i], min_prob, take);
      if (done) return;
      if (full) break;
    }
    Neutron<R>* tmp = tbs2;
    tbs2 = tbs;
    tbs = tmp;
    ntbs = s2;
    if (!ntbs) break;
  }
  for (int i = 0; i < ntbs; ++i) {
    if (out_index >= max_sc) break;
    Neutron<R>& m = tbs[i];
    const R x = m.x, y = m.y, z = m.z;
    ms_propagate_out(c, m);
    const R dx = m.x - x, dy = m.y - y, dz = m.z - z;
    const R dist = m_sqrt(dx * dx + dy * dy + dz * dz);
    const R atten = ms_atten_coeff(m, c);
    m.p *= m_exp(-atten * dist);
    emit(m);
    ++out_index;
  }
}

// Whether a component after the multiple scatterer draws random numbers
// (a sample or a source): then the rest of the chain runs on the outputs
// after the whole scattering tree, in order, as the reference's generated
// kernel does (run_script.py:66-92); otherwise each output runs it as soon
// as it is final, which gives the same tallies without holding the outputs.
__device__ __forceinline__ bool ms_downstream_draws(const mcv_chain& ch,
                                                    int c) {
  for (int k = c + 1; k < ch.ncomp; ++k) {
    const int op = ch.comp[k].opcode;
    if (op == MCV_OP_HSS || op == MCV_OP_HMS || op == MCV_OP_SOURCE_SIMPLE ||
        op == MCV_OP_SNS_SOURCE)
      return true;
  }
  return false;
}

}  // namespace mcv
