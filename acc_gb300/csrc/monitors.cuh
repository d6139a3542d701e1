// monitors.cuh -- monitors and detectors.  Each tallies (N, sum p, sum p^2)
// into a float64 [3][nbins] array with global atomics, the layout and
// update of psd_monitor.py:61-65, 93-95.  Gates are written as negated
// "inside" tests so that a NaN coordinate is never binned.
#pragma once

#include <cooperative_groups.h>

#include "common.cuh"
#include "sample.cuh"
#include "track.cuh"

namespace mcv {

// propagate to z = 0 without moving the neutron (prop_z0, acc/neutron.py:60-66);
// false when that plane lies in the neutron's past.
template <typename R>
__device__ __forceinline__ bool to_z0(const Neutron<R>& n, R& x, R& y) {
  R dt = -n.z / n.vz;
  x = n.x + n.vx * dt;
  y = n.y + n.vy * dt;
  if constexpr (sizeof(R) == 8) {
    double t0 = n.t.val(), t = t0 + dt;
    return !(t0 > t);
  } else {
    return !(dt < 0.f);
  }
}

template <typename R>
__device__ __forceinline__ int bin_of(R v, R lo, R hi, int nb) {
  if constexpr (sizeof(R) == 8) {
    return clampi(m_floori((v - lo) / (hi - lo) * nb), nb);
  } else {
    return clampi(m_floori((v - lo) * (R(nb) / (hi - lo))), nb);
  }
}

// PSD_monitor.propagate (acc/components/monitors/psd_monitor.py:66-83)
template <typename R, typename Trk>
__device__ __forceinline__ void psd_monitor(const Neutron<R>& n,
                                            const mcv_component& c,
                                            const Tally& tl, Trk& trk) {
  R xmin = prm<R>(c, 0), xmax = prm<R>(c, 1), ymin = prm<R>(c, 2),
    ymax = prm<R>(c, 3);
  int nx = c.ip[0], ny = c.ip[1];
  R x, y;
  if (!to_z0(n, x, y)) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  int ix = bin_of(x, xmin, xmax, nx), iy = bin_of(y, ymin, ymax, ny);
  trk.tally(tl, (uint64_t)ix * ny + iy, n.p);
}

// Wavelength_monitor.propagate (wavelength_monitor.py:52-74)
template <typename R, typename Trk>
__device__ __forceinline__ void wavelength_monitor(const Neutron<R>& n,
                                                   const mcv_component& c,
                                                   const Tally& tl, Trk& trk) {
  R xmin = prm<R>(c, 0), xmax = prm<R>(c, 1), ymin = prm<R>(c, 2),
    ymax = prm<R>(c, 3), Lmin = prm<R>(c, 4), Lmax = prm<R>(c, 5);
  R x, y;
  if (!to_z0(n, x, y)) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  R v = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  R L = R(2 * kPi) / (v * R(kV2K));
  if (!(L > Lmin && L < Lmax)) return;
  trk.tally(tl, (uint64_t)bin_of(L, Lmin, Lmax, c.ip[0]), n.p);
}

// Energy monitor: the wavelength monitor binned in E = v^2 VS2E
// (acc/neutron.py:69-71)
template <typename R, typename Trk>
__device__ __forceinline__ void energy_monitor(const Neutron<R>& n,
                                               const mcv_component& c,
                                               const Tally& tl, Trk& trk) {
  R xmin = prm<R>(c, 0), xmax = prm<R>(c, 1), ymin = prm<R>(c, 2),
    ymax = prm<R>(c, 3), Emin = prm<R>(c, 4), Emax = prm<R>(c, 5);
  R x, y;
  if (!to_z0(n, x, y)) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  R E = (n.vx * n.vx + n.vy * n.vy + n.vz * n.vz) * R(kVS2E);
  if (!(E > Emin && E < Emax)) return;
  trk.tally(tl, (uint64_t)bin_of(E, Emin, Emax, c.ip[0]), n.p);
}

// PosDiv_monitor.propagate (posdiv_monitor.py:67-89)
template <typename R, typename Trk>
__device__ __forceinline__ void posdiv_monitor(const Neutron<R>& n,
                                               const mcv_component& c,
                                               const Tally& tl, Trk& trk) {
  R xmin = prm<R>(c, 0), xmax = prm<R>(c, 1), ymin = prm<R>(c, 2),
    ymax = prm<R>(c, 3), maxdiv = prm<R>(c, 4);
  int npos = c.ip[0], ndiv = c.ip[1];
  R x, y;
  if (!to_z0(n, x, y)) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  R div = m_atan(n.vx / n.vz) * R(180. / kPi);
  if (!(div < maxdiv && div > -maxdiv)) return;
  int ix = bin_of(x, xmin, xmax, npos);
  int id = bin_of(div + maxdiv, R(0), 2 * maxdiv, ndiv);
  trk.tally(tl, (uint64_t)ix * ndiv + id, n.p);
}

// PSD_monitor_4Pi.propagate (psd_monitor_4pi.py:56-79) with the +0.5 of
// its theta index (line 72); sin(theta) is clamped to [-1, 1] and a
// neutron that misses the sphere is not tallied.
template <typename R, typename Trk>
__device__ __forceinline__ void psd_monitor_4pi(Neutron<R>& n,
                                                const mcv_component& c,
                                                const Tally& tl, Trk& trk) {
  R radius = prm<R>(c, 0);
  int nphi = c.ip[0], ntheta = c.ip[1];
  R t1, t2;
  if (!isect_sphere<R>(n.x, n.y, n.z, n.vx, n.vy, n.vz, radius, t1, t2))
    return;
  if (m_isnan(t1)) return;
  if (t2 < 0) return;
  if (t1 < 0) t1 = t2;
  prop_dt(n, t1);
  R phi = m_atan2(n.x, n.z);
  R sy = n.y / radius;
  if (m_isnan(sy)) return;
  sy = sy > 1 ? R(1) : (sy < -1 ? R(-1) : sy);
  R theta = m_asin(sy);
  int iphi = (int)(nphi * (phi / 2 / R(kPi) + R(0.5)));
  if (iphi >= nphi) iphi = nphi - 1;
  else if (iphi < 0) iphi = 0;
  int itheta = (int)(ntheta * (theta + R(kPi) / 2) / R(kPi) + R(0.5));
  if (itheta >= ntheta) itheta = ntheta - 1;
  else if (itheta < 0) itheta = 0;
  trk.tally(tl, (uint64_t)iphi * ntheta + itheta, n.p);
}

// IQE_monitor.propagate (iqe_monitor.py:80-113), angle gates included
template <typename R, typename Trk>
__device__ __forceinline__ void iqe_monitor(const Neutron<R>& n,
                                            const mcv_component& c,
                                            const Tally& tl, Trk& trk) {
  R Ei = prm<R>(c, 0), Qmin = prm<R>(c, 1), Qmax = prm<R>(c, 2),
    Emin = prm<R>(c, 3), Emax = prm<R>(c, 4);
  R max_in = prm<R>(c, 5), min_in = prm<R>(c, 6), max_out = prm<R>(c, 7),
    min_out = prm<R>(c, 8);
  R vx = n.vx, vy = n.vy, vz = n.vz;
  R angle_in = m_atan2(vx, vz) / R(kPi) * R(180.);
  R angle_out;
  if (vy != 0) {
    R theta = m_atan(m_sqrt(vx * vx + vz * vz) / vy) / R(kPi) * R(180.);
    angle_out = vy > 0 ? R(90.) - theta : R(90.) + theta;
  } else {
    angle_out = R(0.);
  }
  if (min_in < angle_in && angle_in < max_in && min_out < angle_out &&
      angle_out < max_out) {
    R vi = m_sqrt(Ei) * R(kSE2V);
    R Q = m_sqrt(vx * vx + vy * vy + (vz - vi) * (vz - vi)) * R(kV2K);
    R E = Ei - (vx * vx + vy * vy + vz * vz) * R(kVS2E);
    if (Q >= Qmin && Q < Qmax && E >= Emin && E < Emax) {
      int iQ = bin_of(Q, Qmin, Qmax, c.ip[0]), iE = bin_of(E, Emin, Emax, c.ip[1]);
      trk.tally(tl, (uint64_t)iQ * c.ip[1] + iE, n.p);
    }
  }
}

// theta x tof 4pi shell: the sphere crossing of PSD_monitor_4Pi binned by
// the polar angle from +z, atan2(hypot(x, y), z), and the time of flight.
template <typename R, typename Trk>
__device__ __forceinline__ void theta_tof_4pi(Neutron<R>& n,
                                              const mcv_component& c,
                                              const Tally& tl, Trk& trk) {
  R radius = prm<R>(c, 0), tmin = prm<R>(c, 1), tmax = prm<R>(c, 2);
  int nth = c.ip[0], nt = c.ip[1];
  R t1, t2;
  if (!isect_sphere<R>(n.x, n.y, n.z, n.vx, n.vy, n.vz, radius, t1, t2))
    return;
  if (m_isnan(t1)) return;
  if (t2 < 0) return;
  if (t1 < 0) t1 = t2;
  prop_dt(n, t1);
  R rho = m_sqrt(n.x * n.x + n.y * n.y);
  R theta = m_atan2(rho, n.z);
  if (m_isnan(theta)) return;
  R t = n.t.val();
  if (!(t >= tmin && t < tmax)) return;
  int ith = bin_of(theta, R(0), R(kPi), nth);
  int it = bin_of(t, tmin, tmax, nt);
  trk.tally(tl, (uint64_t)ith * nt + it, n.p);
}

// exit through the side of the vertical (axis y) cylinder x^2 + z^2 = R^2
// from inside; NaN when it leaves through a cap.
template <typename R>
__device__ __forceinline__ R vcyl_exit(const Neutron<R>& n, R Rad, R H) {
  const R NaN = R(__int_as_float(0x7fc00000));
  R a = n.vx * n.vx + n.vz * n.vz;
  R b = n.x * n.vx + n.z * n.vz;
  R cc = n.x * n.x + n.z * n.z - Rad * Rad;
  R k = b * b - a * cc;
  if (k < 0 || a == 0) return NaN;
  R t = (-b + m_sqrt(k)) / a;
  if (t < 0) return NaN;
  R y = n.y + n.vy * t;
  if (!(m_fabs(y) < H / 2)) return NaN;
  return t;
}

// cylinder detector binned in I(Q,E): Q and E as iqe_monitor.py:96-110
template <typename R, typename Trk>
__device__ __forceinline__ void cyl_iqe(Neutron<R>& n, const mcv_component& c,
                                        const Tally& tl, Trk& trk) {
  R Rad = prm<R>(c, 0), H = prm<R>(c, 1), Ei = prm<R>(c, 2),
    Qmin = prm<R>(c, 3), Qmax = prm<R>(c, 4), Emin = prm<R>(c, 5),
    Emax = prm<R>(c, 6);
  R t = vcyl_exit(n, Rad, H);
  if (m_isnan(t)) return;
  prop_dt(n, t);
  R vx = n.vx, vy = n.vy, vz = n.vz;
  R vi = m_sqrt(Ei) * R(kSE2V);
  R Q = m_sqrt(vx * vx + vy * vy + (vz - vi) * (vz - vi)) * R(kV2K);
  R E = Ei - (vx * vx + vy * vy + vz * vz) * R(kVS2E);
  if (Q >= Qmin && Q < Qmax && E >= Emin && E < Emax) {
    int iQ = bin_of(Q, Qmin, Qmax, c.ip[0]), iE = bin_of(E, Emin, Emax, c.ip[1]);
    trk.tally(tl, (uint64_t)iQ * c.ip[1] + iE, n.p);
  }
}

// banked cylinder detector: banks are azimuthal windows of phi = atan2(x, z)
template <typename R, typename Trk>
__device__ __forceinline__ void banked(Neutron<R>& n, const mcv_component& c,
                                       const Tally& tl, Trk& trk) {
  R Rad = prm<R>(c, 0), H = prm<R>(c, 1), a0 = prm<R>(c, 2), w = prm<R>(c, 3),
    g = prm<R>(c, 4), tmin = prm<R>(c, 5), tmax = prm<R>(c, 6);
  int nb = c.ip[0], ntube = c.ip[1], npix = c.ip[2], ntof = c.ip[3];
  R t = vcyl_exit(n, Rad, H);
  if (m_isnan(t)) return;
  prop_dt(n, t);
  R phi = m_atan2(n.x, n.z);
  R rel = phi - a0;
  if (!(rel >= 0)) return;
  int b = m_floori(rel / (w + g));
  if (b >= nb) return;
  R inb = rel - b * (w + g);
  if (inb >= w) return;
  R tt = n.t.val();
  if (!(tt >= tmin && tt < tmax)) return;
  int tube = bin_of(inb, R(0), w, ntube);
  int pix = bin_of(n.y + H / 2, R(0), H, npix);
  int it = bin_of(tt, tmin, tmax, ntof);
  uint64_t bin = (((uint64_t)b * ntube + tube) * npix + pix) * ntof + it;
  trk.tally(tl, bin, n.p);
}

// Save the neutron as it reaches the component (the NeutronToStorage
// monitor of mcvine, which acc/test/instrument_factory.py:104-113 places
// before and after a component): one row of 11 64-bit words -- the
// neutron's index, then x y z vx vy vz sx sy t p in float64 -- at a slot
// that the lanes arriving together reserve with one atomic on word 0.
// Slots past the capacity (table_len rows) are counted but not written.
// `wdown` undoes the FP32 kernels' weight scale.
template <typename R>
__device__ __forceinline__ void neutron_to_storage(const Neutron<R>& n,
                                                   uint64_t index,
                                                   const mcv_component& c,
                                                   double wdown) {
  namespace cg = cooperative_groups;
  auto* words = reinterpret_cast<unsigned long long*>(c.tally);
  cg::coalesced_group g = cg::coalesced_threads();
  unsigned long long base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(words, (unsigned long long)g.size());
  base = g.shfl(base, 0);
  const unsigned long long slot = base + g.thread_rank();
  if (slot >= c.table_len) return;
  double* row = c.tally + 1 + 11 * slot;
  words[1 + 11 * slot] = index;
  row[1] = (double)n.x;
  row[2] = (double)n.y;
  row[3] = (double)n.z;
  row[4] = (double)n.vx;
  row[5] = (double)n.vy;
  row[6] = (double)n.vz;
  row[7] = (double)n.sx;
  row[8] = (double)n.sy;
  row[9] = n.t.dval();
  row[10] = (double)n.p * wdown;
}

}  // namespace mcv
