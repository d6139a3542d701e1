// sample.cuh -- the homogeneous single scatterer: shape intersection,
// scattering point and the isotropic / powder / gridded S(Q,E) kernels.
#pragma once

#include "common.cuh"
#include "track.cuh"

namespace mcv {

constexpr double kGeomEps = 1e-10;  // acc/geometry/__init__.py:2
enum { kOutside = 1, kOnBorder = 0, kInside = -1 };

// ============================================================ intersections
// cu_device_intersect_sphere (acc/geometry/arrow_intersect.py:154-168).  In
// FP32 the discriminant v^2 R^2 - |r x v|^2 is recomputed in FP64 when it is
// within 1e-4 of v^2 R^2 of zero (near tangency).
template <typename R>
__device__ __forceinline__ bool isect_sphere(R x, R y, R z, R vx, R vy, R vz,
                                             R Rad, R& t1, R& t2) {
  R r0dotv = x * vx + y * vy + z * vz;
  R cx = y * vz - z * vy, cy = z * vx - x * vz, cz = x * vy - y * vx;
  R v2 = vx * vx + vy * vy + vz * vz;
  R r0Xv2 = cx * cx + cy * cy + cz * cz;
  R vR2 = v2 * Rad * Rad;
  R disc = vR2 - r0Xv2;
  if constexpr (sizeof(R) == 4) {
    if (fabsf(disc) < 1e-4f * vR2) {
      double X = x, Y = y, Z = z, VX = vx, VY = vy, VZ = vz, RR = Rad;
      double CX = Y * VZ - Z * VY, CY = Z * VX - X * VZ, CZ = X * VY - Y * VX;
      double V2 = VX * VX + VY * VY + VZ * VZ;
      disc = (float)(V2 * RR * RR - (CX * CX + CY * CY + CZ * CZ));
    }
  }
  if (disc < 0) return false;
  R s = m_sqrt(disc);
  t1 = -(r0dotv + s) / v2;
  t2 = -(r0dotv - s) / v2;
  return true;
}

// intersectCylinderSide / TopBottom / cu_device_intersect_cylinder
// (arrow_intersect.py:178-267); cylinder x^2 + y^2 = R^2, |z| < H/2.
template <typename R>
__device__ __forceinline__ bool isect_cylinder(R x, R y, R z, R vx, R vy,
                                               R vz, R Rad, R H, R& o1,
                                               R& o2) {
  const R NaN = R(__int_as_float(0x7fc00000));
  // side
  R a = vx * vx + vy * vy, b = x * vx + y * vy, c = x * x + y * y - Rad * Rad;
  R k = b * b - a * c;
  if constexpr (sizeof(R) == 4) {
    if (fabsf(k) < 1e-4f * fmaxf(b * b, fabsf(a * c))) {
      double A = (double)vx * vx + (double)vy * vy;
      double B = (double)x * vx + (double)y * vy;
      double C = (double)x * x + (double)y * y - (double)Rad * Rad;
      k = (float)(B * B - A * C);
    }
  }
  R hh = H / R(2);
  int n1 = 0;
  R t1 = NaN, t2 = NaN;
  if (!(k < 0 || a == 0)) {
    bool done = false;
    if (k == 0) {
      R t = -b / a;
      if (m_fabs(z + vz * t) < hh) {
        n1 = 1;
        t1 = t;
        done = true;
      }
    }
    if (!done) {
      R sk = m_sqrt(k);
      R ta = (-b + sk) / a, tb = (-b - sk) / a;
      bool ga = m_fabs(z + vz * ta) < hh, gb = m_fabs(z + vz * tb) < hh;
      if (ga && gb) { n1 = 2; t1 = tb; t2 = ta; }
      else if (ga) { n1 = 1; t1 = ta; }
      else if (gb) { n1 = 1; t1 = tb; }
    }
  }
  // caps
  int n2 = 0;
  R t3 = NaN, t4 = NaN;
  if (vz != 0) {
    R r2 = Rad * Rad;
    R ta = (hh - z) / vz;
    R xa = x + vx * ta, ya = y + vy * ta;
    bool ga = xa * xa + ya * ya <= r2;
    R tb = (-hh - z) / vz;
    R xb = x + vx * tb, yb = y + vy * tb;
    bool gb = xb * xb + yb * yb <= r2;
    if (ga && gb) {
      n2 = 2;
      if (ta < tb) { t3 = ta; t4 = tb; }
      else { t3 = tb; t4 = ta; }
    } else if (ga) { n2 = 1; t3 = ta; }
    else if (gb) { n2 = 1; t3 = tb; }
  }
  int nn = n1 + n2;
  if (nn == 0) return false;
  if (nn == 1) {
    if (n1 == 1) { o1 = t1; o2 = t1; }
    else { o1 = t3; o2 = t3; }
  } else if (nn == 2) {
    if (n1 == 1) {
      if (t1 > t3) { o1 = t3; o2 = t1; }
      else { o1 = t1; o2 = t3; }
    } else if (n1 == 0) { o1 = t3; o2 = t4; }
    else { o1 = t1; o2 = t2; }
  } else if (nn == 3) {
    if (n1 == 1) { o1 = t3 < t1 ? t3 : t1; o2 = t4 > t1 ? t4 : t1; }
    else { o1 = t1 < t3 ? t1 : t3; o2 = t2 > t3 ? t2 : t3; }
  } else {
    o1 = t3 < t1 ? t3 : t1;
    o2 = t4 > t2 ? t4 : t2;
  }
  return true;
}

// cu_device_intersect_rectangle / update_intersections / intersect_box
// (acc/geometry/onbox.py:8-56)
template <typename R>
__device__ __forceinline__ R rect_hit(R rx, R ry, R rz, R vx, R vy, R vz, R X,
                                      R Y) {
  R t = -rz / vz;
  R r1x = rx + vx * t, r1y = ry + vy * t;
  if (m_fabs(r1x) > X / 2 || m_fabs(r1y) > Y / 2)
    t = R(__int_as_float(0x7fc00000));
  return t;
}
template <typename R>
__device__ __forceinline__ void update_hits(R& t1, R& t2, R t) {
  if (!isfinite(t)) return;
  if (!isfinite(t1)) { t1 = t; return; }
  if (!isfinite(t2)) {
    if (t > t1) t2 = t;
    else { t2 = t1; t1 = t; }
    return;
  }
  if (t < t1) t1 = t;
  else if (t < t2) return;
  else t2 = t;
}
template <typename R>
__device__ __forceinline__ bool isect_box(R x, R y, R z, R vx, R vy, R vz,
                                          R X, R Y, R Z, R& t1, R& t2) {
  t1 = R(__int_as_float(0x7fc00000));
  t2 = t1;
  if (vz != 0) {
    update_hits(t1, t2, rect_hit(x, y, z - Z / 2, vx, vy, vz, X, Y));
    update_hits(t1, t2, rect_hit(x, y, z + Z / 2, vx, vy, vz, X, Y));
  }
  if (vx != 0) {
    update_hits(t1, t2, rect_hit(y, z, x - X / 2, vy, vz, vx, Y, Z));
    update_hits(t1, t2, rect_hit(y, z, x + X / 2, vy, vz, vx, Y, Z));
  }
  if (vy != 0) {
    update_hits(t1, t2, rect_hit(z, x, y - Y / 2, vz, vx, vy, Z, X));
    update_hits(t1, t2, rect_hit(z, x, y + Y / 2, vz, vx, vy, Z, X));
  }
  return !m_isnan(t1);
}

template <typename R>
__device__ __forceinline__ bool isect_prim(int kind, const mcv_component& c,
                                           int base, R x, R y, R z, R vx,
                                           R vy, R vz, R& t1, R& t2) {
  // the render wrappers (arrow_intersect.py:47-86) report no hit when t1
  // is NaN
  bool ok = false;
  if (kind == MCV_SHAPE_SPHERE)
    ok = isect_sphere<R>(x, y, z, vx, vy, vz, prm<R>(c, base), t1, t2);
  else if (kind == MCV_SHAPE_CYLINDER)
    ok = isect_cylinder<R>(x, y, z, vx, vy, vz, prm<R>(c, base),
                           prm<R>(c, base + 1), t1, t2);
  else if (kind == MCV_SHAPE_BOX)
    ok = isect_box<R>(x, y, z, vx, vy, vz, prm<R>(c, base),
                      prm<R>(c, base + 1), prm<R>(c, base + 2), t1, t2);
  return ok && !m_isnan(t1);
}

// point location (acc/geometry/locate.py:354-421).  FP64 uses the
// reference's epsilon; FP32 a float-resolvable one, 2e-6 of the shape's
// largest dimension, because 1e-10 m is below float resolution at these
// coordinates.
template <typename R>
__device__ __forceinline__ int locate_prim(int kind, const mcv_component& c,
                                           int base, R x, R y, R z) {
  R e;
  if constexpr (sizeof(R) == 4) {
    R s = prm<R>(c, base);
    if (kind != MCV_SHAPE_SPHERE) s = fmaxf(s, prm<R>(c, base + 1));
    if (kind == MCV_SHAPE_BOX) s = fmaxf(s, prm<R>(c, base + 2));
    e = 2e-6f * s;
  } else {
    e = R(kGeomEps);
  }
  if (kind == MCV_SHAPE_SPHERE) {
    R Rad = prm<R>(c, base), d2 = x * x + y * y + z * z;
    if (d2 > (Rad + e) * (Rad + e)) return kOutside;
    if (d2 < (Rad - e) * (Rad - e)) return kInside;
    return kOnBorder;
  }
  if (kind == MCV_SHAPE_CYLINDER) {
    R Rad = prm<R>(c, base), H = prm<R>(c, base + 1);
    if (m_fabs(z) - H / R(2) > e) return kOutside;
    R r2 = x * x + y * y;
    if (r2 > (Rad + e) * (Rad + e)) return kOutside;
    if (H / R(2) - m_fabs(z) > e && r2 < (Rad - e) * (Rad - e)) return kInside;
    return kOnBorder;
  }
  if (kind == MCV_SHAPE_BOX) {
    R W = prm<R>(c, base), H = prm<R>(c, base + 1), D = prm<R>(c, base + 2);
    if (m_fabs(x) - R(0.5) * W > e) return kOutside;
    if (m_fabs(y) - R(0.5) * H > e) return kOutside;
    if (m_fabs(z) - R(0.5) * D > e) return kOutside;
    if (-R(0.5) * W < x && x < R(0.5) * W && -R(0.5) * H < y &&
        y < R(0.5) * H && -R(0.5) * D < z && z < R(0.5) * D)
      return kInside;
    return kOnBorder;
  }
  return kOutside;
}

template <typename R>
__device__ __forceinline__ int locate_shape(const mcv_component& c, R x, R y,
                                            R z) {
  int op = c.ip[0];
  int l1 = locate_prim<R>(c.ip[2], c, 0, x, y, z);
  if (op == MCV_CSG_PRIMITIVE) return l1;
  int l2 = locate_prim<R>(c.ip[3], c, 4, x, y, z);
  if (op == MCV_CSG_DIFFERENCE) {
    if (l1 == kOutside || l2 == kInside) return kOutside;
    if (l1 == kOnBorder || l2 == kOnBorder) return kOnBorder;
    return kInside;
  }
  if (op == MCV_CSG_UNION) {
    if (l1 == kInside || l2 == kInside) return kInside;
    if (l1 == kOutside && l2 == kOutside) return kOutside;
    return kOnBorder;
  }
  if (l1 == kOutside || l2 == kOutside) return kOutside;
  if (l1 == kInside && l2 == kInside) return kInside;
  return kOnBorder;
}

// Up to four sorted hit times in registers.  A primitive gives two; a
// binary CSG node keeps the on-border hits of both operands merged in order,
// which is what intersectComposite (arrow_intersect.py:126-142) builds with
// insert_into_sorted_list (_utils.py:4-32).
template <typename R>
struct Hits {
  R t0, t1, t2, t3;
  int n;
  __device__ __forceinline__ R get(int i) const {
    return i == 0 ? t0 : i == 1 ? t1 : i == 2 ? t2 : t3;
  }
};

template <typename R>
__device__ __forceinline__ void cswap(R& a, R& b) {
  R lo = a < b ? a : b, hi = a < b ? b : a;
  a = lo;
  b = hi;
}

template <typename R>
__device__ __forceinline__ Hits<R> intersect_shape(const mcv_component& c,
                                                   R x, R y, R z, R vx, R vy,
                                                   R vz) {
  Hits<R> h;
  const R inf = R(__int_as_float(0x7f800000));
  h.t0 = h.t1 = h.t2 = h.t3 = inf;
  h.n = 0;
  R a1, a2;
  bool ha = isect_prim<R>(c.ip[2], c, 0, x, y, z, vx, vy, vz, a1, a2);
  if (c.ip[0] == MCV_CSG_PRIMITIVE) {
    if (ha) {
      h.t0 = a1;
      h.t1 = a2;
      h.n = 2;
    }
    return h;
  }
  R b1, b2;
  bool hb = isect_prim<R>(c.ip[3], c, 4, x, y, z, vx, vy, vz, b1, b2);
  R cand[4] = {a1, a2, b1, b2};
  bool ok[4] = {ha, ha, hb, hb};
  R s0 = inf, s1 = inf, s2 = inf, s3 = inf;
  int n = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (ok[k]) {
      R t = cand[k];
      if (locate_shape<R>(c, x + vx * t, y + vy * t, z + vz * t) ==
          kOnBorder) {
        if (n == 0) s0 = t;
        else if (n == 1) s1 = t;
        else if (n == 2) s2 = t;
        else s3 = t;
        ++n;
      }
    }
  }
  cswap(s0, s1);
  cswap(s2, s3);
  cswap(s0, s2);
  cswap(s1, s3);
  cswap(s1, s2);
  h.t0 = s0;
  h.t1 = s1;
  h.t2 = s2;
  h.t3 = s3;
  h.n = n;
  return h;
}

// Hit times of a ray with the shape, computed from the ray's closest
// approach to the shape origin and shifted back by the time to get there
// (FP32: avoids cancelling a long flight against a short chord).
template <typename R>
__device__ __forceinline__ Hits<R> intersect_shape_from(const mcv_component& c,
                                                        R x, R y, R z, R vx,
                                                        R vy, R vz) {
  if constexpr (sizeof(R) == 8) {
    return intersect_shape<R>(c, x, y, z, vx, vy, vz);
  } else {
    float t0 = -(x * vx + y * vy + z * vz) / (vx * vx + vy * vy + vz * vz);
    Hits<float> h = intersect_shape<float>(c, fmaf(vx, t0, x), fmaf(vy, t0, y),
                                           fmaf(vz, t0, z), vx, vy, vz);
    h.t0 += t0;
    h.t1 += t0;
    h.t2 += t0;
    h.t3 += t0;
    return h;
  }
}

// =========================================================== HSS helpers
// _calc_time_to_point_of_scattering_impl
// (homogeneous_single_scatterer.py:121-159) on hit times measured from
// "now" (FP64 path).
template <typename R>
__device__ __forceinline__ void time_to_scatter_ref(const Hits<R>& h, R rand,
                                                    R& T, R& ttravel,
                                                    R& tin) {
  R tps0 = 0, tps1 = 0, tpg0 = 0, tpg1 = 0;
  T = 0;
  int sign = 0, ip = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i < h.n) {
      R t = h.get(i);
      if (!(t < 0)) {
        if (sign == 0) sign = (i % 2 == 0) ? -1 : 1;
        else sign = -sign;
        T += sign * t;
        if (sign > 0) {
          if (ip == 0) { tps0 = T; tpg0 = t; }
          else { tps1 = T; tpg1 = t; }
          ++ip;
        }
      }
    }
  }
  tin = rand * T;
  if (ip == 0) {
    ttravel = 0;
  } else if (ip == 1 || tin < tps0) {
    ttravel = tin - tps0 + tpg0;
  } else {
    ttravel = tin - tps1 + tpg1;
  }
}

// total_time_in_shape (homogeneous_single_scatterer.py:161-178)
template <typename R>
__device__ __forceinline__ R total_time_in_shape(const Hits<R>& h) {
  R T = 0;
  int sign = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (i < h.n) {
      R t = h.get(i);
      if (!(t < 0)) {
        if (sign == 0) sign = (i % 2 == 0) ? -1 : 1;
        else sign = -sign;
        T += sign * t;
      }
    }
  }
  return T;
}

// ================================================================ kernels
// isotropic.S (acc/kernels/isotropic.py:5-21)
template <typename R, typename Rng>
__device__ __forceinline__ void isotropic_S(Neutron<R>& n, Rng& rng) {
  R cos_t = R(rng.next()) * 2 - 1;
  R u2 = rng.next();
  if (cos_t > 1) cos_t = 1;
  R sin_t = m_sqrt(1 - cos_t * cos_t);
  R sin_p, cos_p;
  m_sincos_2pi(u2, &sin_p, &cos_p);
  R vi = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  n.vx = vi * sin_t * cos_p;
  n.vy = vi * sin_t * sin_p;
  n.vz = vi * cos_t;
}

// vec3._rotate (acc/vec3.py:77-105)
template <typename R>
__device__ __forceinline__ void rotate3(R& vx, R& vy, R& vz, R cx, R cy, R cz,
                                        R angle, R eps) {
  R cl = m_sqrt(cx * cx + cy * cy + cz * cz);
  R ci = R(1.0) / cl;
  cx *= ci;
  cy *= ci;
  cz *= ci;
  R sf = vx * cx + vy * cy + vz * cz;
  R px = cx * sf, py = cy * sf, pz = cz * sf;
  R lpl = m_sqrt(px * px + py * py + pz * pz);
  R lv = m_sqrt(vx * vx + vy * vy + vz * vz);
  if (m_fabs(1 - lpl / lv) < eps) return;
  R qx = vx - px, qy = vy - py, qz = vz - pz;
  R ql = m_sqrt(qx * qx + qy * qy + qz * qz);
  R qi = R(1.) / ql;
  qx *= qi;
  qy *= qi;
  qz *= qi;
  R ex = qy * cz - qz * cy, ey = qz * cx - qx * cz, ez = qx * cy - qy * cx;
  R ca, sa;
  if constexpr (sizeof(R) == 4) {
    sincosf(angle, &sa, &ca);
  } else {
    sincos(angle, &sa, &ca);
  }
  qx *= ca;
  qy *= ca;
  qz *= ca;
  ex *= sa;
  ey *= sa;
  ez *= sa;
  R rx = qx - ex, ry = qy - ey, rz = qz - ez;
  rx *= ql;
  ry *= ql;
  rz *= ql;
  vx = rx + px;
  vy = ry + py;
  vz = rz + pz;
}

// powder table rows: {q_v, w_v, my_s_v2, cumulative my_s_v2}
template <typename R>
__device__ __forceinline__ const R* powder_table(const mcv_component& c);
template <>
__device__ __forceinline__ const float* powder_table<float>(
    const mcv_component& c) {
  return c.ftable;
}
template <>
__device__ __forceinline__ const double* powder_table<double>(
    const mcv_component& c) {
  return (const double*)c.table;
}

// number of peaks with q_v/2 <= v (q_v ascending)
template <typename R>
__device__ __forceinline__ int powder_reach(const R* pk, int np, R vl) {
  int lo = 0, hi = np;  // first index with vl < q/2
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (vl < __ldg(&pk[4 * mid]) / 2) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

// powderdiffr.scattering_coefficient (acc/kernels/powderdiffr.py:10-25).
// FP64 sums the peaks in order as the reference does; FP32 reads the
// prefix sum at the reachable count.
template <typename R>
__device__ __forceinline__ R powder_coeff(const Neutron<R>& n,
                                          const mcv_component& c) {
  const R* pk = powder_table<R>(c);
  int np = c.ip[4];
  R vl = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  R xs_v2 = 0;
  if constexpr (sizeof(R) == 4) {
    int k = powder_reach(pk, np, vl);
    xs_v2 = k > 0 ? __ldg(&pk[4 * (k - 1) + 3]) : 0.f;
  } else {
    for (int i = 0; i < np; ++i)
      if (vl >= __ldg(&pk[4 * i]) / 2) xs_v2 += __ldg(&pk[4 * i + 2]);
  }
  return xs_v2 / (vl * vl) / prm<R>(c, 10);
}

// powderdiffr.scatter (acc/kernels/powderdiffr.py:27-109), including the
// reference's peak count: without a break in `for peakindex in range(1,
// Npeaks)` the count is Npeaks-1.
template <typename R, typename Rng, typename Trk>
__device__ __forceinline__ void powder_scatter(Neutron<R>& n, Rng& rng,
                                               const mcv_component& c,
                                               Trk& trk) {
  const R* pk = powder_table<R>(c);
  int np = c.ip[4];
  R ucvol = prm<R>(c, 10), d_phi = prm<R>(c, 11);
  R vx = n.vx, vy = n.vy, vz = n.vz;
  R vl = m_sqrt(vx * vx + vy * vy + vz * vz);
  if (vl < __ldg(&pk[0]) / 2) {
    n.p = R(-1);
    return;
  }
  int nreach;
  if (np <= 1) {
    nreach = 1;
  } else {
    int k = powder_reach(pk, np, vl);  // >= 1 here
    nreach = k < np ? k : np - 1;
  }
  int peak = 0;
  if (nreach > 1) {
    peak = (int)(R(rng.next()) * nreach);
    if (peak >= nreach) peak = nreach - 1;
  }
  R rt = R(rng.next()) * 2 - 1;
  R q = __ldg(&pk[4 * peak]), w = __ldg(&pk[4 * peak + 1]),
    s = __ldg(&pk[4 * peak + 2]);
  trk.powder_peak(peak, s);
  R arg = q * (1 + w * rt) / (R(2.0) * vl);
  R scatter_xs = s / (vl * vl);
  scatter_xs *= nreach;
  R theta = m_asin(arg);
  R alpha = 0, alpha0;
  const R DEG2RAD = R(kPi / 180.0);
  if (d_phi != 0) {
    R a = sin(d_phi * DEG2RAD / 2) / sin(2 * theta);
    if (a < -1 || a > 1) d_phi = 0;
    else alpha = 2 * m_asin(a);
  }
  if (d_phi != 0) {
    alpha = m_fabs(alpha);
    R r = rng.next();
    alpha0 = 2 * r * alpha;
    if (alpha0 > alpha) alpha0 = R(kPi) + (alpha0 - R(1.5) * alpha);
    else alpha0 = alpha0 - R(0.5) * alpha;
  } else {
    R r = R(rng.next()) * 2 - 1;
    alpha0 = R(kPi) * r;
  }
  R nx, ny, nz;
  if (m_fabs(vx) < m_fabs(vz)) { nx = 1; ny = 0; nz = 0; }
  else { nx = 0; ny = 0; nz = 1; }
  // vtmp = v x n
  R tx = vy * nz - vz * ny, ty = vz * nx - vx * nz, tz = vx * ny - vy * nx;
  R ox = vx, oy = vy, oz = vz;
  const R eps = R(1e-7);
  rotate3<R>(ox, oy, oz, tx, ty, tz, 2 * theta, eps);
  rotate3<R>(ox, oy, oz, vx, vy, vz, alpha0, eps);
  n.vx = ox;
  n.vy = oy;
  n.vz = oz;
  if (m_isnan(ox) || m_isnan(oy) || m_isnan(oz)) {
    n.p = R(-1);
    return;
  }
  n.p *= scatter_xs / ucvol;
}

// Bilinear lookup of the S(Q,E) grid (node (iq, ie) at Qmin + iq dQ,
// Emin + ie dE; indices clamp to [0, n-2] as SANS2D_ongrid.py:37-50 does).
// Grid coordinate of a value drawn as lo + u (hi - lo) on an n-node grid
// spanning [lo, hi]: u (n - 1).  In FP32 it is formed exactly from the
// uniform's 24-bit integer k (u = k 2^-24): node = k (n-1) >> 24,
// fraction = (k (n-1) mod 2^24) 2^-24.
// scale of the FP32 S(Q,E) interpolation (an exact power of two)
constexpr float kSqeScale = 0x1p64f;

__device__ __forceinline__ void grid_coord(float u, int n, int& i, float& f) {
  uint64_t prod = (uint64_t)(uint32_t)(u * 16777216.f) * (uint64_t)(n - 1);
  i = (int)(prod >> 24);
  f = (float)(uint32_t)(prod & 0xFFFFFFu) * 5.9604644775390625e-08f;
  if (i > n - 2) {
    i = n - 2;
    f = 1.f;
  }
}

template <typename R, typename Trk>
__device__ __forceinline__ R sqe_lookup(const mcv_component& c, R Q, R E,
                                        R uQ, R uE, Trk& trk) {
  const float* tab = c.ftable;
  int nQ = c.ip[4], nE = c.ip[5];
  int iq, ie;
  R fx, fy;
  if constexpr (sizeof(R) == 4) {
    grid_coord(uQ, nQ, iq, fx);
    grid_coord(uE, nE, ie, fy);
  } else {
    R Qmin = prm<R>(c, 10), Qmax = prm<R>(c, 11), Emin = prm<R>(c, 12),
      Emax = prm<R>(c, 13);
    R dQ = (Qmax - Qmin) / (nQ - 1), dE = (Emax - Emin) / (nE - 1);
    iq = (int)((Q - Qmin) / dQ);
    ie = (int)((E - Emin) / dE);
    iq = iq < 0 ? 0 : (iq > nQ - 2 ? nQ - 2 : iq);
    ie = ie < 0 ? 0 : (ie > nE - 2 ? nE - 2 : ie);
    fx = (Q - Qmin) / dQ - iq;
    fy = (E - Emin) / dE - ie;
  }
  // FP32: the nodes are scaled by 2^64 (exact) so that table tails below
  // float's normal range (subnormal entries) interpolate at full precision;
  // the caller divides the scale out of the weight.
  const R ks = sizeof(R) == 4 ? R(kSqeScale) : R(1);
  R f00 = __ldg(&tab[iq * nE + ie]) * ks;
  R f10 = __ldg(&tab[(iq + 1) * nE + ie]) * ks;
  R f01 = __ldg(&tab[iq * nE + ie + 1]) * ks;
  R f11 = __ldg(&tab[(iq + 1) * nE + ie + 1]) * ks;
  // bilinear_interp (SANS2D_ongrid.py:16-22)
  R a00 = f00, a10 = f10 - f00, a01 = f01 - f00, a11 = f11 - f10 - f01 + f00;
  R S = a00 + a10 * fx + a01 * fy + a11 * fx * fy;
  trk.sqe(iq * nE + ie, nE, fx, fy, (double)S / (double)ks);
  return S;
}

// Gridded S(Q,E) kernel: the kinematics of E_Q._S (acc/kernels/E_Q.py:37-99)
// with (Q, E) uniform over the table box and S from the grid; sin(theta)
// from the factored (Q^2 - (ki-kf)^2)((ki+kf)^2 - Q^2) / (2 ki kf)^2.
template <typename R, typename Rng, typename Trk>
__device__ __forceinline__ void sqe_scatter(Neutron<R>& n, Rng& rng,
                                            const mcv_component& c,
                                            Trk& trk) {
  R Qmin = prm<R>(c, 10), Qmax = prm<R>(c, 11), Emin = prm<R>(c, 12),
    Emax = prm<R>(c, 13);
  R vx = n.vx, vy = n.vy, vz = n.vz;
  R vi = m_sqrt(vx * vx + vy * vy + vz * vz);
  R Ei = vi * vi * R(kVS2E);
  R uQ = rng.next(), uE = rng.next();
  R Q = uQ * (Qmax - Qmin) + Qmin;
  R E = uE * (Emax - Emin) + Emin;
  R u3 = rng.next();
  R Ef = Ei - E;
  if (Ef <= 0) {
    n.p = R(-1);
    return;
  }
  R vf = m_sqrt(Ef) * R(kSE2V);
  R ki = R(kV2K) * vi, kf = R(kV2K) * vf;
  // 1 - cos^2 in factored form, well conditioned near 0 and 180 degrees
  R Q2 = Q * Q, dk = ki - kf, sk = ki + kf;
  R sint2 = (Q2 - dk * dk) * (sk * sk - Q2) / (4 * ki * ki * kf * kf);
  if (sint2 < 0) {
    n.p = R(-1);
    return;
  }
  R cost = (ki * ki + kf * kf - Q2) / (2 * ki * kf);
  R sint = m_sqrt(sint2);
  R sp, cp;
  m_sincos_2pi(u3, &sp, &cp);
  R v2 = vf * sint * cp, v3 = vf * sint * sp, v1 = vf * cost;
  R inv = R(1.0) / vi;
  R e1x = vx * inv, e1y = vy * inv, e1z = vz * inv;
  R nx, ny, nz;
  if (m_fabs(e1x) > R(1e-1) || m_fabs(e1y) > R(1e-1)) { nx = 0; ny = 0; nz = 1; }
  else { nx = 1; ny = 0; nz = 0; }
  R e2x = ny * e1z - nz * e1y, e2y = nz * e1x - nx * e1z,
    e2z = nx * e1y - ny * e1x;
  R l2 = R(1.0) / m_sqrt(e2x * e2x + e2y * e2y + e2z * e2z);
  e2x *= l2;
  e2y *= l2;
  e2z *= l2;
  R e3x = e1y * e2z - e1z * e2y, e3y = e1z * e2x - e1x * e2z,
    e3z = e1x * e2y - e1y * e2x;
  n.vx = e1x * v1 + e2x * v2 + e3x * v3;
  n.vy = e1y * v1 + e2y * v2 + e3y * v3;
  n.vz = e1z * v1 + e2z * v2 + e3z * v3;
  R S = sqe_lookup<R>(c, Q, E, uQ, uE, trk);
  R prob_f = S * (vf / vi) * Q * (Qmax - Qmin) * (Emax - Emin) / (kf * ki) / 2;
  if constexpr (sizeof(R) == 4) {
    // prob_f carries the table scale 2^64: take it out of the factor when
    // the factor stays normal, else out of the weight first (p is near
    // 2^64 times its relative size, so p * 2^-64 stays normal)
    const float f = prob_f * (1.f / kSqeScale);
    n.p = f >= 0x1p-126f ? n.p * f : (n.p * (1.f / kSqeScale)) * prob_f;
  } else {
    n.p *= prob_f;
  }
}

// Outgoing velocity of a (Q, E) transfer (constant_qe.py:38-67,
// E_Q.py:64-92): vf cos(t) along the incident direction e1,
// vf sin(t) cos(phi) along e2 = unit(n x e1), vf sin(t) sin(phi) along
// e3 = e1 x e2, with n = z unless e1 lies within 0.1 of it (then x).
template <typename R>
__device__ __forceinline__ void qe_velocity(Neutron<R>& n, R vi, R vf,
                                            R cost, R sint, R uphi) {
  R sp, cp;
  m_sincos_2pi(uphi, &sp, &cp);
  R v2 = vf * sint * cp, v3 = vf * sint * sp, v1 = vf * cost;
  R inv = R(1.0) / vi;
  R e1x = n.vx * inv, e1y = n.vy * inv, e1z = n.vz * inv;
  R nx, ny, nz;
  if (m_fabs(e1x) > R(1e-1) || m_fabs(e1y) > R(1e-1)) { nx = 0; ny = 0; nz = 1; }
  else { nx = 1; ny = 0; nz = 0; }
  R e2x = ny * e1z - nz * e1y, e2y = nz * e1x - nx * e1z,
    e2z = nx * e1y - ny * e1x;
  R l2 = R(1.0) / m_sqrt(e2x * e2x + e2y * e2y + e2z * e2z);
  e2x *= l2;
  e2y *= l2;
  e2z *= l2;
  R e3x = e1y * e2z - e1z * e2y, e3y = e1z * e2x - e1x * e2z,
    e3z = e1x * e2y - e1y * e2x;
  n.vx = e1x * v1 + e2x * v2 + e3x * v3;
  n.vy = e1y * v1 + e2y * v2 + e3y * v3;
  n.vz = e1z * v1 + e2z * v2 + e3z * v3;
}

// constant_qe.S (acc/kernels/constant_qe.py:15-67): the fixed transfer
// (Q, E) = (prm 10, prm 11), one draw for the azimuth.  A transfer the
// neutron cannot make (E above Ei, |cos(theta)| > 1) leaves the
// reference's velocity NaN; here it absorbs the neutron.  FP32 forms
// sin^2(theta) from the factored (Q^2 - (ki-kf)^2)((ki+kf)^2 - Q^2) /
// (2 ki kf)^2, which keeps its precision near 0 and 180 degrees.
template <typename R, typename Rng>
__device__ __forceinline__ void constant_qe_scatter(Neutron<R>& n, Rng& rng,
                                                    const mcv_component& c) {
  const R Q = prm<R>(c, 10), E = prm<R>(c, 11);
  const R vi = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  const R Ei = vi * vi * R(kVS2E);
  const R Ef = Ei - E;
  const R uphi = rng.next();
  if (!(Ef >= R(0))) {
    n.p = R(-1);
    return;
  }
  const R vf = m_sqrt(Ef) * R(kSE2V);
  const R ki = R(kV2K) * vi, kf = R(kV2K) * vf;
  const R cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
  R s2;
  if constexpr (sizeof(R) == 4) {
    const R Q2 = Q * Q, dk = ki - kf, sk = ki + kf;
    s2 = (Q2 - dk * dk) * (sk * sk - Q2) / (4 * ki * ki * kf * kf);
  } else {
    s2 = 1.0 - cost * cost;
  }
  if (!(s2 >= R(0))) {
    n.p = R(-1);
    return;
  }
  qe_velocity<R>(n, vi, vf, cost, m_sqrt(s2), uphi);
}

// The E_Q kernel's E(Q) and S(Q) programs: postfix {opcode, argument}
// pairs (MCV_EXPR_*) in the working precision (the FP32 kernels read the
// float copy), run on a stack of MCV_EXPR_STACK values.  A malformed
// program (stack under- or overflow, unknown opcode, not exactly one value
// left) gives NaN and never reads or writes outside the stack.  POWI is
// x**n by binary powering, MOD Python's float % (sign of the divisor).
template <typename R>
__device__ __forceinline__ R expr_unary(int op, R x) {
  if constexpr (sizeof(R) == 4) {
    switch (op) {
      case MCV_EXPR_NEG: return -x;
      case MCV_EXPR_EXP: return expf(x);
      case MCV_EXPR_LOG: return logf(x);
      case MCV_EXPR_LOG10: return log10f(x);
      case MCV_EXPR_SQRT: return sqrtf(x);
      case MCV_EXPR_SIN: return sinf(x);
      case MCV_EXPR_COS: return cosf(x);
      case MCV_EXPR_TAN: return tanf(x);
      case MCV_EXPR_ASIN: return asinf(x);
      case MCV_EXPR_ACOS: return acosf(x);
      case MCV_EXPR_ATAN: return atanf(x);
      case MCV_EXPR_SINH: return sinhf(x);
      case MCV_EXPR_COSH: return coshf(x);
      case MCV_EXPR_TANH: return tanhf(x);
      case MCV_EXPR_ASINH: return asinhf(x);
      case MCV_EXPR_ACOSH: return acoshf(x);
      case MCV_EXPR_ATANH: return atanhf(x);
      case MCV_EXPR_ERF: return erff(x);
      case MCV_EXPR_ERFC: return erfcf(x);
      case MCV_EXPR_FABS: return fabsf(x);
      case MCV_EXPR_FLOOR: return floorf(x);
      case MCV_EXPR_CEIL: return ceilf(x);
      default: return __int_as_float(0x7fffffff);
    }
  } else {
    switch (op) {
      case MCV_EXPR_NEG: return -x;
      case MCV_EXPR_EXP: return exp(x);
      case MCV_EXPR_LOG: return log(x);
      case MCV_EXPR_LOG10: return log10(x);
      case MCV_EXPR_SQRT: return sqrt(x);
      case MCV_EXPR_SIN: return sin(x);
      case MCV_EXPR_COS: return cos(x);
      case MCV_EXPR_TAN: return tan(x);
      case MCV_EXPR_ASIN: return asin(x);
      case MCV_EXPR_ACOS: return acos(x);
      case MCV_EXPR_ATAN: return atan(x);
      case MCV_EXPR_SINH: return sinh(x);
      case MCV_EXPR_COSH: return cosh(x);
      case MCV_EXPR_TANH: return tanh(x);
      case MCV_EXPR_ASINH: return asinh(x);
      case MCV_EXPR_ACOSH: return acosh(x);
      case MCV_EXPR_ATANH: return atanh(x);
      case MCV_EXPR_ERF: return erf(x);
      case MCV_EXPR_ERFC: return erfc(x);
      case MCV_EXPR_FABS: return fabs(x);
      case MCV_EXPR_FLOOR: return floor(x);
      case MCV_EXPR_CEIL: return ceil(x);
      default: return __longlong_as_double(0x7ff8000000000000ll);
    }
  }
}

template <typename R>
__device__ __forceinline__ R expr_binary(int op, R a, R b) {
  switch (op) {
    case MCV_EXPR_ADD: return a + b;
    case MCV_EXPR_SUB: return a - b;
    case MCV_EXPR_MUL: return a * b;
    case MCV_EXPR_DIV: return a / b;
    case MCV_EXPR_MIN: return b < a ? b : a;
    case MCV_EXPR_MAX: return b > a ? b : a;
    default: break;
  }
  if constexpr (sizeof(R) == 4) {
    if (op == MCV_EXPR_POW) return powf(a, b);
    if (op == MCV_EXPR_ATAN2) return atan2f(a, b);
    R r = fmodf(a, b);
    return (r != 0.f && ((r < 0.f) != (b < 0.f))) ? r + b : r;
  } else {
    if (op == MCV_EXPR_POW) return pow(a, b);
    if (op == MCV_EXPR_ATAN2) return atan2(a, b);
    R r = fmod(a, b);
    return (r != 0.0 && ((r < 0.0) != (b < 0.0))) ? r + b : r;
  }
}

template <typename R>
__device__ __noinline__ R expr_eval(const R* __restrict__ prog, int nops,
                                    R Q) {
  R st[MCV_EXPR_STACK];
  int sp = 0;
  const R nan = R(0) / R(0);
  for (int i = 0; i < nops; ++i) {
    const int op = (int)__ldg(&prog[2 * i]);
    const R arg = __ldg(&prog[2 * i + 1]);
    if (op == MCV_EXPR_CONST || op == MCV_EXPR_Q) {
      if (sp >= MCV_EXPR_STACK) return nan;
      st[sp++] = op == MCV_EXPR_CONST ? arg : Q;
      continue;
    }
    if (sp < 1) return nan;
    const R x = st[sp - 1];
    if (op >= MCV_EXPR_ADD && op <= MCV_EXPR_MOD && op != MCV_EXPR_NEG &&
        op != MCV_EXPR_POWI) {
      if (sp < 2) return nan;
      st[sp - 2] = expr_binary<R>(op, st[sp - 2], x);
      --sp;
      continue;
    }
    if (op == MCV_EXPR_POWI) {
      const int e = (int)arg;
      unsigned m = e < 0 ? 0u - (unsigned)e : (unsigned)e;
      R r = R(1), b = x;
      while (m) {
        if (m & 1u) r *= b;
        m >>= 1;
        if (m) b *= b;
      }
      st[sp - 1] = e < 0 ? R(1) / r : r;
      continue;
    }
    st[sp - 1] = expr_unary<R>(op, x);
  }
  return sp == 1 ? st[0] : nan;
}

// The S of makeS (acc/kernels/E_Q.py:37-98): up to max_iter draws of Q
// uniform on [Qmin, Qmax), each rejected while E(Q) exceeds Ei or the
// transfer is kinematically closed (cos^2 > 1); none accepted -> p = 0.
// Weight S(Q) (vf/vi) Q (Qmax-Qmin) / (2 ki kf) / tries.
template <typename R, typename Rng>
__device__ __forceinline__ void e_q_scatter(Neutron<R>& n, Rng& rng,
                                            const mcv_component& c) {
  const R Qmin = prm<R>(c, 10), Qmax = prm<R>(c, 11);
  const int max_iter = (int)c.dp[12];
  const int nE = c.ip[4], nS = c.ip[5];
  const R* progE = sizeof(R) == 4 ? (const R*)c.ftable : (const R*)c.table;
  const R* progS = progE + 2 * nE;
  const R vi = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  const R Ei = vi * vi * R(kVS2E);
  const R ki = R(kV2K) * vi;
  R Q = 0, vf = 0, kf = 0, cost = 0, cost2 = 0;
  int itr = 0;
  bool found = false;
  if (c.dp[13] != 0.0) {
    // E does not depend on Q (dp 13, set by the host): evaluated once.
    // FP64: every try draws its Q and tests the same arithmetic as below;
    // when the neutron cannot lose E at all, every one of the max_iter
    // tries fails, and their draws are skipped without being formed.
    const R E = expr_eval<R>(progE, nE, Qmin);
    const R Ef = Ei - E;
    if (Ef < R(0)) {
      rng.skip(max_iter);
      n.p = R(0);
      return;
    }
    vf = m_sqrt(Ef) * R(kSE2V);
    kf = R(kV2K) * vf;
    if constexpr (sizeof(R) == 4) {
      // FP32: the loop's outcome drawn directly.  A try accepts Q exactly
      // when |ki - kf| <= Q <= ki + kf (cos^2 <= 1), an interval of
      // [Qmin, Qmax) taken with probability a; the failed tries before
      // the first success are geometric (P(>= k) = (1 - a)^k, drawn by
      // inversion) and the accepted Q is uniform on the interval, so
      // (tries, Q) has the reference's distribution from two draws
      // instead of up to max_iter.  Near the threshold (Ef -> 0, a -> 0)
      // the loop takes tens of tries, on some lanes of a warp only.
      const R lo = m_fabs(ki - kf) > Qmin ? m_fabs(ki - kf) : Qmin;
      const R hi = ki + kf < Qmax ? ki + kf : Qmax;
      if (!(hi > lo)) {
        n.p = R(0);
        return;
      }
      const R a = (hi - lo) / (Qmax - Qmin);
      int fails = 0;
      if (a < R(1)) {
        const R u = rng.next();
        const float r = logf(1.f - u) / log1pf(-a);
        if (!(r < float(max_iter))) {
          n.p = R(0);
          return;
        }
        fails = (int)r;
      }
      if (fails >= max_iter) {
        n.p = R(0);
        return;
      }
      itr = fails;
      Q = lo + rng.next() * (hi - lo);
      cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
      cost = cost > R(1) ? R(1) : (cost < R(-1) ? R(-1) : cost);
      cost2 = cost * cost;
      found = true;
    }
    for (; !found && itr < max_iter; ++itr) {
      Q = rng.next() * (Qmax - Qmin);
      Q += Qmin;
      cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
      cost2 = cost * cost;
      if (cost2 > R(1)) continue;
      found = true;
      break;
    }
  } else {
    for (; itr < max_iter; ++itr) {
      Q = rng.next() * (Qmax - Qmin);
      Q += Qmin;
      const R E = expr_eval<R>(progE, nE, Q);
      const R Ef = Ei - E;
      if (Ef < R(0)) continue;
      vf = m_sqrt(Ef) * R(kSE2V);
      kf = R(kV2K) * vf;
      cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
      cost2 = cost * cost;
      if (cost2 > R(1)) continue;
      found = true;
      break;
    }
  }
  if (!found) {
    n.p = R(0);
    return;
  }
  R s2;
  if constexpr (sizeof(R) == 4) {
    const R Q2 = Q * Q, dk = ki - kf, sk = ki + kf;
    s2 = (Q2 - dk * dk) * (sk * sk - Q2) / (4 * ki * ki * kf * kf);
    s2 = s2 > R(0) ? s2 : R(0);
  } else {
    s2 = 1.0 - cost2;
  }
  const R uphi = rng.next();
  qe_velocity<R>(n, vi, vf, cost, m_sqrt(s2), uphi);
  const R S = expr_eval<R>(progS, nS, Q);
  const R prob_f = S * (vf / vi) * Q * (Qmax - Qmin) / (kf * ki) / 2;
  n.p *= prob_f / R(itr + 1);
}

// The scattering coefficient: the kernel's constant sigma, the powder's
// speed-dependent one, or a composite's: the sum over its elements (the
// element slots follow the component, header: COMPOSITE), scaled by dp[10]
// (1/N when averaged, composite.py:95-99), when an element's depends on the
// speed; else dp[9] holds that sum.
template <typename R, bool kX = false>
__device__ __forceinline__ R hss_sigma(const Neutron<R>& n,
                                       const mcv_component& c) {
  if (c.ip[1] == MCV_KERNEL_POWDER) return powder_coeff<R>(n, c);
  if constexpr (kX) {
    if (c.ip[1] == MCV_KERNEL_COMPOSITE && (c.ip[5] & 1)) {
      const mcv_component* e = &c + 1;
      R s = R(0);
      for (int i = 0; i < c.ip[4]; ++i)
        s += e[i].ip[1] == MCV_KERNEL_POWDER ? powder_coeff<R>(n, e[i])
                                             : prm<R>(e[i], 9);
      return s * prm<R>(c, 10);
    }
  }
  return prm<R>(c, 9);
}

template <typename R>
__device__ __forceinline__ R hss_mu(const Neutron<R>& n,
                                    const mcv_component& c) {
  // calc_absorption_coeff (acc/kernels/__init__.py:156-161)
  R v = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  return prm<R>(c, 8) / v * 2200;
}

// SANS2D_ongrid's S (acc/kernels/SANS2D_ongrid.py:16-56): (Qx, Qy) drawn
// uniformly over the grid's box; vx -= Qx K2V, vy -= Qy K2V and vz from
// vi^2 - vx^2 vy^2 (the reference's expression: a product where
// |v| = vi would need a sum; kept); p *= S bilinear on cells of width
// (Qmax - Qmin) / n, indices clamped to [0, n-2].
template <typename R, typename Rng>
__device__ __forceinline__ void sans2d_scatter(Neutron<R>& n, Rng& rng,
                                               const mcv_component& c) {
  const R Qxmin = prm<R>(c, 10), Qxmax = prm<R>(c, 11),
          Qymin = prm<R>(c, 12), Qymax = prm<R>(c, 13);
  const int nx = c.ip[4], ny = c.ip[5];
  const R vi = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  R Qx = rng.next() * (Qxmax - Qxmin);
  Qx += Qxmin;
  R Qy = rng.next() * (Qymax - Qymin);
  Qy += Qymin;
  n.vx -= Qx * R(kK2V);
  n.vy -= Qy * R(kK2V);
  n.vz = m_sqrt(vi * vi - n.vx * n.vx * n.vy * n.vy);
  const R dQx = (Qxmax - Qxmin) / nx, dQy = (Qymax - Qymin) / ny;
  int xi = (int)((Qx - Qxmin) / dQx), yi = (int)((Qy - Qymin) / dQy);
  xi = xi < 0 ? 0 : (xi > nx - 2 ? nx - 2 : xi);
  yi = yi < 0 ? 0 : (yi > ny - 2 ? ny - 2 : yi);
  const R xf = (Qx - Qxmin) / dQx - xi, yf = (Qy - Qymin) / dQy - yi;
  const R* S = sizeof(R) == 4 ? (const R*)c.ftable : (const R*)c.table;
  const R f00 = __ldg(&S[xi * ny + yi]), f10 = __ldg(&S[(xi + 1) * ny + yi]);
  const R f01 = __ldg(&S[xi * ny + yi + 1]),
          f11 = __ldg(&S[(xi + 1) * ny + yi + 1]);
  // bilinear_interp (SANS2D_ongrid.py:16-22)
  const R a00 = f00, a10 = f10 - f00, a01 = f01 - f00,
          a11 = f11 - f10 - f01 + f00;
  n.p *= a00 + a10 * xf + a01 * yf + a11 * xf * yf;
}

// DGSSXResKernel.scatter (acc/kernels/DGSSXResKernel.py:19-98): towards
// a target disc of the given radius (choose_direction: uniform in cos(theta)
// over the cone, a rotation about an axis built with the reference's
// in-place vec3.cross, whose later components read the ones it already
// replaced, then about the target direction by phi), arriving at a time of
// flight uniform in tof_target +- dtof / 2.
// p *= solid angle / 4 pi * dtof * (2 Ef / tof) * vf / vi.  The flight time
// tof - t is formed in double in both precisions (times near 1 s apart by
// milliseconds).
template <typename R, typename Rng>
__device__ __forceinline__ void dgssxres_scatter(Neutron<R>& n, Rng& rng,
                                                 const mcv_component& c) {
  const R tx = prm<R>(c, 15) - n.x, ty = prm<R>(c, 16) - n.y,
          tz = prm<R>(c, 17) - n.z;
  const R rad = prm<R>(c, 18);
  const R l2 = tx * tx + ty * ty + tz * tz;
  R cmax = m_sqrt(l2 / (rad * rad + l2));
  if (rad < R(0)) cmax = -cmax;
  R solid, theta;
  if constexpr (sizeof(R) == 4) {
    // the cone of a small target has cos(theta) within ~1e-5 of 1, where
    // 1 - r and acos(r) lose most of float's digits: form 1 - cos(theta_max)
    // as sin^2 / (1 + cos) and theta as 2 asin(sqrt((1 - r) / 2))
    const R omc = rad < R(0) ? R(1) - cmax
                             : (rad * rad / (rad * rad + l2)) / (R(1) + cmax);
    solid = R(2 * kPi) * omc;
    const R om = rng.next() * omc;  // 1 - r
    theta = R(2) * asinf(m_sqrt(R(0.5) * om));
  } else {
    solid = R(2 * kPi) * (R(1) - cmax);
    R r = rng.next();
    r = r * (cmax - R(1)) + R(1);
    theta = acos(r);
  }
  const R phi = rng.next() * R(2 * kPi);
  R nx, ny, nz;
  if (tx == R(0) && tz == R(0)) { nx = 1; ny = 0; nz = 0; }
  else { nx = -tz; ny = 0; nz = tx; }
  nx = ny * tz - nz * ty;
  ny = nz * tx - nx * tz;
  nz = nx * ty - ny * tx;
  R dx = tx, dy = ty, dz = tz;
  rotate3<R>(dx, dy, dz, nx, ny, nz, theta, R(1e-7));
  rotate3<R>(dx, dy, dz, tx, ty, tz, phi, R(1e-7));
  const R inv = R(1) / m_sqrt(dx * dx + dy * dy + dz * dz);
  const double u = rng.next();
  const double tof_t = c.dp[19], dtof = c.dp[20];
  const double tmin = tof_t - 0.5 * dtof, tmax = tof_t + 0.5 * dtof;
  const double tof = u * (tmax - tmin) + tmin;
  double tn;
  if constexpr (sizeof(R) == 4) tn = n.t.dval();
  else tn = n.t.val();
  const R vf = R(double(m_sqrt(l2)) / (tof - tn));
  const R Ef = vf * vf * R(kVS2E);
  const R dEdt = R(2) * Ef / R(tof);
  const R prob = solid / R(4 * kPi) * R(dtof) * dEdt;
  const R vi = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
  n.vx = dx * inv * vf;
  n.vy = dy * inv * vf;
  n.vz = dz * inv * vf;
  n.p *= prob * (vf / vi);
}

// One kernel's scatter (p *= sigma, then its S).  kX: the constant-(Q, E)
// and E(Q) kernels are compiled into the instantiations for the rarer
// components only.
template <typename R, bool kX = false, typename Rng, typename Trk>
__device__ __forceinline__ void hss_kernel_leaf(Neutron<R>& n, Rng& rng,
                                                const mcv_component& c,
                                                Trk& trk) {
  switch (c.ip[1]) {
    case MCV_KERNEL_ISOTROPIC:
      n.p *= prm<R>(c, 9);  // kernels/__init__.py:42
      trk.sigma_factor(prm<R>(c, 9));
      isotropic_S<R>(n, rng);
      break;
    case MCV_KERNEL_POWDER:
      powder_scatter<R>(n, rng, c, trk);
      break;
    case MCV_KERNEL_SQE_GRID:
      n.p *= prm<R>(c, 9);
      trk.sigma_factor(prm<R>(c, 9));
      sqe_scatter<R>(n, rng, c, trk);
      break;
    case MCV_KERNEL_CONSTANT_QE:
      if constexpr (kX) {
        n.p *= prm<R>(c, 9);  // kernels/__init__.py:85
        constant_qe_scatter<R>(n, rng, c);
      }
      break;
    case MCV_KERNEL_E_Q:
      if constexpr (kX) {
        n.p *= prm<R>(c, 9);  // kernels/__init__.py:103
        e_q_scatter<R>(n, rng, c);
      }
      break;
    case MCV_KERNEL_SANS2D:
      if constexpr (kX) {
        n.p *= prm<R>(c, 9);  // kernels/__init__.py:119
        sans2d_scatter<R>(n, rng, c);
      }
      break;
    case MCV_KERNEL_DGSSXRES:
      if constexpr (kX) {
        n.p *= prm<R>(c, 9);  // kernels/__init__.py:138
        dgssxres_scatter<R>(n, rng, c);
      }
      break;
    default:
      break;
  }
}

// The composite kernel's scatter (composite.py:62-75, 101-104): one uniform
// picks element i, the first whose running weight exceeds it (the last one
// otherwise); the element scatters, and p /= its weight.
template <typename R, typename Rng, typename Trk>
__device__ __noinline__ void composite_scatter(Neutron<R>& n, Rng& rng,
                                               const mcv_component& c,
                                               Trk& trk) {
  const R r = rng.next();
  const mcv_component* e = &c + 1;
  const int last = c.ip[4] - 1;
  int i = 0;
  while (i < last && !(r < prm<R>(e[i], 23))) ++i;
  hss_kernel_leaf<R, true>(n, rng, e[i], trk);
  n.p /= prm<R>(e[i], 22);
}

template <typename R, bool kX = false, typename Rng, typename Trk>
__device__ __forceinline__ void hss_kernel(Neutron<R>& n, Rng& rng,
                                           const mcv_component& c, Trk& trk) {
  if constexpr (kX) {
    if (c.ip[1] == MCV_KERNEL_COMPOSITE) {
      composite_scatter<R>(n, rng, c, trk);
      return;
    }
  }
  hss_kernel_leaf<R, kX>(n, rng, c, trk);
}

// The weight factor exp(-(mu(v) + sigma(v)) L) seen by the tracker:
// d/dmu2200 = -2200 L / v; d/dsigma = -L for a constant scattering
// coefficient, d/ds_j = -L / (v^2 Vcell) for the K reachable powder peaks.
template <typename R, typename Trk>
__device__ __forceinline__ void track_atten(const Neutron<R>& n,
                                            const mcv_component& c, R L,
                                            Trk& trk) {
  if constexpr (Trk::kActive) {
    R v = m_sqrt(n.vx * n.vx + n.vy * n.vy + n.vz * n.vz);
    if (c.ip[1] == MCV_KERNEL_POWDER) {
      trk.atten(R(-2200) * L / v, R(0));
      int K = powder_reach(powder_table<R>(c), c.ip[4], v);
      trk.powder_atten(K, -L / (v * v * prm<R>(c, 10)));
    } else {
      trk.atten(R(-2200) * L / v, -L);
    }
  }
}

// HomogeneousSingleScatterer.propagate
// (acc/components/samples/homogeneous_single_scatterer.py:62-100), FP64:
// the reference's sequence.
template <bool kX, typename Rng, typename Trk>
__device__ __forceinline__ void hss(Neutron<double>& n, Rng& rng,
                                    const mcv_component& c, Trk& trk) {
  double x = n.x, y = n.y, z = n.z, vx = n.vx, vy = n.vy, vz = n.vz;
  Hits<double> h = intersect_shape<double>(c, x, y, z, vx, vy, vz);
  if (h.n < 2) return;
  if (h.get(h.n - 1) <= 0) return;
  double rand = rng.next();
  double T, ttravel, tin;
  time_to_scatter_ref<double>(h, rand, T, ttravel, tin);
  double dt = ttravel;
  if (dt <= 0) return;
  prop_dt(n, dt);
  double v = sqrt(vx * vx + vy * vy + vz * vz);
  double dist = v * tin;
  double fulllen = v * T;
  double sigma = hss_sigma<double, kX>(n, c);
  double mu = hss_mu<double>(n, c);
  double atten = exp(-(mu + sigma) * dist);
  n.p *= fulllen * atten;
  track_atten<double>(n, c, dist, trk);
  hss_kernel<double, kX>(n, rng, c, trk);
  if (n.p <= 0) return;
  h = intersect_shape<double>(c, n.x, n.y, n.z, n.vx, n.vy, n.vz);
  double dt3 = total_time_in_shape<double>(h);
  prop_dt(n, dt3);
  sigma = hss_sigma<double, kX>(n, c);
  mu = hss_mu<double>(n, c);
  // the reference uses the incident speed v here (line 98)
  double atten2 = exp(-(mu + sigma) * v * dt3);
  n.p *= atten2;
  track_atten<double>(n, c, v * dt3, trk);
}

// FP32 form of the same propagate.  The incoming ray is first moved to its
// closest approach p0 to the shape's origin (tau = 0 there, "now" is at
// tau_now = -t0), all hit times are measured on that tau axis, and every
// length that the reference forms as a difference of times measured from
// "now" is formed as a difference of tau values.  In exact arithmetic this
// is the reference's sequence; in float it avoids cancelling metre-scale
// flight times against centimetre-scale chords.
template <bool kX, typename Rng, typename Trk>
__device__ __forceinline__ void hss(Neutron<float>& n, Rng& rng,
                                    const mcv_component& c, Trk& trk) {
  float vx = n.vx, vy = n.vy, vz = n.vz;
  float v2 = vx * vx + vy * vy + vz * vz;
  float t0 = -(n.x * vx + n.y * vy + n.z * vz) / v2;
  float px = fmaf(vx, t0, n.x), py = fmaf(vy, t0, n.y), pz = fmaf(vz, t0, n.z);
  float tau_now = -t0;
  Hits<float> h = intersect_shape<float>(c, px, py, pz, vx, vy, vz);
  if (h.n < 2) return;
  if (h.get(h.n - 1) <= tau_now) return;
  float rand = rng.next();
  // segments ahead of "now": (enter, exit) pairs of the sorted hits; when
  // the first hit ahead has odd index the neutron is inside and the first
  // segment starts at "now".
  float T = 0.f, seg_a[2] = {0.f, 0.f}, seg_b[2] = {0.f, 0.f};
  int nseg = 0;
  int i0 = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    if (i < h.n && h.get(i) < tau_now) i0 = i + 1;
  int j = i0;
  if (i0 & 1) {
    seg_a[0] = tau_now;
    seg_b[0] = h.get(i0);
    nseg = 1;
    j = i0 + 1;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    if (nseg < 2 && j + 1 < h.n) {
      float a = h.get(j), b = h.get(j + 1);
      if (nseg == 0) { seg_a[0] = a; seg_b[0] = b; }
      else { seg_a[1] = a; seg_b[1] = b; }
      ++nseg;
      j += 2;
    }
  }
  float L0 = seg_b[0] - seg_a[0], L1 = nseg > 1 ? seg_b[1] - seg_a[1] : 0.f;
  T = L0 + L1;
  float tin = rand * T;
  // scattering point on the tau axis (reference: the first segment whose
  // cumulative in-shape time exceeds tin, else the last one)
  float tau_s = (nseg == 1 || tin < L0) ? seg_b[0] - (L0 - tin)
                                        : seg_b[1] - (T - tin);
  float dt = tau_s - tau_now;
  if (!(dt > 0.f) || nseg == 0) return;
  n.x = fmaf(vx, tau_s, px);
  n.y = fmaf(vy, tau_s, py);
  n.z = fmaf(vz, tau_s, pz);
  n.t.add(t0);
  n.t.add(tau_s);
  float v = sqrtf(v2);
  float dist = v * tin, fulllen = v * T;
  float sigma = hss_sigma<float, kX>(n, c);
  float mu = hss_mu<float>(n, c);
  n.p *= fulllen * __expf(-(mu + sigma) * dist);
  track_atten<float>(n, c, dist, trk);
  hss_kernel<float, kX>(n, rng, c, trk);
  if (n.p <= 0.f) return;
  h = intersect_shape<float>(c, n.x, n.y, n.z, n.vx, n.vy, n.vz);
  float dt3 = total_time_in_shape<float>(h);
  prop_dt(n, dt3);
  sigma = hss_sigma<float, kX>(n, c);
  mu = hss_mu<float>(n, c);
  n.p *= __expf(-(mu + sigma) * v * dt3);
  track_atten<float>(n, c, v * dt3, trk);
}

}  // namespace mcv
