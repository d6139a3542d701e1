// components.cuh -- device restatements of the mcvine/acc components.
//
// Each function is written for the two working precisions.  The FP64 forms
// keep the reference's operation order (they are the "plain" kernels).  The
// FP32 forms compute the same quantities with float-friendly conditioning:
// reciprocal square roots instead of divisions, 1 - tanh(x) evaluated as
// 2 / (1 + e^(2x)), a sample ray re-centred on its closest approach before
// intersecting, and an FP64 discriminant only near tangency.
#pragma once

#include "common.cuh"
#include "track.cuh"

namespace mcv {

// ===================================================================== source
// Source_simple.propagate (acc/components/sources/source_simple.py:114-162)
// with randvec_target_rect (:17-42) for the target on the z axis, where the
// two normalised perpendiculars are (-1,0,0) and (0,-1,0).
template <typename R, typename Rng>
__device__ __forceinline__ void source_simple(Neutron<R>& n, Rng& rng,
                                              const mcv_component& c) {
  const R width = prm<R>(c, 0), height = prm<R>(c, 1), radius = prm<R>(c, 2);
  const R Lambda0 = prm<R>(c, 3), dLambda = prm<R>(c, 4), E0 = prm<R>(c, 5),
          dE = prm<R>(c, 6);
  const R xw = prm<R>(c, 7), yh = prm<R>(c, 8), dist = prm<R>(c, 9),
          pmul = prm<R>(c, 10);
  R r1 = rng.next(), r2 = rng.next(), r3 = rng.next(), r4 = rng.next(),
    r5 = rng.next();
  R x, y;
  if (c.ip[0]) {
    x = width * (r1 - R(0.5));
    y = height * (r2 - R(0.5));
  } else {
    R r = m_sqrt_uniform(r2) * radius, s, co;
    m_sincos_2pi(r1, &s, &co);
    x = r * co;
    y = r * s;
  }
  R tdx = xw * (r3 * 2 - 1) / R(2.0);
  R tdy = yh * (r4 * 2 - 1) / R(2.0);
  R dist2 = m_sqrt(tdx * tdx + tdy * tdy + dist * dist);
  R solidangle = (xw * yh * dist) / (dist2 * dist2 * dist2);
  R dx = -tdx - x, dy = -tdy - y;
  R v;
  if (c.ip[1]) {
    R L = Lambda0 + dLambda * (r5 * 2 - 1);
    v = R(kK2V) * (R(2 * kPi) / L);
  } else {
    R E = E0 + dE * (r5 * 2 - 1);
    v = R(kSE2V) * m_sqrt(E);
  }
  n.x = x;
  n.y = y;
  n.z = R(0);
  if constexpr (sizeof(R) == 4) {
    R inv = m_rsqrt(dx * dx + dy * dy + dist * dist);
    R vs = v * inv;
    n.vx = vs * dx;
    n.vy = vs * dy;
    n.vz = vs * dist;
  } else {
    R dist1 = m_sqrt(dx * dx + dy * dy + dist * dist);
    n.vx = v * dx / dist1;
    n.vy = v * dy / dist1;
    n.vz = v * dist / dist1;
  }
  n.sx = R(0);
  n.sy = R(0);
  n.t.set(R(0));
  n.p = pmul * solidangle;
}

// ==================================================== stored neutrons
// NeutronFromStorage.propagate (acc/components/sources/
// neutronfromstorage.py:68-82): neutron i is stored neutron i mod N
// (table: N x 10 [x y z vx vy vz sx sy t p], float64; ftable its float
// copy).
template <typename R>
__device__ __forceinline__ void storage_source(Neutron<R>& n, uint64_t index,
                                               const mcv_component& c) {
  const uint64_t N = c.table_len / 10;
  const uint64_t row = (index % N) * 10;
  double v[10];
  if constexpr (sizeof(R) == 4) {
#pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = __ldg(&c.ftable[row + k]);
  } else {
    const double* d = static_cast<const double*>(c.table);
#pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = __ldg(&d[row + k]);
  }
  n.x = R(v[0]);
  n.y = R(v[1]);
  n.z = R(v[2]);
  n.vx = R(v[3]);
  n.vy = R(v[4]);
  n.vz = R(v[5]);
  n.sx = R(v[6]);
  n.sy = R(v[7]);
  n.t.set(R(v[8]));
  n.p = R(v[9]);
}

// ================================================== SNS moderator source
// SNS_source (acc/components/sources/SNS_source.py:20-207): E and the
// emission time from the moderator's cumulative tables (the host computes
// them as _SNS_source_utils.py:187-223 does).  FP64 inverts them per
// neutron with the reference's zero_find, whose two loops, unbounded in the
// reference, stop after 64 / 200 passes, as in the oracle; FP32 reads
// inverse tables the host builds with the same zero_find
// (sns_generate_f32).
constexpr int kSnsExpandMax = 64;
constexpr int kSnsBisectMax = 200;

// a table column, or P(t) interpolated between two E rows at weight wl
struct SnsVec {
  const double* a;
  const double* b;  // null: plain column
  double wl;
  __device__ __forceinline__ double at(int i) const {
    return b ? __ldg(&a[i]) * wl + __ldg(&b[i]) * (1 - wl) : __ldg(&a[i]);
  }
};

// quadint (SNS_source.py:59-64)
__device__ __forceinline__ double sns_quadint(double xdes, double x1,
                                              double x2, double x3,
                                              double y1, double y2,
                                              double y3) {
  double t1 = ((xdes - x2) * (xdes - x3) * y1) / ((x1 - x2) * (x1 - x3));
  double t2 = ((xdes - x1) * (xdes - x3) * y2) / ((x2 - x1) * (x2 - x3));
  double t3 = ((xdes - x1) * (xdes - x2) * y3) / ((x3 - x1) * (x3 - x2));
  return t1 + t2 + t3;
}

// quadfuncint (:66-75).  The reference scans up from index 1 for the first
// point not below xdes; on the ascending tables a binary search finds the
// same index.  Past the last point the reference reads beyond the array
// (undefined); the last bracket extrapolates here.  Index -1 wraps to the
// last point, as numba indexes.
__device__ __forceinline__ double sns_quadfuncint(double xdes, int xylen,
                                                  const double* vecx,
                                                  const SnsVec& vecy) {
  int lo = 1, hi = xylen;  // first idx in [1, xylen) with !(vecx < xdes)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&vecx[mid]) < xdes) lo = mid + 1;
    else hi = mid;
  }
  int idx = lo >= xylen ? xylen - 1 : lo;
  const double xi = __ldg(&vecx[idx]);
  if (xi == xdes) return vecy.at(idx);
  const int i0 = idx - 2 < 0 ? idx - 2 + xylen : idx - 2;
  return sns_quadint(xdes, __ldg(&vecx[i0]), __ldg(&vecx[idx - 1]), xi,
                     vecy.at(i0), vecy.at(idx - 1), vecy.at(idx));
}

// zero_find (:78-96)
__device__ __forceinline__ double sns_zero_find(const double* vecx, int len,
                                                const SnsVec& vecy,
                                                double yval, double xmin,
                                                double xmax, double tol) {
  double xl = xmin;
  double xh = pow(10.0, (log10(xmin) + yval * (log10(xmax) - log10(xmin))));
  double f = sns_quadfuncint(xl, len, vecx, vecy) - yval;
  double fmid = sns_quadfuncint(xh, len, vecx, vecy) - yval;
  for (int k = 0; k < kSnsExpandMax && fmid * f >= 0.0; ++k) {
    xh = xh + (xh - xl) * 2.0;
    fmid = sns_quadfuncint(xh, len, vecx, vecy) - yval;
  }
  double dx = xh - xl, rtb = xl;
  for (int k = 0; k < kSnsBisectMax &&
                  fabs(sns_quadfuncint(rtb, len, vecx, vecy) - yval) > tol;
       ++k) {
    dx = dx * 0.5;
    const double xmid = rtb + dx;
    fmid = sns_quadfuncint(xmid, len, vecx, vecy) - yval;
    if (fmid < 0) rtb = xmid;
  }
  return rtb;
}

// generate (:22-54): E (meV) and t (s) from two uniforms.  Out of line:
// one copy for the kernels that contain a source.
static __device__ __noinline__ void sns_generate(const mcv_component& c,
                                                 double randE, double randt,
                                                 double* Eout,
                                                 double* tout) {
  const int nE = c.ip[1], nt = c.ip[2];
  const int Eidx_start = c.ip[3], Eidx_stop = c.ip[4];
  const int tidx_start = c.ip[5], tidx_stop = c.ip[6];
  const double* Es = static_cast<const double*>(c.table);
  const double* Pvec = Es + nE;
  const double* ts = Pvec + nE;
  const double* Ptmat = ts + nt;
  const double EPmin = c.dp[6], EPmax = c.dp[7];
  double randp = EPmin + randE * (EPmax - EPmin);
  const SnsVec pv{Pvec, nullptr, 0.0};
  const double Eval = sns_zero_find(Es, nE, pv, randp, __ldg(&Es[Eidx_start]),
                                    __ldg(&Es[Eidx_stop]), 1e-7);
  int lo = 0, hi = nE;  // first idx with !(Es < Eval): the reference's scan
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&Es[mid]) < Eval) lo = mid + 1;
    else hi = mid;
  }
  // the reference's bracket Eidxh = lo, Eidxl = lo - 1 (:38-46), in
  // bounds: index -1 wraps to the last energy as numba's indexing does
  // (its weight wl is then 0 when Eval == Es[0]); an Eval above the last
  // tabulated energy, where the reference reads one row past its table,
  // takes the last row.
  int Eidxh = lo, Eidxl = lo - 1;
  double wl = 0.0;
  if (lo >= nE) {
    Eidxh = nE - 1;
    Eidxl = nE - 1;
  } else {
    if (Eidxl < 0) Eidxl = nE - 1;
    wl = (__ldg(&Es[Eidxh]) - Eval) / (__ldg(&Es[Eidxh]) - __ldg(&Es[Eidxl]));
  }
  const SnsVec pt{Ptmat + (size_t)Eidxl * nt, Ptmat + (size_t)Eidxh * nt, wl};
  const double p0 = pt.at(tidx_start), p1 = pt.at(tidx_stop - 1);
  randp = p0 + randt * (p1 - p0);
  double tval = 0;
  if (randp > 0.0)
    tval = sns_zero_find(ts, nt, pt, randp, __ldg(&ts[tidx_start]),
                         __ldg(&ts[tidx_stop - 1]), 1e-5);
  *Eout = Eval * 1000.0;
  *tout = tval * 1e-6;
}

// FP32 draw of E (meV) and t (s) from the host's inverse tables (ftable,
// layout in the header): E by linear interpolation in u; t from one of the
// two energy rows that bracket E, picked with probability proportional to
// the reference's row weight (wl, 1 - wl) times the row's mass in the t
// window, with the uniform rescaled into the pick, which samples the
// mixture the reference inverts (SNS_source.py:38-52).  Returns false for
// a u outside [u_lo, u_hi] or rows without mass: the caller then takes
// the FP64 sampler.
__device__ __forceinline__ bool sns_generate_f32(const mcv_component& c,
                                                 float randE, float randt,
                                                 double* Eout,
                                                 double* tout) {
  if (!c.ftable) return false;
  const int nE = c.ip[1];
  const float* Einv = c.ftable;
  const float* Es = Einv + (MCV_SNS_E_NODES + 1);
  const float* mass = Es + nE;
  const float* Tinv = mass + nE;
  float E;
  if (randE >= c.fp[16] && randE <= c.fp[17]) {
    const float s = randE * float(MCV_SNS_E_NODES);
    const int k = min((int)s, MCV_SNS_E_NODES - 1);
    const float e0 = __ldg(&Einv[k]);
    E = fmaf(s - float(k), __ldg(&Einv[k + 1]) - e0, e0);
  } else {
    // outside the regular range: the draw is u = k 2^-24, and the host
    // tabulated zero_find's energy for each such k
    const float* Etail = Tinv + (size_t)nE * (MCV_SNS_T_NODES + 1);
    const int k = (int)(randE * 16777216.f);
    const int nlo = (int)c.fp[18], nhi = (int)c.fp[19];
    if (k < nlo) {
      E = __ldg(&Etail[k]);
    } else if (k >= (1 << 24) - nhi && k < (1 << 24)) {
      E = __ldg(&Etail[nlo + k - ((1 << 24) - nhi)]);
    } else {
      return false;
    }
  }
  int lo = 0, hi = nE;  // first row with !(Es < E)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&Es[mid]) < E) lo = mid + 1;
    else hi = mid;
  }
  int Eh = lo, El = lo - 1;
  float wl = 0.f;
  if (lo >= nE) {
    Eh = nE - 1;
    El = nE - 1;
  } else {
    if (El < 0) El = nE - 1;
    wl = (__ldg(&Es[Eh]) - E) / (__ldg(&Es[Eh]) - __ldg(&Es[El]));
  }
  const float ml = wl * __ldg(&mass[El]), mh = (1.f - wl) * __ldg(&mass[Eh]);
  if (!(ml + mh > 0.f)) return false;
  const float pl = ml / (ml + mh);
  const bool low = randt < pl;
  const int row = low ? El : Eh;
  const float ut = low ? randt / pl : (randt - pl) / (1.f - pl);
  const float* T = Tinv + (size_t)row * (MCV_SNS_T_NODES + 1);
  const float st = fminf(ut, 1.f) * float(MCV_SNS_T_NODES);
  const int j = min((int)st, MCV_SNS_T_NODES - 1);
  const float t0 = __ldg(&T[j]);
  const float t = fmaf(st - float(j), __ldg(&T[j + 1]) - t0, t0);
  *Eout = double(E) * 1000.0;
  *tout = double(t) * 1e-6;
  return true;
}

// SNS_source.propagate (:157-207)
template <typename R, typename Rng>
__device__ __forceinline__ void sns_source(Neutron<R>& n, Rng& rng,
                                           const mcv_component& c) {
  const R randx = rng.next(), randy = rng.next();
  const R rand_theta = rng.next(), rand_phi = rng.next();
  const double randE = rng.next(), randt = rng.next();
  const R xwidth = prm<R>(c, 0), yheight = prm<R>(c, 1),
          radius = prm<R>(c, 2);
  const R focus_xw = prm<R>(c, 3), focus_yh = prm<R>(c, 4),
          dist = prm<R>(c, 5);
  R x, y, z = R(0);
  if (c.ip[7] & 1) {
    // STS_source.propagate (STS_source.py:242-259)
    const R tanMOa = prm<R>(c, 9), cylx = prm<R>(c, 10), cylz = prm<R>(c, 11);
    const R cylphi1 = prm<R>(c, 12), cylphi2 = prm<R>(c, 13);
    const R MR = prm<R>(c, 14), MOa = prm<R>(c, 15);
    if (c.ip[0]) {
      y = yheight * (randy - R(0.5));
      if (c.ip[7] & 2) {
        x = xwidth * (randx - R(0.5));
        z = m_sqrt(MR * MR - (x - cylx) * (x - cylx)) + cylz;
      } else {
        const R ang = -cylphi1 + randx * (cylphi1 + cylphi2) + MOa;
        z = cylz + MR * cos(ang);
        x = cylx + MR * sin(ang);
      }
    } else {
      R s, co;
      m_sincos_2pi(randx, &s, &co);
      const R r = m_sqrt_uniform(randy) * radius;
      x = r * co;
      y = r * s;
      z = tanMOa * x;
    }
  } else if (c.ip[0]) {
    x = xwidth * (randx - R(0.5));
    y = yheight * (randy - R(0.5));
  } else {
    R s, co;
    m_sincos_2pi(randx, &s, &co);
    const R r = m_sqrt_uniform(randy) * radius;
    x = r * co;
    y = r * s;
  }
  const R hdivmax = atan((focus_xw / R(2.0) - x) / dist);
  const R hdivmin = atan(-(focus_xw / R(2.0) + x) / dist);
  const R vdivmax = atan((focus_yh / R(2.0) - y) / dist);
  const R vdivmin = atan(-(focus_yh / R(2.0) + y) / dist);
  const R theta = hdivmin + (hdivmax - hdivmin) * rand_theta;
  const R phi = vdivmin + (vdivmax - vdivmin) * rand_phi;
  double E, t;
  if constexpr (sizeof(R) == 4) {
    if (!sns_generate_f32(c, float(randE), float(randt), &E, &t))
      sns_generate(c, randE, randt, &E, &t);
  } else {
    sns_generate(c, randE, randt, &E, &t);
  }
  const R v = R(kSE2V * sqrt(E));
  n.x = x;
  n.y = y;
  n.z = z;
  n.vx = v * cos(phi) * sin(theta);
  n.vy = v * sin(phi);
  n.vz = v * cos(phi) * cos(theta);
  n.sx = R(0);
  n.sy = R(0);
  n.t.set(R(t));
  n.p = prm<R>(c, 8);
}

// ====================================================================== guide
// calc_reflectivity (acc/components/optics/_guide_utils.py:6-23)
__device__ __forceinline__ double reflectivity(double Q, double R0, double Qc,
                                               double alpha, double m,
                                               double W) {
  double R = R0;
  if (Q > Qc) {
    double tmp = (Q - m * Qc) / W;
    if (tmp < 10)
      R *= (1 - tanh(tmp)) * (1 - alpha * (Q - Qc)) / 2;
    else
      R = 0;
  }
  return R;
}
// (1 - tanh(x)) / 2 == 1 / (1 + e^(2x)), which has no cancellation in
// float; expf (not the fast __expf, whose error grows with |x|) because the
// supermirror edge is steep: d ln R / dQ = 2 / W per bounce.
__device__ __forceinline__ float reflectivity(float Q, float R0, float Qc,
                                              float alpha, float m, float W) {
  float R = R0;
  if (Q > Qc) {
    float tmp = (Q - m * Qc) / W;
    if (tmp < 10.f)
      R *= (1.f - alpha * (Q - Qc)) / (1.f + expf(2.f * tmp));
    else
      R = 0.f;
  }
  return R;
}

// Guide.propagate (acc/components/optics/guide.py:66-162), split into the
// entry (propagate to z=0, absorb outside the opening: lines 74-83) and one
// pass of the bounce loop (lines 85-159) so that the path-regeneration
// kernel can advance a guide one bounce per step with the same arithmetic.
// The loop's locals live in the neutron itself; they are what the reference
// writes back at line 160.

// false when the neutron is absorbed at the opening (only p changes then)
template <typename R>
__device__ __forceinline__ bool guide_enter(Neutron<R>& n,
                                            const mcv_component& c) {
  const R hw1 = prm<R>(c, 2), hh1 = prm<R>(c, 3);
  R dt = -n.z / n.vz;
  R x = n.x + n.vx * dt;
  R y = n.y + n.vy * dt;
  if (x <= -hw1 || x >= hw1 || y <= -hh1 || y >= hh1) {
    n.p = R(-1);  // absorb (acc/neutron.py:25-28)
    return false;
  }
  n.x = x;
  n.y = y;
  n.z = R(0);
  n.t.add(dt);
  return true;
}

// One pass of the bounce loop in FP32, without branches: lanes of a warp
// reach the same bounce with different walls ahead, so every candidate
// time is formed and the earliest is kept by selects (same comparison order
// as the reference, guide.py:100-123); the reflection and the reflectivity
// are selected the same way.  Division by a zero normal product gives an
// infinity that the "approaching" test never selects.
template <typename Trk>
__device__ __forceinline__ bool guide_bounce_fp32(Neutron<float>& n,
                                                  const mcv_component& c,
                                                  Trk& trk) {
  const float ww = prm<float>(c, 0), hh = prm<float>(c, 1),
              hw1 = prm<float>(c, 2), hh1 = prm<float>(c, 3),
              l = prm<float>(c, 4);
  const float x = n.x, y = n.y, z = n.z, vx = n.vx, vy = n.vy, vz = n.vz;
  const float av = l * vx, bv = ww * vz, ah = l * vy, bh = hh * vz;
  const float vn1 = bv + av, vn2 = bv - av, vn3 = bh + ah, vn4 = bh - ah;
  const float cv1 = -hw1 * l - z * ww, cv2 = x * l;
  const float ch1 = -hh1 * l - z * hh, ch2 = y * l;
  float t1 = (l - z) / vz;
  int i = 0;
  const float s1 = (cv1 - cv2) / vn1, s2 = (cv1 + cv2) / vn2;
  const float s3 = (ch1 - ch2) / vn3, s4 = (ch1 + ch2) / vn4;
  if (vn1 < 0.f && s1 < t1) { t1 = s1; i = 1; }
  if (vn2 < 0.f && s2 < t1) { t1 = s2; i = 2; }
  if (vn3 < 0.f && s3 < t1) { t1 = s3; i = 3; }
  if (vn4 < 0.f && s4 < t1) { t1 = s4; i = 4; }
  if (i == 0) return true;  // the neutron left the guide
  n.x = fmaf(vx, t1, x);
  n.y = fmaf(vy, t1, y);
  n.z = fmaf(vz, t1, z);
  n.t.add(t1);
  const bool xw = i <= 2;
  const float vdn = i == 1 ? vn1 : i == 2 ? vn2 : i == 3 ? vn3 : vn4;
  const float lw = xw ? ww : hh;
  // mirror parallel to z: the reflection flips one component exactly,
  // q = 2 V2K |v_perp|; inclined mirror: v -= 2 (v.n) n / |n|^2
  const float rn = rsqrtf(fmaf(l, l, lw * lw));
  const float d = 2.f * vdn * (rn * rn);
  const float sg = (i == 1 || i == 3) ? -1.f : 1.f;
  const bool flat = lw == 0.f;
  const float vperp = xw ? vx : vy;
  const float q = flat ? float(2 * kV2K) * fabsf(vperp)
                       : float(kV2K) * (-2.f) * vdn * rn;
  const float vperp_new = flat ? -vperp : fmaf(sg * d, l, vperp);
  n.vx = xw ? vperp_new : vx;
  n.vy = xw ? vy : vperp_new;
  n.vz = flat ? vz : fmaf(-d, lw, vz);
  const float R0 = prm<float>(c, 5), Qc = prm<float>(c, 6),
              alpha = prm<float>(c, 7), m = prm<float>(c, 8),
              W = prm<float>(c, 9);
  trk.reflect(q, R0, Qc, alpha, m, W);
  // calc_reflectivity (_guide_utils.py:6-23) with (1 - tanh x) / 2 =
  // 1 / (1 + e^(2x)), evaluated for every lane and selected
  const float tmp = (q - m * Qc) / W;
  const float edge = R0 * (1.f - alpha * (q - Qc)) / (1.f + expf(2.f * tmp));
  const float refl = q > Qc ? (tmp < 10.f ? edge : 0.f) : R0;
  n.p *= refl;
  return n.p <= 0.f;
}

// One pass of the bounce loop in FP64, in the reference's operation order.
template <typename Trk>
__device__ __forceinline__ bool guide_bounce_fp64(Neutron<double>& n,
                                                  const mcv_component& c,
                                                  Trk& trk) {
  const double ww = c.dp[0], hh = c.dp[1], hw1 = c.dp[2], hh1 = c.dp[3],
               l = c.dp[4];
  double x = n.x, y = n.y, z = n.z, vx = n.vx, vy = n.vy, vz = n.vz;
  double av = l * vx, bv = ww * vz, ah = l * vy, bh = hh * vz;
  double vdotn_v1 = bv + av, vdotn_v2 = bv - av;
  double vdotn_h1 = bh + ah, vdotn_h2 = bh - ah;
  double cv1 = -hw1 * l - z * ww, cv2 = x * l;
  double ch1 = -hh1 * l - z * hh, ch2 = y * l;
  double t1 = (l - z) / vz, t2;
  int i = 0;
  if (vdotn_v1 < 0) {
    t2 = (cv1 - cv2) / vdotn_v1;
    if (t2 < t1) { t1 = t2; i = 1; }
  }
  if (vdotn_v2 < 0) {
    t2 = (cv1 + cv2) / vdotn_v2;
    if (t2 < t1) { t1 = t2; i = 2; }
  }
  if (vdotn_h1 < 0) {
    t2 = (ch1 - ch2) / vdotn_h1;
    if (t2 < t1) { t1 = t2; i = 3; }
  }
  if (vdotn_h2 < 0) {
    t2 = (ch1 + ch2) / vdotn_h2;
    if (t2 < t1) { t1 = t2; i = 4; }
  }
  if (i == 0) return true;  // the neutron left the guide
  n.x = x + vx * t1;
  n.y = y + vy * t1;
  n.z = z + vz * t1;
  n.t.add(t1);
  double vdn = (i == 1) ? vdotn_v1 : (i == 2) ? vdotn_v2 : (i == 3) ? vdotn_h1
                                                                   : vdotn_h2;
  double lw = (i <= 2) ? ww : hh;  // the mirror's slope term
  double nlen2 = l * l + lw * lw;
  double q = kV2K * (-2) * vdn / sqrt(nlen2);
  double d = 2 * vdn / nlen2;
  if (i == 1) {
    n.vx = vx - d * l;
    n.vz = vz - d * ww;
  } else if (i == 2) {
    n.vx = vx + d * l;
    n.vz = vz - d * ww;
  } else if (i == 3) {
    n.vy = vy - d * l;
    n.vz = vz - d * hh;
  } else {
    n.vy = vy + d * l;
    n.vz = vz - d * hh;
  }
  const double R0 = c.dp[5], Qc = c.dp[6], alpha = c.dp[7], m = c.dp[8],
               W = c.dp[9];
  trk.reflect(q, R0, Qc, alpha, m, W);
  n.p *= reflectivity(q, R0, Qc, alpha, m, W);
  return n.p <= 0;
}

// one pass of the bounce loop; true when the neutron has left the guide
// (it stays at its last reflection point, guide.py:122-123) or its weight
// is gone
template <typename R, typename Trk>
__device__ __forceinline__ bool guide_bounce(Neutron<R>& n,
                                             const mcv_component& c,
                                             Trk& trk) {
  if constexpr (sizeof(R) == 4)
    return guide_bounce_fp32(n, c, trk);
  else
    return guide_bounce_fp64(n, c, trk);
}

// The whole guide; returns 1 when the bounce loop ran out of its
// MCV_MAX_BOUNCES iterations.
template <typename R, typename Trk>
__device__ __forceinline__ int guide(Neutron<R>& n, const mcv_component& c,
                                     Trk& trk) {
  if (!guide_enter(n, c)) return 0;
  for (int nb = 0; nb < MCV_MAX_BOUNCES; ++nb)
    if (guide_bounce(n, c, trk)) return 0;
  return 1;
}

// guide_tapering.Guide.propagate (acc/components/optics/guide_tapering.py
// :140-291): nseg equal segments, each a tapered channel, read from the
// component's table (rows w1 w2 h1 h2 ww hh whalf hhalf lwhalf lhhalf;
// then, when ip[1] > 0, the narrowest width and height of each block of
// ip[1] segments).  Returns 1 when a bounce loop ran out of
// MCV_MAX_BOUNCES iterations.
template <typename R>
__device__ __forceinline__ const R* taper_table(const mcv_component& c) {
  if constexpr (sizeof(R) == 4)
    return c.ftable;
  else
    return static_cast<const double*>(c.table);
}

template <typename R>
__device__ __forceinline__ int guide_tapering(Neutron<R>& n,
                                              const mcv_component& c) {
  const int nseg = c.ip[0];
  const R* d = taper_table<R>(c);
  const R *w1 = d, *w2 = d + nseg, *h1 = d + 2 * nseg, *h2 = d + 3 * nseg,
          *ww = d + 4 * nseg, *hh = d + 5 * nseg, *whalf = d + 6 * nseg,
          *hhalf = d + 7 * nseg;
  const R l_seg = prm<R>(c, 0), R0 = prm<R>(c, 1), Qcx = prm<R>(c, 2),
          Qcy = prm<R>(c, 3), alphax = prm<R>(c, 4), alphay = prm<R>(c, 5),
          mx = prm<R>(c, 6), my = prm<R>(c, 7), W = prm<R>(c, 8);
  R x = n.x, y = n.y, z = n.z, vx = n.vx, vy = n.vy, vz = n.vz;
  Tof<R> t = n.t;
  R prob = n.p;
  // propagate to z=0 (:163-167)
  R dt = -z / vz;
  x += vx * dt;
  y += vy * dt;
  z = R(0);
  t.add(dt);
  int overflow = 0;
  const int blk = c.ip[1];
  const int nblk = blk > 0 ? (nseg + blk - 1) / blk : 0;
  const R* bminw = d + 10 * nseg;
  const R* bminh = bminw + nblk;
  for (int seg = 0; seg < nseg; ++seg) {
    if (blk > 0 && vz > R(0) && seg % blk == 0) {
      // Quiet blocks: a forward flight that stays inside the block's
      // narrowest opening at the block's entrance and exit planes stays
      // inside every segment's channel in between (|x(z)| is convex along
      // the ray, the walls are planar): each segment of the block would
      // pass its entrance check and its quiet test.  The neutron goes to
      // the entrance of the block's last segment, where those segments
      // would have left it.  The margin keeps flights within rounding of
      // a wall on the per-segment path.
      const int b = seg / blk;
      const int send = seg + blk < nseg ? seg + blk : nseg;
      const R ta = (seg * l_seg - z) / vz, tb = (send * l_seg - z) / vz;
      const R keep = sizeof(R) == 4 ? R(0.5 - 0.5e-4) : R(0.5 - 0.5e-9);
      const R hw = keep * __ldg(&bminw[b]), hh2 = keep * __ldg(&bminh[b]);
      const R xa = x + vx * ta, xb = x + vx * tb;
      const R ya = y + vy * ta, yb = y + vy * tb;
      if (m_fabs(xa) < hw && m_fabs(xb) < hw && m_fabs(ya) < hh2 &&
          m_fabs(yb) < hh2) {
        dt = ((send - 1) * l_seg - z) / vz;
        x += vx * dt;
        y += vy * dt;
        z += vz * dt;
        seg = send - 1;
        continue;
      }
    }
    const R zr = seg * l_seg;
    const R w1s = __ldg(&w1[seg]), hhalfs = __ldg(&hhalf[seg]);
    const R wws = __ldg(&ww[seg]), hhs = __ldg(&hh[seg]),
            whalfs = __ldg(&whalf[seg]);
    // propagate to the segment entrance (:171-175)
    dt = (zr - z) / vz;
    x += vx * dt;
    y += vy * dt;
    z += vz * dt;
    if (x <= R(-0.5) * w1s || x >= R(0.5) * w1s || y <= -hhalfs ||
        y >= hhalfs) {
      n.p = R(0);
      return 0;
    }
    // shift origin to the center of the channel hit (:180-186)
    x += R(0.5) * w1s;
    const R edge = floor(x / w1s) * w1s;
    if (x - edge > w1s) {
      n.p = R(0);
      return 0;
    }
    x -= (edge + R(0.5) * w1s);
    const R hadj = edge + (R(0.5) * w1s) - R(0.5) * w1s;
    if (vz > R(0)) {
      // inside at the entrance and at the exit plane: a straight forward
      // flight between two points inside the (planar) walls crosses none
      // of them, so the bounce loop would leave at once without moving
      // the neutron; go to the next segment with the same state
      const R tex = (zr + l_seg - z) / vz;
      R xe, ye;
      if constexpr (sizeof(R) == 4) {
        xe = fmaf(vx, tex, x);
        ye = fmaf(vy, tex, y);
      } else {
        xe = x + vx * tex;
        ye = y + vy * tex;
      }
      if (m_fabs(xe) < R(0.5) * __ldg(&w2[seg]) &&
          m_fabs(ye) < R(0.5) * __ldg(&h2[seg])) {
        x += hadj;
        continue;
      }
    }
    int nb;
    for (nb = 0; nb < MCV_MAX_BOUNCES; ++nb) {
      const R av = l_seg * vx, bv = wws * vz, ah = l_seg * vy, bh = hhs * vz;
      const R vdotn_v1 = bv + av, vdotn_v2 = bv - av;
      const R vdotn_h1 = bh + ah, vdotn_h2 = bh - ah;
      const R cv1 = -whalfs * l_seg - (z - zr) * wws, cv2 = x * l_seg;
      const R ch1 = -hhalfs * l_seg - (z - zr) * hhs, ch2 = y * l_seg;
      R t1 = (zr + l_seg - z) / vz, t2;
      int i = 0;
      if (vdotn_v1 < 0) {
        t2 = (cv1 - cv2) / vdotn_v1;
        if (t2 < t1) { t1 = t2; i = 1; }
      }
      if (vdotn_v2 < 0) {
        t2 = (cv1 + cv2) / vdotn_v2;
        if (t2 < t1) { t1 = t2; i = 2; }
      }
      if (vdotn_h1 < 0) {
        t2 = (ch1 - ch2) / vdotn_h1;
        if (t2 < t1) { t1 = t2; i = 3; }
      }
      if (vdotn_h2 < 0) {
        t2 = (ch1 + ch2) / vdotn_h2;
        if (t2 < t1) { t1 = t2; i = 4; }
      }
      if (i == 0) break;  // left the segment
      x += vx * t1;
      y += vy * t1;
      z += vz * t1;
      t.add(t1);
      const R vdn = i == 1 ? vdotn_v1 : i == 2 ? vdotn_v2
                                               : i == 3 ? vdotn_h1 : vdotn_h2;
      const R slope = i <= 2 ? wws : hhs;
      const R nlen2 = l_seg * l_seg + slope * slope;
      const R q = R(kV2K) * R(-2.0) * vdn / m_sqrt(nlen2);
      const R dd = R(2.0) * vdn / nlen2;
      if (i == 1) {
        vx = vx - dd * l_seg;
        vz = vz - dd * wws;
      } else if (i == 2) {
        vx = vx + dd * l_seg;
        vz = vz - dd * wws;
      } else if (i == 3) {
        vy = vy - dd * l_seg;
        vz = vz - dd * hhs;
      } else {
        vy = vy + dd * l_seg;
        vz = vz - dd * hhs;
      }
      // an m = 0 mirror ends the segment's loop (:256-258)
      if ((i <= 2 && mx == R(0)) || (i > 2 && my == R(0))) {
        x += hadj;
        break;
      }
      R m, Rf;
      if (i <= 2) {
        m = mx;
        if (m <= R(0)) m = m_fabs(mx * __ldg(&w1[0]) / w1s);
        Rf = reflectivity(q, R0, Qcx, alphax, m, W);
      } else {
        m = my;
        if (m <= R(0)) m = m_fabs(my * __ldg(&h1[0]) / __ldg(&h1[seg]));
        Rf = reflectivity(q, R0, Qcy, alphay, m, W);
      }
      if (Rf > R(1e-10)) {
        prob *= Rf;
      } else {
        n.p = R(0);
        return 0;
      }
    }
    if (nb == MCV_MAX_BOUNCES) overflow = 1;
    x += hadj;
  }
  n.x = x;
  n.y = y;
  n.z = z;
  n.vx = vx;
  n.vy = vy;
  n.vz = vz;
  n.t = t;
  n.p = prob;
  return overflow;
}

// ============================================================ mesh guide
// inside_convex_polygon (acc/components/optics/geometry2d.py:12-33): the
// point is on one side of every edge (cross products of one sign); an
// edge it lies on (|cross| < 1e-14) is skipped.
template <typename R>
__device__ __forceinline__ bool inside_convex_polygon(R px, R py,
                                                      const R* poly, int nv) {
  R ax = __ldg(&poly[0]), ay = __ldg(&poly[1]);
  R prev = (__ldg(&poly[2]) - ax) * (py - ay) - (__ldg(&poly[3]) - ay) * (px - ax);
  bool prev_side = prev <= R(0);
  for (int k = 1; k < nv; ++k) {
    const int k2 = k + 1 < nv ? k + 1 : 0;
    ax = __ldg(&poly[2 * k]);
    ay = __ldg(&poly[2 * k + 1]);
    const R sign = (__ldg(&poly[2 * k2]) - ax) * (py - ay) -
                   (__ldg(&poly[2 * k2 + 1]) - ay) * (px - ax);
    if (m_fabs(sign) < R(1e-14)) continue;
    const bool side = sign <= R(0);
    if (m_fabs(prev) < R(1e-14)) {
      prev_side = side;
      continue;
    }
    if (prev_side != side) return false;
  }
  return true;
}

// Guide_anyshape._propagate (acc/components/optics/guide_anyshape.py:
// 96-158): each pass takes, among the faces whose plane the neutron reaches
// at t > 0, the nearest hit that lies inside the face's polygon (the
// reference sorts every positive hit time and takes the first inside one:
// the same face, ties aside), moves there less 1e-14 of the way, and
// reflects off the face with the supermirror reflectivity; none -> the
// neutron has left the guide, where it stays (no propagation to the exit).
// Returns 1 when MCV_ANYSHAPE_MAX_BOUNCES passes did not let it out.
template <typename R>
__device__ __forceinline__ int guide_anyshape(Neutron<R>& n,
                                              const mcv_component& c) {
  const int nf = c.ip[0], nv = c.ip[1], stride = 12 + 2 * nv;
  const R* F = sizeof(R) == 4 ? (const R*)c.ftable : (const R*)c.table;
  const R R0 = prm<R>(c, 0), Qc = prm<R>(c, 1), alpha = prm<R>(c, 2),
          m = prm<R>(c, 3), W = prm<R>(c, 4);
  // FP32: the reference backs a hit off by 1e-14 of its flight so that
  // the next pass does not find the same face again; in float that is
  // below resolution, so the face just left is skipped instead (a
  // reflection from a plane moves away from it: in exact arithmetic it
  // cannot be next).  FP64 keeps the reference's sequence.
  int last = -1;
  for (int nb = 0; nb < MCV_ANYSHAPE_MAX_BOUNCES; ++nb) {
    R best = R(0);
    int bi = -1;
    for (int f = 0; f < nf; ++f) {
      if (sizeof(R) == 4 && f == last) continue;
      const R* g = F + (size_t)f * stride;
      const R cx = __ldg(&g[0]), cy = __ldg(&g[1]), cz = __ldg(&g[2]);
      const R nx = __ldg(&g[9]), ny = __ldg(&g[10]), nz = __ldg(&g[11]);
      // intersect_plane (:22-29)
      const R dist = (cx - n.x) * nx + (cy - n.y) * ny + (cz - n.z) * nz;
      const R vn = n.vx * nx + n.vy * ny + n.vz * nz;
      const R t = dist / vn;
      if (!(t > R(0)) || (bi >= 0 && !(t < best))) continue;
      const R qx = n.x + n.vx * t - cx, qy = n.y + n.vy * t - cy,
              qz = n.z + n.vz * t - cz;
      const R u = qx * __ldg(&g[3]) + qy * __ldg(&g[4]) + qz * __ldg(&g[5]);
      const R w = qx * __ldg(&g[6]) + qy * __ldg(&g[7]) + qz * __ldg(&g[8]);
      if (inside_convex_polygon<R>(u, w, g + 12, nv)) {
        best = t;
        bi = f;
      }
    }
    if (bi < 0) return 0;
    const R* g = F + (size_t)bi * stride;
    const R nx = __ldg(&g[9]), ny = __ldg(&g[10]), nz = __ldg(&g[11]);
    const R t = best - best * R(1e-14);
    const R vq = -(n.vx * nx + n.vy * ny + n.vz * nz) * R(2);
    const R Rf = reflectivity(m_fabs(vq) * R(kV2K), R0, Qc, alpha, m, W);
    if (!(n.p * Rf > R(0))) {
      // absorb (acc/neutron.py:27-28) before the move is written back
      n.p = R(-1);
      return 0;
    }
    n.p *= Rf;
    n.x += n.vx * t;
    n.y += n.vy * t;
    n.z += n.vz * t;
    n.t.add(t);
    n.vx += nx * vq;
    n.vy += ny * vq;
    n.vz += nz * vq;
    last = bi;
  }
  return 1;
}

// The gravity form (acc/components/optics/guide_anyshape_gravity.py:
// 25-182): a face plane is reached where n.(r + v t + g t^2 / 2 - c) = 0
// (intersect_plane: both roots of the quadratic, the linear root when
// |g.n| / 2 < 1e-10); each pass takes the earliest root t > 0 at or past
// 1e-10 s whose point lies inside its face (no back-off), moves along the
// parabola (propagate_with_gravity: v' = v + g t, r' = r + (v + v') t / 2)
// and reflects.  An absorbed neutron keeps the hit's position and time.
// Past the last reflection a neutron short of z_max is carried to the
// plane z = z_max without advancing its time, taking the first root when
// it is positive and also when only the second one is (the reference's
// choice, kept).  FP32: on the face just left a root below 1e-6 s is the
// neutron's own position again (float rounding on the face), so it is
// skipped there; a genuine return onto the same face takes milliseconds.
template <typename R>
__device__ __forceinline__ void gravity_roots(R px, R py, R pz, R vx, R vy,
                                              R vz, R gx, R gy, R gz, R cx,
                                              R cy, R cz, R nx, R ny, R nz,
                                              R& t0, R& t1) {
  const R A = (gx * nx + gy * ny + gz * nz) / R(2);
  const R B = vx * nx + vy * ny + vz * nz;
  const R C = (px * nx + py * ny + pz * nz) - (cx * nx + cy * ny + cz * nz);
  if (m_fabs(A) < R(1e-10)) {
    t0 = -C / B;
    t1 = R(-1);
    return;
  }
  const R d = B * B - R(4) * A * C;
  if (d < R(0)) {
    t0 = t1 = R(-1);
    return;
  }
  const R s = m_sqrt(d);
  t0 = (-B - s) / R(2) / A;
  t1 = (-B + s) / R(2) / A;
}

template <typename R>
__device__ __forceinline__ int guide_anyshape_gravity(Neutron<R>& n,
                                                      const mcv_component& c) {
  const int nf = c.ip[0], nv = c.ip[1], stride = 12 + 2 * nv;
  const R* F = sizeof(R) == 4 ? (const R*)c.ftable : (const R*)c.table;
  const R R0 = prm<R>(c, 0), Qc = prm<R>(c, 1), alpha = prm<R>(c, 2),
          m = prm<R>(c, 3), W = prm<R>(c, 4);
  const R gx = prm<R>(c, 5), gy = prm<R>(c, 6), gz = prm<R>(c, 7);
  int last = -1, overflow = 1;
  for (int nb = 0; nb < MCV_ANYSHAPE_MAX_BOUNCES; ++nb) {
    R best = R(0);
    int bi = -1;
    for (int f = 0; f < nf; ++f) {
      const R* g = F + (size_t)f * stride;
      const R cx = __ldg(&g[0]), cy = __ldg(&g[1]), cz = __ldg(&g[2]);
      R t[2];
      gravity_roots<R>(n.x, n.y, n.z, n.vx, n.vy, n.vz, gx, gy, gz, cx, cy, cz,
                       __ldg(&g[9]), __ldg(&g[10]), __ldg(&g[11]), t[0], t[1]);
      const R tmin = (sizeof(R) == 4 && f == last) ? R(1e-6) : R(1e-10);
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const R tk = t[k];
        if (!(tk > R(0)) || tk < tmin || (bi >= 0 && !(tk < best))) continue;
        const R wx = n.vx + gx * tk, wy = n.vy + gy * tk, wz = n.vz + gz * tk;
        const R qx = n.x + (n.vx + wx) * (R(0.5) * tk) - cx,
                qy = n.y + (n.vy + wy) * (R(0.5) * tk) - cy,
                qz = n.z + (n.vz + wz) * (R(0.5) * tk) - cz;
        const R u = qx * __ldg(&g[3]) + qy * __ldg(&g[4]) + qz * __ldg(&g[5]);
        const R w = qx * __ldg(&g[6]) + qy * __ldg(&g[7]) + qz * __ldg(&g[8]);
        if (inside_convex_polygon<R>(u, w, g + 12, nv)) {
          best = tk;
          bi = f;
        }
      }
    }
    if (bi < 0) {
      overflow = 0;
      break;
    }
    const R* g = F + (size_t)bi * stride;
    const R nx = __ldg(&g[9]), ny = __ldg(&g[10]), nz = __ldg(&g[11]);
    const R t = best;
    const R wx = n.vx + gx * t, wy = n.vy + gy * t, wz = n.vz + gz * t;
    n.x = n.x + (n.vx + wx) * (R(0.5) * t);
    n.y = n.y + (n.vy + wy) * (R(0.5) * t);
    n.z = n.z + (n.vz + wz) * (R(0.5) * t);
    n.vx = wx;
    n.vy = wy;
    n.vz = wz;
    n.t.add(t);
    const R vq = -(wx * nx + wy * ny + wz * nz) * R(2);
    const R Rf = reflectivity(m_fabs(vq) * R(kV2K), R0, Qc, alpha, m, W);
    if (!(n.p * Rf > R(0))) {
      n.p = R(-1);  // absorb (acc/neutron.py:27-28)
      return 0;
    }
    n.p *= Rf;
    n.vx += nx * vq;
    n.vy += ny * vq;
    n.vz += nz * vq;
    last = bi;
  }
  const R zmax = prm<R>(c, 8);
  if (n.z < zmax) {
    R t0, t1;
    gravity_roots<R>(n.x, n.y, n.z, n.vx, n.vy, n.vz, gx, gy, gz, R(0), R(0),
                     zmax, R(0), R(0), R(1), t0, t1);
    if (!(t0 > R(0)) && !(t1 > R(0))) return overflow;
    const R t = t0;  // also when only t1 > 0 (the reference's choice)
    const R wx = n.vx + gx * t, wy = n.vy + gy * t, wz = n.vz + gz * t;
    n.x = n.x + (n.vx + wx) * (R(0.5) * t);
    n.y = n.y + (n.vy + wy) * (R(0.5) * t);
    n.z = n.z + (n.vz + wz) * (R(0.5) * t);
    n.vx = wx;
    n.vy = wy;
    n.vz = wz;
  }
  return overflow;
}

// Slit / Beamstop (acc/components/optics/slit.py:71-108,
// beamstop.py:75-112); dp = {xmin, xmax, ymin, ymax, radius^2, cut}
// (`up`: the chain's FP32 weight scale, which the cut is compared in)
template <typename R>
__device__ __forceinline__ void slit_or_beamstop(Neutron<R>& n,
                                                 const mcv_component& c,
                                                 bool stop, R up) {
  R xmin = prm<R>(c, 0), xmax = prm<R>(c, 1), ymin = prm<R>(c, 2),
    ymax = prm<R>(c, 3), r2 = prm<R>(c, 4), cut = prm<R>(c, 5) * up;
  R x = n.x, y = n.y, z = n.z, vx = n.vx, vy = n.vy, vz = n.vz;
  if ((z < 0 && vz <= 0) || (z > 0 && vz >= 0)) return;
  if (n.p < cut) {
    n.p = R(-1);
    return;
  }
  R dt = R(0);
  if (z != 0) {
    dt = -z / vz;
    x += vx * dt;
    y += vy * dt;
  }
  bool in;
  if (r2 != 0) in = x * x + y * y <= r2;
  else in = xmin <= x && x <= xmax && ymin <= y && y <= ymax;
  if (stop ? in : !in) {
    n.p = R(-1);
    return;
  }
  n.x = x;
  n.y = y;
  n.z = R(0);
  if (z != 0) n.t.add(dt);
}

}  // namespace mcv
