/*
 * oracle.c -- CPU FP64 restatement of mcvine/acc's per-neutron propagation
 * chain.  TEST INFRASTRUCTURE ONLY: this file is the checker that the CUDA
 * engine is compared against (and the timed CPU baseline); no product code
 * path may call it.
 *
 * Each function restates the reference function cited beside it (paths are
 * relative to the mcvine/acc source tree).  The reference is Python/Numba;
 * the arithmetic below keeps its operation order so that FP64 results agree
 * with the reference to rounding.  Compile with -ffp-contract=off so that the
 * result does not depend on whether the host fuses multiply-adds.
 *
 * Components with no reference counterpart (energy monitor, theta x tof
 * shell, cylinder I(Q,E) detector, banked detector, gridded S(Q,E) kernel)
 * are restated from the nearest reference template named at each function.
 *
 * Uniform random numbers come from Philox4x32-10 (Salmon, Moraes, Dror,
 * Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), counter
 * (neutron index lo, hi, draw block, stream), key (seed lo, seed hi); each
 * 128-bit block gives five 24-bit integers u and so five float32-exact
 * uniforms u * 2^-24 in [0, 1), the resolution of the float32 uniforms the
 * reference draws
 * (xoroshiro128p_uniform_float32, e.g. source_simple.py:128-132).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/acc_gb300.h"

/* mcni.utils.conversion constants (the reference imports them from mcni;
 * V2K appears in acc/components/optics/guide_baseline.py:16-17). */
#define V2K 1.58825361e-3
#define K2V (1.0 / V2K)
#define SE2V 437.393377
#define VS2E 5.22703725e-6
#define GEOM_EPSILON 1e-10 /* acc/geometry/__init__.py:2 */
#define LOC_OUTSIDE 1      /* acc/geometry/location.py */
#define LOC_ONBORDER 0
#define LOC_INSIDE (-1)

/* ------------------------------------------------------------------ RNG */
static inline uint32_t mulhilo32(uint32_t a, uint32_t b, uint32_t* hi) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  *hi = (uint32_t)(p >> 32);
  return (uint32_t)p;
}

void oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                          uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0, hi1;
    uint32_t lo0 = mulhilo32(0xD2511F53u, c0, &hi0);
    uint32_t lo1 = mulhilo32(0xCD9E8D57u, c2, &hi1);
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

typedef struct {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t buf[5];
  int pos;           /* next uniform in buf; 5 = empty */
  const float* inj;  /* injected uniforms, or NULL   */
  int inj_pos, inj_stride;
  int overrun;
} rng_t;

static void rng_init(rng_t* r, uint64_t seed, uint64_t index, uint32_t stream,
                     const float* inj, int stride) {
  r->key[0] = (uint32_t)seed;
  r->key[1] = (uint32_t)(seed >> 32);
  r->ctr[0] = (uint32_t)index;
  r->ctr[1] = (uint32_t)(index >> 32);
  r->ctr[2] = 0;
  r->ctr[3] = stream;
  r->pos = 5;
  r->inj = inj;
  r->inj_pos = 0;
  r->inj_stride = stride;
  r->overrun = 0;
}

static double rng_uniform(rng_t* r) {
  if (r->inj) {
    if (r->inj_pos >= r->inj_stride) {
      r->overrun = 1;
      return 0.5;
    }
    return (double)r->inj[r->inj_pos++];
  }
  if (r->pos == 5) {
    /* one 128-bit block w0..w3 gives five 24-bit uniforms: bits 0-23,
     * 24-47, 48-71, 72-95 and 96-119 of w0 | w1 << 32 | w2 << 64 | w3 << 96 */
    uint32_t w[4];
    oracle_philox4x32_10(r->ctr, r->key, w);
    r->ctr[2]++;
    r->buf[0] = w[0] & 0xFFFFFFu;
    r->buf[1] = (w[0] >> 24) | ((w[1] & 0xFFFFu) << 8);
    r->buf[2] = (w[1] >> 16) | ((w[2] & 0xFFu) << 16);
    r->buf[3] = w[2] >> 8;
    r->buf[4] = w[3] & 0xFFFFFFu;
    r->pos = 0;
  }
  return (double)r->buf[r->pos++] * (1.0 / 16777216.0);
}

/* ------------------------------------------------------ neutron / vec3 */
typedef struct {
  double x, y, z, vx, vy, vz, sx, sy, t, p;
} neutron_t;

/* vec3.abs2rel + mXv (acc/vec3.py:148-159, acc/neutron.py:18-23) */
static void apply_transform(neutron_t* n, const double* m, const double* o) {
  double tx = n->x - o[0], ty = n->y - o[1], tz = n->z - o[2];
  double rx = m[0] * tx + m[1] * ty + m[2] * tz;
  double ry = m[3] * tx + m[4] * ty + m[5] * tz;
  double rz = m[6] * tx + m[7] * ty + m[8] * tz;
  double vx = m[0] * n->vx + m[1] * n->vy + m[2] * n->vz;
  double vy = m[3] * n->vx + m[4] * n->vy + m[5] * n->vz;
  double vz = m[6] * n->vx + m[7] * n->vy + m[8] * n->vz;
  n->x = rx; n->y = ry; n->z = rz;
  n->vx = vx; n->vy = vy; n->vz = vz;
}

/* prop_dt_inplace (acc/neutron.py:44-51) */
static inline void prop_dt(neutron_t* n, double dt) {
  n->x = n->x + n->vx * dt;
  n->y = n->y + n->vy * dt;
  n->z = n->z + n->vz * dt;
  n->t = n->t + dt;
}

static inline double length3(double a, double b, double c) {
  return sqrt(a * a + b * b + c * c);
}

static void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

/* vec3.normalize (acc/vec3.py:28-31): scale by 1/length */
static void normalize3(double* v) {
  double l = length3(v[0], v[1], v[2]);
  double s = 1.0 / l;
  v[0] *= s; v[1] *= s; v[2] *= s;
}

/* vec3._rotate (acc/vec3.py:77-105) */
void oracle_rotate(double* v, const double* c, double angle, double epsilon) {
  double c1[3] = {c[0], c[1], c[2]};
  normalize3(c1);
  double sf = v[0] * c1[0] + v[1] * c1[1] + v[2] * c1[2];
  double vpl[3] = {c1[0] * sf, c1[1] * sf, c1[2] * sf};
  if (fabs(1 - length3(vpl[0], vpl[1], vpl[2]) / length3(v[0], v[1], v[2])) <
      epsilon)
    return;
  double vpp[3] = {v[0] - vpl[0], v[1] - vpl[1], v[2] - vpl[2]};
  double vpp_len = length3(vpp[0], vpp[1], vpp[2]);
  double inv = 1. / vpp_len;
  vpp[0] *= inv; vpp[1] *= inv; vpp[2] *= inv;
  double e3[3];
  cross3(vpp, c1, e3);
  double ca = cos(angle), sa = sin(angle);
  vpp[0] *= ca; vpp[1] *= ca; vpp[2] *= ca;
  e3[0] *= sa; e3[1] *= sa; e3[2] *= sa;
  double r[3] = {vpp[0] - e3[0], vpp[1] - e3[1], vpp[2] - e3[2]};
  r[0] *= vpp_len; r[1] *= vpp_len; r[2] *= vpp_len;
  v[0] = r[0] + vpl[0];
  v[1] = r[1] + vpl[1];
  v[2] = r[2] + vpl[2];
}

/* ------------------------------------------------------------- source */
/* randvec_target_rect (acc/components/sources/source_simple.py:17-42) */
static double randvec_target_rect(const double* target, double width,
                                  double height, double rand1, double rand2,
                                  double* vecout) {
  double dx = width * (rand1 * 2 - 1) / 2.0;
  double dy = height * (rand2 * 2 - 1) / 2.0;
  double dist = length3(target[0], target[1], target[2]);
  double vertical[3] = {0.0, 1.0, 0.0};
  double p1[3], p2[3];
  cross3(target, vertical, p1);
  normalize3(p1);
  cross3(target, p1, p2);
  normalize3(p2);
  p1[0] *= dx; p1[1] *= dx; p1[2] *= dx;
  p2[0] *= dy; p2[1] *= dy; p2[2] *= dy;
  double tmp[3] = {p1[0] + target[0], p1[1] + target[1], p1[2] + target[2]};
  vecout[0] = p2[0] + tmp[0];
  vecout[1] = p2[1] + tmp[1];
  vecout[2] = p2[2] + tmp[2];
  double dist2 = sqrt(dx * dx + dy * dy + dist * dist);
  return (width * height * dist) / (dist2 * dist2 * dist2);
}

/* Source_simple.propagate (source_simple.py:114-162) */
static void source_simple(neutron_t* n, rng_t* rng, const mcv_component* c) {
  const double* d = c->dp;
  int square = c->ip[0], wl_distr = c->ip[1];
  double width = d[0], height = d[1], radius = d[2];
  double Lambda0 = d[3], dLambda = d[4], E0 = d[5], dE = d[6];
  double xw = d[7], yh = d[8], dist = d[9], pmul = d[10];
  double r1 = rng_uniform(rng), r2 = rng_uniform(rng), r3 = rng_uniform(rng);
  double r4 = rng_uniform(rng), r5 = rng_uniform(rng);
  double x, y;
  if (square) {
    x = width * (r1 - 0.5);
    y = height * (r2 - 0.5);
  } else {
    double chi = 2 * M_PI * r1;
    /* math.sqrt of a float32 uniform: a float32 root under Numba */
    double r = (double)sqrtf((float)r2) * radius;
    x = r * cos(chi);
    y = r * sin(chi);
  }
  n->x = x; n->y = y; n->z = 0.;
  double target[3] = {0.0, 0.0, dist};
  double vec_f[3];
  double solidangle = randvec_target_rect(target, xw, yh, r3, r4, vec_f);
  double dx = vec_f[0] - x, dy = vec_f[1] - y;
  double dist1 = sqrt(dx * dx + dy * dy + dist * dist);
  double v;
  if (wl_distr) {
    double L = Lambda0 + dLambda * (r5 * 2 - 1);
    v = K2V * (2 * M_PI / L);
  } else {
    double E = E0 + dE * (r5 * 2 - 1);
    v = SE2V * sqrt(E);
  }
  n->vx = v * dx / dist1;
  n->vy = v * dy / dist1;
  n->vz = v * dist / dist1;
  n->sx = 0; n->sy = 0;
  n->t = 0;
  n->p = pmul * solidangle;
}

/* -------------------------------------------------------------- guide */
/* ------------------------------------------------ SNS moderator source */
/* SNS_source (acc/components/sources/SNS_source.py:20-207).  Table
 * (float64): Es[nE], Pvec[nE], ts[nt], Ptmat[nE][nt]; ip: 0 square 1 nE
 * 2 nt 3 Eidx_start 4 Eidx_stop 5 tidx_start 6 tidx_stop; dp: 0 xwidth
 * 1 yheight 2 radius 3 focus_xw 4 focus_yh 5 dist 6 EPmin 7 EPmax 8 prob.
 * The two loops of zero_find, unbounded in the reference, stop after
 * SNS_EXPAND_MAX / SNS_BISECT_MAX passes (the GPU kernels use the same
 * caps). */
#define SNS_EXPAND_MAX 64
#define SNS_BISECT_MAX 200

/* a row of values: a table column, or P(t) interpolated between two E
 * rows at weight wl (generate, :44-47) */
typedef struct {
  const double* a;
  const double* b; /* NULL: plain column */
  double wl;
} snsvec_t;

static inline double snsvec_at(const snsvec_t* v, int i) {
  return v->b ? v->a[i] * v->wl + v->b[i] * (1 - v->wl) : v->a[i];
}

/* quadint (:59-64) */
static double sns_quadint(double xdes, double x1, double x2, double x3,
                          double y1, double y2, double y3) {
  double t1 = ((xdes - x2) * (xdes - x3) * y1) / ((x1 - x2) * (x1 - x3));
  double t2 = ((xdes - x1) * (xdes - x3) * y2) / ((x2 - x1) * (x2 - x3));
  double t3 = ((xdes - x1) * (xdes - x2) * y3) / ((x3 - x1) * (x3 - x2));
  return t1 + t2 + t3;
}

/* quadfuncint (:66-75).  Past the last point the reference reads beyond
 * the array (undefined); here the last bracket extrapolates.  Index -1
 * wraps to the last point, as numba indexes. */
static double sns_quadfuncint(double xdes, int xylen, const double* vecx,
                              const snsvec_t* vecy) {
  int idx = 1;
  while (idx < xylen && vecx[idx] < xdes) idx += 1;
  if (idx >= xylen) idx = xylen - 1;
  if (vecx[idx] == xdes) return snsvec_at(vecy, idx);
  int i0 = idx - 2 < 0 ? idx - 2 + xylen : idx - 2;
  return sns_quadint(xdes, vecx[i0], vecx[idx - 1], vecx[idx],
                     snsvec_at(vecy, i0), snsvec_at(vecy, idx - 1),
                     snsvec_at(vecy, idx));
}

/* zero_find (:78-96) */
static double sns_zero_find(const double* vecx, int len,
                            const snsvec_t* vecy, double yval, double xmin,
                            double xmax, double tol) {
  double xl = xmin;
  double xh = pow(10, (log10(xmin) + yval * (log10(xmax) - log10(xmin))));
  double f = sns_quadfuncint(xl, len, vecx, vecy) - yval;
  double fmid = sns_quadfuncint(xh, len, vecx, vecy) - yval;
  for (int k = 0; k < SNS_EXPAND_MAX && fmid * f >= 0.0; ++k) {
    xh = xh + (xh - xl) * 2.0;
    fmid = sns_quadfuncint(xh, len, vecx, vecy) - yval;
  }
  double dx = xh - xl, rtb = xl;
  for (int k = 0; k < SNS_BISECT_MAX &&
                  fabs(sns_quadfuncint(rtb, len, vecx, vecy) - yval) > tol;
       ++k) {
    dx = dx * 0.5;
    double xmid = rtb + dx;
    fmid = sns_quadfuncint(xmid, len, vecx, vecy) - yval;
    if (fmid < 0) rtb = xmid;
  }
  return rtb;
}

/* generate (:22-54): E (meV) and t (s) from two uniforms */
static void sns_generate(const mcv_component* c, double randE, double randt,
                         double* Eout, double* tout) {
  const int nE = c->ip[1], nt = c->ip[2];
  const int Eidx_start = c->ip[3], Eidx_stop = c->ip[4];
  const int tidx_start = c->ip[5], tidx_stop = c->ip[6];
  const double* Es = (const double*)c->table;
  const double* Pvec = Es + nE;
  const double* ts = Pvec + nE;
  const double* Ptmat = ts + nt;
  const double EPmin = c->dp[6], EPmax = c->dp[7];
  double randp = EPmin + randE * (EPmax - EPmin);
  snsvec_t pv = {Pvec, NULL, 0.};
  double Eval = sns_zero_find(Es, nE, &pv, randp, Es[Eidx_start],
                              Es[Eidx_stop], 1e-7);
  int idx1 = 0;
  while (idx1 < nE && Es[idx1] < Eval) idx1 += 1;
  /* the reference's bracket (:38-46) kept in bounds: index -1 wraps to
   * the last energy as numba's indexing does (weight 0 when Eval ==
   * Es[0]); above the last tabulated energy, where the reference reads one
   * row past its table, the last row */
  int Eidxh = idx1, Eidxl = idx1 - 1;
  double wl = 0.0;
  if (idx1 >= nE) {
    Eidxh = nE - 1;
    Eidxl = nE - 1;
  } else {
    if (Eidxl < 0) Eidxl = nE - 1;
    wl = (Es[Eidxh] - Eval) / (Es[Eidxh] - Es[Eidxl]);
  }
  snsvec_t pt = {Ptmat + (size_t)Eidxl * nt, Ptmat + (size_t)Eidxh * nt, wl};
  double p0 = snsvec_at(&pt, tidx_start), p1 = snsvec_at(&pt, tidx_stop - 1);
  randp = p0 + randt * (p1 - p0);
  double tval = 0;
  if (randp > 0.0)
    tval = sns_zero_find(ts, nt, &pt, randp, ts[tidx_start],
                         ts[tidx_stop - 1], 1e-5);
  *Eout = Eval * 1000.0;
  *tout = tval * 1e-6;
}

/* SNS_source.propagate (:157-207) */
static void sns_source(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double randx = rng_uniform(rng), randy = rng_uniform(rng);
  double rand_theta = rng_uniform(rng), rand_phi = rng_uniform(rng);
  double randE = rng_uniform(rng), randt = rng_uniform(rng);
  const double xwidth = c->dp[0], yheight = c->dp[1], radius = c->dp[2];
  const double focus_xw = c->dp[3], focus_yh = c->dp[4], dist = c->dp[5];
  double x, y, z = 0.;
  if (c->ip[7] & 1) {
    /* STS_source.propagate (STS_source.py:242-259) */
    const double tanMOa = c->dp[9], cylx = c->dp[10], cylz = c->dp[11];
    const double cylphi1 = c->dp[12], cylphi2 = c->dp[13];
    const double MR = c->dp[14], MOa = c->dp[15];
    if (c->ip[0]) {
      y = yheight * (randy - 0.5);
      if (c->ip[7] & 2) {
        x = xwidth * (randx - 0.5);
        z = sqrt(MR * MR - (x - cylx) * (x - cylx)) + cylz;
      } else {
        double ang = -cylphi1 + randx * (cylphi1 + cylphi2) + MOa;
        z = cylz + MR * cos(ang);
        x = cylx + MR * sin(ang);
      }
    } else {
      double chi = 2.0 * M_PI * randx,
           r = (double)sqrtf((float)randy) * radius;
      x = r * cos(chi);
      y = r * sin(chi);
      z = tanMOa * x;
    }
  } else if (c->ip[0]) {
    x = xwidth * (randx - 0.5);
    y = yheight * (randy - 0.5);
  } else {
    double chi = 2 * M_PI * randx,
           r = (double)sqrtf((float)randy) * radius;
    x = r * cos(chi);
    y = r * sin(chi);
  }
  double hdivmax = atan((focus_xw / 2.0 - x) / dist);
  double hdivmin = atan(-(focus_xw / 2.0 + x) / dist);
  double vdivmax = atan((focus_yh / 2.0 - y) / dist);
  double vdivmin = atan(-(focus_yh / 2.0 + y) / dist);
  double theta = hdivmin + (hdivmax - hdivmin) * rand_theta;
  double phi = vdivmin + (vdivmax - vdivmin) * rand_phi;
  double E, t;
  sns_generate(c, randE, randt, &E, &t);
  double v = SE2V * sqrt(E);
  n->x = x;
  n->y = y;
  n->z = z;
  n->vx = v * cos(phi) * sin(theta);
  n->vy = v * sin(phi);
  n->vz = v * cos(phi) * cos(theta);
  n->t = t;
  n->p = c->dp[8];
}

/* generate() alone, for tests */
void oracle_sns_generate(const mcv_component* c, double randE, double randt,
                         double* E, double* t) {
  sns_generate(c, randE, randt, E, t);
}

/* calc_reflectivity (acc/components/optics/_guide_utils.py:6-23) */
double oracle_reflectivity(double Q, double R0, double Qc, double alpha,
                           double m, double W) {
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

/* Guide.propagate (acc/components/optics/guide.py:66-162).  Returns 1 if
 * the bounce loop ran out.  *nrefl (if given) = reflections made, -1 when
 * the neutron misses the opening. */
static int guide(neutron_t* n, const mcv_component* c, int* nrefl) {
  const double* d = c->dp;
  double ww = d[0], hh = d[1], hw1 = d[2], hh1 = d[3], l = d[4];
  double R0 = d[5], Qc = d[6], alpha = d[7], m = d[8], W = d[9];
  double x = n->x, y = n->y, z = n->z, vx = n->vx, vy = n->vy, vz = n->vz;
  double t = n->t, prob = n->p;
  double dt = -z / vz;
  x += vx * dt;
  y += vy * dt;
  z = 0.;
  t += dt;
  if (nrefl) *nrefl = -1;
  if (x <= -hw1 || x >= hw1 || y <= -hh1 || y >= hh1) {
    n->p = -1; /* absorb (acc/neutron.py:25-28) */
    return 0;
  }
  int overflow = 1, refl = 0;
  for (int nb = 0; nb < MCV_MAX_BOUNCES; ++nb) {
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
    if (i == 0) { overflow = 0; break; }
    x += vx * t1;
    y += vy * t1;
    z += vz * t1;
    t += t1;
    double nlen2, q, dd;
    if (i == 1) {
      nlen2 = l * l + ww * ww;
      q = V2K * (-2) * vdotn_v1 / sqrt(nlen2);
      dd = 2 * vdotn_v1 / nlen2;
      vx = vx - dd * l;
      vz = vz - dd * ww;
    } else if (i == 2) {
      nlen2 = l * l + ww * ww;
      q = V2K * (-2) * vdotn_v2 / sqrt(nlen2);
      dd = 2 * vdotn_v2 / nlen2;
      vx = vx + dd * l;
      vz = vz - dd * ww;
    } else if (i == 3) {
      nlen2 = l * l + hh * hh;
      q = V2K * (-2) * vdotn_h1 / sqrt(nlen2);
      dd = 2 * vdotn_h1 / nlen2;
      vy = vy - dd * l;
      vz = vz - dd * hh;
    } else {
      nlen2 = l * l + hh * hh;
      q = V2K * (-2) * vdotn_h2 / sqrt(nlen2);
      dd = 2 * vdotn_h2 / nlen2;
      vy = vy + dd * l;
      vz = vz - dd * hh;
    }
    double R = oracle_reflectivity(q, R0, Qc, alpha, m, W);
    prob *= R;
    ++refl;
    if (prob <= 0) { overflow = 0; break; }
  }
  if (nrefl) *nrefl = refl;
  n->x = x; n->y = y; n->z = z;
  n->vx = vx; n->vy = vy; n->vz = vz;
  n->t = t;
  n->p = prob;
  return overflow;
}

/* guide_tapering.Guide.propagate
 * (acc/components/optics/guide_tapering.py:140-291): nseg equal segments,
 * each a tapered channel; table rows w1 w2 h1 h2 ww hh whalf hhalf lwhalf
 * lhhalf (float64, nseg each).  Returns 1 if a bounce loop ran out. */
/* inside_convex_polygon (acc/components/optics/geometry2d.py:12-33) */
static int inside_convex_polygon(double px, double py, const double* poly,
                                 int nv) {
  double prev = (poly[2] - poly[0]) * (py - poly[1]) -
                (poly[3] - poly[1]) * (px - poly[0]);
  int prev_side = prev <= 0;
  for (int k = 1; k < nv; ++k) {
    int k2 = (k + 1) % nv;
    double ax = poly[2 * k], ay = poly[2 * k + 1];
    double sign = (poly[2 * k2] - ax) * (py - ay) - (poly[2 * k2 + 1] - ay) * (px - ax);
    if (fabs(sign) < 1e-14) continue;
    int side = sign <= 0;
    if (fabs(prev) < 1e-14) {
      prev_side = side;
      continue;
    }
    if (prev_side != side) return 0;
  }
  return 1;
}

/* insert_into_sorted_list_with_indexes (acc/geometry/_utils.py:35-65) */
static int insert_sorted_idx(int index, double d, int* index_list, double* l,
                             int N, int cap) {
  if (N >= cap) return N;
  if (N == 0) {
    l[0] = d;
    index_list[0] = index;
    return 1;
  }
  int minidx = 0, maxidx = N - 1, idx;
  while (minidx < maxidx - 1) {
    int mid = (minidx + maxidx) / 2;
    if (d > l[mid]) minidx = mid;
    else maxidx = mid;
  }
  if (minidx == maxidx) {
    idx = minidx;
    if (d > l[idx]) idx += 1;
  } else {
    if (d >= l[maxidx]) idx = maxidx + 1;
    else if (d <= l[minidx]) idx = minidx;
    else idx = minidx + 1;
  }
  for (int i = N; i > idx; --i) {
    l[i] = l[i - 1];
    index_list[i] = index_list[i - 1];
  }
  l[idx] = d;
  index_list[idx] = index;
  return N + 1;
}

/* Guide_anyshape._propagate (acc/components/optics/guide_anyshape.py:
 * 96-158), in the reference's order: every positive plane hit sorted, the
 * first inside its face taken; the move is written back after the
 * reflectivity (an absorbed neutron keeps its place).  Returns 1 when the
 * bounce limit is reached. */
static int guide_anyshape(neutron_t* n, const mcv_component* c) {
  int nf = c->ip[0], nv = c->ip[1], stride = 12 + 2 * nv;
  const double* F = (const double*)c->table;
  double R0 = c->dp[0], Qc = c->dp[1], alpha = c->dp[2], m = c->dp[3],
         W = c->dp[4];
  double tl[MCV_ANYSHAPE_MAX_FACES + 1];
  int il[MCV_ANYSHAPE_MAX_FACES + 1];
  for (int nb = 0; nb < MCV_ANYSHAPE_MAX_BOUNCES; ++nb) {
    int ninter = 0;
    for (int f = 0; f < nf; ++f) {
      const double* g = F + (size_t)f * stride;
      double dist = (g[0] - n->x) * g[9] + (g[1] - n->y) * g[10] +
                    (g[2] - n->z) * g[11];
      double vn = n->vx * g[9] + n->vy * g[10] + n->vz * g[11];
      double t = dist / vn;
      if (t > 0)
        ninter = insert_sorted_idx(f, t, il, tl, ninter, MCV_ANYSHAPE_MAX_FACES + 1);
    }
    if (!ninter) return 0;
    int found = -1;
    double t = 0;
    for (int k = 0; k < ninter; ++k) {
      const double* g = F + (size_t)il[k] * stride;
      t = tl[k];
      double qx = n->vx * t + n->x - g[0], qy = n->vy * t + n->y - g[1],
             qz = n->vz * t + n->z - g[2];
      double u = qx * g[3] + qy * g[4] + qz * g[5];
      double w = qx * g[6] + qy * g[7] + qz * g[8];
      if (inside_convex_polygon(u, w, g + 12, nv)) {
        found = il[k];
        break;
      }
    }
    if (found < 0) return 0;
    const double* g = F + (size_t)found * stride;
    t -= t * 1e-14;
    double x = n->x + n->vx * t, y = n->y + n->vy * t, z = n->z + n->vz * t;
    double tt = n->t + t;
    double vq = -(n->vx * g[9] + n->vy * g[10] + n->vz * g[11]) * 2;
    double R = oracle_reflectivity(fabs(vq) * V2K, R0, Qc, alpha, m, W);
    double prob = n->p * R;
    if (prob <= 0) {
      n->p = -1;
      return 0;
    }
    n->vx += g[9] * vq;
    n->vy += g[10] * vq;
    n->vz += g[11] * vq;
    n->x = x;
    n->y = y;
    n->z = z;
    n->t = tt;
    n->p = prob;
  }
  return 1;
}

/* intersect_plane of guide_anyshape_gravity.py:25-41: the roots of
 * A t^2 + B t + C = 0, A = g.n / 2, B = v.n, C = r.n - c.n */
static void gravity_roots(const double* r, const double* v, const double* g,
                          const double* c, const double* nrm, double* out) {
  double A = (g[0] * nrm[0] + g[1] * nrm[1] + g[2] * nrm[2]) / 2;
  double B = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2];
  double C = (r[0] * nrm[0] + r[1] * nrm[1] + r[2] * nrm[2]) -
             (c[0] * nrm[0] + c[1] * nrm[1] + c[2] * nrm[2]);
  if (fabs(A) < 1e-10) {
    out[0] = -C / B;
    out[1] = -1;
    return;
  }
  double d = B * B - 4 * A * C;
  if (d < 0) {
    out[0] = out[1] = -1;
    return;
  }
  double s = sqrt(d);
  out[0] = (-B - s) / 2 / A;
  out[1] = (-B + s) / 2 / A;
}

/* propagate_with_gravity (:43-55) */
static void gravity_move(const double* r, const double* v, const double* g,
                         double t, double* r2, double* v2) {
  double tmp[3];
  for (int k = 0; k < 3; ++k) v2[k] = v[k] + g[k] * t;
  for (int k = 0; k < 3; ++k) tmp[k] = (v[k] + v2[k]) * (0.5 * t);
  for (int k = 0; k < 3; ++k) r2[k] = r[k] + tmp[k];
}

/* Guide_anyshape_gravity._propagate (:57-182), in the reference's order:
 * both positive roots of every face sorted, the first at or past 1e-10 s
 * inside its face taken; then the carry to z = z_max (without advancing
 * the time; the first root also when only the second is positive, as the
 * reference has it) */
static int guide_anyshape_gravity(neutron_t* n, const mcv_component* c) {
  int nf = c->ip[0], nv = c->ip[1], stride = 12 + 2 * nv;
  const double* F = (const double*)c->table;
  double R0 = c->dp[0], Qc = c->dp[1], alpha = c->dp[2], m = c->dp[3],
         W = c->dp[4];
  double g[3] = {c->dp[5], c->dp[6], c->dp[7]}, zmax = c->dp[8];
  double tl[MCV_ANYSHAPE_MAX_FACES + 1];
  int il[MCV_ANYSHAPE_MAX_FACES + 1];
  int overflow = 1;
  for (int nb = 0; nb < MCV_ANYSHAPE_MAX_BOUNCES; ++nb) {
    double r[3] = {n->x, n->y, n->z}, v[3] = {n->vx, n->vy, n->vz};
    int ninter = 0;
    for (int f = 0; f < nf; ++f) {
      const double* gf = F + (size_t)f * stride;
      double roots[2];
      gravity_roots(r, v, g, gf, gf + 9, roots);
      /* the reference's list holds 100 entries (max_numfaces, :240); a
       * root that finds it full is dropped */
      if (roots[0] > 0)
        ninter = insert_sorted_idx(f, roots[0], il, tl, ninter, MCV_ANYSHAPE_MAX_FACES + 1);
      if (roots[1] > 0)
        ninter = insert_sorted_idx(f, roots[1], il, tl, ninter, MCV_ANYSHAPE_MAX_FACES + 1);
    }
    if (!ninter) { overflow = 0; break; }
    int found = -1;
    double t = 0, r2[3], v2[3];
    for (int k = 0; k < ninter; ++k) {
      const double* gf = F + (size_t)il[k] * stride;
      t = tl[k];
      gravity_move(r, v, g, t, r2, v2);
      if (t < 1e-10) continue;
      double q[3] = {r2[0] - gf[0], r2[1] - gf[1], r2[2] - gf[2]};
      double u = q[0] * gf[3] + q[1] * gf[4] + q[2] * gf[5];
      double w = q[0] * gf[6] + q[1] * gf[7] + q[2] * gf[8];
      if (inside_convex_polygon(u, w, gf + 12, nv)) { found = il[k]; break; }
    }
    if (found < 0) { overflow = 0; break; }
    const double* gf = F + (size_t)found * stride;
    n->t += t;
    n->x = r2[0]; n->y = r2[1]; n->z = r2[2];
    n->vx = v2[0]; n->vy = v2[1]; n->vz = v2[2];
    double vq = -(v2[0] * gf[9] + v2[1] * gf[10] + v2[2] * gf[11]) * 2;
    double R = oracle_reflectivity(fabs(vq) * V2K, R0, Qc, alpha, m, W);
    double prob = n->p * R;
    if (prob <= 0) { n->p = -1; return 0; }
    n->vx += gf[9] * vq;
    n->vy += gf[10] * vq;
    n->vz += gf[11] * vq;
    n->p = prob;
  }
  if (n->z < zmax) {
    double r[3] = {n->x, n->y, n->z}, v[3] = {n->vx, n->vy, n->vz};
    double cz[3] = {0, 0, zmax}, nz[3] = {0, 0, 1}, roots[2], r2[3], v2[3];
    gravity_roots(r, v, g, cz, nz, roots);
    double t;
    if (roots[0] > 0) t = roots[0];
    else if (roots[1] > 0) t = roots[0];
    else return overflow;
    gravity_move(r, v, g, t, r2, v2);
    n->x = r2[0]; n->y = r2[1]; n->z = r2[2];
    n->vx = v2[0]; n->vy = v2[1]; n->vz = v2[2];
  }
  return overflow;
}

static int guide_tapering(neutron_t* n, const mcv_component* c) {
  const int nseg = c->ip[0];
  const double* d = (const double*)c->table;
  const double *w1 = d, *hh = d + 5 * nseg, *ww = d + 4 * nseg,
               *whalf = d + 6 * nseg, *hhalf = d + 7 * nseg, *h1 = d + 2 * nseg;
  const double l_seg = c->dp[0], R0 = c->dp[1], Qcx = c->dp[2],
               Qcy = c->dp[3], alphax = c->dp[4], alphay = c->dp[5],
               mx = c->dp[6], my = c->dp[7], W = c->dp[8];
  double x = n->x, y = n->y, z = n->z, vx = n->vx, vy = n->vy, vz = n->vz;
  double t = n->t, prob = n->p;
  /* propagate to z=0 (:163-167) */
  double dt = -z / vz;
  x += vx * dt;
  y += vy * dt;
  z = 0.0;
  t += dt;
  int overflow = 0;
  for (int seg = 0; seg < nseg; ++seg) {
    double zr = seg * l_seg;
    /* propagate to segment entrance (:171-175) */
    dt = (zr - z) / vz;
    x += vx * dt;
    y += vy * dt;
    z += vz * dt;
    if (x <= -0.5 * w1[seg] || x >= 0.5 * w1[seg] || y <= -hhalf[seg] ||
        y >= hhalf[seg]) {
      n->p = 0;
      return 0;
    }
    /* shift origin to center of channel hit (:180-186) */
    x += 0.5 * w1[seg];
    double edge = floor(x / w1[seg]) * w1[seg];
    if (x - edge > w1[seg]) {
      n->p = 0;
      return 0;
    }
    x -= (edge + 0.5 * w1[seg]);
    double hadj = edge + (0.5 * w1[seg]) - 0.5 * w1[seg];
    int nb;
    for (nb = 0; nb < MCV_MAX_BOUNCES; ++nb) {
      double av = l_seg * vx, bv = ww[seg] * vz;
      double ah = l_seg * vy, bh = hh[seg] * vz;
      double vdotn_v1 = bv + av, vdotn_v2 = bv - av;
      double vdotn_h1 = bh + ah, vdotn_h2 = bh - ah;
      double cv1 = -whalf[seg] * l_seg - (z - zr) * ww[seg], cv2 = x * l_seg;
      double ch1 = -hhalf[seg] * l_seg - (z - zr) * hh[seg], ch2 = y * l_seg;
      double t1 = (zr + l_seg - z) / vz, t2;
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
      if (i == 0) break; /* left the segment */
      x += vx * t1;
      y += vy * t1;
      z += vz * t1;
      t += t1;
      double nlen2, q, dd;
      if (i == 1) {
        nlen2 = l_seg * l_seg + ww[seg] * ww[seg];
        q = V2K * (-2.0) * vdotn_v1 / sqrt(nlen2);
        dd = 2.0 * vdotn_v1 / nlen2;
        vx = vx - dd * l_seg;
        vz = vz - dd * ww[seg];
      } else if (i == 2) {
        nlen2 = l_seg * l_seg + ww[seg] * ww[seg];
        q = V2K * (-2.0) * vdotn_v2 / sqrt(nlen2);
        dd = 2.0 * vdotn_v2 / nlen2;
        vx = vx + dd * l_seg;
        vz = vz - dd * ww[seg];
      } else if (i == 3) {
        nlen2 = l_seg * l_seg + hh[seg] * hh[seg];
        q = V2K * (-2.0) * vdotn_h1 / sqrt(nlen2);
        dd = 2.0 * vdotn_h1 / nlen2;
        vy = vy - dd * l_seg;
        vz = vz - dd * hh[seg];
      } else {
        nlen2 = l_seg * l_seg + hh[seg] * hh[seg];
        q = V2K * (-2.0) * vdotn_h2 / sqrt(nlen2);
        dd = 2.0 * vdotn_h2 / nlen2;
        vy = vy + dd * l_seg;
        vz = vz - dd * hh[seg];
      }
      /* an m = 0 mirror ends the segment's loop (:256-258) */
      if ((i <= 2 && mx == 0) || (i > 2 && my == 0)) {
        x += hadj;
        break;
      }
      double m, R;
      if (i <= 2) {
        m = mx;
        if (m <= 0.0) m = fabs(mx * w1[0] / w1[seg]);
        R = oracle_reflectivity(q, R0, Qcx, alphax, m, W);
      } else {
        m = my;
        if (m <= 0.0) m = fabs(my * h1[0] / h1[seg]);
        R = oracle_reflectivity(q, R0, Qcy, alphay, m, W);
      }
      if (R > 1e-10) {
        prob *= R;
      } else {
        n->p = 0;
        return 0;
      }
    }
    if (nb == MCV_MAX_BOUNCES) overflow = 1;
    x += hadj;
  }
  n->x = x; n->y = y; n->z = z;
  n->vx = vx; n->vy = vy; n->vz = vz;
  n->t = t;
  n->p = prob;
  return overflow;
}

/* Slit.propagate / Beamstop.propagate (acc/components/optics/slit.py:71-108,
 * beamstop.py:75-112); dp = {xmin, xmax, ymin, ymax, radius^2, cut} */
static void slit_or_beamstop(neutron_t* n, const mcv_component* c, int stop) {
  const double* d = c->dp;
  double xmin = d[0], xmax = d[1], ymin = d[2], ymax = d[3], r2 = d[4],
         cut = d[5];
  double x = n->x, y = n->y, z = n->z, vx = n->vx, vy = n->vy, vz = n->vz;
  if ((z < 0 && vz <= 0) || (z > 0 && vz >= 0)) return;
  double t = n->t;
  if (n->p < cut) { n->p = -1; return; }
  if (z != 0) {
    double dt = -z / vz;
    x += vx * dt;
    y += vy * dt;
    t += dt;
  }
  int in;
  if (r2 != 0) in = x * x + y * y <= r2;
  else in = xmin <= x && x <= xmax && ymin <= y && y <= ymax;
  if (stop ? in : !in) { n->p = -1; return; }
  n->x = x;
  n->y = y;
  n->z = 0.;
  n->t = t;
}

/* ------------------------------------------------------------ geometry */
/* cu_device_intersect_sphere (acc/geometry/arrow_intersect.py:154-168) */
void oracle_intersect_sphere(double x, double y, double z, double vx,
                             double vy, double vz, double R, double* t1,
                             double* t2) {
  double r0dotv = x * vx + y * vy + z * vz;
  double cx = y * vz - z * vy, cy = z * vx - x * vz, cz = x * vy - y * vx;
  double v2 = vx * vx + vy * vy + vz * vz;
  double r0Xv2 = cx * cx + cy * cy + cz * cz;
  double b2m4ac = v2 * R * R - r0Xv2;
  *t1 = NAN;
  *t2 = NAN;
  if (b2m4ac < 0) return;
  double s = sqrt(b2m4ac);
  *t1 = -(r0dotv + s) / v2;
  *t2 = -(r0dotv - s) / v2;
}

/* intersectCylinderSide (arrow_intersect.py:178-204) */
static int cyl_side(double x, double y, double z, double vx, double vy,
                    double vz, double R, double H, double* t1o, double* t2o) {
  double a = vx * vx + vy * vy;
  double b = x * vx + y * vy;
  double c = x * x + y * y - R * R;
  double k = b * b - a * c;
  double hh = H / 2.;
  *t1o = NAN;
  *t2o = NAN;
  if (k < 0 || a == 0) return 0;
  if (k == 0) {
    double t = -b / a;
    if (fabs(z + vz * t) < hh) {
      *t1o = t;
      return 1;
    }
  }
  k = sqrt(k);
  double t1 = (-b + k) / a, t2 = (-b - k) / a;
  int good1 = fabs(z + vz * t1) < hh, good2 = fabs(z + vz * t2) < hh;
  if (good1) {
    if (good2) { *t1o = t2; *t2o = t1; return 2; }
    *t1o = t1;
    return 1;
  }
  if (good2) { *t1o = t2; return 1; }
  return 0;
}

/* intersectCylinderTopBottom (arrow_intersect.py:213-239) */
static int cyl_caps(double x, double y, double z, double vx, double vy,
                    double vz, double R, double H, double* t1o, double* t2o) {
  *t1o = NAN;
  *t2o = NAN;
  if (vz == 0) return 0;
  double hh = H / 2, r2 = R * R;
  double t1 = (hh - z) / vz;
  double x1 = x + vx * t1, y1 = y + vy * t1;
  int good1 = x1 * x1 + y1 * y1 <= r2;
  double t2 = (-hh - z) / vz;
  x1 = x + vx * t2;
  y1 = y + vy * t2;
  int good2 = x1 * x1 + y1 * y1 <= r2;
  if (good1) {
    if (good2) {
      if (t1 < t2) { *t1o = t1; *t2o = t2; }
      else { *t1o = t2; *t2o = t1; }
      return 2;
    }
    *t1o = t1;
    return 1;
  }
  if (good2) { *t1o = t2; return 1; }
  return 0;
}

static inline double pymin(double a, double b) { return b < a ? b : a; }
static inline double pymax(double a, double b) { return b > a ? b : a; }

/* cu_device_intersect_cylinder (arrow_intersect.py:241-267); the n==0
 * branch of the reference falls through to NaNs, i.e. no intersection. */
void oracle_intersect_cylinder(double x, double y, double z, double vx,
                               double vy, double vz, double R, double H,
                               double* o1, double* o2) {
  double t1, t2, t3, t4;
  int n1 = cyl_side(x, y, z, vx, vy, vz, R, H, &t1, &t2);
  int n2 = cyl_caps(x, y, z, vx, vy, vz, R, H, &t3, &t4);
  int n = n1 + n2;
  if (n == 0) { *o1 = NAN; *o2 = NAN; }
  else if (n == 1) {
    if (n1 == 1) { *o1 = t1; *o2 = t1; }
    else { *o1 = t3; *o2 = t3; }
  } else if (n == 2) {
    if (n1 == 1) {
      if (t1 > t3) { *o1 = t3; *o2 = t1; }
      else { *o1 = t1; *o2 = t3; }
    } else if (n1 == 0) { *o1 = t3; *o2 = t4; }
    else { *o1 = t1; *o2 = t2; }
  } else if (n == 3) {
    if (n1 == 1) { *o1 = pymin(t1, t3); *o2 = pymax(t1, t4); }
    else { *o1 = pymin(t3, t1); *o2 = pymax(t3, t2); }
  } else {
    *o1 = pymin(t1, t3);
    *o2 = pymax(t2, t4);
  }
}

/* cu_device_intersect_rectangle (acc/geometry/onbox.py:8-18): the plane
 * z = 0 of a frame where the rectangle is X x Y.  The reference declares it
 * float32; restated in float64 like its CUDASIM known-answer tests. */
static double rect_hit(double rx, double ry, double rz, double vx, double vy,
                       double vz, double X, double Y) {
  double t = -rz / vz;
  double r1x = rx + vx * t, r1y = ry + vy * t;
  if (fabs(r1x) > X / 2 || fabs(r1y) > Y / 2) t = NAN;
  return t;
}

/* cu_device_update_intersections (onbox.py:20-36) */
static void update_hits(double* t1, double* t2, double t) {
  if (!isfinite(t)) return;
  if (!isfinite(*t1)) { *t1 = t; return; }
  if (!isfinite(*t2)) {
    if (t > *t1) *t2 = t;
    else { *t2 = *t1; *t1 = t; }
    return;
  }
  if (t < *t1) *t1 = t;
  else if (t < *t2) return;
  else *t2 = t;
}

/* cu_device_intersect_box (onbox.py:38-56) */
void oracle_intersect_box(double x, double y, double z, double vx, double vy,
                          double vz, double X, double Y, double Z, double* o1,
                          double* o2) {
  double t1 = NAN, t2 = NAN;
  if (vz != 0) {
    update_hits(&t1, &t2, rect_hit(x, y, z - Z / 2, vx, vy, vz, X, Y));
    update_hits(&t1, &t2, rect_hit(x, y, z + Z / 2, vx, vy, vz, X, Y));
  }
  if (vx != 0) {
    update_hits(&t1, &t2, rect_hit(y, z, x - X / 2, vy, vz, vx, Y, Z));
    update_hits(&t1, &t2, rect_hit(y, z, x + X / 2, vy, vz, vx, Y, Z));
  }
  if (vy != 0) {
    update_hits(&t1, &t2, rect_hit(z, x, y - Y / 2, vz, vx, vy, Z, X));
    update_hits(&t1, &t2, rect_hit(z, x, y + Y / 2, vz, vx, vy, Z, X));
  }
  *o1 = t1;
  *o2 = t2;
}

/* locate functions (acc/geometry/locate.py:354-392) */
static int locate_prim(int kind, const double* p, double x, double y,
                       double z) {
  const double e = GEOM_EPSILON;
  if (kind == MCV_SHAPE_SPHERE) {
    double R = p[0], d2 = x * x + y * y + z * z;
    if (d2 > (R + e) * (R + e)) return LOC_OUTSIDE;
    if (d2 < (R - e) * (R - e)) return LOC_INSIDE;
    return LOC_ONBORDER;
  }
  if (kind == MCV_SHAPE_CYLINDER) {
    double R = p[0], H = p[1];
    if (fabs(z) - H / 2. > e) return LOC_OUTSIDE;
    double r2 = x * x + y * y;
    if (r2 > (R + e) * (R + e)) return LOC_OUTSIDE;
    if (H / 2. - fabs(z) > e && r2 < (R - e) * (R - e)) return LOC_INSIDE;
    return LOC_ONBORDER;
  }
  if (kind == MCV_SHAPE_BOX) {
    double W = p[0], H = p[1], D = p[2];
    if (fabs(x) - 0.5 * W > e) return LOC_OUTSIDE;
    if (fabs(y) - 0.5 * H > e) return LOC_OUTSIDE;
    if (fabs(z) - 0.5 * D > e) return LOC_OUTSIDE;
    if (-0.5 * W < x && x < 0.5 * W && -0.5 * H < y && y < 0.5 * H &&
        -0.5 * D < z && z < 0.5 * D)
      return LOC_INSIDE;
    return LOC_ONBORDER;
  }
  return LOC_OUTSIDE;
}

/* locate wrt the HSS shape: primitive, difference (locate.py:395-404),
 * union (:338-352), intersection (:407-421). */
int oracle_locate(const mcv_component* c, double x, double y, double z) {
  int op = c->ip[0];
  int l1 = locate_prim(c->ip[2], c->dp + 0, x, y, z);
  if (op == MCV_CSG_PRIMITIVE) return l1;
  int l2 = locate_prim(c->ip[3], c->dp + 4, x, y, z);
  if (op == MCV_CSG_DIFFERENCE) {
    if (l1 == LOC_OUTSIDE || l2 == LOC_INSIDE) return LOC_OUTSIDE;
    if (l1 == LOC_ONBORDER || l2 == LOC_ONBORDER) return LOC_ONBORDER;
    return LOC_INSIDE;
  }
  if (op == MCV_CSG_UNION) {
    if (l1 == LOC_INSIDE || l2 == LOC_INSIDE) return LOC_INSIDE;
    if (l1 == LOC_OUTSIDE && l2 == LOC_OUTSIDE) return LOC_OUTSIDE;
    return LOC_ONBORDER;
  }
  /* intersection */
  if (l1 == LOC_OUTSIDE || l2 == LOC_OUTSIDE) return LOC_OUTSIDE;
  if (l1 == LOC_INSIDE && l2 == LOC_INSIDE) return LOC_INSIDE;
  return LOC_ONBORDER;
}

/* insert_into_sorted_list (acc/geometry/_utils.py:4-32), capacity len */
int oracle_insert_sorted(double d, double* l, int N, int len) {
  if (N >= len) return N;
  if (N == 0) { l[0] = d; return 1; }
  int minidx = 0, maxidx = N - 1, idx = minidx;
  while (minidx < maxidx - 1) {
    int mididx = (minidx + maxidx) / 2;
    double mid = l[mididx];
    if (d > mid) minidx = mididx;
    else maxidx = mididx;
  }
  if (minidx == maxidx) {
    idx = minidx;
    if (d > l[idx]) idx = idx + 1;
  } else {
    if (d >= l[maxidx]) idx = maxidx + 1;
    else if (d <= l[minidx]) idx = minidx;
    else idx = minidx + 1;
  }
  for (int i = N; i > idx; --i) l[i] = l[i - 1];
  l[idx] = d;
  return N + 1;
}

/* intersect a primitive: the intersectSphere/Cylinder/Block wrappers of
 * ArrowIntersectFuncFactory (arrow_intersect.py:47-86) */
static int intersect_prim(int kind, const double* p, double x, double y,
                          double z, double vx, double vy, double vz,
                          double* ts) {
  double t1, t2;
  if (kind == MCV_SHAPE_SPHERE)
    oracle_intersect_sphere(x, y, z, vx, vy, vz, p[0], &t1, &t2);
  else if (kind == MCV_SHAPE_CYLINDER)
    oracle_intersect_cylinder(x, y, z, vx, vy, vz, p[0], p[1], &t1, &t2);
  else if (kind == MCV_SHAPE_BOX)
    oracle_intersect_box(x, y, z, vx, vy, vz, p[0], p[1], p[2], &t1, &t2);
  else
    return 0;
  if (isnan(t1)) return 0;
  ts[0] = t1;
  ts[1] = t2;
  return 2;
}

/* intersect the HSS shape; composite per intersectComposite
 * (arrow_intersect.py:126-142) */
int oracle_intersect(const mcv_component* c, double x, double y, double z,
                     double vx, double vy, double vz, double* ts) {
  int op = c->ip[0];
  if (op == MCV_CSG_PRIMITIVE)
    return intersect_prim(c->ip[2], c->dp + 0, x, y, z, vx, vy, vz, ts);
  double ts1[MCV_MAX_INTERSECTIONS], ts2[MCV_MAX_INTERSECTIONS];
  int N1 = intersect_prim(c->ip[2], c->dp + 0, x, y, z, vx, vy, vz, ts1);
  int N2 = intersect_prim(c->ip[3], c->dp + 4, x, y, z, vx, vy, vz, ts2);
  int N = 0;
  for (int i = 0; i < N1; ++i) {
    double t = ts1[i];
    if (oracle_locate(c, x + vx * t, y + vy * t, z + vz * t) == LOC_ONBORDER) {
      ts[N] = t;
      N += 1;
    }
  }
  for (int i = 0; i < N2; ++i) {
    double t = ts2[i];
    if (oracle_locate(c, x + vx * t, y + vy * t, z + vz * t) == LOC_ONBORDER) {
      if (N < MCV_MAX_INTERSECTIONS) ts[N] = t;
      N = oracle_insert_sorted(t, ts, N, MCV_MAX_INTERSECTIONS);
    }
  }
  return N;
}

/* ---------------------------------------- propagation helpers (KATs) */
/* forward_intersect (acc/geometry/propagation.py:11-22) */
static int forward_intersect(const mcv_component* c, const neutron_t* n,
                             double* ts) {
  int N = oracle_intersect(c, n->x, n->y, n->z, n->vx, n->vy, n->vz, ts);
  int Nm = N;
  for (int i = 0; i < N; ++i)
    if (ts[i] >= 0) { Nm = i; break; }
  int Np = N - Nm;
  for (int i = 0; i < Np; ++i) ts[i] = ts[i + Nm];
  return Np;
}

/* _propagate_out (propagation.py:52-59) */
void oracle_propagate_out(const mcv_component* c, double* st) {
  neutron_t* n = (neutron_t*)st;
  double ts[MCV_MAX_INTERSECTIONS];
  int N = forward_intersect(c, n, ts);
  if (N == 0) return;
  prop_dt(n, ts[N - 1]);
}

/* _tof_before_first_exit (propagation.py:154-191); returns -1 where the
 * reference raises (point outside the shape). */
double oracle_tof_before_first_exit(const mcv_component* c, const double* st) {
  const neutron_t* n = (const neutron_t*)st;
  double ts[MCV_MAX_INTERSECTIONS];
  int loc = oracle_locate(c, n->x, n->y, n->z);
  if (loc == LOC_OUTSIDE) return -1.0;
  int N = forward_intersect(c, n, ts);
  if (N == 0) return 0.;
  if (loc == LOC_INSIDE) return ts[0];
  double t = 0.;
  for (int i = 0; i < N; ++i) {
    double mx = n->x + ts[i] / 2 * n->vx, my = n->y + ts[i] / 2 * n->vy,
           mz = n->z + ts[i] / 2 * n->vz;
    int l1 = oracle_locate(c, mx, my, mz);
    if (l1 == LOC_OUTSIDE) return 0.;
    if (l1 == LOC_INSIDE) { t = ts[i]; break; }
  }
  return t;
}

/* _propagate_to_next_incident_surface (propagation.py:61-105); returns 1
 * where the reference raises (point inside the shape). */
int oracle_propagate_to_next_incident_surface(const mcv_component* c,
                                              double* st) {
  neutron_t* n = (neutron_t*)st;
  double ts[MCV_MAX_INTERSECTIONS];
  int loc = oracle_locate(c, n->x, n->y, n->z);
  if (loc == LOC_INSIDE) return 1;
  int N = forward_intersect(c, n, ts);
  if (N == 0) return 0;
  double t;
  if (loc == LOC_OUTSIDE) t = ts[0];
  else {
    int found = 0;
    for (int i = 0; i < N; ++i) {
      double mx = n->x + ts[i] / 2 * n->vx, my = n->y + ts[i] / 2 * n->vy,
             mz = n->z + ts[i] / 2 * n->vz;
      int l1 = oracle_locate(c, mx, my, mz);
      if (l1 == LOC_INSIDE) return 0;
      if (l1 == LOC_OUTSIDE) { t = ts[i]; found = 1; break; }
    }
    if (!found) return 0;
  }
  prop_dt(n, t);
  return 0;
}

/* _propagate_to_next_exiting_surface (propagation.py:107-152) */
void oracle_propagate_to_next_exiting_surface(const mcv_component* c,
                                              double* st) {
  neutron_t* n = (neutron_t*)st;
  double ts[MCV_MAX_INTERSECTIONS];
  int loc = oracle_locate(c, n->x, n->y, n->z);
  double t;
  if (loc == LOC_INSIDE) {
    forward_intersect(c, n, ts);
    t = ts[0];
  } else {
    if (loc == LOC_OUTSIDE) oracle_propagate_to_next_incident_surface(c, st);
    int N = forward_intersect(c, n, ts);
    int found = 0;
    for (int i = 0; i < N; ++i) {
      double mx = n->x + ts[i] / 2 * n->vx, my = n->y + ts[i] / 2 * n->vy,
             mz = n->z + ts[i] / 2 * n->vz;
      int l1 = oracle_locate(c, mx, my, mz);
      if (l1 == LOC_OUTSIDE) return;
      if (l1 == LOC_INSIDE) { t = ts[i]; found = 1; break; }
    }
    if (!found) return;
  }
  prop_dt(n, t);
}

/* -------------------------------------------------------- HSS helpers */
/* _calc_time_to_point_of_scattering_impl
 * (acc/components/samples/homogeneous_single_scatterer.py:121-159).
 * out = {total_time_in_shape, total_time_travel_to_scattering_point,
 *        time_travelled_in_shape_to_scattering_point} */
void oracle_time_to_scatter(const double* ts, int ninter, double rand,
                            double* out) {
  double tps[MCV_MAX_INTERSECTIONS], tpg[MCV_MAX_INTERSECTIONS];
  double T = 0.0;
  int sign = 0, ip = 0, i = 0;
  for (i = 0; i < ninter; ++i) {
    double t = ts[i];
    if (t < 0) continue;
    if (sign == 0) sign = (i % 2 == 0) ? -1 : 1;
    else sign *= -1;
    T += sign * t;
    if (sign > 0) {
      tps[ip] = T;
      tpg[ip] = t;
      ip += 1;
    }
  }
  double ttistsp = rand * T;
  if (ip > 0) {
    for (i = 0; i < ip; ++i)
      if (ttistsp < tps[i]) break;
    if (i == ip) i = ip - 1; /* python for-loop variable keeps its last value */
  } else {
    i = -1;
  }
  out[0] = T;
  out[1] = i >= 0 ? ttistsp - tps[i] + tpg[i] : 0.0;
  out[2] = ttistsp;
}

/* total_time_in_shape (homogeneous_single_scatterer.py:161-178) */
double oracle_total_time_in_shape(const double* ts, int ninter) {
  double T = 0;
  int sign = 0;
  for (int i = 0; i < ninter; ++i) {
    double t = ts[i];
    if (t < 0) continue;
    if (sign == 0) sign = (i % 2 == 0) ? -1 : 1;
    else sign *= -1;
    T += sign * t;
  }
  return T;
}

/* time_to_enter (homogeneous_single_scatterer.py:180-195) */
double oracle_time_to_enter(const double* ts, int ninter) {
  for (int i = 0; i < ninter; ++i) {
    double t = ts[i];
    if (t < 0) continue;
    return (i % 2 == 0) ? t : 0;
  }
  return 0;
}

/* ------------------------------------------------------------ kernels */
/* calc_absorption_coeff (acc/kernels/__init__.py:156-161) */
static inline double abs_coeff(const neutron_t* n, double mu) {
  double v = length3(n->vx, n->vy, n->vz);
  return mu / v * 2200;
}

/* isotropic.S (acc/kernels/isotropic.py:5-21) */
static void isotropic_S(neutron_t* n, rng_t* rng) {
  double cos_t = rng_uniform(rng) * 2 - 1;
  double phi = rng_uniform(rng) * (2 * M_PI);
  if (cos_t > 1) cos_t = 1;
  double sin_t = sqrt(1 - cos_t * cos_t);
  double sin_p = sin(phi), cos_p = cos(phi);
  double vi = length3(n->vx, n->vy, n->vz);
  n->vx = vi * sin_t * cos_p;
  n->vy = vi * sin_t * sin_p;
  n->vz = vi * cos_t;
}

/* powderdiffr.scattering_xs / scattering_coefficient
 * (acc/kernels/powderdiffr.py:10-25); peaks = npeaks x {q_v, w_v, my_s_v2,
 * cumulative my_s_v2} */
static double powder_coeff(const neutron_t* n, const mcv_component* c) {
  const double* pk = (const double*)c->table;
  int Np = c->ip[4];
  double vl = length3(n->vx, n->vy, n->vz);
  double xs_v2 = 0.0;
  for (int i = 0; i < Np; ++i)
    if (vl >= pk[4 * i + 0] / 2) xs_v2 += pk[4 * i + 2];
  return xs_v2 / (vl * vl) / c->dp[10];
}

/* powderdiffr.scatter (acc/kernels/powderdiffr.py:27-109) */
static void powder_scatter(neutron_t* n, rng_t* rng, const mcv_component* c) {
  const double* pk = (const double*)c->table;
  int Npeaks = c->ip[4];
  double ucvol = c->dp[10], d_phi = c->dp[11];
  const double eps = 1e-7, DEG2RAD = M_PI / 180.0;
  double v[3] = {n->vx, n->vy, n->vz};
  double vl = length3(v[0], v[1], v[2]);
  if (vl < pk[0] / 2) { n->p = -1; return; }
  /* `for peakindex in range(1, Npeaks): if vl < q_v[peakindex]/2: break`
   * then `Npeaks = peakindex`: with a break the reachable count is the
   * breaking index; without one python leaves the loop variable at
   * Npeaks-1, so the last peak is never picked (reference quirk).  A single
   * peak leaves the variable unbound in the reference; it counts as 1. */
  int Nreach;
  if (Npeaks <= 1) {
    Nreach = 1;
  } else {
    int j;
    for (j = 1; j < Npeaks; ++j)
      if (vl < pk[4 * j] / 2) break;
    Nreach = j < Npeaks ? j : Npeaks - 1;
  }
  int peakindex;
  if (Nreach > 1) peakindex = (int)(rng_uniform(rng) * Nreach);
  else peakindex = 0;
  double rt = rng_uniform(rng) * 2 - 1;
  double q = pk[4 * peakindex], w = pk[4 * peakindex + 1],
         s = pk[4 * peakindex + 2];
  double arg = q * (1 + w * rt) / (2.0 * vl);
  double scatter_xs = s / (vl * vl);
  scatter_xs *= Nreach;
  double theta = asin(arg);
  double alpha = 0, alpha0;
  if (d_phi != 0) {
    double a = sin(d_phi * DEG2RAD / 2) / sin(2 * theta);
    if (a < -1 || a > 1) d_phi = 0;
    else alpha = 2 * asin(a);
  }
  if (d_phi != 0) {
    alpha = fabs(alpha);
    double r = rng_uniform(rng);
    alpha0 = 2 * r * alpha;
    if (alpha0 > alpha) alpha0 = M_PI + (alpha0 - 1.5 * alpha);
    else alpha0 = alpha0 - 0.5 * alpha;
  } else {
    double r = rng_uniform(rng) * 2 - 1;
    alpha0 = M_PI * r;
  }
  double nn[3];
  if (fabs(v[0]) < fabs(v[2])) { nn[0] = 1; nn[1] = 0; nn[2] = 0; }
  else { nn[0] = 0; nn[1] = 0; nn[2] = 1; }
  double vtmp[3], vout[3] = {v[0], v[1], v[2]};
  cross3(v, nn, vtmp);
  oracle_rotate(vout, vtmp, 2 * theta, eps);
  oracle_rotate(vout, v, alpha0, eps);
  n->vx = vout[0]; n->vy = vout[1]; n->vz = vout[2];
  if (isnan(vout[0]) || isnan(vout[1]) || isnan(vout[2])) { n->p = -1; return; }
  n->p *= scatter_xs / ucvol;
}

/* bilinear_interp (acc/kernels/SANS2D_ongrid.py:16-22) */
static inline double bilinear(double x, double y, double f00, double f01,
                              double f10, double f11) {
  double a00 = f00, a10 = f10 - f00, a01 = f01 - f00,
         a11 = f11 - f10 - f01 + f00;
  return a00 + a10 * x + a01 * y + a11 * x * y;
}

/* Bilinear lookup of the S(Q,E) grid: node (iq, ie) sits at
 * (Qmin + iq dQ, Emin + ie dE), dQ = (Qmax-Qmin)/(nQ-1); indices clamp to
 * [0, n-2] as SANS2D_ongrid.py:37-50 does. */
double oracle_sqe_lookup(const mcv_component* c, double Q, double E) {
  const float* S = (const float*)c->table;
  int nQ = c->ip[4], nE = c->ip[5];
  double Qmin = c->dp[10], Qmax = c->dp[11], Emin = c->dp[12], Emax = c->dp[13];
  double dQ = (Qmax - Qmin) / (nQ - 1), dE = (Emax - Emin) / (nE - 1);
  int iq = (int)((Q - Qmin) / dQ), ie = (int)((E - Emin) / dE);
  if (iq < 0) iq = 0;
  if (ie < 0) ie = 0;
  if (iq > nQ - 2) iq = nQ - 2;
  if (ie > nE - 2) ie = nE - 2;
  double fx = (Q - Qmin) / dQ - iq, fy = (E - Emin) / dE - ie;
  double f00 = S[iq * nE + ie], f10 = S[(iq + 1) * nE + ie];
  double f01 = S[iq * nE + ie + 1], f11 = S[(iq + 1) * nE + ie + 1];
  return bilinear(fx, fy, f00, f01, f10, f11);
}

/* Gridded S(Q,E) kernel.  No reference counterpart: restated from the
 * kinematics of E_Q._S (acc/kernels/E_Q.py:37-99) with (Q, E) drawn
 * uniformly over the table box (one draw each, no rejection loop) and S
 * from the bilinear grid (SANS2D_ongrid.py:16-56).  Weight
 * S (vf/vi) Q (Qmax-Qmin)(Emax-Emin) / (2 ki kf); kinematically closed
 * (Q, E) absorb.  sin(theta) comes from the factored
 * (Q^2 - (ki-kf)^2)((ki+kf)^2 - Q^2) / (2 ki kf)^2 instead of 1 - cos^2. */
static void sqe_scatter(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double Qmin = c->dp[10], Qmax = c->dp[11], Emin = c->dp[12], Emax = c->dp[13];
  double v[3] = {n->vx, n->vy, n->vz};
  double vi = length3(v[0], v[1], v[2]);
  double Ei = vi * vi * VS2E;
  double Q = rng_uniform(rng) * (Qmax - Qmin) + Qmin;
  double E = rng_uniform(rng) * (Emax - Emin) + Emin;
  double phi = rng_uniform(rng) * 2.0 * M_PI;
  double Ef = Ei - E;
  if (Ef <= 0) { n->p = -1; return; }
  double vf = sqrt(Ef) * SE2V;
  double ki = V2K * vi, kf = V2K * vf;
  /* 1 - cos^2 in factored form, well conditioned near 0 and 180 deg */
  double Q2 = Q * Q, dk = ki - kf, sk = ki + kf;
  double sint2 = (Q2 - dk * dk) * (sk * sk - Q2) / (4 * ki * ki * kf * kf);
  if (sint2 < 0) { n->p = -1; return; }
  double cost = (ki * ki + kf * kf - Q2) / (2 * ki * kf);
  double sint = sqrt(sint2);
  double v2 = vf * sint * cos(phi), v3 = vf * sint * sin(phi), v1 = vf * cost;
  double e1[3] = {v[0], v[1], v[2]}, e2[3], e3[3], nrm[3];
  normalize3(e1);
  if (fabs(e1[0]) > 1e-1 || fabs(e1[1]) > 1e-1) { nrm[0] = 0; nrm[1] = 0; nrm[2] = 1; }
  else { nrm[0] = 1; nrm[1] = 0; nrm[2] = 0; }
  cross3(nrm, e1, e2);
  normalize3(e2);
  cross3(e1, e2, e3);
  n->vx = e1[0] * v1 + e2[0] * v2 + e3[0] * v3;
  n->vy = e1[1] * v1 + e2[1] * v2 + e3[1] * v3;
  n->vz = e1[2] * v1 + e2[2] * v2 + e3[2] * v3;
  double S = oracle_sqe_lookup(c, Q, E);
  double prob_f = S * (vf / vi) * Q * (Qmax - Qmin) * (Emax - Emin) / (kf * ki) / 2;
  n->p *= prob_f;
}

/* Outgoing velocity of a (Q, E) transfer, shared by the constant-(Q, E)
 * and E(Q) kernels (constant_qe.py:38-67, E_Q.py:64-92): v1 = vf cos(t)
 * along the incident direction e1, v2 = vf sin(t) cos(phi) along
 * e2 = unit(n x e1), v3 = vf sin(t) sin(phi) along e3 = e1 x e2, with
 * n = z unless e1 lies within 0.1 of it (then x). */
static void qe_velocity(neutron_t* n, double vf, double cost, double sint,
                        double phi) {
  double v2 = vf * sint * cos(phi), v3 = vf * sint * sin(phi);
  double v1 = vf * cost;
  double e1[3] = {n->vx, n->vy, n->vz}, e2[3], e3[3], nrm[3];
  normalize3(e1);
  if (fabs(e1[0]) > 1e-1 || fabs(e1[1]) > 1e-1) { nrm[0] = 0; nrm[1] = 0; nrm[2] = 1; }
  else { nrm[0] = 1; nrm[1] = 0; nrm[2] = 0; }
  cross3(nrm, e1, e2);
  normalize3(e2);
  cross3(e1, e2, e3);
  n->vx = e1[0] * v1 + e2[0] * v2 + e3[0] * v3;
  n->vy = e1[1] * v1 + e2[1] * v2 + e3[1] * v3;
  n->vz = e1[2] * v1 + e2[2] * v2 + e3[2] * v3;
}

/* constant_qe.S (acc/kernels/constant_qe.py:15-67): scatter to the fixed
 * (Q, E) = (dp[10], dp[11]) with one draw for the azimuth.  The reference
 * has no guard for a transfer the neutron cannot make (E above Ei, or
 * |cos(theta)| > 1), where its velocity turns NaN; here such a neutron is
 * absorbed (p = -1), after the azimuth draw. */
static void constant_qe_S(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double Q = c->dp[10], E = c->dp[11];
  double vi = length3(n->vx, n->vy, n->vz);
  double Ei = vi * vi * VS2E;
  double Ef = Ei - E;
  double phi = rng_uniform(rng) * 2.0 * M_PI;
  if (!(Ef >= 0)) { n->p = -1; return; }
  double vf = sqrt(Ef) * SE2V;
  double ki = V2K * vi, kf = V2K * vf;
  double cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
  double s2 = 1.0 - cost * cost;
  if (!(s2 >= 0)) { n->p = -1; return; }
  qe_velocity(n, vf, cost, sqrt(s2), phi);
}

/* E_Q kernel programs: postfix {opcode, argument} pairs (MCV_EXPR_*),
 * run with a stack of MCV_EXPR_STACK values; a malformed program (stack
 * under- or overflow, unknown opcode, not exactly one value left) gives
 * NaN.  POWI is x**n by binary powering. */
static double expr_powi(double x, int n) {
  unsigned m = n < 0 ? 0u - (unsigned)n : (unsigned)n;
  double r = 1.0, b = x;
  while (m) {
    if (m & 1u) r *= b;
    m >>= 1;
    if (m) b *= b;
  }
  return n < 0 ? 1.0 / r : r;
}

static double expr_mod(double a, double b) {
  /* Python's float %: the remainder takes the sign of b */
  double r = fmod(a, b);
  if (r != 0 && ((r < 0) != (b < 0))) r += b;
  return r;
}

double oracle_expr_eval(const double* prog, int nops, double Q) {
  double st[MCV_EXPR_STACK];
  int sp = 0;
  for (int i = 0; i < nops; ++i) {
    int op = (int)prog[2 * i];
    double arg = prog[2 * i + 1];
    if (op == MCV_EXPR_CONST || op == MCV_EXPR_Q) {
      if (sp >= MCV_EXPR_STACK) return NAN;
      st[sp++] = op == MCV_EXPR_CONST ? arg : Q;
      continue;
    }
    if (sp < 1) return NAN;
    double x = st[sp - 1], r;
    if (op >= MCV_EXPR_ADD && op <= MCV_EXPR_MOD && op != MCV_EXPR_NEG &&
        op != MCV_EXPR_POWI) {
      if (sp < 2) return NAN;
      double a = st[sp - 2], b = x;
      switch (op) {
        case MCV_EXPR_ADD: r = a + b; break;
        case MCV_EXPR_SUB: r = a - b; break;
        case MCV_EXPR_MUL: r = a * b; break;
        case MCV_EXPR_DIV: r = a / b; break;
        case MCV_EXPR_POW: r = pow(a, b); break;
        case MCV_EXPR_ATAN2: r = atan2(a, b); break;
        case MCV_EXPR_MIN: r = b < a ? b : a; break;
        case MCV_EXPR_MAX: r = b > a ? b : a; break;
        default: r = expr_mod(a, b); break;
      }
      st[sp - 2] = r;
      --sp;
      continue;
    }
    switch (op) {
      case MCV_EXPR_NEG: r = -x; break;
      case MCV_EXPR_POWI: r = expr_powi(x, (int)arg); break;
      case MCV_EXPR_EXP: r = exp(x); break;
      case MCV_EXPR_LOG: r = log(x); break;
      case MCV_EXPR_LOG10: r = log10(x); break;
      case MCV_EXPR_SQRT: r = sqrt(x); break;
      case MCV_EXPR_SIN: r = sin(x); break;
      case MCV_EXPR_COS: r = cos(x); break;
      case MCV_EXPR_TAN: r = tan(x); break;
      case MCV_EXPR_ASIN: r = asin(x); break;
      case MCV_EXPR_ACOS: r = acos(x); break;
      case MCV_EXPR_ATAN: r = atan(x); break;
      case MCV_EXPR_SINH: r = sinh(x); break;
      case MCV_EXPR_COSH: r = cosh(x); break;
      case MCV_EXPR_TANH: r = tanh(x); break;
      case MCV_EXPR_ASINH: r = asinh(x); break;
      case MCV_EXPR_ACOSH: r = acosh(x); break;
      case MCV_EXPR_ATANH: r = atanh(x); break;
      case MCV_EXPR_ERF: r = erf(x); break;
      case MCV_EXPR_ERFC: r = erfc(x); break;
      case MCV_EXPR_FABS: r = fabs(x); break;
      case MCV_EXPR_FLOOR: r = floor(x); break;
      case MCV_EXPR_CEIL: r = ceil(x); break;
      default: return NAN;
    }
    st[sp - 1] = r;
  }
  return sp == 1 ? st[0] : NAN;
}

/* The S of makeS (acc/kernels/E_Q.py:37-98): up to max_iter draws of
 * Q uniform on [Qmin, Qmax), each rejected while E(Q) exceeds Ei or the
 * transfer is kinematically closed (cos^2 > 1); none accepted -> p = 0.
 * Weight S(Q) (vf/vi) Q (Qmax-Qmin) / (2 ki kf) / tries. */
static void e_q_S(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double Qmin = c->dp[10], Qmax = c->dp[11];
  int max_iter = (int)c->dp[12];
  const double* progE = (const double*)c->table;
  const double* progS = progE + 2 * c->ip[4];
  double vi = length3(n->vx, n->vy, n->vz);
  double Ei = vi * vi * VS2E;
  double Q = 0, vf = 0, ki = 0, kf = 0, cost = 0, cost2 = 0;
  int itr, found = 0;
  for (itr = 0; itr < max_iter; ++itr) {
    Q = rng_uniform(rng) * (Qmax - Qmin);
    Q += Qmin;
    double E = oracle_expr_eval(progE, c->ip[4], Q);
    double Ef = Ei - E;
    if (Ef < 0) continue;
    vf = sqrt(Ef) * SE2V;
    ki = V2K * vi;
    kf = V2K * vf;
    cost = (ki * ki + kf * kf - Q * Q) / (2 * ki * kf);
    cost2 = cost * cost;
    if (cost2 > 1) continue;
    found = 1;
    break;
  }
  if (!found) { n->p = 0; return; }
  double sint = sqrt(1.0 - cost2);
  double phi = rng_uniform(rng) * 2.0 * M_PI;
  qe_velocity(n, vf, cost, sint, phi);
  double S = oracle_expr_eval(progS, c->ip[5], Q);
  double prob_f = S * (vf / vi) * Q * (Qmax - Qmin) / (kf * ki) / 2;
  n->p *= prob_f / (itr + 1);
}

/* SANS2D_ongrid's S (acc/kernels/SANS2D_ongrid.py:16-56): (Qx, Qy)
 * uniform over the grid's box; vx -= Qx K2V, vy -= Qy K2V, vz from
 * vi^2 - vx^2 vy^2 (the reference's product, kept); p *= S bilinear on
 * cells of width (Qmax - Qmin) / n, indices clamped to [0, n-2];
 * S[nx][ny] x-major */
static void sans2d_S(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double Qxmin = c->dp[10], Qxmax = c->dp[11], Qymin = c->dp[12],
         Qymax = c->dp[13];
  int nx = c->ip[4], ny = c->ip[5];
  const double* S = (const double*)c->table;
  double vi = length3(n->vx, n->vy, n->vz);
  double Qx = rng_uniform(rng) * (Qxmax - Qxmin);
  Qx += Qxmin;
  double Qy = rng_uniform(rng) * (Qymax - Qymin);
  Qy += Qymin;
  n->vx -= Qx * K2V;
  n->vy -= Qy * K2V;
  n->vz = sqrt(vi * vi - n->vx * n->vx * n->vy * n->vy);
  double dQx = (Qxmax - Qxmin) / nx, dQy = (Qymax - Qymin) / ny;
  int xi = (int)((Qx - Qxmin) / dQx), yi = (int)((Qy - Qymin) / dQy);
  if (xi < 0) xi = 0;
  if (xi > nx - 2) xi = nx - 2;
  if (yi < 0) yi = 0;
  if (yi > ny - 2) yi = ny - 2;
  double xf = (Qx - Qxmin) / dQx - xi, yf = (Qy - Qymin) / dQy - yi;
  double f00 = S[xi * ny + yi], f10 = S[(xi + 1) * ny + yi];
  double f01 = S[xi * ny + yi + 1], f11 = S[(xi + 1) * ny + yi + 1];
  n->p *= bilinear(xf, yf, f00, f01, f10, f11);
}

/* DGSSXResKernel.scatter (acc/kernels/DGSSXResKernel.py:19-98): towards a
 * target disc (choose_direction :19-58, with the reference's in-place
 * vec3.cross whose later components read the ones it already replaced),
 * arriving at a time of flight uniform in tof_target +- dtof / 2;
 * p *= solid angle / 4 pi * dtof * (2 Ef / tof) * vf / vi */
static void dgssxres_S(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double td[3] = {c->dp[15] - n->x, c->dp[16] - n->y, c->dp[17] - n->z};
  double rad = c->dp[18], tof_t = c->dp[19], dtof = c->dp[20];
  double l2 = td[0] * td[0] + td[1] * td[1] + td[2] * td[2];
  double cmax = sqrt(l2 / (rad * rad + l2));
  if (rad < 0.0) cmax *= -1.0;
  double solid = 2.0 * M_PI * (1.0 - cmax);
  double r = rng_uniform(rng);
  r = r * (cmax - 1.0) + 1.0;
  double theta = acos(r);
  double phi = rng_uniform(rng) * 2.0 * M_PI;
  double nm[3];
  if (td[0] == 0.0 && td[2] == 0.0) { nm[0] = 1; nm[1] = 0; nm[2] = 0; }
  else { nm[0] = -td[2]; nm[1] = 0; nm[2] = td[0]; }
  nm[0] = nm[1] * td[2] - nm[2] * td[1];
  nm[1] = nm[2] * td[0] - nm[0] * td[2];
  nm[2] = nm[0] * td[1] - nm[1] * td[0];
  double d[3] = {td[0], td[1], td[2]};
  oracle_rotate(d, nm, theta, 1e-7);
  oracle_rotate(d, td, phi, 1e-7);
  normalize3(d);
  double u = rng_uniform(rng);
  double tmin = tof_t - 0.5 * dtof, tmax = tof_t + 0.5 * dtof;
  double tof = u * (tmax - tmin) + tmin;
  double vf = sqrt(l2) / (tof - n->t);
  double Ef = vf * vf * VS2E;
  double dEdt = 2.0 * Ef / tof;
  double prob = solid / 4.0 / M_PI * dtof * dEdt;
  double vi = length3(n->vx, n->vy, n->vz);
  n->vx = d[0] * vf;
  n->vy = d[1] * vf;
  n->vz = d[2] * vf;
  n->p *= prob * (vf / vi);
}

/* ---------------------------------------------------------------- HSS */
/* the scattering coefficient; a composite's sums its elements' (the slots
 * after the component), scaled by dp[10] (1/N when averaged,
 * composite.py:95-99) */
static double hss_sigma(const neutron_t* n, const mcv_component* c) {
  if (c->ip[1] == MCV_KERNEL_POWDER) return powder_coeff(n, c);
  if (c->ip[1] == MCV_KERNEL_COMPOSITE && (c->ip[5] & 1)) {
    const mcv_component* e = c + 1;
    double s = 0.0;
    for (int i = 0; i < c->ip[4]; ++i)
      s += e[i].ip[1] == MCV_KERNEL_POWDER ? powder_coeff(n, &e[i]) : e[i].dp[9];
    return s * c->dp[10];
  }
  return c->dp[9];
}

/* the kernel's scatter function (scatter_func_factory.render,
 * acc/kernels/__init__.py:10-22, 36-44): p *= sigma for the kernels with a
 * constant scattering coefficient, then the kernel's S */
static void kernel_scatter(neutron_t* n, rng_t* rng, const mcv_component* c) {
  if (c->ip[1] == MCV_KERNEL_COMPOSITE) {
    /* composite.py:62-75, 101-104: one uniform picks the first element
     * whose running weight exceeds it (else the last); the element
     * scatters; p /= its weight */
    double r = rng_uniform(rng);
    const mcv_component* e = c + 1;
    int i = 0, last = c->ip[4] - 1;
    while (i < last && !(r < e[i].dp[23])) ++i;
    kernel_scatter(n, rng, &e[i]);
    n->p /= e[i].dp[22];
    return;
  }
  switch (c->ip[1]) {
    case MCV_KERNEL_ISOTROPIC:
      n->p *= c->dp[9]; /* kernels/__init__.py:42 */
      isotropic_S(n, rng);
      break;
    case MCV_KERNEL_POWDER:
      powder_scatter(n, rng, c);
      break;
    case MCV_KERNEL_SQE_GRID:
      n->p *= c->dp[9];
      sqe_scatter(n, rng, c);
      break;
    case MCV_KERNEL_CONSTANT_QE:
      n->p *= c->dp[9]; /* kernels/__init__.py:85 */
      constant_qe_S(n, rng, c);
      break;
    case MCV_KERNEL_E_Q:
      n->p *= c->dp[9]; /* kernels/__init__.py:103 */
      e_q_S(n, rng, c);
      break;
    case MCV_KERNEL_SANS2D:
      n->p *= c->dp[9]; /* kernels/__init__.py:119 */
      sans2d_S(n, rng, c);
      break;
    case MCV_KERNEL_DGSSXRES:
      n->p *= c->dp[9]; /* kernels/__init__.py:138 */
      dgssxres_S(n, rng, c);
      break;
    default:
      break;
  }
}

/* HomogeneousSingleScatterer.propagate
 * (acc/components/samples/homogeneous_single_scatterer.py:62-100) */
static void hss(neutron_t* n, rng_t* rng, const mcv_component* c) {
  double x = n->x, y = n->y, z = n->z, vx = n->vx, vy = n->vy, vz = n->vz;
  double ts[MCV_MAX_INTERSECTIONS];
  int ninter = oracle_intersect(c, x, y, z, vx, vy, vz, ts);
  if (ninter < 2) return;
  if (ts[ninter - 1] <= 0) return;
  double rand = rng_uniform(rng);
  double o[3];
  oracle_time_to_scatter(ts, ninter, rand, o);
  double dt = o[1];
  if (dt <= 0) return;
  prop_dt(n, dt);
  double v = sqrt(vx * vx + vy * vy + vz * vz);
  double dist = v * o[2];
  double fulllen = v * o[0];
  double sigma = hss_sigma(n, c);
  double mu = abs_coeff(n, c->dp[8]);
  double atten = exp(-(mu + sigma) * dist);
  n->p *= fulllen * atten;
  kernel_scatter(n, rng, c);
  if (n->p <= 0) return;
  ninter = oracle_intersect(c, n->x, n->y, n->z, n->vx, n->vy, n->vz, ts);
  double dt3 = oracle_total_time_in_shape(ts, ninter);
  prop_dt(n, dt3);
  sigma = hss_sigma(n, c);
  mu = abs_coeff(n, c->dp[8]);
  /* the reference uses the incident speed v here (line 98) */
  double atten2 = exp(-(mu + sigma) * v * dt3);
  n->p *= atten2;
}

/* ------------------------------------------------ multiple scattering */
/* HomogeneousMultipleScatterer
 * (acc/components/samples/homogeneous_multiple_scatterer.py:22-342) for
 * one neutron: up to max_scattered_neutrons output neutrons.  Parameters
 * as for the HSS component, plus ip[6] = max_scattered_neutrons,
 * ip[7] = max_ms_loops | max_ms_loops_path1 << 16 and
 * dp[14] = minimum_neutron_event_probability. */
#define ORACLE_MS_CAP 64

static double atten_coeff(const neutron_t* n, const mcv_component* c) {
  /* _calc_atten_coeff (:67-71) */
  return hss_sigma(n, c) + abs_coeff(n, c->dp[8]);
}

static int is_moving(const neutron_t* n) {
  /* acc/neutron.py:39-42, MIN_VELOCITY = 1e-6 */
  return sqrt(n->vx * n->vx + n->vy * n->vy + n->vz * n->vz) > 1.e-6;
}

/* _is_exiting (acc/geometry/propagation.py:24-50) */
static int is_exiting(const mcv_component* c, const neutron_t* n) {
  double ts[MCV_MAX_INTERSECTIONS];
  int loc = oracle_locate(c, n->x, n->y, n->z);
  if (loc == LOC_INSIDE) return 0;
  int N = forward_intersect(c, n, ts);
  if (N == 0) return 1;
  if (loc == LOC_OUTSIDE) return 0;
  double previous = 0.;
  for (int it = 0; it < N; ++it) {
    double now = ts[it], middle = (previous + now) / 2.;
    if (oracle_locate(c, n->x + n->vx * middle, n->y + n->vy * middle,
                      n->z + n->vz * middle) != LOC_ONBORDER)
      return 0;
    previous = now;
  }
  return 1;
}

/* _propagate_to_next_exiting_surface_with_attenuation (:73-84) */
static void exit_with_attenuation(const mcv_component* c, neutron_t* n) {
  double tof = oracle_tof_before_first_exit(c, (const double*)n);
  double v = sqrt(n->vx * n->vx + n->vy * n->vy + n->vz * n->vz);
  double distance = tof * v;
  double atten = atten_coeff(n, c);
  double transmission_prob = exp(-atten * distance);
  oracle_propagate_to_next_exiting_surface(c, (double*)n);
  n->p *= transmission_prob;
}

/* _interactM1 (:86-121): the transmitted and the scattered neutron.  The
 * absorbed copy (:106-110) is overwritten by the scattered one and the
 * kernels' absorb is a no-op (kernels/__init__.py:164-166), so it is not
 * formed.  A neutron outside the shape after propagating to the incident
 * surface, where the reference raises, gives no output. */
static int interact_m1(const mcv_component* c, rng_t* rng, neutron_t* out,
                       neutron_t* n) {
  double vx = n->vx, vy = n->vy, vz = n->vz;
  if (oracle_locate(c, n->x, n->y, n->z) != LOC_INSIDE)
    oracle_propagate_to_next_incident_surface(c, (double*)n);
  double tof = oracle_tof_before_first_exit(c, (const double*)n);
  if (!(tof > 0.)) return 0; /* 0: :97; < 0 or NaN: the reference raises */
  double v = sqrt(vx * vx + vy * vy + vz * vz);
  double distance = tof * v;
  double sigma = hss_sigma(n, c);
  double mu = abs_coeff(n, c->dp[8]);
  double transmission_prob = exp(-(mu + sigma) * distance);
  out[0] = *n;
  oracle_propagate_to_next_exiting_surface(c, (double*)&out[0]);
  out[0].p *= transmission_prob;
  double rand = rng_uniform(rng);
  double x = distance * rand;
  double prob = distance * exp(-(mu + sigma) * x);
  out[1] = *n;
  out[1].p *= prob;
  prop_dt(&out[1], x / v);
  kernel_scatter(&out[1], rng, c);
  return 2;
}

/* _interactM_path1 (:123-177), out holding `cap` neutrons */
static int interact_m_path1(const mcv_component* c, rng_t* rng,
                            neutron_t* out, int cap, const neutron_t* n0) {
  const int max_sc = c->ip[6], loops1 = c->ip[7] >> 16;
  const double min_prob = c->dp[14];
  neutron_t buf_a[ORACLE_MS_CAP], buf_b[ORACLE_MS_CAP], scattered[2];
  neutron_t *tbs = buf_a, *tbs2 = buf_b;
  if (n0->p < min_prob) return 0;
  int ntbs = 1, out_index = 0;
  const int lim = max_sc < cap ? max_sc : cap;
  tbs[0] = *n0;
  for (int iloop = 0; iloop < loops1; ++iloop) {
    int s2 = 0;
    for (int i = 0; i < ntbs; ++i) {
      int ns = interact_m1(c, rng, scattered, &tbs[i]);
      for (int j = 0; j < ns; ++j) {
        neutron_t* s1 = &scattered[j];
        if (s1->p < min_prob) continue;
        if (oracle_locate(c, s1->x, s1->y, s1->z) != LOC_INSIDE) {
          out[out_index++] = *s1;
          if (out_index >= lim) return out_index;
          continue;
        }
        tbs2[s2++] = *s1;
        if (s2 >= max_sc) break;
      }
      if (s2 >= max_sc) break;
    }
    neutron_t* tmp = tbs2;
    tbs2 = tbs;
    tbs = tmp;
    ntbs = s2;
    if (!ntbs) break;
  }
  for (int i = 0; i < ntbs; ++i) {
    if (out_index >= lim) break;
    out[out_index++] = tbs[i];
  }
  return out_index;
}

/* _scatterM (:196-256): the output neutrons of one incident neutron */
static int scatter_m(const mcv_component* c, rng_t* rng, neutron_t* out,
                     const neutron_t* n0) {
  const int max_sc = c->ip[6], loops = c->ip[7] & 0xffff;
  const double min_prob = c->dp[14];
  neutron_t buf_a[ORACLE_MS_CAP], buf_b[ORACLE_MS_CAP],
      scattered[ORACLE_MS_CAP];
  neutron_t *tbs = buf_a, *tbs2 = buf_b;
  if (is_exiting(c, n0)) {
    out[0] = *n0;
    return 1;
  }
  int ntbs = 1, out_index = 0;
  tbs[0] = *n0;
  for (int iloop = 0; iloop < loops; ++iloop) {
    int s2 = 0;
    for (int i = 0; i < ntbs; ++i) {
      int ns1 = interact_m_path1(c, rng, scattered, max_sc, &tbs[i]);
      for (int j = 0; j < ns1; ++j) {
        neutron_t* s1 = &scattered[j];
        if (s1->p < min_prob) continue;
        if (!is_moving(s1)) continue;
        if (oracle_locate(c, s1->x, s1->y, s1->z) == LOC_INSIDE)
          exit_with_attenuation(c, s1);
        if (is_exiting(c, s1)) {
          out[out_index++] = *s1;
          if (out_index >= max_sc) return out_index;
          continue;
        }
        tbs2[s2++] = *s1;
        if (s2 >= max_sc) break;
      }
      if (s2 >= max_sc) break;
    }
    neutron_t* tmp = tbs2;
    tbs2 = tbs;
    tbs = tmp;
    ntbs = s2;
    if (!ntbs) break;
  }
  for (int i = 0; i < ntbs; ++i) {
    if (out_index >= max_sc) break;
    neutron_t* m = &tbs[i];
    double x = m->x, y = m->y, z = m->z;
    oracle_propagate_out(c, (double*)m);
    double dx = m->x - x, dy = m->y - y, dz = m->z - z;
    double dist = sqrt(dx * dx + dy * dy + dz * dz);
    double atten = atten_coeff(m, c);
    m->p *= exp(-atten * dist);
    out[out_index++] = *m;
  }
  return out_index;
}

/* ----------------------------------------------------------- monitors */
typedef struct {
  double* out; /* [3][nbins] */
  uint64_t nbins;
  int atomic;
} tally_t;

static inline void tally_add(const tally_t* tl, uint64_t bin, double p) {
  if (!tl || !tl->out) return;
  double* o = tl->out;
  if (tl->atomic) {
#pragma omp atomic
    o[bin] += 1;
#pragma omp atomic
    o[tl->nbins + bin] += p;
#pragma omp atomic
    o[2 * tl->nbins + bin] += p * p;
  } else {
    o[bin] += 1;
    o[tl->nbins + bin] += p;
    o[2 * tl->nbins + bin] += p * p;
  }
}

static inline int clampi(int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); }

/* PSD_monitor.propagate (acc/components/monitors/psd_monitor.py:66-83) */
static void psd_monitor(const neutron_t* n, const mcv_component* c,
                        const tally_t* tl) {
  const double* d = c->dp;
  double xmin = d[0], xmax = d[1], ymin = d[2], ymax = d[3];
  int nx = c->ip[0], ny = c->ip[1];
  double dt = -n->z / n->vz;
  double x = n->x + n->vx * dt, y = n->y + n->vy * dt, t = n->t + dt;
  if (n->t > t) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  int ix = clampi((int)floor((x - xmin) / (xmax - xmin) * nx), nx);
  int iy = clampi((int)floor((y - ymin) / (ymax - ymin) * ny), ny);
  tally_add(tl, (uint64_t)ix * ny + iy, n->p);
}

/* PSD_monitor_4Pi.propagate (psd_monitor_4pi.py:56-79), including the +0.5
 * in the theta index (line 72).  A neutron that misses the sphere is not
 * tallied. */
static void psd_monitor_4pi(neutron_t* n, const mcv_component* c,
                            const tally_t* tl) {
  double radius = c->dp[0];
  int nphi = c->ip[0], ntheta = c->ip[1];
  double t1, t2;
  oracle_intersect_sphere(n->x, n->y, n->z, n->vx, n->vy, n->vz, radius, &t1,
                          &t2);
  if (isnan(t1)) return;
  if (t2 < 0) return;
  if (t1 < 0) t1 = t2;
  prop_dt(n, t1);
  double phi = atan2(n->x, n->z);
  double sy = n->y / radius;
  if (!(sy == sy)) return;
  if (sy > 1) sy = 1;
  if (sy < -1) sy = -1;
  double theta = asin(sy);
  int iphi = (int)(nphi * (phi / 2 / M_PI + 0.5));
  if (iphi >= nphi) iphi = nphi - 1;
  else if (iphi < 0) iphi = 0;
  int itheta = (int)(ntheta * (theta + M_PI / 2) / M_PI + 0.5);
  if (itheta >= ntheta) itheta = ntheta - 1;
  else if (itheta < 0) itheta = 0;
  tally_add(tl, (uint64_t)iphi * ntheta + itheta, n->p);
}

/* Wavelength_monitor.propagate (wavelength_monitor.py:52-74) */
static void wavelength_monitor(const neutron_t* n, const mcv_component* c,
                               const tally_t* tl) {
  const double* d = c->dp;
  double xmin = d[0], xmax = d[1], ymin = d[2], ymax = d[3], Lmin = d[4],
         Lmax = d[5];
  int nchan = c->ip[0];
  double dt = -n->z / n->vz;
  double x = n->x + n->vx * dt, y = n->y + n->vy * dt, t = n->t + dt;
  if (n->t > t) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  double v = sqrt(n->vx * n->vx + n->vy * n->vy + n->vz * n->vz);
  double L = 2 * M_PI / (v * V2K);
  if (!(L > Lmin && L < Lmax)) return;
  int iL = clampi((int)floor((L - Lmin) / (Lmax - Lmin) * nchan), nchan);
  tally_add(tl, (uint64_t)iL, n->p);
}

/* Energy monitor: no reference counterpart; the wavelength monitor
 * (wavelength_monitor.py:52-74) with E = v^2 VS2E (acc/neutron.py:69-71). */
static void energy_monitor(const neutron_t* n, const mcv_component* c,
                           const tally_t* tl) {
  const double* d = c->dp;
  double xmin = d[0], xmax = d[1], ymin = d[2], ymax = d[3], Emin = d[4],
         Emax = d[5];
  int nchan = c->ip[0];
  double dt = -n->z / n->vz;
  double x = n->x + n->vx * dt, y = n->y + n->vy * dt, t = n->t + dt;
  if (n->t > t) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  double v2 = n->vx * n->vx + n->vy * n->vy + n->vz * n->vz;
  double E = v2 * VS2E;
  if (!(E > Emin && E < Emax)) return;
  int iE = clampi((int)floor((E - Emin) / (Emax - Emin) * nchan), nchan);
  tally_add(tl, (uint64_t)iE, n->p);
}

/* PosDiv_monitor.propagate (posdiv_monitor.py:67-89) */
static void posdiv_monitor(const neutron_t* n, const mcv_component* c,
                           const tally_t* tl) {
  const double* d = c->dp;
  double xmin = d[0], xmax = d[1], ymin = d[2], ymax = d[3], maxdiv = d[4];
  int npos = c->ip[0], ndiv = c->ip[1];
  double dt = -n->z / n->vz;
  double x = n->x + n->vx * dt, y = n->y + n->vy * dt, t = n->t + dt;
  if (n->t > t) return;
  if (!(x > xmin && x < xmax && y > ymin && y < ymax)) return;
  double div = atan(n->vx / n->vz) * (180. / M_PI);
  if (!(div < maxdiv && div > -maxdiv)) return;
  int ix = clampi((int)floor((x - xmin) / (xmax - xmin) * npos), npos);
  int idiv = clampi((int)floor((div + maxdiv) / (2 * maxdiv) * ndiv), ndiv);
  tally_add(tl, (uint64_t)ix * ndiv + idiv, n->p);
}

/* IQE_monitor.propagate (iqe_monitor.py:80-113) */
static void iqe_monitor(const neutron_t* n, const mcv_component* c,
                        const tally_t* tl) {
  const double* d = c->dp;
  double Ei = d[0], Qmin = d[1], Qmax = d[2], Emin = d[3], Emax = d[4];
  double max_in = d[5], min_in = d[6], max_out = d[7], min_out = d[8];
  int nQ = c->ip[0], nE = c->ip[1];
  double vx = n->vx, vy = n->vy, vz = n->vz;
  double angle_in = atan2(vx, vz) / M_PI * 180.;
  double angle_out;
  if (vy != 0) {
    double theta = atan(sqrt(vx * vx + vz * vz) / vy) / M_PI * 180.;
    angle_out = vy > 0 ? 90. - theta : 90. + theta;
  } else {
    angle_out = 0.;
  }
  if (min_in < angle_in && angle_in < max_in && min_out < angle_out &&
      angle_out < max_out) {
    double vi = sqrt(Ei) * SE2V;
    double Q = sqrt(vx * vx + vy * vy + (vz - vi) * (vz - vi)) * V2K;
    double E = Ei - (vx * vx + vy * vy + vz * vz) * VS2E;
    if (Q >= Qmin && Q < Qmax && E >= Emin && E < Emax) {
      int iQ = clampi((int)floor((Q - Qmin) / (Qmax - Qmin) * nQ), nQ);
      int iE = clampi((int)floor((E - Emin) / (Emax - Emin) * nE), nE);
      tally_add(tl, (uint64_t)iQ * nE + iE, n->p);
    }
  }
}

/* theta x tof 4pi shell: no reference counterpart; the sphere crossing of
 * PSD_monitor_4Pi (psd_monitor_4pi.py:56-66) binned by the polar angle from
 * +z, atan2(hypot(x, y), z), and the time of flight. */
static void theta_tof_4pi(neutron_t* n, const mcv_component* c,
                          const tally_t* tl) {
  double radius = c->dp[0], tmin = c->dp[1], tmax = c->dp[2];
  int nth = c->ip[0], nt = c->ip[1];
  double t1, t2;
  oracle_intersect_sphere(n->x, n->y, n->z, n->vx, n->vy, n->vz, radius, &t1,
                          &t2);
  if (isnan(t1)) return;
  if (t2 < 0) return;
  if (t1 < 0) t1 = t2;
  prop_dt(n, t1);
  double theta = atan2(sqrt(n->x * n->x + n->y * n->y), n->z);
  if (!(theta == theta)) return;
  if (!(n->t >= tmin && n->t < tmax)) return;
  int ith = clampi((int)floor(theta / M_PI * nth), nth);
  int it = clampi((int)floor((n->t - tmin) / (tmax - tmin) * nt), nt);
  tally_add(tl, (uint64_t)ith * nt + it, n->p);
}

/* Vertical cylinder (axis y) crossing from inside: the exit time of
 * x^2 + z^2 = R^2 (the side term of intersectCylinderSide,
 * arrow_intersect.py:178-204, with the axis along y).  Returns NaN if the
 * neutron leaves through a cap or does not move horizontally. */
static double vcyl_exit(const neutron_t* n, double R, double H) {
  double a = n->vx * n->vx + n->vz * n->vz;
  double b = n->x * n->vx + n->z * n->vz;
  double c = n->x * n->x + n->z * n->z - R * R;
  double k = b * b - a * c;
  if (k < 0 || a == 0) return NAN;
  double t = (-b + sqrt(k)) / a;
  if (t < 0) return NAN;
  double y = n->y + n->vy * t;
  if (fabs(y) >= H / 2) return NAN;
  return t;
}

/* Cylindrical I(Q,E) detector: no reference counterpart; the exit crossing
 * of a vertical cylinder, then Q and E as IQE_monitor.propagate
 * (iqe_monitor.py:96-110) computes them. */
static void cyl_iqe(neutron_t* n, const mcv_component* c, const tally_t* tl) {
  const double* d = c->dp;
  double R = d[0], H = d[1], Ei = d[2], Qmin = d[3], Qmax = d[4], Emin = d[5],
         Emax = d[6];
  int nQ = c->ip[0], nE = c->ip[1];
  double t = vcyl_exit(n, R, H);
  if (isnan(t)) return;
  prop_dt(n, t);
  double vx = n->vx, vy = n->vy, vz = n->vz;
  double vi = sqrt(Ei) * SE2V;
  double Q = sqrt(vx * vx + vy * vy + (vz - vi) * (vz - vi)) * V2K;
  double E = Ei - (vx * vx + vy * vy + vz * vz) * VS2E;
  if (Q >= Qmin && Q < Qmax && E >= Emin && E < Emax) {
    int iQ = clampi((int)floor((Q - Qmin) / (Qmax - Qmin) * nQ), nQ);
    int iE = clampi((int)floor((E - Emin) / (Emax - Emin) * nE), nE);
    tally_add(tl, (uint64_t)iQ * nE + iE, n->p);
  }
}

/* Banked cylinder detector: no reference counterpart.  Vertical cylinder
 * of radius R and height H; banks are azimuthal windows
 * [a0 + b (w + g), a0 + b (w + g) + w) of phi = atan2(x, z); tubes split a
 * bank evenly in phi, pixels split the height, then a tof histogram. */
static void banked(neutron_t* n, const mcv_component* c, const tally_t* tl) {
  const double* d = c->dp;
  double R = d[0], H = d[1], a0 = d[2], w = d[3], g = d[4], tmin = d[5],
         tmax = d[6];
  int nb = c->ip[0], ntube = c->ip[1], npix = c->ip[2], ntof = c->ip[3];
  double t = vcyl_exit(n, R, H);
  if (isnan(t)) return;
  prop_dt(n, t);
  double phi = atan2(n->x, n->z);
  double rel = phi - a0;
  if (!(rel >= 0)) return;
  int b = (int)floor(rel / (w + g));
  if (b >= nb) return;
  double inb = rel - b * (w + g);
  if (inb >= w) return;
  if (!(n->t >= tmin && n->t < tmax)) return;
  int tube = clampi((int)floor(inb / w * ntube), ntube);
  int pix = clampi((int)floor((n->y + H / 2) / H * npix), npix);
  int it = clampi((int)floor((n->t - tmin) / (tmax - tmin) * ntof), ntof);
  uint64_t bin = (((uint64_t)b * ntube + tube) * npix + pix) * ntof + it;
  tally_add(tl, bin, n->p);
}

/* ------------------------------------------------------------ chains */
static uint64_t comp_nbins(const mcv_component* c) {
  switch (c->opcode) {
    case MCV_OP_PSD_MONITOR:
    case MCV_OP_PSD_MONITOR_4PI:
    case MCV_OP_POSDIV_MONITOR:
    case MCV_OP_IQE_MONITOR:
    case MCV_OP_THETA_TOF_4PI:
    case MCV_OP_CYL_IQE_DETECTOR:
      return (uint64_t)c->ip[0] * (uint64_t)c->ip[1];
    case MCV_OP_WAVELENGTH_MONITOR:
    case MCV_OP_ENERGY_MONITOR:
      return (uint64_t)c->ip[0];
    case MCV_OP_BANKED_DETECTOR:
      return (uint64_t)c->ip[0] * c->ip[1] * c->ip[2] * c->ip[3];
    default:
      return 0;
  }
}

typedef struct {
  uint64_t processed, bounce_overflow, nonfinite, rng_overrun;
} ostat_t;

/* One component on one neutron. */
static void run_component(neutron_t* n, rng_t* rng, const mcv_component* c,
                          const tally_t* tl, ostat_t* st) {
  switch (c->opcode) {
    case MCV_OP_ARM: break;
    case MCV_OP_SOURCE_SIMPLE: source_simple(n, rng, c); break;
    case MCV_OP_SNS_SOURCE: sns_source(n, rng, c); break;
    case MCV_OP_NEUTRON_STORAGE: {
      /* NeutronFromStorage.propagate (neutronfromstorage.py:68-82) */
      uint64_t N = c->table_len / 10;
      uint64_t idx = (uint64_t)rng->ctr[0] | ((uint64_t)rng->ctr[1] << 32);
      memcpy(n, (const double*)c->table + (idx % N) * 10, sizeof *n);
      break;
    }
    case MCV_OP_NEUTRON_TO_STORAGE: {
      /* mcvine's NeutronToStorage (placed by
         acc/test/instrument_factory.py:104-113): the neutron as it arrives,
         in this component's frame, one row [index, 10 values] a neutron */
      uint64_t* words = (uint64_t*)c->tally;
      uint64_t slot = __atomic_fetch_add(&words[0], 1, __ATOMIC_RELAXED);
      if (slot < c->table_len) {
        words[1 + 11 * slot] =
            (uint64_t)rng->ctr[0] | ((uint64_t)rng->ctr[1] << 32);
        memcpy(c->tally + 2 + 11 * slot, n, 10 * sizeof(double));
      }
      break;
    }
    case MCV_OP_GUIDE: st->bounce_overflow += guide(n, c, NULL); break;
    case MCV_OP_GUIDE_TAPERING:
      st->bounce_overflow += guide_tapering(n, c);
      break;
    case MCV_OP_GUIDE_ANYSHAPE:
      st->bounce_overflow += (c->ip[2] & 1) ? guide_anyshape_gravity(n, c)
                                            : guide_anyshape(n, c);
      break;
    case MCV_OP_HSS: hss(n, rng, c); break;
    case MCV_OP_PSD_MONITOR: psd_monitor(n, c, tl); break;
    case MCV_OP_PSD_MONITOR_4PI: psd_monitor_4pi(n, c, tl); break;
    case MCV_OP_WAVELENGTH_MONITOR: wavelength_monitor(n, c, tl); break;
    case MCV_OP_POSDIV_MONITOR: posdiv_monitor(n, c, tl); break;
    case MCV_OP_IQE_MONITOR: iqe_monitor(n, c, tl); break;
    case MCV_OP_ENERGY_MONITOR: energy_monitor(n, c, tl); break;
    case MCV_OP_THETA_TOF_4PI: theta_tof_4pi(n, c, tl); break;
    case MCV_OP_CYL_IQE_DETECTOR: cyl_iqe(n, c, tl); break;
    case MCV_OP_BANKED_DETECTOR: banked(n, c, tl); break;
    case MCV_OP_SLIT: slit_or_beamstop(n, c, 0); break;
    case MCV_OP_BEAMSTOP: slit_or_beamstop(n, c, 1); break;
    default: break;
  }
}

/*
 * Run the chain over neutrons [first, first+ncount).  A neutron leaves the
 * chain after the first component that leaves its weight not positive (the
 * p > 0 filter of ComponentBase.process, ComponentBase.py:100-102).
 * Tallies go into comp[k].tally (host memory here).  stats: processed,
 * bounce_overflow, nonfinite, rng_overrun.
 */
int oracle_run_chain(const mcv_chain* chain, uint64_t ncount, uint64_t first,
                     uint64_t seed, const float* uniforms, int stride,
                     double* out_neutrons, int32_t* out_last, int nthreads,
                     uint64_t* stats) {
  int nc = chain->ncomp;
  if (nc < 1 || nc > MCV_MAX_COMPONENTS) return MCV_EINVAL;
  uint64_t total_bins = 0;
  for (int k = 0; k < nc; ++k) total_bins += comp_nbins(&chain->comp[k]);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  /* private tallies per thread when small, atomics when large */
  int use_private = nthreads > 1 && total_bins * 3 * 8 * (uint64_t)nthreads <
                                        ((uint64_t)1 << 30);
  ostat_t gst = {0, 0, 0, 0};
  double** priv = NULL;
  if (use_private) {
    priv = (double**)calloc((size_t)nthreads * nc, sizeof(double*));
    for (int th = 0; th < nthreads; ++th)
      for (int k = 0; k < nc; ++k) {
        uint64_t nb = comp_nbins(&chain->comp[k]);
        if (nb && chain->comp[k].tally)
          priv[th * nc + k] = (double*)calloc(3 * nb, sizeof(double));
      }
  }
#pragma omp parallel num_threads(nthreads)
  {
    int th = 0;
#ifdef _OPENMP
    th = omp_get_thread_num();
#endif
    tally_t tl[MCV_MAX_COMPONENTS];
    for (int k = 0; k < nc; ++k) {
      tl[k].nbins = comp_nbins(&chain->comp[k]);
      tl[k].out = use_private ? priv[th * nc + k] : chain->comp[k].tally;
      tl[k].atomic = !use_private && nthreads > 1;
    }
    ostat_t st = {0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)ncount; ++ii) {
      uint64_t idx = first + (uint64_t)ii;
      rng_t rng;
      rng_init(&rng, seed, idx, 0, uniforms ? uniforms + (uint64_t)ii * stride : NULL,
               stride);
      neutron_t n;
      memset(&n, 0, sizeof n);
      int last = -1;
      st.processed++;
      for (int k = 0; k < nc; ++k) {
        const mcv_component* c = &chain->comp[k];
        if (k > 0) apply_transform(&n, chain->rot[k], chain->off[k]);
        last = k;
        if (c->opcode == MCV_OP_HMS) {
          /* fan-out: the rest of the chain for every output neutron, in
           * order, on the same stream (run_script.py:66-92, 245-260) */
          neutron_t outs[ORACLE_MS_CAP];
          int nout = scatter_m(c, &rng, outs, &n);
          for (int j = 0; j < nout; ++j) {
            n = outs[j];
            for (int k2 = k + 1; k2 < nc; ++k2) {
              apply_transform(&n, chain->rot[k2], chain->off[k2]);
              last = k2;
              run_component(&n, &rng, &chain->comp[k2], &tl[k2], &st);
              if (!(n.p > 0)) {
                if (isnan(n.p)) st.nonfinite++;
                break;
              }
            }
          }
          break;
        }
        run_component(&n, &rng, c, &tl[k], &st);
        if (!(n.p > 0)) {
          if (isnan(n.p)) st.nonfinite++;
          break;
        }
      }
      st.rng_overrun += rng.overrun;
      if (out_neutrons) memcpy(out_neutrons + (uint64_t)ii * 10, &n, sizeof n);
      if (out_last) out_last[ii] = last;
    }
#pragma omp critical
    {
      gst.processed += st.processed;
      gst.bounce_overflow += st.bounce_overflow;
      gst.nonfinite += st.nonfinite;
      gst.rng_overrun += st.rng_overrun;
    }
  }
  if (use_private) {
    for (int k = 0; k < nc; ++k) {
      uint64_t nb = comp_nbins(&chain->comp[k]);
      double* dst = chain->comp[k].tally;
      if (!nb || !dst) continue;
      for (int th = 0; th < nthreads; ++th) {
        double* src = priv[th * nc + k];
        for (uint64_t b = 0; b < 3 * nb; ++b) dst[b] += src[b];
        free(src);
      }
    }
    free(priv);
  }
  if (stats) {
    stats[0] = gst.processed;
    stats[1] = gst.bounce_overflow;
    stats[2] = gst.nonfinite;
    stats[3] = gst.rng_overrun;
  }
  return gst.rng_overrun ? MCV_EINVAL : MCV_OK;
}

/*
 * Reflections per guide traversal: hist[k * nbins + min(r, nbins - 1)]
 * counts the neutrons that entered guide component k and made r
 * reflections there (the last bin collects r >= nbins - 1).  Same streams
 * and sequence as oracle_run_chain, without tallies; used to describe the
 * divergence of the guide chain, not to check results.
 */
int oracle_guide_reflections(const mcv_chain* chain, uint64_t ncount,
                             uint64_t first, uint64_t seed, int nthreads,
                             uint64_t* hist, int nbins) {
  int nc = chain->ncomp;
  if (nc < 1 || nc > MCV_MAX_COMPONENTS || nbins < 1 || !hist)
    return MCV_EINVAL;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  memset(hist, 0, sizeof(uint64_t) * (size_t)nc * nbins);
#pragma omp parallel num_threads(nthreads)
  {
    uint64_t* h = (uint64_t*)calloc((size_t)nc * nbins, sizeof(uint64_t));
    ostat_t st = {0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)ncount; ++ii) {
      rng_t rng;
      rng_init(&rng, seed, first + (uint64_t)ii, 0, NULL, 0);
      neutron_t n;
      memset(&n, 0, sizeof n);
      for (int k = 0; k < nc; ++k) {
        const mcv_component* c = &chain->comp[k];
        if (k > 0) apply_transform(&n, chain->rot[k], chain->off[k]);
        if (c->opcode == MCV_OP_GUIDE) {
          int r;
          guide(&n, c, &r);
          if (r >= 0) h[(size_t)k * nbins + (r < nbins ? r : nbins - 1)]++;
        } else {
          run_component(&n, &rng, c, NULL, &st);
        }
        if (!(n.p > 0)) break;
      }
    }
#pragma omp critical
    for (size_t b = 0; b < (size_t)nc * nbins; ++b) hist[b] += h[b];
    free(h);
  }
  return MCV_OK;
}

/*
 * Buffered mode (ComponentBase.process, ComponentBase.py:79-129): apply the
 * components to neutrons[n][10] in place; component k draws from stream k+1.
 * Neutrons whose weight is not positive are skipped by later components.
 */
int oracle_process_buffer(const mcv_chain* chain, double* neutrons, uint64_t n,
                          uint64_t first, uint64_t seed, int nthreads,
                          uint64_t* stats) {
  int nc = chain->ncomp;
  if (nc < 1 || nc > MCV_MAX_COMPONENTS) return MCV_EINVAL;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  ostat_t gst = {0, 0, 0, 0};
#pragma omp parallel num_threads(nthreads)
  {
    tally_t tl[MCV_MAX_COMPONENTS];
    for (int k = 0; k < nc; ++k) {
      tl[k].nbins = comp_nbins(&chain->comp[k]);
      tl[k].out = chain->comp[k].tally;
      tl[k].atomic = nthreads > 1;
    }
    ostat_t st = {0, 0, 0, 0};
#pragma omp for schedule(static)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
      neutron_t nt;
      memcpy(&nt, neutrons + (uint64_t)ii * 10, sizeof nt);
      st.processed++;
      for (int k = 0; k < nc; ++k) {
        const mcv_component* c = &chain->comp[k];
        int source = c->opcode == MCV_OP_SOURCE_SIMPLE ||
                     c->opcode == MCV_OP_SNS_SOURCE ||
                     c->opcode == MCV_OP_NEUTRON_STORAGE;
        if (!source && !(nt.p > 0)) break;
        if (k > 0) apply_transform(&nt, chain->rot[k], chain->off[k]);
        rng_t rng;
        rng_init(&rng, seed, first + (uint64_t)ii, (uint32_t)(k + 1), NULL, 0);
        run_component(&nt, &rng, c, &tl[k], &st);
      }
      memcpy(neutrons + (uint64_t)ii * 10, &nt, sizeof nt);
    }
#pragma omp critical
    {
      gst.processed += st.processed;
      gst.bounce_overflow += st.bounce_overflow;
    }
  }
  if (stats) {
    stats[0] = gst.processed;
    stats[1] = gst.bounce_overflow;
    stats[2] = gst.nonfinite;
    stats[3] = 0;
  }
  return MCV_OK;
}

/* single-component probes used by the known-answer tests */
int oracle_guide_one(const mcv_component* c, double* st) {
  return guide((neutron_t*)st, c, NULL);
}
void oracle_source_one(const mcv_component* c, const float* u, double* st) {
  rng_t rng;
  rng_init(&rng, 0, 0, 0, u, 5);
  source_simple((neutron_t*)st, &rng, c);
}
void oracle_hss_one(const mcv_component* c, const float* u, int nu,
                    double* st) {
  rng_t rng;
  rng_init(&rng, 0, 0, 0, u, nu);
  hss((neutron_t*)st, &rng, c);
}
/* The HSS kernel's scatter (p *= sigma, then S) on one neutron state,
 * uniforms from Philox (seed, index) stream 0. */
void oracle_kernel_scatter_one(const mcv_component* c, double* st,
                               uint64_t seed, uint64_t index) {
  rng_t rng;
  rng_init(&rng, seed, index, 0, NULL, 0);
  kernel_scatter((neutron_t*)st, &rng, c);
}
/* The mesh guide on one neutron state; returns 1 at the bounce limit. */
int oracle_anyshape_one(const mcv_component* c, double* st) {
  return (c->ip[2] & 1) ? guide_anyshape_gravity((neutron_t*)st, c)
                        : guide_anyshape((neutron_t*)st, c);
}
void oracle_apply_transform(const double* rot, const double* off, double* st) {
  apply_transform((neutron_t*)st, rot, off);
}
int oracle_sizeof_chain(void) { return (int)sizeof(mcv_chain); }
int oracle_sizeof_component(void) { return (int)sizeof(mcv_component); }

/* The multiple scatterer's steps on one neutron state (tests): which = 0
 * _interactM1, 1 _interactM_path1, 2 _scatterM; out holds up to
 * ORACLE_MS_CAP states; uniforms from Philox (seed, index) stream 0 or
 * from `uniforms` (count `stride`) when given.  Returns the number of
 * output neutrons. */
int oracle_ms_step(const mcv_component* c, int which, double* st,
                   uint64_t seed, uint64_t index, const float* uniforms,
                   int stride, double* out) {
  rng_t rng;
  rng_init(&rng, seed, index, 0, uniforms, stride);
  neutron_t* n = (neutron_t*)st;
  neutron_t o[ORACLE_MS_CAP];
  int N = 0;
  if (which == 0) N = interact_m1(c, &rng, o, n);
  else if (which == 1) N = interact_m_path1(c, &rng, o, c->ip[6], n);
  else N = scatter_m(c, &rng, o, n);
  memcpy(out, o, sizeof(neutron_t) * (size_t)N);
  return N;
}
