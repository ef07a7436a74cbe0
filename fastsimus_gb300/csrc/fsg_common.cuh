// Shared device math for the GB300 simus/pfield sweep kernels.
//
// Precision scheme.  A Green's term is
//     G(s, src, f) = amp * exp(-alpha_f r) * exp(i (k_f r mod 2 pi)),
//     amp = obliquity(theta) * directivity(theta) / sqrt(r) / n_sub
// (_pfield_math.py:202-247, simus.py:306-313).  k_f r reaches a few thousand radians, so the
// distance r and the product k_f r are carried as double-float pairs (an FP32 value plus an
// FP32 error term, ~48-bit significand).  GB300 executes FP64 at a small fraction of its FP32
// rate, so this pair arithmetic on the FP32 pipe is how the kernels get FP64-class phase
// accuracy.  Between exact "anchors" the term is advanced by the geometric recurrence
// G(f + df) = G(f) * exp((-d_alpha + i d_k) r) in plain FP32; anchors re-start it every
// kAnchor steps so rounding drift stays at the 1e-6 level.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fsg {

constexpr int kAnchor = 32;     // frequency steps between exact anchors (receive side, tables)
constexpr int kTxAnchor = 64;   // frequency steps between exact anchors on the transmit side
constexpr int kSrcPerThread = 16;
constexpr int kThreads = 256;

constexpr double kPi = 3.14159265358979323846;
constexpr double kTwoPiD = 2.0 * kPi;
// Cody-Waite split of 2*pi: kTwoPiHi * n is exact for the n that occur (|n| < 2^12).
constexpr float kTwoPiHi = (float)kTwoPiD;
constexpr float kTwoPiLo = (float)(kTwoPiD - (double)kTwoPiHi);
constexpr float kInvTwoPi = (float)(1.0 / kTwoPiD);
constexpr float kHalfPiF = (float)(kPi / 2.0);

struct dfl {
  float hi, lo;
};

__host__ __device__ inline dfl split_double(double v) {
  float hi = (float)v;
  float lo = (float)(v - (double)hi);
  return {hi, lo};
}

__device__ __forceinline__ dfl two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  dfl s = two_sum(a.hi, b.hi);
  float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, lo);
}

__device__ __forceinline__ dfl df_sqr(dfl a) {
  float p = __fmul_rn(a.hi, a.hi);
  float e = fmaf(a.hi, a.hi, -p);
  e = fmaf(2.0f * a.hi, a.lo, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  float s = __fsqrt_rn(a.hi);
  float e = __fadd_rn(fmaf(-s, s, a.hi), a.lo);
  return fast_two_sum(s, __fdiv_rn(e, 2.0f * s));
}

// (k * r) reduced to about [-pi, pi]; k and r double-float.  Absolute error ~2e-7 rad.
__device__ __forceinline__ float df_phase(float2 k, float r_hi, float r_lo) {
  float p = __fmul_rn(k.x, r_hi);
  float e = fmaf(k.x, r_hi, -p);
  e = fmaf(k.x, r_lo, e);
  e = fmaf(k.y, r_hi, e);
  float n = rintf(p * kInvTwoPi);
  float x = fmaf(-n, kTwoPiHi, p);  // exact
  x = __fadd_rn(x, e);
  return fmaf(-n, kTwoPiLo, x);
}

// exp(i k r) with accurate sin/cos (~1 ulp): used for recurrence steps, whose error compounds.
__device__ __forceinline__ float2 df_cis_accurate(float2 k, float r_hi, float r_lo) {
  float p = __fmul_rn(k.x, r_hi);
  float e = fmaf(k.x, r_hi, -p);
  e = fmaf(k.x, r_lo, e);
  e = fmaf(k.y, r_hi, e);
  float n = rintf(p * kInvTwoPi);
  float x = fmaf(-n, kTwoPiHi, p);  // exact
  float t = fmaf(-n, kTwoPiLo, e);  // remaining small phase
  float s, c;
  sincosf(x, &s, &c);
  return make_float2(fmaf(-t, s, c), fmaf(t, c, s));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 acc) {  // acc + a*b
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
  return acc;
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }

// Two complex recurrences advanced at once on the packed FP32x2 pipe (sm_100+ FFMA2/FMUL2):
// lane 0 of each float2 belongs to chain a, lane 1 to chain b, with real and imaginary parts
// in separate pairs (gr, gi) and the steps as (sr, si, sn = -si).  Four packed instructions
// replace eight scalar ones; each lane rounds exactly like the scalar fmaf/mul sequence.
__device__ __forceinline__ void cstep2(float2& gr, float2& gi, float2 sr, float2 si, float2 sn) {
  const float2 tr = __fmul2_rn(gr, sr);
  const float2 ti = __fmul2_rn(gi, sr);
  const float2 nr = __ffma2_rn(gi, sn, tr);  // gr sr - gi si
  const float2 ni = __ffma2_rn(gr, si, ti);  // gr si + gi sr
  gr = nr;
  gi = ni;
}

// Per-sweep physical constants (kernel argument, by value).
struct SweepConst {
  float2 dk;        // frequency-step wavenumber 2 pi df / c, double-float
  float dalpha;     // frequency-step attenuation, Np/m
  float inv_nsub;   // 1 / n_sub (mean over sub-elements)
  float2 min_dist;  // lambda_c / 2 distance clip, double-float
  float dir_coef;   // k_c * seg_length / 2 (centre-frequency directivity argument per sin(theta))
  float baffle_val; // impedance ratio for FSG_BAFFLE_IMPEDANCE
  int baffle;       // 0 soft, 1 rigid, 2 impedance
  int ffd;          // full-frequency directivity (directivity applied per frequency)
  float half_seg;   // seg_length / 2: the per-frequency directivity argument is k_f * half_seg * sin(theta)
};

// sin(x)/x for |x| <= 2 pi as its Taylor series to x^26 in u = x^2 (truncation < 3e-9 there;
// FP32 rounding adds at most ~3e-6 absolute at the end of the range, where the terms are
// largest): the per-frequency directivity of full_frequency_directivity
// (_simus_strategies.py:59-62, _pfield_strategies.py:77-81).
constexpr int kSincTerms = 14;
__device__ __forceinline__ float sinc_coef(int n) {  // (-1)^n / (2n + 1)!
  constexpr float c[kSincTerms] = {1.0f,
                                   -1.0f / 6.0f,
                                   1.0f / 120.0f,
                                   -1.0f / 5040.0f,
                                   1.0f / 362880.0f,
                                   -1.0f / 39916800.0f,
                                   1.0f / 6227020800.0f,
                                   -1.0f / 1307674368000.0f,
                                   1.0f / 355687428096000.0f,
                                   -1.0f / 121645100408832000.0f,
                                   1.0f / 51090942171709440000.0f,
                                   -1.0f / 25852016738884976640000.0f,
                                   1.0f / 15511210043330985984000000.0f,
                                   -1.0f / 10888869450418352160768000000.0f};
  return c[n];
}

__device__ __forceinline__ float sinc_poly(float x) {
  const float u = x * x;
  float p = sinc_coef(kSincTerms - 1);
#pragma unroll
  for (int n = kSincTerms - 2; n >= 0; --n) p = fmaf(p, u, sinc_coef(n));
  return p;
}

// sinc_poly of both lanes on the packed FP32x2 pipe.
__device__ __forceinline__ float2 sinc_poly2(float2 x) {
  const float2 u = __fmul2_rn(x, x);
  float2 p = make_float2(sinc_coef(kSincTerms - 1), sinc_coef(kSincTerms - 1));
#pragma unroll
  for (int n = kSincTerms - 2; n >= 0; --n) p = __ffma2_rn(p, u, make_float2(sinc_coef(n), sinc_coef(n)));
  return p;
}

// sin(x)/x: Taylor series for |x| < 2 (truncation error < 3e-9), sinf(x)/x beyond.
__device__ __forceinline__ float sinc_rad(float x) {
  if (fabsf(x) < 2.0f) {
    const float x2 = x * x;
    float p = -1.0f / 6227020800.0f;  // -1/13!
    p = fmaf(p, x2, 1.0f / 39916800.0f);
    p = fmaf(p, x2, -1.0f / 362880.0f);
    p = fmaf(p, x2, 1.0f / 5040.0f);
    p = fmaf(p, x2, -1.0f / 120.0f);
    p = fmaf(p, x2, 1.0f / 6.0f);
    return fmaf(-p, x2, 1.0f);  // 1 - x^2/6 + x^4/120 - ...
  }
  return __fdiv_rn(sinf(x), x);
}

// Geometry of one (point, source) pair: clipped distance (double-float), amplitude
// obliquity * directivity / sqrt(r) / n_sub and the per-step multiplier
// exp((-d_alpha + i d_k) r).  Follows _distances_and_angles (_pfield_math.py:70-118),
// _obliquity_factor (:165-199), the centre-frequency sinc (simus.py:310-313) and the step of
// _init_exponentials (:240-245).  The angle theta = asin(dx / r) - theta_e enters only
// through sin(theta) and cos(theta), formed from a = dx / r and the element rotation
// (cos theta_e, sin theta_e); |theta| >= pi/2 (the 1e-16 horizon floor) is cos(theta) <= 0.
struct SrcGeo {
  float r_hi, r_lo, amp;
  float2 step;
  float sth;  // sin(theta)
};

__device__ __forceinline__ SrcGeo source_geometry(dfl xs, dfl zs, float4 sp, float2 rot, const SweepConst& C) {
  dfl dx = df_add(xs, dfl{-sp.x, -sp.y});
  dfl dz = df_add(zs, dfl{-sp.z, -sp.w});
  dfl r = df_sqrt(df_add(df_sqr(dx), df_sqr(dz)));
  // a = (dx + 1e-16) / (r + 1e-16) on the unclipped distance; a = 1 when the point sits on the source
  float a = (r.hi > 0.0f) ? __fdiv_rn(dx.hi, r.hi) : 1.0f;
  a = fminf(1.0f, fmaxf(-1.0f, a));
  const float ca = sqrtf((1.0f - a) * (1.0f + a));  // cos(asin(a)) >= 0
  const float sth = fmaf(a, rot.x, -ca * rot.y);   // sin(asin(a) - theta_e)
  const float cth = fmaf(ca, rot.x, a * rot.y);    // cos(asin(a) - theta_e)
  if (r.hi < C.min_dist.x || (r.hi == C.min_dist.x && r.lo < C.min_dist.y)) r = dfl{C.min_dist.x, C.min_dist.y};
  float ob = (C.baffle == 0) ? cth : ((C.baffle == 1) ? 1.0f : __fdiv_rn(cth, cth + C.baffle_val));
  if (cth <= 0.0f) ob = 1e-16f;
  const float dir = C.ffd ? 1.0f : sinc_rad(C.dir_coef * sth);
  SrcGeo g;
  g.r_hi = r.hi;
  g.r_lo = r.lo;
  g.amp = ob * dir * rsqrtf(r.hi) * C.inv_nsub;
  const float mag = (C.dalpha != 0.0f) ? expf(-C.dalpha * r.hi) : 1.0f;
  const float2 cis = df_cis_accurate(C.dk, r.hi, r.lo);
  g.step = make_float2(mag * cis.x, mag * cis.y);
  g.sth = sth;
  return g;
}

// Exact anchor value amp * exp(-alpha r) * exp(i (k r mod 2 pi)) (_pfield_math.py:231-245).
__device__ __forceinline__ float2 anchor_value(float r_hi, float r_lo, float amp, float2 k, float alpha) {
  float ph = df_phase(k, r_hi, r_lo);
  float s, c;
  __sincosf(ph, &s, &c);
  float m = amp * __expf(-alpha * r_hi);
  return make_float2(m * c, m * s);
}

}  // namespace fsg
