// Float-float ("ff") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2), giving ~48-bit significands on the FP32
// pipe.  On GB300 the FP64 pipe delivers ~1/62 of the FP32 rate, so the mixed
// form uses ff wherever it needs more than FP32 accuracy.
//
// Error-free transformations (Knuth two_sum, Dekker/FMA two_prod) and the
// usual double-single algorithms; sincos and exp use 256-entry ff tables with
// short FP32 polynomials for the reduced argument.  All functions are
// __host__ __device__ so that tests compile them on the host (build with FP
// contraction off on the host; on the device, contraction only turns a*b+c
// into fused operations, which these algorithms tolerate).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#ifdef __CUDACC__
#define FF_HD __host__ __device__ __forceinline__
#else
#define FF_HD inline
#endif

namespace gb {

struct ff {
  float hi, lo;
};

FF_HD float __int_as_float_hd(int i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i);
#else
  float f;
  std::memcpy(&f, &i, sizeof f);
  return f;
#endif
}

FF_HD ff ff_make(float hi, float lo) {
  ff r;
  r.hi = hi;
  r.lo = lo;
  return r;
}
FF_HD ff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return ff_make(s, e);
}
FF_HD ff quick_two_sum(float a, float b) {  // requires |a| >= |b| (or a == 0)
  const float s = a + b;
  const float e = b - (s - a);
  return ff_make(s, e);
}
FF_HD ff two_prod(float a, float b) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  return ff_make(p, e);
}
FF_HD ff ff_from_double(double d) {
  const float h = (float)d;
  return ff_make(h, (float)(d - (double)h));
}
FF_HD double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
FF_HD ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }
// Addition with an absolute error of a few u^2 (|a| + |b|) (u = 2^-24): the
// leading parts exactly by two_sum, the low parts in FP32.  Under heavy
// cancellation the relative error of the result grows, its absolute error
// does not; every use in the kernels needs only the absolute bound.
FF_HD ff ff_add(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}
// Addition with a relative error of a few u^2 even under cancellation.
FF_HD ff ff_add_accurate(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  const ff t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
FF_HD ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }
FF_HD ff ff_addf(ff a, float b) {
  ff s = two_sum(a.hi, b);
  s.lo += a.lo;
  return quick_two_sum(s.hi, s.lo);
}
FF_HD ff ff_mul(ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
FF_HD ff ff_mulf(ff a, float b) {
  ff p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// a * b + c with ff accumulation.
FF_HD ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

// 1 / a (one Newton step on the FP32 reciprocal).
FF_HD ff ff_rcp(ff a) {
  const float y = 1.0f / a.hi;
  const ff ay = ff_mulf(a, y);
  const float e = (1.0f - ay.hi) - ay.lo;
  return quick_two_sum(y, y * e);
}
FF_HD ff ff_div(ff a, ff b) { return ff_mul(a, ff_rcp(b)); }

// sqrt(x) and 1/sqrt(x) for x > 0.
FF_HD void ff_sqrt_rsqrt(ff x, ff &r, ff &rinv) {
  const float y = 1.0f / sqrtf(x.hi);
  const float s = x.hi * y;
  const ff s2 = two_prod(s, s);
  const float d = ((x.hi - s2.hi) - s2.lo) + x.lo;  // x - s^2
  r = quick_two_sum(s, 0.5f * d * y);
  const ff xy = ff_mulf(x, y);
  const ff xyy = ff_mulf(xy, y);
  const float e = (1.0f - xyy.hi) - xyy.lo;  // 1 - x y^2
  rinv = quick_two_sum(y, 0.5f * y * e);
}

// ---------------------------------------------------------------------------
// exp: e^t = 2^(k/256) e^rho, k = round(256 t / ln 2), |rho| <= ln 2/512.
// tab[j] = 2^(j/256) as ff.  Relative error ~1e-12 for |t| < 80.
// ---------------------------------------------------------------------------
constexpr float kFfInvC = 369.32993f;               // 256 / ln 2 (only selects k)
constexpr float kFfC_hi = 0.0027076062f;            // ln 2 / 256 = hi + mid (+ 3e-19)
constexpr float kFfC_mid = -7.4400555e-12f;

// k = round(t / C) without conversion instructions: adding 1.5 * 2^23 leaves
// the rounded integer in the low mantissa bits (|t| < 1e4).
FF_HD int __float_as_int_hd(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_int(f);
#else
  int i;
  std::memcpy(&i, &f, sizeof i);
  return i;
#endif
}
constexpr float kFfRoundMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kFfRoundMagicBits = 0x4B400000;

FF_HD ff ff_exp(ff t, const ff *tab) {
  const float rv = fmaf(t.hi, kFfInvC, kFfRoundMagic);
  const float kf = rv - kFfRoundMagic;
  const int k = __float_as_int_hd(rv) - kFfRoundMagicBits;
  // rho = t - kf * C, C = C_hi + C_mid: kf * C_hi exact via two_prod, the
  // leading difference exact via two_sum, then the small parts; the tail
  // polynomial takes rho.lo to first order.
  const ff kc = two_prod(kf, kFfC_hi);
  const ff rh = two_sum(t.hi, -kc.hi);
  const ff rho = two_sum(rh.hi, rh.lo + ((t.lo - kc.lo) - kf * kFfC_mid));
  const float r = rho.hi, lo = rho.lo;
  const float tail = lo * (1.0f + r) +
                     r * r * (0.5f + r * (0.16666667f + r * (0.041666668f + r * 0.0083333338f)));
  const ff eps = two_sum(r, tail);  // e^rho - 1
  const ff T = tab[k & 255];
  const ff Te = ff_mul(T, eps);  // |T eps| < 0.006 T: fast two-sum below
  ff v = quick_two_sum(T.hi, Te.hi);
  v.lo += T.lo + Te.lo;
  v = quick_two_sum(v.hi, v.lo);
  const int e = k >> 8;
  if (e > -120 && e < 120) {
    const float sc = __int_as_float_hd((e + 127) << 23);  // 2^e, exact scaling
    v.hi *= sc;
    v.lo *= sc;
  } else {
    v.hi = ldexpf(v.hi, e);
    v.lo = ldexpf(v.lo, e);
  }
  return v;
}

// ln z for an ff z > 0: a start value l0 ~ ln z.hi, then
// ln z = l0 + log1p(w), w = z e^-l0 - 1, with log1p(w) = w - w^2/2 (|w| < 1e-5).
FF_HD ff ff_log(ff z, const ff *exptab) {
#ifdef __CUDA_ARCH__
  const float l0 = __logf(z.hi);
#else
  const float l0 = logf(z.hi);
#endif
  const ff e = ff_exp(ff_make(-l0, 0.0f), exptab);  // e^-l0
  const ff w = ff_addf(ff_mul(e, z), -1.0f);      // z e^-l0 - 1
  const ff lw = ff_addf(w, -0.5f * w.hi * w.hi);
  return ff_addf(lw, l0);
}

// ln z for a positive FP32 z.
FF_HD ff ff_log_f(float z, const ff *exptab) { return ff_log(ff_make(z, 0.0f), exptab); }

// ---------------------------------------------------------------------------
// sin, cos of x in [0, pi]: x = j (pi/256) + d, |d| <= pi/512;
// stab[j] = {sin, cos}(j pi / 256) as ff (j = 0..256).
// ---------------------------------------------------------------------------
constexpr float kFfPiOver256_hi = 0.012271847f;      // pi/256 = hi + lo (+ 1e-17)
constexpr float kFfPiOver256_lo = -3.4149522e-10f;
constexpr float kFf256OverPi = 81.48733f;

FF_HD void ff_sincos(ff x, const ff *stab_sin, const ff *stab_cos, ff &sx, ff &cx) {
  const float rv = fmaf(x.hi, kFf256OverPi, kFfRoundMagic);
  const float jf = rv - kFfRoundMagic;
  const int j = __float_as_int_hd(rv) - kFfRoundMagicBits;
  const ff jc = two_prod(jf, kFfPiOver256_hi);
  ff d = ff_sub(x, jc);
  d = ff_addf(d, -jf * kFfPiOver256_lo);
  const float dh = d.hi, d2 = dh * dh;
  // sin d = d - d^3/6 + d^5/120 ; cos d - 1 = -d^2/2 + d^4/24 - d^6/720
  const float sd_tail = d.lo - dh * d2 * (0.16666667f - d2 * 0.0083333338f);
  const ff sd = two_sum(dh, sd_tail);
  const float cm1 = -d2 * (0.5f - d2 * (0.041666668f - d2 * 0.0013888889f)) - dh * d.lo;
  const ff S = stab_sin[j], C = stab_cos[j];
  // sin x = S cos d + C sin d = S + S (cos d - 1) + C sin d
  sx = ff_add(S, ff_add(ff_mulf(S, cm1), ff_mul(C, sd)));
  // cos x = C cos d - S sin d = C + C (cos d - 1) - S sin d
  cx = ff_add(C, ff_sub(ff_mulf(C, cm1), ff_mul(S, sd)));
}

}  // namespace gb
