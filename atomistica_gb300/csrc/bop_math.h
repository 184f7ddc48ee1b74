// Functional forms of the Tersoff and Kumagai bond-order potentials, as
// __host__ __device__ functors templated on the arithmetic type of the
// three-body terms (double for the drop-in, float for the mixed form).
//
//   Tersoff   src/potentials/bop/tersoff/tersoff_func.f90:32-232
//   Kumagai   src/potentials/bop/kumagai/kumagai_func.f90:32-242
//   Brenner   src/potentials/bop/brenner/brenner_func.f90:32-225, derived
//             constants brenner_module.f90:196-214
//   trig_off  src/support/cutoff.f90:152-196
//   pair idx  src/macros.inc:123
//
// Two algebraic rewrites keep the FP32 form accurate (both are exact in real
// arithmetic):
//   * Tersoff g = omega*(1 + c^2/d^2 - c^2/(d^2+(h-cos)^2)) is evaluated as
//     omega*(1 + c^2 (h-cos)^2 / (d^2 (d^2+(h-cos)^2))): for Si, c^2/d^2 ~ 4e7
//     and the reference form cancels three digits.  The Brenner g (h + cos,
//     constants of the (i,k) pair) is the same function of hc = -h - cos.
//   * bo powers use exp(n log z): z^(n-1) = z^n / z, arg^(e-1) = arg^e / arg.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "../../include/atomistica_gb300.h"

namespace gb {

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

GB_HD int pair_index(int i, int j, int nel) {
  int a = i + j * nel, b = j + i * nel;
  int x = i * (i + 1) / 2, y = j * (j + 1) / 2;
  return (a < b ? a : b) - (x < y ? x : y);
}

template <class R>
GB_HD R gexp(R x);
template <>
GB_HD double gexp<double>(double x) {
  return exp(x);
}
template <>
GB_HD float gexp<float>(float x) {
  return expf(x);
}
template <class R>
GB_HD R glog(R x);
template <>
GB_HD double glog<double>(double x) {
  return log(x);
}
template <>
GB_HD float glog<float>(float x) {
  return logf(x);
}

// Parameters in the form the kernels consume (derived on the host from the
// reference layout, tersoff_params.f90 / kumagai_params.f90).
struct TersoffDev {
  int nel;
  double A[6], B[6], xi[6], lambda[6], mu[6], omega[6], mubo[6];
  int m[6];
  double r1[6], r2[6], r1sq[6], r2sq[6], fac[6];
  double n[3], e[3], betan[3], lbetan[3], c2[3], d2[3], c2d2inv[3], h[3];
};

struct KumagaiDev {
  int nel;
  double A[1], B[1], lambda1[1], lambda2[1];
  double eta[1], delta[1], alpha[1];
  int beta[1];
  double c1[1], c2[1], c3[1], c4[1], c5[1], h[1];
  double r1[1], r2[1], r1sq[1], r2sq[1], fac[1];
};

// Brenner form: every constant per symmetric pair; VR = VR_f e^{-expR (r-r0)},
// VA = -VA_f e^{-expA (r-r0)}, g from (gamma, c, d, -h) of the (i,k) pair,
// b = (1 + zeta^n)^bo_exp of the (i,j) pair, h(dr) as Tersoff with (mu, m).
// Arrays of 9: Juslin (below) keeps its constants per ordered pair.
struct BrennerDev {
  int nel;
  double r0[9], VR_f[9], VA_f[9], expR[9], expA[9];
  double gamma[9], c2[9], d2[9], c2d2inv[9], hneg[9];
  double n[9], bo_exp[9], bo_fac[9];
  double mu[9];
  int m[9];
  double r1[9], r2[9], r1sq[9], r2sq[9], fac[9];
};

inline BrennerDev make_brenner_dev(const gb_brenner_params_t &p) {
  BrennerDev d{};
  d.nel = p.nel;
  const int np = p.nel * (p.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    d.r0[q] = p.r0[q];
    d.expR[q] = p.beta[q] * std::sqrt(2 * p.S[q]);
    d.expA[q] = p.beta[q] * std::sqrt(2 / p.S[q]);
    d.VR_f[q] = p.D0[q] / (p.S[q] - 1);
    d.VA_f[q] = p.S[q] * p.D0[q] / (p.S[q] - 1);
    d.gamma[q] = p.gamma[q];
    d.c2[q] = p.c[q] * p.c[q];
    d.d2[q] = p.d[q] * p.d[q];
    d.c2d2inv[q] = d.c2[q] / d.d2[q];
    d.hneg[q] = -p.h[q];
    d.n[q] = p.n[q];
    d.bo_exp[q] = -0.5 / p.n[q];
    d.bo_fac[q] = 0.5 * d.bo_exp[q] * p.n[q];
    d.mu[q] = p.mu[q];
    d.m[q] = p.m[q];
    d.r1[q] = p.r1[q];
    d.r2[q] = p.r2[q];
    d.r1sq[q] = p.r1[q] * p.r1[q];
    d.r2sq[q] = p.r2[q] * p.r2[q];
    d.fac[q] = M_PI / (p.r2[q] - p.r1[q]);
  }
  return d;
}

// Juslin form (juslin_func.f90, juslin_module.f90:322-377): the Brenner
// functions with every pair constant per ORDERED element pair (t = j + i nel,
// src/macros.inc:139) and h(dr) = omega e^{(alpha dr)^m} with (alpha, omega,
// m) per element triplet (k + nel (j + nel i), src/macros.inc:146).
struct JuslinDev : BrennerDev {
  double alpha[27], omega[27];
  int m3[27];
};

inline JuslinDev make_juslin_dev(const gb_juslin_params_t &p) {
  JuslinDev d{};
  d.nel = p.nel;
  const int np = p.nel * p.nel;
  for (int q = 0; q < np; q++) {
    d.r0[q] = p.r0[q];
    d.expR[q] = p.beta[q] * std::sqrt(2 * p.S[q]);
    d.expA[q] = p.beta[q] * std::sqrt(2 / p.S[q]);
    d.VR_f[q] = p.D0[q] / (p.S[q] - 1);
    d.VA_f[q] = p.S[q] * p.D0[q] / (p.S[q] - 1);
    d.gamma[q] = p.gamma[q];
    d.c2[q] = p.c[q] * p.c[q];
    d.d2[q] = p.d[q] * p.d[q];
    d.c2d2inv[q] = d.c2[q] / d.d2[q];
    d.hneg[q] = -p.h[q];
    d.n[q] = p.n[q];
    d.bo_exp[q] = -0.5 / p.n[q];
    d.bo_fac[q] = 0.5 * d.bo_exp[q] * p.n[q];
    d.r1[q] = p.r1[q];
    d.r2[q] = p.r2[q];
    d.r1sq[q] = p.r1[q] * p.r1[q];
    d.r2sq[q] = p.r2[q] * p.r2[q];
    d.fac[q] = M_PI / (p.r2[q] - p.r1[q]);
  }
  for (int q = 0; q < np * p.nel; q++) {
    d.alpha[q] = p.alpha[q];
    d.omega[q] = p.omega[q];
    d.m3[q] = p.m[q];
  }
  return d;
}

inline TersoffDev make_tersoff_dev(const gb_tersoff_params_t &p) {
  TersoffDev d{};
  d.nel = p.nel;
  const int np = p.nel * (p.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    d.A[q] = p.A[q];
    d.B[q] = p.B[q];
    d.xi[q] = p.xi[q];
    d.lambda[q] = p.lambda[q];
    d.mu[q] = p.mu[q];
    d.omega[q] = p.omega[q];
    d.mubo[q] = p.mubo[q];
    d.m[q] = p.m[q];
    d.r1[q] = p.r1[q];
    d.r2[q] = p.r2[q];
    d.r1sq[q] = p.r1[q] * p.r1[q];
    d.r2sq[q] = p.r2[q] * p.r2[q];
    d.fac[q] = M_PI / (p.r2[q] - p.r1[q]);
  }
  for (int q = 0; q < p.nel; q++) {
    d.n[q] = p.n[q];
    d.e[q] = -0.5 / p.n[q];
    d.betan[q] = std::pow(p.beta[q], p.n[q]);
    d.lbetan[q] = p.n[q] * std::log(p.beta[q]);
    d.c2[q] = p.c[q] * p.c[q];
    d.d2[q] = p.d[q] * p.d[q];
    d.c2d2inv[q] = p.c[q] * p.c[q] / (p.d[q] * p.d[q]);
    d.h[q] = p.h[q];
  }
  return d;
}

inline KumagaiDev make_kumagai_dev(const gb_kumagai_params_t &p) {
  KumagaiDev d{};
  d.nel = 1;
  d.A[0] = p.A[0];
  d.B[0] = p.B[0];
  d.lambda1[0] = p.lambda1[0];
  d.lambda2[0] = p.lambda2[0];
  d.eta[0] = p.eta[0];
  d.delta[0] = p.delta[0];
  d.alpha[0] = p.alpha[0];
  d.beta[0] = p.beta[0];
  d.c1[0] = p.c1[0];
  d.c2[0] = p.c2[0];
  d.c3[0] = p.c3[0];
  d.c4[0] = p.c4[0];
  d.c5[0] = p.c5[0];
  d.h[0] = p.h[0];
  d.r1[0] = p.r1[0];
  d.r2[0] = p.r2[0];
  d.r1sq[0] = p.r1[0] * p.r1[0];
  d.r2sq[0] = p.r2[0] * p.r2[0];
  d.fac[0] = M_PI / (p.r2[0] - p.r1[0]);
  return d;
}

// trig_off_f (cutoff.f90:171-196): r <= r1 -> (1,0); r >= r2 -> (0,0).
GB_HD void trig_off(double r, double r1, double r2, double fac, double &val, double &dval) {
  if (r <= r1) {
    val = 1.0;
    dval = 0.0;
  } else if (r >= r2) {
    val = 0.0;
    dval = 0.0;
  } else {
    const double x = fac * (r - r1);
    double s, c;
#ifdef __CUDA_ARCH__
    sincos(x, &s, &c);
#else
    s = std::sin(x);
    c = std::cos(x);
#endif
    val = 0.5 * (1.0 + c);
    dval = -0.5 * fac * s;
  }
}

struct TersoffPot {
  static constexpr bool kTripletH = false;  // h constants per element triplet
  // g and b constants per centre element (false) or per element pair (true)
  static constexpr bool kPairTerms = false;
  TersoffDev p;
  GB_HD int nel() const { return p.nel; }
  GB_HD int pair(int i, int j) const { return pair_index(i, j, p.nel); }
  GB_HD double r1(int t) const { return p.r1[t]; }
  GB_HD double r2(int t) const { return p.r2[t]; }
  GB_HD double r1sq(int t) const { return p.r1sq[t]; }
  GB_HD double r2sq(int t) const { return p.r2sq[t]; }
  GB_HD double fac(int t) const { return p.fac[t]; }
  // VA, VR (tersoff_func.f90:32-78): FP64 in both forms.
  GB_HD void VA(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.mu[t] * r);
    v = -p.B[t] * ex;
    dv = p.B[t] * p.mu[t] * ex;
  }
  GB_HD void VR(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.lambda[t] * r);
    v = p.A[t] * ex;
    dv = -p.A[t] * p.lambda[t] * ex;
  }
  // g(cos theta) (tersoff_func.f90:86-114), element of the centre atom.
  template <class R>
  GB_HD void g(int eli, int ikpot, R cs, R &val, R &dval) const {
    const R om = (R)p.omega[ikpot];
    const R hc = (R)p.h[eli] - cs;
    const R d2 = (R)p.d2[eli];
    const R den = d2 + hc * hc;
    const R inv = R(1) / den;
    val = om * (R(1) + (R)p.c2d2inv[eli] * hc * hc * inv);
    dval = R(-2) * om * (R)p.c2[eli] * hc * inv * inv;
  }
  // g as a function of hc = h - cos theta (the mixed form evaluates hc from
  // FP64 unit vectors).
  template <class R>
  GB_HD void g_hc(int eli, int ikpot, R hc, R &val, R &dval) const {
    const R om = (R)p.omega[ikpot];
    const R d2 = (R)p.d2[eli];
    const R den = d2 + hc * hc;
    const R inv = R(1) / den;
    val = om * (R(1) + (R)p.c2d2inv[eli] * hc * hc * inv);
    dval = R(-2) * om * (R)p.c2[eli] * hc * inv * inv;
  }
  // h - cos theta is the argument of g_hc (centre element; the pair is unused)
  GB_HD double hpar(int eli, int /*ikpot*/) const { return p.h[eli]; }
  // h(r_ij - r_ik) (tersoff_func.f90:168-211), pair (i,k).
  template <class R>
  GB_HD void h(int /*eli*/, int /*ijpot*/, int ikpot, R dr, R &val, R &dval) const {
    const double mu = p.mubo[ikpot];
    if (mu == 0.0) {
      val = R(1);
      dval = R(0);
      return;
    }
    const int m = p.m[ikpot];
    const R mu2 = R(2) * (R)mu;
    if (m == 1) {
      val = gexp<R>(mu2 * dr);
      dval = mu2 * val;
    } else if (m == 3) {
      const R arg = mu2 * dr;
      val = gexp<R>(arg * arg * arg);
      dval = mu2 * R(m) * arg * arg * val;
    } else {
      const R arg = mu2 * dr;
      R pw = R(1);
      for (int q = 0; q < m - 1; q++) pw *= arg;
      val = gexp<R>(pw * arg);
      dval = mu2 * R(m) * pw * val;
    }
  }
  // Pair-term coefficients: VA = -Bc e^{-cA r}, VR = Ac e^{-cR r}.
  GB_HD double cA(int t) const { return p.mu[t]; }
  GB_HD double Bc(int t) const { return p.B[t]; }
  GB_HD double cR(int t) const { return p.lambda[t]; }
  GB_HD double Ac(int t) const { return p.A[t]; }
#ifdef __CUDACC__
  // |d ln b / d ln zeta| (for the mixed form's error estimate).
  __device__ __forceinline__ float bsens(int eli, float zeta) const {
    if (!(zeta > 0.0f)) return 0.0f;
    const float x = (float)p.betan[eli] * __expf((float)p.n[eli] * __logf(zeta));
    return fabsf((float)(p.e[eli] * p.n[eli])) * x / (1.0f + x);
  }
#endif
  // bo (tersoff_func.f90:122-160): b = xi (1 + beta^n z^n)^(-1/(2n)),
  // dfb = -1/4 fc VA xi beta^n z^(n-1) arg^(e-1).
  template <class R>
  GB_HD void bo(int eli, int t, R z, R fc, R VA, R &b, R &dfb) const {
    if (z > R(0)) {
      const R n = (R)p.n[eli], e = (R)p.e[eli], bn = (R)p.betan[eli];
      const R zn = gexp<R>(n * glog<R>(z));
      const R arg = R(1) + bn * zn;
      const R ae = gexp<R>(e * glog<R>(arg));
      b = (R)p.xi[t] * ae;
      dfb = R(-0.25) * fc * VA * (R)p.xi[t] * bn * (zn / z) * (ae / arg);
    } else {
      b = R(1);
      dfb = R(0);
    }
  }
};

struct KumagaiPot {
  static constexpr bool kTripletH = false;  // h constants per element triplet
  static constexpr bool kPairTerms = false;
  KumagaiDev p;
  GB_HD double hpar(int eli, int /*ikpot*/) const { return p.h[eli]; }
  // g as a function of hc = h - cos theta.
  template <class R>
  GB_HD void g_hc(int eli, int /*ikpot*/, R hcos, R &val, R &dval) const {
    const R c1 = (R)p.c1[eli], c2 = (R)p.c2[eli], c3 = (R)p.c3[eli], c4 = (R)p.c4[eli],
            c5 = (R)p.c5[eli];
    const R hcos2 = hcos * hcos;
    const R tmp = hcos / (c3 + hcos2);
    const R go = c2 * tmp;
    const R ga1 = c4 * gexp<R>(-c5 * hcos2);
    const R v = go * (R(1) + ga1);
    dval = R(-2) * (R(1) - hcos * tmp) * v + R(2) * c5 * hcos2 * go * ga1;
    val = c1 + hcos * v;
  }
  GB_HD int nel() const { return 1; }
  GB_HD int pair(int /*i*/, int /*j*/) const { return 0; }
  GB_HD double r1(int t) const { return p.r1[t]; }
  GB_HD double r2(int t) const { return p.r2[t]; }
  GB_HD double r1sq(int t) const { return p.r1sq[t]; }
  GB_HD double r2sq(int t) const { return p.r2sq[t]; }
  GB_HD double fac(int t) const { return p.fac[t]; }
  GB_HD void VA(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.lambda2[t] * r);
    v = -p.B[t] * ex;
    dv = p.B[t] * p.lambda2[t] * ex;
  }
  GB_HD void VR(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.lambda1[t] * r);
    v = p.A[t] * ex;
    dv = -p.A[t] * p.lambda1[t] * ex;
  }
  // g (kumagai_func.f90:86-131).
  template <class R>
  GB_HD void g(int eli, int /*ikpot*/, R cs, R &val, R &dval) const {
    const R c1 = (R)p.c1[eli], c2 = (R)p.c2[eli], c3 = (R)p.c3[eli], c4 = (R)p.c4[eli],
            c5 = (R)p.c5[eli], hh = (R)p.h[eli];
    const R hcos = hh - cs;
    const R hcos2 = hcos * hcos;
    const R tmp = hcos / (c3 + hcos2);
    const R go = c2 * tmp;
    const R ga1 = c4 * gexp<R>(-c5 * hcos2);
    const R v = go * (R(1) + ga1);
    dval = R(-2) * (R(1) - hcos * tmp) * v + R(2) * c5 * hcos2 * go * ga1;
    val = c1 + hcos * v;
  }
  // h (kumagai_func.f90:179-221); the beta == 3 branch omits alpha in the
  // exponent exactly as the reference does (:211-213).
  template <class R>
  GB_HD void h(int /*eli*/, int /*ijpot*/, int ikpot, R dr, R &val, R &dval) const {
    const R alpha = (R)p.alpha[ikpot];
    if (p.alpha[ikpot] == 0.0) {
      val = R(1);
      dval = R(0);
      return;
    }
    const int beta = p.beta[ikpot];
    if (beta == 1) {
      val = gexp<R>(alpha * dr);
      dval = alpha * val;
    } else if (beta == 3) {
      val = gexp<R>(dr * dr * dr);
      dval = R(3) * alpha * dr * dr * val;
    } else {
      R pw = R(1);
      for (int q = 0; q < beta - 1; q++) pw *= dr;
      val = gexp<R>(alpha * pw * dr);
      dval = R(beta) * alpha * pw * val;
    }
  }
  GB_HD double cA(int t) const { return p.lambda2[t]; }
  GB_HD double Bc(int t) const { return p.B[t]; }
  GB_HD double cR(int t) const { return p.lambda1[t]; }
  GB_HD double Ac(int t) const { return p.A[t]; }
#ifdef __CUDACC__
  __device__ __forceinline__ float bsens(int eli, float zeta) const {
    if (!(zeta > 0.0f)) return 0.0f;
    const float x = __expf((float)p.eta[eli] * __logf(zeta));
    return fabsf((float)(p.delta[eli] * p.eta[eli])) * x / (1.0f + x);
  }
#endif
  // bo (kumagai_func.f90:139-171): b = (1 + z^eta)^(-delta).
  template <class R>
  GB_HD void bo(int eli, int /*t*/, R z, R fc, R VA, R &b, R &dfb) const {
    if (z > R(0)) {
      const R eta = (R)p.eta[eli], delta = -(R)p.delta[eli];
      const R ze = gexp<R>(eta * glog<R>(z));
      const R arg = R(1) + ze;
      const R ad = gexp<R>(delta * glog<R>(arg));
      b = ad;
      dfb = R(0.5) * fc * VA * eta * (ze / z) * delta * (ad / arg);
    } else {
      b = R(1);
      dfb = R(0);
    }
  }
};

struct BrennerPot {
  static constexpr bool kTripletH = false;  // h constants per element triplet
  static constexpr bool kPairTerms = true;
  BrennerDev p;
  GB_HD int nel() const { return p.nel; }
  GB_HD int pair(int i, int j) const { return pair_index(i, j, p.nel); }
  GB_HD double r1(int t) const { return p.r1[t]; }
  GB_HD double r2(int t) const { return p.r2[t]; }
  GB_HD double r1sq(int t) const { return p.r1sq[t]; }
  GB_HD double r2sq(int t) const { return p.r2sq[t]; }
  GB_HD double fac(int t) const { return p.fac[t]; }
  // VA, VR (brenner_func.f90:32-78)
  GB_HD void VA(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.expA[t] * (r - p.r0[t]));
    v = -p.VA_f[t] * ex;
    dv = p.VA_f[t] * p.expA[t] * ex;
  }
  GB_HD void VR(int t, double r, double &v, double &dv) const {
    const double ex = exp(-p.expR[t] * (r - p.r0[t]));
    v = p.VR_f[t] * ex;
    dv = -p.VR_f[t] * p.expR[t] * ex;
  }
  // g as a function of hc = -h - cos theta of the (i,k) pair
  template <class R>
  GB_HD void g_hc(int /*eli*/, int ikpot, R hc, R &val, R &dval) const {
    const R ga = (R)p.gamma[ikpot];
    const R inv = R(1) / ((R)p.d2[ikpot] + hc * hc);
    val = ga * (R(1) + (R)p.c2d2inv[ikpot] * hc * hc * inv);
    dval = R(-2) * ga * (R)p.c2[ikpot] * hc * inv * inv;
  }
  // g(cos theta) (brenner_func.f90:86-103)
  template <class R>
  GB_HD void g(int eli, int ikpot, R cs, R &val, R &dval) const {
    g_hc<R>(eli, ikpot, (R)p.hneg[ikpot] - cs, val, dval);
  }
  GB_HD double hpar(int /*eli*/, int ikpot) const { return p.hneg[ikpot]; }
  // h (brenner_func.f90:178-214), pair (i,k)
  template <class R>
  GB_HD void h(int /*eli*/, int /*ijpot*/, int ikpot, R dr, R &val, R &dval) const {
    const double mu = p.mu[ikpot];
    if (mu == 0.0) {
      val = R(1);
      dval = R(0);
      return;
    }
    const int m = p.m[ikpot];
    const R mu2 = R(2) * (R)mu;
    if (m == 1) {
      val = gexp<R>(mu2 * dr);
      dval = mu2 * val;
    } else {
      const R arg = mu2 * dr;
      R pw = R(1);
      for (int q = 0; q < m - 1; q++) pw *= arg;
      val = gexp<R>(pw * arg);
      dval = mu2 * R(m) * pw * val;
    }
  }
  // bo (brenner_func.f90:122-170) of the (i,j) pair: b = (1 + zeta^n)^(-1/(2n)),
  // dfb = -1/4 fc VA zeta^(n-1) (1 + zeta^n)^(-1/(2n)-1); n = 1 without the
  // zeta > 0 test.
  template <class R>
  GB_HD void bo(int /*eli*/, int t, R z, R fc, R VA, R &b, R &dfb) const {
    const R e = (R)p.bo_exp[t];
    if (p.n[t] == 1.0) {
      const R arg = R(1) + z;
      b = gexp<R>(e * glog<R>(arg));
      dfb = (R)p.bo_fac[t] * fc * VA * (b / arg);
    } else if (z > R(0)) {
      const R zn = gexp<R>((R)p.n[t] * glog<R>(z));
      const R arg = R(1) + zn;
      b = gexp<R>(e * glog<R>(arg));
      dfb = (R)p.bo_fac[t] * fc * VA * (zn / z) * (b / arg);
    } else {
      b = R(1);
      dfb = R(0);
    }
  }
};

// Juslin: Brenner's VA, VR, g and b on ordered pairs; h per triplet
// (juslin_func.f90:257-294).  For pairs t = j + i nel the triplet (i, j, k)
// of bonds ij (t) and ik (ikpot) is ikpot + nel (t - i).
struct JuslinPot : BrennerPot {
  static constexpr bool kTripletH = true;
  double alpha[27], omega[27];
  int m3[27];
  explicit JuslinPot(const JuslinDev &d) : BrennerPot{d} {
    for (int q = 0; q < 27; q++) {
      alpha[q] = d.alpha[q];
      omega[q] = d.omega[q];
      m3[q] = d.m3[q];
    }
  }
  GB_HD int pair(int i, int j) const { return j + i * p.nel; }
  template <class R>
  GB_HD void h(int eli, int ijpot, int ikpot, R dr, R &val, R &dval) const {
    const int q = ikpot + p.nel * (ijpot - eli);
    const R al = (R)alpha[q], om = (R)omega[q];
    const int m = m3[q];
    if (m == 1) {
      val = om * gexp<R>(al * dr);
      dval = al * val;
    } else if (m == 3) {
      const R arg = al * dr;
      val = om * gexp<R>(arg * arg * arg);
      dval = R(3) * al * arg * arg * val;
    } else {
      const R arg = al * dr;
      R pw = R(1);
      for (int k = 0; k < m - 1; k++) pw *= arg;
      val = om * gexp<R>(pw * arg);
      dval = R(m) * pw * al * val;
    }
  }
};

}  // namespace gb
