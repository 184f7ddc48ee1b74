// Functional forms of the Tersoff and Kumagai bond-order potentials, as
// __host__ __device__ functors templated on the arithmetic type of the
// three-body terms (double for the drop-in, float for the mixed form).
//
//   Tersoff   src/potentials/bop/tersoff/tersoff_func.f90:32-232
//   Kumagai   src/potentials/bop/kumagai/kumagai_func.f90:32-242
//   trig_off  src/support/cutoff.f90:152-196
//   pair idx  src/macros.inc:123
//
// Two algebraic rewrites keep the FP32 form accurate (both are exact in real
// arithmetic):
//   * Tersoff g = omega*(1 + c^2/d^2 - c^2/(d^2+(h-cos)^2)) is evaluated as
//     omega*(1 + c^2 (h-cos)^2 / (d^2 (d^2+(h-cos)^2))): for Si, c^2/d^2 ~ 4e7
//     and the reference form cancels three digits.
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

// ---------------------------------------------------------------------------
// Accurate exponential for the mixed form: e^t = 2^(k/256) e^rho with
// k = floor(256 t / ln 2) and 0 <= rho < ln 2 / 256.  2^(j/256) comes from a
// 256-entry FP64 table (in shared memory), e^rho - 1 from a degree-4
// polynomial in FP32 (|rho| < 0.0028, so its FP32 rounding is ~3e-10
// relative to e^t).  About six FP64 operations instead of the ~25 of exp().
// Valid for |t| < 700.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
// 2^(j/256), j = 0..255, correctly rounded.
static __device__ const double kExp2Tab[256] = {
    0x1.0000000000000p+0, 0x1.00b1afa5abcbfp+0, 0x1.0163da9fb3335p+0, 0x1.02168143b0281p+0,
    0x1.02c9a3e778061p+0, 0x1.037d42e11bbccp+0, 0x1.04315e86e7f85p+0, 0x1.04e5f72f654b1p+0,
    0x1.059b0d3158574p+0, 0x1.0650a0e3c1f89p+0, 0x1.0706b29ddf6dep+0, 0x1.07bd42b72a836p+0,
    0x1.0874518759bc8p+0, 0x1.092bdf66607e0p+0, 0x1.09e3ecac6f383p+0, 0x1.0a9c79b1f3919p+0,
    0x1.0b5586cf9890fp+0, 0x1.0c0f145e46c85p+0, 0x1.0cc922b7247f7p+0, 0x1.0d83b23395decp+0,
    0x1.0e3ec32d3d1a2p+0, 0x1.0efa55fdfa9c5p+0, 0x1.0fb66affed31bp+0, 0x1.1073028d7233ep+0,
    0x1.11301d0125b51p+0, 0x1.11edbab5e2ab6p+0, 0x1.12abdc06c31ccp+0, 0x1.136a814f204abp+0,
    0x1.1429aaea92de0p+0, 0x1.14e95934f312ep+0, 0x1.15a98c8a58e51p+0, 0x1.166a45471c3c2p+0,
    0x1.172b83c7d517bp+0, 0x1.17ed48695bbc0p+0, 0x1.18af9388c8deap+0, 0x1.1972658375d2fp+0,
    0x1.1a35beb6fcb75p+0, 0x1.1af99f8138a1cp+0, 0x1.1bbe084045cd4p+0, 0x1.1c82f95281c6bp+0,
    0x1.1d4873168b9aap+0, 0x1.1e0e75eb44027p+0, 0x1.1ed5022fcd91dp+0, 0x1.1f9c18438ce4dp+0,
    0x1.2063b88628cd6p+0, 0x1.212be3578a819p+0, 0x1.21f49917ddc96p+0, 0x1.22bdda27912d1p+0,
    0x1.2387a6e756238p+0, 0x1.2451ffb82140ap+0, 0x1.251ce4fb2a63fp+0, 0x1.25e85711ece75p+0,
    0x1.26b4565e27cddp+0, 0x1.2780e341ddf29p+0, 0x1.284dfe1f56381p+0, 0x1.291ba7591bb70p+0,
    0x1.29e9df51fdee1p+0, 0x1.2ab8a66d10f13p+0, 0x1.2b87fd0dad990p+0, 0x1.2c57e39771b2fp+0,
    0x1.2d285a6e4030bp+0, 0x1.2df961f641589p+0, 0x1.2ecafa93e2f56p+0, 0x1.2f9d24abd886bp+0,
    0x1.306fe0a31b715p+0, 0x1.31432edeeb2fdp+0, 0x1.32170fc4cd831p+0, 0x1.32eb83ba8ea32p+0,
    0x1.33c08b26416ffp+0, 0x1.3496266e3fa2dp+0, 0x1.356c55f929ff1p+0, 0x1.36431a2de883bp+0,
    0x1.371a7373aa9cbp+0, 0x1.37f26231e754ap+0, 0x1.38cae6d05d866p+0, 0x1.39a401b7140efp+0,
    0x1.3a7db34e59ff7p+0, 0x1.3b57fbfec6cf4p+0, 0x1.3c32dc313a8e5p+0, 0x1.3d0e544ede173p+0,
    0x1.3dea64c123422p+0, 0x1.3ec70df1c5175p+0, 0x1.3fa4504ac801cp+0, 0x1.40822c367a024p+0,
    0x1.4160a21f72e2ap+0, 0x1.423fb2709468ap+0, 0x1.431f5d950a897p+0, 0x1.43ffa3f84b9d4p+0,
    0x1.44e086061892dp+0, 0x1.45c2042a7d232p+0, 0x1.46a41ed1d0057p+0, 0x1.4786d668b3237p+0,
    0x1.486a2b5c13cd0p+0, 0x1.494e1e192aed2p+0, 0x1.4a32af0d7d3dep+0, 0x1.4b17dea6db7d7p+0,
    0x1.4bfdad5362a27p+0, 0x1.4ce41b817c114p+0, 0x1.4dcb299fddd0dp+0, 0x1.4eb2d81d8abffp+0,
    0x1.4f9b2769d2ca7p+0, 0x1.508417f4531eep+0, 0x1.516daa2cf6642p+0, 0x1.5257de83f4eefp+0,
    0x1.5342b569d4f82p+0, 0x1.542e2f4f6ad27p+0, 0x1.551a4ca5d920fp+0, 0x1.56070dde910d2p+0,
    0x1.56f4736b527dap+0, 0x1.57e27dbe2c4cfp+0, 0x1.58d12d497c7fdp+0, 0x1.59c0827ff07ccp+0,
    0x1.5ab07dd485429p+0, 0x1.5ba11fba87a03p+0, 0x1.5c9268a5946b7p+0, 0x1.5d84590998b93p+0,
    0x1.5e76f15ad2148p+0, 0x1.5f6a320dceb71p+0, 0x1.605e1b976dc09p+0, 0x1.6152ae6cdf6f4p+0,
    0x1.6247eb03a5585p+0, 0x1.633dd1d1929fdp+0, 0x1.6434634ccc320p+0, 0x1.652b9febc8fb7p+0,
    0x1.6623882552225p+0, 0x1.671c1c70833f6p+0, 0x1.68155d44ca973p+0, 0x1.690f4b19e9538p+0,
    0x1.6a09e667f3bcdp+0, 0x1.6b052fa75173ep+0, 0x1.6c012750bdabfp+0, 0x1.6cfdcddd47645p+0,
    0x1.6dfb23c651a2fp+0, 0x1.6ef9298593ae5p+0, 0x1.6ff7df9519484p+0, 0x1.70f7466f42e87p+0,
    0x1.71f75e8ec5f74p+0, 0x1.72f8286ead08ap+0, 0x1.73f9a48a58174p+0, 0x1.74fbd35d7cbfdp+0,
    0x1.75feb564267c9p+0, 0x1.77024b1ab6e09p+0, 0x1.780694fde5d3fp+0, 0x1.790b938ac1cf6p+0,
    0x1.7a11473eb0187p+0, 0x1.7b17b0976cfdbp+0, 0x1.7c1ed0130c132p+0, 0x1.7d26a62ff86f0p+0,
    0x1.7e2f336cf4e62p+0, 0x1.7f3878491c491p+0, 0x1.80427543e1a12p+0, 0x1.814d2add106d9p+0,
    0x1.82589994cce13p+0, 0x1.8364c1eb941f7p+0, 0x1.8471a4623c7adp+0, 0x1.857f4179f5b21p+0,
    0x1.868d99b4492edp+0, 0x1.879cad931a436p+0, 0x1.88ac7d98a6699p+0, 0x1.89bd0a478580fp+0,
    0x1.8ace5422aa0dbp+0, 0x1.8be05bad61778p+0, 0x1.8cf3216b5448cp+0, 0x1.8e06a5e0866d9p+0,
    0x1.8f1ae99157736p+0, 0x1.902fed0282c8ap+0, 0x1.9145b0b91ffc6p+0, 0x1.925c353aa2fe2p+0,
    0x1.93737b0cdc5e5p+0, 0x1.948b82b5f98e5p+0, 0x1.95a44cbc8520fp+0, 0x1.96bdd9a7670b3p+0,
    0x1.97d829fde4e50p+0, 0x1.98f33e47a22a2p+0, 0x1.9a0f170ca07bap+0, 0x1.9b2bb4d53fe0dp+0,
    0x1.9c49182a3f090p+0, 0x1.9d674194bb8d5p+0, 0x1.9e86319e32323p+0, 0x1.9fa5e8d07f29ep+0,
    0x1.a0c667b5de565p+0, 0x1.a1e7aed8eb8bbp+0, 0x1.a309bec4a2d33p+0, 0x1.a42c980460ad8p+0,
    0x1.a5503b23e255dp+0, 0x1.a674a8af46052p+0, 0x1.a799e1330b358p+0, 0x1.a8bfe53c12e59p+0,
    0x1.a9e6b5579fdbfp+0, 0x1.ab0e521356ebap+0, 0x1.ac36bbfd3f37ap+0, 0x1.ad5ff3a3c2774p+0,
    0x1.ae89f995ad3adp+0, 0x1.afb4ce622f2ffp+0, 0x1.b0e07298db666p+0, 0x1.b20ce6c9a8952p+0,
    0x1.b33a2b84f15fbp+0, 0x1.b468415b749b1p+0, 0x1.b59728de5593ap+0, 0x1.b6c6e29f1c52ap+0,
    0x1.b7f76f2fb5e47p+0, 0x1.b928cf22749e4p+0, 0x1.ba5b030a1064ap+0, 0x1.bb8e0b79a6f1fp+0,
    0x1.bcc1e904bc1d2p+0, 0x1.bdf69c3f3a207p+0, 0x1.bf2c25bd71e09p+0, 0x1.c06286141b33dp+0,
    0x1.c199bdd85529cp+0, 0x1.c2d1cd9fa652cp+0, 0x1.c40ab5fffd07ap+0, 0x1.c544778fafb22p+0,
    0x1.c67f12e57d14bp+0, 0x1.c7ba88988c933p+0, 0x1.c8f6d9406e7b5p+0, 0x1.ca3405751c4dbp+0,
    0x1.cb720dcef9069p+0, 0x1.ccb0f2e6d1675p+0, 0x1.cdf0b555dc3fap+0, 0x1.cf3155b5bab74p+0,
    0x1.d072d4a07897cp+0, 0x1.d1b532b08c968p+0, 0x1.d2f87080d89f2p+0, 0x1.d43c8eacaa1d6p+0,
    0x1.d5818dcfba487p+0, 0x1.d6c76e862e6d3p+0, 0x1.d80e316c98398p+0, 0x1.d955d71ff6075p+0,
    0x1.da9e603db3285p+0, 0x1.dbe7cd63a8315p+0, 0x1.dd321f301b460p+0, 0x1.de7d5641c0658p+0,
    0x1.dfc97337b9b5fp+0, 0x1.e11676b197d17p+0, 0x1.e264614f5a129p+0, 0x1.e3b333b16ee12p+0,
    0x1.e502ee78b3ff6p+0, 0x1.e653924676d76p+0, 0x1.e7a51fbc74c83p+0, 0x1.e8f7977cdb740p+0,
    0x1.ea4afa2a490dap+0, 0x1.eb9f4867cca6ep+0, 0x1.ecf482d8e67f1p+0, 0x1.ee4aaa2188510p+0,
    0x1.efa1bee615a27p+0, 0x1.f0f9c1cb6412ap+0, 0x1.f252b376bba97p+0, 0x1.f3ac948dd7274p+0,
    0x1.f50765b6e4540p+0, 0x1.f6632798844f8p+0, 0x1.f7bfdad9cbe14p+0, 0x1.f91d802243c89p+0,
    0x1.fa7c1819e90d8p+0, 0x1.fbdba3692d514p+0, 0x1.fd3c22b8f71f1p+0, 0x1.fe9d96b2a23d9p+0,
};

__device__ __forceinline__ double exp_acc(double t, const double *__restrict__ tab2) {
  const double kScale = 369.3299304675746;           // 256 / ln 2
  const double kC_hi = 2.7076061740622863e-03;       // ln 2 / 256, high part
  const double kC_lo = 9.058776616587108e-20;        // low part
  const double kf = floor(t * kScale);
  const int k = (int)kf;
  double rho = fma(-kf, kC_hi, t);
  rho = fma(-kf, kC_lo, rho);
  const float r = (float)rho;
  const float eps = r * (1.0f + r * (0.5f + r * (0.16666667f + r * 0.041666668f)));
  const double T = tab2[k & 255];
  const double v = fma(T, (double)eps, T);
  const long long e = (long long)((k >> 8) + 1023) << 52;
  return v * __longlong_as_double(e);
}
#endif

struct TersoffPot {
  TersoffDev p;
  GB_HD int nel() const { return p.nel; }
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
  GB_HD double hpar(int eli) const { return p.h[eli]; }
  // h(r_ij - r_ik) (tersoff_func.f90:168-211), pair (i,k).
  template <class R>
  GB_HD void h(int ikpot, R dr, R &val, R &dval) const {
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
  // Bond order of the mixed form from an FP32 zeta, accurate to ~1e-9
  // relative: ln zeta by one Newton step on logf, x = beta^n zeta^n and P from
  // exp_acc, b = xi (1 + expm1(e log1p(x))) combined in FP64.
  __device__ __forceinline__ void bo_mixed(int eli, int t, float zeta, double fc, double VA,
                                           const double *tab2, double &b, double &P) const {
    if (!(zeta > 0.0f)) {
      b = 1.0;
      P = 0.0;
      return;
    }
    const float l0 = logf(zeta);
    const double lnz = (double)l0 + fma((double)zeta, exp_acc(-(double)l0, tab2), -1.0);
    const double tx = fma(p.n[eli], lnz, p.lbetan[eli]);
    const double x = exp_acc(tx, tab2);
    const float L = log1pf((float)x);
    const float u = (float)p.e[eli] * L;
    b = p.xi[t] * (1.0 + (double)expm1f(u));
    const double arg = (tx - lnz) + (double)((float)(p.e[eli] - 1.0) * L);
    P = -0.25 * fc * VA * p.xi[t] * exp_acc(arg, tab2);
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
  KumagaiDev p;
  GB_HD double hpar(int eli) const { return p.h[eli]; }
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
  GB_HD void h(int ikpot, R dr, R &val, R &dval) const {
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
  // Bond order of the mixed form (see TersoffPot::bo_mixed).
  __device__ __forceinline__ void bo_mixed(int eli, int /*t*/, float zeta, double fc, double VA,
                                           const double *tab2, double &b, double &P) const {
    if (!(zeta > 0.0f)) {
      b = 1.0;
      P = 0.0;
      return;
    }
    const float l0 = logf(zeta);
    const double lnz = (double)l0 + fma((double)zeta, exp_acc(-(double)l0, tab2), -1.0);
    const double eta = p.eta[eli], delta = p.delta[eli];
    const double x = exp_acc(eta * lnz, tab2);
    const float L = log1pf((float)x);
    b = 1.0 + (double)expm1f((float)(-delta) * L);
    const double arg = (eta - 1.0) * lnz + (double)((float)(-delta - 1.0) * L);
    P = 0.5 * fc * VA * eta * (-delta) * exp_acc(arg, tab2);
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

}  // namespace gb
