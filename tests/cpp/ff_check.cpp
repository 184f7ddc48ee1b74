// Host-compiled accuracy check of the float-float kernels' math
// (atomistica_gb300/csrc/ff.h).  Prints the max relative errors against
// long double references; tests/test_ff_math.py compiles and runs it.
#include <cmath>
#include <cstdio>
#include <random>

#include "ff.h"

using namespace gb;

int main() {
  ff etab[256], stab[257], ctab[257];
  for (int j = 0; j < 256; j++) etab[j] = ff_from_double(std::exp2((double)j / 256.0));
  for (int j = 0; j <= 256; j++) {
    const long double x = (long double)j * 3.14159265358979323846264338327950288L / 256.0L;
    stab[j] = ff_from_double((double)std::sin(x));
    ctab[j] = ff_from_double((double)std::cos(x));
  }
  std::mt19937_64 rng(1);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double e_exp = 0, e_log = 0, e_sin = 0, e_cos = 0, e_sqrt = 0, e_rsqrt = 0, e_rcp = 0, e_mul = 0;
  for (int it = 0; it < 200000; it++) {
    const double t = -30.0 + 45.0 * U(rng);
    const ff tf = ff_from_double(t);
    const long double tr = (long double)tf.hi + (long double)tf.lo;
    const ff v = ff_exp(tf, etab);
    const long double ref = std::exp(tr);
    e_exp = std::fmax(e_exp, (double)std::fabs(((long double)v.hi + v.lo) / ref - 1.0L));
    const float z = (float)std::exp(20.0 * U(rng) - 8.0);
    const ff l = ff_log_f(z, etab);
    e_log = std::fmax(e_log, (double)std::fabs(((long double)l.hi + l.lo) - std::log((long double)z)));
    const double x = 3.14159265358979 * U(rng);
    const ff xf = ff_from_double(x);
    const long double xr = (long double)xf.hi + xf.lo;
    ff sx, cx;
    ff_sincos(xf, stab, ctab, sx, cx);
    e_sin = std::fmax(e_sin, (double)std::fabs(((long double)sx.hi + sx.lo) - std::sin(xr)));
    e_cos = std::fmax(e_cos, (double)std::fabs(((long double)cx.hi + cx.lo) - std::cos(xr)));
    const double q = 0.2 + 12.0 * U(rng);
    const ff qf = ff_from_double(q);
    const long double qr = (long double)qf.hi + qf.lo;
    ff r, ri;
    ff_sqrt_rsqrt(qf, r, ri);
    e_sqrt = std::fmax(e_sqrt, (double)std::fabs(((long double)r.hi + r.lo) / std::sqrt(qr) - 1.0L));
    e_rsqrt = std::fmax(e_rsqrt,
                        (double)std::fabs(((long double)ri.hi + ri.lo) * std::sqrt(qr) - 1.0L));
    const ff rc = ff_rcp(qf);
    e_rcp = std::fmax(e_rcp, (double)std::fabs(((long double)rc.hi + rc.lo) * qr - 1.0L));
    const ff m = ff_mul(qf, xf);
    e_mul = std::fmax(e_mul, (double)std::fabs(((long double)m.hi + m.lo) / (qr * xr) - 1.0L));
  }
  std::printf("%.3e %.3e %.3e %.3e %.3e %.3e %.3e %.3e\n", e_exp, e_log, e_sin, e_cos, e_sqrt,
              e_rsqrt, e_rcp, e_mul);
  return 0;
}
