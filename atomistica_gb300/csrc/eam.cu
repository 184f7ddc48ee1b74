// Tabulated alloy EAM on GB300 (replaces
// src/potentials/eam/tabulated_alloy_eam.f90:147-259 (setfl reader) and
// :423-627 (kernel), with the natural cubic spline of
// src/support/simple_spline.f90:127-195, 373-614).
//
//   eam_density  four lanes per atom i (strided over its list entries):
//                rho_i = sum_j rho_{el j}(r_ij) (no extrapolation: an argument
//                outside the table raises an error as in the serial reference),
//                rho clamped at 0, F_i and F'_i with index-clamped
//                extrapolation (:506-554).
//   eam_pair     four lanes per atom i: for each entry (i->j) the i-side term of
//                the reference (:561-607) and the j-side term of the mirror
//                entry (j->i) (same r, exactly negated pair vector), so that
//                f_i = sum_j [df_ij - df_ji] is a gather: no atomics, no
//                reverse index.  The mask applies to the i side of each entry
//                as in the reference (:488).
// Spline coefficients are built on the host in FP64 with the reference's
// operation order and uploaded as 8 doubles per interval
// {y, c1, c2, c3, d1, d2, d3, 0}: a value gather is one 32-byte sector.
// rho and phi of a setfl file share one r grid, so a pair locates its
// interval once for all of its splines; the interval coordinate is
// r is the correctly rounded square root and the interval coordinate rounds
// as the reference's division, so B is bitwise the reference's; 1/r comes
// from a reciprocal square root refined by a Newton step (within an ulp).

#include <cuda_runtime.h>

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <type_traits>

#include "elements.h"
#include "potential.h"

namespace gb {

// ---------------------------------------------------------------------------
// Host spline builder (simple_spline_init, :127-195; scale_y_axis :756-773).
// ---------------------------------------------------------------------------
void SplineHost::init(int n_, double x0_, double dx_, const double *yy) {
  const double sig = 0.5;
  n = n_;
  x0 = x0_;
  dx = dx_;
  y.assign(yy, yy + n);
  d2y.assign(n, 0.0);
  std::vector<double> u(n, 0.0);
  c1.assign(n - 1, 0.0);
  c2.assign(n - 1, 0.0);
  c3.assign(n - 1, 0.0);
  d1.assign(n - 1, 0.0);
  d2.assign(n - 1, 0.0);
  d3.assign(n - 1, 0.0);
  for (int i = 1; i < n - 1; i++) {
    const double p = sig * d2y[i - 1] + 2;
    d2y[i] = (sig - 1) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / dx - (y[i] - y[i - 1]) / dx) / (2 * dx) - sig * u[i - 1]) / p;
  }
  const double qn = 0.0, un = 0.0;
  d2y[n - 1] = (un - qn * u[n - 2]) / (qn * d2y[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; k--) d2y[k] = d2y[k] * d2y[k + 1] + u[k];
  const double dx2 = dx * dx;
  for (int k = 0; k < n - 1; k++) {
    c1[k] = y[k + 1] - y[k] - (2 * d2y[k] + d2y[k + 1]) * dx2 / 6;
    c2[k] = d2y[k] * dx2 / 2;
    c3[k] = (d2y[k + 1] - d2y[k]) * dx2 / 6;
  }
  for (int k = 0; k < n - 1; k++) {
    d1[k] = c1[k] / dx;
    d2[k] = 2 * c2[k] / dx;
    d3[k] = 3 * c3[k] / dx;
  }
  cut = x0 + dx * (n - 1);
}

void SplineHost::scale_y(double fac) {
  for (auto *v : {&y, &d2y, &c1, &c2, &c3, &d1, &d2, &d3})
    for (auto &x : *v) x = fac * x;
}

// setfl reader (tabulated_alloy_eam.f90:178-253).
int eam_read_setfl(const char *fn, EamTables &t) {
  std::ifstream in(fn);
  if (!in) {
    set_error(std::string("Could not open file '") + fn + "'.");
    return GB_ERROR_FILE_NOT_FOUND;
  }
  std::string line;
  for (int i = 0; i < 3; i++)
    if (!std::getline(in, line)) {
      set_error("setfl: premature end of file in header");
      return GB_ERROR_IO_EOF;
    }
  if (!std::getline(in, line)) {
    set_error("setfl: premature end of file");
    return GB_ERROR_IO_EOF;
  }
  {
    // "nel el_1 ... el_nel" (:196-198); at most MAX_EAM_ELS = 10 (:60)
    std::istringstream ss(line);
    ss >> t.nel;
    if (!ss || t.nel <= 0 || t.nel > 10) {
      set_error("setfl: bad element count line (1 to 10 elements): " + line);
      return GB_ERROR_IO;
    }
    t.names.assign(t.nel, std::string());
    for (int e = 0; e < t.nel; e++) ss >> t.names[e];
    if (!ss) {
      set_error("setfl: element count line lists fewer names than elements: " + line);
      return GB_ERROR_IO;
    }
  }
  int nF = 0, nr = 0;
  double dF = 0, dr = 0;
  if (!std::getline(in, line)) {
    set_error("setfl: premature end of file");
    return GB_ERROR_IO_EOF;
  }
  {
    std::istringstream ss(line);
    ss >> nF >> dF >> nr >> dr >> t.cutoff;
    if (!ss || nF < 2 || nr < 2 || !(dF > 0) || !(dr > 0)) {
      set_error("setfl: bad grid line: " + line);
      return GB_ERROR_IO;
    }
  }
  auto read_values = [&](int n, std::vector<double> &v) {
    v.clear();
    v.reserve(n + 2);
    std::string tok;
    while ((int)v.size() < n && (in >> tok)) v.push_back(std::strtod(tok.c_str(), nullptr));
    std::getline(in, line);
    return (int)v.size() == n;
  };
  t.Z.assign(t.nel, 0);
  t.F.assign(t.nel, SplineHost());
  t.rho.assign(t.nel, SplineHost());
  t.phi.assign((size_t)t.nel * t.nel, SplineHost());
  std::vector<double> v;
  for (int e = 0; e < t.nel; e++) {
    if (!std::getline(in, line)) {
      set_error("setfl: premature end of file");
      return GB_ERROR_IO_EOF;
    }
    std::istringstream ss(line);
    ss >> t.Z[e];
    if (!ss || t.Z[e] <= 0) {
      set_error("setfl: bad element line: " + line);
      return GB_ERROR_IO;
    }
    // the atomic number must name the element of the header (:206-213)
    const char *name = element_name(t.Z[e]);
    if (!name || t.names[e] != name) {
      set_error("Atomic number " + std::to_string(t.Z[e]) + " is element " +
                (name ? name : "?") + " and does not match element name " + t.names[e] +
                " found in data file.");
      return GB_ERROR_IO;
    }
    if (!read_values(nF, v)) {
      set_error("setfl: premature end of file in F(rho)");
      return GB_ERROR_IO_EOF;
    }
    t.F[e].init(nF, 0.0, dF, v.data());
    if (!read_values(nr, v)) {
      set_error("setfl: premature end of file in rho(r)");
      return GB_ERROR_IO_EOF;
    }
    v.push_back(0.0);
    v.push_back(0.0);
    t.rho[e].init(nr + 2, 0.0, dr, v.data());
  }
  for (int i = 0; i < t.nel; i++)
    for (int j = 0; j <= i; j++) {
      if (!read_values(nr, v)) {
        set_error("setfl: premature end of file in r*phi(r)");
        return GB_ERROR_IO_EOF;
      }
      v.push_back(0.0);
      v.push_back(0.0);
      SplineHost s;
      s.init(nr + 2, 0.0, dr, v.data());
      s.scale_y(0.5);
      t.phi[(size_t)i * t.nel + j] = s;
      t.phi[(size_t)j * t.nel + i] = s;
    }
  return 0;
}

// funcfl reader (tabulated_eam.f90:147-200): comment; "Z mass a0 lattice";
// "nF dF nr dr cutoff"; F(rho) [nF], Z(r) [nr], rho(r) [nr]; no padding; Z
// scaled by sqrt(Hartree Bohr / 2) with the constants of Units.f90:74-76.
int eam_read_funcfl(const char *fn, EamTables &t) {
  std::ifstream in(fn);
  if (!in) {
    set_error(std::string("Could not open file '") + fn + "'.");
    return GB_ERROR_FILE_NOT_FOUND;
  }
  std::string line;
  if (!std::getline(in, line) || !std::getline(in, line)) {
    set_error("funcfl: premature end of file in header");
    return GB_ERROR_IO_EOF;
  }
  t.nel = 1;
  t.Z.assign(1, 0);
  {
    std::istringstream ss(line);
    ss >> t.Z[0];
    if (!ss || t.Z[0] <= 0) {
      set_error("funcfl: bad element line: " + line);
      return GB_ERROR_IO;
    }
  }
  int nF = 0, nr = 0;
  double dF = 0, dr = 0;
  if (!std::getline(in, line)) {
    set_error("funcfl: premature end of file");
    return GB_ERROR_IO_EOF;
  }
  {
    std::istringstream ss(line);
    ss >> nF >> dF >> nr >> dr >> t.cutoff;
    if (!ss || nF < 2 || nr < 2 || !(dF > 0) || !(dr > 0)) {
      set_error("funcfl: bad grid line: " + line);
      return GB_ERROR_IO;
    }
  }
  auto read_values = [&](int n, std::vector<double> &v) {
    v.clear();
    std::string tok;
    while ((int)v.size() < n && (in >> tok)) v.push_back(std::strtod(tok.c_str(), nullptr));
    return (int)v.size() == n;
  };
  std::vector<double> v;
  t.F.assign(1, SplineHost());
  t.rho.assign(1, SplineHost());
  t.phi.assign(1, SplineHost());
  if (!read_values(nF, v)) {
    set_error("funcfl: premature end of file in F(rho)");
    return GB_ERROR_IO_EOF;
  }
  t.F[0].init(nF, 0.0, dF, v.data());
  if (!read_values(nr, v)) {
    set_error("funcfl: premature end of file in Z(r)");
    return GB_ERROR_IO_EOF;
  }
  t.phi[0].init(nr, 0.0, dr, v.data());
  if (!read_values(nr, v)) {
    set_error("funcfl: premature end of file in rho(r)");
    return GB_ERROR_IO_EOF;
  }
  t.rho[0].init(nr, 0.0, dr, v.data());
  const double hartree = 27.2113961, bohr = 0.529177249;
  t.phi[0].scale_y(std::sqrt(0.5 * hartree * bohr));
  t.funcfl = true;
  return 0;
}

int eam_upload(EamTables &t) {
  std::vector<const SplineHost *> all;
  for (auto &s : t.F) all.push_back(&s);
  for (auto &s : t.rho) all.push_back(&s);
  for (auto &s : t.phi) all.push_back(&s);
  size_t total = 0;
  for (auto *s : all) total += 8 * (size_t)(s->n - 1);
  std::vector<double> h(total);
  std::vector<size_t> offs;
  size_t o = 0;
  for (auto *s : all) {
    offs.push_back(o);
    for (int k = 0; k < s->n - 1; k++) {
      double *d = &h[o + 8 * (size_t)k];
      d[0] = s->y[k];
      d[1] = s->c1[k];
      d[2] = s->c2[k];
      d[3] = s->c3[k];
      d[4] = s->d1[k];
      d[5] = s->d2[k];
      d[6] = s->d3[k];
      d[7] = 0.0;
    }
    o += 8 * (size_t)(s->n - 1);
  }
  GB_CHECK(t.dev.ensure(sizeof(double) * std::max<size_t>(total, 1)));
  GB_CUDA(cudaMemcpy(t.dev.p, h.data(), sizeof(double) * total, cudaMemcpyHostToDevice));
  auto mk = [&](const SplineHost &s, size_t off) {
    SplineDev d;
    d.tab = t.dev.as<double>() + off;
    d.n = s.n;
    d.x0 = s.x0;
    d.dx = s.dx;
    d.rdx = 1.0 / s.dx;
    d.cut = s.cut;
    return d;
  };
  t.dF.clear();
  t.drho.clear();
  t.dphi.clear();
  size_t q = 0;
  for (auto &s : t.F) t.dF.push_back(mk(s, offs[q++]));
  for (auto &s : t.rho) t.drho.push_back(mk(s, offs[q++]));
  for (auto &s : t.phi) t.dphi.push_back(mk(s, offs[q++]));
  return 0;
}

namespace {

constexpr int kMaxEamEl = 10;  // MAX_EAM_ELS (tabulated_alloy_eam.f90:60)

struct EamArgs {
  int nat;
  int nel;
  const Pos4 *pos;
  const int *el;  // table index or -1
  const int *seed, *nbr, *shift, *mask;
  double A[3][3];
  double cutoff_sq;
  SplineDev F[kMaxEamEl], rho[kMaxEamEl], phi[kMaxEamEl * kMaxEamEl];
  double *Fi, *dFi;      // per atom
  double *f, *epa, *wpa;  // outputs (device, accumulated)
  double *part;           // 10 per block
  int *status;
  ReplayCheck chk;        // a replayed evaluation writes no forces when invalid
  int fset;               // f is written for every atom (1) or accumulated into (0)
  // Per-entry cache written by the density pass and read by the force pass
  // (tables on one shared r grid): spline coordinate B, 1/r, and the
  // interval as 2 k + (coordinate out of the table ? 1 : 0), or -1 for an
  // entry the force pass skips (unknown element, beyond the cutoff).
  double *cB, *cRinv;
  int *cK;
};

// simple_spline_f_and_df with extrapolate=.true. (:536-614).
__device__ __forceinline__ void spline_fdf_extrap(const SplineDev &s, double x, double &f,
                                                  double &df) {
  const double xf = (x - s.x0) / s.dx + 1;
  const double fl = floor(xf);
  int i = (fl < -1e9) ? -1000000000 : (fl > 1e9 ? 1000000000 : (int)fl);
  if (i < 1)
    i = 1;
  else if (i >= s.n)
    i = s.n - 1;
  const double B = xf - i;
  const double2 *t = reinterpret_cast<const double2 *>(s.tab + 8 * (size_t)(i - 1));
  const double2 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2), d = __ldg(t + 3);
  f = a.x + B * (a.y + B * (b.x + B * b.y));
  df = c.x + B * (c.y + B * d.x);
}

// GET_DRJ (macros.inc:76): r_i - r_j + matmul(Abox, dc), reference order.
__device__ __forceinline__ void get_drj(const EamArgs &a, const Pos4 &pi, const Pos4 &pj,
                                        int sh, double d[3]) {
  int s0, s1, s2;
  unpack_shift(sh, s0, s1, s2);
  d[0] = __dsub_rn(pi.x, pj.x);
  d[1] = __dsub_rn(pi.y, pj.y);
  d[2] = __dsub_rn(pi.z, pj.z);
  if (s0 | s1 | s2) {
    const double sx = s0, sy = s1, sz = s2;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double as = __dmul_rn(a.A[c][0], sx);
      as = __dadd_rn(as, __dmul_rn(a.A[c][1], sy));
      as = __dadd_rn(as, __dmul_rn(a.A[c][2], sz));
      d[c] = __dadd_rn(d[c], as);
    }
  }
}

__device__ __forceinline__ double norm2_ref(const double d[3]) {
  double s = __dmul_rn(d[0], d[0]);
  s = __dadd_rn(s, __dmul_rn(d[1], d[1]));
  s = __dadd_rn(s, __dmul_rn(d[2], d[2]));
  return s;
}

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

constexpr int kEamThreads = 256;
// Lanes per atom: an atom's list entries are strided over a group of 4
// consecutive lanes (about 11 entries per lane for the ~43 neighbours of fcc
// at 5 A), 8 atoms per warp.
constexpr int kEamLanes = 4;

__device__ __forceinline__ double group_sum(double x) {
#pragma unroll
  for (int o = 1; o < kEamLanes; o <<= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Interval of r on the grid that rho and phi share in a setfl file (nr + 2
// points from 0 with step dr): 0-based k and local coordinate B of
// simple_spline (:373-434), with k clamped to the table for the
// extrapolating phi; ok = false where the non-extrapolating rho is out of
// range (an error in the reference).
// The quotient (r - x0) / dx is formed as the product with 1/dx and one
// residual correction (Markstein), which rounds as the division does: near
// the end of a setfl table (the zero padding) the spline's slope changes by
// ~1e5 eV/A^2, so B must round exactly as in the reference.
__device__ __forceinline__ void r_interval(const SplineDev &s, double r, double &B, int &k,
                                           bool &ok) {
  const double u = r - s.x0;
  double q = u * s.rdx;
  q = fma(fma(-q, s.dx, u), s.rdx, q);
  const double xf = q + 1.0;
  // floor as one rounding-down conversion (r is finite and below the cutoff
  // at every call, and the conversion saturates)
  int i = __double2int_rd(xf);
  ok = i >= 1 && (i < s.n || r <= s.cut);
  i = min(max(i, 1), s.n - 1);
  B = xf - i;
  k = i - 1;
}

// The reference's SPLINE_* macros (spline.inc; funcfl EAM):
// xf = (x - x0) * (1/dx) + 1, i = int(xf); an index outside the table (an
// out-of-bounds read in the reference) is clamped and reported.
__device__ __forceinline__ void inline_interval(const SplineDev &s, double x, double &B, int &k,
                                                bool &ok) {
  const double xf = __dadd_rn(__dmul_rn(__dsub_rn(x, s.x0), s.rdx), 1.0);
  int i = (int)fmin(fmax(xf, -1.0e9), 1.0e9);
  ok = i >= 1 && i < s.n;
  i = min(max(i, 1), s.n - 1);
  B = xf - i;
  k = i - 1;
}

__device__ __forceinline__ void interval_fdf(const SplineDev &s, int k, double B, double &f,
                                             double &df) {
  const double2 *t = reinterpret_cast<const double2 *>(s.tab + 8 * (size_t)k);
  const double2 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2), d = __ldg(t + 3);
  f = a.x + B * (a.y + B * (b.x + B * b.y));
  df = c.x + B * (c.y + B * d.x);
}

__device__ __forceinline__ double interval_f(const SplineDev &s, int k, double B) {
  const double2 *t = reinterpret_cast<const double2 *>(s.tab + 8 * (size_t)k);
  const double2 a = __ldg(t), b = __ldg(t + 1);
  return a.x + B * (a.y + B * (b.x + B * b.y));
}

__device__ __forceinline__ double interval_df(const SplineDev &s, int k, double B) {
  const double2 *t = reinterpret_cast<const double2 *>(s.tab + 8 * (size_t)k + 4);
  const double2 c = __ldg(t), d = __ldg(t + 1);
  return c.x + B * (c.y + B * d.x);
}


template <bool kFuncfl, bool kCache>
__global__ void __launch_bounds__(kEamThreads) eam_density(const EamArgs a) {
  const int gt = blockIdx.x * kEamThreads + threadIdx.x;
  const int i = gt / kEamLanes, sub = gt % kEamLanes;
  int eli = -1;
  bool on = false;
  if (i < a.nat) {
    eli = a.el[i];
    on = eli >= 0 && !(a.mask && a.mask[i] == 0);
  }
  double rho = 0.0;
  bool bad = false;
  // kCache: every entry of an atom of a known element (the force pass visits
  // them whether or not the atom is in the mask) gets its cache row; the
  // density itself only for atoms in the mask.
  if (kCache ? eli >= 0 : on) {
    const Pos4 pi = a.pos[i];
    const int s = a.seed[i], e = a.seed[i + 1];
    for (int b = s + sub; b < e; b += kEamLanes) {
      const int j = a.nbr[b];
      const int elj = a.el[j];
      if (elj < 0) {
        if (kCache) a.cK[b] = -1;
        continue;
      }
      double d[3];
      get_drj(a, pi, a.pos[j], a.shift[b], d);
      const double r2 = norm2_ref(d);
      if (r2 < a.cutoff_sq) {
        double B;
        int k;
        bool ok;
        // kCache: 1/r is cached as well, and r derived from it (the correctly
        // rounded square root, see sqrt_from_rsqrt)
        const double rinv = kCache ? rsqrt_refined(r2) : 0.0;
        const double r = kCache ? sqrt_from_rsqrt(r2, rinv) : sqrt(r2);
        if (kFuncfl)
          inline_interval(a.rho[elj], r, B, k, ok);
        else
          r_interval(a.rho[elj], r, B, k, ok);
        if (kCache) {
          a.cB[b] = B;
          a.cRinv[b] = rinv;
          a.cK[b] = 2 * k + (ok ? 0 : 1);
        }
        if (on) {
          bad |= !ok;
          rho += interval_f(a.rho[elj], k, B);
        }
      } else if (kCache) {
        a.cK[b] = -1;
      }
    }
  }
  rho = group_sum(rho);  // (every lane takes part in the shuffles)
  if (bad) atomicOr(a.status, 1);
  if (i < a.nat && sub == 0) {
    double F = 0.0, dF = 0.0;
    if (on) {
      if (rho < 0.0) rho = 0.0;
      if (kFuncfl) {
        double B;
        int k;
        bool ok;
        inline_interval(a.F[eli], rho, B, k, ok);
        if (!ok) atomicOr(a.status, 1);
        interval_fdf(a.F[eli], k, B, F, dF);
      } else {
        spline_fdf_extrap(a.F[eli], rho, F, dF);
      }
    }
    a.Fi[i] = F;
    a.dFi[i] = dF;
  }
}

// Virial components kept once (the pair virial is symmetric):
// xx, yy, zz, xy, xz, yz; Fortran (c2 + 3 c) order of the 9 on output.
__device__ __forceinline__ int sym_index(int c2, int c) {
  return c2 == c ? c : 2 + c2 + c;  // (0,1) -> 3, (0,2) -> 4, (1,2) -> 5
}

template <bool kEpa, bool kWat, bool kFuncfl, bool kCache>
__global__ void __launch_bounds__(kEamThreads) eam_pair(const EamArgs a) {
  __shared__ double sred[kEamThreads / 32][7];
  const int gt = blockIdx.x * kEamThreads + threadIdx.x;
  const int i = gt / kEamLanes, sub = gt % kEamLanes;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double w6[6] = {0, 0, 0, 0, 0, 0};  // total virial of this lane's entries
  double F3[3] = {0.0, 0.0, 0.0};
  double Wa[6] = {0, 0, 0, 0, 0, 0};  // per-atom virial of atom i
  double Ei = 0.0;
  const int eli = i < a.nat ? a.el[i] : -1;
  const bool mi = eli >= 0 && !(a.mask && a.mask[i] == 0);
  if (eli >= 0) {
    const double dFi = mi ? a.dFi[i] : 0.0;
    const Pos4 pi = a.pos[i];
    bool bad = false;
    const int s = a.seed[i], e = a.seed[i + 1];
    for (int b = s + sub; b < e; b += kEamLanes) {
      const int j = a.nbr[b];
      // rho and phi share the r grid: one interval for all three splines
      double B, rinv;
      int k, elj;
      bool ok;
      double d[3];
      if (kCache) {
        // the density pass's coordinate, 1/r and interval of this entry
        const int kk = a.cK[b];
        if (kk < 0) continue;
        elj = a.el[j];
        get_drj(a, pi, a.pos[j], a.shift[b], d);
        B = a.cB[b];
        rinv = a.cRinv[b];
        k = kk >> 1;
        ok = (kk & 1) == 0;
      } else {
        elj = a.el[j];
        if (elj < 0) continue;
        get_drj(a, pi, a.pos[j], a.shift[b], d);
        const double r2 = norm2_ref(d);
        if (!(r2 < a.cutoff_sq)) continue;
        const double r = sqrt(r2);  // rounded as the reference's (table coordinate)
        rinv = rsqrt_refined(r2);
        if (kFuncfl)
          inline_interval(a.phi[eli * a.nel + elj], r, B, k, ok);
        else
          r_interval(a.phi[eli * a.nel + elj], r, B, k, ok);
      }
      const bool mj = !(a.mask && a.mask[j] == 0);
      const SplineDev &sp = a.phi[eli * a.nel + elj];
      double phi, dphi, pair;
      if (kFuncfl) {
        // Z(r): pair energy Z^2 / r, its derivative 2 Z Z' / r - Z^2 / r^2
        // (tabulated_eam.f90:301-304)
        double z, dz;
        interval_fdf(sp, k, B, z, dz);
        phi = z * z * rinv;
        pair = 2 * z * dz * rinv - phi * rinv;
      } else {
        interval_fdf(sp, k, B, phi, dphi);
        pair = (dphi - phi * rinv) * rinv;
        phi = phi * rinv;
      }
      double fac_i = 0.0;
      // f_i += (sc_i + sc_j) d: the i-side term df = sc_i d and the j-side
      // term of the mirror entry, -df' = sc_j d, added as one coefficient
      double sc_f = 0.0;
      if (mi) {
        // i-side of entry (i->j), :577-607: df = sc d, f_i += df,
        // w += -d (x) df
        bad |= !ok;
        fac_i = interval_df(a.rho[elj], k, B);
        const double sc = -(dFi * fac_i + pair) * rinv;
        Ei += phi;
        sc_f = sc;
        const double df[3] = {sc * d[0], sc * d[1], sc * d[2]};
        const double w[6] = {-d[0] * df[0], -d[1] * df[1], -d[2] * df[2],
                             -d[0] * df[1], -d[0] * df[2], -d[1] * df[2]};
#pragma unroll
        for (int c = 0; c < 6; c++) {
          w6[c] += w[c];
          if (kWat) Wa[c] += 0.5 * w[c];
        }
      }
      if (mj) {
        // j-side of the mirror entry (j->i): dr' = -d, acts on i with -df'.
        bad |= !ok;
        const double fac_j = (mi && elj == eli) ? fac_i : interval_df(a.rho[eli], k, B);
        const double sc = -(a.dFi[j] * fac_j + pair) * rinv;
        sc_f += sc;
        if (kWat) {
          const double dfp[3] = {-sc * d[0], -sc * d[1], -sc * d[2]};
          Wa[0] += 0.5 * (d[0] * dfp[0]);
          Wa[1] += 0.5 * (d[1] * dfp[1]);
          Wa[2] += 0.5 * (d[2] * dfp[2]);
          Wa[3] += 0.5 * (d[0] * dfp[1]);
          Wa[4] += 0.5 * (d[0] * dfp[2]);
          Wa[5] += 0.5 * (d[1] * dfp[2]);
        }
      }
      F3[0] = fma(sc_f, d[0], F3[0]);
      F3[1] = fma(sc_f, d[1], F3[1]);
      F3[2] = fma(sc_f, d[2], F3[2]);
    }
    if (bad) atomicOr(a.status, 1);
  }
  // group sums (every lane takes part in the shuffles)
#pragma unroll
  for (int c = 0; c < 3; c++) F3[c] = group_sum(F3[c]);
  Ei = group_sum(Ei);
  if (kWat)
#pragma unroll
    for (int c = 0; c < 6; c++) Wa[c] = group_sum(Wa[c]);
  double e_tot = 0.0;
  if (a.fset && eli < 0 && i < a.nat && sub == 0 && !replay_invalid(a.chk))
#pragma unroll
    for (int c = 0; c < 3; c++) a.f[3 * (size_t)i + c] = 0.0;  // (skipped atom, written)
  if (eli >= 0) {
    if (mi) Ei += a.Fi[i];
    if (sub == 0 && !replay_invalid(a.chk)) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        if (a.fset)
          a.f[3 * (size_t)i + c] = F3[c];
        else
          a.f[3 * (size_t)i + c] += F3[c];
      }
      if (kEpa && mi) a.epa[i] += Ei;
      if (kWat)
#pragma unroll
        for (int q = 0; q < 9; q++) a.wpa[9 * (size_t)i + q] += Wa[sym_index(q % 3, q / 3)];
      if (mi) e_tot = Ei;
    }
  }
  // Block partials: energy and virial.
#pragma unroll
  for (int c = 0; c < 6; c++) w6[c] = warp_sum(w6[c]);
  e_tot = warp_sum(e_tot);
  if (lane == 0) {
    sred[wib][0] = e_tot;
#pragma unroll
    for (int c = 0; c < 6; c++) sred[wib][1 + c] = w6[c];
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    const int col = threadIdx.x == 0 ? 0 : 1 + sym_index((threadIdx.x - 1) % 3,
                                                         (threadIdx.x - 1) / 3);
    double s = 0.0;
    for (int w = 0; w < kEamThreads / 32; w++) s += sred[w][col];
    a.part[10 * (size_t)blockIdx.x + threadIdx.x] = s;
  }
}

}  // namespace

// Whether every rho and phi table of the file lies on one r grid (the
// density pass's interval of an entry is then the force pass's too).
static bool eam_shared_grid(const EamTables &t) {
  if (t.drho.empty()) return false;
  const SplineDev &g = t.drho[0];
  auto same = [&](const SplineDev &q) {
    return q.n == g.n && q.x0 == g.x0 && q.dx == g.dx && q.rdx == g.rdx && q.cut == g.cut;
  };
  for (const auto &q : t.drho)
    if (!same(q)) return false;
  for (const auto &q : t.dphi)
    if (!same(q)) return false;
  return true;
}

int eam_cache_ensure(Potential &pot, int64_t entries) {
  if (entries < 0) entries = 0;
  return pot.eam_cache.ensure(20 * (size_t)std::max<int64_t>(entries, 1));
}

int eam_compute(Potential &pot, const Particles &p, Neighbors &nl, const Outputs &o,
                bool want_wat, ReplayCheck chk, bool capture) {
  cudaStream_t s = pot.stream;
  const int nat = p.nat;
  EamTables &t = *pot.eam;
  if (nat == 0) {
    GB_CUDA(cudaMemsetAsync(o.red, 0, sizeof(double) * 10, s));
    return 0;
  }
  if (t.nel > kMaxEamEl) {
    set_error("TabulatedAlloyEAM: more than 10 elements in the setfl file.");
    return GB_ERROR_ARGUMENT;
  }
  EamArgs a;
  a.nat = nat;
  a.nel = t.nel;
  a.pos = nl.pos4.as<Pos4>();
  a.el = pot.el.as<int>();
  a.seed = nl.seed.as<int>();
  a.nbr = nl.nbr.as<int>();
  a.shift = nl.shift.as<int>();
  a.mask = o.mask;
  std::memcpy(a.A, p.A, sizeof(a.A));
  a.cutoff_sq = t.cutoff * t.cutoff;
  for (int q = 0; q < t.nel; q++) {
    a.F[q] = t.dF[q];
    a.rho[q] = t.drho[q];
  }
  for (int q = 0; q < t.nel * t.nel; q++) a.phi[q] = t.dphi[q];
  GB_CHECK(pot.atom_dF.ensure(sizeof(double) * 2 * nat));
  a.Fi = pot.atom_dF.as<double>();
  a.dFi = a.Fi + nat;
  a.f = o.f;
  a.epa = o.epot_per_at;
  a.wpa = o.wpot_per_at;
  const int blocks = (int)(((int64_t)nat * kEamLanes + kEamThreads - 1) / kEamThreads);
  GB_CHECK(pot.tile_part.ensure(sizeof(double) * 10 * blocks + 64));
  a.part = pot.tile_part.as<double>();
  a.status = o.status;
  a.chk = chk;
  a.fset = o.f_set ? 1 : 0;
  const bool ff = t.funcfl;
  // The per-entry cache needs one r grid for every rho and phi table (true
  // of setfl and funcfl files) and room for the list: its entries now, or the
  // captured capacity (sized before the capture began).
  const int64_t entries = capture ? (int64_t)nat * nl.stage_cap : (int64_t)nl.nentries;
  const bool cache = eam_shared_grid(t) && eam_cache_ensure(pot, entries) == 0;
  clear_error();
  a.cB = nullptr;
  a.cRinv = nullptr;
  a.cK = nullptr;
  if (cache) {
    const size_t cap = pot.eam_cache.bytes / 20;
    a.cB = pot.eam_cache.as<double>();
    a.cRinv = a.cB + cap;
    a.cK = reinterpret_cast<int *>(a.cRinv + cap);
  }
  if (ff)
    cache ? eam_density<true, true><<<blocks, kEamThreads, 0, s>>>(a)
          : eam_density<true, false><<<blocks, kEamThreads, 0, s>>>(a);
  else
    cache ? eam_density<false, true><<<blocks, kEamThreads, 0, s>>>(a)
          : eam_density<false, false><<<blocks, kEamThreads, 0, s>>>(a);
  note_launch();
  const bool epa = o.epot_per_at != nullptr;
  // the funcfl kernel of the reference leaves wpot_per_at untouched
  const bool wat = want_wat && !ff;
  if (!capture) GB_CUDA(cudaEventRecord(pot.kev[0], s));
  auto pair = [&](auto epa_t, auto wat_t, auto ff_t) {
    if (cache)
      eam_pair<decltype(epa_t)::value, decltype(wat_t)::value, decltype(ff_t)::value, true>
          <<<blocks, kEamThreads, 0, s>>>(a);
    else
      eam_pair<decltype(epa_t)::value, decltype(wat_t)::value, decltype(ff_t)::value, false>
          <<<blocks, kEamThreads, 0, s>>>(a);
    note_launch();
  };
  using T = std::true_type;
  using F = std::false_type;
  if (ff) {
    if (epa)
      pair(T{}, F{}, T{});
    else
      pair(F{}, F{}, T{});
  } else if (epa && wat) {
    pair(T{}, T{}, F{});
  } else if (epa) {
    pair(T{}, F{}, F{});
  } else if (wat) {
    pair(F{}, T{}, F{});
  } else {
    pair(F{}, F{}, F{});
  }
  if (!capture) GB_CUDA(cudaEventRecord(pot.kev[1], s));
  GB_CUDA(cudaGetLastError());
  GB_CHECK(pot.red_stage.ensure(reduce_stage_bytes(blocks) + 64));
  GB_CHECK(reduce_partials(a.part, blocks, 10, o.red, pot.red_stage.as<double>(), s));
  return 0;
}

}  // namespace gb
