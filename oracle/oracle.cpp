// ============================================================================
// TEST INFRASTRUCTURE ONLY — the CPU FP64 oracle.
//
// A plain C++17 (+OpenMP) restatement of Atomistica's per-step force path, used
// by tests/ as the checker and by bench.py as the timed CPU baseline.  Nothing
// in the atomistica_gb300 product links, loads or calls this file.
//
// Every routine follows the reference loop structure and operation order:
//   * neighbour list      src/python/f90/python_neighbors.f90:570-959
//   * reciprocal cell     src/support/f_linearalgebra.f90:505-552 (gauss)
//   * BOP kernel          src/potentials/bop/bop_kernel.f90:420-1068, 1074-1529,
//                         1613-1628 (non-screened branch)
//   * BOP glue            src/potentials/bop/default_bind_to_func.f90:73-144,
//                         src/potentials/bop/default_compute_func.f90:54-95
//   * Tersoff functions   src/potentials/bop/tersoff/tersoff_func.f90:32-232
//   * Kumagai functions   src/potentials/bop/kumagai/kumagai_func.f90:32-242
//   * Brenner functions   src/potentials/bop/brenner/brenner_func.f90:32-225,
//                         brenner_module.f90:119-243 (derived constants,
//                         interaction range)
//   * trig_off cutoff     src/support/cutoff.f90:152-196
//   * screened BOP        bop_kernel.f90:682-995 (pass 1), 1171-1527 and
//                         1531-1611 (pass 2 and the screening forces),
//                         default_bind_to_func.f90:45-71, 94-121;
//                         exp_cutoff src/support/cutoff.f90:232-293
//   * cubic spline        src/support/simple_spline.f90:127-195, 373-651, 756-773
//   * alloy EAM           src/potentials/eam/tabulated_alloy_eam.f90:147-259,
//                         423-627
//   * pair index          src/macros.inc:123
//
// Parity pins: the reference ships no golden energy/force vectors and its
// Fortran cannot be compiled here (no Fortran compiler).  The oracle is pinned
// by the reference's own known-answer tests re-expressed without ASE (see
// tests/test_oracle_pins.py): FD force/virial consistency, the Si(100)
// surface energy 2.309 J/m^2, bulk Ec/a0/elastic constants within 5 %, mask
// additivity, the pbc bit-equality and the neighbour-list tests.
//
// Build with -ffp-contract=off so that the FP64 distance tests follow the
// reference operation order exactly (no fused multiply-add).
// ============================================================================

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Cell geometry.  A[a][k] is Fortran Abox(a,k): column k is lattice vector k.
// ---------------------------------------------------------------------------

struct Box {
  double A[3][3];
  double B[3][3];  // A^-1 (Bbox)
  int pbc[3];
};

// Gauss elimination with the pivot choice of gauss() in
// src/support/f_linearalgebra.f90:505-552, applied to each unit vector as in
// gaussn (:599-637, the non-LAPACK branch).
int gauss_solve(const double Ain[3][3], const double b[3], double x[3]) {
  const int n = 3;
  double A[3][4];
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < n; k++) A[j][k] = Ain[j][k];
    A[j][n] = b[j];
  }
  int indx[3] = {0, 0, 0};  // 0 = not yet used as pivot, else pivot step (1-based)
  for (int i = 0; i < n; i++) {
    int max_indx = -1;
    double maxv = -1.0;
    for (int j = 0; j < n; j++) {
      if (indx[j] != 0) continue;
      double v = std::fabs(A[j][i]);
      if (v > maxv) {
        maxv = v;
        max_indx = j;
      }
    }
    indx[max_indx] = i + 1;
    if (A[max_indx][i] == 0.0) return -1;
    double fac[3], row[4];
    for (int j = 0; j < n; j++) fac[j] = A[j][i] / A[max_indx][i];
    for (int k = 0; k < n + 1; k++) row[k] = A[max_indx][k];
    for (int j = 0; j < n; j++) {
      if (indx[j] != 0) continue;
      for (int k = i; k < n + 1; k++) A[j][k] = A[j][k] - fac[j] * row[k];
    }
  }
  double Ap[3][4];
  for (int j = 0; j < n; j++)
    for (int k = 0; k < n + 1; k++) Ap[indx[j] - 1][k] = A[j][k];
  for (int j = n - 1; j >= 0; j--) {
    if (Ap[j][j] == 0.0) return -1;
    x[j] = Ap[j][n] / Ap[j][j];
    for (int m = 0; m < j; m++) Ap[m][n] = Ap[m][n] - Ap[m][j] * x[j];
  }
  return 0;
}

int make_box(const double *cell_rows, const int *pbc, Box &box) {
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) box.A[a][k] = cell_rows[3 * k + a];
  for (int c = 0; c < 3; c++) {
    double e[3] = {0, 0, 0}, x[3];
    e[c] = 1.0;
    if (gauss_solve(box.A, e, x) != 0) return -1;
    for (int a = 0; a < 3; a++) box.B[a][c] = x[a];
  }
  for (int k = 0; k < 3; k++) box.pbc[k] = pbc[k] != 0;
  return 0;
}

// ---------------------------------------------------------------------------
// Neighbour list: python_neighbors.f90 binning_init (:765-871), binning_update
// (:904-959) and fill_neighbor_list (:570-754).  Compact CSR instead of the
// sentinel-separated per-thread chunks; same per-atom entry order.
// ---------------------------------------------------------------------------

struct NList {
  std::vector<int64_t> seed;  // nat+1 CSR offsets
  std::vector<int> nbr;
  std::vector<int> dc;  // 3 ints per entry
};

struct Binning {
  int n_cells[3];
  double rec[3][3];
  int dx, dy, dz;
  std::vector<int> d;  // 3 per stencil entry
};

void binning_init(const Box &box, double cutoff, double bin_size, Binning &bn) {
  double box_size[3];
  for (int x = 0; x < 3; x++) {
    double s = 0.0;
    for (int a = 0; a < 3; a++) s = s + box.A[a][x] * box.A[a][x];
    box_size[x] = std::sqrt(s);
  }
  for (int x = 0; x < 3; x++) {
    int nc = (int)(box_size[x] / bin_size);
    bn.n_cells[x] = nc < 3 ? 3 : nc;
  }
  double cs[3][3];  // cs[a][x] = cell_size(a, x)
  for (int x = 0; x < 3; x++) {
    for (int a = 0; a < 3; a++) cs[a][x] = box.A[a][x] / bn.n_cells[x];
    for (int k = 0; k < 3; k++) bn.rec[x][k] = box.B[x][k] * bn.n_cells[x];
  }
  auto col = [&](int x, double v[3]) {
    for (int a = 0; a < 3; a++) v[a] = cs[a][x];
  };
  auto cross = [](const double u[3], const double v[3], double w[3]) {
    w[0] = u[1] * v[2] - u[2] * v[1];
    w[1] = u[2] * v[0] - u[0] * v[2];
    w[2] = u[0] * v[1] - u[1] * v[0];
  };
  auto dot = [](const double u[3], const double v[3]) {
    double s = u[0] * v[0];
    s = s + u[1] * v[1];
    s = s + u[2] * v[2];
    return s;
  };
  double c1[3], c2[3], c3[3], nx[3], ny[3], nz[3];
  col(0, c1);
  col(1, c2);
  col(2, c3);
  cross(c2, c3, nx);
  cross(c3, c1, ny);
  cross(c1, c2, nz);
  double cv = dot(c1, nx);
  // nx = cv*nx/dot_product(nx, nx) etc. (python_neighbors.f90:838-840); the
  // right-hand side uses the old vector.
  const double dnx = dot(nx, nx), dny = dot(ny, ny), dnz = dot(nz, nz);
  for (int a = 0; a < 3; a++) {
    nx[a] = cv * nx[a] / dnx;
    ny[a] = cv * ny[a] / dny;
    nz[a] = cv * nz[a] / dnz;
  }
  bn.dx = (int)(cutoff / std::sqrt(dot(nx, nx))) + 1;
  bn.dy = (int)(cutoff / std::sqrt(dot(ny, ny))) + 1;
  bn.dz = (int)(cutoff / std::sqrt(dot(nz, nz))) + 1;
  bn.d.clear();
  for (int x = -bn.dx; x <= bn.dx; x++)
    for (int y = -bn.dy; y <= bn.dy; y++)
      for (int z = -bn.dz; z <= bn.dz; z++) {
        bn.d.push_back(x);
        bn.d.push_back(y);
        bn.d.push_back(z);
      }
}

// floor(matmul(rec_cell_size, r)) (0-based), python_neighbors.f90:641.
inline void raw_cell(const Binning &bn, const double *ri, int c[3]) {
  for (int x = 0; x < 3; x++) {
    double s = bn.rec[x][0] * ri[0];
    s = s + bn.rec[x][1] * ri[1];
    s = s + bn.rec[x][2] * ri[2];
    c[x] = (int)std::floor(s);
  }
}

int build_neighbors(int nat, const double *r, const Box &box, double cutoff,
                    NList &nl) {
  Binning bn;
  binning_init(box, cutoff, cutoff, bn);
  const int ncx = bn.n_cells[0], ncy = bn.n_cells[1], ncz = bn.n_cells[2];
  // binning_update: singly linked list per cell in increasing atom id.
  std::vector<int> seed((size_t)ncx * ncy * ncz, -1), last(seed.size(), -1),
      next(nat, -1);
  for (int i = 0; i < nat; i++) {
    int c[3];
    raw_cell(bn, &r[3 * i], c);
    for (int k = 0; k < 3; k++) {
      const int n = bn.n_cells[k];
      if (box.pbc[k]) {
        while (c[k] < 0) c[k] += n;
        while (c[k] > n - 1) c[k] -= n;
      } else {
        if (c[k] < 0) c[k] = 0;
        if (c[k] > n - 1) c[k] = n - 1;
      }
    }
    size_t ci = ((size_t)c[2] * ncy + c[1]) * ncx + c[0];
    if (seed[ci] == -1) {
      seed[ci] = i;
      last[ci] = i;
    } else {
      next[last[ci]] = i;
      last[ci] = i;
    }
  }
  const double cutoff_sq = cutoff * cutoff;
  const int n_d = (int)bn.d.size() / 3;
  // Per-atom lists are built independently, then concatenated in atom order.
  std::vector<std::vector<int>> lj(nat), ls(nat);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < nat; i++) {
    int celli[3], shift[3] = {0, 0, 0};
    raw_cell(bn, &r[3 * i], celli);
    for (int k = 0; k < 3; k++) {
      const int n = bn.n_cells[k];
      if (box.pbc[k]) {
        while (celli[k] < 0) {
          celli[k] += n;
          shift[k] += 1;
        }
        while (celli[k] > n - 1) {
          celli[k] -= n;
          shift[k] -= 1;
        }
      } else {
        if (celli[k] < 0) celli[k] = 0;
        if (celli[k] > n - 1) celli[k] = n - 1;
      }
    }
    for (int x = 0; x < n_d; x++) {
      int cur[3], shift1[3];
      for (int k = 0; k < 3; k++) {
        cur[k] = celli[k] + bn.d[3 * x + k];
        shift1[k] = shift[k];
      }
      bool exists = true;
      for (int k = 0; k < 3; k++) {
        const int n = bn.n_cells[k];
        if (box.pbc[k]) {
          while (cur[k] < 0) {
            cur[k] += n;
            shift1[k] += 1;
          }
          while (cur[k] > n - 1) {
            cur[k] -= n;
            shift1[k] -= 1;
          }
        }
        if (cur[k] < 0 || cur[k] > n - 1) exists = false;
      }
      if (!exists) continue;
      int j = seed[((size_t)cur[2] * ncy + cur[1]) * ncx + cur[0]];
      while (j != -1) {
        int cellj[3], shift2[3];
        raw_cell(bn, &r[3 * j], cellj);
        for (int k = 0; k < 3; k++) {
          shift2[k] = shift1[k];
          const int n = bn.n_cells[k];
          if (box.pbc[k]) {
            while (cellj[k] < 0) {
              cellj[k] += n;
              shift2[k] -= 1;
            }
            while (cellj[k] > n - 1) {
              cellj[k] -= n;
              shift2[k] += 1;
            }
          }
        }
        if (i != j || shift2[0] != 0 || shift2[1] != 0 || shift2[2] != 0) {
          // delta_r = r_i - r_j + matmul(Abox, shift2)   (:708)
          double dr[3];
          for (int a = 0; a < 3; a++) {
            double as = box.A[a][0] * (double)shift2[0];
            as = as + box.A[a][1] * (double)shift2[1];
            as = as + box.A[a][2] * (double)shift2[2];
            dr[a] = (r[3 * i + a] - r[3 * j + a]) + as;
          }
          double d2 = dr[0] * dr[0];
          d2 = d2 + dr[1] * dr[1];
          d2 = d2 + dr[2] * dr[2];
          if (d2 < cutoff_sq) {
            lj[i].push_back(j);
            ls[i].push_back(shift2[0]);
            ls[i].push_back(shift2[1]);
            ls[i].push_back(shift2[2]);
          }
        }
        j = next[j];
      }
    }
  }
  nl.seed.assign(nat + 1, 0);
  for (int i = 0; i < nat; i++) nl.seed[i + 1] = nl.seed[i] + (int64_t)lj[i].size();
  nl.nbr.resize(nl.seed[nat]);
  nl.dc.resize(3 * nl.seed[nat]);
  for (int i = 0; i < nat; i++) {
    std::copy(lj[i].begin(), lj[i].end(), nl.nbr.begin() + nl.seed[i]);
    std::copy(ls[i].begin(), ls[i].end(), nl.dc.begin() + 3 * nl.seed[i]);
  }
  return 0;
}

// Pair index, src/macros.inc:123 (0-based in and out).
inline int pair_index(int i, int j, int nel) {
  int a = std::min(i + j * nel, j + i * nel);
  int b = std::min(i * (i + 1) / 2, j * (j + 1) / 2);
  return a - b;
}

// trig_off cutoff, src/support/cutoff.f90:152-196.
struct TrigOff {
  double r1, r2, fac;
  void init(double a, double b) {
    r1 = a;
    r2 = b;
    fac = M_PI / (r2 - r1);
  }
  void f(double r, double &val, double &dval) const {
    if (r <= r1) {
      val = 1.0;
      dval = 0.0;
    } else if (r >= r2) {
      val = 0.0;
      dval = 0.0;
    } else {
      double x = fac * (r - r1);
      val = 0.5 * (1.0 + std::cos(x));
      dval = -0.5 * fac * std::sin(x);
    }
  }
};

// exp_cutoff (the CUTOFF_T of the screened potentials), cutoff.f90:232-293:
// f(x) = exp(-8 x^3) corrected so that f, f' and f'' vanish at x = 1.
struct ExpCutoff {
  double r1, r2, fac1, fac2, c, d, off;
  void init(double a, double b) {
    r1 = a;
    r2 = b;
    fac1 = 1.0 / (r2 - r1);
    const double val1 = std::exp(-8.0);
    const double dval1 = -24 * val1;
    const double ddval1 = -48 * val1 - 24 * dval1;
    c = (-3 * dval1 + ddval1) / 3;
    d = (2 * dval1 - ddval1) / 4;
    fac2 = 1.0 / (1 - val1 - c - d);
    off = val1 + c + d;
  }
  void f(double r, double &val, double &dval) const {
    if (r <= r1) {
      val = 1.0;
      dval = 0.0;
    } else if (r >= r2) {
      val = 0.0;
      dval = 0.0;
    } else {
      const double x = fac1 * (r - r1);
      const double x2 = x * x;
      val = std::exp(-8 * x * x2);
      dval = -24 * x2 * val;
      dval = fac1 * fac2 * (dval + 3 * c * x2 + 4 * d * x * x2);
      val = fac2 * (val + c * x * x2 + d * x2 * x2 - off);
    }
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Parameter sets (layout of BOP_DB_TYPE, tersoff_params.f90:27-97 and
// kumagai_params.f90:27-96; 0-based element/pair indices).
// ---------------------------------------------------------------------------

extern "C" {

struct orc_tersoff_params {
  int nel;
  int Z[3];
  double A[6], B[6], xi[6], lambda[6], mu[6], omega[6], mubo[6];
  int m[6];
  double beta[3], n[3], c[3], d[3], h[3];
  double r1[6], r2[6];
};

// Extra parameters of the screened variants (tersoff_params.f90:81-90 under
// SCREENING): outer (attractive/repulsive) and bond-order cutoffs, screening
// window Cmin < C < Cmax; per pair.  The inner cutoff is r1/r2 of the base set.
struct orc_scr_params {
  double or1[9], or2[9], bor1[9], bor2[9], Cmin[9], Cmax[9];
};

struct orc_kumagai_params {
  int nel;
  int Z[1];
  double A[1], B[1], lambda1[1], lambda2[1];
  double eta[1], delta[1], alpha[1];
  int beta[1];
  double c1[1], c2[1], c3[1], c4[1], c5[1], h[1];
  double r1[1], r2[1];
};

// Brenner-form parameter set (brenner_params.f90:27-65): every array per
// symmetric element pair.
struct orc_brenner_params {
  int nel;
  int Z[3];
  double D0[6], r0[6], S[6], beta[6], gamma[6], c[6], d[6], h[6], mu[6], n[6];
  int m[6];
  double r1[6], r2[6];
};

// Juslin parameter set (juslin_params.f90:31-70): pair arrays per ordered
// element pair j + i nel (macros.inc:139), h constants per element triplet
// k + nel (j + nel i) (macros.inc:146).
struct orc_juslin_params {
  int nel;
  int Z[3];
  double D0[9], r0[9], S[9], beta[9], gamma[9], c[9], d[9], h[9], n[9];
  double alpha[27], omega[27];
  int m[27];
  double r1[9], r2[9];
};

}  // extern "C"

namespace {

// Tersoff functional form, tersoff_func.f90:32-232.
struct TersoffFn {
  const orc_tersoff_params &p;
  explicit TersoffFn(const orc_tersoff_params &q) : p(q) {}
  int nel() const { return p.nel; }
  int npairs() const { return p.nel * (p.nel + 1) / 2; }
  int pair(int i, int j) const { return pair_index(i, j, p.nel); }
  bool cdr_guard() const { return true; }
  double r1(int ij) const { return p.r1[ij]; }
  double r2(int ij) const { return p.r2[ij]; }
  void VA(int ij, double dr, double &val, double &dval) const {
    double e = std::exp(-p.mu[ij] * dr);
    val = -p.B[ij] * e;
    dval = p.B[ij] * p.mu[ij] * e;
  }
  void VR(int ij, double dr, double &val, double &dval) const {
    double e = std::exp(-p.lambda[ij] * dr);
    val = p.A[ij] * e;
    dval = -p.A[ij] * p.lambda[ij] * e;
  }
  void g(int ktypi, int ikpot, double costh, double &val, double &dval) const {
    double omega = p.omega[ikpot];
    double h_c = p.h[ktypi] - costh;
    double c_sq = p.c[ktypi] * p.c[ktypi];
    double d_sq = p.d[ktypi] * p.d[ktypi];
    double h = d_sq + h_c * h_c;
    val = omega * (1.0 + c_sq / d_sq - c_sq / h);
    dval = -2 * omega * c_sq * h_c / (h * h);
  }
  void bo(int ktypi, int ijpot, double zij, double fcij, double faij, double &bij,
          double &dfbij) const {
    if (zij > 0.0) {
      double e = -0.5 / p.n[ktypi];
      double b = std::pow(p.beta[ktypi], p.n[ktypi]);
      double arg = 1.0 + b * std::pow(zij, p.n[ktypi]);
      bij = p.xi[ijpot] * std::pow(arg, e);
      dfbij = -0.25 * fcij * faij * p.xi[ijpot] * b * std::pow(zij, p.n[ktypi] - 1.0) *
              std::pow(arg, e - 1.0);
    } else {
      bij = 1.0;
      dfbij = 0.0;
    }
  }
  void h(int /*eli*/, int /*elj*/, int /*elk*/, int ikpot, double dr, double &val,
         double &dval) const {
    double mu = p.mubo[ikpot];
    if (mu == 0.0) {
      val = 1.0;
      dval = 0.0;
    } else {
      int m = p.m[ikpot];
      if (m == 1) {
        val = std::exp(2 * mu * dr);
        dval = 2 * mu * val;
      } else if (m == 3) {
        double arg = 2 * mu * dr;
        val = std::exp(arg * arg * arg);
        dval = 2 * mu * m * arg * arg * val;
      } else {
        val = std::exp(std::pow(2 * mu * dr, m));
        dval = 2 * mu * m * std::pow(2 * mu * dr, m - 1) * val;
      }
    }
  }
};

// Kumagai functional form, kumagai_func.f90:32-242.
struct KumagaiFn {
  const orc_kumagai_params &p;
  explicit KumagaiFn(const orc_kumagai_params &q) : p(q) {}
  int nel() const { return p.nel; }
  int npairs() const { return 1; }
  int pair(int /*i*/, int /*j*/) const { return 0; }
  bool cdr_guard() const { return true; }
  double r1(int ij) const { return p.r1[ij]; }
  double r2(int ij) const { return p.r2[ij]; }
  void VA(int ij, double dr, double &val, double &dval) const {
    double e = std::exp(-p.lambda2[ij] * dr);
    val = -p.B[ij] * e;
    dval = p.B[ij] * p.lambda2[ij] * e;
  }
  void VR(int ij, double dr, double &val, double &dval) const {
    double e = std::exp(-p.lambda1[ij] * dr);
    val = p.A[ij] * e;
    dval = -p.A[ij] * p.lambda1[ij] * e;
  }
  void g(int ktypi, int /*ikpot*/, double costh, double &val, double &dval) const {
    double c1 = p.c1[ktypi], c2 = p.c2[ktypi], c3 = p.c3[ktypi], c4 = p.c4[ktypi],
           c5 = p.c5[ktypi], h = p.h[ktypi];
    double h_cos = h - costh;
    double h_cos_sq = h_cos * h_cos;
    double tmp = h_cos / (c3 + h_cos_sq);
    double go = c2 * tmp;
    double ga1 = c4 * std::exp(-c5 * h_cos_sq);
    double v = go * (1.0 + ga1);
    dval = -2 * (1.0 - h_cos * tmp) * v + 2 * c5 * h_cos_sq * go * ga1;
    val = c1 + h_cos * v;
  }
  void bo(int ktypi, int /*ijpot*/, double zij, double fcij, double faij, double &bij,
          double &dfbij) const {
    if (zij > 0.0) {
      double eta = p.eta[ktypi];
      double delta = -p.delta[ktypi];
      double arg = 1.0 + std::pow(zij, eta);
      bij = std::pow(arg, delta);
      dfbij = 0.5 * fcij * faij * eta * std::pow(zij, eta - 1.0) * delta *
              std::pow(arg, delta - 1.0);
    } else {
      bij = 1.0;
      dfbij = 0.0;
    }
  }
  void h(int /*eli*/, int /*elj*/, int /*elk*/, int ikpot, double dr, double &val,
         double &dval) const {
    double alpha = p.alpha[ikpot];
    if (alpha == 0.0) {
      val = 1.0;
      dval = 0.0;
    } else {
      int beta = p.beta[ikpot];
      if (beta == 1) {
        val = std::exp(alpha * dr);
        dval = alpha * val;
      } else if (beta == 3) {
        // kumagai_func.f90:211-213 omits alpha in the exponent; kept as is.
        val = std::exp(dr * dr * dr);
        dval = 3 * alpha * dr * dr * val;
      } else {
        val = std::exp(alpha * std::pow(dr, beta));
        dval = beta * alpha * std::pow(dr, beta - 1) * val;
      }
    }
  }
};

// Brenner functional form, brenner_func.f90:32-225, with the derived
// constants of BIND_TO_FUNC (brenner_module.f90:196-214): bo_exp = -1/(2n),
// bo_fac = bo_exp n / 2, expR = beta sqrt(2 S), expA = beta sqrt(2 / S),
// VR_f = D0 / (S - 1), VA_f = S D0 / (S - 1), c_d = c^2 / d^2.
struct BrennerFn {
  const orc_brenner_params &p;
  double bo_exp[6], bo_fac[6], bo_exp1[6], expR[6], expA[6], c_sq[6], d_sq[6], c_d[6],
      VR_f[6], VA_f[6];
  explicit BrennerFn(const orc_brenner_params &q) : p(q) {
    const int np = p.nel * (p.nel + 1) / 2;
    for (int i = 0; i < np; i++) {
      bo_exp[i] = -0.5 / p.n[i];
      bo_fac[i] = 0.5 * bo_exp[i] * p.n[i];
      bo_exp1[i] = bo_exp[i] - 1.0;
      expR[i] = p.beta[i] * std::sqrt(2 * p.S[i]);
      expA[i] = p.beta[i] * std::sqrt(2 / p.S[i]);
      c_sq[i] = p.c[i] * p.c[i];
      d_sq[i] = p.d[i] * p.d[i];
      c_d[i] = c_sq[i] / d_sq[i];
      VR_f[i] = p.D0[i] / (p.S[i] - 1);
      VA_f[i] = p.S[i] * p.D0[i] / (p.S[i] - 1);
    }
  }
  int nel() const { return p.nel; }
  int npairs() const { return p.nel * (p.nel + 1) / 2; }
  int pair(int i, int j) const { return pair_index(i, j, p.nel); }
  bool cdr_guard() const { return true; }
  double r1(int ij) const { return p.r1[ij]; }
  double r2(int ij) const { return p.r2[ij]; }
  void VA(int ij, double dr, double &val, double &dval) const {
    const double e = std::exp(-expA[ij] * (dr - p.r0[ij]));
    val = -VA_f[ij] * e;
    dval = VA_f[ij] * expA[ij] * e;
  }
  void VR(int ij, double dr, double &val, double &dval) const {
    const double e = std::exp(-expR[ij] * (dr - p.r0[ij]));
    val = VR_f[ij] * e;
    dval = -VR_f[ij] * expR[ij] * e;
  }
  // angular term of the (i,k) pair; the sign convention is h + cos theta
  void g(int /*ktypi*/, int ikpot, double costh, double &val, double &dval) const {
    const double hc = p.h[ikpot] + costh;
    const double h = d_sq[ikpot] + hc * hc;
    val = p.gamma[ikpot] * (1 + c_d[ikpot] - c_sq[ikpot] / h);
    dval = 2 * p.gamma[ikpot] * c_sq[ikpot] * hc / (h * h);
  }
  // bond order of the (i,j) pair; n = 1 takes the branch without the
  // zeta > 0 test (brenner_func.f90:146-150)
  void bo(int /*ktypi*/, int ijpot, double zij, double fcij, double faij, double &bij,
          double &dfbij) const {
    if (p.n[ijpot] == 1.0) {
      const double arg = 1.0 + zij;
      bij = std::pow(arg, bo_exp[ijpot]);
      dfbij = bo_fac[ijpot] * fcij * faij * std::pow(arg, bo_exp1[ijpot]);
    } else if (zij > 0.0) {
      const double arg = 1.0 + std::pow(zij, p.n[ijpot]);
      bij = std::pow(arg, bo_exp[ijpot]);
      dfbij = bo_fac[ijpot] * fcij * faij * std::pow(zij, p.n[ijpot] - 1.0) *
              std::pow(arg, bo_exp1[ijpot]);
    } else {
      bij = 1.0;
      dfbij = 0.0;
    }
  }
  void h(int /*eli*/, int /*elj*/, int /*elk*/, int ikpot, double dr, double &val,
         double &dval) const {
    const double mu = p.mu[ikpot];
    if (mu == 0.0) {
      val = 1.0;
      dval = 0.0;
    } else {
      const int m = p.m[ikpot];
      if (m == 1) {
        val = std::exp(2 * mu * dr);
        dval = 2 * mu * val;
      } else if (m == 3) {
        const double arg = 2 * mu * dr;
        val = std::exp(arg * arg * arg);
        dval = 6 * mu * arg * arg * val;
      } else {
        val = std::exp(std::pow(2 * mu * dr, m));
        dval = 2 * mu * m * std::pow(2 * mu * dr, m - 1) * val;
      }
    }
  }
};

// Juslin functional form, juslin_func.f90:25-313, with the derived constants
// of BIND_TO_FUNC (juslin_module.f90:322-377).  The caller's set is first
// completed by the mirror fill of juslin_module.f90:273-300 (an ordered pair
// with r0 < 0 takes the constants of its mirror).  VA, VR, g and bo are
// Brenner's; h is omega e^{(alpha dr)^m} of the triplet (i, j, k).
struct JuslinFn {
  orc_juslin_params p;
  double bo_exp[9], bo_fac[9], bo_exp1[9], expR[9], expA[9], c_sq[9], d_sq[9], c_d[9], VR_f[9],
      VA_f[9];
  explicit JuslinFn(const orc_juslin_params &q) : p(q) {
    const int nel = p.nel;
    for (int i = 0; i < nel; i++)
      for (int j = 0; j < nel; j++) {
        const int a = j + i * nel, b = i + j * nel;
        if (p.r0[a] < 0.0) {
          p.D0[a] = p.D0[b];
          p.r0[a] = p.r0[b];
          p.S[a] = p.S[b];
          p.beta[a] = p.beta[b];
          p.gamma[a] = p.gamma[b];
          p.c[a] = p.c[b];
          p.d[a] = p.d[b];
          p.h[a] = p.h[b];
          p.n[a] = p.n[b];
          p.r1[a] = p.r1[b];
          p.r2[a] = p.r2[b];
        }
      }
    for (int i = 0; i < nel * nel; i++) {
      bo_exp[i] = -0.5 / p.n[i];
      bo_fac[i] = 0.5 * bo_exp[i] * p.n[i];
      bo_exp1[i] = bo_exp[i] - 1.0;
      expR[i] = p.beta[i] * std::sqrt(2 * p.S[i]);
      expA[i] = p.beta[i] * std::sqrt(2 / p.S[i]);
      c_sq[i] = p.c[i] * p.c[i];
      d_sq[i] = p.d[i] * p.d[i];
      c_d[i] = c_sq[i] / d_sq[i];
      VR_f[i] = p.D0[i] / (p.S[i] - 1);
      VA_f[i] = p.S[i] * p.D0[i] / (p.S[i] - 1);
    }
  }
  int nel() const { return p.nel; }
  int npairs() const { return p.nel * p.nel; }
  int pair(int i, int j) const { return j + i * p.nel; }
  bool cdr_guard() const { return false; }
  double r1(int ij) const { return p.r1[ij]; }
  double r2(int ij) const { return p.r2[ij]; }
  void VA(int ij, double dr, double &val, double &dval) const {
    const double e = std::exp(-expA[ij] * (dr - p.r0[ij]));
    val = -VA_f[ij] * e;
    dval = VA_f[ij] * expA[ij] * e;
  }
  void VR(int ij, double dr, double &val, double &dval) const {
    const double e = std::exp(-expR[ij] * (dr - p.r0[ij]));
    val = VR_f[ij] * e;
    dval = -VR_f[ij] * expR[ij] * e;
  }
  void g(int /*ktypi*/, int ikpot, double costh, double &val, double &dval) const {
    const double hc = p.h[ikpot] + costh;
    const double h = d_sq[ikpot] + hc * hc;
    val = p.gamma[ikpot] * (1 + c_d[ikpot] - c_sq[ikpot] / h);
    dval = 2.0 * p.gamma[ikpot] * c_sq[ikpot] * hc / (h * h);
  }
  void bo(int /*ktypi*/, int ijpot, double zij, double fcij, double faij, double &bij,
          double &dfbij) const {
    if (p.n[ijpot] == 1.0) {
      const double arg = 1.0 + zij;
      bij = std::pow(arg, bo_exp[ijpot]);
      dfbij = bo_fac[ijpot] * fcij * faij * std::pow(arg, bo_exp1[ijpot]);
    } else if (zij > 0.0) {
      const double arg = 1.0 + std::pow(zij, p.n[ijpot]);
      bij = std::pow(arg, bo_exp[ijpot]);
      dfbij = bo_fac[ijpot] * fcij * faij * std::pow(zij, p.n[ijpot] - 1.0) *
              std::pow(arg, bo_exp1[ijpot]);
    } else {
      bij = 1.0;
      dfbij = 0.0;
    }
  }
  // juslin_func.f90:257-294; TRIPLET_INDEX_NS(ktypi, ktypj, ktypk)
  void h(int eli, int elj, int elk, int /*ikpot*/, double dr, double &val,
         double &dval) const {
    const int t = elk + p.nel * (elj + p.nel * eli);
    const double alpha = p.alpha[t], omega = p.omega[t];
    const int m = p.m[t];
    if (m == 1) {
      val = omega * std::exp(alpha * dr);
      dval = alpha * val;
    } else if (m == 3) {
      const double arg = alpha * dr;
      val = omega * std::exp(arg * arg * arg);
      dval = 3 * alpha * arg * arg * val;
    } else {
      const double arg = alpha * dr;
      val = omega * std::exp(std::pow(arg, m));
      dval = m * std::pow(arg, m - 1) * alpha * val;
    }
  }
};

struct BopOut {
  double *epot, *f, *wpot, *epot_per_at, *epot_per_bond, *f_per_bond, *wpot_per_at,
      *wpot_per_bond;
};

// BOP_KERNEL, bop_kernel.f90 (non-screened, PYTHON build).  el[i] is the
// 0-based database index or -1.  Per-bond outputs are indexed by the compact
// neighbour-list slot (the reference's nbb).
template <class Fn>
int bop_kernel(const Fn &fn, int nat, const double *r, const Box &box, const int *el,
               const NList &nl, const int *mask, const BopOut &o, int nthreads,
               int natloc = -1) {
  // natloc < nat: the LAMMPS build, bonds of the first natloc atoms only
  // (bop_kernel.f90:562, 1075 loop i = 1, natloc)
  if (natloc < 0) natloc = nat;
  const int nel = fn.nel();
  (void)nel;
  const int npairs = fn.npairs();
  std::vector<TrigOff> cut_in(npairs);
  std::vector<double> cut_in_l(npairs), cut_in_h(npairs), cut_in_h2(npairs);
  for (int i = 0; i < npairs; i++) {
    cut_in[i].init(fn.r1(i), fn.r2(i));
    cut_in_l[i] = fn.r1(i);
    cut_in_h[i] = fn.r2(i);
    cut_in_h2[i] = fn.r2(i) * fn.r2(i);
  }
  // Pass 1 (bop_kernel.f90:562-1068): internal short bond list.
  struct Bond {
    int j, nbb, typ;
    int dc[3];
    double len, nm[3], fc, dfc;
  };
  std::vector<int64_t> neb_seed(nat + 1, 0);
  std::vector<std::vector<Bond>> bonds_of(nat);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
  for (int i = 0; i < natloc; i++) {
    const int eli = el[i];
    if (eli < 0) continue;
    for (int64_t jn = nl.seed[i]; jn < nl.seed[i + 1]; jn++) {
      const int j = nl.nbr[jn];
      const int elj = el[j];
      if (elj < 0) continue;
      const int *dc = &nl.dc[3 * jn];
      double rij[3];
      for (int a = 0; a < 3; a++) {
        double as = box.A[a][0] * (double)dc[0];
        as = as + box.A[a][1] * (double)dc[1];
        as = as + box.A[a][2] * (double)dc[2];
        rij[a] = (r[3 * j + a] - r[3 * i + a]) - as;
      }
      double rlij = rij[0] * rij[0];
      rlij = rlij + rij[1] * rij[1];
      rlij = rlij + rij[2] * rij[2];
      const int el2ij = fn.pair(eli, elj);
      Bond b;
      b.j = j;
      b.nbb = (int)jn;
      b.typ = el2ij;
      b.dc[0] = dc[0];
      b.dc[1] = dc[1];
      b.dc[2] = dc[2];
      if (rlij < cut_in_l[el2ij] * cut_in_l[el2ij]) {
        b.fc = 1.0;
        b.dfc = 0.0;
      } else if (rlij < cut_in_h2[el2ij]) {
        double rl = std::sqrt(rlij);
        cut_in[el2ij].f(rl, b.fc, b.dfc);
      } else {
        continue;
      }
      rlij = std::sqrt(rlij);
      b.len = rlij;
      for (int a = 0; a < 3; a++) b.nm[a] = rij[a] / rlij;
      bonds_of[i].push_back(b);
    }
  }
  int nebmax = 0;
  for (int i = 0; i < nat; i++) nebmax = std::max(nebmax, (int)bonds_of[i].size());

  // Pass 2 (bop_kernel.f90:1074-1529) with thread-private pe/f/wpot_per_at
  // (tls.f90) reduced in thread order at the end.
  int nt = nthreads;
  std::vector<std::vector<double>> tpe(nt), tf(nt), twat(nt);
  std::vector<double> twpot(9 * nt, 0.0);
  const bool want_wat = o.wpot_per_at != nullptr;
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num();
#else
    const int tid = 0;
#endif
    std::vector<double> &pe = tpe[tid];
    std::vector<double> &f = tf[tid];
    std::vector<double> &wat = twat[tid];
    pe.assign(nat, 0.0);
    f.assign(3 * (size_t)nat, 0.0);
    if (want_wat) wat.assign(9 * (size_t)nat, 0.0);
    double wpot[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    std::vector<double> dbidk(3 * (size_t)std::max(nebmax, 1));
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < natloc; i++) {
      const int eli = el[i];
      if (eli < 0) continue;
      double fi[3] = {0, 0, 0};
      const std::vector<Bond> &bi = bonds_of[i];
      const int nb = (int)bi.size();
      for (int ij = 0; ij < nb; ij++) {
        const Bond &B = bi[ij];
        const int j = B.j;
        int maskfac = 2;
        if (mask) {
          if (mask[i] == 0 && mask[j] == 0)
            maskfac = 0;
          else if (mask[i] == 0 || mask[j] == 0)
            maskfac = 1;
        }
        const int el2ij = B.typ;
        double rlij = B.len;
        if (!(maskfac > 0 && rlij < cut_in_h[el2ij])) continue;
        double fj[3] = {0, 0, 0};
        const int elj = el[j];
        (void)elj;
        const double rlijr = 1.0 / rlij;
        double rnij[3] = {B.nm[0], B.nm[1], B.nm[2]};
        double rij[3] = {rlij * rnij[0], rlij * rnij[1], rlij * rnij[2]};
        const double fcarij = B.fc, dfcarijr = B.dfc;
        double VAij, dVAij, VRij, dVRij;
        fn.VA(el2ij, rlij, VAij, dVAij);
        fn.VR(el2ij, rlij, VRij, dVRij);
        VAij = 0.5 * maskfac * VAij;
        dVAij = 0.5 * maskfac * dVAij;
        VRij = 0.5 * maskfac * VRij;
        dVRij = 0.5 * maskfac * dVRij;
        double wij[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double wijb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double zij = 0.0;
        double dbidi[3] = {0, 0, 0}, dbidj[3] = {0, 0, 0};
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;
          const Bond &K = bi[ik];
          const int ikpot = K.typ;
          const double rlik = K.len;
          if (!(rlik < cut_in_h[ikpot])) {
            dbidk[3 * ik] = dbidk[3 * ik + 1] = dbidk[3 * ik + 2] = 0.0;
            continue;
          }
          const double *rnik = K.nm;
          double rik[3] = {rlik * rnik[0], rlik * rnik[1], rlik * rnik[2]};
          const double fcik = K.fc, dfcikr = K.dfc;
          double h_Dr, dh_dDr;
          fn.h(eli, el[j], el[K.j], ikpot, rlij - rlik, h_Dr, dh_dDr);
          double costh = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
          double g_costh, dg_dcosth;
          fn.g(eli, ikpot, costh, g_costh, dg_dcosth);
          double dkc[3];
          for (int a = 0; a < 3; a++) dkc[a] = rnik[a] * rlik - rnij[a] * rlij;
          double disjk = std::sqrt(dkc[0] * dkc[0] + dkc[1] * dkc[1] + dkc[2] * dkc[2]);
          for (int a = 0; a < 3; a++) dkc[a] = dkc[a] / disjk;
          const double dcsdij = 1.0 / rlik - costh * rlijr;
          const double dcsdik = rlijr - costh / rlik;
          const double dcsdjk = -disjk * rlijr / rlik;
          double dcsdi[3], dcsdj[3], dcsdk[3];
          for (int a = 0; a < 3; a++) {
            dcsdi[a] = -dcsdij * rnij[a] - dcsdik * rnik[a];
            dcsdj[a] = dcsdij * rnij[a] - dcsdjk * dkc[a];
            dcsdk[a] = dcsdik * rnik[a] + dcsdjk * dkc[a];
          }
          const double dzfac = fcik * dg_dcosth * h_Dr;
          double dgdi[3], dgdj[3], dgdk[3];
          for (int a = 0; a < 3; a++) {
            dgdi[a] = dzfac * dcsdi[a];
            dgdj[a] = dzfac * dcsdj[a];
            dgdk[a] = dzfac * dcsdk[a];
          }
          zij = zij + fcik * g_costh * h_Dr;
          const double dzdrij = g_costh * fcik * dh_dDr;
          const double dzdrik = g_costh * (dfcikr * h_Dr - fcik * dh_dDr);
          double df[3];
          for (int a = 0; a < 3; a++) {
            dbidi[a] = dbidi[a] - dzdrij * rnij[a] - dzdrik * rnik[a] + dgdi[a];
            df[a] = dzdrij * rnij[a] + dgdj[a];
            dbidj[a] = dbidj[a] + df[a];
            dbidk[3 * ik + a] = dzdrik * rnik[a] + dgdk[a];
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++)
              wijb[a][c] = wijb[a][c] - rij[a] * df[c] - rik[a] * dbidk[3 * ik + c];
        }
        double bij, dbij_dzij;
        fn.bo(eli, el2ij, zij, fcarij, VAij, bij, dbij_dzij);
        double dffac = 0.5 * fcarij * (VRij + bij * VAij);
        pe[i] = pe[i] + dffac;
        pe[j] = pe[j] + dffac;
        if (o.epot_per_bond) o.epot_per_bond[B.nbb] += dffac;
        dffac = 0.5 * (dVRij * fcarij + bij * dVAij * fcarij + VRij * dfcarijr +
                       bij * VAij * dfcarijr);
        double df[3];
        for (int a = 0; a < 3; a++) {
          df[a] = dffac * rnij[a];
          fi[a] = fi[a] + df[a];
          fj[a] = fj[a] - df[a];
        }
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++)
            wij[a][c] = wij[a][c] + rij[a] * df[c] - dbij_dzij * wijb[a][c];
        if (o.f_per_bond)
          for (int a = 0; a < 3; a++) o.f_per_bond[3 * (size_t)B.nbb + a] += df[a];
        for (int a = 0; a < 3; a++) fi[a] = fi[a] - dbij_dzij * dbidi[a];
        for (int a = 0; a < 3; a++) fj[a] = fj[a] - dbij_dzij * dbidj[a];
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;  // k == j and kdc == jdc (:1459)
          const int k = bi[ik].j;
          for (int a = 0; a < 3; a++)
            f[3 * (size_t)k + a] += -dbij_dzij * dbidk[3 * ik + a];
        }
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++) wpot[a][c] += wij[a][c];
        if (o.wpot_per_bond)
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++)
              o.wpot_per_bond[9 * (size_t)B.nbb + 3 * c + a] += wij[a][c];
        if (want_wat)
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) {
              wat[9 * (size_t)i + 3 * c + a] += wij[a][c] / 2;
              wat[9 * (size_t)j + 3 * c + a] += wij[a][c] / 2;
            }
        for (int a = 0; a < 3; a++) f[3 * (size_t)j + a] += fj[a];
      }
      for (int a = 0; a < 3; a++) f[3 * (size_t)i + a] += fi[a];
    }
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) twpot[9 * tid + 3 * a + c] = wpot[a][c];
  }
  // Reductions (bop_kernel.f90:1613-1628, tls_reduce).
  double esum = 0.0;
  for (int t = 0; t < nt; t++) {
    if (tpe[t].empty()) continue;
    double s = 0.0;
    for (int i = 0; i < nat; i++) s += tpe[t][i];
    esum += 0.5 * s;
    for (size_t q = 0; q < 3 * (size_t)nat; q++) o.f[q] += tf[t][q];
    if (o.epot_per_at)
      for (int i = 0; i < nat; i++) o.epot_per_at[i] += 0.5 * tpe[t][i];
    if (want_wat)
      for (size_t q = 0; q < 9 * (size_t)nat; q++) o.wpot_per_at[q] += twat[t][q];
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) o.wpot[3 * c + a] += twpot[9 * t + 3 * a + c];
  }
  *o.epot += esum;
  return 0;
}

// BOP_KERNEL with SCREENING defined (TersoffScr, KumagaiScr; PYTHON build,
// neither SIN_S nor PARTIAL_SCREENING).  Differences to the plain kernel:
//   * pass 1 (bop_kernel.f90:682-995): a bond beyond the inner cutoff r1 is
//     tested for screening by every neighbour k of i (in list order, stopping
//     at the first full screen or once ln S drops below screening_threshold):
//     C = (2 (x_ik + x_jk) - (x_ik - x_jk)^2 - 1) / (1 - (x_ik - x_jk)^2),
//     x = r^2 / r_ij^2; C <= Cmin screens fully, Cmin < C < Cmax adds
//     -((Cmax - C)/(C - Cmin))^2 to ln S and records k with dS/dr_ik,
//     dS/dr_jk.  A screened bond beyond r2 is dropped; the others get
//     fc_ar = (1 - fc_in) S fc_out + fc_in and fc_bo likewise (exp_cutoff);
//   * pass 2: VA/VR up to or2 with fc_ar, zeta terms up to bor2 with fc_bo;
//     the screening neighbours of bond ij take forces from the pair term
//     (:1531-1560), and those of bond ik from d zeta_ij / d S_ik accumulated
//     over ij (sfacbo, :1462-1471, applied in the loop :1571-1611).
template <class Fn>
int bop_kernel_scr(const Fn &fn, const orc_scr_params &sp, int nat, const double *r,
                   const Box &box, const int *el, const NList &nl, const int *mask,
                   const BopOut &o, int nthreads, int natloc = -1) {
  if (natloc < 0) natloc = nat;
  const int nel = fn.nel();
  (void)nel;
  const int npairs = fn.npairs();
  std::vector<ExpCutoff> cut_in(npairs), cut_out(npairs), cut_bo(npairs);
  std::vector<double> cut_in_l(npairs), cut_in_h(npairs), cut_in_h2(npairs), cut_out_l(npairs),
      cut_out_h(npairs), cut_bo_h(npairs), max_cut_sq(npairs), Cmin(npairs), Cmax(npairs),
      dC(npairs), C_dr_cut(npairs);
  for (int q = 0; q < npairs; q++) {
    cut_in[q].init(fn.r1(q), fn.r2(q));
    cut_in_l[q] = fn.r1(q);
    cut_in_h[q] = fn.r2(q);
    cut_in_h2[q] = fn.r2(q) * fn.r2(q);
    cut_out[q].init(sp.or1[q], sp.or2[q]);
    cut_out_l[q] = sp.or1[q];
    cut_out_h[q] = sp.or2[q];
    cut_bo[q].init(sp.bor1[q], sp.bor2[q]);
    cut_bo_h[q] = sp.bor2[q];
    const double mc = std::max(std::max(cut_in_h[q], cut_out_h[q]), cut_bo_h[q]);
    max_cut_sq[q] = mc * mc;
    Cmin[q] = sp.Cmin[q];
    Cmax[q] = sp.Cmax[q];
    dC[q] = Cmax[q] - Cmin[q];
    // default_bind_to_func.f90:62-68; Juslin without the guard
    // (juslin_module.f90:305-307)
    C_dr_cut[q] =
        (Cmax[q] > 2.0 || !fn.cdr_guard()) ? Cmax[q] * Cmax[q] / (4 * (Cmax[q] - 1)) : 1.0;
  }
  const double screening_threshold = std::log(1e-6);
  const double dot_threshold = (double)1e-10f;  // a default-real literal in tersoff_type.f90:86

  struct ScrEntry {
    int k, kn;
    double arik, arjk, boik, bojk;
  };
  struct Bond {
    int j, nbb, typ;
    double len, nm[3], fcar, dfcar, fcbo, dfcbo;
    int s0, s1;  // screening entries [s0, s1) of the atom's ScrEntry list
  };
  auto get_rik = [&](int i, int64_t kn, double rik[3]) {
    const int k = nl.nbr[kn];
    const int *dc = &nl.dc[3 * kn];
    for (int a = 0; a < 3; a++) {
      double as = box.A[a][0] * (double)dc[0];
      as = as + box.A[a][1] * (double)dc[1];
      as = as + box.A[a][2] * (double)dc[2];
      rik[a] = (r[3 * k + a] - r[3 * i + a]) - as;
    }
  };
  std::vector<std::vector<Bond>> bonds_of(nat);
  std::vector<std::vector<ScrEntry>> scr_of(nat);
  // Pass 1.
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
  for (int i = 0; i < natloc; i++) {
    const int eli = el[i];
    if (eli < 0) continue;
    std::vector<Bond> &bonds = bonds_of[i];
    std::vector<ScrEntry> &scr = scr_of[i];
    const int64_t jbeg = nl.seed[i], jend = nl.seed[i + 1];
    for (int64_t jn = jbeg; jn < jend; jn++) {
      const int j = nl.nbr[jn];
      const int elj = el[j];
      if (elj < 0) continue;
      const int *dcj = &nl.dc[3 * jn];
      double rij[3];
      get_rik(i, jn, rij);
      double rlij = rij[0] * rij[0];
      rlij = rlij + rij[1] * rij[1];
      rlij = rlij + rij[2] * rij[2];
      const int el2ij = fn.pair(eli, elj);
      Bond b;
      b.j = j;
      b.nbb = (int)jn;
      b.typ = el2ij;
      b.s0 = b.s1 = (int)scr.size();
      if (rlij < cut_in_l[el2ij] * cut_in_l[el2ij]) {
        // region (a): no screening
        b.fcar = b.fcbo = 1.0;
        b.dfcar = b.dfcbo = 0.0;
      } else if (rlij < max_cut_sq[el2ij] && cut_out_l[el2ij] < cut_out_h[el2ij]) {
        bool screened = false, need_derivative = false;
        double sij = 0.0, dsijdrij = 0.0;
        const int ineb = (int)scr.size();
        for (int64_t kn = jbeg; !(screened || sij < screening_threshold) && kn < jend; kn++) {
          const int k = nl.nbr[kn];
          double rik[3];
          get_rik(i, kn, rik);
          double rr = rik[0] * rik[0];
          rr = rr + rik[1] * rik[1];
          rr = rr + rik[2] * rik[2];
          if (!(rr < C_dr_cut[el2ij] * rlij)) continue;
          const int *dck = &nl.dc[3 * kn];
          if (!(k != j || dck[0] != dcj[0] || dck[1] != dcj[1] || dck[2] != dcj[2])) continue;
          double dot_ij_ik = rij[0] * rik[0];
          dot_ij_ik = dot_ij_ik + rij[1] * rik[1];
          dot_ij_ik = dot_ij_ik + rij[2] * rik[2];
          const double rlik = rr;
          double rjk[3];
          for (int a = 0; a < 3; a++) rjk[a] = -rij[a] + rik[a];
          double dot_ij_jk = rij[0] * rjk[0];
          dot_ij_jk = dot_ij_jk + rij[1] * rjk[1];
          dot_ij_jk = dot_ij_jk + rij[2] * rjk[2];
          double rljk = rjk[0] * rjk[0];
          rljk = rljk + rjk[1] * rjk[1];
          rljk = rljk + rjk[2] * rjk[2];
          if (!(dot_ij_ik > dot_threshold && dot_ij_jk < -dot_threshold)) continue;
          const double xik = rlik / rlij, xjk = rljk / rlij;
          const double xm = xik - xjk, xp = xik + xjk;
          double fac = 1.0 / (1 - xm * xm);
          const double C = (2 * xp - xm * xm - 1) * fac;
          if (C <= Cmin[el2ij]) {
            screened = true;
          } else if (C < Cmax[el2ij]) {
            need_derivative = true;
            const double Cmax_C = Cmax[el2ij] - C, C_Cmin = C - Cmin[el2ij];
            const double t = Cmax_C / C_Cmin;
            sij = sij - t * t;
            const double dCdrik = 4 * xik * fac * (1 + (C - 1) * xm);
            const double dCdrjk = 4 * xjk * fac * (1 - (C - 1) * xm);
            const double dCdrij = -(dCdrik + dCdrjk);
            fac = 2 * Cmax_C * dC[el2ij] / (C_Cmin * C_Cmin * C_Cmin);
            dsijdrij = dsijdrij + fac * dCdrij;
            ScrEntry e;
            e.k = k;
            e.kn = (int)kn;
            e.arik = fac * dCdrik / rlik;
            e.arjk = fac * dCdrjk / rljk;
            e.boik = e.bojk = 0.0;
            scr.push_back(e);
          }
        }
        if ((screened || sij < screening_threshold) && rlij > cut_in_h2[el2ij]) {
          scr.resize(ineb);  // fully screened: not a bond
          continue;
        }
        const double rl = std::sqrt(rlij);
        double fcin, dfcin;
        if (screened) {
          cut_in[el2ij].f(rl, fcin, dfcin);
          b.fcar = b.fcbo = fcin;
          b.dfcar = b.dfcbo = dfcin;
          scr.resize(ineb);
        } else if (need_derivative) {
          sij = std::exp(sij);
          double fcar, dfcar, fcbo, dfcbo;
          cut_in[el2ij].f(rl, fcin, dfcin);
          cut_out[el2ij].f(rl, fcar, dfcar);
          cut_bo[el2ij].f(rl, fcbo, dfcbo);
          b.fcar = (1.0 - fcin) * sij * fcar + fcin;
          b.dfcar = (1.0 - fcin) * sij * (dfcar + fcar * dsijdrij / rl) - dfcin * sij * fcar + dfcin;
          b.fcbo = (1.0 - fcin) * sij * fcbo + fcin;
          b.dfcbo = (1.0 - fcin) * sij * (dfcbo + fcbo * dsijdrij / rl) - dfcin * sij * fcbo + dfcin;
          for (size_t q = ineb; q < scr.size(); q++) {
            ScrEntry &e = scr[q];
            e.boik = e.arik * sij * fcbo * (1.0 - fcin);
            e.bojk = e.arjk * sij * fcbo * (1.0 - fcin);
            e.arik = e.arik * sij * fcar * (1.0 - fcin);
            e.arjk = e.arjk * sij * fcar * (1.0 - fcin);
          }
        } else {
          double fcar, dfcar, fcbo, dfcbo;
          cut_out[el2ij].f(rl, fcar, dfcar);
          cut_bo[el2ij].f(rl, fcbo, dfcbo);
          if (rl < cut_in_h[el2ij]) {
            cut_in[el2ij].f(rl, fcin, dfcin);
            b.fcar = (1.0 - fcin) * fcar + fcin;
            b.dfcar = (1.0 - fcin) * dfcar - dfcin * fcar + dfcin;
            b.fcbo = (1.0 - fcin) * fcbo + fcin;
            b.dfcbo = (1.0 - fcin) * dfcbo - dfcin * fcbo + dfcin;
          } else {
            b.fcar = fcar;
            b.dfcar = dfcar;
            b.fcbo = fcbo;
            b.dfcbo = dfcbo;
          }
        }
        b.s0 = ineb;
        b.s1 = (int)scr.size();
      } else if (rlij < cut_in_h2[el2ij]) {
        double fcin, dfcin;
        cut_in[el2ij].f(std::sqrt(rlij), fcin, dfcin);
        b.fcar = b.fcbo = fcin;
        b.dfcar = b.dfcbo = dfcin;
      } else {
        continue;
      }
      rlij = std::sqrt(rlij);
      b.len = rlij;
      for (int a = 0; a < 3; a++) b.nm[a] = rij[a] / rlij;
      bonds.push_back(b);
    }
  }
  int nebmax = 0;
  for (int i = 0; i < nat; i++) nebmax = std::max(nebmax, (int)bonds_of[i].size());

  // Pass 2 and the screening-force loop, thread-private accumulators (tls.f90).
  int nt = nthreads;
  std::vector<std::vector<double>> tpe(nt), tf(nt), twat(nt);
  std::vector<double> twpot(9 * nt, 0.0);
  std::vector<std::vector<double>> sfacbo_of(nat);
  const bool want_wat = o.wpot_per_at != nullptr;
  auto add_w = [&](std::vector<double> &wat, double wpot[3][3], int i, int j, int nbb,
                   const double wij[3][3]) {
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) wpot[a][c] += wij[a][c];
    if (o.wpot_per_bond)
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) o.wpot_per_bond[9 * (size_t)nbb + 3 * c + a] += wij[a][c];
    if (want_wat)
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++) {
          wat[9 * (size_t)i + 3 * c + a] += wij[a][c] / 2;
          wat[9 * (size_t)j + 3 * c + a] += wij[a][c] / 2;
        }
  };
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num();
#else
    const int tid = 0;
#endif
    std::vector<double> &pe = tpe[tid];
    std::vector<double> &f = tf[tid];
    std::vector<double> &wat = twat[tid];
    pe.assign(nat, 0.0);
    f.assign(3 * (size_t)nat, 0.0);
    if (want_wat) wat.assign(9 * (size_t)nat, 0.0);
    double wpot[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    std::vector<double> dbidk(3 * (size_t)std::max(nebmax, 1)), zfaci(std::max(nebmax, 1));
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < natloc; i++) {
      const int eli = el[i];
      if (eli < 0) continue;
      double fi[3] = {0, 0, 0};
      const std::vector<Bond> &bi = bonds_of[i];
      const std::vector<ScrEntry> &scr = scr_of[i];
      const int nb = (int)bi.size();
      std::vector<double> &sfacbo = sfacbo_of[i];
      sfacbo.assign(nb, 0.0);
      for (int ij = 0; ij < nb; ij++) {
        const Bond &B = bi[ij];
        const int j = B.j;
        int maskfac = 2;
        if (mask) {
          if (mask[i] == 0 && mask[j] == 0)
            maskfac = 0;
          else if (mask[i] == 0 || mask[j] == 0)
            maskfac = 1;
        }
        const int el2ij = B.typ;
        const double rlij = B.len;
        if (!(maskfac > 0 && rlij < cut_out_h[el2ij])) continue;
        double fj[3] = {0, 0, 0};
        const double rlijr = 1.0 / rlij;
        const double rnij[3] = {B.nm[0], B.nm[1], B.nm[2]};
        const double rij[3] = {rlij * rnij[0], rlij * rnij[1], rlij * rnij[2]};
        const double fcarij = B.fcar, dfcarijr = B.dfcar;
        double VAij, dVAij, VRij, dVRij;
        fn.VA(el2ij, rlij, VAij, dVAij);
        fn.VR(el2ij, rlij, VRij, dVRij);
        VAij = 0.5 * maskfac * VAij;
        dVAij = 0.5 * maskfac * dVAij;
        VRij = 0.5 * maskfac * VRij;
        dVRij = 0.5 * maskfac * dVRij;
        double wij[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double wijb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        double zij = 0.0;
        double dbidi[3] = {0, 0, 0}, dbidj[3] = {0, 0, 0};
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;
          const Bond &K = bi[ik];
          const int ikpot = K.typ;
          const double rlik = K.len;
          if (!(rlik < cut_bo_h[ikpot])) {
            zfaci[ik] = 0.0;
            dbidk[3 * ik] = dbidk[3 * ik + 1] = dbidk[3 * ik + 2] = 0.0;
            continue;
          }
          const double *rnik = K.nm;
          const double rik[3] = {rlik * rnik[0], rlik * rnik[1], rlik * rnik[2]};
          const double fcik = K.fcbo, dfcikr = K.dfcbo;
          double h_Dr, dh_dDr;
          fn.h(eli, el[j], el[K.j], ikpot, rlij - rlik, h_Dr, dh_dDr);
          const double costh = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
          double g_costh, dg_dcosth;
          fn.g(eli, ikpot, costh, g_costh, dg_dcosth);
          double dkc[3];
          for (int a = 0; a < 3; a++) dkc[a] = rnik[a] * rlik - rnij[a] * rlij;
          const double disjk = std::sqrt(dkc[0] * dkc[0] + dkc[1] * dkc[1] + dkc[2] * dkc[2]);
          for (int a = 0; a < 3; a++) dkc[a] = dkc[a] / disjk;
          const double dcsdij = 1.0 / rlik - costh * rlijr;
          const double dcsdik = rlijr - costh / rlik;
          const double dcsdjk = -disjk * rlijr / rlik;
          double dcsdi[3], dcsdj[3], dcsdk[3];
          for (int a = 0; a < 3; a++) {
            dcsdi[a] = -dcsdij * rnij[a] - dcsdik * rnik[a];
            dcsdj[a] = dcsdij * rnij[a] - dcsdjk * dkc[a];
            dcsdk[a] = dcsdik * rnik[a] + dcsdjk * dkc[a];
          }
          const double dzfac = fcik * dg_dcosth * h_Dr;
          double dgdi[3], dgdj[3], dgdk[3];
          for (int a = 0; a < 3; a++) {
            dgdi[a] = dzfac * dcsdi[a];
            dgdj[a] = dzfac * dcsdj[a];
            dgdk[a] = dzfac * dcsdk[a];
          }
          zfaci[ik] = g_costh * h_Dr;
          zij = zij + fcik * g_costh * h_Dr;
          const double dzdrij = g_costh * fcik * dh_dDr;
          const double dzdrik = g_costh * (dfcikr * h_Dr - fcik * dh_dDr);
          double df[3];
          for (int a = 0; a < 3; a++) {
            dbidi[a] = dbidi[a] - dzdrij * rnij[a] - dzdrik * rnik[a] + dgdi[a];
            df[a] = dzdrij * rnij[a] + dgdj[a];
            dbidj[a] = dbidj[a] + df[a];
            dbidk[3 * ik + a] = dzdrik * rnik[a] + dgdk[a];
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++)
              wijb[a][c] = wijb[a][c] - rij[a] * df[c] - rik[a] * dbidk[3 * ik + c];
        }
        double bij, dbij_dzij;
        fn.bo(eli, el2ij, zij, fcarij, VAij, bij, dbij_dzij);
        double dffac = 0.5 * fcarij * (VRij + bij * VAij);
        pe[i] = pe[i] + dffac;
        pe[j] = pe[j] + dffac;
        if (o.epot_per_bond) o.epot_per_bond[B.nbb] += dffac;
        dffac = 0.5 * (dVRij * fcarij + bij * dVAij * fcarij + VRij * dfcarijr +
                       bij * VAij * dfcarijr);
        double df[3];
        for (int a = 0; a < 3; a++) {
          df[a] = dffac * rnij[a];
          fi[a] = fi[a] + df[a];
          fj[a] = fj[a] - df[a];
        }
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++)
            wij[a][c] = wij[a][c] + rij[a] * df[c] - dbij_dzij * wijb[a][c];
        if (o.f_per_bond)
          for (int a = 0; a < 3; a++) o.f_per_bond[3 * (size_t)B.nbb + a] += df[a];
        for (int a = 0; a < 3; a++) fi[a] = fi[a] - dbij_dzij * dbidi[a];
        for (int a = 0; a < 3; a++) fj[a] = fj[a] - dbij_dzij * dbidj[a];
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;  // k == j and kdc == jdc (:1459)
          const int k = bi[ik].j;
          for (int a = 0; a < 3; a++)
            f[3 * (size_t)k + a] += -dbij_dzij * dbidk[3 * ik + a];
          if (bi[ik].s0 < bi[ik].s1) sfacbo[ik] = sfacbo[ik] + zfaci[ik] * dbij_dzij;
        }
        // forces on the screening neighbours of bond ij from the pair term
        const double dffac2 = 0.5 * (VRij + bij * VAij);
        for (int q = B.s0; q < B.s1; q++) {
          const ScrEntry &e = scr[q];
          double rik[3], rjk[3];
          get_rik(i, e.kn, rik);
          for (int a = 0; a < 3; a++) rjk[a] = -rij[a] + rik[a];
          for (int a = 0; a < 3; a++) {
            const double d1 = dffac2 * e.arik * rik[a];
            fi[a] = fi[a] + d1;
            f[3 * (size_t)e.k + a] += -d1;
            df[a] = d1;
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) wij[a][c] = wij[a][c] + rik[a] * df[c];
          for (int a = 0; a < 3; a++) {
            const double d2 = dffac2 * e.arjk * rjk[a];
            fj[a] = fj[a] + d2;
            f[3 * (size_t)e.k + a] += -d2;
            df[a] = d2;
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) wij[a][c] = wij[a][c] + rjk[a] * df[c];
        }
        add_w(wat, wpot, i, j, B.nbb, wij);
        for (int a = 0; a < 3; a++) f[3 * (size_t)j + a] += fj[a];
      }
      for (int a = 0; a < 3; a++) f[3 * (size_t)i + a] += fi[a];
    }
    // Screening forces through the bond-order cutoff (:1571-1611).
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < natloc; i++) {
      if (el[i] < 0) continue;
      double fi[3] = {0, 0, 0};
      const std::vector<Bond> &bi = bonds_of[i];
      const std::vector<ScrEntry> &scr = scr_of[i];
      for (int ij = 0; ij < (int)bi.size(); ij++) {
        const Bond &B = bi[ij];
        double fj[3] = {0, 0, 0};
        double wij[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        const double rij[3] = {B.len * B.nm[0], B.len * B.nm[1], B.len * B.nm[2]};
        const double sfac = sfacbo_of[i][ij];
        for (int q = B.s0; q < B.s1; q++) {
          const ScrEntry &e = scr[q];
          const double boik = sfac * e.boik, bojk = sfac * e.bojk;
          double rik[3], rjk[3], df[3];
          get_rik(i, e.kn, rik);
          for (int a = 0; a < 3; a++) rjk[a] = -rij[a] + rik[a];
          for (int a = 0; a < 3; a++) {
            df[a] = boik * rik[a];
            fi[a] = fi[a] + df[a];
            f[3 * (size_t)e.k + a] += -df[a];
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) wij[a][c] = wij[a][c] + rik[a] * df[c];
          for (int a = 0; a < 3; a++) {
            df[a] = bojk * rjk[a];
            fj[a] = fj[a] + df[a];
            f[3 * (size_t)e.k + a] += -df[a];
          }
          for (int a = 0; a < 3; a++)
            for (int c = 0; c < 3; c++) wij[a][c] = wij[a][c] + rjk[a] * df[c];
        }
        add_w(wat, wpot, i, B.j, B.nbb, wij);
        for (int a = 0; a < 3; a++) f[3 * (size_t)B.j + a] += fj[a];
      }
      for (int a = 0; a < 3; a++) f[3 * (size_t)i + a] += fi[a];
    }
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) twpot[9 * tid + 3 * a + c] = wpot[a][c];
  }
  double esum = 0.0;
  for (int t = 0; t < nt; t++) {
    if (tpe[t].empty()) continue;
    double s = 0.0;
    for (int i = 0; i < nat; i++) s += tpe[t][i];
    esum += 0.5 * s;
    for (size_t q = 0; q < 3 * (size_t)nat; q++) o.f[q] += tf[t][q];
    if (o.epot_per_at)
      for (int i = 0; i < nat; i++) o.epot_per_at[i] += 0.5 * tpe[t][i];
    if (want_wat)
      for (size_t q = 0; q < 9 * (size_t)nat; q++) o.wpot_per_at[q] += twat[t][q];
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) o.wpot[3 * c + a] += twpot[9 * t + 3 * a + c];
  }
  *o.epot += esum;
  return 0;
}

// ---------------------------------------------------------------------------
// Natural cubic spline on a uniform grid, simple_spline.f90.
// ---------------------------------------------------------------------------

struct Spline {
  int n = 0;
  double x0 = 0, dx = 1, cut = 0;
  std::vector<double> y, d2y, c1, c2, c3, d1, d2, d3;

  void init(int n_, double x0_, double dx_, const double *yy) {
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
    d2y[0] = 0.0;
    u[0] = 0.0;
    for (int i = 1; i < n - 1; i++) {
      double p = sig * d2y[i - 1] + 2;
      d2y[i] = (sig - 1) / p;
      u[i] = (6.0 * ((y[i + 1] - y[i]) / dx - (y[i] - y[i - 1]) / dx) / (2 * dx) -
              sig * u[i - 1]) /
             p;
    }
    const double qn = 0.0, un = 0.0;
    d2y[n - 1] = (un - qn * u[n - 2]) / (qn * d2y[n - 2] + 1.0);
    for (int k = n - 2; k >= 0; k--) d2y[k] = d2y[k] * d2y[k + 1] + u[k];
    for (int k = 0; k < n - 1; k++) {
      c1[k] = y[k + 1] - y[k] - (2 * d2y[k] + d2y[k + 1]) * (dx * dx) / 6;
      c2[k] = d2y[k] * (dx * dx) / 2;
      c3[k] = (d2y[k + 1] - d2y[k]) * (dx * dx) / 6;
    }
    for (int k = 0; k < n - 1; k++) {
      d1[k] = c1[k] / dx;
      d2[k] = 2 * c2[k] / dx;
      d3[k] = 3 * c3[k] / dx;
    }
    cut = x0 + dx * (n - 1);
  }
  void scale_y(double fac) {
    for (auto &v : y) v = fac * v;
    for (auto &v : d2y) v = fac * v;
    for (auto &v : c1) v = fac * v;
    for (auto &v : c2) v = fac * v;
    for (auto &v : c3) v = fac * v;
    for (auto &v : d1) v = fac * v;
    for (auto &v : d2) v = fac * v;
    for (auto &v : d3) v = fac * v;
  }
  // simple_spline_f (:373-434); 1-based interval index as in the reference.
  double f(double x, int *err) const {
    double xf;
    int i;
    if (x == cut) {
      xf = n;
      i = n - 1;
    } else {
      xf = (x - x0) / dx + 1;
      i = (int)std::floor(xf);
    }
    if (i < 1 || i >= n) {
      if (err) *err = -1;
      return 1.0;
    }
    double B = xf - i;
    int k = i - 1;
    return y[k] + B * (c1[k] + B * (c2[k] + B * c3[k]));
  }
  double df(double x, int *err) const {
    double xf;
    int i;
    if (x == cut) {
      xf = n;
      i = n - 1;
    } else {
      xf = (x - x0) / dx + 1;
      i = (int)std::floor(xf);
    }
    if (i < 1 || i >= n) {
      if (err) *err = -1;
      return 1.0;
    }
    double B = xf - i;
    int k = i - 1;
    return d1[k] + B * (d2[k] + B * d3[k]);
  }
  void f_and_df_extrap(double x, double &fv, double &dfv) const {
    double xf = (x - x0) / dx + 1;
    int i = (int)std::floor(xf);
    if (i < 1)
      i = 1;
    else if (i >= n)
      i = n - 1;
    double B = xf - i;
    int k = i - 1;
    fv = y[k] + B * (c1[k] + B * (c2[k] + B * c3[k]));
    dfv = d1[k] + B * (d2[k] + B * d3[k]);
  }
};

// The SPLINE_* macros of src/spline.inc (used by tabulated_eam.f90):
// xf = (x - x0) * (1/dx) + 1, i = int(xf) (truncation), no range check.
struct InlineSpline {
  const Spline *s;
  double rdx;
  explicit InlineSpline(const Spline &q) : s(&q), rdx(1.0 / q.dx) {}
  void at(double x, double &B, int &k, int *err) const {
    const double xf = (x - s->x0) * rdx + 1.0;
    int i = (int)xf;
    if (i < 1 || i >= s->n) {  // out of the table: undefined in the reference
      if (err) *err = -1;
      i = std::min(std::max(i, 1), s->n - 1);
    }
    B = xf - i;
    k = i - 1;
  }
  double f(double x, int *err) const {
    double B;
    int k;
    at(x, B, k, err);
    return s->y[k] + B * (s->c1[k] + B * (s->c2[k] + B * s->c3[k]));
  }
  double df(double x, int *err) const {
    double B;
    int k;
    at(x, B, k, err);
    return s->d1[k] + B * (s->d2[k] + B * s->d3[k]);
  }
};

// Single-element funcfl EAM (tabulated_eam.f90:147-200): F(rho), the
// effective charge Z(r) scaled by sqrt(Hartree Bohr / 2) (Units.f90:74-76),
// rho(r); no padding.
struct FuncflEAM {
  int Z = 0;
  double mass = 0, a0 = 0, cutoff = 0;
  Spline F, Zr, rho;
};

int funcfl_read(const char *fn, FuncflEAM &e) {
  std::ifstream in(fn);
  if (!in) return -1;
  std::string line;
  if (!std::getline(in, line)) return -2;  // comment
  if (!std::getline(in, line)) return -2;
  {
    std::istringstream ss(line);
    ss >> e.Z >> e.mass >> e.a0;
    if (!ss) return -3;
  }
  int nF, nr;
  double dF, dr;
  if (!std::getline(in, line)) return -2;
  {
    std::istringstream ss(line);
    ss >> nF >> dF >> nr >> dr >> e.cutoff;
    if (!ss) return -3;
  }
  auto read_values = [&](int n, std::vector<double> &v) {
    v.clear();
    std::string tok;
    while ((int)v.size() < n && (in >> tok)) v.push_back(std::strtod(tok.c_str(), nullptr));
    return (int)v.size() == n;
  };
  std::vector<double> v;
  if (!read_values(nF, v)) return -4;
  e.F.init(nF, 0.0, dF, v.data());
  if (!read_values(nr, v)) return -4;
  e.Zr.init(nr, 0.0, dr, v.data());
  if (!read_values(nr, v)) return -4;
  e.rho.init(nr, 0.0, dr, v.data());
  const double hartree = 27.2113961, bohr = 0.529177249;
  e.Zr.scale_y(std::sqrt(0.5 * hartree * bohr));
  return 0;
}

// tabulated_eam_energy_and_forces_kernel (tabulated_eam.f90:230-330): every
// atom is of the potential's element (elements = "*"); no mask, no per-atom
// virial (the reference leaves wpot_per_at untouched).
int funcfl_kernel(const FuncflEAM &e, int nat, const double *r, const Box &box, const NList &nl,
                  double *epot, double *fout, double *wpot, double *epot_per_at, int nthreads) {
  const double cutoff_sq = e.cutoff * e.cutoff;
  const InlineSpline sF(e.F), sZ(e.Zr), srho(e.rho);
  int nt = nthreads;
  std::vector<std::vector<double>> tsca(nt), tvec(nt);
  std::vector<double> tw(9 * nt, 0.0);
  int err_all = 0;
#pragma omp parallel num_threads(nthreads) reduction(| : err_all)
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num();
#else
    const int tid = 0;
#endif
    auto &sca = tsca[tid];
    auto &vec = tvec[tid];
    sca.assign(nat, 0.0);
    vec.assign(3 * (size_t)nat, 0.0);
    double w[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    std::vector<int> neb;
    std::vector<double> neb_dr, neb_abs;
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < nat; i++) {
      double rho = 0.0;
      neb.clear();
      neb_dr.clear();
      neb_abs.clear();
      int err = 0;
      for (int64_t ni = nl.seed[i]; ni < nl.seed[i + 1]; ni++) {
        const int j = nl.nbr[ni];
        const int *dc = &nl.dc[3 * ni];
        double dr[3];
        for (int a = 0; a < 3; a++) {
          double as = box.A[a][0] * (double)dc[0];
          as = as + box.A[a][1] * (double)dc[1];
          as = as + box.A[a][2] * (double)dc[2];
          dr[a] = (r[3 * i + a] - r[3 * j + a]) + as;
        }
        double abs_dr = dr[0] * dr[0];
        abs_dr = abs_dr + dr[1] * dr[1];
        abs_dr = abs_dr + dr[2] * dr[2];
        if (abs_dr < cutoff_sq) {
          abs_dr = std::sqrt(abs_dr);
          rho = rho + srho.f(abs_dr, &err);
          neb.push_back(j);
          neb_dr.insert(neb_dr.end(), dr, dr + 3);
          neb_abs.push_back(abs_dr);
        }
      }
      if (rho < 0.0) rho = 0.0;
      double B;
      int k;
      sF.at(rho, B, k, &err);
      const double Fi = e.F.y[k] + B * (e.F.c1[k] + B * (e.F.c2[k] + B * e.F.c3[k]));
      const double dFi = e.F.d1[k] + B * (e.F.d2[k] + B * e.F.d3[k]);
      if (err) err_all |= 1;
      sca[i] = sca[i] + Fi;
      double esum = 0.0, fori[3] = {0, 0, 0};
      for (size_t q = 0; q < neb.size(); q++) {
        const double rr = neb_abs[q];
        int e2 = 0;
        sZ.at(rr, B, k, &e2);
        double phi = e.Zr.y[k] + B * (e.Zr.c1[k] + B * (e.Zr.c2[k] + B * e.Zr.c3[k]));
        double dphi = e.Zr.d1[k] + B * (e.Zr.d2[k] + B * e.Zr.d3[k]);
        dphi = 2 * phi * dphi / rr;
        phi = phi * phi / rr;
        dphi = dphi - phi / rr;
        esum = esum + phi;
        const double fac = srho.df(rr, &e2);
        if (e2) err_all |= 1;
        const double *dr = &neb_dr[3 * q];
        const double sc = -((dFi * fac + dphi) / rr);
        double df[3];
        for (int a = 0; a < 3; a++) df[a] = sc * dr[a];
        const int j = neb[q];
        for (int a = 0; a < 3; a++) {
          fori[a] = fori[a] + df[a];
          vec[3 * (size_t)j + a] = vec[3 * (size_t)j + a] - df[a];
        }
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++) w[a][c] = w[a][c] + (-dr[a] * df[c]);
      }
      sca[i] = sca[i] + esum;
      for (int a = 0; a < 3; a++) vec[3 * (size_t)i + a] += fori[a];
    }
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) tw[9 * tid + 3 * a + c] = w[a][c];
  }
  double esum = 0.0;
  for (int t = 0; t < nt; t++) {
    if (tsca[t].empty()) continue;
    for (int i = 0; i < nat; i++) esum += tsca[t][i];
    for (size_t q = 0; q < 3 * (size_t)nat; q++) fout[q] += tvec[t][q];
    if (epot_per_at)
      for (int i = 0; i < nat; i++) epot_per_at[i] += tsca[t][i];
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) wpot[3 * c + a] += tw[9 * t + 3 * a + c];
  }
  *epot = esum;
  return err_all ? -5 : 0;
}

struct EAM {
  int nel = 0;
  std::vector<int> Z;
  double cutoff = 0;
  std::vector<Spline> F, rho, phi;  // phi[i*nel+j], symmetric copies
};

// setfl reader, tabulated_alloy_eam.f90:147-259 (read_ascii takes
// whitespace-separated values across lines).
int eam_read(const char *fn, EAM &e) {
  std::ifstream in(fn);
  if (!in) return -1;
  std::string line;
  for (int i = 0; i < 3; i++)
    if (!std::getline(in, line)) return -2;
  if (!std::getline(in, line)) return -2;
  {
    std::istringstream ss(line);
    ss >> e.nel;
    if (!ss || e.nel <= 0) return -3;
  }
  int nF, nr;
  double dF, dr;
  if (!std::getline(in, line)) return -2;
  {
    std::istringstream ss(line);
    ss >> nF >> dF >> nr >> dr >> e.cutoff;
    if (!ss) return -3;
  }
  auto read_values = [&](int n, std::vector<double> &v) {
    v.clear();
    std::string tok;
    while ((int)v.size() < n && (in >> tok)) v.push_back(std::strtod(tok.c_str(), nullptr));
    std::getline(in, line);  // rest of the last line
    return (int)v.size() == n;
  };
  e.Z.resize(e.nel);
  e.F.resize(e.nel);
  e.rho.resize(e.nel);
  e.phi.resize((size_t)e.nel * e.nel);
  std::vector<double> v;
  for (int i = 0; i < e.nel; i++) {
    if (!std::getline(in, line)) return -2;
    std::istringstream ss(line);
    ss >> e.Z[i];
    if (!read_values(nF, v)) return -4;
    e.F[i].init(nF, 0.0, dF, v.data());
    if (!read_values(nr, v)) return -4;
    v.push_back(0.0);
    v.push_back(0.0);
    e.rho[i].init(nr + 2, 0.0, dr, v.data());
  }
  for (int i = 0; i < e.nel; i++)
    for (int j = 0; j <= i; j++) {
      if (!read_values(nr, v)) return -4;
      v.push_back(0.0);
      v.push_back(0.0);
      Spline s;
      s.init(nr + 2, 0.0, dr, v.data());
      s.scale_y(0.5);
      e.phi[(size_t)i * e.nel + j] = s;
      e.phi[(size_t)j * e.nel + i] = s;
    }
  return 0;
}

// tabulated_alloy_eam_energy_and_forces_kernel (:423-627).  db[i] is the
// 0-based table index of atom i or -1.
int eam_kernel(const EAM &e, int nat, const double *r, const Box &box, const int *db,
               const NList &nl, const int *mask, double *epot, double *fout, double *wpot,
               double *epot_per_at, double *wpot_per_at, int nthreads) {
  const double cutoff_sq = e.cutoff * e.cutoff;
  int nt = nthreads;
  std::vector<std::vector<double>> tsca(nt), tvec(nt), twat(nt);
  std::vector<double> tw(9 * nt, 0.0), te(nt, 0.0);
  int err_all = 0;
  const bool want_wat = wpot_per_at != nullptr;
#pragma omp parallel num_threads(nthreads) reduction(| : err_all)
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num();
#else
    const int tid = 0;
#endif
    auto &sca = tsca[tid];
    auto &vec = tvec[tid];
    auto &wat = twat[tid];
    sca.assign(nat, 0.0);
    vec.assign(3 * (size_t)nat, 0.0);
    if (want_wat) wat.assign(9 * (size_t)nat, 0.0);
    double w[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    std::vector<int> neb;
    std::vector<double> neb_dr, neb_abs;
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < nat; i++) {
      if (mask && mask[i] == 0) continue;
      const int dbi = db[i];
      if (dbi < 0) continue;
      double rho = 0.0;
      neb.clear();
      neb_dr.clear();
      neb_abs.clear();
      for (int64_t ni = nl.seed[i]; ni < nl.seed[i + 1]; ni++) {
        const int j = nl.nbr[ni];
        const int dbj = db[j];
        if (dbj < 0) continue;
        const int *dc = &nl.dc[3 * ni];
        double dr[3];
        for (int a = 0; a < 3; a++) {
          double as = box.A[a][0] * (double)dc[0];
          as = as + box.A[a][1] * (double)dc[1];
          as = as + box.A[a][2] * (double)dc[2];
          dr[a] = (r[3 * i + a] - r[3 * j + a]) + as;
        }
        double abs_dr = dr[0] * dr[0];
        abs_dr = abs_dr + dr[1] * dr[1];
        abs_dr = abs_dr + dr[2] * dr[2];
        if (abs_dr < cutoff_sq) {
          abs_dr = std::sqrt(abs_dr);
          int err = 0;
          double drho = e.rho[dbj].f(abs_dr, &err);
          if (err) err_all |= 1;
          rho = rho + drho;
          neb.push_back(j);
          neb_dr.insert(neb_dr.end(), dr, dr + 3);
          neb_abs.push_back(abs_dr);
        }
      }
      if (rho < 0.0) rho = 0.0;
      double Fi, dFi;
      e.F[dbi].f_and_df_extrap(rho, Fi, dFi);
      sca[i] = sca[i] + Fi;
      double fori[3] = {0, 0, 0};
      for (size_t q = 0; q < neb.size(); q++) {
        const int j = neb[q];
        const int dbj = db[j];
        const double *dr = &neb_dr[3 * q];
        const double abs_dr = neb_abs[q];
        double phi, dphi;
        e.phi[(size_t)dbi * e.nel + dbj].f_and_df_extrap(abs_dr, phi, dphi);
        const double r_abs_dr = 1.0 / abs_dr;
        sca[i] = sca[i] + phi * r_abs_dr;
        int err = 0;
        const double fac = e.rho[dbj].df(abs_dr, &err);
        if (err) err_all |= 1;
        double df[3];
        for (int a = 0; a < 3; a++)
          df[a] = -(dFi * fac + (dphi - phi * r_abs_dr) * r_abs_dr) * r_abs_dr * dr[a];
        for (int a = 0; a < 3; a++) {
          fori[a] = fori[a] + df[a];
          vec[3 * (size_t)j + a] = vec[3 * (size_t)j + a] - df[a];
        }
        for (int a = 0; a < 3; a++)
          for (int c = 0; c < 3; c++) {
            double wij = -dr[a] * df[c];
            w[a][c] = w[a][c] + wij;
            if (want_wat) {
              wat[9 * (size_t)i + 3 * c + a] += wij / 2;
              wat[9 * (size_t)j + 3 * c + a] += wij / 2;
            }
          }
      }
      for (int a = 0; a < 3; a++) vec[3 * (size_t)i + a] += fori[a];
    }
    double s = 0.0;
    for (int i = 0; i < nat; i++) s += sca[i];
    te[tid] = s;
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) tw[9 * tid + 3 * a + c] = w[a][c];
  }
  double esum = 0.0;
  for (int t = 0; t < nt; t++) {
    if (tsca[t].empty()) continue;
    esum += te[t];
    for (size_t q = 0; q < 3 * (size_t)nat; q++) fout[q] += tvec[t][q];
    if (epot_per_at)
      for (int i = 0; i < nat; i++) epot_per_at[i] += tsca[t][i];
    if (want_wat)
      for (size_t q = 0; q < 9 * (size_t)nat; q++) wpot_per_at[q] += twat[t][q];
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++) wpot[3 * c + a] += tw[9 * t + 3 * a + c];
  }
  *epot += esum;
  return err_all ? -2 : 0;
}

int resolve_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  nthreads = 1;
#endif
  return nthreads < 1 ? 1 : nthreads;
}

// View an externally supplied CSR list as an NList (copying).
void nl_from_arrays(int nat, const int64_t *seed, const int *nbr, const int *dc, NList &nl) {
  nl.seed.assign(seed, seed + nat + 1);
  nl.nbr.assign(nbr, nbr + seed[nat]);
  nl.dc.assign(dc, dc + 3 * seed[nat]);
}

}  // namespace

// ============================================================================
// C entry points (ctypes, tests and bench.py's CPU baseline only).
// ============================================================================

extern "C" {

struct orc_nlist {
  NList nl;
};

// Builds the full directed neighbour list.  Returns a handle or NULL.
orc_nlist *orc_neighbors_build(int nat, const double *r, const double *cell, const int *pbc,
                               double cutoff) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return nullptr;
  orc_nlist *h = new orc_nlist;
  build_neighbors(nat, r, box, cutoff, h->nl);
  return h;
}

int64_t orc_neighbors_size(const orc_nlist *h) { return (int64_t)h->nl.nbr.size(); }

void orc_neighbors_copy(const orc_nlist *h, int64_t *seed, int *nbr, int *dc) {
  std::copy(h->nl.seed.begin(), h->nl.seed.end(), seed);
  std::copy(h->nl.nbr.begin(), h->nl.nbr.end(), nbr);
  std::copy(h->nl.dc.begin(), h->nl.dc.end(), dc);
}

void orc_neighbors_free(orc_nlist *h) { delete h; }

void orc_cell_inverse(const double *cell, double *Bbox_rowmajor) {
  Box box;
  int pbc[3] = {1, 1, 1};
  make_box(cell, pbc, box);
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) Bbox_rowmajor[3 * a + k] = box.B[a][k];
}

static int map_elements(int nat, const int *Z, int nel, const int *dbZ, std::vector<int> &el) {
  el.assign(nat, -1);
  for (int i = 0; i < nat; i++)
    for (int q = 0; q < nel; q++)
      if (Z[i] == dbZ[q]) el[i] = q;
  return 0;
}

// Interaction range requested by BIND_TO_FUNC for the elements present
// (default_bind_to_func.f90:123-144).
static double bop_range(int nat, const std::vector<int> &el, int nel, const double *r2) {
  std::vector<int> present(nel, 0);
  for (int i = 0; i < nat; i++)
    if (el[i] >= 0) present[el[i]] = 1;
  double range = 0.0;
  for (int a = 0; a < nel; a++)
    for (int b = 0; b < nel; b++)
      if (present[a] && present[b]) range = std::max(range, r2[pair_index(a, b, nel)]);
  return range;
}

double orc_tersoff_cutoff(const orc_tersoff_params *p, int nat, const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return bop_range(nat, el, p->nel, p->r2);
}

double orc_kumagai_cutoff(const orc_kumagai_params *p, int nat, const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return bop_range(nat, el, p->nel, p->r2);
}

// energy_and_forces on an explicit neighbour list.  Outputs are accumulated
// into (f, wpot, per-atom, per-bond) as the reference does; epot is set.
int orc_tersoff_kernel(const orc_tersoff_params *p, int nat, const double *r,
                       const double *cell, const int *pbc, const int *Z,
                       const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                       double *epot, double *f, double *wpot, double *epot_per_at,
                       double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                       double *wpot_per_bond, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc, nl);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return bop_kernel(TersoffFn(*p), nat, r, box, el.data(), nl, mask, o,
                    resolve_threads(nthreads));
}

int orc_kumagai_kernel(const orc_kumagai_params *p, int nat, const double *r,
                       const double *cell, const int *pbc, const int *Z,
                       const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                       double *epot, double *f, double *wpot, double *epot_per_at,
                       double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                       double *wpot_per_bond, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc, nl);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return bop_kernel(KumagaiFn(*p), nat, r, box, el.data(), nl, mask, o,
                    resolve_threads(nthreads));
}

// Full COMPUTE_FUNC: neighbour build + kernel (no per-bond outputs).
int orc_tersoff_compute(const orc_tersoff_params *p, int nat, const double *r,
                        const double *cell, const int *pbc, const int *Z, const int *mask,
                        double *epot, double *f, double *wpot, double *epot_per_at,
                        double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  double cutoff = bop_range(nat, el, p->nel, p->r2);
  NList nl;
  if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
  else nl.seed.assign(nat + 1, 0);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return bop_kernel(TersoffFn(*p), nat, r, box, el.data(), nl, mask, o,
                    resolve_threads(nthreads));
}

int orc_kumagai_compute(const orc_kumagai_params *p, int nat, const double *r,
                        const double *cell, const int *pbc, const int *Z, const int *mask,
                        double *epot, double *f, double *wpot, double *epot_per_at,
                        double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  double cutoff = bop_range(nat, el, p->nel, p->r2);
  NList nl;
  if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
  else nl.seed.assign(nat + 1, 0);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return bop_kernel(KumagaiFn(*p), nat, r, box, el.data(), nl, mask, o,
                    resolve_threads(nthreads));
}

// Interaction range of the screened variants for the elements present
// (default_bind_to_func.f90:117-144): sqrt(C_dr_cut(pair)) times the largest
// of all pairs' max(r2, or2, bor2).
static double scr_range(int nat, const std::vector<int> &el, int nel, const double *r2,
                        const orc_scr_params &sp) {
  const int npairs = nel * (nel + 1) / 2;
  double mx = 0.0;
  for (int q = 0; q < npairs; q++) {
    const double m = std::max(std::max(r2[q], sp.or2[q]), sp.bor2[q]);
    mx = std::max(mx, m * m);
  }
  std::vector<int> present(nel, 0);
  for (int i = 0; i < nat; i++)
    if (el[i] >= 0) present[el[i]] = 1;
  double range = 0.0;
  for (int a = 0; a < nel; a++)
    for (int b = 0; b < nel; b++)
      if (present[a] && present[b]) {
        const int q = pair_index(a, b, nel);
        const double cdr = sp.Cmax[q] > 2.0 ? sp.Cmax[q] * sp.Cmax[q] / (4 * (sp.Cmax[q] - 1))
                                            : 1.0;
        range = std::max(range, std::sqrt(cdr) * std::sqrt(mx));
      }
  return range;
}

double orc_tersoff_scr_cutoff(const orc_tersoff_params *p, const orc_scr_params *sp, int nat,
                              const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return scr_range(nat, el, p->nel, p->r2, *sp);
}

double orc_kumagai_scr_cutoff(const orc_kumagai_params *p, const orc_scr_params *sp, int nat,
                              const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return scr_range(nat, el, p->nel, p->r2, *sp);
}

int orc_tersoff_scr_kernel(const orc_tersoff_params *p, const orc_scr_params *sp, int nat,
                           const double *r, const double *cell, const int *pbc, const int *Z,
                           const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                           double *epot, double *f, double *wpot, double *epot_per_at,
                           double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                           double *wpot_per_bond, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc, nl);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return bop_kernel_scr(TersoffFn(*p), *sp, nat, r, box, el.data(), nl, mask, o,
                        resolve_threads(nthreads));
}

int orc_kumagai_scr_kernel(const orc_kumagai_params *p, const orc_scr_params *sp, int nat,
                           const double *r, const double *cell, const int *pbc, const int *Z,
                           const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                           double *epot, double *f, double *wpot, double *epot_per_at,
                           double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                           double *wpot_per_bond, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc, nl);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return bop_kernel_scr(KumagaiFn(*p), *sp, nat, r, box, el.data(), nl, mask, o,
                        resolve_threads(nthreads));
}

// Neighbour build + screened kernel (the CPU baseline's timed unit).
int orc_tersoff_scr_compute(const orc_tersoff_params *p, const orc_scr_params *sp, int nat,
                            const double *r, const double *cell, const int *pbc, const int *Z,
                            const int *mask, double *epot, double *f, double *wpot,
                            double *epot_per_at, double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  double cutoff = scr_range(nat, el, p->nel, p->r2, *sp);
  NList nl;
  if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
  else nl.seed.assign(nat + 1, 0);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return bop_kernel_scr(TersoffFn(*p), *sp, nat, r, box, el.data(), nl, mask, o,
                        resolve_threads(nthreads));
}

int orc_kumagai_scr_compute(const orc_kumagai_params *p, const orc_scr_params *sp, int nat,
                            const double *r, const double *cell, const int *pbc, const int *Z,
                            const int *mask, double *epot, double *f, double *wpot,
                            double *epot_per_at, double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  double cutoff = scr_range(nat, el, p->nel, p->r2, *sp);
  NList nl;
  if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
  else nl.seed.assign(nat + 1, 0);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return bop_kernel_scr(KumagaiFn(*p), *sp, nat, r, box, el.data(), nl, mask, o,
                        resolve_threads(nthreads));
}

// Brenner entry points.  The screened interaction range differs from the
// default bind_to: sqrt(C_dr_cut) times max(r2, or2, bor2) of the same pair
// (brenner_module.f90:191-243), not of all pairs.
static double brenner_scr_range(int nat, const std::vector<int> &el, const orc_brenner_params &p,
                                const orc_scr_params &sp) {
  const int nel = p.nel;
  std::vector<int> present(nel, 0);
  for (int i = 0; i < nat; i++)
    if (el[i] >= 0) present[el[i]] = 1;
  double range = 0.0;
  for (int a = 0; a < nel; a++)
    for (int b = 0; b < nel; b++)
      if (present[a] && present[b]) {
        const int q = pair_index(a, b, nel);
        const double cdr = sp.Cmax[q] > 2.0 ? sp.Cmax[q] * sp.Cmax[q] / (4 * (sp.Cmax[q] - 1))
                                            : 1.0;
        const double mc = std::max(std::max(p.r2[q], sp.or2[q]), sp.bor2[q]);
        range = std::max(range, std::sqrt(cdr) * std::sqrt(mc * mc));
      }
  return range;
}

double orc_brenner_cutoff(const orc_brenner_params *p, int nat, const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return bop_range(nat, el, p->nel, p->r2);
}

double orc_brenner_scr_cutoff(const orc_brenner_params *p, const orc_scr_params *sp, int nat,
                              const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  return brenner_scr_range(nat, el, *p, *sp);
}

// sp == NULL: Brenner; else BrennerScr.  nl_seed == NULL: the list is built
// here (compute); else it is the caller's (kernel).
static int brenner_run(const orc_brenner_params *p, const orc_scr_params *sp, int nat,
                       const double *r, const double *cell, const int *pbc, const int *Z,
                       const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                       const BopOut &o, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  NList nl;
  if (seed) {
    nl_from_arrays(nat, seed, nbr, dc, nl);
  } else {
    const double cutoff =
        sp ? brenner_scr_range(nat, el, *p, *sp) : bop_range(nat, el, p->nel, p->r2);
    if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
    else nl.seed.assign(nat + 1, 0);
  }
  *o.epot = 0.0;
  const BrennerFn fn(*p);
  const int nt = resolve_threads(nthreads);
  return sp ? bop_kernel_scr(fn, *sp, nat, r, box, el.data(), nl, mask, o, nt)
            : bop_kernel(fn, nat, r, box, el.data(), nl, mask, o, nt);
}

int orc_brenner_kernel(const orc_brenner_params *p, int nat, const double *r, const double *cell,
                       const int *pbc, const int *Z, const int64_t *seed, const int *nbr,
                       const int *dc, const int *mask, double *epot, double *f, double *wpot,
                       double *epot_per_at, double *epot_per_bond, double *f_per_bond,
                       double *wpot_per_at, double *wpot_per_bond, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return brenner_run(p, nullptr, nat, r, cell, pbc, Z, seed, nbr, dc, mask, o, nthreads);
}

int orc_brenner_scr_kernel(const orc_brenner_params *p, const orc_scr_params *sp, int nat,
                           const double *r, const double *cell, const int *pbc, const int *Z,
                           const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                           double *epot, double *f, double *wpot, double *epot_per_at,
                           double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                           double *wpot_per_bond, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return brenner_run(p, sp, nat, r, cell, pbc, Z, seed, nbr, dc, mask, o, nthreads);
}

int orc_brenner_compute(const orc_brenner_params *p, int nat, const double *r, const double *cell,
                        const int *pbc, const int *Z, const int *mask, double *epot, double *f,
                        double *wpot, double *epot_per_at, double *wpot_per_at, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return brenner_run(p, nullptr, nat, r, cell, pbc, Z, nullptr, nullptr, nullptr, mask, o,
                     nthreads);
}

int orc_brenner_scr_compute(const orc_brenner_params *p, const orc_scr_params *sp, int nat,
                            const double *r, const double *cell, const int *pbc, const int *Z,
                            const int *mask, double *epot, double *f, double *wpot,
                            double *epot_per_at, double *wpot_per_at, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return brenner_run(p, sp, nat, r, cell, pbc, Z, nullptr, nullptr, nullptr, mask, o, nthreads);
}

// Juslin entry points.  The screening parameters take the mirror fill of
// juslin_module.f90:273-300 as well; the screened range is sqrt(C_dr_cut) of
// the pair times the largest max(r2, or2, bor2) of all pairs
// (juslin_module.f90:381-404), C_dr_cut without the Cmax > 2 guard.
static orc_scr_params juslin_fill_scr(const orc_juslin_params &p, const orc_scr_params &sp) {
  orc_scr_params q = sp;
  const int nel = p.nel;
  for (int i = 0; i < nel; i++)
    for (int j = 0; j < nel; j++) {
      const int a = j + i * nel, b = i + j * nel;
      if (p.r0[a] < 0.0) {
        q.or1[a] = q.or1[b];
        q.or2[a] = q.or2[b];
        q.bor1[a] = q.bor1[b];
        q.bor2[a] = q.bor2[b];
        q.Cmin[a] = q.Cmin[b];
        q.Cmax[a] = q.Cmax[b];
      }
    }
  return q;
}

static double juslin_range(int nat, const std::vector<int> &el, const JuslinFn &fn,
                           const orc_scr_params *sp) {
  const int nel = fn.nel();
  (void)nel;
  std::vector<int> present(nel, 0);
  for (int i = 0; i < nat; i++)
    if (el[i] >= 0) present[el[i]] = 1;
  double mx = 0.0;
  if (sp)
    for (int q = 0; q < nel * nel; q++) {
      const double m = std::max(std::max(fn.p.r2[q], sp->or2[q]), sp->bor2[q]);
      mx = std::max(mx, m * m);
    }
  double range = 0.0;
  for (int a = 0; a < nel; a++)
    for (int b = 0; b < nel; b++)
      if (present[a] && present[b]) {
        const int q = fn.pair(a, b);
        if (!sp) {
          range = std::max(range, fn.p.r2[q]);
        } else {
          const double cdr = sp->Cmax[q] * sp->Cmax[q] / (4 * (sp->Cmax[q] - 1));
          range = std::max(range, std::sqrt(cdr) * std::sqrt(mx));
        }
      }
  return range;
}

static double juslin_cutoff(const orc_juslin_params *p, const orc_scr_params *sp, int nat,
                            const int *Z) {
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  const JuslinFn fn(*p);
  if (!sp) return juslin_range(nat, el, fn, nullptr);
  const orc_scr_params q = juslin_fill_scr(*p, *sp);
  return juslin_range(nat, el, fn, &q);
}

// sp == NULL: Juslin; else JuslinScr.  seed == NULL: the list is built here.
static int juslin_run(const orc_juslin_params *p, const orc_scr_params *sp, int nat,
                      const double *r, const double *cell, const int *pbc, const int *Z,
                      const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                      const BopOut &o, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> el;
  map_elements(nat, Z, p->nel, p->Z, el);
  const JuslinFn fn(*p);
  orc_scr_params q{};
  if (sp) q = juslin_fill_scr(*p, *sp);
  NList nl;
  if (seed) {
    nl_from_arrays(nat, seed, nbr, dc, nl);
  } else {
    const double cutoff = juslin_range(nat, el, fn, sp ? &q : nullptr);
    if (cutoff > 0) build_neighbors(nat, r, box, cutoff, nl);
    else nl.seed.assign(nat + 1, 0);
  }
  *o.epot = 0.0;
  const int nt = resolve_threads(nthreads);
  return sp ? bop_kernel_scr(fn, q, nat, r, box, el.data(), nl, mask, o, nt)
            : bop_kernel(fn, nat, r, box, el.data(), nl, mask, o, nt);
}

double orc_juslin_cutoff(const orc_juslin_params *p, int nat, const int *Z) {
  return juslin_cutoff(p, nullptr, nat, Z);
}

double orc_juslin_scr_cutoff(const orc_juslin_params *p, const orc_scr_params *sp, int nat,
                             const int *Z) {
  return juslin_cutoff(p, sp, nat, Z);
}

int orc_juslin_kernel(const orc_juslin_params *p, int nat, const double *r, const double *cell,
                      const int *pbc, const int *Z, const int64_t *seed, const int *nbr,
                      const int *dc, const int *mask, double *epot, double *f, double *wpot,
                      double *epot_per_at, double *epot_per_bond, double *f_per_bond,
                      double *wpot_per_at, double *wpot_per_bond, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return juslin_run(p, nullptr, nat, r, cell, pbc, Z, seed, nbr, dc, mask, o, nthreads);
}

int orc_juslin_scr_kernel(const orc_juslin_params *p, const orc_scr_params *sp, int nat,
                          const double *r, const double *cell, const int *pbc, const int *Z,
                          const int64_t *seed, const int *nbr, const int *dc, const int *mask,
                          double *epot, double *f, double *wpot, double *epot_per_at,
                          double *epot_per_bond, double *f_per_bond, double *wpot_per_at,
                          double *wpot_per_bond, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, epot_per_bond, f_per_bond, wpot_per_at, wpot_per_bond};
  return juslin_run(p, sp, nat, r, cell, pbc, Z, seed, nbr, dc, mask, o, nthreads);
}

int orc_juslin_compute(const orc_juslin_params *p, int nat, const double *r, const double *cell,
                       const int *pbc, const int *Z, const int *mask, double *epot, double *f,
                       double *wpot, double *epot_per_at, double *wpot_per_at, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return juslin_run(p, nullptr, nat, r, cell, pbc, Z, nullptr, nullptr, nullptr, mask, o,
                    nthreads);
}

int orc_juslin_scr_compute(const orc_juslin_params *p, const orc_scr_params *sp, int nat,
                           const double *r, const double *cell, const int *pbc, const int *Z,
                           const int *mask, double *epot, double *f, double *wpot,
                           double *epot_per_at, double *wpot_per_at, int nthreads) {
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  return juslin_run(p, sp, nat, r, cell, pbc, Z, nullptr, nullptr, nullptr, mask, o, nthreads);
}

// The LAMMPS contract (bop_kernel.f90 under LAMMPS): nat = local + ghost
// atoms with explicit positions, a shift-free list over all of them, bonds of
// the first natloc atoms; kind 0 Tersoff, 1 Kumagai, 2 Brenner, 3 Juslin; sp != NULL:
// screened.
int orc_bop_ghost(int kind, const void *params, const orc_scr_params *sp, int nat, int natloc,
                  const double *r, const int *Z, const int64_t *seed, const int *nbr,
                  const int *mask, double *epot, double *f, double *wpot, double *epot_per_at,
                  double *wpot_per_at, int nthreads) {
  const double eye[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const int nopbc[3] = {0, 0, 0};
  Box box;
  if (make_box(eye, nopbc, box) != 0) return -1;
  const int64_t n = seed[nat];
  std::vector<int> dc(3 * (size_t)std::max<int64_t>(n, 1), 0);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc.data(), nl);
  *epot = 0.0;
  BopOut o{epot, f, wpot, epot_per_at, nullptr, nullptr, wpot_per_at, nullptr};
  std::vector<int> el;
  const int nt = resolve_threads(nthreads);
  if (kind == 0) {
    const orc_tersoff_params *p = static_cast<const orc_tersoff_params *>(params);
    map_elements(nat, Z, p->nel, p->Z, el);
    return sp ? bop_kernel_scr(TersoffFn(*p), *sp, nat, r, box, el.data(), nl, mask, o, nt,
                               natloc)
              : bop_kernel(TersoffFn(*p), nat, r, box, el.data(), nl, mask, o, nt, natloc);
  }
  if (kind == 3) {
    const orc_juslin_params *p = static_cast<const orc_juslin_params *>(params);
    map_elements(nat, Z, p->nel, p->Z, el);
    const JuslinFn fn(*p);
    if (!sp) return bop_kernel(fn, nat, r, box, el.data(), nl, mask, o, nt, natloc);
    const orc_scr_params q = juslin_fill_scr(*p, *sp);
    return bop_kernel_scr(fn, q, nat, r, box, el.data(), nl, mask, o, nt, natloc);
  }
  if (kind == 2) {
    const orc_brenner_params *p = static_cast<const orc_brenner_params *>(params);
    map_elements(nat, Z, p->nel, p->Z, el);
    const BrennerFn fn(*p);
    return sp ? bop_kernel_scr(fn, *sp, nat, r, box, el.data(), nl, mask, o, nt, natloc)
              : bop_kernel(fn, nat, r, box, el.data(), nl, mask, o, nt, natloc);
  }
  const orc_kumagai_params *p = static_cast<const orc_kumagai_params *>(params);
  map_elements(nat, Z, p->nel, p->Z, el);
  return sp ? bop_kernel_scr(KumagaiFn(*p), *sp, nat, r, box, el.data(), nl, mask, o, nt, natloc)
            : bop_kernel(KumagaiFn(*p), nat, r, box, el.data(), nl, mask, o, nt, natloc);
}

struct orc_funcfl {
  FuncflEAM e;
};

orc_funcfl *orc_funcfl_load(const char *fn, int *err) {
  orc_funcfl *h = new orc_funcfl;
  const int rc = funcfl_read(fn, h->e);
  if (err) *err = rc;
  if (rc != 0) {
    delete h;
    return nullptr;
  }
  return h;
}
void orc_funcfl_free(orc_funcfl *h) { delete h; }
double orc_funcfl_cutoff(const orc_funcfl *h) { return h->e.cutoff; }

// Neighbour build with the file's cutoff + kernel.
int orc_funcfl_compute(const orc_funcfl *h, int nat, const double *r, const double *cell,
                       const int *pbc, double *epot, double *f, double *wpot,
                       double *epot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  NList nl;
  build_neighbors(nat, r, box, h->e.cutoff, nl);
  return funcfl_kernel(h->e, nat, r, box, nl, epot, f, wpot, epot_per_at,
                       resolve_threads(nthreads));
}

struct orc_eam {
  EAM e;
};

orc_eam *orc_eam_load(const char *fn, int *ierr) {
  orc_eam *h = new orc_eam;
  int rc = eam_read(fn, h->e);
  if (ierr) *ierr = rc;
  if (rc != 0) {
    delete h;
    return nullptr;
  }
  return h;
}

void orc_eam_free(orc_eam *h) { delete h; }
double orc_eam_cutoff(const orc_eam *h) { return h->e.cutoff; }
int orc_eam_nel(const orc_eam *h) { return h->e.nel; }

// Spline table export: which = 0 (F), 1 (rho), 2 (phi, i*nel+j).
// Returns n; fills x0dx[3] = {x0, dx, cut} and coef (8*n slots: y, d2y, then
// c1,c2,c3,d1,d2,d3 each n-1 long, padded to n) when coef != NULL.
int orc_eam_table(const orc_eam *h, int which, int idx, double *x0dx, double *coef) {
  const Spline *s = nullptr;
  if (which == 0) s = &h->e.F[idx];
  else if (which == 1) s = &h->e.rho[idx];
  else s = &h->e.phi[idx];
  if (x0dx) {
    x0dx[0] = s->x0;
    x0dx[1] = s->dx;
    x0dx[2] = s->cut;
  }
  if (coef) {
    const int n = s->n;
    const std::vector<double> *arr[8] = {&s->y, &s->d2y, &s->c1, &s->c2,
                                         &s->c3, &s->d1, &s->d2, &s->d3};
    for (int q = 0; q < 8; q++) {
      for (int k = 0; k < n; k++) coef[(size_t)q * n + k] = k < (int)arr[q]->size() ? (*arr[q])[k] : 0.0;
    }
  }
  return s->n;
}

int orc_eam_kernel(const orc_eam *h, int nat, const double *r, const double *cell,
                   const int *pbc, const int *Z, const int64_t *seed, const int *nbr,
                   const int *dc, const int *mask, double *epot, double *f, double *wpot,
                   double *epot_per_at, double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> db;
  map_elements(nat, Z, h->e.nel, h->e.Z.data(), db);
  NList nl;
  nl_from_arrays(nat, seed, nbr, dc, nl);
  *epot = 0.0;
  return eam_kernel(h->e, nat, r, box, db.data(), nl, mask, epot, f, wpot, epot_per_at,
                    wpot_per_at, resolve_threads(nthreads));
}

int orc_eam_compute(const orc_eam *h, int nat, const double *r, const double *cell,
                    const int *pbc, const int *Z, const int *mask, double *epot, double *f,
                    double *wpot, double *epot_per_at, double *wpot_per_at, int nthreads) {
  Box box;
  if (make_box(cell, pbc, box) != 0) return -1;
  std::vector<int> db;
  map_elements(nat, Z, h->e.nel, h->e.Z.data(), db);
  NList nl;
  build_neighbors(nat, r, box, h->e.cutoff, nl);
  *epot = 0.0;
  return eam_kernel(h->e, nat, r, box, db.data(), nl, mask, epot, f, wpot, epot_per_at,
                    wpot_per_at, resolve_threads(nthreads));
}

int orc_max_threads(void) { return resolve_threads(0); }

}  // extern "C"
