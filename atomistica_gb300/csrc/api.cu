// C-ABI of the potentials (replaces the generated shims
// python_<mod>_{new,free,bind_to,energy_and_forces}, src/python/gen_factory.py:98-356,
// and COMPUTE_FUNC / BIND_TO_FUNC, src/potentials/bop/default_compute_func.f90:25-100,
// default_bind_to_func.f90:25-146, src/potentials/eam/tabulated_alloy_eam.f90:297-415).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "bop_math.h"
#include "elements.h"
#include "potential.h"

using namespace gb;

namespace gb {
namespace {

// Default parameter sets: Tersoff_PRB_39_5566_SiC (tersoff_params.f90:99-138)
// and Kumagai_CompMaterSci_39_457_Si (kumagai_params.f90:97-132).
gb_tersoff_params_t default_tersoff() {
  gb_tersoff_params_t p{};
  p.nel = 2;
  p.Z[0] = 6;
  p.Z[1] = 14;
  const double A[3] = {1.3936e3, std::sqrt(1.3936e3 * 1.8308e3), 1.8308e3};
  const double B[3] = {3.4674e2, std::sqrt(3.4674e2 * 4.7118e2), 4.7118e2};
  const double xi[3] = {1.0, 0.9776e0, 1.0};
  const double lam[3] = {3.4879e0, (3.4879e0 + 2.4799e0) / 2, 2.4799e0};
  const double mu[3] = {2.2119e0, (2.2119e0 + 1.7322e0) / 2, 1.7322e0};
  const double r1[3] = {1.80, std::sqrt(1.80 * 2.70), 2.70};
  const double r2[3] = {2.10, std::sqrt(2.10 * 3.00), 3.00};
  for (int q = 0; q < 3; q++) {
    p.A[q] = A[q];
    p.B[q] = B[q];
    p.xi[q] = xi[q];
    p.lambda[q] = lam[q];
    p.mu[q] = mu[q];
    p.omega[q] = 1.0;
    p.mubo[q] = 0.0;
    p.m[q] = 1;
    p.r1[q] = r1[q];
    p.r2[q] = r2[q];
  }
  const double beta[2] = {1.5724e-7, 1.1000e-6}, n[2] = {7.2751e-1, 7.8734e-1},
               c[2] = {3.8049e4, 1.0039e5}, d[2] = {4.3484e0, 1.6217e1},
               h[2] = {-5.7058e-1, -5.9825e-1};
  for (int q = 0; q < 2; q++) {
    p.beta[q] = beta[q];
    p.n[q] = n[q];
    p.c[q] = c[q];
    p.d[q] = d[q];
    p.h[q] = h[q];
  }
  return p;
}

gb_kumagai_params_t default_kumagai() {
  gb_kumagai_params_t p{};
  p.nel = 1;
  p.Z[0] = 14;
  p.A[0] = 3281.5905;
  p.B[0] = 121.00047;
  p.lambda1[0] = 3.2300135;
  p.lambda2[0] = 1.3457970;
  p.eta[0] = 1.0000000;
  p.delta[0] = 0.53298909;
  p.alpha[0] = 2.3890327;
  p.beta[0] = 1;
  p.c1[0] = 0.20173476;
  p.c2[0] = 730418.72;
  p.c3[0] = 1000000.0;
  p.c4[0] = 1.0000000;
  p.c5[0] = 26.000000;
  p.h[0] = -0.36500000;
  p.r1[0] = 2.70;
  p.r2[0] = 3.30;
  return p;
}

// Tersoff_PRB_39_5566_SiC__Scr (tersoff_params.f90:99-138 under SCREENING):
// m = 3, mubo = 1 / dimer length, inner cutoff r1 < r2 = 1.2 r1.
gb_tersoff_params_t default_tersoff_scr() {
  gb_tersoff_params_t p = default_tersoff();
  const double mubo[3] = {0.69103023078057590, 0.56580821386164815, 0.43569872294774004};
  const double r1[3] = {2.00, std::sqrt(2.00 * 2.50), 2.50};
  for (int q = 0; q < 3; q++) {
    p.mubo[q] = mubo[q];
    p.m[q] = 3;
    p.r1[q] = r1[q];
    p.r2[q] = r1[q] * 1.2;
  }
  return p;
}

gb_screening_params_t default_screening_tersoff() {
  gb_screening_params_t s{};
  const double o1[3] = {2.00, std::sqrt(2.00 * 3.00), 3.00};
  for (int q = 0; q < 3; q++) {
    s.or1[q] = s.bor1[q] = o1[q];
    s.or2[q] = s.bor2[q] = o1[q] * 2.0;
    s.Cmin[q] = 1.0;
    s.Cmax[q] = 3.0;
  }
  return s;
}

// Kumagai_CompMaterSci_39_457_Si__Scr (kumagai_params.f90:119-128).
gb_kumagai_params_t default_kumagai_scr() {
  gb_kumagai_params_t p = default_kumagai();
  p.r1[0] = 2.50;
  p.r2[0] = 2.50 * 1.2;
  return p;
}

gb_screening_params_t default_screening_kumagai() {
  gb_screening_params_t s{};
  s.or1[0] = s.bor1[0] = 3.00;
  s.or2[0] = s.bor2[0] = 3.00 * 2.0;
  s.Cmin[0] = 1.0;
  s.Cmax[0] = 3.0;
  return s;
}

// Erhart_PRB_71_035211_SiC (brenner_params.f90:67-117, non-screened values;
// el = C, Si).
gb_brenner_params_t default_brenner() {
  gb_brenner_params_t p{};
  p.nel = 2;
  p.Z[0] = 6;
  p.Z[1] = 14;
  const double D0[3] = {6.00, 4.36, 3.24}, r0[3] = {1.4276, 1.79, 2.232},
               S[3] = {2.167, 1.847, 1.842}, beta[3] = {2.0099, 1.6991, 1.4761},
               gamma[3] = {0.11233, 0.011877, 0.114354}, c[3] = {181.910, 273987.0, 2.00494},
               d[3] = {6.28433, 180.314, 0.81472}, h[3] = {0.5556, 0.68, 0.259},
               r1[3] = {1.85, 2.20, 2.68}, r2[3] = {2.15, 2.60, 2.96};
  for (int q = 0; q < 3; q++) {
    p.D0[q] = D0[q];
    p.r0[q] = r0[q];
    p.S[q] = S[q];
    p.beta[q] = beta[q];
    p.gamma[q] = gamma[q];
    p.c[q] = c[q];
    p.d[q] = d[q];
    p.h[q] = h[q];
    p.mu[q] = 0.0;
    p.n[q] = 1.0;
    p.m[q] = 1;
    p.r1[q] = r1[q];
    p.r2[q] = r2[q];
  }
  return p;
}

// The same set under SCREENING (brenner_params.f90:92-104): mu = 1/1.4276,
// 1/1.79, 1/1.842, m = 3, inner cutoff r1 < r2 = 1.2 r1; the outer and
// bond-order cutoffs and the C window are those of the screened Tersoff set.
gb_brenner_params_t default_brenner_scr() {
  gb_brenner_params_t p = default_brenner();
  const double mu[3] = {1.0 / 1.4276, 1.0 / 1.79, 1.0 / 1.842};
  const double r1[3] = {2.00, std::sqrt(2.00 * 2.50), 2.50};
  for (int q = 0; q < 3; q++) {
    p.mu[q] = mu[q];
    p.m[q] = 3;
    p.r1[q] = r1[q];
    p.r2[q] = r1[q] * 1.2;
  }
  return p;
}

// The checks of the reference's bind_to (brenner_module.f90:200-210) and
// the ones the kernels need.
int check_brenner(const gb_brenner_params_t &p) {
  if (p.nel < 1 || p.nel > 3) {
    set_error("Brenner: nel must be 1..3 (BRENNER_MAX_EL = 3)");
    return GB_ERROR_ARGUMENT;
  }
  const int np = p.nel * (p.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    if (!(p.r2[q] > p.r1[q]) || !(p.r1[q] >= 0)) {
      set_error("Brenner: need 0 <= r1 < r2 for every pair");
      return GB_ERROR_ARGUMENT;
    }
    if (p.d[q] == 0.0) {
      set_error("Brenner: d = 0! This leads to problems computing c**2/d**2. Please specify "
                "d != 0.");
      return GB_ERROR_ARGUMENT;
    }
    if (!(p.S[q] > 1.0)) {
      set_error("Brenner: S <= 1! This leads to problems computing (S-1)**(-1). Please "
                "specify S > 1.");
      return GB_ERROR_ARGUMENT;
    }
    if (!(p.n[q] != 0.0)) {
      set_error("Brenner: n must be nonzero");
      return GB_ERROR_ARGUMENT;
    }
    if (p.mu[q] != 0.0 && p.m[q] < 1) {
      set_error("Brenner: m must be >= 1 when mu != 0");
      return GB_ERROR_ARGUMENT;
    }
  }
  return 0;
}

// Juslin_J_Appl_Phys_98_123520_WCH (juslin_params.f90:75-108; el = W, C, H;
// ordered pairs, r0 = -1 marks the pairs (C,W) and (H,W) that take their
// mirror's constants).  screened: the SCREENING values of r1, r2.
gb_juslin_params_t default_juslin(bool screened) {
  gb_juslin_params_t p{};
  p.nel = 3;
  p.Z[0] = 74;
  p.Z[1] = 6;
  p.Z[2] = 1;
  const double D0[9] = {5.41861, 6.64, 2.748, 0.0, 6.0, 3.6422, 0.0, 3.642, 4.7509};
  const double r0[9] = {2.34095, 1.90547, 1.727, -1.0, 1.39, 1.1199, -1.0, 1.1199, 0.74144};
  const double S[9] = {1.92708, 2.96149, 1.2489, 0.0, 1.22, 1.69077, 0.0, 1.69077, 2.3432};
  const double beta[9] = {1.38528, 1.80370, 1.52328, 0.0, 2.1, 1.9583, 0.0, 1.9583, 1.9436};
  const double gamma[9] = {0.00188227, 0.072855, 0.0054, 0.0, 0.00020813,
                           0.00020813, 0.0,      12.33,  12.33};
  const double c[9] = {2.14969, 1.10304, 1.788, 0.0, 330.0, 330.0, 0.0, 0.0, 0.0};
  const double d[9] = {0.17126, 0.33018, 0.8255, 0.0, 3.5, 3.5, 0.0, 1.0, 1.0};
  const double h[9] = {-0.27780, 0.75107, 0.38912, 0.0, 1.0, 1.0, 0.0, 1.0, 1.0};
  const double r1[9] = {3.20, 2.60, screened ? 2.68 : 1.95, 0.0, 1.70, 1.30, 0.0, 1.30, 1.10};
  const double r2[9] = {3.80, 3.00, screened ? 2.96 : 2.35, 0.0, 2.00, 1.80, 0.0, 1.80, 1.70};
  for (int q = 0; q < 9; q++) {
    p.D0[q] = D0[q];
    p.r0[q] = r0[q];
    p.S[q] = S[q];
    p.beta[q] = beta[q];
    p.gamma[q] = gamma[q];
    p.c[q] = c[q];
    p.d[q] = d[q];
    p.h[q] = h[q];
    p.n[q] = 1.0;
    p.r1[q] = r1[q];
    p.r2[q] = r2[q];
  }
  // alpha = 0.45876 for (W,W,W), (W,C,W), (W,H,W); alpha = 4 for (C,C,H),
  // (C,H,C), (C,H,H), (H,C,C), (H,C,H), (H,H,C), (H,H,H); omega of (C,H,C),
  // (C,H,H), (H,C,C), (H,C,H) as tabulated; every other triplet alpha = 0,
  // omega = 1; m = 1 throughout.
  const int a1[3] = {0, 3, 6}, a4[7] = {14, 16, 17, 22, 23, 25, 26};
  for (int q = 0; q < 27; q++) {
    p.alpha[q] = 0.0;
    p.omega[q] = 1.0;
    p.m[q] = 1;
  }
  for (int q : a1) p.alpha[q] = 0.45876;
  for (int q : a4) p.alpha[q] = 4.0;
  p.omega[16] = 2.94586;
  p.omega[17] = 4.54415;
  p.omega[22] = 0.33946;
  p.omega[23] = 0.22006;
  return p;
}

gb_screening_params_t default_screening_juslin() {
  gb_screening_params_t s{};
  const gb_juslin_params_t p = default_juslin(true);
  for (int q = 0; q < 9; q++) {
    s.or1[q] = s.bor1[q] = p.r1[q];
    s.or2[q] = s.bor2[q] = p.r2[q];
    s.Cmin[q] = q == 3 || q == 6 ? 0.0 : 1.0;
    s.Cmax[q] = q == 3 || q == 6 ? 0.0 : 3.0;
  }
  return s;
}

// The mirror fill of the reference's bind_to (juslin_module.f90:273-300): an
// ordered pair (i, j) with r0 < 0 takes every constant of (j, i), screening
// cutoffs included.  (The reference indexes this loop with the maximal
// element count 3; for nel = 3, the only published sets, that is the
// kernel's index.)
void fill_juslin(gb_juslin_params_t &p, gb_screening_params_t *sc) {
  const int nel = p.nel;
  for (int i = 0; i < nel; i++)
    for (int j = 0; j < nel; j++) {
      const int a = j + i * nel, b = i + j * nel;
      if (!(p.r0[a] < 0.0)) continue;
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
      if (sc) {
        sc->or1[a] = sc->or1[b];
        sc->or2[a] = sc->or2[b];
        sc->bor1[a] = sc->bor1[b];
        sc->bor2[a] = sc->bor2[b];
        sc->Cmin[a] = sc->Cmin[b];
        sc->Cmax[a] = sc->Cmax[b];
      }
    }
}

// The checks of the reference's bind_to (juslin_module.f90:331-343) and the
// ones the kernels need.
int check_juslin(const gb_juslin_params_t &p) {
  if (p.nel < 1 || p.nel > 3) {
    set_error("Juslin: nel must be 1..3 (JUSLIN_MAX_EL = 3)");
    return GB_ERROR_ARGUMENT;
  }
  const int np = p.nel * p.nel;
  for (int q = 0; q < np; q++) {
    if (!(p.r2[q] > p.r1[q]) || !(p.r1[q] >= 0)) {
      set_error("Juslin: need 0 <= r1 < r2 for every pair");
      return GB_ERROR_ARGUMENT;
    }
    if (p.d[q] == 0.0) {
      set_error("Juslin: d = 0! This leads to problems computing c**2/d**2. Please specify "
                "d != 0.");
      return GB_ERROR_ARGUMENT;
    }
    if (!(p.S[q] > 1.0)) {
      set_error("Juslin: S <= 1! This leads to problems computing (S-1)**(-1). Please "
                "specify S > 1.");
      return GB_ERROR_ARGUMENT;
    }
    if (!(p.n[q] != 0.0)) {
      set_error("Juslin: n must be nonzero");
      return GB_ERROR_ARGUMENT;
    }
  }
  for (int q = 0; q < np * p.nel; q++)
    if (p.alpha[q] != 0.0 && p.m[q] < 1) {
      set_error("Juslin: m must be >= 1 where alpha != 0");
      return GB_ERROR_ARGUMENT;
    }
  return 0;
}

int check_screening(const gb_screening_params_t &s, int npairs) {
  for (int q = 0; q < npairs; q++) {
    if (!(s.or2[q] > s.or1[q]) || !(s.bor2[q] > s.bor1[q]) || !(s.Cmax[q] > s.Cmin[q])) {
      set_error("screening: need or1 < or2, bor1 < bor2 and Cmin < Cmax for every pair");
      return GB_ERROR_ARGUMENT;
    }
  }
  return 0;
}

int check_tersoff(const gb_tersoff_params_t &p) {
  if (p.nel < 1 || p.nel > 3) {
    set_error("Tersoff: nel must be 1..3");
    return GB_ERROR_ARGUMENT;
  }
  const int np = p.nel * (p.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    if (!(p.r2[q] > p.r1[q]) || !(p.r1[q] >= 0)) {
      set_error("Tersoff: need 0 <= r1 < r2 for every pair");
      return GB_ERROR_ARGUMENT;
    }
    if (p.mubo[q] != 0.0 && p.m[q] < 1) {
      set_error("Tersoff: m must be >= 1 when mubo != 0");
      return GB_ERROR_ARGUMENT;
    }
  }
  for (int q = 0; q < p.nel; q++)
    if (!(p.n[q] != 0.0) || !(p.d[q] != 0.0)) {
      set_error("Tersoff: n and d must be nonzero");
      return GB_ERROR_ARGUMENT;
    }
  return 0;
}

int check_kumagai(const gb_kumagai_params_t &p) {
  if (p.nel != 1) {
    set_error("Kumagai: exactly one element is supported (KUMAGAI_MAX_EL = 1)");
    return GB_ERROR_ARGUMENT;
  }
  if (!(p.r2[0] > p.r1[0]) || !(p.r1[0] >= 0)) {
    set_error("Kumagai: need 0 <= r1 < r2");
    return GB_ERROR_ARGUMENT;
  }
  if (p.alpha[0] != 0.0 && p.beta[0] < 1) {
    set_error("Kumagai: beta must be >= 1");
    return GB_ERROR_ARGUMENT;
  }
  return 0;
}

}  // namespace

const double *bop_r1(const Potential &pot) {
  if (pot.kind == kJuslin) return pot.jp.r1;
  return pot.kind == kTersoff ? pot.tp.r1 : pot.kind == kBrenner ? pot.bp.r1 : pot.kp.r1;
}
const double *bop_r2(const Potential &pot) {
  if (pot.kind == kJuslin) return pot.jp.r2;
  return pot.kind == kTersoff ? pot.tp.r2 : pot.kind == kBrenner ? pot.bp.r2 : pot.kp.r2;
}

double bop_pair_range(const Potential &pot, int t) {
  const double *r2 = bop_r2(pot);
  if (!pot.screened) return r2[t];
  const int np = pot_npairs(pot);
  double mx = 0.0;
  for (int q = 0; q < np; q++) {
    if (pot.kind == kBrenner && q != t) continue;  // BrennerScr: the pair's own cutoffs
    const double m = std::max(std::max(r2[q], pot.scr.or2[q]), pot.scr.bor2[q]);
    mx = std::max(mx, m * m);
  }
  const double cmax = pot.scr.Cmax[t];
  // JuslinScr: no Cmax > 2 guard (juslin_module.f90:305-307)
  const double cdr =
      (cmax > 2.0 || pot.kind == kJuslin) ? cmax * cmax / (4 * (cmax - 1)) : 1.0;
  return std::sqrt(cdr) * std::sqrt(mx);
}

int pot_nel(const Potential &pot) {
  if (pot.kind == kTersoff) return pot.tp.nel;
  if (pot.kind == kKumagai) return 1;
  if (pot.kind == kBrenner) return pot.bp.nel;
  if (pot.kind == kJuslin) return pot.jp.nel;
  return pot.eam->nel;
}
int pot_Z(const Potential &pot, int q) {
  if (pot.kind == kTersoff) return pot.tp.Z[q];
  if (pot.kind == kKumagai) return pot.kp.Z[q];
  if (pot.kind == kBrenner) return pot.bp.Z[q];
  if (pot.kind == kJuslin) return pot.jp.Z[q];
  return pot.eam->Z[q];
}
int pot_npairs(const Potential &pot) {
  const int nel = pot_nel(pot);
  return pot.kind == kJuslin ? nel * nel : nel * (nel + 1) / 2;
}
int pot_pair(const Potential &pot, int a, int b) {
  return pot.kind == kJuslin ? b + a * pot_nel(pot) : pair_index(a, b, pot_nel(pot));
}

cudaStream_t pot_stream(Potential &pot) {
  if (!pot.stream) {
    cudaStreamCreateWithFlags(&pot.stream, cudaStreamNonBlocking);
    pot.own_stream = true;
  }
  if (!pot.ev[0]) {
    for (int q = 0; q < 4; q++) cudaEventCreate(&pot.ev[q]);
    for (int q = 0; q < 2; q++) cudaEventCreate(&pot.kev[q]);
  }
  return pot.stream;
}

namespace {


// Z -> internal element index (Z2db, default_compute_func.f90:62-66).
int update_element_map(Potential &pot, const Particles &p) {
  if (pot.el_for == &p && pot.el_zrev == p.z_rev && pot.el.p) return 0;
  const int nel = pot_nel(pot);
  std::vector<int> el(std::max(p.nat, 1), -1);
  const bool all = pot.kind == kEAM && pot.eam->funcfl;  // one table for every element
  const std::vector<int> &flt = pot.el_filter;
  for (int i = 0; i < p.nat; i++) {
    // the element filter (IS_EL2(els, eli), tabulated_alloy_eam.f90:316-335):
    // atoms of other elements are skipped as i and as j, like atoms of
    // elements without parameters
    if (!flt.empty() && std::find(flt.begin(), flt.end(), p.hZ[i]) == flt.end()) continue;
    for (int q = 0; q < nel; q++)
      if (all || p.hZ[i] == pot_Z(pot, q)) el[i] = q;
  }
  GB_CHECK(pot.el.ensure(sizeof(int) * el.size()));
  GB_CUDA(cudaMemcpyAsync(pot.el.p, el.data(), sizeof(int) * el.size(), cudaMemcpyHostToDevice,
                          pot_stream(pot)));
  GB_CUDA(cudaStreamSynchronize(pot.stream));
  pot.el_for = &p;
  pot.el_zrev = p.z_rev;
  return 0;
}

struct Stage {
  double *caller = nullptr;
  double *dev = nullptr;
  size_t n = 0;
  bool host = false;
};

int stage_in(double *caller, size_t n, DevBuf &tmp, cudaStream_t s, Stage &st) {
  st.caller = caller;
  st.n = n;
  st.dev = nullptr;
  st.host = false;
  if (!caller) return 0;
  if (is_device_ptr(caller)) {
    st.dev = caller;
    return 0;
  }
  GB_CHECK(tmp.ensure(sizeof(double) * std::max<size_t>(n, 1)));
  st.dev = tmp.as<double>();
  st.host = true;
  if (n) GB_CUDA(cudaMemcpyAsync(st.dev, caller, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  return 0;
}

int stage_out(const Stage &st, cudaStream_t s) {
  if (st.host && st.n)
    GB_CUDA(cudaMemcpyAsync(st.caller, st.dev, sizeof(double) * st.n, cudaMemcpyDeviceToHost, s));
  return 0;
}

__global__ void add_arrays(double *__restrict__ dst, const double *__restrict__ src, size_t n) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x)
    dst[k] += src[k];
}

int add_into(double *dst, const double *src, size_t n, cudaStream_t s) {
  if (!n) return 0;
  const int T = 256;
  const size_t blocks = std::min<size_t>((n + T - 1) / T, 65535);
  add_arrays<<<(unsigned)blocks, T, 0, s>>>(dst, src, n);
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// CUDA graph of a whole single-structure evaluation (gb_potential_set_graph).
// After an eager evaluation has sized every buffer, the next evaluation of
// the same particles, list, cell and force buffer captures the list build
// (single staged pass, no host decision), the tile kernel with a plan that
// has head room, the gather, the sums and the copies of the status words and
// results to pinned memory; later evaluations replay it.  A replay whose
// list or tile plan overflowed leaves the forces as they were (the gather
// checks the status words on the device) and is redone eagerly.
// ---------------------------------------------------------------------------
void drop_single_graph(Potential &pot) {
  if (pot.graph_exec) cudaGraphExecDestroy(pot.graph_exec);
  if (pot.graph) cudaGraphDestroy(pot.graph);
  pot.graph_exec = nullptr;
  pot.graph = nullptr;
  pot.graph_kernels = 0;
  pot.graph_bufs.clear();
}

// Device (and pinned) buffers whose addresses a captured evaluation holds.
std::vector<const void *> single_graph_buffers(const Potential &pot, const Particles &p,
                                               const Neighbors &nl) {
  return {p.r.p,          pot.el.p,       nl.pos4.p,      nl.posff.p,    nl.atom_cell.p,
          nl.atom_wrap.p, nl.cell_count.p, nl.cell_start.p, nl.cell_atoms.p, nl.counts.p,
          nl.spos.p,      nl.swrap.p,     nl.seed.p,      nl.nbr.p,      nl.shift.p,
          nl.rev.p,       nl.stage.p,     nl.scan_tmp.p,  nl.stats.p,    nl.hstats.p,
          pot.bond_G.p,   pot.bond_e.p,   pot.tile_part.p, pot.red.p,    pot.hred.p,
          pot.red_stage.p, pot.out_f.p, pot.eam_cache.p};
}

bool single_graph_current(const Potential &pot, const Particles &p, const Neighbors &nl,
                          const double *fd, bool set_f, cudaStream_t s) {
  return pot.graph_exec && pot.graph_p == &p && pot.graph_nl == &nl && pot.graph_nat == p.nat &&
         pot.graph_cell_rev == p.cell_rev && pot.graph_fd == fd && pot.graph_set_f == set_f &&
         pot.graph_prec == pot.precision && pot.graph_stream == s &&
         pot.graph_tile_request == pot.tile_request &&
         pot.graph_cutoff == nl.interaction_range && pot.el_for == &p &&
         pot.graph_bufs == single_graph_buffers(pot, p, nl);
}

// Captures the evaluation into pot.graph (nothing runs).  fd: the force
// array (device, or mapped page-locked host memory) the graph accumulates
// into, or writes for every atom when set_f.
void single_capture(Potential &pot, Particles &p, Neighbors &nl, double *fd, bool set_f,
                    cudaStream_t s) {
  drop_single_graph(pot);
  const int nat = p.nat;
  const int cap = nl.stage_cap;
  const bool bop = pot.kind != kEAM;
  const int nbt0 = pot.last_plan[0], ntrip0 = pot.last_plan[1];
  if (cap <= 0 || nat <= 0 || !nl.valid || nl.built_for != &p || (bop && nbt0 <= 0)) return;
  const int64_t capacity = (int64_t)nat * cap;
  if (capacity > (int64_t)INT_MAX / 3) return;
  const bool mixed = pot.precision == GB_PRECISION_MIXED;
  int max_nbt = nbt0, max_ntrip = ntrip0;
  if (bop) {
    const int apt = pot.tile_atoms;
    const int ntiles = (nat + apt - 1) / apt;
    // Tile plan with head room for the next configurations (checked per tile
    // by the kernel): as much as fits without fewer resident CTAs per SM than
    // the exact plan of this evaluation, at most +25 % bonds / +50 % slots.
    const int occ0 = bop_tile_ctas_per_sm(pot, bop_tile_smem(mixed, nbt0, ntrip0));
    for (int step = 16; step >= 1; step--) {
      const int nb = std::min(apt * cap, nbt0 + nbt0 * step / 64 + step);
      const int nt = std::min(apt * trip_slots(cap), ntrip0 + ntrip0 * step / 32 + 4 * step);
      const size_t sm = bop_tile_smem(mixed, nb, nt);
      if (sm <= bop_tile_smem_budget() && bop_tile_ctas_per_sm(pot, sm) >= occ0) {
        max_nbt = nb;
        max_ntrip = nt;
        break;
      }
    }
    if (pot.bond_G.ensure(sizeof(double) * 3 * capacity) ||
        pot.bond_e.ensure(sizeof(double) * capacity) ||
        pot.tile_part.ensure(sizeof(double) * 10 * (size_t)ntiles + 64) ||
        pot.red_stage.ensure(reduce_stage_bytes(ntiles) + 64)) {
      clear_error();
      return;
    }
  } else if (eam_cache_ensure(pot, capacity)) {
    clear_error();
    return;
  }
  // every buffer at its captured size now: nothing may be allocated inside
  // (the EAM kernels' per-atom and per-block buffers depend on nat only and
  // were sized by the eager call).  A list array that grows here loses the
  // eager call's list: the list is then marked for a rebuild.
  const void *list0[3] = {nl.nbr.p, nl.shift.p, nl.rev.p};
  const int grow = nl.nbr.ensure(sizeof(int) * capacity) ||
                   nl.shift.ensure(sizeof(int) * capacity) ||
                   nl.rev.ensure(sizeof(int) * capacity) ||
                   nl.stage.ensure(sizeof(int2) * capacity) ||
                   pot.red.ensure(sizeof(double) * 16) || pot.hred.ensure(sizeof(double) * 16);
  if (nl.nbr.p != list0[0] || nl.shift.p != list0[1] || nl.rev.p != list0[2]) {
    nl.valid = false;
    nl.rev_valid = false;
  }
  if (grow) {
    clear_error();
    return;
  }
  BinParams bp;
  if (bin_params(p.A, p.B, p.pbc, nl.interaction_range, 0, bp)) {
    clear_error();
    return;
  }
  const int ncells = bp.n[0] * bp.n[1] * bp.n[2];
  Outputs o;
  o.f = fd;
  o.f_set = set_f;  // (every atom's force written: no zeroing first)
  o.red = pot.red.as<double>();
  o.status = reinterpret_cast<int *>(o.red + 12);
  BopSystem sys;
  sys.nat = nat;
  std::memcpy(sys.A, p.A, sizeof(sys.A));
  sys.capture = true;
  sys.nb_capacity = capacity;
  sys.max_nbt = max_nbt;
  sys.max_ntrip = max_ntrip;
  sys.check.nl = nl.stats.as<int>();
  sys.check.tile = o.status;
  sys.check.cap = cap;
  // capturing runs nothing: the eager evaluation's list state stays valid
  const bool rev_valid0 = nl.rev_valid, posff_valid0 = nl.posff_valid;
  const bool plan_ready0 = nl.plan_ready, valid0 = nl.valid;
  const int plan0[2] = {pot.last_plan[0], pot.last_plan[1]};
  const int tile_atoms0 = pot.tile_atoms;
  nl.rev_valid = false;
  nl.rev_pending = false;
  const uint64_t launches0 = gb_kernel_launches();
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    pot.graph_failed = true;
    return;
  }
  int rc = 0;
  if (cudaMemsetAsync(o.status, 0, sizeof(int) * 4, s) != cudaSuccess) rc = -1;
  if (rc == 0) rc = nl_build(nl, nat, p.r.as<double>(), bp, nullptr, nullptr, ncells, s, true);
  if (rc == 0)
    rc = bop ? bop_run(pot, sys, nl, o, false, false)
             : eam_compute(pot, p, nl, o, false, sys.check, true);
  if (rc == 0 && cudaMemcpyAsync(pot.hred.p, o.red, sizeof(double) * 14, cudaMemcpyDeviceToHost,
                                 s) != cudaSuccess)
    rc = -1;
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  note_launch(-(int)(gb_kernel_launches() - launches0));  // captured, not run
  nl.rev_valid = rev_valid0;
  nl.rev_pending = false;
  nl.posff_valid = posff_valid0;
  nl.plan_ready = plan_ready0;
  nl.valid = valid0;
  pot.last_plan[0] = plan0[0];
  pot.last_plan[1] = plan0[1];
  pot.tile_atoms = tile_atoms0;
  cudaGraphExec_t x = nullptr;
  if (rc != 0 || ce != cudaSuccess || !g || cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    clear_error();
    pot.graph_failed = true;
    return;
  }
  size_t nn = 0;
  cudaGraphGetNodes(g, nullptr, &nn);
  std::vector<cudaGraphNode_t> nodes(nn);
  if (nn) cudaGraphGetNodes(g, nodes.data(), &nn);
  int kernels = 0;
  for (size_t k = 0; k < nn; k++) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
      kernels++;
  }
  pot.graph = g;
  pot.graph_exec = x;
  pot.graph_kernels = kernels;
  pot.graph_cap = cap;
  pot.graph_p = &p;
  pot.graph_nl = &nl;
  pot.graph_nat = nat;
  pot.graph_cell_rev = p.cell_rev;
  pot.graph_cutoff = nl.interaction_range;
  pot.graph_fd = fd;
  pot.graph_set_f = set_f;
  pot.graph_prec = pot.precision;
  pot.graph_stream = s;
  pot.graph_tile_request = pot.tile_request;
  pot.graph_bufs = single_graph_buffers(pot, p, nl);
}

// Energy (set) and virial (accumulated) from the pinned result row hr, after
// the checks of the force kernels' status word.
int finish_results(Potential &pot, const double *hr, double *epot, double *wpot) {
  const int st = reinterpret_cast<const int *>(hr + 12)[0];
  pot.last_status = st;
  pot.last_hot = reinterpret_cast<const int *>(hr + 12)[2];
  if (st & 1) {
    set_error("Spline argument outside of the defined interval (EAM density table).");
    return GB_ERROR_DOMAIN;
  }
  if (st & 2) {
    set_error("Internal error: bond-order tile plan mismatch.");
    return GB_ERROR_UNSPECIFIED;
  }
  if (st & 4) {
    set_error("Internal neighbor list exhausted: an atom has more bonds after screening than "
              "the screened kernel supports (32).");
    return GB_ERROR_CAPACITY;
  }
  // epot is set; wpot accumulated (gen_factory.py:283, potential.c:468-479).
  if (is_device_ptr(epot)) {
    GB_CUDA(cudaMemcpy(epot, hr, sizeof(double), cudaMemcpyHostToDevice));
  } else {
    *epot = hr[0];
  }
  if (is_device_ptr(wpot)) {
    double w[9];
    GB_CUDA(cudaMemcpy(w, wpot, sizeof(w), cudaMemcpyDeviceToHost));
    for (int q = 0; q < 9; q++) w[q] += hr[1 + q];
    GB_CUDA(cudaMemcpy(wpot, w, sizeof(w), cudaMemcpyHostToDevice));
  } else {
    for (int q = 0; q < 9; q++) wpot[q] += hr[1 + q];
  }
  return 0;
}

// Replays the captured evaluation; done = false when its list or tile plan
// overflowed (the forces are then as before the call; with set_f they are
// written by the eager call that follows).
int single_replay(Potential &pot, Particles &p, Neighbors &nl, double *f, double *fd,
                  bool staged, bool set_f, double *epot, double *wpot, cudaStream_t s,
                  bool &done) {
  done = false;
  const size_t nf = 3 * (size_t)p.nat;
  GB_CUDA(cudaEventRecord(pot.ev[0], s));
  if (staged && !set_f)
    GB_CUDA(cudaMemcpyAsync(fd, f, sizeof(double) * nf, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaGraphLaunch(pot.graph_exec, s));
  if (staged) GB_CUDA(cudaMemcpyAsync(f, fd, sizeof(double) * nf, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaEventRecord(pot.ev[3], s));
  GB_CUDA(cudaStreamSynchronize(s));
  note_launch(pot.graph_kernels);
  const int *hs = nl.hstats.as<int>();
  const double *hr = pot.hred.as<double>();
  const int *st = reinterpret_cast<const int *>(hr + 12);
  if (!(hs[0] <= pot.graph_cap && (hs[1] & (1 | 2 | 8)) == 0 && (hs[5] & 4) == 0 &&
        (st[0] & 2) == 0)) {
    drop_single_graph(pot);
    nl.valid = false;
    return 0;
  }
  nl.nentries = hs[4];
  nl.maxz = hs[0];
  nl.valid = true;
  nl.built_for = &p;
  nl.built_pos_rev = p.pos_rev;
  nl.built_cell_rev = p.cell_rev;
  nl.built_nat = p.nat;
  nl.cutoff = nl.interaction_range;
  nl.rev_valid = pot.kind != kEAM;  // (the bond-order evaluation builds the reverse index)
  nl.rev_pending = false;
  nl.posff_valid = nl.want_posff;
  nl.plan_ready = false;
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, pot.ev[0], pot.ev[3]);
  cudaGetLastError();
  pot.timing[0] = pot.timing[1] = pot.timing[3] = 0.0;
  pot.timing[2] = ms;
  pot.last_bonds = nl.nentries;
  GB_CHECK(finish_results(pot, hr, epot, wpot));
  done = true;
  return 0;
}

int energy_and_forces(Potential &pot, Particles &p, Neighbors &nl, double *epot, double *f,
                      double *wpot, const int *mask, double *epa, double *epb, double *fpb,
                      double *wpa, double *wpb, int flags = 0) {
  const bool set_f = (flags & GB_FORCES_SET) != 0;  // f is written, not accumulated into
  if (!epot || !f || !wpot) {
    set_error("energy_and_forces: epot, f and wpot are required");
    return GB_ERROR_ARGUMENT;
  }
  // Optional arguments outside the class's features are refused as by the
  // generated shims (gen_factory.py:302-351): TabulatedAlloyEAM has
  // mask,per_at (tabulated_alloy_eam.f90:24), TabulatedEAM per_at
  // (tabulated_eam.f90:24).
  if (pot.kind == kEAM) {
    const char *cls = pot.eam->funcfl ? "TabulatedEAM" : "TabulatedAlloyEAM";
    const char *bad = epb ? "epot_per_bond" : fpb ? "f_per_bond" : wpb ? "wpot_per_bond"
                      : (pot.eam->funcfl && mask) ? "mask" : nullptr;
    if (bad) {
      set_error(std::string("*") + bad + "* argument present but not supported by potential " +
                cls + ".");
      return GB_ERROR_ARGUMENT;
    }
  }
  if (pot.kind == kEAM && pot.precision != GB_PRECISION_FP64) {
    set_error("TabulatedAlloyEAM has only the FP64 form.");
    return GB_ERROR_ARGUMENT;
  }
  cudaStream_t s = pot_stream(pot);
  if (p.stream && p.stream != s) {
    GB_CUDA(cudaEventRecord(pot.ev[3], p.stream));
    GB_CUDA(cudaStreamWaitEvent(s, pot.ev[3], 0));
  }
  GB_CUDA(cudaEventRecord(pot.ev[0], s));
  GB_CHECK(update_element_map(pot, p));
  const int nat = p.nat;
  // CUDA-graph replay of a whole evaluation (outputs: energy, forces, virial)
  pot.last_replayed = false;
  const bool graph_ok = pot.use_graph && !pot.graph_failed && !pot.screened && nat > 0 &&
                        !mask && !epa && !wpa && !epb && !fpb && !wpb;
  double *gfd = nullptr;
  if (graph_ok) {
    // the forces go to the caller's device array, to page-locked host memory
    // directly when they are written (not accumulated), or through the
    // staging buffer out_f (copied in and out around the replay)
    const bool fh = !is_device_ptr(f);
    gfd = !fh ? f : (set_f && pot.kind != kEAM ? mapped_host_ptr(f) : nullptr);
    if (!gfd) {
      GB_CHECK(pot.out_f.ensure(sizeof(double) * 3 * std::max<size_t>(nat, 1)));
      gfd = pot.out_f.as<double>();
    }
    const bool staged = gfd == pot.out_f.as<double>();
    if (single_graph_current(pot, p, nl, gfd, set_f, s)) {
      bool done = false;
      GB_CHECK(single_replay(pot, p, nl, f, gfd, staged, set_f, epot, wpot, s, done));
      if (done) {
        pot.last_replayed = true;
        pot.graph_unused = 0;
        return 0;
      }
    }
  }
  // Host forces (accumulated into): their upload runs on a second stream
  // while the neighbour list is built.
  Stage sf, sepa, swpa, sepb, sfpb, swpb;
  const bool f_host = nat > 0 && !is_device_ptr(f);
  if (f_host && !set_f) {
    if (!pot.aux) {
      GB_CUDA(cudaStreamCreateWithFlags(&pot.aux, cudaStreamNonBlocking));
      GB_CUDA(cudaEventCreateWithFlags(&pot.aux_ev, cudaEventDisableTiming));
    }
    GB_CUDA(cudaEventRecord(pot.aux_ev, s));  // the buffer's previous use is done
    GB_CUDA(cudaStreamWaitEvent(pot.aux, pot.aux_ev, 0));
    GB_CHECK(stage_in(f, 3 * (size_t)nat, pot.out_f, pot.aux, sf));
    GB_CUDA(cudaEventRecord(pot.aux_ev, pot.aux));
  }
  nl.stream = s;
  if (pot.precision == GB_PRECISION_MIXED) nl.want_posff = true;
  // Forces that are written (not accumulated) go straight to their array:
  // a device array, or page-locked host memory, which the gather writes over
  // the host link while it computes (no staging copy).
  // (the EAM pair kernel writes an atom's three values from one lane, which
  // suits device memory only)
  double *f_direct = nullptr;
  if (set_f && nat > 0) f_direct = !f_host ? f : pot.kind != kEAM ? mapped_host_ptr(f) : nullptr;
  if (pot.kind != kEAM && !pot.screened) {
    // the bond-order kernels need the reverse index, and the list build can
    // plan their tiles (the size of the previous evaluation's tiles)
    nl.want_rev = true;
    nl.plan_apt = pot.tile_atoms;
  } else {
    nl.plan_apt = 0;
  }
  GB_CHECK(neighbors_update(nl, p, s));
  GB_CUDA(cudaEventRecord(pot.ev[1], s));

  const size_t nb = (size_t)nl.nentries;
  if (f_direct) {
    // written by the force kernels in store mode (every atom)
    sf.caller = sf.dev = f_direct;
    sf.n = 3 * (size_t)nat;
    sf.host = false;
  } else if (set_f) {
    // nothing to upload: the forces start from zero on the device
    if (f_host) {
      GB_CHECK(pot.out_f.ensure(sizeof(double) * 3 * std::max<size_t>(nat, 1)));
      sf.caller = f;
      sf.dev = pot.out_f.as<double>();
      sf.n = 3 * (size_t)nat;
      sf.host = true;
    } else {
      sf.caller = sf.dev = f;
      sf.n = 3 * (size_t)nat;
      sf.host = false;
    }
    if (nat) GB_CUDA(cudaMemsetAsync(sf.dev, 0, sizeof(double) * 3 * nat, s));
  } else if (f_host) {
    GB_CUDA(cudaStreamWaitEvent(s, pot.aux_ev, 0));
  } else {
    GB_CHECK(stage_in(f, 3 * (size_t)nat, pot.out_f, s, sf));
  }
  GB_CHECK(stage_in(epa, nat, pot.out_epa, s, sepa));
  GB_CHECK(stage_in(wpa, 9 * (size_t)nat, pot.out_wpa, s, swpa));
  GB_CHECK(stage_in(epb, nb, pot.out_epb, s, sepb));
  GB_CHECK(stage_in(fpb, 3 * nb, pot.out_fpb, s, sfpb));
  GB_CHECK(stage_in(wpb, 9 * nb, pot.out_wpb, s, swpb));
  Outputs o;
  o.f = sf.dev;
  o.f_set = f_direct != nullptr;
  o.epot_per_at = sepa.dev;
  o.wpot_per_at = swpa.dev;
  o.epot_per_bond = sepb.dev;
  o.f_per_bond = sfpb.dev;
  o.wpot_per_bond = swpb.dev;
  if (mask) {
    if (is_device_ptr(mask)) {
      o.mask = mask;
    } else {
      GB_CHECK(pot.mask_d.ensure(sizeof(int) * std::max(nat, 1)));
      if (nat)
        GB_CUDA(cudaMemcpyAsync(pot.mask_d.p, mask, sizeof(int) * nat, cudaMemcpyHostToDevice, s));
      o.mask = pot.mask_d.as<int>();
    }
  }
  GB_CHECK(pot.red.ensure(sizeof(double) * 16));
  o.red = pot.red.as<double>();
  o.status = reinterpret_cast<int *>(o.red + 12);
  GB_CUDA(cudaMemsetAsync(o.status, 0, sizeof(int) * 4, s));

  const bool want_wat = wpa != nullptr || wpb != nullptr;
  const bool want_pb = epb || fpb || wpb;
  if (pot.kind == kEAM) {
    GB_CHECK(eam_compute(pot, p, nl, o, want_wat));
  } else {
    GB_CHECK(bop_compute(pot, p, nl, o, want_wat, want_pb));
    if (epb) GB_CHECK(add_into(sepb.dev, pot.bond_e.as<double>(), nb, s));
    if (fpb) GB_CHECK(add_into(sfpb.dev, pot.bond_fr.as<double>(), 3 * nb, s));
    if (wpb) GB_CHECK(add_into(swpb.dev, pot.bond_w.as<double>(), 9 * nb, s));
  }
  GB_CUDA(cudaEventRecord(pot.ev[2], s));
  GB_CHECK(stage_out(sf, s));
  GB_CHECK(stage_out(sepa, s));
  GB_CHECK(stage_out(swpa, s));
  GB_CHECK(stage_out(sepb, s));
  GB_CHECK(stage_out(sfpb, s));
  GB_CHECK(stage_out(swpb, s));
  GB_CHECK(pot.hred.ensure(sizeof(double) * 16));
  double *hr = pot.hred.as<double>();
  GB_CUDA(cudaMemcpyAsync(hr, o.red, sizeof(double) * 14, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaEventRecord(pot.ev[3], s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaGetLastError());
  GB_CHECK(neighbors_check_reverse(nl, nullptr));  // (when the tile plan came with the list)
  float ms[4] = {0, 0, 0, 0};
  cudaEventElapsedTime(&ms[0], pot.ev[0], pot.ev[1]);
  cudaEventElapsedTime(&ms[1], pot.ev[1], pot.ev[2]);
  cudaEventElapsedTime(&ms[2], pot.ev[0], pot.ev[3]);
  if (nat > 0) cudaEventElapsedTime(&ms[3], pot.kev[0], pot.kev[1]);
  cudaGetLastError();
  for (int q = 0; q < 4; q++) pot.timing[q] = ms[q];
  pot.last_bonds = pot.kind == kEAM ? 0 : nl.nentries;
  GB_CHECK(finish_results(pot, hr, epot, wpot));
  if (graph_ok && !single_graph_current(pot, p, nl, gfd, set_f, s)) {
    // a caller whose calls never match the previous capture (e.g. a new
    // force array every call) would pay a capture per call: after three
    // captures in a row that were never replayed, stay eager
    if (pot.graph_exec && ++pot.graph_unused >= 3) {
      drop_single_graph(pot);
      pot.graph_failed = true;
    } else {
      single_capture(pot, p, nl, gfd, set_f, s);
    }
  }
  return 0;
}

int bind_to(Potential &pot, Particles &p, Neighbors &nl) {
  // Elements present in the particles (p%nel / el2Z).
  std::vector<int> zs(p.hZ.begin(), p.hZ.end());
  std::sort(zs.begin(), zs.end());
  zs.erase(std::unique(zs.begin(), zs.end()), zs.end());
  const int nel = pot_nel(pot);
  auto dbidx = [&](int Z) {
    for (int q = 0; q < nel; q++)
      if (pot_Z(pot, q) == Z) return q;
    return -1;
  };
  if (pot.kind == kEAM) {
    // tabulated_alloy_eam_bind_to (:297-350): the cutoff for every pair.
    if (!zs.empty() && pot.eam->cutoff > nl.interaction_range) {
      nl.interaction_range = pot.eam->cutoff;
      nl.valid = false;
    }
  } else {
    // default_bind_to_func.f90:123-144: cut_in_h of each present pair.
    for (int zi : zs)
      for (int zj : zs) {
        const int ii = dbidx(zi), jj = dbidx(zj);
        if (ii < 0 || jj < 0) continue;
        const int t = pot_pair(pot, ii, jj);
        const double c = bop_pair_range(pot, t);
        if (c > nl.interaction_range) {
          nl.interaction_range = c;
          nl.valid = false;
        }
      }
  }
  pot.el_for = nullptr;
  return update_element_map(pot, p);
}

__global__ void fill_i32(int *__restrict__ p, int64_t n, int v) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    p[k] = v;
}

__global__ void ghost_pos4(int nat, const double *__restrict__ r, Pos4 *__restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  Pos4 q;
  q.x = r[3 * (size_t)i];
  q.y = r[3 * (size_t)i + 1];
  q.z = r[3 * (size_t)i + 2];
  q.w = 0.0;
  p[i] = q;
}

// The LAMMPS contract (bop_kernel.f90:577-597 under LAMMPS,
// pair_atomistica.cpp:386-545): nat = local + ghost atoms with explicit
// positions, a full list (CSR, 0-based) over all of them without image
// shifts; bonds are computed for the first natloc atoms only and forces are
// returned for all nat atoms (the caller sums the ghost forces back onto
// their owners).  epot and wpot are the sums over the local atoms' bonds.
// LAMMPS's per-atom virial layout, vatom (nat,6) = Fortran (6,nat), from the
// (3,3,nat) per-atom virial w (element (a,c,i) at a + 3c + 9i): the
// reference's LAMMPS build accumulates -w11, -w22, -w33, -w21, -w31, -w32
// (SUM_VIRIAL under LAMMPS, macros.inc:202; bop_kernel.f90:1514-1517).
__global__ void per_at_virial_to_voigt(int nat, const double *__restrict__ w,
                                       double *__restrict__ v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const double *a = w + 9 * (size_t)i;
  double *o = v + 6 * (size_t)i;
  o[0] -= a[0];
  o[1] -= a[4];
  o[2] -= a[8];
  o[3] -= a[1];
  o[4] -= a[2];
  o[5] -= a[5];
}

int energy_and_forces_ghost(Potential &pot, int nat, int natloc, const double *r, const int *Z,
                            const int *seed, const int *nbr, double *epot, double *f,
                            double *wpot, const int *mask, double *epa, double *wpa,
                            bool voigt) {
  if (!epot || !f || !wpot || nat < 0 || natloc < 0 || natloc > nat ||
      (nat > 0 && (!r || !Z || !seed))) {
    set_error("energy_and_forces_ghost: invalid arguments");
    return GB_ERROR_ARGUMENT;
  }
  if (pot.kind == kEAM) {
    set_error("energy_and_forces_ghost: ghost-atom lists are supported for the bond-order "
              "potentials");
    return GB_ERROR_ARGUMENT;
  }
  cudaStream_t s = pot_stream(pot);
  Neighbors &nl = pot.gnl;
  // list: CSR offsets (host copy for the sizes), entries, zero shifts
  std::vector<int> hseed(nat + 1, 0);
  if (is_device_ptr(seed))
    GB_CUDA(cudaMemcpy(hseed.data(), seed, sizeof(int) * (nat + 1), cudaMemcpyDeviceToHost));
  else
    std::memcpy(hseed.data(), seed, sizeof(int) * (nat + 1));
  const int64_t n = hseed[nat];
  int maxz = 0;
  for (int i = 0; i < nat; i++) {
    if (hseed[i + 1] < hseed[i] || hseed[0] != 0) {
      set_error("energy_and_forces_ghost: seed must be non-decreasing CSR offsets from 0");
      return GB_ERROR_ARGUMENT;
    }
    maxz = std::max(maxz, hseed[i + 1] - hseed[i]);
  }
  if (n > 0 && !nbr) {
    set_error("energy_and_forces_ghost: neighbor array missing");
    return GB_ERROR_ARGUMENT;
  }
  GB_CHECK(nl.seed.ensure(sizeof(int) * (nat + 1)));
  GB_CHECK(nl.nbr.ensure(sizeof(int) * std::max<int64_t>(n, 1)));
  GB_CHECK(nl.shift.ensure(sizeof(int) * std::max<int64_t>(n, 1)));
  // status words of the reverse-index build (allocated by nl_build otherwise)
  GB_CHECK(nl.stats.ensure(sizeof(int) * 8));
  GB_CHECK(nl.hstats.ensure(sizeof(int) * 8));
  GB_CUDA(cudaMemsetAsync(nl.stats.p, 0, sizeof(int) * 8, s));
  GB_CUDA(cudaMemcpyAsync(nl.seed.p, hseed.data(), sizeof(int) * (nat + 1),
                          cudaMemcpyHostToDevice, s));
  if (n > 0) {
    GB_CUDA(cudaMemcpyAsync(nl.nbr.p, nbr, sizeof(int) * n, cudaMemcpyDefault, s));
    const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 4096);
    fill_i32<<<blocks, 256, 0, s>>>(nl.shift.as<int>(), n, pack_shift(0, 0, 0));  // no image shifts
    note_launch();
  }
  // positions
  GB_CHECK(nl.pos4.ensure(sizeof(Pos4) * std::max(nat, 1)));
  if (nat > 0) {
    const double *rd = r;
    if (!is_device_ptr(r)) {
      GB_CHECK(pot.g_r.ensure(sizeof(double) * 3 * (size_t)nat));
      GB_CUDA(cudaMemcpyAsync(pot.g_r.p, r, sizeof(double) * 3 * (size_t)nat,
                              cudaMemcpyHostToDevice, s));
      rd = pot.g_r.as<double>();
    }
    ghost_pos4<<<(nat + 127) / 128, 128, 0, s>>>(nat, rd, nl.pos4.as<Pos4>());
    note_launch();
  }
  nl.nentries = n;
  nl.maxz = maxz;
  nl.valid = true;
  nl.rev_valid = false;
  nl.rev_pending = false;
  nl.plan_ready = false;
  nl.posff_valid = false;
  nl.built_for = nullptr;  // (not a particles-bound list)
  // element map from Z
  {
    std::vector<int> hz(std::max(nat, 1), 0);
    if (nat > 0) {
      if (is_device_ptr(Z))
        GB_CUDA(cudaMemcpy(hz.data(), Z, sizeof(int) * nat, cudaMemcpyDeviceToHost));
      else
        std::memcpy(hz.data(), Z, sizeof(int) * nat);
    }
    const int nel = pot_nel(pot);
    std::vector<int> el(std::max(nat, 1), -1);
    for (int i = 0; i < nat; i++)
      for (int q = 0; q < nel; q++)
        if (hz[i] == pot_Z(pot, q)) el[i] = q;
    GB_CHECK(pot.el.ensure(sizeof(int) * el.size()));
    GB_CUDA(cudaMemcpyAsync(pot.el.p, el.data(), sizeof(int) * el.size(), cudaMemcpyHostToDevice,
                            s));
    GB_CUDA(cudaStreamSynchronize(s));
    pot.el_for = nullptr;  // the map belongs to this call
  }
  Stage sf, sepa, swpa;
  GB_CHECK(stage_in(f, 3 * (size_t)nat, pot.out_f, s, sf));
  GB_CHECK(stage_in(epa, nat, pot.out_epa, s, sepa));
  GB_CHECK(stage_in(wpa, (voigt ? 6 : 9) * (size_t)nat, pot.out_wpa, s, swpa));
  Outputs o;
  o.f = sf.dev;
  o.epot_per_at = sepa.dev;
  o.wpot_per_at = swpa.dev;
  if (voigt && wpa) {
    // the (3,3,nat) per-atom virial goes to a zeroed scratch, converted below
    GB_CHECK(pot.g_wpa9.ensure(sizeof(double) * 9 * (size_t)std::max(nat, 1)));
    GB_CUDA(cudaMemsetAsync(pot.g_wpa9.p, 0, sizeof(double) * 9 * (size_t)std::max(nat, 1), s));
    o.wpot_per_at = pot.g_wpa9.as<double>();
  }
  if (mask) {
    if (is_device_ptr(mask)) {
      o.mask = mask;
    } else {
      GB_CHECK(pot.mask_d.ensure(sizeof(int) * std::max(nat, 1)));
      if (nat)
        GB_CUDA(cudaMemcpyAsync(pot.mask_d.p, mask, sizeof(int) * nat, cudaMemcpyHostToDevice, s));
      o.mask = pot.mask_d.as<int>();
    }
  }
  GB_CHECK(pot.red.ensure(sizeof(double) * 16));
  o.red = pot.red.as<double>();
  o.status = reinterpret_cast<int *>(o.red + 12);
  GB_CUDA(cudaMemsetAsync(o.status, 0, sizeof(int) * 4, s));
  // the ghosts' own entries carry no bond terms: start every entry from zero
  const int64_t nb = std::max<int64_t>(n, 1);
  const bool want_wat = wpa != nullptr;
  GB_CHECK(pot.bond_G.ensure(sizeof(double) * 3 * nb));
  GB_CHECK(pot.bond_e.ensure(sizeof(double) * nb));
  GB_CUDA(cudaMemsetAsync(pot.bond_G.p, 0, sizeof(double) * 3 * nb, s));
  GB_CUDA(cudaMemsetAsync(pot.bond_e.p, 0, sizeof(double) * nb, s));
  if (want_wat) {
    GB_CHECK(pot.bond_w.ensure(sizeof(double) * 9 * nb));
    GB_CUDA(cudaMemsetAsync(pot.bond_w.p, 0, sizeof(double) * 9 * nb, s));
  }
  BopSystem sys;
  sys.nat = natloc;
  sys.nat_all = nat;
  if (pot.precision == GB_PRECISION_MIXED) nl.want_posff = true;
  GB_CHECK(bop_run(pot, sys, nl, o, want_wat, false));
  if (voigt && wpa && nat > 0) {
    per_at_virial_to_voigt<<<(nat + 255) / 256, 256, 0, s>>>(nat, o.wpot_per_at, swpa.dev);
    note_launch();
  }
  GB_CHECK(stage_out(sf, s));
  GB_CHECK(stage_out(sepa, s));
  GB_CHECK(stage_out(swpa, s));
  GB_CHECK(pot.hred.ensure(sizeof(double) * 16));
  double *hr = pot.hred.as<double>();
  GB_CUDA(cudaMemcpyAsync(hr, o.red, sizeof(double) * 14, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaGetLastError());
  const int st = reinterpret_cast<const int *>(hr + 12)[0];
  pot.last_status = st;
  pot.last_bonds = n;
  if (st & 2) {
    set_error("Internal error: bond-order tile plan mismatch.");
    return GB_ERROR_UNSPECIFIED;
  }
  if (st & 4) {
    set_error("Internal neighbor list exhausted: an atom has more bonds after screening than "
              "the screened kernel supports (32).");
    return GB_ERROR_CAPACITY;
  }
  if (is_device_ptr(epot)) {
    GB_CUDA(cudaMemcpy(epot, hr, sizeof(double), cudaMemcpyHostToDevice));
  } else {
    *epot = hr[0];
  }
  if (is_device_ptr(wpot)) {
    double w[9];
    GB_CUDA(cudaMemcpy(w, wpot, sizeof(w), cudaMemcpyDeviceToHost));
    for (int q = 0; q < 9; q++) w[q] += hr[1 + q];
    GB_CUDA(cudaMemcpy(wpot, w, sizeof(w), cudaMemcpyHostToDevice));
  } else {
    for (int q = 0; q < 9; q++) wpot[q] += hr[1 + q];
  }
  return 0;
}

}  // namespace
}  // namespace gb

extern "C" {

int gb_tersoff_new(gb_potential_t **h, const gb_tersoff_params_t *params) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_tersoff_params_t p = params ? *params : default_tersoff();
  GB_CHECK(check_tersoff(p));
  *h = new gb_potential;
  (*h)->pot.kind = kTersoff;
  (*h)->pot.tp = p;
  return 0;
}

int gb_kumagai_new(gb_potential_t **h, const gb_kumagai_params_t *params) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_kumagai_params_t p = params ? *params : default_kumagai();
  GB_CHECK(check_kumagai(p));
  *h = new gb_potential;
  (*h)->pot.kind = kKumagai;
  (*h)->pot.kp = p;
  return 0;
}

int gb_tersoff_scr_new(gb_potential_t **h, const gb_tersoff_params_t *params,
                       const gb_screening_params_t *scr) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_tersoff_params_t p = params ? *params : default_tersoff_scr();
  gb_screening_params_t sc = scr ? *scr : default_screening_tersoff();
  GB_CHECK(check_tersoff(p));
  GB_CHECK(check_screening(sc, p.nel * (p.nel + 1) / 2));
  *h = new gb_potential;
  (*h)->pot.kind = kTersoff;
  (*h)->pot.tp = p;
  (*h)->pot.screened = true;
  (*h)->pot.scr = sc;
  return 0;
}

int gb_kumagai_scr_new(gb_potential_t **h, const gb_kumagai_params_t *params,
                       const gb_screening_params_t *scr) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_kumagai_params_t p = params ? *params : default_kumagai_scr();
  gb_screening_params_t sc = scr ? *scr : default_screening_kumagai();
  GB_CHECK(check_kumagai(p));
  GB_CHECK(check_screening(sc, 1));
  *h = new gb_potential;
  (*h)->pot.kind = kKumagai;
  (*h)->pot.kp = p;
  (*h)->pot.screened = true;
  (*h)->pot.scr = sc;
  return 0;
}

int gb_brenner_new(gb_potential_t **h, const gb_brenner_params_t *params) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_brenner_params_t p = params ? *params : default_brenner();
  GB_CHECK(check_brenner(p));
  *h = new gb_potential;
  (*h)->pot.kind = kBrenner;
  (*h)->pot.bp = p;
  return 0;
}

int gb_brenner_scr_new(gb_potential_t **h, const gb_brenner_params_t *params,
                       const gb_screening_params_t *scr) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_brenner_params_t p = params ? *params : default_brenner_scr();
  gb_screening_params_t sc = scr ? *scr : default_screening_tersoff();
  GB_CHECK(check_brenner(p));
  GB_CHECK(check_screening(sc, p.nel * (p.nel + 1) / 2));
  *h = new gb_potential;
  (*h)->pot.kind = kBrenner;
  (*h)->pot.bp = p;
  (*h)->pot.screened = true;
  (*h)->pot.scr = sc;
  return 0;
}

int gb_juslin_new(gb_potential_t **h, const gb_juslin_params_t *params) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_juslin_params_t p = params ? *params : default_juslin(false);
  if (p.nel < 1 || p.nel > 3) return check_juslin(p);
  fill_juslin(p, nullptr);
  GB_CHECK(check_juslin(p));
  *h = new gb_potential;
  (*h)->pot.kind = kJuslin;
  (*h)->pot.jp = p;
  return 0;
}

int gb_juslin_scr_new(gb_potential_t **h, const gb_juslin_params_t *params,
                      const gb_screening_params_t *scr) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  gb_juslin_params_t p = params ? *params : default_juslin(true);
  gb_screening_params_t sc = scr ? *scr : default_screening_juslin();
  if (p.nel < 1 || p.nel > 3) return check_juslin(p);
  fill_juslin(p, &sc);
  GB_CHECK(check_juslin(p));
  GB_CHECK(check_screening(sc, p.nel * p.nel));
  for (int q = 0; q < p.nel * p.nel; q++)
    if (!(sc.Cmax[q] > 1.0)) {
      set_error("JuslinScr: Cmax must be > 1 (C_dr_cut = Cmax^2 / (4 (Cmax - 1)))");
      return GB_ERROR_ARGUMENT;
    }
  *h = new gb_potential;
  (*h)->pot.kind = kJuslin;
  (*h)->pot.jp = p;
  (*h)->pot.screened = true;
  (*h)->pot.scr = sc;
  return 0;
}

int gb_tabulated_eam_new(gb_potential_t **h, const char *fn) {
  clear_error();
  if (!h || !fn) return GB_ERROR_ARGUMENT;
  std::unique_ptr<EamTables> t(new EamTables);
  GB_CHECK(eam_read_funcfl(fn, *t));
  GB_CHECK(eam_upload(*t));
  *h = new gb_potential;
  (*h)->pot.kind = kEAM;
  (*h)->pot.eam = std::move(t);
  return 0;
}

int gb_tabulated_alloy_eam_new(gb_potential_t **h, const char *fn) {
  clear_error();
  if (!h || !fn) return GB_ERROR_ARGUMENT;
  std::unique_ptr<EamTables> t(new EamTables);
  GB_CHECK(eam_read_setfl(fn, *t));
  GB_CHECK(eam_upload(*t));
  *h = new gb_potential;
  (*h)->pot.kind = kEAM;
  (*h)->pot.eam = std::move(t);
  return 0;
}

void gb_potential_free(gb_potential_t *h) {
  if (!h) return;
  Potential &pot = h->pot;
  drop_single_graph(pot);
  for (int q = 0; q < 4; q++)
    if (pot.ev[q]) cudaEventDestroy(pot.ev[q]);
  for (int q = 0; q < 2; q++)
    if (pot.kev[q]) cudaEventDestroy(pot.kev[q]);
  if (pot.aux_ev) cudaEventDestroy(pot.aux_ev);
  if (pot.aux) cudaStreamDestroy(pot.aux);
  if (pot.own_stream && pot.stream) cudaStreamDestroy(pot.stream);
  delete h;
}

int gb_potential_set_precision(gb_potential_t *h, int precision) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  if (precision != GB_PRECISION_FP64 && precision != GB_PRECISION_MIXED) {
    set_error("precision must be GB_PRECISION_FP64 or GB_PRECISION_MIXED");
    return GB_ERROR_ARGUMENT;
  }
  if (h->pot.kind == kEAM && precision != GB_PRECISION_FP64) {
    set_error("TabulatedAlloyEAM has only the FP64 form.");
    return GB_ERROR_ARGUMENT;
  }
  if (h->pot.screened && precision != GB_PRECISION_FP64) {
    set_error("The screened potentials have only the FP64 form.");
    return GB_ERROR_ARGUMENT;
  }
  h->pot.precision = precision;
  return 0;
}

int gb_potential_set_stream(gb_potential_t *h, void *stream) {
  if (!h) return GB_ERROR_ARGUMENT;
  Potential &pot = h->pot;
  if (pot.own_stream && pot.stream) cudaStreamDestroy(pot.stream);
  pot.own_stream = false;
  pot.stream = (cudaStream_t)stream;
  if (!stream) pot_stream(pot);
  return 0;
}

double gb_potential_get_cutoff(const gb_potential_t *h) {
  if (!h) return -1.0;
  const Potential &pot = h->pot;
  if (pot.kind == kEAM) return pot.eam->cutoff;
  double c = 0.0;
  const int np = pot_npairs(pot);
  for (int q = 0; q < np; q++) c = std::max(c, bop_pair_range(pot, q));
  return c;
}

int gb_potential_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl, int *ierror) {
  clear_error();
  int rc = (h && p && nl) ? bind_to(h->pot, p->p, nl->nl) : GB_ERROR_ARGUMENT;
  if (ierror) *ierror = rc;
  return rc;
}

int gb_potential_energy_and_forces_ghost(gb_potential_t *h, int nat, int natloc,
                                         const double *r, const int *Z, const int *seed,
                                         const int *nbr, double *epot, double *f, double *wpot,
                                         const int *mask, double *epot_per_at,
                                         double *wpot_per_at, int *ierror) {
  clear_error();
  int rc = h ? energy_and_forces_ghost(h->pot, nat, natloc, r, Z, seed, nbr, epot, f, wpot, mask,
                                       epot_per_at, wpot_per_at, false)
             : GB_ERROR_ARGUMENT;
  if (ierror) *ierror = rc;
  return rc;
}

int gb_potential_energy_and_forces_lammps(gb_potential_t *h, int nat, int natloc,
                                          const double *r, const int *Z, const int *seed,
                                          const int *nbr, double *epot, double *f, double *wpot,
                                          const int *mask, double *epot_per_at, double *vatom,
                                          int *ierror) {
  clear_error();
  int rc = h ? energy_and_forces_ghost(h->pot, nat, natloc, r, Z, seed, nbr, epot, f, wpot, mask,
                                       epot_per_at, vatom, true)
             : GB_ERROR_ARGUMENT;
  if (ierror) *ierror = rc;
  return rc;
}

int gb_potential_energy_and_forces_flags(gb_potential_t *h, gb_particles_t *p,
                                         gb_neighbors_t *nl, const double *q, double *epot,
                                         double *f, double *wpot, const int *mask, double *epa,
                                         double *epb, double *fpb, double *wpa, double *wpb,
                                         int flags, int *ierror) {
  (void)q;
  clear_error();
  int rc = (h && p && nl)
               ? energy_and_forces(h->pot, p->p, nl->nl, epot, f, wpot, mask, epa, epb, fpb, wpa,
                                   wpb, flags)
               : GB_ERROR_ARGUMENT;
  if (ierror) *ierror = rc;
  return rc;
}

int gb_potential_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                   const double *q, double *epot, double *f, double *wpot,
                                   const int *mask, double *epa, double *epb, double *fpb,
                                   double *wpa, double *wpb, int *ierror) {
  (void)q;
  clear_error();
  int rc = (h && p && nl)
               ? energy_and_forces(h->pot, p->p, nl->nl, epot, f, wpot, mask, epa, epb, fpb, wpa,
                                   wpb)
               : GB_ERROR_ARGUMENT;
  if (ierror) *ierror = rc;
  return rc;
}

int gb_tersoff_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl, int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_tersoff_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epa, double *epb, double *fpb,
                                 double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}
int gb_kumagai_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl, int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_kumagai_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epa, double *epb, double *fpb,
                                 double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}
int gb_brenner_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl, int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_brenner_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                 const double *q, double *epot, double *f, double *wpot,
                                 const int *mask, double *epa, double *epb, double *fpb,
                                 double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}
int gb_juslin_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl, int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_juslin_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                const double *q, double *epot, double *f, double *wpot,
                                const int *mask, double *epa, double *epb, double *fpb,
                                double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}
int gb_tabulated_alloy_eam_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                   int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_tabulated_alloy_eam_energy_and_forces(gb_potential_t *h, gb_particles_t *p,
                                             gb_neighbors_t *nl, const double *q, double *epot,
                                             double *f, double *wpot, const int *mask,
                                             double *epa, double *epb, double *fpb,
                                             double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}
int gb_tabulated_eam_bind_to(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                             int *ierror) {
  return gb_potential_bind_to(h, p, nl, ierror);
}
int gb_tabulated_eam_energy_and_forces(gb_potential_t *h, gb_particles_t *p, gb_neighbors_t *nl,
                                       const double *q, double *epot, double *f, double *wpot,
                                       const int *mask, double *epa, double *epb, double *fpb,
                                       double *wpa, double *wpb, int *ierror) {
  return gb_potential_energy_and_forces(h, p, nl, q, epot, f, wpot, mask, epa, epb, fpb, wpa, wpb,
                                        ierror);
}

int gb_potential_set_elements(gb_potential_t *h, const char *elements) {
  clear_error();
  if (!h || !elements) {
    set_error("set_elements: missing argument");
    return GB_ERROR_ARGUMENT;
  }
  Potential &pot = h->pot;
  if (pot.kind != kEAM) {
    set_error("set_elements: only the EAM potentials have an element filter");
    return GB_ERROR_ARGUMENT;
  }
  // filter_from_string (src/core/filter.f90:55-120): "*" = all elements,
  // else comma-separated symbols (or atomic numbers), each read into two
  // characters; an unknown symbol is an error.
  std::vector<int> flt;
  const std::string str(elements);
  std::string trimmed = str;
  trimmed.erase(trimmed.find_last_not_of(' ') + 1);
  if (trimmed != "*") {
    size_t start = 0;
    while (true) {
      const size_t comma = str.find(',', start);
      const std::string tok = str.substr(start, comma == std::string::npos ? std::string::npos
                                                                            : comma - start);
      const std::string sym = tok.substr(0, 2);
      const int Z = element_Z(sym);
      if (Z <= 0) {
        set_error("Unknown element '" + sym + "'.");
        return GB_ERROR_ARGUMENT;
      }
      flt.push_back(Z);
      if (comma == std::string::npos) break;
      start = comma + 1;
    }
  }
  pot.el_filter = flt;
  pot.el_for = nullptr;  // rebuild the element map on the next call
  return 0;
}

int gb_tabulated_alloy_eam_table(const gb_potential_t *h, int which, int idx, double *x0dx,
                                 double *coef) {
  clear_error();
  if (!h || h->pot.kind != kEAM) return GB_ERROR_ARGUMENT;
  const EamTables &t = *h->pot.eam;
  const SplineHost *s = nullptr;
  if (which == 0 && idx >= 0 && idx < t.nel) s = &t.F[idx];
  if (which == 1 && idx >= 0 && idx < t.nel) s = &t.rho[idx];
  if (which == 2 && idx >= 0 && idx < t.nel * t.nel) s = &t.phi[idx];
  if (!s) return GB_ERROR_ARGUMENT;
  if (x0dx) {
    x0dx[0] = s->x0;
    x0dx[1] = s->dx;
    x0dx[2] = s->cut;
  }
  if (coef) {
    const std::vector<double> *arr[8] = {&s->y, &s->d2y, &s->c1, &s->c2,
                                         &s->c3, &s->d1, &s->d2, &s->d3};
    for (int c = 0; c < 8; c++)
      for (int k = 0; k < s->n; k++)
        coef[(size_t)c * s->n + k] = k < (int)arr[c]->size() ? (*arr[c])[k] : 0.0;
  }
  return s->n;
}

int gb_potential_last_timing(const gb_potential_t *h, double *ms) {
  if (!h || !ms) return GB_ERROR_ARGUMENT;
  for (int q = 0; q < 4; q++) ms[q] = h->pot.timing[q];
  return 0;
}

int gb_potential_set_graph(gb_potential_t *h, int on) {
  if (!h) return GB_ERROR_ARGUMENT;
  h->pot.use_graph = on != 0;
  h->pot.graph_failed = false;
  h->pot.graph_unused = 0;
  if (!on) drop_single_graph(h->pot);
  return 0;
}

int gb_potential_set_tile_atoms(gb_potential_t *h, int atoms) {
  if (!h || atoms < 0) return GB_ERROR_ARGUMENT;
  h->pot.tile_request = atoms;
  return 0;
}

int gb_potential_last_stats(const gb_potential_t *h, int64_t *stats) {
  if (!h || !stats) return GB_ERROR_ARGUMENT;
  stats[0] = h->pot.last_bonds;
  stats[1] = h->pot.last_hot;
  stats[2] = h->pot.tile_atoms;
  stats[3] = h->pot.last_replayed ? 1 : 0;
  return 0;
}

}  // extern "C"
