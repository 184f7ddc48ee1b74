// Host-side generator of the random structures of the synthetic workloads:
// uniform positions in a triclinic cell with every pair (over all periodic
// images) at least dmin apart, by random sequential addition.
//
// Candidates are drawn from a counter-free xoshiro256** stream seeded by
// splitmix64, so a (nat, cell, dmin, seed) gives the same positions on every
// host (integer generator, no FMA contraction in host code).  Accepted atoms
// are kept in a periodic grid of bins at least dmin high, so a candidate is
// tested against the 27 surrounding bins only; cells too thin for a 3-bin
// grid along an axis are tested against all atoms and all images within
// dmin instead.
#include <cmath>
#include <cstdint>
#include <vector>

#include "internal.h"

namespace gb {
namespace {

struct Xoshiro {
  uint64_t s[4];
  explicit Xoshiro(uint64_t seed) {
    for (int k = 0; k < 4; k++) {  // splitmix64
      seed += 0x9e3779b97f4a7c15ull;
      uint64_t z = seed;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      s[k] = z ^ (z >> 31);
    }
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }  // [0, 1)
};

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int gb_random_packing(int nat, const double *cell, double dmin, uint64_t seed,
                                 int64_t max_tries, double *pos) {
  clear_error();
  if (nat < 0 || !cell || (nat > 0 && !pos) || !(dmin > 0.0)) return GB_ERROR_ARGUMENT;
  if (nat == 0) return 0;
  // rows of cell are the lattice vectors; r = f @ cell
  double A[3][3], B[3][3];
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) A[a][k] = cell[3 * k + a];  // A[:, k] = vector k
  if (cell_inverse(A, B) != 0) {
    set_error("random_packing: singular cell");
    return GB_ERROR_ARGUMENT;
  }
  // plane spacing along lattice direction k: 1 / |row k of A^-1|
  double h[3];
  int nimg[3], ng[3];
  for (int k = 0; k < 3; k++) {
    h[k] = 1.0 / std::sqrt(B[k][0] * B[k][0] + B[k][1] * B[k][1] + B[k][2] * B[k][2]);
    nimg[k] = (int)std::ceil(dmin / h[k]);
    ng[k] = (int)std::floor(h[k] / dmin);
  }
  const double d2min = dmin * dmin;
  auto disp2 = [&](const double *fa, const double *fb, int s0, int s1, int s2) {
    const double df[3] = {fa[0] - fb[0] + s0, fa[1] - fb[1] + s1, fa[2] - fb[2] + s2};
    double d2 = 0.0;
    for (int c = 0; c < 3; c++) {
      const double x = df[0] * cell[c] + df[1] * cell[3 + c] + df[2] * cell[6 + c];
      d2 += x * x;
    }
    return d2;
  };
  // an atom must also clear its own periodic images
  {
    const double z[3] = {0, 0, 0};
    for (int s0 = -nimg[0]; s0 <= nimg[0]; s0++)
      for (int s1 = -nimg[1]; s1 <= nimg[1]; s1++)
        for (int s2 = -nimg[2]; s2 <= nimg[2]; s2++)
          if ((s0 | s1 | s2) != 0 && disp2(z, z, s0, s1, s2) < d2min) {
            set_error("random_packing: cell too small for dmin");
            return GB_ERROR_ARGUMENT;
          }
  }
  Xoshiro rng(seed);
  std::vector<double> frac(3 * (size_t)nat);
  const bool grid = ng[0] >= 3 && ng[1] >= 3 && ng[2] >= 3;
  std::vector<std::vector<int>> bins;
  if (grid) bins.resize((size_t)ng[0] * ng[1] * ng[2]);
  int n = 0;
  for (int64_t tries = 0; n < nat; tries++) {
    if (tries >= max_tries) {
      set_error("random_packing: no room left after the maximum number of candidates");
      return GB_ERROR_DOMAIN;
    }
    double f[3];
    for (int c = 0; c < 3; c++) f[c] = rng.uniform();
    bool ok = true;
    if (grid) {
      int g[3];
      for (int c = 0; c < 3; c++) g[c] = std::min((int)(f[c] * ng[c]), ng[c] - 1);
      for (int o0 = -1; o0 <= 1 && ok; o0++)
        for (int o1 = -1; o1 <= 1 && ok; o1++)
          for (int o2 = -1; o2 <= 1 && ok; o2++) {
            int b[3] = {g[0] + o0, g[1] + o1, g[2] + o2}, w[3];
            for (int c = 0; c < 3; c++) {
              w[c] = b[c] < 0 ? -1 : (b[c] >= ng[c] ? 1 : 0);
              b[c] -= w[c] * ng[c];
            }
            for (int j : bins[((size_t)b[0] * ng[1] + b[1]) * ng[2] + b[2]])
              if (disp2(&frac[3 * (size_t)j], f, w[0], w[1], w[2]) < d2min) {
                ok = false;
                break;
              }
          }
      if (ok) bins[((size_t)g[0] * ng[1] + g[1]) * ng[2] + g[2]].push_back(n);
    } else {
      for (int j = 0; j < n && ok; j++)
        for (int s0 = -nimg[0]; s0 <= nimg[0] && ok; s0++)
          for (int s1 = -nimg[1]; s1 <= nimg[1] && ok; s1++)
            for (int s2 = -nimg[2]; s2 <= nimg[2] && ok; s2++)
              if (disp2(&frac[3 * (size_t)j], f, s0, s1, s2) < d2min) ok = false;
    }
    if (!ok) continue;
    for (int c = 0; c < 3; c++) frac[3 * (size_t)n + c] = f[c];
    n++;
  }
  for (int i = 0; i < nat; i++)
    for (int c = 0; c < 3; c++) {
      const double *fi = &frac[3 * (size_t)i];
      pos[3 * (size_t)i + c] = fi[0] * cell[c] + fi[1] * cell[3 + c] + fi[2] * cell[6 + c];
    }
  return 0;
}
