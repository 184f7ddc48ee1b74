// Batch of independent structures (batch.cu) and the helpers shared with the
// differentiation path (autodiff.cu).
#pragma once

#include <vector>

#include "potential.h"

namespace gb {

struct Batch {
  int nstruct = 0, nat = 0;
  std::vector<int> atom_off;  // nstruct + 1
  std::vector<double> A;      // 9 per structure: A[a][k], column k = lattice vector k
  std::vector<double> B;      // inverses
  std::vector<int> pbc;       // 3 per structure
  std::vector<int> hZ;        // nat
  uint64_t geom_rev = 0, pos_rev = 0;
  DevBuf r, sid, bps, Acells, Acells_ff, tiles, red_seg, el;
  DevBuf tan_G, tan_part, tan_f, tan_dpos, tan_red;  // tangent evaluation scratch
  HostBuf hseg;
  // cached derived state
  uint64_t built_geom = ~0ull, built_pos = ~0ull, el_geom = ~0ull;
  const Potential *el_pot = nullptr;
  double built_cutoff = -1.0;
  int ncells = 0, tiles_apt = 0, ntiles = 0;
  int64_t tiles_nentries = -1;
  Neighbors nl;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
};

cudaStream_t batch_stream(Batch &b);
// Element index of every atom for the potential; per-structure binning for
// the cutoff; tiles of at most apt atoms inside each structure.
int batch_elements(Batch &b, Potential &pot, cudaStream_t s);
int batch_binning(Batch &b, double cutoff, cudaStream_t s);
int batch_tiles(Batch &b, int apt, cudaStream_t s);
double batch_cutoff(const Batch &b, const Potential &pot);

}  // namespace gb

struct gb_batch {
  gb::Batch b;
};
