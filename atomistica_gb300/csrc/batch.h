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
  std::vector<int> zu;        // distinct atomic numbers of the batch (sorted)
  uint64_t geom_rev = 0, pos_rev = 0;
  DevBuf r, sid, bps, Acells, Acells_ff, tiles, red_seg, red_piece, el;
  DevBuf tan_G, tan_part, tan_f, tan_dpos, tan_red;  // tangent evaluation scratch
  HostBuf hseg;
  // cached derived state
  uint64_t built_geom = ~0ull, built_pos = ~0ull, el_geom = ~0ull;
  const Potential *el_pot = nullptr;
  double built_cutoff = -1.0;
  int ncells = 0, tiles_apt = 0, ntiles = 0, npiece = 0;
  int64_t tiles_nentries = -1;
  // Tiles of the bond-order kernels (batch_tiles_work): cut inside each
  // structure by a bond budget from the per-atom counts of the list built
  // when they were cut; kept while the geometry is unchanged.
  int tiles_budget = 0;      // bonds per tile; 0: the tiles are of fixed atom count
  int tile_max_atoms = 0;    // most atoms in one tile
  uint64_t tiles_geom = ~0ull, tiles_pos = ~0ull;  // geometry / positions they were cut for
  Neighbors nl;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // Tile autotuning: the bond budget per tile timed fastest for (geometry,
  // potential, precision).
  bool autotune = false;
  int tuned_apt = 0;
  uint64_t tuned_geom = ~0ull;
  const Potential *tuned_pot = nullptr;
  int tuned_prec = -1, tune_candidates = 0;
  // CUDA graph of the whole evaluation (list build, tiles, gather, sums):
  // replayed while geometry, potential, tiles and every buffer it uses are
  // unchanged; any overflow seen after a replay falls back to the eager path.
  bool use_graph = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_failed = false;
  uint64_t graph_geom = ~0ull;
  const Potential *graph_pot = nullptr;
  int graph_prec = -1, graph_apt = 0, graph_kernels = 0;
  int graph_cap = 0, graph_ncells = 0;  // list capacity per atom, cells: baked into the graph
  int graph_kind = 0;       // 0: one evaluation; 1: a velocity-Verlet step around it
  double graph_dt = 0.0;
  // Velocity Verlet (verlet.f90:100-235): velocities, masses and the forces
  // at the current positions (valid while md_f_pos == pos_rev).
  DevBuf md_v, md_m, md_f;
  uint64_t md_f_pos = ~0ull;
  std::vector<double> md_e, md_w;  // per-structure energies / virials of the last step
  std::vector<const void *> graph_bufs;
  DevBuf gf;  // forces accumulated by the graph
  // A graph of one evaluation captured for a device force array of the
  // caller accumulates into that array directly (graph_fout); a call with
  // another array drops such a graph, and later graphs use gf.
  double *graph_fout = nullptr;
  bool graph_direct_off = false;
  int64_t info[4] = {0, 0, 0, 0};  // last call: replayed, bonds/tile, kernels in graph, tuned
  ~Batch();
};

cudaStream_t batch_stream(Batch &b);
// Element index of every atom for the potential; per-structure binning for
// the cutoff; tiles of at most apt atoms inside each structure.
int batch_elements(Batch &b, Potential &pot, cudaStream_t s);
int batch_binning(Batch &b, double cutoff, cudaStream_t s);
int batch_tiles(Batch &b, int apt, cudaStream_t s);
int batch_tiles_work(Batch &b, int budget, cudaStream_t s, bool recut = false);
double batch_cutoff(const Batch &b, const Potential &pot);

}  // namespace gb

struct gb_batch {
  gb::Batch b;
};
