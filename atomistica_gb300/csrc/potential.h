// Internal potential object shared by bop.cu, eam.cu and api.cu.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "internal.h"

namespace gb {

enum PotKind { kTersoff = 0, kKumagai = 1, kEAM = 2, kBrenner = 3, kJuslin = 4 };

// Uniform natural cubic spline tables (simple_spline.f90:127-195) built on the
// host.  Device layout: 8 doubles per interval k = {y_k, c1_k, c2_k, c3_k,
// d1_k, d2_k, d3_k, 0} so that one value-gather is one 32-byte sector and a
// value+derivative gather is two.
struct SplineHost {
  int n = 0;
  double x0 = 0, dx = 1, cut = 0;
  std::vector<double> y, d2y, c1, c2, c3, d1, d2, d3;
  void init(int n, double x0, double dx, const double *yy);
  void scale_y(double fac);
};

struct SplineDev {
  const double *tab;  // 8*(n-1) doubles
  int n;
  double x0, dx, cut;
  double rdx;  // 1 / dx
};

struct EamTables {
  int nel = 0;
  std::vector<int> Z;
  std::vector<std::string> names;  // element names of the setfl header
  double cutoff = 0;
  // Single-element funcfl file (TabulatedEAM, tabulated_eam.f90): phi[0]
  // holds the scaled effective charge Z(r), the pair term is Z^2 / r, the
  // splines are evaluated as the reference's SPLINE_* macros, every atom is
  // of the file's element.
  bool funcfl = false;
  std::vector<SplineHost> F, rho, phi;  // phi[i*nel+j]
  DevBuf dev;                           // all tables, packed
  std::vector<SplineDev> dF, drho, dphi;
};

int eam_read_setfl(const char *fn, EamTables &t);
int eam_read_funcfl(const char *fn, EamTables &t);
int eam_upload(EamTables &t);

struct Outputs {
  // Device pointers (accumulated into); NULL when not requested.
  double *f = nullptr;
  bool f_set = false;  // f is written (every atom), not accumulated into
  double *epot_per_at = nullptr;
  double *wpot_per_at = nullptr;
  double *epot_per_bond = nullptr;
  double *f_per_bond = nullptr;
  double *wpot_per_bond = nullptr;
  const int *mask = nullptr;
  // Device result of the reductions: [0] epot, [1..9] wpot Fortran order.
  double *red = nullptr;
  // Device status word: bit 0 spline argument out of range, bit 1 tile plan
  // mismatch.
  int *status = nullptr;
};

struct Potential {
  PotKind kind = kTersoff;
  int precision = GB_PRECISION_FP64;
  gb_tersoff_params_t tp{};
  gb_kumagai_params_t kp{};
  gb_brenner_params_t bp{};
  gb_juslin_params_t jp{};      // ordered-pair entries filled as juslin_module.f90:273-300
  bool screened = false;        // TersoffScr / KumagaiScr / BrennerScr / JuslinScr
  gb_screening_params_t scr{};  // their outer / bond-order cutoffs, Cmin, Cmax
  std::unique_ptr<EamTables> eam;

  cudaStream_t stream = nullptr;
  bool own_stream = false;

  // Element filter of the EAM potentials (the `elements` property,
  // tabulated_alloy_eam.f90:72, tabulated_eam.f90): atomic numbers the
  // potential acts on; empty = "*" (all).
  std::vector<int> el_filter;

  // Element map for the bound particles.
  DevBuf el;
  const Particles *el_for = nullptr;
  uint64_t el_zrev = ~0ull;

  // Scratch.
  DevBuf bond_G, bond_e, bond_w, bond_fr, tile_part, red;
  DevBuf atom_dF;
  DevBuf eam_cache;  // per list entry: spline coordinate, 1/r, interval (EAM density pass)
  DevBuf red_stage;  // first-stage sums of the tile partials
  DevBuf out_f, out_epa, out_wpa, out_epb, out_fpb, out_wpb, mask_d;
  // Ghost-atom calls (a caller's list over local + ghost atoms, no image
  // shifts): the list, positions and element map live here.
  Neighbors gnl;
  DevBuf g_r;
  DevBuf g_wpa9;  // (3,3,nat) per-atom virial before the LAMMPS Voigt conversion
  HostBuf hred;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t kev[2] = {nullptr, nullptr};  // around the dominant force kernel
  cudaStream_t aux = nullptr;   // host->device force upload, overlapped with the list build
  cudaEvent_t aux_ev = nullptr;
  double timing[4] = {0, 0, 0, 0};
  int tile_atoms = 32;
  int tile_request = 0;     // atoms per tile requested (0: automatic)
  int last_status = 0;
  int last_hot = 0;         // bonds recomputed on the accurate path (mixed form)
  int64_t last_bonds = 0;   // directed bonds of the last bond-order call
  int last_plan[2] = {0, 0};  // largest bonds / (ij, ik) slots per tile of the last call

  // CUDA graph of a whole single-structure evaluation (gb_potential_set_graph):
  // list build, tile kernel, gather, sums and the status / result copies,
  // captured after an eager evaluation and replayed while the particles,
  // list, cell, force buffer and every device buffer are unchanged.
  bool use_graph = false;
  bool graph_failed = false;  // capture not possible (or not useful): stay eager
  int graph_unused = 0;       // captures in a row that were never replayed
  bool last_replayed = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int graph_kernels = 0, graph_cap = 0, graph_nat = 0, graph_prec = 0, graph_tile_request = 0;
  bool graph_set_f = false;
  const void *graph_p = nullptr, *graph_nl = nullptr;
  uint64_t graph_cell_rev = 0;
  double graph_cutoff = 0.0;
  double *graph_fd = nullptr;
  cudaStream_t graph_stream = nullptr;
  std::vector<const void *> graph_bufs;
};

// Interaction range requested by bind_to for element pair t (database
// indices): r2, or for the screened variants sqrt(C_dr_cut(t)) times the
// largest cutoff of all pairs (default_bind_to_func.f90:117-144; BrennerScr:
// of pair t itself, brenner_module.f90:229-243).
double bop_pair_range(const Potential &pot, int t);

// Kernel launches (on pot.stream) for an up-to-date neighbour list.
int bop_compute(Potential &pot, const Particles &p, Neighbors &nl, const Outputs &o,
                bool want_wat, bool want_per_bond);
// (chk, capture: a captured evaluation, see ReplayCheck; no event records)
// Per-entry cache of the EAM density pass (spline coordinate, 1/r and
// interval of each list entry, 20 bytes), sized for `entries` list entries.
int eam_cache_ensure(Potential &pot, int64_t entries);
int eam_compute(Potential &pot, const Particles &p, Neighbors &nl, const Outputs &o,
                bool want_wat, ReplayCheck chk = ReplayCheck{}, bool capture = false);
// Element count / atomic number of element q of the potential; its stream.
int pot_nel(const Potential &pot);
// Number of element-pair entries (nel (nel + 1) / 2 symmetric pairs; Juslin:
// nel^2 ordered pairs) and the entry of the database elements (a, b).
int pot_npairs(const Potential &pot);
int pot_pair(const Potential &pot, int a, int b);
int pot_Z(const Potential &pot, int q);
// Inner cutoffs r1, r2 per pair of a bond-order potential.
const double *bop_r1(const Potential &pot);
const double *bop_r2(const Potential &pot);
cudaStream_t pot_stream(Potential &pot);

// Deterministic fixed-order sum of tile partials: red[c] = sum_t part[t*nc+c].
// Deterministic sum of nrows rows of nc (= 10) doubles into red[0..nc); with a
// stage buffer of reduce_stage_bytes(nrows) bytes large inputs use two passes.
constexpr int kRedRowsPerBlock = 256;
size_t reduce_stage_bytes(int nrows);
int reduce_partials(const double *part, int nrows, int nc, double *red, double *stage,
                    cudaStream_t s);
// Per-segment sums of 10-column rows: out[q][.] = sum of rows [seg[q], seg[q+1]).
int reduce_segments(const double *part, const int *seg, int nseg, double *out, cudaStream_t s);
int reduce_seg_pieces(const double *part, const int *piece0, int npiece, const int *seg_piece,
                      int nseg, double *psum, double *out, cudaStream_t s);

// The system a bond-order evaluation runs on: one structure (cell A), or a
// batch of structures whose tiles (cut by the caller, at most apt atoms, never
// across structures) carry their structure's cell and whose energy/virial sums
// go per structure into red_seg (nseg x 10: energy, virial).
struct BopSystem {
  int nat = 0;      // atoms whose bonds are computed (the tiles)
  int nat_all = 0;  // atoms of the list, forces gathered for all (ghost atoms; 0: nat)
  double A[3][3] = {{0}};
  const int *tile_atom0 = nullptr;   // device, ntiles + 1
  const int *tile_struct = nullptr;  // device, ntiles
  const double *Acells = nullptr;    // device, 9 per structure
  const float2 *Acells_ff = nullptr; // device, 9 float-float pairs per structure
  int ntiles = 0, apt = 0;
  // Captured evaluation (CUDA graph): no host synchronisation; buffers sized
  // for nb_capacity list entries; tile plan max_nbt / max_ntrip given.
  bool capture = false;
  int64_t nb_capacity = 0;
  const int *el = nullptr;           // device element map (nullptr: the potential's)
  int max_nbt = 0, max_ntrip = 0;
  const int *seg = nullptr;          // device, tile offsets of the structures (nseg + 1)
  int nseg = 0;
  double *red_seg = nullptr;         // device, nseg x 10
  // Pieces of the structures' tile rows (at most 32 rows each): piece p is
  // rows [piece0[p], piece0[p + 1]), structure q has pieces
  // [seg_piece[q], seg_piece[q + 1]); piece_sum (npiece x 10) is scratch.
  // nullptr: the structures' rows are summed by one block each.
  const int *piece0 = nullptr;
  const int *seg_piece = nullptr;
  int npiece = 0;
  double *piece_sum = nullptr;
  // A captured evaluation's gathers check the replay's validity.
  ReplayCheck check;
};
int bop_run(Potential &pot, const BopSystem &sys, Neighbors &nl, const Outputs &o,
            bool want_wat, bool want_pb);
// Atoms per tile for a list whose largest coordination is maxz.
// Shared memory of a tile with nbt bonds and ntrip (ij, ik) slots, and the
// largest a tile may use (bytes).
size_t bop_tile_smem(bool mixed, int nbt, int ntrip);
size_t bop_tile_smem_budget();
// Resident tile CTAs per SM of the evaluation pot would launch with smem.
int bop_tile_ctas_per_sm(const Potential &pot, size_t smem);

}  // namespace gb

// Opaque handle type of the C-ABI.
struct gb_potential {
  gb::Potential pot;
};
