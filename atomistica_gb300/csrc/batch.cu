// Batched bond-order evaluation: many independent periodic structures of
// uneven size and shape (each with its own triclinic cell and pbc flags) in
// one neighbour build and one tile-kernel launch.
//
//   * atoms of all structures are concatenated; sid[i] is the structure of
//     atom i; each structure has its own binning parameters (its cells are
//     numbered consecutively after the previous structure's), so the cell
//     lists are segmented and one pair-search launch covers every structure;
//   * bond-order tiles never cross a structure and carry their structure's
//     cell; the per-tile energy/virial rows are summed per structure;
//   * forces come from the same gather as a single structure.
//
// Per structure the results equal a separate evaluation of that structure
// (the same neighbour entries in the same order, the same kernels); the
// reference has no batched entry point.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "batch.h"
#include "bop_math.h"

namespace gb {


cudaStream_t batch_stream(Batch &b) {
  if (!b.stream) {
    cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking);
    b.own_stream = true;
  }
  return b.stream;
}

// Element index of every atom for this potential (Z2db).
int batch_elements(Batch &b, Potential &pot, cudaStream_t s) {
  if (b.el_pot == &pot && b.el_geom == b.geom_rev && b.el.p) return 0;
  const int nel = pot_nel(pot);
  std::vector<int> el(std::max(b.nat, 1), -1);
  for (int i = 0; i < b.nat; i++)
    for (int q = 0; q < nel; q++)
      if (b.hZ[i] == pot_Z(pot, q)) el[i] = q;
  GB_CHECK(b.el.ensure(sizeof(int) * el.size()));
  GB_CUDA(cudaMemcpyAsync(b.el.p, el.data(), sizeof(int) * el.size(), cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  b.el_pot = &pot;
  b.el_geom = b.geom_rev;
  return 0;
}

// Interaction range: the largest r2 over the element pairs present
// (default_bind_to_func.f90:123-144).
double batch_cutoff(const Batch &b, const Potential &pot) {
  const std::vector<int> &zs = b.zu;
  const int nel = pot_nel(pot);
  auto dbidx = [&](int Z) {
    for (int q = 0; q < nel; q++)
      if (pot_Z(pot, q) == Z) return q;
    return -1;
  };
  double cut = 0.0;
  for (int zi : zs)
    for (int zj : zs) {
      const int ii = dbidx(zi), jj = dbidx(zj);
      if (ii < 0 || jj < 0) continue;
      const int t = pot_pair(pot, ii, jj);
      cut = std::max(cut, bop_pair_range(pot, t));
    }
  return cut;
}

// Per-structure binning parameters for the cutoff (cells numbered in
// structure order).
int batch_binning(Batch &b, double cutoff, cudaStream_t s) {
  if (b.built_geom == b.geom_rev && b.built_cutoff == cutoff) return 0;
  std::vector<BinParams> h(std::max(b.nstruct, 1));
  long long base = 0;
  for (int q = 0; q < b.nstruct; q++) {
    double A[3][3], B[3][3];
    std::memcpy(A, &b.A[9 * q], sizeof(A));
    std::memcpy(B, &b.B[9 * q], sizeof(B));
    GB_CHECK(bin_params(A, B, &b.pbc[3 * q], cutoff, (int)base, h[q]));
    base += (long long)h[q].n[0] * h[q].n[1] * h[q].n[2];
    if (base > (1ll << 28)) {
      set_error("batch: too many cells in total (cells or cutoff out of range)");
      return GB_ERROR_DOMAIN;
    }
  }
  GB_CHECK(b.bps.ensure(sizeof(BinParams) * h.size()));
  GB_CUDA(cudaMemcpyAsync(b.bps.p, h.data(), sizeof(BinParams) * h.size(),
                          cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  b.ncells = (int)base;
  b.built_geom = b.geom_rev;
  b.built_cutoff = cutoff;
  b.nl.valid = false;
  return 0;
}

// Uploads a tiling: tile_atom0 [nt + 1] | tile_struct [nt] | seg [nstruct + 1]
// | piece0 [np + 1] | seg_piece [nstruct + 1], where the pieces cut each
// structure's rows [seg[q], seg[q + 1]) into runs of at most 32 rows for the
// two-step per-structure sums.
int upload_tiles(Batch &b, const std::vector<int> &atom0, const std::vector<int> &strct,
                 const std::vector<int> &seg, cudaStream_t s) {
  const int nt = (int)strct.size();
  std::vector<int> piece0, seg_piece(b.nstruct + 1, 0);
  for (int q = 0; q < b.nstruct; q++) {
    seg_piece[q] = (int)piece0.size();
    for (int r = seg[q]; r < seg[q + 1]; r += 32) piece0.push_back(r);
  }
  seg_piece[b.nstruct] = (int)piece0.size();
  const int np = (int)piece0.size();
  piece0.push_back(nt);
  std::vector<int> all;
  all.reserve(atom0.size() + strct.size() + seg.size() + piece0.size() + seg_piece.size());
  const std::vector<int> *parts[] = {&atom0, &strct, &seg, &piece0, &seg_piece};
  for (const std::vector<int> *v : parts) all.insert(all.end(), v->begin(), v->end());
  GB_CHECK(b.tiles.ensure(sizeof(int) * all.size()));
  GB_CUDA(cudaMemcpyAsync(b.tiles.p, all.data(), sizeof(int) * all.size(),
                          cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  b.ntiles = nt;
  b.npiece = np;
  return 0;
}

// Tiles of at most apt atoms inside each structure; per-structure tile
// offsets for the energy/virial sums.
int batch_tiles(Batch &b, int apt, cudaStream_t s) {
  if (b.tiles_budget == 0 && b.tiles_apt == apt && b.tiles_nentries == b.nl.nentries &&
      b.ntiles > 0 && b.built_geom == b.geom_rev)
    return 0;
  std::vector<int> atom0, strct, seg(b.nstruct + 1, 0);
  for (int q = 0; q < b.nstruct; q++) {
    seg[q] = (int)strct.size();
    for (int a = b.atom_off[q]; a < b.atom_off[q + 1]; a += apt) {
      atom0.push_back(a);
      strct.push_back(q);
    }
  }
  seg[b.nstruct] = (int)strct.size();
  atom0.push_back(b.nat);
  GB_CHECK(upload_tiles(b, atom0, strct, seg, s));
  b.tiles_apt = apt;
  b.tiles_budget = 0;
  b.graph_geom = ~0ull;  // a captured graph holds the previous tiles: capture again
  b.tile_max_atoms = apt;
  b.tiles_nentries = b.nl.nentries;
  return 0;
}

// Tiles of the bond-order kernels, balanced by work: inside each structure,
// consecutive atoms join a tile while it keeps at most kMaxTileAtoms atoms,
// `budget` bonds and 6 budget (ij, ik) slots (a first atom always joins), so
// a tile's work matches the CTA's threads whatever the coordination (tiles
// of a fixed atom count leave threads idle where it is low and overflow
// shared memory where it is high).  The counts come from the list built
// last; the tiles are kept while the geometry is unchanged: any tiling is
// correct (every evaluation plans its exact per-tile maxima), only the
// balance depends on the counts.
int batch_tiles_work(Batch &b, int budget, cudaStream_t s, bool recut) {
  constexpr int kMaxTileAtoms = 64;
  if (!recut && b.tiles_budget == budget && b.tiles_geom == b.geom_rev && b.ntiles > 0) return 0;
  std::vector<int> seed(b.nat + 1, 0);
  if (b.nat > 0)
    GB_CUDA(cudaMemcpyAsync(seed.data(), b.nl.seed.p, sizeof(int) * (b.nat + 1),
                            cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  const int64_t tmax = 6 * (int64_t)budget;
  std::vector<int> atom0, strct, seg(b.nstruct + 1, 0);
  int most = 1;
  for (int q = 0; q < b.nstruct; q++) {
    seg[q] = (int)strct.size();
    int na = 0;
    int64_t nb = 0, nt = 0;
    for (int a = b.atom_off[q]; a < b.atom_off[q + 1]; a++) {
      const int64_t z = seed[a + 1] - seed[a];
      if (na > 0 && (na == kMaxTileAtoms || nb + z > budget ||
                     nt + trip_slots((int)z) > tmax)) {
        most = std::max(most, na);
        na = 0;
      }
      if (na == 0) {
        atom0.push_back(a);
        strct.push_back(q);
        nb = nt = 0;
      }
      na++;
      nb += z;
      nt += trip_slots((int)z);
    }
    if (na > 0) most = std::max(most, na);
  }
  seg[b.nstruct] = (int)strct.size();
  atom0.push_back(b.nat);
  GB_CHECK(upload_tiles(b, atom0, strct, seg, s));
  b.tiles_apt = budget;
  b.tiles_budget = budget;
  b.tile_max_atoms = most;
  b.tiles_geom = b.geom_rev;
  b.tiles_pos = b.built_pos;
  b.graph_geom = ~0ull;  // a captured graph holds the previous tiles: capture again
  b.tiles_nentries = b.nl.nentries;
  return 0;
}

Batch::~Batch() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
}

namespace {

// Velocity Verlet (verlet.f90:100-235): v += 0.5 f / m dt; r += v dt
// (step1) ... forces ... v += 0.5 f / m dt (step2).  Atoms with m <= 0 do
// not move (the reference's group filter p%g(i) > 0).
__global__ void md_kick_drift(int nat, double *__restrict__ r, double *__restrict__ v,
                              const double *__restrict__ f, const double *__restrict__ m,
                              double dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const double mi = m[i];
  if (!(mi > 0.0)) return;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double vv = v[3 * (size_t)i + c] + 0.5 * f[3 * (size_t)i + c] / mi * dt;
    v[3 * (size_t)i + c] = vv;
    r[3 * (size_t)i + c] = r[3 * (size_t)i + c] + vv * dt;
  }
}

// step2 with the new forces f, which also become the stored forces fout.
// nls / pst (captured steps): the list build's and the force kernels' status
// words; a step whose list or tile plan overflowed leaves v and fout as they
// are (the host redoes the evaluation).
__global__ void md_kick(int nat, double *__restrict__ v, const double *__restrict__ f,
                        const double *__restrict__ m, double dt, double *__restrict__ fout,
                        const int *__restrict__ nls, const int *__restrict__ pst, int cap) {
  if (nls && !(nls[0] <= cap && (nls[1] & 3) == 0 && (nls[4] & 4) == 0 && (pst[0] & 2) == 0))
    return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const double mi = m[i];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const double fc = f[3 * (size_t)i + c];
    if (mi > 0.0) v[3 * (size_t)i + c] = v[3 * (size_t)i + c] + 0.5 * fc / mi * dt;
    fout[3 * (size_t)i + c] = fc;
  }
}

void drop_graph(Batch &b) {
  if (b.graph_exec) cudaGraphExecDestroy(b.graph_exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.graph_exec = nullptr;
  b.graph = nullptr;
  b.graph_kernels = 0;
  b.graph_bufs.clear();
  b.graph_fout = nullptr;
}

// Device buffers a captured evaluation writes or reads (their addresses are
// baked into the graph).
std::vector<const void *> graph_buffers(const Batch &b, const Potential &pot) {
  const Neighbors &nl = b.nl;
  return {b.r.p, b.sid.p, b.bps.p, b.Acells.p, b.Acells_ff.p, b.tiles.p, b.red_seg.p, b.el.p,
          b.gf.p, b.hseg.p, b.md_v.p, b.md_m.p, b.md_f.p, nl.pos4.p, nl.posff.p, nl.atom_cell.p,
          nl.atom_wrap.p,
          nl.cell_count.p, nl.cell_start.p, nl.cell_atoms.p, nl.counts.p, nl.spos.p, nl.swrap.p,
          nl.seed.p, nl.nbr.p, nl.shift.p, nl.rev.p, nl.stage.p, nl.scan_tmp.p, nl.stats.p,
          nl.hstats.p, pot.bond_G.p, pot.bond_e.p, pot.tile_part.p, pot.red.p, pot.hred.p};
}

BopSystem batch_system(const Batch &b) {
  BopSystem sys;
  sys.nat = b.nat;
  const int *t = b.tiles.as<int>();
  sys.tile_atom0 = t;
  sys.tile_struct = t + b.ntiles + 1;
  sys.seg = t + 2 * b.ntiles + 1;
  sys.nseg = b.nstruct;
  sys.red_seg = b.red_seg.as<double>();
  sys.piece0 = t + 2 * b.ntiles + 1 + b.nstruct + 1;
  sys.seg_piece = sys.piece0 + b.npiece + 1;
  sys.npiece = b.npiece;
  sys.piece_sum = b.red_piece.as<double>();
  sys.Acells = b.Acells.as<double>();
  sys.Acells_ff = reinterpret_cast<const float2 *>(b.Acells_ff.p);
  sys.ntiles = b.ntiles;
  sys.apt = b.tiles_apt;
  sys.el = b.el.as<int>();
  return sys;
}

// Tile kernel, gather and per-structure sums into fdev (accumulated), then
// the per-structure rows and the status words to pinned host memory.
int batch_forces(Batch &b, Potential &pot, double *fdev, cudaStream_t s, BopSystem sys) {
  GB_CHECK(pot.red.ensure(sizeof(double) * 16));
  GB_CHECK(pot.hred.ensure(sizeof(double) * 16));
  GB_CHECK(b.red_seg.ensure(sizeof(double) * 10 * std::max(b.nstruct, 1)));
  GB_CHECK(b.red_piece.ensure(sizeof(double) * 10 * std::max(b.npiece, 1)));
  GB_CHECK(b.hseg.ensure(sizeof(double) * 10 * std::max(b.nstruct, 1) + 64));
  sys.red_seg = b.red_seg.as<double>();  // (allocated just now on the first call)
  sys.piece_sum = b.red_piece.as<double>();
  Outputs o;
  o.f = fdev;
  o.red = pot.red.as<double>();
  o.status = reinterpret_cast<int *>(o.red + 12);
  GB_CUDA(cudaMemsetAsync(o.status, 0, sizeof(int) * 4, s));
  GB_CHECK(bop_run(pot, sys, b.nl, o, false, false));
  GB_CUDA(cudaMemcpyAsync(b.hseg.p, b.red_seg.p, sizeof(double) * 10 * b.nstruct,
                          cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(pot.hred.p, o.red, sizeof(double) * 14, cudaMemcpyDeviceToHost, s));
  return 0;
}

// Device outputs of batch_finish: epot[q] = row q's energy, wpot[q] += its
// virial (rows of 10: energy, then the virial in Fortran order).
__global__ void seg_results(int nseg, const double *__restrict__ rows, double *__restrict__ epot,
                            double *__restrict__ wpot) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= 10 * nseg) return;
  const int q = k / 10, c = k % 10;
  if (c == 0)
    epot[q] = rows[k];
  else
    wpot[9 * (size_t)q + c - 1] += rows[k];
}

// epot set, wpot accumulated, per structure (as energy_and_forces).  Device
// arrays are written on the stream from the device rows (no host copy);
// host arrays from the page-locked copy of the rows.
int batch_finish(Batch &b, Potential &pot, double *epot, double *wpot, cudaStream_t s) {
  const double *hs = b.hseg.as<double>();
  const double *hr = pot.hred.as<double>();
  const int st = reinterpret_cast<const int *>(hr + 12)[0];
  pot.last_status = st;
  pot.last_hot = reinterpret_cast<const int *>(hr + 12)[2];
  pot.last_bonds = b.nl.nentries;
  if (st & 2) {
    set_error("Internal error: bond-order tile plan mismatch.");
    return GB_ERROR_UNSPECIFIED;
  }
  const bool ed = is_device_ptr(epot), wd = is_device_ptr(wpot);
  if (ed && wd) {
    seg_results<<<(10 * b.nstruct + 255) / 256, 256, 0, s>>>(b.nstruct, b.red_seg.as<double>(),
                                                             epot, wpot);
    note_launch();
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaStreamSynchronize(s));  // results complete on return, as for host arrays
    return 0;
  }
  std::vector<double> e(b.nstruct), w(9 * (size_t)b.nstruct);
  if (wd)
    GB_CUDA(cudaMemcpy(w.data(), wpot, sizeof(double) * w.size(), cudaMemcpyDeviceToHost));
  else
    std::memcpy(w.data(), wpot, sizeof(double) * w.size());
  for (int q = 0; q < b.nstruct; q++) {
    e[q] = hs[10 * q];
    for (int c = 0; c < 9; c++) w[9 * q + c] += hs[10 * q + 1 + c];
  }
  if (ed)
    GB_CUDA(cudaMemcpy(epot, e.data(), sizeof(double) * e.size(), cudaMemcpyHostToDevice));
  else
    std::memcpy(epot, e.data(), sizeof(double) * e.size());
  if (wd)
    GB_CUDA(cudaMemcpy(wpot, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice));
  else
    std::memcpy(wpot, w.data(), sizeof(double) * w.size());
  return 0;
}

// Bond budget per tile: the autotuned value when current, else one bond per
// thread of the mixed kernel (two per thread of the FP64 one).  Tuning times
// the force part for budgets 256, 192 and 128 on scratch forces and keeps
// the fastest.
int batch_choose_budget(Batch &b, Potential &pot, cudaStream_t s) {
  constexpr int kBudgets[3] = {256, 192, 128};
  const bool current = b.tuned_apt > 0 && b.tuned_geom == b.geom_rev && b.tuned_pot == &pot &&
                       b.tuned_prec == pot.precision;
  if (!b.autotune) return kBudgets[0];
  if (current) return b.tuned_apt;
  GB_CHECK(b.gf.ensure(sizeof(double) * 3 * std::max(b.nat, 1)));
  int best = kBudgets[0], ncand = 0;
  float best_ms = 0.0f;
  for (int budget : kBudgets) {
    GB_CHECK(batch_tiles_work(b, budget, s));
    GB_CUDA(cudaMemsetAsync(b.gf.p, 0, sizeof(double) * 3 * b.nat, s));
    float ms = 0.0f;
    for (int rep = 0; rep < 2; rep++) {  // the first run warms up
      GB_CUDA(cudaEventRecord(pot.ev[1], s));
      GB_CHECK(batch_forces(b, pot, b.gf.as<double>(), s, batch_system(b)));
      GB_CUDA(cudaEventRecord(pot.ev[2], s));
      GB_CUDA(cudaStreamSynchronize(s));
      GB_CUDA(cudaEventElapsedTime(&ms, pot.ev[1], pot.ev[2]));
    }
    ncand++;
    if (ncand == 1 || ms < best_ms) {
      best_ms = ms;
      best = budget;
    }
  }
  b.tuned_apt = best;
  b.tuned_geom = b.geom_rev;
  b.tuned_pot = &pot;
  b.tuned_prec = pot.precision;
  b.tune_candidates = ncand;
  return best;
}

// Captures the whole evaluation (list build included) after an eager one
// has sized everything; failures leave the eager path in use.
// kind 0: one evaluation into gf; kind 1: a whole velocity-Verlet step of
// time step dt (step1, gf = 0, evaluation, checked step2 into md_v / md_f).
void batch_capture(Batch &b, Potential &pot, cudaStream_t s, int kind = 0, double dt = 0.0,
                   double *fcall = nullptr) {
  drop_graph(b);
  const int cap = b.nl.stage_cap;
  if (cap <= 0 || b.nat == 0) return;
  const int64_t capacity = (int64_t)b.nat * cap;
  // Tile plan with head room for the next configurations (checked per tile
  // by the kernel): as much as fits without fewer resident CTAs per SM than
  // the exact plan of this evaluation, at most +25 % bonds / +50 % slots.
  const int apt = b.tile_max_atoms;  // most atoms in one tile
  const int nbt0 = pot.last_plan[0], ntrip0 = pot.last_plan[1];
  if (nbt0 == 0) return;
  const bool mixed = pot.precision == GB_PRECISION_MIXED;
  const int occ0 = bop_tile_ctas_per_sm(pot, bop_tile_smem(mixed, nbt0, ntrip0));
  int max_nbt = nbt0, max_ntrip = ntrip0;
  for (int step = 16; step >= 1; step--) {  // head room step/16 of the maxima
    const int nb = std::min(apt * cap, nbt0 + nbt0 * step / 64 + step);
    const int nt = std::min(apt * trip_slots(cap), ntrip0 + ntrip0 * step / 32 + 4 * step);
    const size_t sm = bop_tile_smem(mixed, nb, nt);
    if (sm <= bop_tile_smem_budget() && bop_tile_ctas_per_sm(pot, sm) >= occ0) {
      max_nbt = nb;
      max_ntrip = nt;
      break;
    }
  }
  Neighbors &nl = b.nl;
  // a list array that grows here loses the eager call's list: rebuild it next
  const void *list0[3] = {nl.nbr.p, nl.shift.p, nl.rev.p};
  const bool grew = nl.nbr.ensure(sizeof(int) * capacity) ||
                    nl.shift.ensure(sizeof(int) * capacity) ||
                    nl.rev.ensure(sizeof(int) * capacity);
  if (nl.nbr.p != list0[0] || nl.shift.p != list0[1] || nl.rev.p != list0[2]) {
    nl.valid = false;
    nl.rev_valid = false;
  }
  if (grew || nl.stage.ensure(sizeof(int2) * capacity) ||
      pot.bond_G.ensure(sizeof(double) * 3 * capacity) ||
      pot.bond_e.ensure(sizeof(double) * capacity) ||
      pot.tile_part.ensure(sizeof(double) * 10 * b.ntiles + 64) ||
      b.gf.ensure(sizeof(double) * 3 * b.nat)) {
    clear_error();
    return;
  }
  // One evaluation for a device force array: the graph's gather adds into
  // that array, and only when the replay is valid (the gather checks the
  // list build's and the tile kernel's status words on the device), so an
  // overflowed replay leaves the caller's forces untouched.
  double *fout = b.gf.as<double>();
  b.graph_fout = nullptr;
  BopSystem sys = batch_system(b);
  if (kind == 0 && fcall && !b.graph_direct_off && is_device_ptr(fcall) &&
      !pot.red.ensure(sizeof(double) * 16)) {
    fout = fcall;
    b.graph_fout = fcall;
    sys.check.nl = nl.stats.as<int>();
    sys.check.tile = reinterpret_cast<int *>(pot.red.as<double>() + 12);
    sys.check.cap = cap;
  }
  clear_error();
  sys.capture = true;
  sys.nb_capacity = capacity;
  sys.max_nbt = max_nbt;
  sys.max_ntrip = max_ntrip;
  // Capturing runs nothing: the list, reverse index and ff positions of the
  // eager evaluation stay valid on the device; restore their flags after.
  const bool rev_valid0 = nl.rev_valid, posff_valid0 = nl.posff_valid;
  const int plan0[2] = {pot.last_plan[0], pot.last_plan[1]};
  nl.rev_valid = false;
  nl.rev_pending = false;
  nl.posff_valid = nl.want_posff;
  const uint64_t launches0 = gb_kernel_launches();
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  BinParams dummy{};
  const int T = 256, nbk = (b.nat + T - 1) / T;
  int rc = 0;
  if (kind == 1) {
    md_kick_drift<<<nbk, T, 0, s>>>(b.nat, b.r.as<double>(), b.md_v.as<double>(),
                                    b.md_f.as<double>(), b.md_m.as<double>(), dt);
    note_launch();
    if (cudaMemsetAsync(b.gf.p, 0, sizeof(double) * 3 * b.nat, s) != cudaSuccess) rc = -1;
  }
  if (rc == 0)
    rc = nl_build(nl, b.nat, b.r.as<double>(), dummy, b.bps.as<BinParams>(), b.sid.as<int>(),
                  b.ncells, s, true);
  if (rc == 0) rc = batch_forces(b, pot, fout, s, sys);
  if (rc == 0 && kind == 1) {
    md_kick<<<nbk, T, 0, s>>>(b.nat, b.md_v.as<double>(), b.gf.as<double>(), b.md_m.as<double>(),
                              dt, b.md_f.as<double>(), nl.stats.as<int>(),
                              reinterpret_cast<const int *>(pot.red.as<double>() + 12), cap);
    note_launch();
  }
  const cudaError_t ce = cudaStreamEndCapture(s, &g);
  note_launch(-(int)(gb_kernel_launches() - launches0));  // captured, not run
  nl.rev_valid = rev_valid0;
  nl.rev_pending = false;
  nl.posff_valid = posff_valid0;
  pot.last_plan[0] = plan0[0];
  pot.last_plan[1] = plan0[1];
  if (rc != 0 || ce != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    clear_error();
    b.graph_failed = true;
    return;
  }
  cudaGraphExec_t x = nullptr;
  if (cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
    cudaGraphDestroy(g);
    cudaGetLastError();
    b.graph_failed = true;
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
  b.graph = g;
  b.graph_exec = x;
  b.graph_kernels = kernels;
  b.graph_geom = b.geom_rev;
  b.graph_pot = &pot;
  b.graph_prec = pot.precision;
  b.graph_apt = b.tiles_apt;
  b.graph_cap = cap;
  b.graph_ncells = b.ncells;
  b.graph_kind = kind;
  b.graph_dt = dt;
  b.graph_bufs = graph_buffers(b, pot);
  (void)mixed;
}

bool graph_current(const Batch &b, const Potential &pot, int kind = 0, double dt = 0.0) {
  return b.graph_exec && b.graph_kind == kind && (kind == 0 || b.graph_dt == dt) &&
         b.graph_geom == b.geom_rev && b.graph_pot == &pot &&
         b.graph_prec == pot.precision && b.graph_apt == b.tiles_apt &&
         b.graph_ncells == b.ncells &&
         b.graph_bufs == graph_buffers(b, pot);
}

// Replays the graph; true when its results are valid (no capacity, plan or
// list problem), in which case the caller's outputs are written.
int batch_replay(Batch &b, Potential &pot, double *epot, double *f, double *wpot,
                 cudaStream_t s, bool &done) {
  done = false;
  const size_t nf = 3 * (size_t)b.nat;
  const bool direct = b.graph_fout != nullptr;
  if (direct && f != b.graph_fout) {
    // another force array: this graph would add into the old one
    drop_graph(b);
    b.graph_direct_off = true;
    return 0;
  }
  if (!direct)
    GB_CUDA(cudaMemcpyAsync(b.gf.p, f, sizeof(double) * nf, cudaMemcpyDefault, s));
  GB_CUDA(cudaGraphLaunch(b.graph_exec, s));
  GB_CUDA(cudaStreamSynchronize(s));
  note_launch(b.graph_kernels);
  const int *hs = b.nl.hstats.as<int>();
  const int *st = reinterpret_cast<const int *>(pot.hred.as<double>() + 12);
  const bool ok = hs[0] <= b.graph_cap && (hs[1] & (1 | 2 | 8)) == 0 && (hs[5] & 4) == 0 &&
                  (st[0] & 2) == 0;
  if (!ok) {
    drop_graph(b);
    b.nl.valid = false;
    return 0;
  }
  b.nl.nentries = hs[4];
  b.nl.maxz = hs[0];
  b.nl.valid = true;
  b.nl.rev_valid = true;
  b.nl.rev_pending = false;
  b.nl.posff_valid = b.nl.want_posff;
  b.built_pos = b.pos_rev;
  if (!direct) GB_CUDA(cudaMemcpy(f, b.gf.p, sizeof(double) * nf, cudaMemcpyDefault));
  GB_CHECK(batch_finish(b, pot, epot, wpot, s));
  done = true;
  return 0;
}

// Checks, stream order, elements, cutoff and binning of an evaluation.
int batch_prepare(Batch &b, Potential &pot, cudaStream_t &s, double &cutoff) {
  if (pot.kind == kEAM || pot.screened) {
    set_error("batch_energy_and_forces: batches support the non-screened bond-order potentials");
    return GB_ERROR_ARGUMENT;
  }
  if (b.nat > 0 && !b.r.p) {
    set_error("batch_energy_and_forces: positions not set");
    return GB_ERROR_ARGUMENT;
  }
  s = pot_stream(pot);
  if (b.stream && b.stream != s) {
    GB_CUDA(cudaEventRecord(pot.ev[3], b.stream));
    GB_CUDA(cudaStreamWaitEvent(s, pot.ev[3], 0));
  }
  GB_CUDA(cudaEventRecord(pot.ev[0], s));
  GB_CHECK(batch_elements(b, pot, s));
  cutoff = batch_cutoff(b, pot);
  if (!(cutoff > 0.0)) {
    set_error("batch_energy_and_forces: no element of the batch is known to the potential");
    return GB_ERROR_ARGUMENT;
  }
  GB_CHECK(batch_binning(b, cutoff, s));
  if (pot.precision == GB_PRECISION_MIXED) b.nl.want_posff = true;
  b.nl.want_rev = true;  // the compaction also builds the reverse index
  return 0;
}

// One evaluation without graphs: list (if the positions changed), tiles,
// forces accumulated into f, energies set / virials accumulated.
int batch_eager(Batch &b, Potential &pot, double *epot, double *f, double *wpot, cudaStream_t s,
                double cutoff) {
  if (!(b.nl.valid && b.built_pos == b.pos_rev && b.nl.posff_valid == b.nl.want_posff)) {
    b.nl.valid = false;
    b.nl.rev_valid = false;
    b.nl.rev_pending = false;
    BinParams dummy{};
    GB_CHECK(nl_build(b.nl, b.nat, b.r.as<double>(), dummy, b.bps.as<BinParams>(),
                      b.sid.as<int>(), b.ncells, s));
    b.nl.cutoff = cutoff;
    b.nl.valid = true;
    b.built_pos = b.pos_rev;
  }
  GB_CUDA(cudaEventRecord(pot.ev[1], s));
  const int budget = batch_choose_budget(b, pot, s);
  GB_CHECK(batch_tiles_work(b, budget, s));
  const size_t nf = 3 * (size_t)b.nat;
  double *fd = f;
  const bool f_host = b.nat > 0 && !is_device_ptr(f);
  if (f_host) {
    GB_CHECK(pot.out_f.ensure(sizeof(double) * std::max<size_t>(nf, 1)));
    fd = pot.out_f.as<double>();
    GB_CUDA(cudaMemcpyAsync(fd, f, sizeof(double) * nf, cudaMemcpyHostToDevice, s));
  }
  int rc = batch_forces(b, pot, fd, s, batch_system(b));
  if (rc == GB_ERROR_CAPACITY && b.tiles_pos != b.built_pos) {
    // tiles cut for other positions (e.g. before a compression) no longer
    // fit: cut them again from this list (the failed call changed no output)
    clear_error();
    GB_CHECK(batch_tiles_work(b, budget, s, true));
    rc = batch_forces(b, pot, fd, s, batch_system(b));
  }
  GB_CHECK(rc);
  GB_CUDA(cudaEventRecord(pot.ev[2], s));
  if (f_host) GB_CUDA(cudaMemcpyAsync(f, fd, sizeof(double) * nf, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaEventRecord(pot.ev[3], s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaGetLastError());
  float ms[4] = {0, 0, 0, 0};
  cudaEventElapsedTime(&ms[0], pot.ev[0], pot.ev[1]);
  cudaEventElapsedTime(&ms[1], pot.ev[1], pot.ev[2]);
  cudaEventElapsedTime(&ms[2], pot.ev[0], pot.ev[3]);
  cudaEventElapsedTime(&ms[3], pot.kev[0], pot.kev[1]);
  cudaGetLastError();
  for (int q = 0; q < 4; q++) pot.timing[q] = ms[q];
  GB_CHECK(batch_finish(b, pot, epot, wpot, s));
  b.info[1] = b.tiles_apt;
  b.info[3] = b.tune_candidates;
  return 0;
}

// Replays a captured velocity-Verlet step; ok = false when its list or tile
// plan overflowed (positions and the first half kick are applied, the second
// half kick is not: the caller redoes the evaluation).
int batch_replay_md(Batch &b, Potential &pot, cudaStream_t s, bool &ok) {
  GB_CUDA(cudaGraphLaunch(b.graph_exec, s));
  GB_CUDA(cudaStreamSynchronize(s));
  note_launch(b.graph_kernels);
  b.pos_rev++;  // the step moved the atoms
  const int *hs = b.nl.hstats.as<int>();
  const int *st = reinterpret_cast<const int *>(pot.hred.as<double>() + 12);
  ok = hs[0] <= b.graph_cap && (hs[1] & (1 | 2 | 8)) == 0 && (hs[5] & 4) == 0 &&
       (st[0] & 2) == 0;
  if (!ok) {
    drop_graph(b);
    b.nl.valid = false;
    return 0;
  }
  b.nl.nentries = hs[4];
  b.nl.maxz = hs[0];
  b.nl.valid = true;
  b.nl.rev_valid = true;
  b.nl.rev_pending = false;
  b.nl.posff_valid = b.nl.want_posff;
  b.built_pos = b.pos_rev;
  b.md_f_pos = b.pos_rev;
  return 0;
}

}  // namespace

int batch_energy_and_forces(Batch &b, Potential &pot, double *epot, double *f, double *wpot) {
  if (!epot || !f || !wpot) {
    set_error("batch_energy_and_forces: epot, f and wpot are required");
    return GB_ERROR_ARGUMENT;
  }
  b.info[0] = 0;
  if (b.nstruct == 0) return 0;
  cudaStream_t s;
  double cutoff;
  GB_CHECK(batch_prepare(b, pot, s, cutoff));
  if (b.use_graph && graph_current(b, pot)) {
    bool done = false;
    GB_CHECK(batch_replay(b, pot, epot, f, wpot, s, done));
    if (done) {
      b.info[0] = 1;
      b.info[1] = b.tiles_apt;
      b.info[2] = b.graph_kernels;
      return 0;
    }
  }
  GB_CHECK(batch_eager(b, pot, epot, f, wpot, s, cutoff));
  if (b.use_graph && !b.graph_failed && !graph_current(b, pot)) batch_capture(b, pot, s, 0, 0.0, f);
  b.info[2] = b.graph_kernels;
  return 0;
}

// nsteps velocity-Verlet steps of time step dt; epot / wpot (per structure,
// optional) of the last step.  With graphs on, a step after the first eager
// one is captured whole and replayed.
int batch_md_run(Batch &b, Potential &pot, double dt, int nsteps, double *epot, double *wpot) {
  if (nsteps < 0 || !(dt == dt)) {
    set_error("md_run: nsteps >= 0 and a finite dt are required");
    return GB_ERROR_ARGUMENT;
  }
  if (b.nstruct == 0 || b.nat == 0) return 0;
  if (!b.md_v.p || !b.md_m.p) {
    set_error("md_run: velocities and masses not set (gb_batch_md_set_state)");
    return GB_ERROR_ARGUMENT;
  }
  cudaStream_t s;
  double cutoff;
  GB_CHECK(batch_prepare(b, pot, s, cutoff));
  const size_t nf = 3 * (size_t)b.nat;
  GB_CHECK(b.gf.ensure(sizeof(double) * nf));
  GB_CHECK(b.md_f.ensure(sizeof(double) * nf));
  b.md_e.assign(b.nstruct, 0.0);
  b.md_w.assign(9 * (size_t)b.nstruct, 0.0);
  const int T = 256, nbk = (b.nat + T - 1) / T;
  auto eval_into_md_f = [&](bool kick) -> int {
    // forces at the current positions into gf, then (kick) step2 and md_f
    GB_CUDA(cudaMemsetAsync(b.gf.p, 0, sizeof(double) * nf, s));
    std::fill(b.md_w.begin(), b.md_w.end(), 0.0);
    GB_CHECK(batch_eager(b, pot, b.md_e.data(), b.gf.as<double>(), b.md_w.data(), s, cutoff));
    if (kick) {
      md_kick<<<nbk, T, 0, s>>>(b.nat, b.md_v.as<double>(), b.gf.as<double>(),
                                b.md_m.as<double>(), dt, b.md_f.as<double>(), nullptr, nullptr, 0);
      note_launch();
    } else {
      GB_CUDA(cudaMemcpyAsync(b.md_f.p, b.gf.p, sizeof(double) * nf, cudaMemcpyDeviceToDevice, s));
    }
    GB_CUDA(cudaStreamSynchronize(s));
    GB_CUDA(cudaGetLastError());
    b.md_f_pos = b.pos_rev;
    return 0;
  };
  if (b.md_f_pos != b.pos_rev) GB_CHECK(eval_into_md_f(false));  // forces at the start
  b.info[0] = 0;
  for (int step = 0; step < nsteps; step++) {
    if (b.use_graph && graph_current(b, pot, 1, dt)) {
      bool ok = false;
      GB_CHECK(batch_replay_md(b, pot, s, ok));
      if (ok) {
        std::fill(b.md_w.begin(), b.md_w.end(), 0.0);
        GB_CHECK(batch_finish(b, pot, b.md_e.data(), b.md_w.data(), s));
        b.info[0] = 1;
        continue;
      }
      GB_CHECK(eval_into_md_f(true));  // an overflowed replay: the evaluation again
      continue;
    }
    md_kick_drift<<<nbk, T, 0, s>>>(b.nat, b.r.as<double>(), b.md_v.as<double>(),
                                    b.md_f.as<double>(), b.md_m.as<double>(), dt);
    note_launch();
    b.pos_rev++;
    GB_CHECK(eval_into_md_f(true));
    if (b.use_graph && !b.graph_failed) batch_capture(b, pot, s, 1, dt);
  }
  b.info[2] = b.graph_kernels;
  if (epot) {
    if (is_device_ptr(epot))
      GB_CUDA(cudaMemcpy(epot, b.md_e.data(), sizeof(double) * b.nstruct, cudaMemcpyHostToDevice));
    else
      std::memcpy(epot, b.md_e.data(), sizeof(double) * b.nstruct);
  }
  if (wpot) {
    if (is_device_ptr(wpot))
      GB_CUDA(cudaMemcpy(wpot, b.md_w.data(), sizeof(double) * b.md_w.size(),
                         cudaMemcpyHostToDevice));
    else
      std::memcpy(wpot, b.md_w.data(), sizeof(double) * b.md_w.size());
  }
  return 0;
}

}  // namespace gb

// ===========================================================================
// C-ABI.
// ===========================================================================
using namespace gb;

extern "C" {

int gb_batch_new(gb_batch_t **out) {
  clear_error();
  if (!out) return GB_ERROR_ARGUMENT;
  *out = new gb_batch;
  return 0;
}

void gb_batch_free(gb_batch_t *h) {
  if (!h) return;
  if (h->b.own_stream && h->b.stream) cudaStreamDestroy(h->b.stream);
  delete h;
}

int gb_batch_set_stream(gb_batch_t *h, void *stream) {
  if (!h) return GB_ERROR_ARGUMENT;
  if (h->b.own_stream && h->b.stream) cudaStreamDestroy(h->b.stream);
  h->b.stream = static_cast<cudaStream_t>(stream);
  h->b.own_stream = false;
  return 0;
}

int gb_batch_set_structures(gb_batch_t *h, int nstruct, const int *nat, const double *cells,
                            const int *pbc, const int *Z) {
  clear_error();
  if (!h || nstruct < 0 || (nstruct > 0 && (!nat || !cells))) return GB_ERROR_ARGUMENT;
  Batch &b = h->b;
  std::vector<int> off(nstruct + 1, 0);
  for (int q = 0; q < nstruct; q++) {
    if (nat[q] < 0) {
      set_error("batch: negative atom count");
      return GB_ERROR_ARGUMENT;
    }
    off[q + 1] = off[q] + nat[q];
  }
  const int total = off[nstruct];
  if (total > 0 && !Z) return GB_ERROR_ARGUMENT;
  std::vector<double> A(9 * (size_t)nstruct), B(9 * (size_t)nstruct);
  std::vector<int> pb(3 * (size_t)nstruct, 1);
  for (int q = 0; q < nstruct; q++) {
    double a[3][3], bi[3][3];
    // cells: per structure 3 rows = lattice vectors (C layout), A[a][k] = cell[k][a]
    for (int x = 0; x < 3; x++)
      for (int k = 0; k < 3; k++) a[x][k] = cells[9 * (size_t)q + 3 * k + x];
    if (cell_inverse(a, bi) != 0) {
      set_error("Gauss elimination failed (singular cell) for structure " + std::to_string(q));
      return GB_ERROR_ARGUMENT;
    }
    std::memcpy(&A[9 * (size_t)q], a, sizeof(a));
    std::memcpy(&B[9 * (size_t)q], bi, sizeof(bi));
    if (pbc)
      for (int k = 0; k < 3; k++) pb[3 * (size_t)q + k] = pbc[3 * (size_t)q + k] != 0;
  }
  cudaStream_t s = batch_stream(b);
  std::vector<int> sid(std::max(total, 1), 0);
  for (int q = 0; q < nstruct; q++)
    for (int i = off[q]; i < off[q + 1]; i++) sid[i] = q;
  std::vector<float2> aff(9 * (size_t)std::max(nstruct, 1));
  for (size_t k = 0; k < A.size(); k++) {
    const float hi = (float)A[k];
    aff[k] = make_float2(hi, (float)(A[k] - (double)hi));
  }
  GB_CHECK(b.sid.ensure(sizeof(int) * sid.size()));
  GB_CHECK(b.Acells.ensure(sizeof(double) * std::max<size_t>(A.size(), 9)));
  GB_CHECK(b.Acells_ff.ensure(sizeof(float2) * aff.size()));
  GB_CHECK(b.r.ensure(sizeof(double) * 3 * std::max(total, 1)));
  GB_CUDA(cudaMemcpyAsync(b.sid.p, sid.data(), sizeof(int) * sid.size(), cudaMemcpyHostToDevice,
                          s));
  if (!A.empty())
    GB_CUDA(cudaMemcpyAsync(b.Acells.p, A.data(), sizeof(double) * A.size(),
                            cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaMemcpyAsync(b.Acells_ff.p, aff.data(), sizeof(float2) * aff.size(),
                          cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  b.nstruct = nstruct;
  b.nat = total;
  b.atom_off = off;
  b.A = A;
  b.B = B;
  b.pbc = pb;
  b.hZ.assign(Z ? Z : nullptr, Z ? Z + total : nullptr);
  b.zu = b.hZ;
  std::sort(b.zu.begin(), b.zu.end());
  b.zu.erase(std::unique(b.zu.begin(), b.zu.end()), b.zu.end());
  b.geom_rev++;
  b.pos_rev++;
  b.nl.valid = false;
  b.ntiles = 0;
  return 0;
}

int gb_batch_set_positions(gb_batch_t *h, const double *r) {
  clear_error();
  if (!h || (!r && h->b.nat > 0)) return GB_ERROR_ARGUMENT;
  Batch &b = h->b;
  if (b.nat > 0) {
    cudaStream_t s = batch_stream(b);
    GB_CUDA(cudaMemcpyAsync(b.r.p, r, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
    if (!is_device_ptr(r)) GB_CUDA(cudaStreamSynchronize(s));
  }
  b.pos_rev++;
  return 0;
}

int gb_batch_get_nat(const gb_batch_t *h) { return h ? h->b.nat : -1; }

int gb_batch_set_options(gb_batch_t *h, int use_graph, int autotune) {
  if (!h) return GB_ERROR_ARGUMENT;
  Batch &b = h->b;
  b.use_graph = use_graph != 0;
  b.autotune = autotune != 0;
  b.graph_failed = false;
  if (!b.use_graph) drop_graph(b);
  if (!b.autotune) b.tuned_apt = 0;
  return 0;
}

int gb_batch_last_info(const gb_batch_t *h, int64_t *info) {
  if (!h || !info) return GB_ERROR_ARGUMENT;
  for (int k = 0; k < 4; k++) info[k] = h->b.info[k];
  return 0;
}

int gb_batch_md_set_state(gb_batch_t *h, const double *v, const double *m) {
  clear_error();
  if (!h || (h->b.nat > 0 && (!v || !m))) return GB_ERROR_ARGUMENT;
  Batch &b = h->b;
  const size_t n = (size_t)std::max(b.nat, 1);
  GB_CHECK(b.md_v.ensure(sizeof(double) * 3 * n));
  GB_CHECK(b.md_m.ensure(sizeof(double) * n));
  if (b.nat > 0) {
    cudaStream_t s = batch_stream(b);
    GB_CUDA(cudaMemcpyAsync(b.md_v.p, v, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
    GB_CUDA(cudaMemcpyAsync(b.md_m.p, m, sizeof(double) * b.nat, cudaMemcpyDefault, s));
    GB_CUDA(cudaStreamSynchronize(s));
  }
  b.md_f_pos = ~0ull;  // forces are recomputed at the next md_run
  return 0;
}

int gb_batch_md_get_state(gb_batch_t *h, double *r, double *v, double *f) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  Batch &b = h->b;
  if (b.nat == 0) return 0;
  const size_t nb = sizeof(double) * 3 * b.nat;
  if (r) GB_CUDA(cudaMemcpy(r, b.r.p, nb, cudaMemcpyDefault));
  if (v) {
    if (!b.md_v.p) return GB_ERROR_ARGUMENT;
    GB_CUDA(cudaMemcpy(v, b.md_v.p, nb, cudaMemcpyDefault));
  }
  if (f) {
    if (!b.md_f.p || b.md_f_pos != b.pos_rev) {
      set_error("md_get_state: no forces at the current positions (run md_run first)");
      return GB_ERROR_ARGUMENT;
    }
    GB_CUDA(cudaMemcpy(f, b.md_f.p, nb, cudaMemcpyDefault));
  }
  return 0;
}

int gb_batch_md_run(gb_batch_t *h, gb_potential_t *pot, double dt, int nsteps, double *epot,
                    double *wpot) {
  clear_error();
  if (!h || !pot) return GB_ERROR_ARGUMENT;
  return batch_md_run(h->b, pot->pot, dt, nsteps, epot, wpot);
}

int gb_batch_energy_and_forces(gb_batch_t *h, gb_potential_t *pot, double *epot, double *f,
                               double *wpot) {
  clear_error();
  if (!h || !pot) return GB_ERROR_ARGUMENT;
  return batch_energy_and_forces(h->b, pot->pot, epot, f, wpot);
}

}  // extern "C"
