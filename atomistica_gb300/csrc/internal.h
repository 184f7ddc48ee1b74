// Internal types shared by the CUDA translation units of libatomistica_gb300.
// Nothing here crosses the C-ABI; the public surface is include/atomistica_gb300.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/atomistica_gb300.h"

namespace gb {

// ---------------------------------------------------------------------------
// Error state.  The C-ABI returns an int code (error.f90:81-86 convention:
// 0 = none, negative = error) and keeps the message in a thread-local buffer.
// ---------------------------------------------------------------------------
void set_error(const std::string &msg);
void clear_error();

#define GB_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      ::gb::set_error(std::string("CUDA error in " #call ": ") +                   \
                      cudaGetErrorString(e_));                                     \
      return GB_ERROR_CUDA;                                                        \
    }                                                                              \
  } while (0)

#define GB_CHECK(expr)        \
  do {                        \
    int rc_ = (expr);         \
    if (rc_ != 0) return rc_; \
  } while (0)

// Growable device buffer (grows, never shrinks — like the reference's
// internal neighbour buffers, bop_kernel.f90:307-414).
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);
  void release();
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
  ~DevBuf() { release(); }
};

// Pinned host staging buffer.
struct HostBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);
  void release();
  template <class T>
  T *as() const {
    return reinterpret_cast<T *>(p);
  }
  ~HostBuf() { release(); }
};

// Host-side count of kernel launches issued by this library (diagnostics).
void note_launch(int n = 1);

// Does the pointer refer to device (or managed) memory?
bool is_device_ptr(const void *ptr);
// The device address of page-locked host memory that kernels may access
// directly (mapped, as every page-locked allocation is under unified
// addressing), or nullptr for other memory.
double *mapped_host_ptr(void *ptr);

// ---------------------------------------------------------------------------
// Particles (python_particles.f90:85-140, set_cell :286-346).
// ---------------------------------------------------------------------------
struct Particles {
  int nat = 0;
  double A[3][3] = {{0}};  // A[a][k] = Abox(a,k): column k = lattice vector k
  double B[3][3] = {{0}};  // Bbox = A^-1 (Gauss elimination, gauss() order)
  int pbc[3] = {1, 1, 1};
  bool cell_set = false;
  uint64_t pos_rev = 0, cell_rev = 0, z_rev = 0;
  DevBuf r;      // double[3*nat], caller layout (nat,3)
  DevBuf Z;      // int[nat]
  std::vector<int> hZ;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
};

// Packed integer image shift: three 10-bit signed fields (range +-511).
__host__ __device__ inline int32_t pack_shift(int s0, int s1, int s2) {
  return (int32_t)((uint32_t)(s0 + 512) | ((uint32_t)(s1 + 512) << 10) |
                   ((uint32_t)(s2 + 512) << 20));
}
__host__ __device__ inline void unpack_shift(int32_t p, int &s0, int &s1, int &s2) {
  uint32_t u = (uint32_t)p;
  s0 = (int)(u & 1023u) - 512;
  s1 = (int)((u >> 10) & 1023u) - 512;
  s2 = (int)((u >> 20) & 1023u) - 512;
}
constexpr int kMaxShift = 511;

// Validity of a replayed (CUDA-graph) evaluation, read on the device by the
// kernels that write the caller's outputs: nl = the list build's status words
// (nl[0] largest coordination, nl[1] flags, nl[4] reverse-index flags), tile
// = the force kernels' status word, cap = the captured per-atom capacity.
// nl == nullptr: no check.
struct ReplayCheck {
  const int *nl = nullptr;
  const int *tile = nullptr;
  int cap = 0;
};
__device__ __forceinline__ bool replay_invalid(const ReplayCheck &c) {
  return c.nl && !(c.nl[0] <= c.cap && (c.nl[1] & (1 | 2 | 8)) == 0 && (c.nl[4] & 4) == 0 &&
                   (c.tile[0] & 2) == 0);
}

// 1/sqrt(x) to about an ulp: the hardware reciprocal square root refined by
// one Newton step, y (1 + (1/2 - x/2 y^2)).
__device__ __forceinline__ double rsqrt_refined(double x) {
  const double y = rsqrt(x);
  const double e = fma(-0.5 * x * y, y, 0.5);
  return fma(y, e, y);
}
// sqrt(x) from y = rsqrt_refined(x): s = x y and one correction with the
// residual x - s^2 computed by an FMA (Markstein's method); it equals the
// correctly rounded square root for every argument the tests draw (see
// gb_diag_sqrt_check), so a kernel that needs both sqrt(x) and 1/sqrt(x)
// pays for one hardware approximation.
__device__ __forceinline__ double sqrt_from_rsqrt(double x, double y) {
  const double s = x * y;
  const double e = fma(-s, s, x);
  return fma(e, 0.5 * y, s);
}

// A block's per-atom forces (3 doubles per atom; atom blockIdx.x * kThreads +
// threadIdx.x) written out through shared memory, so that consecutive
// threads store consecutive doubles: coalesced lines in device memory, and
// whole lines over the host link when f is page-locked host memory.  fset:
// written, else accumulated into.  Every thread of the block takes part.
template <int kThreads>
__device__ __forceinline__ void store_block_forces(double *__restrict__ f, int nat,
                                                   const double F[3], int fset) {
  __shared__ double sf[3 * kThreads];
  const int t = threadIdx.x;
  const int a0 = blockIdx.x * kThreads;
  sf[3 * t] = F[0];
  sf[3 * t + 1] = F[1];
  sf[3 * t + 2] = F[2];
  __syncthreads();
  const int n = 3 * (nat - a0 < kThreads ? nat - a0 : kThreads);
  for (int k = t; k < n; k += kThreads) {
    const size_t q = 3 * (size_t)a0 + k;
    if (fset)
      f[q] = sf[k];
    else
      f[q] += sf[k];
  }
}

// (ij, ik) slots of an atom with z bonds in the bond-order tile kernels: its
// z x z block, one slot longer for even z > 0, so that consecutive atoms'
// blocks start an odd number of slots apart and the rows that a warp's
// lanes write and read at one time (several atoms at once) fall into
// different shared-memory banks.
#ifndef GB_TRIP_PAD
#define GB_TRIP_PAD 1
#endif
__host__ __device__ __forceinline__ int trip_slots(int z) {
  return z * z + ((GB_TRIP_PAD && z > 0 && !(z & 1)) ? 1 : 0);
}
// Largest staging buffer of the single-pass neighbour build (bytes).
constexpr size_t kStageMaxBytes = size_t(2) << 30;

// Binning and pair-search parameters of one periodic cell.
struct BinParams {
  double rec[3][3];
  float recf[3][3];  // rec rounded to float (cell prefilter)
  double A[3][3];
  float Af[3][3];  // A rounded to float, and max |A_ak|
  float Amax;
  int n[3];
  int pbc[3];
  int dx, dy, dz;
  int cell_base;  // first cell of this structure in a batch (0 otherwise)
  double cutoff_sq;
  float cutoff_f;                    // cutoff rounded up to float
  float cutoff_sq_lo, cutoff_sq_hi;  // float bracket of cutoff^2
};

// Position padded to 32 bytes: one DRAM sector per gather.
struct __align__(32) Pos4 {
  double x, y, z, w;
};

struct Cell {
  double A[3][3];
  int pbc[3];
};

// ---------------------------------------------------------------------------
// Neighbour list (python_neighbors.f90:51-139) — full directed CSR with
// per-entry image shifts, rebuilt when positions or cell changed.
// ---------------------------------------------------------------------------
struct Neighbors {
  int avgn = 100;
  double interaction_range = 0.0;
  double cutoff = 0.0;
  bool valid = false;
  const Particles *built_for = nullptr;
  uint64_t built_pos_rev = ~0ull, built_cell_rev = ~0ull;
  int built_nat = -1;

  // Binning (neighbors_binning_init, :765-871).
  int n_cells[3] = {0, 0, 0};
  double rec[3][3] = {{0}};
  int dx = 0, dy = 0, dz = 0;

  DevBuf pos4;        // Pos4[nat]: positions padded for one-sector gathers
  DevBuf posff;       // float4[2 nat]: positions as float-float (hi, lo)
  bool want_posff = false;  // written by the build (a mixed-form potential uses the list)
  bool posff_valid = false;
  DevBuf atom_cell;   // int[nat]: wrapped linear cell index
  DevBuf atom_wrap;   // int[nat]: packed wrap counts q (pbc dims)
  DevBuf cell_count;  // int[ncells+1]
  DevBuf cell_start;  // int[ncells+1]
  DevBuf cell_atoms;  // int[nat]: atoms sorted by (cell, id)
  DevBuf counts;      // int[nat+1]
  DevBuf spos;        // float4[nat]: cell-sorted float positions, .w = atom id
  DevBuf swrap;       // int[nat]: wrap counts in cell-sorted order
  DevBuf seed;        // int[nat+1] CSR offsets
  DevBuf nbr;         // int[capacity]
  DevBuf shift;       // int32 packed shifts [capacity]
  DevBuf rev;         // int[capacity]: reverse entry (built on demand)
  DevBuf stage;       // int2[nat * stage_cap]: staged entries of the single pass
  int stage_cap = 0;  // per-atom capacity of the single pass (0: two passes)
  DevBuf scan_tmp;
  DevBuf stats;       // device-side status words
  HostBuf hstats;
  bool rev_valid = false;
  bool rev_pending = false;  // reverse index built, symmetry flag not yet read
  // Set by a bond-order potential before a single-structure build: the
  // staged compaction also writes the reverse index, and the tile plan for
  // tiles of plan_apt atoms is computed before the build's one read-back.
  bool want_rev = false;
  int plan_apt = 0;
  bool plan_ready = false;  // hplan holds the plan of this list for plan_done_apt
  int plan_done_apt = 0;
  int hplan[2] = {0, 0};    // most bonds and (ij, ik) slots in one tile
  int64_t nentries = 0;
  int maxz = 0;
  cudaStream_t stream = nullptr;
};

// Tile plan of the bond-order kernels (launch only): out[0] = most bonds and
// out[1] = most (ij, ik) slots of the tiles of apt consecutive atoms (or of
// the caller's tiles, tile_atom0 != nullptr); out[0..1] must start at zero.
int bop_plan_launch(int nat, int apt, int ntiles, const int *tile_atom0, const int *seed,
                    int *out, cudaStream_t s);

// Builds/refreshes the list for p if positions or cell changed
// (neighbors_update, :430-456).
int neighbors_update(Neighbors &nl, Particles &p, cudaStream_t stream);
// Binning parameters of one cell (rows of A: Abox(a, k) with column k the
// lattice vector k; B = A^-1); cell_base offsets the cell numbers.
int bin_params(const double A[3][3], const double B[3][3], const int pbc[3], double cutoff,
               int cell_base, BinParams &bp);
// 3x3 inverse by the reference's Gauss elimination (0 on success).
int cell_inverse(const double A[3][3], double B[3][3]);
// List build of nat atoms at r (device (nat,3)); a batch passes per-structure
// parameters bps (device) and per-atom structure ids sid.
// capture: no host synchronisation (for CUDA-graph capture); needs a
// previous build (staged pass with capacity nl.stage_cap) and buffers sized
// for nat * stage_cap entries; the status words land in nl.hstats.
int nl_build(Neighbors &nl, int nat, const double *r, const BinParams &bp0,
             const BinParams *bps, const int *sid, int ncells, cudaStream_t stream,
             bool capture = false);
// Reverse-entry index of the list.  With sync = false the symmetry check is
// deferred: call neighbors_check_reverse (stream = nullptr once the caller
// has synchronised the stream itself) before rev is read.
int neighbors_build_reverse(Neighbors &nl, int nat, cudaStream_t stream,
                            bool sync = true);
int neighbors_check_reverse(Neighbors &nl, cudaStream_t stream);

// Device-wide exclusive scan of int32 (n+1 outputs, out[n] = total).
int exclusive_scan_i32(const int *in, int *out, int n, DevBuf &tmp, cudaStream_t stream);

// Cell for kernels.
Cell make_cell(const Particles &p);

}  // namespace gb

// Opaque handle types of the C-ABI.
struct gb_particles {
  gb::Particles p;
};
struct gb_neighbors {
  gb::Neighbors nl;
};
