// Particles, neighbour list and shared utilities of libatomistica_gb300.
//
// Neighbour build (replaces python_neighbors.f90:430-959):
//   K1  nl_assign_cells   per atom: FP64 cell coordinate floor(rec . r) with the
//                         reference operation order, pbc wrap / clamp, padded
//                         Pos4 copy of the position, cell histogram.
//   K1b exclusive scan    cell offsets.
//   K1c nl_scatter        atoms into their cell slots (atomic slot claim).
//   K1d nl_sort_cells     per-cell sort by atom id, so that every cell lists its
//                         atoms in increasing id as the reference's linked
//                         list does (binning_update, :904-959), written as
//                         float positions (+ id, wrap) in cell-sorted order
//                         (nl_sort_big_cells: the same for crowded cells).
//   K2  nl_pairs<count>   per atom (cell-sorted thread order): stencil loop in
//                         the reference order; each candidate is decided by an
//                         FP32 test with a rigorous error bound, and only the
//                         few inside the uncertainty band take the reference's
//                         FP64 test |r_i - r_j + A s|^2 < cutoff^2 (no FMA
//                         contraction, reference order, :708-711), so the
//                         decision always equals the reference's -> counts.
//   K2b exclusive scan    CSR offsets.
//   K2c nl_pairs<fill>    same loop, writes j and the packed image shift
//                         (steady state: one pass that also stages the
//                         entries, then nl_compact / nl_compact_reverse).
// The resulting per-atom entry order equals the reference's (stencil offset
// x-major/z-minor, then atom id), so pair sets and per-bond indices match.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>

#include "internal.h"

namespace gb {

// ---------------------------------------------------------------------------
// Error state.
// ---------------------------------------------------------------------------
static thread_local std::string g_error;
static std::atomic<unsigned long long> g_launches{0};
void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
void set_error(const std::string &msg) { g_error = msg; }
void clear_error() { g_error.clear(); }

int DevBuf::ensure(size_t n) {
  if (n <= bytes && p) return 0;
  size_t nb = std::max<size_t>(n, 256);
  nb = std::max(nb, bytes + bytes / 2);
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, nb);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc(") + std::to_string(nb) + ") failed: " +
              cudaGetErrorString(e));
    return GB_ERROR_CUDA;
  }
  if (p) cudaFree(p);
  p = q;
  bytes = nb;
  return 0;
}
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int HostBuf::ensure(size_t n) {
  if (n <= bytes && p) return 0;
  size_t nb = std::max<size_t>(n, 256);
  nb = std::max(nb, bytes + bytes / 2);
  void *q = nullptr;
  cudaError_t e = cudaMallocHost(&q, nb);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMallocHost failed: ") + cudaGetErrorString(e));
    return GB_ERROR_CUDA;
  }
  if (p) cudaFreeHost(p);
  p = q;
  bytes = nb;
  return 0;
}
void HostBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
}

bool is_device_ptr(const void *ptr) {
  if (!ptr) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

double *mapped_host_ptr(void *ptr) {
  if (!ptr) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<double *>(a.devicePointer) : nullptr;
}

Cell make_cell(const Particles &p) {
  Cell c;
  std::memcpy(c.A, p.A, sizeof(c.A));
  for (int k = 0; k < 3; k++) c.pbc[k] = p.pbc[k];
  return c;
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32: block-local scans, recursive scan of block sums.
// ---------------------------------------------------------------------------
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;

__global__ void scan_tiles(const int *__restrict__ in, int *__restrict__ out, int n,
                           int *__restrict__ tile_sums) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPerThread;
  int v[kScanPerThread];
  int s = 0;
#pragma unroll
  for (int q = 0; q < kScanPerThread; q++) {
    int idx = base + q;
    v[q] = idx < n ? in[idx] : 0;
    s += v[q];
  }
  // Warp-inclusive scan of per-thread sums.
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int w = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = w;
  }
  __syncthreads();
  int run = incl - s + (wid > 0 ? warp_tot[wid - 1] : 0);
#pragma unroll
  for (int q = 0; q < kScanPerThread; q++) {
    int idx = base + q;
    if (idx < n) out[idx] = run;
    run += v[q];
  }
  if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = run;
}

__global__ void scan_add(int *__restrict__ out, int n, const int *__restrict__ tile_offs) {
  const int idx = blockIdx.x * kScanTile + threadIdx.x;
  const int add = tile_offs[blockIdx.x];
  for (int q = 0; q < kScanPerThread; q++) {
    int k = idx + q * kScanThreads;
    if (k < n && k < (blockIdx.x + 1) * kScanTile) out[k] += add;
  }
}

// Second pass of the two-pass scan (tiles <= kScanFlatTiles): the block
// adds the sum of the tile sums before it (integer sums: exact in any order)
// and the last block writes the total out[n].
constexpr int kScanFlatTiles = 2048;
__global__ void scan_add_prefix(int *__restrict__ out, int n, const int *__restrict__ tile_sums,
                                int tiles) {
  __shared__ int warp_tot[kScanThreads / 32];
  int s = 0;
  for (int t = threadIdx.x; t < (int)blockIdx.x; t += kScanThreads) s += tile_sums[t];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) warp_tot[wid] = s;
  __syncthreads();
  int add = 0;
#pragma unroll
  for (int w = 0; w < kScanThreads / 32; w++) add += warp_tot[w];
  if (add != 0) {
    const int idx = blockIdx.x * kScanTile + threadIdx.x;
    for (int q = 0; q < kScanPerThread; q++) {
      const int k = idx + q * kScanThreads;
      if (k < n) out[k] += add;
    }
  }
  if (blockIdx.x == tiles - 1 && threadIdx.x == 0) out[n] = add + tile_sums[tiles - 1];
}

__global__ void scan_total(const int *__restrict__ in, int *__restrict__ out, int n) {
  // out[n] = out[n-1] + in[n-1]
  if (n == 0)
    out[0] = 0;
  else
    out[n] = out[n - 1] + in[n - 1];
}

int scan_rec(const int *in, int *out, int n, int *tmp, cudaStream_t s) {
  if (n <= 0) return 0;
  const int tiles = (n + kScanTile - 1) / kScanTile;
  int *sums = tmp;
  int *offs = tmp + tiles + 1;
  scan_tiles<<<tiles, kScanThreads, 0, s>>>(in, out, n, sums);
  note_launch();
  if (tiles > 1) {
    scan_rec(sums, offs, tiles, tmp + 2 * (tiles + 1), s);
    scan_add<<<tiles, kScanThreads, 0, s>>>(out, n, offs);
    note_launch();
  }
  return 0;
}

size_t scan_tmp_ints(int n) {
  size_t t = 0;
  while (n > 0) {
    int tiles = (n + kScanTile - 1) / kScanTile;
    t += 2 * (size_t)(tiles + 1);
    if (tiles <= 1) break;
    n = tiles;
  }
  return t + 64;
}

}  // namespace

// Small inputs (n <= 16384): one block of 1024 threads and the total out[n],
// one launch.  Warp w scans elements [512 w, 512 w + 512) as 16 rows of 32
// (coalesced loads and stores, 16 independent shuffle scans per warp), then
// the 32 warp totals are scanned and added.
constexpr int kScanSmallThreads = 1024, kScanSmallPer = 16;
__global__ void __launch_bounds__(kScanSmallThreads)
    scan_small(const int *__restrict__ in, int *__restrict__ out, int n) {
  __shared__ int warp_tot[kScanSmallThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int base = wid * (32 * kScanSmallPer) + lane;
  int v[kScanSmallPer];
#pragma unroll
  for (int q = 0; q < kScanSmallPer; q++) v[q] = base + 32 * q < n ? in[base + 32 * q] : 0;
  int run = 0;
#pragma unroll
  for (int q = 0; q < kScanSmallPer; q++) {
    int x = v[q];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += t;
    }
    const int row = __shfl_sync(0xffffffffu, x, 31);
    v[q] = run + x - v[q];  // exclusive within the warp's chunk
    run += row;
  }
  if (lane == 0) warp_tot[wid] = run;
  __syncthreads();
  if (wid == 0) {
    int w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  const int off = wid > 0 ? warp_tot[wid - 1] : 0;
#pragma unroll
  for (int q = 0; q < kScanSmallPer; q++)
    if (base + 32 * q < n) out[base + 32 * q] = v[q] + off;
  if (threadIdx.x == 0) out[n] = warp_tot[kScanSmallThreads / 32 - 1];
}

int exclusive_scan_i32(const int *in, int *out, int n, DevBuf &tmp, cudaStream_t stream) {
  GB_CHECK(tmp.ensure(scan_tmp_ints(n) * sizeof(int)));
  const int tiles = (n + kScanTile - 1) / kScanTile;
  if (n > 0 && n <= kScanSmallThreads * kScanSmallPer) {
    scan_small<<<1, kScanSmallThreads, 0, stream>>>(in, out, n);
    note_launch();
  } else if (n > 0 && tiles <= kScanFlatTiles) {
    // two launches: tile scans, then the tile offsets and the total
    scan_tiles<<<tiles, kScanThreads, 0, stream>>>(in, out, n, tmp.as<int>());
    note_launch();
    scan_add_prefix<<<tiles, kScanThreads, 0, stream>>>(out, n, tmp.as<int>(), tiles);
    note_launch();
  } else {
    scan_rec(in, out, n, tmp.as<int>(), stream);
    scan_total<<<1, 1, 0, stream>>>(in, out, n);
    note_launch();
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------------------
// Host-side cell inverse (gauss(), f_linearalgebra.f90:505-552).
// ---------------------------------------------------------------------------
static int gauss_solve3(const double Ain[3][3], const double b[3], double x[3]) {
  double A[3][4];
  for (int j = 0; j < 3; j++) {
    for (int k = 0; k < 3; k++) A[j][k] = Ain[j][k];
    A[j][3] = b[j];
  }
  int indx[3] = {0, 0, 0};
  for (int i = 0; i < 3; i++) {
    int mi = -1;
    double mv = -1.0;
    for (int j = 0; j < 3; j++) {
      if (indx[j]) continue;
      double v = std::fabs(A[j][i]);
      if (v > mv) {
        mv = v;
        mi = j;
      }
    }
    indx[mi] = i + 1;
    if (A[mi][i] == 0.0) return -1;
    double fac[3], row[4];
    for (int j = 0; j < 3; j++) fac[j] = A[j][i] / A[mi][i];
    for (int k = 0; k < 4; k++) row[k] = A[mi][k];
    for (int j = 0; j < 3; j++) {
      if (indx[j]) continue;
      for (int k = i; k < 4; k++) A[j][k] = A[j][k] - fac[j] * row[k];
    }
  }
  double Ap[3][4];
  for (int j = 0; j < 3; j++)
    for (int k = 0; k < 4; k++) Ap[indx[j] - 1][k] = A[j][k];
  for (int j = 2; j >= 0; j--) {
    if (Ap[j][j] == 0.0) return -1;
    x[j] = Ap[j][3] / Ap[j][j];
    for (int m = 0; m < j; m++) Ap[m][3] = Ap[m][3] - Ap[m][j] * x[j];
  }
  return 0;
}

int cell_inverse(const double A[3][3], double B[3][3]) {
  for (int c = 0; c < 3; c++) {
    double e[3] = {0, 0, 0}, x[3];
    e[c] = 1.0;
    if (gauss_solve3(A, e, x) != 0) return -1;
    for (int a = 0; a < 3; a++) B[a][c] = x[a];
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Neighbour build kernels.
// ---------------------------------------------------------------------------
namespace {


__device__ __forceinline__ int floor_div(int a, int n) {
  int q = a / n;
  if ((a % n != 0) && ((a < 0) != (n < 0))) q--;
  return q;
}

// floor(matmul(rec_cell_size, r)) with the reference's summation order and no
// FMA contraction (python_neighbors.f90:641).  The FP32 value s_f of each row
// is within 8 u S (S = sum |rec_a x_a|, u = 2^-24; 5.1 u S is the bound of the
// FP32 and FP64 roundings) of the FP64 value, so floor(s_f -/+ e) agreeing
// decides the cell; otherwise (an atom within ~1e-5 cells of a boundary) the
// FP64 evaluation does.
// (a call, not inlined: kept out of line so that the rare FP64 evaluation is
// not executed under predicates for every atom)
__device__ __noinline__ int raw_cell_fp64(const double *rec_row, double x, double y, double z) {
  double sd = __dmul_rn(rec_row[0], x);
  sd = __dadd_rn(sd, __dmul_rn(rec_row[1], y));
  sd = __dadd_rn(sd, __dmul_rn(rec_row[2], z));
  double f = floor(sd);
  f = fmin(fmax(f, -1.0e9), 1.0e9);
  return (int)f;
}

__device__ __forceinline__ void raw_cell(const BinParams &bp, double x, double y, double z,
                                         float xf, float yf, float zf, int c[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float p0 = __fmul_rn(bp.recf[k][0], xf), p1 = __fmul_rn(bp.recf[k][1], yf),
                p2 = __fmul_rn(bp.recf[k][2], zf);
    const float sf = __fadd_rn(__fadd_rn(p0, p1), p2);
    const float e = 4.8e-7f * (fabsf(p0) + fabsf(p1) + fabsf(p2)) + 1.0e-37f;
    const float fl = floorf(sf - e);
    if (fl == floorf(sf + e) && fabsf(fl) < 1.0e9f)
      c[k] = (int)fl;
    else
      c[k] = raw_cell_fp64(bp.rec[k], x, y, z);
  }
}

// Linear cell index, z fastest: the 2 dz + 1 cells of one (x, y) stencil row
// are contiguous in the cell-sorted atom order.
__device__ __forceinline__ int cell_linear(const BinParams &bp, int cx, int cy, int cz) {
  return bp.cell_base + (cx * bp.n[1] + cy) * bp.n[2] + cz;
}

__device__ __forceinline__ int pack_wrap(int q0, int q1, int q2) {
  return pack_shift(q0, q1, q2);
}

// kBatch: atom i belongs to structure sid[i] with binning parameters
// bps[sid[i]] (cells of all structures numbered consecutively).
template <bool kBatch>
__global__ void nl_assign_cells(int nat, const double *__restrict__ r, BinParams bp0,
                                const BinParams *__restrict__ bps, const int *__restrict__ sid,
                                Pos4 *__restrict__ pos4, float4 *__restrict__ posff,
                                int *__restrict__ atom_cell,
                                int *__restrict__ atom_wrap, int *__restrict__ cell_count,
                                int *__restrict__ status) {
  // (blockDim.x is a multiple of 32: every lane reaches the warp reduction)
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < nat;
  double x = 0.0, y = 0.0, z = 0.0;
  if (in) {
    x = r[3 * i];
    y = r[3 * i + 1];
    z = r[3 * i + 2];
  }
  const bool finite = isfinite(x) && isfinite(y) && isfinite(z);
  const float xf = (float)x, yf = (float)y, zf = (float)z;
  {
    // max |coordinate| (rounded up) for the pair prefilter's error bound: one
    // atomic per block (a single address: per-warp atomics serialised there).
    __shared__ unsigned wmax[32];
    const float m = finite ? fmaxf(fabsf(xf), fmaxf(fabsf(yf), fabsf(zf))) * (1.0f + 1.2e-7f)
                           : 0.0f;
    const unsigned mw = __reduce_max_sync(0xffffffffu, (unsigned)__float_as_int(m));
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = mw;
    __syncthreads();
    if (threadIdx.x < 32) {
      const unsigned v = threadIdx.x < (blockDim.x >> 5) ? wmax[threadIdx.x] : 0u;
      const unsigned bm = __reduce_max_sync(0xffffffffu, v);
      if (threadIdx.x == 0) atomicMax(&status[3], (int)bm);
    }
  }
  if (!in) return;
  const BinParams &bp = kBatch ? bps[sid[i]] : bp0;
  pos4[i] = Pos4{x, y, z, 0.0};
  if (posff) {
    // float-float copy (hi, lo) for the mixed-precision kernels
    posff[2 * i] = make_float4(xf, yf, zf, 0.0f);
    posff[2 * i + 1] = make_float4((float)(x - (double)xf), (float)(y - (double)yf),
                                   (float)(z - (double)zf), 0.0f);
  }
  if (!finite) {
    atomicOr(&status[1], 1);  // non-finite position
    atom_cell[i] = 0;
    atom_wrap[i] = pack_wrap(0, 0, 0);
    atomicAdd(&cell_count[0], 1);
    return;
  }
  int c[3], q[3];
  raw_cell(bp, x, y, z, xf, yf, zf, c);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    q[k] = 0;
    if (bp.pbc[k]) {
      q[k] = floor_div(c[k], bp.n[k]);
      c[k] -= q[k] * bp.n[k];
    } else {
      c[k] = min(max(c[k], 0), bp.n[k] - 1);
    }
    if (q[k] > kMaxShift || q[k] < -kMaxShift) atomicOr(&status[1], 2);
  }
  const int ci = cell_linear(bp, c[0], c[1], c[2]);
  atom_cell[i] = ci;
  atom_wrap[i] = pack_wrap(max(min(q[0], kMaxShift), -kMaxShift),
                           max(min(q[1], kMaxShift), -kMaxShift),
                           max(min(q[2], kMaxShift), -kMaxShift));
  atomicAdd(&cell_count[ci], 1);
}

__global__ void nl_scatter(int nat, const int *__restrict__ atom_cell,
                           const int *__restrict__ cell_start, int *__restrict__ cell_fill,
                           int *__restrict__ cell_atoms) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const int c = atom_cell[i];
  const int slot = cell_start[c] + atomicAdd(&cell_fill[c], 1);
  cell_atoms[slot] = i;
}

// Sort each cell's atoms by id: insertion sort for small cells, a
// rank-by-count pass (one block per cell) for the rare crowded cell.
constexpr int kSmallCell = 48;

// The sorted slot t of atom i: float copy of its position with the atom id
// in .w and its wrap counts, so that the candidate loop reads one 16-byte
// record per candidate.
__device__ __forceinline__ void put_sorted(int t, int i, const Pos4 *__restrict__ pos4,
                                           const int *__restrict__ atom_wrap,
                                           float4 *__restrict__ spos, int *__restrict__ swrap) {
  const Pos4 p = pos4[i];
  spos[t] = make_float4((float)p.x, (float)p.y, (float)p.z, __int_as_float(i));
  swrap[t] = atom_wrap[i];
}

// Per cell (a thread each): the cell's atoms sorted by id (insertion sort),
// written to their sorted slots; crowded cells are left to nl_sort_big_cells.
__global__ void nl_sort_cells(int ncells, const int *__restrict__ cell_start,
                              const int *__restrict__ cell_atoms, int *__restrict__ big_cells,
                              int *__restrict__ n_big, const Pos4 *__restrict__ pos4,
                              const int *__restrict__ atom_wrap, float4 *__restrict__ spos,
                              int *__restrict__ swrap) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  const int s = cell_start[c], e = cell_start[c + 1];
  const int m = e - s;
  if (m == 0) return;
  if (m > kSmallCell) {
    big_cells[atomicAdd(n_big, 1)] = c;
    return;
  }
  int v[kSmallCell];
  for (int q = 0; q < m; q++) v[q] = cell_atoms[s + q];
  for (int q = 1; q < m; q++) {
    int key = v[q];
    int p = q - 1;
    while (p >= 0 && v[p] > key) {
      v[p + 1] = v[p];
      p--;
    }
    v[p + 1] = key;
  }
  for (int q = 0; q < m; q++) put_sorted(s + q, v[q], pos4, atom_wrap, spos, swrap);
}

// Crowded cells (rare), a block each: rank by count into tmp, then the
// sorted slots from tmp (one block per cell, so a barrier orders the two).
__global__ void nl_sort_big_cells(const int *__restrict__ big_cells, const int *__restrict__ n_big,
                                  const int *__restrict__ cell_start,
                                  const int *__restrict__ cell_atoms, int *__restrict__ tmp,
                                  const Pos4 *__restrict__ pos4,
                                  const int *__restrict__ atom_wrap, float4 *__restrict__ spos,
                                  int *__restrict__ swrap) {
  const int nbig = *n_big;
  for (int bc = blockIdx.x; bc < nbig; bc += gridDim.x) {
    const int c = big_cells[bc];
    const int s = cell_start[c], e = cell_start[c + 1];
    for (int q = s + threadIdx.x; q < e; q += blockDim.x) {
      const int me = cell_atoms[q];
      int rank = 0;
      for (int t = s; t < e; t++) rank += cell_atoms[t] < me;
      tmp[s + rank] = me;
    }
    __syncthreads();
    for (int q = s + threadIdx.x; q < e; q += blockDim.x)
      put_sorted(q, tmp[q], pos4, atom_wrap, spos, swrap);
  }
}

// Exact reference test |r_i - r_j + A s|^2 < cutoff^2: FP64, no FMA
// contraction, reference operation order (python_neighbors.f90:708-711).
__device__ __forceinline__ bool exact_pair_test(const BinParams &bp, const Pos4 &ri,
                                                const Pos4 &rj, int s0, int s1, int s2) {
  const double sx = (double)s0, sy = (double)s1, sz = (double)s2;
  const double rij[3] = {__dsub_rn(ri.x, rj.x), __dsub_rn(ri.y, rj.y), __dsub_rn(ri.z, rj.z)};
  double d[3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    double as = __dmul_rn(bp.A[a][0], sx);
    as = __dadd_rn(as, __dmul_rn(bp.A[a][1], sy));
    as = __dadd_rn(as, __dmul_rn(bp.A[a][2], sz));
    d[a] = __dadd_rn(rij[a], as);
  }
  double d2 = __dmul_rn(d[0], d[0]);
  d2 = __dadd_rn(d2, __dmul_rn(d[1], d[1]));
  d2 = __dadd_rn(d2, __dmul_rn(d[2], d[2]));
  return d2 < bp.cutoff_sq;
}

// Candidate loop.  Every candidate is first tested in FP32 against a
// rigorous error bound of the FP32 evaluation (positions rounded to float,
// the image term and the squared norm); only candidates whose FP32 distance
// falls inside the uncertainty band around the cutoff take the exact FP64
// test.  The decision is therefore always the reference's, while almost all
// arithmetic runs on the FP32 pipe.
//
// Error bound: with u = 2^-24, X = max |coordinate| and T = sum_k |A_ak s_k|,
// each component of the FP32 difference vector is within
// E = u (4X + 8T + 4 cutoff + 4) of the exact one, and
// |d2_f - d2| <= 2 E (3.47 |d| + 9 E) + 12 u d2 (a factor-2 margin included);
// |d| <= (d2 + 1) / 2 replaces the square root.
//
// Stencil order (python_neighbors.f90:862-869): x, then y, then z offsets,
// each cell's atoms by increasing id.  With the z-fastest cell layout the z
// offsets of one (x, y) row that do not cross the periodic boundary form one
// contiguous run of the cell-sorted atoms, visited in that same order.
//
// kMode: kPairsCount (counts), kPairsFill (CSR j and packed shift at seed[i]),
// kPairsCountStage (counts, and the first `cap` entries of each atom into
// stage[i * cap ..], compacted afterwards when no atom has more).
constexpr int kPairsCount = 0, kPairsFill = 1, kPairsCountStage = 2;

__device__ __forceinline__ bool wrap_cell(const BinParams &bp, int k, int &c, int &s) {
  const int n = bp.n[k];
  if (c >= 0 && c < n) return true;
  if (!bp.pbc[k]) return false;
  const int q = floor_div(c, n);
  c -= q * n;
  s -= q;
  return true;
}

// One candidate: atom j at sorted slot jq for atom i (position pi), seen
// through the run's image shift s = (sx, sy, sz) (s1zero: s = 0; o = A s in
// FP32, Erun the run's error term) plus j's own wrap.  Returns the reference's
// decision; j, the packed shift and whether the shift is outside the packed
// range are returned for an accepted pair.
__device__ __forceinline__ bool pair_test(const BinParams &bp, const float4 &pi, int i, int jq,
                                          const float4 *__restrict__ spos,
                                          const int *__restrict__ swrap,
                                          const Pos4 *__restrict__ pos4, int sx, int sy, int sz,
                                          bool s1zero, float ox, float oy, float oz, float Erun,
                                          float Ebase, float eA, int packed1, float clo,
                                          float chi, bool &have_ri, Pos4 &ri, int &j,
                                          int &packed, bool &range_bad) {
  const float u = 5.9604645e-8f;
  const int kZeroWrap = pack_shift(0, 0, 0);
  const float4 pj = spos[jq];
  j = __float_as_int(pj.w);
  const int wj = swrap[jq];
  int s2x = sx, s2y = sy, s2z = sz;
  bool zero_shift = s1zero;
  float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
  float E = Erun;
  if (wj == kZeroWrap) {
    dx += ox;
    dy += oy;
    dz += oz;
  } else {
    int w0, w1, w2;
    unpack_shift(wj, w0, w1, w2);
    s2x += w0;
    s2y += w1;
    s2z += w2;
    zero_shift = (s2x | s2y | s2z) == 0;
    const float fx = (float)s2x, fy = (float)s2y, fz = (float)s2z;
    dx += bp.Af[0][0] * fx + bp.Af[0][1] * fy + bp.Af[0][2] * fz;
    dy += bp.Af[1][0] * fx + bp.Af[1][1] * fy + bp.Af[1][2] * fz;
    dz += bp.Af[2][0] * fx + bp.Af[2][1] * fy + bp.Af[2][2] * fz;
    E = Ebase + eA * (fabsf(fx) + fabsf(fy) + fabsf(fz));
  }
  if (j == i && zero_shift) return false;
  const float d2f = dx * dx + dy * dy + dz * dz;
  const float B = 2.0f * E * (1.735f * (d2f + 1.0f) + 9.0f * E) + 12.0f * u * d2f;
  bool accept;
  if (d2f + B < clo) {
    accept = true;
  } else if (d2f - B > chi) {
    accept = false;
  } else {
    if (!have_ri) {
      ri = pos4[i];
      have_ri = true;
    }
    accept = exact_pair_test(bp, ri, pos4[j], s2x, s2y, s2z);
  }
  if (accept) {
    packed = wj == kZeroWrap ? packed1 : pack_shift(s2x, s2y, s2z);
    range_bad = s2x > kMaxShift || s2x < -kMaxShift || s2y > kMaxShift || s2y < -kMaxShift ||
                s2z > kMaxShift || s2z < -kMaxShift;
  }
  return accept;
}

// Shortcuts of the candidate loops.  A warp runs a candidate step for all
// its lanes at once, so the common cases are kept short and the band test of
// pair_test is left to the rare ones:
//   d2' = |(p_i + A s) - p_j|^2 in FP32 (the run's image offset added to p_i
//         first), for a j without own wrap (its image offset is the run's);
//   reject  d2' > thi (about nine candidates in ten), or j = i in a run
//           without image shift;
//   accept  d2' < tlo;
//   otherwise (the FP32 band around the cutoff, a wrapped j) pair_test.
// thi and tlo are where pair_test's band test (d2f -+ B against chi / clo,
// B = a d2f + b, a = 3.47 E + 12 u, b = 3.47 E + 18 E^2) starts to reject /
// still accepts: thi = (chi + b) / (1 - a) raised and tlo = (clo - b) /
// (1 + a) lowered by a relative 1e-6.  Each component error of the lean
// evaluation is within the same E as pair_test's order for every pair
// closer than the cutoff (u (3X + 4T + |d|) <= E), so both shortcuts make
// the reference's decision.
__device__ __forceinline__ void band_thresholds(float clo, float chi, float E, float &tlo,
                                                float &thi) {
  const float u = 5.9604645e-8f;
  const float a = 3.47f * E + 12.0f * u, b = 3.47f * E + 18.0f * E * E;
  thi = (chi + b) / (1.0f - a) * (1.0f + 1e-6f);
  tlo = (clo - b) / (1.0f + a) * (1.0f - 1e-6f);
}
// Whether a packed image shift is outside the packed range.
__device__ __forceinline__ bool shift_out_of_range(int sx, int sy, int sz) {
  return sx > kMaxShift || sx < -kMaxShift || sy > kMaxShift || sy < -kMaxShift ||
         sz > kMaxShift || sz < -kMaxShift;
}

// An accepted entry number pos of atom i, as kMode stores it.
template <int kMode>
__device__ __forceinline__ void pair_store(int i, int pos, int j, int packed, bool range_bad,
                                           int seed_i, int *__restrict__ nbr,
                                           int *__restrict__ shift, int2 *__restrict__ stage,
                                           int cap, int *__restrict__ status) {
  if (kMode == kPairsFill) {
    nbr[seed_i + pos] = j;
    shift[seed_i + pos] = packed;
  } else {
    if (kMode == kPairsCountStage && pos < cap)
      stage[(size_t)i * cap + pos] = make_int2(j, packed);
    if (range_bad) atomicOr(&status[1], 2);
  }
}

// The whole stencil of atom i (sorted slot t, cell (cx0, cy0, cz0), wrap q)
// walked on one thread in the reference's order; returns its entry count.
// kLean: the candidate steps take the shortcuts above (the batch walk); else
// every candidate takes pair_test (the single-structure walk, where the
// shortcuts' extra registers cost more than they save).
template <int kMode, bool kLean>
__device__ __forceinline__ int pairs_walk(const BinParams &bp, int i, int t, const float4 &pi,
                                          int cx0, int cy0, int cz0, int q0, int q1, int q2,
                                          float Ebase, float eA, const Pos4 *__restrict__ pos4,
                                          const float4 *__restrict__ spos,
                                          const int *__restrict__ swrap,
                                          const int *__restrict__ cell_start, int seed_i,
                                          int *__restrict__ nbr, int *__restrict__ shift,
                                          int2 *__restrict__ stage, int cap,
                                          int *__restrict__ status) {
  const int kZeroWrap = pack_shift(0, 0, 0);
  int cnt = 0;
  bool have_ri = false;
  Pos4 ri;
  const float clo = bp.cutoff_sq_lo, chi = bp.cutoff_sq_hi;  // (once per atom)
  for (int x = -bp.dx; x <= bp.dx; x++) {
    int cx = cx0 + x, sx = -q0;
    if (!wrap_cell(bp, 0, cx, sx)) continue;
    for (int y = -bp.dy; y <= bp.dy; y++) {
      int cy = cy0 + y, sy = -q1;
      if (!wrap_cell(bp, 1, cy, sy)) continue;
      const int row = cell_linear(bp, cx, cy, 0);
      int z = -bp.dz;
      while (z <= bp.dz) {
        int cz = cz0 + z, sz = -q2;
        if (!wrap_cell(bp, 2, cz, sz)) {
          z++;
          continue;
        }
        const int run = min(bp.dz - z + 1, bp.n[2] - cz);
        const int js = cell_start[row + cz], je = cell_start[row + cz + run];
        z += run;
        // image offset A s1 of this run (atoms j with zero wrap use it as is)
        const bool s1zero = (sx | sy | sz) == 0;
        float ox = 0.0f, oy = 0.0f, oz = 0.0f, Erun = Ebase;
        if (!s1zero) {
          const float fx = (float)sx, fy = (float)sy, fz = (float)sz;
          ox = bp.Af[0][0] * fx + bp.Af[0][1] * fy + bp.Af[0][2] * fz;
          oy = bp.Af[1][0] * fx + bp.Af[1][1] * fy + bp.Af[1][2] * fz;
          oz = bp.Af[2][0] * fx + bp.Af[2][1] * fy + bp.Af[2][2] * fz;
          Erun += eA * (fabsf(fx) + fabsf(fy) + fabsf(fz));
        }
        const int packed1 = pack_shift(sx, sy, sz);
        if (!kLean) {
          for (int jq = js; jq < je; jq++) {
            int j, packed;
            bool range_bad;
            if (pair_test(bp, pi, i, jq, spos, swrap, pos4, sx, sy, sz, s1zero, ox, oy, oz, Erun,
                          Ebase, eA, packed1, clo, chi, have_ri, ri, j, packed, range_bad)) {
              pair_store<kMode>(i, cnt, j, packed, range_bad, seed_i, nbr, shift, stage, cap,
                                status);
              cnt++;
            }
          }
          continue;
        }
        const bool run_bad = shift_out_of_range(sx, sy, sz);
        float tlo, thi;
        band_thresholds(clo, chi, Erun, tlo, thi);
        const float px = pi.x + ox, py = pi.y + oy, pz = pi.z + oz;
        const int self_slot = s1zero ? t : -1;
        for (int jq = js; jq < je; jq++) {
          const float4 pj = spos[jq];
          const int wj = swrap[jq];
          const float dx = px - pj.x, dy = py - pj.y, dz = pz - pj.z;
          const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          const bool plain = wj == kZeroWrap;
          if (plain && (d2 > thi || jq == self_slot)) continue;
          int j = __float_as_int(pj.w), packed = packed1;
          bool range_bad = run_bad;
          bool acc = plain && d2 < tlo;
          if (!acc)
            acc = pair_test(bp, pi, i, jq, spos, swrap, pos4, sx, sy, sz, s1zero, ox, oy, oz, Erun,
                            Ebase, eA, packed1, clo, chi, have_ri, ri, j, packed, range_bad);
          if (acc) {
            pair_store<kMode>(i, cnt, j, packed, range_bad, seed_i, nbr, shift, stage, cap,
                              status);
            cnt++;
          }
        }
      }
    }
  }
  return cnt;
}

// Threads per block and resident threads per SM asked of the compiler (1536
// for a single structure, 1024 for batches): the pair search is bound by the
// latency of its candidate loads, and more resident warps (fewer registers,
// a few spilled) hide more of it (measured at 1,048,576 atoms).
#ifndef GB_PAIRS_THREADS
#define GB_PAIRS_THREADS 128
#endif
#ifndef GB_PAIRS_MIN_BLOCKS
#define GB_PAIRS_MIN_BLOCKS (1536 / GB_PAIRS_THREADS)
#endif
#ifndef GB_PAIRS_MIN_BLOCKS_BATCH
#define GB_PAIRS_MIN_BLOCKS_BATCH (1024 / GB_PAIRS_THREADS)
#endif
constexpr int kPairsThreads = GB_PAIRS_THREADS;

template <int kMode, bool kBatch>
__global__ void __launch_bounds__(kPairsThreads,
                                  kBatch ? GB_PAIRS_MIN_BLOCKS_BATCH : GB_PAIRS_MIN_BLOCKS)
    nl_pairs(int nat, BinParams bp0, const BinParams *__restrict__ bps,
             const int *__restrict__ sid, const Pos4 *__restrict__ pos4,
             const int *__restrict__ atom_cell, const float4 *__restrict__ spos,
             const int *__restrict__ swrap, const int *__restrict__ cell_start,
             int *__restrict__ counts, const int *__restrict__ seed, int *__restrict__ nbr,
             int *__restrict__ shift, int2 *__restrict__ stage, int cap, int clamp,
             int *__restrict__ status) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  // lanes with an atom (blockDim.x is a multiple of 32): they sum their
  // counts into the 64-bit list total at the end
  const unsigned active = __ballot_sync(0xffffffffu, t < nat);
  if (t >= nat) return;
  const float4 pi = spos[t];
  const int i = __float_as_int(pi.w);
  const BinParams &bp = kBatch ? bps[sid[i]] : bp0;
  int ci = atom_cell[i] - bp.cell_base;
  const int cz0 = ci % bp.n[2];
  ci /= bp.n[2];
  const int cy0 = ci % bp.n[1];
  const int cx0 = ci / bp.n[1];
  int q0, q1, q2;
  unpack_shift(swrap[t], q0, q1, q2);
  const float u = 5.9604645e-8f;
  const float X = __int_as_float(status[3]);
  const float Ebase = u * (4.0f * X + 4.0f * bp.cutoff_f + 4.0f);
  const float eA = 8.0f * u * bp.Amax;
  const int seed_i = kMode == kPairsFill ? seed[i] : 0;
  // Inside the cell grid (no row of the stencil needs a periodic wrap, the
  // atom is not wrapped): every row is one run of 2 dz + 1 cells with a zero
  // image shift, so a whole warp of such atoms takes a lean walk (the same
  // rows, runs, candidates and decisions as pairs_walk, with the shortcut
  // candidate steps; a wrapped j still brings its own shift through
  // pair_test).
  const bool deep = !kBatch && (q0 | q1 | q2) == 0 && cx0 >= bp.dx &&
                    cx0 < bp.n[0] - bp.dx && cy0 >= bp.dy && cy0 < bp.n[1] - bp.dy &&
                    cz0 >= bp.dz && cz0 < bp.n[2] - bp.dz;
  int cnt = 0;
  if (__all_sync(active, deep)) {
    const int kZeroWrap = pack_shift(0, 0, 0);
    const float clo = bp.cutoff_sq_lo, chi = bp.cutoff_sq_hi;
    float tlo0, thi0;
    band_thresholds(clo, chi, Ebase, tlo0, thi0);
    bool have_ri = false;
    Pos4 ri;
    for (int x = -bp.dx; x <= bp.dx; x++) {
      for (int y = -bp.dy; y <= bp.dy; y++) {
        const int row = cell_linear(bp, cx0 + x, cy0 + y, 0);
        const int js = cell_start[row + cz0 - bp.dz], je = cell_start[row + cz0 + bp.dz + 1];
        for (int jq = js; jq < je; jq++) {
          const float4 pj = spos[jq];
          const int wj = swrap[jq];
          const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
          const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
          const bool plain = wj == kZeroWrap;
          if (plain && (d2 > thi0 || jq == t)) continue;
          int j = __float_as_int(pj.w), packed = kZeroWrap;
          bool range_bad = false;
          bool acc = plain && d2 < tlo0;
          if (!acc)
            acc = pair_test(bp, pi, i, jq, spos, swrap, pos4, 0, 0, 0, true, 0.0f, 0.0f, 0.0f,
                            Ebase, Ebase, eA, kZeroWrap, clo, chi, have_ri, ri, j, packed,
                            range_bad);
          if (acc) {
            pair_store<kMode>(i, cnt, j, packed, range_bad, seed_i, nbr, shift, stage, cap,
                              status);
            cnt++;
          }
        }
      }
    }
  } else {
    cnt = pairs_walk<kMode, kBatch>(bp, i, t, pi, cx0, cy0, cz0, q0, q1, q2, Ebase, eA, pos4,
                                    spos, swrap, cell_start, seed_i, nbr, shift, stage, cap,
                                    status);
  }
  if (kMode != kPairsFill) {
    // clamp: the staged single pass without a host check (captured graphs)
    // keeps at most cap entries per atom; status[0] still records the true
    // maximum, which the caller compares with cap afterwards.
    counts[i] = clamp ? min(cnt, cap) : cnt;
    atomicMax(&status[0], cnt);
    // 64-bit total of the entries (status[6..7]): the CSR offsets are int32,
    // and a total beyond 2^31 - 1 must be refused before the scan's wrapped
    // result is used.  A count of 2^26 or more per atom is refused outright.
    if (cnt >= (1 << 26)) atomicOr(&status[1], 8);
    const unsigned wsum = __reduce_add_sync(active, (unsigned)min(cnt, (1 << 26) - 1));
    if ((threadIdx.x & 31) == __ffs(active) - 1)
      atomicAdd(reinterpret_cast<unsigned long long *>(status + 6), (unsigned long long)wsum);
  }
}

// Small structures (too few atoms to fill the GPU with one thread per atom):
// the candidates of an atom are dealt to a group of kPairLanes lanes, so that
// its walk does not run serially on one thread.  The group's lanes lay out
// the atom's stencil rows (row k on lane k mod 8; per row at most two runs of
// consecutive cells, as the row splits where it crosses the periodic
// boundary in z) with their image shifts in a shared table, take a prefix
// over the runs in stencil order and deal the candidates c = 0, 1, ... to the
// lanes in turn (lane g takes c = g, g + 8, ...); the group's ballot places
// the accepted entries in exactly the order of the one-thread walk.  An atom
// with more than 16 rows or more than two runs in a row is walked by the
// group's first lane.
constexpr int kPairLanes = 8;
constexpr int kPairRows = 16;
constexpr int kPairSlots = 2 * kPairRows;
#ifndef GB_PAIR_GROUP_MAX_ATOMS
#define GB_PAIR_GROUP_MAX_ATOMS 32768
#endif
constexpr int kPairGroupMaxAtoms = GB_PAIR_GROUP_MAX_ATOMS;

template <int kMode>
__global__ void __launch_bounds__(128)
    nl_pairs_grp(int nat, BinParams bp, const Pos4 *__restrict__ pos4,
                 const int *__restrict__ atom_cell, const float4 *__restrict__ spos,
                 const int *__restrict__ swrap, const int *__restrict__ cell_start,
                 int *__restrict__ counts, const int *__restrict__ seed, int *__restrict__ nbr,
                 int *__restrict__ shift, int2 *__restrict__ stage, int cap, int clamp,
                 int *__restrict__ status) {
  constexpr int G = kPairLanes;
  __shared__ int s_js[128 / G][kPairSlots], s_sh[128 / G][kPairSlots];
  __shared__ int s_pre[128 / G][kPairSlots + 1];
  const int lane = threadIdx.x & 31, g = threadIdx.x & (G - 1), grp = threadIdx.x / G;
  const unsigned gmask = 0xFFu << (lane & 24);
  const int t = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G);
  int cnt = 0, i = -1;
  if (t < nat) {  // (uniform over the group)
    const float4 pi = spos[t];
    i = __float_as_int(pi.w);
    int ci = atom_cell[i];
    const int cz0 = ci % bp.n[2];
    ci /= bp.n[2];
    const int cy0 = ci % bp.n[1];
    const int cx0 = ci / bp.n[1];
    int q0, q1, q2;
    unpack_shift(swrap[t], q0, q1, q2);
    const float u = 5.9604645e-8f;
    const float X = __int_as_float(status[3]);
    const float Ebase = u * (4.0f * X + 4.0f * bp.cutoff_f + 4.0f);
    const float eA = 8.0f * u * bp.Amax;
    const int seed_i = kMode == kPairsFill ? seed[i] : 0;
    const int ny = 2 * bp.dy + 1, nrows = (2 * bp.dx + 1) * ny;
    bool over = nrows > kPairRows;
    int js[2][2], len[2][2], sh[2][2];
#pragma unroll
    for (int m = 0; m < 2; m++) {
#pragma unroll
      for (int p = 0; p < 2; p++) {
        js[m][p] = 0;
        len[m][p] = 0;
        sh[m][p] = 0;
      }
      const int k = g + G * m;
      if (over || k >= nrows) continue;
      int cx = cx0 + k / ny - bp.dx, sx = -q0;
      int cy = cy0 + k % ny - bp.dy, sy = -q1;
      if (!wrap_cell(bp, 0, cx, sx) || !wrap_cell(bp, 1, cy, sy)) continue;
      const int row = cell_linear(bp, cx, cy, 0);
      int z = -bp.dz, np = 0;
      while (z <= bp.dz) {
        int cz = cz0 + z, sz = -q2;
        if (!wrap_cell(bp, 2, cz, sz)) {
          z++;
          continue;
        }
        const int run = min(bp.dz - z + 1, bp.n[2] - cz);
        if (np < 2) {
          js[m][np] = cell_start[row + cz];
          len[m][np] = cell_start[row + cz + run] - js[m][np];
          sh[m][np] = pack_shift(sx, sy, sz);
        }
        np++;
        z += run;
      }
      if (np > 2) over = true;
    }
    over = __any_sync(gmask, over);
    if (!over) {
      // slots 2k + p (row k, run p) in stencil order: exclusive prefix
      int base = 0;
#pragma unroll
      for (int m = 0; m < 2; m++) {
        const int rl = len[m][0] + len[m][1];
        int inc = rl;
#pragma unroll
        for (int o = 1; o < G; o <<= 1) {
          const int v = __shfl_up_sync(gmask, inc, o, G);
          if (g >= o) inc += v;
        }
        const int k = g + G * m;
        if (k < nrows) {
          const int p0 = base + inc - rl;
#pragma unroll
          for (int p = 0; p < 2; p++) {
            s_js[grp][2 * k + p] = js[m][p];
            s_sh[grp][2 * k + p] = sh[m][p];
          }
          s_pre[grp][2 * k] = p0;
          s_pre[grp][2 * k + 1] = p0 + len[m][0];
        }
        base += __shfl_sync(gmask, inc, G - 1, G);
      }
      if (g == 0) s_pre[grp][2 * nrows] = base;
      __syncwarp(gmask);
      const int total = base;
      bool have_ri = false;
      Pos4 ri;
      const float clo = bp.cutoff_sq_lo, chi = bp.cutoff_sq_hi;
      int r = 0, rs = -1, sx = 0, sy = 0, sz = 0, packed1 = 0;
      bool s1zero = true;
      float ox = 0.0f, oy = 0.0f, oz = 0.0f, Erun = Ebase;
      for (int c0 = 0; c0 < total; c0 += G) {
        const int c = c0 + g;
        bool accept = false, range_bad = false;
        int j = 0, packed = 0;
        if (c < total) {
          while (s_pre[grp][r + 1] <= c) r++;
          if (r != rs) {  // the run's image offset, as pairs_walk forms it
            rs = r;
            packed1 = s_sh[grp][r];
            unpack_shift(packed1, sx, sy, sz);
            s1zero = (sx | sy | sz) == 0;
            ox = oy = oz = 0.0f;
            Erun = Ebase;
            if (!s1zero) {
              const float fx = (float)sx, fy = (float)sy, fz = (float)sz;
              ox = bp.Af[0][0] * fx + bp.Af[0][1] * fy + bp.Af[0][2] * fz;
              oy = bp.Af[1][0] * fx + bp.Af[1][1] * fy + bp.Af[1][2] * fz;
              oz = bp.Af[2][0] * fx + bp.Af[2][1] * fy + bp.Af[2][2] * fz;
              Erun += eA * (fabsf(fx) + fabsf(fy) + fabsf(fz));
            }
          }
          const int jq = s_js[grp][r] + (c - s_pre[grp][r]);
          accept = pair_test(bp, pi, i, jq, spos, swrap, pos4, sx, sy, sz, s1zero, ox, oy, oz,
                             Erun, Ebase, eA, packed1, clo, chi, have_ri, ri, j, packed, range_bad);
        }
        const unsigned mine = (__ballot_sync(gmask, accept) >> (lane & 24)) & 0xFFu;
        if (accept)
          pair_store<kMode>(i, cnt + __popc(mine & ((1u << g) - 1u)), j, packed, range_bad,
                            seed_i, nbr, shift, stage, cap, status);
        cnt += __popc(mine);
      }
    } else if (g == 0) {
      cnt = pairs_walk<kMode, false>(bp, i, t, pi, cx0, cy0, cz0, q0, q1, q2, Ebase, eA, pos4,
                                     spos, swrap, cell_start, seed_i, nbr, shift, stage, cap,
                                     status);
    }
    cnt = __shfl_sync(gmask, cnt, 0, G);
  }
  if (kMode != kPairsFill) {
    // as nl_pairs: counts (clamped for a captured build), the largest count,
    // the refusal of 2^26 or more per atom and the 64-bit total; one atomic
    // per warp for the last two
    const bool lead = g == 0 && i >= 0;
    if (lead) {
      counts[i] = clamp ? min(cnt, cap) : cnt;
      if (cnt >= (1 << 26)) atomicOr(&status[1], 8);
    }
    const unsigned mx = __reduce_max_sync(0xffffffffu, lead ? (unsigned)cnt : 0u);
    const unsigned wsum =
        __reduce_add_sync(0xffffffffu, lead ? (unsigned)min(cnt, (1 << 26) - 1) : 0u);
    if (lane == 0) {
      atomicMax(&status[0], (int)min(mx, (unsigned)INT_MAX));
      atomicAdd(reinterpret_cast<unsigned long long *>(status + 6), (unsigned long long)wsum);
    }
  }
}

// CSR from the staged entries (every atom has at most cap of them).
// Staged entries to the CSR: G consecutive lanes per atom take its entries k
// = lane, lane + G, ..., so that a group's loads of the staged row and its
// stores to nbr / shift are contiguous runs (one thread per atom wrote each
// entry to a different sector of its warp's stores).
template <int G>
__global__ void nl_compact(int nat, int cap, const int *__restrict__ seed,
                           const int2 *__restrict__ stage, int *__restrict__ nbr,
                           int *__restrict__ shift) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(t / G), lane = (int)(t % G);
  if (i >= nat) return;
  const int s = seed[i], n = seed[i + 1] - s;
  const int2 *src = stage + (size_t)i * cap;
  for (int k = lane; k < n; k += G) {
    const int2 v = src[k];
    nbr[s + k] = v.x;
    shift[s + k] = v.y;
  }
}

// Lanes per atom for nl_compact from the staging capacity (an upper bound of
// the entries per atom, 1.25 x the previous maximum + 4).
cudaError_t launch_compact(int nat, int cap, const int *seed, const int2 *stage, int *nbr,
                           int *shift, cudaStream_t stream) {
  const int g = cap <= 16 ? 4 : cap <= 48 ? 8 : 16;
  const unsigned blocks = (unsigned)(((int64_t)nat * g + 127) / 128);
  if (g == 4)
    nl_compact<4><<<blocks, 128, 0, stream>>>(nat, cap, seed, stage, nbr, shift);
  else if (g == 8)
    nl_compact<8><<<blocks, 128, 0, stream>>>(nat, cap, seed, stage, nbr, shift);
  else
    nl_compact<16><<<blocks, 128, 0, stream>>>(nat, cap, seed, stage, nbr, shift);
  note_launch();
  return cudaGetLastError();
}

// nl_compact and the reverse index in one pass: entry k of atom i, staged as
// (j, s) at stage[i cap + k], goes to nbr / shift at seed[i] + k, and its
// reverse (j -> i, -s) is looked up among j's staged entries instead of in the
// compacted arrays: rev = seed[j] + its position.  Four entries of i at a
// time per thread, so that their loads (seed[j], then the first 32-byte
// sector of j's staged row: its first four entries; cap is a multiple of 4)
// overlap.
#ifndef GB_COMPACT_LANES
#define GB_COMPACT_LANES 2
#endif
constexpr int kCompactLanes = GB_COMPACT_LANES;  // threads per atom

__global__ void nl_compact_reverse(int nat, int cap, const int *__restrict__ seed,
                                   const int2 *__restrict__ stage, int *__restrict__ nbr,
                                   int *__restrict__ shift, int *__restrict__ rev,
                                   int *__restrict__ status) {
  // kCompactLanes threads per atom take its entries in turn (entry k on lane
  // k mod kCompactLanes), four at a time
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = t / kCompactLanes, lane = t % kCompactLanes;
  if (i >= nat) return;
  const int s = seed[i], n = seed[i + 1] - s;
  const int2 *src = stage + (size_t)i * cap;
  for (int k0 = lane; k0 < n; k0 += 4 * kCompactLanes) {
    int2 v[4];
    int want[4], cj[4], nj[4], found[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = k0 + q * kCompactLanes;
      v[q] = k < n ? src[k] : make_int2(i, 0);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = k0 + q * kCompactLanes;
      if (k < n) {
        nbr[s + k] = v[q].x;
        shift[s + k] = v[q].y;
      }
      int s0, s1, s2;
      unpack_shift(v[q].y, s0, s1, s2);
      want[q] = pack_shift(-s0, -s1, -s2);
      cj[q] = seed[v[q].x];
      nj[q] = k < n ? seed[v[q].x + 1] - cj[q] : 0;
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      found[q] = -1;
      if (nj[q] > 0) {
        const int4 *row = reinterpret_cast<const int4 *>(stage + (size_t)v[q].x * cap);
        const int4 e01 = row[0], e23 = row[1];
        const int ex[4] = {e01.x, e01.z, e23.x, e23.z}, ey[4] = {e01.y, e01.w, e23.y, e23.w};
#pragma unroll
        for (int c = 3; c >= 0; c--)
          if (c < nj[q] && ex[c] == i && ey[c] == want[q]) found[q] = c;
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int k = k0 + q * kCompactLanes;
      if (k >= n) continue;
      const int2 *row = stage + (size_t)v[q].x * cap;
      for (int c = 4; c < nj[q] && found[q] < 0; c++) {
        const int2 e = row[c];
        if (e.x == i && e.y == want[q]) found[q] = c;
      }
      if (found[q] < 0) atomicOr(&status[1], 4);
      rev[s + k] = found[q] < 0 ? -1 : cj[q] + found[q];
    }
  }
}

// rev[b] = entry (j -> i, -s) of the entry b = (i -> j, s).
// One thread per atom i: each entry b = (i -> j, s) searches atom j's entries
// for (j -> i, -s), four candidates per step.
__global__ void nl_reverse(int nat, const int *__restrict__ seed, const int *__restrict__ nbr,
                           const int *__restrict__ shift, int *__restrict__ rev,
                           int *__restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const int b1 = seed[i + 1];
  for (int b = seed[i]; b < b1; b++) {
    const int j = nbr[b];
    int s0, s1, s2;
    unpack_shift(shift[b], s0, s1, s2);
    const int want = pack_shift(-s0, -s1, -s2);
    const int c0 = seed[j], c1 = seed[j + 1];
    int found = -1;
    for (int c = c0; c < c1 && found < 0; c += 4) {
      int nj[4], sj[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        nj[q] = c + q < c1 ? nbr[c + q] : -1;
        sj[q] = c + q < c1 ? shift[c + q] : 0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (found < 0 && nj[q] == i && sj[q] == want) found = c + q;
    }
    if (found < 0) atomicOr(&status[1], 4);
    rev[b] = found;
  }
}

// The same for long lists (large cutoffs, e.g. the screened potentials): a
// warp per atom i, its lanes over the entries of i.
__global__ void nl_reverse_dense(int nat, const int *__restrict__ seed,
                                 const int *__restrict__ nbr, const int *__restrict__ shift,
                                 int *__restrict__ rev, int *__restrict__ status) {
  const int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= nat) return;
  const int b1 = seed[i + 1];
  for (int b = seed[i] + lane; b < b1; b += 32) {
    const int j = nbr[b];
    int s0, s1, s2;
    unpack_shift(shift[b], s0, s1, s2);
    const int want = pack_shift(-s0, -s1, -s2);
    const int c0 = seed[j], c1 = seed[j + 1];
    int found = -1;
    for (int c = c0; c < c1 && found < 0; c += 4) {
      int nj[4], sj[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        nj[q] = c + q < c1 ? nbr[c + q] : -1;
        sj[q] = c + q < c1 ? shift[c + q] : 0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (found < 0 && nj[q] == i && sj[q] == want) found = c + q;
    }
    if (found < 0) atomicOr(&status[1], 4);
    rev[b] = found;
  }
}

}  // namespace

// Host-side binning_init (python_neighbors.f90:765-871) for one cell:
// n_cells = max(3, int(|a_k| / cutoff)), rec_cell_size = n_cells * Bbox,
// stencil half-widths from the cell's plane spacings; plus the derived
// fields of the pair search.  cell_base offsets the cell numbers (batches).
int bin_params(const double A[3][3], const double B[3][3], const int pbc[3], double cutoff,
               int cell_base, BinParams &bp) {
  const double bin_size = cutoff;
  double box_size[3];
  for (int x = 0; x < 3; x++) {
    double s = 0.0;
    for (int a = 0; a < 3; a++) s = s + A[a][x] * A[a][x];
    box_size[x] = std::sqrt(s);
  }
  for (int x = 0; x < 3; x++) {
    double v = box_size[x] / bin_size;
    int nc = v > 1e6 ? 1000000 : (int)v;
    bp.n[x] = nc < 3 ? 3 : nc;
  }
  double cs[3][3];
  for (int x = 0; x < 3; x++) {
    for (int a = 0; a < 3; a++) cs[a][x] = A[a][x] / bp.n[x];
    for (int k = 0; k < 3; k++) bp.rec[x][k] = B[x][k] * bp.n[x];
  }
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
  for (int a = 0; a < 3; a++) {
    c1[a] = cs[a][0];
    c2[a] = cs[a][1];
    c3[a] = cs[a][2];
  }
  cross(c2, c3, nx);
  cross(c3, c1, ny);
  cross(c1, c2, nz);
  const double cv = dot(c1, nx);
  const double dnx = dot(nx, nx), dny = dot(ny, ny), dnz = dot(nz, nz);
  for (int a = 0; a < 3; a++) {
    nx[a] = cv * nx[a] / dnx;
    ny[a] = cv * ny[a] / dny;
    nz[a] = cv * nz[a] / dnz;
  }
  bp.dx = (int)(cutoff / std::sqrt(dot(nx, nx))) + 1;
  bp.dy = (int)(cutoff / std::sqrt(dot(ny, ny))) + 1;
  bp.dz = (int)(cutoff / std::sqrt(dot(nz, nz))) + 1;
  if ((long long)bp.n[0] * bp.n[1] * bp.n[2] > (1ll << 28)) {
    set_error("neighbors_update: too many cells (cell or cutoff out of range)");
    return GB_ERROR_DOMAIN;
  }
  if ((2ll * bp.dx + 1) * (2ll * bp.dy + 1) * (2ll * bp.dz + 1) > 100000000ll) {
    set_error("neighbors_update: cutoff too large for this cell");
    return GB_ERROR_DOMAIN;
  }
  bp.cell_base = cell_base;
  bp.Amax = 0.0f;
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) {
      bp.recf[a][k] = (float)bp.rec[a][k];
      bp.A[a][k] = A[a][k];
      bp.Af[a][k] = (float)A[a][k];
      bp.Amax = std::max(bp.Amax, std::fabs(bp.Af[a][k]));
    }
  for (int k = 0; k < 3; k++) bp.pbc[k] = pbc[k];
  bp.cutoff_sq = cutoff * cutoff;
  bp.cutoff_f = (float)(cutoff * (1.0 + 1e-6));
  bp.cutoff_sq_lo = (float)(bp.cutoff_sq * (1.0 - 1e-6));
  bp.cutoff_sq_hi = (float)(bp.cutoff_sq * (1.0 + 1e-6));
  return 0;
}

// Builds the list of nat atoms at r (device, (nat,3)) on the stream.  A
// batch passes per-structure parameters bps (device) and the atoms'
// structure ids sid; bp0 is then unused.
int nl_build(Neighbors &nl, int nat, const double *r, const BinParams &bp0,
             const BinParams *bps, const int *sid, int ncells, cudaStream_t stream,
             bool capture) {
  const bool batch = bps != nullptr;
  if (capture && nl.stage_cap <= 0) {
    set_error("nl_build: a captured build needs the staged single pass (build once first)");
    return GB_ERROR_ARGUMENT;
  }
  GB_CHECK(nl.pos4.ensure(sizeof(Pos4) * std::max(nat, 1)));
  if (nl.want_posff) GB_CHECK(nl.posff.ensure(sizeof(float4) * 2 * std::max(nat, 1)));
  nl.posff_valid = nl.want_posff;
  GB_CHECK(nl.atom_cell.ensure(sizeof(int) * std::max(nat, 1)));
  GB_CHECK(nl.atom_wrap.ensure(sizeof(int) * std::max(nat, 1)));
  GB_CHECK(nl.cell_count.ensure(sizeof(int) * (ncells + 1)));
  GB_CHECK(nl.cell_start.ensure(sizeof(int) * (ncells + 1)));
  GB_CHECK(nl.cell_atoms.ensure(sizeof(int) * 2 * std::max(nat, 1)));
  GB_CHECK(nl.counts.ensure(sizeof(int) * (nat + 1)));
  GB_CHECK(nl.spos.ensure(sizeof(float4) * std::max(nat, 1)));
  GB_CHECK(nl.swrap.ensure(sizeof(int) * std::max(nat, 1)));
  GB_CHECK(nl.seed.ensure(sizeof(int) * (nat + 1)));
  GB_CHECK(nl.stats.ensure(sizeof(int) * 16 + sizeof(int) * (size_t)(ncells + 1)));
  GB_CHECK(nl.hstats.ensure(sizeof(int) * 16));
  // [0] maxz [1] flags [2] n_big [3] max |coordinate| [4] reverse-index flags
  // [6..7] 64-bit entry total [8..9] tile plan (most bonds, most slots)
  int *status = nl.stats.as<int>();
  int *big_cells = status + 16;
  GB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 16, stream));
  nl.plan_ready = false;
  GB_CUDA(cudaMemsetAsync(nl.cell_count.p, 0, sizeof(int) * (ncells + 1), stream));
  const int T = 256;
  const int nb = (nat + T - 1) / T;
  float4 *posff = nl.want_posff ? nl.posff.as<float4>() : nullptr;
  if (nat > 0) {
    if (batch)
      nl_assign_cells<true><<<nb, T, 0, stream>>>(
          nat, r, bp0, bps, sid, nl.pos4.as<Pos4>(), posff, nl.atom_cell.as<int>(),
          nl.atom_wrap.as<int>(), nl.cell_count.as<int>(), status);
    else
      nl_assign_cells<false><<<nb, T, 0, stream>>>(
          nat, r, bp0, nullptr, nullptr, nl.pos4.as<Pos4>(), posff, nl.atom_cell.as<int>(),
          nl.atom_wrap.as<int>(), nl.cell_count.as<int>(), status);
    note_launch();
  }
  GB_CHECK(exclusive_scan_i32(nl.cell_count.as<int>(), nl.cell_start.as<int>(), ncells,
                              nl.scan_tmp, stream));
  GB_CUDA(cudaMemsetAsync(nl.cell_count.p, 0, sizeof(int) * (ncells + 1), stream));
  int *cell_atoms = nl.cell_atoms.as<int>();
  auto pairs = [&](auto mode_tag, int *counts, const int *seed, int *nbr, int *shift,
                   int2 *stage, int cap, int clamp = 0) {
    constexpr int kMode = decltype(mode_tag)::value;
    if (batch)
      nl_pairs<kMode, true><<<(nat + kPairsThreads - 1) / kPairsThreads, kPairsThreads, 0,
                              stream>>>(
          nat, bp0, bps, sid, nl.pos4.as<Pos4>(), nl.atom_cell.as<int>(), nl.spos.as<float4>(),
          nl.swrap.as<int>(), nl.cell_start.as<int>(), counts, seed, nbr, shift, stage, cap,
          clamp, status);
    else if (nat <= kPairGroupMaxAtoms)
      nl_pairs_grp<kMode><<<(unsigned)(((int64_t)nat * kPairLanes + 127) / 128), 128, 0,
                            stream>>>(nat, bp0, nl.pos4.as<Pos4>(), nl.atom_cell.as<int>(),
                                      nl.spos.as<float4>(), nl.swrap.as<int>(),
                                      nl.cell_start.as<int>(), counts, seed, nbr, shift, stage,
                                      cap, clamp, status);
    else
      nl_pairs<kMode, false><<<(nat + kPairsThreads - 1) / kPairsThreads, kPairsThreads, 0,
                               stream>>>(
          nat, bp0, nullptr, nullptr, nl.pos4.as<Pos4>(), nl.atom_cell.as<int>(),
          nl.spos.as<float4>(), nl.swrap.as<int>(), nl.cell_start.as<int>(), counts, seed, nbr,
          shift, stage, cap, clamp, status);
    note_launch();
  };
  if (nat > 0) {
    nl_scatter<<<nb, T, 0, stream>>>(nat, nl.atom_cell.as<int>(), nl.cell_start.as<int>(),
                                     nl.cell_count.as<int>(), cell_atoms);
    note_launch();
    nl_sort_cells<<<(ncells + T - 1) / T, T, 0, stream>>>(
        ncells, nl.cell_start.as<int>(), cell_atoms, big_cells, &status[2], nl.pos4.as<Pos4>(),
        nl.atom_wrap.as<int>(), nl.spos.as<float4>(), nl.swrap.as<int>());
    note_launch();
    nl_sort_big_cells<<<std::min(ncells, 128), 256, 0, stream>>>(
        big_cells, &status[2], nl.cell_start.as<int>(), cell_atoms, cell_atoms + nat,
        nl.pos4.as<Pos4>(), nl.atom_wrap.as<int>(), nl.spos.as<float4>(), nl.swrap.as<int>());
    note_launch();
    // Single pass (count + staged entries) once a previous build has sized
    // the per-atom capacity; count-only pass otherwise.
    if (nl.stage_cap > 0) {
      GB_CHECK(nl.stage.ensure(sizeof(int2) * (size_t)nat * nl.stage_cap));
      pairs(std::integral_constant<int, kPairsCountStage>(), nl.counts.as<int>(), nullptr,
            nullptr, nullptr, nl.stage.as<int2>(), nl.stage_cap, capture ? 1 : 0);
    } else {
      pairs(std::integral_constant<int, kPairsCount>(), nl.counts.as<int>(), nullptr, nullptr,
            nullptr, nullptr, 0);
    }
  }
  GB_CHECK(exclusive_scan_i32(nl.counts.as<int>(), nl.seed.as<int>(), nat, nl.scan_tmp, stream));
  int *hs = nl.hstats.as<int>();
  if (capture) {
    // No host decisions: compact the staged entries (at most cap per atom, so
    // at most nat * cap in all; the buffers were sized for that) and leave
    // the status words in hstats for the caller to check after the replay.
    if (nat > 0 && nl.want_rev && nl.stage_cap <= 32) {
      // (rev sized for nat * cap entries by the caller, like nbr and shift)
      nl_compact_reverse<<<(unsigned)(((int64_t)nat * kCompactLanes + 127) / 128), 128, 0,
                           stream>>>(
          nat, nl.stage_cap, nl.seed.as<int>(), nl.stage.as<int2>(), nl.nbr.as<int>(),
          nl.shift.as<int>(), nl.rev.as<int>(), status + 3);
      note_launch();
      GB_CUDA(cudaMemcpyAsync(hs + 5, status + 4, sizeof(int), cudaMemcpyDeviceToHost, stream));
      nl.rev_pending = true;
    } else if (nat > 0) {
      GB_CUDA(launch_compact(nat, nl.stage_cap, nl.seed.as<int>(), nl.stage.as<int2>(),
                             nl.nbr.as<int>(), nl.shift.as<int>(), stream));
    }
    GB_CUDA(cudaMemcpyAsync(hs, status, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
    GB_CUDA(cudaMemcpyAsync(hs + 4, nl.seed.as<int>() + nat, sizeof(int), cudaMemcpyDeviceToHost,
                            stream));
    return 0;
  }
  // The bond-order tile plan of this list, for the tiles the potential asked
  // for, goes back with the list's sizes (one host synchronisation for both).
  const int plan_apt = batch ? 0 : nl.plan_apt;
  if (plan_apt > 0 && nat > 0)
    GB_CHECK(bop_plan_launch(nat, plan_apt, (nat + plan_apt - 1) / plan_apt, nullptr,
                             nl.seed.as<int>(), status + 8, stream));
  // Read back: maxz, flags, n_big, total entries (int32 scan and 64-bit sum),
  // the tile plan.
  GB_CUDA(cudaMemcpyAsync(hs, status, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
  GB_CUDA(cudaMemcpyAsync(hs + 4, nl.seed.as<int>() + nat, sizeof(int), cudaMemcpyDeviceToHost,
                          stream));
  GB_CUDA(cudaMemcpyAsync(hs + 6, status + 6, sizeof(int) * 4, cudaMemcpyDeviceToHost, stream));
  GB_CUDA(cudaStreamSynchronize(stream));
  GB_CUDA(cudaGetLastError());
  if (plan_apt > 0 && nat > 0) {
    nl.hplan[0] = hs[8];
    nl.hplan[1] = hs[9];
    nl.plan_done_apt = plan_apt;
    nl.plan_ready = true;
  }
  if (hs[1] & 1) {
    set_error("Non-finite particle position.");
    return GB_ERROR_DOMAIN;
  }
  if (hs[1] & 2) {
    set_error("Particle or image shift outside the supported range (|shift| <= 511 cells).");
    return GB_ERROR_DOMAIN;
  }
  unsigned long long total64 = 0;
  std::memcpy(&total64, hs + 6, sizeof(total64));
  if ((hs[1] & 8) || total64 > (unsigned long long)INT_MAX) {
    set_error("Neighbor list overflow (" + std::to_string(total64) +
              " entries, more than the 2^31 - 1 of the int32 offsets).");
    return GB_ERROR_CAPACITY;
  }
  const int64_t total = hs[4];
  GB_CHECK(nl.nbr.ensure(sizeof(int) * std::max<int64_t>(total, 1)));
  GB_CHECK(nl.shift.ensure(sizeof(int) * std::max<int64_t>(total, 1)));
  const int maxz = hs[0];
  if (nat > 0) {
    if (nl.stage_cap > 0 && maxz <= nl.stage_cap && nl.want_rev &&
        total <= 24 * (int64_t)nat) {
      // compaction and reverse index together (the symmetry flag is read
      // by the caller's next synchronisation, as after neighbors_build_reverse)
      GB_CHECK(nl.rev.ensure(sizeof(int) * std::max<int64_t>(total, 1)));
      nl_compact_reverse<<<(unsigned)(((int64_t)nat * kCompactLanes + 127) / 128), 128, 0,
                           stream>>>(
          nat, nl.stage_cap, nl.seed.as<int>(), nl.stage.as<int2>(), nl.nbr.as<int>(),
          nl.shift.as<int>(), nl.rev.as<int>(), status + 3);
      note_launch();
      GB_CUDA(cudaMemcpyAsync(hs + 5, status + 4, sizeof(int), cudaMemcpyDeviceToHost, stream));
      nl.rev_pending = true;
    } else if (nl.stage_cap > 0 && maxz <= nl.stage_cap) {
      GB_CUDA(launch_compact(nat, nl.stage_cap, nl.seed.as<int>(), nl.stage.as<int2>(),
                             nl.nbr.as<int>(), nl.shift.as<int>(), stream));
    } else {
      pairs(std::integral_constant<int, kPairsFill>(), nullptr, nl.seed.as<int>(),
            nl.nbr.as<int>(), nl.shift.as<int>(), nullptr, 0);
    }
  }
  // Capacity of the next build's single pass: this build's maximum plus a
  // margin, while the stage stays below kStageMaxBytes.
  {
    const int cap = ((maxz + maxz / 4 + 4) + 3) & ~3;
    nl.stage_cap = (size_t)nat * cap * sizeof(int2) <= kStageMaxBytes ? cap : 0;
  }
  GB_CUDA(cudaGetLastError());
  nl.nentries = total;
  nl.maxz = maxz;
  return 0;
}

int neighbors_update(Neighbors &nl, Particles &p, cudaStream_t stream) {
  if (!p.cell_set) {
    set_error("neighbors_update: cell not set");
    return GB_ERROR_ARGUMENT;
  }
  if (p.nat > 0 && !p.r.p) {
    set_error("neighbors_update: positions not set");
    return GB_ERROR_ARGUMENT;
  }
  if (nl.valid && nl.built_for == &p && nl.built_pos_rev == p.pos_rev &&
      nl.built_cell_rev == p.cell_rev && nl.built_nat == p.nat && nl.cutoff == nl.interaction_range)
    return 0;
  // cutoff = interaction_range + verlet_shell (0 on the Python path, :478)
  const double cutoff = nl.interaction_range;
  if (!(cutoff > 0.0)) {
    set_error("Cutoff needs to be larger than zero.");
    return GB_ERROR_ARGUMENT;
  }
  nl.valid = false;
  nl.rev_valid = false;
  nl.rev_pending = false;
  BinParams bp;
  GB_CHECK(bin_params(p.A, p.B, p.pbc, cutoff, 0, bp));
  for (int k = 0; k < 3; k++) nl.n_cells[k] = bp.n[k];
  std::memcpy(nl.rec, bp.rec, sizeof(nl.rec));
  nl.dx = bp.dx;
  nl.dy = bp.dy;
  nl.dz = bp.dz;
  const int ncells = bp.n[0] * bp.n[1] * bp.n[2];
  GB_CHECK(nl_build(nl, p.nat, p.r.as<double>(), bp, nullptr, nullptr, ncells, stream, false));
  nl.cutoff = cutoff;
  nl.valid = true;
  nl.built_for = &p;
  nl.built_pos_rev = p.pos_rev;
  nl.built_cell_rev = p.cell_rev;
  nl.built_nat = p.nat;
  return 0;
}

int neighbors_build_reverse(Neighbors &nl, int nat, cudaStream_t stream, bool sync) {
  if (nl.rev_valid || nl.rev_pending) return sync ? neighbors_check_reverse(nl, stream) : 0;
  GB_CHECK(nl.rev.ensure(sizeof(int) * std::max<int64_t>(nl.nentries, 1)));
  // The symmetry flag goes to stats[4] (the kernels set bit 4 of their
  // status[1]), so that the list build's own words stats[0..3] stay intact.
  int *status = nl.stats.as<int>() + 3;
  GB_CUDA(cudaMemsetAsync(status + 1, 0, sizeof(int), stream));
  if (nat > 0) {
    if (nl.nentries > 24 * (int64_t)nat)  // long lists: a warp per atom
      nl_reverse_dense<<<(unsigned)(((int64_t)nat * 32 + 127) / 128), 128, 0, stream>>>(
          nat, nl.seed.as<int>(), nl.nbr.as<int>(), nl.shift.as<int>(), nl.rev.as<int>(), status);
    else
      nl_reverse<<<(nat + 127) / 128, 128, 0, stream>>>(nat, nl.seed.as<int>(), nl.nbr.as<int>(),
                                                       nl.shift.as<int>(), nl.rev.as<int>(),
                                                       status);
    note_launch();
  }
  int *hs = nl.hstats.as<int>();
  // (hstats[5]: the list build's own status words stay in hstats[0..4])
  GB_CUDA(cudaMemcpyAsync(hs + 5, status + 1, sizeof(int), cudaMemcpyDeviceToHost, stream));
  nl.rev_pending = true;
  return sync ? neighbors_check_reverse(nl, stream) : 0;
}

int neighbors_check_reverse(Neighbors &nl, cudaStream_t stream) {
  if (!nl.rev_pending) return 0;
  if (stream) GB_CUDA(cudaStreamSynchronize(stream));
  nl.rev_pending = false;
  if (nl.hstats.as<int>()[5] & 4) {
    set_error("Internal error: neighbour list is not symmetric.");
    return GB_ERROR_UNSPECIFIED;
  }
  nl.rev_valid = true;
  return 0;
}

}  // namespace gb

// ===========================================================================
// C-ABI: particles and neighbours.
// ===========================================================================
using namespace gb;


static cudaStream_t particles_stream(Particles &p) {
  if (!p.stream) {
    cudaStreamCreateWithFlags(&p.stream, cudaStreamNonBlocking);
    p.own_stream = true;
  }
  return p.stream;
}

extern "C" {

const char *gb_get_error(void) { return g_error.c_str(); }
const char *gb_version(void) { return "atomistica_gb300 0.1.0 (sm_103a)"; }

uint64_t gb_kernel_launches(void) { return g_launches.load(); }

int gb_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int gb_particles_new(gb_particles_t **p) {
  clear_error();
  if (!p) return GB_ERROR_ARGUMENT;
  *p = new gb_particles;
  return 0;
}

void gb_particles_free(gb_particles_t *p) {
  if (!p) return;
  if (p->p.own_stream && p->p.stream) cudaStreamDestroy(p->p.stream);
  delete p;
}

int gb_particles_allocate(gb_particles_t *h, int nat) {
  clear_error();
  if (!h || nat < 0) {
    set_error("particles_allocate: invalid arguments");
    return GB_ERROR_ARGUMENT;
  }
  Particles &p = h->p;
  GB_CHECK(p.r.ensure(sizeof(double) * 3 * std::max(nat, 1)));
  GB_CHECK(p.Z.ensure(sizeof(int) * std::max(nat, 1)));
  p.nat = nat;
  p.hZ.assign(nat, 0);
  GB_CUDA(cudaMemsetAsync(p.r.p, 0, sizeof(double) * 3 * std::max(nat, 1), particles_stream(p)));
  GB_CUDA(cudaMemsetAsync(p.Z.p, 0, sizeof(int) * std::max(nat, 1), particles_stream(p)));
  GB_CUDA(cudaStreamSynchronize(particles_stream(p)));
  p.pos_rev++;
  p.z_rev++;
  return 0;
}

int gb_particles_get_nat(const gb_particles_t *h) { return h ? h->p.nat : -1; }

int gb_particles_set_cell(gb_particles_t *h, const double *cell, const int *pbc) {
  clear_error();
  if (!h || !cell) return GB_ERROR_ARGUMENT;
  Particles &p = h->p;
  double A[3][3];
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) A[a][k] = cell[3 * k + a];
  double B[3][3];
  if (cell_inverse(A, B) != 0) {
    set_error("Gauss elimination failed (singular cell).");
    return GB_ERROR_ARGUMENT;
  }
  bool changed = !p.cell_set || std::memcmp(A, p.A, sizeof(A)) != 0;
  std::memcpy(p.A, A, sizeof(A));
  std::memcpy(p.B, B, sizeof(B));
  for (int k = 0; k < 3; k++) {
    int v = pbc ? (pbc[k] != 0) : 1;
    if (v != p.pbc[k]) changed = true;
    p.pbc[k] = v;
  }
  p.cell_set = true;
  if (changed) p.cell_rev++;
  return 0;
}

int gb_particles_set_positions(gb_particles_t *h, const double *r) {
  clear_error();
  if (!h || (!r && h->p.nat > 0)) return GB_ERROR_ARGUMENT;
  Particles &p = h->p;
  if (p.nat == 0) {
    p.pos_rev++;
    return 0;
  }
  cudaStream_t s = particles_stream(p);
  const size_t bytes = sizeof(double) * 3 * p.nat;
  GB_CUDA(cudaMemcpyAsync(p.r.p, r, bytes, cudaMemcpyDefault, s));
  if (!is_device_ptr(r)) GB_CUDA(cudaStreamSynchronize(s));
  p.pos_rev++;
  return 0;
}

int gb_particles_set_Z(gb_particles_t *h, const int *Z) {
  clear_error();
  if (!h || (!Z && h->p.nat > 0)) return GB_ERROR_ARGUMENT;
  Particles &p = h->p;
  if (p.nat == 0) return 0;
  cudaStream_t s = particles_stream(p);
  GB_CUDA(cudaMemcpyAsync(p.hZ.data(), Z, sizeof(int) * p.nat, cudaMemcpyDefault, s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaMemcpyAsync(p.Z.p, p.hZ.data(), sizeof(int) * p.nat, cudaMemcpyHostToDevice, s));
  GB_CUDA(cudaStreamSynchronize(s));
  p.z_rev++;
  return 0;
}

int gb_particles_set_stream(gb_particles_t *h, void *stream) {
  if (!h) return GB_ERROR_ARGUMENT;
  Particles &p = h->p;
  if (p.own_stream && p.stream) cudaStreamDestroy(p.stream);
  p.own_stream = false;
  p.stream = (cudaStream_t)stream;
  if (!stream) particles_stream(p);
  return 0;
}

int gb_neighbors_new(gb_neighbors_t **nl, int avgn) {
  clear_error();
  if (!nl) return GB_ERROR_ARGUMENT;
  *nl = new gb_neighbors;
  (*nl)->nl.avgn = avgn > 0 ? avgn : 100;
  return 0;
}

void gb_neighbors_free(gb_neighbors_t *nl) { delete nl; }

int gb_neighbors_request_interaction_range(gb_neighbors_t *h, double cutoff) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  if (cutoff > h->nl.interaction_range) {
    h->nl.interaction_range = cutoff;
    h->nl.valid = false;
  }
  return 0;
}

double gb_neighbors_get_interaction_range(const gb_neighbors_t *h) {
  return h ? h->nl.interaction_range : -1.0;
}

int gb_neighbors_update(gb_neighbors_t *h, gb_particles_t *p) {
  clear_error();
  if (!h || !p) return GB_ERROR_ARGUMENT;
  cudaStream_t s = h->nl.stream ? h->nl.stream : particles_stream(p->p);
  if (p->p.stream && p->p.stream != s) GB_CUDA(cudaStreamSynchronize(p->p.stream));
  return neighbors_update(h->nl, p->p, s);
}

int64_t gb_neighbors_get_size(const gb_neighbors_t *h) {
  return (h && h->nl.valid) ? h->nl.nentries : -1;
}

namespace gb {
namespace {
__global__ void nl_export(int nat, const int *__restrict__ seed, const int *__restrict__ nbr,
                          const int *__restrict__ shift, int64_t *__restrict__ oseed,
                          int *__restrict__ oj, int *__restrict__ odc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nat) return;
  if (oseed) oseed[i] = seed[i];
  if (i == nat) return;
  for (int b = seed[i]; b < seed[i + 1]; b++) {
    if (oj) oj[b] = nbr[b];
    if (odc) {
      int s0, s1, s2;
      unpack_shift(shift[b], s0, s1, s2);
      odc[3 * b] = s0;
      odc[3 * b + 1] = s1;
      odc[3 * b + 2] = s2;
    }
  }
}
}  // namespace
}  // namespace gb

int gb_neighbors_get(gb_neighbors_t *h, gb_particles_t *ph, int64_t *seed, int *j, int *dc) {
  clear_error();
  if (!h || !ph) return GB_ERROR_ARGUMENT;
  Neighbors &nl = h->nl;
  Particles &p = ph->p;
  cudaStream_t s = nl.stream ? nl.stream : particles_stream(p);
  GB_CHECK(neighbors_update(nl, p, s));
  const int nat = p.nat;
  const int64_t n = nl.nentries;
  DevBuf tmp;
  const size_t bs = sizeof(int64_t) * (nat + 1), bj = sizeof(int) * n, bd = sizeof(int) * 3 * n;
  GB_CHECK(tmp.ensure(bs + bj + bd + 64));
  char *base = tmp.as<char>();
  int64_t *dseed = (seed && is_device_ptr(seed)) ? seed : (int64_t *)base;
  int *dj = (j && is_device_ptr(j)) ? j : (int *)(base + bs);
  int *ddc = (dc && is_device_ptr(dc)) ? dc : (int *)(base + bs + bj);
  nl_export<<<(nat + 1 + 127) / 128, 128, 0, s>>>(nat, nl.seed.as<int>(), nl.nbr.as<int>(),
                                                 nl.shift.as<int>(), seed ? dseed : nullptr,
                                                 j ? dj : nullptr, dc ? ddc : nullptr);
  note_launch();
  GB_CUDA(cudaGetLastError());
  if (seed && dseed != seed) GB_CUDA(cudaMemcpyAsync(seed, dseed, bs, cudaMemcpyDeviceToHost, s));
  if (j && dj != j && n) GB_CUDA(cudaMemcpyAsync(j, dj, bj, cudaMemcpyDeviceToHost, s));
  if (dc && ddc != dc && n) GB_CUDA(cudaMemcpyAsync(dc, ddc, bd, cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int gb_neighbors_set_stream(gb_neighbors_t *h, void *stream) {
  if (!h) return GB_ERROR_ARGUMENT;
  h->nl.stream = (cudaStream_t)stream;
  return 0;
}

}  // extern "C"
