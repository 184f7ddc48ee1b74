// Tersoff / Kumagai energy, force and virial on GB300 (replaces BOP_KERNEL,
// src/potentials/bop/bop_kernel.f90:420-1628, non-screened branch).
//
// Work decomposition (one launch of bop_tile per call, then one gather):
//
//   bop_tile   one CTA per tile of `apt` consecutive atoms; a thread per bond
//              (directed neighbour entry), strided over the tile's bonds.
//     phase 1  bond geometry from positions and integer image shifts, with
//              r^2 evaluated exactly as the neighbour test (FP64, no FMA), the
//              cutoff regions of pass 1 (:627-680, :997-1058) and trig_off.
//              Unit vectors, lengths and cutoff values go to shared memory.
//     phase 2  per bond ij: the k loop over the other bonds of i (:1171-1343)
//              gives zeta_ij, d zeta/d r_j and, per (ij, ik), d zeta/d r_k,
//              which is kept in shared memory (no per-triplet global
//              storage).  Then b_ij, P_ij = d E / d zeta_ij (bo, :1356),
//              the pair energy (:1366) and the radial force (:1376-1402).
//     phase 3  per bond ik: G_ik = force that centre i exerts on the end atom
//              of bond ik = (its own j-role term) - sum_j P_ij d zeta_ij/d r_k.
//   bop_gather one thread per atom a: F_a = sum_{b in out(a)} (G[rev b] - G[b]),
//              using the reverse-entry index of the symmetric list.  The self
//              term -sum G[b] equals the reference's f_i by translation
//              invariance.  No atomics anywhere: results are bitwise
//              reproducible run to run.
//
// The total virial is -sum_b r_b (x) G_b (equal to sum_ij w_ij of :1404); the
// per-atom virial (requested) follows the reference exactly: w_ij = r_ij (x)
// df - P_ij wijb_ij, half to i and half to j (:1510-1518).
//
// Precision forms: bop_tile (FP64 drop-in, this file) and bop_tile_mx (mixed:
// FP32 three-body terms, float-float geometry, pair terms, bond order and
// accumulation on the FP32 pipe, FP64 recomputation of the bonds whose
// estimated error is large; bop_mixed.cuh).

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "bop_math.h"
#include "ff.h"
#include "ff_tables.h"
#include "potential.h"

namespace gb {

namespace {

constexpr int kBopThreads = 128;
// Largest dynamic shared memory a tile kernel is allowed to request (bytes).
constexpr size_t kSmemBudgetAll = 208 * 1024;
constexpr int kMaxApt = 64;

// Bond meta word: owner local atom (bits 0-7), pair type (8-11), flags
// (12: in short list, 13: active as ij, 14: usable as k), maskfac (16-17).
constexpr int kFlagShort = 1 << 12;
constexpr int kFlagIJ = 1 << 13;
constexpr int kFlagK = 1 << 14;

struct BopArgs {
  int nat;
  int apt;
  const Pos4 *pos;
  const int *el;
  const int *seed;
  const int *nbr;
  const int *shift;
  const int *mask;
  double A[3][3];
  double *G;        // 3 per bond
  double *ebond;    // 1 per bond
  double *wbond;    // 9 per bond (per-atom virial only)
  double *frbond;   // 3 per bond (f_per_bond only)
  double *tile_part;  // 10 per tile
  // Batches of structures: tile t covers atoms [tile_atom0[t], tile_atom0[t+1])
  // of structure tile_struct[t], whose cell is Acells[9 s ..] (FP64) /
  // Acells_ff (float-float pairs); the mixed kernel then writes one partial
  // row per tile.  nullptr for a single structure (uniform tiles of apt).
  const int *tile_atom0 = nullptr;
  const int *tile_struct = nullptr;
  const double *Acells = nullptr;
  const float2 *Acells_ff = nullptr;
  int ntiles = 0;
  // Batches, mixed kernel: a counter (zero at launch) from which the
  // persistent CTAs take their tiles in turn; nullptr = the static schedule.
  int *tile_queue = nullptr;
};

__device__ __forceinline__ void tile_range(const BopArgs &a, int tile, int &a0, int &a1) {
  if (a.tile_atom0) {
    a0 = a.tile_atom0[tile];
    a1 = a.tile_atom0[tile + 1];
  } else {
    a0 = tile * a.apt;
    a1 = min(a0 + a.apt, a.nat);
  }
}

// Shared-memory layout of one tile (nbt bonds, ntrip (ij, ik) slots).
struct SmemLayout {
  int *aseed, *toff, *el, *meta, *hot;
  double *rn64, *r64, *rinv64, *fc64, *dfc64, *P, *G, *E;  // per bond
  double *t;                                               // 3 per (ij, ik) slot
  int nbt, ntrip;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

template <class R>
__host__ __device__ inline size_t bop_smem_bytes(int nbt, int ntrip) {
  size_t o = align16(sizeof(int) * (3 * kMaxApt + 2 + 2 * (size_t)nbt));
  o += align16(sizeof(double) * (size_t)nbt * 12);
  o += align16(sizeof(double) * (size_t)ntrip * 3);
  return o + 64;
}

__device__ inline SmemLayout carve(unsigned char *sm, int nbt, int ntrip) {
  SmemLayout L;
  L.nbt = nbt;
  L.ntrip = ntrip;
  int *ip = reinterpret_cast<int *>(sm);
  L.aseed = ip;
  L.toff = ip + kMaxApt + 1;
  L.el = ip + 2 * kMaxApt + 2;
  L.meta = ip + 3 * kMaxApt + 2;
  L.hot = L.meta + nbt;
  size_t o = align16(sizeof(int) * (3 * kMaxApt + 2 + 2 * (size_t)nbt));
  double *dp = reinterpret_cast<double *>(sm + o);
  L.rn64 = dp;
  L.r64 = dp + 3 * nbt;
  L.rinv64 = dp + 4 * nbt;
  L.fc64 = dp + 5 * nbt;
  L.dfc64 = dp + 6 * nbt;
  L.P = dp + 7 * nbt;
  L.G = dp + 8 * nbt;
  L.E = dp + 11 * nbt;
  o += align16(sizeof(double) * (size_t)nbt * 12);
  L.t = reinterpret_cast<double *>(sm + o);
  return L;
}

// Deterministic block sum of NC doubles per thread into out[0..NC).
template <int NC>
__device__ inline void block_sum(double (&v)[NC], double *out, double *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int nw = kBopThreads / 32;
#pragma unroll
  for (int c = 0; c < NC; c++) {
    double x = v[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) scratch[wid * NC + c] = x;
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double s = 0.0;
    for (int w = 0; w < nw; w++) s += scratch[w * NC + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// k loop of bond ij = lb in FP64 (bop_kernel.f90:1171-1343): zeta_ij,
// d zeta/d r_j (dbj), d zeta_ij/d r_k into trow (component c at
// trow[c*ntrip + q]) and, for the per-atom virial, sum_k r_ik (x) dzeta/dr_k.
template <class Pot, bool kWat>
__device__ __forceinline__ void kloop64(const Pot &pot, const SmemLayout &L, int lb, int s, int z,
                                        int eli, double *trow, double &zeta, double dbj[3],
                                        double wk[9]) {
  const int nbt = L.nbt, ntrip = L.ntrip;
  const double rnij[3] = {L.rn64[lb], L.rn64[nbt + lb], L.rn64[2 * nbt + lb]};
  const double rlij = L.r64[lb], rinvj = L.rinv64[lb];
  const int ijpot = (L.meta[lb] >> 8) & 0xf;
  for (int q = 0; q < z; q++) {
    const int lk = s + q;
    if (lk == lb) continue;
    const int mk = L.meta[lk];
    if (!(mk & kFlagK)) {
      trow[q] = 0.0;
      trow[ntrip + q] = 0.0;
      trow[2 * ntrip + q] = 0.0;
      continue;
    }
    const int ikpot = (mk >> 8) & 0xf;
    const double rnik[3] = {L.rn64[lk], L.rn64[nbt + lk], L.rn64[2 * nbt + lk]};
    const double rlik = L.r64[lk], rinvk = L.rinv64[lk], fcik = L.fc64[lk], dfcik = L.dfc64[lk];
    double hv, dh;
    pot.template h<double>(eli, ijpot, ikpot, rlij - rlik, hv, dh);
    const double cs = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
    double gv, dg;
    pot.template g<double>(eli, ikpot, cs, gv, dg);
    const double dzfac = fcik * dg * hv;
    zeta += fcik * gv * hv;
    const double dzdrij = gv * fcik * dh;
    const double dzdrik = gv * (dfcik * hv - fcik * dh);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      // d cos/d r_j = (n_ik - cos n_ij)/r_ij ; d cos/d r_k = (n_ij - cos n_ik)/r_ik
      const double dcj = (rnik[c] - cs * rnij[c]) * rinvj;
      const double dck = (rnij[c] - cs * rnik[c]) * rinvk;
      dbj[c] += dzdrij * rnij[c] + dzfac * dcj;
      const double dk = dzdrik * rnik[c] + dzfac * dck;
      trow[c * ntrip + q] = dk;
      if (kWat)
#pragma unroll
        for (int c1 = 0; c1 < 3; c1++) wk[3 * c1 + c] += rnik[c1] * rlik * dk;
    }
  }
}

// Energy, radial force, G partial and per-bond outputs of bond ij
// (bop_kernel.f90:1356-1518).  The energy goes to L.E (summed later in a
// fixed order).
template <bool kWat, bool kPB>
__device__ __forceinline__ void finalize_bond(const BopArgs &a, const SmemLayout &L, int lb, int b,
                                              double bij, double P, const double dbj[3],
                                              const double wk[9], double VA, double dVA,
                                              double VR, double dVR) {
  const int nbt = L.nbt;
  const double fcij = L.fc64[lb], dfcij = L.dfc64[lb];
  const double e_b = 0.5 * fcij * (VR + bij * VA);
  const double dff = 0.5 * (dVR * fcij + bij * dVA * fcij + VR * dfcij + bij * VA * dfcij);
  const double rn64[3] = {L.rn64[lb], L.rn64[nbt + lb], L.rn64[2 * nbt + lb]};
  double dfr[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    dfr[c] = dff * rn64[c];
    L.G[c * nbt + lb] = -dfr[c] - P * dbj[c];
  }
  L.P[lb] = P;
  L.E[lb] = e_b;
  if (a.ebond) a.ebond[b] = e_b;
  if (kPB) {
    a.frbond[3 * (size_t)b] = dfr[0];
    a.frbond[3 * (size_t)b + 1] = dfr[1];
    a.frbond[3 * (size_t)b + 2] = dfr[2];
  }
  if (kWat) {
    // w_ij = r_ij (x) df - P wijb, wijb = -r_ij (x) dbidj - sum_k r_ik (x) dbidk
    const double r = L.r64[lb];
    const double rij[3] = {r * rn64[0], r * rn64[1], r * rn64[2]};
#pragma unroll
    for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
      for (int c2 = 0; c2 < 3; c2++)
        a.wbond[9 * (size_t)b + c1 + 3 * c2] =
            rij[c1] * dfr[c2] + P * (rij[c1] * dbj[c2]) + P * wk[3 * c1 + c2];
  }
}

// Mixed form: bonds whose estimated FP32 force error exceeds this (eV/A) are
// recomputed in float-float arithmetic.  The estimate is conservative: at
// the 2.33 g/cm^3, sigma = 0.25 A amorphous Si workload (1,048,576 atoms)
// the largest force error against FP64 is 1.6e-6 eV/A with 2e-6 (2.3 % of
// the bonds recomputed), 2.3e-6 with 4e-6 (0.6 %), 3.2e-6 with 6e-6
// (0.23 %), 3.5e-6 with 8e-6 (0.09 %), 4.8e-6 with 1.2e-5 (0.02 %), 5.2e-6
// with 1.6e-5 and 6.8e-6 with 3.2e-5 (no bond recomputed); on the 2048
// random packings 3.9e-6 (2e-6) and 4.2e-6 (6e-6 to 3.2e-5).  Each tile that
// has a hot bond runs the dependent float-float chain while its other warps
// wait, so fewer hot bonds mean fewer tiles paying for it: 1.2e-5 keeps the
// largest error below half the 1e-5 eV/A bound.
#ifndef GB_MX_HOT_THRESHOLD
#define GB_MX_HOT_THRESHOLD 1.2e-5f
#endif
constexpr float kHotThreshold = GB_MX_HOT_THRESHOLD;
// Juslin's W-C-H random packings (3 g/cm^3, 1.1 A minimum separation; H-H
// contacts with forces of hundreds of eV/A) reach 7.5e-6 eV/A with 8e-6 and
// 9.7e-6 with 1.2e-5: their threshold stays at 2e-6.
#ifndef GB_MX_HOT_THRESHOLD_JUSLIN
#define GB_MX_HOT_THRESHOLD_JUSLIN 2.0e-6f
#endif
constexpr float kHotThresholdJuslin = GB_MX_HOT_THRESHOLD_JUSLIN;
// 1: the mixed kernel takes a batch's tiles from a counter (dynamic
// schedule); 0: the static round-robin schedule for batches too.
#ifndef GB_MX_TILE_QUEUE
#define GB_MX_TILE_QUEUE 1
#endif

template <class Pot, class R, bool kWat, bool kPB>
__global__ void __launch_bounds__(kBopThreads)
    bop_tile(const BopArgs a, const Pot pot, int max_nbt, int max_ntrip, int *status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double red_scratch[(kBopThreads / 32) * 9];
  __shared__ double sA[3][3];  // this tile's cell
  static_assert(std::is_same<R, double>::value, "bop_tile is the FP64 form");
  const int tid = threadIdx.x;
  int a0, a1;
  tile_range(a, blockIdx.x, a0, a1);
  if (tid < 9)
    sA[tid / 3][tid % 3] = a.Acells ? a.Acells[9 * a.tile_struct[blockIdx.x] + tid]
                                    : a.A[tid / 3][tid % 3];
  const int na = a1 - a0;
  const int b0 = a.seed[a0];
  const int nbt = a.seed[a1] - b0;

  // Tile bookkeeping: local atom seeds, triplet offsets, owners.
  int ntrip = 0;
  {
    int *aseed = reinterpret_cast<int *>(sm);
    int *toff = aseed + kMaxApt + 1;
    int *el = aseed + 2 * kMaxApt + 2;
    for (int q = tid; q <= na; q += kBopThreads) aseed[q] = a.seed[a0 + q] - b0;
    for (int q = tid; q < na; q += kBopThreads) el[q] = a.el[a0 + q];
    __syncthreads();
    if (tid == 0) {
      int s = 0;
      for (int q = 0; q < na; q++) {
        toff[q] = s;
        const int z = aseed[q + 1] - aseed[q];
        s += trip_slots(z);
      }
      toff[na] = s;
    }
    __syncthreads();
    ntrip = toff[na];
  }
  if (nbt > max_nbt || ntrip > max_ntrip) {
    // Plan mismatch: report and leave this tile's outputs untouched.
    if (tid == 0) atomicOr(status, 2);
    return;
  }
  SmemLayout L = carve(sm, nbt, ntrip);
  for (int q = tid; q < na; q += kBopThreads)
    for (int lb = L.aseed[q]; lb < L.aseed[q + 1]; lb++) L.meta[lb] = q;
  __syncthreads();

  const int nel = pot.nel();

  // ---- Phase 1: bond geometry (pass 1, bop_kernel.f90:562-1068). ----
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int ai = L.meta[lb];
    const int i = a0 + ai;
    const int b = b0 + lb;
    const int j = a.nbr[b];
    const int eli = L.el[ai];
    const int elj = a.el[j];
    int meta = ai;
    double fc = 0.0, dfc = 0.0, r = 1.0, rinv = 1.0;
    double rn[3] = {0.0, 0.0, 0.0};
    if (eli >= 0 && elj >= 0) {
      const Pos4 pi = a.pos[i], pj = a.pos[j];
      int s0, s1, s2;
      unpack_shift(a.shift[b], s0, s1, s2);
      // rij = r_j - r_i - matmul(cell, dc) (:593), reference order, no FMA.
      double rij[3] = {__dsub_rn(pj.x, pi.x), __dsub_rn(pj.y, pi.y), __dsub_rn(pj.z, pi.z)};
      if (s0 | s1 | s2) {
        const double sx = s0, sy = s1, sz = s2;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          double as = __dmul_rn(sA[c][0], sx);
          as = __dadd_rn(as, __dmul_rn(sA[c][1], sy));
          as = __dadd_rn(as, __dmul_rn(sA[c][2], sz));
          rij[c] = __dsub_rn(rij[c], as);
        }
      }
      double r2 = __dmul_rn(rij[0], rij[0]);
      r2 = __dadd_rn(r2, __dmul_rn(rij[1], rij[1]));
      r2 = __dadd_rn(r2, __dmul_rn(rij[2], rij[2]));
      const int t = pot.pair(eli, elj);
      meta |= t << 8;
      bool in_short = false;
      if (r2 < pot.r1sq(t)) {
        fc = 1.0;
        dfc = 0.0;
        in_short = true;
      } else if (r2 < pot.r2sq(t)) {
        in_short = true;
      }
      if (in_short) {
        if (!(r2 < pot.r1sq(t)))
          trig_off(__dsqrt_rn(r2), pot.r1(t), pot.r2(t), pot.fac(t), fc, dfc);
        r = __dsqrt_rn(r2);
#pragma unroll
        for (int c = 0; c < 3; c++) rn[c] = rij[c] / r;
        rinv = 1.0 / r;
        int mf = 2;
        if (a.mask) {
          const int mi = a.mask[i], mj = a.mask[j];
          if (mi == 0 && mj == 0)
            mf = 0;
          else if (mi == 0 || mj == 0)
            mf = 1;
        }
        meta |= kFlagShort | (mf << 16);
        if (r < pot.r2(t)) {
          meta |= kFlagK;
          if (mf > 0) meta |= kFlagIJ;
        }
      }
    }
    L.meta[lb] = meta;
#pragma unroll
    for (int c = 0; c < 3; c++) L.rn64[c * nbt + lb] = rn[c];
    L.r64[lb] = r;
    L.rinv64[lb] = rinv;
    L.fc64[lb] = fc;
    L.dfc64[lb] = dfc;
  }
  __syncthreads();

  // ---- Phase 2: zeta, bond order, pair terms (pass 2, :1074-1529). ----
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int b = b0 + lb;
    const int meta = L.meta[lb];
    if (!(meta & kFlagIJ)) {
      L.P[lb] = 0.0;
      L.G[lb] = 0.0;
      L.G[nbt + lb] = 0.0;
      L.G[2 * nbt + lb] = 0.0;
      L.E[lb] = 0.0;
      if (a.ebond) a.ebond[b] = 0.0;
      if (kPB) {
        a.frbond[3 * (size_t)b] = 0.0;
        a.frbond[3 * (size_t)b + 1] = 0.0;
        a.frbond[3 * (size_t)b + 2] = 0.0;
      }
      if (kWat)
        for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)b + c] = 0.0;
      continue;
    }
    const int ai = meta & 0xff;
    const int t = (meta >> 8) & 0xf;
    const int mf = (meta >> 16) & 3;
    const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, p = lb - s;
    double *trow = L.t + L.toff[ai] + p * z;
    const int eli = L.el[ai];
    const double r = L.r64[lb];
    const double hm = 0.5 * mf;
    const double fcij = L.fc64[lb];
    double VA, dVA, VR, dVR;
    // VA, VR (tersoff_func.f90:32-78) scaled by maskfac/2 (:1133-1139)
    pot.VA(t, r, VA, dVA);
    pot.VR(t, r, VR, dVR);
    VA *= hm;
    dVA *= hm;
    VR *= hm;
    dVR *= hm;
    double zeta = 0.0, dbj[3] = {0.0, 0.0, 0.0}, wk[9];
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) wk[c] = 0.0;
    kloop64<Pot, kWat>(pot, L, lb, s, z, eli, trow, zeta, dbj, wk);
    double bij, P;
    pot.template bo<double>(eli, t, zeta, fcij, VA, bij, P);
    finalize_bond<kWat, kPB>(a, L, lb, b, bij, P, dbj, wk, VA, dVA, VR, dVR);
  }
  __syncthreads();

  // ---- Phase 3: forces on the end atoms (k-role), total virial. ----
  double eacc[1] = {0.0};
  double wacc[9];
#pragma unroll
  for (int c = 0; c < 9; c++) wacc[c] = 0.0;
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int b = b0 + lb;
    const int meta = L.meta[lb];
    eacc[0] += L.E[lb];
    double G[3] = {L.G[lb], L.G[nbt + lb], L.G[2 * nbt + lb]};
    if (meta & kFlagK) {
      const int ai = meta & 0xff;
      const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, q = lb - s;
      const double *tcol = L.t + L.toff[ai] + q;
      for (int p = 0; p < z; p++) {
        const int lp = s + p;
        if (lp == lb) continue;
        if (!(L.meta[lp] & kFlagIJ)) continue;
        const double P = L.P[lp];
        const double *tv = tcol + p * z;
#pragma unroll
        for (int c = 0; c < 3; c++) G[c] -= P * tv[c * ntrip];
      }
      const double r = L.r64[lb];
      const double rb[3] = {r * L.rn64[lb], r * L.rn64[nbt + lb], r * L.rn64[2 * nbt + lb]};
#pragma unroll
      for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
        for (int c2 = 0; c2 < 3; c2++) wacc[c1 + 3 * c2] -= rb[c1] * G[c2];
    }
    a.G[3 * (size_t)b] = G[0];
    a.G[3 * (size_t)b + 1] = G[1];
    a.G[3 * (size_t)b + 2] = G[2];
  }
  double *part = a.tile_part + 10 * (size_t)blockIdx.x;
  block_sum<1>(eacc, part, red_scratch);
  block_sum<9>(wacc, part + 1, red_scratch);
}

}  // namespace
}  // namespace gb

constexpr int kGatherThreads = 128;  // threads per block of the per-atom gathers
#include "bop_mixed.cuh"
#include "bop_scr.cuh"

namespace gb {
namespace {

// Per-atom gather through the reverse-entry index.
template <bool kEpa, bool kWat>
__global__ void bop_gather(int nat, const int *__restrict__ seed, const int *__restrict__ rev,
                           const double *__restrict__ G, const double *__restrict__ ebond,
                           const double *__restrict__ wbond, double *__restrict__ f,
                           double *__restrict__ epa, double *__restrict__ wpa, ReplayCheck chk,
                           int fset) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (replay_invalid(chk)) return;  // (uniform over the grid)
  double F[3] = {0.0, 0.0, 0.0};
  double E = 0.0;
  double W[9];
  if (kWat)
#pragma unroll
    for (int c = 0; c < 9; c++) W[c] = 0.0;
  const int s = i < nat ? seed[i] : 0, e = i < nat ? seed[i + 1] : 0;
  for (int b = s; b < e; b++) {
    const int rb = rev[b];
    if (rb < 0) continue;  // (an incomplete list; reported by the reverse build)
#pragma unroll
    for (int c = 0; c < 3; c++) F[c] += G[3 * (size_t)rb + c] - G[3 * (size_t)b + c];
    if (kEpa) E += ebond[b] + ebond[rb];
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) W[c] += wbond[9 * (size_t)b + c] + wbond[9 * (size_t)rb + c];
  }
  store_block_forces<kGatherThreads>(f, nat, F, fset);
  if (i >= nat) return;
  if (kEpa) epa[i] += 0.5 * E;
  if (kWat)
#pragma unroll
    for (int c = 0; c < 9; c++) wpa[9 * (size_t)i + c] += 0.5 * W[c];
}

// Tile plan: the largest bond count and (ij, ik) slot count of the tiles.
// Each warp walks tiles w, w + (warps in the grid), ..., its lanes over a
// tile's atoms (at most 64), keeps its maxima, and the block adds them to the
// result with one atomic per value (same-address atomics from every tile
// would serialise).
constexpr int kPlanThreads = 256;
__global__ void __launch_bounds__(kPlanThreads)
    bop_plan(int nat, int apt, int ntiles, const int *__restrict__ tile_atom0,
             const int *__restrict__ seed, int *__restrict__ out) {
  __shared__ int smax[2][kPlanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (int)(gridDim.x * (kPlanThreads / 32));
  int mb = 0, mt = 0;
  for (int tile = (int)blockIdx.x * (kPlanThreads / 32) + wid; tile < ntiles; tile += nw) {
    const int a0 = tile_atom0 ? tile_atom0[tile] : tile * apt;
    const int a1 = tile_atom0 ? tile_atom0[tile + 1] : min(a0 + apt, nat);
    int ntrip = 0;
    for (int q = a0 + lane; q < a1; q += 32) ntrip += trip_slots(seed[q + 1] - seed[q]);
    mt = max(mt, (int)__reduce_add_sync(0xffffffffu, ntrip));
    mb = max(mb, seed[a1] - seed[a0]);
  }
  if (lane == 0) {
    smax[0][wid] = mb;
    smax[1][wid] = mt;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    int m = 0;
    for (int w = 0; w < kPlanThreads / 32; w++) m = max(m, smax[threadIdx.x][w]);
    atomicMax(&out[threadIdx.x], m);
  }
}

// Deterministic sum of rows of kRedCols doubles: block q sums rows
// [q*rpb, min((q+1)*rpb, nrows)) into out[q*kRedCols ..] (coalesced row
// reads, fixed shuffle tree, then the warps in order).
constexpr int kRedCols = 10;
__global__ void reduce_rows_kernel(const double *__restrict__ part, int nrows, int rpb,
                                   double *__restrict__ out) {
  __shared__ double sh[32 * kRedCols];
  const int r0 = blockIdx.x * rpb, r1 = min(r0 + rpb, nrows);
  double acc[kRedCols];
#pragma unroll
  for (int c = 0; c < kRedCols; c++) acc[c] = 0.0;
  for (int t = r0 + threadIdx.x; t < r1; t += blockDim.x)
#pragma unroll
    for (int c = 0; c < kRedCols; c++) acc[c] += part[(size_t)t * kRedCols + c];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int c = 0; c < kRedCols; c++) {
    double x = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[wid * kRedCols + c] = x;
  }
  __syncthreads();
  if ((int)threadIdx.x < kRedCols) {
    double x = 0.0;
    for (int w = 0; w < nw; w++) x += sh[w * kRedCols + threadIdx.x];
    out[(size_t)blockIdx.x * kRedCols + threadIdx.x] = x;
  }
}

// Dynamic plus static shared memory above 48 KB needs an opt-in per kernel:
// raise the dynamic limit once per kernel and device to the budget of the
// largest tile (on the first launch, which is always an eager one, so that no
// attribute call happens while a stream is being captured into a graph).
template <auto Kern>
cudaError_t allow_smem(size_t smem) {
  if (smem > kSmemBudgetAll) return cudaErrorInvalidValue;
  static int done_for = -1;  // one per kernel (template argument)
  int dev = 0;
  cudaGetDevice(&dev);
  if (done_for == dev) return cudaSuccess;
  const cudaError_t e =
      cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudgetAll);
  if (e == cudaSuccess) done_for = dev;
  return e;
}

// Resident CTAs of a kernel on this device (for the persistent grid).
template <class K>
int resident_ctas(K kern, int threads, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess)
    return 0;
  return sms * std::max(per_sm, 1);
}

// Launches the tile kernel; *rows = number of energy/virial partial rows
// written to args.tile_part (one per tile, or one per CTA of the persistent
// mixed kernel).
template <class Pot, class R, bool kWat, bool kPB>
int launch_tile(const BopArgs &args, const Pot &pot, const float4 *posff, int ntiles, int max_nbt,
                int max_ntrip, int *status, cudaStream_t s, int *rows) {
  constexpr bool kMix = std::is_same<R, float>::value;
  const size_t smem =
      kMix ? bop_smem_bytes_mx(max_nbt, max_ntrip) : bop_smem_bytes<R>(max_nbt, max_ntrip);
  cudaError_t e = cudaSuccess;
  if (kMix) {
    auto kern = bop_tile_mx<Pot, kWat, kPB>;
    e = allow_smem<bop_tile_mx<Pot, kWat, kPB>>(smem);
    if (e == cudaSuccess) {
      const int resident = resident_ctas(kern, kMxThreads, smem);
      const int grid = resident > 0 ? std::min(ntiles, resident) : ntiles;
      MxParams mp = make_mx(pot, args.A);
      mp.hot = std::is_same<Pot, JuslinPot>::value ? kHotThresholdJuslin : kHotThreshold;
      kern<<<grid, kMxThreads, smem, s>>>(args, pot, mp, posff, max_nbt, max_ntrip, status);
      note_launch();
      *rows = grid;
    }
  } else {
    auto kern = bop_tile<Pot, double, kWat, kPB>;
    e = allow_smem<bop_tile<Pot, double, kWat, kPB>>(smem);
    if (e == cudaSuccess) {
      kern<<<ntiles, kBopThreads, smem, s>>>(args, pot, max_nbt, max_ntrip, status);
      note_launch();
      *rows = ntiles;
    }
  }
  if (e != cudaSuccess) {
    set_error(std::string("bop: shared memory request too large: ") + cudaGetErrorString(e));
    return GB_ERROR_CAPACITY;
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

// Calls f with the device functor of the potential's bond-order form and
// returns its result.
template <class F>
int with_bop(const Potential &pot, F &&f) {
  switch (pot.kind) {
    case kTersoff:
      return f(TersoffPot{make_tersoff_dev(pot.tp)});
    case kKumagai:
      return f(KumagaiPot{make_kumagai_dev(pot.kp)});
    case kBrenner:
      return f(BrennerPot{make_brenner_dev(pot.bp)});
    case kJuslin:
      return f(JuslinPot(make_juslin_dev(pot.jp)));
    default:
      set_error("not a bond-order potential");
      return GB_ERROR_ARGUMENT;
  }
}

// R = double: FP64 drop-in; R = float: mixed form (posff: ff positions).
template <class Pot, class R>
int dispatch_tile(const BopArgs &args, const Pot &pot, const float4 *posff, int ntiles,
                  int max_nbt, int max_ntrip, int *status, bool wat, bool pb, cudaStream_t s,
                  int *rows) {
  if (wat && pb)
    return launch_tile<Pot, R, true, true>(args, pot, posff, ntiles, max_nbt, max_ntrip, status,
                                           s, rows);
  if (wat)
    return launch_tile<Pot, R, true, false>(args, pot, posff, ntiles, max_nbt, max_ntrip, status,
                                            s, rows);
  if (pb)
    return launch_tile<Pot, R, false, true>(args, pot, posff, ntiles, max_nbt, max_ntrip, status,
                                            s, rows);
  return launch_tile<Pot, R, false, false>(args, pot, posff, ntiles, max_nbt, max_ntrip, status,
                                           s, rows);
}

// Per-atom gather of the bond forces (FP64 G, or ff G for the mixed form).
// chk: a captured evaluation's gather leaves the outputs as they are when
// the replayed list or tile plan overflowed (ReplayCheck, internal.h).
int launch_gather(bool mixed, int nat, const int *seed, const int *rev, const double *G,
                  const double *ebond, const double *wbond, double *f, double *epa, double *wpa,
                  cudaStream_t s, ReplayCheck chk = ReplayCheck{}, bool fset = false) {
  const int T = kGatherThreads, nb = (nat + T - 1) / T;
  const float2 *Gf = reinterpret_cast<const float2 *>(G);
  const int fs = fset ? 1 : 0;
  if (mixed) {
    if (epa && wpa) bop_gather_mx<true, true><<<nb, T, 0, s>>>(nat, seed, rev, Gf, ebond, wbond, f, epa, wpa, chk, fs);
    else if (epa) bop_gather_mx<true, false><<<nb, T, 0, s>>>(nat, seed, rev, Gf, ebond, wbond, f, epa, wpa, chk, fs);
    else if (wpa) bop_gather_mx<false, true><<<nb, T, 0, s>>>(nat, seed, rev, Gf, ebond, wbond, f, epa, wpa, chk, fs);
    else bop_gather_mx<false, false><<<nb, T, 0, s>>>(nat, seed, rev, Gf, ebond, wbond, f, epa, wpa, chk, fs);
  } else {
    if (epa && wpa) bop_gather<true, true><<<nb, T, 0, s>>>(nat, seed, rev, G, ebond, wbond, f, epa, wpa, chk, fs);
    else if (epa) bop_gather<true, false><<<nb, T, 0, s>>>(nat, seed, rev, G, ebond, wbond, f, epa, wpa, chk, fs);
    else if (wpa) bop_gather<false, true><<<nb, T, 0, s>>>(nat, seed, rev, G, ebond, wbond, f, epa, wpa, chk, fs);
    else bop_gather<false, false><<<nb, T, 0, s>>>(nat, seed, rev, G, ebond, wbond, f, epa, wpa, chk, fs);
  }
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

}  // namespace

// Per-segment sums: block q adds rows [seg[q], seg[q+1]) in order.
__global__ void reduce_segments_kernel(const double *__restrict__ part,
                                       const int *__restrict__ seg, double *__restrict__ out) {
  __shared__ double sh[2 * kRedCols];
  const int r0 = seg[blockIdx.x], r1 = seg[blockIdx.x + 1];
  double acc[kRedCols];
#pragma unroll
  for (int c = 0; c < kRedCols; c++) acc[c] = 0.0;
  for (int t = r0 + threadIdx.x; t < r1; t += blockDim.x)
#pragma unroll
    for (int c = 0; c < kRedCols; c++) acc[c] += part[(size_t)t * kRedCols + c];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < kRedCols; c++) {
    double x = acc[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[wid * kRedCols + c] = x;
  }
  __syncthreads();
  if ((int)threadIdx.x < kRedCols)
    out[(size_t)blockIdx.x * kRedCols + threadIdx.x] =
        sh[threadIdx.x] + (blockDim.x > 32 ? sh[kRedCols + threadIdx.x] : 0.0);
}

// Per-structure sums in two steps, so that a structure with many tiles is
// summed by many warps: the sum of each piece (a run of at most 32 of one
// structure's tile rows), then per structure the sum of its pieces.  Each
// warp takes three pieces (or structures), a lane per (piece, column), and
// adds the rows in order: one FP64 add per row and column.
constexpr int kPerWarp = 32 / kRedCols;
static_assert(kPerWarp >= 1, "one column per lane");

__global__ void reduce_pieces_kernel(const double *__restrict__ part,
                                     const int *__restrict__ piece0, int npiece,
                                     double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int p = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kPerWarp + lane / kRedCols;
  const int c = lane % kRedCols;
  if (lane >= kPerWarp * kRedCols || p >= npiece) return;
  double v = 0.0;
  for (int r = piece0[p]; r < piece0[p + 1]; r++) v += part[(size_t)r * kRedCols + c];
  out[(size_t)p * kRedCols + c] = v;
}

__global__ void reduce_seg_pieces_kernel(const double *__restrict__ psum,
                                         const int *__restrict__ seg_piece, int nseg,
                                         double *__restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int q = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kPerWarp + lane / kRedCols;
  const int c = lane % kRedCols;
  if (lane >= kPerWarp * kRedCols || q >= nseg) return;
  double v = 0.0;
  for (int p = seg_piece[q]; p < seg_piece[q + 1]; p++) v += psum[(size_t)p * kRedCols + c];
  out[(size_t)q * kRedCols + c] = v;
}

int reduce_seg_pieces(const double *part, const int *piece0, int npiece, const int *seg_piece,
                      int nseg, double *psum, double *out, cudaStream_t s) {
  if (nseg <= 0) return 0;
  if (npiece > 0) {
    const int64_t warps = (npiece + kPerWarp - 1) / kPerWarp;
    reduce_pieces_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(part, piece0,
                                                                            npiece, psum);
    note_launch();
  }
  const int64_t warps = (nseg + kPerWarp - 1) / kPerWarp;
  reduce_seg_pieces_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(
      psum, seg_piece, nseg, out);
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

int reduce_segments(const double *part, const int *seg, int nseg, double *out, cudaStream_t s) {
  if (nseg <= 0) return 0;
  reduce_segments_kernel<<<nseg, 64, 0, s>>>(part, seg, out);
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

size_t reduce_stage_bytes(int nrows) {
  return sizeof(double) * kRedCols * (size_t)((nrows + kRedRowsPerBlock - 1) / kRedRowsPerBlock);
}

int reduce_partials(const double *part, int nrows, int nc, double *red, double *stage,
                    cudaStream_t s) {
  if (nc != kRedCols) {
    set_error("reduce_partials: unsupported column count");
    return GB_ERROR_ARGUMENT;
  }
  // 64 threads per block: the shuffle tree's FP64 adds run on one SM's FP64
  // units, so a wide block would be bound by them.
  if (stage == nullptr || nrows <= 2 * kRedRowsPerBlock) {
    reduce_rows_kernel<<<1, 64, 0, s>>>(part, nrows, std::max(nrows, 1), red);
    note_launch();
  } else {
    const int nb = (nrows + kRedRowsPerBlock - 1) / kRedRowsPerBlock;
    reduce_rows_kernel<<<nb, 64, 0, s>>>(part, nrows, kRedRowsPerBlock, stage);
    note_launch();
    reduce_rows_kernel<<<1, 64, 0, s>>>(stage, nb, nb, red);
    note_launch();
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

static const size_t kSmemBudget = 200 * 1024;

namespace {

template <class Pot, bool kWat, bool kPB>
int launch_scr1(const BopArgs &args, const Pot &pot, const ScrDev &sd, int blocks, int *status,
                cudaStream_t s) {
  const size_t smem = sizeof(ScrWarpMem) * kScrWarps;
  const cudaError_t ae = allow_smem<bop_scr_atom<Pot, kWat, kPB>>(smem);
  GB_CUDA(ae);
  bop_scr_atom<Pot, kWat, kPB><<<blocks, kScrThreads, smem, s>>>(args, pot, sd, status);
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

template <class Pot>
int launch_scr(const BopArgs &args, const Pot &pot, const ScrDev &sd, int blocks, int *status,
               bool wat, bool pb, cudaStream_t s) {
  if (wat && pb) return launch_scr1<Pot, true, true>(args, pot, sd, blocks, status, s);
  if (wat) return launch_scr1<Pot, true, false>(args, pot, sd, blocks, status, s);
  if (pb) return launch_scr1<Pot, false, true>(args, pot, sd, blocks, status, s);
  return launch_scr1<Pot, false, false>(args, pot, sd, blocks, status, s);
}

// Screened variants: one thread per atom over the whole list (bop_scr.cuh),
// then the same gather and sums as the tile kernels.
int bop_run_scr(Potential &pot, const BopSystem &sys, Neighbors &nl, const Outputs &o,
                bool want_wat, bool want_pb) {
  cudaStream_t s = pot.stream;
  const int nat = sys.nat;
  const int nat_all = sys.nat_all > 0 ? sys.nat_all : nat;
  if (sys.tile_atom0) {
    set_error("batches support the non-screened bond-order potentials");
    return GB_ERROR_ARGUMENT;
  }
  if (pot.precision != GB_PRECISION_FP64) {
    set_error("The screened potentials have only the FP64 form.");
    return GB_ERROR_ARGUMENT;
  }
  if (nat == 0) {
    GB_CUDA(cudaMemsetAsync(o.red, 0, sizeof(double) * 10, s));
    return 0;
  }
  GB_CHECK(neighbors_build_reverse(nl, nat_all, s, true));
  const int64_t nb = std::max<int64_t>(nl.nentries, 1);
  GB_CHECK(pot.bond_G.ensure(sizeof(double) * 3 * nb));
  GB_CHECK(pot.bond_e.ensure(sizeof(double) * nb));
  if (want_wat) GB_CHECK(pot.bond_w.ensure(sizeof(double) * 9 * nb));
  if (want_pb) GB_CHECK(pot.bond_fr.ensure(sizeof(double) * 3 * nb));
  const int blocks = (nat + kScrWarps - 1) / kScrWarps;  // a warp per atom
  GB_CHECK(pot.tile_part.ensure(sizeof(double) * 10 * blocks + 64));
  BopArgs args;
  args.nat = nat;
  args.apt = 1;
  args.pos = nl.pos4.as<Pos4>();
  args.el = pot.el.as<int>();
  args.seed = nl.seed.as<int>();
  args.nbr = nl.nbr.as<int>();
  args.shift = nl.shift.as<int>();
  args.mask = o.mask;
  std::memcpy(args.A, sys.A, sizeof(args.A));
  args.G = pot.bond_G.as<double>();
  args.ebond = (o.epot_per_at || o.epot_per_bond) ? pot.bond_e.as<double>() : nullptr;
  args.wbond = want_wat ? pot.bond_w.as<double>() : nullptr;
  args.frbond = want_pb ? pot.bond_fr.as<double>() : nullptr;
  args.tile_part = pot.tile_part.as<double>();
  GB_CUDA(cudaEventRecord(pot.kev[0], s));
  {
    const ScrDev sd =
        make_scr_dev(bop_r1(pot), bop_r2(pot), pot_npairs(pot), pot.scr, pot.kind != kJuslin);
    GB_CHECK(with_bop(pot, [&](const auto &P) {
      return launch_scr(args, P, sd, blocks, o.status, want_wat, want_pb, s);
    }));
  }
  GB_CUDA(cudaEventRecord(pot.kev[1], s));
  GB_CHECK(launch_gather(false, nat_all, nl.seed.as<int>(), nl.rev.as<int>(), args.G,
                         args.ebond, args.wbond, o.f, o.epot_per_at,
                         want_wat ? o.wpot_per_at : nullptr, s, ReplayCheck{}, o.f_set));
  GB_CHECK(pot.red_stage.ensure(reduce_stage_bytes(blocks) + 64));
  GB_CHECK(reduce_partials(args.tile_part, blocks, 10, o.red, pot.red_stage.as<double>(), s));
  pot.tile_atoms = 1;
  pot.last_plan[0] = pot.last_plan[1] = 0;
  return 0;
}

}  // namespace

int bop_run(Potential &pot, const BopSystem &sys, Neighbors &nl, const Outputs &o,
            bool want_wat, bool want_pb) {
  if (pot.screened) return bop_run_scr(pot, sys, nl, o, want_wat, want_pb);
  cudaStream_t s = pot.stream;
  const int nat = sys.nat;
  const int nat_all = sys.nat_all > 0 ? sys.nat_all : nat;
  const bool batch = sys.tile_atom0 != nullptr;
  if (nat == 0) {
    GB_CUDA(cudaMemsetAsync(o.red, 0, sizeof(double) * 10, s));
    if (batch && sys.nseg > 0)
      GB_CUDA(cudaMemsetAsync(sys.red_seg, 0, sizeof(double) * 10 * sys.nseg, s));
    return 0;
  }
  GB_CHECK(neighbors_build_reverse(nl, nat_all, s, false));  // checked after the plan read-back
  const bool mixed = pot.precision == GB_PRECISION_MIXED;
  // Atoms per tile: largest power of two <= kMaxApt whose worst tile fits.
  const int maxz = std::max(nl.maxz, 1);
  int apt = batch ? sys.apt : kMaxApt;
  auto fits = [&](int aptc) {
    const size_t worst = bop_smem_bytes<double>(aptc * maxz, aptc * trip_slots(maxz));
    return worst <= kSmemBudget;
  };
  if (batch) {
    // tiles were cut by the caller (at most kMaxApt atoms each); their exact
    // plan is checked against shared memory below
  } else if (pot.tile_request > 0) {
    apt = std::min(pot.tile_request, kMaxApt);
    while (apt > 1 && !fits(apt)) apt >>= 1;
  } else {
    while (apt > 1 && !fits(apt)) apt >>= 1;
    // Keep roughly one bond per thread.
    while (apt > 1 && (int64_t)apt * std::max(1, (int)(nl.nentries / std::max(nat, 1))) >
                          2 * kBopThreads)
      apt >>= 1;
  }
  if (!batch && !fits(apt)) {
    set_error("Internal neighbor list exhausted: an atom has " + std::to_string(maxz) +
              " neighbours within the cutoff, more than the bond-order kernel supports.");
    return GB_ERROR_CAPACITY;
  }
  const int ntiles = batch ? sys.ntiles : (nat + apt - 1) / apt;
  // A captured evaluation sizes everything for the list capacity and uses
  // the tile plan given by the caller (checked per tile by the kernel).
  const int64_t nb = std::max<int64_t>(sys.capture ? sys.nb_capacity : nl.nentries, 1);
  GB_CHECK(pot.bond_G.ensure(sizeof(double) * 3 * nb));
  GB_CHECK(pot.bond_e.ensure(sizeof(double) * nb));
  if (want_wat) GB_CHECK(pot.bond_w.ensure(sizeof(double) * 9 * nb));
  if (want_pb) GB_CHECK(pot.bond_fr.ensure(sizeof(double) * 3 * nb));
  GB_CHECK(pot.tile_part.ensure(sizeof(double) * 10 * ntiles + 64));
  // Plan: exact max bonds / triplets per tile.  A single structure's list
  // build may have planned these tiles already (read back with the list's
  // sizes); the reverse index is then checked by the caller after its
  // final synchronisation.
  int *plan = reinterpret_cast<int *>(pot.tile_part.as<double>() + 10 * (size_t)ntiles);
  GB_CUDA(cudaMemsetAsync(plan, 0, sizeof(int) * 4, s));
  int max_nbt = sys.max_nbt, max_ntrip = sys.max_ntrip;
  const bool preplanned = !batch && !sys.capture && nat_all == nat && nl.plan_ready &&
                          nl.plan_done_apt == apt;
  if (preplanned) {
    max_nbt = nl.hplan[0];
    max_ntrip = nl.hplan[1];
  } else {
    GB_CHECK(bop_plan_launch(nat, apt, ntiles, sys.tile_atom0, nl.seed.as<int>(), plan, s));
  }
  if (!sys.capture && !preplanned) {
    GB_CHECK(pot.hred.ensure(64));
    int *hplan = pot.hred.as<int>();
    GB_CUDA(cudaMemcpyAsync(hplan, plan, sizeof(int) * 2, cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    GB_CHECK(neighbors_check_reverse(nl, nullptr));
    max_nbt = hplan[0];
    max_ntrip = hplan[1];
    if (batch && bop_tile_smem(mixed, max_nbt, max_ntrip) > kSmemBudget) {
      set_error("Internal neighbor list exhausted: a tile of " + std::to_string(max_nbt) +
                " bonds does not fit the bond-order kernel's shared memory.");
      return GB_ERROR_CAPACITY;
    }
  }
  pot.last_plan[0] = max_nbt;
  pot.last_plan[1] = max_ntrip;

  BopArgs args;
  args.nat = nat;
  args.apt = apt;
  args.pos = nl.pos4.as<Pos4>();
  args.el = sys.el ? sys.el : pot.el.as<int>();
  args.seed = nl.seed.as<int>();
  args.nbr = nl.nbr.as<int>();
  args.shift = nl.shift.as<int>();
  args.mask = o.mask;
  std::memcpy(args.A, sys.A, sizeof(args.A));
  args.tile_atom0 = sys.tile_atom0;
  args.tile_struct = sys.tile_struct;
  args.Acells = sys.Acells;
  args.Acells_ff = sys.Acells_ff;
  args.ntiles = ntiles;
  args.G = pot.bond_G.as<double>();
  // per-bond energies only when per-atom or per-bond energies are requested
  args.ebond = (o.epot_per_at || o.epot_per_bond) ? pot.bond_e.as<double>() : nullptr;
  args.wbond = want_wat ? pot.bond_w.as<double>() : nullptr;
  args.frbond = want_pb ? pot.bond_fr.as<double>() : nullptr;
  args.tile_part = pot.tile_part.as<double>();
  // Batch tiles carry their own partial rows, so the order in which CTAs
  // take them does not change any sum: they are handed out by a counter
  // (plan[2], zeroed with the plan above).
  if (batch && mixed && GB_MX_TILE_QUEUE) args.tile_queue = plan + 2;
  int *status = o.status;
  int rc, rows = ntiles;
  if (mixed && !nl.posff_valid) {
    GB_CHECK(nl.posff.ensure(sizeof(float4) * 2 * (size_t)nat_all));
    bop_posff<<<(nat_all + 127) / 128, 128, 0, s>>>(nat_all, args.pos, nl.posff.as<float4>());
    note_launch();
    nl.posff_valid = true;
  }
  const float4 *posff = mixed ? nl.posff.as<float4>() : nullptr;
  if (!sys.capture) GB_CUDA(cudaEventRecord(pot.kev[0], s));
  rc = with_bop(pot, [&](const auto &P) {
    using PotT = std::decay_t<decltype(P)>;
    return mixed ? dispatch_tile<PotT, float>(args, P, posff, ntiles, max_nbt, max_ntrip, status,
                                              want_wat, want_pb, s, &rows)
                 : dispatch_tile<PotT, double>(args, P, posff, ntiles, max_nbt, max_ntrip, status,
                                               want_wat, want_pb, s, &rows);
  });
  GB_CHECK(rc);
  if (!sys.capture) GB_CUDA(cudaEventRecord(pot.kev[1], s));
  GB_CHECK(launch_gather(mixed, nat_all, nl.seed.as<int>(), nl.rev.as<int>(), args.G,
                         args.ebond, args.wbond, o.f, o.epot_per_at,
                         want_wat ? o.wpot_per_at : nullptr, s, sys.check, o.f_set));
  if (batch) {
    if (sys.piece0)
      GB_CHECK(reduce_seg_pieces(args.tile_part, sys.piece0, sys.npiece, sys.seg_piece, sys.nseg,
                                 sys.piece_sum, sys.red_seg, s));
    else
      GB_CHECK(reduce_segments(args.tile_part, sys.seg, sys.nseg, sys.red_seg, s));
    GB_CUDA(cudaMemsetAsync(o.red, 0, sizeof(double) * 10, s));
  } else {
    GB_CHECK(pot.red_stage.ensure(reduce_stage_bytes(rows) + 64));
    GB_CHECK(reduce_partials(args.tile_part, rows, 10, o.red, pot.red_stage.as<double>(), s));
  }
  pot.tile_atoms = apt;
  return 0;
}

int bop_compute(Potential &pot, const Particles &p, Neighbors &nl, const Outputs &o,
                bool want_wat, bool want_pb) {
  BopSystem sys;
  sys.nat = p.nat;
  std::memcpy(sys.A, p.A, sizeof(sys.A));
  return bop_run(pot, sys, nl, o, want_wat, want_pb);
}

int bop_plan_launch(int nat, int apt, int ntiles, const int *tile_atom0, const int *seed,
                    int *out, cudaStream_t s) {
  if (ntiles <= 0) return 0;
  const int blocks = std::min((ntiles + kPlanThreads / 32 - 1) / (kPlanThreads / 32), 152 * 4);
  bop_plan<<<blocks, kPlanThreads, 0, s>>>(nat, apt, ntiles, tile_atom0, seed, out);
  note_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

size_t bop_tile_smem(bool mixed, int nbt, int ntrip) {
  return mixed ? bop_smem_bytes_mx(nbt, ntrip) : bop_smem_bytes<double>(nbt, ntrip);
}

size_t bop_tile_smem_budget() { return kSmemBudget; }

namespace {
template <auto Kern>
int ctas_per_sm(int threads, size_t smem) {
  if (allow_smem<Kern>(smem) != cudaSuccess) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, Kern, threads, smem) != cudaSuccess)
    return 0;
  return per_sm;
}
}  // namespace

int bop_tile_ctas_per_sm(const Potential &pot, size_t smem) {
  const bool mixed = pot.precision == GB_PRECISION_MIXED;
  const int n = with_bop(pot, [&](const auto &P) {
    using PotT = std::decay_t<decltype(P)>;
    return mixed ? ctas_per_sm<bop_tile_mx<PotT, false, false>>(kMxThreads, smem)
                 : ctas_per_sm<bop_tile<PotT, double, false, false>>(kBopThreads, smem);
  });
  return std::max(n, 0);
}


}  // namespace gb

// ===========================================================================
// Allocation-free variant of the bond-order evaluation.
//
// Some callers cannot call cudaMalloc: codes embedded in a host framework that
// has already reserved the device memory for its own pool (so cudaMalloc
// fails or would fragment that pool), and MD loops that must not allocate
// inside a time step.  For them
// gb_bop_energy_and_forces_noalloc evaluates Tersoff, Kumagai or Brenner on a
// neighbour list the caller supplies, using only the file-scope scratch array
// below for every intermediate buffer.  The array is sized for at most
// kNoallocMaxAtoms atoms and kNoallocMaxEntries list entries; every GPU that
// loads this library holds it (kNoallocBytes = 12,976,896 bytes, about 13 MB)
// until the process exits.  The call waits for its stream to read the list
// size, the list checks and the tile plan back, so it blocks the host.
// ===========================================================================

namespace gb {
namespace {

constexpr int kNoallocMaxAtoms = 16384;
constexpr int kNoallocMaxEntries = 262144;

constexpr size_t na_align(size_t x) { return (x + 255) & ~size_t(255); }
// Scratch layout (byte offsets).
constexpr size_t kNaStatus = 0;                                            // 64 ints
constexpr size_t kNaRed = kNaStatus + 256;                                 // 16 doubles
constexpr size_t kNaPos = kNaRed + 256;                                    // Pos4[A]
constexpr size_t kNaEl = na_align(kNaPos + 32 * (size_t)kNoallocMaxAtoms);  // int[A]
constexpr size_t kNaSeed = na_align(kNaEl + 4 * (size_t)kNoallocMaxAtoms);  // int[A+1]
constexpr size_t kNaShift = na_align(kNaSeed + 4 * ((size_t)kNoallocMaxAtoms + 1));
constexpr size_t kNaRev = na_align(kNaShift + 4 * (size_t)kNoallocMaxEntries);
constexpr size_t kNaG = na_align(kNaRev + 4 * (size_t)kNoallocMaxEntries);   // 3 doubles/entry
constexpr size_t kNaE = na_align(kNaG + 24 * (size_t)kNoallocMaxEntries);    // 1 double/entry
constexpr size_t kNaPart = na_align(kNaE + 8 * (size_t)kNoallocMaxEntries);  // 10 doubles/tile
constexpr size_t kNaPosff = na_align(kNaPart + 80 * (size_t)kNoallocMaxAtoms);  // 2 float4/atom
constexpr size_t kNoallocBytes = na_align(kNaPosff + 32 * (size_t)kNoallocMaxAtoms);
static_assert(kNoallocBytes == 12976896, "scratch size quoted in the header");

}  // namespace
}  // namespace gb

// The scratch itself.  Host code must not use this name as an address (on the
// host it is only a stand-in): the device address is obtained with
// cudaGetSymbolAddress, once per device, in noalloc_scratch() below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[gb::kNoallocBytes];

namespace gb {
namespace {

constexpr int kNoallocMaxDevices = 64;
unsigned char *g_noalloc_ptr[kNoallocMaxDevices] = {nullptr};

// Device address of the scratch for the current device (set-up on the first
// call per device).
int noalloc_scratch(unsigned char **out) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_error("noalloc: device index out of range");
    return GB_ERROR_ARGUMENT;
  }
  if (!g_noalloc_ptr[dev]) {
    void *ptr = nullptr;
    GB_CUDA(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
    g_noalloc_ptr[dev] = static_cast<unsigned char *>(ptr);
  }
  *out = g_noalloc_ptr[dev];
  return 0;
}

// Per atom: padded position, element index (Z -> parameter-set index), int32
// offsets, max neighbour count.  status[0] = max z, status[1] = flags.  The
// offsets are validated here, before any kernel walks the list: seed[0] = 0,
// non-decreasing, every offset within [0, n] (n = seed[nat], already checked
// against the scratch capacity on the host).
__global__ void noalloc_prepare(int nat, int64_t n, const double *__restrict__ r,
                                const int *__restrict__ Z, int nel, int z0, int z1, int z2,
                                const int64_t *__restrict__ seed, Pos4 *__restrict__ pos,
                                int *__restrict__ el, int *__restrict__ seed32,
                                int *__restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > nat) return;
  const int64_t si = seed[i];
  if (si < 0 || si > n || (i == 0 && si != 0)) atomicOr(&status[1], 16);
  seed32[i] = (int)(si < 0 ? 0 : si > n ? n : si);
  if (i == nat) return;
  pos[i] = Pos4{r[3 * i], r[3 * i + 1], r[3 * i + 2], 0.0};
  const int z = Z[i];
  el[i] = (nel > 0 && z == z0) ? 0 : (nel > 1 && z == z1) ? 1 : (nel > 2 && z == z2) ? 2 : -1;
  const int64_t cnt = seed[i + 1] - si;
  if (cnt < 0) atomicOr(&status[1], 1);
  atomicMax(&status[0], (int)(cnt < 0 ? 0 : cnt > n ? n : cnt));
}

// Per entry: packed image shift; neighbour index range check.
__global__ void noalloc_pack(int nat, int n, const int *__restrict__ j, const int *__restrict__ dc,
                             int *__restrict__ shift, int *__restrict__ status) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const int s0 = dc[3 * b], s1 = dc[3 * b + 1], s2 = dc[3 * b + 2];
  if (s0 > kMaxShift || s0 < -kMaxShift || s1 > kMaxShift || s1 < -kMaxShift ||
      s2 > kMaxShift || s2 < -kMaxShift)
    atomicOr(&status[1], 2);
  const int jj = j[b];
  if (jj < 0 || jj >= nat) atomicOr(&status[1], 4);
  shift[b] = pack_shift(s0, s1, s2);
}

// rev[b] = entry (j -> i, -s) of entry b = (i -> j, s); the list must be the
// full symmetric list of gb_neighbors_get.
__global__ void noalloc_reverse(int nat, const int *__restrict__ seed, const int *__restrict__ nbr,
                                const int *__restrict__ shift, int *__restrict__ rev,
                                int *__restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  for (int b = seed[i]; b < seed[i + 1]; b++) {
    const int jj = nbr[b];
    int found = -1;
    if (jj >= 0 && jj < nat) {
      int s0, s1, s2;
      unpack_shift(shift[b], s0, s1, s2);
      const int want = pack_shift(-s0, -s1, -s2);
      for (int c = seed[jj]; c < seed[jj + 1]; c++)
        if (nbr[c] == i && shift[c] == want) {
          found = c;
          break;
        }
    }
    if (found < 0) {
      atomicOr(&status[1], 8);
      found = b;  // keeps the gather in bounds; the call reports an error
    }
    rev[b] = found;
  }
}

__global__ void noalloc_finish(const double *__restrict__ red, double *__restrict__ epot,
                               double *__restrict__ wpot) {
  if (threadIdx.x == 0) epot[0] = red[0];
  if (threadIdx.x < 9) wpot[threadIdx.x] += red[1 + threadIdx.x];
}

}  // namespace
}  // namespace gb

extern "C" int gb_bop_energy_and_forces_noalloc(gb_potential_t *h, int nat, const double *r,
                                                const double *cell, const int *Z,
                                                const int64_t *seed, const int *j, const int *dc,
                                                double *epot, double *f, double *wpot,
                                                void *stream) {
  using namespace gb;
  clear_error();
  if (!h || !cell || !epot || !f || !wpot || (nat > 0 && (!r || !Z || !seed))) {
    set_error("noalloc: missing argument");
    return GB_ERROR_ARGUMENT;
  }
  Potential &pot = h->pot;
  if ((pot.kind != kTersoff && pot.kind != kKumagai && pot.kind != kBrenner) || pot.screened) {
    set_error("noalloc: only the non-screened bond-order potentials (Tersoff, Kumagai, "
              "Brenner) are supported");
    return GB_ERROR_ARGUMENT;
  }
  if (nat < 0 || nat > kNoallocMaxAtoms) {
    set_error("noalloc: nat = " + std::to_string(nat) + " exceeds the maximum of " +
              std::to_string(kNoallocMaxAtoms) + " atoms");
    return GB_ERROR_CAPACITY;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  unsigned char *base = nullptr;
  GB_CHECK(noalloc_scratch(&base));
  int *status = reinterpret_cast<int *>(base + kNaStatus);
  double *red = reinterpret_cast<double *>(base + kNaRed);
  // The status words and reduction slots keep the previous call's values:
  // clear them.
  GB_CUDA(cudaMemsetAsync(status, 0, 256 + 256, s));
  if (nat == 0) {
    noalloc_finish<<<1, 32, 0, s>>>(red, epot, wpot);
    note_launch();
    GB_CUDA(cudaGetLastError());
    return 0;
  }
  int64_t n64 = 0;
  GB_CUDA(cudaMemcpyAsync(&n64, seed + nat, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (n64 < 0 || n64 > kNoallocMaxEntries) {
    set_error("noalloc: the neighbour list has " + std::to_string(n64) +
              " entries, more than the maximum of " + std::to_string(kNoallocMaxEntries));
    return GB_ERROR_CAPACITY;
  }
  const int n = (int)n64;
  if (n > 0 && (!j || !dc)) {
    set_error("noalloc: missing neighbour list arrays");
    return GB_ERROR_ARGUMENT;
  }
  Pos4 *pos = reinterpret_cast<Pos4 *>(base + kNaPos);
  int *el = reinterpret_cast<int *>(base + kNaEl);
  int *seed32 = reinterpret_cast<int *>(base + kNaSeed);
  int *shift = reinterpret_cast<int *>(base + kNaShift);
  int *rev = reinterpret_cast<int *>(base + kNaRev);
  double *G = reinterpret_cast<double *>(base + kNaG);
  double *ebond = reinterpret_cast<double *>(base + kNaE);
  double *part = reinterpret_cast<double *>(base + kNaPart);
  const int nel = pot_nel(pot);
  const int z0 = pot_Z(pot, 0), z1 = nel > 1 ? pot_Z(pot, 1) : -1,
            z2 = nel > 2 ? pot_Z(pot, 2) : -1;
  // Status words: [0] max z, [1] list flags, [4..5] tile plan, [8..15] the
  // tile kernel's own status (separate slots: the mixed kernel counts its
  // hot bonds in its status[2]).
  int *plan = status + 4;
  int *kstatus = status + 8;
  noalloc_prepare<<<(nat + 1 + 127) / 128, 128, 0, s>>>(nat, n64, r, Z, nel, z0, z1, z2, seed,
                                                       pos, el, seed32, status);
  note_launch();
  if (n > 0) {
    noalloc_pack<<<(n + 255) / 256, 256, 0, s>>>(nat, n, j, dc, shift, status);
    note_launch();
  }
  GB_CUDA(cudaGetLastError());
  // The offsets and neighbour indices are checked before any kernel walks
  // the list (noalloc_reverse and the tile kernel index through both).
  int hs[2] = {0, 0};
  GB_CUDA(cudaMemcpyAsync(hs, status, sizeof(hs), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  auto list_error = [](int flags) {
    set_error(std::string("noalloc: invalid neighbour list (") +
              ((flags & 16) ? "offsets not within [0, seed[nat]] or seed[0] != 0 " : "") +
              ((flags & 1) ? "decreasing offsets " : "") +
              ((flags & 2) ? "image shift beyond +-511 " : "") +
              ((flags & 4) ? "neighbour index out of range " : "") +
              ((flags & 8) ? "list not symmetric" : "") + ")");
    return GB_ERROR_ARGUMENT;
  };
  if (hs[1]) return list_error(hs[1]);
  // Tile size as in bop_compute.
  const int maxz = std::max(hs[0], 1);
  int apt = kMaxApt;
  auto fits = [&](int aptc) {
    return bop_smem_bytes<double>(aptc * maxz, aptc * trip_slots(maxz)) <= kSmemBudget;
  };
  while (apt > 1 && !fits(apt)) apt >>= 1;
  while (apt > 1 && (int64_t)apt * std::max(1, n / nat) > 2 * kBopThreads) apt >>= 1;
  if (!fits(apt)) {
    set_error("noalloc: an atom has " + std::to_string(maxz) +
              " neighbours, more than the bond-order kernel supports");
    return GB_ERROR_CAPACITY;
  }
  const int ntiles = (nat + apt - 1) / apt;
  noalloc_reverse<<<(nat + 127) / 128, 128, 0, s>>>(nat, seed32, j, shift, rev, status);
  note_launch();
  GB_CHECK(bop_plan_launch(nat, apt, ntiles, nullptr, seed32, plan, s));
  int hp[6] = {0, 0, 0, 0, 0, 0};
  GB_CUDA(cudaMemcpyAsync(hp, status, sizeof(hp), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (hp[1]) return list_error(hp[1]);

  BopArgs args;
  args.nat = nat;
  args.apt = apt;
  args.pos = pos;
  args.el = el;
  args.seed = seed32;
  args.nbr = j;
  args.shift = shift;
  args.mask = nullptr;
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) args.A[a][k] = cell[3 * k + a];
  args.G = G;
  args.ebond = ebond;
  args.wbond = nullptr;
  args.frbond = nullptr;
  args.tile_part = part;
  const bool mixed = pot.precision == GB_PRECISION_MIXED;
  float4 *posff = reinterpret_cast<float4 *>(base + kNaPosff);
  if (mixed) {
    bop_posff<<<(nat + 127) / 128, 128, 0, s>>>(nat, pos, posff);
    note_launch();
  }
  int rows = ntiles;
  const int rc = with_bop(pot, [&](const auto &P) {
    using PotT = std::decay_t<decltype(P)>;
    return mixed ? dispatch_tile<PotT, float>(args, P, posff, ntiles, hp[4], hp[5], kstatus,
                                              false, false, s, &rows)
                 : dispatch_tile<PotT, double>(args, P, posff, ntiles, hp[4], hp[5], kstatus,
                                               false, false, s, &rows);
  });
  GB_CHECK(rc);
  GB_CHECK(launch_gather(mixed, nat, seed32, rev, G, ebond, nullptr, f, nullptr, nullptr, s));
  GB_CHECK(reduce_partials(part, rows, 10, red, nullptr, s));
  noalloc_finish<<<1, 32, 0, s>>>(red, epot, wpot);
  note_launch();
  GB_CUDA(cudaGetLastError());
  int hst = 0;
  GB_CUDA(cudaMemcpyAsync(&hst, kstatus, sizeof(int), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaStreamSynchronize(s));
  if (hst) {
    set_error("noalloc: internal error (tile plan mismatch)");
    return GB_ERROR_UNSPECIFIED;
  }
  return 0;
}
