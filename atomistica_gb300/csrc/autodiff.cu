// Tangent (forward-mode) evaluation of single-element Tersoff energies and
// forces over a batch of structures, for parameter fitting.
//
// Every quantity of the bond-order evaluation carries (value, derivative)
// along one direction: a direction in the space of the 14 continuous Tersoff
// parameters (A, B, lambda, mu, beta, n, c, d, h, R = r1, S = r2, xi, omega,
// mubo; tersoff_func.f90:32-211, cutoff.f90:171-196) and/or a direction v in
// the positions.  One pass gives E, F and their derivatives dE, dF along the
// direction; with a position direction v, dF = -H v (H the Hessian of E), so
// the vector-Jacobian products of E and F with respect to positions need one
// pass and those with respect to the parameters one pass per parameter.
//
// Decomposition as the FP64 tile kernel (bop.cu): one CTA per tile (tiles of
// the batch), a thread per directed bond, zeta and its derivatives per bond,
// d zeta/d r_k per (ij, ik) slot in shared memory, per-bond forces G gathered
// per atom through the reverse-entry index; no atomics.  Derivatives of the
// cutoff region and of the list itself are taken at fixed region membership
// (the cutoff function and its derivative vanish at r = S, so E and F are C1
// across it).  mubo = 0 takes the reference's h = 1 branch
// (tersoff_func.f90:190) only when mubo has no derivative; otherwise
// h = exp((2 mubo (r_ij - r_ik))^m) is differentiated.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "batch.h"

namespace gb {
namespace {

struct Dual {
  double v, d;
};
__host__ __device__ __forceinline__ Dual mk(double v, double d = 0.0) { return Dual{v, d}; }
__host__ __device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__host__ __device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__host__ __device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__host__ __device__ __forceinline__ Dual operator*(Dual a, Dual b) {
  return {a.v * b.v, a.d * b.v + a.v * b.d};
}
__host__ __device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
__host__ __device__ __forceinline__ Dual operator*(double s, Dual a) { return {s * a.v, s * a.d}; }
__host__ __device__ __forceinline__ Dual operator+(double s, Dual a) { return {s + a.v, a.d}; }
__host__ __device__ __forceinline__ Dual dexp(Dual a) {
  const double e = exp(a.v);
  return {e, e * a.d};
}
__host__ __device__ __forceinline__ Dual dlog(Dual a) { return {log(a.v), a.d / a.v}; }
__host__ __device__ __forceinline__ Dual dsqrt(Dual a) {
  const double s = sqrt(a.v);
  return {s, a.d / (2.0 * s)};
}
__host__ __device__ __forceinline__ void dsincos(Dual a, Dual &s, Dual &c) {
  const double sv = sin(a.v), cv = cos(a.v);
  s = {sv, cv * a.d};
  c = {cv, -sv * a.d};
}

// Single-element Tersoff parameters with their derivatives along the
// direction, and the derived quantities.
struct TersoffTangent {
  Dual A, B, lam, mu, beta, n, c, d, h, r1, r2, xi, om, mubo;
  int m;
  bool h_one;  // mubo == 0 with no derivative: h = 1 (tersoff_func.f90:190-192)
  Dual c2, d2, e, fac;
};

constexpr int kTThreads = 128;
constexpr int kTMaxApt = 64;
constexpr int kTFlagShort = 1 << 12, kTFlagIJ = 1 << 13, kTFlagK = 1 << 14;

struct TangentArgs {
  int nat;
  const int *tile_atom0, *tile_struct;
  const double *Acells;
  const Pos4 *pos;
  const double *dpos;  // (nat,3) position direction or nullptr
  const int *el;
  const int *seed, *nbr, *shift;
  Dual *G;             // 3 per bond
  double *tile_part;   // 10 per tile: [E.v, E.d, 0...]
};

__host__ __device__ inline size_t talign(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ inline size_t tangent_smem(int nbt, int ntrip) {
  size_t o = talign(sizeof(int) * (2 * kTMaxApt + 2 + (size_t)nbt));
  o += talign(sizeof(Dual) * (size_t)nbt * 12);
  o += talign(sizeof(Dual) * (size_t)ntrip * 3);
  return o + 64;
}

__global__ void __launch_bounds__(kTThreads)
    tangent_tile(const TangentArgs a, const TersoffTangent p, int max_nbt, int max_ntrip,
                 int *status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double sA[9];
  __shared__ double red[2 * (kTThreads / 32)];
  const int tid = threadIdx.x, tile = blockIdx.x;
  const int a0 = a.tile_atom0[tile], a1 = a.tile_atom0[tile + 1];
  if (tid < 9) sA[tid] = a.Acells[9 * a.tile_struct[tile] + tid];
  const int na = a1 - a0;
  const int b0 = a.seed[a0];
  const int nbt = a.seed[a1] - b0;
  int *aseed = reinterpret_cast<int *>(sm);
  int *toff = aseed + kTMaxApt + 1;
  int *meta = aseed + 2 * kTMaxApt + 2;
  for (int q = tid; q <= na; q += kTThreads) aseed[q] = a.seed[a0 + q] - b0;
  __syncthreads();
  if (tid == 0) {
    int s = 0;
    for (int q = 0; q < na; q++) {
      toff[q] = s;
      const int z = aseed[q + 1] - aseed[q];
      s += z * z;
    }
    toff[na] = s;
  }
  __syncthreads();
  const int ntrip = toff[na];
  if (nbt > max_nbt || ntrip > max_ntrip || na > kTMaxApt) {
    if (tid == 0) atomicOr(status, 2);
    return;
  }
  size_t o = talign(sizeof(int) * (2 * kTMaxApt + 2 + (size_t)nbt));
  Dual *D = reinterpret_cast<Dual *>(sm + o);
  Dual *rn = D, *rl = D + 3 * nbt, *rinv = D + 4 * nbt, *fc = D + 5 * nbt, *dfc = D + 6 * nbt,
       *P = D + 7 * nbt, *E = D + 8 * nbt, *Gs = D + 9 * nbt;
  o += talign(sizeof(Dual) * (size_t)nbt * 12);
  Dual *T = reinterpret_cast<Dual *>(sm + o);
  for (int q = tid; q < na; q += kTThreads)
    for (int lb = aseed[q]; lb < aseed[q + 1]; lb++) meta[lb] = q;
  __syncthreads();

  // Phase 1: bond geometry.
  for (int lb = tid; lb < nbt; lb += kTThreads) {
    const int ai = meta[lb];
    const int i = a0 + ai, b = b0 + lb, j = a.nbr[b];
    int mt = ai;
    Dual f = mk(0.0), df = mk(0.0), r = mk(1.0), ri = mk(1.0);
    Dual n3[3] = {mk(0.0), mk(0.0), mk(0.0)};
    if (a.el[i] >= 0 && a.el[j] >= 0) {
      const Pos4 pi = a.pos[i], pj = a.pos[j];
      int s0, s1, s2;
      unpack_shift(a.shift[b], s0, s1, s2);
      const double pv[3] = {pj.x - pi.x, pj.y - pi.y, pj.z - pi.z};
      Dual rij[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double as = sA[3 * c] * s0 + sA[3 * c + 1] * s1 + sA[3 * c + 2] * s2;
        const double dd = a.dpos ? a.dpos[3 * (size_t)j + c] - a.dpos[3 * (size_t)i + c] : 0.0;
        rij[c] = mk(pv[c] - as, dd);
      }
      const Dual r2 = rij[0] * rij[0] + rij[1] * rij[1] + rij[2] * rij[2];
      if (r2.v < p.r2.v * p.r2.v) {
        r = dsqrt(r2);
        ri = mk(1.0) / r;
#pragma unroll
        for (int c = 0; c < 3; c++) n3[c] = rij[c] * ri;
        if (r.v <= p.r1.v) {
          f = mk(1.0);
        } else {
          Dual sx, cx;
          dsincos(p.fac * (r - p.r1), sx, cx);
          f = 0.5 * (1.0 + cx);
          df = -0.5 * (p.fac * sx);
        }
        mt |= kTFlagShort | kTFlagK | kTFlagIJ;
      }
    }
    meta[lb] = mt;
#pragma unroll
    for (int c = 0; c < 3; c++) rn[c * nbt + lb] = n3[c];
    rl[lb] = r;
    rinv[lb] = ri;
    fc[lb] = f;
    dfc[lb] = df;
  }
  __syncthreads();

  // Phase 2: per bond ij, zeta and its derivatives, b, P, energy, j-role G.
  for (int lb = tid; lb < nbt; lb += kTThreads) {
    const int mt = meta[lb];
    if (!(mt & kTFlagIJ)) {
      P[lb] = mk(0.0);
      E[lb] = mk(0.0);
#pragma unroll
      for (int c = 0; c < 3; c++) Gs[c * nbt + lb] = mk(0.0);
      continue;
    }
    const int ai = mt & 0xff;
    const int s = aseed[ai], z = aseed[ai + 1] - s, pq = lb - s;
    Dual *trow = T + toff[ai] + pq * z;
    const Dual r = rl[lb];
    const Dual eA = dexp(-(p.mu * r)), eR = dexp(-(p.lam * r));
    const Dual VA = -(p.B * eA), dVA = p.B * p.mu * eA;
    const Dual VR = p.A * eR, dVR = -(p.A * p.lam * eR);
    const Dual nij[3] = {rn[lb], rn[nbt + lb], rn[2 * nbt + lb]};
    Dual zeta = mk(0.0), dbj[3] = {mk(0.0), mk(0.0), mk(0.0)};
    for (int q = 0; q < z; q++) {
      const int lk = s + q;
      if (lk == lb) continue;
      if (!(meta[lk] & kTFlagK)) {
        trow[q] = mk(0.0);
        trow[ntrip + q] = mk(0.0);
        trow[2 * ntrip + q] = mk(0.0);
        continue;
      }
      const Dual nik[3] = {rn[lk], rn[nbt + lk], rn[2 * nbt + lk]};
      Dual hv = mk(1.0), dh = mk(0.0);
      if (!p.h_one) {
        const Dual x = 2.0 * (p.mubo * (r - rl[lk]));
        Dual pw = mk(1.0);
        for (int k = 1; k < p.m; k++) pw = pw * x;
        hv = dexp(pw * x);
        dh = 2.0 * (p.mubo * ((double)p.m * (pw * hv)));
      }
      const Dual cs = nik[0] * nij[0] + nik[1] * nij[1] + nik[2] * nij[2];
      // g = omega (1 + c^2 hc^2 / (d^2 (d^2 + hc^2))), hc = h - cos theta
      const Dual hc = p.h - cs;
      const Dual den = p.d2 + hc * hc;
      const Dual gv = p.om * (1.0 + (p.c2 * hc * hc) / (p.d2 * den));
      const Dual dg = -2.0 * ((p.om * p.c2 * hc) / (den * den));
      const Dual fk = fc[lk];
      zeta = zeta + fk * gv * hv;
      const Dual dzfac = fk * dg * hv;
      const Dual dzdrij = gv * fk * dh;
      const Dual dzdrik = gv * (dfc[lk] * hv - fk * dh);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const Dual dcj = (nik[c] - cs * nij[c]) * rinv[lb];
        const Dual dck = (nij[c] - cs * nik[c]) * rinv[lk];
        dbj[c] = dbj[c] + dzdrij * nij[c] + dzfac * dcj;
        trow[c * ntrip + q] = dzdrik * nik[c] + dzfac * dck;
      }
    }
    // b = xi (1 + beta^n zeta^n)^e, e = -1/(2n); P = dE/dzeta
    Dual bij = mk(1.0), Pij = mk(0.0);
    if (zeta.v > 0.0) {
      const Dual x = dexp(p.n * (dlog(p.beta) + dlog(zeta)));
      const Dual l1x = dlog(1.0 + x);
      const Dual ae = dexp(p.e * l1x);
      bij = p.xi * ae;
      Pij = -0.25 * (fc[lb] * VA * p.xi * (x / zeta) * (ae / (1.0 + x)));
    }
    const Dual f = fc[lb], dfv = dfc[lb];
    E[lb] = 0.5 * (f * (VR + bij * VA));
    const Dual dff = 0.5 * (dVR * f + bij * dVA * f + VR * dfv + bij * VA * dfv);
    P[lb] = Pij;
#pragma unroll
    for (int c = 0; c < 3; c++) Gs[c * nbt + lb] = -(dff * nij[c]) - Pij * dbj[c];
  }
  __syncthreads();

  // Phase 3: k-role forces, energy.
  double ev = 0.0, ed = 0.0;
  for (int lb = tid; lb < nbt; lb += kTThreads) {
    const int mt = meta[lb];
    ev += E[lb].v;
    ed += E[lb].d;
    Dual G[3] = {Gs[lb], Gs[nbt + lb], Gs[2 * nbt + lb]};
    if (mt & kTFlagK) {
      const int ai = mt & 0xff;
      const int s = aseed[ai], z = aseed[ai + 1] - s, q = lb - s;
      const Dual *tcol = T + toff[ai] + q;
      for (int pq = 0; pq < z; pq++) {
        const int lp = s + pq;
        if (lp == lb || !(meta[lp] & kTFlagIJ)) continue;
        const Dual *tv = tcol + pq * z;
#pragma unroll
        for (int c = 0; c < 3; c++) G[c] = G[c] - P[lp] * tv[c * ntrip];
      }
    }
    Dual *Go = a.G + 3 * (size_t)(b0 + lb);
    Go[0] = G[0];
    Go[1] = G[1];
    Go[2] = G[2];
  }
  // tile energy (fixed tree)
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    ev += __shfl_down_sync(0xffffffffu, ev, off);
    ed += __shfl_down_sync(0xffffffffu, ed, off);
  }
  if ((tid & 31) == 0) {
    red[2 * (tid >> 5)] = ev;
    red[2 * (tid >> 5) + 1] = ed;
  }
  __syncthreads();
  if (tid < 10) {
    double v = 0.0;
    if (tid < 2)
      for (int w = 0; w < kTThreads / 32; w++) v += red[2 * w + tid];
    a.tile_part[10 * (size_t)tile + tid] = v;
  }
}

// F_a = sum_b (G[rev b] - G[b]) (value and derivative).
__global__ void tangent_gather(int nat, const int *__restrict__ seed,
                               const int *__restrict__ rev, const Dual *__restrict__ G,
                               double *__restrict__ f, double *__restrict__ df) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  double fv[3] = {0, 0, 0}, fd[3] = {0, 0, 0};
  for (int b = seed[i]; b < seed[i + 1]; b++) {
    const int rb = rev[b];
    if (rb < 0) continue;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const Dual gr = G[3 * (size_t)rb + c], gb = G[3 * (size_t)b + c];
      fv[c] += gr.v - gb.v;
      fd[c] += gr.d - gb.d;
    }
  }
#pragma unroll
  for (int c = 0; c < 3; c++) {
    f[3 * (size_t)i + c] = fv[c];
    df[3 * (size_t)i + c] = fd[c];
  }
}

TersoffTangent make_tangent(const double *q, const double *dq, int m) {
  TersoffTangent p;
  auto D = [&](int k) { return mk(q[k], dq ? dq[k] : 0.0); };
  p.A = D(0);
  p.B = D(1);
  p.lam = D(2);
  p.mu = D(3);
  p.beta = D(4);
  p.n = D(5);
  p.c = D(6);
  p.d = D(7);
  p.h = D(8);
  p.r1 = D(9);
  p.r2 = D(10);
  p.xi = D(11);
  p.om = D(12);
  p.mubo = D(13);
  p.m = m;
  p.h_one = p.mubo.v == 0.0 && p.mubo.d == 0.0;
  p.c2 = p.c * p.c;
  p.d2 = p.d * p.d;
  p.e = mk(-0.5) / p.n;
  p.fac = mk(M_PI) / (p.r2 - p.r1);
  return p;
}

}  // namespace

int batch_tersoff_tangent(Batch &b, int Z, int m, const double *params, const double *dparams,
                          const double *dr, double *epot, double *depot, double *f, double *df,
                          cudaStream_t s) {
  if (!params || !epot || !depot || !f || !df) {
    set_error("tersoff_tangent: params, epot, depot, f and df are required");
    return GB_ERROR_ARGUMENT;
  }
  if (b.nstruct == 0) return 0;
  if (b.nat > 0 && !b.r.p) {
    set_error("tersoff_tangent: positions not set");
    return GB_ERROR_ARGUMENT;
  }
  if (m < 1 || !(params[10] > params[9]) || !(params[9] > 0.0) || !(params[5] > 0.0) ||
      !(params[4] > 0.0)) {
    set_error("tersoff_tangent: invalid parameters (need 0 < R < S, n > 0, beta > 0, m >= 1)");
    return GB_ERROR_ARGUMENT;
  }
  if (!s) s = batch_stream(b);
  // elements: Z -> 0, others unknown to the potential
  std::vector<int> el(std::max(b.nat, 1), -1);
  for (int i = 0; i < b.nat; i++) el[i] = b.hZ[i] == Z ? 0 : -1;
  GB_CHECK(b.el.ensure(sizeof(int) * el.size()));
  GB_CUDA(cudaMemcpyAsync(b.el.p, el.data(), sizeof(int) * el.size(), cudaMemcpyHostToDevice, s));
  b.el_pot = nullptr;  // the element map no longer belongs to a potential
  const double cutoff = params[10];
  GB_CHECK(batch_binning(b, cutoff, s));
  if (!(b.nl.valid && b.built_pos == b.pos_rev)) {
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
  GB_CHECK(neighbors_build_reverse(b.nl, b.nat, s, true));
  // tiles whose worst case fits the tangent layout
  const int maxz = std::max(b.nl.maxz, 1);
  int apt = kTMaxApt;
  while (apt > 1 && tangent_smem(apt * maxz, apt * maxz * maxz) > 200 * 1024) apt >>= 1;
  if (tangent_smem(apt * maxz, apt * maxz * maxz) > 200 * 1024) {
    set_error("tersoff_tangent: an atom has too many neighbours for the tangent kernel");
    return GB_ERROR_CAPACITY;
  }
  GB_CHECK(batch_tiles(b, apt, s));
  const int ntiles = b.ntiles;
  const int64_t nb = std::max<int64_t>(b.nl.nentries, 1);
  DevBuf &G = b.tan_G, &part = b.tan_part, &fo = b.tan_f, &dp = b.tan_dpos, &red = b.tan_red;
  GB_CHECK(G.ensure(sizeof(Dual) * 3 * nb));
  GB_CHECK(part.ensure(sizeof(double) * 10 * std::max(ntiles, 1) + 64));
  GB_CHECK(fo.ensure(sizeof(double) * 6 * std::max(b.nat, 1)));
  GB_CHECK(red.ensure(sizeof(double) * 10 * std::max(b.nstruct, 1) + 64));
  const double *dpos = nullptr;
  if (dr) {
    if (is_device_ptr(dr)) {
      dpos = dr;
    } else {
      GB_CHECK(dp.ensure(sizeof(double) * 3 * std::max(b.nat, 1)));
      GB_CUDA(cudaMemcpyAsync(dp.p, dr, sizeof(double) * 3 * b.nat, cudaMemcpyHostToDevice, s));
      dpos = dp.as<double>();
    }
  }
  int *status = reinterpret_cast<int *>(part.as<double>() + 10 * (size_t)std::max(ntiles, 1));
  GB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, s));
  TangentArgs a;
  a.nat = b.nat;
  const int *t = b.tiles.as<int>();
  a.tile_atom0 = t;
  a.tile_struct = t + ntiles + 1;
  a.Acells = b.Acells.as<double>();
  a.pos = b.nl.pos4.as<Pos4>();
  a.dpos = dpos;
  a.el = b.el.as<int>();
  a.seed = b.nl.seed.as<int>();
  a.nbr = b.nl.nbr.as<int>();
  a.shift = b.nl.shift.as<int>();
  a.G = G.as<Dual>();
  a.tile_part = part.as<double>();
  const int max_nbt = apt * maxz, max_ntrip = apt * maxz * maxz;
  const size_t smem = tangent_smem(max_nbt, max_ntrip);
  if (smem > 48 * 1024)
    GB_CUDA(cudaFuncSetAttribute(tangent_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
  const TersoffTangent p = make_tangent(params, dparams, m);
  if (ntiles > 0) {
    tangent_tile<<<ntiles, kTThreads, smem, s>>>(a, p, max_nbt, max_ntrip, status);
    note_launch();
  }
  double *fv = fo.as<double>(), *fd = fv + 3 * (size_t)b.nat;
  if (b.nat > 0) {
    tangent_gather<<<(b.nat + 127) / 128, 128, 0, s>>>(b.nat, b.nl.seed.as<int>(),
                                                       b.nl.rev.as<int>(), a.G, fv, fd);
    note_launch();
  }
  GB_CHECK(reduce_segments(part.as<double>(), t + 2 * ntiles + 1, b.nstruct, red.as<double>(), s));
  std::vector<double> hred(10 * (size_t)b.nstruct);
  int hst[4];
  GB_CUDA(cudaMemcpyAsync(hred.data(), red.p, sizeof(double) * hred.size(),
                          cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(hst, status, sizeof(hst), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(f, fv, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
  GB_CUDA(cudaMemcpyAsync(df, fd, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaGetLastError());
  if (hst[0] & 2) {
    set_error("Internal error: tangent tile plan mismatch.");
    return GB_ERROR_UNSPECIFIED;
  }
  std::vector<double> e(b.nstruct), de(b.nstruct);
  for (int q = 0; q < b.nstruct; q++) {
    e[q] = hred[10 * q];
    de[q] = hred[10 * q + 1];
  }
  GB_CUDA(cudaMemcpy(epot, e.data(), sizeof(double) * e.size(), cudaMemcpyDefault));
  GB_CUDA(cudaMemcpy(depot, de.data(), sizeof(double) * de.size(), cudaMemcpyDefault));
  return 0;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_batch_tersoff_tangent(gb_batch_t *h, int Z, int m, const double *params,
                                        const double *dparams, const double *dr, double *epot,
                                        double *depot, double *f, double *df) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  return batch_tersoff_tangent(h->b, Z, m, params, dparams, dr, epot, depot, f, df, nullptr);
}
