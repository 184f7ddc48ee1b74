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
// Per-bond Dual slots: rn (3), r, 1/r, fc, dfc/dr, P, E, G (3), and for the
// adjoint dfc/dR, dfc/dS.
constexpr int kTBondSlots = 14;
__host__ __device__ inline size_t tangent_smem(int nbt, int ntrip) {
  size_t o = talign(sizeof(int) * (2 * kTMaxApt + 2 + (size_t)nbt));
  o += talign(sizeof(Dual) * (size_t)nbt * kTBondSlots);
  o += talign(sizeof(Dual) * (size_t)ntrip * 3);
  return o + 64;
}

// Parameter order of the gradients (and of the parameter vector).
enum TParam { tA, tB, tLam, tMu, tBeta, tN, tC, tD, tH, tR, tS, tXi, tOm, tMubo, kTParams };
// Columns of a tile row: E (value, derivative), dE/dtheta (14 values, 14
// derivatives along the position direction), 2 spare.
constexpr int kTRow = 32;

// kAdj = false: the tangent evaluation (E, F and their derivatives along a
// direction in parameters and positions).  kAdj = true: in addition the
// reverse-mode gradient dE/dtheta of the 14 parameters, written by hand
// below, with every quantity still a Dual along the position direction v:
// one pass gives dE/dtheta and D_v(dE/dtheta) = d(v . dE/dr)/dtheta, the
// parameter gradient of the force-matching term, next to D_v F = -H v.
template <bool kAdj>
__global__ void __launch_bounds__(kTThreads)
    tangent_tile(const TangentArgs a, const TersoffTangent p, int max_nbt, int max_ntrip,
                 int *status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double sA[9];
  __shared__ double red[(kAdj ? kTRow : 2) * (kTThreads / 32)];
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
       *P = D + 7 * nbt, *E = D + 8 * nbt, *Gs = D + 9 * nbt, *dfcR = D + 12 * nbt,
       *dfcS = D + 13 * nbt;
  o += talign(sizeof(Dual) * (size_t)nbt * kTBondSlots);
  Dual *T = reinterpret_cast<Dual *>(sm + o);
  for (int q = tid; q < na; q += kTThreads)
    for (int lb = aseed[q]; lb < aseed[q + 1]; lb++) meta[lb] = q;
  __syncthreads();

  // Phase 1: bond geometry.
  for (int lb = tid; lb < nbt; lb += kTThreads) {
    const int ai = meta[lb];
    const int i = a0 + ai, b = b0 + lb, j = a.nbr[b];
    int mt = ai;
    Dual f = mk(0.0), df = mk(0.0), r = mk(1.0), ri = mk(1.0), fR = mk(0.0), fS = mk(0.0);
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
          const Dual x = p.fac * (r - p.r1);
          dsincos(x, sx, cx);
          f = 0.5 * (1.0 + cx);
          df = -0.5 * (p.fac * sx);
          if (kAdj) {
            // x = pi (r - R) / (S - R): dx/dR = (x - pi) / (S - R), dx/dS = -x / (S - R)
            const Dual w = p.r2 - p.r1;
            fR = -0.5 * (sx * ((x - mk(M_PI)) / w));
            fS = 0.5 * (sx * (x / w));
          }
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
    if (kAdj) {
      dfcR[lb] = fR;
      dfcS[lb] = fS;
    }
  }
  __syncthreads();

  // Phase 2: per bond ij, zeta and its derivatives, b, P, energy, j-role G;
  // with kAdj also the bond's share of dE/dtheta.
  Dual gth[kAdj ? kTParams : 1];
#pragma unroll
  for (int q = 0; q < (kAdj ? kTParams : 1); q++) gth[q] = mk(0.0);
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
    // kAdj: d zeta / d (c, d, h, omega, mubo, R, S)
    Dual zc = mk(0.0), zd = mk(0.0), zh = mk(0.0), zom = mk(0.0), zmu = mk(0.0),
         zR = mk(0.0), zS = mk(0.0);
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
      Dual hv = mk(1.0), dh = mk(0.0), dhmu = mk(0.0);
      if (!p.h_one) {
        const Dual drr = r - rl[lk];
        const Dual x = 2.0 * (p.mubo * drr);
        Dual pw = mk(1.0);
        for (int k = 1; k < p.m; k++) pw = pw * x;
        hv = dexp(pw * x);
        dh = 2.0 * (p.mubo * ((double)p.m * (pw * hv)));
        // h = exp((2 mubo dr)^m): dh/dmubo = 2 m dr (2 mubo dr)^(m-1) h
        if (kAdj) dhmu = 2.0 * (drr * ((double)p.m * (pw * hv)));
      }
      const Dual cs = nik[0] * nij[0] + nik[1] * nij[1] + nik[2] * nij[2];
      // g = omega (1 + c^2 hc^2 / (d^2 (d^2 + hc^2))), hc = h - cos theta
      const Dual hc = p.h - cs;
      const Dual den = p.d2 + hc * hc;
      const Dual gv = p.om * (1.0 + (p.c2 * hc * hc) / (p.d2 * den));
      const Dual dg = -2.0 * ((p.om * p.c2 * hc) / (den * den));
      const Dual fk = fc[lk];
      if (kAdj) {
        // g = omega G0, G0 = 1 + c^2 hc^2 / (d^2 den), den = d^2 + hc^2
        const Dual fh = fk * hv;
        const Dual G0 = 1.0 + (p.c2 * hc * hc) / (p.d2 * den);
        const Dual dd2 = p.d2 * den;
        zom = zom + fh * G0;
        zc = zc + fh * (2.0 * (p.om * p.c * hc * hc) / dd2);
        zd = zd - fh * (2.0 * (p.om * p.c2 * hc * hc * p.d * (2.0 * p.d2 + hc * hc)) /
                        (dd2 * dd2));
        zh = zh + fh * (2.0 * (p.om * p.c2 * hc) / (den * den));
        zmu = zmu + fk * gv * dhmu;
        zR = zR + dfcR[lk] * gv * hv;
        zS = zS + dfcS[lk] * gv * hv;
      }
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
    Dual bxi = mk(0.0), bbeta = mk(0.0), bn = mk(0.0);  // d b / d (xi, beta, n)
    if (zeta.v > 0.0) {
      const Dual lbz = dlog(p.beta) + dlog(zeta);
      const Dual x = dexp(p.n * lbz);
      const Dual l1x = dlog(1.0 + x);
      const Dual ae = dexp(p.e * l1x);
      bij = p.xi * ae;
      Pij = -0.25 * (fc[lb] * VA * p.xi * (x / zeta) * (ae / (1.0 + x)));
      if (kAdj) {
        // ln b = ln xi - ln(1 + x) / (2 n), x = (beta zeta)^n
        bxi = ae;
        bbeta = -0.5 * (bij * x / (p.beta * (1.0 + x)));
        bn = bij * (l1x / (2.0 * (p.n * p.n)) - (x * lbz) / (2.0 * (p.n * (1.0 + x))));
      }
    }
    const Dual f = fc[lb], dfv = dfc[lb];
    E[lb] = 0.5 * (f * (VR + bij * VA));
    if (kAdj) {
      // e = f (VR + b VA) / 2 with VR = A e^{-lambda r}, VA = -B e^{-mu r}
      const Dual hf = 0.5 * f, v = VR + bij * VA, hfVA = hf * VA;
      gth[tA] = gth[tA] + hf * eR;
      gth[tLam] = gth[tLam] - hf * (r * VR);
      gth[tB] = gth[tB] - hf * (bij * eA);
      gth[tMu] = gth[tMu] - hf * (bij * (r * VA));
      gth[tXi] = gth[tXi] + hfVA * bxi;
      gth[tBeta] = gth[tBeta] + hfVA * bbeta;
      gth[tN] = gth[tN] + hfVA * bn;
      gth[tR] = gth[tR] + 0.5 * (dfcR[lb] * v) + Pij * zR;
      gth[tS] = gth[tS] + 0.5 * (dfcS[lb] * v) + Pij * zS;
      gth[tC] = gth[tC] + Pij * zc;
      gth[tD] = gth[tD] + Pij * zd;
      gth[tH] = gth[tH] + Pij * zh;
      gth[tOm] = gth[tOm] + Pij * zom;
      gth[tMubo] = gth[tMubo] + Pij * zmu;
    }
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
  // tile sums (fixed trees): energy, and with kAdj dE/dtheta
  constexpr int kCols = kAdj ? kTRow : 2;
  double col[kCols];
  col[0] = ev;
  col[1] = ed;
  if (kAdj) {
#pragma unroll
    for (int q = 0; q < kTParams; q++) {
      col[2 + q] = gth[q].v;
      col[2 + kTParams + q] = gth[q].d;
    }
#pragma unroll
    for (int q = 2 + 2 * kTParams; q < kCols; q++) col[q] = 0.0;
  }
#pragma unroll
  for (int q = 0; q < kCols; q++) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) col[q] += __shfl_down_sync(0xffffffffu, col[q], off);
    if ((tid & 31) == 0) red[kCols * (tid >> 5) + q] = col[q];
  }
  __syncthreads();
  const int rowlen = kAdj ? kTRow : 10;
  if (tid < rowlen) {
    double v = 0.0;
    if (tid < kCols)
      for (int w = 0; w < kTThreads / 32; w++) v += red[kCols * w + tid];
    a.tile_part[rowlen * (size_t)tile + tid] = v;
  }
}

// Per-structure sums of the kTRow-column tile rows, rows in order.
__global__ void adjoint_segments(const double *__restrict__ part, const int *__restrict__ seg,
                                 double *__restrict__ out) {
  const int q = blockIdx.x, c = threadIdx.x;
  double v = 0.0;
  for (int t = seg[q]; t < seg[q + 1]; t++) v += part[kTRow * (size_t)t + c];
  out[kTRow * (size_t)q + c] = v;
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

// One tile pass over the batch.  adj = false: tangent along (dparams, dr);
// outputs epot/depot (nstruct), f/df (nat,3).  adj = true: dparams must be
// NULL; additionally dEdp / dvdEdp (nstruct,14): dE_s/dtheta and its
// derivative along dr.  Output pointers may be host or device memory.
int batch_tersoff_eval(Batch &b, int Z, int m, const double *params, const double *dparams,
                       const double *dr, bool adj, double *epot, double *depot, double *f,
                       double *df, double *dEdp, double *dvdEdp, cudaStream_t s) {
  if (!params || !epot || !f || (!adj && (!depot || !df))) {
    set_error("tersoff_tangent: params, epot, depot, f and df are required");
    return GB_ERROR_ARGUMENT;
  }
  if (adj && (dparams || !dEdp)) {
    set_error("tersoff_adjoint: dE/dparams is required; no parameter direction");
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
  const int rowlen = adj ? kTRow : 10;
  const int64_t nb = std::max<int64_t>(b.nl.nentries, 1);
  DevBuf &G = b.tan_G, &part = b.tan_part, &fo = b.tan_f, &dp = b.tan_dpos, &red = b.tan_red;
  GB_CHECK(G.ensure(sizeof(Dual) * 3 * nb));
  GB_CHECK(part.ensure(sizeof(double) * rowlen * std::max(ntiles, 1) + 64));
  GB_CHECK(fo.ensure(sizeof(double) * 6 * std::max(b.nat, 1)));
  GB_CHECK(red.ensure(sizeof(double) * rowlen * std::max(b.nstruct, 1) + 64));
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
  int *status = reinterpret_cast<int *>(part.as<double>() + rowlen * (size_t)std::max(ntiles, 1));
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
  TersoffTangent p = make_tangent(params, dparams, m);
  if (adj) p.h_one = false;  // mubo is differentiated even at 0
  if (ntiles > 0) {
    if (adj) {
      if (smem > 48 * 1024)
        GB_CUDA(cudaFuncSetAttribute(tangent_tile<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      tangent_tile<true><<<ntiles, kTThreads, smem, s>>>(a, p, max_nbt, max_ntrip, status);
    } else {
      if (smem > 48 * 1024)
        GB_CUDA(cudaFuncSetAttribute(tangent_tile<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      tangent_tile<false><<<ntiles, kTThreads, smem, s>>>(a, p, max_nbt, max_ntrip, status);
    }
    note_launch();
  }
  double *fv = fo.as<double>(), *fd = fv + 3 * (size_t)b.nat;
  if (b.nat > 0) {
    tangent_gather<<<(b.nat + 127) / 128, 128, 0, s>>>(b.nat, b.nl.seed.as<int>(),
                                                       b.nl.rev.as<int>(), a.G, fv, fd);
    note_launch();
  }
  if (adj) {
    adjoint_segments<<<b.nstruct, kTRow, 0, s>>>(part.as<double>(), t + 2 * ntiles + 1,
                                                  red.as<double>());
    note_launch();
  } else {
    GB_CHECK(reduce_segments(part.as<double>(), t + 2 * ntiles + 1, b.nstruct, red.as<double>(),
                             s));
  }
  std::vector<double> hred(rowlen * (size_t)b.nstruct);
  int hst[4];
  GB_CUDA(cudaMemcpyAsync(hred.data(), red.p, sizeof(double) * hred.size(),
                          cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(hst, status, sizeof(hst), cudaMemcpyDeviceToHost, s));
  GB_CUDA(cudaMemcpyAsync(f, fv, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
  if (df) GB_CUDA(cudaMemcpyAsync(df, fd, sizeof(double) * 3 * b.nat, cudaMemcpyDefault, s));
  GB_CUDA(cudaStreamSynchronize(s));
  GB_CUDA(cudaGetLastError());
  if (hst[0] & 2) {
    set_error("Internal error: tangent tile plan mismatch.");
    return GB_ERROR_UNSPECIFIED;
  }
  std::vector<double> e(b.nstruct), de(b.nstruct);
  for (int q = 0; q < b.nstruct; q++) {
    e[q] = hred[rowlen * q];
    de[q] = hred[rowlen * q + 1];
  }
  GB_CUDA(cudaMemcpy(epot, e.data(), sizeof(double) * e.size(), cudaMemcpyDefault));
  if (depot) GB_CUDA(cudaMemcpy(depot, de.data(), sizeof(double) * de.size(), cudaMemcpyDefault));
  if (adj) {
    std::vector<double> gv((size_t)kTParams * b.nstruct), gd((size_t)kTParams * b.nstruct);
    for (int q = 0; q < b.nstruct; q++)
      for (int k = 0; k < kTParams; k++) {
        gv[(size_t)kTParams * q + k] = hred[rowlen * q + 2 + k];
        gd[(size_t)kTParams * q + k] = hred[rowlen * q + 2 + kTParams + k];
      }
    GB_CUDA(cudaMemcpy(dEdp, gv.data(), sizeof(double) * gv.size(), cudaMemcpyDefault));
    if (dvdEdp)
      GB_CUDA(cudaMemcpy(dvdEdp, gd.data(), sizeof(double) * gd.size(), cudaMemcpyDefault));
  }
  return 0;
}

int batch_tersoff_tangent(Batch &b, int Z, int m, const double *params, const double *dparams,
                          const double *dr, double *epot, double *depot, double *f, double *df,
                          cudaStream_t s) {
  return batch_tersoff_eval(b, Z, m, params, dparams, dr, false, epot, depot, f, df, nullptr,
                            nullptr, s);
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

extern "C" int gb_batch_tersoff_adjoint(gb_batch_t *h, int Z, int m, const double *params,
                                        const double *v, double *epot, double *f, double *hv,
                                        double *dE_dparams, double *dv_dE_dparams) {
  clear_error();
  if (!h) return GB_ERROR_ARGUMENT;
  return batch_tersoff_eval(h->b, Z, m, params, nullptr, v, true, epot, nullptr, f, hv,
                            dE_dparams, dv_dE_dparams, nullptr);
}
