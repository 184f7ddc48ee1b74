// Screened bond-order kernel (TersoffScr, KumagaiScr; included by bop.cu).
//
// The SCREENING branch of bop_kernel.f90 (pass 1 :682-995, pass 2
// :1171-1560 and the bond-order screening forces :1571-1611) with exp_cutoff
// cutoffs (cutoff.f90:232-293), FP64, one warp per atom i (its list
// displacements kept in shared memory):
//   pass 1  every list entry (i, j) is a candidate bond.  Inside the inner
//           cutoff r1 it is a bond with fc = 1; up to the largest cutoff its
//           screening by the other neighbours k of i is evaluated in list
//           order (C <= Cmin screens fully, Cmin < C < Cmax multiplies S by
//           exp(-((Cmax - C)/(C - Cmin))^2); the loop stops at a full screen
//           or once ln S < ln 1e-6); a screened bond beyond r2 is dropped, the
//           others get fc_ar = (1 - fc_in) S fc_out + fc_in, fc_bo likewise;
//   pass 2  the bond-order terms on the atom's bonds (VA/VR up to or2 with
//           fc_ar, zeta terms up to bor2 with fc_bo) and the forces on the
//           screening neighbours of each bond from its pair term;
//   then    the screening forces through fc_bo, scaled by the accumulated
//           d E / d fc_bo of the bond (sfacbo).
// Lanes take the candidate bonds (each runs its screening loop in list order);
// the kept bonds are compacted in list order.  The bond-order terms take a
// lane per bond ij, the forces on the k atoms a lane per bond ik (recomputing
// d zeta_ij / d r_k for the active ij in order), and the screening forces a
// bond at a time with the lanes over its screening entries: the entries of a
// bond are not stored, pass 1 records where its loop stopped and the same
// test picks them again.  Forces are written as G[b] = force on the end atom
// of list entry b from atom i's terms and gathered through the reverse index,
// as in the tile kernels; entries and per-bond outputs of atom i are written
// only by atom i's warp, in a fixed order (no atomics).  The decisions of the screening loop (the
// distance window, the dot-product signs, C against Cmin/Cmax and the ln S
// threshold) use unfused FP64 operations in the reference's order.

namespace gb {
namespace {

constexpr int kScrThreads = kBopThreads;  // block_sum assumes kBopThreads
constexpr int kScrMaxBonds = 32;          // bonds per atom after screening (a lane each)

struct ExpCutDev {
  double r1, r2, fac1, fac2, c, d, off;
};

inline ExpCutDev make_exp_cut(double a, double b) {
  ExpCutDev q;
  q.r1 = a;
  q.r2 = b;
  q.fac1 = 1.0 / (b - a);
  const double val1 = std::exp(-8.0);
  const double dval1 = -24 * val1;
  const double ddval1 = -48 * val1 - 24 * dval1;
  q.c = (-3 * dval1 + ddval1) / 3;
  q.d = (2 * dval1 - ddval1) / 4;
  q.fac2 = 1.0 / (1 - val1 - q.c - q.d);
  q.off = val1 + q.c + q.d;
  return q;
}

__device__ __forceinline__ void exp_cut(const ExpCutDev &q, double r, double &val, double &dval) {
  if (r <= q.r1) {
    val = 1.0;
    dval = 0.0;
  } else if (r >= q.r2) {
    val = 0.0;
    dval = 0.0;
  } else {
    const double x = q.fac1 * (r - q.r1);
    const double x2 = x * x;
    const double v = exp(-8 * x * x2);
    const double dv = -24 * x2 * v;
    dval = q.fac1 * q.fac2 * (dv + 3 * q.c * x2 + 4 * q.d * x * x2);
    val = q.fac2 * (v + q.c * x * x2 + q.d * x2 * x2 - q.off);
  }
}

struct ScrPair {
  ExpCutDev in, out, bo;
  double in_l2, in_h, in_h2, out_l, out_h, bo_h, max_cut_sq, Cmin, Cmax, dC, C_dr_cut;
};
struct ScrDev {
  ScrPair pr[9];
  double thr_s, thr_dot;  // ln 1e-6; 1e-10 as a default-real literal
};

// guard: C_dr_cut = 1 for Cmax <= 2 (default_bind_to_func.f90:62-68,
// brenner_module.f90:198-204); the Juslin module takes Cmax^2 / (4 (Cmax - 1))
// for every pair (juslin_module.f90:305-307).
inline ScrDev make_scr_dev(const double *r1, const double *r2, int npairs,
                           const gb_screening_params_t &s, bool guard = true) {
  ScrDev d{};
  for (int q = 0; q < npairs; q++) {
    ScrPair &p = d.pr[q];
    p.in = make_exp_cut(r1[q], r2[q]);
    p.out = make_exp_cut(s.or1[q], s.or2[q]);
    p.bo = make_exp_cut(s.bor1[q], s.bor2[q]);
    p.in_l2 = r1[q] * r1[q];
    p.in_h = r2[q];
    p.in_h2 = r2[q] * r2[q];
    p.out_l = s.or1[q];
    p.out_h = s.or2[q];
    p.bo_h = s.bor2[q];
    const double mc = std::max(std::max(r2[q], s.or2[q]), s.bor2[q]);
    p.max_cut_sq = mc * mc;
    p.Cmin = s.Cmin[q];
    p.Cmax = s.Cmax[q];
    p.dC = s.Cmax[q] - s.Cmin[q];
    p.C_dr_cut = (s.Cmax[q] > 2.0 || !guard) ? s.Cmax[q] * s.Cmax[q] / (4 * (s.Cmax[q] - 1))
                                             : 1.0;
  }
  d.thr_s = std::log(1e-6);
  d.thr_dot = (double)1e-10f;
  return d;
}

// r_k - r_i - A s of list entry kn (python_neighbors / bop_kernel.f90:593
// order, unfused).
__device__ __forceinline__ int scr_disp(const BopArgs &a, const Pos4 &pi, int kn, double d[3]) {
  const int k = a.nbr[kn];
  const Pos4 pk = a.pos[k];
  d[0] = __dsub_rn(pk.x, pi.x);
  d[1] = __dsub_rn(pk.y, pi.y);
  d[2] = __dsub_rn(pk.z, pi.z);
  int s0, s1, s2;
  unpack_shift(a.shift[kn], s0, s1, s2);
  if (s0 | s1 | s2) {
    const double sx = s0, sy = s1, sz = s2;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      double as = __dmul_rn(a.A[c][0], sx);
      as = __dadd_rn(as, __dmul_rn(a.A[c][1], sy));
      as = __dadd_rn(as, __dmul_rn(a.A[c][2], sz));
      d[c] = __dsub_rn(d[c], as);
    }
  }
  return k;
}

__device__ __forceinline__ double dot_rn(const double x[3], const double y[3]) {
  double s = __dmul_rn(x[0], y[0]);
  s = __dadd_rn(s, __dmul_rn(x[1], y[1]));
  return __dadd_rn(s, __dmul_rn(x[2], y[2]));
}

__device__ __forceinline__ void outer_add(double w[9], const double x[3], const double y[3]) {
#pragma unroll
  for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
    for (int c2 = 0; c2 < 3; c2++) w[c1 + 3 * c2] += x[c1] * y[c2];
}

constexpr int kScrWarps = kScrThreads / 32;  // atoms per block (a warp each)
constexpr int kScrCache = 192;               // list entries per atom kept in shared memory

// A bond of the atom after screening (shared memory, list order).
struct ScrBond {
  int jn, typ, need, kn_end;  // kn_end: where the screening loop stopped
  int active;                 // maskfac > 0 and within the outer cutoff
  int maskfac;
  double len, nm[3], fcar, dfcar, fcbo, dfcbo;
  double sij, fcin, fcar0, fcbo0;  // for the screening entries (need != 0)
  double dbdz, dffac2, sfacbo;     // from pass 2
};

struct ScrD4 {
  double x, y, z, w;
};

// Shared memory of one warp.
struct ScrWarpMem {
  ScrD4 rk[kScrCache];  // r_k - r_i of the atom's entries and its square
  int k[kScrCache], sh[kScrCache];
  ScrBond b[kScrMaxBonds];
};

// The atom's list entry kn: displacement, its square, end atom and shift
// (from the shared-memory copy when the list fits, else from the arrays).
__device__ __forceinline__ int scr_get(const BopArgs &a, const Pos4 &pi, const ScrWarpMem &W,
                                       bool cached, int s, int kn, double d[3], double &rr,
                                       int &sh) {
  if (cached) {
    const ScrD4 v = W.rk[kn - s];
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
    rr = v.w;
    sh = W.sh[kn - s];
    return W.k[kn - s];
  }
  const int k = scr_disp(a, pi, kn, d);
  rr = dot_rn(d, d);
  sh = a.shift[kn];
  return k;
}

// One step of the screening loop (bop_kernel.f90:733-799) for neighbour
// (k, rik) of bond (j, rij): 0 no effect, 1 full screen (C <= Cmin),
// 2 partial screen with t = (Cmax - C)/(C - Cmin) and the raw derivatives
// dS/dr_ij (dsij), dS/dr_ik / r_ik^2 (rik_raw), dS/dr_jk / r_jk^2 (rjk_raw).
__device__ __forceinline__ int scr_step(const ScrDev &sd, const ScrPair &P, int j, int shj,
                                        const double rij[3], double rlij, double rlim, int k,
                                        int shk, const double rik[3], double rlik, double &t,
                                        double &dsij, double &rik_raw, double &rjk_raw) {
  if (!(rlik < rlim)) return 0;
  if (k == j && shk == shj) return 0;
  const double dot_ij_ik = dot_rn(rij, rik);
  double rjk[3];
#pragma unroll
  for (int c = 0; c < 3; c++) rjk[c] = __dadd_rn(-rij[c], rik[c]);
  const double dot_ij_jk = dot_rn(rij, rjk);
  const double rljk = dot_rn(rjk, rjk);
  if (!(dot_ij_ik > sd.thr_dot && dot_ij_jk < -sd.thr_dot)) return 0;
  const double xik = __ddiv_rn(rlik, rlij), xjk = __ddiv_rn(rljk, rlij);
  const double xm = __dsub_rn(xik, xjk), xp = __dadd_rn(xik, xjk);
  const double xm2 = __dmul_rn(xm, xm);
  const double fac = __ddiv_rn(1.0, __dsub_rn(1.0, xm2));
  const double C = __dmul_rn(__dsub_rn(__dsub_rn(__dmul_rn(2.0, xp), xm2), 1.0), fac);
  if (C <= P.Cmin) return 1;
  if (!(C < P.Cmax)) return 0;
  const double Cmax_C = __dsub_rn(P.Cmax, C), C_Cmin = __dsub_rn(C, P.Cmin);
  t = __ddiv_rn(Cmax_C, C_Cmin);
  const double dCdrik = 4 * xik * fac * (1 + (C - 1) * xm);
  const double dCdrjk = 4 * xjk * fac * (1 - (C - 1) * xm);
  const double dCdrij = -(dCdrik + dCdrjk);
  const double f2 = 2 * Cmax_C * P.dC / (C_Cmin * C_Cmin * C_Cmin);
  dsij = f2 * dCdrij;
  rik_raw = f2 * dCdrik / rlik;
  rjk_raw = f2 * dCdrjk / rljk;
  return 2;
}

__device__ __forceinline__ double warp_sum_d(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Forces on the screening neighbours of need-bond Bj (the partial entries in
// [s, kn_end) of its screening loop), lanes over the entries: G[kn] gets
// -(d1 + d2), with d1 = f_ik r_ik, d2 = f_jk r_jk and (f_ik, f_jk) =
// scale (rik_raw, rjk_raw); the bond's own G[jn] gets sum d2 and its virial
// sum r_ik (x) d1 + r_jk (x) d2 (warp sums in a fixed order).
template <bool kWat>
__device__ __forceinline__ void scr_entry_forces(const BopArgs &a, const ScrDev &sd,
                                                 const Pos4 &pi, const ScrWarpMem &W,
                                                 bool cached, int s, int lane, const ScrBond &Bj,
                                                 double scale, double wacc[9]) {
  const ScrPair &P = sd.pr[Bj.typ];
  double r0[3], rl0;
  int sh0;
  const int j = scr_get(a, pi, W, cached, s, Bj.jn, r0, rl0, sh0);
  const double rlim = __dmul_rn(P.C_dr_cut, rl0);
  const double rij[3] = {Bj.len * Bj.nm[0], Bj.len * Bj.nm[1], Bj.len * Bj.nm[2]};
  double fj[3] = {0.0, 0.0, 0.0}, w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int kn = s + lane; kn < Bj.kn_end; kn += 32) {
    double rik[3], rlik;
    int shk;
    const int k = scr_get(a, pi, W, cached, s, kn, rik, rlik, shk);
    double t, dsij, rik_raw, rjk_raw;
    if (scr_step(sd, P, j, sh0, r0, rl0, rlim, k, shk, rik, rlik, t, dsij, rik_raw, rjk_raw) != 2)
      continue;
    const double fik = scale * (rik_raw * Bj.sij * (Bj.need == 1 ? Bj.fcar0 : Bj.fcbo0) *
                                (1.0 - Bj.fcin));
    const double fjk = scale * (rjk_raw * Bj.sij * (Bj.need == 1 ? Bj.fcar0 : Bj.fcbo0) *
                                (1.0 - Bj.fcin));
    double rjk[3], d1[3], d2[3];
    double *Gk = a.G + 3 * (size_t)kn;
#pragma unroll
    for (int c = 0; c < 3; c++) {
      rjk[c] = -rij[c] + rik[c];
      d1[c] = fik * rik[c];
      d2[c] = fjk * rjk[c];
      fj[c] += d2[c];
      Gk[c] += -d1[c] - d2[c];
    }
    outer_add(w, rik, d1);
    outer_add(w, rjk, d2);
  }
#pragma unroll
  for (int c = 0; c < 3; c++) fj[c] = warp_sum_d(fj[c]);
#pragma unroll
  for (int c = 0; c < 9; c++) w[c] = warp_sum_d(w[c]);
  if (lane == 0) {
    double *Gj = a.G + 3 * (size_t)Bj.jn;
#pragma unroll
    for (int c = 0; c < 3; c++) Gj[c] += fj[c];
#pragma unroll
    for (int c = 0; c < 9; c++) wacc[c] += w[c];
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)Bj.jn + c] += w[c];
  }
  __syncwarp();
}

template <class Pot, bool kWat, bool kPB>
__global__ void __launch_bounds__(kScrThreads)
    bop_scr_atom(const BopArgs a, const Pot pot, const ScrDev sd, int *status) {
  extern __shared__ __align__(16) unsigned char scr_sm[];
  __shared__ double red_scratch[(kScrThreads / 32) * 9];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  ScrWarpMem &W = reinterpret_cast<ScrWarpMem *>(scr_sm)[wid];
  const int i = blockIdx.x * kScrWarps + wid;
  double eacc[1] = {0.0};
  double wacc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int eli = i < a.nat ? a.el[i] : -1;
  if (i < a.nat) {
    const int s = a.seed[i], e = a.seed[i + 1];
    for (int b = s + lane; b < e; b += 32) {  // this atom's entries start from zero
#pragma unroll
      for (int c = 0; c < 3; c++) a.G[3 * (size_t)b + c] = 0.0;
      if (a.ebond) a.ebond[b] = 0.0;
      if (kPB)
#pragma unroll
        for (int c = 0; c < 3; c++) a.frbond[3 * (size_t)b + c] = 0.0;
      if (kWat)
#pragma unroll
        for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)b + c] = 0.0;
    }
  }
  if (eli >= 0) {  // (uniform over the warp)
    const int s = a.seed[i], e = a.seed[i + 1];
    const Pos4 pi = a.pos[i];
    const int nel = pot.nel();
    const bool cached = e - s <= kScrCache;
    if (cached)
      for (int kn = s + lane; kn < e; kn += 32) {
        double d[3];
        const int k = scr_disp(a, pi, kn, d);
        W.rk[kn - s] = ScrD4{d[0], d[1], d[2], dot_rn(d, d)};
        W.k[kn - s] = k;
        W.sh[kn - s] = a.shift[kn];
      }
    __syncwarp();
    // ---- Pass 1: candidates over the lanes, kept bonds compacted in list
    // order. ----
    int nb = 0;
    bool overflow = false;
    for (int base = s; base < e; base += 32) {
      const int jn = base + lane;
      bool keep = false;
      ScrBond bd;
      if (jn < e) {
        double rij[3], rlij;
        int shj;
        const int j = scr_get(a, pi, W, cached, s, jn, rij, rlij, shj);
        const int elj = a.el[j];
        if (elj >= 0) {
          const int t = pot.pair(eli, elj);
          const ScrPair &P = sd.pr[t];
          bd.jn = jn;
          bd.typ = t;
          bd.need = 0;
          bd.kn_end = s;
          bd.sij = bd.fcin = bd.fcar0 = bd.fcbo0 = 0.0;
          keep = true;
          if (rlij < P.in_l2) {
            bd.fcar = bd.fcbo = 1.0;
            bd.dfcar = bd.dfcbo = 0.0;
          } else if (rlij < P.max_cut_sq && P.out_l < P.out_h) {
            bool screened = false, need = false;
            double sij = 0.0, dsijdrij = 0.0;
            const double rlim = __dmul_rn(P.C_dr_cut, rlij);
            int kn = s;
            for (; !(screened || sij < sd.thr_s) && kn < e; kn++) {
              double rik[3], rlik;
              int shk;
              const int k = scr_get(a, pi, W, cached, s, kn, rik, rlik, shk);
              double tt, dsij, u, v;
              const int r = scr_step(sd, P, j, shj, rij, rlij, rlim, k, shk, rik, rlik, tt, dsij,
                                     u, v);
              if (r == 1) {
                screened = true;
              } else if (r == 2) {
                need = true;
                sij = __dsub_rn(sij, __dmul_rn(tt, tt));
                dsijdrij = dsijdrij + dsij;
              }
            }
            bd.kn_end = kn;
            if ((screened || sij < sd.thr_s) && rlij > P.in_h2) {
              keep = false;  // fully screened
            } else {
              const double rl = sqrt(rlij);
              double fcin, dfcin;
              if (screened) {
                exp_cut(P.in, rl, fcin, dfcin);
                bd.fcar = bd.fcbo = fcin;
                bd.dfcar = bd.dfcbo = dfcin;
              } else if (need) {
                sij = exp(sij);
                double fcar, dfcar, fcbo, dfcbo;
                exp_cut(P.in, rl, fcin, dfcin);
                exp_cut(P.out, rl, fcar, dfcar);
                exp_cut(P.bo, rl, fcbo, dfcbo);
                bd.fcar = (1.0 - fcin) * sij * fcar + fcin;
                bd.dfcar =
                    (1.0 - fcin) * sij * (dfcar + fcar * dsijdrij / rl) - dfcin * sij * fcar + dfcin;
                bd.fcbo = (1.0 - fcin) * sij * fcbo + fcin;
                bd.dfcbo =
                    (1.0 - fcin) * sij * (dfcbo + fcbo * dsijdrij / rl) - dfcin * sij * fcbo + dfcin;
                bd.need = 1;
                bd.sij = sij;
                bd.fcin = fcin;
                bd.fcar0 = fcar;
                bd.fcbo0 = fcbo;
              } else {
                double fcar, dfcar, fcbo, dfcbo;
                exp_cut(P.out, rl, fcar, dfcar);
                exp_cut(P.bo, rl, fcbo, dfcbo);
                if (rl < P.in_h) {
                  exp_cut(P.in, rl, fcin, dfcin);
                  bd.fcar = (1.0 - fcin) * fcar + fcin;
                  bd.dfcar = (1.0 - fcin) * dfcar - dfcin * fcar + dfcin;
                  bd.fcbo = (1.0 - fcin) * fcbo + fcin;
                  bd.dfcbo = (1.0 - fcin) * dfcbo - dfcin * fcbo + dfcin;
                } else {
                  bd.fcar = fcar;
                  bd.dfcar = dfcar;
                  bd.fcbo = fcbo;
                  bd.dfcbo = dfcbo;
                }
              }
            }
          } else if (rlij < P.in_h2) {
            double fcin, dfcin;
            exp_cut(P.in, sqrt(rlij), fcin, dfcin);
            bd.fcar = bd.fcbo = fcin;
            bd.dfcar = bd.dfcbo = dfcin;
          } else {
            keep = false;
          }
          if (keep) {
            const double rl = sqrt(rlij);
            bd.len = rl;
#pragma unroll
            for (int c = 0; c < 3; c++) bd.nm[c] = rij[c] / rl;
            int mf = 2;
            if (a.mask) {
              const int mi = a.mask[i], mj = a.mask[j];
              if (mi == 0 && mj == 0)
                mf = 0;
              else if (mi == 0 || mj == 0)
                mf = 1;
            }
            bd.maskfac = mf;
            bd.active = mf > 0 && rl < P.out_h;
            bd.dbdz = bd.dffac2 = bd.sfacbo = 0.0;
          }
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      const int pos = nb + __popc(bal & ((1u << lane) - 1u));
      if (keep && pos < kScrMaxBonds) W.b[pos] = bd;
      nb += __popc(bal);
      if (nb > kScrMaxBonds) {
        overflow = true;
        break;
      }
    }
    __syncwarp();
    if (overflow) {
      if (lane == 0) atomicOr(status, 4);
    } else {
      // ---- Pass 2a: lane ij, the bond order and the forces on i and j
      // (the force on i itself is minus the sum of its entries' G by
      // translation invariance; it is not accumulated). ----
      if (lane < nb && W.b[lane].active) {
        ScrBond &Bj = W.b[lane];
        const int t = Bj.typ;
        const double rlij = Bj.len, rlijr = 1.0 / rlij;
        const double rnij[3] = {Bj.nm[0], Bj.nm[1], Bj.nm[2]};
        const double rij[3] = {rlij * rnij[0], rlij * rnij[1], rlij * rnij[2]};
        const double fcarij = Bj.fcar, dfcarijr = Bj.dfcar;
        double VA, dVA, VR, dVR;
        pot.VA(t, rlij, VA, dVA);
        pot.VR(t, rlij, VR, dVR);
        const double hm = 0.5 * Bj.maskfac;
        VA *= hm;
        dVA *= hm;
        VR *= hm;
        dVR *= hm;
        double wij[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, wijb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double zij = 0.0, dbidj[3] = {0.0, 0.0, 0.0};
        for (int ik = 0; ik < nb; ik++) {
          if (ik == lane) continue;
          const ScrBond &Bk = W.b[ik];
          const int ikpot = Bk.typ;
          const double rlik = Bk.len;
          if (!(rlik < sd.pr[ikpot].bo_h)) continue;
          const double rnik[3] = {Bk.nm[0], Bk.nm[1], Bk.nm[2]};
          const double rik[3] = {rlik * rnik[0], rlik * rnik[1], rlik * rnik[2]};
          const double fcik = Bk.fcbo, dfcikr = Bk.dfcbo;
          double h_Dr, dh_dDr;
          pot.template h<double>(eli, t, ikpot, rlij - rlik, h_Dr, dh_dDr);
          const double costh = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
          double g_costh, dg_dcosth;
          pot.template g_hc<double>(eli, ikpot, pot.hpar(eli, ikpot) - costh, g_costh, dg_dcosth);
          double dkc[3];
#pragma unroll
          for (int c = 0; c < 3; c++) dkc[c] = rnik[c] * rlik - rnij[c] * rlij;
          const double disjk = sqrt(dkc[0] * dkc[0] + dkc[1] * dkc[1] + dkc[2] * dkc[2]);
#pragma unroll
          for (int c = 0; c < 3; c++) dkc[c] = dkc[c] / disjk;
          const double dcsdij = 1.0 / rlik - costh * rlijr;
          const double dcsdik = rlijr - costh / rlik;
          const double dcsdjk = -disjk * rlijr / rlik;
          const double dzfac = fcik * dg_dcosth * h_Dr;
          zij = zij + fcik * g_costh * h_Dr;
          const double dzdrij = g_costh * fcik * dh_dDr;
          const double dzdrik = g_costh * (dfcikr * h_Dr - fcik * dh_dDr);
          double df[3], dk[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const double dcsdj = dcsdij * rnij[c] - dcsdjk * dkc[c];
            const double dcsdk = dcsdik * rnik[c] + dcsdjk * dkc[c];
            df[c] = dzdrij * rnij[c] + dzfac * dcsdj;
            dbidj[c] = dbidj[c] + df[c];
            dk[c] = dzdrik * rnik[c] + dzfac * dcsdk;
          }
#pragma unroll
          for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
            for (int c2 = 0; c2 < 3; c2++)
              wijb[c1 + 3 * c2] -= rij[c1] * df[c2] + rik[c1] * dk[c2];
        }
        double bij, dbdz;
        pot.template bo<double>(eli, t, zij, fcarij, VA, bij, dbdz);
        const double dffac = 0.5 * fcarij * (VR + bij * VA);
        eacc[0] += dffac;
        if (a.ebond) a.ebond[Bj.jn] = dffac;
        const double dffr =
            0.5 * (dVR * fcarij + bij * dVA * fcarij + VR * dfcarijr + bij * VA * dfcarijr);
        double df[3], fj[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          df[c] = dffr * rnij[c];
          fj[c] = -df[c] - dbdz * dbidj[c];
        }
        outer_add(wij, rij, df);
#pragma unroll
        for (int c = 0; c < 9; c++) wij[c] -= dbdz * wijb[c];
        if (kPB)
#pragma unroll
          for (int c = 0; c < 3; c++) a.frbond[3 * (size_t)Bj.jn + c] = df[c];
#pragma unroll
        for (int c = 0; c < 9; c++) wacc[c] += wij[c];
        if (kWat)
#pragma unroll
          for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)Bj.jn + c] += wij[c];
        double *Gj = a.G + 3 * (size_t)Bj.jn;
#pragma unroll
        for (int c = 0; c < 3; c++) Gj[c] += fj[c];
        Bj.dbdz = dbdz;
        Bj.dffac2 = 0.5 * (VR + bij * VA);
      }
      __syncwarp();
      // ---- Pass 2b: lane ik, the k-role forces -dbdz_ij d zeta_ij / d r_k
      // over the active bonds ij in order, and d E / d fc_bo of bond ik
      // (sfacbo, :1462-1471). ----
      if (lane < nb) {
        ScrBond &Bk = W.b[lane];
        const int ikpot = Bk.typ;
        const double rlik = Bk.len;
        if (rlik < sd.pr[ikpot].bo_h) {
          const double rnik[3] = {Bk.nm[0], Bk.nm[1], Bk.nm[2]};
          const double fcik = Bk.fcbo, dfcikr = Bk.dfcbo;
          double Gk[3] = {0.0, 0.0, 0.0}, sfac = 0.0;
          for (int ij = 0; ij < nb; ij++) {
            if (ij == lane) continue;
            const ScrBond &Bj = W.b[ij];
            if (!Bj.active) continue;
            const double rlij = Bj.len, rlijr = 1.0 / rlij;
            const double rnij[3] = {Bj.nm[0], Bj.nm[1], Bj.nm[2]};
            double h_Dr, dh_dDr;
            pot.template h<double>(eli, Bj.typ, ikpot, rlij - rlik, h_Dr, dh_dDr);
            const double costh = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
            double g_costh, dg_dcosth;
            pot.template g_hc<double>(eli, ikpot, pot.hpar(eli, ikpot) - costh, g_costh, dg_dcosth);
            double dkc[3];
#pragma unroll
            for (int c = 0; c < 3; c++) dkc[c] = rnik[c] * rlik - rnij[c] * rlij;
            const double disjk = sqrt(dkc[0] * dkc[0] + dkc[1] * dkc[1] + dkc[2] * dkc[2]);
#pragma unroll
            for (int c = 0; c < 3; c++) dkc[c] = dkc[c] / disjk;
            const double dcsdik = rlijr - costh / rlik;
            const double dcsdjk = -disjk * rlijr / rlik;
            const double dzfac = fcik * dg_dcosth * h_Dr;
            const double dzdrik = g_costh * (dfcikr * h_Dr - fcik * dh_dDr);
#pragma unroll
            for (int c = 0; c < 3; c++) {
              const double dcsdk = dcsdik * rnik[c] + dcsdjk * dkc[c];
              Gk[c] += -Bj.dbdz * (dzdrik * rnik[c] + dzfac * dcsdk);
            }
            if (Bk.need) sfac = sfac + g_costh * h_Dr * Bj.dbdz;
          }
          double *G = a.G + 3 * (size_t)Bk.jn;
#pragma unroll
          for (int c = 0; c < 3; c++) G[c] += Gk[c];
          Bk.sfacbo = sfac;
        }
      }
      __syncwarp();
      // ---- Screening forces: through fc_ar from the pair term of each
      // active need-bond (:1531-1560), then through fc_bo scaled by sfacbo
      // (:1571-1611); lanes over the bond's screening entries. ----
      for (int q = 0; q < nb; q++) {
        const ScrBond &Bj = W.b[q];
        if (Bj.need && Bj.active)
          scr_entry_forces<kWat>(a, sd, pi, W, cached, s, lane, Bj, Bj.dffac2, wacc);
      }
      for (int q = 0; q < nb; q++) {
        ScrBond Bj = W.b[q];
        if (Bj.need && Bj.sfacbo != 0.0) {
          Bj.need = 2;  // (selects fc_bo in scr_entry_forces)
          scr_entry_forces<kWat>(a, sd, pi, W, cached, s, lane, Bj, Bj.sfacbo, wacc);
        }
      }
    }
  }
  double *part = a.tile_part + 10 * (size_t)blockIdx.x;
  block_sum<1>(eacc, part, red_scratch);
  block_sum<9>(wacc, part + 1, red_scratch);
}

}  // namespace
}  // namespace gb
