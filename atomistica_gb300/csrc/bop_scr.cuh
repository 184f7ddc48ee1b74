// Screened bond-order kernel (TersoffScr, KumagaiScr; included by bop.cu).
//
// The SCREENING branch of bop_kernel.f90 (pass 1 :682-995, pass 2
// :1171-1560 and the bond-order screening forces :1571-1611) with exp_cutoff
// cutoffs (cutoff.f90:232-293), FP64, one thread per atom i:
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
// The screening entries of a bond are not stored: the screening loop is
// rerun (same code, same early exit, so the same entries) when its forces are
// applied.  Forces are written as G[b] = force on the end atom of list entry b
// from atom i's terms and gathered through the reverse index, as in the tile
// kernels; bonds, entries and per-bond outputs of atom i are written only by
// atom i's thread (no atomics).  The decisions of the screening loop (the
// distance window, the dot-product signs, C against Cmin/Cmax and the ln S
// threshold) use unfused FP64 operations in the reference's order.

namespace gb {
namespace {

constexpr int kScrThreads = kBopThreads;  // block_sum assumes kBopThreads
constexpr int kScrMaxBonds = 32;          // bonds per atom after screening

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
  ScrPair pr[6];
  double thr_s, thr_dot;  // ln 1e-6; 1e-10 as a default-real literal
};

inline ScrDev make_scr_dev(const double *r1, const double *r2, int npairs,
                           const gb_screening_params_t &s) {
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
    p.C_dr_cut = s.Cmax[q] > 2.0 ? s.Cmax[q] * s.Cmax[q] / (4 * (s.Cmax[q] - 1)) : 1.0;
  }
  d.thr_s = std::log(1e-6);
  d.thr_dot = (double)1e-10f;
  return d;
}

struct ScrBond {
  int jn, typ, need;
  double len, nm[3], fcar, dfcar, fcbo, dfcbo;
  double sij, fcin, fcar0, fcbo0;  // for the screening entries (need != 0)
};

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

// The screening loop of candidate bond (i, jn) (bop_kernel.f90:715-800).
// visit(kn, k, dS/dr_ik / r_ik^2, dS/dr_jk / r_jk^2, r_ik) for every
// partially screening neighbour before the loop stops.
template <class Visit>
__device__ __forceinline__ void scr_screen(const BopArgs &a, const ScrDev &sd, const ScrPair &P,
                                           const Pos4 &pi, int s, int e, int jn, int j,
                                           const double rij[3], double rlij, bool &screened,
                                           bool &need, double &sij, double &dsijdrij,
                                           Visit visit) {
  screened = false;
  need = false;
  sij = 0.0;
  dsijdrij = 0.0;
  const int shj = a.shift[jn];
  const double rlim = __dmul_rn(P.C_dr_cut, rlij);
  for (int kn = s; !(screened || sij < sd.thr_s) && kn < e; kn++) {
    double rik[3];
    const int k = scr_disp(a, pi, kn, rik);
    const double rlik = dot_rn(rik, rik);
    if (!(rlik < rlim)) continue;
    if (k == j && a.shift[kn] == shj) continue;
    const double dot_ij_ik = dot_rn(rij, rik);
    double rjk[3];
#pragma unroll
    for (int c = 0; c < 3; c++) rjk[c] = __dadd_rn(-rij[c], rik[c]);
    const double dot_ij_jk = dot_rn(rij, rjk);
    const double rljk = dot_rn(rjk, rjk);
    if (!(dot_ij_ik > sd.thr_dot && dot_ij_jk < -sd.thr_dot)) continue;
    const double xik = __ddiv_rn(rlik, rlij), xjk = __ddiv_rn(rljk, rlij);
    const double xm = __dsub_rn(xik, xjk), xp = __dadd_rn(xik, xjk);
    const double xm2 = __dmul_rn(xm, xm);
    const double fac = __ddiv_rn(1.0, __dsub_rn(1.0, xm2));
    const double C = __dmul_rn(__dsub_rn(__dsub_rn(__dmul_rn(2.0, xp), xm2), 1.0), fac);
    if (C <= P.Cmin) {
      screened = true;
    } else if (C < P.Cmax) {
      need = true;
      const double Cmax_C = __dsub_rn(P.Cmax, C), C_Cmin = __dsub_rn(C, P.Cmin);
      const double t = __ddiv_rn(Cmax_C, C_Cmin);
      sij = __dsub_rn(sij, __dmul_rn(t, t));
      const double dCdrik = 4 * xik * fac * (1 + (C - 1) * xm);
      const double dCdrjk = 4 * xjk * fac * (1 - (C - 1) * xm);
      const double dCdrij = -(dCdrik + dCdrjk);
      const double f2 = 2 * Cmax_C * P.dC / (C_Cmin * C_Cmin * C_Cmin);
      dsijdrij = dsijdrij + f2 * dCdrij;
      visit(kn, k, f2 * dCdrik / rlik, f2 * dCdrjk / rljk, rik);
    }
  }
}

__device__ __forceinline__ void outer_add(double w[9], const double x[3], const double y[3]) {
#pragma unroll
  for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
    for (int c2 = 0; c2 < 3; c2++) w[c1 + 3 * c2] += x[c1] * y[c2];
}

template <class Pot, bool kWat, bool kPB>
__global__ void __launch_bounds__(kScrThreads)
    bop_scr_atom(const BopArgs a, const Pot pot, const ScrDev sd, int *status) {
  __shared__ double red_scratch[(kScrThreads / 32) * 9];
  const int i = blockIdx.x * kScrThreads + threadIdx.x;
  double eacc[1] = {0.0};
  double wacc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  const int eli = i < a.nat ? a.el[i] : -1;
  if (i < a.nat) {
    const int s = a.seed[i], e = a.seed[i + 1];
    for (int b = s; b < e; b++) {  // this atom's entries start from zero
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
  if (eli >= 0) {
    const int s = a.seed[i], e = a.seed[i + 1];
    const Pos4 pi = a.pos[i];
    const int nel = pot.nel();
    ScrBond B[kScrMaxBonds];
    int nb = 0;
    bool overflow = false;
    // ---- Pass 1: bonds after screening. ----
    for (int jn = s; jn < e && !overflow; jn++) {
      const int j = a.nbr[jn];
      const int elj = a.el[j];
      if (elj < 0) continue;
      double rij[3];
      scr_disp(a, pi, jn, rij);
      const double rlij = dot_rn(rij, rij);
      const int t = pair_index(eli, elj, nel);
      const ScrPair &P = sd.pr[t];
      ScrBond bd;
      bd.jn = jn;
      bd.typ = t;
      bd.need = 0;
      bd.sij = bd.fcin = bd.fcar0 = bd.fcbo0 = 0.0;
      if (rlij < P.in_l2) {
        bd.fcar = bd.fcbo = 1.0;
        bd.dfcar = bd.dfcbo = 0.0;
      } else if (rlij < P.max_cut_sq && P.out_l < P.out_h) {
        bool screened, need;
        double sij, dsijdrij;
        scr_screen(a, sd, P, pi, s, e, jn, j, rij, rlij, screened, need, sij, dsijdrij,
                   [](int, int, double, double, const double *) {});
        if ((screened || sij < sd.thr_s) && rlij > P.in_h2) continue;  // fully screened
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
          bd.dfcar = (1.0 - fcin) * sij * (dfcar + fcar * dsijdrij / rl) - dfcin * sij * fcar + dfcin;
          bd.fcbo = (1.0 - fcin) * sij * fcbo + fcin;
          bd.dfcbo = (1.0 - fcin) * sij * (dfcbo + fcbo * dsijdrij / rl) - dfcin * sij * fcbo + dfcin;
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
      } else if (rlij < P.in_h2) {
        double fcin, dfcin;
        exp_cut(P.in, sqrt(rlij), fcin, dfcin);
        bd.fcar = bd.fcbo = fcin;
        bd.dfcar = bd.dfcbo = dfcin;
      } else {
        continue;
      }
      const double rl = sqrt(rlij);
      bd.len = rl;
#pragma unroll
      for (int c = 0; c < 3; c++) bd.nm[c] = rij[c] / rl;
      if (nb == kScrMaxBonds) {
        overflow = true;
        break;
      }
      B[nb++] = bd;
    }
    if (overflow) {
      atomicOr(status, 4);
    } else {
      // ---- Pass 2 (the force on i itself is minus the sum of its entries'
      // G by translation invariance; it is not accumulated here). ----
      double dbidk[kScrMaxBonds][3];
      double zfaci[kScrMaxBonds], sfacbo[kScrMaxBonds];
      for (int q = 0; q < nb; q++) sfacbo[q] = 0.0;
      for (int ij = 0; ij < nb; ij++) {
        const ScrBond &Bj = B[ij];
        const int j = a.nbr[Bj.jn];
        int maskfac = 2;
        if (a.mask) {
          const int mi = a.mask[i], mj = a.mask[j];
          if (mi == 0 && mj == 0)
            maskfac = 0;
          else if (mi == 0 || mj == 0)
            maskfac = 1;
        }
        const int t = Bj.typ;
        const double rlij = Bj.len;
        if (!(maskfac > 0 && rlij < sd.pr[t].out_h)) continue;
        double fj[3] = {0.0, 0.0, 0.0};
        const double rlijr = 1.0 / rlij;
        const double rnij[3] = {Bj.nm[0], Bj.nm[1], Bj.nm[2]};
        const double rij[3] = {rlij * rnij[0], rlij * rnij[1], rlij * rnij[2]};
        const double fcarij = Bj.fcar, dfcarijr = Bj.dfcar;
        double VA, dVA, VR, dVR;
        pot.VA(t, rlij, VA, dVA);
        pot.VR(t, rlij, VR, dVR);
        const double hm = 0.5 * maskfac;
        VA *= hm;
        dVA *= hm;
        VR *= hm;
        dVR *= hm;
        double wij[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, wijb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double zij = 0.0, dbidi[3] = {0.0, 0.0, 0.0}, dbidj[3] = {0.0, 0.0, 0.0};
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;
          const ScrBond &Bk = B[ik];
          const int ikpot = Bk.typ;
          const double rlik = Bk.len;
          if (!(rlik < sd.pr[ikpot].bo_h)) {
            zfaci[ik] = 0.0;
            dbidk[ik][0] = dbidk[ik][1] = dbidk[ik][2] = 0.0;
            continue;
          }
          const double *rnik = Bk.nm;
          const double rik[3] = {rlik * rnik[0], rlik * rnik[1], rlik * rnik[2]};
          const double fcik = Bk.fcbo, dfcikr = Bk.dfcbo;
          double h_Dr, dh_dDr;
          pot.template h<double>(ikpot, rlij - rlik, h_Dr, dh_dDr);
          const double costh = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
          double g_costh, dg_dcosth;
          pot.template g_hc<double>(eli, ikpot, pot.hpar(eli) - costh, g_costh, dg_dcosth);
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
          zfaci[ik] = g_costh * h_Dr;
          zij = zij + fcik * g_costh * h_Dr;
          const double dzdrij = g_costh * fcik * dh_dDr;
          const double dzdrik = g_costh * (dfcikr * h_Dr - fcik * dh_dDr);
          double df[3];
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const double dcsdi = -dcsdij * rnij[c] - dcsdik * rnik[c];
            const double dcsdj = dcsdij * rnij[c] - dcsdjk * dkc[c];
            const double dcsdk = dcsdik * rnik[c] + dcsdjk * dkc[c];
            dbidi[c] = dbidi[c] - dzdrij * rnij[c] - dzdrik * rnik[c] + dzfac * dcsdi;
            df[c] = dzdrij * rnij[c] + dzfac * dcsdj;
            dbidj[c] = dbidj[c] + df[c];
            dbidk[ik][c] = dzdrik * rnik[c] + dzfac * dcsdk;
          }
#pragma unroll
          for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
            for (int c2 = 0; c2 < 3; c2++)
              wijb[c1 + 3 * c2] -= rij[c1] * df[c2] + rik[c1] * dbidk[ik][c2];
        }
        double bij, dbdz;
        pot.template bo<double>(eli, t, zij, fcarij, VA, bij, dbdz);
        const double dffac = 0.5 * fcarij * (VR + bij * VA);
        eacc[0] += dffac;
        if (a.ebond) a.ebond[Bj.jn] = dffac;
        const double dffr =
            0.5 * (dVR * fcarij + bij * dVA * fcarij + VR * dfcarijr + bij * VA * dfcarijr);
        double df[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          df[c] = dffr * rnij[c];
          fj[c] -= df[c];
        }
        outer_add(wij, rij, df);
#pragma unroll
        for (int c = 0; c < 9; c++) wij[c] -= dbdz * wijb[c];
        if (kPB)
#pragma unroll
          for (int c = 0; c < 3; c++) a.frbond[3 * (size_t)Bj.jn + c] = df[c];
#pragma unroll
        for (int c = 0; c < 3; c++) fj[c] -= dbdz * dbidj[c];
        for (int ik = 0; ik < nb; ik++) {
          if (ik == ij) continue;
          double *Gk = a.G + 3 * (size_t)B[ik].jn;
#pragma unroll
          for (int c = 0; c < 3; c++) Gk[c] += -dbdz * dbidk[ik][c];
          if (B[ik].need) sfacbo[ik] = sfacbo[ik] + zfaci[ik] * dbdz;
        }
        if (Bj.need) {
          // forces on the screening neighbours from the pair term (:1531-1560):
          // the screening loop again on the bond's original vector
          const double dffac2 = 0.5 * (VR + bij * VA);
          const double om = 1.0 - Bj.fcin, sij = Bj.sij, fcar0 = Bj.fcar0;
          double r0[3];
          scr_disp(a, pi, Bj.jn, r0);
          bool sc, nd;
          double sj, dsj;
          scr_screen(a, sd, sd.pr[t], pi, s, e, Bj.jn, j, r0, dot_rn(r0, r0), sc, nd, sj, dsj,
                     [&](int kn, int, double rawik, double rawjk, const double *rik) {
                       const double arik = rawik * sij * fcar0 * om;
                       const double arjk = rawjk * sij * fcar0 * om;
                       double rjk[3], d1[3], d2[3];
                       double *Gk = a.G + 3 * (size_t)kn;
#pragma unroll
                       for (int c = 0; c < 3; c++) {
                         rjk[c] = -rij[c] + rik[c];
                         d1[c] = dffac2 * arik * rik[c];
                         d2[c] = dffac2 * arjk * rjk[c];
                         fj[c] += d2[c];
                         Gk[c] += -d1[c] - d2[c];
                       }
                       outer_add(wij, rik, d1);
                       outer_add(wij, rjk, d2);
                     });
        }
#pragma unroll
        for (int c = 0; c < 9; c++) wacc[c] += wij[c];
        if (kWat)
#pragma unroll
          for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)Bj.jn + c] += wij[c];
        double *Gj = a.G + 3 * (size_t)Bj.jn;
#pragma unroll
        for (int c = 0; c < 3; c++) Gj[c] += fj[c];
      }
      // ---- Screening forces through fc_bo (:1571-1611). ----
      for (int ij = 0; ij < nb; ij++) {
        const ScrBond &Bj = B[ij];
        if (!Bj.need || sfacbo[ij] == 0.0) continue;
        const int j = a.nbr[Bj.jn];
        const double sfac = sfacbo[ij], om = 1.0 - Bj.fcin, sij = Bj.sij, fcbo0 = Bj.fcbo0;
        const double rij[3] = {Bj.len * Bj.nm[0], Bj.len * Bj.nm[1], Bj.len * Bj.nm[2]};
        double fj[3] = {0.0, 0.0, 0.0};
        double wij[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        double r0[3];
        scr_disp(a, pi, Bj.jn, r0);
        bool sc, nd;
        double sj, dsj;
        scr_screen(a, sd, sd.pr[Bj.typ], pi, s, e, Bj.jn, j, r0, dot_rn(r0, r0), sc, nd, sj, dsj,
                   [&](int kn, int, double rawik, double rawjk, const double *rik) {
                     const double boik = sfac * (rawik * sij * fcbo0 * om);
                     const double bojk = sfac * (rawjk * sij * fcbo0 * om);
                     double rjk[3], d1[3], d2[3];
                     double *Gk = a.G + 3 * (size_t)kn;
#pragma unroll
                     for (int c = 0; c < 3; c++) {
                       rjk[c] = -rij[c] + rik[c];
                       d1[c] = boik * rik[c];
                       d2[c] = bojk * rjk[c];
                       fj[c] += d2[c];
                       Gk[c] += -d1[c] - d2[c];
                     }
                     outer_add(wij, rik, d1);
                     outer_add(wij, rjk, d2);
                   });
#pragma unroll
        for (int c = 0; c < 9; c++) wacc[c] += wij[c];
        if (kWat)
#pragma unroll
          for (int c = 0; c < 9; c++) a.wbond[9 * (size_t)Bj.jn + c] += wij[c];
        double *Gj = a.G + 3 * (size_t)Bj.jn;
#pragma unroll
        for (int c = 0; c < 3; c++) Gj[c] += fj[c];
      }
    }
  }
  double *part = a.tile_part + 10 * (size_t)blockIdx.x;
  block_sum<1>(eacc, part, red_scratch);
  block_sum<9>(wacc, part + 1, red_scratch);
}

}  // namespace
}  // namespace gb
