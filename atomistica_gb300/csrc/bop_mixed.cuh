// The mixed-precision bond-order tile kernel (included by bop.cu).
//
// Same decomposition as the FP64 tile kernel (phases 1-3, then a gather), but
// every quantity whose error is amplified into the forces is carried in
// float-float (ff.h) on the FP32 pipe instead of FP64:
//   phase 1  r_ij from ff positions, r and 1/r (ff sqrt), unit vectors and the
//            trig cutoff (ff sin/cos) in ff;
//   phase 2  the three-body k loop in FP32 with h - cos theta from an ff dot
//            product; VA, VR, the bond order b and P = dE/dzeta in ff (ff exp,
//            ln zeta by a Newton step); the energy, radial force and G partial
//            in ff.  A bond whose estimated FP32 error (from |P| sum_k
//            |dzeta/dr_k| and |dVA| d ln b/d ln zeta) exceeds kHotThreshold is
//            recomputed in FP64 (phase 2b);
//   phase 3  G_ik -= P_ij dzeta_ij/dr_k and the virial in ff.
// The only FP64 arithmetic left is the hot-bond recomputation, the conversion
// of per-bond energies and per-atom forces to FP64 and the tile reductions.
// Run-to-run results are bitwise reproducible (no atomics in any sum).

namespace gb {
namespace {

struct MxPair {
  ff cA, cR, Ac, Bc, xi, r1, fac;
};
struct MxElem {
  ff n, lbetan, e, h, eta, delta;
};
struct MxParams {
  int kind;  // 0 Tersoff, 1 Kumagai
  MxPair pr[6];
  MxElem el[3];
  ff A[3][3];
};

inline ff ffh(double d) { return ff_from_double(d); }

inline MxParams make_mx(const TersoffDev &d, const double A[3][3]) {
  MxParams m{};
  m.kind = 0;
  const int np = d.nel * (d.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    m.pr[q].cA = ffh(d.mu[q]);
    m.pr[q].cR = ffh(d.lambda[q]);
    m.pr[q].Ac = ffh(d.A[q]);
    m.pr[q].Bc = ffh(d.B[q]);
    m.pr[q].xi = ffh(d.xi[q]);
    m.pr[q].r1 = ffh(d.r1[q]);
    m.pr[q].fac = ffh(d.fac[q]);
  }
  for (int q = 0; q < d.nel; q++) {
    m.el[q].n = ffh(d.n[q]);
    m.el[q].lbetan = ffh(d.lbetan[q]);
    m.el[q].e = ffh(d.e[q]);
    m.el[q].h = ffh(d.h[q]);
  }
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) m.A[a][k] = ffh(A[a][k]);
  return m;
}

inline MxParams make_mx(const KumagaiDev &d, const double A[3][3]) {
  MxParams m{};
  m.kind = 1;
  m.pr[0].cA = ffh(d.lambda2[0]);
  m.pr[0].cR = ffh(d.lambda1[0]);
  m.pr[0].Ac = ffh(d.A[0]);
  m.pr[0].Bc = ffh(d.B[0]);
  m.pr[0].xi = ffh(1.0);
  m.pr[0].r1 = ffh(d.r1[0]);
  m.pr[0].fac = ffh(d.fac[0]);
  m.el[0].eta = ffh(d.eta[0]);
  m.el[0].delta = ffh(d.delta[0]);
  m.el[0].h = ffh(d.h[0]);
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) m.A[a][k] = ffh(A[a][k]);
  return m;
}

// Fast ff addition (no special care for catastrophic cancellation).
__device__ __forceinline__ ff ff_add_fast(ff a, ff b) {
  ff s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}

struct MxLayout {
  int *aseed, *toff, *el, *meta, *hot;
  ff *rn;  // 3 * nbt (component-major)
  ff *r, *rinv, *fc, *dfc, *P, *E;
  ff *G;  // 3 * nbt
  ff *t;  // 3 * ntrip
  int nbt, ntrip;
};

__host__ __device__ inline size_t bop_smem_bytes_mx(int nbt, int ntrip) {
  size_t o = align16(sizeof(int) * (3 * kMaxApt + 2 + 2 * (size_t)nbt));
  o += align16(sizeof(ff) * (size_t)nbt * 12);
  o += align16(sizeof(ff) * (size_t)ntrip * 3);
  return o + 64;
}

__device__ inline MxLayout carve_mx(unsigned char *sm, int nbt, int ntrip) {
  MxLayout L;
  L.nbt = nbt;
  L.ntrip = ntrip;
  int *ip = reinterpret_cast<int *>(sm);
  L.aseed = ip;
  L.toff = ip + kMaxApt + 1;
  L.el = ip + 2 * kMaxApt + 2;
  L.meta = ip + 3 * kMaxApt + 2;
  L.hot = L.meta + nbt;
  size_t o = align16(sizeof(int) * (3 * kMaxApt + 2 + 2 * (size_t)nbt));
  ff *fp = reinterpret_cast<ff *>(sm + o);
  L.rn = fp;
  L.r = fp + 3 * nbt;
  L.rinv = fp + 4 * nbt;
  L.fc = fp + 5 * nbt;
  L.dfc = fp + 6 * nbt;
  L.P = fp + 7 * nbt;
  L.E = fp + 8 * nbt;
  L.G = fp + 9 * nbt;
  o += align16(sizeof(ff) * (size_t)nbt * 12);
  L.t = reinterpret_cast<ff *>(sm + o);
  return L;
}

// Bond order in ff from an FP32 zeta (Tersoff: b = xi (1 + beta^n z^n)^e,
// P = -1/4 fc VA xi beta^n z^(n-1) (1+x)^(e-1); Kumagai: b = (1 + z^eta)^-delta,
// P = 1/2 fc VA eta z^(eta-1) (-delta) (1+x)^(-delta-1)).
__device__ __forceinline__ void bo_ff(const MxParams &mp, int eli, int t, float zeta, ff fc,
                                      ff VA, const ff *etab, ff &b, ff &P) {
  if (!(zeta > 0.0f)) {
    b = ff_make(1.0f, 0.0f);
    P = ff_make(0.0f, 0.0f);
    return;
  }
  const MxElem &E = mp.el[eli];
  const ff lnz = ff_log_f(zeta, etab);
  if (mp.kind == 0) {
    const ff tx = ff_add(ff_mul(E.n, lnz), E.lbetan);
    const ff x = ff_exp(tx, etab);
    const float L = log1pf(x.hi + x.lo);
    const float u = E.e.hi * L;
    b = ff_mul(mp.pr[t].xi, two_sum(1.0f, expm1f(u)));
    const ff arg = ff_addf(ff_sub(tx, lnz), (E.e.hi - 1.0f) * L);
    P = ff_mul(ff_mulf(ff_mul(ff_mul(fc, VA), mp.pr[t].xi), -0.25f), ff_exp(arg, etab));
  } else {
    const ff x = ff_exp(ff_mul(E.eta, lnz), etab);
    const float L = log1pf(x.hi + x.lo);
    b = two_sum(1.0f, expm1f(-E.delta.hi * L));
    const ff arg = ff_addf(ff_mul(ff_addf(E.eta, -1.0f), lnz), (-E.delta.hi - 1.0f) * L);
    P = ff_mul(ff_mul(ff_mul(ff_mul(fc, VA), E.eta), ff_neg(E.delta)),
               ff_mulf(ff_exp(arg, etab), 0.5f));
  }
}

// Three-body k loop in FP32 (h - cos theta from an ff dot product).
template <class Pot, bool kWat>
__device__ __forceinline__ void kloop_mx(const Pot &pot, const MxParams &mp, const MxLayout &L,
                                         int lb, int s, int z, int eli, ff *trow, float &zeta,
                                         float dbj[3], float wk[9], float &sumdk) {
  const int nbt = L.nbt, ntrip = L.ntrip;
  const ff rnij[3] = {L.rn[lb], L.rn[nbt + lb], L.rn[2 * nbt + lb]};
  const float rlij = L.r[lb].hi, rinvj = L.rinv[lb].hi;
  const ff h = mp.el[eli].h;
  for (int q = 0; q < z; q++) {
    const int lk = s + q;
    if (lk == lb) continue;
    const int mk = L.meta[lk];
    if (!(mk & kFlagK)) {
      trow[q] = ff_make(0.0f, 0.0f);
      trow[ntrip + q] = ff_make(0.0f, 0.0f);
      trow[2 * ntrip + q] = ff_make(0.0f, 0.0f);
      continue;
    }
    const int ikpot = (mk >> 8) & 0xf;
    const ff rnik[3] = {L.rn[lk], L.rn[nbt + lk], L.rn[2 * nbt + lk]};
    const float rlik = L.r[lk].hi, rinvk = L.rinv[lk].hi, fcik = L.fc[lk].hi,
                dfcik = L.dfc[lk].hi;
    // cos theta in ff
    ff csf = two_prod(rnik[0].hi, rnij[0].hi);
    csf = ff_add_fast(csf, two_prod(rnik[1].hi, rnij[1].hi));
    csf = ff_add_fast(csf, two_prod(rnik[2].hi, rnij[2].hi));
    csf.lo += rnik[0].hi * rnij[0].lo + rnik[0].lo * rnij[0].hi + rnik[1].hi * rnij[1].lo +
              rnik[1].lo * rnij[1].hi + rnik[2].hi * rnij[2].lo + rnik[2].lo * rnij[2].hi;
    const ff hc = ff_sub(h, csf);
    const float cs = csf.hi + csf.lo;
    float hv, dh;
    pot.template h<float>(ikpot, rlij - rlik, hv, dh);
    float gv, dg;
    pot.template g_hc<float>(eli, ikpot, hc.hi + hc.lo, gv, dg);
    const float dzfac = fcik * dg * hv;
    zeta += fcik * gv * hv;
    const float dzdrij = gv * fcik * dh;
    const float dzdrik = gv * (dfcik * hv - fcik * dh);
    const float rnjf[3] = {rnij[0].hi, rnij[1].hi, rnij[2].hi};
    const float rnkf[3] = {rnik[0].hi, rnik[1].hi, rnik[2].hi};
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float dcj = (rnkf[c] - cs * rnjf[c]) * rinvj;
      const float dck = (rnjf[c] - cs * rnkf[c]) * rinvk;
      dbj[c] += dzdrij * rnjf[c] + dzfac * dcj;
      const float dk = dzdrik * rnkf[c] + dzfac * dck;
      trow[c * ntrip + q] = ff_make(dk, 0.0f);
      sumdk += fabsf(dk);
      if (kWat)
#pragma unroll
        for (int c1 = 0; c1 < 3; c1++) wk[3 * c1 + c] += rnkf[c1] * rlik * dk;
    }
  }
}

// FP64 k loop for the hot bonds, from the ff geometry.
template <class Pot, bool kWat>
__device__ __forceinline__ void kloop_mx64(const Pot &pot, const MxLayout &L, int lb, int s, int z,
                                           int eli, ff *trow, double &zeta, double dbj[3],
                                           double wk[9]) {
  const int nbt = L.nbt, ntrip = L.ntrip;
  const double rnij[3] = {ff_to_double(L.rn[lb]), ff_to_double(L.rn[nbt + lb]),
                          ff_to_double(L.rn[2 * nbt + lb])};
  const double rlij = ff_to_double(L.r[lb]), rinvj = ff_to_double(L.rinv[lb]);
  for (int q = 0; q < z; q++) {
    const int lk = s + q;
    if (lk == lb) continue;
    const int mk = L.meta[lk];
    if (!(mk & kFlagK)) {
      trow[q] = ff_make(0.0f, 0.0f);
      trow[ntrip + q] = ff_make(0.0f, 0.0f);
      trow[2 * ntrip + q] = ff_make(0.0f, 0.0f);
      continue;
    }
    const int ikpot = (mk >> 8) & 0xf;
    const double rnik[3] = {ff_to_double(L.rn[lk]), ff_to_double(L.rn[nbt + lk]),
                            ff_to_double(L.rn[2 * nbt + lk])};
    const double rlik = ff_to_double(L.r[lk]), rinvk = ff_to_double(L.rinv[lk]);
    const double fcik = ff_to_double(L.fc[lk]), dfcik = ff_to_double(L.dfc[lk]);
    double hv, dh;
    pot.template h<double>(ikpot, rlij - rlik, hv, dh);
    const double cs = rnik[0] * rnij[0] + rnik[1] * rnij[1] + rnik[2] * rnij[2];
    double gv, dg;
    pot.template g<double>(eli, ikpot, cs, gv, dg);
    const double dzfac = fcik * dg * hv;
    zeta += fcik * gv * hv;
    const double dzdrij = gv * fcik * dh;
    const double dzdrik = gv * (dfcik * hv - fcik * dh);
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const double dcj = (rnik[c] - cs * rnij[c]) * rinvj;
      const double dck = (rnij[c] - cs * rnik[c]) * rinvk;
      dbj[c] += dzdrij * rnij[c] + dzfac * dcj;
      const double dk = dzdrik * rnik[c] + dzfac * dck;
      trow[c * ntrip + q] = ff_from_double(dk);
      if (kWat)
#pragma unroll
        for (int c1 = 0; c1 < 3; c1++) wk[3 * c1 + c] += rnik[c1] * rlik * dk;
    }
  }
}

// Energy, radial force and G partial in ff; FP64 per-bond outputs.
template <bool kWat, bool kPB>
__device__ __forceinline__ void finalize_mx(const BopArgs &a, const MxLayout &L, int lb, int b,
                                            ff bij, ff P, const ff dbj[3], const double wk[9],
                                            ff VA, ff dVA, ff VR, ff dVR) {
  const int nbt = L.nbt;
  const ff fc = L.fc[lb], dfc = L.dfc[lb];
  const ff v = ff_add(VR, ff_mul(bij, VA));    // VR + b VA
  const ff dv = ff_add(dVR, ff_mul(bij, dVA));  // dVR + b dVA
  const ff e_b = ff_mulf(ff_mul(fc, v), 0.5f);
  const ff dff = ff_mulf(ff_add(ff_mul(fc, dv), ff_mul(dfc, v)), 0.5f);
  ff dfr[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    dfr[c] = ff_mul(dff, L.rn[c * nbt + lb]);
    L.G[c * nbt + lb] = ff_neg(ff_add(dfr[c], ff_mul(P, dbj[c])));
  }
  L.P[lb] = P;
  L.E[lb] = e_b;
  a.ebond[b] = ff_to_double(e_b);
  if (kPB) {
    a.frbond[3 * (size_t)b] = ff_to_double(dfr[0]);
    a.frbond[3 * (size_t)b + 1] = ff_to_double(dfr[1]);
    a.frbond[3 * (size_t)b + 2] = ff_to_double(dfr[2]);
  }
  if (kWat) {
    const double r = ff_to_double(L.r[lb]);
    const double P64 = ff_to_double(P);
    double rij[3], dfr64[3], dbj64[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      rij[c] = r * ff_to_double(L.rn[c * nbt + lb]);
      dfr64[c] = ff_to_double(dfr[c]);
      dbj64[c] = ff_to_double(dbj[c]);
    }
#pragma unroll
    for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
      for (int c2 = 0; c2 < 3; c2++)
        a.wbond[9 * (size_t)b + c1 + 3 * c2] =
            rij[c1] * dfr64[c2] + P64 * (rij[c1] * dbj64[c2]) + P64 * wk[3 * c1 + c2];
  }
}

template <class Pot, bool kWat, bool kPB>
__global__ void __launch_bounds__(kBopThreads)
    bop_tile_mx(const BopArgs a, const Pot pot, const MxParams mp, const float4 *__restrict__ posff,
                int max_nbt, int max_ntrip, int *status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double red_scratch[(kBopThreads / 32) * 10];
  __shared__ ff s_exp[256], s_sin[257], s_cos[257];
  __shared__ int s_nhot;
  const int tid = threadIdx.x;
  for (int q = tid; q < 256; q += kBopThreads)
    s_exp[q] = ff_make(kFfExp2Tab[2 * q], kFfExp2Tab[2 * q + 1]);
  for (int q = tid; q < 257; q += kBopThreads) {
    s_sin[q] = ff_make(kFfSinTab[2 * q], kFfSinTab[2 * q + 1]);
    s_cos[q] = ff_make(kFfCosTab[2 * q], kFfCosTab[2 * q + 1]);
  }
  if (tid == 0) s_nhot = 0;
  const int a0 = blockIdx.x * a.apt;
  const int a1 = min(a0 + a.apt, a.nat);
  const int na = a1 - a0;
  const int b0 = a.seed[a0];
  const int nbt = a.seed[a1] - b0;
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
        s += z * z;
      }
      toff[na] = s;
    }
    __syncthreads();
    ntrip = toff[na];
  }
  if (nbt > max_nbt || ntrip > max_ntrip) {
    if (tid == 0) atomicOr(status, 2);
    return;
  }
  MxLayout L = carve_mx(sm, nbt, ntrip);
  for (int q = tid; q < na; q += kBopThreads)
    for (int lb = L.aseed[q]; lb < L.aseed[q + 1]; lb++) L.meta[lb] = q;
  __syncthreads();
  const int nel = pot.nel();

  // ---- Phase 1: bond geometry in ff. ----
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int ai = L.meta[lb];
    const int i = a0 + ai;
    const int b = b0 + lb;
    const int j = a.nbr[b];
    const int eli = L.el[ai];
    const int elj = a.el[j];
    int meta = ai;
    ff fc = ff_make(0.0f, 0.0f), dfc = ff_make(0.0f, 0.0f), r = ff_make(1.0f, 0.0f),
       rinv = ff_make(1.0f, 0.0f);
    ff rn[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
    if (eli >= 0 && elj >= 0) {
      const float4 pih = posff[2 * i], pil = posff[2 * i + 1];
      const float4 pjh = posff[2 * j], pjl = posff[2 * j + 1];
      ff rij[3] = {ff_sub(ff_make(pjh.x, pjl.x), ff_make(pih.x, pil.x)),
                   ff_sub(ff_make(pjh.y, pjl.y), ff_make(pih.y, pil.y)),
                   ff_sub(ff_make(pjh.z, pjl.z), ff_make(pih.z, pil.z))};
      int s0, s1, s2;
      unpack_shift(a.shift[b], s0, s1, s2);
      if (s0 | s1 | s2) {
        const float sx = (float)s0, sy = (float)s1, sz = (float)s2;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          ff as = ff_mulf(mp.A[c][0], sx);
          as = ff_add(as, ff_mulf(mp.A[c][1], sy));
          as = ff_add(as, ff_mulf(mp.A[c][2], sz));
          rij[c] = ff_sub(rij[c], as);
        }
      }
      ff r2 = ff_mul(rij[0], rij[0]);
      r2 = ff_add_fast(r2, ff_mul(rij[1], rij[1]));
      r2 = ff_add_fast(r2, ff_mul(rij[2], rij[2]));
      const int t = pair_index(eli, elj, nel);
      meta |= t << 8;
      const float r2f = r2.hi + r2.lo;
      if (r2f < (float)pot.r2sq(t)) {
        ff_sqrt_rsqrt(r2, r, rinv);
#pragma unroll
        for (int c = 0; c < 3; c++) rn[c] = ff_mul(rij[c], rinv);
        const float rf = r.hi + r.lo;
        if (r2f < (float)pot.r1sq(t) || rf <= (float)pot.r1(t)) {
          fc = ff_make(1.0f, 0.0f);
        } else if (rf < (float)pot.r2(t)) {
          const MxPair &pp = mp.pr[t];
          const ff x = ff_mul(pp.fac, ff_sub(r, pp.r1));
          ff sx, cx;
          ff_sincos(x, s_sin, s_cos, sx, cx);
          fc = ff_mulf(ff_addf(cx, 1.0f), 0.5f);
          dfc = ff_mulf(ff_mul(pp.fac, sx), -0.5f);
        }
        int mf = 2;
        if (a.mask) {
          const int mi = a.mask[i], mj = a.mask[j];
          if (mi == 0 && mj == 0)
            mf = 0;
          else if (mi == 0 || mj == 0)
            mf = 1;
        }
        meta |= kFlagShort | (mf << 16);
        if (rf < (float)pot.r2(t)) {
          meta |= kFlagK;
          if (mf > 0) meta |= kFlagIJ;
        }
      }
    }
    L.meta[lb] = meta;
#pragma unroll
    for (int c = 0; c < 3; c++) L.rn[c * nbt + lb] = rn[c];
    L.r[lb] = r;
    L.rinv[lb] = rinv;
    L.fc[lb] = fc;
    L.dfc[lb] = dfc;
  }
  __syncthreads();

  // ---- Phase 2: FP32 three-body terms, ff scalar chain. ----
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int b = b0 + lb;
    const int meta = L.meta[lb];
    if (!(meta & kFlagIJ)) {
      L.P[lb] = ff_make(0.0f, 0.0f);
      L.E[lb] = ff_make(0.0f, 0.0f);
      L.G[lb] = ff_make(0.0f, 0.0f);
      L.G[nbt + lb] = ff_make(0.0f, 0.0f);
      L.G[2 * nbt + lb] = ff_make(0.0f, 0.0f);
      a.ebond[b] = 0.0;
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
    ff *trow = L.t + L.toff[ai] + p * z;
    const int eli = L.el[ai];
    const MxPair &pp = mp.pr[t];
    const float hm = 0.5f * mf;
    const ff r = L.r[lb];
    const ff VA = ff_mulf(ff_mul(pp.Bc, ff_exp(ff_neg(ff_mul(pp.cA, r)), s_exp)), -hm);
    const ff dVA = ff_neg(ff_mul(pp.cA, VA));
    const ff VR = ff_mulf(ff_mul(pp.Ac, ff_exp(ff_neg(ff_mul(pp.cR, r)), s_exp)), hm);
    const ff dVR = ff_neg(ff_mul(pp.cR, VR));
    float zeta = 0.0f, dbj[3] = {0.0f, 0.0f, 0.0f}, wk[9], sumdk = 0.0f;
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) wk[c] = 0.0f;
    kloop_mx<Pot, kWat>(pot, mp, L, lb, s, z, eli, trow, zeta, dbj, wk, sumdk);
    // A zeta below 1e-30 would overflow the FP32 range inside ln/exp: such a
    // bond (and any non-finite estimate) takes the FP64 path.
    const bool tiny = zeta > 0.0f && zeta < 1.0e-30f;
    ff bij, P;
    bo_ff(mp, eli, t, tiny ? 1.0f : zeta, L.fc[lb], VA, s_exp, bij, P);
    const float est = 2.4e-7f * fabsf(dVA.hi) * L.fc[lb].hi * pot.bsens(eli, zeta) +
                      3.0e-7f * fabsf(P.hi) *
                          (sumdk + fabsf(dbj[0]) + fabsf(dbj[1]) + fabsf(dbj[2]));
    if (tiny || !(est <= kHotThreshold)) {
      L.hot[atomicAdd(&s_nhot, 1)] = lb;
    } else {
      const ff dbjf[3] = {ff_make(dbj[0], 0.0f), ff_make(dbj[1], 0.0f), ff_make(dbj[2], 0.0f)};
      double wkd[9];
      if (kWat)
#pragma unroll
        for (int c = 0; c < 9; c++) wkd[c] = wk[c];
      finalize_mx<kWat, kPB>(a, L, lb, b, bij, P, dbjf, wkd, VA, dVA, VR, dVR);
    }
  }
  __syncthreads();
  // ---- Phase 2b: FP64 recomputation of the hot bonds. ----
  {
    const int nhot = s_nhot;
    for (int hq = tid; hq < nhot; hq += kBopThreads) {
      const int lb = L.hot[hq];
      const int b = b0 + lb;
      const int meta = L.meta[lb];
      const int ai = meta & 0xff;
      const int t = (meta >> 8) & 0xf;
      const int mf = (meta >> 16) & 3;
      const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, p = lb - s;
      ff *trow = L.t + L.toff[ai] + p * z;
      const int eli = L.el[ai];
      const MxPair &pp = mp.pr[t];
      const float hm = 0.5f * mf;
      const ff r = L.r[lb];
      const ff VA = ff_mulf(ff_mul(pp.Bc, ff_exp(ff_neg(ff_mul(pp.cA, r)), s_exp)), -hm);
      const ff dVA = ff_neg(ff_mul(pp.cA, VA));
      const ff VR = ff_mulf(ff_mul(pp.Ac, ff_exp(ff_neg(ff_mul(pp.cR, r)), s_exp)), hm);
      const ff dVR = ff_neg(ff_mul(pp.cR, VR));
      double zeta = 0.0, dbj[3] = {0.0, 0.0, 0.0}, wk[9];
      if (kWat)
#pragma unroll
        for (int c = 0; c < 9; c++) wk[c] = 0.0;
      kloop_mx64<Pot, kWat>(pot, L, lb, s, z, eli, trow, zeta, dbj, wk);
      double b64, P64;
      pot.template bo<double>(eli, t, zeta, ff_to_double(L.fc[lb]), ff_to_double(VA), b64, P64);
      const ff dbjf[3] = {ff_from_double(dbj[0]), ff_from_double(dbj[1]), ff_from_double(dbj[2])};
      finalize_mx<kWat, kPB>(a, L, lb, b, ff_from_double(b64), ff_from_double(P64), dbjf, wk, VA,
                             dVA, VR, dVR);
    }
  }
  __syncthreads();

  // ---- Phase 3: k-role forces and the virial in ff. ----
  ff eacc = ff_make(0.0f, 0.0f);
  ff wacc[9];
#pragma unroll
  for (int c = 0; c < 9; c++) wacc[c] = ff_make(0.0f, 0.0f);
  for (int lb = tid; lb < nbt; lb += kBopThreads) {
    const int b = b0 + lb;
    const int meta = L.meta[lb];
    eacc = ff_add(eacc, L.E[lb]);
    ff G[3] = {L.G[lb], L.G[nbt + lb], L.G[2 * nbt + lb]};
    if (meta & kFlagK) {
      const int ai = meta & 0xff;
      const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, q = lb - s;
      const ff *tcol = L.t + L.toff[ai] + q;
      for (int pq = 0; pq < z; pq++) {
        const int lp = s + pq;
        if (lp == lb) continue;
        if (!(L.meta[lp] & kFlagIJ)) continue;
        const ff P = L.P[lp];
        const ff *tv = tcol + pq * z;
#pragma unroll
        for (int c = 0; c < 3; c++) G[c] = ff_sub(G[c], ff_mul(P, tv[c * ntrip]));
      }
      const ff r = L.r[lb];
      ff rb[3];
#pragma unroll
      for (int c = 0; c < 3; c++) rb[c] = ff_mul(r, L.rn[c * nbt + lb]);
#pragma unroll
      for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
        for (int c2 = 0; c2 < 3; c2++)
          wacc[c1 + 3 * c2] = ff_sub(wacc[c1 + 3 * c2], ff_mul(rb[c1], G[c2]));
    }
    float2 *Gout = reinterpret_cast<float2 *>(a.G) + 3 * (size_t)b;
    Gout[0] = make_float2(G[0].hi, G[0].lo);
    Gout[1] = make_float2(G[1].hi, G[1].lo);
    Gout[2] = make_float2(G[2].hi, G[2].lo);
  }
  double part_v[10];
  part_v[0] = ff_to_double(eacc);
#pragma unroll
  for (int c = 0; c < 9; c++) part_v[1 + c] = ff_to_double(wacc[c]);
  block_sum<10>(part_v, a.tile_part + 10 * (size_t)blockIdx.x, red_scratch);
}

// Gather of the ff bond forces: F_a = sum_b (G[rev b] - G[b]) in ff.
template <bool kEpa, bool kWat>
__global__ void bop_gather_mx(int nat, const int *__restrict__ seed, const int *__restrict__ rev,
                              const float2 *__restrict__ G, const double *__restrict__ ebond,
                              const double *__restrict__ wbond, double *__restrict__ f,
                              double *__restrict__ epa, double *__restrict__ wpa) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  ff F[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
  double E = 0.0;
  double W[9];
  if (kWat)
#pragma unroll
    for (int c = 0; c < 9; c++) W[c] = 0.0;
  const int s = seed[i], e = seed[i + 1];
  for (int b = s; b < e; b++) {
    const int rb = rev[b];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float2 gr = G[3 * (size_t)rb + c], gb = G[3 * (size_t)b + c];
      F[c] = ff_add(F[c], ff_sub(ff_make(gr.x, gr.y), ff_make(gb.x, gb.y)));
    }
    if (kEpa) E += ebond[b] + ebond[rb];
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) W[c] += wbond[9 * (size_t)b + c] + wbond[9 * (size_t)rb + c];
  }
#pragma unroll
  for (int c = 0; c < 3; c++) f[3 * (size_t)i + c] += ff_to_double(F[c]);
  if (kEpa) epa[i] += 0.5 * E;
  if (kWat)
#pragma unroll
    for (int c = 0; c < 9; c++) wpa[9 * (size_t)i + c] += 0.5 * W[c];
}

// ff positions (hi, lo) of every atom: 2 float4 per atom.
__global__ void bop_posff(int nat, const Pos4 *__restrict__ pos, float4 *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nat) return;
  const Pos4 p = pos[i];
  const ff x = ff_from_double(p.x), y = ff_from_double(p.y), z = ff_from_double(p.z);
  out[2 * i] = make_float4(x.hi, y.hi, z.hi, 0.0f);
  out[2 * i + 1] = make_float4(x.lo, y.lo, z.lo, 0.0f);
}

}  // namespace
}  // namespace gb
