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
//            |dzeta/dr_k| and |dVA| d ln b/d ln zeta) exceeds MxParams::hot is
//            recomputed in FP64 (phase 2b);
//   phase 3  G_ik -= P_ij dzeta_ij/dr_k and the virial in ff.
// The only FP64 arithmetic left is the hot-bond recomputation, the conversion
// of per-bond energies and per-atom forces to FP64 and the tile reductions.
// Run-to-run results are bitwise reproducible (no atomics in any sum).

#ifndef GB_MX_THREADS
#define GB_MX_THREADS 256
#endif
#ifndef GB_MX_MIN_BLOCKS
#define GB_MX_MIN_BLOCKS 3
#endif

namespace gb {
namespace {

constexpr int kMxThreads = GB_MX_THREADS;  // threads per tile (mixed form)
static_assert(kMaxApt <= 64, "the triplet-offset scan takes two atoms per lane");

struct MxPair {
  ff cA, cR, Ac, Bc, xi, r1, fac;
  float r1sq, r2sq, r2;  // cutoff tests in FP32
  // h(dr) = exp(hae (hs dr)^hm), dh/d dr = had hm hs (hs dr)^(hm-1) h;
  // hm = 0: h = 1.  Tersoff: hae = had = 1, hs = 2 mubo, hm = m; Kumagai:
  // hae = alpha (1 for beta = 3, kumagai_func.f90:211-213), had = alpha,
  // hs = 1, hm = beta.
  ff hae, had, hs;
  int hm;
  ff om;  // Tersoff omega of the (i,k) pair
};
struct MxElem {
  ff n, lbetan, e, h, eta, delta;
  ff c2, d2, c2d2;                 // Tersoff g
  ff c1, kc2, c3, c4, c5;          // Kumagai g
  float sens;                      // |d ln b / d ln x| prefactor (|e n|, |delta eta|)
};
// el[] holds the g and bond-order constants per centre element (Tersoff,
// Kumagai) or per element pair (Brenner: g of the (i,k) pair, b of the (i,j)
// pair; the kernels index it through el_g / el_b).
// Juslin's h(dr) = om e^{(hs dr)^hm} per element triplet (hm = 0: h = om).
struct MxTrip {
  ff hs, om;
  int hm;
};
struct MxParams {
  int kind;  // 0 Tersoff, Brenner and Juslin, 1 Kumagai
  int nel;
  float hot;  // estimated force error (eV/A) above which a bond is recomputed
  MxPair pr[9];
  MxElem el[9];
  MxTrip tr[27];  // Juslin only
  ff A[3][3];
};

// Index into MxParams::el of the g constants (centre element eli, pair ikpot)
// and of the bond-order constants (pair t); kPP: per-pair constants.
template <bool kPP>
__host__ __device__ __forceinline__ int el_g(int eli, int ikpot) {
  return kPP ? ikpot : eli;
}
template <bool kPP>
__host__ __device__ __forceinline__ int el_b(int eli, int t) {
  return kPP ? t : eli;
}

inline ff ffh(double d) { return ff_from_double(d); }

inline void mx_cutoffs(MxPair &q, double r1, double r2, double fac) {
  q.r1 = ffh(r1);
  q.fac = ffh(fac);
  q.r1sq = (float)(r1 * r1);
  q.r2sq = (float)(r2 * r2);
  q.r2 = (float)r2;
}

inline MxParams make_mx(const TersoffDev &d, const double A[3][3]) {
  MxParams m{};
  m.kind = 0;
  const int np = d.nel * (d.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    MxPair &pq = m.pr[q];
    pq.cA = ffh(d.mu[q]);
    pq.cR = ffh(d.lambda[q]);
    pq.Ac = ffh(d.A[q]);
    pq.Bc = ffh(d.B[q]);
    pq.xi = ffh(d.xi[q]);
    mx_cutoffs(pq, d.r1[q], d.r2[q], d.fac[q]);
    pq.hae = ffh(1.0);
    pq.had = ffh(1.0);
    pq.hs = ffh(2.0 * d.mubo[q]);
    pq.hm = d.mubo[q] == 0.0 ? 0 : d.m[q];
    pq.om = ffh(d.omega[q]);
  }
  for (int q = 0; q < d.nel; q++) {
    MxElem &e = m.el[q];
    e.n = ffh(d.n[q]);
    e.lbetan = ffh(d.lbetan[q]);
    e.e = ffh(d.e[q]);
    e.h = ffh(d.h[q]);
    e.c2 = ffh(d.c2[q]);
    e.d2 = ffh(d.d2[q]);
    e.c2d2 = ffh(d.c2d2inv[q]);
    e.sens = (float)std::fabs(d.e[q] * d.n[q]);
  }
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) m.A[a][k] = ffh(A[a][k]);
  return m;
}

// Brenner: VA = -Bc e^{-cA r} with Bc = VA_f e^{expA r0} (and VR alike), the
// Tersoff g with gamma for omega and -h for h, the Tersoff b with beta = xi = 1
// and the pair's n; all constants per pair.
inline MxParams make_mx(const BrennerDev &d, const double A[3][3], int np = -1) {
  MxParams m{};
  m.kind = 0;
  m.nel = d.nel;
  if (np < 0) np = d.nel * (d.nel + 1) / 2;
  for (int q = 0; q < np; q++) {
    MxPair &pq = m.pr[q];
    pq.cA = ffh(d.expA[q]);
    pq.cR = ffh(d.expR[q]);
    pq.Ac = ffh(d.VR_f[q] * std::exp(d.expR[q] * d.r0[q]));
    pq.Bc = ffh(d.VA_f[q] * std::exp(d.expA[q] * d.r0[q]));
    pq.xi = ffh(1.0);
    mx_cutoffs(pq, d.r1[q], d.r2[q], d.fac[q]);
    pq.hae = ffh(1.0);
    pq.had = ffh(1.0);
    pq.hs = ffh(2.0 * d.mu[q]);
    pq.hm = d.mu[q] == 0.0 ? 0 : d.m[q];
    pq.om = ffh(d.gamma[q]);
    MxElem &e = m.el[q];
    e.n = ffh(d.n[q]);
    e.lbetan = ffh(0.0);
    e.e = ffh(d.bo_exp[q]);
    e.h = ffh(d.hneg[q]);
    e.c2 = ffh(d.c2[q]);
    e.d2 = ffh(d.d2[q]);
    e.c2d2 = ffh(d.c2d2inv[q]);
    e.sens = (float)std::fabs(d.bo_exp[q] * d.n[q]);
  }
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) m.A[a][k] = ffh(A[a][k]);
  return m;
}

inline MxParams make_mx(const KumagaiDev &d, const double A[3][3]) {
  MxParams m{};
  m.kind = 1;
  MxPair &p0 = m.pr[0];
  p0.cA = ffh(d.lambda2[0]);
  p0.cR = ffh(d.lambda1[0]);
  p0.Ac = ffh(d.A[0]);
  p0.Bc = ffh(d.B[0]);
  p0.xi = ffh(1.0);
  mx_cutoffs(p0, d.r1[0], d.r2[0], d.fac[0]);
  p0.hae = ffh(d.beta[0] == 3 ? 1.0 : d.alpha[0]);
  p0.had = ffh(d.alpha[0]);
  p0.hs = ffh(1.0);
  p0.hm = d.alpha[0] == 0.0 ? 0 : d.beta[0];
  p0.om = ffh(1.0);
  MxElem &e = m.el[0];
  e.n = ffh(d.eta[0]);
  e.lbetan = ffh(0.0);
  e.eta = ffh(d.eta[0]);
  e.delta = ffh(d.delta[0]);
  e.h = ffh(d.h[0]);
  e.c1 = ffh(d.c1[0]);
  e.kc2 = ffh(d.c2[0]);
  e.c3 = ffh(d.c3[0]);
  e.c4 = ffh(d.c4[0]);
  e.c5 = ffh(d.c5[0]);
  e.sens = (float)std::fabs(d.delta[0] * d.eta[0]);
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) m.A[a][k] = ffh(A[a][k]);
  return m;
}

// Juslin: Brenner's constants on the nel^2 ordered pairs and h per triplet.
inline MxParams make_mx(const JuslinPot &P, const double A[3][3]) {
  MxParams m = make_mx(P.p, A, P.p.nel * P.p.nel);
  for (int q = 0; q < P.p.nel * P.p.nel * P.p.nel; q++) {
    m.tr[q].hs = ffh(P.alpha[q]);
    m.tr[q].om = ffh(P.omega[q]);
    m.tr[q].hm = P.alpha[q] == 0.0 ? 0 : P.m3[q];
  }
  return m;
}
template <class Pot>
inline MxParams make_mx(const Pot &P, const double A[3][3]) {
  return make_mx(P.p, A);
}


// acc += a b with an unnormalised accumulator (hi: running FP32 sum, lo:
// its rounding errors and the low parts); ff_norm before use.
__device__ __forceinline__ void ff_acc_mul(ff &acc, ff a, ff b) {
  ff p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  const ff s = two_sum(acc.hi, p.hi);
  acc.hi = s.hi;
  acc.lo += s.lo + p.lo;
}
__device__ __forceinline__ void ff_acc(ff &acc, ff a) {
  const ff s = two_sum(acc.hi, a.hi);
  acc.hi = s.hi;
  acc.lo += s.lo + a.lo;
}
__device__ __forceinline__ ff ff_norm(ff a) { return two_sum(a.hi, a.lo); }

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

// ---- Three-body functions on the MxParams copies of the parameters. ----
// Their element argument is the index into MxParams::el (el_g / el_b).
// g as a function of hc = h - cos theta, and d g / d cos theta
// (tersoff_func.f90:86-114 in the stable form g = omega (1 + c^2 hc^2 /
// (d^2 (d^2 + hc^2))); kumagai_func.f90:86-131).
__device__ __forceinline__ void g_f(const MxParams &mp, int eli, int ikpot, float hc, float &val,
                                    float &dval) {
  const MxElem &E = mp.el[eli];
  const float hc2 = hc * hc;
  if (mp.kind == 0) {
    const float om = mp.pr[ikpot].om.hi;
    const float inv = 1.0f / (E.d2.hi + hc2);
    val = om * (1.0f + E.c2d2.hi * hc2 * inv);
    dval = -2.0f * om * E.c2.hi * hc * inv * inv;
  } else {
    const float tmp = hc / (E.c3.hi + hc2);
    const float go = E.kc2.hi * tmp;
    const float ga1 = E.c4.hi * expf(-E.c5.hi * hc2);
    const float v = go * (1.0f + ga1);
    dval = -2.0f * (1.0f - hc * tmp) * v + 2.0f * E.c5.hi * hc2 * go * ga1;
    val = E.c1.hi + hc * v;
  }
}

__device__ __forceinline__ void g_ff(const MxParams &mp, int eli, int ikpot, ff hc,
                                     const ff *etab, ff &val, ff &dval) {
  const MxElem &E = mp.el[eli];
  const ff hc2 = ff_mul(hc, hc);
  if (mp.kind == 0) {
    const ff om = mp.pr[ikpot].om;
    const ff inv = ff_rcp(ff_add(E.d2, hc2));
    val = ff_mul(om, ff_addf(ff_mul(ff_mul(E.c2d2, hc2), inv), 1.0f));
    dval = ff_mulf(ff_mul(ff_mul(ff_mul(om, E.c2), hc), ff_mul(inv, inv)), -2.0f);
  } else {
    const ff tmp = ff_div(hc, ff_add(E.c3, hc2));
    const ff go = ff_mul(E.kc2, tmp);
    const ff ga1 = ff_mul(E.c4, ff_exp(ff_neg(ff_mul(E.c5, hc2)), etab));
    const ff v = ff_mul(go, ff_addf(ga1, 1.0f));
    const ff t1 = ff_mulf(ff_mul(ff_addf(ff_neg(ff_mul(hc, tmp)), 1.0f), v), -2.0f);
    const ff t2 = ff_mulf(ff_mul(ff_mul(E.c5, hc2), ff_mul(go, ga1)), 2.0f);
    dval = ff_add(t1, t2);
    val = ff_add(E.c1, ff_mul(hc, v));
  }
}

// Juslin's h (juslin_func.f90:257-294) of triplet q.
__device__ __forceinline__ void h3_f(const MxTrip &q, float dr, float &val, float &dval) {
  if (q.hm == 0) {
    val = q.om.hi;
    dval = 0.0f;
    return;
  }
  const float x = q.hs.hi * dr;
  float pw = 1.0f;
  for (int k = 1; k < q.hm; k++) pw *= x;
  val = q.om.hi * expf(pw * x);
  dval = (float)q.hm * q.hs.hi * pw * val;
}

__device__ __forceinline__ void h3_ff(const MxTrip &q, ff dr, const ff *etab, ff &val,
                                      ff &dval) {
  if (q.hm == 0) {
    val = q.om;
    dval = ff_make(0.0f, 0.0f);
    return;
  }
  const ff x = ff_mul(q.hs, dr);
  ff pw = ff_make(1.0f, 0.0f);
  for (int k = 1; k < q.hm; k++) pw = ff_mul(pw, x);
  val = ff_mul(q.om, ff_exp(ff_mul(pw, x), etab));
  dval = ff_mul(ff_mulf(q.hs, (float)q.hm), ff_mul(pw, val));
}

// h(dr), dr = r_ij - r_ik (tersoff_func.f90:168-211, kumagai_func.f90:179-221).
__device__ __forceinline__ void h_f(const MxPair &q, float dr, float &val, float &dval) {
  if (q.hm == 0) {
    val = 1.0f;
    dval = 0.0f;
    return;
  }
  const float x = q.hs.hi * dr;
  float pw = 1.0f;
  for (int k = 1; k < q.hm; k++) pw *= x;
  val = expf(q.hae.hi * pw * x);
  dval = q.had.hi * (float)q.hm * q.hs.hi * pw * val;
}

__device__ __forceinline__ void h_ff(const MxPair &q, ff dr, const ff *etab, ff &val, ff &dval) {
  if (q.hm == 0) {
    val = ff_make(1.0f, 0.0f);
    dval = ff_make(0.0f, 0.0f);
    return;
  }
  const ff x = ff_mul(q.hs, dr);
  ff pw = ff_make(1.0f, 0.0f);
  for (int k = 1; k < q.hm; k++) pw = ff_mul(pw, x);
  val = ff_exp(ff_mul(q.hae, ff_mul(pw, x)), etab);
  dval = ff_mul(ff_mulf(ff_mul(q.had, q.hs), (float)q.hm), ff_mul(pw, val));
}

// |d ln b / d ln zeta| = sens x / (1 + x), x = beta^n zeta^n (Kumagai: zeta^eta).
__device__ __forceinline__ float bsens_f(const MxParams &mp, int eli, float zeta) {
  if (!(zeta > 0.0f)) return 0.0f;
  const MxElem &E = mp.el[eli];
  const float x = __expf(E.n.hi * __logf(zeta) + E.lbetan.hi);
  return E.sens * x / (1.0f + x);
}

// Bond order of a bond on the FP32 path, from its FP32 zeta (tersoff_func.f90
// :122-160, kumagai_func.f90:139-171): ln zeta, x = beta^n zeta^n and the
// exponent of P in ff, so that b and P carry only the error of zeta (the
// error estimate's first term); log1p(x) and expm1 in FP32, where their
// error is of the order of zeta's.
__device__ __forceinline__ void bo_f(const MxParams &mp, int eli, int t, float zeta, ff fc, ff VA,
                                     const ff *etab, ff &b, ff &P, ff &x, float &L) {
  x = ff_make(0.0f, 0.0f);
  L = 0.0f;
  if (!(zeta > 0.0f)) {
    b = ff_make(1.0f, 0.0f);
    P = ff_make(0.0f, 0.0f);
    return;
  }
  const MxElem &E = mp.el[eli];
  const ff lnz = ff_log_f(zeta, etab);
  if (mp.kind == 0) {
    const ff tx = ff_add(ff_mul(E.n, lnz), E.lbetan);  // ln x
    x = ff_exp(tx, etab);
    L = log1pf(x.hi + x.lo);
    b = ff_mul(mp.pr[t].xi, two_sum(1.0f, expm1f(E.e.hi * L)));
    const ff arg = ff_addf(ff_sub(tx, lnz), (E.e.hi - 1.0f) * L);
    P = ff_mul(ff_mulf(ff_mul(ff_mul(fc, VA), mp.pr[t].xi), -0.25f), ff_exp(arg, etab));
  } else {
    x = ff_exp(ff_mul(E.eta, lnz), etab);
    L = log1pf(x.hi + x.lo);
    b = two_sum(1.0f, expm1f(-E.delta.hi * L));
    const ff arg = ff_addf(ff_mul(ff_addf(E.eta, -1.0f), lnz), (-E.delta.hi - 1.0f) * L);
    P = ff_mul(ff_mul(ff_mul(ff_mul(fc, VA), E.eta), ff_neg(E.delta)),
               ff_mulf(ff_exp(arg, etab), 0.5f));
  }
}

// b and P of a hot bond at zeta0 + dz, from the FP32 pass's x0 = x(zeta0),
// L0 = log1p(x0) (FP32) and P0 (exact for zeta0 and L0): x to first order in
// dz / zeta0 (~1e-7), then L = ln(1 + x) and b in ff, and
// P = P0 (1 + (n - 1) dz / zeta0 + (e - 1) (L - L0)) (Kumagai: n -> eta,
// e -> -delta); the neglected terms are ~1e-14 relative.
__device__ __forceinline__ void bo_hot(const MxParams &mp, int eli, int t, ff P0, ff x0,
                                       float zeta0, float L0, float dz, const ff *etab, ff &b,
                                       ff &P) {
  const MxElem &E = mp.el[eli];
  const float dzr = dz / zeta0;
  const float n = E.n.hi;  // x ~ zeta^n (Kumagai: n = eta)
  const ff x = ff_add(x0, ff_mulf(x0, n * dzr));
  const ff L = ff_log(ff_addf(x, 1.0f), etab);
  const float dL = (L.hi - L0) + L.lo;
  if (mp.kind == 0) {
    b = ff_mul(mp.pr[t].xi, ff_exp(ff_mul(E.e, L), etab));
    P = ff_add(P0, ff_mulf(P0, (n - 1.0f) * dzr + (E.e.hi - 1.0f) * dL));
  } else {
    b = ff_exp(ff_mul(ff_neg(E.delta), L), etab);
    P = ff_add(P0, ff_mulf(P0, (n - 1.0f) * dzr + (-E.delta.hi - 1.0f) * dL));
  }
}

// Three-body k loop of bond lb in FP32 (h - cos theta from an ff dot
// product, bop_kernel.f90:1171-1343).  Also returns sum_k |d zeta/d r_k| for
// the error estimate.
template <bool kWat, bool kPP, bool kTri>
__device__ __forceinline__ void kloop_mx(const MxParams &mp, const MxLayout &L, int lb, int s,
                                         int z, int eli, ff *trow, float &zeta, float dbj[3],
                                         float wk[9], float &sumdk) {
  const int nbt = L.nbt, ntrip = L.ntrip;
  // kTri: triplet (i, j, k) = ikpot + nel (ijpot - eli) of the ordered pairs
  const int tri0 = kTri ? mp.nel * (((L.meta[lb] >> 8) & 0xf) - eli) : 0;
  const ff rnij[3] = {L.rn[lb], L.rn[nbt + lb], L.rn[2 * nbt + lb]};
  const float rlij = L.r[lb].hi, rinvj = L.rinv[lb].hi;
  const ff h0 = mp.el[eli].h;
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
    // cos theta = s2.hi + clo and h - cos theta, both to ~1e-14 absolute
    const ff p0 = two_prod(rnik[0].hi, rnij[0].hi), p1 = two_prod(rnik[1].hi, rnij[1].hi),
             p2 = two_prod(rnik[2].hi, rnij[2].hi);
    const ff s1 = two_sum(p0.hi, p1.hi);
    const ff s2 = two_sum(s1.hi, p2.hi);
    float clo = ((s1.lo + s2.lo) + (p0.lo + p1.lo + p2.lo));
    clo = fmaf(rnik[0].hi, rnij[0].lo, clo);
    clo = fmaf(rnik[0].lo, rnij[0].hi, clo);
    clo = fmaf(rnik[1].hi, rnij[1].lo, clo);
    clo = fmaf(rnik[1].lo, rnij[1].hi, clo);
    clo = fmaf(rnik[2].hi, rnij[2].lo, clo);
    clo = fmaf(rnik[2].lo, rnij[2].hi, clo);
    const float cs = s2.hi + clo;
    const ff h = kPP ? mp.el[ikpot].h : h0;
    const ff dh0 = two_sum(h.hi, -s2.hi);
    const float hcf = dh0.hi + ((dh0.lo + h.lo) - clo);
    float hv, dh;
    if (kTri)
      h3_f(mp.tr[tri0 + ikpot], rlij - rlik, hv, dh);
    else
      h_f(mp.pr[ikpot], rlij - rlik, hv, dh);
    float gv, dg;
    g_f(mp, el_g<kPP>(eli, ikpot), ikpot, hcf, gv, dg);
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

// The same k loop in ff arithmetic for the hot bonds, over the slots
// q = q0, q0 + dq, ... of bond lb's row (the partial sums of zeta, d zeta /
// d r_j and the virial term are added up across the lanes afterwards).
template <bool kWat, bool kPP, bool kTri>
__device__ __forceinline__ void kloop_ff(const MxParams &mp, const MxLayout &L, int lb, int s,
                                         int z, int eli, ff *trow, const ff *etab, int q0,
                                         int dq, ff &zeta, ff dbj[3], ff wk[9]) {
  const int nbt = L.nbt, ntrip = L.ntrip;
  const int tri0 = kTri ? mp.nel * (((L.meta[lb] >> 8) & 0xf) - eli) : 0;
  const ff rnij[3] = {L.rn[lb], L.rn[nbt + lb], L.rn[2 * nbt + lb]};
  const ff rlij = L.r[lb], rinvj = L.rinv[lb];
  const ff h0 = mp.el[eli].h;
  for (int q = q0; q < z; q += dq) {
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
    const ff rlik = L.r[lk], rinvk = L.rinv[lk], fcik = L.fc[lk], dfcik = L.dfc[lk];
    ff hv, dh;
    if (kTri)
      h3_ff(mp.tr[tri0 + ikpot], ff_sub(rlij, rlik), etab, hv, dh);
    else
      h_ff(mp.pr[ikpot], ff_sub(rlij, rlik), etab, hv, dh);
    ff cs = ff_mul(rnik[0], rnij[0]);
    cs = ff_add(cs, ff_mul(rnik[1], rnij[1]));
    cs = ff_add(cs, ff_mul(rnik[2], rnij[2]));
    ff gv, dg;
    g_ff(mp, el_g<kPP>(eli, ikpot), ikpot, ff_sub(kPP ? mp.el[ikpot].h : h0, cs), etab, gv,
         dg);
    const ff fh = ff_mul(fcik, hv);
    const ff dzfac = ff_mul(fh, dg);
    zeta = ff_add(zeta, ff_mul(fh, gv));
    const ff dzdrij = ff_mul(ff_mul(gv, fcik), dh);
    const ff dzdrik = ff_mul(gv, ff_sub(ff_mul(dfcik, hv), ff_mul(fcik, dh)));
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const ff dcj = ff_mul(ff_sub(rnik[c], ff_mul(cs, rnij[c])), rinvj);
      const ff dck = ff_mul(ff_sub(rnij[c], ff_mul(cs, rnik[c])), rinvk);
      dbj[c] = ff_add(dbj[c], ff_add(ff_mul(dzdrij, rnij[c]), ff_mul(dzfac, dcj)));
      const ff dk = ff_add(ff_mul(dzdrik, rnik[c]), ff_mul(dzfac, dck));
      trow[c * ntrip + q] = dk;
      if (kWat)
#pragma unroll
        for (int c1 = 0; c1 < 3; c1++)
          wk[3 * c1 + c] = ff_add(wk[3 * c1 + c], ff_mul(ff_mul(rnik[c1], rlik), dk));
    }
  }
}

__device__ __forceinline__ ff ff_shfl_xor(ff v, int o) {
  ff r;
  r.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
  r.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
  return r;
}

// Energy, radial force and G partial in ff; FP64 per-bond outputs.
template <bool kWat, bool kPB>
__device__ __forceinline__ void finalize_mx(const BopArgs &a, const MxLayout &L, int lb, int b,
                                            ff bij, ff P, const ff dbj[3], const ff wk[9],
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
  if (a.ebond) a.ebond[b] = (double)e_b.hi + (double)e_b.lo;
  if (kPB) {
    a.frbond[3 * (size_t)b] = ff_to_double(dfr[0]);
    a.frbond[3 * (size_t)b + 1] = ff_to_double(dfr[1]);
    a.frbond[3 * (size_t)b + 2] = ff_to_double(dfr[2]);
  }
  if (kWat) {
    // w_ij = r_ij (x) df + P (r_ij (x) dbj + sum_k r_ik (x) dk) (bop_kernel.f90:1404)
    const ff r = L.r[lb];
    ff rij[3];
#pragma unroll
    for (int c = 0; c < 3; c++) rij[c] = ff_mul(r, L.rn[c * nbt + lb]);
#pragma unroll
    for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
      for (int c2 = 0; c2 < 3; c2++) {
        const ff w = ff_add(ff_mul(rij[c1], dfr[c2]),
                                 ff_mul(P, ff_add(ff_mul(rij[c1], dbj[c2]), wk[3 * c1 + c2])));
        a.wbond[9 * (size_t)b + c1 + 3 * c2] = ff_to_double(w);
      }
  }
}

// Deterministic tile sums: the energy in ff (warp xor tree), the nine virial
// components in FP32 (a warp reduce-scatter butterfly: lanes l, l ^ m swap
// half of their components for m = 16, 8, 4, 2, then m = 1, leaving
// component c = 8 b4 + 4 b3 + 2 b2 + b1 (b_k: bit k of the lane) in lanes 2c,
// 2c + 1), then the warps in order; written as FP64 (out[0] energy, out[1..9]
// the virial).  The FP32 virial is accurate to ~1e-7 of sum |r (x) G|.
__device__ inline void block_sum_tile(ff e, const float (&w)[9], double *out, ff *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int nw = kMxThreads / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e = ff_add(e, ff_shfl_xor(e, o));
  float x[16];
#pragma unroll
  for (int c = 0; c < 16; c++) x[c] = c < 9 ? w[c] : 0.0f;
#pragma unroll
  for (int lev = 0; lev < 4; lev++) {
    const int m = 16 >> lev, H = 8 >> lev;
    const bool up = (lane & m) != 0;
#pragma unroll
    for (int q = 0; q < H; q++) {
      const float send = up ? x[q] : x[q + H];
      const float keep = up ? x[q + H] : x[q];
      x[q] = keep + __shfl_xor_sync(0xffffffffu, send, m);
    }
  }
  const float r = x[0] + __shfl_xor_sync(0xffffffffu, x[0], 1);
  const int c = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 +
                ((lane >> 1) & 1);
  if ((lane & 1) == 0 && c < 9) scratch[wid * 10 + 1 + c] = ff_make(r, 0.0f);
  if (lane == 0) scratch[wid * 10] = e;
  __syncthreads();
  if (threadIdx.x < 10) {
    double sum = 0.0;
    for (int q = 0; q < nw; q++) sum += ff_to_double(scratch[q * 10 + threadIdx.x]);
    out[threadIdx.x] = sum;
  }
}

// The tile index that thread 0 took from the queue at the start of the
// current tile (the barrier orders its write before every thread's read).
__device__ __forceinline__ int next_queued_tile(const int &s_next) {
  __syncthreads();
  return s_next;
}

template <class Pot, bool kWat, bool kPB>
__global__ void __launch_bounds__(kMxThreads, GB_MX_MIN_BLOCKS)
    bop_tile_mx(const BopArgs a, const Pot pot, const MxParams mp, const float4 *__restrict__ posff,
                int max_nbt, int max_ntrip, int *status) {
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ ff red_scratch[(kMxThreads / 32) * 10];
  __shared__ ff s_exp[256], s_sin[257], s_cos[257];
  __shared__ int s_nhot, s_next;
  __shared__ ff sAf[9];
  const int tid = threadIdx.x;
  for (int q = tid; q < 256; q += kMxThreads)
    s_exp[q] = ff_make(kFfExp2Tab[2 * q], kFfExp2Tab[2 * q + 1]);
  for (int q = tid; q < 257; q += kMxThreads) {
    s_sin[q] = ff_make(kFfSinTab[2 * q], kFfSinTab[2 * q + 1]);
    s_cos[q] = ff_make(kFfCosTab[2 * q], kFfCosTab[2 * q + 1]);
  }
  // Persistent CTAs.  A single structure: tiles blockIdx.x, blockIdx.x +
  // gridDim.x, ... (a static schedule, so the per-CTA energy and virial sums
  // are reproducible).  A batch (one partial row per tile): the next tile
  // from the counter a.tile_queue, taken at the start of the current one.
  ff eacc = ff_make(0.0f, 0.0f);
  float wacc[9];
#pragma unroll
  for (int c = 0; c < 9; c++) wacc[c] = 0.0f;
  const int ntiles = a.tile_atom0 ? a.ntiles : (a.nat + a.apt - 1) / a.apt;
  int *const queue = a.tile_atom0 ? a.tile_queue : nullptr;
  if (queue) {
    if (tid == 0) s_next = atomicAdd(queue, 1);
    __syncthreads();
  }
  for (int tile = queue ? s_next : blockIdx.x; tile < ntiles;
       tile = queue ? next_queued_tile(s_next) : tile + gridDim.x) {
    __syncthreads();  // the previous tile is done with shared memory (and s_next)
    if (tid == 0) {
      s_nhot = 0;
      if (queue) s_next = atomicAdd(queue, 1);
    }
    if (tid < 9) {  // this tile's cell
      const float2 v = a.Acells_ff ? a.Acells_ff[9 * a.tile_struct[tile] + tid]
                                   : make_float2(mp.A[tid / 3][tid % 3].hi,
                                                 mp.A[tid / 3][tid % 3].lo);
      sAf[tid] = ff_make(v.x, v.y);
    }
    int a0, a1;
    tile_range(a, tile, a0, a1);
    const int na = a1 - a0;
    const int b0 = a.seed[a0];
    const int nbt = a.seed[a1] - b0;
    int ntrip = 0;
    {
      int *aseed = reinterpret_cast<int *>(sm);
      int *toff = aseed + kMaxApt + 1;
      int *el = aseed + 2 * kMaxApt + 2;
      for (int q = tid; q <= na; q += kMxThreads) aseed[q] = a.seed[a0 + q] - b0;
      for (int q = tid; q < na; q += kMxThreads) el[q] = a.el[a0 + q];
      __syncthreads();
      if (tid < 32) {
        // triplet-slot offsets: exclusive scan of trip_slots(z) over the tile's atoms
        // (na <= 64: two atoms per lane)
        const int q0 = 2 * tid, q1 = 2 * tid + 1;
        const int z0 = q0 < na ? aseed[q0 + 1] - aseed[q0] : 0;
        const int z1 = q1 < na ? aseed[q1 + 1] - aseed[q1] : 0;
        const int own = trip_slots(z0) + trip_slots(z1);
        int inc = own;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, inc, o);
          if (tid >= o) inc += v;
        }
        const int ex = inc - own;
        if (q0 < na) toff[q0] = ex;
        if (q1 < na) toff[q1] = ex + trip_slots(z0);
        if (tid == 31) toff[na] = inc;
      }
      __syncthreads();
      ntrip = toff[na];
    }
    if (nbt > max_nbt || ntrip > max_ntrip) {  // uniform over the block
      if (tid == 0) atomicOr(status, 2);
      continue;
    }
    MxLayout L = carve_mx(sm, nbt, ntrip);
    for (int q = tid; q < na; q += kMxThreads)
      for (int lb = L.aseed[q]; lb < L.aseed[q + 1]; lb++) L.meta[lb] = q;
    __syncthreads();
    const int nel = pot.nel();

    // ---- Phase 1: bond geometry in ff. ----
    for (int lb = tid; lb < nbt; lb += kMxThreads) {
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
            ff as = ff_mulf(sAf[3 * c], sx);
            as = ff_add(as, ff_mulf(sAf[3 * c + 1], sy));
            as = ff_add(as, ff_mulf(sAf[3 * c + 2], sz));
            rij[c] = ff_sub(rij[c], as);
          }
        }
        ff r2 = ff_mul(rij[0], rij[0]);
        r2 = ff_add(r2, ff_mul(rij[1], rij[1]));
        r2 = ff_add(r2, ff_mul(rij[2], rij[2]));
        const int t = pot.pair(eli, elj);
        meta |= t << 8;
        const float r2f = r2.hi + r2.lo;
        const MxPair &pp = mp.pr[t];
        if (r2f < pp.r2sq) {
          ff_sqrt_rsqrt(r2, r, rinv);
#pragma unroll
          for (int c = 0; c < 3; c++) rn[c] = ff_mul(rij[c], rinv);
          const float rf = r.hi + r.lo;
          if (r2f < pp.r1sq || rf <= pp.r1.hi) {
            fc = ff_make(1.0f, 0.0f);
          } else if (rf < pp.r2) {
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
          if (rf < pp.r2) {
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
    for (int lb = tid; lb < nbt; lb += kMxThreads) {
      const int b = b0 + lb;
      const int meta = L.meta[lb];
      if (!(meta & kFlagIJ)) {
        L.P[lb] = ff_make(0.0f, 0.0f);
        L.E[lb] = ff_make(0.0f, 0.0f);
        L.G[lb] = ff_make(0.0f, 0.0f);
        L.G[nbt + lb] = ff_make(0.0f, 0.0f);
        L.G[2 * nbt + lb] = ff_make(0.0f, 0.0f);
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
      kloop_mx<kWat, Pot::kPairTerms, Pot::kTripletH>(mp, L, lb, s, z, eli, trow, zeta, dbj, wk,
                                                       sumdk);
      // A zeta below 1e-30 would overflow the FP32 range inside ln/exp: such a
      // bond (and any non-finite estimate) takes the accurate path.
      const bool tiny = zeta > 0.0f && zeta < 1.0e-30f;
      ff bij, P, x0;
      float L0;
      const int eb = el_b<Pot::kPairTerms>(eli, t);
      bo_f(mp, eb, t, tiny ? 1.0f : zeta, L.fc[lb], VA, s_exp, bij, P, x0, L0);
      // Error estimate (eV/A) of this bond's forces on the FP32 path: the FP32
      // zeta through d b / d ln zeta, the FP32 log1p/expm1 of b, and the FP32
      // three-body derivatives multiplied by P.
      const float fva = fabsf(dVA.hi) * L.fc[lb].hi;
      const float est = fva * (2.4e-7f * bsens_f(mp, eb, zeta) +
                               1.5e-7f * fabsf(bij.hi - mp.pr[t].xi.hi)) +
                        3.0e-7f * fabsf(P.hi) *
                            (sumdk + fabsf(dbj[0]) + fabsf(dbj[1]) + fabsf(dbj[2]));
      if (tiny || !(est <= mp.hot)) {
        L.hot[atomicAdd(&s_nhot, 1)] = lb;
        // kept for the accurate pass (which overwrites these slots)
        L.P[lb] = VA;
        L.E[lb] = VR;
        L.G[lb] = P;
        L.G[nbt + lb] = x0;
        L.G[2 * nbt + lb] = ff_make(tiny ? 0.0f : zeta, L0);
      } else {
        const ff dbjf[3] = {ff_make(dbj[0], 0.0f), ff_make(dbj[1], 0.0f), ff_make(dbj[2], 0.0f)};
        ff wkf[9];
        if (kWat)
#pragma unroll
          for (int c = 0; c < 9; c++) wkf[c] = ff_make(wk[c], 0.0f);
        finalize_mx<kWat, kPB>(a, L, lb, b, bij, P, dbjf, wkf, VA, dVA, VR, dVR);
      }
    }
    __syncthreads();
    // ---- Phase 2b: the hot bonds again, k loop and bond order in ff. ----
    // kHotLanes lanes per hot bond share its k loop; the partial sums are added
    // by a fixed xor tree, then the group's first lane finishes the bond.
    {
      constexpr int kHotLanes = 8;
      constexpr int kGroups = kMxThreads / kHotLanes;
      const int nhot = s_nhot;
      if (tid == 0 && nhot > 0) atomicAdd(&status[2], nhot);  // diagnostic count
      const int gl = tid & (kHotLanes - 1);
      for (int base = 0; base < nhot; base += kGroups) {
        const int hq = base + tid / kHotLanes;
        const bool act = hq < nhot;
        ff zeta = ff_make(0.0f, 0.0f), wk[9];
        ff dbj[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
        if (kWat)
#pragma unroll
          for (int c = 0; c < 9; c++) wk[c] = ff_make(0.0f, 0.0f);
        int lb = 0;
        if (act) {
          lb = L.hot[hq];
          const int ai = L.meta[lb] & 0xff;
          const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, p = lb - s;
          kloop_ff<kWat, Pot::kPairTerms, Pot::kTripletH>(mp, L, lb, s, z, L.el[ai],
                                                           L.t + L.toff[ai] + p * z, s_exp, gl,
                                                           kHotLanes, zeta, dbj, wk);
        }
#pragma unroll
        for (int o = 1; o < kHotLanes; o <<= 1) {
          zeta = ff_add(zeta, ff_shfl_xor(zeta, o));
#pragma unroll
          for (int c = 0; c < 3; c++) dbj[c] = ff_add(dbj[c], ff_shfl_xor(dbj[c], o));
          if (kWat)
#pragma unroll
            for (int c = 0; c < 9; c++) wk[c] = ff_add(wk[c], ff_shfl_xor(wk[c], o));
        }
        if (act && gl == 0) {
          const int b = b0 + lb;
          const int meta = L.meta[lb];
          const int ai = meta & 0xff;
          const int t = (meta >> 8) & 0xf;
          const int eli = L.el[ai];
          const MxPair &pp = mp.pr[t];
          const ff VA = L.P[lb], VR = L.E[lb];  // from the FP32 pass
          const ff dVA = ff_neg(ff_mul(pp.cA, VA));
          const ff dVR = ff_neg(ff_mul(pp.cR, VR));
          ff bij, P;
          const ff zl = L.G[2 * nbt + lb];  // (FP32-pass zeta, L0)
          if (zl.hi > 0.0f && zeta.hi > 1.0e-30f) {
            bo_hot(mp, el_b<Pot::kPairTerms>(eli, t), t, L.G[lb], L.G[nbt + lb], zl.hi, zl.lo,
                   (zeta.hi - zl.hi) + zeta.lo, s_exp, bij, P);
          } else {
            // FP64 bond order for a vanishing zeta (outside the FP32 range of ln/exp)
            double b64, P64;
            pot.template bo<double>(eli, t, ff_to_double(zeta), ff_to_double(L.fc[lb]),
                                    ff_to_double(VA), b64, P64);
            bij = ff_from_double(b64);
            P = ff_from_double(P64);
          }
          finalize_mx<kWat, kPB>(a, L, lb, b, bij, P, dbj, wk, VA, dVA, VR, dVR);
        }
      }
    }
    __syncthreads();

    // ---- Phase 3: k-role forces (ff) and the virial (FP32 per thread). ----
    for (int lb = tid; lb < nbt; lb += kMxThreads) {
      const int b = b0 + lb;
      const int meta = L.meta[lb];
      ff_acc(eacc, L.E[lb]);
      ff G[3] = {L.G[lb], L.G[nbt + lb], L.G[2 * nbt + lb]};
      if (meta & kFlagK) {
        const int ai = meta & 0xff;
        const int s = L.aseed[ai], z = L.aseed[ai + 1] - s, q = lb - s;
        const ff *tcol = L.t + L.toff[ai] + q;
        for (int pq = 0; pq < z; pq++) {
          const int lp = s + pq;
          if (lp == lb) continue;
          if (!(L.meta[lp] & kFlagIJ)) continue;
          const ff mP = ff_neg(L.P[lp]);
          const ff *tv = tcol + pq * z;
#pragma unroll
          for (int c = 0; c < 3; c++) ff_acc_mul(G[c], mP, tv[c * ntrip]);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) G[c] = ff_norm(G[c]);
        const float r = L.r[lb].hi;
        float rb[3];
#pragma unroll
        for (int c = 0; c < 3; c++) rb[c] = r * L.rn[c * nbt + lb].hi;
#pragma unroll
        for (int c1 = 0; c1 < 3; c1++)
#pragma unroll
          for (int c2 = 0; c2 < 3; c2++)
            wacc[c1 + 3 * c2] = fmaf(-rb[c1], G[c2].hi + G[c2].lo, wacc[c1 + 3 * c2]);
      }
      float2 *Gout = reinterpret_cast<float2 *>(a.G) + 3 * (size_t)b;
      Gout[0] = make_float2(G[0].hi, G[0].lo);
      Gout[1] = make_float2(G[1].hi, G[1].lo);
      Gout[2] = make_float2(G[2].hi, G[2].lo);
    }
    if (a.tile_atom0) {  // batches: one partial row per tile (structure sums)
      block_sum_tile(ff_norm(eacc), wacc, a.tile_part + 10 * (size_t)tile, red_scratch);
      eacc = ff_make(0.0f, 0.0f);
#pragma unroll
      for (int c = 0; c < 9; c++) wacc[c] = 0.0f;
    }
  }  // tiles
  if (!a.tile_atom0)
    block_sum_tile(ff_norm(eacc), wacc, a.tile_part + 10 * (size_t)blockIdx.x, red_scratch);
}

// Gather of the ff bond forces: F_a = sum_b (G[rev b] - G[b]) in ff.
template <bool kEpa, bool kWat>
__global__ void bop_gather_mx(int nat, const int *__restrict__ seed, const int *__restrict__ rev,
                              const float2 *__restrict__ G, const double *__restrict__ ebond,
                              const double *__restrict__ wbond, double *__restrict__ f,
                              double *__restrict__ epa, double *__restrict__ wpa,
                              ReplayCheck chk, int fset) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (replay_invalid(chk)) return;  // (uniform over the grid)
  ff F[3] = {ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f), ff_make(0.0f, 0.0f)};
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
    for (int c = 0; c < 3; c++) {
      const float2 gr = G[3 * (size_t)rb + c], gb = G[3 * (size_t)b + c];
      F[c] = ff_add(F[c], ff_sub(ff_make(gr.x, gr.y), ff_make(gb.x, gb.y)));
    }
    if (kEpa) E += ebond[b] + ebond[rb];
    if (kWat)
#pragma unroll
      for (int c = 0; c < 9; c++) W[c] += wbond[9 * (size_t)b + c] + wbond[9 * (size_t)rb + c];
  }
  const double Fd[3] = {ff_to_double(F[0]), ff_to_double(F[1]), ff_to_double(F[2])};
  store_block_forces<kGatherThreads>(f, nat, Fd, fset);
  if (i >= nat) return;
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
