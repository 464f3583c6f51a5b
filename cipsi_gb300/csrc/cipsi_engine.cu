// cipsi_engine.cu -- GB300 (sm_103a) engine for the CIPSI second-order
// perturbation / selection step (the work of cip/pertu.f + cip/diexcit.f).
//
// Algorithm (same perturber set, owners and weights as the reference, which
// walks excitation lists one candidate at a time, cip/igene.f, pert1.f):
//
//   * S determinants are alpha/beta occupation bitstrings, W 64-bit words per
//     spin (W = 1 for norb <= 64, 2 for norb <= 128).
//   * One CTA owns one generator k at a time (persistent grid, atomic work
//     queue).  It first gathers nb(k) = { j in S : degree(j,k) <= 4 } with the
//     mask of k's electrons that j lacks.
//   * Candidates I = k - R + A are processed in blocks of fixed removed
//     electrons R (|R| = 1 or 2).  For a block, L_R = { j in nb(k) :
//     |(k - R) \ j| <= 2 } is compacted into shared memory; it contains every
//     S determinant that can be within two excitations of any I of the block.
//     Each thread then takes added spin orbitals A and scans L_R only.
//   * The reference's loop structure decides which excitations of k are
//     examined (rank-change classes gated by the content of S,
//     igene.f:34-35,89-90,199-200,296-298), the owner test (pert1.f:104-118,
//     diexcit.f:246-259), the scan for interacting S determinants
//     (pert1.f:129-144, diexcit.f:267-285), the spin-flip weights
//     (pert1.f:150-164, diexcit.f:304-316), the MP / EN denominators and
//     selection (pert1.f:171-295, diexcit.f:327-478).  All of that is
//     restated here per candidate, as set rules on bitstrings.
//   * Matrix elements use canonical (alpha string, beta string) phases; S
//     coefficients are converted once on the host from the reference's
//     excitation-list phase, so <I|H|Psi>^2 is identical.
//   * (pq|rs) are read as real*4 (as cip stores them, cip/reijkl.f:27) and
//     widened to double; everything else is double.  E2 sums are Kahan
//     compensated per thread and reduced in a fixed order (deterministic).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cipsi_gb300.h"

namespace {

constexpr int kNClass = CIPSI_NCLASS;
constexpr int kMaxRoots = CIPSI_MAX_ROOTS;
constexpr int kThreads = 256;
constexpr int kMaxSym = 8;
constexpr int kMaxElec = 64;
constexpr int kMaxOrb = 128;
constexpr int kRowCap = 128;  // per-warp list of |K' \ j| = 2 entries holding a1

// counters[] slots
enum {
  C_IETAT = 0,
  C_NPROC,
  C_NSEL,
  C_NCAND,
  C_NCMP,
  C_NP1,
  C_NP2,
  C_ALGB,
  C_LRFALLBACK,
  C_NCOUNTERS
};

struct Params {
  int norb, noca, nel, ncf, metat, nsym, isym;
  int ngen;
  const int32_t* gens;       // generator indices (0-based); -1 = pertu block
  const uint8_t* gen_dmask;  // allowed rank changes per generator, bit (D+2)
  int nunits;                // work units: (generator slot, range of R blocks
  const int32_t* unit_g;     //   or, for the pertu block, of candidates)
  const int32_t* unit_r0;
  const int32_t* unit_r1;
  const uint64_t* S;         // ncf x 2W words (alpha words, beta words)
  const uint8_t* ygen;
  const int32_t* nesp;
  const uint8_t* yef;
  const double* c;           // ncf x metat, canonical phase
  const float* eri;
  const int32_t* pairtab;    // norb x norb: pair index | irrep << 24
  const int32_t* ntttt;     // [irrep 1..nsym] first packed index (1-based)
  const double* F;           // packed i*(i+1)/2 + j (i >= j, 0-based)
  const double* J;
  const double* K;
  const double* fmpb;        // 2*norb by spin orbital
  const int8_t* orbsym;      // 0-based irreps
  int its[kMaxSym][kMaxSym]; // 0-based product table
  double e[kMaxRoots], eb[kMaxRoots], emp[kMaxRoots], teste[kMaxRoots], taum[kMaxRoots];
  int yen, ysele, ymoyen, ywdeg, symvar, nclass;
  double tau, teseff;
  double aval[kNClass];
  long long aval_bits[kNClass];  // bit patterns of aval (non-negative, ascending)
  int pertu_ref, pertu_mono;
  // scratch
  int32_t* nb_j;             // per block: ncf entries
  uint64_t* nb_emask;
  int32_t* lr_idx;           // per block: ncf entries (fallback path)
  int lr_cap;                // shared-memory capacity of L_R
  // outputs
  double* gen_part;          // ngen x (5 * metat)
  unsigned long long* counters;
  unsigned long long* dpivot_bits;
  unsigned long long* hist_nom;      // nclass
  unsigned long long* hist_nam;      // nclass x metat
  double* hist_tab;                  // 2 x nclass x metat (tabmp, tabvp)
  uint64_t* sel_bits;                // cap x 2W
  int32_t* sel_owner;
  double* sel_xam;
  double* sel_evp;                   // cap x metat
  long long sel_cap;
  int* work;                         // work counter
};

// ------------------------------------------------------------ bit helpers
template <int W>
__device__ __forceinline__ int popc_between(const uint64_t* s, int lo, int hi) {
  // number of set bits strictly between orbital positions lo < hi
  int cnt = 0;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    const int base = w * 64;
    const int from = max(lo + 1 - base, 0);
    const int to = min(hi - base, 64);
    if (from < to) {
      const uint64_t hiMask = (to >= 64) ? ~0ull : ((1ull << to) - 1ull);
      const uint64_t loMask = (1ull << from) - 1ull;
      cnt += __popcll(s[w] & hiMask & ~loMask);
    }
  }
  return cnt;
}

template <int W>
__device__ __forceinline__ int first_bit(const uint64_t* s) {
#pragma unroll
  for (int w = 0; w < W; ++w)
    if (s[w]) return w * 64 + __ffsll((long long)s[w]) - 1;
  return -1;
}

template <int W>
__device__ __forceinline__ int last_bit(const uint64_t* s) {
#pragma unroll
  for (int w = W - 1; w >= 0; --w)
    if (s[w]) return w * 64 + 63 - __clzll((long long)s[w]);
  return -1;
}

__device__ __forceinline__ int tri(int i, int j) {
  return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
}

// (ij|kl) as cip/ai.f looks it up: packed pair indices, zero across irreps
__device__ __forceinline__ double ai(const Params& p, int i, int j, int k, int l) {
  const int pij = __ldg(&p.pairtab[i * p.norb + j]);
  const int pkl = __ldg(&p.pairtab[k * p.norb + l]);
  const int s1 = pij >> 24, s2 = pkl >> 24;
  if (s1 != s2) return 0.0;
  const long long a = pij & 0xFFFFFF, b = pkl & 0xFFFFFF;
  const long long lo = a < b ? a : b, hi = a < b ? b : a;
  const long long idx = lo + hi * (hi - 1) / 2 + __ldg(&p.ntttt[s1]) - 2;
  return (double)__ldg(&p.eri[idx]);
}

// <I|H|J> for degree 1 or 2, canonical phases.  u = I bits, v = J bits
// (alpha words then beta words).  rankI / rankJ: excitation degree relative
// to the reference determinant; the one-difference element sums over the
// holes and particles of the more excited determinant as cip/hntd.f does.
template <int W>
__device__ double hmat(const Params& p, const uint64_t* u, const uint64_t* v, int rankI, int rankJ,
                       const uint64_t* hf, int& kind) {
  uint64_t remv[2 * W], addv[2 * W];
  int nrem[2] = {0, 0};
#pragma unroll
  for (int q = 0; q < 2 * W; ++q) {
    const uint64_t x = u[q] ^ v[q];
    remv[q] = x & v[q];  // occupied in J only
    addv[q] = x & u[q];  // occupied in I only
    nrem[q / W] += __popcll(remv[q]);
  }
  const int norb = p.norb;
  if (nrem[0] + nrem[1] == 1) {
    kind = 1;
    const int s = nrem[0] ? 0 : 1;
    const int pp = first_bit<W>(remv + s * W);
    const int qq = first_bit<W>(addv + s * W);
    const int lo = pp < qq ? pp : qq, hi = pp < qq ? qq : pp;
    const int sign = (popc_between<W>(v + s * W, lo, hi) & 1) ? -1 : 1;
    double val = __ldg(&p.F[tri(pp, qq)]);
    const uint64_t* D = (rankI > rankJ) ? u : v;
    // holes of D (occupied in the reference, empty in D)
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
#pragma unroll
      for (int w = 0; w < W; ++w) {
        uint64_t h = hf[sp * W + w] & ~D[sp * W + w];
        while (h) {
          const int r = w * 64 + __ffsll((long long)h) - 1;
          h &= h - 1;
          val -= ai(p, pp, qq, r, r);
          if (sp == s) val += ai(p, pp, r, qq, r);
        }
        uint64_t t = D[sp * W + w] & ~hf[sp * W + w];
        while (t) {
          const int r = w * 64 + __ffsll((long long)t) - 1;
          t &= t - 1;
          val += ai(p, pp, qq, r, r);
          if (sp == s) val -= ai(p, pp, r, qq, r);
        }
      }
    }
    (void)norb;
    return sign * val;
  }
  kind = 2;
  if (nrem[0] == 1 && nrem[1] == 1) {
    const int pa = first_bit<W>(remv), qa = first_bit<W>(addv);
    const int pb = first_bit<W>(remv + W), qb = first_bit<W>(addv + W);
    const int sa = popc_between<W>(v, min(pa, qa), max(pa, qa));
    const int sb = popc_between<W>(v + W, min(pb, qb), max(pb, qb));
    const double val = ai(p, pa, qa, pb, qb);
    return ((sa + sb) & 1) ? -val : val;
  }
  const int s = nrem[0] == 2 ? 0 : 1;
  const uint64_t* rm = remv + s * W;
  const uint64_t* ad = addv + s * W;
  const int p1 = first_bit<W>(rm), p2 = last_bit<W>(rm);
  const int q1 = first_bit<W>(ad), q2 = last_bit<W>(ad);
  uint64_t mid[W];
#pragma unroll
  for (int w = 0; w < W; ++w) mid[w] = v[s * W + w];
  const int s1 = popc_between<W>(mid, min(p1, q1), max(p1, q1));
  mid[p1 >> 6] &= ~(1ull << (p1 & 63));
  mid[q1 >> 6] |= (1ull << (q1 & 63));
  const int s2 = popc_between<W>(mid, min(p2, q2), max(p2, q2));
  const double val = ai(p, p1, q1, p2, q2) - ai(p, p1, q2, p2, q1);
  return ((s1 + s2) & 1) ? -val : val;
}

// hmp (cip/hmp.f) and hdig (cip/hdig.f) of I, written over the sets of
// holes H and particles P of I relative to the reference determinant.
template <int W>
__device__ void diag_terms(const Params& p, const uint64_t* u, const uint64_t* hf, double& hmpi,
                           double& hdigi, bool want_hdig) {
  int hs[24], ps[24];  // spin orbital codes: orb + spin * norb
  int nh = 0, np = 0;
#pragma unroll
  for (int sp = 0; sp < 2; ++sp) {
#pragma unroll
    for (int w = 0; w < W; ++w) {
      uint64_t h = hf[sp * W + w] & ~u[sp * W + w];
      while (h && nh < 24) {
        hs[nh++] = w * 64 + __ffsll((long long)h) - 1 + sp * p.norb;
        h &= h - 1;
      }
      uint64_t t = u[sp * W + w] & ~hf[sp * W + w];
      while (t && np < 24) {
        ps[np++] = w * 64 + __ffsll((long long)t) - 1 + sp * p.norb;
        t &= t - 1;
      }
    }
  }
  double mp = 0.0;
  for (int i = 0; i < np; ++i) mp += __ldg(&p.fmpb[ps[i]]);
  for (int i = 0; i < nh; ++i) mp -= __ldg(&p.fmpb[hs[i]]);
  hmpi = mp;
  if (!want_hdig) {
    hdigi = 0.0;
    return;
  }
  const int n = p.norb;
  double e = 0.0;
  for (int i = 0; i < np; ++i) {
    const int o = ps[i] % n;
    e += __ldg(&p.F[tri(o, o)]);
  }
  for (int i = 0; i < nh; ++i) {
    const int o = hs[i] % n;
    e -= __ldg(&p.F[tri(o, o)]);
  }
  auto jk = [&](int a, int b) -> double {
    const int oa = a % n, ob = b % n;
    const int t = tri(oa, ob);
    double x = __ldg(&p.J[t]);
    if ((a / n) == (b / n)) x -= __ldg(&p.K[t]);
    return x;
  };
  // same-position terms of the reference's pair sum, 0.5*(J_tt-K_tt+J_pp-K_pp)
  for (int i = 0; i < nh; ++i) e += 0.5 * jk(hs[i], hs[i]);
  for (int i = 0; i < np; ++i) e += 0.5 * jk(ps[i], ps[i]);
  for (int i = 0; i < nh; ++i)
    for (int j = i + 1; j < nh; ++j) e += jk(hs[i], hs[j]);
  for (int i = 0; i < np; ++i)
    for (int j = i + 1; j < np; ++j) e += jk(ps[i], ps[j]);
  for (int i = 0; i < nh; ++i)
    for (int j = 0; j < np; ++j) e -= jk(hs[i], ps[j]);
  hdigi = e;
}

// bit patterns of 0.05, 1e-6 and +inf
constexpr long long kBits005 = 0x3fa999999999999all;
constexpr long long kBits1em6 = 0x3eb0c6f7a0b5ed8dll;
constexpr long long kBitsInf = 0x7ff0000000000000ll;
// a < b for a >= 0 (a may be NaN: false), b >= 0
__device__ __forceinline__ bool lt_nonneg(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return x < y && x <= kBitsInf;
}
// max of a >= 0 (not NaN) and b >= 0 (may be NaN: fmax ignores it)
__device__ __forceinline__ double max_nonneg(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  if (y > kBitsInf) return a;
  return __longlong_as_double(x > y ? x : y);
}

__device__ __forceinline__ void kahan_add(double& s, double& c, double x) {
  const double y = x - c;
  const double t = s + y;
  c = (t - s) - y;
  s = t;
}

// Block-wide order-preserving compaction: calls emit(slot, i) for every i in
// [0, n) with pred(i), slots dense and increasing with i (deterministic).
// Must be called by every thread of the block.
template <typename Pred, typename Emit>
__device__ int ordered_compact(int n, Pred pred, Emit emit, int* warp_tmp /* >= 33 ints */) {
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  int total = 0;
  for (int base = 0; base < n; base += blockDim.x) {
    const int i = base + tid;
    const bool keep = i < n && pred(i);
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_tmp[wid] = __popc(m);
    __syncthreads();
    if (wid == 0) {
      const int v = lane < nw ? warp_tmp[lane] : 0;
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane < nw) warp_tmp[lane] = x - v;  // exclusive prefix
      if (lane == 31) warp_tmp[32] = x;       // round total
    }
    __syncthreads();
    if (keep) emit(total + warp_tmp[wid] + __popc(m & ((1u << lane) - 1u)), i);
    total += warp_tmp[32];
    __syncthreads();
  }
  return total;
}

template <int R>
struct Acc {
  double e2mp[R], cmp[R], e2vp[R], cvp[R], e2b[R], cb[R], psimp[R], psivp[R];
  unsigned long long ietat, nproc, nsel, ncand, ncmp, np1, np2, algb;
  double dpivot;
  __device__ void zero() {
#pragma unroll
    for (int m = 0; m < R; ++m) {
      e2mp[m] = cmp[m] = e2vp[m] = cvp[m] = e2b[m] = cb[m] = psimp[m] = psivp[m] = 0.0;
    }
    ietat = nproc = nsel = ncand = ncmp = np1 = np2 = algb = 0ull;
    dpivot = 0.0;
  }
};

// One thread's histogram (cip/isto.f): class sums and counts, indexed by
// class at run time, so it lives in local memory (L1-resident); one FP64 add
// per contribution, no atomics; merged into the block's at kernel end.
template <int R>
struct HistPriv {
  double tab[kNClass][2][R];
  unsigned long long nom[kNClass];
  unsigned long long nam[kNClass][R];
  __device__ void zero() {
    for (int c = 0; c < kNClass; ++c) {
      nom[c] = 0ull;
      for (int m = 0; m < R; ++m) {
        tab[c][0][m] = tab[c][1][m] = 0.0;
        nam[c][m] = 0ull;
      }
    }
  }
};

struct SmemHist {
  unsigned long long nom[kNClass];
  unsigned long long nam[kNClass * kMaxRoots];
  double tab[2 * kNClass * kMaxRoots];
};

// histogram class of a non-negative value (cip/isto.f: first i with
// val < aval(i)); compared as IEEE bit patterns, which order non-negative
// doubles exactly as the values (integer pipe instead of FP64 compares)
__device__ __forceinline__ int hist_class(const Params& p, double val) {
  const long long v = __double_as_longlong(val);
  const int nc = p.nclass - 1;
  int c = 0;
  for (int i = 0; i < nc; ++i) c += (v >= p.aval_bits[i]) ? 1 : 0;
  return c;
}

// Everything the reference does with one candidate after its interaction
// scan: denominators, E2, selection, histogram, unit-60 record.  Called by
// all 32 lanes of a warp; `live` marks the lanes holding a perturber.
template <int W, int R>
__device__ void finish_candidate(const Params& p, bool live, const uint64_t* u, double hmpi,
                                 double hvpi, const double* bc, int owner1 /*1-based, 0 = pertu*/,
                                 double fmul, int nmul, bool ybis, bool is_pert1, Acc<R>& acc,
                                 HistPriv<R>& hp) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  double xam = 0.0;
  bool ydeg = false;
  double vil[R], semp[R], sevp[R];
  // the reference adds each term and then term*fmul (spin-flip weight,
  // pert1.f:280-287); one compensated add of term*(1+fmul) is used here
  const double wgt = ybis ? 1.0 + fmul : 1.0;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    vil[m] = 0.0;
    semp[m] = sevp[m] = 0.0;
    if (!live || m >= p.metat) continue;
    const double bcalc = bc[m];
    const double dmp = p.emp[m] - hmpi;
    double eivp = 0.0, cimp, xim, deno, eim;
    if (p.yen) {
      // the three denominators share one FP64 division (GB300's FP64 rate is
      // 1/64 of FP32): r = 1/(dmp*dvp*db), 1/dmp = dvp*db*r, etc.
      const double dvp = p.e[m] - hvpi;
      const double db = p.eb[m] - hvpi;
      const double pvb = dvp * db;
      const double prod = dmp * pvb;
      double civp, cib;
      if (fabs(prod) > 1.0e-280 && fabs(prod) < 1.0e280) {
        const double r = 1.0 / prod;
        cimp = bcalc * (pvb * r);
        civp = bcalc * ((dmp * db) * r);
        cib = bcalc * ((dmp * dvp) * r);
      } else {  // a denominator at (or near) zero or huge: divide one by one
        cimp = bcalc / dmp;
        civp = bcalc / dvp;
        cib = bcalc / db;
      }
      eivp = bcalc * civp;
      kahan_add(acc.e2vp[m], acc.cvp[m], eivp * wgt);
      acc.psivp[m] = fma(civp * civp, wgt, acc.psivp[m]);
      kahan_add(acc.e2b[m], acc.cb[m], (bcalc * cib) * wgt);
      xim = p.ysele ? fabs(eivp) : fabs(civp);
      deno = dvp;
      eim = eivp;
    } else {
      cimp = bcalc / dmp;
    }
    const double eimp = bcalc * cimp;
    kahan_add(acc.e2mp[m], acc.cmp[m], eimp * wgt);
    acc.psimp[m] = fma(cimp * cimp, wgt, acc.psimp[m]);
    if (!p.yen) {
      xim = p.ysele ? fabs(eimp) : fabs(cimp);
      deno = dmp;
      eim = eimp;
    }
    // comparisons of magnitudes on their IEEE bit patterns (exact for
    // non-negative doubles; NaN compares as in the reference: never below)
    const long long bdeno = __double_as_longlong(deno) & 0x7fffffffffffffffll;
    const long long beim = __double_as_longlong(eim) & 0x7fffffffffffffffll;
    if (!(bdeno > kBits005 && bdeno <= kBitsInf) && !(beim < kBits1em6) && p.ywdeg) ydeg = true;
    if (lt_nonneg(xim, p.teste[m])) acc.dpivot = max_nonneg(acc.dpivot, xim);
    if (p.ymoyen) {
      xim = xim * p.taum[m];
      vil[m] = xim;
      xam = max_nonneg(xam, xim);
    }
    semp[m] = eimp;
    sevp[m] = eivp;
  }
  if (live) {
    acc.ietat += (unsigned long long)(long long)(nmul + 1);
    acc.nproc += 1;
  }
  // histogram (cip/isto.f; pert1 calls it always, diexcit only if ymoyen)
  if (live && (is_pert1 || p.ymoyen) && xam >= p.teseff) {
    const double fm = fmul + 1.0;
    const int cls = hist_class(p, xam);
    hp.nom[cls] += (unsigned long long)(1 + nmul);
#pragma unroll
    for (int m = 0; m < R; ++m) {
      if (m >= p.metat || vil[m] < p.teseff) continue;
      hp.tab[cls][0][m] += semp[m] * fm;
      hp.tab[cls][1][m] += sevp[m] * fm;
      hp.nam[hist_class(p, vil[m])][m] += (unsigned long long)(1 + nmul);
    }
  }
  if (ydeg) xam = 1.0;
  // unit-60 record (pie.f): one slot reservation per warp
  const bool sel = live && xam > p.tau && p.ymoyen;
  const unsigned sm = __ballot_sync(kFull, sel);
  if (sm) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(&p.counters[C_NSEL], (unsigned long long)__popc(sm));
    base = __shfl_sync(kFull, base, 0);
    if (sel) {
      const unsigned long long slot = base + __popc(sm & ((1u << lane) - 1u));
      if ((long long)slot < p.sel_cap) {
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) p.sel_bits[slot * 2 * W + q] = u[q];
        p.sel_owner[slot] = owner1;
        p.sel_xam[slot] = xam;
        // ENvp per root written by cipsym (cipsym/pert1.f:244): eivp*(fmul+1)
#pragma unroll
        for (int m = 0; m < R; ++m)
          if (m < p.metat) p.sel_evp[slot * p.metat + m] = p.symvar ? sevp[m] * (fmul + 1.0) : 0.0;
      }
    }
  }
}

template <int R>
__device__ void block_flush(const Params& p, Acc<R>& acc, int gslot, double* red) {
  // reduce 5*metat sums over the block in a fixed order; write gen_part[gslot]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int nq = 5 * p.metat;
  for (int q = 0; q < nq; ++q) {
    const int m = q % p.metat, which = q / p.metat;
    double v = 0.0;
#pragma unroll
    for (int mm = 0; mm < R; ++mm)
      if (mm == m) {
        v = which == 0   ? acc.e2mp[mm] - acc.cmp[mm]
            : which == 1 ? acc.e2vp[mm] - acc.cvp[mm]
            : which == 2 ? acc.e2b[mm] - acc.cb[mm]
            : which == 3 ? acc.psimp[mm]
                         : acc.psivp[mm];
      }
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[q * 32 + wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    double s = 0.0, c = 0.0;
    for (int w = 0; w < nw; ++w) kahan_add(s, c, red[threadIdx.x * 32 + w]);
    p.gen_part[(long long)gslot * nq + threadIdx.x] = s - c;
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < R; ++m) {
    acc.e2mp[m] = acc.cmp[m] = acc.e2vp[m] = acc.cvp[m] = acc.e2b[m] = acc.cb[m] = 0.0;
    acc.psimp[m] = acc.psivp[m] = 0.0;
  }
}

// Per-warp queue of perturbers that survived the interaction scan.  The
// FP64 epilogue (denominators, E2, selection) then runs on full warps: the
// FP64 pipe of GB300 is narrow, and a warp instruction costs the same with
// 32 lanes or with the few that would be live at the candidate level.
constexpr int kQCap = 64;
template <int W, int R>
struct WarpQueue {
  uint64_t u[2 * W][kQCap];
  double bc[R][kQCap];
  double hmp[kQCap], hvp[kQCap], fmul[kQCap];
  int nmul[kQCap], owner[kQCap];
  unsigned char flags[kQCap];  // bit 0 ybis, bit 1 is_pert1
};

// Enqueue the live lanes' perturbers (called by a whole warp); runs the
// epilogue on every full batch of 32.
template <int W, int R>
__device__ void enqueue_candidate(const Params& p, WarpQueue<W, R>& q, int& qn, bool live,
                                  const uint64_t* u, double hmpi, double hvpi, const double* bc,
                                  int owner1, double fmul, int nmul, bool ybis, bool is_pert1,
                                  Acc<R>& acc, HistPriv<R>& hp);

template <int W, int R>
__device__ __noinline__ void drain_queue(const Params& p, WarpQueue<W, R>& q, int& qn, bool all, Acc<R>& acc,
                            HistPriv<R>& hp) {
  const int lane = threadIdx.x & 31;
  while (qn >= 32 || (all && qn > 0)) {
    const int base = qn >= 32 ? qn - 32 : 0;
    const int cnt = qn >= 32 ? 32 : qn;
    const bool live = lane < cnt;
    const int e = base + (live ? lane : 0);
    uint64_t u[2 * W];
#pragma unroll
    for (int w = 0; w < 2 * W; ++w) u[w] = q.u[w][e];
    double bc[R];
#pragma unroll
    for (int m = 0; m < R; ++m) bc[m] = q.bc[m][e];
    const unsigned char f = q.flags[e];
    finish_candidate<W, R>(p, live, u, q.hmp[e], q.hvp[e], bc, q.owner[e], q.fmul[e], q.nmul[e],
                           (f & 1) != 0, (f & 2) != 0, acc, hp);
    __syncwarp();
    qn = base;
  }
}

template <int W, int R>
__device__ void enqueue_candidate(const Params& p, WarpQueue<W, R>& q, int& qn, bool live,
                                  const uint64_t* u, double hmpi, double hvpi, const double* bc,
                                  int owner1, double fmul, int nmul, bool ybis, bool is_pert1,
                                  Acc<R>& acc, HistPriv<R>& hp) {
  const int lane = threadIdx.x & 31;
  const unsigned lm = __ballot_sync(0xffffffffu, live);
  if (live) {
    const int e = qn + __popc(lm & ((1u << lane) - 1u));
#pragma unroll
    for (int w = 0; w < 2 * W; ++w) q.u[w][e] = u[w];
#pragma unroll
    for (int m = 0; m < R; ++m) q.bc[m][e] = bc[m];
    q.hmp[e] = hmpi;
    q.hvp[e] = hvpi;
    q.fmul[e] = fmul;
    q.nmul[e] = nmul;
    q.owner[e] = owner1;
    q.flags[e] = (unsigned char)((ybis ? 1 : 0) | (is_pert1 ? 2 : 0));
  }
  qn += __popc(lm);
  __syncwarp();
  drain_queue<W, R>(p, q, qn, false, acc, hp);
}

// ------------------------------------------------------------------ kernel
struct BlockShared {
  double vdg[2 * kMaxOrb];  // hdig(K'+a) - hdig(K') without the pair term
  double hK, mK;            // hdig(K'), hmp(K')
  int dn_so[48];            // spin orbitals where K' differs from the reference
  int dn_sg[48];            // +1 (occupied virtual) / -1 (empty reference orbital)
  int ndn;
  uint64_t kbits[2 * 2];
  int occ[kMaxElec];      // spin orbital code (orb + spin*norb) of k's electrons
  int vir[2][kMaxOrb];    // virtual orbitals of k per spin
  int nvir[2];
  int nel_s[2];
  int nnb;
  int nlr;
  int gen;
  int kidx;
  int rank_k;
};

template <int W, int R>
__global__ void __launch_bounds__(kThreads, 2) k_pt2(Params p) {
  extern __shared__ __align__(16) unsigned char dyn[];
  __shared__ BlockShared sh;
  __shared__ SmemHist hist;
  __shared__ double red[5 * kMaxRoots * 32];
  __shared__ int ctmp[33];
  __shared__ int16_t wrow[(kThreads / 32) * kRowCap];

  const int tid = threadIdx.x;
  // shared L_R arrays (fast path)
  uint64_t* lr_bits = reinterpret_cast<uint64_t*>(dyn);          // cap x 2W
  int32_t* lr_j = reinterpret_cast<int32_t*>(lr_bits + (size_t)p.lr_cap * 2 * W);
  // per-warp epilogue queues, 16-byte aligned after the L_R arrays
  const size_t qoff = (((size_t)p.lr_cap * (2 * W * 8 + 4)) + 15) & ~(size_t)15;
  WarpQueue<W, R>& wq = reinterpret_cast<WarpQueue<W, R>*>(dyn + qoff)[threadIdx.x >> 5];
  int qn = 0;
  int32_t* my_nb_j = p.nb_j + (size_t)blockIdx.x * p.ncf;
  uint64_t* my_nb_em = p.nb_emask + (size_t)blockIdx.x * p.ncf;
  int32_t* my_lr_idx = p.lr_idx + (size_t)blockIdx.x * p.ncf;

  for (int i = tid; i < kNClass; i += blockDim.x) hist.nom[i] = 0;
  for (int i = tid; i < kNClass * kMaxRoots; i += blockDim.x) hist.nam[i] = 0;
  for (int i = tid; i < 2 * kNClass * kMaxRoots; i += blockDim.x) hist.tab[i] = 0.0;

  uint64_t hf[2 * W];
#pragma unroll
  for (int s = 0; s < 2; ++s)
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const int lo = w * 64;
      const int n = min(max(p.noca - lo, 0), 64);
      hf[s * W + w] = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
    }

  Acc<R> acc;
  acc.zero();
  HistPriv<R> hp;
  hp.zero();
  const int ncf = p.ncf;

  for (;;) {
    __syncthreads();
    if (tid == 0) sh.gen = atomicAdd(p.work, 1);
    __syncthreads();
    const int unit = sh.gen;
    if (unit >= p.nunits) break;
    const int g = p.unit_g[unit];
    const int ur0 = p.unit_r0[unit], ur1 = p.unit_r1[unit];
    const int k = p.gens[g];

    if (k < 0) {
      // ---------------- pertu: reference and its singles, no owner test
      // candidates: t = 0 -> reference (if pertu_ref), then singles
      const int no = p.noca, nv = p.norb - p.noca;
      for (int t0 = ur0; t0 < ur1; t0 += blockDim.x) {
        const int t = t0 + tid;
        bool live = t < ur1;
        uint64_t u[2 * W];
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) u[q] = hf[q];
        const int tt = p.pertu_ref ? t - 1 : t;  // tt < 0: the reference itself
        if (live && tt >= 0) {
          const int s = tt / (no * nv);
          const int rem = tt % (no * nv);
          const int o = rem / nv, vv = no + rem % nv;
          if (p.its[p.orbsym[o]][p.orbsym[vv]] != p.isym - 1) live = false;
          u[s * W + (o >> 6)] &= ~(1ull << (o & 63));
          u[s * W + (vv >> 6)] |= (1ull << (vv & 63));
        }
        double bc[R];
#pragma unroll
        for (int m = 0; m < R; ++m) bc[m] = 0.0;
        double hmpi = 0.0, hvpi = 0.0;
        if (live) {
          acc.ncand++;
          int rankI = 0;
#pragma unroll
          for (int q = 0; q < 2 * W; ++q) rankI += __popcll(hf[q] & ~u[q]);
          int nint = 0;
          bool drop = false;
          for (int j = 0; j < ncf; ++j) {
            const uint64_t* v = p.S + (size_t)j * 2 * W;
            int x = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) x += __popcll(u[q] ^ __ldg(&v[q]));
            acc.ncmp++;
            if (x > 4) continue;
            if (x == 0) {
              drop = true;
              break;
            }
            uint64_t vv[2 * W];
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) vv[q] = __ldg(&v[q]);
            int rankJ = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) rankJ += __popcll(hf[q] & ~vv[q]);
            int kind;
            const double h = hmat<W>(p, u, vv, rankI, rankJ, hf, kind);
            if (kind == 1) acc.np1++; else acc.np2++;
            ++nint;
#pragma unroll
            for (int m = 0; m < R; ++m)
              if (m < p.metat) bc[m] += h * __ldg(&p.c[(size_t)j * p.metat + m]);
          }
          if (drop || nint == 0) live = false;
          if (live) diag_terms<W>(p, u, hf, hmpi, hvpi, p.yen != 0);
        }
        enqueue_candidate<W, R>(p, wq, qn, live, u, hmpi, hvpi, bc, 0, 0.0, 0, false, true, acc, hp);
      }
      drain_queue<W, R>(p, wq, qn, true, acc, hp);
      block_flush<R>(p, acc, unit, red);
      continue;
    }

    // ---------------- generator k: neighbours within degree 4
    if (tid == 0) {
      sh.kidx = k;
      sh.nnb = 0;
    }
    if (tid < 2 * W) sh.kbits[tid] = p.S[(size_t)k * 2 * W + tid];
    __syncthreads();
    uint64_t kb[2 * W];
#pragma unroll
    for (int q = 0; q < 2 * W; ++q) kb[q] = sh.kbits[q];
    if (tid == 0) {
      // electron list and virtual lists of k
      int ne = 0;
      for (int s = 0; s < 2; ++s) {
        int nes = 0, nv = 0;
        for (int o = 0; o < p.norb; ++o) {
          if ((kb[s * W + (o >> 6)] >> (o & 63)) & 1ull) {
            sh.occ[ne++] = o + s * p.norb;
            ++nes;
          } else {
            sh.vir[s][nv++] = o;
          }
        }
        sh.nel_s[s] = nes;
        sh.nvir[s] = nv;
      }
      int rk = 0;
      for (int q = 0; q < 2 * W; ++q) rk += __popcll(hf[q] & ~kb[q]);
      sh.rank_k = rk;
    }
    __syncthreads();
    const int nel = sh.nel_s[0] + sh.nel_s[1];
    const int nnb = ordered_compact(
        ncf,
        [&](int j) {
          int x = 0;
#pragma unroll
          for (int q = 0; q < 2 * W; ++q) x += __popcll(kb[q] ^ __ldg(&p.S[(size_t)j * 2 * W + q]));
          return x <= 8;
        },
        [&](int slot, int j) {
          // electrons of k missing in j, as a mask over k's electron indices
          uint64_t em = 0;
#pragma unroll
          for (int q = 0; q < 2 * W; ++q) {
            uint64_t miss = kb[q] & ~__ldg(&p.S[(size_t)j * 2 * W + q]);
            while (miss) {
              const int b = __ffsll((long long)miss) - 1;
              miss &= miss - 1;
              // electron index = occupied bits of k before this bit
              int idx = 0;
              const int s = q / W, w = q % W;
              if (s == 1) idx += sh.nel_s[0];
              for (int w2 = 0; w2 < w; ++w2) idx += __popcll(kb[s * W + w2]);
              idx += __popcll(kb[q] & ((1ull << b) - 1ull));
              em |= 1ull << idx;
            }
          }
          my_nb_j[slot] = j;
          my_nb_em[slot] = em;
        },
        ctmp);
    const int rank_k = sh.rank_k;
    const uint8_t dmask = p.gen_dmask[g];
    const int k1 = k + 1;  // 1-based owner index
    const int nespk = p.nesp[k];
    const bool yefk = p.yef[k] != 0;

    // ---------------- blocks of removed electrons R (this unit's range)
    for (int r = ur0; r < ur1; ++r) {
      int e1, e2 = -1;
      if (r < nel) {
        e1 = r;
      } else {
        // pair index -> (e1 < e2)
        int t = r - nel;
        e1 = 0;
        while (t >= nel - 1 - e1) {
          t -= nel - 1 - e1;
          ++e1;
        }
        e2 = e1 + 1 + t;
      }
      const int so1 = sh.occ[e1];
      const int so2 = e2 >= 0 ? sh.occ[e2] : -1;
      const int sp1 = so1 / p.norb, o1 = so1 % p.norb;
      const int sp2 = so2 >= 0 ? so2 / p.norb : -1, o2 = so2 >= 0 ? so2 % p.norb : -1;
      const int nRr = e2 >= 0 ? 2 : 1;
      const int hfR = (o1 < p.noca ? 1 : 0) + (e2 >= 0 && o2 < p.noca ? 1 : 0);
      // achievable rank changes D = hfR + aV - |R| (aV = added HF-virtuals)
      bool any = false;
      for (int aV = 0; aV <= nRr; ++aV) {
        const int D = hfR + aV - nRr;
        if (dmask & (1u << (D + 2))) any = true;
      }
      if (!any) continue;
      const uint64_t rmask = (1ull << e1) | (e2 >= 0 ? (1ull << e2) : 0ull);
      // L_R, partitioned: entries with |K' \ j| <= 1 first, then those with
      // |K' \ j| = 2; each part in ascending j, so every sum over interacting
      // determinants runs in a fixed order (bitwise reproducible results)
      auto lr_store = [&](int slot, int t) {
        const int j = my_nb_j[t];
        if (slot < p.lr_cap) {
          lr_j[slot] = j;
          const uint64_t* v = p.S + (size_t)j * 2 * W;
#pragma unroll
          for (int q = 0; q < 2 * W; ++q) lr_bits[(size_t)slot * 2 * W + q] = __ldg(&v[q]);
        }
        my_lr_idx[slot] = j;
      };
      auto lr_m = [&](int t) {
        const uint64_t em = my_nb_em[t];
        return __popcll(em) - __popcll(em & rmask);
      };
      const int n01 = ordered_compact(nnb, [&](int t) { return lr_m(t) <= 1; }, lr_store, ctmp);
      const int n2 = ordered_compact(
          nnb, [&](int t) { return lr_m(t) == 2; }, [&](int slot, int t) { lr_store(n01 + slot, t); },
          ctmp);
      const int nlr = n01 + n2;
      const bool fast = nlr <= p.lr_cap;
      if (!fast && tid == 0) atomicAdd(&p.counters[C_LRFALLBACK], 1ull);
      // K' = k - R
      uint64_t kp[2 * W];
#pragma unroll
      for (int q = 0; q < 2 * W; ++q) kp[q] = kb[q];
      kp[sp1 * W + (o1 >> 6)] &= ~(1ull << (o1 & 63));
      if (e2 >= 0) kp[sp2 * W + (o2 >> 6)] &= ~(1ull << (o2 & 63));
      // diagonal energies of I = K' + A from those of K' (cip/hdig.f, hmp.f
      // written over occupation changes dn relative to the reference):
      //   hdig = sum_r dn_r F_rr + 1/2 sum_rs dn_r dn_s (J_rs - [same spin] K_rs)
      //   hmp  = sum_r dn_r fmpb_r
      if (tid == 0) {
        int nd = 0;
        for (int sp = 0; sp < 2; ++sp)
          for (int w = 0; w < W; ++w) {
            uint64_t h = hf[sp * W + w] & ~kp[sp * W + w];
            while (h) {
              const int b = __ffsll((long long)h) - 1;
              h &= h - 1;
              sh.dn_so[nd] = w * 64 + b + sp * p.norb;
              sh.dn_sg[nd++] = -1;
            }
            uint64_t t2 = kp[sp * W + w] & ~hf[sp * W + w];
            while (t2) {
              const int b = __ffsll((long long)t2) - 1;
              t2 &= t2 - 1;
              sh.dn_so[nd] = w * 64 + b + sp * p.norb;
              sh.dn_sg[nd++] = 1;
            }
          }
        sh.ndn = nd;
      }
      __syncthreads();
      {
        const int ndn = sh.ndn, n = p.norb;
        for (int a = tid; a < 2 * n; a += blockDim.x) {
          const int oa = a % n, sa = a / n;
          double g = 0.0;
          for (int i = 0; i < ndn; ++i) {
            const int r = sh.dn_so[i];
            const int t = tri(oa, r % n);
            double x = __ldg(&p.J[t]);
            if (sa == r / n) x -= __ldg(&p.K[t]);
            g += sh.dn_sg[i] * x;
          }
          const int ta = tri(oa, oa);
          sh.vdg[a] = __ldg(&p.F[ta]) + g + 0.5 * (__ldg(&p.J[ta]) - __ldg(&p.K[ta]));
        }
        if (tid == 32) {
          double e = 0.0, mp = 0.0;
          for (int i = 0; i < ndn; ++i) {
            const int r = sh.dn_so[i], orr = r % n;
            e += sh.dn_sg[i] * __ldg(&p.F[tri(orr, orr)]);
            mp += sh.dn_sg[i] * __ldg(&p.fmpb[r]);
            for (int j = 0; j < ndn; ++j) {
              const int q = sh.dn_so[j];
              const int t = tri(orr, q % n);
              double x = __ldg(&p.J[t]);
              if (r / n == q / n) x -= __ldg(&p.K[t]);
              e += 0.5 * sh.dn_sg[i] * sh.dn_sg[j] * x;
            }
          }
          sh.hK = e;
          sh.mK = mp;
        }
      }
      __syncthreads();
      const int symR = e2 >= 0 ? p.its[p.orbsym[o1]][p.orbsym[o2]] : p.orbsym[o1];
      // added-orbital space
      const int nv1 = sh.nvir[sp1];
      int nA;
      if (nRr == 1) {
        nA = nv1;
      } else if (sp1 == sp2) {
        nA = nv1 * (nv1 - 1) / 2;
      } else {
        nA = sh.nvir[0] * sh.nvir[1];
      }
      // One candidate I = K' + {a1[, a2]}: rank-change class, symmetry and
      // spin-pattern rules, then a scan of L_R entries [0, nscan) plus the
      // listed entries rb[0..nrb) (owner test, already in S, <I|H|j>), then
      // the E2 / selection epilogue.  Called by whole warps.
      auto candidate = [&](bool live, int a1, int a2, int sa1, int sa2, int nscan, const int16_t* rb,
                           int nrb) {
        int D = 0;
        bool ysyspi = true;
        if (live) {
          const int aV = (a1 >= p.noca ? 1 : 0) + (a2 >= 0 && a2 >= p.noca ? 1 : 0);
          D = hfR + aV - nRr;
          if (!(dmask & (1u << (D + 2)))) live = false;
          const int symA = a2 >= 0 ? p.its[p.orbsym[a1]][p.orbsym[a2]] : p.orbsym[a1];
          if (p.its[symR][symA] != 0) live = false;
          // diexcit spin patterns for generators without a flip partner
          if (live && D == 2) {
            if (sp1 != sp2) {
              // alpha hole orbital o1, beta hole o2, alpha particle a1, beta particle a2
              ysyspi = !(o1 == o2 && a1 == a2);
              const bool unflipped = (o1 < o2) || (o1 == o2 && a1 <= a2);
              if (!yefk && !unflipped) live = false;
            } else if (!yefk && sp1 == 1) {
              live = false;
            }
          }
        }
        uint64_t u[2 * W];
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) u[q] = kp[q];
        double bc[R];
#pragma unroll
        for (int m = 0; m < R; ++m) bc[m] = 0.0;
        int nint = 0, nnz = 0, lesp = 0;
        if (live) {
          acc.ncand++;
          u[sa1 * W + (a1 >> 6)] |= (1ull << (a1 & 63));
          if (a2 >= 0) u[sa2 * W + (a2 >> 6)] |= (1ull << (a2 & 63));
          const int rankI = rank_k + D;
          bool drop = false;
          // one S determinant of L_R against I: owner test, already-in-S
          // test, <I|H|j> accumulation; returns true when I is dropped
          auto visit = [&](int i, int x) -> bool {
            uint64_t vv[2 * W];
            int j;
            if (fast) {
              j = lr_j[i];
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) vv[q] = lr_bits[(size_t)i * 2 * W + q];
            } else {
              j = my_lr_idx[i];
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) vv[q] = __ldg(&p.S[(size_t)j * 2 * W + q]);
            }
            if (j < k) return p.ygen[j] != 0;
            if (x == 0) return true;
            int rankJ = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) rankJ += __popcll(hf[q] & ~vv[q]);
            int kind;
            const double h = hmat<W>(p, u, vv, rankI, rankJ, hf, kind);
            if (kind == 1) acc.np1++; else acc.np2++;
            ++nint;
            if (h != 0.0) ++nnz;
            if (j > k && j <= k + nespk) ++lesp;
#pragma unroll
            for (int m = 0; m < R; ++m)
              if (m < p.metat) bc[m] += h * __ldg(&p.c[(size_t)j * p.metat + m]);
            return false;
          };
          for (int i0 = 0; i0 < nscan && !drop; i0 += 4) {
            // four independent compares per step (latency of the loads overlaps)
            int xs[4];
#pragma unroll
            for (int g4 = 0; g4 < 4; ++g4) {
              const int i = i0 + g4;
              int x = 99;
              if (i < nscan) {
                x = 0;
                if (fast) {
#pragma unroll
                  for (int q = 0; q < 2 * W; ++q) x += __popcll(u[q] ^ lr_bits[(size_t)i * 2 * W + q]);
                } else {
                  const int jj = my_lr_idx[i];
#pragma unroll
                  for (int q = 0; q < 2 * W; ++q) x += __popcll(u[q] ^ __ldg(&p.S[(size_t)jj * 2 * W + q]));
                }
              }
              xs[g4] = x;
            }
            if (xs[0] > 4 && xs[1] > 4 && xs[2] > 4 && xs[3] > 4) continue;
#pragma unroll 1
            for (int g4 = 0; g4 < 4 && !drop; ++g4)
              if (xs[g4] <= 4) drop = visit(i0 + g4, xs[g4]);
          }
          for (int q2 = 0; q2 < nrb && !drop; ++q2) {
            const int i = rb[q2];
            int x = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) x += __popcll(u[q] ^ lr_bits[(size_t)i * 2 * W + q]);
            if (x <= 4) drop = visit(i, x);
          }
          acc.ncmp += (unsigned long long)(nscan + nrb);
          if (drop || nint == 0) live = false;
          if (live && D == 2 && nnz == 0) live = false;  // diexcit drops zero couplings
        }
        const bool is_pert1 = (D != 2);
        double fmul = 0.0, hmpi = 0.0, hvpi = 0.0;
        int nmul = 0;
        bool ybis = false;
        if (live) {
          if (is_pert1) {
            if (nespk != 0) {
              ybis = true;
              fmul = (1.0 / (double)(lesp + 1)) * (double)(nespk + 1) - 1.0;
              nmul = (int)fmul;
            }
          } else {
            int nespf = nespk;
            ybis = nespf > 0;
            if (yefk || ysyspi) {
              ybis = true;
              if (!yefk) nespf = nespf + nespf + 1;
            }
            fmul = (1.0 / (double)(lesp + 1)) * (double)(nespf + 1) - 1.0;
            nmul = (int)fmul;
          }
          hmpi = sh.mK + __ldg(&p.fmpb[a1 + sa1 * p.norb]);
          hvpi = sh.hK + sh.vdg[a1 + sa1 * p.norb];
          if (a2 >= 0) {
            hmpi += __ldg(&p.fmpb[a2 + sa2 * p.norb]);
            const int tq = tri(a1, a2);
            double gq = __ldg(&p.J[tq]);
            if (sa1 == sa2) gq -= __ldg(&p.K[tq]);
            hvpi += sh.vdg[a2 + sa2 * p.norb] + gq;
          }
        }
        enqueue_candidate<W, R>(p, wq, qn, live, u, hmpi, hvpi, bc, k1, fmul, nmul, ybis, is_pert1, acc, hp);
      };
      if (nRr == 1 || !fast) {
        // flat: threads take candidates, every candidate scans all of L_R
        for (int t0 = 0; t0 < nA; t0 += blockDim.x) {
          const int t = t0 + tid;
          const bool live = t < nA;
          int a1 = 0, a2 = -1, sa1 = sp1, sa2 = sp2;
          if (live) {
            if (nRr == 1) {
              a1 = sh.vir[sp1][t];
            } else if (sp1 == sp2) {
              // t -> (x < y) over nv1 virtuals
              int x = 0, tt = t;
              while (tt >= nv1 - 1 - x) {
                tt -= nv1 - 1 - x;
                ++x;
              }
              a1 = sh.vir[sp1][x];
              a2 = sh.vir[sp1][x + 1 + tt];
            } else {
              a1 = sh.vir[0][t / sh.nvir[1]];
              a2 = sh.vir[1][t % sh.nvir[1]];
              sa1 = 0;
              sa2 = 1;
            }
          }
          candidate(live, a1, a2, sa1, sa2, nlr, nullptr, 0);
        }
      } else {
        // rows: one warp per first added orbital a1; an entry with
        // |K' \ j| = 2 interacts only if it occupies both added orbitals, so
        // the warp lists the ones that occupy a1 and its lanes (columns a2)
        // scan the |K' \ j| <= 1 part plus that short list
        const int lane = tid & 31, wid = tid >> 5, nwarps = blockDim.x >> 5;
        const bool same = sp1 == sp2;
        const int sr = same ? sp1 : 0, sc = same ? sp1 : 1;
        const int nrows = same ? nv1 - 1 : sh.nvir[0];
        int16_t* rowbuf = wrow + wid * kRowCap;
        for (int row = wid; row < nrows; row += nwarps) {
          const int a1 = sh.vir[sr][row];
          const int w1 = sr * W + (a1 >> 6);
          const uint64_t b1 = 1ull << (a1 & 63);
          int nrb = 0;
          for (int i0 = n01; i0 < nlr; i0 += 32) {
            const int i = i0 + lane;
            const bool has = i < nlr && (lr_bits[(size_t)i * 2 * W + w1] & b1);
            const unsigned bm = __ballot_sync(0xffffffffu, has);
            if (has) {
              const int pos = nrb + __popc(bm & ((1u << lane) - 1u));
              if (pos < kRowCap) rowbuf[pos] = (int16_t)i;
            }
            nrb += __popc(bm);
          }
          __syncwarp();
          const bool overflow = nrb > kRowCap;
          const int ncols = same ? nv1 - 1 - row : sh.nvir[1];
          for (int c0 = 0; c0 < ncols; c0 += 32) {
            const int c = c0 + lane;
            const bool live = c < ncols;
            const int a2 = live ? (same ? sh.vir[sc][row + 1 + c] : sh.vir[sc][c]) : 0;
            if (!overflow)
              candidate(live, a1, a2, sr, sc, n01, rowbuf, nrb);
            else
              candidate(live, a1, a2, sr, sc, nlr, nullptr, 0);
          }
          __syncwarp();
        }
      }
      __syncthreads();
    }
    drain_queue<W, R>(p, wq, qn, true, acc, hp);
    block_flush<R>(p, acc, unit, red);
  }

  // block totals of the integer counters and the histogram
  __syncthreads();
  {
    unsigned long long v[8] = {acc.ietat, acc.nproc, 0ull, acc.ncand, acc.ncmp, acc.np1, acc.np2, 0ull};
    for (int q = 0; q < 8; ++q) {
      unsigned long long x = v[q];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if ((tid & 31) == 0 && x) atomicAdd(&p.counters[q], x);
    }
    unsigned long long db = __double_as_longlong(acc.dpivot);
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long y = __shfl_down_sync(0xffffffffu, db, o);
      db = y > db ? y : db;
    }
    if ((tid & 31) == 0) atomicMax(p.dpivot_bits, db);
  }
  // this thread's histogram into the block's
  for (int c = 0; c < p.nclass; ++c) {
    if (hp.nom[c]) atomicAdd(&hist.nom[c], hp.nom[c]);
    for (int m = 0; m < R && m < p.metat; ++m) {
      if (hp.tab[c][0][m] != 0.0) atomicAdd(&hist.tab[c * kMaxRoots + m], hp.tab[c][0][m]);
      if (hp.tab[c][1][m] != 0.0)
        atomicAdd(&hist.tab[kNClass * kMaxRoots + c * kMaxRoots + m], hp.tab[c][1][m]);
      if (hp.nam[c][m]) atomicAdd(&hist.nam[c * kMaxRoots + m], hp.nam[c][m]);
    }
  }
  __syncthreads();
  for (int i = tid; i < p.nclass; i += blockDim.x)
    if (hist.nom[i]) atomicAdd(&p.hist_nom[i], hist.nom[i]);
  for (int i = tid; i < p.nclass * kMaxRoots; i += blockDim.x) {
    const int c = i / kMaxRoots, m = i % kMaxRoots;
    if (m >= p.metat) continue;
    if (hist.nam[i]) atomicAdd(&p.hist_nam[c * p.metat + m], hist.nam[i]);
    if (hist.tab[i] != 0.0) atomicAdd(&p.hist_tab[c * p.metat + m], hist.tab[i]);
    const double tv = hist.tab[kNClass * kMaxRoots + i];
    if (tv != 0.0) atomicAdd(&p.hist_tab[p.nclass * p.metat + c * p.metat + m], tv);
  }
}

// fixed-order Kahan reduction of the per-generator partial sums
__global__ void k_reduce(const double* part, int ngen, int nq, double* out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double s = 0.0, c = 0.0;
  for (int g = 0; g < ngen; ++g) kahan_add(s, c, part[(long long)g * nq + q]);
  out[q] = s - c;
}

}  // namespace

// =================================================================== host

struct cipsi_ctx {
  cipsi_dims d{};
  int device = 0;
  int W = 1;
  std::string err;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  bool have_int = false, have_space = false, have_roots = false;
  // host copies needed for set-up
  std::vector<int32_t> itsym, its;
  std::vector<int32_t> rank;
  std::vector<uint64_t> Sbits;
  std::vector<uint8_t> ygen, ysaut, yef1;
  std::vector<int32_t> nesp;
  std::vector<double> sigma;
  std::vector<double> croot;  // metat*ncf reference phase (column-major)
  double e[kMaxRoots]{}, eb[kMaxRoots]{}, emp[kMaxRoots]{}, teste[kMaxRoots]{}, taum[kMaxRoots]{};
  // device buffers
  uint64_t* dS = nullptr;
  uint8_t *dygen = nullptr, *dyef = nullptr;
  int32_t* dnesp = nullptr;
  double* dc = nullptr;
  float* deri = nullptr;
  int32_t* dpairtab = nullptr;
  int32_t* dntttt = nullptr;
  double *dF = nullptr, *dJ = nullptr, *dK = nullptr, *dfmpb = nullptr;
  int8_t* dorbsym = nullptr;
  int64_t ninte = 0;
  // per-run buffers
  int32_t* dunits = nullptr;
  int units_cap = 0;
  int nunits = 0;
  std::vector<int32_t> hunits;
  int32_t* dgens = nullptr;
  uint8_t* dgmask = nullptr;
  int gens_cap = 0;
  int32_t* dnb_j = nullptr;
  uint64_t* dnb_em = nullptr;
  int32_t* dlr_idx = nullptr;
  size_t scratch_blocks = 0;
  double* dgen_part = nullptr;
  size_t gen_part_cap = 0;
  unsigned long long* dcounters = nullptr;  // counters + dpivot + hist
  double* dhist_tab = nullptr;
  double* dred = nullptr;
  int* dwork = nullptr;
  uint64_t* dsel_bits = nullptr;
  int32_t* dsel_owner = nullptr;
  double *dsel_xam = nullptr, *dsel_evp = nullptr;
  long long sel_cap = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // pending run
  int ngen = 0;
  int nclass = kNClass;
  bool pending = false;
  cipsi_opts last_opts{};
  long long nsel = 0;  // records of the last fetched run
};

namespace {

int fail(cipsi_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                        \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(ctx, CIPSI_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int upload(cipsi_ctx* ctx, T** dptr, const T* h, size_t n) {
  if (*dptr) cudaFree(*dptr);
  *dptr = nullptr;
  CK(cudaMalloc((void**)dptr, std::max<size_t>(n, 1) * sizeof(T)));
  if (n) CK(cudaMemcpyAsync(*dptr, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return 0;
}

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

}  // namespace

extern "C" {

int cipsi_ctx_create(cipsi_ctx** out, const cipsi_dims* dims, int32_t device) {
  if (!out || !dims) return CIPSI_ERR_ARG;
  *out = nullptr;
  cipsi_ctx* ctx = new cipsi_ctx();
  ctx->d = *dims;
  ctx->device = device;
  const cipsi_dims& d = *dims;
  if (d.norb < 2 || d.norb > kMaxOrb) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "norb must be in [2, 128]");
  }
  if (d.noca < 1 || d.noca >= d.norb || 2 * d.noca > kMaxElec) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "noca must be in [1, min(norb-1, 32)]");
  }
  if (d.nsym < 1 || d.nsym > kMaxSym || d.isym < 1 || d.isym > d.nsym) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "nsym must be in [1, 8] and isym in [1, nsym]");
  }
  if (d.isz != 0) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "only isz = 0 (Ms = 0) is supported");
  }
  if (d.metat < 1 || d.metat > kMaxRoots) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "metat must be in [1, 8]");
  }
  if (d.ncf < 1) {
    *out = ctx;
    return fail(ctx, CIPSI_ERR_ARG, "ncf must be positive");
  }
  ctx->W = d.norb <= 64 ? 1 : 2;
  *out = ctx;
  CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
  ctx->stream = ctx->own_stream;
  CK(cudaEventCreate(&ctx->ev0));
  CK(cudaEventCreate(&ctx->ev1));
  return CIPSI_OK;
}

void cipsi_ctx_destroy(cipsi_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  dfree(ctx->dS); dfree(ctx->dygen); dfree(ctx->dyef); dfree(ctx->dnesp); dfree(ctx->dc);
  dfree(ctx->deri); dfree(ctx->dpairtab); dfree(ctx->dntttt); dfree(ctx->dF); dfree(ctx->dJ);
  dfree(ctx->dK); dfree(ctx->dfmpb); dfree(ctx->dorbsym); dfree(ctx->dgens); dfree(ctx->dgmask);
  dfree(ctx->dunits);
  dfree(ctx->dnb_j); dfree(ctx->dnb_em); dfree(ctx->dlr_idx); dfree(ctx->dgen_part);
  dfree(ctx->dcounters); dfree(ctx->dhist_tab); dfree(ctx->dred); dfree(ctx->dwork);
  dfree(ctx->dsel_bits); dfree(ctx->dsel_owner); dfree(ctx->dsel_xam); dfree(ctx->dsel_evp);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

const char* cipsi_last_error(const cipsi_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int cipsi_set_stream(cipsi_ctx* ctx, void* stream) {
  if (!ctx) return CIPSI_ERR_ARG;
  ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
  return CIPSI_OK;
}

static int set_integrals_common(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                                const double* f, const double* aj, const double* ak,
                                const int16_t* ij0, const int32_t* ntttt, int64_t ninte) {
  const int n = ctx->d.norb, ns = ctx->d.nsym;
  if (!itsym || !its || !f || !aj || !ak || !ij0 || !ntttt || ninte < 1)
    return fail(ctx, CIPSI_ERR_ARG, "set_integrals: null array or empty integral list");
  CK(cudaSetDevice(ctx->device));
  ctx->itsym.assign(itsym, itsym + n);
  ctx->its.assign(its, its + ns * ns);
  std::vector<int8_t> orbsym(n);
  for (int i = 0; i < n; ++i) {
    if (itsym[i] < 1 || itsym[i] > ns) return fail(ctx, CIPSI_ERR_ARG, "itsym out of range");
    orbsym[i] = (int8_t)(itsym[i] - 1);
  }
  for (int i = 0; i < ns * ns; ++i)
    if (its[i] < 1 || its[i] > ns) return fail(ctx, CIPSI_ERR_ARG, "its out of range");
  // pair table: pair index (1-based) | irrep (1-based) << 24, as cip/ai.f reads ij0
  std::vector<int32_t> pt((size_t)n * n);
  auto IJ0 = [&](int i, int j) -> int { return ij0[(size_t)(j - 1) * n + (i - 1)]; };
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n; ++j) {
      const int mi = std::min(i, j), ma = std::max(i, j);
      const int pidx = IJ0(mi, ma);
      const int irr = (mi == ma) ? 1 : IJ0(ma, mi);
      if (pidx < 1 || irr < 1 || irr > ns)
        return fail(ctx, CIPSI_ERR_ARG, "ij0 holds an invalid pair index or irrep");
      pt[(size_t)(i - 1) * n + (j - 1)] = pidx | (irr << 24);
    }
  std::vector<int32_t> nt(ns + 1, 0);
  for (int s = 0; s < ns; ++s) nt[s + 1] = ntttt[s];
  const size_t nter = (size_t)n * (n + 1) / 2;
  std::vector<double> F(f, f + nter);
  // cip/ijkf.f:34-37 zeroes |F| < 1e-10
  for (auto& x : F)
    if (std::fabs(x) < 1.0e-10) x = 0.0;
  int rc;
  if ((rc = upload(ctx, &ctx->dorbsym, orbsym.data(), orbsym.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dpairtab, pt.data(), pt.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dntttt, nt.data(), nt.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dF, F.data(), F.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dJ, aj, nter))) return rc;
  if ((rc = upload(ctx, &ctx->dK, ak, nter))) return rc;
  ctx->ninte = ninte;
  return CIPSI_OK;
}

int cipsi_set_integrals(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its, const double* f,
                        const double* aj, const double* ak, const int16_t* ij0,
                        const int32_t* ntttt, const float* bijkl, int64_t ninte) {
  if (!ctx) return CIPSI_ERR_ARG;
  int rc = set_integrals_common(ctx, itsym, its, f, aj, ak, ij0, ntttt, ninte);
  if (rc) return rc;
  if (!bijkl) return fail(ctx, CIPSI_ERR_ARG, "bijkl is null");
  if ((rc = upload(ctx, &ctx->deri, bijkl, (size_t)ninte))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_int = true;
  return CIPSI_OK;
}

int cipsi_set_integrals_fp64(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                             const double* f, const double* aj, const double* ak,
                             const int16_t* ij0, const int32_t* ntttt, const double* pqrs,
                             int64_t ninte) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (!pqrs) return fail(ctx, CIPSI_ERR_ARG, "pqrs is null");
  std::vector<float> b((size_t)ninte);
  for (int64_t i = 0; i < ninte; ++i) b[i] = (float)pqrs[i];  // real*8 -> real*4 (RN)
  return cipsi_set_integrals(ctx, itsym, its, f, aj, ak, ij0, ntttt, b.data(), ninte);
}

int cipsi_set_space(cipsi_ctx* ctx, const int32_t* ne, const int32_t* nd, const int32_t* trou,
                    const int32_t* part, int64_t ntp, const uint8_t* ygen, const uint8_t* ysaut,
                    const int32_t* nesp, const uint8_t* yef1) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (!ne || !nd || !trou || !part || !ygen || !ysaut || !nesp || !yef1)
    return fail(ctx, CIPSI_ERR_ARG, "set_space: null array");
  const int ncf = ctx->d.ncf, n = ctx->d.norb, W = ctx->W, noca = ctx->d.noca;
  CK(cudaSetDevice(ctx->device));
  ctx->Sbits.assign((size_t)ncf * 2 * W, 0ull);
  ctx->rank.assign(ncf, 0);
  ctx->sigma.assign(ncf, 1.0);
  for (int k = 0; k < ncf; ++k) {
    const int nec = ne[k];
    if (nec < 0 || nec > 16 || (nec > 0 && (nd[k] < 0 || nd[k] + nec > ntp)))
      return fail(ctx, CIPSI_ERR_ARG, "set_space: bad ne/nd at determinant " + std::to_string(k + 1));
    // reference determinant bits over 2*norb spin orbitals
    std::vector<uint64_t> full(4, 0ull);  // spin orbital so (0-based) -> bit so
    auto setb = [&](int so, bool on) {
      if (on) full[so >> 6] |= 1ull << (so & 63);
      else full[so >> 6] &= ~(1ull << (so & 63));
    };
    auto getb = [&](int so) { return (full[so >> 6] >> (so & 63)) & 1ull; };
    for (int o = 0; o < noca; ++o) {
      setb(o, true);
      setb(o + n, true);
    }
    int sign = 1;
    for (int i = 0; i < nec; ++i) {
      const int h = trou[nd[k] + i], pp = part[nd[k] + i];
      if (h < 1 || h > 2 * n || pp < 1 || pp > 2 * n)
        return fail(ctx, CIPSI_ERR_ARG, "set_space: spin orbital out of range");
      const int h0 = h - 1, p0 = pp - 1;
      if (!getb(h0) || getb(p0))
        return fail(ctx, CIPSI_ERR_ARG, "set_space: invalid excitation list at determinant " +
                                            std::to_string(k + 1));
      // phase of a+_p a_h on the canonical string (reference pair convention)
      const int lo = std::min(h0, p0), hi = std::max(h0, p0);
      int cnt = 0;
      for (int so = lo + 1; so < hi; ++so) cnt += (int)getb(so);
      if (cnt & 1) sign = -sign;
      setb(h0, false);
      setb(p0, true);
    }
    ctx->sigma[k] = sign;
    ctx->rank[k] = nec;
    int nal = 0, nbe = 0;
    for (int o = 0; o < n; ++o) {
      if (getb(o)) {
        ctx->Sbits[(size_t)k * 2 * W + (o >> 6)] |= 1ull << (o & 63);
        ++nal;
      }
      if (getb(o + n)) {
        ctx->Sbits[(size_t)k * 2 * W + W + (o >> 6)] |= 1ull << (o & 63);
        ++nbe;
      }
    }
    if (nal != noca || nbe != noca)
      return fail(ctx, CIPSI_ERR_ARG, "set_space: determinant with Ms != 0");
  }
  ctx->ygen.assign(ygen, ygen + ncf);
  ctx->ysaut.assign(ysaut, ysaut + ncf);
  ctx->yef1.assign(yef1, yef1 + ncf);
  ctx->nesp.assign(nesp, nesp + ncf);
  for (int k = 0; k < ncf; ++k) {
    ctx->ygen[k] = ctx->ygen[k] ? 1 : 0;
    ctx->ysaut[k] = ctx->ysaut[k] ? 1 : 0;
    ctx->yef1[k] = ctx->yef1[k] ? 1 : 0;
  }
  int rc;
  if ((rc = upload(ctx, &ctx->dS, ctx->Sbits.data(), ctx->Sbits.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dygen, ctx->ygen.data(), ctx->ygen.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dyef, ctx->yef1.data(), ctx->yef1.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dnesp, ctx->nesp.data(), ctx->nesp.size()))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_space = true;
  ctx->have_roots = false;  // coefficients need the phases of this space
  return CIPSI_OK;
}

int cipsi_set_roots(cipsi_ctx* ctx, const double* c, const double* e, const double* eb,
                    const double* emp, const double* teste, const double* taum,
                    const double* fmpb) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (!ctx->have_space) return fail(ctx, CIPSI_ERR_STATE, "set_roots before set_space");
  if (!c || !e || !eb || !emp || !teste || !taum || !fmpb)
    return fail(ctx, CIPSI_ERR_ARG, "set_roots: null array");
  const int ncf = ctx->d.ncf, mt = ctx->d.metat, n = ctx->d.norb;
  CK(cudaSetDevice(ctx->device));
  std::vector<double> cc((size_t)ncf * mt);
  for (int k = 0; k < ncf; ++k)
    for (int m = 0; m < mt; ++m) cc[(size_t)k * mt + m] = ctx->sigma[k] * c[(size_t)m * ncf + k];
  for (int m = 0; m < mt; ++m) {
    ctx->e[m] = e[m];
    ctx->eb[m] = eb[m];
    ctx->emp[m] = emp[m];
    ctx->teste[m] = teste[m];
    ctx->taum[m] = taum[m];
  }
  int rc;
  if ((rc = upload(ctx, &ctx->dc, cc.data(), cc.size()))) return rc;
  if ((rc = upload(ctx, &ctx->dfmpb, fmpb, (size_t)2 * n))) return rc;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_roots = true;
  return CIPSI_OK;
}

}  // extern "C"

static size_t queue_bytes(int W, int R) {
  switch (W * 16 + R) {
    case 16 + 1: return sizeof(WarpQueue<1, 1>);
    case 16 + 2: return sizeof(WarpQueue<1, 2>);
    case 16 + 4: return sizeof(WarpQueue<1, 4>);
    case 16 + 8: return sizeof(WarpQueue<1, 8>);
    case 32 + 1: return sizeof(WarpQueue<2, 1>);
    case 32 + 2: return sizeof(WarpQueue<2, 2>);
    case 32 + 4: return sizeof(WarpQueue<2, 4>);
    default: return sizeof(WarpQueue<2, 8>);
  }
}

template <int W, int R>
static cudaError_t launch_pt2(const Params& p, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e = cudaFuncSetAttribute(k_pt2<W, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_pt2<W, R><<<grid, kThreads, smem, st>>>(p);
  return cudaGetLastError();
}

extern "C" {

int cipsi_run_pt2_async(cipsi_ctx* ctx, const cipsi_opts* o) {
  if (!ctx || !o) return CIPSI_ERR_ARG;
  if (!ctx->have_int || !ctx->have_space || !ctx->have_roots)
    return fail(ctx, CIPSI_ERR_STATE, "run before set_integrals / set_space / set_roots");
  if (o->nclass < 2 || o->nclass > kNClass) return fail(ctx, CIPSI_ERR_ARG, "nclass must be in [2, 10]");
  CK(cudaSetDevice(ctx->device));
  const int ncf = ctx->d.ncf, W = ctx->W, mt = ctx->d.metat;
  // flags on the content of S (pertu.f:52-61)
  bool yd = false, ym = false, yf = false;
  for (int k = 0; k < ncf; ++k) {
    if (ctx->rank[k] == 1) ym = true;
    if (ctx->rank[k] == 0) yd = true;
    if (ctx->rank[k] == 2) yf = true;
  }
  if (ym) yf = true;
  std::vector<int32_t> gens;
  std::vector<uint8_t> gmask;
  const bool pertu_ref = yf && !yd && ctx->d.isym == 1;  // isz == 0, !yion
  const bool pertu_mono = yf && ym;
  if (o->run_pertu && (pertu_ref || pertu_mono)) {
    gens.push_back(-1);
    gmask.push_back(0);
  }
  for (int k = 0; k < ncf; ++k) {
    if (!ctx->ygen[k] || ctx->ysaut[k]) continue;
    if (o->gen_mask && !o->gen_mask[k]) continue;
    const int nec = ctx->rank[k];
    // allowed rank changes, bit (D + 2); D = +2 (diexcit) always
    uint8_t m = 1u << 4;
    if (!((nec == 0 && ym) || (nec == 1 && yd))) {
      m |= 1u << 3;  // +1
      const bool stop1 = nec < 1 || (ym && nec == 1) || (nec == 2 && yd);
      if (!stop1) {
        m |= 1u << 2;  // 0
        if (!((nec == 3 && yd) || (nec == 2 && ym))) {
          m |= 1u << 1;  // -1
          if (!((nec == 2 && (yd || yf)) || (nec == 3 && ym) || (nec == 4 && yd))) m |= 1u << 0;
        }
      }
    }
    gens.push_back(k);
    gmask.push_back(m);
  }
  const int ngen = (int)gens.size();
  ctx->ngen = ngen;
  // work units: a generator's R blocks are split into chunks of at most
  // kRChunk blocks that have an allowed rank-change class, so one heavy
  // generator does not serialise on one SM; low-rank generators (which meet
  // most of S) are queued first.
  constexpr int kRChunk = 6;
  constexpr int kPertuChunk = 128;
  std::vector<int32_t> ug, ur0, ur1;
  {
    const int n = ctx->d.norb, noca = ctx->d.noca, nel = 2 * noca;
    const int nR = nel + nel * (nel - 1) / 2;
    std::vector<int> order(ngen);
    for (int g = 0; g < ngen; ++g) order[g] = g;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
      const int ra = gens[a] < 0 ? -1 : ctx->rank[gens[a]];
      const int rb = gens[b] < 0 ? -1 : ctx->rank[gens[b]];
      return ra < rb;
    });
    std::vector<int> hfe(nel);
    for (int g : order) {
      const int k = gens[g];
      if (k < 0) {
        const int ntot = (pertu_ref ? 1 : 0) + (pertu_mono ? 2 * noca * (n - noca) : 0);
        for (int t = 0; t < ntot; t += kPertuChunk) {
          ug.push_back(g);
          ur0.push_back(t);
          ur1.push_back(std::min(ntot, t + kPertuChunk));
        }
        continue;
      }
      // electrons of k: alpha orbitals ascending, then beta; HF-occupied?
      int ne = 0;
      for (int sp = 0; sp < 2; ++sp)
        for (int o = 0; o < n; ++o)
          if ((ctx->Sbits[(size_t)k * 2 * W + sp * W + (o >> 6)] >> (o & 63)) & 1ull) hfe[ne++] = o < noca;
      const uint8_t m = gmask[g];
      auto allowed = [&](int r) {
        int hfR, nRr;
        if (r < nel) {
          hfR = hfe[r];
          nRr = 1;
        } else {
          int t = r - nel, e1 = 0;
          while (t >= nel - 1 - e1) {
            t -= nel - 1 - e1;
            ++e1;
          }
          hfR = hfe[e1] + hfe[e1 + 1 + t];
          nRr = 2;
        }
        for (int aV = 0; aV <= nRr; ++aV)
          if (m & (1u << (hfR + aV - nRr + 2))) return true;
        return false;
      };
      int cnt = 0, start = -1;
      for (int r = 0; r < nR; ++r) {
        if (!allowed(r)) continue;
        if (start < 0) start = r;
        if (++cnt == kRChunk) {
          ug.push_back(g);
          ur0.push_back(start);
          ur1.push_back(r + 1);
          cnt = 0;
          start = -1;
        }
      }
      if (start >= 0) {
        ug.push_back(g);
        ur0.push_back(start);
        ur1.push_back(nR);
      }
    }
  }
  const int nunits = (int)ug.size();
  ctx->nunits = nunits;
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  // shared L_R capacity: enough for every neighbour list when it fits
  const size_t per_entry = (size_t)2 * W * 8 + 4;
  const size_t qbytes = (size_t)(kThreads / 32) * queue_bytes(W, mt <= 1 ? 1 : mt <= 2 ? 2 : mt <= 4 ? 4 : 8);
  const size_t smem_budget = (size_t)200 * 1024 - qbytes;  // L_R share of the dynamic smem
  int lr_cap = (int)std::min<size_t>((size_t)ncf, smem_budget / per_entry);
  const size_t smem = (((size_t)lr_cap * per_entry + 15) & ~(size_t)15) + qbytes + 16;
  const int blocks_per_sm = smem <= 95 * 1024 ? 2 : 1;
  int grid = std::max(1, std::min(nunits, dev_sms * blocks_per_sm));
  // buffers
  if ((size_t)grid > ctx->scratch_blocks || !ctx->dnb_j) {
    dfree(ctx->dnb_j); dfree(ctx->dnb_em); dfree(ctx->dlr_idx);
    CK(cudaMalloc(&ctx->dnb_j, (size_t)grid * ncf * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dnb_em, (size_t)grid * ncf * sizeof(uint64_t)));
    CK(cudaMalloc(&ctx->dlr_idx, (size_t)grid * ncf * sizeof(int32_t)));
    ctx->scratch_blocks = grid;
  }
  if (ngen > ctx->gens_cap) {
    dfree(ctx->dgens); dfree(ctx->dgmask);
    CK(cudaMalloc(&ctx->dgens, (size_t)std::max(ngen, 1) * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dgmask, (size_t)std::max(ngen, 1)));
    ctx->gens_cap = ngen;
  }
  if (nunits > ctx->units_cap) {
    dfree(ctx->dunits);
    CK(cudaMalloc(&ctx->dunits, (size_t)std::max(nunits, 1) * 3 * sizeof(int32_t)));
    ctx->units_cap = nunits;
  }
  if (ngen) {
    CK(cudaMemcpyAsync(ctx->dgens, gens.data(), ngen * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->dgmask, gmask.data(), ngen, cudaMemcpyHostToDevice, ctx->stream));
  }
  if (nunits) {
    ctx->hunits.resize((size_t)3 * nunits);
    std::copy(ug.begin(), ug.end(), ctx->hunits.begin());
    std::copy(ur0.begin(), ur0.end(), ctx->hunits.begin() + nunits);
    std::copy(ur1.begin(), ur1.end(), ctx->hunits.begin() + 2 * nunits);
    CK(cudaMemcpyAsync(ctx->dunits, ctx->hunits.data(), (size_t)3 * nunits * sizeof(int32_t),
                       cudaMemcpyHostToDevice, ctx->stream));
  }
  const size_t nq = (size_t)5 * mt;
  if ((size_t)std::max(nunits, 1) * nq > ctx->gen_part_cap) {
    dfree(ctx->dgen_part);
    ctx->gen_part_cap = (size_t)std::max(nunits, 1) * nq;
    CK(cudaMalloc(&ctx->dgen_part, ctx->gen_part_cap * sizeof(double)));
  }
  // counters [C_NCOUNTERS] + dpivot + nom[10] + nam[10*8]
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  if (!ctx->dcounters) {
    CK(cudaMalloc(&ctx->dcounters, ncount * sizeof(unsigned long long)));
    CK(cudaMalloc(&ctx->dhist_tab, 2 * kNClass * kMaxRoots * sizeof(double)));
    CK(cudaMalloc(&ctx->dred, 5 * kMaxRoots * sizeof(double)));
    CK(cudaMalloc(&ctx->dwork, sizeof(int)));
  }
  if (ctx->sel_cap == 0) {
    ctx->sel_cap = 1 << 20;
    CK(cudaMalloc(&ctx->dsel_bits, (size_t)ctx->sel_cap * 2 * W * sizeof(uint64_t)));
    CK(cudaMalloc(&ctx->dsel_owner, (size_t)ctx->sel_cap * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dsel_xam, (size_t)ctx->sel_cap * sizeof(double)));
    CK(cudaMalloc(&ctx->dsel_evp, (size_t)ctx->sel_cap * mt * sizeof(double)));
  }
  CK(cudaMemsetAsync(ctx->dcounters, 0, ncount * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dhist_tab, 0, 2 * kNClass * kMaxRoots * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->dwork, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->dgen_part, 0, (size_t)std::max(nunits, 1) * nq * sizeof(double), ctx->stream));

  Params p{};
  p.norb = ctx->d.norb;
  p.noca = ctx->d.noca;
  p.nel = 2 * ctx->d.noca;
  p.ncf = ncf;
  p.metat = mt;
  p.nsym = ctx->d.nsym;
  p.isym = ctx->d.isym;
  p.ngen = ngen;
  p.gens = ctx->dgens;
  p.gen_dmask = ctx->dgmask;
  p.nunits = nunits;
  p.unit_g = ctx->dunits;
  p.unit_r0 = ctx->dunits + nunits;
  p.unit_r1 = ctx->dunits + 2 * nunits;
  p.S = ctx->dS;
  p.ygen = ctx->dygen;
  p.nesp = ctx->dnesp;
  p.yef = ctx->dyef;
  p.c = ctx->dc;
  p.eri = ctx->deri;
  p.pairtab = ctx->dpairtab;
  p.ntttt = ctx->dntttt;
  p.F = ctx->dF;
  p.J = ctx->dJ;
  p.K = ctx->dK;
  p.fmpb = ctx->dfmpb;
  p.orbsym = ctx->dorbsym;
  for (int i = 0; i < ctx->d.nsym; ++i)
    for (int j = 0; j < ctx->d.nsym; ++j) p.its[i][j] = ctx->its[(size_t)j * ctx->d.nsym + i] - 1;
  for (int m = 0; m < mt; ++m) {
    p.e[m] = ctx->e[m];
    p.eb[m] = ctx->eb[m];
    p.emp[m] = ctx->emp[m];
    p.teste[m] = ctx->teste[m];
    p.taum[m] = ctx->taum[m];
  }
  p.yen = o->yen;
  p.ysele = o->ysele;
  p.ymoyen = o->ymoyen;
  p.ywdeg = o->ywdeg;
  p.symvar = o->sym_variant;
  p.nclass = o->nclass;
  p.tau = o->tau;
  p.teseff = o->teseff;
  for (int i = 0; i < kNClass; ++i) {
    p.aval[i] = o->aval[i];
    std::memcpy(&p.aval_bits[i], &o->aval[i], 8);
  }
  for (int i = 0; i + 1 < o->nclass; ++i)
    if (!(o->aval[i] >= 0.0) || (i > 0 && !(o->aval[i] > o->aval[i - 1])))
      return fail(ctx, CIPSI_ERR_ARG, "aval must be non-negative and increasing");
  p.pertu_ref = pertu_ref ? 1 : 0;
  p.pertu_mono = pertu_mono ? 1 : 0;
  p.nb_j = ctx->dnb_j;
  p.nb_emask = ctx->dnb_em;
  p.lr_idx = ctx->dlr_idx;
  p.lr_cap = lr_cap;
  p.gen_part = ctx->dgen_part;
  p.counters = ctx->dcounters;
  p.dpivot_bits = ctx->dcounters + C_NCOUNTERS;
  p.hist_nom = ctx->dcounters + C_NCOUNTERS + 1;
  p.hist_nam = ctx->dcounters + C_NCOUNTERS + 1 + kNClass;
  p.hist_tab = ctx->dhist_tab;
  p.sel_bits = ctx->dsel_bits;
  p.sel_owner = ctx->dsel_owner;
  p.sel_xam = ctx->dsel_xam;
  p.sel_evp = ctx->dsel_evp;
  p.sel_cap = ctx->sel_cap;
  p.work = ctx->dwork;

  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (nunits > 0) {
    cudaError_t e;
    const int R = mt <= 1 ? 1 : mt <= 2 ? 2 : mt <= 4 ? 4 : 8;
    if (W == 1) {
      e = R == 1 ? launch_pt2<1, 1>(p, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<1, 2>(p, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<1, 4>(p, grid, smem, ctx->stream)
                 : launch_pt2<1, 8>(p, grid, smem, ctx->stream);
    } else {
      e = R == 1 ? launch_pt2<2, 1>(p, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<2, 2>(p, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<2, 4>(p, grid, smem, ctx->stream)
                 : launch_pt2<2, 8>(p, grid, smem, ctx->stream);
    }
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_pt2 launch: ") + cudaGetErrorString(e));
    k_reduce<<<1, 64, 0, ctx->stream>>>(ctx->dgen_part, nunits, (int)nq, ctx->dred);
    CK(cudaGetLastError());
  } else {
    CK(cudaMemsetAsync(ctx->dred, 0, nq * sizeof(double), ctx->stream));
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->nclass = o->nclass;
  ctx->pending = true;
  ctx->last_opts = *o;
  return CIPSI_OK;
}

int cipsi_fetch_result(cipsi_ctx* ctx, cipsi_result* r) {
  if (!ctx || !r) return CIPSI_ERR_ARG;
  if (!ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "fetch_result without a run");
  CK(cudaSetDevice(ctx->device));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->pending = false;
  const int mt = ctx->d.metat;
  memset(r, 0, sizeof(*r));
  std::vector<double> red(5 * mt);
  CK(cudaMemcpy(red.data(), ctx->dred, red.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (int m = 0; m < mt; ++m) {
    r->e2mp[m] = red[0 * mt + m];
    r->e2vp[m] = red[1 * mt + m];
    r->e2b[m] = red[2 * mt + m];
    r->psimp[m] = red[3 * mt + m];
    r->psivp[m] = red[4 * mt + m];
  }
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  std::vector<unsigned long long> cnt(ncount);
  CK(cudaMemcpy(cnt.data(), ctx->dcounters, ncount * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  std::vector<double> tab(2 * kNClass * kMaxRoots);
  CK(cudaMemcpy(tab.data(), ctx->dhist_tab, tab.size() * sizeof(double), cudaMemcpyDeviceToHost));
  r->ietat = (int64_t)cnt[C_IETAT];
  r->n_processed = (int64_t)cnt[C_NPROC];
  r->n_candidates = (int64_t)cnt[C_NCAND];
  r->n_compares = (int64_t)cnt[C_NCMP];
  r->n_pairs_1 = (int64_t)cnt[C_NP1];
  r->n_pairs_2 = (int64_t)cnt[C_NP2];
  {
    unsigned long long b = cnt[C_NCOUNTERS];
    double dp;
    memcpy(&dp, &b, 8);
    r->dpivot = dp;
  }
  const int nc = ctx->nclass;
  for (int i = 0; i < nc; ++i) r->nom[i] = (int64_t)cnt[C_NCOUNTERS + 1 + i];
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < mt; ++m) {
      r->nam[c * kMaxRoots + m] = (int64_t)cnt[C_NCOUNTERS + 1 + kNClass + c * mt + m];
      r->tabmp[c * kMaxRoots + m] = tab[c * mt + m];
      r->tabvp[c * kMaxRoots + m] = tab[nc * mt + c * mt + m];
    }
  // algorithmic bytes of the E2 loop (per interacting pair: metat coefficients
  // + integrals as stored; per perturber: diagonal terms), see the docs
  const double avg_rank = 4.0;
  r->alg_bytes = (int64_t)(cnt[C_NP2] * (8.0 * mt + 2 * 4.0 + 8.0) +
                           cnt[C_NP1] * (8.0 * mt + 8.0 + 2.0 * avg_rank * 2 * 4.0) +
                           cnt[C_NPROC] * (8.0 * avg_rank + 8.0 * (avg_rank + avg_rank * avg_rank) + 8.0 * mt));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  r->kernel_ms = ms;
  // selection: records stay on the device until cipsi_selection_get/raw
  const long long nsel = (long long)cnt[C_NSEL];
  if (nsel > ctx->sel_cap)
    return fail(ctx, CIPSI_ERR_OVERFLOW,
                "selection buffer overflow: " + std::to_string(nsel) + " records > capacity " +
                    std::to_string(ctx->sel_cap) + " (cipsi_run_pt2 grows the buffer and reruns)");
  ctx->nsel = nsel;
  r->n_selected = nsel;
  return CIPSI_OK;
}

int cipsi_run_pt2(cipsi_ctx* ctx, const cipsi_opts* opts, cipsi_result* res) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    int rc = cipsi_run_pt2_async(ctx, opts);
    if (rc) return rc;
    rc = cipsi_fetch_result(ctx, res);
    if (rc != CIPSI_ERR_OVERFLOW) return rc;
    // grow the selection buffer to what the run needed and redo
    unsigned long long nsel = 0;
    CK(cudaMemcpy(&nsel, ctx->dcounters + C_NSEL, 8, cudaMemcpyDeviceToHost));
    dfree(ctx->dsel_bits); dfree(ctx->dsel_owner); dfree(ctx->dsel_xam); dfree(ctx->dsel_evp);
    ctx->sel_cap = (long long)(nsel + nsel / 8 + 1024);
    const int W = ctx->W, mt = ctx->d.metat;
    CK(cudaMalloc(&ctx->dsel_bits, (size_t)ctx->sel_cap * 2 * W * sizeof(uint64_t)));
    CK(cudaMalloc(&ctx->dsel_owner, (size_t)ctx->sel_cap * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dsel_xam, (size_t)ctx->sel_cap * sizeof(double)));
    CK(cudaMalloc(&ctx->dsel_evp, (size_t)ctx->sel_cap * mt * sizeof(double)));
  }
  return fail(ctx, CIPSI_ERR_OVERFLOW, "selection buffer could not be grown");
}

int cipsi_selection_raw(cipsi_ctx* ctx, int64_t first, int64_t count, uint64_t* bits,
                        int32_t* owner, double* xam, double* evp) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (first < 0 || count < 0 || first + count > ctx->nsel)
    return fail(ctx, CIPSI_ERR_ARG, "selection: range outside the selection");
  if (count == 0) return CIPSI_OK;
  CK(cudaSetDevice(ctx->device));
  const int W = ctx->W, mt = ctx->d.metat;
  if (bits)
    CK(cudaMemcpyAsync(bits, ctx->dsel_bits + (size_t)first * 2 * W, (size_t)count * 2 * W * 8,
                       cudaMemcpyDeviceToHost, ctx->stream));
  if (owner)
    CK(cudaMemcpyAsync(owner, ctx->dsel_owner + first, (size_t)count * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (xam) CK(cudaMemcpyAsync(xam, ctx->dsel_xam + first, (size_t)count * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (evp)
    CK(cudaMemcpyAsync(evp, ctx->dsel_evp + (size_t)first * mt, (size_t)count * mt * 8,
                       cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return CIPSI_OK;
}

int cipsi_selection_get(cipsi_ctx* ctx, int64_t first, int64_t count, int32_t* nec, int32_t* holes,
                        int32_t* parts, double* xam, double* evp, int32_t* owner) {
  if (!ctx) return CIPSI_ERR_ARG;
  const int W = ctx->W, n = ctx->d.norb, noca = ctx->d.noca;
  std::vector<uint64_t> bits((size_t)std::max<int64_t>(count, 0) * 2 * W);
  int rc = cipsi_selection_raw(ctx, first, count, bits.data(), owner, xam, evp);
  if (rc) return rc;
  for (int64_t i = 0; i < count; ++i) {
    int nh = 0, np = 0;
    int32_t* h = holes ? holes + i * 8 : nullptr;
    int32_t* pp = parts ? parts + i * 8 : nullptr;
    for (int q = 0; q < 8; ++q) {
      if (h) h[q] = 0;
      if (pp) pp[q] = 0;
    }
    for (int s = 0; s < 2; ++s)
      for (int w = 0; w < W; ++w) {
        const uint64_t word = bits[(size_t)i * 2 * W + s * W + w];
        const int lo = w * 64;
        const int nref = std::min(std::max(noca - lo, 0), 64);
        const uint64_t ref = nref >= 64 ? ~0ull : ((1ull << nref) - 1ull);
        uint64_t hm = ref & ~word, pm = word & ~ref;
        while (hm) {
          const int b = __builtin_ctzll(hm);
          hm &= hm - 1;
          if (h && nh < 8) h[nh] = lo + b + 1 + s * n;
          ++nh;
        }
        while (pm) {
          const int b = __builtin_ctzll(pm);
          pm &= pm - 1;
          if (pp && np < 8) pp[np] = lo + b + 1 + s * n;
          ++np;
        }
      }
    if (nh > 8) return fail(ctx, CIPSI_ERR_OVERFLOW, "selected determinant with excitation degree > 8");
    if (nec) nec[i] = nh;
  }
  return CIPSI_OK;
}


// ------------------------------------------------- run without allocation
// cipsi_run_pt2_static runs k_pt2 + k_reduce with every per-run buffer taken
// from one file-scope device array instead of cudaMalloc'd context buffers.
// Layout of the array (each region 256-byte aligned): counters + dpivot +
// histogram counts | histogram sums | reduced sums | work counter |
// generator list | generator masks | work units | per-unit partial sums |
// per-block neighbour scratch (nb_j, nb_emask, lr_idx).  The generator and
// unit lists are staged in file-scope host arrays of fixed size.

}  // extern "C"

namespace {

constexpr size_t kStaticScratchBytes = (size_t)32 << 20;  // 32 MiB
constexpr int kStaticMaxUnits = 1 << 18;
constexpr int kStaticMaxGens = 1 << 17;
constexpr int kStaticMaxDevices = 64;

static __device__ __align__(256) unsigned char g_pt2_scratch[kStaticScratchBytes];

// host staging of the generator and unit lists (copied to the device array)
static int32_t g_static_gens[kStaticMaxGens];
static uint8_t g_static_gmask[kStaticMaxGens];
static int32_t g_static_units[3 * kStaticMaxUnits];

// device address of g_pt2_scratch, looked up once per device
static unsigned char* g_static_ptr[kStaticMaxDevices];
static bool g_static_ready[kStaticMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int cipsi_run_pt2_static(cipsi_ctx* ctx, const cipsi_opts* o, cipsi_result* r) {
  if (!ctx || !o || !r) return CIPSI_ERR_ARG;
  if (!ctx->have_int || !ctx->have_space || !ctx->have_roots)
    return fail(ctx, CIPSI_ERR_STATE, "run before set_integrals / set_space / set_roots");
  if (ctx->pending)
    return fail(ctx, CIPSI_ERR_STATE, "an asynchronous run is pending: fetch its result first");
  if (o->nclass < 2 || o->nclass > kNClass) return fail(ctx, CIPSI_ERR_ARG, "nclass must be in [2, 10]");
  for (int i = 0; i + 1 < o->nclass; ++i)
    if (!(o->aval[i] >= 0.0) || (i > 0 && !(o->aval[i] > o->aval[i - 1])))
      return fail(ctx, CIPSI_ERR_ARG, "aval must be non-negative and increasing");
  if (ctx->device < 0 || ctx->device >= kStaticMaxDevices)
    return fail(ctx, CIPSI_ERR_ARG, "device ordinal out of range for the static scratch table");
  CK(cudaSetDevice(ctx->device));
  // set-up, once per device, with that device current
  if (!g_static_ready[ctx->device]) {
    void* ptr = nullptr;
    CK(cudaGetSymbolAddress(&ptr, g_pt2_scratch));
    g_static_ptr[ctx->device] = static_cast<unsigned char*>(ptr);
    g_static_ready[ctx->device] = true;
  }
  unsigned char* base = g_static_ptr[ctx->device];
  const int ncf = ctx->d.ncf, W = ctx->W, mt = ctx->d.metat;

  // generators and their allowed rank changes (pertu.f:52-61, igene.f:34-35,
  // 89-90, 199-200, 296-298; same rules as cipsi_run_pt2_async)
  bool yd = false, ym = false, yf = false;
  int maxrank = 0;
  for (int k = 0; k < ncf; ++k) {
    if (ctx->rank[k] == 1) ym = true;
    if (ctx->rank[k] == 0) yd = true;
    if (ctx->rank[k] == 2) yf = true;
    maxrank = std::max(maxrank, ctx->rank[k]);
  }
  if (ym) yf = true;
  const bool pertu_ref = yf && !yd && ctx->d.isym == 1;
  const bool pertu_mono = yf && ym;
  int ngen = 0;
  auto too_many_gens = [&]() {
    return fail(ctx, CIPSI_ERR_OVERFLOW,
                "cipsi_run_pt2_static: more than " + std::to_string(kStaticMaxGens) + " generators");
  };
  if (o->run_pertu && (pertu_ref || pertu_mono)) {
    g_static_gens[ngen] = -1;
    g_static_gmask[ngen++] = 0;
  }
  for (int k = 0; k < ncf; ++k) {
    if (!ctx->ygen[k] || ctx->ysaut[k]) continue;
    if (o->gen_mask && !o->gen_mask[k]) continue;
    const int nec = ctx->rank[k];
    uint8_t m = 1u << 4;
    if (!((nec == 0 && ym) || (nec == 1 && yd))) {
      m |= 1u << 3;
      const bool stop1 = nec < 1 || (ym && nec == 1) || (nec == 2 && yd);
      if (!stop1) {
        m |= 1u << 2;
        if (!((nec == 3 && yd) || (nec == 2 && ym))) {
          m |= 1u << 1;
          if (!((nec == 2 && (yd || yf)) || (nec == 3 && ym) || (nec == 4 && yd))) m |= 1u << 0;
        }
      }
    }
    if (ngen == kStaticMaxGens) return too_many_gens();
    g_static_gens[ngen] = k;
    g_static_gmask[ngen++] = m;
  }

  // work units in the order of cipsi_run_pt2_async: generators by rank
  // (pertu block first), each split into chunks of at most 6 allowed R blocks
  constexpr int kRChunk = 6;
  constexpr int kPertuChunk = 128;
  const int n = ctx->d.norb, noca = ctx->d.noca, nel = 2 * noca;
  const int nR = nel + nel * (nel - 1) / 2;
  int nunits = 0;
  int32_t* ug = g_static_units;
  int32_t* ur0 = g_static_units + kStaticMaxUnits;
  int32_t* ur1 = g_static_units + 2 * kStaticMaxUnits;
  auto push_unit = [&](int g, int a, int b) {
    if (nunits == kStaticMaxUnits) return false;
    ug[nunits] = g;
    ur0[nunits] = a;
    ur1[nunits] = b;
    ++nunits;
    return true;
  };
  auto too_many_units = [&]() {
    return fail(ctx, CIPSI_ERR_OVERFLOW,
                "cipsi_run_pt2_static: more than " + std::to_string(kStaticMaxUnits) + " work units");
  };
  int hfe[2 * 128];
  for (int rk = -1; rk <= maxrank; ++rk) {
    for (int g = 0; g < ngen; ++g) {
      const int k = g_static_gens[g];
      if ((k < 0 ? -1 : ctx->rank[k]) != rk) continue;
      if (k < 0) {
        const int ntot = (pertu_ref ? 1 : 0) + (pertu_mono ? 2 * noca * (n - noca) : 0);
        for (int t = 0; t < ntot; t += kPertuChunk)
          if (!push_unit(g, t, std::min(ntot, t + kPertuChunk))) return too_many_units();
        continue;
      }
      int ne = 0;
      for (int sp = 0; sp < 2; ++sp)
        for (int orb = 0; orb < n; ++orb)
          if ((ctx->Sbits[(size_t)k * 2 * W + sp * W + (orb >> 6)] >> (orb & 63)) & 1ull)
            hfe[ne++] = orb < noca;
      const uint8_t m = g_static_gmask[g];
      int cnt = 0, start = -1;
      for (int rb = 0; rb < nR; ++rb) {
        int hfR, nRr;
        if (rb < nel) {
          hfR = hfe[rb];
          nRr = 1;
        } else {
          int t = rb - nel, e1 = 0;
          while (t >= nel - 1 - e1) {
            t -= nel - 1 - e1;
            ++e1;
          }
          hfR = hfe[e1] + hfe[e1 + 1 + t];
          nRr = 2;
        }
        bool ok = false;
        for (int aV = 0; aV <= nRr; ++aV)
          if (m & (1u << (hfR + aV - nRr + 2))) ok = true;
        if (!ok) continue;
        if (start < 0) start = rb;
        if (++cnt == kRChunk) {
          if (!push_unit(g, start, rb + 1)) return too_many_units();
          cnt = 0;
          start = -1;
        }
      }
      if (start >= 0 && !push_unit(g, start, nR)) return too_many_units();
    }
  }

  // launch shape as in cipsi_run_pt2_async, then fewer blocks if the
  // per-block neighbour scratch would not fit in the array
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int R = mt <= 1 ? 1 : mt <= 2 ? 2 : mt <= 4 ? 4 : 8;
  const size_t per_entry = (size_t)2 * W * 8 + 4;
  const size_t qbytes = (size_t)(kThreads / 32) * queue_bytes(W, R);
  const size_t smem_budget = (size_t)200 * 1024 - qbytes;
  const int lr_cap = (int)std::min<size_t>((size_t)ncf, smem_budget / per_entry);
  const size_t smem = (((size_t)lr_cap * per_entry + 15) & ~(size_t)15) + qbytes + 16;
  const int blocks_per_sm = smem <= 95 * 1024 ? 2 : 1;
  const size_t nq = (size_t)5 * mt;
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  const size_t off_counters = 0;
  const size_t off_tab = align256(off_counters + ncount * sizeof(unsigned long long));
  const size_t off_red = align256(off_tab + 2 * kNClass * kMaxRoots * sizeof(double));
  const size_t off_work = align256(off_red + 5 * kMaxRoots * sizeof(double));
  const size_t off_gens = align256(off_work + sizeof(int));
  const size_t off_gmask = align256(off_gens + (size_t)std::max(ngen, 1) * sizeof(int32_t));
  const size_t off_units = align256(off_gmask + (size_t)std::max(ngen, 1));
  const size_t off_part = align256(off_units + (size_t)3 * std::max(nunits, 1) * sizeof(int32_t));
  const size_t off_nb = align256(off_part + (size_t)std::max(nunits, 1) * nq * sizeof(double));
  const size_t per_block = 3 * align256((size_t)ncf * sizeof(uint64_t));
  int grid = std::max(1, std::min(nunits, dev_sms * blocks_per_sm));
  if (off_nb + per_block > kStaticScratchBytes)
    return fail(ctx, CIPSI_ERR_OVERFLOW,
                "cipsi_run_pt2_static: the run needs " + std::to_string(off_nb + per_block) +
                    " bytes of scratch, more than the static " + std::to_string(kStaticScratchBytes) +
                    " (ncf = " + std::to_string(ncf) + ", work units = " + std::to_string(nunits) +
                    "); use cipsi_run_pt2");
  grid = (int)std::min<size_t>((size_t)grid, (kStaticScratchBytes - off_nb) / per_block);
  const size_t nb_stride = align256((size_t)ncf * sizeof(uint64_t));
  unsigned char* nb0 = base + off_nb;

  // zero what the kernels accumulate into; upload the lists
  CK(cudaMemsetAsync(base, 0, off_gens, ctx->stream));
  CK(cudaMemsetAsync(base + off_part, 0, (size_t)std::max(nunits, 1) * nq * sizeof(double), ctx->stream));
  if (ngen) {
    CK(cudaMemcpyAsync(base + off_gens, g_static_gens, (size_t)ngen * sizeof(int32_t),
                       cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(base + off_gmask, g_static_gmask, (size_t)ngen, cudaMemcpyHostToDevice, ctx->stream));
  }
  int32_t* dunits = reinterpret_cast<int32_t*>(base + off_units);
  if (nunits) {
    CK(cudaMemcpyAsync(dunits, ug, (size_t)nunits * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(dunits + nunits, ur0, (size_t)nunits * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(dunits + 2 * nunits, ur1, (size_t)nunits * sizeof(int32_t), cudaMemcpyHostToDevice,
                       ctx->stream));
  }

  Params p{};
  p.norb = ctx->d.norb;
  p.noca = ctx->d.noca;
  p.nel = nel;
  p.ncf = ncf;
  p.metat = mt;
  p.nsym = ctx->d.nsym;
  p.isym = ctx->d.isym;
  p.ngen = ngen;
  p.gens = reinterpret_cast<const int32_t*>(base + off_gens);
  p.gen_dmask = base + off_gmask;
  p.nunits = nunits;
  p.unit_g = dunits;
  p.unit_r0 = dunits + nunits;
  p.unit_r1 = dunits + 2 * nunits;
  p.S = ctx->dS;
  p.ygen = ctx->dygen;
  p.nesp = ctx->dnesp;
  p.yef = ctx->dyef;
  p.c = ctx->dc;
  p.eri = ctx->deri;
  p.pairtab = ctx->dpairtab;
  p.ntttt = ctx->dntttt;
  p.F = ctx->dF;
  p.J = ctx->dJ;
  p.K = ctx->dK;
  p.fmpb = ctx->dfmpb;
  p.orbsym = ctx->dorbsym;
  for (int i = 0; i < ctx->d.nsym; ++i)
    for (int j = 0; j < ctx->d.nsym; ++j) p.its[i][j] = ctx->its[(size_t)j * ctx->d.nsym + i] - 1;
  for (int m = 0; m < mt; ++m) {
    p.e[m] = ctx->e[m];
    p.eb[m] = ctx->eb[m];
    p.emp[m] = ctx->emp[m];
    p.teste[m] = ctx->teste[m];
    p.taum[m] = ctx->taum[m];
  }
  p.yen = o->yen;
  p.ysele = o->ysele;
  p.ymoyen = o->ymoyen;
  p.ywdeg = o->ywdeg;
  p.symvar = o->sym_variant;
  p.nclass = o->nclass;
  p.tau = o->tau;
  p.teseff = o->teseff;
  for (int i = 0; i < kNClass; ++i) {
    p.aval[i] = o->aval[i];
    std::memcpy(&p.aval_bits[i], &o->aval[i], 8);
  }
  p.pertu_ref = pertu_ref ? 1 : 0;
  p.pertu_mono = pertu_mono ? 1 : 0;
  // nb_j, nb_emask, lr_idx: grid x ncf entries each (k_pt2 indexes block b at
  // b * ncf), in three regions of grid * nb_stride >= grid * ncf * 8 bytes
  p.nb_j = reinterpret_cast<int32_t*>(nb0);
  p.nb_emask = reinterpret_cast<uint64_t*>(nb0 + (size_t)grid * nb_stride);
  p.lr_idx = reinterpret_cast<int32_t*>(nb0 + (size_t)2 * grid * nb_stride);
  p.lr_cap = lr_cap;
  p.gen_part = reinterpret_cast<double*>(base + off_part);
  unsigned long long* dcounters = reinterpret_cast<unsigned long long*>(base + off_counters);
  p.counters = dcounters;
  p.dpivot_bits = dcounters + C_NCOUNTERS;
  p.hist_nom = dcounters + C_NCOUNTERS + 1;
  p.hist_nam = dcounters + C_NCOUNTERS + 1 + kNClass;
  p.hist_tab = reinterpret_cast<double*>(base + off_tab);
  // no record storage: selected perturbers are counted only
  p.sel_bits = nullptr;
  p.sel_owner = nullptr;
  p.sel_xam = nullptr;
  p.sel_evp = nullptr;
  p.sel_cap = 0;
  p.work = reinterpret_cast<int*>(base + off_work);
  double* dred = reinterpret_cast<double*>(base + off_red);

  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (nunits > 0) {
    cudaError_t e;
    if (W == 1) {
      e = R == 1 ? launch_pt2<1, 1>(p, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<1, 2>(p, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<1, 4>(p, grid, smem, ctx->stream)
                 : launch_pt2<1, 8>(p, grid, smem, ctx->stream);
    } else {
      e = R == 1 ? launch_pt2<2, 1>(p, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<2, 2>(p, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<2, 4>(p, grid, smem, ctx->stream)
                 : launch_pt2<2, 8>(p, grid, smem, ctx->stream);
    }
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_pt2 launch: ") + cudaGetErrorString(e));
    k_reduce<<<1, 64, 0, ctx->stream>>>(p.gen_part, nunits, (int)nq, dred);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));

  // results (same fields as cipsi_fetch_result; no records are kept)
  double red[5 * kMaxRoots];
  unsigned long long cnt[C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots];
  double tab[2 * kNClass * kMaxRoots];
  CK(cudaMemcpy(red, dred, nq * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(cnt, dcounters, ncount * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(tab, p.hist_tab, 2 * kNClass * kMaxRoots * sizeof(double), cudaMemcpyDeviceToHost));
  memset(r, 0, sizeof(*r));
  for (int m = 0; m < mt; ++m) {
    r->e2mp[m] = red[0 * mt + m];
    r->e2vp[m] = red[1 * mt + m];
    r->e2b[m] = red[2 * mt + m];
    r->psimp[m] = red[3 * mt + m];
    r->psivp[m] = red[4 * mt + m];
  }
  r->ietat = (int64_t)cnt[C_IETAT];
  r->n_processed = (int64_t)cnt[C_NPROC];
  r->n_candidates = (int64_t)cnt[C_NCAND];
  r->n_compares = (int64_t)cnt[C_NCMP];
  r->n_pairs_1 = (int64_t)cnt[C_NP1];
  r->n_pairs_2 = (int64_t)cnt[C_NP2];
  {
    const unsigned long long b = cnt[C_NCOUNTERS];
    double dp;
    memcpy(&dp, &b, 8);
    r->dpivot = dp;
  }
  const int nc = o->nclass;
  for (int i = 0; i < nc; ++i) r->nom[i] = (int64_t)cnt[C_NCOUNTERS + 1 + i];
  for (int c = 0; c < nc; ++c)
    for (int m = 0; m < mt; ++m) {
      r->nam[c * kMaxRoots + m] = (int64_t)cnt[C_NCOUNTERS + 1 + kNClass + c * mt + m];
      r->tabmp[c * kMaxRoots + m] = tab[c * mt + m];
      r->tabvp[c * kMaxRoots + m] = tab[nc * mt + c * mt + m];
    }
  const double avg_rank = 4.0;
  r->alg_bytes = (int64_t)(cnt[C_NP2] * (8.0 * mt + 2 * 4.0 + 8.0) +
                           cnt[C_NP1] * (8.0 * mt + 8.0 + 2.0 * avg_rank * 2 * 4.0) +
                           cnt[C_NPROC] * (8.0 * avg_rank + 8.0 * (avg_rank + avg_rank * avg_rank) + 8.0 * mt));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  r->kernel_ms = ms;
  r->n_selected = (int64_t)cnt[C_NSEL];
  return CIPSI_OK;
}

}  // extern "C"
