#pragma once
// pt2_kernel.cuh -- the perturbation / selection kernel k_pt2 of the GB300
// engine (the work of cip/pertu.f + cip/diexcit.f); included by pt2_w1.cu and
// pt2_w2.cu, which instantiate it for 1 and 2 words per spin string.
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

#include <algorithm>
#include <cmath>

#include "pt2_common.cuh"

namespace cipsi_dev {
namespace {

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

// Word updates and half selections of the small bitstring arrays with
// compile-time indices only: a run-time index into a local array makes the
// compiler place it in local memory (stack), one of the kernel's largest
// traffic sources.
template <int N>
__device__ __forceinline__ void or_word(uint64_t* x, int idx, uint64_t m) {
#pragma unroll
  for (int q = 0; q < N; ++q) x[q] |= (q == idx) ? m : 0ull;
}
template <int N>
__device__ __forceinline__ void clear_word(uint64_t* x, int idx, uint64_t m) {
#pragma unroll
  for (int q = 0; q < N; ++q) x[q] &= (q == idx) ? ~m : ~0ull;
}
template <int N>
__device__ __forceinline__ uint64_t get_word(const uint64_t* x, int idx) {
  uint64_t r = 0ull;
#pragma unroll
  for (int q = 0; q < N; ++q) r = (q == idx) ? x[q] : r;
  return r;
}
// out[w] = x[s * W + w] (s = 0: alpha words, 1: beta words)
template <int W>
__device__ __forceinline__ void pick_spin(const uint64_t* x, int s, uint64_t* out) {
#pragma unroll
  for (int w = 0; w < W; ++w) out[w] = s ? x[W + w] : x[w];
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
  if (p.eri64) return __ldg(&p.eri64[idx]);
  return (double)__ldg(&p.eri[idx]);
}

// adjoint of ai(): add w to dE/d(ij|kl) at its packed position (nothing
// when the irreps differ: the integral is zero by symmetry)
__device__ __forceinline__ void ai_adj(const Params& p, int i, int j, int k, int l, double w) {
  const int pij = __ldg(&p.pairtab[i * p.norb + j]);
  const int pkl = __ldg(&p.pairtab[k * p.norb + l]);
  const int s1 = pij >> 24, s2 = pkl >> 24;
  if (s1 != s2) return;
  const long long a = pij & 0xFFFFFF, b = pkl & 0xFFFFFF;
  const long long lo = a < b ? a : b, hi = a < b ? b : a;
  const long long idx = lo + hi * (hi - 1) / 2 + __ldg(&p.ntttt[s1]) - 2;
  atomicAdd(&p.g_eri[idx], w);
}

// Compact L_R entry of a determinant j for a block of removed electrons R
// (K' = k - R): bits 0-31 the spin orbitals of E = j \ K' (code orb +
// spin * norb, one byte each; |E| = |R| + m <= 4, unused bytes repeat the
// first code), bits 32-33 m = |K' \ j|, bits 34-63 the index j.
__device__ __forceinline__ uint64_t lr_entry(uint32_t ebytes, int ne, int m, int j) {
  const uint32_t first = ebytes & 0xFFu;
  for (int q = ne; q < 4; ++q) ebytes |= first << (8 * q);
  return (uint64_t)ebytes | ((uint64_t)m << 32) | ((uint64_t)j << 34);
}
__device__ __forceinline__ int lr_entry_j(uint64_t e) { return (int)(e >> 34); }
// true when some byte of x equals the byte repeated in c4 (a zero byte of
// x ^ c4; the borrow test flags a byte only if it or a lower byte is zero)
__device__ __forceinline__ bool has_byte(uint32_t x, uint32_t c4) {
  const uint32_t v = x ^ c4;
  return ((v - 0x01010101u) & ~v & 0x80808080u) != 0u;
}
// bit difference |I xor j| = 2 (m + |A \ E|) of I = K' + A, A = {c1[, c2]}
// (c1x4, c2x4: the codes repeated in four bytes)
__device__ __forceinline__ int lr_diff(uint64_t e, uint32_t c1x4, uint32_t c2x4, bool two) {
  const uint32_t E = (uint32_t)e;
  int d = (int)((e >> 32) & 3u);
  d += has_byte(E, c1x4) ? 0 : 1;
  if (two) d += has_byte(E, c2x4) ? 0 : 1;
  return 2 * d;
}

// <I|H|J> for degree 1 or 2, canonical phases.  u = I bits, v = J bits
// (alpha words then beta words).  rankI / rankJ: excitation degree relative
// to the reference determinant; the one-difference element sums over the
// holes and particles of the more excited determinant as cip/hntd.f does.
template <int W>
__device__ __forceinline__ double hmat(const Params& p, const uint64_t* u, const uint64_t* v, int rankI, int rankJ,
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
    uint64_t rs[W], as[W], vs[W];
    pick_spin<W>(remv, s, rs);
    pick_spin<W>(addv, s, as);
    pick_spin<W>(v, s, vs);
    const int pp = first_bit<W>(rs);
    const int qq = first_bit<W>(as);
    const int lo = pp < qq ? pp : qq, hi = pp < qq ? qq : pp;
    const int sign = (popc_between<W>(vs, lo, hi) & 1) ? -1 : 1;
    double val = __ldg(&p.F[tri(pp, qq)]);
    const bool dI = rankI > rankJ;
    uint64_t D[2 * W];
#pragma unroll
    for (int q = 0; q < 2 * W; ++q) D[q] = dI ? u[q] : v[q];
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
  uint64_t rm[W], ad[W], mid[W];
  pick_spin<W>(remv, s, rm);
  pick_spin<W>(addv, s, ad);
  pick_spin<W>(v, s, mid);
  const int p1 = first_bit<W>(rm), p2 = last_bit<W>(rm);
  const int q1 = first_bit<W>(ad), q2 = last_bit<W>(ad);
  const int s1 = popc_between<W>(mid, min(p1, q1), max(p1, q1));
  clear_word<W>(mid, p1 >> 6, 1ull << (p1 & 63));
  or_word<W>(mid, q1 >> 6, 1ull << (q1 & 63));
  const int s2 = popc_between<W>(mid, min(p2, q2), max(p2, q2));
  const double val = ai(p, p1, q1, p2, q2) - ai(p, p1, q2, p2, q1);
  return ((s1 + s2) & 1) ? -val : val;
}

// Adjoint of hmat: adds w * d<I|H|J>/d(integral) to the gradients (F
// off-diagonal terms to g_F, (pq|rs) to g_eri), same cases and phases.
// with_eri false: the F term only (one-electron adjoint; two-difference
// elements then add nothing).
template <int W>
__device__ void hmat_adj(const Params& p, const uint64_t* u, const uint64_t* v, int rankI, int rankJ,
                         const uint64_t* hf, double w, bool with_eri) {
  if (w == 0.0) return;
  uint64_t remv[2 * W], addv[2 * W];
  int nrem[2] = {0, 0};
#pragma unroll
  for (int q = 0; q < 2 * W; ++q) {
    const uint64_t x = u[q] ^ v[q];
    remv[q] = x & v[q];
    addv[q] = x & u[q];
    nrem[q / W] += __popcll(remv[q]);
  }
  if (nrem[0] + nrem[1] == 1) {
    const int s = nrem[0] ? 0 : 1;
    uint64_t rs[W], as[W], vs[W];
    pick_spin<W>(remv, s, rs);
    pick_spin<W>(addv, s, as);
    pick_spin<W>(v, s, vs);
    const int pp = first_bit<W>(rs);
    const int qq = first_bit<W>(as);
    const int lo = pp < qq ? pp : qq, hi = pp < qq ? qq : pp;
    const double sw = (popc_between<W>(vs, lo, hi) & 1) ? -w : w;
    atomicAdd(&p.g_F[tri(pp, qq)], sw);
    if (!with_eri) return;
    const bool dI = rankI > rankJ;
    uint64_t D[2 * W];
#pragma unroll
    for (int q = 0; q < 2 * W; ++q) D[q] = dI ? u[q] : v[q];
#pragma unroll
    for (int sp = 0; sp < 2; ++sp) {
#pragma unroll
      for (int ww = 0; ww < W; ++ww) {
        uint64_t h = hf[sp * W + ww] & ~D[sp * W + ww];
        while (h) {
          const int r = ww * 64 + __ffsll((long long)h) - 1;
          h &= h - 1;
          ai_adj(p, pp, qq, r, r, -sw);
          if (sp == s) ai_adj(p, pp, r, qq, r, sw);
        }
        uint64_t t = D[sp * W + ww] & ~hf[sp * W + ww];
        while (t) {
          const int r = ww * 64 + __ffsll((long long)t) - 1;
          t &= t - 1;
          ai_adj(p, pp, qq, r, r, sw);
          if (sp == s) ai_adj(p, pp, r, qq, r, -sw);
        }
      }
    }
    return;
  }
  if (!with_eri) return;
  if (nrem[0] == 1 && nrem[1] == 1) {
    const int pa = first_bit<W>(remv), qa = first_bit<W>(addv);
    const int pb = first_bit<W>(remv + W), qb = first_bit<W>(addv + W);
    const int sa = popc_between<W>(v, min(pa, qa), max(pa, qa));
    const int sb = popc_between<W>(v + W, min(pb, qb), max(pb, qb));
    ai_adj(p, pa, qa, pb, qb, ((sa + sb) & 1) ? -w : w);
    return;
  }
  const int s = nrem[0] == 2 ? 0 : 1;
  uint64_t rm[W], ad[W], mid[W];
  pick_spin<W>(remv, s, rm);
  pick_spin<W>(addv, s, ad);
  pick_spin<W>(v, s, mid);
  const int p1 = first_bit<W>(rm), p2 = last_bit<W>(rm);
  const int q1 = first_bit<W>(ad), q2 = last_bit<W>(ad);
  const int s1 = popc_between<W>(mid, min(p1, q1), max(p1, q1));
  clear_word<W>(mid, p1 >> 6, 1ull << (p1 & 63));
  or_word<W>(mid, q1 >> 6, 1ull << (q1 & 63));
  const int s2 = popc_between<W>(mid, min(p2, q2), max(p2, q2));
  const double sw = ((s1 + s2) & 1) ? -w : w;
  ai_adj(p, p1, q1, p2, q2, sw);
  ai_adj(p, p1, q2, p2, q1, -sw);
}

// E2 sums of one thread, Kahan-compensated, and its counters
template <int R>
struct Acc {
  double e2mp[R], cmp[R], e2vp[R], cvp[R], e2b[R], cb[R], psimp[R], psivp[R];
  unsigned long long ietat, nproc;
  double dpivot;
  __device__ void zero() {
#pragma unroll
    for (int m = 0; m < R; ++m) {
      e2mp[m] = cmp[m] = e2vp[m] = cvp[m] = e2b[m] = cb[m] = psimp[m] = psivp[m] = 0.0;
    }
    ietat = nproc = 0ull;
    dpivot = 0.0;
  }
};

// Per-perturber derivative factors of the E2 sums (pert1.f:151-191):
//   t_mp = b^2/(emp - hmp), t_vp = b^2/(e - hdig), t_b = b^2/(eb - hdig),
// each weighted by wgt; gb[m] = dE/db_m, gh = dE/dhdig, gm = dE/dhmp, and
// the root-energy gradients accumulated into gr[3][R] (e, eb, emp).  The
// terms themselves go to acc (the forward's E2 sums and norms, from the same
// quotients b/d).
template <int R>
__device__ __forceinline__ void adj_factors(const Params& p, const double* bc, double hmpi, double hvpi,
                                            double wgt, double* gb, double& gh, double& gm,
                                            double (*gr)[R], Acc<R>& acc) {
  gh = 0.0;
  gm = 0.0;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    gb[m] = 0.0;
    if (m >= p.metat) continue;
    const double b = bc[m];
    const double dmp = p.emp[m] - hmpi;
    double qmp, qvp = 0.0, qb = 0.0;
    if (p.yen) {
      // one division for the three quotients, as in the forward epilogue
      const double dvp = p.e[m] - hvpi, db = p.eb[m] - hvpi;
      const double pvb = dvp * db, prod = dmp * pvb;
      if (((unsigned)(__double_as_longlong(prod) >> 52) & 0x7FFu) - 93u < 1860u) {
        const double br = b / prod;
        qmp = br * pvb;
        qvp = br * (dmp * db);
        qb = br * (dmp * dvp);
      } else {
        qmp = b / dmp;
        qvp = b / dvp;
        qb = b / db;
      }
    } else {
      qmp = b / dmp;
    }
    const double tmp = wgt * p.seed_mp[m] * qmp * qmp;
    gb[m] = wgt * p.seed_mp[m] * (2.0 * qmp);
    gm += tmp;
    gr[2][m] -= tmp;
    kahan_add(acc.e2mp[m], acc.cmp[m], (b * qmp) * wgt);
    acc.psimp[m] = fma(qmp * qmp, wgt, acc.psimp[m]);
    if (p.yen) {
      const double tv = wgt * p.seed_vp[m] * qvp * qvp;
      const double tb = wgt * p.seed_b[m] * qb * qb;
      gb[m] += wgt * (p.seed_vp[m] * (2.0 * qvp) + p.seed_b[m] * (2.0 * qb));
      gh += tv + tb;
      gr[0][m] -= tv;
      gr[1][m] -= tb;
      kahan_add(acc.e2vp[m], acc.cvp[m], (b * qvp) * wgt);
      kahan_add(acc.e2b[m], acc.cb[m], (b * qb) * wgt);
      acc.psivp[m] = fma(qvp * qvp, wgt, acc.psivp[m]);
    }
  }
}

// adjoint of diag_terms: dE/dhmp = gm and dE/dhdig = gh spread over fmpb,
// F, J, K of the holes and particles of I (slice of this block)
template <int W>
__device__ void diag_terms_adj(const Params& p, const uint64_t* u, const uint64_t* hf, double gh,
                               double gm, double* sl) {
  int hs[24], ps[24];
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
  const int n = p.norb, nt = n * (n + 1) / 2;
  double* sF = sl;
  double* sJ = sl + nt;
  double* sK = sl + 2 * nt;
  double* sf = sl + 3 * nt;
  for (int i = 0; i < np; ++i) atomicAdd(&sf[ps[i]], gm);
  for (int i = 0; i < nh; ++i) atomicAdd(&sf[hs[i]], -gm);
  if (gh == 0.0) return;
  for (int i = 0; i < np; ++i) atomicAdd(&sF[tri(ps[i] % n, ps[i] % n)], gh);
  for (int i = 0; i < nh; ++i) atomicAdd(&sF[tri(hs[i] % n, hs[i] % n)], -gh);
  auto jk = [&](int a, int b, double c) {
    const int t = tri(a % n, b % n);
    atomicAdd(&sJ[t], c);
    if ((a / n) == (b / n)) atomicAdd(&sK[t], -c);
  };
  for (int i = 0; i < nh; ++i) jk(hs[i], hs[i], 0.5 * gh);
  for (int i = 0; i < np; ++i) jk(ps[i], ps[i], 0.5 * gh);
  for (int i = 0; i < nh; ++i)
    for (int j = i + 1; j < nh; ++j) jk(hs[i], hs[j], gh);
  for (int i = 0; i < np; ++i)
    for (int j = i + 1; j < np; ++j) jk(ps[i], ps[j], gh);
  for (int i = 0; i < nh; ++i)
    for (int j = 0; j < np; ++j) jk(hs[i], ps[j], -gh);
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

// Spin-flip weight fmul = (1/(lesp+1)) * (nespf+1) - 1 (pert1.f:150-164,
// diexcit.f:304-316), rounded step by step as the reference does (no fused
// multiply-add).  lesp is 0 or 1 for almost every perturber: those two
// reciprocals are exact constants, so the FP64 division is only taken for
// lesp >= 2.
__device__ __forceinline__ double spin_weight(int nespf, int lesp) {
  if (lesp == 0) return (double)nespf;  // 1 * (nespf + 1) - 1, exact
  const double inv = lesp == 1 ? 0.5 : 1.0 / (double)(lesp + 1);
  return __dsub_rn(__dmul_rn(inv, (double)(nespf + 1)), 1.0);
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


// Block-wide order-preserving two-way partition of [0, n): i with
// part(i) == 0 gets the slots 0..n0-1, i with part(i) == 1 the slots
// n0..n0+n1-1, each part in increasing i (deterministic, whatever the
// scheduling); part(i) < 0 drops i.  Each warp owns one
// contiguous chunk: it counts both parts, the warps' offsets come from one
// exchange in shared memory, and the warp emits its chunk again at those
// offsets.  Two block barriers whatever n.  Must be called by every thread
// of the block; part() is evaluated twice per index.
template <typename Part, typename Emit>
__device__ int2 ordered_partition2(int n, Part part, Emit emit, int* warp_tmp /* >= 2 * warps ints */) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int chunk = (((n + nw - 1) / nw) + 31) & ~31;
  const int lo = min(n, wid * chunk), hi = min(n, lo + chunk);
  int c0 = 0, c1 = 0;
  for (int base = lo; base < hi; base += 32) {
    const int i = base + lane;
    const int pt = i < hi ? part(i) : -1;
    c0 += __popc(__ballot_sync(kFull, pt == 0));
    c1 += __popc(__ballot_sync(kFull, pt == 1));
  }
  if (lane == 0) {
    warp_tmp[wid] = c0;
    warp_tmp[nw + wid] = c1;
  }
  __syncthreads();
  int o0 = 0, o1 = 0, n0 = 0, n1 = 0;
  for (int w = 0; w < nw; ++w) {
    const int a = warp_tmp[w], b = warp_tmp[nw + w];
    if (w < wid) {
      o0 += a;
      o1 += b;
    }
    n0 += a;
    n1 += b;
  }
  const unsigned below = (1u << lane) - 1u;
  for (int base = lo; base < hi; base += 32) {
    const int i = base + lane;
    const int pt = i < hi ? part(i) : -1;
    const unsigned m0 = __ballot_sync(kFull, pt == 0);
    const unsigned m1 = __ballot_sync(kFull, pt == 1);
    if (pt == 0) emit(o0 + __popc(m0 & below), i);
    if (pt == 1) emit(n0 + o1 + __popc(m1 & below), i);
    o0 += __popc(m0);
    o1 += __popc(m1);
  }
  __syncthreads();
  return make_int2(n0, n1);
}

// Counters of the candidate scan.  Kept apart from Acc: Acc is passed by
// reference to the out-of-line queue drain, so it lives in local memory,
// and these are incremented in the scan loop itself (registers).
struct ScanCounts {
  unsigned long long ncand, ncmp, np1, np2;
  __device__ void zero() { ncand = ncmp = np1 = np2 = 0ull; }
};

// One thread's histogram (cip/isto.f): class sums and counts, indexed by
// class at run time, so it lives in local memory (L1-resident); one FP64 add
// per contribution, no atomics; merged into the block's at kernel end.
template <int R>
struct HistPriv {
  double tab[kNClass][2][R];
  unsigned int nom[kNClass];  // per-thread counts stay far below 2^32
  unsigned int nam[kNClass][R];
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
                                 double hvpi, const double* bc, int slot /*in the work unit*/,
                                 double fmul, int nmul, bool ybis, bool is_pert1, Acc<R>& acc,
                                 HistPriv<R>& hp) {
  constexpr unsigned kFull = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  double xam = 0.0;
  bool ydeg = false;
  // weighted E2 terms per root: term * (1 + fmul), which is also what the
  // histogram (isto.f, fm = fmul + 1) and cipsym's unit-60 value
  // (cipsym/pert1.f:244, eivp * (fmul + 1)) use
  double vil[R], semp[R], sevp[R];
  // the reference adds each term and then term*fmul (spin-flip weight,
  // pert1.f:280-287); one compensated add of term*(1+fmul) is used here.
  // fmul = 0 whenever ybis is false, so wgt = fmul + 1 for every perturber.
  const double wgt = ybis ? 1.0 + fmul : 1.0;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    vil[m] = 0.0;
    semp[m] = sevp[m] = 0.0;
    if (!live || m >= p.metat) continue;
    const double bcalc = bc[m];
    const double dmp = p.emp[m] - hmpi;
    double eivp = 0.0, tvp = 0.0, cimp, xim, deno, eim;
    if (p.yen) {
      // the three denominators share one FP64 division (GB300's FP64 rate is
      // 1/64 of FP32): br = b/(dmp*dvp*db), b/dmp = dvp*db*br, etc.
      const double dvp = p.e[m] - hvpi;
      const double db = p.eb[m] - hvpi;
      const double pvb = dvp * db;
      const double prod = dmp * pvb;
      double civp, cib;
      // 1e-280 < |prod| < 1e280 tested on the exponent field (integer pipe):
      // binary exponent in [-930, 929]
      const unsigned pex = (unsigned)(__double_as_longlong(prod) >> 52) & 0x7FFu;
      if (pex - 93u < 1860u) {
        const double br = bcalc / prod;
        cimp = br * pvb;
        civp = br * (dmp * db);
        cib = br * (dmp * dvp);
      } else {  // a denominator at (or near) zero or huge: divide one by one
        cimp = bcalc / dmp;
        civp = bcalc / dvp;
        cib = bcalc / db;
      }
      eivp = bcalc * civp;
      tvp = eivp * wgt;
      kahan_add(acc.e2vp[m], acc.cvp[m], tvp);
      acc.psivp[m] = fma(civp * civp, wgt, acc.psivp[m]);
      kahan_add(acc.e2b[m], acc.cb[m], (bcalc * cib) * wgt);
      xim = p.ysele ? fabs(eivp) : fabs(civp);
      deno = dvp;
      eim = eivp;
    } else {
      cimp = bcalc / dmp;
    }
    const double eimp = bcalc * cimp;
    const double tmp = eimp * wgt;
    kahan_add(acc.e2mp[m], acc.cmp[m], tmp);
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
    semp[m] = tmp;
    sevp[m] = tvp;
  }
  if (live) {
    acc.ietat += (unsigned long long)(long long)(nmul + 1);
    acc.nproc += 1;
  }
  // histogram (cip/isto.f; pert1 calls it always, diexcit only if ymoyen)
  if (live && (is_pert1 || p.ymoyen) && xam >= p.teseff) {
    const int cls = hist_class(p, xam);
    hp.nom[cls] += (unsigned)(1 + nmul);
#pragma unroll
    for (int m = 0; m < R; ++m) {
      if (m >= p.metat || vil[m] < p.teseff) continue;
      hp.tab[cls][0][m] += semp[m];  // eimp * (fmul + 1)
      hp.tab[cls][1][m] += sevp[m];  // eivp * (fmul + 1)
      hp.nam[hist_class(p, vil[m])][m] += (unsigned)(1 + nmul);
    }
  }
  if (ydeg) xam = 1.0;
  // unit-60 record (pie.f): counted per warp; kept, when asked, at the
  // candidate's slot of this CTA's staging region (compacted in slot order
  // when the work unit is done, unit_compact)
  const bool sel = live && xam > p.tau && p.ymoyen;
  const unsigned sm = __ballot_sync(kFull, sel);
  if (sm && lane == 0) atomicAdd(&p.counters[C_NSEL], (unsigned long long)__popc(sm));
  if (sel && p.rec_mode && slot >= p.st_cap) atomicAdd(&p.counters[C_STAGE_OVF], 1ull);  // host sizing error
  if (sel && p.rec_mode && slot < p.st_cap) {
    const size_t s = (size_t)blockIdx.x * p.st_cap + slot;
#pragma unroll
    for (int q = 0; q < 2 * W; ++q) p.st_bits[s * 2 * W + q] = u[q];
    p.st_xam[s] = xam;
    // ENvp per root written by cipsym (cipsym/pert1.f:244): eivp*(fmul+1)
#pragma unroll
    for (int m = 0; m < R; ++m)
      if (m < p.metat) p.st_evp[s * p.metat + m] = p.symvar ? sevp[m] : 0.0;
    atomicOr(&p.st_mask[(size_t)blockIdx.x * (p.st_cap >> 5) + (slot >> 5)], 1u << (slot & 31));
  }
}

// End of a work unit (whole block): the staged records of its flagged
// slots go, in slot order, to one segment of the record pool, reserved with
// a single atomic; the unit table notes the segment.  The slot mask is
// cleared for the next unit.  Records beyond the pool's capacity are
// counted but not stored (the host sees pool_count > pool_cap).
template <int W>
__device__ __noinline__ void unit_compact(const Params& p, int unit, int nslots, int* tmp /* >= 32 ints */,
                             long long& sbase /* shared */) {
  constexpr unsigned kFull = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  __syncthreads();  // every warp's staging stores and mask bits are done
  const int nwords = (min(nslots, p.st_cap) + 31) >> 5;
  uint32_t* mask = p.st_mask + (size_t)blockIdx.x * (p.st_cap >> 5);
  const size_t st0 = (size_t)blockIdx.x * p.st_cap;
  // each thread owns a contiguous range of mask words
  const int per = (nwords + (int)blockDim.x - 1) / (int)blockDim.x;
  const int w0 = min(nwords, tid * per), w1 = min(nwords, w0 + per);
  int cnt = 0;
  for (int w = w0; w < w1; ++w) cnt += __popc(__ldcg(&mask[w]));
  // block exclusive scan of cnt (thread order = slot order)
  int incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) tmp[wid] = incl;
  __syncthreads();
  if (tid == 0) {
    int acc = 0;
    for (int w = 0; w < nw; ++w) {
      const int v = tmp[w];
      tmp[w] = acc;
      acc += v;
    }
    long long base = 0;
    if (acc) base = (long long)atomicAdd(p.pool_count, (unsigned long long)acc);
    p.unit_pool[unit] = base;
    p.unit_nsel[unit] = acc;
    sbase = base;
  }
  __syncthreads();
  long long pos = sbase + tmp[wid] + (incl - cnt);
  for (int w = w0; w < w1; ++w) {
    uint32_t m = __ldcg(&mask[w]);
    if (m) mask[w] = 0u;
    while (m) {
      const int b = __ffs(m) - 1;
      m &= m - 1u;
      if (pos < p.pool_cap) {
        const size_t s = st0 + (size_t)(w * 32 + b);
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) p.pool_bits[(size_t)pos * 2 * W + q] = __ldcg(&p.st_bits[s * 2 * W + q]);
        p.pool_xam[pos] = __ldcg(&p.st_xam[s]);
        for (int mm = 0; mm < p.metat; ++mm) p.pool_evp[(size_t)pos * p.metat + mm] = __ldcg(&p.st_evp[s * p.metat + mm]);
      }
      ++pos;
    }
  }
  __syncthreads();
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


// Enqueue the live lanes' perturbers (called by a whole warp); runs the
// epilogue on every full batch of 32.
template <int W, int R>
__device__ void enqueue_candidate(const Params& p, WarpQueue<W, R>& q, int& qn, bool live,
                                  const uint64_t* u, double hmpi, double hvpi, const double* bc,
                                  int slot, double fmul, int nmul, bool ybis, bool is_pert1,
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
    finish_candidate<W, R>(p, live, u, q.hmp[e], q.hvp[e], bc, q.slot[e], q.fmul[e], q.nmul[e],
                           (f & 1) != 0, (f & 2) != 0, acc, hp);
    __syncwarp();
    qn = base;
  }
}

template <int W, int R>
__device__ void enqueue_candidate(const Params& p, WarpQueue<W, R>& q, int& qn, bool live,
                                  const uint64_t* u, double hmpi, double hvpi, const double* bc,
                                  int slot, double fmul, int nmul, bool ybis, bool is_pert1,
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
    q.slot[e] = slot;
    q.flags[e] = (unsigned char)((ybis ? 1 : 0) | (is_pert1 ? 2 : 0));
  }
  qn += __popc(lm);
  __syncwarp();
  // the drain is out of line; calling it only with a full batch spares the
  // register saves of a call on every other candidate round
  if (qn >= 32) drain_queue<W, R>(p, q, qn, false, acc, hp);
}

// Block totals of the integer counters and the histogram into the
// geometry's global counters; then reset them for the next geometry.
template <int R>
__device__ void flush_totals(const Params& p, Acc<R>& acc, HistPriv<R>& hp, SmemHist& hist,
                             unsigned long long ncand, unsigned long long ncmp, unsigned long long np1,
                             unsigned long long np2) {
  const int tid = threadIdx.x;
  // block totals of the integer counters and the histogram
  __syncthreads();
  {
    unsigned long long v[8] = {acc.ietat, acc.nproc, 0ull, ncand, ncmp, np1, np2, 0ull};
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
    if (hp.nom[c]) atomicAdd(&hist.nom[c], (unsigned long long)hp.nom[c]);
    for (int m = 0; m < R && m < p.metat; ++m) {
      if (hp.tab[c][0][m] != 0.0) atomicAdd(&hist.tab[c * kMaxRoots + m], hp.tab[c][0][m]);
      if (hp.tab[c][1][m] != 0.0)
        atomicAdd(&hist.tab[kNClass * kMaxRoots + c * kMaxRoots + m], hp.tab[c][1][m]);
      if (hp.nam[c][m]) atomicAdd(&hist.nam[c * kMaxRoots + m], (unsigned long long)hp.nam[c][m]);
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
  __syncthreads();
  acc.ietat = acc.nproc = 0ull;
  acc.dpivot = 0.0;
  hp.zero();
  for (int i = tid; i < kNClass; i += blockDim.x) hist.nom[i] = 0;
  for (int i = tid; i < kNClass * kMaxRoots; i += blockDim.x) hist.nam[i] = 0;
  for (int i = tid; i < 2 * kNClass * kMaxRoots; i += blockDim.x) hist.tab[i] = 0.0;
  __syncthreads();
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
  long long unit_base;    // pool segment of the unit being compacted
};

template <int W, int R, bool B, bool ADJ>
__global__ void __launch_bounds__(kThreads, 2) k_pt2(Params p0, BatchArgs ba) {
  extern __shared__ __align__(16) unsigned char dyn[];
  // the current geometry's parameters, in shared memory (device functions
  // then read them through a shared-memory reference instead of a local
  // copy of the kernel argument)
  __shared__ Params sgeo;
  const Params& p = sgeo;
  __shared__ BlockShared sh;
  __shared__ SmemHist hist;
  __shared__ double red[5 * kMaxRoots * 32];
  __shared__ int ctmp[33];
  __shared__ int16_t wrow[(kThreads / 32) * kRowCap];
  __shared__ int hitl[kThreads * kHitCap];  // per-thread lists of scan hits

  const int tid = threadIdx.x;
  // shared L_R arrays (fast path)
  // (lr_cap is the same for every geometry of a batched launch)
  // L_R entries (compact form, lr_entry) up to lr_cap in shared memory; the
  // rest of a longer list stays in the block's global scratch
  uint64_t* lr_ent = reinterpret_cast<uint64_t*>(dyn);
  // per-warp epilogue queues, 16-byte aligned after the L_R entries
  const size_t qoff = (((size_t)p0.lr_cap * 8) + 15) & ~(size_t)15;
  WarpQueue<W, R>& wq = reinterpret_cast<WarpQueue<W, R>*>(dyn + qoff)[threadIdx.x >> 5];
  int qn = 0;

  for (int i = tid; i < kNClass; i += blockDim.x) hist.nom[i] = 0;
  for (int i = tid; i < kNClass * kMaxRoots; i += blockDim.x) hist.nam[i] = 0;
  for (int i = tid; i < 2 * kNClass * kMaxRoots; i += blockDim.x) hist.tab[i] = 0.0;

  // per-geometry state
  int32_t* my_nb_j = nullptr;
  uint64_t* my_nb_em = nullptr;
  uint64_t* my_lr_ent = nullptr;
  uint64_t hf[2 * W];
  int ncf = 0;
  auto geo_init = [&]() {
    my_nb_j = p.nb_j + (size_t)blockIdx.x * p.nb_stride;
    my_nb_em = p.nb_emask + (size_t)blockIdx.x * p.nb_stride;
    my_lr_ent = p.lr_ent + (size_t)blockIdx.x * p.nb_stride;
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const int lo = w * 64;
        const int n = min(max(p.noca - lo, 0), 64);
        hf[s * W + w] = (n >= 64) ? ~0ull : ((1ull << n) - 1ull);
      }
    ncf = p.ncf;
  };
  if (!B) {
    if (tid == 0) sgeo = p0;
    __syncthreads();
    geo_init();
  }
  int cur_geo = -1;

  Acc<R> acc;
  acc.zero();
  ScanCounts sc;
  sc.zero();
  HistPriv<R> hp;
  hp.zero();
  // adjoint: per-thread root-energy gradients and per-block accumulators of
  // dE/dhdig and dE/dhmp over one block of removed electrons (K' terms:
  // adj_sh[0..1]; per added spin orbital: adj_gv, adj_gf)
  __shared__ double adj_gv[ADJ ? 2 * kMaxOrb : 1], adj_gf[ADJ ? 2 * kMaxOrb : 1], adj_sh[2];
  double adjr[3][R];
  double adj_gK = 0.0, adj_gM = 0.0;
  double* adj_sl = nullptr;
  if (ADJ) {
#pragma unroll
    for (int m = 0; m < R; ++m) adjr[0][m] = adjr[1][m] = adjr[2][m] = 0.0;
    for (int i = tid; i < 2 * kMaxOrb; i += blockDim.x) adj_gv[i] = adj_gf[i] = 0.0;
    adj_sl = p0.g_slice + (size_t)blockIdx.x * p0.slice_stride;
  }

  for (;;) {
    __syncthreads();
    if (tid == 0) sh.gen = atomicAdd(B ? ba.work : p0.work, 1);
    __syncthreads();
    int unit = sh.gen;
    if (unit >= (B ? ba.nunits : p0.nunits)) break;
    if (B) {
      const int gi = ba.unit_geo[unit];
      if (gi != cur_geo) {
        if (cur_geo >= 0) {
          flush_totals<R>(p, acc, hp, hist, sc.ncand, sc.ncmp, sc.np1, sc.np2);
          sc.zero();
        }
        __syncthreads();
        const int* src = reinterpret_cast<const int*>(ba.geo + gi);
        int* dst = reinterpret_cast<int*>(&sgeo);
        for (int i = tid; i < (int)(sizeof(Params) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
        __syncthreads();
        cur_geo = gi;
        geo_init();
      }
      unit = ba.unit_local[unit];
    }
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
          clear_word<2 * W>(u, s * W + (o >> 6), 1ull << (o & 63));
          or_word<2 * W>(u, s * W + (vv >> 6), 1ull << (vv & 63));
        }
        double bc[R];
#pragma unroll
        for (int m = 0; m < R; ++m) bc[m] = 0.0;
        double hmpi = 0.0, hvpi = 0.0;
        if (live) {
          sc.ncand++;
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
            sc.ncmp++;
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
            if (kind == 1) sc.np1++; else sc.np2++;
            ++nint;
#pragma unroll
            for (int m = 0; m < R; ++m)
              if (m < p.metat) bc[m] += h * __ldg(&p.c[(size_t)j * p.metat + m]);
          }
          if (drop || nint == 0) live = false;
          if (live) diag_terms<W>(p, u, hf, hmpi, hvpi, p.yen != 0);
        }
        if (ADJ) {
          if (live) {
            double gb[R], gh, gm;
            adj_factors<R>(p, bc, hmpi, hvpi, 1.0, gb, gh, gm, adjr, acc);
            acc.ietat += 1;
            acc.nproc += 1;
            int rankI = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) rankI += __popcll(hf[q] & ~u[q]);
            for (int j = 0; j < ncf; ++j) {
              const uint64_t* v = p.S + (size_t)j * 2 * W;
              uint64_t vv[2 * W];
              int x = 0;
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) {
                vv[q] = __ldg(&v[q]);
                x += __popcll(u[q] ^ vv[q]);
              }
              if (x > 4 || x == 0 || (p.adj_1e && x == 4)) continue;
              int rankJ = 0;
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) rankJ += __popcll(hf[q] & ~vv[q]);
              double w = 0.0;
#pragma unroll
              for (int m = 0; m < R; ++m)
                if (m < p.metat) w += gb[m] * __ldg(&p.c[(size_t)j * p.metat + m]);
              hmat_adj<W>(p, u, vv, rankI, rankJ, hf, w, !p.adj_1e);
            }
            diag_terms_adj<W>(p, u, hf, p.yen ? gh : 0.0, gm, adj_sl);
          }
        } else {
          enqueue_candidate<W, R>(p, wq, qn, live, u, hmpi, hvpi, bc, t - ur0, 0.0, 0, false, true, acc, hp);
        }
      }
      drain_queue<W, R>(p, wq, qn, true, acc, hp);
      if (!ADJ && p.rec_mode) unit_compact<W>(p, unit, ur1 - ur0, ctmp, sh.unit_base);
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
          if ((get_word<2 * W>(kb, s * W + (o >> 6)) >> (o & 63)) & 1ull) {
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
    const int nnb = ordered_partition2(
        ncf,
        [&](int j) {
          int x = 0;
#pragma unroll
          for (int q = 0; q < 2 * W; ++q) x += __popcll(kb[q] ^ __ldg(&p.S[(size_t)j * 2 * W + q]));
          return x <= 8 ? 0 : -1;
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
        ctmp).x;
    const int rank_k = sh.rank_k;
    const uint8_t dmask = p.gen_dmask[g];
    const int nespk = p.nesp[k];
    const bool yefk = p.yef[k] != 0;
    int slot0 = 0;  // first candidate slot of the current block in the unit

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
      const int bslot = slot0;
      slot0 += (int)block_candidates(nRr, sp1 == sp2, sh.nvir[sp1], sh.nvir[0], sh.nvir[1]);
      const uint64_t rmask = (1ull << e1) | (e2 >= 0 ? (1ull << e2) : 0ull);
      // K' = k - R
      uint64_t kp[2 * W];
#pragma unroll
      for (int q = 0; q < 2 * W; ++q) kp[q] = kb[q];
      clear_word<2 * W>(kp, sp1 * W + (o1 >> 6), 1ull << (o1 & 63));
      if (e2 >= 0) clear_word<2 * W>(kp, sp2 * W + (o2 >> 6), 1ull << (o2 & 63));
      auto lr_m = [&](int t) {
        const uint64_t em = my_nb_em[t];
        return __popcll(em) - __popcll(em & rmask);
      };
      // L_R, partitioned: entries with |K' \ j| <= 1 first, then those with
      // |K' \ j| = 2; each part in ascending j, so every sum over interacting
      // determinants runs in a fixed order (bitwise reproducible results).
      // Entry of j: m = |K' \ j| and E = j \ K' (at most 4 spin orbitals),
      // since for I = K' + A, |I \ j| = m + |A \ E|.
      auto lr_store = [&](int slot, int t) {
        const int j = my_nb_j[t];
        const uint64_t* v = p.S + (size_t)j * 2 * W;
        uint32_t ebytes = 0;
        int ne = 0;
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) {
          uint64_t d = __ldg(&v[q]) & ~kp[q];
          while (d) {
            const int b = __ffsll((long long)d) - 1;
            d &= d - 1;
            const uint32_t code = (uint32_t)((q % W) * 64 + b + (q / W) * p.norb);
            if (ne < 4) ebytes |= code << (8 * ne);
            ++ne;
          }
        }
        const uint64_t ent = lr_entry(ebytes, ne, lr_m(t), j);
        if (slot < p.lr_cap)
          lr_ent[slot] = ent;
        else
          my_lr_ent[slot] = ent;
      };
      // diagonal energies of I = K' + A from those of K' (cip/hdig.f, hmp.f
      // written over occupation changes dn relative to the reference):
      //   hdig = sum_r dn_r F_rr + 1/2 sum_rs dn_r dn_s (J_rs - [same spin] K_rs)
      //   hmp  = sum_r dn_r fmpb_r
      // (listed by thread 0 before the partition below, whose first barrier
      // publishes it)
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
      const int2 nparts = ordered_partition2(
          nnb,
          [&](int t) {
            const int m = lr_m(t);
            return m <= 1 ? 0 : (m == 2 ? 1 : -1);
          },
          lr_store, ctmp);
      const int n01 = nparts.x;
      const int nlr = nparts.x + nparts.y;
      const bool fast = nlr <= p.lr_cap;
      if (!fast && tid == 0) atomicAdd(&p.counters[C_LRFALLBACK], 1ull);
      auto ent_at = [&](int i) -> uint64_t { return i < p.lr_cap ? lr_ent[i] : my_lr_ent[i]; };
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
        if ((tid >> 5) == (int)(blockDim.x >> 5) - 1) {
          // the last warp: the ndn + ndn^2 terms of hdig(K') and hmp(K')
          // spread over its lanes, then summed by shuffles in a fixed order
          const int lane = tid & 31;
          double e = 0.0, mp = 0.0;
          for (int t = lane; t < ndn * (ndn + 1); t += 32) {
            if (t < ndn) {
              const int r = sh.dn_so[t], orr = r % n;
              e += sh.dn_sg[t] * __ldg(&p.F[tri(orr, orr)]);
              mp += sh.dn_sg[t] * __ldg(&p.fmpb[r]);
            } else {
              const int i = (t - ndn) / ndn, j = (t - ndn) % ndn;
              const int r = sh.dn_so[i], q = sh.dn_so[j];
              const int tq = tri(r % n, q % n);
              double x = __ldg(&p.J[tq]);
              if (r / n == q / n) x -= __ldg(&p.K[tq]);
              e += 0.5 * sh.dn_sg[i] * sh.dn_sg[j] * x;
            }
          }
          for (int o = 16; o > 0; o >>= 1) {
            e += __shfl_down_sync(0xffffffffu, e, o);
            mp += __shfl_down_sync(0xffffffffu, mp, o);
          }
          if (lane == 0) {
            sh.hK = e;
            sh.mK = mp;
          }
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
                           int nrb, int slot) {
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
        // The scan runs in two phases so that the expensive part (the
        // Slater-Condon element and its integral gathers) runs with the warp
        // converged: phase A compares I with every entry and applies the
        // owner and already-in-S tests from the entry alone, keeping the
        // lane's remaining hits in its list; phase B then takes the t-th hit
        // of every lane at once.  Visiting each hit as it is found would run
        // the element once per hitting lane (hits fall at different
        // positions for different lanes), i.e. one lane at a time.  Both
        // loops below are warp-uniform (nscan and nrb are the same for the
        // whole warp); a lane's hits keep their scan order, so the sums are
        // the same as with in-place visits.
        bool drop = !live;
        int nh = 0;
        int* hl = hitl + threadIdx.x * kHitCap;
        // adjoint: the first two one-difference partners j (and their count),
        // for the one-electron second pass
        int s1n = 0, s1j0 = 0, s1j1 = 0;
        const int rankI = rank_k + D;
        const bool two = a2 >= 0;
        const uint32_t c1x4 = live ? (uint32_t)(a1 + sa1 * p.norb) * 0x01010101u : 0u;
        const uint32_t c2x4 = live && two ? (uint32_t)(a2 + sa2 * p.norb) * 0x01010101u : 0u;
        if (live) {
          sc.ncand++;
          or_word<2 * W>(u, sa1 * W + (a1 >> 6), 1ull << (a1 & 63));
          if (a2 >= 0) or_word<2 * W>(u, sa2 * W + (a2 >> 6), 1ull << (a2 & 63));
        }
        // phase A on one entry: j < k is the owner test (a generator below k
        // within two excitations owns I), x == 0 means I is in S
        auto hit = [&](int i, int x) {
          const int j = lr_entry_j(ent_at(i));
          if (j < k) {
            if (p.ygen[j]) drop = true;
            return;
          }
          if (x == 0) {
            drop = true;
            return;
          }
          hl[nh++] = i;
        };
        // phase B: <I|H|j> of the listed hits, lanes in step
        auto flush = [&]() {
          const int maxh = __reduce_max_sync(0xffffffffu, drop ? 0 : nh);
          for (int t = 0; t < maxh; ++t) {
            if (!drop && t < nh) {
              const int j = lr_entry_j(ent_at(hl[t]));
              uint64_t vv[2 * W];
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) vv[q] = __ldg(&p.S[(size_t)j * 2 * W + q]);
              int rankJ = 0;
#pragma unroll
              for (int q = 0; q < 2 * W; ++q) rankJ += __popcll(hf[q] & ~vv[q]);
              int kind;
              const double h = hmat<W>(p, u, vv, rankI, rankJ, hf, kind);
              if (kind == 1) sc.np1++; else sc.np2++;
              if (ADJ && kind == 1) {
                s1j1 = s1n == 1 ? j : s1j1;
                s1j0 = s1n == 0 ? j : s1j0;
                ++s1n;
              }
              ++nint;
              if (h != 0.0) ++nnz;
              if (j > k && j <= k + nespk) ++lesp;
#pragma unroll
              for (int m = 0; m < R; ++m)
                if (m < p.metat) bc[m] += h * __ldg(&p.c[(size_t)j * p.metat + m]);
            }
          }
          nh = 0;
        };
        for (int i0 = 0; i0 < nscan; i0 += 4) {
          if (__all_sync(0xffffffffu, drop)) break;
          if (__any_sync(0xffffffffu, !drop && nh > kHitCap - 4)) flush();
          if (!drop) {
            // four independent compares per step (latency of the loads
            // overlaps); the hits are walked as a bit mask and each one's
            // difference picked by selects, so nothing here is indexed at
            // run time (a run-time index into a local array puts it on the
            // stack)
            const int x0 = lr_diff(ent_at(i0), c1x4, c2x4, two);
            const int x1 = i0 + 1 < nscan ? lr_diff(ent_at(i0 + 1), c1x4, c2x4, two) : 99;
            const int x2 = i0 + 2 < nscan ? lr_diff(ent_at(i0 + 2), c1x4, c2x4, two) : 99;
            const int x3 = i0 + 3 < nscan ? lr_diff(ent_at(i0 + 3), c1x4, c2x4, two) : 99;
            unsigned hits = (x0 <= 4 ? 1u : 0u) | (x1 <= 4 ? 2u : 0u) | (x2 <= 4 ? 4u : 0u) | (x3 <= 4 ? 8u : 0u);
            while (hits && !drop) {
              const int g4 = __ffs(hits) - 1;
              hits &= hits - 1u;
              hit(i0 + g4, g4 == 0 ? x0 : g4 == 1 ? x1 : g4 == 2 ? x2 : x3);
            }
          }
        }
        for (int q2 = 0; q2 < nrb; ++q2) {
          if (__all_sync(0xffffffffu, drop)) break;
          if (__any_sync(0xffffffffu, !drop && nh >= kHitCap)) flush();
          if (!drop) {
            const int i = rb[q2];
            const int x = lr_diff(ent_at(i), c1x4, c2x4, two);
            if (x <= 4) hit(i, x);
          }
        }
        flush();
        if (live) {
          sc.ncmp += (unsigned long long)(nscan + nrb);
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
              fmul = spin_weight(nespk, lesp);
              nmul = (int)fmul;
            }
          } else {
            int nespf = nespk;
            ybis = nespf > 0;
            if (yefk || ysyspi) {
              ybis = true;
              if (!yefk) nespf = nespf + nespf + 1;
            }
            fmul = spin_weight(nespf, lesp);
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
        if (ADJ) {
          double gb[R], gh = 0.0, gm = 0.0;
#pragma unroll
          for (int m = 0; m < R; ++m) gb[m] = 0.0;
          if (live) {
            adj_factors<R>(p, bc, hmpi, hvpi, ybis ? 1.0 + fmul : 1.0, gb, gh, gm, adjr, acc);
            acc.ietat += (unsigned long long)(long long)(nmul + 1);
            acc.nproc += 1;
            if (!p.yen) gh = 0.0;
          }
          // second pass over the same entries: dE/dH_Ij = sum_m gb[m] c_jm,
          // spread over the integrals of <I|H|j>.  Two phases as in the first
          // pass: each lane lists the entries that interact with its I, then
          // the warp takes the t-th listed entry of every lane at once, so
          // hmat_adj runs with the warp in step instead of once per hitting
          // lane.  The loops are warp-uniform (nscan, nrb); dead lanes list
          // nothing.  One-electron adjoint: only the one-difference partners
          // matter; those the first pass noted (up to two) are done here,
          // and the scan runs only for lanes with more.
          const bool with_eri = !p.adj_1e;
          const bool rescan = live && (with_eri || s1n > 2);
          const auto adj_one = [&](int j) {
            uint64_t vv[2 * W];
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) vv[q] = __ldg(&p.S[(size_t)j * 2 * W + q]);
            int rankJ = 0;
#pragma unroll
            for (int q = 0; q < 2 * W; ++q) rankJ += __popcll(hf[q] & ~vv[q]);
            double w = 0.0;
#pragma unroll
            for (int m = 0; m < R; ++m)
              if (m < p.metat) w += gb[m] * __ldg(&p.c[(size_t)j * p.metat + m]);
            hmat_adj<W>(p, u, vv, rank_k + D, rankJ, hf, w, with_eri);
          };
          if (!with_eri && live && s1n <= 2) {
            if (s1n > 0) adj_one(s1j0);
            if (s1n > 1) adj_one(s1j1);
          }
          const bool two = a2 >= 0;
          const uint32_t c1x4 = rescan ? (uint32_t)(a1 + sa1 * p.norb) * 0x01010101u : 0u;
          const uint32_t c2x4 = rescan && two ? (uint32_t)(a2 + sa2 * p.norb) * 0x01010101u : 0u;
          const int xmax = with_eri ? 4 : 2;
          int nh = 0;
          int* hl = hitl + threadIdx.x * kHitCap;
          auto note = [&](int i) {
            const int x = lr_diff(ent_at(i), c1x4, c2x4, two);
            if (x <= xmax && x != 0 && lr_entry_j(ent_at(i)) >= k) hl[nh++] = i;
          };
          auto flush_adj = [&]() {
            const int maxh = __reduce_max_sync(0xffffffffu, nh);
            for (int t = 0; t < maxh; ++t)
              if (t < nh) adj_one(lr_entry_j(ent_at(hl[t])));
            nh = 0;
          };
          if (__any_sync(0xffffffffu, rescan)) {
            for (int i = 0; i < nscan; ++i) {
              if (__any_sync(0xffffffffu, nh == kHitCap)) flush_adj();
              if (rescan) note(i);
            }
            for (int q2 = 0; q2 < nrb; ++q2) {
              if (__any_sync(0xffffffffu, nh == kHitCap)) flush_adj();
              if (rescan) note(rb[q2]);
            }
            flush_adj();
          }
          if (!live) return;
          // diagonal terms: hdig(I) = hdig(K') + vdg[a1] + vdg[a2] + G(a1,a2),
          // hmp(I) = hmp(K') + fmpb[a1] + fmpb[a2]
          adj_gK += gh;
          adj_gM += gm;
          atomicAdd(&adj_gv[a1 + sa1 * p.norb], gh);
          atomicAdd(&adj_gf[a1 + sa1 * p.norb], gm);
          if (a2 >= 0) {
            atomicAdd(&adj_gv[a2 + sa2 * p.norb], gh);
            atomicAdd(&adj_gf[a2 + sa2 * p.norb], gm);
            const int nt = p.norb * (p.norb + 1) / 2;
            const int tq = tri(a1, a2);
            atomicAdd(&adj_sl[nt + tq], gh);
            if (sa1 == sa2) atomicAdd(&adj_sl[2 * nt + tq], -gh);
          }
          return;
        }
        enqueue_candidate<W, R>(p, wq, qn, live, u, hmpi, hvpi, bc, slot, fmul, nmul, ybis, is_pert1, acc, hp);
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
          candidate(live, a1, a2, sa1, sa2, nlr, nullptr, 0, bslot + t);
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
        // rows in zig-zag order over the warps (row lengths fall with the
        // row index for same-spin pairs): even stripes forward, odd backward
        for (int t = 0; t * nwarps < nrows; ++t) {
          const int row = (t & 1) ? t * nwarps + (nwarps - 1 - wid) : t * nwarps + wid;
          if (row >= nrows) continue;
          const int a1 = sh.vir[sr][row];
          const uint32_t r1x4 = (uint32_t)(a1 + sr * p.norb) * 0x01010101u;
          int nrb = 0;
          for (int i0 = n01; i0 < nlr; i0 += 32) {
            const int i = i0 + lane;
            const bool has = i < nlr && has_byte((uint32_t)ent_at(i), r1x4);
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
            // a row list that overflowed falls back to the whole of L_R (one
            // call site: the candidate code is instantiated once for rows)
            // slot: the pair's index in the flat enumeration (row-major
            // over a1 < a2 for one spin, a1 x a2 for opposite spins)
            const int tflat = same ? row * (nv1 - 1) - row * (row - 1) / 2 + c : row * sh.nvir[1] + c;
            candidate(live, a1, a2, sr, sc, overflow ? nlr : n01, rowbuf, overflow ? 0 : nrb, bslot + tflat);
          }
          __syncwarp();
        }
      }
      __syncthreads();
      if (ADJ) {
        // expand this block's dE/dhdig and dE/dhmp sums over F, J, K, fmpb
        if (tid < 2) adj_sh[tid] = 0.0;
        __syncthreads();
        double gk = adj_gK, gmk = adj_gM;
        for (int o = 16; o > 0; o >>= 1) {
          gk += __shfl_down_sync(0xffffffffu, gk, o);
          gmk += __shfl_down_sync(0xffffffffu, gmk, o);
        }
        if ((tid & 31) == 0) {
          atomicAdd(&adj_sh[0], gk);
          atomicAdd(&adj_sh[1], gmk);
        }
        adj_gK = adj_gM = 0.0;
        __syncthreads();
        const int n = p.norb, nt = n * (n + 1) / 2, ndn = sh.ndn;
        double* sF = adj_sl;
        double* sJ = adj_sl + nt;
        double* sK = adj_sl + 2 * nt;
        double* sf = adj_sl + 3 * nt;
        if (tid == 0) {
          // hdig(K') = sum_i dn_i F_rr + 1/2 sum_ij dn_i dn_j (J - [same spin] K)
          const double G = adj_sh[0], M = adj_sh[1];
          for (int i = 0; i < ndn; ++i) {
            const int r = sh.dn_so[i], orr = r % n;
            atomicAdd(&sf[r], sh.dn_sg[i] * M);
            if (G == 0.0) continue;
            atomicAdd(&sF[tri(orr, orr)], sh.dn_sg[i] * G);
            for (int j = 0; j < ndn; ++j) {
              const int q = sh.dn_so[j];
              const int t = tri(orr, q % n);
              const double c = 0.5 * sh.dn_sg[i] * sh.dn_sg[j] * G;
              atomicAdd(&sJ[t], c);
              if (r / n == q / n) atomicAdd(&sK[t], -c);
            }
          }
        }
        for (int a = tid; a < 2 * n; a += blockDim.x) {
          // vdg[a] = F_aa + sum_i dn_i (J - [same spin] K)(a, r_i) + 1/2 (J_aa - K_aa)
          const double gv = adj_gv[a];
          if (adj_gf[a] != 0.0) atomicAdd(&sf[a], adj_gf[a]);
          if (gv == 0.0) continue;
          const int oa = a % n, sa = a / n;
          const int ta = tri(oa, oa);
          atomicAdd(&sF[ta], gv);
          atomicAdd(&sJ[ta], 0.5 * gv);
          atomicAdd(&sK[ta], -0.5 * gv);
          for (int i = 0; i < ndn; ++i) {
            const int r = sh.dn_so[i];
            const int t = tri(oa, r % n);
            atomicAdd(&sJ[t], sh.dn_sg[i] * gv);
            if (sa == r / n) atomicAdd(&sK[t], -sh.dn_sg[i] * gv);
          }
        }
        __syncthreads();
        for (int i = tid; i < 2 * n; i += blockDim.x) adj_gv[i] = adj_gf[i] = 0.0;
        __syncthreads();
      }
    }
    drain_queue<W, R>(p, wq, qn, true, acc, hp);
    if (!ADJ && p.rec_mode) unit_compact<W>(p, unit, slot0, ctmp, sh.unit_base);
    block_flush<R>(p, acc, unit, red);
  }

  if (!B || cur_geo >= 0) flush_totals<R>(p, acc, hp, hist, sc.ncand, sc.ncmp, sc.np1, sc.np2);
  if (ADJ) {
#pragma unroll
    for (int k3 = 0; k3 < 3; ++k3)
#pragma unroll
      for (int m = 0; m < R; ++m) {
        double v = adjr[k3][m];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0 && m < p0.metat && v != 0.0) atomicAdd(&p0.g_roots[k3 * p0.metat + m], v);
      }
  }
}

}  // namespace

template <int W, int R, bool B, bool ADJ>
cudaError_t launch_pt2(const Params& p, const BatchArgs& ba, int grid, size_t smem, cudaStream_t st) {
  cudaError_t e =
      cudaFuncSetAttribute(k_pt2<W, R, B, ADJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_pt2<W, R, B, ADJ><<<grid, kThreads, smem, st>>>(p, ba);
  return cudaGetLastError();
}

}  // namespace cipsi_dev
