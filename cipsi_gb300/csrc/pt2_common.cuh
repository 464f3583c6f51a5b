// pt2_common.cuh -- types shared by the perturbation kernels (pt2_kernel.cuh,
// compiled in pt2_w1.cu / pt2_w2.cu) and the host side (cipsi_engine.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/cipsi_gb300.h"

namespace cipsi_dev {

constexpr int kNClass = CIPSI_NCLASS;
constexpr int kMaxRoots = CIPSI_MAX_ROOTS;
constexpr int kThreads = 256;
constexpr int kMaxSym = 8;
constexpr int kMaxElec = 64;
constexpr int kMaxOrb = 128;
constexpr int kRowCap = 128;  // per-warp list of |K' \ j| = 2 entries holding a1
constexpr int kHitCap = 8;    // per-thread list of scan hits awaiting their matrix elements

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
  C_STAGE_OVF,  // selected candidates whose slot lay outside the staging region (must stay 0)
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
  uint64_t* lr_ent;          // per block: ncf compact L_R entries beyond lr_cap
  int lr_cap;                // shared-memory capacity of L_R
  int nb_stride;             // entries per block in nb_j / nb_emask / lr_ent
  // outputs
  double* gen_part;          // ngen x (5 * metat)
  unsigned long long* counters;
  unsigned long long* dpivot_bits;
  unsigned long long* hist_nom;      // nclass
  unsigned long long* hist_nam;      // nclass x metat
  double* hist_tab;                  // 2 x nclass x metat (tabmp, tabvp)
  double* red;                       // 5 x metat reduced sums (k_reduce output)
  // unit-60 records.  A selected candidate is staged in its CTA's region at
  // its slot (its position in the work unit's candidate order) and flagged
  // in the region's slot mask; when the unit is done the CTA compacts the
  // flagged slots, in slot order, into one segment of the record pool and
  // notes the segment in the unit table.  k_gather then lays the segments
  // out in unit order, so the records come out in (unit, candidate) order
  // whatever the scheduling.
  int rec_mode;                      // 0: selection counted only; 1: records kept
  int st_cap;                        // slots per CTA region (multiple of 32)
  uint64_t* st_bits;                 // grid x st_cap x 2W
  double* st_xam;                    // grid x st_cap
  double* st_evp;                    // grid x st_cap x metat
  uint32_t* st_mask;                 // grid x st_cap / 32
  uint64_t* pool_bits;               // pool_cap x 2W
  double* pool_xam;                  // pool_cap
  double* pool_evp;                  // pool_cap x metat
  long long pool_cap;
  unsigned long long* pool_count;    // records placed in the pool (may exceed pool_cap: then not stored)
  long long* unit_pool;              // per unit: first pool record of its segment
  int32_t* unit_nsel;                // per unit: records of its segment
  int* work;                         // work counter
  // (pq|rs) as doubles: the caller's FP64 integrals (derivative checks) or
  // the real*4 ones widened on the device; null = read the real*4 `eri`
  const double* eri64;
  // adjoint launch (k_pt2<..., ADJ = true>): seeds dE/d e2mp[m], e2vp[m],
  // e2b[m] and the gradient outputs
  double seed_mp[kMaxRoots], seed_vp[kMaxRoots], seed_b[kMaxRoots];
  double* g_eri;    // ninte: dE/d(pq|rs) in the packed order
  double* g_F;      // n(n+1)/2: dE/dF (off-diagonal terms of one-difference elements)
  double* g_slice;  // per block: [F | J | K] packed triangles, then fmpb[2n]
  int slice_stride; // doubles per block slice (3 n(n+1)/2 + 2n)
  double* g_roots;  // 3 x metat: dE/d e, d eb, d emp
  // one-electron adjoint: no (pq|rs) gradient (g_eri unused), so only the
  // single-excitation elements (their F term) take part in the second pass
  int adj_1e;
};

static_assert(sizeof(Params) % sizeof(int) == 0, "Params is copied as ints");

// Batched launch: many geometries (each with its own Params) in one
// persistent launch.  Global unit u belongs to geometry unit_geo[u] and is
// unit unit_local[u] of that geometry's unit list.
struct BatchArgs {
  const Params* geo;
  const int32_t* unit_geo;
  const int32_t* unit_local;
  int nunits;
  int* work;
};

__device__ __forceinline__ void kahan_add(double& s, double& c, double x) {
  const double y = x - c;
  const double t = s + y;
  c = (t - s) - y;
  s = t;
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
  int nmul[kQCap], slot[kQCap];  // slot: the candidate's position in its work unit
  unsigned char flags[kQCap];  // bit 0 ybis, bit 1 is_pert1
};

// Candidates of one block of removed electrons R: nv added orbitals for
// |R| = 1, nv(nv-1)/2 same-spin pairs, nva * nvb opposite-spin pairs (nv:
// empty orbitals of the generator in the spin(s) of R).  A work unit's
// candidate slots are numbered block after block (blocks with no allowed
// rank-change class take none), then by the candidate's index in its block:
// the added orbital, or the pair (a1 < a2) in row-major order.
__host__ __device__ inline long long block_candidates(int nR, bool same_spin, int nv1, int nva, int nvb) {
  if (nR == 1) return nv1;
  return same_spin ? (long long)nv1 * (nv1 - 1) / 2 : (long long)nva * nvb;
}

// k_pt2<W, R, B, ADJ> launched with `smem` bytes of dynamic shared memory
// (pt2_w1.cu / pt2_w2.cu: forward, plain and batched; pt2_adj.cu: adjoint).
template <int W, int R, bool B, bool ADJ = false>
cudaError_t launch_pt2(const Params& p, const BatchArgs& ba, int grid, size_t smem, cudaStream_t st);

// The Hamiltonian over a determinant list by rows (hbuild.cu): pass 1
// counts, per row i, the columns j < min(i, jmax) within two excitations;
// pass 2 writes them, in increasing j, from rowptr[i] on.
struct HBuildArgs {
  Params p;                 // integrals (pairtab, ntttt, eri / eri64, F) and norb
  const uint64_t* S;        // n x 2W words
  const int8_t* sigma;      // n: phase of each determinant's excitation list
  int n;                    // determinants (rows)
  int jmax;                 // columns j < min(i, jmax)
  uint64_t hf[4];           // the reference determinant (2W words)
  int32_t* count;           // pass 1 output: columns per row
  const long long* rowptr;  // pass 2 input: first pair of each row
  int32_t* col;             // pass 2 outputs
  double* val;
};

template <int W>
cudaError_t launch_hpairs(const HBuildArgs& a, bool fill, cudaStream_t st);

}  // namespace cipsi_dev
