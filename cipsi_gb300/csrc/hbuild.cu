// hbuild.cu -- the Hamiltonian over a list of determinants, lower triangle by
// rows, as moy builds it for the S + selected list (moy/moy.f:117-199):
// row i holds every column j < min(i, jmax) within two excitations of i,
// in increasing j, with <i|H|j> in the phase of the reference's excitation
// lists (the value moy's hntd returns).
//
// Two passes over the same pair scan:
//   k_hpairs<W, false>  counts the columns of every row (degree <= 2);
//   k_hpairs<W, true>   writes (j, <i|H|j>) at the row's offset (an
//                       exclusive scan of the counts).
// One thread owns one row; a CTA owns 256 consecutive rows and streams the
// columns below them through shared memory in tiles, so every lane of a
// warp reads the same column (a broadcast) and each column tile comes from
// L2 once per 256 rows.  The degree test is XOR + popcount over the 2W
// words of the two bitstrings.  In the fill pass a lane notes its hits in a
// short list and the warp evaluates the listed matrix elements together
// (lanes hit at different columns: evaluating each hit where it is found
// would run the Slater-Condon code once per hitting lane).
//
// Matrix elements: hmat() of the perturbation kernel (canonical alpha-then-
// beta string phase, the one-difference sum taken over the holes and
// particles of the more excited determinant -- the column when the ranks
// are equal, as moy/hntd.f picks it), times sigma_i * sigma_j, the
// excitation-list phases of the two determinants.  Identical determinants
// (popcount 0) give 0, as hntd does.
#include "pt2_kernel.cuh"

namespace cipsi_dev {
namespace {

constexpr int kHRows = 256;  // rows (threads) per CTA
constexpr int kHTile = 512;  // columns per shared-memory tile
constexpr int kHHits = 8;    // per-thread list of hits awaiting their elements

template <int W, bool FILL>
__global__ void __launch_bounds__(kHRows) k_hpairs(HBuildArgs a) {
  __shared__ uint64_t tile[kHTile * 2 * W];
  __shared__ int hitl[FILL ? kHRows * kHHits : 1];
  __shared__ Params sp;
  if (threadIdx.x == 0) sp = a.p;
  // heavy (high) row blocks first: row i scans i columns
  const int rb = (int)gridDim.x - 1 - (int)blockIdx.x;
  const int row0 = rb * kHRows;
  const int i = row0 + (int)threadIdx.x;
  const bool row_ok = i < a.n;
  const int jend = row_ok ? min(i, a.jmax) : 0;
  const int jblock = min(min(row0 + kHRows - 1, a.n - 1), a.jmax);  // the block's largest jend
  uint64_t u[2 * W], hf[2 * W];
#pragma unroll
  for (int q = 0; q < 2 * W; ++q) {
    u[q] = row_ok ? a.S[(size_t)i * 2 * W + q] : 0ull;
    hf[q] = a.hf[q];
  }
  int rankI = 0;
#pragma unroll
  for (int q = 0; q < 2 * W; ++q) rankI += __popcll(hf[q] & ~u[q]);
  const double sgi = row_ok ? (double)a.sigma[i] : 0.0;
  int cnt = 0;
  long long out = (FILL && row_ok) ? a.rowptr[i] : 0;
  int nh = 0;
  int* hl = hitl + (FILL ? threadIdx.x * kHHits : 0);
  __syncthreads();
  const Params& p = sp;
  // the listed hits of every lane of the warp, evaluated in step
  auto flush = [&]() {
    const int maxh = __reduce_max_sync(0xffffffffu, nh);
    for (int t = 0; t < maxh; ++t) {
      if (t < nh) {
        const int j = hl[t];
        uint64_t v[2 * W];
        int diff = 0, rankJ = 0;
#pragma unroll
        for (int q = 0; q < 2 * W; ++q) {
          v[q] = __ldg(&a.S[(size_t)j * 2 * W + q]);
          diff += __popcll(u[q] ^ v[q]);
          rankJ += __popcll(hf[q] & ~v[q]);
        }
        double h = 0.0;
        if (diff != 0) {
          int kind;
          h = hmat<W>(p, u, v, rankI, rankJ, hf, kind);
        }
        a.col[out] = j;
        a.val[out] = sgi * (double)__ldg(&a.sigma[j]) * h;
        ++out;
      }
    }
    nh = 0;
  };
  for (int j0 = 0; j0 < jblock; j0 += kHTile) {
    const int nt = min(kHTile, jblock - j0);
    __syncthreads();
    for (int x = threadIdx.x; x < nt * 2 * W; x += kHRows) tile[x] = __ldg(&a.S[(size_t)j0 * 2 * W + x]);
    __syncthreads();
    for (int t = 0; t < nt; ++t) {
      int d = 0;
#pragma unroll
      for (int q = 0; q < 2 * W; ++q) d += __popcll(u[q] ^ tile[t * 2 * W + q]);
      const bool hit = (j0 + t < jend) && d <= 4;
      if (FILL) {
        if (hit) hl[nh++] = j0 + t;
        if (__any_sync(0xffffffffu, nh == kHHits)) flush();
      } else {
        cnt += hit ? 1 : 0;
      }
    }
  }
  if (FILL) {
    flush();
  } else if (row_ok) {
    a.count[i] = cnt;
  }
}

}  // namespace

template <int W>
cudaError_t launch_hpairs(const HBuildArgs& a, bool fill, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  const int grid = (a.n + kHRows - 1) / kHRows;
  if (fill)
    k_hpairs<W, true><<<grid, kHRows, 0, st>>>(a);
  else
    k_hpairs<W, false><<<grid, kHRows, 0, st>>>(a);
  return cudaGetLastError();
}

template cudaError_t launch_hpairs<1>(const HBuildArgs&, bool, cudaStream_t);
template cudaError_t launch_hpairs<2>(const HBuildArgs&, bool, cudaStream_t);

}  // namespace cipsi_dev
