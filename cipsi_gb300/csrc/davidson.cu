// davidson.cu -- the lowest eigenpairs of the CI matrix that moy writes to
// unit 1 (the work of bd, CIPSI_sources/bd/bigdia.f), on the GPU.
//
// The matrix is H = L + L^T, L being the elements moy stores (row i: the
// columns j < i, then the diagonal as half its value, moy/moy.f:150-190,
// as bd/getmat.f rebuilds it).  It is assembled once as a full CSR matrix in
// device memory; the iteration is a block Davidson method:
//
//   V (n x k) orthonormal, W = H V;  Rayleigh-Ritz on V^T W (host, k <= 64);
//   Ritz vectors X = V S, residuals R = W S - X Theta;  converged when every
//   residual norm is below `tol`;  corrections T = R / (theta - diag(H))
//   (the diagonal preconditioner of Davidson's method), made orthogonal to
//   V twice and orthonormalised through their Gram matrix; V grows by T
//   until it would exceed kmax columns, then restarts from the Ritz vectors.
//
// Kernels: k_spmm (H times a block of vectors: one warp per row, the row's
// nonzeros over the lanes, a shuffle reduction per vector), k_gram (V^T T:
// one CTA per output element, fixed-order tree sums, so results are
// reproducible run to run), k_combine (X = V S, thread per row), k_precond.
// HBM-bound: each product reads the 12 bytes of every nonzero once, and the
// vectors (8 bytes per row and vector) stay L2-resident up to ~10^6 rows.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cipsi_gb300.h"
#include "symeig.h"

namespace {

constexpr int kMaxBlock = 16;  // vectors per block product

template <int NV>
__global__ void __launch_bounds__(256) k_spmm(int n, const long long* __restrict__ rowptr,
                                              const int32_t* __restrict__ col, const double* __restrict__ val,
                                              const double* __restrict__ X, int ldx, double* __restrict__ Y,
                                              int ldy, int nv) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = 0.0;
    const long long a = rowptr[row], b = rowptr[row + 1];
    for (long long t = a + lane; t < b; t += 32) {
      const int c = __ldg(&col[t]);
      const double h = __ldg(&val[t]);
#pragma unroll
      for (int v = 0; v < NV; ++v)
        if (v < nv) acc[v] = fma(h, __ldg(&X[(size_t)v * ldx + c]), acc[v]);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      double x = acc[v];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0 && v < nv) Y[(size_t)v * ldy + row] = x;
    }
  }
}

// G[a * kb + b] = sum_i A[a * lda + i] * B[b * ldb + i]; one CTA per (a, b)
__global__ void __launch_bounds__(256) k_gram(int n, const double* __restrict__ A, int lda, int ka,
                                              const double* __restrict__ B, int ldb, int kb, double* __restrict__ G) {
  __shared__ double red[256];
  const int a = blockIdx.x / kb, b = blockIdx.x % kb;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(A[(size_t)a * lda + i], B[(size_t)b * ldb + i], s);
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) G[(size_t)a * kb + b] = red[0];
  (void)ka;
}

// Y[:, b] = beta * Y[:, b] + sum_a A[:, a] S[a * kb + b]   (S: ka x kb, row-major)
__global__ void __launch_bounds__(256) k_combine(int n, const double* __restrict__ A, int lda, int ka,
                                                 const double* __restrict__ S, int kb, double beta,
                                                 double* __restrict__ Y, int ldy) {
  extern __shared__ double sS[];
  for (int i = threadIdx.x; i < ka * kb; i += blockDim.x) sS[i] = S[i];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int b = 0; b < kb; ++b) {
      double y = beta == 0.0 ? 0.0 : beta * Y[(size_t)b * ldy + i];
      for (int a = 0; a < ka; ++a) y = fma(A[(size_t)a * lda + i], sS[a * kb + b], y);
      Y[(size_t)b * ldy + i] = y;
    }
  }
}

// T[:, b] = R[:, b] / (theta_b - d_i), the denominator kept away from zero
__global__ void k_precond(int n, const double* __restrict__ R, int ldr, const double* __restrict__ diag,
                          const double* __restrict__ theta, int kb, double* __restrict__ T, int ldt) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int b = 0; b < kb; ++b) {
      double den = theta[b] - diag[i];
      if (std::fabs(den) < 1e-8) den = den < 0.0 ? -1e-8 : 1e-8;
      T[(size_t)b * ldt + i] = R[(size_t)b * ldr + i] / den;
    }
}

struct Dev {
  std::string err;
  bool ok = true;
  bool check(cudaError_t e, const char* what) {
    if (e != cudaSuccess && ok) {
      ok = false;
      err = std::string(what) + ": " + cudaGetErrorString(e);
    }
    return e == cudaSuccess;
  }
};

void seterr(char* errbuf, int32_t errlen, const std::string& m) {
  if (errbuf && errlen > 0) std::snprintf(errbuf, (size_t)errlen, "%s", m.c_str());
}

}  // namespace

extern "C" int cipsi_davidson(int32_t n, int64_t nel, const int32_t* itab, const int32_t* jtab, const double* val,
                              int32_t nroots, double tol, int32_t maxiter, int32_t device, double* evals,
                              double* evecs, int32_t* iters, double* resid, char* errbuf, int32_t errlen) {
  using cipsi_host::sym_eig;
  if (n < 1 || nel < 0 || nroots < 1 || nroots > n || !itab || !jtab || !val || !evals || !evecs) {
    seterr(errbuf, errlen, "cipsi_davidson: bad arguments");
    return CIPSI_ERR_ARG;
  }
  if (nroots > 8) {
    seterr(errbuf, errlen, "cipsi_davidson: at most 8 roots");
    return CIPSI_ERR_ARG;
  }
  // full CSR of H = L + L^T (host), diagonal kept for the preconditioner
  std::vector<long long> rowptr((size_t)n + 1, 0);
  std::vector<double> diag(n, 0.0);
  for (int64_t t = 0; t < nel; ++t) {
    const int i = itab[t] - 1, j = jtab[t] - 1;
    if (i < 0 || i >= n || j < 0 || j >= n || j > i) {
      seterr(errbuf, errlen, "cipsi_davidson: element " + std::to_string(t + 1) + " outside the lower triangle");
      return CIPSI_ERR_ARG;
    }
    if (i == j) {
      diag[i] += 2.0 * val[t];
      continue;
    }
    ++rowptr[i + 1];
    ++rowptr[j + 1];
  }
  for (int i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i] + 1;  // + the diagonal slot
  std::vector<long long> fill(rowptr.begin(), rowptr.end() - 1);
  const long long nnz = rowptr[n];
  std::vector<int32_t> col((size_t)nnz);
  std::vector<double> hv((size_t)nnz);
  for (int i = 0; i < n; ++i) {
    col[fill[i]] = i;
    hv[fill[i]++] = diag[i];
  }
  for (int64_t t = 0; t < nel; ++t) {
    const int i = itab[t] - 1, j = jtab[t] - 1;
    if (i == j) continue;
    col[fill[i]] = j;
    hv[fill[i]++] = val[t];
    col[fill[j]] = i;
    hv[fill[j]++] = val[t];
  }
  // block size and subspace limit
  const int nb = std::min(n, std::min(kMaxBlock, nroots + 2));
  const int kmax = std::min(n, std::max(4 * nb, 24));
  Dev d;
  d.check(cudaSetDevice(device), "cudaSetDevice");
  cudaStream_t st = nullptr;
  d.check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
  long long* drow = nullptr;
  int32_t* dcol = nullptr;
  double *dval = nullptr, *ddiag = nullptr, *V = nullptr, *Wm = nullptr, *X = nullptr, *AX = nullptr, *T = nullptr,
         *AT = nullptr, *dG = nullptr, *dS = nullptr, *dth = nullptr;
  auto alloc = [&](void** p, size_t bytes, const char* what) { d.check(cudaMalloc(p, std::max<size_t>(bytes, 8)), what); };
  alloc((void**)&drow, rowptr.size() * 8, "rowptr");
  alloc((void**)&dcol, (size_t)nnz * 4, "col");
  alloc((void**)&dval, (size_t)nnz * 8, "val");
  alloc((void**)&ddiag, (size_t)n * 8, "diag");
  alloc((void**)&V, (size_t)n * kmax * 8, "V");
  alloc((void**)&Wm, (size_t)n * kmax * 8, "W");
  alloc((void**)&X, (size_t)n * nb * 8, "X");
  alloc((void**)&AX, (size_t)n * nb * 8, "AX");
  alloc((void**)&T, (size_t)n * nb * 8, "T");
  alloc((void**)&AT, (size_t)n * nb * 8, "AT");
  alloc((void**)&dG, (size_t)kmax * kmax * 8, "G");
  alloc((void**)&dS, (size_t)kmax * kmax * 8, "S");
  alloc((void**)&dth, (size_t)kmax * 8, "theta");
  if (d.ok) {
    d.check(cudaMemcpyAsync(drow, rowptr.data(), rowptr.size() * 8, cudaMemcpyHostToDevice, st), "copy");
    d.check(cudaMemcpyAsync(dcol, col.data(), (size_t)nnz * 4, cudaMemcpyHostToDevice, st), "copy");
    d.check(cudaMemcpyAsync(dval, hv.data(), (size_t)nnz * 8, cudaMemcpyHostToDevice, st), "copy");
    d.check(cudaMemcpyAsync(ddiag, diag.data(), (size_t)n * 8, cudaMemcpyHostToDevice, st), "copy");
  }
  int sms = 0;
  d.check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attr");
  const int ewgrid = std::max(1, std::min((n + 255) / 256, 8 * sms));
  const int spgrid = std::max(1, std::min((n * 32 + 255) / 256, 32 * sms));
  auto spmm = [&](const double* Xin, double* Yout, int nv) {
    for (int v0 = 0; v0 < nv && d.ok; v0 += kMaxBlock) {
      const int m = std::min(kMaxBlock, nv - v0);
      if (m <= 1)
        k_spmm<1><<<spgrid, 256, 0, st>>>(n, drow, dcol, dval, Xin + (size_t)v0 * n, n, Yout + (size_t)v0 * n, n, m);
      else if (m <= 4)
        k_spmm<4><<<spgrid, 256, 0, st>>>(n, drow, dcol, dval, Xin + (size_t)v0 * n, n, Yout + (size_t)v0 * n, n, m);
      else if (m <= 8)
        k_spmm<8><<<spgrid, 256, 0, st>>>(n, drow, dcol, dval, Xin + (size_t)v0 * n, n, Yout + (size_t)v0 * n, n, m);
      else
        k_spmm<16><<<spgrid, 256, 0, st>>>(n, drow, dcol, dval, Xin + (size_t)v0 * n, n, Yout + (size_t)v0 * n, n, m);
      d.check(cudaGetLastError(), "k_spmm");
    }
  };
  auto gram = [&](const double* A, int ka, const double* B, int kb, std::vector<double>& G) {
    G.assign((size_t)ka * kb, 0.0);
    if (!d.ok || ka == 0 || kb == 0) return;
    k_gram<<<ka * kb, 256, 0, st>>>(n, A, n, ka, B, n, kb, dG);
    d.check(cudaGetLastError(), "k_gram");
    d.check(cudaMemcpyAsync(G.data(), dG, G.size() * 8, cudaMemcpyDeviceToHost, st), "copy G");
    d.check(cudaStreamSynchronize(st), "sync");
  };
  auto combine = [&](const double* A, int ka, const std::vector<double>& S, int kb, double beta, double* Y) {
    if (!d.ok || kb == 0) return;
    d.check(cudaMemcpyAsync(dS, S.data(), S.size() * 8, cudaMemcpyHostToDevice, st), "copy S");
    k_combine<<<ewgrid, 256, (size_t)ka * kb * 8, st>>>(n, A, n, ka, dS, kb, beta, Y, n);
    d.check(cudaGetLastError(), "k_combine");
  };
  // T (nt columns): remove the components along V (two passes), then make
  // the columns orthonormal through their Gram matrix, dropping directions
  // with no weight left; returns the columns kept (written back into T)
  auto orthonormalise = [&](int k, int nt) -> int {
    // the scale of the corrections before projection: a direction is
    // dropped when projecting leaves less than 1e-10 of that scale
    std::vector<double> G0;
    gram(T, nt, T, nt, G0);
    double scale2 = 0.0;
    for (int q = 0; q < nt; ++q) scale2 = std::max(scale2, G0[(size_t)q * nt + q]);
    for (int pass = 0; pass < 2 && k > 0; ++pass) {
      std::vector<double> C;
      gram(V, k, T, nt, C);  // k x nt
      for (auto& x : C) x = -x;
      combine(V, k, C, nt, 1.0, T);
    }
    std::vector<double> G, w, U;
    gram(T, nt, T, nt, G);
    if (!d.ok) return 0;
    sym_eig(nt, G, w, U);
    std::vector<int> keep;
    for (int q = nt - 1; q >= 0; --q)
      if (w[q] > 1e-20 * scale2 && w[q] > 0.0) keep.push_back(q);
    const int nk = (int)keep.size();
    if (nk == 0) return 0;
    std::vector<double> Sx((size_t)nt * nk);
    for (int c = 0; c < nk; ++c)
      for (int r = 0; r < nt; ++r) Sx[(size_t)r * nk + c] = U[(size_t)r * nt + keep[c]] / std::sqrt(w[keep[c]]);
    combine(T, nt, Sx, nk, 0.0, AT);  // AT as scratch for the new columns
    d.check(cudaMemcpyAsync(T, AT, (size_t)n * nk * 8, cudaMemcpyDeviceToDevice, st), "copy T");
    // once more against V: the Gram step can bring back rounding-level overlap
    if (k > 0) {
      std::vector<double> C;
      gram(V, k, T, nk, C);
      for (auto& x : C) x = -x;
      combine(V, k, C, nk, 1.0, T);
      gram(T, nk, T, nk, G);
      if (!d.ok) return 0;
      sym_eig(nk, G, w, U);
      std::vector<double> S2((size_t)nk * nk);
      for (int c = 0; c < nk; ++c)
        for (int r = 0; r < nk; ++r) S2[(size_t)r * nk + c] = U[(size_t)r * nk + c] / std::sqrt(std::max(w[c], 1e-300));
      combine(T, nk, S2, nk, 0.0, AT);
      d.check(cudaMemcpyAsync(T, AT, (size_t)n * nk * 8, cudaMemcpyDeviceToDevice, st), "copy T");
    }
    return nk;
  };
  // start: unit vectors on the nb smallest diagonal elements
  {
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return diag[a] < diag[b]; });
    std::vector<double> v0((size_t)n * nb, 0.0);
    for (int b = 0; b < nb; ++b) v0[(size_t)b * n + ord[b]] = 1.0;
    if (d.ok) d.check(cudaMemcpyAsync(V, v0.data(), v0.size() * 8, cudaMemcpyHostToDevice, st), "copy V0");
    spmm(V, Wm, nb);
  }
  int k = nb, it = 0;
  std::vector<double> theta, Sm, res(nroots, 0.0);
  bool converged = false;
  for (it = 1; it <= std::max(1, maxiter) && d.ok; ++it) {
    std::vector<double> Hs, w, U;
    gram(V, k, Wm, k, Hs);
    if (!d.ok) break;
    for (int a = 0; a < k; ++a)  // symmetrise (rounding)
      for (int b = a + 1; b < k; ++b) Hs[(size_t)a * k + b] = Hs[(size_t)b * k + a] = 0.5 * (Hs[(size_t)a * k + b] + Hs[(size_t)b * k + a]);
    sym_eig(k, Hs, w, U);
    const int nx = std::min(nb, k);
    Sm.assign((size_t)k * nx, 0.0);
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < nx; ++b) Sm[(size_t)a * nx + b] = U[(size_t)a * k + b];
    theta.assign(w.begin(), w.begin() + nx);
    combine(V, k, Sm, nx, 0.0, X);
    combine(Wm, k, Sm, nx, 0.0, AX);
    // residuals R = AX - X theta (into T)
    d.check(cudaMemcpyAsync(T, AX, (size_t)n * nx * 8, cudaMemcpyDeviceToDevice, st), "copy R");
    {
      std::vector<double> D((size_t)nx * nx, 0.0);
      for (int b = 0; b < nx; ++b) D[(size_t)b * nx + b] = -theta[b];
      combine(X, nx, D, nx, 1.0, T);
    }
    std::vector<double> RR;
    gram(T, nx, T, nx, RR);
    if (!d.ok) break;
    double worst = 0.0;
    for (int b = 0; b < nroots; ++b) {
      res[b] = std::sqrt(std::max(RR[(size_t)b * nx + b], 0.0));
      worst = std::max(worst, res[b]);
    }
    if (worst <= tol) {
      converged = true;
      break;
    }
    // restart from the Ritz vectors when V is full
    if (k + nx > kmax) {
      d.check(cudaMemcpyAsync(V, X, (size_t)n * nx * 8, cudaMemcpyDeviceToDevice, st), "restart V");
      d.check(cudaMemcpyAsync(Wm, AX, (size_t)n * nx * 8, cudaMemcpyDeviceToDevice, st), "restart W");
      k = nx;
    }
    // corrections of the roots not yet converged (the extra block vectors
    // always): their residual columns, divided by theta - diag(H)
    std::vector<int> todo;
    for (int b = 0; b < nx; ++b)
      if (b >= nroots || res[b] > tol) todo.push_back(b);
    const int nu = (int)todo.size();
    {
      std::vector<double> sel((size_t)nx * nu, 0.0), th(nu);
      for (int c = 0; c < nu; ++c) {
        sel[(size_t)todo[c] * nu + c] = 1.0;
        th[c] = theta[todo[c]];
      }
      combine(T, nx, sel, nu, 0.0, AT);
      d.check(cudaMemcpyAsync(dth, th.data(), nu * 8, cudaMemcpyHostToDevice, st), "theta");
      k_precond<<<ewgrid, 256, 0, st>>>(n, AT, n, ddiag, dth, nu, T, n);
      d.check(cudaGetLastError(), "k_precond");
    }
    const int nt = std::min(orthonormalise(k, nu), kmax - k);
    if (nt <= 0) break;  // the space is exhausted (n small)
    d.check(cudaMemcpyAsync(V + (size_t)k * n, T, (size_t)n * nt * 8, cudaMemcpyDeviceToDevice, st), "append V");
    spmm(V + (size_t)k * n, Wm + (size_t)k * n, nt);
    k += nt;
  }
  std::vector<double> xo((size_t)n * nb);
  if (d.ok) {
    d.check(cudaMemcpyAsync(xo.data(), X, (size_t)n * std::min(nb, k) * 8, cudaMemcpyDeviceToHost, st), "copy X");
    d.check(cudaStreamSynchronize(st), "sync");
  }
  for (void* p : {(void*)drow, (void*)dcol, (void*)dval, (void*)ddiag, (void*)V, (void*)Wm, (void*)X, (void*)AX,
                  (void*)T, (void*)AT, (void*)dG, (void*)dS, (void*)dth})
    if (p) cudaFree(p);
  if (st) cudaStreamDestroy(st);
  if (!d.ok) {
    seterr(errbuf, errlen, "cipsi_davidson: " + d.err);
    return CIPSI_ERR_CUDA;
  }
  // each vector's largest component made positive (a fixed sign convention)
  for (int b = 0; b < nroots; ++b) {
    double* x = xo.data() + (size_t)b * n;
    int imax = 0;
    for (int i = 1; i < n; ++i)
      if (std::fabs(x[i]) > std::fabs(x[imax])) imax = i;
    const double sg = x[imax] < 0.0 ? -1.0 : 1.0;
    for (int i = 0; i < n; ++i) evecs[(size_t)b * n + i] = sg * x[i];
    evals[b] = theta[b];
    if (resid) resid[b] = res[b];
  }
  if (iters) *iters = it;
  if (!converged) {
    seterr(errbuf, errlen, "cipsi_davidson: not converged after " + std::to_string(maxiter) + " iterations");
    return CIPSI_ERR_OVERFLOW;
  }
  return CIPSI_OK;
}
