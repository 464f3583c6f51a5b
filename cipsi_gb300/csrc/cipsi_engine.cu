// cipsi_engine.cu -- host side of the GB300 engine for the CIPSI second-order
// perturbation / selection step: contexts, run planning, launches, results,
// the batched multi-geometry launch and the allocation-free entry point.
// The kernel itself is in pt2_kernel.cuh (algorithm described there).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "pt2_common.cuh"

using namespace cipsi_dev;

namespace {

// fixed-order Kahan reduction of the per-unit partial sums: block q sums
// column q; thread t takes a contiguous range of units, then thread 0 adds
// the per-thread sums in thread order (bitwise reproducible)
constexpr int kReduceThreads = 256;
__global__ void __launch_bounds__(kReduceThreads) k_reduce(const double* part, int nunits, int nq,
                                                           double* out) {
  __shared__ double ps[kReduceThreads], pc[kReduceThreads];
  const int q = blockIdx.x;
  const int per = (nunits + kReduceThreads - 1) / kReduceThreads;
  const int u0 = threadIdx.x * per, u1 = min(nunits, u0 + per);
  double s = 0.0, c = 0.0;
  for (int u = u0; u < u1; ++u) kahan_add(s, c, part[(long long)u * nq + q]);
  ps[threadIdx.x] = s;
  pc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, C = 0.0;
    for (int t = 0; t < kReduceThreads; ++t) {
      kahan_add(S, C, ps[t]);
      kahan_add(S, C, -pc[t]);
    }
    out[q] = S - C;
  }
}

// k_reduce for every geometry of a batch: block (q, b) sums column q of
// geometry b's per-unit partials into its reduced sums
__global__ void __launch_bounds__(kReduceThreads) k_reduce_batch(const Params* geo) {
  __shared__ double ps[kReduceThreads], pc[kReduceThreads];
  const Params& p = geo[blockIdx.y];
  const int nq = 5 * p.metat;
  const int q = blockIdx.x;
  if (q >= nq) return;
  const int nunits = p.nunits;
  const int per = (nunits + kReduceThreads - 1) / kReduceThreads;
  const int u0 = threadIdx.x * per, u1 = min(nunits, u0 + per);
  double s = 0.0, c = 0.0;
  for (int u = u0; u < u1; ++u) kahan_add(s, c, p.gen_part[(long long)u * nq + q]);
  ps[threadIdx.x] = s;
  pc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0.0, C = 0.0;
    for (int t = 0; t < kReduceThreads; ++t) {
      kahan_add(S, C, ps[t]);
      kahan_add(S, C, -pc[t]);
    }
    p.red[q] = S - C;
  }
}

// adjoint: sum the per-block slices [F | J | K | fmpb] over blocks
__global__ void k_slice_reduce(const double* sl, int nblocks, int stride, int nt, double* gF, double* gJ,
                               double* gK, double* gf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= stride) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += sl[(size_t)b * stride + i];
  if (i < nt) gF[i] += s;
  else if (i < 2 * nt) gJ[i - nt] = s;
  else if (i < 3 * nt) gK[i - 2 * nt] = s;
  else gf[i - 3 * nt] = s;
}

// Output offsets of the unit segments: unit_out[u] = base + the records of
// units u0..u-1 (exclusive scan of unit_nsel over [u0, u1), one block);
// *total = the records of [u0, u1).
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_scan_units(const int32_t* nsel, long long* out, int u0, int u1,
                                                             long long base, unsigned long long* total) {
  __shared__ long long wsum[kScanThreads / 32];
  __shared__ long long carry;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid == 0) carry = base;
  __syncthreads();
  for (int c0 = u0; c0 < u1; c0 += kScanThreads) {
    const int u = c0 + tid;
    const long long v = u < u1 ? nsel[u] : 0;
    long long incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const long long y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) wsum[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      long long w = wsum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const long long before = carry + (wid ? wsum[wid - 1] : 0) + (incl - v);
    if (u < u1) out[u] = before;
    __syncthreads();
    if (tid == 0) carry += wsum[kScanThreads / 32 - 1];
    __syncthreads();
  }
  if (tid == 0 && total) *total = (unsigned long long)(carry - base);
}

// Records of units [u0, u1) from their pool segments to the output arrays
// at unit_out[u] - out_base (unit order), with the owner (1-based generator
// index, 0 for pertu's candidates) taken from the unit; records beyond
// out_cap are dropped (the run reports an overflow).
struct GatherArgs {
  const uint64_t* pool_bits;
  const double* pool_xam;
  const double* pool_evp;
  long long pool_cap;
  const long long* unit_pool;
  const int32_t* unit_nsel;
  const long long* unit_out;
  const int32_t* unit_g;
  const int32_t* gens;
  int u0, u1, words, metat;
  long long out_base, out_cap;
  uint64_t* out_bits;
  int32_t* out_owner;
  double* out_xam;
  double* out_evp;
};
__global__ void __launch_bounds__(256) k_gather(GatherArgs a) {
  for (int u = a.u0 + blockIdx.x; u < a.u1; u += gridDim.x) {
    const int n = a.unit_nsel[u];
    if (n == 0) continue;
    const long long src = a.unit_pool[u];
    const long long dst = a.unit_out[u] - a.out_base;
    const int k = a.gens[a.unit_g[u]];
    const int owner = k < 0 ? 0 : k + 1;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const long long d = dst + i, q = src + i;
      if (d >= a.out_cap || q >= a.pool_cap) break;
      for (int w = 0; w < a.words; ++w) a.out_bits[d * a.words + w] = a.pool_bits[q * a.words + w];
      a.out_owner[d] = owner;
      a.out_xam[d] = a.pool_xam[q];
      for (int m = 0; m < a.metat; ++m) a.out_evp[d * a.metat + m] = a.pool_evp[q * a.metat + m];
    }
  }
}

// zero what every geometry of a batch accumulates into (block b: geometry b)
__global__ void k_batch_clear(const Params* geo) {
  const Params& p = geo[blockIdx.x];
  const int ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  for (int i = threadIdx.x; i < ncount; i += blockDim.x) p.counters[i] = 0ull;
  for (int i = threadIdx.x; i < 2 * kNClass * kMaxRoots; i += blockDim.x) p.hist_tab[i] = 0.0;
  const long long npart = (long long)max(p.nunits, 1) * 5 * p.metat;
  for (long long i = threadIdx.x; i < npart; i += blockDim.x) p.gen_part[i] = 0.0;
  if (threadIdx.x == 0 && p.pool_count) *p.pool_count = 0ull;
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
  double* deri64 = nullptr;  // FP64 storage of (pq|rs) (cipsi_set_integrals_f64store)
  double* deri_w = nullptr;  // the real*4 (pq|rs) widened to double (small integral sets)
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
  uint64_t* dlr_ent = nullptr;
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
  // record path: per-CTA staging (slot-indexed), the pool of unit segments,
  // the unit table (segment, records, output offset)
  uint64_t* dst_bits = nullptr;
  double *dst_xam = nullptr, *dst_evp = nullptr;
  uint32_t* dst_mask = nullptr;
  size_t st_slots = 0;  // allocated grid x st_cap slots
  uint64_t* dpool_bits = nullptr;
  double *dpool_xam = nullptr, *dpool_evp = nullptr;
  long long pool_cap = 0;
  unsigned long long* dpool_count = nullptr;
  long long* dunit_pool = nullptr;
  int32_t* dunit_nsel = nullptr;
  long long* dunit_out = nullptr;
  unsigned long long* dscan_total = nullptr;
  int unit_tab_cap = 0;
  // streamed runs (cipsi_run_pt2_stream): two device record buffers, a copy
  // stream, a ring of pinned host buffers; per-unit record counts of the
  // last run, reused to size the chunks of a run with the same plan
  uint64_t* dout_bits[2] = {nullptr, nullptr};
  int32_t* dout_owner[2] = {nullptr, nullptr};
  double* dout_xam[2] = {nullptr, nullptr};
  double* dout_evp[2] = {nullptr, nullptr};
  long long out_cap = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_gathered[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
  cudaEvent_t ev_host[2] = {nullptr, nullptr};
  void* hbuf[2] = {nullptr, nullptr};
  long long hbuf_cap = 0;
  int stream_chunks = 0;  // chunks of the last streamed run
  std::vector<int32_t> last_unit_nsel;
  unsigned long long last_plan_sig = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk = nullptr;  // evk: end of k_pt2
  long long last_launches = 0;
  // launch tuning (cipsi_set_tuning): R blocks per work unit for generators
  // of excitation rank >= 2 (rank 0/1 generators get one block per unit),
  // and CTAs per SM (0 = as many as the shared-memory L_R size allows)
  int tune_r_chunk = 6;
  int tune_ctas = 0;
  // set by a batched run: the event that marks its end (fetch waits on it),
  // and whether ev0/ev1 time this context's own launch
  cudaEvent_t ext_done = nullptr;
  bool ev_valid = false;
  // bumped whenever a device buffer is (re)allocated: a batch built on this
  // context refuses to run after that
  unsigned long long buf_gen = 0;
  // pending run
  int ngen = 0;
  int nclass = kNClass;
  bool pending = false;
  cipsi_opts last_opts{};
  long long nsel = 0;  // records of the last fetched run
  // caller-provided record arrays in pinned host memory (cipsi_set_selection_sink):
  // the kernel writes the unit-60 records there directly
  bool sink = false;
  uint64_t* sink_bits = nullptr;
  int32_t* sink_owner = nullptr;
  double *sink_xam = nullptr, *sink_evp = nullptr;
  long long sink_cap = 0;
  void* sink_host[4] = {nullptr, nullptr, nullptr, nullptr};  // the caller's addresses
  // the Hamiltonian over the space (cipsi_hamiltonian_build): phases of the
  // determinants, the caller's Fock matrix when given, pairs by rows
  int8_t* dsigma = nullptr;
  double* dFraw = nullptr;
  int32_t* dh_count = nullptr;
  long long* dh_rowptr = nullptr;
  int32_t* dh_col = nullptr;
  double* dh_val = nullptr;
  long long h_cap = 0;
  std::vector<long long> h_rowptr;
  bool have_h = false;
  float h_ms = 0.f;
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

// Integral sets up to this size are also kept widened to double on the
// device (13 MB for 60 orbitals; the 120-orbital set stays real*4 only, so
// that it still fits in L2).  The values are the real*4 ones, exactly; the
// kernel then loads a double per integral instead of converting a float.
constexpr size_t kWidenMaxBytes = (size_t)48 << 20;

__global__ void k_widen(const float* __restrict__ in, double* __restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}

template <typename T>
int upload(cipsi_ctx* ctx, T** dptr, const T* h, size_t n) {
  if (*dptr) cudaFree(*dptr);
  *dptr = nullptr;
  ++ctx->buf_gen;
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
  CK(cudaEventCreate(&ctx->evk));
  return CIPSI_OK;
}

void cipsi_ctx_destroy(cipsi_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  dfree(ctx->dS); dfree(ctx->dygen); dfree(ctx->dyef); dfree(ctx->dnesp); dfree(ctx->dc);
  dfree(ctx->deri); dfree(ctx->dpairtab); dfree(ctx->dntttt); dfree(ctx->dF); dfree(ctx->dJ);
  dfree(ctx->dK); dfree(ctx->dfmpb); dfree(ctx->dorbsym); dfree(ctx->dgens); dfree(ctx->dgmask);
  dfree(ctx->deri64);
  dfree(ctx->deri_w);
  dfree(ctx->dunits);
  dfree(ctx->dnb_j); dfree(ctx->dnb_em); dfree(ctx->dlr_ent); dfree(ctx->dgen_part);
  dfree(ctx->dcounters); dfree(ctx->dhist_tab); dfree(ctx->dred); dfree(ctx->dwork);
  dfree(ctx->dsel_bits); dfree(ctx->dsel_owner); dfree(ctx->dsel_xam); dfree(ctx->dsel_evp);
  dfree(ctx->dst_bits); dfree(ctx->dst_xam); dfree(ctx->dst_evp); dfree(ctx->dst_mask);
  dfree(ctx->dpool_bits); dfree(ctx->dpool_xam); dfree(ctx->dpool_evp); dfree(ctx->dpool_count);
  dfree(ctx->dunit_pool); dfree(ctx->dunit_nsel); dfree(ctx->dunit_out); dfree(ctx->dscan_total);
  dfree(ctx->dsigma); dfree(ctx->dFraw); dfree(ctx->dh_count); dfree(ctx->dh_rowptr);
  dfree(ctx->dh_col); dfree(ctx->dh_val);
  for (int i = 0; i < 2; ++i) {
    dfree(ctx->dout_bits[i]); dfree(ctx->dout_owner[i]); dfree(ctx->dout_xam[i]); dfree(ctx->dout_evp[i]);
    if (ctx->hbuf[i]) cudaFreeHost(ctx->hbuf[i]);
    for (cudaEvent_t e : {ctx->ev_gathered[i], ctx->ev_copied[i], ctx->ev_host[i]})
      if (e) cudaEventDestroy(e);
  }
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->evk) cudaEventDestroy(ctx->evk);
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
  if (ctx->deri64) {
    ++ctx->buf_gen;
    dfree(ctx->deri64);
  }
  dfree(ctx->deri_w);
  if ((size_t)ninte * sizeof(double) <= kWidenMaxBytes) {
    CK(cudaMalloc((void**)&ctx->deri_w, (size_t)ninte * sizeof(double)));
    const int grid = (int)std::min<int64_t>((ninte + 255) / 256, 4096);
    k_widen<<<grid, 256, 0, ctx->stream>>>(ctx->deri, ctx->deri_w, ninte);
    CK(cudaGetLastError());
  }
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

int cipsi_set_integrals_f64store(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                                 const double* f, const double* aj, const double* ak,
                                 const int16_t* ij0, const int32_t* ntttt, const double* pqrs,
                                 int64_t ninte) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (!pqrs) return fail(ctx, CIPSI_ERR_ARG, "pqrs is null");
  int rc = set_integrals_common(ctx, itsym, its, f, aj, ak, ij0, ntttt, ninte);
  if (rc) return rc;
  if ((rc = upload(ctx, &ctx->deri64, pqrs, (size_t)ninte))) return rc;
  dfree(ctx->deri_w);
  if (!ctx->deri) {
    const float zero = 0.f;
    if ((rc = upload(ctx, &ctx->deri, &zero, 1))) return rc;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->have_int = true;
  return CIPSI_OK;
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



namespace {

int roots_pad(int mt) { return mt <= 1 ? 1 : mt <= 2 ? 2 : mt <= 4 ? 4 : 8; }

int check_run_args(cipsi_ctx* ctx, const cipsi_opts* o) {
  if (!ctx || !o) return CIPSI_ERR_ARG;
  if (!ctx->have_int || !ctx->have_space || !ctx->have_roots)
    return fail(ctx, CIPSI_ERR_STATE, "run before set_integrals / set_space / set_roots");
  if (o->nclass < 2 || o->nclass > kNClass) return fail(ctx, CIPSI_ERR_ARG, "nclass must be in [2, 10]");
  for (int i = 0; i + 1 < o->nclass; ++i)
    if (!(o->aval[i] >= 0.0) || (i > 0 && !(o->aval[i] > o->aval[i - 1])))
      return fail(ctx, CIPSI_ERR_ARG, "aval must be non-negative and increasing");
  return CIPSI_OK;
}

// Generators, their allowed rank changes and the work units of one run.
struct RunPlan {
  std::vector<int32_t> gens;   // generator indices (0-based); -1 = pertu block
  std::vector<uint8_t> gmask;  // allowed rank changes, bit (D + 2)
  std::vector<int32_t> ug, ur0, ur1;
  std::vector<long long> uslots;  // candidate slots per unit (block_candidates over its allowed blocks)
  long long max_slots = 0;
  bool pertu_ref = false, pertu_mono = false;
};

void plan_run(const cipsi_ctx* ctx, const cipsi_opts* o, int r_chunk, RunPlan& pl) {
  const int ncf = ctx->d.ncf, W = ctx->W;
  // flags on the content of S (pertu.f:52-61)
  bool yd = false, ym = false, yf = false;
  for (int k = 0; k < ncf; ++k) {
    if (ctx->rank[k] == 1) ym = true;
    if (ctx->rank[k] == 0) yd = true;
    if (ctx->rank[k] == 2) yf = true;
  }
  if (ym) yf = true;
  std::vector<int32_t>& gens = pl.gens;
  std::vector<uint8_t>& gmask = pl.gmask;
  const bool pertu_ref = yf && !yd && ctx->d.isym == 1;  // isz == 0, !yion
  const bool pertu_mono = yf && ym;
  pl.pertu_ref = pertu_ref;
  pl.pertu_mono = pertu_mono;
  if (o->run_pertu && (pertu_ref || pertu_mono)) {
    gens.push_back(-1);
    gmask.push_back(0);
  }
  for (int k = 0; k < ncf; ++k) {
    if (!ctx->ygen[k] || ctx->ysaut[k]) continue;
    if (o->gen_mask && !o->gen_mask[k]) continue;
    const int nec = ctx->rank[k];
    // allowed rank changes, bit (D + 2); D = +2 (diexcit) always
    // (igene.f:34-35, 89-90, 199-200, 296-298)
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
  // work units: a generator's R blocks that have an allowed rank-change class
  // are split into chunks (one block per unit for generators of rank 0 and 1,
  // which meet most of S; r_chunk blocks for the others), so one heavy
  // generator does not serialise on one SM; low-rank generators are queued
  // first.
  const int kRChunkHigh = std::max(1, r_chunk);
  constexpr int kPertuChunk = 128;
  std::vector<int32_t>& ug = pl.ug;
  std::vector<int32_t>& ur0 = pl.ur0;
  std::vector<int32_t>& ur1 = pl.ur1;
  const int n = ctx->d.norb, noca = ctx->d.noca, nel = 2 * noca;
  const int nR = nel + nel * (nel - 1) / 2;
  std::vector<int> order(ngen);
  for (int g = 0; g < ngen; ++g) order[g] = g;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    const int ra = gens[a] < 0 ? -1 : ctx->rank[gens[a]];
    const int rb = gens[b] < 0 ? -1 : ctx->rank[gens[b]];
    return ra < rb;
  });
  std::vector<int> hfe(nel), spe(nel);
  auto push = [&](int g, int a, int b, long long slots) {
    ug.push_back(g);
    ur0.push_back(a);
    ur1.push_back(b);
    pl.uslots.push_back(slots);
    pl.max_slots = std::max(pl.max_slots, slots);
  };
  for (int g : order) {
    const int k = gens[g];
    if (k < 0) {
      const int ntot = (pertu_ref ? 1 : 0) + (pertu_mono ? 2 * noca * (n - noca) : 0);
      for (int t = 0; t < ntot; t += kPertuChunk) push(g, t, std::min(ntot, t + kPertuChunk), std::min(ntot, t + kPertuChunk) - t);
      continue;
    }
    // electrons of k: alpha orbitals ascending, then beta; HF-occupied?
    int ne = 0, nes[2] = {0, 0};
    for (int sp = 0; sp < 2; ++sp)
      for (int orb = 0; orb < n; ++orb)
        if ((ctx->Sbits[(size_t)k * 2 * W + sp * W + (orb >> 6)] >> (orb & 63)) & 1ull) {
          spe[ne] = sp;
          hfe[ne++] = orb < noca;
          ++nes[sp];
        }
    const int nv[2] = {n - nes[0], n - nes[1]};
    const uint8_t m = gmask[g];
    // rank-change class allowed for block r?  Its candidates (slots).
    auto block = [&](int r, long long& cands) {
      int hfR, nRr, e1, e2 = -1;
      if (r < nel) {
        e1 = r;
        hfR = hfe[r];
        nRr = 1;
      } else {
        int t = r - nel;
        e1 = 0;
        while (t >= nel - 1 - e1) {
          t -= nel - 1 - e1;
          ++e1;
        }
        e2 = e1 + 1 + t;
        hfR = hfe[e1] + hfe[e2];
        nRr = 2;
      }
      cands = block_candidates(nRr, e2 >= 0 && spe[e1] == spe[e2], nv[spe[e1]], nv[0], nv[1]);
      for (int aV = 0; aV <= nRr; ++aV)
        if (m & (1u << (hfR + aV - nRr + 2))) return true;
      return false;
    };
    const int kRChunk = ctx->rank[k] <= 1 ? 1 : kRChunkHigh;
    int cnt = 0, start = -1, last = -1;
    long long slots = 0;
    for (int r = 0; r < nR; ++r) {
      long long c;
      if (!block(r, c)) continue;
      if (start < 0) start = r;
      last = r;
      slots += c;
      if (++cnt == kRChunk) {
        push(g, start, r + 1, slots);
        cnt = 0;
        start = -1;
        slots = 0;
      }
    }
    if (start >= 0) push(g, start, last + 1, slots);
  }
}

// Shared-memory L_R capacity, dynamic shared memory and CTAs per SM.
// ctas: 0 = 200 KB per CTA (two CTAs per SM when the list fits in half),
// 1 = one CTA per SM, 2 = sized so that two CTAs fit per SM.
struct LaunchShape {
  int lr_cap;
  size_t smem;
  int blocks_per_sm;
};

// adj: the adjoint launch.  Its static shared memory exceeds the forward's
// by ~4 KB (the per-block dE/dhdig and dE/dhmp sums), which its L_R list
// gives back so that two CTAs still fit per SM; it never fills the
// epilogue queues (its drains find them empty), so they take no space.
LaunchShape launch_shape(int W, int R, int ncf_max, int ctas, bool adj = false) {
  const size_t per_entry = 8;  // compact L_R entry
  const size_t qbytes = adj ? 0 : (size_t)(kThreads / 32) * queue_bytes(W, R);
  // two CTAs per SM unless one is asked for: the part of a long L_R list
  // beyond shared memory is read from the block's global scratch, 8 bytes
  // per entry, which costs less than halving the resident warps
  // (the kernel's static shared memory, ~28 KB, comes on top: two CTAs of
  // 82 + 28 KB, or one of 192 + 28 KB, fit the SM's 228 KB)
  const size_t smem_total = (ctas == 1 ? (size_t)192 * 1024 : (size_t)82 * 1024) - (adj ? 4096 : 0);
  const size_t smem_budget = smem_total > qbytes + 16 ? smem_total - qbytes - 16 : 0;
  LaunchShape ls;
  ls.lr_cap = (int)std::min<size_t>((size_t)ncf_max, smem_budget / per_entry);
  ls.smem = (((size_t)ls.lr_cap * per_entry + 15) & ~(size_t)15) + qbytes + 16;
  ls.blocks_per_sm = ctas == 1 ? 1 : ls.smem <= (adj ? 82 : 86) * 1024 ? 2 : 1;
  return ls;
}

// The record pool (unit segments), for `cap` records.
int grow_pool(cipsi_ctx* ctx, long long cap) {
  const int W = ctx->W, mt = ctx->d.metat;
  ++ctx->buf_gen;
  dfree(ctx->dpool_bits); dfree(ctx->dpool_xam); dfree(ctx->dpool_evp);
  ctx->pool_cap = 0;
  CK(cudaMalloc(&ctx->dpool_bits, (size_t)cap * 2 * W * sizeof(uint64_t)));
  CK(cudaMalloc(&ctx->dpool_xam, (size_t)cap * sizeof(double)));
  CK(cudaMalloc(&ctx->dpool_evp, (size_t)cap * mt * sizeof(double)));
  ctx->pool_cap = cap;
  return CIPSI_OK;
}

// The device record arrays (cipsi_selection_get / raw), for `cap` records.
int grow_sel(cipsi_ctx* ctx, long long cap) {
  const int W = ctx->W, mt = ctx->d.metat;
  ++ctx->buf_gen;
  dfree(ctx->dsel_bits); dfree(ctx->dsel_owner); dfree(ctx->dsel_xam); dfree(ctx->dsel_evp);
  ctx->sel_cap = 0;
  CK(cudaMalloc(&ctx->dsel_bits, (size_t)cap * 2 * W * sizeof(uint64_t)));
  CK(cudaMalloc(&ctx->dsel_owner, (size_t)cap * sizeof(int32_t)));
  CK(cudaMalloc(&ctx->dsel_xam, (size_t)cap * sizeof(double)));
  CK(cudaMalloc(&ctx->dsel_evp, (size_t)cap * mt * sizeof(double)));
  ctx->sel_cap = cap;
  return CIPSI_OK;
}

// Device buffers of one run on ctx (generator and unit lists, per-unit
// partial sums, counters, histogram, records), sized for the plan; the lists
// are uploaded on stream st.
int prepare_run(cipsi_ctx* ctx, const RunPlan& pl, cudaStream_t st) {
  const int mt = ctx->d.metat;
  const int ngen = (int)pl.gens.size(), nunits = (int)pl.ug.size();
  ctx->ngen = ngen;
  ctx->nunits = nunits;
  if (ngen > ctx->gens_cap) {
    ++ctx->buf_gen;
    dfree(ctx->dgens); dfree(ctx->dgmask);
    CK(cudaMalloc(&ctx->dgens, (size_t)std::max(ngen, 1) * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dgmask, (size_t)std::max(ngen, 1)));
    ctx->gens_cap = ngen;
  }
  if (nunits > ctx->units_cap) {
    ++ctx->buf_gen;
    dfree(ctx->dunits);
    CK(cudaMalloc(&ctx->dunits, (size_t)std::max(nunits, 1) * 3 * sizeof(int32_t)));
    ctx->units_cap = nunits;
  }
  if (ngen) {
    CK(cudaMemcpyAsync(ctx->dgens, pl.gens.data(), ngen * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(ctx->dgmask, pl.gmask.data(), ngen, cudaMemcpyHostToDevice, st));
  }
  if (nunits) {
    ctx->hunits.resize((size_t)3 * nunits);
    std::copy(pl.ug.begin(), pl.ug.end(), ctx->hunits.begin());
    std::copy(pl.ur0.begin(), pl.ur0.end(), ctx->hunits.begin() + nunits);
    std::copy(pl.ur1.begin(), pl.ur1.end(), ctx->hunits.begin() + 2 * nunits);
    CK(cudaMemcpyAsync(ctx->dunits, ctx->hunits.data(), (size_t)3 * nunits * sizeof(int32_t),
                       cudaMemcpyHostToDevice, st));
  }
  const size_t nq = (size_t)5 * mt;
  if ((size_t)std::max(nunits, 1) * nq > ctx->gen_part_cap) {
    ++ctx->buf_gen;
    dfree(ctx->dgen_part);
    ctx->gen_part_cap = (size_t)std::max(nunits, 1) * nq;
    CK(cudaMalloc(&ctx->dgen_part, ctx->gen_part_cap * sizeof(double)));
  }
  // counters [C_NCOUNTERS] + dpivot + nom[10] + nam[10*8]
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  if (!ctx->dcounters) {
    ++ctx->buf_gen;
    CK(cudaMalloc(&ctx->dcounters, ncount * sizeof(unsigned long long)));
    CK(cudaMalloc(&ctx->dhist_tab, 2 * kNClass * kMaxRoots * sizeof(double)));
    CK(cudaMalloc(&ctx->dred, 5 * kMaxRoots * sizeof(double)));
    CK(cudaMalloc(&ctx->dwork, sizeof(int)));
  }
  if (ctx->pool_cap == 0) {
    const int rc = grow_pool(ctx, 1 << 20);
    if (rc) return rc;
  }
  if (ctx->sel_cap == 0) {
    const int rc = grow_sel(ctx, 1 << 20);
    if (rc) return rc;
  }
  if (nunits > ctx->unit_tab_cap) {
    ++ctx->buf_gen;
    dfree(ctx->dunit_pool); dfree(ctx->dunit_nsel); dfree(ctx->dunit_out);
    CK(cudaMalloc(&ctx->dunit_pool, (size_t)nunits * sizeof(long long)));
    CK(cudaMalloc(&ctx->dunit_nsel, (size_t)nunits * sizeof(int32_t)));
    CK(cudaMalloc(&ctx->dunit_out, (size_t)nunits * sizeof(long long)));
    ctx->unit_tab_cap = nunits;
  }
  if (!ctx->dpool_count) {
    ++ctx->buf_gen;
    CK(cudaMalloc(&ctx->dpool_count, sizeof(unsigned long long)));
    CK(cudaMalloc(&ctx->dscan_total, sizeof(unsigned long long)));
  }
  return CIPSI_OK;
}

// Per-CTA record staging for `grid` CTAs of st_cap slots each.
int ensure_staging(cipsi_ctx* ctx, int grid, long long st_cap) {
  const size_t slots = (size_t)grid * (size_t)st_cap;
  if (slots <= ctx->st_slots && ctx->dst_mask) return CIPSI_OK;
  ++ctx->buf_gen;
  dfree(ctx->dst_bits); dfree(ctx->dst_xam); dfree(ctx->dst_evp); dfree(ctx->dst_mask);
  const int W = ctx->W, mt = ctx->d.metat;
  CK(cudaMalloc(&ctx->dst_bits, slots * 2 * W * sizeof(uint64_t)));
  CK(cudaMalloc(&ctx->dst_xam, slots * sizeof(double)));
  CK(cudaMalloc(&ctx->dst_evp, slots * mt * sizeof(double)));
  CK(cudaMalloc(&ctx->dst_mask, slots / 32 * sizeof(uint32_t)));
  CK(cudaMemset(ctx->dst_mask, 0, slots / 32 * sizeof(uint32_t)));
  ctx->st_slots = slots;
  return CIPSI_OK;
}

// Staging slots per CTA for a plan: its largest unit, in whole mask words.
long long staging_cap(const RunPlan& pl) { return std::max<long long>(32, (pl.max_slots + 31) / 32 * 32); }

// Kernel parameters of one run on ctx (everything but the neighbour scratch
// and the L_R capacity).
void fill_params(const cipsi_ctx* ctx, const cipsi_opts* o, const RunPlan& pl, Params& p) {
  const int mt = ctx->d.metat, nunits = (int)pl.ug.size();
  p.norb = ctx->d.norb;
  p.noca = ctx->d.noca;
  p.nel = 2 * ctx->d.noca;
  p.ncf = ctx->d.ncf;
  p.metat = mt;
  p.nsym = ctx->d.nsym;
  p.isym = ctx->d.isym;
  p.ngen = (int)pl.gens.size();
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
  p.eri64 = ctx->deri64 ? ctx->deri64 : ctx->deri_w;
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
  p.pertu_ref = pl.pertu_ref ? 1 : 0;
  p.pertu_mono = pl.pertu_mono ? 1 : 0;
  p.gen_part = ctx->dgen_part;
  p.counters = ctx->dcounters;
  p.dpivot_bits = ctx->dcounters + C_NCOUNTERS;
  p.hist_nom = ctx->dcounters + C_NCOUNTERS + 1;
  p.hist_nam = ctx->dcounters + C_NCOUNTERS + 1 + kNClass;
  p.hist_tab = ctx->dhist_tab;
  p.red = ctx->dred;
  p.rec_mode = 1;
  p.st_cap = (int)staging_cap(pl);
  p.st_bits = ctx->dst_bits;
  p.st_xam = ctx->dst_xam;
  p.st_evp = ctx->dst_evp;
  p.st_mask = ctx->dst_mask;
  p.pool_bits = ctx->dpool_bits;
  p.pool_xam = ctx->dpool_xam;
  p.pool_evp = ctx->dpool_evp;
  p.pool_cap = ctx->pool_cap;
  p.pool_count = ctx->dpool_count;
  p.unit_pool = ctx->dunit_pool;
  p.unit_nsel = ctx->dunit_nsel;
  p.work = ctx->dwork;
}

// Output arrays of a run's records: the caller's pinned sink or the
// context's device arrays.
void record_target(const cipsi_ctx* ctx, GatherArgs& a) {
  if (ctx->sink) {
    a.out_bits = ctx->sink_bits;
    a.out_owner = ctx->sink_owner;
    a.out_xam = ctx->sink_xam;
    a.out_evp = ctx->sink_evp;
    a.out_cap = ctx->sink_cap;
  } else {
    a.out_bits = ctx->dsel_bits;
    a.out_owner = ctx->dsel_owner;
    a.out_xam = ctx->dsel_xam;
    a.out_evp = ctx->dsel_evp;
    a.out_cap = ctx->sel_cap;
  }
}

// Scan + gather of units [u0, u1) of run `p` (records at output offset
// out_base.. of the target in `a`), enqueued on st.
cudaError_t enqueue_gather(const cipsi_ctx* ctx, const Params& p, int u0, int u1, long long out_base, GatherArgs a,
                           cudaStream_t st, int dev_sms) {
  if (u1 <= u0) return cudaSuccess;
  k_scan_units<<<1, kScanThreads, 0, st>>>(p.unit_nsel, ctx->dunit_out, u0, u1, out_base, ctx->dscan_total);
  a.pool_bits = p.pool_bits;
  a.pool_xam = p.pool_xam;
  a.pool_evp = p.pool_evp;
  a.pool_cap = p.pool_cap;
  a.unit_pool = p.unit_pool;
  a.unit_nsel = p.unit_nsel;
  a.unit_out = ctx->dunit_out;
  a.unit_g = p.unit_g;
  a.gens = p.gens;
  a.u0 = u0;
  a.u1 = u1;
  a.words = 2 * ctx->W;
  a.metat = ctx->d.metat;
  a.out_base = out_base;
  const int grid = std::max(1, std::min(u1 - u0, 4 * dev_sms));
  k_gather<<<grid, 256, 0, st>>>(a);
  return cudaGetLastError();
}

// Per-CTA neighbour scratch (nb_j, nb_emask, lr_ent) for `grid` CTAs.
int ensure_neighbour_scratch(cipsi_ctx* ctx, int grid) {
  if ((size_t)grid <= ctx->scratch_blocks && ctx->dnb_j) return CIPSI_OK;
  const int ncf = ctx->d.ncf;
  ++ctx->buf_gen;
  dfree(ctx->dnb_j); dfree(ctx->dnb_em); dfree(ctx->dlr_ent);
  CK(cudaMalloc(&ctx->dnb_j, (size_t)grid * ncf * sizeof(int32_t)));
  CK(cudaMalloc(&ctx->dnb_em, (size_t)grid * ncf * sizeof(uint64_t)));
  CK(cudaMalloc(&ctx->dlr_ent, (size_t)grid * ncf * sizeof(uint64_t)));
  ctx->scratch_blocks = grid;
  return CIPSI_OK;
}

// the plain (one geometry) forward launch of k_pt2<W, R>
cudaError_t launch_plain(const Params& p, int W, int R, int grid, size_t smem, cudaStream_t st) {
  if (W == 1)
    return R == 1 ? launch_pt2<1, 1, false>(p, BatchArgs{}, grid, smem, st)
         : R == 2 ? launch_pt2<1, 2, false>(p, BatchArgs{}, grid, smem, st)
         : R == 4 ? launch_pt2<1, 4, false>(p, BatchArgs{}, grid, smem, st)
                  : launch_pt2<1, 8, false>(p, BatchArgs{}, grid, smem, st);
  return R == 1 ? launch_pt2<2, 1, false>(p, BatchArgs{}, grid, smem, st)
       : R == 2 ? launch_pt2<2, 2, false>(p, BatchArgs{}, grid, smem, st)
       : R == 4 ? launch_pt2<2, 4, false>(p, BatchArgs{}, grid, smem, st)
                : launch_pt2<2, 8, false>(p, BatchArgs{}, grid, smem, st);
}

}  // namespace

extern "C" {

int cipsi_set_tuning(cipsi_ctx* ctx, int32_t r_chunk, int32_t ctas_per_sm) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (r_chunk < 1 || r_chunk > 4096) return fail(ctx, CIPSI_ERR_ARG, "r_chunk must be in [1, 4096]");
  if (ctas_per_sm < 0 || ctas_per_sm > 2) return fail(ctx, CIPSI_ERR_ARG, "ctas_per_sm must be 0, 1 or 2");
  ctx->tune_r_chunk = r_chunk;
  ctx->tune_ctas = ctas_per_sm;
  return CIPSI_OK;
}

int cipsi_set_selection_sink(cipsi_ctx* ctx, uint64_t* bits, int32_t* owner, double* xam, double* evp,
                             int64_t capacity) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "an asynchronous run is pending: fetch its result first");
  ++ctx->buf_gen;
  if (!bits) {
    ctx->sink = false;
    ctx->sink_bits = nullptr;
    ctx->sink_owner = nullptr;
    ctx->sink_xam = ctx->sink_evp = nullptr;
    ctx->sink_cap = 0;
    ctx->nsel = 0;
    return CIPSI_OK;
  }
  if (!owner || !xam || !evp || capacity < 1)
    return fail(ctx, CIPSI_ERR_ARG, "selection sink: null array or capacity < 1");
  CK(cudaSetDevice(ctx->device));
  void* host[4] = {bits, owner, xam, evp};
  void* dev[4] = {nullptr, nullptr, nullptr, nullptr};
  for (int i = 0; i < 4; ++i) {
    cudaPointerAttributes a{};
    CK(cudaPointerGetAttributes(&a, host[i]));
    if (a.type != cudaMemoryTypeHost)
      return fail(ctx, CIPSI_ERR_ARG, "selection sink: arrays must be pinned host memory (cudaHostAlloc or "
                                      "cudaHostRegister)");
    CK(cudaHostGetDevicePointer(&dev[i], host[i], 0));
  }
  ctx->sink = true;
  ctx->sink_bits = static_cast<uint64_t*>(dev[0]);
  ctx->sink_owner = static_cast<int32_t*>(dev[1]);
  ctx->sink_xam = static_cast<double*>(dev[2]);
  ctx->sink_evp = static_cast<double*>(dev[3]);
  ctx->sink_cap = capacity;
  for (int i = 0; i < 4; ++i) ctx->sink_host[i] = host[i];
  ctx->nsel = 0;
  return CIPSI_OK;
}

int cipsi_run_pt2_async(cipsi_ctx* ctx, const cipsi_opts* o) {
  int rc = check_run_args(ctx, o);
  if (rc) return rc;
  CK(cudaSetDevice(ctx->device));
  const int ncf = ctx->d.ncf, W = ctx->W, mt = ctx->d.metat;
  RunPlan pl;
  plan_run(ctx, o, ctx->tune_r_chunk, pl);
  const int nunits = (int)pl.ug.size();
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const LaunchShape ls = launch_shape(W, roots_pad(mt), ncf, ctx->tune_ctas);
  const int grid = std::max(1, std::min(nunits, dev_sms * ls.blocks_per_sm));
  rc = ensure_neighbour_scratch(ctx, grid);
  if (rc) return rc;
  rc = prepare_run(ctx, pl, ctx->stream);
  if (rc) return rc;
  rc = ensure_staging(ctx, grid, staging_cap(pl));
  if (rc) return rc;
  const size_t nq = (size_t)5 * mt;
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  CK(cudaMemsetAsync(ctx->dcounters, 0, ncount * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dhist_tab, 0, 2 * kNClass * kMaxRoots * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->dwork, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->dpool_count, 0, sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dgen_part, 0, (size_t)std::max(nunits, 1) * nq * sizeof(double), ctx->stream));

  Params p{};
  fill_params(ctx, o, pl, p);
  p.nb_j = ctx->dnb_j;
  p.nb_emask = ctx->dnb_em;
  p.lr_ent = ctx->dlr_ent;
  p.lr_cap = ls.lr_cap;
  p.nb_stride = ncf;

  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (nunits > 0) {
    cudaError_t e = launch_plain(p, W, roots_pad(mt), grid, ls.smem, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_pt2 launch: ") + cudaGetErrorString(e));
    CK(cudaEventRecord(ctx->evk, ctx->stream));
    ctx->last_launches = 4;
    GatherArgs ga{};
    record_target(ctx, ga);
    e = enqueue_gather(ctx, p, 0, nunits, 0, ga, ctx->stream, dev_sms);
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("record gather: ") + cudaGetErrorString(e));
    k_reduce<<<(unsigned)nq, kReduceThreads, 0, ctx->stream>>>(ctx->dgen_part, nunits, (int)nq, ctx->dred);
    CK(cudaGetLastError());
  } else {
    CK(cudaEventRecord(ctx->evk, ctx->stream));
    ctx->last_launches = 0;
    CK(cudaMemsetAsync(ctx->dred, 0, nq * sizeof(double), ctx->stream));
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  ctx->ev_valid = true;
  ctx->nclass = o->nclass;
  ctx->pending = true;
  ctx->last_opts = *o;
  return CIPSI_OK;
}

int cipsi_fetch_result(cipsi_ctx* ctx, cipsi_result* r) {
  if (!ctx || !r) return CIPSI_ERR_ARG;
  if (!ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "fetch_result without a run");
  CK(cudaSetDevice(ctx->device));
  if (ctx->ext_done) {
    CK(cudaEventSynchronize(ctx->ext_done));
    ctx->ext_done = nullptr;
  }
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
  float ms = -1.f, mk = -1.f;  // batched runs: the batch's time is reported by the batch
  if (ctx->ev_valid) {
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    CK(cudaEventElapsedTime(&mk, ctx->ev0, ctx->evk));
  }
  r->kernel_ms = ms;
  r->pt2_ms = mk;
  r->launches = ctx->ev_valid ? ctx->last_launches : 0;
  // selection: records stay on the device (or in the sink) until
  // cipsi_selection_get/raw
  const long long nsel = (long long)cnt[C_NSEL];
  r->n_selected = nsel;
  if (cnt[C_STAGE_OVF])
    return fail(ctx, CIPSI_ERR_CUDA, "internal error: a selected candidate's slot lay outside its staging region");
  // the records are valid when every unit segment found room in the pool;
  // the output arrays then hold the first out_cap of them, in unit order
  const long long out_cap = ctx->sink ? ctx->sink_cap : ctx->sel_cap;
  ctx->nsel = nsel > ctx->pool_cap ? 0 : std::min(nsel, out_cap);
  if (nsel > ctx->pool_cap || nsel > out_cap)
    return fail(ctx, CIPSI_ERR_OVERFLOW,
                "selection buffer overflow: " + std::to_string(nsel) + " records > capacity " +
                    std::to_string(std::min(out_cap, ctx->pool_cap)) +
                    (nsel > ctx->pool_cap ? " (counted only; cipsi_run_pt2 grows the buffers and reruns)"
                     : ctx->sink         ? " (the sink holds the first records; the rest were counted only)"
                                         : " (cipsi_run_pt2 grows the buffer and reruns)"));
  return CIPSI_OK;
}

int cipsi_run_pt2(cipsi_ctx* ctx, const cipsi_opts* opts, cipsi_result* res) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    int rc = cipsi_run_pt2_async(ctx, opts);
    if (rc) return rc;
    rc = cipsi_fetch_result(ctx, res);
    if (rc != CIPSI_ERR_OVERFLOW) return rc;
    // grow the pool (and the device record arrays) to what the run needed
    // and redo; a caller's sink that is too small stays the caller's
    const long long nsel = res->n_selected;
    const long long cap = nsel + nsel / 8 + 1024;
    if (nsel <= ctx->pool_cap && ctx->sink) return rc;
    if (nsel > ctx->pool_cap && (rc = grow_pool(ctx, cap))) return rc;
    if (!ctx->sink && nsel > ctx->sel_cap && (rc = grow_sel(ctx, cap))) return rc;
  }
  return fail(ctx, CIPSI_ERR_OVERFLOW, "selection buffer could not be grown");
}

}  // extern "C"

// ------------------------------------------------------- streamed records
// cipsi_run_pt2_stream: the run in chunks of consecutive work units whose
// candidate slots fit the record pool (a unit never selects more records
// than it has slots), so any selection size runs in bounded device memory.
// Per chunk, on the context stream: k_pt2 over the chunk's units, the unit
// scan and the gather into one of two device record buffers; the copy
// stream then brings the chunk to a ring of two pinned host buffers piece
// by piece, and the caller's consumer gets each piece, in record order,
// while the GPU computes the next chunk.

namespace {

int ensure_stream_buffers(cipsi_ctx* ctx, long long cap, bool host, long long hb_cap) {
  const int W = ctx->W, mt = ctx->d.metat;
  if (cap > ctx->out_cap) {
    ++ctx->buf_gen;
    for (int i = 0; i < 2; ++i) {
      dfree(ctx->dout_bits[i]); dfree(ctx->dout_owner[i]); dfree(ctx->dout_xam[i]); dfree(ctx->dout_evp[i]);
    }
    ctx->out_cap = 0;
    for (int i = 0; i < 2; ++i) {
      CK(cudaMalloc(&ctx->dout_bits[i], (size_t)cap * 2 * W * sizeof(uint64_t)));
      CK(cudaMalloc(&ctx->dout_owner[i], (size_t)cap * sizeof(int32_t)));
      CK(cudaMalloc(&ctx->dout_xam[i], (size_t)cap * sizeof(double)));
      CK(cudaMalloc(&ctx->dout_evp[i], (size_t)cap * mt * sizeof(double)));
    }
    ctx->out_cap = cap;
  }
  if (!ctx->copy_stream) {
    CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
      CK(cudaEventCreateWithFlags(&ctx->ev_gathered[i], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->ev_copied[i], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ctx->ev_host[i], cudaEventDisableTiming));
    }
  }
  if (host && hb_cap > ctx->hbuf_cap) {
    for (int i = 0; i < 2; ++i)
      if (ctx->hbuf[i]) {
        cudaFreeHost(ctx->hbuf[i]);
        ctx->hbuf[i] = nullptr;
      }
    ctx->hbuf_cap = 0;
    const size_t bytes = (size_t)hb_cap * (2 * W * 8 + 8 + 8 + mt * 8);
    for (int i = 0; i < 2; ++i) CK(cudaHostAlloc(&ctx->hbuf[i], bytes, cudaHostAllocDefault));
    ctx->hbuf_cap = hb_cap;
  }
  return CIPSI_OK;
}

// the counters, histogram and sums of a finished run into *r (as
// cipsi_fetch_result), reading on the context stream
int read_results(cipsi_ctx* ctx, int nclass, cipsi_result* r) {
  const int mt = ctx->d.metat;
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  std::vector<double> red(5 * mt), tab(2 * kNClass * kMaxRoots);
  std::vector<unsigned long long> cnt(ncount);
  CK(cudaMemcpyAsync(red.data(), ctx->dred, red.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cnt.data(), ctx->dcounters, ncount * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaMemcpyAsync(tab.data(), ctx->dhist_tab, tab.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
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
  r->n_selected = (int64_t)cnt[C_NSEL];
  {
    const unsigned long long b = cnt[C_NCOUNTERS];
    memcpy(&r->dpivot, &b, 8);
  }
  for (int i = 0; i < nclass; ++i) r->nom[i] = (int64_t)cnt[C_NCOUNTERS + 1 + i];
  for (int c = 0; c < nclass; ++c)
    for (int m = 0; m < mt; ++m) {
      r->nam[c * kMaxRoots + m] = (int64_t)cnt[C_NCOUNTERS + 1 + kNClass + c * mt + m];
      r->tabmp[c * kMaxRoots + m] = tab[c * mt + m];
      r->tabvp[c * kMaxRoots + m] = tab[nclass * mt + c * mt + m];
    }
  const double avg_rank = 4.0;
  r->alg_bytes = (int64_t)(cnt[C_NP2] * (8.0 * mt + 2 * 4.0 + 8.0) +
                           cnt[C_NP1] * (8.0 * mt + 8.0 + 2.0 * avg_rank * 2 * 4.0) +
                           cnt[C_NPROC] * (8.0 * avg_rank + 8.0 * (avg_rank + avg_rank * avg_rank) + 8.0 * mt));
  if (cnt[C_STAGE_OVF])
    return fail(ctx, CIPSI_ERR_CUDA, "internal error: a selected candidate's slot lay outside its staging region");
  return CIPSI_OK;
}

}  // namespace

extern "C" {

int cipsi_run_pt2_stream(cipsi_ctx* ctx, const cipsi_opts* o, int64_t chunk_records, cipsi_record_fn fn,
                         void* user, cipsi_result* r) {
  int rc = check_run_args(ctx, o);
  if (rc) return rc;
  if (!r) return fail(ctx, CIPSI_ERR_ARG, "run_pt2_stream: null result");
  if (ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "an asynchronous run is pending: fetch its result first");
  CK(cudaSetDevice(ctx->device));
  const int ncf = ctx->d.ncf, W = ctx->W, mt = ctx->d.metat;
  RunPlan pl;
  plan_run(ctx, o, ctx->tune_r_chunk, pl);
  const int nunits = (int)pl.ug.size();
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const LaunchShape ls = launch_shape(W, roots_pad(mt), ncf, ctx->tune_ctas);
  const int grid = std::max(1, std::min(nunits, dev_sms * ls.blocks_per_sm));
  if ((rc = ensure_neighbour_scratch(ctx, grid))) return rc;
  if ((rc = prepare_run(ctx, pl, ctx->stream))) return rc;
  if ((rc = ensure_staging(ctx, grid, staging_cap(pl)))) return rc;
  // chunk capacity: what was asked, else what about half the free device
  // memory holds (pool + two record buffers), at most 2^29 records; at
  // least the largest unit's slots
  const long long rec_bytes = 2 * W * 8 + 8 + 8 * mt;
  long long cap = chunk_records;
  if (cap <= 0) {
    size_t fr = 0, tot = 0;
    CK(cudaMemGetInfo(&fr, &tot));
    const double have = (double)fr + (double)(ctx->pool_cap + 2 * ctx->out_cap) * (rec_bytes + 4);
    cap = std::min<long long>(1ll << 29, (long long)(0.45 * have / (3.0 * (rec_bytes + 4))));
    // with a consumer, about eight chunks once the run has more than 8M
    // slots: each chunk's records are delivered while the next computes,
    // so only the last chunk's delivery follows the kernels
    if (fn) {
      long long total = 0;
      for (long long x : pl.uslots) total += x;
      cap = std::min(cap, std::max<long long>(total / 8 + 1, 1ll << 20));
    }
  }
  cap = std::max(cap, std::max<long long>(pl.max_slots, 1024));
  if (ctx->pool_cap < cap && (rc = grow_pool(ctx, cap))) return rc;
  const long long hb_cap = std::min<long long>(cap, 1ll << 24);
  if ((rc = ensure_stream_buffers(ctx, cap, fn != nullptr, hb_cap))) return rc;
  // chunks: consecutive units whose slots add up to at most cap
  std::vector<int> cut{0};
  {
    long long acc = 0;
    for (int u = 0; u < nunits; ++u) {
      if (acc + pl.uslots[u] > cap && u > cut.back()) {
        cut.push_back(u);
        acc = 0;
      }
      acc += pl.uslots[u];
    }
    if (cut.back() != nunits) cut.push_back(nunits);
  }
  const int nchunks = (int)cut.size() - 1;
  // per chunk: records gathered and records placed in the pool (pinned)
  unsigned long long* hcnt = nullptr;
  CK(cudaHostAlloc((void**)&hcnt, (size_t)std::max(1, 2 * nchunks) * sizeof(unsigned long long),
                   cudaHostAllocDefault));
  struct HostFree {
    unsigned long long* p;
    ~HostFree() { if (p) cudaFreeHost(p); }
  } hold{hcnt};

  const size_t nq = (size_t)5 * mt;
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  CK(cudaMemsetAsync(ctx->dcounters, 0, ncount * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dhist_tab, 0, 2 * kNClass * kMaxRoots * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->dgen_part, 0, (size_t)std::max(nunits, 1) * nq * sizeof(double), ctx->stream));
  Params p{};
  fill_params(ctx, o, pl, p);
  p.nb_j = ctx->dnb_j;
  p.nb_emask = ctx->dnb_em;
  p.lr_ent = ctx->dlr_ent;
  p.lr_cap = ls.lr_cap;
  p.nb_stride = ncf;
  const size_t words = 2 * (size_t)W;

  long long delivered = 0;  // records handed to the consumer so far
  long long piece_no = 0;
  auto deliver = [&](int c) -> int {
    const int b = c & 1;
    CK(cudaEventSynchronize(ctx->ev_gathered[b]));
    const long long n = (long long)hcnt[2 * c];
    if ((long long)hcnt[2 * c + 1] > ctx->pool_cap)
      return fail(ctx, CIPSI_ERR_OVERFLOW, "internal error: a chunk's records overflowed the pool");
    CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_gathered[b], 0));
    const long long npieces = (n + hb_cap - 1) / hb_cap;
    for (long long j = 0; j <= npieces; ++j) {
      if (j < npieces) {
        const long long off = j * hb_cap, cnt = std::min(hb_cap, n - off);
        unsigned char* hb = static_cast<unsigned char*>(ctx->hbuf[(piece_no + j) & 1]);
        CK(cudaMemcpyAsync(hb, ctx->dout_bits[b] + off * words, (size_t)cnt * words * 8, cudaMemcpyDeviceToHost,
                           ctx->copy_stream));
        hb += (size_t)hb_cap * words * 8;
        CK(cudaMemcpyAsync(hb, ctx->dout_owner[b] + off, (size_t)cnt * 4, cudaMemcpyDeviceToHost, ctx->copy_stream));
        hb += (size_t)hb_cap * 8;
        CK(cudaMemcpyAsync(hb, ctx->dout_xam[b] + off, (size_t)cnt * 8, cudaMemcpyDeviceToHost, ctx->copy_stream));
        hb += (size_t)hb_cap * 8;
        CK(cudaMemcpyAsync(hb, ctx->dout_evp[b] + off * mt, (size_t)cnt * mt * 8, cudaMemcpyDeviceToHost,
                           ctx->copy_stream));
        CK(cudaEventRecord(ctx->ev_host[(piece_no + j) & 1], ctx->copy_stream));
      }
      if (j >= 1) {
        const long long off = (j - 1) * hb_cap, cnt = std::min(hb_cap, n - off);
        const int hbi = (int)((piece_no + j - 1) & 1);
        CK(cudaEventSynchronize(ctx->ev_host[hbi]));
        const unsigned char* hb = static_cast<const unsigned char*>(ctx->hbuf[hbi]);
        const uint64_t* hbits = reinterpret_cast<const uint64_t*>(hb);
        const int32_t* hown = reinterpret_cast<const int32_t*>(hb + (size_t)hb_cap * words * 8);
        const double* hxam = reinterpret_cast<const double*>(hb + (size_t)hb_cap * (words * 8 + 8));
        const double* hevp = reinterpret_cast<const double*>(hb + (size_t)hb_cap * (words * 8 + 16));
        if (fn(user, delivered, cnt, (int32_t)words, mt, hbits, hown, hxam, hevp) != 0) {
          cudaStreamSynchronize(ctx->copy_stream);
          return fail(ctx, CIPSI_ERR_ARG, "run_pt2_stream: the record consumer returned an error");
        }
        delivered += cnt;
      }
    }
    piece_no += npieces;
    CK(cudaEventRecord(ctx->ev_copied[b], ctx->copy_stream));
    return CIPSI_OK;
  };

  // k_pt2 of each chunk timed by a pair of events
  std::vector<cudaEvent_t> kev(2 * (size_t)nchunks, nullptr);
  struct EvFree {
    std::vector<cudaEvent_t>& v;
    ~EvFree() {
      for (cudaEvent_t e : v)
        if (e) cudaEventDestroy(e);
    }
  } evhold{kev};
  for (auto& e : kev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  for (int c = 0; c < nchunks; ++c) {
    const int u0 = cut[c], u1 = cut[c + 1], b = c & 1;
    // the record buffer of this chunk was last read by chunk c - 2's copies
    if (c >= 2 && fn) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[b], 0));
    CK(cudaMemsetAsync(ctx->dwork, 0, sizeof(int), ctx->stream));
    CK(cudaMemsetAsync(ctx->dpool_count, 0, sizeof(unsigned long long), ctx->stream));
    Params pc = p;
    pc.nunits = u1 - u0;
    pc.unit_g = p.unit_g + u0;
    pc.unit_r0 = p.unit_r0 + u0;
    pc.unit_r1 = p.unit_r1 + u0;
    pc.gen_part = p.gen_part + (size_t)u0 * nq;
    pc.unit_pool = p.unit_pool + u0;
    pc.unit_nsel = p.unit_nsel + u0;
    const int cgrid = std::max(1, std::min(u1 - u0, grid));
    CK(cudaEventRecord(kev[2 * c], ctx->stream));
    cudaError_t e = launch_plain(pc, W, roots_pad(mt), cgrid, ls.smem, ctx->stream);
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_pt2 launch: ") + cudaGetErrorString(e));
    CK(cudaEventRecord(kev[2 * c + 1], ctx->stream));
    GatherArgs ga{};
    ga.out_bits = ctx->dout_bits[b];
    ga.out_owner = ctx->dout_owner[b];
    ga.out_xam = ctx->dout_xam[b];
    ga.out_evp = ctx->dout_evp[b];
    ga.out_cap = ctx->out_cap;
    e = enqueue_gather(ctx, p, u0, u1, 0, ga, ctx->stream, dev_sms);
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("record gather: ") + cudaGetErrorString(e));
    CK(cudaMemcpyAsync(&hcnt[2 * c], ctx->dscan_total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(&hcnt[2 * c + 1], ctx->dpool_count, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaEventRecord(ctx->ev_gathered[b], ctx->stream));
    if (fn && c >= 1 && (rc = deliver(c - 1))) return rc;
  }
  if (fn && nchunks >= 1 && (rc = deliver(nchunks - 1))) return rc;
  if (nunits > 0) {
    k_reduce<<<(unsigned)nq, kReduceThreads, 0, ctx->stream>>>(ctx->dgen_part, nunits, (int)nq, ctx->dred);
    CK(cudaGetLastError());
  } else {
    CK(cudaMemsetAsync(ctx->dred, 0, nq * sizeof(double), ctx->stream));
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (fn) CK(cudaStreamSynchronize(ctx->copy_stream));
  if ((rc = read_results(ctx, o->nclass, r))) return rc;
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  r->kernel_ms = ms;
  double pt2 = 0.0;
  for (int c = 0; c < nchunks; ++c) {
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, kev[2 * c], kev[2 * c + 1]));
    pt2 += t;
  }
  r->pt2_ms = pt2;
  r->launches = 3ll * nchunks + (nunits > 0 ? 1 : 0);
  for (int c = 0; c < nchunks; ++c)
    if ((long long)hcnt[2 * c + 1] > ctx->pool_cap)
      return fail(ctx, CIPSI_ERR_OVERFLOW, "internal error: a chunk's records overflowed the pool");
  if (fn && delivered != r->n_selected)
    return fail(ctx, CIPSI_ERR_CUDA, "internal error: " + std::to_string(delivered) + " records delivered of " +
                                         std::to_string(r->n_selected) + " selected");
  ctx->nsel = 0;  // the streamed records are the consumer's; none stay readable
  ctx->stream_chunks = nchunks;
  return CIPSI_OK;
}

// Order-sensitive digest of streamed records (a record consumer): per
// field array (bits, owner, xam, evp) a Fletcher-style pair of 64-bit sums
// over its words in record order, s1 = sum w_i and s2 = sum of the running
// s1, continued across calls; big pieces are split over host threads and
// the per-slice pairs combined in order.
int cipsi_record_digest(void* user, int64_t first, int64_t count, int32_t words, int32_t metat,
                        const uint64_t* bits, const int32_t* owner, const double* xam, const double* evp) {
  cipsi_digest* d = static_cast<cipsi_digest*>(user);
  if (!d || first != d->records) return -1;
  struct Pair {
    uint64_t s1 = 0, s2 = 0, n = 0;
  };
  auto fold = [](Pair& acc, const Pair& x) {
    acc.s2 += x.s2 + acc.s1 * x.n;
    acc.s1 += x.s1;
    acc.n += x.n;
  };
  // word i of a field array as a 64-bit integer
  auto run = [&](int field, uint64_t n) {
    auto word = [&](uint64_t i) -> uint64_t {
      if (field == 0) return bits[i];
      if (field == 1) return (uint64_t)(uint32_t)owner[i];
      uint64_t v;
      memcpy(&v, field == 2 ? &xam[i] : &evp[i], 8);
      return v;
    };
    auto slice = [&](uint64_t a, uint64_t b_) {
      Pair x;
      for (uint64_t i = a; i < b_; ++i) {
        x.s1 += word(i);
        x.s2 += x.s1;
      }
      x.n = b_ - a;
      return x;
    };
    const int nt = std::max(1, std::min<int>(d->threads > 0 ? d->threads : 1, (int)(n / 65536 + 1)));
    std::vector<Pair> part(nt);
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t)
      th.emplace_back([&, t]() { part[t] = slice(n * t / nt, n * (t + 1) / nt); });
    part[0] = slice(0, n / nt);
    for (auto& x : th) x.join();
    Pair acc{d->s1[field], d->s2[field], 0};
    for (const Pair& x : part) fold(acc, x);
    d->s1[field] = acc.s1;
    d->s2[field] = acc.s2;
  };
  if (count > 0) {
    run(0, (uint64_t)count * (uint64_t)words);
    run(1, (uint64_t)count);
    run(2, (uint64_t)count);
    run(3, (uint64_t)count * (uint64_t)metat);
  }
  d->records += count;
  return 0;
}

}  // extern "C"

namespace {

// The adjoint launch behind cipsi_run_pt2_adjoint (geri given) and
// cipsi_run_pt2_adjoint_1e (geri null: no (pq|rs) gradient, the second pass
// over singles only).  e2, when given, receives the E2 sums of the same pass.
int run_adjoint(cipsi_ctx* ctx, const cipsi_opts* o, const double* seed, double* e2, double* gF, double* gJ,
                double* gK, double* geri, double* gfmpb, double* groots) {
  int rc = 0;
  if (ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "an asynchronous run is pending: fetch its result first");
  CK(cudaSetDevice(ctx->device));
  const int ncf = ctx->d.ncf, W = ctx->W, mt = ctx->d.metat, n = ctx->d.norb;
  const int nt = n * (n + 1) / 2;
  RunPlan pl;
  plan_run(ctx, o, ctx->tune_r_chunk, pl);
  const int nunits = (int)pl.ug.size();
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int R = roots_pad(mt);
  const LaunchShape ls = launch_shape(W, R, ncf, ctx->tune_ctas, true);
  const int grid = std::max(1, std::min(nunits, dev_sms * ls.blocks_per_sm));
  rc = ensure_neighbour_scratch(ctx, grid);
  if (rc) return rc;
  rc = prepare_run(ctx, pl, ctx->stream);
  if (rc) return rc;
  const size_t nq = (size_t)5 * mt;
  const size_t ncount = C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots;
  CK(cudaMemsetAsync(ctx->dcounters, 0, ncount * sizeof(unsigned long long), ctx->stream));
  CK(cudaMemsetAsync(ctx->dhist_tab, 0, 2 * kNClass * kMaxRoots * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->dwork, 0, sizeof(int), ctx->stream));
  CK(cudaMemsetAsync(ctx->dgen_part, 0, (size_t)std::max(nunits, 1) * nq * sizeof(double), ctx->stream));
  // gradient buffers (this call only)
  const int stride = 3 * nt + 2 * n;
  double *d_eri = nullptr, *d_F = nullptr, *d_J = nullptr, *d_K = nullptr, *d_f = nullptr, *d_sl = nullptr,
         *d_roots = nullptr;
  auto release = [&]() {
    dfree(d_eri); dfree(d_F); dfree(d_J); dfree(d_K); dfree(d_f); dfree(d_sl); dfree(d_roots);
  };
  auto ck = [&](cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    release();
    return fail(ctx, CIPSI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  const bool one_e = geri == nullptr;
  if (!one_e && (rc = ck(cudaMalloc(&d_eri, (size_t)ctx->ninte * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_F, (size_t)nt * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_J, (size_t)nt * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_K, (size_t)nt * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_f, (size_t)2 * n * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_sl, (size_t)grid * stride * sizeof(double)), "cudaMalloc"))) return rc;
  if ((rc = ck(cudaMalloc(&d_roots, (size_t)3 * mt * sizeof(double)), "cudaMalloc"))) return rc;
  if (!one_e && (rc = ck(cudaMemsetAsync(d_eri, 0, (size_t)ctx->ninte * sizeof(double), ctx->stream), "memset")))
    return rc;
  if ((rc = ck(cudaMemsetAsync(d_F, 0, (size_t)nt * sizeof(double), ctx->stream), "memset"))) return rc;
  if ((rc = ck(cudaMemsetAsync(d_sl, 0, (size_t)grid * stride * sizeof(double), ctx->stream), "memset"))) return rc;
  if ((rc = ck(cudaMemsetAsync(d_roots, 0, (size_t)3 * mt * sizeof(double), ctx->stream), "memset"))) return rc;

  Params p{};
  fill_params(ctx, o, pl, p);
  p.nb_j = ctx->dnb_j;
  p.nb_emask = ctx->dnb_em;
  p.lr_ent = ctx->dlr_ent;
  p.lr_cap = ls.lr_cap;
  p.nb_stride = ncf;
  p.rec_mode = 0;  // no records from an adjoint launch
  for (int m = 0; m < mt; ++m) {
    p.seed_mp[m] = seed[m];
    p.seed_vp[m] = seed[mt + m];
    p.seed_b[m] = seed[2 * mt + m];
  }
  p.g_eri = d_eri;
  p.g_F = d_F;
  p.g_slice = d_sl;
  p.slice_stride = stride;
  p.g_roots = d_roots;
  p.adj_1e = one_e ? 1 : 0;
  if (nunits > 0) {
    cudaError_t e;
    if (W == 1) {
      e = R == 1 ? launch_pt2<1, 1, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
        : R == 2 ? launch_pt2<1, 2, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
        : R == 4 ? launch_pt2<1, 4, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
                 : launch_pt2<1, 8, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream);
    } else {
      e = R == 1 ? launch_pt2<2, 1, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
        : R == 2 ? launch_pt2<2, 2, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
        : R == 4 ? launch_pt2<2, 4, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream)
                 : launch_pt2<2, 8, false, true>(p, BatchArgs{}, grid, ls.smem, ctx->stream);
    }
    if ((rc = ck(e, "adjoint k_pt2 launch"))) return rc;
    k_reduce<<<(unsigned)nq, kReduceThreads, 0, ctx->stream>>>(ctx->dgen_part, nunits, (int)nq, ctx->dred);
  } else {
    if ((rc = ck(cudaMemsetAsync(ctx->dred, 0, nq * sizeof(double), ctx->stream), "memset"))) return rc;
  }
  k_slice_reduce<<<(stride + 255) / 256, 256, 0, ctx->stream>>>(d_sl, grid, stride, nt, d_F, d_J, d_K, d_f);
  if ((rc = ck(cudaGetLastError(), "k_slice_reduce"))) return rc;
  struct Out {
    double* host;
    const double* dev;
    size_t n;
  } outs[] = {{geri, d_eri, (size_t)ctx->ninte}, {gF, d_F, (size_t)nt}, {gJ, d_J, (size_t)nt},
              {gK, d_K, (size_t)nt}, {gfmpb, d_f, (size_t)2 * n}, {groots, d_roots, (size_t)3 * mt},
              {e2, ctx->dred, (size_t)3 * mt}};
  for (const Out& x : outs)
    if (x.host && (rc = ck(cudaMemcpyAsync(x.host, x.dev, x.n * sizeof(double), cudaMemcpyDeviceToHost,
                                           ctx->stream), "copy gradients")))
      return rc;
  if ((rc = ck(cudaStreamSynchronize(ctx->stream), "adjoint run"))) return rc;
  release();
  return CIPSI_OK;
}

}  // namespace

extern "C" {

int cipsi_run_pt2_adjoint(cipsi_ctx* ctx, const cipsi_opts* o, const double* seed, double* gF,
                          double* gJ, double* gK, double* geri, double* gfmpb, double* groots) {
  const int rc = check_run_args(ctx, o);
  if (rc) return rc;
  if (!seed || !gF || !gJ || !gK || !geri || !gfmpb || !groots)
    return fail(ctx, CIPSI_ERR_ARG, "run_pt2_adjoint: null seed or gradient array");
  return run_adjoint(ctx, o, seed, nullptr, gF, gJ, gK, geri, gfmpb, groots);
}

int cipsi_run_pt2_adjoint_1e(cipsi_ctx* ctx, const cipsi_opts* o, const double* seed, double* e2, double* gF,
                             double* gJ, double* gK, double* gfmpb, double* groots) {
  const int rc = check_run_args(ctx, o);
  if (rc) return rc;
  if (!seed || !e2 || !gF || !gJ || !gK || !gfmpb || !groots)
    return fail(ctx, CIPSI_ERR_ARG, "run_pt2_adjoint_1e: null seed, energy or gradient array");
  return run_adjoint(ctx, o, seed, e2, gF, gJ, gK, nullptr, gfmpb, groots);
}

int cipsi_selection_raw(cipsi_ctx* ctx, int64_t first, int64_t count, uint64_t* bits,
                        int32_t* owner, double* xam, double* evp) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (first < 0 || count < 0 || first + count > ctx->nsel)
    return fail(ctx, CIPSI_ERR_ARG, "selection: range outside the selection");
  if (count == 0) return CIPSI_OK;
  CK(cudaSetDevice(ctx->device));
  const int W = ctx->W, mt = ctx->d.metat;
  if (ctx->sink) {
    // the records are already in host memory
    auto cp = [](void* dst, const void* src, size_t n) {
      if (dst && dst != src) std::memcpy(dst, src, n);
    };
    cp(bits, static_cast<const uint64_t*>(ctx->sink_host[0]) + (size_t)first * 2 * W, (size_t)count * 2 * W * 8);
    cp(owner, static_cast<const int32_t*>(ctx->sink_host[1]) + first, (size_t)count * 4);
    cp(xam, static_cast<const double*>(ctx->sink_host[2]) + first, (size_t)count * 8);
    cp(evp, static_cast<const double*>(ctx->sink_host[3]) + (size_t)first * mt, (size_t)count * mt * 8);
    return CIPSI_OK;
  }
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


// ------------------------------------------------------ batched geometries
// One persistent launch per (words per spin string, roots) class runs the
// work units of many contexts (Autocip grid geometries of different sizes);
// the launches of all classes, the clearing and the reductions are captured
// once in a CUDA graph and replayed by cipsi_batch_run.

}  // extern "C"

struct cipsi_batch {
  int device = 0;
  std::string err;
  cudaStream_t stream = nullptr;
  std::vector<cipsi_ctx*> ctxs;
  std::vector<cipsi_opts> opts;
  std::vector<unsigned long long> buf_gen;
  Params* dgeo = nullptr;
  struct Class {
    int W = 1, R = 1;
    int big = 0;  // the plain form would run these contexts at one CTA per SM
    std::vector<int> geos;
    int nunits = 0, grid = 0, ncf_max = 0;
    LaunchShape ls{};
    int32_t* dunit_geo = nullptr;
    int32_t* dunit_local = nullptr;
    int* dwork = nullptr;
    int32_t* dnb_j = nullptr;
    uint64_t* dnb_em = nullptr;
    uint64_t* dlr_ent = nullptr;
    // record staging shared by the class's geometries (per CTA)
    long long st_cap = 32;
    uint64_t* dst_bits = nullptr;
    double *dst_xam = nullptr, *dst_evp = nullptr;
    uint32_t* dst_mask = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev_join = nullptr;
  };
  std::vector<Class> classes;
  int max_nq = 0;
  cudaEvent_t ev_fork = nullptr, ev0 = nullptr, ev1 = nullptr, done = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool pending = false;
};

namespace {

int bfail(cipsi_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define BCK(call)                                                                       \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return bfail(b, CIPSI_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <int W>
cudaError_t launch_batch_class(const Params& p0, const BatchArgs& ba, int R, int grid, size_t smem,
                               cudaStream_t st) {
  return R == 1 ? launch_pt2<W, 1, true>(p0, ba, grid, smem, st)
       : R == 2 ? launch_pt2<W, 2, true>(p0, ba, grid, smem, st)
       : R == 4 ? launch_pt2<W, 4, true>(p0, ba, grid, smem, st)
                : launch_pt2<W, 8, true>(p0, ba, grid, smem, st);
}

void batch_free(cipsi_batch* b) {
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto& c : b->classes) {
    dfree(c.dunit_geo); dfree(c.dunit_local); dfree(c.dwork);
    dfree(c.dnb_j); dfree(c.dnb_em); dfree(c.dlr_ent);
    dfree(c.dst_bits); dfree(c.dst_xam); dfree(c.dst_evp); dfree(c.dst_mask);
    if (c.st) cudaStreamDestroy(c.st);
    if (c.ev_join) cudaEventDestroy(c.ev_join);
  }
  dfree(b->dgeo);
  for (cudaEvent_t e : {b->ev_fork, b->ev0, b->ev1, b->done})
    if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

extern "C" {

int cipsi_batch_create(cipsi_batch** out, cipsi_ctx* const* ctxs, int32_t n, const cipsi_opts* opts,
                       int32_t r_chunk, int32_t ctas_per_sm) {
  if (!out) return CIPSI_ERR_ARG;
  *out = nullptr;
  cipsi_batch* b = new cipsi_batch();
  *out = b;
  if (!ctxs || !opts || n < 1) return bfail(b, CIPSI_ERR_ARG, "batch needs at least one context and its options");
  if (r_chunk < 1 || r_chunk > 4096 || ctas_per_sm < 0 || ctas_per_sm > 2)
    return bfail(b, CIPSI_ERR_ARG, "r_chunk must be in [1, 4096] and ctas_per_sm 0, 1 or 2");
  b->device = ctxs[0] ? ctxs[0]->device : 0;
  for (int i = 0; i < n; ++i) {
    cipsi_ctx* ctx = ctxs[i];
    if (!ctx) return bfail(b, CIPSI_ERR_ARG, "null context in batch");
    if (ctx->device != b->device) return bfail(b, CIPSI_ERR_ARG, "all contexts of a batch must use one device");
    if (ctx->pending) return bfail(b, CIPSI_ERR_STATE, "a context of the batch has a pending run");
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == ctx) return bfail(b, CIPSI_ERR_ARG, "a context appears twice in the batch");
    const int rc = check_run_args(ctx, &opts[i]);
    if (rc) return bfail(b, rc, "context " + std::to_string(i) + ": " + ctx->err);
  }
  BCK(cudaSetDevice(b->device));
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  for (cudaEvent_t* e : {&b->ev_fork, &b->done})
    BCK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  BCK(cudaEventCreate(&b->ev0));
  BCK(cudaEventCreate(&b->ev1));
  int dev_sms = 0;
  BCK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, b->device));

  // plan every geometry; per-context buffers as for a plain run
  std::vector<Params> P(n);
  std::vector<long long> work(n), stcap(n);
  b->ctxs.assign(ctxs, ctxs + n);
  b->opts.assign(opts, opts + n);
  for (int i = 0; i < n; ++i) {
    cipsi_ctx* ctx = ctxs[i];
    b->opts[i].gen_mask = nullptr;  // used by the plan below only
    RunPlan pl;
    plan_run(ctx, &opts[i], r_chunk, pl);
    if (prepare_run(ctx, pl, b->stream)) return bfail(b, CIPSI_ERR_CUDA, "context " + std::to_string(i) + ": " + ctx->err);
    fill_params(ctx, &opts[i], pl, P[i]);
    stcap[i] = staging_cap(pl);
    work[i] = (long long)pl.ug.size() * ctx->d.ncf;
    const int W = ctx->W, R = roots_pad(ctx->d.metat);
    // contexts whose shared-memory list needs a whole SM go to their own
    // launch, so the others keep two CTAs per SM as in the plain form
    const int big = ctas_per_sm == 0 && launch_shape(W, R, ctx->d.ncf, 0).blocks_per_sm == 1 ? 1 : 0;
    int c = 0;
    while (c < (int)b->classes.size() &&
           !(b->classes[c].W == W && b->classes[c].R == R && b->classes[c].big == big))
      ++c;
    if (c == (int)b->classes.size()) {
      b->classes.emplace_back();
      b->classes[c].W = W;
      b->classes[c].R = R;
      b->classes[c].big = big;
    }
    b->classes[c].geos.push_back(i);
    b->max_nq = std::max(b->max_nq, 5 * ctx->d.metat);
  }
  BCK(cudaStreamSynchronize(b->stream));  // host plan vectors die here

  // per class: unit order (heaviest geometry first), launch shape, scratch
  for (auto& c : b->classes) {
    std::stable_sort(c.geos.begin(), c.geos.end(), [&](int x, int y) { return work[x] > work[y]; });
    std::vector<int32_t> ugeo, ulocal;
    int mt_max = 1;
    for (int i : c.geos) {
      c.ncf_max = std::max(c.ncf_max, ctxs[i]->d.ncf);
      c.st_cap = std::max(c.st_cap, stcap[i]);
      mt_max = std::max(mt_max, ctxs[i]->d.metat);
      for (int u = 0; u < P[i].nunits; ++u) {
        ugeo.push_back(i);
        ulocal.push_back(u);
      }
    }
    c.nunits = (int)ugeo.size();
    c.ls = launch_shape(c.W, c.R, c.ncf_max, ctas_per_sm);
    c.grid = std::max(1, std::min(c.nunits, dev_sms * c.ls.blocks_per_sm));
    BCK(cudaMalloc(&c.dunit_geo, (size_t)std::max(c.nunits, 1) * sizeof(int32_t)));
    BCK(cudaMalloc(&c.dunit_local, (size_t)std::max(c.nunits, 1) * sizeof(int32_t)));
    BCK(cudaMalloc(&c.dwork, sizeof(int)));
    BCK(cudaMalloc(&c.dnb_j, (size_t)c.grid * c.ncf_max * sizeof(int32_t)));
    BCK(cudaMalloc(&c.dnb_em, (size_t)c.grid * c.ncf_max * sizeof(uint64_t)));
    BCK(cudaMalloc(&c.dlr_ent, (size_t)c.grid * c.ncf_max * sizeof(uint64_t)));
    {
      const size_t slots = (size_t)c.grid * (size_t)c.st_cap;
      BCK(cudaMalloc(&c.dst_bits, slots * 2 * c.W * sizeof(uint64_t)));
      BCK(cudaMalloc(&c.dst_xam, slots * sizeof(double)));
      BCK(cudaMalloc(&c.dst_evp, slots * mt_max * sizeof(double)));
      BCK(cudaMalloc(&c.dst_mask, slots / 32 * sizeof(uint32_t)));
      BCK(cudaMemset(c.dst_mask, 0, slots / 32 * sizeof(uint32_t)));
    }
    if (c.nunits) {
      BCK(cudaMemcpy(c.dunit_geo, ugeo.data(), (size_t)c.nunits * sizeof(int32_t), cudaMemcpyHostToDevice));
      BCK(cudaMemcpy(c.dunit_local, ulocal.data(), (size_t)c.nunits * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    for (int i : c.geos) {
      P[i].nb_j = c.dnb_j;
      P[i].nb_emask = c.dnb_em;
      P[i].lr_ent = c.dlr_ent;
      P[i].nb_stride = c.ncf_max;
      P[i].lr_cap = c.ls.lr_cap;
      P[i].st_cap = (int)c.st_cap;
      P[i].st_bits = c.dst_bits;
      P[i].st_xam = c.dst_xam;
      P[i].st_evp = c.dst_evp;
      P[i].st_mask = c.dst_mask;
    }
    BCK(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    BCK(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming));
  }
  BCK(cudaMalloc(&b->dgeo, (size_t)n * sizeof(Params)));
  BCK(cudaMemcpy(b->dgeo, P.data(), (size_t)n * sizeof(Params), cudaMemcpyHostToDevice));
  for (int i = 0; i < n; ++i) b->buf_gen.push_back(ctxs[i]->buf_gen);

  // capture: clear, the class launches side by side, the reductions
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
  k_batch_clear<<<n, 256, 0, b->stream>>>(b->dgeo);
  BCK(cudaEventRecord(b->ev_fork, b->stream));
  for (auto& c : b->classes) {
    BCK(cudaStreamWaitEvent(c.st, b->ev_fork, 0));
    BCK(cudaMemsetAsync(c.dwork, 0, sizeof(int), c.st));
    if (c.nunits) {
      BatchArgs ba{b->dgeo, c.dunit_geo, c.dunit_local, c.nunits, c.dwork};
      const Params& p0 = P[c.geos[0]];
      cudaError_t e = c.W == 1 ? launch_batch_class<1>(p0, ba, c.R, c.grid, c.ls.smem, c.st)
                               : launch_batch_class<2>(p0, ba, c.R, c.grid, c.ls.smem, c.st);
      if (e != cudaSuccess) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(b->stream, &g);
        if (g) cudaGraphDestroy(g);
        return bfail(b, CIPSI_ERR_CUDA, std::string("batched k_pt2 launch: ") + cudaGetErrorString(e));
      }
    }
    BCK(cudaEventRecord(c.ev_join, c.st));
    BCK(cudaStreamWaitEvent(b->stream, c.ev_join, 0));
  }
  k_reduce_batch<<<dim3((unsigned)b->max_nq, (unsigned)n), kReduceThreads, 0, b->stream>>>(b->dgeo);
  // every geometry's records, in its unit order
  for (int i = 0; i < n; ++i) {
    GatherArgs ga{};
    record_target(ctxs[i], ga);
    const cudaError_t e = enqueue_gather(ctxs[i], P[i], 0, P[i].nunits, 0, ga, b->stream, dev_sms);
    if (e != cudaSuccess) {
      cudaGraph_t g = nullptr;
      cudaStreamEndCapture(b->stream, &g);
      if (g) cudaGraphDestroy(g);
      return bfail(b, CIPSI_ERR_CUDA, std::string("batched record gather: ") + cudaGetErrorString(e));
    }
  }
  BCK(cudaStreamEndCapture(b->stream, &b->graph));
  BCK(cudaGraphInstantiate(&b->exec, b->graph, 0));
  return CIPSI_OK;
}

int cipsi_batch_run(cipsi_batch* b) {
  if (!b || !b->exec) return CIPSI_ERR_ARG;
  for (size_t i = 0; i < b->ctxs.size(); ++i) {
    const cipsi_ctx* ctx = b->ctxs[i];
    if (ctx->buf_gen != b->buf_gen[i])
      return bfail(b, CIPSI_ERR_STATE, "context " + std::to_string(i) +
                                           " reallocated its buffers after the batch was built; rebuild the batch");
    // a result left pending by this batch's previous run is simply replaced
    if (ctx->pending && ctx->ext_done != b->done)
      return bfail(b, CIPSI_ERR_STATE, "context " + std::to_string(i) + " has a pending run");
  }
  BCK(cudaSetDevice(b->device));
  BCK(cudaEventRecord(b->ev0, b->stream));
  BCK(cudaGraphLaunch(b->exec, b->stream));
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaEventRecord(b->done, b->stream));
  for (size_t i = 0; i < b->ctxs.size(); ++i) {
    cipsi_ctx* ctx = b->ctxs[i];
    ctx->ext_done = b->done;
    ctx->ev_valid = false;
    ctx->nclass = b->opts[i].nclass;
    ctx->last_opts = b->opts[i];
    ctx->pending = true;
  }
  b->pending = true;
  return CIPSI_OK;
}

int cipsi_batch_wait(cipsi_batch* b, double* ms) {
  if (!b) return CIPSI_ERR_ARG;
  if (!b->pending) return bfail(b, CIPSI_ERR_STATE, "batch_wait without batch_run");
  BCK(cudaSetDevice(b->device));
  BCK(cudaEventSynchronize(b->done));
  b->pending = false;
  float t = 0.f;
  BCK(cudaEventElapsedTime(&t, b->ev0, b->ev1));
  if (ms) *ms = t;
  return CIPSI_OK;
}

const char* cipsi_batch_last_error(const cipsi_batch* b) { return b ? b->err.c_str() : "null batch"; }

void cipsi_batch_destroy(cipsi_batch* b) {
  if (!b) return;
  batch_free(b);
  for (cipsi_ctx* ctx : b->ctxs)
    if (ctx && ctx->ext_done == b->done) {
      ctx->ext_done = nullptr;
      ctx->pending = false;
    }
  delete b;
}

// ------------------------------------------------- run without allocation
// cipsi_run_pt2_static runs k_pt2 + k_reduce with every per-run buffer taken
// from one file-scope device array instead of cudaMalloc'd context buffers.
// Layout of the array (each region 256-byte aligned): counters + dpivot +
// histogram counts | histogram sums | reduced sums | work counter |
// generator list | generator masks | work units | per-unit partial sums |
// per-block neighbour scratch (nb_j, nb_emask, lr_ent).  The generator and
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
  const LaunchShape ls = launch_shape(W, R, ncf, 0);
  const int lr_cap = ls.lr_cap;
  const size_t smem = ls.smem;
  const int blocks_per_sm = ls.blocks_per_sm;
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
  p.eri64 = ctx->deri64 ? ctx->deri64 : ctx->deri_w;
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
  // nb_j, nb_emask, lr_ent: grid x ncf entries each (k_pt2 indexes block b at
  // b * ncf), in three regions of grid * nb_stride >= grid * ncf * 8 bytes
  p.nb_j = reinterpret_cast<int32_t*>(nb0);
  p.nb_emask = reinterpret_cast<uint64_t*>(nb0 + (size_t)grid * nb_stride);
  p.lr_ent = reinterpret_cast<uint64_t*>(nb0 + (size_t)2 * grid * nb_stride);
  p.lr_cap = lr_cap;
  p.nb_stride = ncf;
  p.gen_part = reinterpret_cast<double*>(base + off_part);
  unsigned long long* dcounters = reinterpret_cast<unsigned long long*>(base + off_counters);
  p.counters = dcounters;
  p.dpivot_bits = dcounters + C_NCOUNTERS;
  p.hist_nom = dcounters + C_NCOUNTERS + 1;
  p.hist_nam = dcounters + C_NCOUNTERS + 1 + kNClass;
  p.hist_tab = reinterpret_cast<double*>(base + off_tab);
  // no record storage: selected perturbers are counted only
  p.rec_mode = 0;
  p.work = reinterpret_cast<int*>(base + off_work);
  double* dred = reinterpret_cast<double*>(base + off_red);

  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (nunits > 0) {
    cudaError_t e;
    if (W == 1) {
      e = R == 1 ? launch_pt2<1, 1, false>(p, BatchArgs{}, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<1, 2, false>(p, BatchArgs{}, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<1, 4, false>(p, BatchArgs{}, grid, smem, ctx->stream)
                 : launch_pt2<1, 8, false>(p, BatchArgs{}, grid, smem, ctx->stream);
    } else {
      e = R == 1 ? launch_pt2<2, 1, false>(p, BatchArgs{}, grid, smem, ctx->stream)
        : R == 2 ? launch_pt2<2, 2, false>(p, BatchArgs{}, grid, smem, ctx->stream)
        : R == 4 ? launch_pt2<2, 4, false>(p, BatchArgs{}, grid, smem, ctx->stream)
                 : launch_pt2<2, 8, false>(p, BatchArgs{}, grid, smem, ctx->stream);
    }
    if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_pt2 launch: ") + cudaGetErrorString(e));
    k_reduce<<<(unsigned)nq, kReduceThreads, 0, ctx->stream>>>(p.gen_part, nunits, (int)nq, dred);
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(ctx->ev1, ctx->stream));

  // results (same fields as cipsi_fetch_result; no records are kept), read
  // on the context's stream: a legacy-stream cudaMemcpy would also wait for
  // every other blocking stream of the device
  double red[5 * kMaxRoots];
  unsigned long long cnt[C_NCOUNTERS + 1 + kNClass + kNClass * kMaxRoots];
  double tab[2 * kNClass * kMaxRoots];
  CK(cudaMemcpyAsync(red, dred, nq * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(cnt, dcounters, ncount * sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(tab, p.hist_tab, 2 * kNClass * kMaxRoots * sizeof(double), cudaMemcpyDeviceToHost,
                     ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
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
  r->pt2_ms = ms;
  r->launches = nunits > 0 ? 2 : 0;
  r->n_selected = (int64_t)cnt[C_NSEL];
  return CIPSI_OK;
}

}  // extern "C"

// ================================================ Hamiltonian over the space
// cipsi_hamiltonian_build / cipsi_hamiltonian_get: the lower triangle of H
// over the determinants given to cipsi_set_space, by rows, as moy writes it
// to its unit 1 (moy/moy.f:117-199) -- row i: the columns j < min(i, jmax)
// within two excitations, in increasing j, with <i|H|j> in the phase of the
// excitation lists.  The elements moy drops (|h| < 1e-10) are kept here;
// the caller filters them when it writes the file.
extern "C" {

int cipsi_hamiltonian_build(cipsi_ctx* ctx, const double* fock, int32_t jmax, int64_t* npairs) {
  if (!ctx || !npairs) return CIPSI_ERR_ARG;
  if (!ctx->have_int || !ctx->have_space)
    return fail(ctx, CIPSI_ERR_STATE, "hamiltonian_build needs set_integrals and set_space");
  if (ctx->pending) return fail(ctx, CIPSI_ERR_STATE, "a run is pending: fetch its result first");
  CK(cudaSetDevice(ctx->device));
  const int n = ctx->d.ncf, W = ctx->W, norb = ctx->d.norb;
  *npairs = 0;
  ctx->have_h = false;
  int rc;
  {
    std::vector<int8_t> sg(n);
    for (int k = 0; k < n; ++k) sg[k] = ctx->sigma[k] < 0 ? -1 : 1;
    if ((rc = upload(ctx, &ctx->dsigma, sg.data(), sg.size()))) return rc;
  }
  const double* dF = ctx->dF;
  if (fock) {
    if ((rc = upload(ctx, &ctx->dFraw, fock, (size_t)norb * (norb + 1) / 2))) return rc;
    dF = ctx->dFraw;
  }
  dfree(ctx->dh_count);
  ++ctx->buf_gen;
  CK(cudaMalloc((void**)&ctx->dh_count, (size_t)n * sizeof(int32_t)));
  HBuildArgs a{};
  a.p.norb = norb;
  a.p.noca = ctx->d.noca;
  a.p.nsym = ctx->d.nsym;
  a.p.eri = ctx->deri;
  a.p.eri64 = ctx->deri64 ? ctx->deri64 : ctx->deri_w;
  a.p.pairtab = ctx->dpairtab;
  a.p.ntttt = ctx->dntttt;
  a.p.F = dF;
  a.S = ctx->dS;
  a.sigma = ctx->dsigma;
  a.n = n;
  a.jmax = jmax < 0 ? n : std::min(jmax, n);
  for (int q = 0; q < 4; ++q) a.hf[q] = 0ull;
  for (int o = 0; o < ctx->d.noca; ++o) {
    a.hf[o >> 6] |= 1ull << (o & 63);
    a.hf[W + (o >> 6)] |= 1ull << (o & 63);
  }
  a.count = ctx->dh_count;
  CK(cudaEventRecord(ctx->ev0, ctx->stream));
  cudaError_t e = W == 1 ? launch_hpairs<1>(a, false, ctx->stream) : launch_hpairs<2>(a, false, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_hpairs (count): ") + cudaGetErrorString(e));
  std::vector<int32_t> cnt(n);
  CK(cudaMemcpyAsync(cnt.data(), ctx->dh_count, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->h_rowptr.assign((size_t)n + 1, 0);
  for (int i = 0; i < n; ++i) ctx->h_rowptr[i + 1] = ctx->h_rowptr[i] + cnt[i];
  const long long total = ctx->h_rowptr[n];
  if ((rc = upload(ctx, &ctx->dh_rowptr, ctx->h_rowptr.data(), ctx->h_rowptr.size()))) return rc;
  if (total > ctx->h_cap || !ctx->dh_col) {
    dfree(ctx->dh_col);
    dfree(ctx->dh_val);
    ++ctx->buf_gen;
    CK(cudaMalloc((void**)&ctx->dh_col, (size_t)std::max(total, 1ll) * sizeof(int32_t)));
    CK(cudaMalloc((void**)&ctx->dh_val, (size_t)std::max(total, 1ll) * sizeof(double)));
    ctx->h_cap = std::max(total, 1ll);
  }
  a.rowptr = ctx->dh_rowptr;
  a.col = ctx->dh_col;
  a.val = ctx->dh_val;
  e = W == 1 ? launch_hpairs<1>(a, true, ctx->stream) : launch_hpairs<2>(a, true, ctx->stream);
  if (e != cudaSuccess) return fail(ctx, CIPSI_ERR_CUDA, std::string("k_hpairs (fill): ") + cudaGetErrorString(e));
  CK(cudaEventRecord(ctx->ev1, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaEventElapsedTime(&ctx->h_ms, ctx->ev0, ctx->ev1));
  ctx->have_h = true;
  *npairs = total;
  return CIPSI_OK;
}

int cipsi_hamiltonian_get(cipsi_ctx* ctx, int32_t row0, int32_t nrows, int64_t* rowptr, int32_t* col,
                          double* val) {
  if (!ctx) return CIPSI_ERR_ARG;
  if (!ctx->have_h) return fail(ctx, CIPSI_ERR_STATE, "hamiltonian_get before hamiltonian_build");
  const int n = ctx->d.ncf;
  if (row0 < 0 || nrows < 0 || row0 + (long long)nrows > n)
    return fail(ctx, CIPSI_ERR_ARG, "hamiltonian_get: rows out of range");
  const long long a = ctx->h_rowptr[row0], b = ctx->h_rowptr[row0 + nrows];
  if (rowptr)
    for (int r = 0; r <= nrows; ++r) rowptr[r] = ctx->h_rowptr[row0 + r] - a;
  CK(cudaSetDevice(ctx->device));
  if (b > a && (col || val)) {
    if (col)
      CK(cudaMemcpyAsync(col, ctx->dh_col + a, (size_t)(b - a) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                         ctx->stream));
    if (val)
      CK(cudaMemcpyAsync(val, ctx->dh_val + a, (size_t)(b - a) * sizeof(double), cudaMemcpyDeviceToHost,
                         ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return CIPSI_OK;
}

float cipsi_hamiltonian_ms(const cipsi_ctx* ctx) { return ctx ? ctx->h_ms : 0.f; }

}  // extern "C"
