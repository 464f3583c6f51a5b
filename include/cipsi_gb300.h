/*
 * cipsi_gb300.h -- C ABI of the GB300 engine for the CIPSI second-order
 * perturbation and selection step (the `cip` / `cipsym` hot path).
 *
 * The engine replaces, in one call, the two subroutine calls that do all the
 * work of the reference program after its set-up:
 *
 *     if(ypertu) call pertu        CIPSI_sources/cip/cip.f:238
 *     if(ypertu) call diexcit      CIPSI_sources/cip/cip.f:241
 *     (CIPSI_sources/cipsym/cip.f:248,251 in the symmetric variant)
 *
 * Those subroutines take no arguments; they read and write COMMON blocks.
 * Each setter below takes the arrays of one group of COMMON variables, with
 * the reference's own layout and meaning, so that a patched cip.f can pass
 * its COMMON storage directly through an ISO_C_BINDING interface whose
 * types mirror the structs below.  All arrays are owned by the caller and copied by the
 * call; nothing is retained.  Indices stored in arrays (spin orbitals,
 * offsets) keep the reference's 1-based values.
 *
 * Return codes: 0 = success, negative = error (cipsi_last_error(ctx) gives a
 * message).  The library never exits the process.  One context drives one
 * GPU; contexts are independent (one per Autocip process / geometry).
 */
#ifndef CIPSI_GB300_H
#define CIPSI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CIPSI_OK 0
#define CIPSI_ERR_ARG (-1)      /* invalid argument or unsupported input */
#define CIPSI_ERR_CUDA (-2)     /* CUDA runtime error                    */
#define CIPSI_ERR_STATE (-3)    /* call order (setters before run)       */
#define CIPSI_ERR_OVERFLOW (-4) /* internal buffer overflow              */

#define CIPSI_MAX_ROOTS 8
#define CIPSI_NCLASS 10

typedef struct cipsi_ctx cipsi_ctx;

/* Sizes: COMMON /cipsi/ (CIPSI_sources/cip/cip.f:36-39). */
typedef struct {
  int32_t norb;  /* number of orbitals (norb)                               */
  int32_t noca;  /* doubly occupied orbitals of the reference det (noca)    */
  int32_t nsym;  /* number of irreducible representations (nsym)            */
  int32_t isym;  /* symmetry of the treated states (isym, 1-based)          */
  int32_t isz;   /* 2*Sz (isz); only 0 is supported                          */
  int32_t metat; /* number of roots (metat), 1..CIPSI_MAX_ROOTS            */
  int32_t ncf;   /* determinants of S including spin-flip partners (ncf)    */
} cipsi_dims;

/* Options: COMMON /cipsi/, /tome/, /hist/ flags used by pertu/diexcit. */
typedef struct {
  int32_t yen;        /* Epstein-Nesbet partitions (ityper = 2)              */
  int32_t ysele;      /* select on energy contributions (iselec = 3)         */
  int32_t ymoyen;     /* histogram + unit-60 selection (ymoyen)              */
  int32_t ywdeg;      /* near-degenerate perturbers are selected (ywdeg)     */
  int32_t sym_variant;/* 1: cipsym (ENvp per root in the selection records)  */
  int32_t nclass;     /* histogram classes (nclass <= 10)                     */
  double tau;         /* unit-60 selection threshold (tau)                    */
  double teseff;      /* histogram threshold (teseff)                         */
  double aval[CIPSI_NCLASS]; /* class upper bounds (aval)                     */
  const uint8_t* gen_mask; /* optional, ncf bytes: 0 = do not run this det as
                              a generator (generator-range sharding); NULL =
                              all.  Owner tests still see every determinant. */
  int32_t run_pertu;  /* 1: include pertu's reference-only and reference-
                         single perturbers (pertu.f:62-108)                   */
} cipsi_opts;

/* Results: the accumulators of COMMON /ic/ and /hist/ after pertu+diexcit. */
typedef struct {
  double e2mp[CIPSI_MAX_ROOTS];  /* MP barycentric E2 (e2mp)                 */
  double e2vp[CIPSI_MAX_ROOTS];  /* EN eigenvalue E2 (e2vp)                  */
  double e2b[CIPSI_MAX_ROOTS];   /* EN barycentric E2 (e2b)                  */
  double psimp[CIPSI_MAX_ROOTS]; /* norm of the first-order function, MP     */
  double psivp[CIPSI_MAX_ROOTS]; /* norm of the first-order function, EN     */
  double dpivot;                 /* largest non-listed contribution (dpivot) */
  int64_t ietat;                 /* effective states generated (ietat)       */
  int64_t n_processed;           /* perturbers that reached the E2 loop      */
  int64_t n_selected;            /* records available through selection_get  */
  int64_t nom[CIPSI_NCLASS];     /* histogram totals (nom)                   */
  int64_t nam[CIPSI_NCLASS * CIPSI_MAX_ROOTS];     /* nam(class, root)       */
  double tabmp[CIPSI_NCLASS * CIPSI_MAX_ROOTS];    /* tabmp(class, root)     */
  double tabvp[CIPSI_NCLASS * CIPSI_MAX_ROOTS];    /* tabvp(class, root)     */
  /* work counters (not in the reference; for throughput and roofline)      */
  int64_t n_candidates;   /* excitations examined                           */
  int64_t n_compares;     /* candidate-vs-S determinant comparisons          */
  int64_t n_pairs_1;      /* interacting (I,K) pairs differing by 1 spin orb */
  int64_t n_pairs_2;      /* interacting (I,K) pairs differing by 2          */
  int64_t alg_bytes;      /* algorithmic bytes (integrals, coefficients,     */
                          /* diagonal terms) read by the E2 loop             */
  double kernel_ms;       /* device time of the perturbation kernels         */
  double pt2_ms;          /* of which the perturbation kernel itself (k_pt2, */
                          /* summed over its launches)                        */
  int64_t launches;       /* kernel launches of the run (k_pt2, record scan  */
                          /* and gather per chunk, final reduction)           */
} cipsi_result;

/* Create a context on CUDA device `device`.
   Replaces the static sizing of pshf.prm (ndetz, doa, metz, kget). */
int cipsi_ctx_create(cipsi_ctx** ctx, const cipsi_dims* dims, int32_t device);
void cipsi_ctx_destroy(cipsi_ctx* ctx);
const char* cipsi_last_error(const cipsi_ctx* ctx);

/* Run the engine's kernels on this CUDA stream (cudaStream_t; NULL = the
   context's own stream). */
int cipsi_set_stream(cipsi_ctx* ctx, void* stream);

/* Integrals: COMMON /jkf/ (f, aj, ak), /ij1/ (ij0, ntttt), /bij/ (bijkl) and
   the symmetry tables itsym, its of /spo/ (cip/ijkf.f:26-43,
   cip/reijkl.f:12-36, cip/ai.f:1-42).
     itsym[norb]        irrep of each orbital (1-based values)
     its[nsym*nsym]     product table, column-major its(i,j)
     f, aj, ak          packed lower triangles ((x(i,j),j=1,i),i=1,norb)
     ij0[norb*norb]     int16 pair map, column-major ij0(i,j)
     ntttt[nsym]        first packed index of each irrep block (1-based)
     bijkl[ninte]       (pq|rs) as stored by cip: real*4                     */
int cipsi_set_integrals(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                        const double* f, const double* aj, const double* ak,
                        const int16_t* ij0, const int32_t* ntttt, const float* bijkl,
                        int64_t ninte);
/* Same, from the real*8 values of the unit-40 file: rounded to real*4 exactly
   as cip/reijkl.f:27 does. */
int cipsi_set_integrals_fp64(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                             const double* f, const double* aj, const double* ak,
                             const int16_t* ij0, const int32_t* ntttt, const double* pqrs,
                             int64_t ninte);

/* Reference space S: COMMON /spo/ (ne, nd, trou, part, ygen) and /degene/
   (ysaut, nesp, yef(.,1)) as built by cip/deter.f:478-567.
     ne[ncf], nd[ncf]   excitation degree and offset: the holes of det k are
                        trou[nd[k]] .. trou[nd[k]+ne[k]-1] (C indexing of
                        trou(nd(k)+1..nd(k)+ne(k)))
     trou[], part[]     hole / particle spin orbitals (1..2*norb)
     ygen, ysaut        generator and spin-flip-partner flags (bytes)
     nesp               number of partners following a determinant
     yef1               yef(k,1): det has a distinct spin-flip partner in S */
int cipsi_set_space(cipsi_ctx* ctx, const int32_t* ne, const int32_t* nd, const int32_t* trou,
                    const int32_t* part, int64_t ntp, const uint8_t* ygen, const uint8_t* ysaut,
                    const int32_t* nesp, const uint8_t* yef1);

/* Zero-order quantities: COMMON /ic/ and /tome/ (cip/cip.f:75-135).
     c[ncf*metat]   S coefficients, column-major per root (reference phase)
     e, eb, emp, teste, taum [metat]   e relative to escf
     fmpb[2*norb]   barycentric MP one-electron energies                    */
int cipsi_set_roots(cipsi_ctx* ctx, const double* c, const double* e, const double* eb,
                    const double* emp, const double* teste, const double* taum,
                    const double* fmpb);

/* pertu + diexcit on the GPU (cip.f:238-241).  Blocks until done. */
int cipsi_run_pt2(cipsi_ctx* ctx, const cipsi_opts* opts, cipsi_result* res);

/* Launch shape of later runs on this context (no counterpart in the
   reference; results do not depend on it beyond summation order):
     r_chunk      removed-electron blocks per work unit for generators of
                  excitation rank >= 2 (rank 0 and 1 generators always get
                  one block per unit); default 6
     ctas_per_sm  0 or 2 = shared-memory list sized so that two CTAs fit
                  per SM (the rest of a longer list is read from global
                  memory), 1 = one CTA per SM with a 200 KB list
   cipsi_gb300.tune (Python) picks both by timing a generator sample. */
int cipsi_set_tuning(cipsi_ctx* ctx, int32_t r_chunk, int32_t ctas_per_sm);

/* Unit-60 records straight into caller memory (no counterpart in the
   reference): pinned host arrays (cudaHostAlloc / cudaHostRegister) of
   `capacity` records, laid out as cipsi_selection_raw returns them (bits
   [capacity*2W], owner, xam, evp [capacity*metat]).  Later runs on this
   context write their records there from the kernel, over the host link,
   while they compute; cipsi_selection_raw then copies from these arrays
   (or does nothing when given the same arrays).  Records beyond `capacity`
   are counted, not stored: cipsi_fetch_result reports CIPSI_ERR_OVERFLOW with
   the results valid and the first `capacity` records kept, and
   cipsi_run_pt2 does not rerun.  bits = NULL returns to device buffers.
   The arrays must stay allocated while the sink is set. */
int cipsi_set_selection_sink(cipsi_ctx* ctx, uint64_t* bits, int32_t* owner, double* xam, double* evp,
                             int64_t capacity);

/* Streamed run (no counterpart in the reference; replaces pie.f's
   buffered writes of lungo records to unit 60, CIPSI_sources/cip/pie.f:
   20-36, for selections too large for device memory): the same work as
   cipsi_run_pt2, in chunks of consecutive work units whose candidate slots
   fit `chunk_records` records (0 = sized from the free device memory, at
   most 2^29, and with fn given at most an eighth of the run's slots, at
   least 2^20, so that delivery overlaps the kernels).  Each chunk's records are copied into pinned host buffers
   while the next chunk computes, and `fn` receives them piece by piece, in
   the order cipsi_selection_get gives, with `first` = the index of the
   piece's first record in the run: bits[count*words] (words = 2W, as
   cipsi_selection_raw), owner[count], xam[count], evp[count*metat].  The
   pointers are valid during the call only.  A non-zero return from fn stops
   the run (CIPSI_ERR_ARG).  fn = NULL keeps each chunk's records in device
   memory only (timing of the device work).  Blocks until done; nothing is
   left for cipsi_selection_get. */
typedef int (*cipsi_record_fn)(void* user, int64_t first, int64_t count, int32_t words, int32_t metat,
                               const uint64_t* bits, const int32_t* owner, const double* xam,
                               const double* evp);
int cipsi_run_pt2_stream(cipsi_ctx* ctx, const cipsi_opts* opts, int64_t chunk_records,
                         cipsi_record_fn fn, void* user, cipsi_result* res);

/* A record consumer for cipsi_run_pt2_stream (user = cipsi_digest*, zero it
   and set `threads` first): an order-sensitive digest of the streamed
   records, per field array (bits, owner, xam, evp) the pair s1 = sum of its
   64-bit words, s2 = sum of the running s1, over the run's records in
   order (unsigned arithmetic modulo 2^64; owner words zero-extended, doubles
   as their bit patterns).  Pieces must arrive in order (first ==
   records).  No counterpart in the reference. */
typedef struct {
  uint64_t s1[4], s2[4];
  int64_t records;
  int32_t threads;
} cipsi_digest;
int cipsi_record_digest(void* user, int64_t first, int64_t count, int32_t words, int32_t metat,
                        const uint64_t* bits, const int32_t* owner, const double* xam, const double* evp);

/* Enqueue the same work on the context stream without waiting; the result is
   collected by cipsi_fetch_result.  Used to time the kernels alone. */
int cipsi_run_pt2_async(cipsi_ctx* ctx, const cipsi_opts* opts);
int cipsi_fetch_result(cipsi_ctx* ctx, cipsi_result* res);

/* Selected perturbers (what pie.f writes to unit 60), records
   [first, first+count) of the last run.  Their order is fixed whatever the
   GPU's scheduling: work units in the run's order (generators by
   excitation rank, then by index; pertu's candidates first), and within a
   unit blocks of removed electrons, then added orbitals, in enumeration
   order.  Two runs on the same inputs give identical arrays.
     nec[count]           excitation degree
     holes/parts[8*count] sorted spin orbitals (1-based), zero padded
     xam[count]           selection value written as v(n)
     evp[metat*count]     ENvp contribution per root (cipsym), else zeros
     owner[count]         generator index (1-based; 0 = pertu)             */
int cipsi_selection_get(cipsi_ctx* ctx, int64_t first, int64_t count, int32_t* nec,
                        int32_t* holes, int32_t* parts, double* xam, double* evp,
                        int32_t* owner);

/* Host-side inputs of one cip/cipsym run, read from a calculation directory
   exactly as CIPSI_sources/cip/cip.f:50-135 does (namelists, units 40, 33,
   60, 59, 4; S with its spin-flip partners, deter.f:478-567; zero order,
   faifoc.f and cip.f:99-135).  Host memory only: no device work. */
typedef struct cipsi_inputs cipsi_inputs;
int cipsi_inputs_read(cipsi_inputs** in, const char* workdir, const char* stdin_path,
                      int32_t sym_variant, char* errbuf, int32_t errlen);
/* Sizes and namelist options of the run (either pointer may be NULL). */
int cipsi_inputs_dims(const cipsi_inputs* in, cipsi_dims* dims, cipsi_opts* opts);
/* Copy the inputs into a context: cipsi_set_integrals + cipsi_set_space +
   cipsi_set_roots from the host arrays (host-to-device copies). */
int cipsi_inputs_upload(const cipsi_inputs* in, cipsi_ctx* ctx);
void cipsi_inputs_free(cipsi_inputs* in);

/* Process-level drop-in for cip.exe (sym_variant = 0) and cipsym.exe
   (sym_variant = 1): reads the &cipfil/&icinp namelists from `stdin_path`
   and the unit files of `workdir` exactly as CIPSI_sources/cip/cip.f:50-242
   does, runs the engine in place of pertu + diexcit, and writes unit 60,
   unit 33 and the listing lines of cip.f:243-254 / cipsym/cip.f:253-254.
   `json_path` (optional) receives the E2 totals and counters; `gen_mask`
   (optional, one byte per determinant of S) limits the generators.  On
   error returns a negative code and copies the message into errbuf. */
int cipsi_cip_main(const char* workdir, const char* stdin_path, int32_t sym_variant,
                   const char* json_path, const uint8_t* gen_mask, int32_t device, char* errbuf,
                   int32_t errlen);

/* The same records without conversion: occupation bitstrings, 2*W 64-bit
   words per record (W = 1 if norb <= 64 else 2; alpha words then beta
   words, bit o of word o/64 = orbital o+1), owner, xam, evp[metat].  Any
   output pointer may be NULL. */
int cipsi_selection_raw(cipsi_ctx* ctx, int64_t first, int64_t count, uint64_t* bits,
                        int32_t* owner, double* xam, double* evp);

/* Read access to an array of the inputs, by the name of its COMMON
   variable: itsym, its, ij0, ntttt, F (f), J (aj), K (ak), eri (bijkl),
   c, e, eb, emp, teste, taum, fmpb, ne, nd, trou, part, ygen, ysaut, nesp,
   yef1, escf.  *data points into `in` (valid until cipsi_inputs_free);
   *type: 1 int32, 2 int16, 3 float32, 4 float64, 5 uint8.  CIPSI_ERR_ARG
   for an unknown name.  Not in the reference (its arrays are COMMONs). */
int cipsi_inputs_array(const cipsi_inputs* in, const char* name, const void** data, int64_t* count,
                       int32_t* type);

/* Same as cipsi_set_integrals_fp64 but (pq|rs) stay in FP64 on the device
   instead of the reference's real*4 (cip/reijkl.f:27): for derivative
   checks, where real*4 steps (~1e-8 relative) would swamp a finite
   difference.  cipsi_set_integrals returns the context to real*4. */
int cipsi_set_integrals_f64store(cipsi_ctx* ctx, const int32_t* itsym, const int32_t* its,
                                 const double* f, const double* aj, const double* ak,
                                 const int16_t* ij0, const int32_t* ntttt, const double* pqrs,
                                 int64_t ninte);

/* Adjoint of cipsi_run_pt2 (no counterpart in the reference): gradients of
   L = sum_m seed[m] e2mp[m] + seed[metat+m] e2vp[m] + seed[2 metat+m] e2b[m]
   with respect to the engine's inputs, the S coefficients held fixed:
     gF, gJ, gK [norb(norb+1)/2]  packed like f, aj, ak
     geri [ninte]                 packed like bijkl
     gfmpb [2 norb]               by spin orbital
     groots [3 metat]             dL/de, dL/deb, dL/demp
   The perturber set, weights and denominators are those of the forward run
   (pert1.f:151-191, diexcit.f:327-376); dL/d<I|H|j> = sum_m dL/db_m c_jm is
   spread over the integrals of each interacting pair (hntd.f:138-163), and
   dL/dhdig, dL/dhmp over F, J, K, fmpb (hdig.f, hmp.f).  Blocks until done;
   allocates its gradient buffers for the call. */
int cipsi_run_pt2_adjoint(cipsi_ctx* ctx, const cipsi_opts* opts, const double* seed, double* gF,
                          double* gJ, double* gK, double* geri, double* gfmpb, double* groots);

/* One-electron adjoint (no counterpart in the reference): the E2 sums and
   the gradients of cipsi_run_pt2_adjoint except the (pq|rs) one, from one
   pass.  e2 [3 metat] receives [e2mp; e2vp; e2b] as cipsi_run_pt2 computes
   them (the same terms; the rounding of a sum may differ in the last bits);
   gF, gJ, gK, gfmpb, groots are complete (J and K enter only hdig, F the
   diagonal terms and the one-difference elements).  Without the (pq|rs)
   gradient the second pass visits only the pairs one excitation apart, so
   the call costs about one forward run: a perturbation h -> h + F mu of the
   one-electron operator (the finite-field runs of Autocip_13/ffield.f90:66-127)
   needs gF, the fmpb gradient and the root-energy gradients only. */
int cipsi_run_pt2_adjoint_1e(cipsi_ctx* ctx, const cipsi_opts* opts, const double* seed, double* e2,
                             double* gF, double* gJ, double* gK, double* gfmpb, double* groots);

/* Batched form: the runs of many contexts (the geometries of an Autocip
   grid, of different sizes) in one persistent launch per class of contexts
   with the same string width (norb <= 64 or not) and padded root count,
   all captured once as a CUDA graph.  No counterpart in the reference, which
   runs one cip process per geometry (Autocip_13/calcul.f90:320).
     cipsi_batch_create  plans every context's run with opts[i] (as
                         cipsi_run_pt2_async would, gen_mask read here only),
                         sizes its buffers and captures the graph; r_chunk
                         and ctas_per_sm as in cipsi_set_tuning.  On failure
                         *b still holds a batch: read cipsi_batch_last_error
                         and destroy it.
     cipsi_batch_run     replays the graph on the batch's own stream (no
                         wait); afterwards cipsi_fetch_result(ctx_i) gives
                         each geometry's result (it waits for the batch) and
                         the selection calls its records; kernel_ms is -1
                         there, cipsi_batch_wait gives the batch's time.
     cipsi_batch_wait    waits for the last replay; *ms = its device time.
   Records beyond a context's selection capacity are counted but not stored
   (cipsi_fetch_result then returns CIPSI_ERR_OVERFLOW for that context; a
   cipsi_run_pt2 on it grows the capacity).  A context whose buffers are
   reallocated after the batch was built (set_* calls, a plain run that grows
   a buffer) makes cipsi_batch_run fail with CIPSI_ERR_STATE: rebuild the
   batch.  Member contexts must not run other work while a replay is in
   flight. */
typedef struct cipsi_batch cipsi_batch;
int cipsi_batch_create(cipsi_batch** b, cipsi_ctx* const* ctxs, int32_t n, const cipsi_opts* opts,
                       int32_t r_chunk, int32_t ctas_per_sm);
int cipsi_batch_run(cipsi_batch* b);
int cipsi_batch_wait(cipsi_batch* b, double* ms);
const char* cipsi_batch_last_error(const cipsi_batch* b);
void cipsi_batch_destroy(cipsi_batch* b);

/* pertu + diexcit like cipsi_run_pt2, but the call allocates no device
   memory.  This entry point has no counterpart in the reference.

   For callers that must not allocate while they run: a program that has
   handed the free device memory to its own pool (cudaMalloc would fail or
   fragment it), or one that keeps other streams busy while E2 is computed
   (cudaMalloc and cudaFree can synchronise the whole device and stall
   them).  The context's inputs (set_integrals / set_space / set_roots) are
   the only device memory it uses besides one 32 MiB array that is part of
   the library's device image.

   Returns the same energies, histogram and counters as cipsi_run_pt2.
   Selected perturbers are counted (n_selected) but not stored: use
   cipsi_run_pt2 when the records are needed.  The records of an earlier
   cipsi_run_pt2 stay readable.  Blocks until done.

   Limits: at most 131072 generators and 262144 work units (a generator
   makes one unit per six allowed excitation blocks), and the per-run
   buffers must fit the 32 MiB array: per-unit sums (40 * metat bytes per
   unit) plus, per thread block, 3 * ncf * 8 bytes of neighbour lists; the
   call runs fewer thread blocks when the lists do not fit for all of them,
   and returns CIPSI_ERR_OVERFLOW with the needed size when even one block
   does not fit.  CIPSI_ERR_STATE if a cipsi_run_pt2_async result is still
   pending on the context.

   The first call on each device looks up the array's device address
   (cudaGetSymbolAddress) with that device current; make that first call
   before any stream capture starts.  Every call clears the counters and
   sums it accumulates into before its kernels run.  All calls in the
   process share the one array (and fixed host staging arrays): two calls
   that overlap in time, from two threads or on two contexts, race and
   corrupt each other's results, so callers must serialise them. */
int cipsi_run_pt2_static(cipsi_ctx* ctx, const cipsi_opts* opts, cipsi_result* res);

/* The Hamiltonian over the determinants given to cipsi_set_space, lower
   triangle by rows, as moy builds it over S + the selected perturbers
   (CIPSI_sources/moy/moy.f:117-199, the double loop over i and j < i with
   its degree test and hntd).  Row i holds every column j < min(i, jmax)
   (jmax < 0: no limit; moy's y_secd sets jmax = |S|) within two
   excitations of i, in increasing j, with <i|H|j> in the phase of the
   reference's excitation lists (the value hntd returns; 0 for identical
   determinants).  moy drops the elements with |h| < 1e-10 when it writes
   unit 1: they are kept here, the caller filters.  The diagonal is not
   included (moy/hdig.f, on the host).  `fock` (optional, packed like f) is
   the Fock matrix the one-difference elements use; moy reads it from unit
   40 as it stands (moy/ijkf.f), while cipsi_set_integrals zeroes
   |F| < 1e-10 as cip/ijkf.f does.  Needs cipsi_set_integrals* and
   cipsi_set_space; blocks until done; *npairs = pairs over all rows.
   The pairs stay on the device until the next build or ctx_destroy. */
int cipsi_hamiltonian_build(cipsi_ctx* ctx, const double* fock, int32_t jmax, int64_t* npairs);
/* Rows row0 .. row0+nrows-1 of the last build: rowptr[nrows+1] (offsets
   into col/val, from 0), col (0-based j) and val; any output may be NULL
   (rowptr alone costs no device copy). */
int cipsi_hamiltonian_get(cipsi_ctx* ctx, int32_t row0, int32_t nrows, int64_t* rowptr, int32_t* col,
                          double* val);
/* Device time of the last build's two kernels, in ms. */
float cipsi_hamiltonian_ms(const cipsi_ctx* ctx);

/* Process-level drop-in for moy.exe (CIPSI_sources/moy/moy.f): reads the
   &moyfil/&moyen namelists from `stdin_path` and, in `workdir`, units 4
   (first record), 40 and 60; builds the determinant list as moy/deter.f
   does (unit-60 records with vs >= tau, by excitation degree, each followed
   by its spin-flip partner, repeats dropped); writes units 64 and 61 (the
   lists), unit 1 (H by rows, |h| >= 1e-10, in 8192-element records), unit
   63 (MP diagonal, ystkmp) and, as moy/morue.f, the second-order energies
   of the determinants beyond S (unit 33 records and the fourth unit-4
   record).  The pairs come from cipsi_hamiltonian_build on `device`.
   `json_path` (optional) receives counts and energies.  Not supported:
   yspipro, yion, spatial degeneracy operations (ntrans > 0). */
int cipsi_moy_main(const char* workdir, const char* stdin_path, const char* json_path, int32_t device,
                   char* errbuf, int32_t errlen);

/* The lowest eigenpairs of the CI matrix that moy writes to unit 1 (the
   work of CIPSI_sources/bd/bigdia.f): the n x n symmetric H = L + L^T, L
   given as nel elements (itab[t], jtab[t], val[t]), 1-based, jtab <= itab,
   each diagonal element stored as half its value (moy/moy.f:150-190,
   bd/getmat.f).  A block Davidson iteration on `device` (davidson.cu),
   converged when every root's residual norm |H x - e x| is at most `tol`:
   evals[nroots] ascending, evecs[n * nroots] (root-major, unit norm, each
   vector's largest component positive), *iters, resid[nroots] (optional).
   nroots <= 8.  Returns CIPSI_ERR_OVERFLOW (results of the last iteration
   filled in) if not converged within maxiter iterations.  Allocates its
   device buffers for the call. */
int cipsi_davidson(int32_t n, int64_t nel, const int32_t* itab, const int32_t* jtab, const double* val,
                   int32_t nroots, double tol, int32_t maxiter, int32_t device, double* evals, double* evecs,
                   int32_t* iters, double* resid, char* errbuf, int32_t errlen);

/* Process-level drop-in for bd.exe (CIPSI_sources/bd/bd.f): reads the
   &bdfil/&option namelists from `stdin_path` and, in `workdir`, unit 1 (the
   matrix moy wrote) and the first two records of unit 4 (metat, ncper,
   escf); computes the lowest metat eigenpairs with cipsi_davidson; writes
   the 'energies var.' record of unit 33, unit 59 (qwvec: ncf, netat, the
   vectors, the total energies), unit 55 (qws) and the listing lines
   ' ncf,netat,ncper,iget' that the Autocip driver reads.  Not supported:
   qnorm, qrvec, qhef, qdcple, and ind, cold, netat or ites given in
   &option. */
int cipsi_bd_main(const char* workdir, const char* stdin_path, const char* json_path, int32_t device,
                  char* errbuf, int32_t errlen);

#ifdef __cplusplus
}
#endif
#endif /* CIPSI_GB300_H */
