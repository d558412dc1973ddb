/*
 * lra.h -- C ABI of liblra, the GB300 (sm_103a) engine for LowRankApprox.jl's
 * sketch-then-factor path (idfact / pqrfact / psvdfact / pheigfact / curfact,
 * sketch / sketchfact, snorm / snormdiff).
 *
 * Conventions (chosen so that a Julia `ccall` shim needs no copies):
 *   - matrices are column-major with an explicit leading dimension (Julia's
 *     `stride(A, 2)`), exactly as the reference passes them to LAPACK
 *     (src/lapack.jl:129-136);
 *   - integer outputs (pivots, skeleton / redundant indices, rows, cols) are
 *     int64 and 1-based, like Julia's `Vector{Int}` (src/pqr.jl:350,357);
 *   - an input pointer may be host or device memory; the library detects
 *     which with cudaPointerGetAttributes and never mutates an input;
 *   - results are returned in library-owned host structs, released with the
 *     matching lra_*_free (a Julia finalizer);
 *   - every entry point returns an lra_status; lra_last_error(ctx) gives the
 *     message.  The Julia shim maps LRA_EINVAL -> ArgumentError,
 *     LRA_EDIM -> DimensionMismatch, LRA_ENOTHERM -> ErrorException
 *     ("matrix must be Hermitian", src/pheig.jl:279).
 *
 * A context owns one CUDA stream, a device workspace arena and pinned host
 * staging.  It is thread-compatible, not thread-safe: use one per host thread.
 */
#ifndef LRA_H
#define LRA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LRA_VERSION_MAJOR 0
#define LRA_VERSION_MINOR 1

/* ---- status codes -------------------------------------------------------- */
typedef enum lra_status {
  LRA_OK = 0,
  LRA_EINVAL = 1,      /* bad option / argument   (ArgumentError)        */
  LRA_EDIM = 2,        /* inconsistent dimensions (DimensionMismatch)     */
  LRA_ENOMEM = 3,      /* device or host allocation failed                */
  LRA_ETIMEDOUT = 4,   /* a bounded device wait gave up                   */
  LRA_ENONFINITE = 5,  /* NaN / Inf in the input                          */
  LRA_ECUDA = 6,       /* CUDA runtime error                              */
  LRA_ERAND = 7,       /* injected random stream too short                */
  LRA_ENOTSUP = 8,     /* combination not supported by this build         */
  LRA_ENOTHERM = 9,    /* pheigfact on a non-Hermitian matrix             */
  LRA_EBUSY = 10       /* server queue full / over HBM budget             */
} lra_status;

/* element types: Float32, Float64, ComplexF32, ComplexF64 (complex arrays
   hold (re, im) pairs, Julia's Complex{T} layout; complex types run on the
   native path whatever opts->precision says) */
typedef enum lra_dtype { LRA_F32 = 0, LRA_F64 = 1, LRA_C32 = 2, LRA_C64 = 3 } lra_dtype;

/* src/LowRankApprox.jl:138 -- the valid sketch symbols */
typedef enum lra_sketch_kind {
  LRA_SKETCH_NONE = 0,
  LRA_SKETCH_RANDN = 1,
  LRA_SKETCH_SPRN = 2,
  LRA_SKETCH_SRFT = 3,
  LRA_SKETCH_SUB = 4
} lra_sketch_kind;

/* pqrfact_retval letters (src/pqr.jl:298-300) as a bit set */
enum { LRA_RET_Q = 1, LRA_RET_R = 2, LRA_RET_T = 4 };

/* arithmetic of the GEMM-shaped stages */
typedef enum lra_precision {
  LRA_PREC_NATIVE = 0, /* plain FP64 (FP32 for Float32 input) on CUDA cores  */
  LRA_PREC_MIXED = 1   /* exact-split BF16 slices on tcgen05 tensor cores,
                          FP64-faithful accumulation; the pivoted QR, norm
                          recomputation, triangular solve and small dense
                          factorizations stay in the input precision        */
} lra_precision;

/*
 * LRAOptions (src/LowRankApprox.jl:77-120), field for field.  The
 * oversampling functions `n -> a*n + b` become affine coefficients
 * {a, b}; arbitrary Julia closures are rejected by the shim.
 */
typedef struct lra_opts {
  double atol;                  /* 0                                      */
  int64_t maxdet_niter;         /* -1                                     */
  double maxdet_tol;            /* -1 (off)                               */
  int64_t nb;                   /* 32                                     */
  double pheig_orthtol;         /* sqrt(eps(T))                           */
  int32_t pqrfact_retval;       /* LRA_RET_Q | LRA_RET_R                  */
  int32_t sketch;               /* LRA_SKETCH_RANDN                       */
  int64_t rank;                 /* -1                                     */
  double rtol;                  /* 5 eps(T)                               */
  int64_t sketch_randn_niter;   /* 0                                      */
  int32_t sketchfact_adap;      /* 1                                      */
  int32_t verb;                 /* 1                                      */
  int64_t sketchfact_randn_samp[2]; /* {1, 8}:  n -> n + 8               */
  int64_t sketchfact_srft_samp[2];  /* {1, 8}:  n -> n + 8               */
  int64_t sketchfact_sub_samp[2];   /* {4, 8}:  n -> 4n + 8              */
  int64_t snorm_niter;          /* 32                                     */
  /* GB300 engine options (no counterpart in LRAOptions) */
  int32_t precision;            /* lra_precision, default LRA_PREC_NATIVE */
  int32_t check_finite;         /* reject NaN/Inf input (default 1)       */
  uint64_t seed;                /* seed of the in-library generator       */
} lra_opts;

/*
 * Injected randomness.  The reference draws its random numbers inside the
 * sketch operators (src/sketch.jl:92,252,339-361,575; src/snorm.jl:18).
 * For reproducible parity the caller may supply them instead; each sketch
 * consumes, per adaptive step, in this order:
 *   randn : l*M values of `gauss` = S (l x M, column-major)
 *   srft  : M values of `gauss` (d_i = +1 if > 0 else -1), then l values of
 *           `ints` (idx_i = 1 + (v - 1) mod M)
 *   sub   : l values of `ints` (rows r_i = 1 + (v - 1) mod M)
 *   sprn  : M values of `ints` used as sort keys (the permutation is their
 *           stable ascending rank order, 1-based), then M values of `gauss`
 *           (row i uses fld(M-i, l) + 1 of them)
 *   snorm : N values of `gauss` (the start vector)
 * where M is the sketched dimension and l the sketch order.  Pointers may be
 * host or device memory.  With rand == NULL the library draws from its own
 * counter-based generator seeded by opts->seed.
 */
typedef struct lra_rand {
  const double* gauss;
  int64_t gauss_len;
  const int64_t* ints;
  int64_t ints_len;
} lra_rand;

/* ---- result types (library-owned host memory) --------------------------- */

/* IDPackedV (src/id.jl:15-92): A[:, rd] ~= A[:, sk] * T */
typedef struct lra_id {
  int32_t dtype;
  int32_t nsteps;     /* adaptive sketch steps taken */
  int64_t k, n;
  int64_t* sk;        /* k, 1-based                  */
  int64_t* rd;        /* n - k, 1-based              */
  void* T;            /* k x (n - k), ld = k         */
} lra_id;

/* PartialQRFactors (src/pqr.jl:14-32); Q, R, T are NULL unless requested */
typedef struct lra_pqr {
  int32_t dtype;
  int32_t retval;     /* LRA_RET_* bits that were filled */
  int64_t m, n, k;
  int64_t* p;         /* n, 1-based column permutation */
  void* Q;            /* m x k, ld = m                 */
  void* R;            /* k x n, ld = k                 */
  void* T;            /* k x (n - k), ld = k           */
} lra_pqr;

/* PartialSVD (src/psvd.jl:4-16): A ~= U * diagm(S) * Vt */
typedef struct lra_psvd {
  int32_t dtype;
  int32_t _pad;
  int64_t m, n, k;
  void* U;            /* m x k, ld = m (NULL for psvdvals) */
  void* S;            /* k                                 */
  void* Vt;           /* k x n, ld = k (NULL for psvdvals) */
} lra_psvd;

/* PartialHermitianEigen (src/pheig.jl:4-7) */
typedef struct lra_pheig {
  int32_t dtype;
  int32_t _pad;
  int64_t n, k;
  void* values;       /* k, ascending              */
  void* vectors;      /* n x k, ld = n (NULL: vals) */
} lra_pheig;

/* CURPackedU / HermitianCURPackedU / SymmetricCURPackedU (src/cur.jl:14-57) */
typedef struct lra_cur {
  int32_t kind;       /* 0 general, 1 Hermitian, 2 symmetric */
  int32_t _pad;
  int64_t kr, kc;
  int64_t* rows;      /* kr, 1-based (== cols for kinds 1, 2) */
  int64_t* cols;      /* kc, 1-based */
} lra_cur;

/* one matrix of a batch */
typedef struct lra_matdesc {
  int64_t m, n, lda;
  const void* A;
} lra_matdesc;

/* ---- context ------------------------------------------------------------- */
typedef struct lra_ctx lra_ctx;

int lra_ctx_create(int device, lra_ctx** ctx);
void lra_ctx_destroy(lra_ctx* ctx);
/* use the caller's cudaStream_t for all work of this context */
int lra_ctx_set_stream(lra_ctx* ctx, void* cuda_stream);
const char* lra_last_error(const lra_ctx* ctx);
const char* lra_status_string(int status);
/* number of kernels this context has launched (instrumentation) */
int64_t lra_ctx_launches(const lra_ctx* ctx);
/* number of launches of the kernel called `name` (the names the launch
   list of a profiler shows, e.g. "geqp3_df_smem_kernel"), cumulative over
   the context's life (instrumentation; no counterpart in the reference) */
int64_t lra_ctx_kernel_launches(const lra_ctx* ctx, const char* name);
/* device time of the last call's stages, ms: sketch, qr, solve, post */
int lra_ctx_stage_ms(const lra_ctx* ctx, double out[4]);

/* The shapes this engine's autotuner picks (the tcgen05 sketch tile N per
   element type and sketch order, the pivoted QR's row count for a thread
   per column, the SRFT kernel form per l'), read when a context is created
   from the table LRA_TUNING names or the one beside liblra.so
   (tuning_gb300.txt, written by lowrankapprox/autotune.py).  set overrides
   one entry of this context (keys "tc_tile_n" with index dtype * 16 +
   ceil(log2 order), "qr_seq_len", "srft_wide" with index log2 l'; index 0
   for the rest: "qr_steps" (adaptive steps a pivoted-QR launch may hold,
   1..8), "qr_sms" (SMs a QR launch may take, 0 all), "tc_split" (most K
   parts of the tensor-core sketch, 0 as many as fill the SMs),
   "jacobi_jb" (FP32 Jacobi block columns 4, 8, 16, 32; 0 by size),
   "jacobi_cluster" (largest cluster of the in-cluster FP32 Jacobi, 2..16;
   0 the largest schedulable, 1 never), "trsm_inv" (1: FP64 triangular
   solves on the tensor-core path by substitution instead of the
   unit-diagonal inverse), "gram_start" (cosine x 1e4 where the FP32 sweeps
   hand over to the Gram polish, 0 by order));
   get writes the table in force and its source as text and returns the
   length it needs (with the terminating zero).  No counterpart in the
   reference, whose BLAS picks its own blocking.                           */
int lra_ctx_set_tuning(lra_ctx* ctx, const char* key, int64_t index, int64_t value);
int lra_ctx_get_tuning(const lra_ctx* ctx, char* buf, int64_t len);

/* Limit of every bounded device-side wait (grid barriers, the pivoted QR's
   exchange between CTAs, the tensor-core sketch's mbarriers), in ns; 0
   restores the default of 4 s.  A wait that runs out makes its call return
   LRA_ETIMEDOUT and leaves the context usable.  The setting belongs to the
   device: it applies to every context on ctx's device.  Failure detection
   of this engine, no counterpart in the reference.                         */
int lra_ctx_set_wait_limit(lra_ctx* ctx, int64_t ns);
/* Self-test of the bounded waits: a two-CTA cooperative kernel meets at a
   grid barrier whose arrival count starts at the grid size, so no arrival
   completes it; both CTAs wait out the limit above and return.  Returns
   LRA_ETIMEDOUT when that happened as designed; any other status means the
   bounded-wait machinery misbehaved.                                       */
int lra_ctx_probe_wait(lra_ctx* ctx);

/* LRAOptions(T) defaults (src/LowRankApprox.jl:96-119) */
int lra_opts_init(lra_opts* opts, int dtype);
/* chkopts! (src/LowRankApprox.jl:133-141) */
int lra_chkopts(const lra_opts* opts);

/* ---- sketches (src/sketch.jl) -------------------------------------------- */

/* sketch(side, trans, A, order) (src/sketch.jl:35-46): writes B, which is
   order x M' (side 'l') or M' x order (side 'r'), into caller memory `B`
   (host or device), leading dimension ldb.                                 */
int lra_sketch(lra_ctx* ctx, int dtype, char side, char trans, int64_t m,
               int64_t n, const void* A, int64_t lda, int64_t order,
               const lra_opts* opts, const lra_rand* rand, void* B,
               int64_t ldb);

/* sketchfact(side, trans, A) (src/sketch.jl:52-63, 223-240): adaptive
   sketch + partial pivoted QR; returns PartialQRFactors with the options'
   pqrfact_retval (Q is the Q of the sketch, as in the reference).  side
   'l': the QR of S op(A) (order x N', pivots over the columns of op(A));
   side 'r': the QR of op(A) S (M' x order, pivots over the sketch's
   columns; its Q is prange's basis of the range of op(A)).                 */
int lra_sketchfact(lra_ctx* ctx, int dtype, char side, char trans, int64_t m,
                   int64_t n, const void* A, int64_t lda, const lra_opts* opts,
                   const lra_rand* rand, lra_pqr** out);

/* prange(trans, A, opts) (src/prange.jl:14-61): an orthonormal basis of the
   range of op(A) for trans 'n' / 'c' (the Q of sketchfact(:right, ...); of
   pqrfact with sketch :none; of the skeleton columns for :sub), or of the
   ranges of A and A' together for trans 'b' (A square).  The result holds
   Q only (m' x k, retval LRA_RET_Q), n = k and p the identity.  maxdet_tol
   >= 0 gives LRA_ENOTSUP.                                                   */
int lra_prange(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n,
               const void* A, int64_t lda, const lra_opts* opts,
               const lra_rand* rand, lra_pqr** out);

/* geqp3_adap! (src/pqr.jl:348-418) on a DEVICE matrix, in place: B (m x n,
   ldb) becomes R (upper) + Householder vectors (below), jpvt (n, int64,
   1-based) the column permutation, tau (min(m,n)) the reflector scalars,
   *k the detected rank.  Replaces the `_LAPACK.laqps!` ccall loop
   (src/lapack.jl:117-139 called from src/pqr.jl:394-416).                   */
int lra_geqp3_adap(lra_ctx* ctx, int dtype, int64_t m, int64_t n, void* B,
                   int64_t ldb, int64_t* jpvt, void* tau, const lra_opts* opts,
                   int64_t* k);

/* The same pivoted QR as lra_geqp3_adap, for callers that cannot allocate
   device memory while they factor: a serving loop that reserved all of its
   memory up front, or a host whose device allocator is owned by another
   framework.  It has no counterpart in the reference.  Its scratch (partial
   norms, pivot candidates, counters, grid barrier) is one fixed 1 MiB device
   array inside liblra, so the matrix may have at most 32768 columns (larger
   n returns LRA_EINVAL); B, jpvt and tau are caller-owned device buffers as
   above.  The first call on a device resolves the array's device address
   (cudaGetSymbolAddress) and caches it by device ordinal, so only the
   device's primary context is supported.  Each call synchronizes the
   context's stream and reads k back.  All calls on a device share the
   array: calls that overlap on the GPU race and must be serialized by the
   caller.  A rank of 0 (opts->rank == 0) returns k = 0 and the identity in
   jpvt.  No cudaMalloc / cudaFree or allocating library routine is called. */
int lra_geqp3_adap_noalloc(lra_ctx* ctx, int dtype, int64_t m, int64_t n, void* B,
                           int64_t ldb, int64_t* jpvt, void* tau,
                           const lra_opts* opts, int64_t* k);

/* n draws of the in-library generator, the one a call with rand == NULL
   uses in place of the reference's randn (src/util.jl:4-11,
   src/sketch.jl:92): Philox-4x32-10 keyed by `seed`, counters from
   `counter` on (each counter gives two values), Box-Muller, rounded to the
   1/32 lattice; written to out (host or device, float64).  On a fresh
   context a call draws its Gaussian sketches in adaptive-step order: step t
   takes order_t * M values at counter c_t, with c_0 = 0 and c_(t+1) = c_t +
   (order_t * M + 1) / 2.  Lets a caller reproduce the sketch a call used.  */
int lra_rand_gauss(lra_ctx* ctx, uint64_t seed, uint64_t counter, int64_t n,
                   double* out);

/* C = alpha op(A) op(B) + beta C in Float64 (column-major device arrays;
   trans 'n' or 't'), computed the way the factorizations compute their
   GEMMs: precision LRA_PREC_MIXED runs the tensor-core product of six
   exact BF16 byte slices per operand (error near 2^-45 of the rows' and
   columns' largest magnitudes), LRA_PREC_NATIVE the FP64 CUDA-core kernel.
   No counterpart in the reference, whose GEMMs are BLAS calls; exported so
   that the product the mixed path relies on can be checked directly.      */
int lra_dgemm(lra_ctx* ctx, int precision, char transa, char transb, int64_t m,
              int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
              const double* B, int64_t ldb, double beta, double* C, int64_t ldc);

/* ---- factorizations --------------------------------------------------------- */

/* idfact(trans, A) (src/id.jl:434-450) */
int lra_idfact(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n,
               const void* A, int64_t lda, const lra_opts* opts,
               const lra_rand* rand, lra_id** out);

/* pqrfact(trans, A) (src/pqr.jl:290-307) */
int lra_pqrfact(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n,
                const void* A, int64_t lda, const lra_opts* opts,
                const lra_rand* rand, lra_pqr** out);

/* psvdfact(A) (src/psvd.jl:238-272); psvdvals (src/psvd.jl:274-290) when
   vals_only != 0 (U and Vt are then NULL).                                  */
int lra_psvdfact(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A,
                 int64_t lda, const lra_opts* opts, const lra_rand* rand,
                 int vals_only, lra_psvd** out);

/* pheigfact(A) (src/pheig.jl:276-296); pheigvals (src/pheig.jl:298-311) */
int lra_pheigfact(lra_ctx* ctx, int dtype, int64_t n, const void* A,
                  int64_t lda, const lra_opts* opts, const lra_rand* rand,
                  int vals_only, lra_pheig** out);

/* curfact(A) (src/cur.jl:532-564) */
int lra_curfact(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A,
                int64_t lda, const lra_opts* opts, const lra_rand* rand,
                lra_cur** out);

/* the middle factor of CUR(A, U) (src/cur.jl:85-93, 100-115): the
   pseudo-inverse of A[rows, cols] (k x k, rows and cols 1-based host arrays
   of k entries each) as a PartialSVD (V, 1 ./ S, U'), with W = A[rows, cols]
   = U diag(S) V' computed on the device.  C = A[:, cols] and R = A[rows, :]
   are plain gathers the caller makes (the reference indexes A for them).
   For HermitianCURPackedU / SymmetricCURPackedU pass cols as rows too; the
   factor is the same pseudo-inverse, held as a PartialSVD.                  */
int lra_cur_middle(lra_ctx* ctx, int dtype, int64_t m, int64_t n,
                   const void* A, int64_t lda, int64_t k, const int64_t* rows,
                   const int64_t* cols, lra_psvd** out);

/* ---- spectral norms (src/snorm.jl) ------------------------------------------ */

/* snorm(A) (src/snorm.jl:14-45) */
int lra_snorm(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A,
              int64_t lda, int hermitian, const lra_opts* opts,
              const lra_rand* rand, double* out);
/* snormdiff(A, B) = snorm(A - B) (src/snorm.jl:50-53, src/linop.jl:176-187) */
int lra_snormdiff(lra_ctx* ctx, int dtype, int64_t m, int64_t n,
                  const void* A, int64_t lda, const void* B, int64_t ldb,
                  const lra_opts* opts, const lra_rand* rand, double* out);
/* snormdiff(A, F) with F = A[:, sk] * [I T] P' applied in factored form */
int lra_snormdiff_id(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n,
                     const void* A, int64_t lda, const lra_id* F,
                     const lra_opts* opts, const lra_rand* rand, double* out);
/* snormdiff(A, F) with F = U * diagm(S) * Vt applied in factored form */
int lra_snormdiff_psvd(lra_ctx* ctx, int dtype, int64_t m, int64_t n,
                       const void* A, int64_t lda, const lra_psvd* F,
                       const lra_opts* opts, const lra_rand* rand,
                       double* out);

/* ---- matrix-free operators (LinearOperator / HermitianLinearOperator,
   src/linop.jl:9-40) -----------------------------------------------------------
   An operator A (m x n) known only through the caller's product: matmat
   writes Y = op(A) X for trans 'n' (op(A) = A: X is n x ncols, Y m x ncols)
   or 'c' (op(A) = A': X is m x ncols, Y n x ncols), column-major DEVICE
   arrays of the operator's element type with leading dimensions ldx, ldy.
   It is called from the host thread of the library call, with X ready in
   the order of `stream` (a cudaStream_t), and must either enqueue its work
   on that stream or finish it before it returns; it returns 0, or nonzero
   to make the call fail with LRA_ECUDA.  hermitian != 0 marks a
   HermitianLinearOperator (m == n, A' = A): matmat is then called with 'n'
   only.  As in the reference (chkopts!, src/LowRankApprox.jl:142-148), a
   factorization of an operator uses the Gaussian sketch whatever
   opts->sketch says; it runs in native precision (the products are the
   caller's) and without the finite check.  A[:, cols] and A[rows, :] are
   formed as products with unit columns (src/linop.jl:56-77).              */
typedef int (*lra_matmat_fn)(void* user, char trans, int64_t ncols, const void* X, int64_t ldx, void* Y,
                             int64_t ldy, void* stream);

typedef struct lra_linop {
  int64_t m, n;
  int32_t dtype;       /* LRA_F32 / LRA_F64 */
  int32_t hermitian;
  lra_matmat_fn matmat;
  void* user;
} lra_linop;

/* sketchfact / idfact / pqrfact / prange / psvdfact (psvdvals) / pheigfact
   (pheigvals) / curfact / snorm of an operator: the entry points above with
   A given as a lra_linop (src/sketch.jl:52-66, src/id.jl:434-450,
   src/pqr.jl:290-307, src/prange.jl:14-61, src/psvd.jl:238-290,
   src/pheig.jl:276-311, src/cur.jl:532-564, src/snorm.jl:14-45)         */
int lra_sketchfact_linop(lra_ctx* ctx, char side, char trans, const lra_linop* A, const lra_opts* opts,
                         const lra_rand* rand, lra_pqr** out);
int lra_idfact_linop(lra_ctx* ctx, char trans, const lra_linop* A, const lra_opts* opts,
                     const lra_rand* rand, lra_id** out);
int lra_pqrfact_linop(lra_ctx* ctx, char trans, const lra_linop* A, const lra_opts* opts,
                      const lra_rand* rand, lra_pqr** out);
int lra_prange_linop(lra_ctx* ctx, char trans, const lra_linop* A, const lra_opts* opts,
                     const lra_rand* rand, lra_pqr** out);
int lra_psvdfact_linop(lra_ctx* ctx, const lra_linop* A, const lra_opts* opts, const lra_rand* rand,
                       int vals_only, lra_psvd** out);
int lra_pheigfact_linop(lra_ctx* ctx, const lra_linop* A, const lra_opts* opts, const lra_rand* rand,
                        int vals_only, lra_pheig** out);
int lra_curfact_linop(lra_ctx* ctx, const lra_linop* A, const lra_opts* opts, const lra_rand* rand,
                      lra_cur** out);
int lra_snorm_linop(lra_ctx* ctx, const lra_linop* A, const lra_opts* opts, const lra_rand* rand,
                    double* out);

/* ---- batches of independent matrices ---------------------------------------- */

/* idfact over `count` matrices of uneven sizes (many independent idfact
   calls, src/id.jl:434-450).  The matrices are spread over up to eight
   worker streams of a private server (below), so that their work overlaps
   on the device; outs[i] receives matrix i's IDPackedV, identical to a
   single lra_idfact call on it.  rand may be NULL or an array of `count`
   streams.                                                                 */
int lra_idfact_batched(lra_ctx* ctx, int dtype, int64_t count,
                       const lra_matdesc* mats, const lra_opts* opts,
                       const lra_rand* rand, lra_id** outs);

/* ---- serving loop (continuous batching) --------------------------------------
   No counterpart in the reference, which factors one matrix per call.  A
   server owns `slots` workers (host thread + context + stream each) on one
   device.  Submitted requests are admitted in arrival order as soon as a
   slot is free and their estimated device memory fits `hbm_budget_bytes`
   beside the requests already running; admitted requests run concurrently.
   Each request runs as a fresh idfact / psvdfact call (the in-library
   generator restarts from opts.seed), so its result is the same whichever
   slot runs it and whatever runs beside it.  A request's A and rand must
   stay valid until its result has been polled.                             */
typedef struct lra_server lra_server;

enum { LRA_REQ_IDFACT = 0, LRA_REQ_PSVDFACT = 1 };

typedef struct lra_request {
  int32_t kind;          /* LRA_REQ_* */
  int32_t dtype;         /* LRA_F32 / LRA_F64 */
  char trans;            /* idfact: 'n' or 'c' (0 means 'n') */
  char _pad[7];
  int64_t m, n, lda;
  const void* A;         /* host or device, column-major */
  lra_opts opts;
  const lra_rand* rand;  /* optional injected randomness */
} lra_request;

typedef struct lra_result {
  int32_t kind;          /* LRA_REQ_* of the request */
  int32_t status;        /* LRA_* status of the factorization */
  lra_id* id;            /* LRA_REQ_IDFACT: free with lra_id_free */
  lra_psvd* psvd;        /* LRA_REQ_PSVDFACT: free with lra_psvd_free */
  double queue_ms;       /* submit -> start */
  double run_ms;         /* start -> done */
  double total_ms;       /* submit -> done */
  int32_t slot;
  int32_t _pad;
  char error[160];       /* lra_last_error text when status != LRA_OK */
} lra_result;

typedef struct lra_server_stats {
  int64_t submitted, completed, rejected, in_flight, queued;
  double p50_ms, p99_ms, mean_ms;  /* submit -> done, completed requests */
  double matrices_per_s;           /* completed / (last done - first submit) */
  int64_t hbm_budget, hbm_in_use;  /* bytes, by the admission estimates */
} lra_server_stats;

int lra_server_create(int device, int slots, int64_t hbm_budget_bytes,
                      lra_server** out);
/* LRA_ENOMEM (and nothing queued) when the request alone exceeds the budget */
int lra_server_submit(lra_server* s, const lra_request* req, uint64_t* ticket);
/* wait_ms < 0 waits for completion, 0 only checks.  LRA_OK: done, *out
   filled and the ticket released; LRA_EBUSY: not done yet.                 */
int lra_server_poll(lra_server* s, uint64_t ticket, int64_t wait_ms,
                    lra_result* out);
int lra_server_get_stats(lra_server* s, lra_server_stats* out);
/* running requests finish, queued ones are dropped, unpolled results freed */
void lra_server_destroy(lra_server* s);

/* ---- freeing ---------------------------------------------------------------- */
void lra_id_free(lra_id* r);
void lra_pqr_free(lra_pqr* r);
void lra_psvd_free(lra_psvd* r);
void lra_pheig_free(lra_pheig* r);
void lra_cur_free(lra_cur* r);

#ifdef __cplusplus
}
#endif

#endif /* LRA_H */
