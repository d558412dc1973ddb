// Internal interfaces of liblra: context, workspace arena, kernel launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/lra.h"
#include "cplx.cuh"

namespace lra {

// Error carried from the point of failure to the C ABI boundary.
struct Error {
  int status;
  std::string msg;
};

[[noreturn]] void fail(int status, const char* fmt, ...);
void check_cuda(cudaError_t e, const char* what);
#define LRA_CUDA(x) ::lra::check_cuda((x), #x)

// Device workspace: bump allocation in chunks that never move while a call
// runs (so earlier pointers stay valid).  All work of a context is ordered
// on its one stream, so rewinding to a mark and reusing memory is safe.
// At the start of a call, several chunks are merged into one.
struct ArenaMark {
  size_t chunk;
  size_t used;
};

class Arena {
 public:
  ~Arena();
  void* alloc(size_t bytes);  // 256-byte aligned
  template <typename T>
  T* alloc_n(size_t n) {
    return static_cast<T*>(alloc(n * sizeof(T)));
  }
  ArenaMark mark() const;
  void release(ArenaMark m);
  // start of a call: merge chunks (synchronizes the stream first)
  void reset(cudaStream_t stream);
  // give every chunk back to the device (synchronizes the stream first)
  void free_all(cudaStream_t stream);
  size_t capacity() const;

 private:
  struct Chunk {
    char* base;
    size_t cap;
    size_t used;
  };
  std::vector<Chunk> chunks_;
  size_t cur_ = 0;
};

}  // namespace lra

// Shapes the autotuner (lowrankapprox/autotune.py) picks, read from its
// table when a context is created (ctx.cpp: load_tuning); the defaults are
// the shapes the sweeps before it had chosen.
struct lra_tuning {
  // tcgen05 sketch tile N (32, 64 or 96 sketch rows per CTA) by element
  // type (0 Float32, 1 Float64) and ceil(log2(sketch order)), 0..15
  int tc_tile_n[2][16];
  // rows below which the double-float pivoted QR sums a column with one
  // thread (a warp per four columns above)
  int qr_seq_len;
  // Float32 SRFT: 1 selects the 512-thread swizzled form for log2(l') when
  // it applies (7..10), 0 the 256-thread padded form
  int srft_wide[11];
  // adaptive sketch steps the shared-memory pivoted QR may factor in one
  // launch (1: one step at a time)
  int qr_steps;
  // SMs a pivoted-QR launch may take (0: all); more when the sketch needs
  // them to fit shared memory.  The serving loop shares the device this way
  int qr_sms;
  // most parts the tensor-core sketch splits K into when its tiles are too
  // few for the SMs (0: as many as fill them, 1: no split)
  int tc_split;
  // columns per block of the FP32 block Jacobi (4, 8, 16, 32; 0: by size)
  int jacobi_jb;
  // largest cluster of the cluster-resident FP32 Jacobi (2..16; 0: the
  // largest that can be scheduled; 1: never, the block-pair kernel instead)
  int jacobi_cluster;
  // FP64 triangular solves on the tensor-core path: 0 multiply by the
  // explicit inverse (k from 65 to 2048), 1 blocked substitution
  int trsm_inv;
  // largest cosine, in units of 1e-4, at which the FP32 sweeps hand the
  // core SVD to the Gram polish (0: min(3e-2, 12 / n))
  int gram_start;
};

struct lra_ctx {
  // device word that kernels with bounded waits set when one gave up,
  // read once at the end of the library call (tc_gemm arms it instead of
  // waiting for its own launch)
  int* dev_err = nullptr;
  bool dev_err_armed = false;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  lra::Arena arena;
  std::string last_error;
  int64_t launches = 0;
  std::unordered_map<std::string, int64_t> launches_by_name;
  double stage_ms[4] = {0, 0, 0, 0};
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  uint64_t rng_counter = 0;  // advances per call of the in-library generator
  // the mixed-precision path sends large Float64 GEMMs to tc_gemm
  bool gemm_tc = false;
  // rtol of the current mixed-precision call (0 otherwise)
  double mixed_rtol = 0;
  // pinned host staging (grown on demand)
  void* pinned = nullptr;
  size_t pinned_cap = 0;
  // side streams of the batched path and their join events (made on first use)
  static constexpr int kAux = 8;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t aux_ev[kAux + 1] = {};
  // the operator of a matrix-free call (lra_*_linop) while it runs, else null
  const lra_linop* linop = nullptr;
  lra_tuning tuning{};
  std::string tuning_source;  // the table file read, or "defaults"
};

namespace lra {

// ---- launchers (defined in the .cu files) ---------------------------------

// C = alpha * op(A) * op(B) + beta * C, column-major, CUDA cores.
template <typename T>
void gemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, T alpha,
          const T* A, int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc);

// op(A) (M x N) cut into `ns` exact BF16 byte slices at per-column
// power-of-two scales (K-major planes, ld = Kp), built once per call and
// reused by every adaptive sketch step.
struct TcSplit {
  int64_t K = 0, N = 0, Kp = 0;
  int ns = 0;
  char trans = 'n';
  int* colexp = nullptr;
  void* slices = nullptr;
};
bool tc_sketch_supported(int64_t order, int64_t M, int64_t N);
template <typename T>
void tc_split(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda, int ns,
              TcSplit* out, bool balanced = false);
// B (order x N, ldb) = S op(A) on tcgen05 tensor cores; S is order x M
// (ld = order) with entries on the 1/32 lattice.
template <typename T>
void tc_sketch(lra_ctx* ctx, const TcSplit& sp, int64_t order, const T* S, T* B, int64_t ldb,
               int* err_slot = nullptr);

// Raises a kernel's dynamic shared memory limit to the most the device
// allows beside its static shared memory.  Always the same value per kernel:
// the attribute is global to the kernel, and a per-call value set by one
// host thread could undercut another thread's launch in between.
void raise_smem_limit(lra_ctx* ctx, const void* kernel);

// LRA_TRACE=1 in the environment: iteration counts of the iterative
// kernels (Jacobi sweeps, pivots) on stderr.
bool trace_on();

// Keeps a stretch of work on the FP64 CUDA-core GEMM (products whose
// result must be orthonormal to working precision).
struct NativeGemmScope {
  lra_ctx* ctx;
  bool saved;
  explicit NativeGemmScope(lra_ctx* c) : ctx(c), saved(c->gemm_tc) { c->gemm_tc = false; }
  ~NativeGemmScope() { ctx->gemm_tc = saved; }
  NativeGemmScope(const NativeGemmScope&) = delete;
  NativeGemmScope& operator=(const NativeGemmScope&) = delete;
};

// C = alpha op(A) op(B) + beta C in Float64 on tcgen05 tensor cores from
// six exact BF16 byte slices of each operand (error near 2^-45 of the
// row / column scales); used by the mixed-precision path.
bool tc_gemm_worthwhile(int64_t m, int64_t n, int64_t k);
void tc_gemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
             int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc);

// The mixed path's pivoted QR of many Float64 sketches at once (a CTA per
// matrix): each B (m x n, ld ldb) is factored in place, its jpvt and tau
// filled and its rank written to k_dev[i], as geqp3_adap would.
struct DfBatchItem {
  int64_t m, n, ldb, kmax;
  double* B;
  int64_t* jpvt;
  double* tau;
};
bool geqp3_df_batch_fits(lra_ctx* ctx, int64_t m, int64_t n);
// lra_idfact_batched's grouped path: whether the batch qualifies, and the run
bool grouped_batch_ok(lra_ctx* ctx, int64_t count, const lra_matdesc* mats, const lra_opts& o, const lra_rand* rand);
void idfact_batched_grouped(lra_ctx* ctx, int64_t count, const lra_matdesc* mats, const lra_opts& o,
                            lra_id** outs);
// -1 when the batch does not qualify for the grouped path, else its status
int try_idfact_batched_grouped(lra_ctx* ctx, int dtype, int64_t count, const lra_matdesc* mats,
                               const lra_opts* opts, const lra_rand* rand, lra_id** outs);
void geqp3_df_batch(lra_ctx* ctx, int64_t count, const DfBatchItem* items, int64_t nb, double atol, double rtol,
                    int64_t* k_dev);

// Rank-adaptive column-pivoted Householder QR (geqp3_adap!), in place.
// pivot == false runs the same Householder QR without pivoting.
// Several adaptive steps' sketches factored by one launch of the
// shared-memory pivoted QR, each on CTAs of its own.  A step whose rank
// comes out below its threshold (k < nt) stops the steps after it at their
// next pivot; the factors (A, jpvt, tau) are written for the first such step
// only.  k[i] is step i's rank (-1 for a step that a lower one stopped).
// Returns the index of that first step, or -1 when every step's rank reached
// its threshold (no factors written).
template <typename T>
struct QrStep {
  int64_t m, n;
  T* A;
  int64_t lda;
  int64_t* jpvt;
  T* tau;
  int64_t kmax, nt;
};
// how many of the leading steps (m[i] x n sketches, i < count) one launch can
// hold together: 0 when the shared-memory kernel does not apply
template <typename T>
int geqp3_steps_fit(lra_ctx* ctx, int count, const int64_t* m, int64_t n);
template <typename T>
int geqp3_adap_steps(lra_ctx* ctx, int count, const QrStep<T>* steps, int64_t nb, double atol, double rtol,
                     int64_t* k);

template <typename T>
int64_t geqp3_adap(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda, int64_t* jpvt,
                   T* tau, int64_t kmax, int64_t nb, double atol, double rtol, bool pivot);

// The same pivoted QR with its scratch in a fixed device array instead of
// the context arena (no device allocation); n <= noalloc_max_cols().
template <typename T>
int64_t geqp3_adap_noalloc(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda, int64_t* jpvt, T* tau,
                           int64_t kmax, int64_t nb, double atol, double rtol);
int64_t noalloc_max_cols();

// X (k x nrhs) <- triu(R)^{-1} X, R k x k (ldr).
template <typename T>
void trsm_left_diag(lra_ctx* ctx, int jb, int64_t nrhs, const T* R, int64_t ldr, T* X, int64_t ldx);
// X <- triu(R)^{-1} X (k <= kBsMax) by back substitution, a thread per column
constexpr int kBsMax = 128;
template <typename T>
void trsm_bs(lra_ctx* ctx, int64_t k, int64_t nrhs, const T* R, int64_t ldr, T* X, int64_t ldx);
// the batch's T = R11^{-1} R12 (R11, R12 from B, ld ldb; T k x nr, ld k)
struct BsItem {
  int64_t k, nr, ldb;
  const double* B;
  double* T;
};
void trsm_bs_batch(lra_ctx* ctx, int64_t count, const BsItem* items);
// the batch's results into one device buffer: at byte offset off, n int64
// (jpvt, 1-based) then nt doubles (T)
struct PackItem {
  int64_t n, nt;
  const int64_t* jpvt;
  const double* T;
  size_t off;
};
void pack_results(lra_ctx* ctx, int64_t count, const PackItem* items, char* out);
template <typename T>
void trsm_upper(lra_ctx* ctx, int64_t k, int64_t nrhs, const T* R, int64_t ldr, T* X,
                int64_t ldx, const T* Yd = nullptr);

// Householder vectors (below the diagonal of V, m x k) applied to X
// (m x nc): X <- Q X (trans 'n') or Q^T X (trans 't').
template <typename T>
void apply_q(lra_ctx* ctx, char trans, int64_t m, int64_t k, const T* V, int64_t ldv,
             const T* tau, T* X, int64_t ldx, int64_t nc);

// Explicit Q (m x k) from Householder vectors (LAPACK xORGQR).
template <typename T>
void orgqr(lra_ctx* ctx, int64_t m, int64_t k, T* V, int64_t ldv, const T* tau);

// One-sided Jacobi SVD of X (n x n, square, in place): on exit X = U * S,
// V (n x n) accumulates the right rotations, S gets the column norms.
template <typename T>
// stop > 0 ends the sweeps once a sweep's largest cosine is below it
void jacobi_svd(lra_ctx* ctx, int64_t n, T* X, int64_t ldx, T* V, int64_t ldv, T* S, bool quadratic_stop = false,
                double stop = 0);

// G = R^T R in place (upper R, lower part zeroed), blocked; false when G is
// not numerically positive definite
template <typename T>
bool potrf_upper(lra_ctx* ctx, int64_t k, T* G, int64_t ldg);
// n (1 or 2) independent factorizations as potrf_upper, in one launch
template <typename T>
void potrf_upper_batch(lra_ctx* ctx, int n, const int64_t* k, T* const* G, const int64_t* ldg, bool* ok);
// cholqr_pre with one pass and chol_v at once (their factorizations batched)
template <typename T>
bool cholqr1_and_chol_v(lra_ctx* ctx, int64_t m, int64_t k, T* X, int64_t ldx, const T* Rpre, int64_t ldr, T* Rc,
                        int64_t nr, const T* Tm, T* Rv, const T* Rpre_inv = nullptr);
// X (m x k) <- X triu(R)^{-1}, blocked (or times the explicit inverse, see
// trsm_by_inverse)
template <typename T>
void trsm_right_upper(lra_ctx* ctx, int64_t m, int64_t k, const T* R, int64_t ldr, T* X, int64_t ldx,
                      const T* Yd = nullptr);
// Y = triu(R)^{-1} diag(R) (k x k, ld ldy); false when k is beyond the
// kernel (2048)
template <typename T>
bool tri_inv_upper(lra_ctx* ctx, int64_t k, const T* R, int64_t ldr, T* Y, int64_t ldy);
// dst = src with rows (side 'l') or columns ('r') divided by diag(R)
template <typename T>
void div_by_diag(lra_ctx* ctx, int64_t m, int64_t n, const T* R, int64_t ldr, char side, const T* src, int64_t lds,
                 T* dst, int64_t ldd);
template <typename T>
bool trsm_by_inverse(const lra_ctx* ctx, int64_t k, int64_t other);

// post.cu: X (m x k) <- X Rpre^{-1} (if Rpre), then `passes` Cholesky QR
// passes; on exit X is orthonormal and the input equals X Rc Rpre.  False
// on a Cholesky breakdown.
template <typename T>
bool cholqr_pre(lra_ctx* ctx, int64_t m, int64_t k, T* X, int64_t ldx, const T* Rpre, int64_t ldr,
                int passes, T* Rc);
// Rv = chol(I + T T^T) for the k x nr matrix T (ld k)
template <typename T>
bool chol_v(lra_ctx* ctx, int64_t k, int64_t nr, const T* Tm, T* Rv);
// SVD of the k x k matrix Mm (ld k): U diag(S) V^T, S descending (returned)
template <typename T>
std::vector<T> small_svd(lra_ctx* ctx, int64_t k, const T* Mm, T* U, T* V, T* S);
template <typename T>
std::vector<T> sort_desc(lra_ctx* ctx, int64_t k, T* S, T* U, T* V);

// Polish sweeps of the mixed-precision path in double-float (X and V
// Float64 in and out, V overwritten); false when n does not fit.
bool jacobi_svd_df(lra_ctx* ctx, int64_t n, double* X, int64_t ldx, double* V, int64_t ldv, double* S);
// jacobi_svd for Float64 with the bulk of the sweeps in FP32 and FP64 polish
template <typename T>
void jacobi_svd_fast(lra_ctx* ctx, int64_t n, T* X, int64_t ldx, T* V, int64_t ldv, T* S);

// exact symmetry test of a square device matrix
template <typename T>
bool is_symmetric(lra_ctx* ctx, int64_t n, const T* A, int64_t lda);

// ---- small elementwise / data-movement kernels (kernels_misc.cu) -----------
template <typename T>
void copy_matrix(lra_ctx* ctx, int64_t m, int64_t n, const T* src, int64_t lds, T* dst,
                 int64_t ldd);
template <typename T>
void transpose(lra_ctx* ctx, int64_t m, int64_t n, const T* src, int64_t lds, T* dst,
               int64_t ldd);
// dst(:, j) = src(:, idx[j] - 1) (1-based idx on the device)
template <typename T>
void gather_cols(lra_ctx* ctx, int64_t m, int64_t k, const T* src, int64_t lds,
                 const int64_t* idx, T* dst, int64_t ldd);
// dst(i, :) = src(idx[i] - 1, :)
template <typename T>
void gather_rows(lra_ctx* ctx, int64_t k, int64_t n, const T* src, int64_t lds,
                 const int64_t* idx, T* dst, int64_t ldd);
// dst(:, idx[j] - 1) = src(:, j)
template <typename T>
void scatter_cols(lra_ctx* ctx, int64_t m, int64_t k, const T* src, int64_t lds,
                  const int64_t* idx, T* dst, int64_t ldd);
template <typename T>
void set_zero(lra_ctx* ctx, T* p, int64_t n);
template <typename T>
void set_identity(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda);
// lower part (below diagonal) of A (m x n) set to zero
template <typename T>
void zero_lower(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda);
// 1/32-lattice rounding of a Gaussian stream, converting to T
template <typename T>
void sketch_from_stream(lra_ctx* ctx, const double* g, int64_t n, T* out, bool lattice);
// in-library lattice Gaussians (Philox-4x32-10, key = seed, counter = base + i)
template <typename T>
void sketch_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, T* out);
// in-library uniform integers in [1, hi] and permutations of 1..n
void ints_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, int64_t hi, int64_t* out);
void perm_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, int64_t* out);
// B(i, j) = 0.5 (B(i, j) + B(j, i)) on both triangles (hermitianize!)
template <typename T>
void symmetrize(lra_ctx* ctx, int64_t n, T* B, int64_t ldb);
// A(i, i) += s
template <typename T>
void add_diag(lra_ctx* ctx, int64_t n, T* A, int64_t lda, T s);
// dst(idx[i] - 1, :) = src(i, :)
template <typename T>
void scatter_rows(lra_ctx* ctx, int64_t k, int64_t n, const T* src, int64_t lds,
                  const int64_t* idx, T* dst, int64_t ldd);
// x *= s
template <typename T>
void scale_vec(lra_ctx* ctx, int64_t n, T* x, T s);
// columns j of X (m x n) divided by s[j] (skipped where s[j] == 0)
template <typename T>
void div_cols(lra_ctx* ctx, int64_t m, int64_t n, T* X, int64_t ldx, const T* s);
// pheigorth!: Gram-Schmidt inside eigenvalue clusters, cl = cluster bounds
template <typename T>
void cluster_orth(lra_ctx* ctx, int64_t n, int64_t k, T* Z, int64_t ldz, const int64_t* cl,
                  int64_t ncl);
// nonfinite check: returns true when every entry is finite
template <typename T>
bool all_finite(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda);
template <typename T>
void all_finite_async(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda, int* bad);

// column 2-norms
template <typename T>
void col_norms(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda, T* out);

// SRFT / subset / sparse-Gaussian sketches (sketch.cu), left side, op(A)
template <typename T>
void srft_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                 const T* d, const int64_t* idx, int64_t order, T* B, int64_t ldb);
template <typename T>
void sub_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                const int64_t* rows, int64_t order, T* B, int64_t ldb);
template <typename T>
void srft_signs(lra_ctx* ctx, const double* g, int64_t n, T* d);
// FFT-based SRFT (srft.cu); false when the shape needs srft_sketch
template <typename T>
bool srft_sketch_fft(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda, const T* d,
                     const int64_t* idx, int64_t order, T* B, int64_t ldb);
template <typename T>
void sprn_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                 const int64_t* perm, const T* g, int64_t order, T* B, int64_t ldb);

// y = op(A) x (gemv), CUDA cores
template <typename T>
void gemv(lra_ctx* ctx, char trans, int64_t m, int64_t n, T alpha, const T* A, int64_t lda,
          const T* x, T beta, T* y);

// kernel-launch accounting (every launcher calls this once per launch)
inline void count_launch(lra_ctx* ctx, int n = 1) { ctx->launches += n; }
void post_launch(lra_ctx* ctx, const char* name);

// the bounded-wait limit of each translation unit that waits (ns; 0: the
// default), and the grid-barrier self-test: returns the barrier's error
// word (4 when its wait ran out) and the number of CTAs that returned
cudaError_t set_wait_limit_qr(uint64_t ns);
cudaError_t set_wait_limit_dense(uint64_t ns);
cudaError_t set_wait_limit_tc(uint64_t ns);
int probe_grid_wait(lra_ctx* ctx, int* returned);

// the tuning table: defaults, then the file named by LRA_TUNING or the
// table beside liblra.so (tuning_gb300.txt); the source is recorded
void load_tuning(lra_tuning* t, std::string* source);
// one entry by name ("tc_tile_n", "qr_seq_len", "srft_wide"), the index
// addressing the table (dtype * 16 + log2 order; log2 l'); false if unknown
bool set_tuning(lra_tuning* t, const char* key, int64_t index, int64_t value);
std::string tuning_text(const lra_tuning& t);

// ---- complex element types (cplx.cu) -------------------------------------------------
// C = alpha op(A) op(B) + beta C, op 'n', 't' or 'c' (conjugate transpose)
template <typename R>
void cgemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, cx<R> alpha, const cx<R>* A,
           int64_t lda, const cx<R>* B, int64_t ldb, cx<R> beta, cx<R>* C, int64_t ldc);
// dst (n x m) = src^H; A <- conj(A)
template <typename R>
void cadjoint(lra_ctx* ctx, int64_t m, int64_t n, const cx<R>* src, int64_t lds, cx<R>* dst, int64_t ldd);
template <typename R>
void cconj(lra_ctx* ctx, int64_t m, int64_t n, cx<R>* A, int64_t lda);
template <typename R>
void ccol_norms(lra_ctx* ctx, int64_t m, int64_t n, const cx<R>* A, int64_t lda, R* out);
// geqp3_adap! with ZLAQPS / CLAQPS rules (pivot) or a plain Householder QR
template <typename R>
int64_t cgeqp3(lra_ctx* ctx, int64_t m, int64_t n, cx<R>* A, int64_t lda, int64_t* jpvt, cx<R>* tau, int64_t kmax,
               int64_t nb, double atol, double rtol, bool pivot);
// X <- Q X ('n') or Q^H X ('c'), Q = H_1 ... H_k of the QR's reflectors
template <typename R>
void capply_q(lra_ctx* ctx, char trans, int64_t m, int64_t k, const cx<R>* V, int64_t ldv, const cx<R>* tau,
              cx<R>* X, int64_t ldx, int64_t nc);
template <typename R>
void corgqr(lra_ctx* ctx, int64_t m, int64_t k, cx<R>* V, int64_t ldv, const cx<R>* tau);
template <typename R>
void ctrsm_upper(lra_ctx* ctx, int64_t k, int64_t nrhs, const cx<R>* R_, int64_t ldr, cx<R>* X, int64_t ldx);
// one-sided Jacobi: X (k x k) <- U, V, S (unsorted) with X = U diag(S) V^H
template <typename R>
void cjacobi_svd(lra_ctx* ctx, int64_t k, cx<R>* X, int64_t ldx, cx<R>* V, int64_t ldv, R* S);
template <typename R>
bool cis_hermitian(lra_ctx* ctx, int64_t n, const cx<R>* A, int64_t lda);
template <typename R>
void chermitianize(lra_ctx* ctx, int64_t n, cx<R>* B, int64_t ldb);
template <typename R>
void cadd_diag(lra_ctx* ctx, int64_t n, cx<R>* A, int64_t lda, R s);
template <typename R>
void cphases(lra_ctx* ctx, const double* g, int64_t n, cx<R>* d);
template <typename R>
void csrft_direct(lra_ctx* ctx, char trans, int64_t M, int64_t N, const cx<R>* A, int64_t lda, const cx<R>* d,
                  const int64_t* idx, int64_t order, cx<R>* B, int64_t ldb);
template <typename R>
void csprn(lra_ctx* ctx, char trans, int64_t M, int64_t N, const cx<R>* A, int64_t lda, const int64_t* perm,
           const cx<R>* g, const int64_t* start, int64_t order, cx<R>* B, int64_t ldb);
template <typename R>
void csub(lra_ctx* ctx, char trans, int64_t N, const cx<R>* A, int64_t lda, const int64_t* rows, int64_t order,
          cx<R>* B, int64_t ldb);
template <typename R>
bool cmaxdet_step(lra_ctx* ctx, int64_t k, int64_t nr, cx<R>* T, int64_t* jpvt, double bound, bool update, cx<R>* R1,
                  int64_t ldr);
template <typename R>
void ccluster_orth(lra_ctx* ctx, int64_t n, int64_t k, cx<R>* Z, int64_t ldz, const int64_t* cl, int64_t ncl);

}  // namespace lra
