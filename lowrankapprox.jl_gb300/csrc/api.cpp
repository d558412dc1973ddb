// C ABI of liblra: option handling, randomness, and the host-side drivers
// of the sketch-then-factor path.  Every numerical stage runs on the GPU;
// the host only sequences launches and reads back the few scalars the
// reference's control flow branches on (the rank of each adaptive step,
// the singular / eigen values that decide the truncation).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <limits>
#include <numeric>
#include <vector>
#include <unordered_map>
#include <map>
#include <mutex>

#include "internal.hpp"

namespace lra {

namespace {

bool is_dev(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

template <typename T>
struct DMat {
  const T* p;
  int64_t ld;
};

template <typename T>
DMat<T> stage_in(lra_ctx* ctx, const void* A, int64_t m, int64_t n, int64_t lda) {
  if (ctx->linop) return DMat<T>{nullptr, std::max<int64_t>(m, 1)};  // matrix-free: no entries to stage
  if (m == 0 || n == 0) return DMat<T>{static_cast<const T*>(A), std::max<int64_t>(lda, 1)};
  if (!A) fail(LRA_EINVAL, "null matrix pointer");
  if (lda < std::max<int64_t>(1, m)) fail(LRA_EDIM, "lda (%lld) < m (%lld)", (long long)lda, (long long)m);
  if (is_dev(A)) return DMat<T>{static_cast<const T*>(A), lda};
  T* d = ctx->arena.alloc_n<T>((size_t)m * n);
  LRA_CUDA(cudaMemcpy2DAsync(d, m * sizeof(T), A, lda * sizeof(T), m * sizeof(T), n, cudaMemcpyHostToDevice,
                             ctx->stream));
  return DMat<T>{d, m};
}

template <typename T>
void to_host(lra_ctx* ctx, void* dst, const T* src, size_t n) {
  if (n == 0) return;
  LRA_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
}

// Result arrays of 1 MiB and more live in page-locked host memory, so that
// the device-to-host copies run at the link's speed (the CUDA runtime stages a
// pageable copy at a fraction of it: 19 vs 180 GB/s measured on a GB300
// node).  Blocks freed through lra_*_free are kept for reuse, up to 2 GiB.
std::mutex g_pin_mu;
std::multimap<size_t, void*> g_pin_free;
std::unordered_map<void*, size_t> g_pin_live;
size_t g_pin_cached = 0;
constexpr size_t kPinMin = (size_t)1 << 20;
constexpr size_t kPinCacheCap = (size_t)2 << 30;

void* hmalloc(size_t bytes) {
  if (bytes >= kPinMin) {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin_free.lower_bound(bytes);
    if (it != g_pin_free.end() && it->first <= 2 * bytes) {
      void* p = it->second;
      const size_t sz = it->first;
      g_pin_free.erase(it);
      g_pin_cached -= sz;
      g_pin_live[p] = sz;
      return p;
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) == cudaSuccess && p) {
      g_pin_live[p] = bytes;
      return p;
    }
    cudaGetLastError();  // no page-locked memory left: pageable below
  }
  void* p = std::malloc(bytes ? bytes : 1);
  if (!p) fail(LRA_ENOMEM, "host allocation of %zu bytes", bytes);
  return p;
}

// A slab holds many result arrays at once (the batched path copies all its
// results in one transfer); it goes back to the cache when the last array in
// it has been freed.  Every array must start strictly inside its slab.
struct Slab {
  size_t size;
  int refs;
  bool pinned;
};
std::map<char*, Slab> g_slabs;  // by base address

char* hslab(size_t bytes, int refs) {
  char* p = nullptr;
  bool pinned = false;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin_free.lower_bound(bytes);
    if (it != g_pin_free.end() && it->first <= 2 * bytes) {
      p = static_cast<char*>(it->second);
      bytes = it->first;
      g_pin_cached -= it->first;
      g_pin_free.erase(it);
      pinned = true;
    }
  }
  if (!p) {
    void* q = nullptr;
    if (cudaHostAlloc(&q, bytes, cudaHostAllocPortable) == cudaSuccess && q) {
      p = static_cast<char*>(q);
      pinned = true;
    } else {
      cudaGetLastError();
      p = static_cast<char*>(std::malloc(bytes));
      if (!p) fail(LRA_ENOMEM, "host allocation of %zu bytes", bytes);
    }
  }
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_slabs[p] = Slab{bytes, refs, pinned};
  return p;
}

void hfree(void* p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin_live.find(p);
    if (it != g_pin_live.end()) {
      const size_t sz = it->second;
      g_pin_live.erase(it);
      if (g_pin_cached + sz <= kPinCacheCap) {
        g_pin_free.emplace(sz, p);
        g_pin_cached += sz;
      } else {
        cudaFreeHost(p);
      }
      return;
    }
    auto sl = g_slabs.upper_bound(static_cast<char*>(p));
    if (sl != g_slabs.begin()) {
      --sl;
      char* base = sl->first;
      if (static_cast<char*>(p) >= base && static_cast<char*>(p) < base + sl->second.size) {
        if (--sl->second.refs == 0) {
          const Slab s = sl->second;
          g_slabs.erase(sl);
          if (!s.pinned) {
            std::free(base);
          } else if (g_pin_cached + s.size <= kPinCacheCap) {
            g_pin_free.emplace(s.size, base);
            g_pin_cached += s.size;
          } else {
            cudaFreeHost(base);
          }
        }
        return;
      }
    }
  }
  std::free(p);
}

// ---- stage timing (CUDA events on the context stream) ----------------------
struct Stage {
  lra_ctx* ctx;
  int idx;
  cudaEvent_t a = nullptr, b = nullptr;
  Stage(lra_ctx* c, int i) : ctx(c), idx(i) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, ctx->stream);
  }
  ~Stage() {
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0;
    if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess) ctx->stage_ms[idx] += ms;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaGetLastError();
  }
};

// ---- randomness ---------------------------------------------------------------
struct RandSrc {
  lra_ctx* ctx;
  const lra_rand* r;
  uint64_t seed;
  int64_t g = 0, q = 0;
  bool gdev = false, qdev = false;

  RandSrc(lra_ctx* c, const lra_rand* rr, uint64_t s) : ctx(c), r(rr), seed(s) {
    if (r) {
      gdev = is_dev(r->gauss);
      qdev = is_dev(r->ints);
    }
  }
  bool injected_gauss() const { return r && r->gauss; }
  bool injected_ints() const { return r && r->ints; }

  // the position in both streams (a step drawn ahead and not used is
  // rewound, so that later draws see the positions of the step-by-step loop)
  struct Pos {
    int64_t g, q;
    uint64_t counter;
  };
  Pos pos() const { return Pos{g, q, ctx->rng_counter}; }
  void seek(const Pos& p) {
    g = p.g;
    q = p.q;
    ctx->rng_counter = p.counter;
  }

  const double* take_gauss_raw(int64_t n) {
    if (g + n > r->gauss_len)
      fail(LRA_ERAND, "gauss stream exhausted: need %lld values at offset %lld, have %lld", (long long)n,
           (long long)g, (long long)r->gauss_len);
    const double* src = r->gauss + g;
    g += n;
    if (gdev) return src;
    double* d = ctx->arena.alloc_n<double>(n);
    LRA_CUDA(cudaMemcpyAsync(d, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return d;
  }

  template <typename T>
  void gauss(int64_t n, T* out, bool lattice) {
    if (n <= 0) return;
    if (injected_gauss()) {
      sketch_from_stream(ctx, take_gauss_raw(n), n, out, lattice);
    } else {
      sketch_philox(ctx, seed, ctx->rng_counter, n, out);
      ctx->rng_counter += (uint64_t)(n + 1) / 2;
    }
  }

  template <typename T>
  void signs(int64_t n, T* d) {
    if (n <= 0) return;
    if (injected_gauss()) {
      srft_signs(ctx, take_gauss_raw(n), n, d);
    } else {
      sketch_philox(ctx, seed, ctx->rng_counter, n, d);
      ctx->rng_counter += (uint64_t)(n + 1) / 2;
      // sign of a lattice Gaussian: map to +-1 through the stream kernel
      double* tmp = ctx->arena.alloc_n<double>(n);
      sketch_philox(ctx, seed ^ 0x5bd1e995ull, ctx->rng_counter, n, tmp);
      ctx->rng_counter += (uint64_t)(n + 1) / 2;
      srft_signs(ctx, tmp, n, d);
    }
  }

  // n indices in [1, hi] (1 + (v - 1) mod hi), or with perm a permutation of
  // 1..n (the stable ascending rank order of n keys)
  void ints(int64_t n, int64_t hi, int64_t* out, bool perm) {
    if (n <= 0) return;
    if (injected_ints()) {
      if (q + n > r->ints_len)
        fail(LRA_ERAND, "int stream exhausted: need %lld values at offset %lld, have %lld", (long long)n,
             (long long)q, (long long)r->ints_len);
      std::vector<int64_t> h(n);
      if (qdev) {
        LRA_CUDA(cudaMemcpyAsync(h.data(), r->ints + q, n * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                 ctx->stream));
        LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      } else {
        std::memcpy(h.data(), r->ints + q, n * sizeof(int64_t));
      }
      q += n;
      std::vector<int64_t> v(n);
      if (perm) {
        std::vector<int64_t> ord(n);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return h[a] < h[b]; });
        for (int64_t i = 0; i < n; ++i) v[i] = ord[i] + 1;
      } else {
        for (int64_t i = 0; i < n; ++i) v[i] = 1 + (((h[i] - 1) % hi) + hi) % hi;
      }
      LRA_CUDA(cudaMemcpyAsync(out, v.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    } else if (perm) {
      perm_philox(ctx, seed, ctx->rng_counter, n, out);
      ctx->rng_counter += (uint64_t)n;
    } else {
      ints_philox(ctx, seed, ctx->rng_counter, n, hi, out);
      ctx->rng_counter += (uint64_t)n;
    }
  }
};

// ---- options --------------------------------------------------------------------
int64_t samp(const lra_opts& o, int64_t n) {
  switch (o.sketch) {
    case LRA_SKETCH_RANDN:
      return o.sketchfact_randn_samp[0] * n + o.sketchfact_randn_samp[1];
    case LRA_SKETCH_SRFT:
      return o.sketchfact_srft_samp[0] * n + o.sketchfact_srft_samp[1];
    case LRA_SKETCH_SUB:
      return o.sketchfact_sub_samp[0] * n + o.sketchfact_sub_samp[1];
    default:
      return n;  // sprn: order = n (src/sketch.jl:680)
  }
}

void chkopts(const lra_opts* o) {
  if (!o) fail(LRA_EINVAL, "opts is NULL");
  if (!(o->atol >= 0)) fail(LRA_EINVAL, "atol");
  if (!(o->nb > 0)) fail(LRA_EINVAL, "nb");
  if (!(o->pheig_orthtol >= 0)) fail(LRA_EINVAL, "pheig_orthtol");
  if (!(o->rtol >= 0)) fail(LRA_EINVAL, "rtol");
  if (o->sketch < LRA_SKETCH_NONE || o->sketch > LRA_SKETCH_SUB) fail(LRA_EINVAL, "sketch");
  if (o->precision != LRA_PREC_NATIVE && o->precision != LRA_PREC_MIXED) fail(LRA_EINVAL, "precision");
  if (o->sketch_randn_niter < 0) fail(LRA_EINVAL, "sketch_randn_niter");
  if (o->pqrfact_retval & ~(LRA_RET_Q | LRA_RET_R | LRA_RET_T)) fail(LRA_EINVAL, "pqrfact_retval");
}

char chktrans(char t) {
  if (t == 'n' || t == 'N') return 'n';
  if (t == 'c' || t == 'C' || t == 't' || t == 'T') return 'c';
  fail(LRA_EINVAL, "trans");
}

int slices_for(const lra_opts& o, int dtype) {
  // 8-bit slices of A until the truncation is far below rtol
  const double target = std::max(o.rtol, dtype == LRA_F64 ? 1e-15 : 1e-7) * 1e-2;
  int s = 1;
  while (s < 7 && std::ldexp(1.0, -8 * s + 1) > target) ++s;
  return s;
}

// ---- matrix-free operators ---------------------------------------------------------
// a dense sub-matrix taken from an operator is factored as a matrix: the
// operator is set aside while this scope lives
struct DenseScope {
  lra_ctx* ctx;
  const lra_linop* saved;
  explicit DenseScope(lra_ctx* c) : ctx(c), saved(c->linop) { c->linop = nullptr; }
  ~DenseScope() { ctx->linop = saved; }
};

// Y = op(L) X through the caller's product (trans 'n': L, 'c': L'; a
// HermitianLinearOperator is its own adjoint), in stream order
template <typename T>
void linop_apply(lra_ctx* ctx, char trans, int64_t ncols, const T* X, int64_t ldx, T* Y, int64_t ldy) {
  const lra_linop* L = ctx->linop;
  if (ncols <= 0) return;
  const char tr = (L->hermitian || trans == 'n') ? 'n' : 'c';
  const int64_t rows = tr == 'n' ? L->m : L->n;
  if (rows <= 0) return;
  if (L->matmat(L->user, tr, ncols, X, ldx, Y, ldy, (void*)ctx->stream) != 0)
    fail(LRA_ECUDA, "the operator's matmat callback returned an error");
  LRA_CUDA(cudaGetLastError());
}

// C (rows x N, ldc) = X (rows x K, ldx) op(L), op(L) K x N: (op(L)' X')'
template <typename T>
void linop_rmul(lra_ctx* ctx, char trans, int64_t rows, int64_t K, int64_t N, const T* X, int64_t ldx, T* C,
                int64_t ldc) {
  if (rows <= 0 || N <= 0) return;
  const ArenaMark mk = ctx->arena.mark();
  T* Xt = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(K, 1) * rows);
  T* Ct = ctx->arena.alloc_n<T>((size_t)N * rows);
  transpose(ctx, rows, K, X, ldx, Xt, std::max<int64_t>(K, 1));
  linop_apply<T>(ctx, trans == 'n' ? 'c' : 'n', rows, Xt, std::max<int64_t>(K, 1), Ct, N);
  transpose(ctx, N, rows, Ct, N, C, ldc);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

// E (N x k): the unit columns e_idx[i] (idx 1-based, device)
template <typename T>
T* unit_cols(lra_ctx* ctx, int64_t N, const int64_t* idx, int64_t k) {
  const int64_t kk = std::max<int64_t>(k, 1);
  T* I = ctx->arena.alloc_n<T>((size_t)kk * kk);
  T* Et = ctx->arena.alloc_n<T>((size_t)kk * std::max<int64_t>(N, 1));
  T* E = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(N, 1) * kk);
  set_identity(ctx, k, k, I, kk);
  set_zero(ctx, Et, kk * N);
  scatter_cols(ctx, k, k, I, kk, idx, Et, kk);
  transpose(ctx, k, N, Et, kk, E, std::max<int64_t>(N, 1));
  return E;
}

// ---- sketches ----------------------------------------------------------------------
template <typename T>
void orthrows(lra_ctx* ctx, int64_t rows, int64_t cols, T* B) {
  // thin = false: Q of the LQ factorization, rows beyond min(rows, cols) zeroed
  const ArenaMark mk = ctx->arena.mark();
  const int64_t kq = std::min(rows, cols);
  T* Wt = ctx->arena.alloc_n<T>((size_t)cols * rows);
  transpose(ctx, rows, cols, B, rows, Wt, cols);
  int64_t* jp = ctx->arena.alloc_n<int64_t>(rows);
  T* tau = ctx->arena.alloc_n<T>(std::max<int64_t>(kq, 1));
  geqp3_adap<T>(ctx, cols, rows, Wt, cols, jp, tau, kq, 32, -1.0, 0.0, false);
  orgqr(ctx, cols, kq, Wt, cols, tau);
  set_zero(ctx, B, rows * cols);
  transpose(ctx, cols, kq, Wt, cols, B, rows);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

// whether the Gaussian sketch runs on the tensor cores: the mixed path
// resolves op(A) to 2^-48 (Float64) / 2^-24 (Float32) of each column's
// scale, so a Float64 rtol below 1e-13 keeps the native GEMM.
bool use_tc(const lra_opts& o, int dtype) {
  if (o.precision != LRA_PREC_MIXED || o.sketch != LRA_SKETCH_RANDN) return false;
  return dtype == LRA_F32 || o.rtol >= 1e-13;
}

// whether the large Float64 GEMMs of a factorization run on the tensor
// cores (tc_gemm: 2^-45 of the operands' row / column scales)
bool use_tc_gemm(const lra_opts& o, int dtype) {
  return o.precision == LRA_PREC_MIXED && dtype == LRA_F64 && o.rtol >= 1e-13;
}

// right_layout: the Gaussian matrix is drawn as M x order (column-major), the
// layout of a right sketch A S (src/sketch.jl:95-98), and used transposed
template <typename T>
void make_sketch(lra_ctx* ctx, const lra_opts& o, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                 int64_t order, RandSrc& rs, T* B, int dtype, TcSplit* split = nullptr, bool right_layout = false) {
  const ArenaMark mk = ctx->arena.mark();
  const char tA = trans == 'c' ? 't' : 'n';
  switch (o.sketch) {
    case LRA_SKETCH_RANDN: {
      const bool tc = use_tc(o, dtype) && tc_sketch_supported(order, M, N);
      T* S = ctx->arena.alloc_n<T>((size_t)order * M);
      if (right_layout) {
        T* Sr = ctx->arena.alloc_n<T>((size_t)order * M);
        rs.gauss(order * M, Sr, o.precision == LRA_PREC_MIXED);
        transpose(ctx, M, order, Sr, std::max<int64_t>(M, 1), S, std::max<int64_t>(order, 1));
      } else {
        rs.gauss(order * M, S, o.precision == LRA_PREC_MIXED);
      }
      // the products with op(A): a GEMM, or the operator's own product for
      // a matrix-free input (sketch_randn_* with A a LinOp, src/linop.jl)
      const bool lin = ctx->linop != nullptr;
      if (lin) {
        linop_rmul<T>(ctx, trans, order, M, N, S, order, B, order);
      } else if (tc) {
        TcSplit local;
        if (!split) split = &local;
        if (split->ns == 0) tc_split<T>(ctx, trans, M, N, A, lda, dtype == LRA_F64 ? 6 : 3, split);
        tc_sketch<T>(ctx, *split, order, S, B, order);
      } else {
        gemm<T>(ctx, 'n', tA, order, N, M, T(1), S, order, A, lda, T(0), B, order);
      }
      if (o.sketch_randn_niter > 0) {
        const bool herm = (M == N) && is_symmetric(ctx, M, A, lda);
        T* Bq = ctx->arena.alloc_n<T>((size_t)order * M);
        for (int64_t it = 0; it < o.sketch_randn_niter; ++it) {
          orthrows(ctx, order, N, B);
          // Bq = Bp op(A)^T (order x M)
          if (lin)
            linop_rmul<T>(ctx, trans == 'n' ? 'c' : 'n', order, N, M, B, order, Bq, order);
          else
            gemm<T>(ctx, 'n', trans == 'c' ? 'n' : 't', order, M, N, T(1), B, order, A, lda, T(0), Bq, order);
          if (herm) {
            copy_matrix(ctx, order, M, Bq, order, B, order);
          } else {
            orthrows(ctx, order, M, Bq);
            if (lin)
              linop_rmul<T>(ctx, trans, order, M, N, Bq, order, B, order);
            else
              gemm<T>(ctx, 'n', tA, order, N, M, T(1), Bq, order, A, lda, T(0), B, order);
          }
        }
      }
      break;
    }
    case LRA_SKETCH_SRFT: {
      T* d = ctx->arena.alloc_n<T>(M);
      rs.signs(M, d);
      int64_t* idx = ctx->arena.alloc_n<int64_t>(order);
      rs.ints(order, M, idx, false);
      if (!srft_sketch_fft<T>(ctx, trans, M, N, A, lda, d, idx, order, B, order))
        srft_sketch<T>(ctx, trans, M, N, A, lda, d, idx, order, B, order);
      break;
    }
    case LRA_SKETCH_SUB: {
      int64_t* rows = ctx->arena.alloc_n<int64_t>(order);
      rs.ints(order, M, rows, false);
      sub_sketch<T>(ctx, trans, M, N, A, lda, rows, order, B, order);
      break;
    }
    case LRA_SKETCH_SPRN: {
      int64_t* perm = ctx->arena.alloc_n<int64_t>(M);
      rs.ints(M, M, perm, true);
      T* g = ctx->arena.alloc_n<T>(M);
      rs.gauss(M, g, false);
      sprn_sketch<T>(ctx, trans, M, N, A, lda, perm, g, order, B, order);
      break;
    }
    default:
      fail(LRA_EINVAL, "sketch");
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

// ---- pivoted QR + post-processing --------------------------------------------------
template <typename T>
struct Fact {
  T* B = nullptr;  // order x N, R in the upper triangle
  int64_t ld = 0, order = 0, N = 0;
  int64_t* jpvt = nullptr;  // N, 1-based
  T* tau = nullptr;
  int64_t k = 0;
  int nsteps = 0;
  T* T_ = nullptr;  // k x (N - k), ld = k
  int64_t swaps = 0;  // maxdet swaps: when > 0, R11 no longer matches sk
  bool embed = true;  // B = S op(A) with S a subspace embedding (randn/srft)
  // after maxdet swaps with an R factor requested: the Householder QR of the
  // updated R1 (k x k, ld k; R above, reflectors below) and its tau
  T* r1 = nullptr;
  T* r1tau = nullptr;
  // R11^-1 diag(R11) (k x k, ld k) when the solve for T computed it, for the
  // post-processing's division by R11 (valid while swaps == 0)
  T* r11inv = nullptr;
};

template <typename T>
void maxdet_dev(lra_ctx* ctx, const lra_opts& o, Fact<T>& F);

// The rank a step whose rank reached its threshold points to: where the
// line through log |R_ii| over the middle half of its pivots crosses the
// rank test's threshold (rtol |R_11|, or atol).  The last pivots of a short
// sketch fall faster than the matrix's spectrum, so they are left out.  A step whose factorization
// stopped below kmax revealed the rank itself.  -1 when the diagonal gives
// no estimate; a large value when it does not decay.  Used only to decide
// how many steps to factor together.
template <typename T>
int64_t predict_rank(lra_ctx* ctx, const Fact<T>& F, int64_t kmax, const lra_opts& o) {
  const int64_t k = F.k;
  if (k <= 1) return -1;
  if (k < kmax) return k;
  std::vector<T> d((size_t)k);
  LRA_CUDA(cudaMemcpy2DAsync(d.data(), sizeof(T), F.B, (size_t)(F.ld + 1) * sizeof(T), sizeof(T), (size_t)k,
                             cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  const double d0 = std::fabs((double)d[0]);
  const double ptol = std::max(o.atol, o.rtol * d0);
  const int64_t i1 = k / 4, i2 = std::max<int64_t>(i1 + 1, (3 * k) / 4);
  const double a = std::fabs((double)d[(size_t)i1]), b = std::fabs((double)d[(size_t)i2]);
  if (!(ptol > 0) || !(a > 0) || !(b > 0) || !std::isfinite(a) || !std::isfinite(b)) return -1;
  if (b <= ptol) return k;
  const double slope = (std::log(b) - std::log(a)) / (double)(i2 - i1);
  if (!(slope < -1e-12)) return std::numeric_limits<int64_t>::max() / 4;
  const double r = (double)i2 + (std::log(ptol) - std::log(b)) / slope;
  return r > 1e15 ? std::numeric_limits<int64_t>::max() / 4 : std::max<int64_t>(k, (int64_t)r);
}

// Steps step, step + 1, ... of sketchfact_dev's loop (thresholds nt, 2 nt,
// ...) up to the first whose threshold exceeds twice the predicted rank (a
// step that reveals the rank stops the ones after it, so a wide margin
// costs their sketches only),
// as many as one shared-memory launch holds, sketched in order and factored
// together.  Returns the number of steps taken when one of them revealed
// its rank (F is then that step's factorization and the random streams stand
// where that step left them), minus that number when none did (the streams
// stand after the last), and 0 when fewer than two steps fit one launch
// (nothing done).
template <typename T>
int sketchfact_steps(lra_ctx* ctx, const lra_opts& o, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                     RandSrc& rs, int dtype, TcSplit* split, int step, int64_t nt, int64_t rank_hint,
                     const ArenaMark& base, Fact<T>& F) {
  const int64_t limit = rank_hint > (int64_t)1 << 40 ? (int64_t)1 << 40 : 2 * rank_hint + 64;
  std::vector<int64_t> orders, nts, ms;
  int64_t t = nt;
  for (int i = 0; i < ctx->tuning.qr_steps && i < 8; ++i) {
    const int64_t order = samp(o, t);
    if (order <= 0) break;
    orders.push_back(order);
    nts.push_back(t);
    ms.push_back(order);
    // the step that should reveal the rank (its threshold above the
    // prediction), or the one whose sketch covers every column, is the last
    if (t > limit || std::min(order, N) >= N) break;
    if (t > ((int64_t)1 << 40)) break;
    t *= 2;
  }
  int cnt = geqp3_steps_fit<T>(ctx, (int)orders.size(), ms.data(), N);
  if (cnt < 2) return 0;
  std::vector<QrStep<T>> st;
  std::vector<RandSrc::Pos> after;
  {
    Stage sg(ctx, 0);
    for (int i = 0; i < cnt; ++i) {
      const int64_t order = orders[(size_t)i];
      const int64_t l = std::min(order, N);
      const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
      QrStep<T> q;
      q.m = order;
      q.n = N;
      q.lda = std::max<int64_t>(order, 1);
      q.A = ctx->arena.alloc_n<T>((size_t)q.lda * N);
      q.jpvt = ctx->arena.alloc_n<int64_t>(N);
      q.tau = ctx->arena.alloc_n<T>(std::max<int64_t>(l, 1));
      q.kmax = kmax;
      q.nt = nts[(size_t)i];
      const RandSrc::Pos before = rs.pos();
      try {
        make_sketch<T>(ctx, o, trans, M, N, A, lda, order, rs, q.A, dtype, split);
      } catch (const Error& e) {
        // an injected stream too short for a step drawn ahead: the launch
        // ends before it (the step-by-step loop meets the same error only if
        // it gets there)
        if (e.status != LRA_ERAND || i == 0) throw;
        rs.seek(before);
        cnt = i;
        break;
      }
      st.push_back(q);
      after.push_back(rs.pos());
    }
  }
  if (cnt < 2) {
    // not enough left to share a launch: back to one step at a time
    rs.seek(after.empty() ? rs.pos() : after[0]);
    if (!after.empty()) {
      // the one sketch drawn is the step's own; factor it here
      const QrStep<T>& q = st[0];
      int64_t k = 0;
      {
        Stage sq(ctx, 1);
        k = geqp3_adap<T>(ctx, q.m, q.n, q.A, q.lda, q.jpvt, q.tau, q.kmax, o.nb, o.atol, o.rtol, true);
      }
      F.order = q.m;
      F.ld = q.lda;
      F.B = q.A;
      F.jpvt = q.jpvt;
      F.tau = q.tau;
      F.k = k;
      F.nsteps = step + 1;
      if (k < q.nt) return 1;
      ctx->arena.release(base);
      return -1;
    }
    return 0;
  }
  std::vector<int64_t> ks((size_t)cnt);
  int c;
  {
    Stage sq(ctx, 1);
    c = geqp3_adap_steps<T>(ctx, cnt, st.data(), o.nb, o.atol, o.rtol, ks.data());
  }
  if (c < 0) {
    ctx->arena.release(base);
    return -cnt;
  }
  const QrStep<T>& q = st[(size_t)c];
  F.order = q.m;
  F.ld = q.lda;
  F.B = q.A;
  F.jpvt = q.jpvt;
  F.tau = q.tau;
  F.k = ks[(size_t)c];
  F.nsteps = step + c + 1;
  rs.seek(after[(size_t)c]);
  return c + 1;
}

template <typename T>
Fact<T> sketchfact_dev(lra_ctx* ctx, const lra_opts& o, char trans, int64_t M, int64_t N, const T* A,
                       int64_t lda, RandSrc& rs, int dtype) {
  const bool adaptive = o.sketchfact_adap || o.rank < 0;
  int64_t nt = adaptive ? o.nb : o.rank;
  Fact<T> F;
  F.N = N;
  // the byte slices of op(A) for the tensor-core sketch outlive the steps
  TcSplit split;
  if (use_tc(o, dtype) && tc_sketch_supported(1, M, N) && M > 0 && N > 0) {
    Stage st(ctx, 0);
    tc_split<T>(ctx, trans, M, N, A, lda, dtype == LRA_F64 ? 6 : 3, &split);
  }
  const ArenaMark base = ctx->arena.mark();
  // Steps factored together: once a step's rank has reached its threshold,
  // the decay of its R diagonal predicts the rank, and the steps up to the
  // one that should reveal it are sketched and factored by one launch of the
  // shared-memory pivoted QR (each on CTAs of its own; a step that reveals
  // its rank stops the later ones).  The first step whose rank comes out
  // below its threshold is the result, the same as one step at a time; the
  // prediction only decides how many steps share a launch.
  const bool ahead = adaptive && !ctx->linop && ctx->tuning.qr_steps > 1 && N > 0 && M > 0;
  int64_t rank_hint = -1;
  for (int step = 0;; ++step) {
    if (step > 62) fail(LRA_EINVAL, "adaptive sketch did not terminate");
    if (ahead && rank_hint >= 0) {
      const int done = sketchfact_steps<T>(ctx, o, trans, M, N, A, lda, rs, dtype, split.ns ? &split : nullptr,
                                           step, nt, rank_hint, base, F);
      if (done > 0) break;
      if (done < 0) {
        // every step of the launch reached its threshold: the rank is at
        // least the last one's, and the next launch takes the steps after
        step += -done - 1;
        for (int i = 0; i < -done; ++i) nt *= 2;
        rank_hint = nt;
        continue;
      }
    }
    const int64_t order = samp(o, nt);
    if (order < 0) fail(LRA_EINVAL, "sketch order %lld", (long long)order);
    const int64_t l = std::min(order, N);
    const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
    F.order = order;
    F.ld = std::max<int64_t>(order, 1);
    F.B = ctx->arena.alloc_n<T>((size_t)F.ld * std::max<int64_t>(N, 1));
    F.jpvt = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(N, 1));
    F.tau = ctx->arena.alloc_n<T>(std::max<int64_t>(l, 1));
    {
      Stage st(ctx, 0);
      make_sketch<T>(ctx, o, trans, M, N, A, lda, order, rs, F.B, dtype, split.ns ? &split : nullptr);
    }
    {
      Stage st(ctx, 1);
      F.k = geqp3_adap<T>(ctx, order, N, F.B, F.ld, F.jpvt, F.tau, kmax, o.nb, o.atol, o.rtol, true);
    }
    F.nsteps = step + 1;
    if (!adaptive || F.k < nt) break;
    if (ahead) rank_hint = predict_rank<T>(ctx, F, kmax, o);
    nt *= 2;
    ctx->arena.release(base);
  }
  return F;
}

// sketchfact(:right, trans, A) (src/sketch.jl:223-240 and twins): the same
// adaptive loop on the right sketch op(A) S (M x order), made as the
// transpose of the left sketch of op(A)' exactly as lra_sketch makes it;
// the pivots run over the sketch's order columns
template <typename T>
Fact<T> sketchfact_right_dev(lra_ctx* ctx, const lra_opts& o, char trans, int64_t M, int64_t N, const T* A,
                             int64_t lda, RandSrc& rs, int dtype) {
  const bool adaptive = o.sketchfact_adap || o.rank < 0;
  int64_t nt = adaptive ? o.nb : o.rank;
  const char tt = trans == 'n' ? 'c' : 'n';
  Fact<T> F;
  F.order = M;
  F.ld = std::max<int64_t>(M, 1);
  const ArenaMark base = ctx->arena.mark();
  for (int step = 0;; ++step) {
    if (step > 62) fail(LRA_EINVAL, "adaptive sketch did not terminate");
    const int64_t order = samp(o, nt);
    if (order < 0) fail(LRA_EINVAL, "sketch order %lld", (long long)order);
    const int64_t l = std::min(order, M);
    const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
    F.N = order;
    F.B = ctx->arena.alloc_n<T>((size_t)F.ld * std::max<int64_t>(order, 1));
    F.jpvt = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(order, 1));
    F.tau = ctx->arena.alloc_n<T>(std::max<int64_t>(l, 1));
    {
      Stage st(ctx, 0);
      const ArenaMark mk = ctx->arena.mark();
      T* Bt = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(order, 1) * std::max<int64_t>(M, 1));
      make_sketch<T>(ctx, o, tt, N, M, A, lda, order, rs, Bt, dtype, nullptr, true);
      if (order > 0 && M > 0) transpose(ctx, order, M, Bt, order, F.B, F.ld);
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      ctx->arena.release(mk);
    }
    {
      Stage st(ctx, 1);
      F.k = geqp3_adap<T>(ctx, M, order, F.B, F.ld, F.jpvt, F.tau, kmax, o.nb, o.atol, o.rtol, true);
    }
    F.nsteps = step + 1;
    if (!adaptive || F.k < nt) break;
    nt *= 2;
    ctx->arena.release(base);
  }
  return F;
}

template <typename T>
void postproc_t(lra_ctx* ctx, const lra_opts& o, Fact<T>& F, bool want_t) {
  const bool maxdet = F.k > 0 && F.k < F.N && o.maxdet_tol >= 0;
  if (!(want_t || maxdet)) return;
  Stage st(ctx, 2);
  const int64_t k = F.k, nr = F.N - k;
  F.T_ = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k, 1) * std::max<int64_t>(nr, 1));
  if (k > 0 && nr > 0) {
    copy_matrix(ctx, k, nr, F.B + k * F.ld, F.ld, F.T_, k);
    if (k <= kBsMax) {
      trsm_bs(ctx, k, nr, F.B, F.ld, F.T_, k);
    } else {
      if (trsm_by_inverse<T>(ctx, k, nr)) {
        F.r11inv = ctx->arena.alloc_n<T>((size_t)k * k);
        tri_inv_upper<T>(ctx, k, F.B, F.ld, F.r11inv, k);
      }
      trsm_upper(ctx, k, nr, F.B, F.ld, F.T_, k, F.r11inv);
    }
  }
  if (maxdet) maxdet_dev<T>(ctx, o, F);
}

// pqrfact_backend! on a dense device matrix (M x N, ld), in place
template <typename T>
Fact<T> pqr_backend_dev(lra_ctx* ctx, const lra_opts& o, T* B, int64_t M, int64_t N, int64_t ld) {
  Fact<T> F;
  F.B = B;
  F.ld = ld;
  F.order = M;
  F.N = N;
  const int64_t l = std::min(M, N);
  const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
  F.jpvt = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(N, 1));
  F.tau = ctx->arena.alloc_n<T>(std::max<int64_t>(l, 1));
  Stage st(ctx, 1);
  F.k = geqp3_adap<T>(ctx, M, N, B, ld, F.jpvt, F.tau, kmax, o.nb, o.atol, o.rtol, true);
  F.nsteps = 0;
  return F;
}

// op(A) as a dense device copy (M x N, ld = M)
template <typename T>
T* dense_op(lra_ctx* ctx, char trans, int64_t m, int64_t n, const DMat<T>& A) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  T* B = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(N, 1));
  if (trans == 'n')
    copy_matrix(ctx, m, n, A.p, A.ld, B, M);
  else
    transpose(ctx, m, n, A.p, A.ld, B, M);
  return B;
}

// the sketch or the full matrix, factored, with T when requested
template <typename T>
Fact<T> id_core(lra_ctx* ctx, const lra_opts& o, char trans, int64_t m, int64_t n, const DMat<T>& A,
                RandSrc& rs, int dtype, bool want_t) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  Fact<T> F;
  if (o.sketch == LRA_SKETCH_NONE) {
    T* B = dense_op(ctx, trans, m, n, A);
    F = pqr_backend_dev<T>(ctx, o, B, M, N, M);
  } else {
    F = sketchfact_dev<T>(ctx, o, trans, M, N, A.p, A.ld, rs, dtype);
    F.embed = o.sketch == LRA_SKETCH_RANDN || o.sketch == LRA_SKETCH_SRFT;
  }
  postproc_t<T>(ctx, o, F, want_t);
  return F;
}

// A[:, sk] = Q R_A through the sketch-preconditioned Cholesky QR; Ask (M x k,
// ld M) becomes Q.  False when R11 does not precondition A[:, sk] (maxdet
// swaps) or a Cholesky factorization broke down; Ask is then left damaged
// and the caller regathers it.
template <typename T>
bool skeleton_qr(lra_ctx* ctx, const Fact<T>& F, int64_t M, T* Ask, T* RA, int dtype) {
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1);
  if (F.swaps > 0) return false;
  const int passes = (dtype == LRA_F64 && F.embed) ? 1 : 2;
  T* Rc = ctx->arena.alloc_n<T>((size_t)kk * kk);
  if (!cholqr_pre<T>(ctx, M, k, Ask, std::max<int64_t>(M, 1), F.B, F.ld, passes, Rc)) return false;
  // R_A = Rc R11
  T* R11 = ctx->arena.alloc_n<T>((size_t)kk * kk);
  copy_matrix(ctx, k, k, F.B, F.ld, R11, kk);
  zero_lower(ctx, k, k, R11, kk);
  gemm<T>(ctx, 'n', 'n', k, k, k, T(1), Rc, kk, R11, kk, T(0), RA, kk);
  return true;
}

// skeleton_qr and R_v = chol(I + T T^T) (chol_v); with one Cholesky QR
// pass the two factorizations share a launch
template <typename T>
bool skeleton_qr_v(lra_ctx* ctx, const Fact<T>& F, int64_t M, T* Ask, T* RA, int64_t nr, T* Rv, int dtype) {
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1);
  if (F.swaps > 0) return false;
  if (!(dtype == LRA_F64 && F.embed)) return skeleton_qr<T>(ctx, F, M, Ask, RA, dtype) && chol_v<T>(ctx, k, nr, F.T_, Rv);
  T* Rc = ctx->arena.alloc_n<T>((size_t)kk * kk);
  if (!cholqr1_and_chol_v<T>(ctx, M, k, Ask, std::max<int64_t>(M, 1), F.B, F.ld, Rc, nr, F.T_, Rv, F.r11inv))
    return false;
  // R_A = Rc R11
  T* R11 = ctx->arena.alloc_n<T>((size_t)kk * kk);
  copy_matrix(ctx, k, k, F.B, F.ld, R11, kk);
  zero_lower(ctx, k, k, R11, kk);
  gemm<T>(ctx, 'n', 'n', k, k, k, T(1), Rc, kk, R11, kk, T(0), RA, kk);
  return true;
}

// getcols(trans, A, idx): M x k device matrix
template <typename T>
T* getcols(lra_ctx* ctx, char trans, int64_t m, int64_t n, const DMat<T>& A, const int64_t* idx, int64_t k) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  T* C = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(k, 1));
  if (ctx->linop) {
    // A[:, cols] of an operator is op(A) times unit columns (src/linop.jl:56-63)
    if (k > 0 && M > 0) linop_apply<T>(ctx, trans, k, unit_cols<T>(ctx, N, idx, k), std::max<int64_t>(N, 1), C, M);
    return C;
  }
  if (trans == 'n') {
    gather_cols(ctx, m, k, A.p, A.ld, idx, C, M);
  } else {
    T* Rw = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k, 1) * std::max<int64_t>(n, 1));
    gather_rows(ctx, k, n, A.p, A.ld, idx, Rw, k);
    transpose(ctx, k, n, Rw, k, C, M);
  }
  return C;
}

}  // namespace

// One step of maxdet_swapcols! (src/pqr.jl:445-476) on the device: find
// max |T| (ties: last index, findmaxabs, src/util.jl:13-23); when it is
// above `bound` and `update` is set, swap p and apply maxdet_update!
// (src/pqr.jl:479-501, T part).  Returns whether max |T| > bound.
template <typename T>
bool maxdet_step(lra_ctx* ctx, int64_t k, int64_t nr, T* Tm, int64_t* jpvt, double bound, bool update, T* R1,
                 int64_t ldr);

namespace {

// strong rank-revealing swaps (maxdet_swapcols!, src/pqr.jl:445-476): T and
// p always; with an R factor requested, R1 = triu(R[:, 1:k]) follows each
// swap (maxdet_update!, src/pqr.jl:494-499) and, after the last one, is
// re-factored by an unpivoted Householder QR (qrfact!(R1), :467), whose
// reflectors then rotate Q (gemqrt!, :468) and whose R replaces R11
// (:469-474).  Without an R factor R1 stays triangular, its QR is the
// identity and Q is left as it is.
template <typename T>
void maxdet_dev(lra_ctx* ctx, const lra_opts& o, Fact<T>& F) {
  const int64_t k = F.k, nr = F.N - k, kk = std::max<int64_t>(k, 1);
  const bool retr = o.pqrfact_retval & LRA_RET_R;
  T* R1 = nullptr;
  if (retr && k > 0) {
    R1 = ctx->arena.alloc_n<T>((size_t)kk * kk);
    copy_matrix(ctx, k, k, F.B, F.ld, R1, kk);
    zero_lower(ctx, k, k, R1, kk);
  }
  const int64_t cap = 64 * (k + nr) + 1000;  // the determinant grows every swap
  int64_t niter = 0;
  while (niter < cap) {
    const bool upd = niter != o.maxdet_niter;
    if (!maxdet_step<T>(ctx, k, nr, F.T_, F.jpvt, 1.0 + o.maxdet_tol, upd, R1, kk)) break;
    if (!upd) break;
    ++niter;
  }
  F.swaps = niter;
  if (niter > 0 && R1) {
    T* tau1 = ctx->arena.alloc_n<T>(kk);
    int64_t* jp = ctx->arena.alloc_n<int64_t>(kk);
    geqp3_adap<T>(ctx, k, k, R1, kk, jp, tau1, k, 32, -1.0, 0.0, false);
    F.r1 = R1;
    F.r1tau = tau1;
  }
}

// R11 of the returned R: the re-factored R1 after maxdet swaps, else the
// pivoted QR's own (k x k upper triangle into R11, ld k)
template <typename T>
void result_r11(lra_ctx* ctx, const Fact<T>& F, T* R11) {
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1);
  if (F.r1)
    copy_matrix(ctx, k, k, F.r1, kk, R11, kk);
  else
    copy_matrix(ctx, k, k, F.B, F.ld, R11, kk);
  zero_lower(ctx, k, k, R11, kk);
}

// Q (M x k, ld ldq) <- Q Qf, Qf the reflectors of the re-factored R1
// (LAPACK.gemqrt!('R', 'N', ...), src/pqr.jl:468), as (Qf^T Q^T)^T
template <typename T>
void maxdet_rotate_q(lra_ctx* ctx, const Fact<T>& F, int64_t M, T* Q, int64_t ldq) {
  const int64_t k = F.k;
  if (!F.r1 || k <= 0 || M <= 0) return;
  T* Qt = ctx->arena.alloc_n<T>((size_t)k * M);
  transpose(ctx, M, k, Q, ldq, Qt, k);
  apply_q(ctx, 't', k, k, F.r1, k, F.r1tau, Qt, k, M);
  transpose(ctx, k, M, Qt, k, Q, ldq);
}

}  // namespace

}  // namespace lra

using namespace lra;

// ======================================================================================
// C ABI
// ======================================================================================

namespace {

// the context's error word, after the stream has drained: a kernel whose
// bounded wait gave up during this call fails the call
void check_dev_err(lra_ctx* ctx) {
  if (!ctx->dev_err_armed) return;
  ctx->dev_err_armed = false;
  int h = 0;
  LRA_CUDA(cudaMemcpy(&h, ctx->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (h != 0) {
    LRA_CUDA(cudaMemset(ctx->dev_err, 0, sizeof(int)));
    fail(LRA_ETIMEDOUT, "tc_gemm: a bounded wait timed out");
  }
}

template <class Fn>
int guarded(lra_ctx* ctx, Fn&& fn) {
  if (!ctx) return LRA_EINVAL;
  try {
    LRA_CUDA(cudaSetDevice(ctx->device));
    ctx->arena.reset(ctx->stream);
    for (double& s : ctx->stage_ms) s = 0;
    ctx->gemm_tc = false;
    ctx->mixed_rtol = 0;
    fn();
    ctx->gemm_tc = false;
    ctx->mixed_rtol = 0;
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    check_dev_err(ctx);
    ctx->last_error.clear();
    return LRA_OK;
  } catch (const lra::Error& e) {
    ctx->gemm_tc = false;
    ctx->mixed_rtol = 0;
    ctx->last_error = e.msg;
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    if (ctx->dev_err) {
      cudaMemset(ctx->dev_err, 0, sizeof(int));
      ctx->dev_err_armed = false;
      cudaGetLastError();
    }
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->last_error = "host allocation failed";
    return LRA_ENOMEM;
  } catch (...) {
    ctx->last_error = "unexpected exception";
    return LRA_ECUDA;
  }
}

template <class Fn>
void dispatch(int dtype, Fn&& fn) {
  if (dtype == LRA_F64)
    fn(double(0));
  else if (dtype == LRA_F32)
    fn(float(0));
  else
    fail(LRA_EINVAL, "dtype");
}

template <typename T>
void check_input(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, const DMat<T>& A) {
  if (ctx->linop) return;  // the operator's entries are not available
  if (o.check_finite && !all_finite(ctx, m, n, A.p, A.ld)) fail(LRA_ENONFINITE, "input has NaN or Inf entries");
}

void check_dims(int64_t m, int64_t n) {
  if (m < 0 || n < 0) fail(LRA_EDIM, "negative dimension");
}

template <typename T>
lra_id* pack_id(lra_ctx* ctx, const Fact<T>& F, int dtype) {
  lra_id* r = static_cast<lra_id*>(hmalloc(sizeof(lra_id)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->nsteps = F.nsteps;
  r->k = F.k;
  r->n = F.N;
  r->sk = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(F.k, 1)));
  r->rd = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(F.N - F.k, 1)));
  r->T = hmalloc(sizeof(T) * std::max<int64_t>(F.k * (F.N - F.k), 1));
  to_host(ctx, r->sk, F.jpvt, F.k);
  to_host(ctx, r->rd, F.jpvt + F.k, F.N - F.k);
  if (F.k > 0 && F.N > F.k) to_host(ctx, r->T, F.T_, (size_t)F.k * (F.N - F.k));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}

}  // namespace

namespace lra {

// ---- lra_idfact_batched, grouped ----------------------------------------------------
// Float64 matrices on the mixed path (tensor-core Gaussian sketch, library
// generator restarted per matrix as for a call on a fresh context): every
// round sketches the unfinished matrices, factors all their sketches in one
// grouped launch (geqp3_df_batch), reads the ranks back once and doubles the
// sketch of those whose rank is not yet revealed (sketchfact_dev's loop);
// the solves T = R11^{-1} R12 run as one grouped launch.  Each result is
// what lra_idfact returns for the matrix on a fresh context.
bool grouped_batch_ok(lra_ctx* ctx, int64_t count, const lra_matdesc* mats, const lra_opts& o, const lra_rand* rand) {
  if (rand || count <= 0) return false;
  if (!use_tc(o, LRA_F64) || o.sketch != LRA_SKETCH_RANDN || o.sketch_randn_niter != 0 || o.maxdet_tol >= 0)
    return false;
  if (!(o.sketchfact_adap || o.rank < 0)) return false;
  for (int64_t i = 0; i < count; ++i) {
    const lra_matdesc& d = mats[i];
    if (d.m < 1 || d.n < 1 || !d.A || d.lda < d.m) return false;
    // the largest sketch the doubling can reach: order(nt) with nt up to 2 n
    int64_t nt = o.nb, order = samp(o, nt);
    while (nt <= 2 * d.n) {
      order = samp(o, nt);
      nt *= 2;
    }
    if (!tc_sketch_supported(order, d.m, d.n) || !geqp3_df_batch_fits(ctx, order, d.n)) return false;
  }
  return true;
}

// The per-matrix launches of a batch (staging, byte slices, sketches) are
// small; they are spread over the context's side streams so that several run
// at once.  fan_out makes the side streams wait for the work issued so far on
// the main stream, fan_in makes the main stream wait for the side streams.
void fan_out(lra_ctx* ctx) {
  for (int i = 0; i < lra_ctx::kAux; ++i)
    if (!ctx->aux[i]) LRA_CUDA(cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking));
  for (cudaEvent_t& e : ctx->aux_ev)
    if (!e) LRA_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  LRA_CUDA(cudaEventRecord(ctx->aux_ev[lra_ctx::kAux], ctx->stream));
  for (int i = 0; i < lra_ctx::kAux; ++i) LRA_CUDA(cudaStreamWaitEvent(ctx->aux[i], ctx->aux_ev[lra_ctx::kAux], 0));
}

void fan_in(lra_ctx* ctx) {
  for (int i = 0; i < lra_ctx::kAux; ++i) {
    LRA_CUDA(cudaEventRecord(ctx->aux_ev[i], ctx->aux[i]));
    LRA_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->aux_ev[i], 0));
  }
}

// runs fn with ctx->stream switched to side stream i (mod the count)
template <typename Fn>
void on_side(lra_ctx* ctx, int64_t i, Fn&& fn) {
  cudaStream_t main = ctx->stream;
  ctx->stream = ctx->aux[i % lra_ctx::kAux];
  try {
    fn();
  } catch (...) {
    ctx->stream = main;
    throw;
  }
  ctx->stream = main;
}

void idfact_batched_grouped(lra_ctx* ctx, int64_t count, const lra_matdesc* mats, const lra_opts& oin,
                            lra_id** outs) {
  lra_opts o = oin;
  o.pqrfact_retval = LRA_RET_T;
  ctx->gemm_tc = use_tc_gemm(o, LRA_F64);
  ctx->mixed_rtol = ctx->gemm_tc ? o.rtol : 0.0;
  const bool adaptive = o.sketchfact_adap || o.rank < 0;
  size_t free_b = 0, total_b = 0;
  LRA_CUDA(cudaMemGetInfo(&free_b, &total_b));
  const double budget = 0.3 * (double)free_b;
  // LRA_TRACE: host-side phase times (each phase waits for the device)
  const bool tr = trace_on();
  double tph[6] = {0, 0, 0, 0, 0, 0};
  auto tnow = [] { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double tlast = tnow();
  auto tmark = [&](int q) {
    if (!tr) return;
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    const double t = tnow();
    tph[q] += t - tlast;
    tlast = t;
  };
  int64_t c0 = 0;
  while (c0 < count) {
    // a chunk whose working set stays inside the budget
    int64_t c1 = c0;
    double bytes = 0;
    while (c1 < count) {
      const double mn = (double)mats[c1].m * (double)mats[c1].n;
      const double est = 40.0 * mn + 64.0 * 512.0 * ((double)mats[c1].m + (double)mats[c1].n);
      if (c1 > c0 && (bytes + est > budget || c1 - c0 >= 1024)) break;
      bytes += est;
      ++c1;
    }
    const int64_t cn = c1 - c0;
    const ArenaMark mk = ctx->arena.mark();
    std::vector<DMat<double>> dA((size_t)cn);
    std::vector<TcSplit> split((size_t)cn);
    int* flags = ctx->arena.alloc_n<int>((size_t)cn);
    LRA_CUDA(cudaMemsetAsync(flags, 0, (size_t)cn * sizeof(int), ctx->stream));
    fan_out(ctx);
    for (int64_t i = 0; i < cn; ++i) {
      const lra_matdesc& d = mats[c0 + i];
      on_side(ctx, i, [&] {
        dA[(size_t)i] = stage_in<double>(ctx, d.A, d.m, d.n, d.lda);
        if (o.check_finite) all_finite_async(ctx, d.m, d.n, dA[(size_t)i].p, dA[(size_t)i].ld, flags + i);
        tc_split<double>(ctx, 'n', d.m, d.n, dA[(size_t)i].p, dA[(size_t)i].ld, 6, &split[(size_t)i]);
      });
    }
    fan_in(ctx);
    tmark(0);
    {
      std::vector<int> hf((size_t)cn);
      LRA_CUDA(cudaMemcpyAsync(hf.data(), flags, (size_t)cn * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int64_t i = 0; i < cn; ++i)
        if (hf[(size_t)i]) fail(LRA_ENONFINITE, "matrix %lld of the batch has NaN or Inf entries", (long long)(c0 + i));
    }
    struct St {
      int64_t nt, order, k = 0;
      uint64_t ctr = 0;
      int nsteps = 0;
      bool done = false;
      double* B = nullptr;
      int64_t* jpvt = nullptr;
      double* tau = nullptr;
    };
    std::vector<St> st((size_t)cn);
    for (auto& s : st) s.nt = adaptive ? o.nb : o.rank;
    int64_t* kdev = ctx->arena.alloc_n<int64_t>((size_t)cn);
    int* errs = ctx->arena.alloc_n<int>((size_t)cn);
    for (int round = 0;; ++round) {
      if (round > 62) fail(LRA_EINVAL, "adaptive sketch did not terminate");
      std::vector<int64_t> act;
      for (int64_t i = 0; i < cn; ++i)
        if (!st[(size_t)i].done) act.push_back(i);
      if (act.empty()) break;
      LRA_CUDA(cudaMemsetAsync(errs, 0, (size_t)cn * sizeof(int), ctx->stream));
      std::vector<DfBatchItem> items;
      items.reserve(act.size());
      fan_out(ctx);
      for (const int64_t i : act) {
        St& s = st[(size_t)i];
        const lra_matdesc& d = mats[c0 + i];
        s.order = samp(o, s.nt);
        if (s.order < 1) fail(LRA_EINVAL, "sketch order %lld", (long long)s.order);
        const int64_t l = std::min(s.order, d.n);
        const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
        s.B = ctx->arena.alloc_n<double>((size_t)s.order * d.n);
        s.jpvt = ctx->arena.alloc_n<int64_t>((size_t)d.n);
        s.tau = ctx->arena.alloc_n<double>((size_t)std::max<int64_t>(l, 1));
        // S stays allocated until the chunk ends: the sketches run on several streams
        double* S = ctx->arena.alloc_n<double>((size_t)s.order * d.m);
        ctx->rng_counter = s.ctr;
        on_side(ctx, i, [&] {
          RandSrc rs(ctx, nullptr, o.seed);
          rs.gauss(s.order * d.m, S, true);
          tc_sketch<double>(ctx, split[(size_t)i], s.order, S, s.B, s.order, errs + i);
        });
        s.ctr = ctx->rng_counter;
        items.push_back(DfBatchItem{s.order, d.n, s.order, kmax, s.B, s.jpvt, s.tau});
      }
      fan_in(ctx);
      std::vector<int64_t> map(act.begin(), act.end());
      tmark(1);
      // the batch writes k of item t to kdev[t]
      geqp3_df_batch(ctx, (int64_t)items.size(), items.data(), o.nb, o.atol, o.rtol, kdev);
      tmark(2);
      std::vector<int64_t> hk(items.size());
      std::vector<int> he((size_t)cn);
      LRA_CUDA(cudaMemcpyAsync(hk.data(), kdev, hk.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaMemcpyAsync(he.data(), errs, (size_t)cn * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      for (size_t t = 0; t < map.size(); ++t) {
        St& s = st[(size_t)map[t]];
        if (he[(size_t)map[t]]) fail(LRA_ETIMEDOUT, "tc_sketch: a bounded wait timed out");
        s.k = hk[t];
        s.nsteps = round + 1;
        if (!adaptive || s.k < s.nt)
          s.done = true;
        else
          s.nt *= 2;
      }
    }
    // T = R11^{-1} R12 (the single path's postproc_t), then the results
    std::vector<double*> Tm((size_t)cn, nullptr);
    std::vector<BsItem> bs;
    for (int64_t i = 0; i < cn; ++i) {
      St& s = st[(size_t)i];
      const int64_t n = mats[c0 + i].n, k = s.k, nr = n - k;
      Tm[(size_t)i] = ctx->arena.alloc_n<double>((size_t)std::max<int64_t>(k, 1) * std::max<int64_t>(nr, 1));
      if (k <= 0 || nr <= 0) continue;
      if (k <= kBsMax) {
        bs.push_back(BsItem{k, nr, s.order, s.B, Tm[(size_t)i]});
      } else {
        copy_matrix(ctx, k, nr, s.B + k * s.order, s.order, Tm[(size_t)i], k);
        trsm_upper(ctx, k, nr, s.B, s.order, Tm[(size_t)i], k);
      }
    }
    tmark(3);
    trsm_bs_batch(ctx, (int64_t)bs.size(), bs.data());
    tmark(4);
    // the results of the chunk packed on the device and copied in one
    // transfer into a page-locked slab: per matrix jpvt (sk then rd) and T,
    // with 8 bytes of padding so that every array starts inside the slab
    std::vector<size_t> off((size_t)cn + 1, 0);
    std::vector<PackItem> pk((size_t)cn);
    for (int64_t i = 0; i < cn; ++i) {
      const int64_t n = mats[c0 + i].n, k = st[(size_t)i].k;
      pk[(size_t)i] = PackItem{n, k * (n - k), st[(size_t)i].jpvt, Tm[(size_t)i], off[(size_t)i]};
      off[(size_t)i + 1] = off[(size_t)i] + 8 * (size_t)(n + k * (n - k) + 1);
    }
    const size_t total = off[(size_t)cn];
    char* dout = ctx->arena.alloc_n<char>(total);
    pack_results(ctx, cn, pk.data(), dout);
    char* slab = hslab(total, (int)(3 * cn));
    LRA_CUDA(cudaMemcpyAsync(slab, dout, total, cudaMemcpyDeviceToHost, ctx->stream));
    for (int64_t i = 0; i < cn; ++i) {
      const St& s = st[(size_t)i];
      const int64_t n = mats[c0 + i].n, k = s.k;
      lra_id* r = static_cast<lra_id*>(hmalloc(sizeof(lra_id)));
      std::memset(r, 0, sizeof *r);
      outs[c0 + i] = r;
      r->dtype = LRA_F64;
      r->nsteps = s.nsteps;
      r->k = k;
      r->n = n;
      char* base = slab + off[(size_t)i];
      r->sk = reinterpret_cast<int64_t*>(base);
      r->rd = reinterpret_cast<int64_t*>(base) + k;
      r->T = base + 8 * (size_t)n;
    }
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    tmark(5);
    ctx->arena.release(mk);
    c0 = c1;
  }
  if (tr)
    std::fprintf(stderr,
                 "[lra] idfact_batched grouped, %lld matrices (ms): stage+split %.2f sketches %.2f qr %.2f "
                 "readback %.2f solve %.2f results %.2f\n",
                 (long long)count, tph[0], tph[1], tph[2], tph[3], tph[4], tph[5]);
}

int try_idfact_batched_grouped(lra_ctx* ctx, int dtype, int64_t count, const lra_matdesc* mats,
                               const lra_opts* opts, const lra_rand* rand, lra_id** outs) {
  if (!ctx || !opts || dtype != LRA_F64) return -1;
  if (opts->precision != LRA_PREC_MIXED) return -1;
  bool ok = false;
  const int st0 = guarded(ctx, [&] {
    chkopts(opts);
    ok = grouped_batch_ok(ctx, count, mats, *opts, rand);
  });
  if (st0 != LRA_OK || !ok) return -1;
  const int st = guarded(ctx, [&] { idfact_batched_grouped(ctx, count, mats, *opts, outs); });
  if (st != LRA_OK)
    for (int64_t i = 0; i < count; ++i) {
      lra_id_free(outs[i]);
      outs[i] = nullptr;
    }
  return st;
}

}  // namespace lra


namespace lra {
namespace {
int64_t psvdrank(const std::vector<double>& s, const lra_opts& o);
std::pair<int64_t, int64_t> pheigrank(const std::vector<double>& w, const lra_opts& o);
}  // namespace
}  // namespace lra

// ======================================================================================
// complex element types (ComplexF32 / ComplexF64): the same drivers on the
// complex kernels of cplx.cu, native precision.  The reference's A' is a
// conjugate transpose throughout; Gaussian draws are crandn's pairs
// (src/util.jl:4-11): entry t of a complex draw is (g[2t], g[2t + 1]).
// ======================================================================================
namespace lra {
namespace {

bool is_cplx(int dtype) { return dtype == LRA_C32 || dtype == LRA_C64; }

template <class Fn>
void dispatch_c(int dtype, Fn&& fn) {
  if (dtype == LRA_C32)
    fn(float{});
  else
    fn(double{});
}

template <typename R>
using CX = cx<R>;

// complex Gaussian draws (n entries) into out
template <typename R>
void cgauss(RandSrc& rs, int64_t n, CX<R>* out) {
  rs.gauss<R>(2 * n, reinterpret_cast<R*>(out), false);
}

// raw Gaussian doubles on the device (the injected stream, or the library's)
template <typename R>
const double* gauss_raw_dev(lra_ctx* ctx, RandSrc& rs, int64_t n) {
  if (rs.injected_gauss()) return rs.take_gauss_raw(n);
  double* d = ctx->arena.alloc_n<double>(std::max<int64_t>(n, 1));
  rs.gauss<double>(n, d, false);
  return d;
}

template <typename R>
void check_input_c(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, const DMat<CX<R>>& A) {
  if (ctx->linop) return;
  if (o.check_finite &&
      !all_finite(ctx, 2 * m, n, reinterpret_cast<const R*>(A.p), 2 * A.ld))
    fail(LRA_ENONFINITE, "input has NaN or Inf entries");
}

// orthcols!(thin = false): Q of the QR in the first min(m, n) columns, zeros after
template <typename R>
void orthcols_c(lra_ctx* ctx, int64_t m, int64_t n, CX<R>* B) {
  const ArenaMark mk = ctx->arena.mark();
  const int64_t kq = std::min(m, n);
  int64_t* jp = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(n, 1));
  CX<R>* tau = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(kq, 1));
  cgeqp3<R>(ctx, m, n, B, std::max<int64_t>(m, 1), jp, tau, kq, 32, -1.0, 0.0, false);
  corgqr<R>(ctx, m, kq, B, std::max<int64_t>(m, 1), tau);
  if (n > kq) set_zero<CX<R>>(ctx, B + kq * m, m * (n - kq));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

// orthrows!(thin = false): rows of the LQ's Q (the QR of B^H), zeros after
template <typename R>
void orthrows_c(lra_ctx* ctx, int64_t m, int64_t n, CX<R>* B) {
  const ArenaMark mk = ctx->arena.mark();
  CX<R>* W = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(n, 1) * std::max<int64_t>(m, 1));
  cadjoint<R>(ctx, m, n, B, std::max<int64_t>(m, 1), W, std::max<int64_t>(n, 1));
  orthcols_c<R>(ctx, n, m, W);
  cadjoint<R>(ctx, n, m, W, std::max<int64_t>(n, 1), B, std::max<int64_t>(m, 1));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

// the operand accessors of the gather-type sketches: the left sketch of
// op(A) reads op(A) itself, the right sketch reads op(A)^T (its output is
// written transposed)
inline char c_mode(char trans, bool right) {
  // 'n': A(t, col) as stored; 'c': conj(A(col, t)); 't': A(col, t); 'j': conj(A(t, col))
  if (!right) return trans == 'n' ? 'n' : 'c';
  return trans == 'n' ? 't' : 'j';
}

// sketch(side, trans, A, order) for complex A (src/sketch.jl:35-46, 87-690):
// left: B (order x N) = S op(A); right: B (M x order) = op(A) S, op(A) M x N
template <typename R>
void make_sketch_c(lra_ctx* ctx, const lra_opts& o, char trans, int64_t M, int64_t N, const CX<R>* A, int64_t lda,
                   int64_t order, RandSrc& rs, CX<R>* B, bool right) {
  const ArenaMark mk = ctx->arena.mark();
  const CX<R> one(1), zero(0);
  const char op = trans == 'n' ? 'n' : 'c', opH = trans == 'n' ? 'c' : 'n';
  const int64_t ldb = right ? std::max<int64_t>(M, 1) : std::max<int64_t>(order, 1);
  switch (o.sketch) {
    case LRA_SKETCH_RANDN: {
      const bool herm = (M == N) && [&] {
        return ctx->linop ? ctx->linop->hermitian != 0 : cis_hermitian<R>(ctx, M, A, lda);
      }();
      if (!right) {
        CX<R>* S = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(order * M, 1));
        cgauss<R>(rs, order * M, S);
        cgemm<R>(ctx, 'n', op, order, N, M, one, S, ldb, A, lda, zero, B, ldb);
        CX<R>* Bq = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(order * M, 1));
        for (int64_t it = 0; it < o.sketch_randn_niter; ++it) {
          orthrows_c<R>(ctx, order, N, B);
          cgemm<R>(ctx, 'n', opH, order, M, N, one, B, ldb, A, lda, zero, Bq, ldb);
          if (herm) {
            copy_matrix<CX<R>>(ctx, order, M, Bq, ldb, B, ldb);
          } else {
            orthrows_c<R>(ctx, order, M, Bq);
            cgemm<R>(ctx, 'n', op, order, N, M, one, Bq, ldb, A, lda, zero, B, ldb);
          }
        }
      } else {
        CX<R>* S = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(N * order, 1));
        cgauss<R>(rs, N * order, S);
        cgemm<R>(ctx, op, 'n', M, order, N, one, A, lda, S, std::max<int64_t>(N, 1), zero, B, ldb);
        CX<R>* Bq = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(N * order, 1));
        const int64_t ldq = std::max<int64_t>(N, 1);
        for (int64_t it = 0; it < o.sketch_randn_niter; ++it) {
          orthcols_c<R>(ctx, M, order, B);
          cgemm<R>(ctx, opH, 'n', N, order, M, one, A, lda, B, ldb, zero, Bq, ldq);
          if (herm) {
            copy_matrix<CX<R>>(ctx, N, order, Bq, ldq, B, ldb);
          } else {
            orthcols_c<R>(ctx, N, order, Bq);
            cgemm<R>(ctx, op, 'n', M, order, N, one, A, lda, Bq, ldq, zero, B, ldb);
          }
        }
      }
      break;
    }
    case LRA_SKETCH_SRFT: {
      // the transform runs over the sketched dimension K: M (left) or N (right)
      const int64_t K = right ? N : M, C = right ? M : N;
      if (K >= ((int64_t)1 << 31)) fail(LRA_ENOTSUP, "complex SRFT of more than 2^31 rows");
      CX<R>* d = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(K, 1));
      cphases<R>(ctx, gauss_raw_dev<R>(ctx, rs, 2 * K), K, d);
      int64_t* idx = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(order, 1));
      rs.ints(order, K, idx, false);
      CX<R>* Bl = right ? ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(order * C, 1)) : B;
      csrft_direct<R>(ctx, c_mode(trans, right), K, C, A, lda, d, idx, order, Bl, std::max<int64_t>(order, 1));
      if (right) transpose<CX<R>>(ctx, order, C, Bl, std::max<int64_t>(order, 1), B, ldb);
      break;
    }
    case LRA_SKETCH_SUB: {
      const int64_t K = right ? N : M, C = right ? M : N;
      int64_t* rows = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(order, 1));
      rs.ints(order, K, rows, false);
      CX<R>* Bl = right ? ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(order * C, 1)) : B;
      csub<R>(ctx, c_mode(trans, right), C, A, lda, rows, order, Bl, std::max<int64_t>(order, 1));
      if (right) transpose<CX<R>>(ctx, order, C, Bl, std::max<int64_t>(order, 1), B, ldb);
      break;
    }
    case LRA_SKETCH_SPRN: {
      const int64_t K = right ? N : M, C = right ? M : N;
      int64_t* perm = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(K, 1));
      rs.ints(K, K, perm, true);
      CX<R>* g = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(K, 1));
      cgauss<R>(rs, K, g);
      std::vector<int64_t> start(order + 1, 0);
      for (int64_t i = 1; i <= order; ++i) start[i] = start[i - 1] + (K - i) / order + 1;
      int64_t* dst = ctx->arena.alloc_n<int64_t>(order + 1);
      LRA_CUDA(cudaMemcpyAsync(dst, start.data(), (order + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                               ctx->stream));
      CX<R>* Bl = right ? ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(order * C, 1)) : B;
      csprn<R>(ctx, c_mode(trans, right), K, C, A, lda, perm, g, dst, order, Bl, std::max<int64_t>(order, 1));
      if (right) transpose<CX<R>>(ctx, order, C, Bl, std::max<int64_t>(order, 1), B, ldb);
      break;
    }
    default:
      fail(LRA_EINVAL, "sketch");
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

template <typename R>
struct CFact {
  CX<R>* B = nullptr;  // rows x N, R in the upper triangle
  int64_t ld = 0, order = 0, N = 0;
  int64_t* jpvt = nullptr;
  CX<R>* tau = nullptr;
  int64_t k = 0;
  int nsteps = 0;
  CX<R>* T_ = nullptr;
  int64_t swaps = 0;
  CX<R>* r1 = nullptr;
  CX<R>* r1tau = nullptr;
};

// geqp3_adap! of a dense rows x N device matrix B (ld), in place
template <typename R>
CFact<R> cpqr_backend(lra_ctx* ctx, const lra_opts& o, CX<R>* B, int64_t rows, int64_t N, int64_t ld) {
  CFact<R> F;
  F.B = B;
  F.ld = ld;
  F.order = rows;
  F.N = N;
  const int64_t l = std::min(rows, N);
  const int64_t kmax = (o.rank < 0 || o.rank > l) ? l : o.rank;
  F.jpvt = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(N, 1));
  F.tau = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(l, 1));
  Stage st(ctx, 1);
  F.k = cgeqp3<R>(ctx, rows, N, B, ld, F.jpvt, F.tau, kmax, o.nb, o.atol, o.rtol, true);
  return F;
}

// sketchfact (src/sketch.jl:223-240 and twins): the adaptive doubling loop
template <typename R>
CFact<R> sketchfact_c(lra_ctx* ctx, const lra_opts& o, char trans, bool right, int64_t M, int64_t N,
                      const CX<R>* A, int64_t lda, RandSrc& rs) {
  const bool adaptive = o.sketchfact_adap || o.rank < 0;
  int64_t nt = adaptive ? o.nb : o.rank;
  CFact<R> F;
  const ArenaMark base = ctx->arena.mark();
  for (int step = 0;; ++step) {
    if (step > 62) fail(LRA_EINVAL, "adaptive sketch did not terminate");
    const int64_t order = samp(o, nt);
    if (order < 0) fail(LRA_EINVAL, "sketch order %lld", (long long)order);
    const int64_t rows = right ? M : order, cols = right ? order : N;
    CX<R>* B = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(rows, 1) * std::max<int64_t>(cols, 1));
    {
      Stage st(ctx, 0);
      make_sketch_c<R>(ctx, o, trans, M, N, A, lda, order, rs, B, right);
    }
    lra_opts oq = o;
    F = cpqr_backend<R>(ctx, oq, B, rows, cols, std::max<int64_t>(rows, 1));
    F.nsteps = step + 1;
    if (!adaptive || F.k < nt) break;
    nt *= 2;
    ctx->arena.release(base);
  }
  return F;
}

// T = R11 \ R12 and maxdet (src/pqr.jl:420-501), as postproc_t does
template <typename R>
void cpostproc(lra_ctx* ctx, const lra_opts& o, CFact<R>& F, bool want_t) {
  const bool maxdet = F.k > 0 && F.k < F.N && o.maxdet_tol >= 0;
  if (!(want_t || maxdet)) return;
  Stage st(ctx, 2);
  const int64_t k = F.k, nr = F.N - k, kk = std::max<int64_t>(k, 1);
  F.T_ = ctx->arena.alloc_n<CX<R>>((size_t)kk * std::max<int64_t>(nr, 1));
  if (k > 0 && nr > 0) {
    copy_matrix<CX<R>>(ctx, k, nr, F.B + k * F.ld, F.ld, F.T_, k);
    ctrsm_upper<R>(ctx, k, nr, F.B, F.ld, F.T_, k);
  }
  if (!maxdet) return;
  const bool retr = o.pqrfact_retval & LRA_RET_R;
  CX<R>* R1 = nullptr;
  if (retr) {
    R1 = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
    copy_matrix<CX<R>>(ctx, k, k, F.B, F.ld, R1, kk);
    zero_lower<CX<R>>(ctx, k, k, R1, kk);
  }
  const int64_t cap = 64 * (k + nr) + 1000;
  int64_t niter = 0;
  while (niter < cap) {
    const bool upd = niter != o.maxdet_niter;
    if (!cmaxdet_step<R>(ctx, k, nr, F.T_, F.jpvt, 1.0 + o.maxdet_tol, upd, R1, kk)) break;
    if (!upd) break;
    ++niter;
  }
  F.swaps = niter;
  if (niter > 0 && R1) {
    CX<R>* t1 = ctx->arena.alloc_n<CX<R>>(kk);
    int64_t* jp = ctx->arena.alloc_n<int64_t>(kk);
    cgeqp3<R>(ctx, k, k, R1, kk, jp, t1, k, 32, -1.0, 0.0, false);
    F.r1 = R1;
    F.r1tau = t1;
  }
}

template <typename R>
void cresult_r11(lra_ctx* ctx, const CFact<R>& F, CX<R>* R11) {
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1);
  if (F.r1)
    copy_matrix<CX<R>>(ctx, k, k, F.r1, kk, R11, kk);
  else
    copy_matrix<CX<R>>(ctx, k, k, F.B, F.ld, R11, kk);
  zero_lower<CX<R>>(ctx, k, k, R11, kk);
}

// Q <- Q Qf after maxdet re-factored R1 (gemqrt!('R', 'N'), src/pqr.jl:468)
template <typename R>
void cmaxdet_rotate_q(lra_ctx* ctx, const CFact<R>& F, int64_t M, CX<R>* Q, int64_t ldq) {
  const int64_t k = F.k;
  if (!F.r1 || k <= 0 || M <= 0) return;
  CX<R>* Qh = ctx->arena.alloc_n<CX<R>>((size_t)k * M);
  cadjoint<R>(ctx, M, k, Q, ldq, Qh, k);                       // Q^H (k x M)
  capply_q<R>(ctx, 'c', k, k, F.r1, k, F.r1tau, Qh, k, M);      // Qf^H Q^H
  cadjoint<R>(ctx, k, M, Qh, k, Q, ldq);
}

// op(A) as a dense device copy (M x N, ld M)
template <typename R>
CX<R>* cdense_op(lra_ctx* ctx, char trans, int64_t m, int64_t n, const DMat<CX<R>>& A) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  CX<R>* B = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(N, 1));
  if (trans == 'n')
    copy_matrix<CX<R>>(ctx, m, n, A.p, A.ld, B, std::max<int64_t>(M, 1));
  else
    cadjoint<R>(ctx, m, n, A.p, A.ld, B, std::max<int64_t>(M, 1));
  return B;
}

// getcols(trans, A, idx) (src/util.jl:25-29): M x k
template <typename R>
CX<R>* cgetcols(lra_ctx* ctx, char trans, int64_t m, int64_t n, const DMat<CX<R>>& A, const int64_t* idx,
                int64_t k) {
  const int64_t M = trans == 'n' ? m : n;
  CX<R>* C = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(k, 1));
  if (trans == 'n') {
    gather_cols<CX<R>>(ctx, m, k, A.p, A.ld, idx, C, std::max<int64_t>(M, 1));
  } else {
    CX<R>* Rw = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(k, 1) * std::max<int64_t>(n, 1));
    gather_rows<CX<R>>(ctx, k, n, A.p, A.ld, idx, Rw, std::max<int64_t>(k, 1));
    cadjoint<R>(ctx, k, n, Rw, std::max<int64_t>(k, 1), C, std::max<int64_t>(M, 1));
  }
  return C;
}

template <typename R>
CFact<R> cid_core(lra_ctx* ctx, const lra_opts& o, char trans, int64_t m, int64_t n, const DMat<CX<R>>& A,
                  RandSrc& rs, bool want_t) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  CFact<R> F;
  if (o.sketch == LRA_SKETCH_NONE) {
    CX<R>* B = cdense_op<R>(ctx, trans, m, n, A);
    F = cpqr_backend<R>(ctx, o, B, M, N, std::max<int64_t>(M, 1));
  } else {
    F = sketchfact_c<R>(ctx, o, trans, false, M, N, A.p, A.ld, rs);
  }
  cpostproc<R>(ctx, o, F, want_t);
  return F;
}

template <typename R>
lra_id* cpack_id(lra_ctx* ctx, const CFact<R>& F, int dtype) {
  lra_id* r = static_cast<lra_id*>(hmalloc(sizeof(lra_id)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->nsteps = F.nsteps;
  r->k = F.k;
  r->n = F.N;
  r->sk = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(F.k, 1)));
  r->rd = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(F.N - F.k, 1)));
  r->T = hmalloc(sizeof(CX<R>) * std::max<int64_t>(F.k * (F.N - F.k), 1));
  to_host(ctx, r->sk, F.jpvt, F.k);
  to_host(ctx, r->rd, F.jpvt + F.k, F.N - F.k);
  if (F.k > 0 && F.N > F.k) to_host(ctx, r->T, F.T_, (size_t)F.k * (F.N - F.k));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}

// the pivoted QR's Q (rows x k) of F and its R = [R11 | R11 T] (k x N)
template <typename R>
void cfact_qr(lra_ctx* ctx, CFact<R>& F, bool rq, bool rr, lra_pqr* r) {
  const int64_t k = F.k, N = F.N, rows = F.order, kk = std::max<int64_t>(k, 1);
  if (rr) {
    CX<R>* Rm = ctx->arena.alloc_n<CX<R>>((size_t)kk * std::max<int64_t>(N, 1));
    cresult_r11<R>(ctx, F, Rm);
    if (N > k && k > 0) {
      if (F.T_)
        cgemm<R>(ctx, 'n', 'n', k, N - k, k, CX<R>(1), Rm, kk, F.T_, kk, CX<R>(0), Rm + k * kk, kk);
      else {
        copy_matrix<CX<R>>(ctx, k, N - k, F.B + k * F.ld, F.ld, Rm + k * kk, kk);
      }
    }
    r->R = hmalloc(sizeof(CX<R>) * std::max<int64_t>(k * N, 1));
    to_host(ctx, r->R, Rm, (size_t)k * N);
    r->retval |= LRA_RET_R;
  }
  if (rq) {
    corgqr<R>(ctx, rows, k, F.B, F.ld, F.tau);
    cmaxdet_rotate_q<R>(ctx, F, rows, F.B, F.ld);
    r->Q = hmalloc(sizeof(CX<R>) * std::max<int64_t>(rows * k, 1));
    if (k > 0 && rows > 0)
      LRA_CUDA(cudaMemcpy2DAsync(r->Q, rows * sizeof(CX<R>), F.B, F.ld * sizeof(CX<R>), rows * sizeof(CX<R>), k,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    r->retval |= LRA_RET_Q;
  }
}

template <typename R>
lra_pqr* new_pqr(int dtype, int64_t m, int64_t n, int64_t k) {
  lra_pqr* r = static_cast<lra_pqr*>(hmalloc(sizeof(lra_pqr)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->m = m;
  r->n = n;
  r->k = k;
  r->p = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(n, 1)));
  return r;
}

// sketchfact(side, trans, A) for complex A
template <typename R>
lra_pqr* csketchfact(lra_ctx* ctx, const lra_opts& o0, char side, char t, int64_t m, int64_t n,
                     const DMat<CX<R>>& A, RandSrc& rs, int dtype) {
  lra_opts o = o0;
  if (o.sketch == LRA_SKETCH_NONE) o.sketch = LRA_SKETCH_RANDN;
  const bool right = side == 'r' || side == 'R';
  const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
  CFact<R> F = sketchfact_c<R>(ctx, o, t, right, M, N, A.p, A.ld, rs);
  const bool rq = o.pqrfact_retval & LRA_RET_Q, rr = o.pqrfact_retval & LRA_RET_R, rt = o.pqrfact_retval & LRA_RET_T;
  cpostproc<R>(ctx, o, F, rt);
  lra_pqr* r = new_pqr<R>(dtype, F.order, F.N, F.k);
  try {
    to_host(ctx, r->p, F.jpvt, F.N);
    if (rt) {
      r->T = hmalloc(sizeof(CX<R>) * std::max<int64_t>(F.k * (F.N - F.k), 1));
      if (F.k > 0 && F.N > F.k) to_host(ctx, r->T, F.T_, (size_t)F.k * (F.N - F.k));
      r->retval |= LRA_RET_T;
    }
    if (rr && !F.T_ && F.k > 0 && F.k < F.N) {
      // R = triu(B[1:k, :]) without maxdet (src/pqr.jl:428)
      CX<R>* Rm = ctx->arena.alloc_n<CX<R>>((size_t)F.k * F.N);
      copy_matrix<CX<R>>(ctx, F.k, F.N, F.B, F.ld, Rm, F.k);
      zero_lower<CX<R>>(ctx, F.k, F.N, Rm, F.k);
      r->R = hmalloc(sizeof(CX<R>) * (size_t)F.k * F.N);
      to_host(ctx, r->R, Rm, (size_t)F.k * F.N);
      r->retval |= LRA_RET_R;
      cfact_qr<R>(ctx, F, rq, false, r);
    } else {
      cfact_qr<R>(ctx, F, rq, rr, r);
    }
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    lra_pqr_free(r);
    throw;
  }
  return r;
}

// pqrfact(trans, A) (src/pqr.jl:290-307)
template <typename R>
lra_pqr* cpqrfact(lra_ctx* ctx, const lra_opts& o, char t, int64_t m, int64_t n, const DMat<CX<R>>& A,
                  RandSrc& rs, int dtype) {
  const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
  const bool rq = o.pqrfact_retval & LRA_RET_Q, rr = o.pqrfact_retval & LRA_RET_R, rt = o.pqrfact_retval & LRA_RET_T;
  lra_pqr* r = new_pqr<R>(dtype, M, N, 0);
  try {
    if (o.sketch == LRA_SKETCH_NONE) {
      CX<R>* B = cdense_op<R>(ctx, t, m, n, A);
      CFact<R> F = cpqr_backend<R>(ctx, o, B, M, N, std::max<int64_t>(M, 1));
      cpostproc<R>(ctx, o, F, rt || rr);
      r->k = F.k;
      to_host(ctx, r->p, F.jpvt, N);
      cfact_qr<R>(ctx, F, rq, rr, r);
      if (rt) {
        r->T = hmalloc(sizeof(CX<R>) * std::max<int64_t>(F.k * (N - F.k), 1));
        if (F.k > 0 && N > F.k) to_host(ctx, r->T, F.T_, (size_t)F.k * (N - F.k));
        r->retval |= LRA_RET_T;
      }
    } else {
      lra_opts oi = o;
      oi.pqrfact_retval = LRA_RET_T;
      CFact<R> F = cid_core<R>(ctx, oi, t, m, n, A, rs, true);
      const int64_t k = F.k, kk = std::max<int64_t>(k, 1);
      r->k = k;
      to_host(ctx, r->p, F.jpvt, N);
      // Q, R11 = qr(A[:, sk]); R = [R11 | R11 T] (pqrr, src/pqr.jl:330-340)
      CX<R>* Ask = cgetcols<R>(ctx, t, m, n, A, F.jpvt, k);
      int64_t* jp = ctx->arena.alloc_n<int64_t>(kk);
      CX<R>* tau = ctx->arena.alloc_n<CX<R>>(kk);
      cgeqp3<R>(ctx, M, k, Ask, std::max<int64_t>(M, 1), jp, tau, k, 32, -1.0, 0.0, false);
      CFact<R> Q;
      Q.B = Ask;
      Q.ld = std::max<int64_t>(M, 1);
      Q.order = M;
      Q.N = N;
      Q.k = k;
      Q.tau = tau;
      if (rr) {
        CX<R>* Rm = ctx->arena.alloc_n<CX<R>>((size_t)kk * std::max<int64_t>(N, 1));
        copy_matrix<CX<R>>(ctx, k, k, Ask, Q.ld, Rm, kk);
        zero_lower<CX<R>>(ctx, k, k, Rm, kk);
        if (N > k && k > 0)
          cgemm<R>(ctx, 'n', 'n', k, N - k, k, CX<R>(1), Rm, kk, F.T_, kk, CX<R>(0), Rm + k * kk, kk);
        r->R = hmalloc(sizeof(CX<R>) * std::max<int64_t>(k * N, 1));
        to_host(ctx, r->R, Rm, (size_t)k * N);
        r->retval |= LRA_RET_R;
      }
      if (rq) cfact_qr<R>(ctx, Q, true, false, r);
      if (rt) {
        r->T = hmalloc(sizeof(CX<R>) * std::max<int64_t>(k * (N - k), 1));
        if (k > 0 && N > k) to_host(ctx, r->T, F.T_, (size_t)k * (N - k));
        r->retval |= LRA_RET_T;
      }
    }
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    lra_pqr_free(r);
    throw;
  }
  return r;
}

// SVD of a k x k device matrix X (ld ldx, destroyed): U (k x k, ld k), S
// descending (host), V (k x k, ld k) with X = U diag(S) V^H
template <typename R>
std::vector<R> csmall_svd(lra_ctx* ctx, int64_t k, CX<R>* X, int64_t ldx, CX<R>* U, CX<R>* V) {
  const int64_t kk = std::max<int64_t>(k, 1);
  std::vector<R> hS(k);
  if (k <= 0) return hS;
  CX<R>* Xw = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  copy_matrix<CX<R>>(ctx, k, k, X, ldx, Xw, kk);
  CX<R>* Vw = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  R* S = ctx->arena.alloc_n<R>(kk);
  cjacobi_svd<R>(ctx, k, Xw, kk, Vw, kk, S);
  to_host(ctx, hS.data(), S, k);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> ord(k);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return hS[a] > hS[b]; });
  std::vector<int64_t> cols(k);
  std::vector<R> sorted(k);
  for (int64_t i = 0; i < k; ++i) {
    cols[i] = ord[i] + 1;
    sorted[i] = hS[ord[i]];
  }
  int64_t* dc = ctx->arena.alloc_n<int64_t>(kk);
  LRA_CUDA(cudaMemcpyAsync(dc, cols.data(), k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  gather_cols<CX<R>>(ctx, k, k, Xw, kk, dc, U, kk);
  gather_cols<CX<R>>(ctx, k, k, Vw, kk, dc, V, kk);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return sorted;
}

// psvdfact / psvdvals (src/psvd.jl:238-290)
template <typename R>
lra_psvd* cpsvd(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, const DMat<CX<R>>& A, RandSrc& rs,
                int dtype, bool vals_only) {
  const bool tall = m >= n;
  const char t = tall ? 'n' : 'c';
  const int64_t M = tall ? m : n, N = tall ? n : m;  // op(A) is M x N
  lra_opts oi = o;
  oi.pqrfact_retval = LRA_RET_T;
  CFact<R> F = cid_core<R>(ctx, oi, t, m, n, A, rs, true);
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1), ldq = std::max<int64_t>(M, 1), ldn = std::max<int64_t>(N, 1);
  Stage st(ctx, 3);
  // Q, R = qr(op(A)[:, sk])
  CX<R>* Q = cgetcols<R>(ctx, t, m, n, A, F.jpvt, k);
  int64_t* jp = ctx->arena.alloc_n<int64_t>(kk);
  CX<R>* tau = ctx->arena.alloc_n<CX<R>>(kk);
  cgeqp3<R>(ctx, M, k, Q, ldq, jp, tau, k, 32, -1.0, 0.0, false);
  CX<R>* Rm = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  copy_matrix<CX<R>>(ctx, k, k, Q, ldq, Rm, kk);
  zero_lower<CX<R>>(ctx, k, k, Rm, kk);
  corgqr<R>(ctx, M, k, Q, ldq, tau);
  // Wh = (R Vhat)^H (N x k): rows sk <- R^H, rows rd <- T^H R^H
  CX<R>* Wh = ctx->arena.alloc_n<CX<R>>((size_t)ldn * kk);
  {
    CX<R>* Rh = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
    cadjoint<R>(ctx, k, k, Rm, kk, Rh, kk);
    CX<R>* Wp = ctx->arena.alloc_n<CX<R>>((size_t)ldn * kk);  // [R^H; T^H R^H] in pivoted row order
    copy_matrix<CX<R>>(ctx, k, k, Rh, kk, Wp, ldn);
    if (N > k && k > 0)
      cgemm<R>(ctx, 'c', 'n', N - k, k, k, CX<R>(1), F.T_, kk, Rh, kk, CX<R>(0), Wp + k, ldn);
    set_zero<CX<R>>(ctx, Wh, ldn * kk);
    CX<R>* Wpt = ctx->arena.alloc_n<CX<R>>((size_t)kk * ldn);
    transpose<CX<R>>(ctx, N, k, Wp, ldn, Wpt, kk);
    CX<R>* Wt = ctx->arena.alloc_n<CX<R>>((size_t)kk * ldn);
    scatter_cols<CX<R>>(ctx, k, N, Wpt, kk, F.jpvt, Wt, kk);
    transpose<CX<R>>(ctx, k, N, Wt, kk, Wh, ldn);
  }
  // Wh = Q2 R2; R2^H = Ux S Vx^H; W = R Vhat = Ux S (Q2 Vx)^H
  int64_t* jp2 = ctx->arena.alloc_n<int64_t>(kk);
  CX<R>* tau2 = ctx->arena.alloc_n<CX<R>>(kk);
  cgeqp3<R>(ctx, N, k, Wh, ldn, jp2, tau2, k, 32, -1.0, 0.0, false);
  CX<R>* R2 = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  copy_matrix<CX<R>>(ctx, k, k, Wh, ldn, R2, kk);
  zero_lower<CX<R>>(ctx, k, k, R2, kk);
  CX<R>* X = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  cadjoint<R>(ctx, k, k, R2, kk, X, kk);
  CX<R>* Ux = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  CX<R>* Vx = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  std::vector<R> hS = csmall_svd<R>(ctx, k, X, kk, Ux, Vx);
  std::vector<double> sd(hS.begin(), hS.end());
  const int64_t kr = psvdrank(sd, o), lkr = std::max<int64_t>(kr, 1);
  lra_psvd* r = static_cast<lra_psvd*>(hmalloc(sizeof(lra_psvd)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->m = m;
  r->n = n;
  r->k = kr;
  r->S = hmalloc(sizeof(R) * lkr);
  std::memcpy(r->S, hS.data(), sizeof(R) * kr);
  if (vals_only) return r;
  // Vfull = Q2 Vx (N x k): the reflectors of Wh applied to [Vx; 0]
  CX<R>* Vf = ctx->arena.alloc_n<CX<R>>((size_t)ldn * lkr);
  set_zero<CX<R>>(ctx, Vf, ldn * lkr);
  copy_matrix<CX<R>>(ctx, k, kr, Vx, kk, Vf, ldn);
  capply_q<R>(ctx, 'n', N, k, Wh, ldn, tau2, Vf, ldn, kr);
  // op(A) = (Q Ux) S Vf^H
  CX<R>* Uf = ctx->arena.alloc_n<CX<R>>((size_t)ldq * lkr);
  cgemm<R>(ctx, 'n', 'n', M, kr, k, CX<R>(1), Q, ldq, Ux, kk, CX<R>(0), Uf, ldq);
  // A = Uf S Vf^H (m >= n), or A = op(A)^H = Vf S Uf^H (m < n)
  CX<R>* Uo = tall ? Uf : Vf;
  CX<R>* Vo = tall ? Vf : Uf;
  const int64_t ldu = tall ? ldq : ldn, ldv = tall ? ldn : ldq;
  CX<R>* Vt = ctx->arena.alloc_n<CX<R>>((size_t)lkr * std::max<int64_t>(n, 1));
  cadjoint<R>(ctx, n, kr, Vo, ldv, Vt, lkr);
  r->U = hmalloc(sizeof(CX<R>) * std::max<int64_t>(m * kr, 1));
  r->Vt = hmalloc(sizeof(CX<R>) * std::max<int64_t>(kr * n, 1));
  if (m > 0 && kr > 0)
    LRA_CUDA(cudaMemcpy2DAsync(r->U, m * sizeof(CX<R>), Uo, ldu * sizeof(CX<R>), m * sizeof(CX<R>), kr,
                               cudaMemcpyDeviceToHost, ctx->stream));
  to_host(ctx, r->Vt, Vt, (size_t)kr * n);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}

// pheigfact / pheigvals (src/pheig.jl:276-311)
template <typename R>
lra_pheig* cpheig(lra_ctx* ctx, const lra_opts& o, int64_t n, const DMat<CX<R>>& A, RandSrc& rs, int dtype,
                  bool vals_only) {
  lra_opts oi = o;
  oi.pqrfact_retval = LRA_RET_T;
  CFact<R> F = cid_core<R>(ctx, oi, 'n', n, n, A, rs, true);
  const int64_t k = F.k, kk = std::max<int64_t>(k, 1), ldn = std::max<int64_t>(n, 1);
  Stage st(ctx, 3);
  // Q, R = qr(Vhat^H): Vhat^H (n x k) has rows sk = I, rows rd = T^H
  CX<R>* Vh = ctx->arena.alloc_n<CX<R>>((size_t)ldn * kk);
  {
    CX<R>* P = ctx->arena.alloc_n<CX<R>>((size_t)kk * ldn);  // Vhat (k x n) in pivoted order
    set_identity<CX<R>>(ctx, k, k, P, kk);
    if (n > k && k > 0) copy_matrix<CX<R>>(ctx, k, n - k, F.T_, kk, P + k * kk, kk);
    CX<R>* Vm = ctx->arena.alloc_n<CX<R>>((size_t)kk * ldn);
    scatter_cols<CX<R>>(ctx, k, n, P, kk, F.jpvt, Vm, kk);
    cadjoint<R>(ctx, k, n, Vm, kk, Vh, ldn);
  }
  int64_t* jp = ctx->arena.alloc_n<int64_t>(kk);
  CX<R>* tau = ctx->arena.alloc_n<CX<R>>(kk);
  cgeqp3<R>(ctx, n, k, Vh, ldn, jp, tau, k, 32, -1.0, 0.0, false);
  CX<R>* Rm = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  copy_matrix<CX<R>>(ctx, k, k, Vh, ldn, Rm, kk);
  zero_lower<CX<R>>(ctx, k, k, Rm, kk);
  // B = R (A[sk, sk] R^H)
  CX<R>* Ass = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  {
    CX<R>* Ac = cgetcols<R>(ctx, 'n', n, n, A, F.jpvt, k);
    gather_rows<CX<R>>(ctx, k, k, Ac, ldn, F.jpvt, Ass, kk);
  }
  CX<R>* Cm = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  cgemm<R>(ctx, 'n', 'c', k, k, k, CX<R>(1), Ass, kk, Rm, kk, CX<R>(0), Cm, kk);
  CX<R>* B = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  cgemm<R>(ctx, 'n', 'n', k, k, k, CX<R>(1), Rm, kk, Cm, kk, CX<R>(0), B, kk);
  chermitianize<R>(ctx, k, B, kk);
  // eigen! through the Jacobi SVD of the positive shift B + s I
  R* cn = ctx->arena.alloc_n<R>(kk);
  ccol_norms<R>(ctx, k, k, B, kk, cn);
  std::vector<R> hcn(k);
  to_host(ctx, hcn.data(), cn, k);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  double fro = 0;
  for (R v : hcn) fro += (double)v * (double)v;
  const R shift = (R)(std::sqrt(fro) * 1.0001 + (fro == 0 ? 1.0 : 0.0));
  cadd_diag<R>(ctx, k, B, kk, shift);
  CX<R>* U = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  CX<R>* Z = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  std::vector<R> hS = csmall_svd<R>(ctx, k, B, kk, U, Z);
  std::vector<double> w(k);
  for (int64_t i = 0; i < k; ++i) w[i] = (double)hS[i] - (double)shift;
  std::vector<int64_t> ord(k);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return w[a] < w[b]; });
  std::vector<double> ws(k);
  for (int64_t i = 0; i < k; ++i) ws[i] = w[ord[i]];
  auto kp = pheigrank(ws, o);
  std::vector<int64_t> sel;
  if (kp.first + kp.second < k) {
    for (int64_t i = 0; i < kp.first; ++i) sel.push_back(i);
    for (int64_t i = k - kp.second; i < k; ++i) sel.push_back(i);
  } else {
    for (int64_t i = 0; i < k; ++i) sel.push_back(i);
  }
  const int64_t ke = (int64_t)sel.size();
  lra_pheig* r = static_cast<lra_pheig*>(hmalloc(sizeof(lra_pheig)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->n = n;
  r->k = ke;
  r->values = hmalloc(sizeof(R) * std::max<int64_t>(ke, 1));
  std::vector<double> vals(ke);
  for (int64_t i = 0; i < ke; ++i) {
    vals[i] = ws[sel[i]];
    static_cast<R*>(r->values)[i] = (R)vals[i];
  }
  if (!vals_only && ke > 0) {
    std::vector<int64_t> cols1(ke);
    for (int64_t i = 0; i < ke; ++i) cols1[i] = ord[sel[i]] + 1;
    int64_t* dcols = ctx->arena.alloc_n<int64_t>(ke);
    LRA_CUDA(cudaMemcpyAsync(dcols, cols1.data(), ke * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    CX<R>* Zs = ctx->arena.alloc_n<CX<R>>((size_t)ldn * ke);
    set_zero<CX<R>>(ctx, Zs, ldn * ke);
    gather_cols<CX<R>>(ctx, k, ke, Z, kk, dcols, Zs, ldn);
    std::vector<int64_t> cl;
    int64_t a = 0;
    while (a < ke) {
      const double va = vals[a];
      int64_t b = a + 1;
      while (b < ke) {
        if (2 * std::fabs((va - vals[b]) / (va + vals[b])) > o.pheig_orthtol) break;
        ++b;
      }
      --b;
      if (b > a) {
        cl.push_back(a);
        cl.push_back(b + 1);
      }
      a = b + 1;
    }
    if (!cl.empty()) {
      int64_t* dcl = ctx->arena.alloc_n<int64_t>(cl.size());
      LRA_CUDA(cudaMemcpyAsync(dcl, cl.data(), cl.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
      ccluster_orth<R>(ctx, k, ke, Zs, ldn, dcl, (int64_t)cl.size() / 2);
    }
    capply_q<R>(ctx, 'n', n, k, Vh, ldn, tau, Zs, ldn, ke);
    r->vectors = hmalloc(sizeof(CX<R>) * (size_t)n * ke);
    to_host(ctx, r->vectors, Zs, (size_t)n * ke);
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return r;
}

// curfact (src/cur.jl:532-606)
template <typename R>
lra_cur* ccurfact(lra_ctx* ctx, const lra_opts& o0, int64_t m, int64_t n, const DMat<CX<R>>& A, RandSrc& rs) {
  lra_opts o = o0;
  o.pqrfact_retval = 0;
  auto sel = [&](char t, int64_t mm, int64_t nn, const DMat<CX<R>>& X) {
    CFact<R> F = cid_core<R>(ctx, o, t, mm, nn, X, rs, false);
    std::vector<int64_t> idx(F.k);
    to_host(ctx, idx.data(), F.jpvt, F.k);
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    return idx;
  };
  lra_cur* r = static_cast<lra_cur*>(hmalloc(sizeof(lra_cur)));
  std::memset(r, 0, sizeof *r);
  std::vector<int64_t> rows, cols;
  if (m == n && cis_hermitian<R>(ctx, n, A.p, A.ld)) {
    cols = sel('n', m, n, A);
    rows = cols;
    r->kind = 1;
  } else if (m >= n) {
    rows = sel('c', m, n, A);
    const int64_t kr = (int64_t)rows.size();
    int64_t* drows = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(kr, 1));
    LRA_CUDA(cudaMemcpyAsync(drows, rows.data(), kr * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    CX<R>* Ar = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(kr, 1) * std::max<int64_t>(n, 1));
    gather_rows<CX<R>>(ctx, kr, n, A.p, A.ld, drows, Ar, std::max<int64_t>(kr, 1));
    cols = sel('n', kr, n, DMat<CX<R>>{Ar, std::max<int64_t>(kr, 1)});
  } else {
    cols = sel('n', m, n, A);
    const int64_t kc = (int64_t)cols.size();
    int64_t* dcols = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(kc, 1));
    LRA_CUDA(cudaMemcpyAsync(dcols, cols.data(), kc * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    CX<R>* Ac = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(m, 1) * std::max<int64_t>(kc, 1));
    gather_cols<CX<R>>(ctx, m, kc, A.p, A.ld, dcols, Ac, std::max<int64_t>(m, 1));
    rows = sel('c', m, kc, DMat<CX<R>>{Ac, std::max<int64_t>(m, 1)});
  }
  if (r->kind == 0) {
    const size_t k = std::min(rows.size(), cols.size());
    rows.resize(k);
    cols.resize(k);
  }
  r->kr = (int64_t)rows.size();
  r->kc = (int64_t)cols.size();
  r->rows = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<size_t>(rows.size(), 1)));
  r->cols = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<size_t>(cols.size(), 1)));
  std::memcpy(r->rows, rows.data(), rows.size() * sizeof(int64_t));
  std::memcpy(r->cols, cols.data(), cols.size() * sizeof(int64_t));
  return r;
}

// prange (src/prange.jl:14-77)
template <typename R>
lra_pqr* cprange(lra_ctx* ctx, const lra_opts& o, char t, int64_t m, int64_t n, const DMat<CX<R>>& A, RandSrc& rs,
                 int dtype) {
  if (t == 'b') {
    if (m != n) fail(LRA_EDIM, "prange(:b): the matrix must be square");
    if (cis_hermitian<R>(ctx, n, A.p, A.ld)) t = 'n';
  }
  auto side_q = [&](char tr, int64_t& k, CX<R>** R11) -> CX<R>* {
    const int64_t M = tr == 'n' ? m : n, N = tr == 'n' ? n : m;
    CFact<R> F;
    if (o.sketch == LRA_SKETCH_NONE) {
      CX<R>* B = cdense_op<R>(ctx, tr, m, n, A);
      F = cpqr_backend<R>(ctx, o, B, M, N, std::max<int64_t>(M, 1));
    } else {
      F = sketchfact_c<R>(ctx, o, tr, true, M, N, A.p, A.ld, rs);
    }
    if (R11 && o.maxdet_tol >= 0) {
      lra_opts oq = o;
      oq.pqrfact_retval = LRA_RET_Q | LRA_RET_R;
      cpostproc<R>(ctx, oq, F, false);
    }
    k = F.k;
    const int64_t kk = std::max<int64_t>(k, 1);
    if (R11) {
      *R11 = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
      cresult_r11<R>(ctx, F, *R11);
    }
    corgqr<R>(ctx, M, k, F.B, F.ld, F.tau);
    cmaxdet_rotate_q<R>(ctx, F, M, F.B, F.ld);
    return F.B;
  };
  const int64_t M = t == 'c' ? n : m;
  int64_t k = 0;
  CX<R>* Q = nullptr;
  if (t == 'b') {
    int64_t kr = 0, kc = 0;
    CX<R>*Rr = nullptr, *Rc = nullptr;
    CX<R>* Qr = side_q('c', kr, &Rr);
    CX<R>* Qc = side_q('n', kc, &Rc);
    const int64_t kb = kr + kc;
    CX<R>* Bc = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(kb, 1));
    if (kr > 0) cgemm<R>(ctx, 'n', 'n', M, kr, kr, CX<R>(1), Qr, M, Rr, kr, CX<R>(0), Bc, M);
    if (kc > 0) cgemm<R>(ctx, 'n', 'n', M, kc, kc, CX<R>(1), Qc, M, Rc, kc, CX<R>(0), Bc + kr * M, M);
    CFact<R> F = cpqr_backend<R>(ctx, o, Bc, M, kb, std::max<int64_t>(M, 1));
    k = F.k;
    corgqr<R>(ctx, M, k, F.B, F.ld, F.tau);
    Q = F.B;
  } else if (o.sketch == LRA_SKETCH_SUB) {
    const int64_t N = t == 'n' ? n : m;
    CFact<R> F = sketchfact_c<R>(ctx, o, t, false, M, N, A.p, A.ld, rs);
    if (o.maxdet_tol >= 0) {
      lra_opts oq = o;
      oq.pqrfact_retval = LRA_RET_Q;
      cpostproc<R>(ctx, oq, F, false);
    }
    const int64_t kc = F.k, kq = std::min(M, kc);
    Q = cgetcols<R>(ctx, t, m, n, A, F.jpvt, kc);
    if (kq > 0) orthcols_c<R>(ctx, M, kc, Q);
    k = kq;
  } else {
    Q = side_q(t, k, nullptr);
  }
  lra_pqr* r = new_pqr<R>(dtype, M, k, k);
  for (int64_t i = 0; i < k; ++i) r->p[i] = i + 1;
  r->Q = hmalloc(sizeof(CX<R>) * std::max<int64_t>(M * k, 1));
  if (k > 0 && M > 0) to_host(ctx, r->Q, Q, (size_t)M * k);
  r->retval = LRA_RET_Q;
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}

// snorm / snormdiff power iteration (src/snorm.jl:14-53), complex vectors
template <typename R, class FwdFn, class AdjFn>
double csnorm_loop(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, bool herm, RandSrc& rs, FwdFn fwd,
                   AdjFn adj) {
  CX<R>* xn = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(n, 1));
  CX<R>* xm = ctx->arena.alloc_n<CX<R>>(std::max<int64_t>(m, 1));
  R* nrm = ctx->arena.alloc_n<R>(1);
  cgauss<R>(rs, n, xn);
  auto norm = [&](const CX<R>* x, int64_t len) {
    ccol_norms<R>(ctx, len, 1, x, std::max<int64_t>(len, 1), nrm);
    R h = 0;
    to_host(ctx, &h, nrm, 1);
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    return (double)h;
  };
  double xnrm = norm(xn, n);
  double s = 1, t = 0;
  int64_t niter = 0;
  while (s > 0 && std::fabs(s - t) > std::max(o.atol, t * o.rtol)) {
    if (niter == o.snorm_niter) break;
    ++niter;
    scale_vec<R>(ctx, 2 * n, reinterpret_cast<R*>(xn), (R)(1.0 / xnrm));
    if (herm) {
      fwd(xn, xm);
      copy_matrix<CX<R>>(ctx, n, 1, xm, std::max<int64_t>(n, 1), xn, std::max<int64_t>(n, 1));
    } else {
      fwd(xn, xm);
      adj(xm, xn);
    }
    xnrm = norm(xn, n);
    t = s;
    s = herm ? xnrm : std::sqrt(xnrm);
  }
  return s;
}


template <typename R>
double csnormdiff_dense(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, const CX<R>* A, int64_t lda,
                        const CX<R>* B, int64_t ldb, bool herm, RandSrc& rs) {
  const CX<R> one(1), mone(-1), zero(0);
  const int64_t lm = std::max<int64_t>(m, 1), ln = std::max<int64_t>(n, 1);
  return csnorm_loop<R>(
      ctx, o, m, n, herm, rs,
      [&](const CX<R>* x, CX<R>* y) {
        cgemm<R>(ctx, 'n', 'n', m, 1, n, one, A, lda, x, ln, zero, y, lm);
        cgemm<R>(ctx, 'n', 'n', m, 1, n, mone, B, ldb, x, ln, one, y, lm);
      },
      [&](const CX<R>* y, CX<R>* x) {
        cgemm<R>(ctx, 'c', 'n', n, 1, m, one, A, lda, y, lm, zero, x, ln);
        cgemm<R>(ctx, 'c', 'n', n, 1, m, mone, B, ldb, y, lm, one, x, ln);
      });
}

// the middle factor of CUR(A, U) (src/cur.jl:85-115): the pseudo-inverse of
// W = A[rows, cols] = Uw diag(S) Vw^H as the PartialSVD (Vw, 1 ./ S, Uw^H)
template <typename R>
lra_psvd* ccur_middle(lra_ctx* ctx, int64_t m, int64_t n, const void* A, int64_t lda, int64_t k,
                      const int64_t* rows, const int64_t* cols, int dtype) {
  const int64_t kk = std::max<int64_t>(k, 1);
  DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
  CX<R>* W = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  if (k > 0) {
    int64_t* dr = ctx->arena.alloc_n<int64_t>(kk);
    int64_t* dc = ctx->arena.alloc_n<int64_t>(kk);
    LRA_CUDA(cudaMemcpyAsync(dr, rows, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    LRA_CUDA(cudaMemcpyAsync(dc, cols, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    CX<R>* Ac = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(m, 1) * kk);
    gather_cols<CX<R>>(ctx, m, k, dA.p, dA.ld, dc, Ac, std::max<int64_t>(m, 1));
    gather_rows<CX<R>>(ctx, k, k, Ac, std::max<int64_t>(m, 1), dr, W, kk);
  }
  CX<R>* Uw = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  CX<R>* Vw = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  std::vector<R> hS = csmall_svd<R>(ctx, k, W, kk, Uw, Vw);
  lra_psvd* r = static_cast<lra_psvd*>(hmalloc(sizeof(lra_psvd)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->m = k;
  r->n = k;
  r->k = k;
  r->S = hmalloc(sizeof(R) * kk);
  for (int64_t i = 0; i < k; ++i) static_cast<R*>(r->S)[i] = hS[i] > R(0) ? R(1) / hS[i] : R(0);
  CX<R>* Uh = ctx->arena.alloc_n<CX<R>>((size_t)kk * kk);
  cadjoint<R>(ctx, k, k, Uw, kk, Uh, kk);
  r->U = hmalloc(sizeof(CX<R>) * (size_t)kk * kk);
  r->Vt = hmalloc(sizeof(CX<R>) * (size_t)kk * kk);
  to_host(ctx, r->U, Vw, (size_t)k * k);
  to_host(ctx, r->Vt, Uh, (size_t)k * k);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}
}  // namespace
}  // namespace lra

extern "C" {

const char* lra_status_string(int s) {
  switch (s) {
    case LRA_OK: return "ok";
    case LRA_EINVAL: return "invalid argument";
    case LRA_EDIM: return "dimension mismatch";
    case LRA_ENOMEM: return "out of memory";
    case LRA_ETIMEDOUT: return "device wait timed out";
    case LRA_ENONFINITE: return "non-finite input";
    case LRA_ECUDA: return "CUDA error";
    case LRA_ERAND: return "random stream exhausted";
    case LRA_ENOTSUP: return "not supported";
    case LRA_ENOTHERM: return "matrix must be Hermitian";
    case LRA_EBUSY: return "busy";
    default: return "unknown status";
  }
}

int lra_ctx_create(int device, lra_ctx** out) {
  if (!out) return LRA_EINVAL;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return LRA_ECUDA;
  }
  if (device < 0 || device >= count) return LRA_EINVAL;
  lra_ctx* c = new (std::nothrow) lra_ctx();
  if (!c) return LRA_ENOMEM;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return LRA_ECUDA;
  }
  c->own_stream = true;
  load_tuning(&c->tuning, &c->tuning_source);
  *out = c;
  return LRA_OK;
}

int lra_ctx_set_tuning(lra_ctx* ctx, const char* key, int64_t index, int64_t value) {
  if (!ctx) return LRA_EINVAL;
  if (!key || !set_tuning(&ctx->tuning, key, index, value)) {
    ctx->last_error = "unknown tuning key or value out of range";
    return LRA_EINVAL;
  }
  return LRA_OK;
}

int lra_ctx_get_tuning(const lra_ctx* ctx, char* buf, int64_t len) {
  if (!ctx) return LRA_EINVAL;
  const std::string s = "# source: " + ctx->tuning_source + "\n" + tuning_text(ctx->tuning);
  if (!buf || len <= 0) return (int)s.size() + 1;
  std::snprintf(buf, (size_t)len, "%s", s.c_str());
  return (int)s.size() + 1;
}

void lra_ctx_destroy(lra_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  for (int i = 0; i < lra_ctx::kAux; ++i) {
    if (ctx->aux[i]) {
      cudaStreamSynchronize(ctx->aux[i]);
      cudaStreamDestroy(ctx->aux[i]);
    }
  }
  for (cudaEvent_t e : ctx->aux_ev)
    if (e) cudaEventDestroy(e);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  if (ctx->dev_err) cudaFree(ctx->dev_err);
  delete ctx;
}

int lra_ctx_set_stream(lra_ctx* ctx, void* stream) {
  if (!ctx) return LRA_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  ctx->stream = static_cast<cudaStream_t>(stream);
  ctx->own_stream = false;
  return LRA_OK;
}

const char* lra_last_error(const lra_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

int64_t lra_ctx_launches(const lra_ctx* ctx) { return ctx ? ctx->launches : 0; }

int64_t lra_ctx_kernel_launches(const lra_ctx* ctx, const char* name) {
  if (!ctx || !name) return 0;
  const auto it = ctx->launches_by_name.find(name);
  return it == ctx->launches_by_name.end() ? 0 : it->second;
}

int lra_ctx_stage_ms(const lra_ctx* ctx, double out[4]) {
  if (!ctx || !out) return LRA_EINVAL;
  for (int i = 0; i < 4; ++i) out[i] = ctx->stage_ms[i];
  return LRA_OK;
}

int lra_ctx_set_wait_limit(lra_ctx* ctx, int64_t ns) {
  if (!ctx) return LRA_EINVAL;
  if (ns < 0) {
    ctx->last_error = "wait limit < 0";
    return LRA_EINVAL;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess || cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
      set_wait_limit_qr((uint64_t)ns) != cudaSuccess || set_wait_limit_dense((uint64_t)ns) != cudaSuccess ||
      set_wait_limit_tc((uint64_t)ns) != cudaSuccess) {
    ctx->last_error = cudaGetErrorString(cudaGetLastError());
    return LRA_ECUDA;
  }
  ctx->last_error.clear();
  return LRA_OK;
}

int lra_ctx_probe_wait(lra_ctx* ctx) {
  int returned = 0, err = 0;
  const int st = guarded(ctx, [&] { err = probe_grid_wait(ctx, &returned); });
  if (st != LRA_OK) return st;
  if (err == 4 && returned == 2) {
    ctx->last_error = "probe: the grid barrier's bounded wait ran out and both CTAs returned";
    return LRA_ETIMEDOUT;
  }
  char msg[128];
  std::snprintf(msg, sizeof msg, "probe: unexpected barrier state (err %d, %d CTAs returned)", err, returned);
  ctx->last_error = msg;
  return LRA_ECUDA;
}

int lra_opts_init(lra_opts* o, int dtype) {
  if (!o) return LRA_EINVAL;
  if (dtype != LRA_F32 && dtype != LRA_F64 && dtype != LRA_C32 && dtype != LRA_C64) return LRA_EINVAL;
  std::memset(o, 0, sizeof *o);
  // eps(real(T)) (src/LowRankApprox.jl:96-119)
  const double eps = (dtype == LRA_F64 || dtype == LRA_C64) ? 2.220446049250313e-16 : 1.1920928955078125e-07;
  o->atol = 0;
  o->maxdet_niter = -1;
  o->maxdet_tol = -1;
  o->nb = 32;
  o->pheig_orthtol = std::sqrt(eps);
  o->pqrfact_retval = LRA_RET_Q | LRA_RET_R;
  o->rank = -1;
  o->rtol = 5 * eps;
  o->sketch = LRA_SKETCH_RANDN;
  o->sketch_randn_niter = 0;
  o->sketchfact_adap = 1;
  o->verb = 1;
  o->sketchfact_randn_samp[0] = 1;
  o->sketchfact_randn_samp[1] = 8;
  o->sketchfact_srft_samp[0] = 1;
  o->sketchfact_srft_samp[1] = 8;
  o->sketchfact_sub_samp[0] = 4;
  o->sketchfact_sub_samp[1] = 8;
  o->snorm_niter = 32;
  o->precision = LRA_PREC_NATIVE;
  o->check_finite = 1;
  o->seed = 0x4c5241ull;
  return LRA_OK;
}

int lra_chkopts(const lra_opts* o) {
  try {
    chkopts(o);
    return LRA_OK;
  } catch (const lra::Error& e) {
    return e.status;
  }
}

int lra_sketch(lra_ctx* ctx, int dtype, char side, char trans, int64_t m, int64_t n, const void* A, int64_t lda,
               int64_t order, const lra_opts* opts, const lra_rand* rand, void* B, int64_t ldb) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (order < 0) fail(LRA_EINVAL, "order");
    const char t = chktrans(trans);
    if (side != 'l' && side != 'r' && side != 'L' && side != 'R') fail(LRA_EINVAL, "side");
    lra_opts o = *opts;
    if (o.sketch == LRA_SKETCH_NONE) o.sketch = LRA_SKETCH_RANDN;  // src/sketch.jl:68-74
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        const bool left = side == 'l' || side == 'L';
        const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
        const int64_t rows = left ? order : M, cols = left ? N : order;
        if (ldb < std::max<int64_t>(rows, 1)) fail(LRA_EDIM, "ldb");
        CX<R>* Bd = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(rows, 1) * std::max<int64_t>(cols, 1));
        make_sketch_c<R>(ctx, o, t, M, N, dA.p, dA.ld, order, rs, Bd, !left);
        if (rows > 0 && cols > 0)
          LRA_CUDA(cudaMemcpy2DAsync(B, ldb * sizeof(CX<R>), Bd, std::max<int64_t>(rows, 1) * sizeof(CX<R>),
                                     rows * sizeof(CX<R>), cols,
                                     is_dev(B) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      // right sketches A S are the transposes of left sketches S^T A^T
      const bool left = side == 'l' || side == 'L';
      const char tt = left ? t : (t == 'n' ? 'c' : 'n');
      const int64_t M = tt == 'n' ? m : n, N = tt == 'n' ? n : m;
      T* Bd = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(order, 1) * std::max<int64_t>(N, 1));
      make_sketch<T>(ctx, o, tt, M, N, dA.p, dA.ld, order, rs, Bd, dtype, nullptr, !left);
      const int64_t rows = left ? order : N, cols = left ? N : order;
      if (ldb < std::max<int64_t>(rows, 1)) fail(LRA_EDIM, "ldb");
      T* src = Bd;
      if (!left) {
        src = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(rows * cols, 1));
        transpose(ctx, order, N, Bd, std::max<int64_t>(order, 1), src, std::max<int64_t>(rows, 1));
      }
      if (rows > 0 && cols > 0)
        LRA_CUDA(cudaMemcpy2DAsync(B, ldb * sizeof(T), src, rows * sizeof(T), rows * sizeof(T), cols,
                                   is_dev(B) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
    });
  });
}

int lra_geqp3_adap(lra_ctx* ctx, int dtype, int64_t m, int64_t n, void* B, int64_t ldb, int64_t* jpvt, void* tau,
                   const lra_opts* opts, int64_t* k) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (!k) fail(LRA_EINVAL, "k is NULL");
    if (m > 0 && n > 0 && (!is_dev(B) || !is_dev(jpvt) || !is_dev(tau)))
      fail(LRA_EINVAL, "lra_geqp3_adap works on device buffers");
    if (ldb < std::max<int64_t>(1, m)) fail(LRA_EDIM, "ldb");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        const int64_t l = std::min(m, n);
        const int64_t kmax = (opts->rank < 0 || opts->rank > l) ? l : opts->rank;
        *k = cgeqp3<R>(ctx, m, n, static_cast<CX<R>*>(B), ldb, jpvt, static_cast<CX<R>*>(tau), kmax, opts->nb,
                       opts->atol, opts->rtol, true);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      const int64_t l = std::min(m, n);
      const int64_t kmax = (opts->rank < 0 || opts->rank > l) ? l : opts->rank;
      *k = geqp3_adap<T>(ctx, m, n, static_cast<T*>(B), ldb, jpvt, static_cast<T*>(tau), kmax, opts->nb,
                         opts->atol, opts->rtol, true);
    });
  });
}

int lra_geqp3_adap_noalloc(lra_ctx* ctx, int dtype, int64_t m, int64_t n, void* B, int64_t ldb, int64_t* jpvt,
                           void* tau, const lra_opts* opts, int64_t* k) {
  // No arena reset and no workspace: this entry point allocates nothing.
  if (!ctx) return LRA_EINVAL;
  try {
    chkopts(opts);
    check_dims(m, n);
    if (!k) fail(LRA_EINVAL, "k is NULL");
    if (n > noalloc_max_cols())
      fail(LRA_EINVAL, "lra_geqp3_adap_noalloc: n = %lld exceeds its limit of %lld columns", (long long)n,
           (long long)noalloc_max_cols());
    if (m <= 0 || n <= 0) fail(LRA_EINVAL, "lra_geqp3_adap_noalloc: empty matrix");
    if (!is_dev(B) || !is_dev(jpvt) || !is_dev(tau)) fail(LRA_EINVAL, "lra_geqp3_adap_noalloc works on device buffers");
    if (ldb < m) fail(LRA_EDIM, "ldb");
    LRA_CUDA(cudaSetDevice(ctx->device));
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      const int64_t l = std::min(m, n);
      const int64_t kmax = (opts->rank < 0 || opts->rank > l) ? l : opts->rank;
      *k = geqp3_adap_noalloc<T>(ctx, m, n, static_cast<T*>(B), ldb, jpvt, static_cast<T*>(tau), kmax, opts->nb,
                                 opts->atol, opts->rtol);
    });
    ctx->last_error.clear();
    return LRA_OK;
  } catch (const lra::Error& e) {
    ctx->gemm_tc = false;
    ctx->mixed_rtol = 0;
    ctx->last_error = e.msg;
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    return e.status;
  } catch (const std::bad_alloc&) {
    ctx->last_error = "host allocation failed";
    return LRA_ENOMEM;
  } catch (...) {
    ctx->last_error = "unexpected exception";
    return LRA_ECUDA;
  }
}

int lra_rand_gauss(lra_ctx* ctx, uint64_t seed, uint64_t counter, int64_t n, double* out) {
  return guarded(ctx, [&] {
    if (n < 0) fail(LRA_EINVAL, "n < 0");
    if (n == 0) return;
    if (!out) fail(LRA_EINVAL, "out is NULL");
    double* d = is_dev(out) ? out : ctx->arena.alloc_n<double>(n);
    sketch_philox<double>(ctx, seed, counter, n, d);
    if (d != out)
      LRA_CUDA(cudaMemcpyAsync(out, d, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  });
}

int lra_dgemm(lra_ctx* ctx, int precision, char transa, char transb, int64_t m, int64_t n, int64_t k,
              double alpha, const double* A, int64_t lda, const double* B, int64_t ldb, double beta, double* C,
              int64_t ldc) {
  return guarded(ctx, [&] {
    auto tr = [](char t) { return t == 'n' || t == 'N' || t == 't' || t == 'T' || t == 'c' || t == 'C'; };
    if (!tr(transa) || !tr(transb)) fail(LRA_EINVAL, "trans must be 'n' or 't'");
    if (m < 0 || n < 0 || k < 0) fail(LRA_EDIM, "negative dimension");
    if (precision != LRA_PREC_NATIVE && precision != LRA_PREC_MIXED) fail(LRA_EINVAL, "precision");
    if (m == 0 || n == 0) return;
    const bool ta = transa != 'n' && transa != 'N', tb = transb != 'n' && transb != 'N';
    if (lda < std::max<int64_t>(1, ta ? k : m) || ldb < std::max<int64_t>(1, tb ? n : k) ||
        ldc < std::max<int64_t>(1, m))
      fail(LRA_EDIM, "leading dimension too small");
    if ((k > 0 && (!is_dev(A) || !is_dev(B))) || !is_dev(C)) fail(LRA_EINVAL, "lra_dgemm takes device arrays");
    if (precision == LRA_PREC_MIXED && k > 0)
      tc_gemm(ctx, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
    else
      gemm<double>(ctx, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  });
}

int lra_idfact(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n, const void* A, int64_t lda,
               const lra_opts* opts, const lra_rand* rand, lra_id** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    const char t = chktrans(trans);
    lra_opts o = *opts;
    o.pqrfact_retval = LRA_RET_T;  // src/id.jl:437
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        CFact<R> F = cid_core<R>(ctx, o, t, m, n, dA, rs, true);
        *out = cpack_id<R>(ctx, F, dtype);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      Fact<T> F = id_core<T>(ctx, o, t, m, n, dA, rs, dtype, true);
      *out = pack_id<T>(ctx, F, dtype);
    });
  });
}

int lra_sketchfact(lra_ctx* ctx, int dtype, char side, char trans, int64_t m, int64_t n, const void* A,
                   int64_t lda, const lra_opts* opts, const lra_rand* rand, lra_pqr** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    const char t = chktrans(trans);
    if (side != 'l' && side != 'L' && side != 'r' && side != 'R') fail(LRA_EINVAL, "side");
    const bool left = side == 'l' || side == 'L';
    lra_opts o = *opts;
    if (o.sketch == LRA_SKETCH_NONE) o.sketch = LRA_SKETCH_RANDN;
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        *out = csketchfact<R>(ctx, o, side, t, m, n, dA, rs, dtype);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      const int64_t Mo = t == 'n' ? m : n, No = t == 'n' ? n : m;
      // left: the pivoted QR of S op(A) (columns of op(A)); right: of op(A) S
      Fact<T> F = left ? sketchfact_dev<T>(ctx, o, t, Mo, No, dA.p, dA.ld, rs, dtype)
                       : sketchfact_right_dev<T>(ctx, o, t, Mo, No, dA.p, dA.ld, rs, dtype);
      const int64_t N = F.N;
      const bool rq = o.pqrfact_retval & LRA_RET_Q, rr = o.pqrfact_retval & LRA_RET_R,
                 rt = o.pqrfact_retval & LRA_RET_T;
      postproc_t<T>(ctx, o, F, rt);
      lra_pqr* r = static_cast<lra_pqr*>(hmalloc(sizeof(lra_pqr)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->m = F.order;
      r->n = N;
      r->k = F.k;
      r->p = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(N, 1)));
      to_host(ctx, r->p, F.jpvt, N);
      const int64_t k = F.k;
      if (rr) {
        T* R = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * N, 1));
        if (F.r1) {
          // after maxdet swaps: R = [R1 | R1 T] with R1 re-factored (src/pqr.jl:469-474)
          result_r11<T>(ctx, F, R);
          if (N > k) gemm<T>(ctx, 'n', 'n', k, N - k, k, T(1), R, k, F.T_, k, T(0), R + k * k, k);
        } else {
          copy_matrix(ctx, k, N, F.B, F.ld, R, std::max<int64_t>(k, 1));
          zero_lower(ctx, k, N, R, std::max<int64_t>(k, 1));
        }
        r->R = hmalloc(sizeof(T) * std::max<int64_t>(k * N, 1));
        to_host(ctx, r->R, R, (size_t)k * N);
        r->retval |= LRA_RET_R;
      }
      if (rt) {
        r->T = hmalloc(sizeof(T) * std::max<int64_t>(k * (N - k), 1));
        if (k > 0 && N > k) to_host(ctx, r->T, F.T_, (size_t)k * (N - k));
        r->retval |= LRA_RET_T;
      }
      if (rq) {
        orgqr(ctx, F.order, k, F.B, F.ld, F.tau);
        maxdet_rotate_q<T>(ctx, F, F.order, F.B, F.ld);
        r->Q = hmalloc(sizeof(T) * std::max<int64_t>(F.order * k, 1));
        if (k > 0)
          LRA_CUDA(cudaMemcpy2DAsync(r->Q, F.order * sizeof(T), F.B, F.ld * sizeof(T), F.order * sizeof(T), k,
                                     cudaMemcpyDeviceToHost, ctx->stream));
        r->retval |= LRA_RET_Q;
      }
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      *out = r;
    });
  });
}

int lra_prange(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n, const void* A, int64_t lda,
               const lra_opts* opts, const lra_rand* rand, lra_pqr** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    char t = (trans == 'b' || trans == 'B') ? 'b' : chktrans(trans);  // prange_chktrans, src/prange.jl:79-80
    const lra_opts& o = *opts;
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        *out = cprange<R>(ctx, o, t, m, n, dA, rs, dtype);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      if (t == 'b') {
        if (m != n) fail(LRA_EDIM, "prange(:b): the matrix must be square");
        if (is_symmetric(ctx, n, dA.p, dA.ld)) t = 'n';  // src/prange.jl:24
      }
      // one side's factorization (src/prange.jl:26-31, 47-52): the pivoted QR
      // of op(A) itself (sketch :none) or of the right sketch op(A) S; Q
      // (M x k, ld M) replaces the reflectors, and R11 is kept on request.
      // With maxdet_tol >= 0 the :b form asks for "qr" (src/prange.jl:25), so
      // the swaps re-factor R1 and rotate Q; with Q alone (:n, :c) they
      // leave Q as it is (maxdet_swapcols!, src/pqr.jl:467-468) and are
      // skipped.
      auto side_q = [&](char tr, int64_t& k, T** R11) -> T* {
        const int64_t M = tr == 'n' ? m : n, N = tr == 'n' ? n : m;
        Fact<T> F;
        if (o.sketch == LRA_SKETCH_NONE) {
          T* B = dense_op(ctx, tr, m, n, dA);
          F = pqr_backend_dev<T>(ctx, o, B, M, N, M);
        } else {
          F = sketchfact_right_dev<T>(ctx, o, tr, M, N, dA.p, dA.ld, rs, dtype);
        }
        if (R11 && o.maxdet_tol >= 0) {
          lra_opts oq = o;
          oq.pqrfact_retval = LRA_RET_Q | LRA_RET_R;
          postproc_t<T>(ctx, oq, F, false);
        }
        k = F.k;
        const int64_t kk = std::max<int64_t>(k, 1);
        if (R11) {
          *R11 = ctx->arena.alloc_n<T>((size_t)kk * kk);
          result_r11<T>(ctx, F, *R11);
        }
        orgqr(ctx, M, k, F.B, F.ld, F.tau);
        maxdet_rotate_q<T>(ctx, F, M, F.B, F.ld);
        return F.B;
      };
      const int64_t M = t == 'c' ? n : m;
      int64_t k = 0;
      T* Q = nullptr;
      if (t == 'b') {
        // src/prange.jl:32-45: the row and column bases scaled by their
        // R11, side by side, and the Q of their pivoted QR
        int64_t kr = 0, kc = 0;
        T *Rr = nullptr, *Rc = nullptr;
        T* Qr = side_q('c', kr, &Rr);
        T* Qc = side_q('n', kc, &Rc);
        const int64_t kb = kr + kc;
        T* Bc = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(M, 1) * std::max<int64_t>(kb, 1));
        if (kr > 0) gemm<T>(ctx, 'n', 'n', M, kr, kr, T(1), Qr, M, Rr, kr, T(0), Bc, M);
        if (kc > 0) gemm<T>(ctx, 'n', 'n', M, kc, kc, T(1), Qc, M, Rc, kc, T(0), Bc + kr * M, M);
        Fact<T> F = pqr_backend_dev<T>(ctx, o, Bc, M, kb, M);
        k = F.k;
        orgqr(ctx, M, k, F.B, F.ld, F.tau);
        Q = F.B;
      } else if (o.sketch == LRA_SKETCH_SUB) {
        // prange_sub (src/prange.jl:63-77): the skeleton columns of op(A)
        // from the left sketch, made orthonormal (orthcols!, src/util.jl)
        const int64_t N = t == 'n' ? n : m;
        Fact<T> F = sketchfact_dev<T>(ctx, o, t, M, N, dA.p, dA.ld, rs, dtype);
        if (o.maxdet_tol >= 0) {
          // the swaps move the skeleton columns prange_sub takes
          lra_opts oq = o;
          oq.pqrfact_retval = LRA_RET_Q;
          postproc_t<T>(ctx, oq, F, false);
        }
        const int64_t kc = F.k, kq = std::min(M, kc);
        Q = getcols<T>(ctx, t, m, n, dA, F.jpvt, kc);
        int64_t* jp = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(kc, 1));
        T* tau = ctx->arena.alloc_n<T>(std::max<int64_t>(kq, 1));
        if (kq > 0) {
          geqp3_adap<T>(ctx, M, kc, Q, std::max<int64_t>(M, 1), jp, tau, kq, 32, -1.0, 0.0, false);
          orgqr(ctx, M, kq, Q, std::max<int64_t>(M, 1), tau);
        }
        k = kq;
      } else {
        Q = side_q(t, k, nullptr);
      }
      lra_pqr* r = static_cast<lra_pqr*>(hmalloc(sizeof(lra_pqr)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->m = M;
      r->n = k;
      r->k = k;
      r->p = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(k, 1)));
      for (int64_t i = 0; i < k; ++i) r->p[i] = i + 1;
      r->Q = hmalloc(sizeof(T) * std::max<int64_t>(M * k, 1));
      if (k > 0 && M > 0)
        LRA_CUDA(cudaMemcpy2DAsync(r->Q, M * sizeof(T), Q, M * sizeof(T), M * sizeof(T), k, cudaMemcpyDeviceToHost,
                                   ctx->stream));
      r->retval = LRA_RET_Q;
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      *out = r;
    });
  });
}

int lra_pqrfact(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n, const void* A, int64_t lda,
                const lra_opts* opts, const lra_rand* rand, lra_pqr** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    const char t = chktrans(trans);
    const lra_opts& o = *opts;
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        *out = cpqrfact<R>(ctx, o, t, m, n, dA, rs, dtype);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
      const bool rq = o.pqrfact_retval & LRA_RET_Q, rr = o.pqrfact_retval & LRA_RET_R,
                 rt = o.pqrfact_retval & LRA_RET_T;
      lra_pqr* r = static_cast<lra_pqr*>(hmalloc(sizeof(lra_pqr)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->m = M;
      r->n = N;
      r->p = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<int64_t>(N, 1)));
      try {
        T* Qd = nullptr;  // M x k, ld = M
        T* R11 = nullptr;  // k x k upper, ld = k
        Fact<T> F;
        if (o.sketch == LRA_SKETCH_NONE) {
          // pqrfact_none (src/pqr.jl:323-327): pivoted QR of op(A) itself
          lra_opts oo = o;
          T* B = dense_op(ctx, t, m, n, dA);
          F = pqr_backend_dev<T>(ctx, oo, B, M, N, M);
          postproc_t<T>(ctx, oo, F, rt || rr);
          const int64_t k = F.k;
          R11 = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * k, 1));
          result_r11<T>(ctx, F, R11);
          if (rq) {
            orgqr(ctx, M, k, F.B, F.ld, F.tau);
            maxdet_rotate_q<T>(ctx, F, M, F.B, F.ld);
            Qd = F.B;
          }
        } else {
          lra_opts oi = o;
          oi.pqrfact_retval = LRA_RET_T;
          F = id_core<T>(ctx, oi, t, m, n, dA, rs, dtype, true);
          const int64_t k = F.k;
          T* Ask = getcols<T>(ctx, t, m, n, dA, F.jpvt, k);
          R11 = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * k, 1));
          Stage st(ctx, 3);
          if (skeleton_qr<T>(ctx, F, M, Ask, R11, dtype)) {
            Qd = Ask;  // Cholesky QR preconditioned by the sketch's R11
          } else {
            Ask = getcols<T>(ctx, t, m, n, dA, F.jpvt, k);
            int64_t* jp = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(k, 1));
            T* tau = ctx->arena.alloc_n<T>(std::max<int64_t>(k, 1));
            geqp3_adap<T>(ctx, M, k, Ask, std::max<int64_t>(M, 1), jp, tau, k, 32, -1.0, 0.0, false);
            copy_matrix(ctx, k, k, Ask, std::max<int64_t>(M, 1), R11, std::max<int64_t>(k, 1));
            if (rq) {
              orgqr(ctx, M, k, Ask, std::max<int64_t>(M, 1), tau);
              Qd = Ask;
            }
          }
        }
        const int64_t k = F.k;
        r->k = k;
        zero_lower(ctx, k, k, R11, std::max<int64_t>(k, 1));
        to_host(ctx, r->p, F.jpvt, N);
        if (rq) {
          r->Q = hmalloc(sizeof(T) * std::max<int64_t>(M * k, 1));
          if (k > 0 && M > 0)
            LRA_CUDA(cudaMemcpy2DAsync(r->Q, M * sizeof(T), Qd, (o.sketch == LRA_SKETCH_NONE ? F.ld : M) * sizeof(T),
                                       M * sizeof(T), k, cudaMemcpyDeviceToHost, ctx->stream));
          r->retval |= LRA_RET_Q;
        }
        if (rr) {
          // R = [R11 | R11 T] (pqrr, src/pqr.jl:330-340)
          T* R = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * N, 1));
          copy_matrix(ctx, k, k, R11, std::max<int64_t>(k, 1), R, std::max<int64_t>(k, 1));
          if (k > 0 && N > k)
            gemm<T>(ctx, 'n', 'n', k, N - k, k, T(1), R11, k, F.T_, k, T(0), R + k * k, k);
          r->R = hmalloc(sizeof(T) * std::max<int64_t>(k * N, 1));
          to_host(ctx, r->R, R, (size_t)k * N);
          r->retval |= LRA_RET_R;
        }
        if (rt) {
          r->T = hmalloc(sizeof(T) * std::max<int64_t>(k * (N - k), 1));
          if (k > 0 && N > k) to_host(ctx, r->T, F.T_, (size_t)k * (N - k));
          r->retval |= LRA_RET_T;
        }
        LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      } catch (...) {
        lra_pqr_free(r);
        throw;
      }
      *out = r;
    });
  });
}

}  // extern "C"

// ======================================================================================
// post-processed factorizations: psvd, pheig, cur; norms; batches
// ======================================================================================

namespace lra {
namespace {

// SVD of the k x N device matrix W (k <= N): W = U diag(S) Vt with U k x k,
// S descending, V (N x k) returned as the Householder reflectors of W^T
// (Q2, tau2) plus V' (k x k) so that Vfull = Q2 [V'; 0].
template <typename T>
struct SmallSvd {
  T* U;     // k x k
  T* S;     // k (device)
  T* Vp;    // k x k
  T* Q2;    // N x k reflectors
  T* tau2;  // k
  std::vector<T> hS;
};

template <typename T>
SmallSvd<T> svd_wide(lra_ctx* ctx, int64_t k, int64_t N, const T* W, int64_t ldw) {
  SmallSvd<T> r;
  r.Q2 = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(N * k, 1));
  transpose(ctx, k, N, W, ldw, r.Q2, std::max<int64_t>(N, 1));
  int64_t* jp = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(k, 1));
  r.tau2 = ctx->arena.alloc_n<T>(std::max<int64_t>(k, 1));
  geqp3_adap<T>(ctx, N, k, r.Q2, std::max<int64_t>(N, 1), jp, r.tau2, k, 32, -1.0, 0.0, false);
  // X = R2^T (k x k)
  T* R2 = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * k, 1));
  copy_matrix(ctx, k, k, r.Q2, std::max<int64_t>(N, 1), R2, std::max<int64_t>(k, 1));
  zero_lower(ctx, k, k, R2, std::max<int64_t>(k, 1));
  r.U = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * k, 1));
  transpose(ctx, k, k, R2, std::max<int64_t>(k, 1), r.U, std::max<int64_t>(k, 1));
  r.Vp = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * k, 1));
  r.S = ctx->arena.alloc_n<T>(std::max<int64_t>(k, 1));
  jacobi_svd<T>(ctx, k, r.U, std::max<int64_t>(k, 1), r.Vp, std::max<int64_t>(k, 1), r.S);
  div_cols(ctx, k, k, r.U, std::max<int64_t>(k, 1), r.S);
  // sort descending (gesdd order) and permute U, V' columns
  r.hS.resize(k);
  to_host(ctx, r.hS.data(), r.S, k);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> ord(k);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return r.hS[a] > r.hS[b]; });
  bool sorted = true;
  for (int64_t i = 0; i < k; ++i) sorted &= ord[i] == i;
  if (!sorted && k > 0) {
    std::vector<int64_t> ord1(k);
    std::vector<T> s2(k);
    for (int64_t i = 0; i < k; ++i) {
      ord1[i] = ord[i] + 1;
      s2[i] = r.hS[ord[i]];
    }
    r.hS = s2;
    int64_t* dord = ctx->arena.alloc_n<int64_t>(k);
    LRA_CUDA(cudaMemcpyAsync(dord, ord1.data(), k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    T* tmp = ctx->arena.alloc_n<T>((size_t)k * k);
    gather_cols(ctx, k, k, r.U, k, dord, tmp, k);
    copy_matrix(ctx, k, k, tmp, k, r.U, k);
    gather_cols(ctx, k, k, r.Vp, k, dord, tmp, k);
    copy_matrix(ctx, k, k, tmp, k, r.Vp, k);
    LRA_CUDA(cudaMemcpyAsync(r.S, r.hS.data(), k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return r;
}

int64_t psvdrank(const std::vector<double>& s, const lra_opts& o) {
  const int64_t k = (int64_t)s.size();
  if (k == 0) return 0;
  const double ptol = std::max(o.atol, o.rtol * s[0]);
  for (int64_t i = 1; i < k; ++i)
    if (s[i] <= ptol) return i;
  return k;
}

// psvdfact for op(A) tall-or-square (M >= N in the reference's branch)
template <typename T>
lra_psvd* psvd_dev(lra_ctx* ctx, const lra_opts& o, char trans, int64_t m, int64_t n, const DMat<T>& dA,
                   RandSrc& rs, int dtype, bool vals_only) {
  const int64_t M = trans == 'n' ? m : n, N = trans == 'n' ? n : m;
  lra_opts oi = o;
  oi.pqrfact_retval = LRA_RET_T;
  Fact<T> F = id_core<T>(ctx, oi, trans, m, n, dA, rs, dtype, true);
  const int64_t k = F.k;
  Stage st(ctx, 3);
  const int64_t ldq = std::max<int64_t>(M, 1), ldk = std::max<int64_t>(k, 1);
  // LRA_TRACE: the post-processing's phases (each waits for the device)
  const bool tr = trace_on();
  auto tnow = [] { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double tl = tr ? tnow() : 0;
  auto tmark = [&](const char* what) {
    if (!tr) return;
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    const double t = tnow();
    std::fprintf(stderr, "[lra] psvd post k=%lld %s %.3f ms\n", (long long)k, what, t - tl);
    tl = t;
  };
  {
    // GEMM-shaped route: A[:, sk] = Q R_A, V^T = Q_v R_v, SVD(R_A R_v^T)
    const ArenaMark mk = ctx->arena.mark();
    T* Q = getcols<T>(ctx, trans, m, n, dA, F.jpvt, k);
    T* RA = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
    T* Rv = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
    tmark("gather");
    const bool ok = skeleton_qr_v<T>(ctx, F, M, Q, RA, N - k, Rv, dtype);
    tmark("skeleton cholesky qr, chol(I + T T')");
    if (ok) {
      T* Mm = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      gemm<T>(ctx, 'n', 't', k, k, k, T(1), RA, ldk, Rv, ldk, T(0), Mm, ldk);
      T* UM = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      T* VM = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      T* S = ctx->arena.alloc_n<T>(ldk);
      std::vector<T> hS = small_svd<T>(ctx, k, Mm, UM, VM, S);
      tmark("core svd");
      std::vector<double> sd(hS.begin(), hS.end());
      const int64_t kk = psvdrank(sd, o), lkk = std::max<int64_t>(kk, 1);
      lra_psvd* r = static_cast<lra_psvd*>(hmalloc(sizeof(lra_psvd)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->k = kk;
      r->S = hmalloc(sizeof(T) * lkk);
      std::memcpy(r->S, hS.data(), sizeof(T) * kk);
      if (vals_only) return r;
      // U = Q U_M(:, 1:kk)
      T* U = ctx->arena.alloc_n<T>((size_t)ldq * lkk);
      gemm<T>(ctx, 'n', 'n', M, kk, k, T(1), Q, ldq, UM, ldk, T(0), U, ldq);
      // Vt = Z^T V,  Z = R_v^{-1} V_M(:, 1:kk):  Vt[:, p] = [Z^T | Z^T T]
      trsm_upper(ctx, k, kk, Rv, ldk, VM, ldk);
      T* Vp = ctx->arena.alloc_n<T>((size_t)lkk * std::max<int64_t>(N, 1));
      transpose(ctx, k, kk, VM, ldk, Vp, lkk);
      if (N > k) gemm<T>(ctx, 't', 'n', kk, N - k, k, T(1), VM, ldk, F.T_, ldk, T(0), Vp + k * lkk, lkk);
      T* Vt = ctx->arena.alloc_n<T>((size_t)lkk * std::max<int64_t>(N, 1));
      scatter_cols(ctx, kk, N, Vp, lkk, F.jpvt, Vt, lkk);
      tmark("factors");
      r->U = hmalloc(sizeof(T) * std::max<int64_t>(M * kk, 1));
      r->Vt = hmalloc(sizeof(T) * std::max<int64_t>(kk * N, 1));
      to_host(ctx, r->U, U, (size_t)M * kk);
      to_host(ctx, r->Vt, Vt, (size_t)kk * N);
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      tmark("to host");
      return r;
    }
    ctx->arena.release(mk);
  }
  // Householder route (the skeleton moved under maxdet, or a Cholesky broke
  // down): Q, R = qr(A[:, sk])
  T* Ask = getcols<T>(ctx, trans, m, n, dA, F.jpvt, k);
  int64_t* jp = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(k, 1));
  T* tau = ctx->arena.alloc_n<T>(std::max<int64_t>(k, 1));
  geqp3_adap<T>(ctx, M, k, Ask, ldq, jp, tau, k, 32, -1.0, 0.0, false);
  T* R = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
  copy_matrix(ctx, k, k, Ask, ldq, R, ldk);
  zero_lower(ctx, k, k, R, ldk);
  // W = R V = [R | R T] P^T  (k x N)
  T* Wp = ctx->arena.alloc_n<T>((size_t)ldk * std::max<int64_t>(N, 1));
  copy_matrix(ctx, k, k, R, ldk, Wp, ldk);
  if (k > 0 && N > k) gemm<T>(ctx, 'n', 'n', k, N - k, k, T(1), R, ldk, F.T_, ldk, T(0), Wp + k * ldk, ldk);
  T* W = ctx->arena.alloc_n<T>((size_t)ldk * std::max<int64_t>(N, 1));
  scatter_cols(ctx, k, N, Wp, ldk, F.jpvt, W, ldk);
  SmallSvd<T> sv = svd_wide<T>(ctx, k, N, W, ldk);
  std::vector<double> sd(sv.hS.begin(), sv.hS.end());
  const int64_t kk = psvdrank(sd, o);
  lra_psvd* r = static_cast<lra_psvd*>(hmalloc(sizeof(lra_psvd)));
  std::memset(r, 0, sizeof *r);
  r->dtype = dtype;
  r->k = kk;
  r->S = hmalloc(sizeof(T) * std::max<int64_t>(kk, 1));
  std::memcpy(r->S, sv.hS.data(), sizeof(T) * kk);
  if (vals_only) return r;
  // U = Q [U~(:, 1:kk); 0]  (M x kk)
  T* U = ctx->arena.alloc_n<T>((size_t)ldq * std::max<int64_t>(kk, 1));
  set_zero(ctx, U, ldq * std::max<int64_t>(kk, 1));
  copy_matrix(ctx, k, kk, sv.U, ldk, U, ldq);
  apply_q<T>(ctx, 'n', M, k, Ask, ldq, tau, U, ldq, kk);
  // V~ = Q2 [V'(:, 1:kk); 0]  (N x kk); Vt = V~^T
  const int64_t ldn = std::max<int64_t>(N, 1);
  T* Vf = ctx->arena.alloc_n<T>((size_t)ldn * std::max<int64_t>(kk, 1));
  set_zero(ctx, Vf, ldn * std::max<int64_t>(kk, 1));
  copy_matrix(ctx, k, kk, sv.Vp, ldk, Vf, ldn);
  apply_q<T>(ctx, 'n', N, k, sv.Q2, ldn, sv.tau2, Vf, ldn, kk);
  r->U = hmalloc(sizeof(T) * std::max<int64_t>(M * kk, 1));
  r->Vt = hmalloc(sizeof(T) * std::max<int64_t>(kk * N, 1));
  T* Vt = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(kk * N, 1));
  transpose(ctx, N, kk, Vf, ldn, Vt, std::max<int64_t>(kk, 1));
  to_host(ctx, r->U, U, (size_t)M * kk);
  to_host(ctx, r->Vt, Vt, (size_t)kk * N);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  return r;
}

// transpose a host matrix (rows x cols, ld = rows) in place into a new buffer
template <typename T>
void* host_transpose(const void* src, int64_t rows, int64_t cols) {
  T* d = static_cast<T*>(hmalloc(sizeof(T) * std::max<int64_t>(rows * cols, 1)));
  const T* s = static_cast<const T*>(src);
  for (int64_t j = 0; j < cols; ++j)
    for (int64_t i = 0; i < rows; ++i) d[j + i * cols] = s[i + j * rows];
  return d;
}

std::pair<int64_t, int64_t> pheigrank(const std::vector<double>& w, const lra_opts& o) {
  const int64_t n = (int64_t)w.size();
  if (n == 0) return {0, 0};
  const double wmax = std::max(std::fabs(w[0]), std::fabs(w[n - 1]));
  // searchsorted(w, 0): first index with w >= 0 .. last index with w <= 0
  int64_t lo = 0;
  while (lo < n && w[lo] < 0) ++lo;
  int64_t hi = lo;
  while (hi < n && w[hi] <= 0) ++hi;
  auto rank1 = [&](std::vector<double> v) {
    int64_t k = (int64_t)v.size();
    k = o.rank >= 0 ? std::min<int64_t>(o.rank, k) : k;
    const double ptol = std::max(o.atol, o.rtol * wmax);
    for (int64_t i = 1; i < k; ++i)
      if (std::fabs(v[i]) <= ptol) return i;
    return k;
  };
  std::vector<double> neg(w.begin(), w.begin() + lo);
  std::vector<double> pos(w.rbegin(), w.rbegin() + (n - hi));
  return {rank1(neg), rank1(pos)};
}

}  // namespace
}  // namespace lra

extern "C" {

int lra_psvdfact(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda, const lra_opts* opts,
                 const lra_rand* rand, int vals_only, lra_psvd** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, *opts, m, n, dA);
        RandSrc rs(ctx, rand, opts->seed);
        *out = cpsvd<R>(ctx, *opts, m, n, dA, rs, dtype, vals_only != 0);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, *opts, m, n, dA);
      RandSrc rs(ctx, rand, opts->seed);
      if (m >= n) {
        lra_psvd* r = psvd_dev<T>(ctx, *opts, 'n', m, n, dA, rs, dtype, vals_only != 0);
        r->m = m;
        r->n = n;
        *out = r;
      } else {
        // the :c branch (src/psvd.jl:256-270) is the same computation on A':
        // A' = U2 S Vt2  =>  A = Vt2' S U2'
        lra_psvd* r = psvd_dev<T>(ctx, *opts, 'c', m, n, dA, rs, dtype, vals_only != 0);
        if (!vals_only) {
          void* U = host_transpose<T>(r->Vt, r->k, m);
          void* Vt = host_transpose<T>(r->U, n, r->k);
          hfree(r->U);
          hfree(r->Vt);
          r->U = U;
          r->Vt = Vt;
        }
        r->m = m;
        r->n = n;
        *out = r;
      }
    });
  });
}

int lra_pheigfact(lra_ctx* ctx, int dtype, int64_t n, const void* A, int64_t lda, const lra_opts* opts,
                  const lra_rand* rand, int vals_only, lra_pheig** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(n, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    const lra_opts& o = *opts;
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, n, n, lda);
        check_input_c<R>(ctx, o, n, n, dA);
        const bool herm = ctx->linop ? ctx->linop->hermitian != 0 : cis_hermitian<R>(ctx, n, dA.p, dA.ld);
        if (!herm) fail(LRA_ENOTHERM, "matrix must be Hermitian");
        RandSrc rs(ctx, rand, o.seed);
        *out = cpheig<R>(ctx, o, n, dA, rs, dtype, vals_only != 0);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, n, n, lda);
      check_input(ctx, o, n, n, dA);
      if (!is_symmetric(ctx, n, dA.p, dA.ld)) fail(LRA_ENOTHERM, "matrix must be Hermitian");
      RandSrc rs(ctx, rand, o.seed);
      lra_opts oi = o;
      oi.pqrfact_retval = LRA_RET_T;
      Fact<T> F = id_core<T>(ctx, oi, 'n', n, n, dA, rs, dtype, true);
      const int64_t k = F.k, ldk = std::max<int64_t>(k, 1), ldn = std::max<int64_t>(n, 1);
      Stage st(ctx, 3);
      // V' = P [I; T'] (n x k) = Q_v R: R = chol(I + T T') (V V' = I + T T'),
      // Q_v = V' R^{-1} is applied in factored form below; the Householder
      // QR of V' remains for a (theoretical) Cholesky breakdown
      T* R = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      T* Vt = nullptr;
      T* tau = nullptr;
      if (!chol_v<T>(ctx, k, n - k, F.T_, R)) {
        Vt = ctx->arena.alloc_n<T>((size_t)ldn * ldk);
        set_zero(ctx, Vt, ldn * ldk);
        T* I = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
        set_identity(ctx, k, k, I, ldk);
        scatter_rows(ctx, k, k, I, ldk, F.jpvt, Vt, ldn);
        if (n > k) {
          T* Tt = ctx->arena.alloc_n<T>((size_t)(n - k) * ldk);
          transpose(ctx, k, n - k, F.T_, ldk, Tt, n - k);
          scatter_rows(ctx, n - k, k, Tt, n - k, F.jpvt + k, Vt, ldn);
        }
        int64_t* jp = ctx->arena.alloc_n<int64_t>(ldk);
        tau = ctx->arena.alloc_n<T>(ldk);
        geqp3_adap<T>(ctx, n, k, Vt, ldn, jp, tau, k, 32, -1.0, 0.0, false);
        copy_matrix(ctx, k, k, Vt, ldn, R, ldk);
        zero_lower(ctx, k, k, R, ldk);
      }
      // B = R (A[sk, sk] R')
      T* Ass = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      if (ctx->linop) {
        // an operator's A[sk, sk]: rows sk of A[:, sk] (src/linop.jl:73-77)
        T* Ac = getcols<T>(ctx, 'n', n, n, dA, F.jpvt, k);
        gather_rows(ctx, k, k, Ac, ldn, F.jpvt, Ass, ldk);
      } else {
        T* Ar = ctx->arena.alloc_n<T>((size_t)ldk * ldn);
        gather_rows(ctx, k, n, dA.p, dA.ld, F.jpvt, Ar, ldk);
        gather_cols(ctx, k, k, Ar, ldk, F.jpvt, Ass, ldk);
      }
      T* C = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      gemm<T>(ctx, 'n', 't', k, k, k, T(1), Ass, ldk, R, ldk, T(0), C, ldk);
      T* B = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      gemm<T>(ctx, 'n', 'n', k, k, k, T(1), R, ldk, C, ldk, T(0), B, ldk);
      symmetrize(ctx, k, B, ldk);
      // eigen! through the one-sided Jacobi SVD of the PSD shift B + s I
      T* cn = ctx->arena.alloc_n<T>(ldk);
      col_norms(ctx, k, k, B, ldk, cn);
      std::vector<T> hcn(k);
      to_host(ctx, hcn.data(), cn, k);
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      double fro = 0;
      for (T v : hcn) fro += (double)v * (double)v;
      const T shift = (T)(std::sqrt(fro) * 1.0001 + (fro == 0 ? 1.0 : 0.0));
      add_diag(ctx, k, B, ldk, shift);
      T* Z = ctx->arena.alloc_n<T>((size_t)ldk * ldk);
      T* S = ctx->arena.alloc_n<T>(ldk);
      jacobi_svd_fast<T>(ctx, k, B, ldk, Z, ldk, S);
      std::vector<T> hS(k);
      to_host(ctx, hS.data(), S, k);
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      std::vector<double> w(k);
      for (int64_t i = 0; i < k; ++i) w[i] = (double)hS[i] - (double)shift;
      std::vector<int64_t> ord(k);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return w[a] < w[b]; });
      std::vector<double> ws(k);
      for (int64_t i = 0; i < k; ++i) ws[i] = w[ord[i]];
      auto kk = pheigrank(ws, o);
      std::vector<int64_t> sel;
      if (kk.first + kk.second < k) {
        for (int64_t i = 0; i < kk.first; ++i) sel.push_back(i);
        for (int64_t i = k - kk.second; i < k; ++i) sel.push_back(i);
      } else {
        for (int64_t i = 0; i < k; ++i) sel.push_back(i);
      }
      const int64_t ke = (int64_t)sel.size();
      lra_pheig* r = static_cast<lra_pheig*>(hmalloc(sizeof(lra_pheig)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->n = n;
      r->k = ke;
      r->values = hmalloc(sizeof(T) * std::max<int64_t>(ke, 1));
      std::vector<double> vals(ke);
      for (int64_t i = 0; i < ke; ++i) {
        vals[i] = ws[sel[i]];
        static_cast<T*>(r->values)[i] = (T)vals[i];
      }
      if (!vals_only && ke > 0) {
        std::vector<int64_t> cols1(ke);
        for (int64_t i = 0; i < ke; ++i) cols1[i] = ord[sel[i]] + 1;
        int64_t* dcols = ctx->arena.alloc_n<int64_t>(ke);
        LRA_CUDA(cudaMemcpyAsync(dcols, cols1.data(), ke * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        T* Zs = ctx->arena.alloc_n<T>((size_t)ldn * ke);
        set_zero(ctx, Zs, ldn * ke);
        gather_cols(ctx, k, ke, Z, ldk, dcols, Zs, ldn);
        // pheigorth!: re-orthonormalize clusters (src/pheig.jl:342-364)
        std::vector<int64_t> cl;
        int64_t a = 0;
        while (a < ke) {
          const double va = vals[a];
          int64_t b = a + 1;
          while (b < ke) {
            const double vb = vals[b];
            if (2 * std::fabs((va - vb) / (va + vb)) > o.pheig_orthtol) break;
            ++b;
          }
          --b;
          if (b > a) {
            cl.push_back(a);
            cl.push_back(b);
          }
          a = b + 1;
        }
        if (!cl.empty()) {
          int64_t* dcl = ctx->arena.alloc_n<int64_t>(cl.size());
          LRA_CUDA(cudaMemcpyAsync(dcl, cl.data(), cl.size() * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
          cluster_orth(ctx, k, ke, Zs, ldn, dcl, (int64_t)cl.size() / 2);
        }
        if (Vt) {
          apply_q<T>(ctx, 'n', n, k, Vt, ldn, tau, Zs, ldn, ke);
        } else {
          // Q_v Z = P [I; T'] (R^{-1} Z): rows sk <- Y, rows rd <- T' Y
          T* Y = ctx->arena.alloc_n<T>((size_t)ldk * ke);
          copy_matrix(ctx, k, ke, Zs, ldn, Y, ldk);
          trsm_upper(ctx, k, ke, R, ldk, Y, ldk);
          set_zero(ctx, Zs, ldn * ke);
          scatter_rows(ctx, k, ke, Y, ldk, F.jpvt, Zs, ldn);
          if (n > k) {
            T* TY = ctx->arena.alloc_n<T>((size_t)(n - k) * ke);
            gemm<T>(ctx, 't', 'n', n - k, ke, k, T(1), F.T_, ldk, Y, ldk, T(0), TY, n - k);
            scatter_rows(ctx, n - k, ke, TY, n - k, F.jpvt + k, Zs, ldn);
          }
        }
        r->vectors = hmalloc(sizeof(T) * (size_t)n * ke);
        to_host(ctx, r->vectors, Zs, (size_t)n * ke);
        LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      }
      *out = r;
    });
  });
}

int lra_cur_middle(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda, int64_t k,
                   const int64_t* rows, const int64_t* cols, lra_psvd** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    check_dims(m, n);
    if (!out || (k > 0 && (!rows || !cols))) fail(LRA_EINVAL, "NULL argument");
    if (k < 0 || k > std::min(m, n)) fail(LRA_EDIM, "k");
    if (dtype != LRA_F32 && dtype != LRA_F64 && !is_cplx(dtype)) fail(LRA_EINVAL, "dtype");
    for (int64_t i = 0; i < k; ++i)
      if (rows[i] < 1 || rows[i] > m || cols[i] < 1 || cols[i] > n) fail(LRA_EINVAL, "row or column index");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        *out = ccur_middle<R>(ctx, m, n, A, lda, k, rows, cols, dtype);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      const int64_t kk = std::max<int64_t>(k, 1);
      // W = A[rows, cols]: gathered where A lives
      T* W = ctx->arena.alloc_n<T>((size_t)kk * kk);
      if (k > 0) {
        if (is_dev(A)) {
          int64_t* di = ctx->arena.alloc_n<int64_t>((size_t)2 * kk);
          LRA_CUDA(cudaMemcpyAsync(di, rows, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
          LRA_CUDA(cudaMemcpyAsync(di + kk, cols, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
          T* Ac = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(m, 1) * kk);
          gather_cols(ctx, m, k, static_cast<const T*>(A), lda, di + kk, Ac, std::max<int64_t>(m, 1));
          gather_rows(ctx, k, k, Ac, std::max<int64_t>(m, 1), di, W, kk);
        } else {
          const T* Ah = static_cast<const T*>(A);
          std::vector<T> h((size_t)k * k);
          for (int64_t j = 0; j < k; ++j)
            for (int64_t i = 0; i < k; ++i) h[i + j * k] = Ah[(rows[i] - 1) + (cols[j] - 1) * lda];
          LRA_CUDA(cudaMemcpyAsync(W, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
          LRA_CUDA(cudaStreamSynchronize(ctx->stream));
        }
      }
      // W = U diag(S) V' by one-sided Jacobi; pinv(W) = V diag(1 ./ S) U'
      T* Ud = ctx->arena.alloc_n<T>((size_t)kk * kk);
      T* Vd = ctx->arena.alloc_n<T>((size_t)kk * kk);
      T* Sd = ctx->arena.alloc_n<T>(kk);
      std::vector<T> hs = small_svd<T>(ctx, k, W, Ud, Vd, Sd);
      T* Ut = ctx->arena.alloc_n<T>((size_t)kk * kk);
      if (k > 0) transpose(ctx, k, k, Ud, k, Ut, k);
      lra_psvd* r = static_cast<lra_psvd*>(hmalloc(sizeof(lra_psvd)));
      std::memset(r, 0, sizeof *r);
      r->dtype = dtype;
      r->m = k;
      r->n = k;
      r->k = k;
      r->S = hmalloc(sizeof(T) * kk);
      for (int64_t i = 0; i < k; ++i) static_cast<T*>(r->S)[i] = T(1) / hs[(size_t)i];
      r->U = hmalloc(sizeof(T) * kk * kk);
      r->Vt = hmalloc(sizeof(T) * kk * kk);
      if (k > 0) {
        to_host(ctx, r->U, Vd, (size_t)k * k);
        to_host(ctx, r->Vt, Ut, (size_t)k * k);
      }
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      *out = r;
    });
  });
}

int lra_curfact(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda, const lra_opts* opts,
                const lra_rand* rand, lra_cur** out) {
  if (out) *out = nullptr;
  return guarded(ctx, [&] {
    chkopts(opts);
    ctx->gemm_tc = use_tc_gemm(*opts, dtype);
    ctx->mixed_rtol = ctx->gemm_tc ? opts->rtol : 0.0;
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    lra_opts o = *opts;
    o.pqrfact_retval = 0;  // src/cur.jl:534
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, o, m, n, dA);
        RandSrc rs(ctx, rand, o.seed);
        *out = ccurfact<R>(ctx, o, m, n, dA, rs);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, o, m, n, dA);
      RandSrc rs(ctx, rand, o.seed);
      auto sel = [&](char t, int64_t mm, int64_t nn, const DMat<T>& X) {
        Fact<T> F = id_core<T>(ctx, o, t, mm, nn, X, rs, dtype, false);
        std::vector<int64_t> idx(F.k);
        to_host(ctx, idx.data(), F.jpvt, F.k);
        LRA_CUDA(cudaStreamSynchronize(ctx->stream));
        return idx;
      };
      lra_cur* r = static_cast<lra_cur*>(hmalloc(sizeof(lra_cur)));
      std::memset(r, 0, sizeof *r);
      std::vector<int64_t> rows, cols;
      if (m == n && is_symmetric(ctx, n, dA.p, dA.ld)) {
        cols = sel('n', m, n, dA);
        rows = cols;
        r->kind = 1;
      } else if (m >= n) {
        rows = sel('c', m, n, dA);
        const int64_t kr = (int64_t)rows.size();
        int64_t* drows = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(kr, 1));
        LRA_CUDA(cudaMemcpyAsync(drows, rows.data(), kr * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        T* Ar = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(kr, 1) * std::max<int64_t>(n, 1));
        if (ctx->linop) {
          // an operator's A[rows, :] is (A' E)' (src/linop.jl:64-71), a dense matrix
          T* Art = getcols<T>(ctx, 'c', m, n, dA, drows, kr);
          transpose(ctx, n, kr, Art, std::max<int64_t>(n, 1), Ar, std::max<int64_t>(kr, 1));
        } else {
          gather_rows(ctx, kr, n, dA.p, dA.ld, drows, Ar, std::max<int64_t>(kr, 1));
        }
        DenseScope dense(ctx);
        cols = sel('n', kr, n, DMat<T>{Ar, std::max<int64_t>(kr, 1)});
      } else {
        cols = sel('n', m, n, dA);
        const int64_t kc = (int64_t)cols.size();
        int64_t* dcols = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(kc, 1));
        LRA_CUDA(cudaMemcpyAsync(dcols, cols.data(), kc * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        T* Ac;
        if (ctx->linop) {
          Ac = getcols<T>(ctx, 'n', m, n, dA, dcols, kc);
        } else {
          Ac = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(m, 1) * std::max<int64_t>(kc, 1));
          gather_cols(ctx, m, kc, dA.p, dA.ld, dcols, Ac, std::max<int64_t>(m, 1));
        }
        DenseScope dense(ctx);
        rows = sel('c', m, kc, DMat<T>{Ac, std::max<int64_t>(m, 1)});
      }
      if (r->kind == 0) {
        const size_t k = std::min(rows.size(), cols.size());
        rows.resize(k);
        cols.resize(k);
      }
      r->kr = (int64_t)rows.size();
      r->kc = (int64_t)cols.size();
      r->rows = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<size_t>(rows.size(), 1)));
      r->cols = static_cast<int64_t*>(hmalloc(sizeof(int64_t) * std::max<size_t>(cols.size(), 1)));
      std::memcpy(r->rows, rows.data(), rows.size() * sizeof(int64_t));
      std::memcpy(r->cols, cols.data(), cols.size() * sizeof(int64_t));
      *out = r;
    });
  });
}

}  // extern "C"

// ---- spectral norms ----------------------------------------------------------------

namespace lra {
namespace {

// power iteration of src/snorm.jl:14-45 with the operator given as callbacks
template <typename T, class FwdFn, class AdjFn>
double snorm_loop(lra_ctx* ctx, const lra_opts& o, int64_t m, int64_t n, bool herm, RandSrc& rs, FwdFn fwd,
                  AdjFn adj) {
  T* xn = ctx->arena.alloc_n<T>(std::max<int64_t>(n, 1));
  T* xm = ctx->arena.alloc_n<T>(std::max<int64_t>(m, 1));
  T* nrm = ctx->arena.alloc_n<T>(1);
  if (rs.injected_gauss())
    sketch_from_stream(ctx, rs.take_gauss_raw(n), n, xn, false);
  else
    rs.gauss(n, xn, false);
  auto norm = [&](const T* x, int64_t len) {
    col_norms(ctx, len, 1, x, std::max<int64_t>(len, 1), nrm);
    T h = 0;
    to_host(ctx, &h, nrm, 1);
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    return (double)h;
  };
  double xnrm = norm(xn, n);
  double s = 1, t = 0;
  int64_t niter = 0;
  while (s > 0 && std::fabs(s - t) > std::max(o.atol, t * o.rtol)) {
    if (niter == o.snorm_niter) break;
    ++niter;
    scale_vec(ctx, n, xn, (T)(1.0 / xnrm));
    if (herm) {
      fwd(xn, xm);
      copy_matrix(ctx, n, 1, xm, std::max<int64_t>(n, 1), xn, std::max<int64_t>(n, 1));
    } else {
      fwd(xn, xm);
      adj(xm, xn);
    }
    xnrm = norm(xn, n);
    t = s;
    s = herm ? xnrm : std::sqrt(xnrm);
  }
  return s;
}

}  // namespace
}  // namespace lra

// ---- matrix-free operators (LinearOperator, src/linop.jl:9-40) ----------------------
namespace lra {
namespace {

// runs an entry point with ctx->linop = L and the options a matrix-free
// input takes: the Gaussian sketch whatever opts->sketch says (chkopts!,
// src/LowRankApprox.jl:142-148), in native precision (the products are the
// operator's), and no finite check (its entries are never formed)
template <class Fn>
int with_linop(lra_ctx* ctx, const lra_linop* L, const lra_opts* opts, Fn&& call) {
  if (!ctx) return LRA_EINVAL;
  const char* bad = nullptr;
  int st = LRA_EINVAL;
  if (!L) {
    bad = "operator is NULL";
  } else if (!L->matmat) {
    bad = "operator has no matmat";
  } else if (L->m < 0 || L->n < 0) {
    bad = "negative dimension";
    st = LRA_EDIM;
  } else if (L->dtype != LRA_F32 && L->dtype != LRA_F64) {
    bad = "dtype";
  } else if (L->hermitian && L->m != L->n) {
    bad = "a Hermitian operator must be square";
    st = LRA_EDIM;
  } else if (!opts) {
    bad = "opts is NULL";
  }
  if (bad) {
    ctx->last_error = bad;
    return st;
  }
  lra_opts o = *opts;
  o.sketch = LRA_SKETCH_RANDN;
  o.precision = LRA_PREC_NATIVE;
  o.check_finite = 0;
  ctx->linop = L;
  int r = LRA_ECUDA;
  try {
    r = call(&o);
  } catch (...) {
    ctx->last_error = "unexpected exception";
  }
  ctx->linop = nullptr;
  return r;
}

inline int64_t lin_ld(const lra_linop* L) { return std::max<int64_t>(L->m, 1); }

}  // namespace
}  // namespace lra

extern "C" {

int lra_snorm(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda, int hermitian,
              const lra_opts* opts, const lra_rand* rand, double* out) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        check_input_c<R>(ctx, *opts, m, n, dA);
        const bool herm = hermitian < 0 ? (m == n && cis_hermitian<R>(ctx, n, dA.p, dA.ld)) : hermitian != 0;
        RandSrc rs(ctx, rand, opts->seed);
        const CX<R> one(1), zero(0);
        *out = csnorm_loop<R>(
            ctx, *opts, m, n, herm, rs,
            [&](const CX<R>* x, CX<R>* y) { cgemm<R>(ctx, 'n', 'n', m, 1, n, one, dA.p, dA.ld, x, std::max<int64_t>(n, 1), zero, y, std::max<int64_t>(m, 1)); },
            [&](const CX<R>* y, CX<R>* x) { cgemm<R>(ctx, 'c', 'n', n, 1, m, one, dA.p, dA.ld, y, std::max<int64_t>(m, 1), zero, x, std::max<int64_t>(n, 1)); });
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      check_input(ctx, *opts, m, n, dA);
      const bool herm = hermitian < 0 ? (m == n && is_symmetric(ctx, n, dA.p, dA.ld)) : hermitian != 0;
      RandSrc rs(ctx, rand, opts->seed);
      const bool lin = ctx->linop != nullptr;
      *out = snorm_loop<T>(
          ctx, *opts, m, n, herm, rs,
          [&](const T* x, T* y) {
            if (lin)
              linop_apply<T>(ctx, 'n', 1, x, std::max<int64_t>(n, 1), y, std::max<int64_t>(m, 1));
            else
              gemv<T>(ctx, 'n', m, n, T(1), dA.p, dA.ld, x, T(0), y);
          },
          [&](const T* y, T* x) {
            if (lin)
              linop_apply<T>(ctx, 'c', 1, y, std::max<int64_t>(m, 1), x, std::max<int64_t>(n, 1));
            else
              gemv<T>(ctx, 't', m, n, T(1), dA.p, dA.ld, y, T(0), x);
          });
    });
  });
}

int lra_snormdiff(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda, const void* B,
                  int64_t ldb, const lra_opts* opts, const lra_rand* rand, double* out) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (!out) fail(LRA_EINVAL, "out is NULL");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        DMat<CX<R>> dB = stage_in<CX<R>>(ctx, B, m, n, ldb);
        const bool herm = m == n && cis_hermitian<R>(ctx, n, dA.p, dA.ld) && cis_hermitian<R>(ctx, n, dB.p, dB.ld);
        RandSrc rs(ctx, rand, opts->seed);
        *out = csnormdiff_dense<R>(ctx, *opts, m, n, dA.p, dA.ld, dB.p, dB.ld, herm, rs);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      DMat<T> dB = stage_in<T>(ctx, B, m, n, ldb);
      const bool herm = m == n && is_symmetric(ctx, n, dA.p, dA.ld) && is_symmetric(ctx, n, dB.p, dB.ld);
      RandSrc rs(ctx, rand, opts->seed);
      *out = snorm_loop<T>(
          ctx, *opts, m, n, herm, rs,
          [&](const T* x, T* y) {
            gemv<T>(ctx, 'n', m, n, T(1), dA.p, dA.ld, x, T(0), y);
            gemv<T>(ctx, 'n', m, n, T(-1), dB.p, dB.ld, x, T(1), y);
          },
          [&](const T* y, T* x) {
            gemv<T>(ctx, 't', m, n, T(1), dA.p, dA.ld, y, T(0), x);
            gemv<T>(ctx, 't', m, n, T(-1), dB.p, dB.ld, y, T(1), x);
          });
    });
  });
}

int lra_snormdiff_id(lra_ctx* ctx, int dtype, char trans, int64_t m, int64_t n, const void* A, int64_t lda,
                     const lra_id* F, const lra_opts* opts, const lra_rand* rand, double* out) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (!out || !F) fail(LRA_EINVAL, "NULL argument");
    const char t = chktrans(trans);
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        if (F->dtype != dtype) fail(LRA_EINVAL, "dtype of F");
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
        if (F->n != N) fail(LRA_EDIM, "ID size");
        const int64_t k = F->k, ldm = std::max<int64_t>(M, 1);
        CX<R>* Aop = cdense_op<R>(ctx, t, m, n, dA);
        int64_t* p = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(N, 1));
        LRA_CUDA(cudaMemcpyAsync(p, F->sk, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        LRA_CUDA(cudaMemcpyAsync(p + k, F->rd, (N - k) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
        CX<R>* Td = ctx->arena.alloc_n<CX<R>>((size_t)std::max<int64_t>(k * (N - k), 1));
        if (k > 0 && N > k)
          LRA_CUDA(cudaMemcpyAsync(Td, F->T, (size_t)k * (N - k) * sizeof(CX<R>), cudaMemcpyHostToDevice, ctx->stream));
        CX<R>* Cm = ctx->arena.alloc_n<CX<R>>((size_t)ldm * std::max<int64_t>(k, 1));
        gather_cols<CX<R>>(ctx, M, k, Aop, ldm, p, Cm, ldm);
        CX<R>* Fp = ctx->arena.alloc_n<CX<R>>((size_t)ldm * std::max<int64_t>(N, 1));
        CX<R>* Fd = ctx->arena.alloc_n<CX<R>>((size_t)ldm * std::max<int64_t>(N, 1));
        copy_matrix<CX<R>>(ctx, M, k, Cm, ldm, Fp, ldm);
        if (k > 0 && N > k)
          cgemm<R>(ctx, 'n', 'n', M, N - k, k, CX<R>(1), Cm, ldm, Td, k, CX<R>(0), Fp + k * ldm, ldm);
        else if (N > k)
          set_zero<CX<R>>(ctx, Fp + k * ldm, ldm * (N - k));
        scatter_cols<CX<R>>(ctx, M, N, Fp, ldm, p, Fd, ldm);
        RandSrc rs(ctx, rand, opts->seed);
        *out = csnormdiff_dense<R>(ctx, *opts, M, N, Aop, ldm, Fd, ldm, false, rs);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      if (F->dtype != dtype) fail(LRA_EINVAL, "dtype of F");
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      // work on op(A) (M x N): F = C [I T] P', C = op(A)[:, sk]
      const int64_t M = t == 'n' ? m : n, N = t == 'n' ? n : m;
      if (F->n != N) fail(LRA_EDIM, "ID size");
      const int64_t k = F->k, ldm = std::max<int64_t>(M, 1);
      T* Aop = dense_op(ctx, t, m, n, dA);
      int64_t* p = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(N, 1));
      LRA_CUDA(cudaMemcpyAsync(p, F->sk, k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
      LRA_CUDA(cudaMemcpyAsync(p + k, F->rd, (N - k) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
      T* Td = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(k * (N - k), 1));
      if (k > 0 && N > k)
        LRA_CUDA(cudaMemcpyAsync(Td, F->T, (size_t)k * (N - k) * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      T* C = ctx->arena.alloc_n<T>((size_t)ldm * std::max<int64_t>(k, 1));
      gather_cols(ctx, M, k, Aop, ldm, p, C, ldm);
      // dense F = C [I T] P' then the difference power iteration
      T* Fd = ctx->arena.alloc_n<T>((size_t)ldm * std::max<int64_t>(N, 1));
      T* Fp = ctx->arena.alloc_n<T>((size_t)ldm * std::max<int64_t>(N, 1));
      copy_matrix(ctx, M, k, C, ldm, Fp, ldm);
      if (k > 0 && N > k) gemm<T>(ctx, 'n', 'n', M, N - k, k, T(1), C, ldm, Td, k, T(0), Fp + k * ldm, ldm);
      else if (N > k) set_zero(ctx, Fp + k * ldm, ldm * (N - k));
      scatter_cols(ctx, M, N, Fp, ldm, p, Fd, ldm);
      RandSrc rs(ctx, rand, opts->seed);
      *out = snorm_loop<T>(
          ctx, *opts, M, N, false, rs,
          [&](const T* x, T* y) {
            gemv<T>(ctx, 'n', M, N, T(1), Aop, ldm, x, T(0), y);
            gemv<T>(ctx, 'n', M, N, T(-1), Fd, ldm, x, T(1), y);
          },
          [&](const T* y, T* x) {
            gemv<T>(ctx, 't', M, N, T(1), Aop, ldm, y, T(0), x);
            gemv<T>(ctx, 't', M, N, T(-1), Fd, ldm, y, T(1), x);
          });
    });
  });
}

int lra_snormdiff_psvd(lra_ctx* ctx, int dtype, int64_t m, int64_t n, const void* A, int64_t lda,
                       const lra_psvd* F, const lra_opts* opts, const lra_rand* rand, double* out) {
  return guarded(ctx, [&] {
    chkopts(opts);
    check_dims(m, n);
    if (!out || !F || !F->U || !F->Vt) fail(LRA_EINVAL, "NULL argument");
    if (is_cplx(dtype)) {
      dispatch_c(dtype, [&](auto z) {
        using R = decltype(z);
        if (F->dtype != dtype) fail(LRA_EINVAL, "dtype of F");
        if (F->m != m || F->n != n) fail(LRA_EDIM, "PSVD size");
        DMat<CX<R>> dA = stage_in<CX<R>>(ctx, A, m, n, lda);
        const int64_t k = F->k, kk = std::max<int64_t>(k, 1), ldm = std::max<int64_t>(m, 1);
        CX<R>* U = ctx->arena.alloc_n<CX<R>>((size_t)ldm * kk);
        CX<R>* Vt = ctx->arena.alloc_n<CX<R>>((size_t)kk * std::max<int64_t>(n, 1));
        LRA_CUDA(cudaMemcpyAsync(U, F->U, (size_t)m * k * sizeof(CX<R>), cudaMemcpyHostToDevice, ctx->stream));
        LRA_CUDA(cudaMemcpyAsync(Vt, F->Vt, (size_t)k * n * sizeof(CX<R>), cudaMemcpyHostToDevice, ctx->stream));
        // US = U diag(S) on the host values of S, then the dense F = US Vt
        std::vector<CX<R>> hU((size_t)m * k);
        std::memcpy(hU.data(), F->U, hU.size() * sizeof(CX<R>));
        const R* hs = static_cast<const R*>(F->S);
        for (int64_t j = 0; j < k; ++j)
          for (int64_t i = 0; i < m; ++i) hU[i + j * m] = hs[j] * hU[i + j * m];
        LRA_CUDA(cudaMemcpyAsync(U, hU.data(), hU.size() * sizeof(CX<R>), cudaMemcpyHostToDevice, ctx->stream));
        CX<R>* Fd = ctx->arena.alloc_n<CX<R>>((size_t)ldm * std::max<int64_t>(n, 1));
        if (k > 0)
          cgemm<R>(ctx, 'n', 'n', m, n, k, CX<R>(1), U, ldm, Vt, kk, CX<R>(0), Fd, ldm);
        else
          set_zero<CX<R>>(ctx, Fd, ldm * n);
        LRA_CUDA(cudaStreamSynchronize(ctx->stream));
        RandSrc rs(ctx, rand, opts->seed);
        *out = csnormdiff_dense<R>(ctx, *opts, m, n, dA.p, dA.ld, Fd, ldm, false, rs);
      });
      return;
    }
    dispatch(dtype, [&](auto z) {
      using T = decltype(z);
      if (F->dtype != dtype) fail(LRA_EINVAL, "dtype of F");
      if (F->m != m || F->n != n) fail(LRA_EDIM, "PSVD size");
      DMat<T> dA = stage_in<T>(ctx, A, m, n, lda);
      const int64_t k = F->k, kk = std::max<int64_t>(k, 1);
      T* U = ctx->arena.alloc_n<T>((size_t)std::max<int64_t>(m, 1) * kk);
      T* S = ctx->arena.alloc_n<T>(kk);
      T* Vt = ctx->arena.alloc_n<T>((size_t)kk * std::max<int64_t>(n, 1));
      T* w = ctx->arena.alloc_n<T>(kk);
      LRA_CUDA(cudaMemcpyAsync(U, F->U, (size_t)m * k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      LRA_CUDA(cudaMemcpyAsync(S, F->S, (size_t)k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      LRA_CUDA(cudaMemcpyAsync(Vt, F->Vt, (size_t)k * n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      // US = U diag(S)
      T* Sinv = ctx->arena.alloc_n<T>(kk);
      std::vector<T> hs(k), hsi(k);
      std::memcpy(hs.data(), F->S, k * sizeof(T));
      for (int64_t i = 0; i < k; ++i) hsi[i] = hs[i] != T(0) ? T(1) / hs[i] : T(0);
      LRA_CUDA(cudaMemcpyAsync(Sinv, hsi.data(), k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
      div_cols(ctx, std::max<int64_t>(m, 1), k, U, std::max<int64_t>(m, 1), Sinv);  // U <- U diag(S)
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      RandSrc rs(ctx, rand, opts->seed);
      *out = snorm_loop<T>(
          ctx, *opts, m, n, false, rs,
          [&](const T* x, T* y) {
            gemv<T>(ctx, 'n', m, n, T(1), dA.p, dA.ld, x, T(0), y);
            gemv<T>(ctx, 'n', k, n, T(1), Vt, kk, x, T(0), w);
            gemv<T>(ctx, 'n', m, k, T(-1), U, std::max<int64_t>(m, 1), w, T(1), y);
          },
          [&](const T* y, T* x) {
            gemv<T>(ctx, 't', m, n, T(1), dA.p, dA.ld, y, T(0), x);
            gemv<T>(ctx, 't', m, k, T(1), U, std::max<int64_t>(m, 1), y, T(0), w);
            gemv<T>(ctx, 't', k, n, T(-1), Vt, kk, w, T(1), x);
          });
    });
  });
}


int lra_sketchfact_linop(lra_ctx* ctx, char side, char trans, const lra_linop* L, const lra_opts* opts,
                         const lra_rand* rand, lra_pqr** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_sketchfact(ctx, L->dtype, side, trans, L->m, L->n, L, lin_ld(L), o, rand, out);
  });
}

int lra_idfact_linop(lra_ctx* ctx, char trans, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                     lra_id** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_idfact(ctx, L->dtype, trans, L->m, L->n, L, lin_ld(L), o, rand, out);
  });
}

int lra_pqrfact_linop(lra_ctx* ctx, char trans, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                      lra_pqr** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_pqrfact(ctx, L->dtype, trans, L->m, L->n, L, lin_ld(L), o, rand, out);
  });
}

int lra_prange_linop(lra_ctx* ctx, char trans, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                     lra_pqr** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_prange(ctx, L->dtype, trans, L->m, L->n, L, lin_ld(L), o, rand, out);
  });
}

int lra_psvdfact_linop(lra_ctx* ctx, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                       int vals_only, lra_psvd** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_psvdfact(ctx, L->dtype, L->m, L->n, L, lin_ld(L), o, rand, vals_only, out);
  });
}

int lra_pheigfact_linop(lra_ctx* ctx, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                        int vals_only, lra_pheig** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    if (L->m != L->n) {
      ctx->last_error = "pheigfact needs a square operator";
      return (int)LRA_EDIM;
    }
    return lra_pheigfact(ctx, L->dtype, L->n, L, lin_ld(L), o, rand, vals_only, out);
  });
}

int lra_curfact_linop(lra_ctx* ctx, const lra_linop* L, const lra_opts* opts, const lra_rand* rand,
                      lra_cur** out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_curfact(ctx, L->dtype, L->m, L->n, L, lin_ld(L), o, rand, out);
  });
}

int lra_snorm_linop(lra_ctx* ctx, const lra_linop* L, const lra_opts* opts, const lra_rand* rand, double* out) {
  return with_linop(ctx, L, opts, [&](const lra_opts* o) {
    return lra_snorm(ctx, L->dtype, L->m, L->n, L, lin_ld(L), -1, o, rand, out);
  });
}

void lra_id_free(lra_id* r) {
  if (!r) return;
  hfree(r->sk);
  hfree(r->rd);
  hfree(r->T);
  hfree(r);
}

void lra_pqr_free(lra_pqr* r) {
  if (!r) return;
  hfree(r->p);
  hfree(r->Q);
  hfree(r->R);
  hfree(r->T);
  hfree(r);
}

void lra_psvd_free(lra_psvd* r) {
  if (!r) return;
  hfree(r->U);
  hfree(r->S);
  hfree(r->Vt);
  hfree(r);
}

void lra_pheig_free(lra_pheig* r) {
  if (!r) return;
  hfree(r->values);
  hfree(r->vectors);
  hfree(r);
}

void lra_cur_free(lra_cur* r) {
  if (!r) return;
  hfree(r->rows);
  hfree(r->cols);
  hfree(r);
}

}  // extern "C"
