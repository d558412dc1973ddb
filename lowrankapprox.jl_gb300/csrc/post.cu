// Post-processing of the ID into PSVD / PHEIG / PQR factors (src/psvd.jl:238-272,
// src/pheig.jl:276-296, src/pqr.jl:297-307) as GEMM-shaped work.
//
// The reference takes Householder QRs of the tall skeleton matrix A[:, sk]
// (m x k) and of (R V)^T (n x k).  Here both become Cholesky QRs that are
// stable because their inputs are well conditioned:
//   * A[:, sk] R11^{-1}, with R11 the triangular factor of the sketch's own
//     pivoted QR on the skeleton columns (S A[:, sk] = Q_B R11), is the
//     preimage of the orthonormal Q_B under the subspace embedding S, so its
//     condition number is that of S on range(A[:, sk]) -- O(10) for a
//     Gaussian sketch -- and its Gram matrix factors stably;
//   * V V^T = I + T T^T, so V^T = P [I; T^T] factors as Q_v R_v with
//     R_v = chol(I + T T^T) without forming Q_v.
// The factorizations of the reference are then recovered exactly:
//   A[:, sk] = Q R_A,  R_A = R_c R11,
//   R V = R_A R_v^T Q_v^T,  SVD(R_A R_v^T) = U_M S V_M^T,
//   U = Q U_M,  Vt = (R_v^{-1} V_M)^T V.
// Every large operation is a GEMM or a blocked triangular solve; only the
// k x k SVD / eigenproblem is iterative.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

template <typename T>
bool cholqr_pre(lra_ctx* ctx, int64_t m, int64_t k, T* X, int64_t ldx, const T* Rpre, int64_t ldr, int passes,
                T* Rc) {
  const int64_t kk = std::max<int64_t>(k, 1);
  set_identity(ctx, k, k, Rc, kk);
  if (k == 0) return true;
  if (Rpre) trsm_right_upper(ctx, m, k, Rpre, ldr, X, ldx);
  const ArenaMark mk = ctx->arena.mark();
  T* G = ctx->arena.alloc_n<T>((size_t)kk * kk);
  T* tmp = ctx->arena.alloc_n<T>((size_t)kk * kk);
  bool ok = true;
  for (int p = 0; p < passes && ok; ++p) {
    gemm<T>(ctx, 't', 'n', k, k, m, T(1), X, ldx, X, ldx, T(0), G, kk);
    ok = potrf_upper(ctx, k, G, kk);
    if (!ok) break;
    trsm_right_upper(ctx, m, k, G, kk, X, ldx);
    // Rc <- G Rc (both upper triangular)
    gemm<T>(ctx, 'n', 'n', k, k, k, T(1), G, kk, Rc, kk, T(0), tmp, kk);
    copy_matrix(ctx, k, k, tmp, kk, Rc, kk);
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return ok;
}

// X (m x k) <- X Rpre^{-1} and one Cholesky QR pass (Rc = its triangular
// factor), together with R_v = chol(I + T T^T) (T k x nr, ld k): the two
// k x k Cholesky factorizations in one launch.  False on a breakdown of
// either.
template <typename T>
bool cholqr1_and_chol_v(lra_ctx* ctx, int64_t m, int64_t k, T* X, int64_t ldx, const T* Rpre, int64_t ldr, T* Rc,
                        int64_t nr, const T* Tm, T* Rv, const T* Rpre_inv) {
  const int64_t kk = std::max<int64_t>(k, 1);
  set_identity(ctx, k, k, Rv, kk);
  if (k == 0) {
    set_identity(ctx, k, k, Rc, kk);
    return true;
  }
  // LRA_TRACE: the phases (each waits for the device)
  const bool tr = trace_on();
  auto tnow = [] { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count(); };
  double tl = tr ? tnow() : 0;
  auto tmark = [&](const char* what) {
    if (!tr) return;
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    const double t = tnow();
    std::fprintf(stderr, "[lra] cholqr k=%lld %s %.3f ms\n", (long long)k, what, t - tl);
    tl = t;
  };
  tmark("start");
  if (nr > 0) gemm<T>(ctx, 'n', 't', k, k, nr, T(1), Tm, kk, Tm, kk, T(1), Rv, kk);
  tmark("I + T T'");
  trsm_right_upper(ctx, m, k, Rpre, ldr, X, ldx, Rpre_inv);
  tmark("X / R11");
  gemm<T>(ctx, 't', 'n', k, k, m, T(1), X, ldx, X, ldx, T(0), Rc, kk);
  tmark("gram");
  const int64_t ks[2] = {k, k}, lds[2] = {kk, kk};
  T* Gs[2] = {Rc, Rv};
  bool ok[2] = {true, true};
  potrf_upper_batch<T>(ctx, 2, ks, Gs, lds, ok);
  tmark("two cholesky");
  if (!ok[0] || !ok[1]) return false;
  trsm_right_upper(ctx, m, k, Rc, kk, X, ldx);
  tmark("X / Rc");
  return true;
}

// R_v = chol(I + T T^T), T k x nr (ld k); false on breakdown
template <typename T>
bool chol_v(lra_ctx* ctx, int64_t k, int64_t nr, const T* Tm, T* Rv) {
  const int64_t kk = std::max<int64_t>(k, 1);
  set_identity(ctx, k, k, Rv, kk);
  if (k == 0) return true;
  if (nr > 0) gemm<T>(ctx, 'n', 't', k, k, nr, T(1), Tm, kk, Tm, kk, T(1), Rv, kk);
  return potrf_upper(ctx, k, Rv, kk);
}

// descending sort of S with the matching columns of U and V (k x k, ld k)
template <typename T>
std::vector<T> sort_desc(lra_ctx* ctx, int64_t k, T* S, T* U, T* V) {
  std::vector<T> hS(k);
  if (k == 0) return hS;
  LRA_CUDA(cudaMemcpyAsync(hS.data(), S, k * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int64_t> ord(k);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return hS[a] > hS[b]; });
  bool sorted = true;
  for (int64_t i = 0; i < k; ++i) sorted &= ord[i] == i;
  if (sorted) return hS;
  std::vector<int64_t> o1(k);
  std::vector<T> s2(k);
  for (int64_t i = 0; i < k; ++i) {
    o1[i] = ord[i] + 1;
    s2[i] = hS[ord[i]];
  }
  const ArenaMark mk = ctx->arena.mark();
  int64_t* d = ctx->arena.alloc_n<int64_t>(k);
  T* tmp = ctx->arena.alloc_n<T>((size_t)k * k);
  LRA_CUDA(cudaMemcpyAsync(d, o1.data(), k * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
  for (T* X : {U, V}) {
    gather_cols(ctx, k, k, X, k, d, tmp, k);
    copy_matrix(ctx, k, k, tmp, k, X, k);
  }
  LRA_CUDA(cudaMemcpyAsync(S, s2.data(), k * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return s2;
}

// SVD of a k x k matrix Mm = U_M diag(S) V_M^T (S descending) by one-sided
// Jacobi on Mm^T, whose columns (the rows of Mm) carry the grading of the
// pivoted factors.  U, V, S are k x k / k device buffers.
template <typename T>
std::vector<T> small_svd(lra_ctx* ctx, int64_t k, const T* Mm, T* U, T* V, T* S) {
  if (k == 0) return {};
  // X = Mm^T; Jacobi: X W = Y diag(S) -> Mm = W diag(S) Y^T: U_M = W, V_M = Y
  transpose(ctx, k, k, Mm, k, V, k);
  jacobi_svd_fast<T>(ctx, k, V, k, U, k, S);
  div_cols(ctx, k, k, V, k, S);
  return sort_desc(ctx, k, S, U, V);
}

template bool cholqr_pre<float>(lra_ctx*, int64_t, int64_t, float*, int64_t, const float*, int64_t, int, float*);
template bool cholqr_pre<double>(lra_ctx*, int64_t, int64_t, double*, int64_t, const double*, int64_t, int,
                                 double*);
template bool cholqr1_and_chol_v<float>(lra_ctx*, int64_t, int64_t, float*, int64_t, const float*, int64_t, float*,
                                        int64_t, const float*, float*, const float*);
template bool cholqr1_and_chol_v<double>(lra_ctx*, int64_t, int64_t, double*, int64_t, const double*, int64_t,
                                         double*, int64_t, const double*, double*, const double*);
template bool chol_v<float>(lra_ctx*, int64_t, int64_t, const float*, float*);
template bool chol_v<double>(lra_ctx*, int64_t, int64_t, const double*, double*);
template std::vector<float> small_svd<float>(lra_ctx*, int64_t, const float*, float*, float*, float*);
template std::vector<double> small_svd<double>(lra_ctx*, int64_t, const double*, double*, double*, double*);
template std::vector<float> sort_desc<float>(lra_ctx*, int64_t, float*, float*, float*);
template std::vector<double> sort_desc<double>(lra_ctx*, int64_t, double*, double*, double*);

}  // namespace lra

// ---- mixed-precision one-sided Jacobi -------------------------------------------
// FP64 runs at 1/64 of the FP32 rate on GB300, so the sweeps that only need to
// bring the columns close to orthogonal run in FP32; the accumulated FP32
// rotation is re-orthonormalized in FP64 (Cholesky QR of a near-identity
// Gram matrix), applied to X in FP64, and FP64 sweeps finish from there --
// they converge quadratically from the FP32 level in one or two sweeps.

namespace lra {

namespace {

template <typename S, typename D>
__global__ void cast_kernel(int64_t m, int64_t n, const S* __restrict__ a, int64_t lda, D* __restrict__ b,
                            int64_t ldb, double scale) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    b[i + j * ldb] = (D)((double)a[i + j * lda] * scale);
  }
}

template <typename S, typename D>
void cast(lra_ctx* ctx, int64_t m, int64_t n, const S* a, int64_t lda, D* b, int64_t ldb, double scale = 1.0) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m * n + 255) / 256, ctx->num_sms * 8));
  cast_kernel<S, D><<<g, 256, 0, ctx->stream>>>(m, n, a, lda, b, ldb, scale);
  post_launch(ctx, "cast_kernel");
}

// max |a| as the bit pattern of a nonnegative double (NaN / Inf as +Inf)
template <typename T>
__global__ void absmax_bits_kernel(int64_t m, int64_t n, const T* __restrict__ a, int64_t lda,
                                   unsigned long long* __restrict__ out) {
  double mx = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    const double v = fabs((double)a[t % m + (t / m) * lda]);
    mx = v <= 1.7976931348623157e308 ? fmax(mx, v) : INFINITY;
  }
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

// X^ = X with every column scaled to unit norm (zero columns stay zero)
__global__ void unit_cols_kernel(int64_t n, const double* __restrict__ X, int64_t ldx, const double* __restrict__ s,
                                 double* __restrict__ Xh) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    Xh[t] = s[j] > 0 ? X[i + j * ldx] / s[j] : 0.0;
  }
}

// T antisymmetric from the Gram matrix of the unit columns: for p < q the
// tangent of the one-sided Jacobi angle of the pair, zeta = (s_q^2 - s_p^2) /
// (2 s_p s_q c_pq), t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)); T_pq = t,
// T_qp = -t.  Angles with |t| > kGramMaxTan (nearly equal norms: a cluster,
// where simultaneous rotations interfere, or a pair the FP32 sweeps left far
// from orthogonal) are left out.  maxc[0] gets the largest |c_pq|, maxc[1]
// the largest over the pairs that rotate, maxc[2] the largest |t| (bits of
// doubles).
constexpr double kGramMaxTan = 0.01;

__global__ void gram_tangent_kernel(int64_t n, const double* __restrict__ Gh, const double* __restrict__ s,
                                    double* __restrict__ T, unsigned long long* __restrict__ maxc) {
  double mc = 0, ma = 0, mt = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % n, col = t / n;
    if (r == col) {
      T[t] = 0;
      continue;
    }
    const int64_t p = r < col ? r : col, q = r < col ? col : r;
    const double c = Gh[p + q * n];
    mc = fmax(mc, fabs(c));
    double tg = 0;
    if (c != 0 && s[p] > 0 && s[q] > 0) {
      const double zeta = (s[q] * s[q] - s[p] * s[p]) / (2.0 * s[p] * s[q] * c);
      tg = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      if (!(fabs(tg) <= kGramMaxTan)) {
        tg = 0;
      } else {
        ma = fmax(ma, fabs(c));
        mt = fmax(mt, fabs(tg));
      }
    }
    T[t] = r < col ? tg : -tg;
  }
  mc = warp_max(mc);
  ma = warp_max(ma);
  mt = warp_max(mt);
  if ((threadIdx.x & 31) == 0) {
    if (mc > 0) atomicMax(maxc, (unsigned long long)__double_as_longlong(mc));
    if (ma > 0) atomicMax(maxc + 1, (unsigned long long)__double_as_longlong(ma));
    if (mt > 0) atomicMax(maxc + 2, (unsigned long long)__double_as_longlong(mt));
  }
}

// W = I + T + T2 / 2, exp(T) to second order: W'W = I + T^4 / 4 for
// antisymmetric T (the third-order terms cancel)
__global__ void gram_rotation_kernel(int64_t n, const double* __restrict__ T, const double* __restrict__ T2,
                                     double* __restrict__ W) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    W[t] = (i == j ? 1.0 : 0.0) + T[t] + 0.5 * T2[t];
  }
}

// W <- W - W T^4 / 8 (one Newton-Schulz step, W (3 I - W'W) / 2, written for
// W'W = I + T^4 / 4: the defect falls to O(T^8) while every product involved
// is small, so no entry of W loses its own relative accuracy), and DW =
// diag(s) W
__global__ void gram_finish_kernel(int64_t n, const double* __restrict__ WT4, const double* __restrict__ s,
                                   double* __restrict__ W, double* __restrict__ DW) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n;
    const double w = WT4 ? W[t] - 0.125 * WT4[t] : W[t];
    W[t] = w;
    DW[t] = s[i] * w;
  }
}

// the pairs whose cosine is above tol (p < q): appended to pairs[] (at most
// cap; count may go past it)
__global__ void gram_bad_pairs_kernel(int64_t n, const double* __restrict__ Gh, double tol, int2* __restrict__ pairs,
                                      int* __restrict__ count, int cap) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t % n, q = t / n;
    if (p >= q || !(fabs(Gh[p + q * n]) > tol)) continue;
    const int i = atomicAdd(count, 1);
    if (i < cap) pairs[i] = make_int2((int)p, (int)q);
  }
}

// one exact one-sided Jacobi rotation per CTA, on disjoint column pairs of X
// (and the same rotation on Wacc): the FP64 dots of the pair, the angle as
// the FP32 sweeps take it, the two columns rotated
__global__ void __launch_bounds__(256) pair_rotate_kernel(int64_t n, double* __restrict__ X, int64_t ldx,
                                                          double* __restrict__ Wacc, const int2* __restrict__ pairs) {
  __shared__ double red[3][8];
  const int2 pq = pairs[blockIdx.x];
  double* xp = X + (int64_t)pq.x * ldx;
  double* xq = X + (int64_t)pq.y * ldx;
  double a = 0, b = 0, g = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = xp[i], w = xq[i];
    a = fma(u, u, a);
    b = fma(w, w, b);
    g = fma(u, w, g);
  }
  a = warp_sum(a);
  b = warp_sum(b);
  g = warp_sum(g);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][wid] = a;
    red[1][wid] = b;
    red[2][wid] = g;
  }
  __syncthreads();
  a = b = g = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    a += red[0][w];
    b += red[1][w];
    g += red[2][w];
  }
  if (g == 0 || !(a > 0) || !(b > 0)) return;
  const double zeta = (b - a) / (2.0 * g);
  const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double c = 1.0 / sqrt(1.0 + t * t), sn = c * t;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = xp[i], w = xq[i];
    xp[i] = c * u - sn * w;
    xq[i] = sn * u + c * w;
  }
  double* vp = Wacc + (int64_t)pq.x * n;
  double* vq = Wacc + (int64_t)pq.y * n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const double u = vp[i], w = vq[i];
    vp[i] = c * u - sn * w;
    vq[i] = sn * u + c * w;
  }
}

}  // namespace

// ---- Gram-matrix polish of a nearly orthogonal X ----------------------------------
// After the FP32 sweeps and X <- X W, the columns of X are orthogonal to
// about 1e-6 relative to their norms.  One-sided Jacobi would finish with a
// sweep or two of pairwise rotations; here every pair's rotation comes from
// the Gram matrix of the unit columns, G^ = X^' X^ (one GEMM: each entry is a
// cosine, accurate to ~2^-45 absolutely on the tensor cores), and all the
// rotations are applied at once, W = exp(T) to second order with T the
// antisymmetric matrix of the pairs' angle tangents.  The cosines square
// every iteration (1e-6 -> ~1e-11 -> rounding).  X <- X^ (diag(s) W) keeps
// each column's error relative to its own norm, which the plain product X W
// would not for a graded X.  Returns false when the largest cosine is still
// above tol after a few iterations (clusters of equal singular values, where
// simultaneous rotations interfere); the caller then finishes with pairwise
// sweeps from the X and Wacc reached so far (pairs of nearly equal norms are
// left to them; an iteration that raised the largest cosine is undone).
// Wacc (n x n, ld n) is multiplied by each W; S gets the column norms of the
// final X.
constexpr double kGramStart = 3e-2;  // largest cosine the FP32 sweeps leave for the Gram polish

// The pairs the simultaneous rotations leave out (nearly equal norms), when
// they are few: exact rotations of those pairs, in rounds of disjoint pairs
// taken largest cosine first.  False (nothing done) when there are none or
// too many; the pairwise sweeps over all pairs then finish instead.
static bool rotate_bad_pairs(lra_ctx* ctx, int64_t n, double* X, int64_t ldx, double* Wacc, const double* Gh,
                             double tol) {
  const int cap = (int)std::min<int64_t>(32 * n, 1 << 22);
  const ArenaMark mk = ctx->arena.mark();
  int2* dp = ctx->arena.alloc_n<int2>((size_t)cap);
  int* cnt = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), ctx->stream));
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * n + 255) / 256, ctx->num_sms * 8));
  gram_bad_pairs_kernel<<<g, 256, 0, ctx->stream>>>(n, Gh, tol, dp, cnt, cap);
  post_launch(ctx, "gram_bad_pairs_kernel");
  int hc = 0;
  LRA_CUDA(cudaMemcpyAsync(&hc, cnt, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  if (trace_on()) std::fprintf(stderr, "[lra] gram polish n=%lld: %d pairs above %.2e\n", (long long)n, hc, tol);
  if (hc <= 0 || hc > cap) {
    ctx->arena.release(mk);
    return false;
  }
  std::vector<int2> hp((size_t)hc);
  std::vector<double> hcos((size_t)hc);
  LRA_CUDA(cudaMemcpyAsync(hp.data(), dp, (size_t)hc * sizeof(int2), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  // the cosines, for the order (host copies of the few Gram entries involved)
  for (int i = 0; i < hc; ++i)
    LRA_CUDA(cudaMemcpyAsync(&hcos[(size_t)i], Gh + hp[(size_t)i].x + (int64_t)hp[(size_t)i].y * n, sizeof(double),
                             cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<int> ord((size_t)hc);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return std::fabs(hcos[(size_t)a]) > std::fabs(hcos[(size_t)b]); });
  std::vector<char> used((size_t)n);
  std::vector<char> done((size_t)hc, 0);
  int left = hc;
  for (int round = 0; left > 0 && round < 1024; ++round) {
    std::fill(used.begin(), used.end(), 0);
    std::vector<int2> sel;
    for (int i : ord) {
      if (done[(size_t)i]) continue;
      const int2 pq = hp[(size_t)i];
      if (used[(size_t)pq.x] || used[(size_t)pq.y]) continue;
      used[(size_t)pq.x] = used[(size_t)pq.y] = 1;
      done[(size_t)i] = 1;
      --left;
      sel.push_back(pq);
    }
    LRA_CUDA(cudaMemcpyAsync(dp, sel.data(), sel.size() * sizeof(int2), cudaMemcpyHostToDevice, ctx->stream));
    pair_rotate_kernel<<<(unsigned)sel.size(), 256, 0, ctx->stream>>>(n, X, ldx, Wacc, dp);
    post_launch(ctx, "pair_rotate_kernel");
    // sel is reused next round: the copy must have been read
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  ctx->arena.release(mk);
  return true;
}

bool gram_polish(lra_ctx* ctx, int64_t n, double* X, int64_t ldx, double* Wacc, double* S, double tol,
                 int max_iter) {
  const ArenaMark mk = ctx->arena.mark();
  const size_t nn = (size_t)n * n;
  double* Xh = ctx->arena.alloc_n<double>(nn);
  double* Gh = ctx->arena.alloc_n<double>(nn);
  double* Tm = ctx->arena.alloc_n<double>(nn);
  double* T2 = ctx->arena.alloc_n<double>(nn);
  double* W = ctx->arena.alloc_n<double>(nn);
  double* DW = ctx->arena.alloc_n<double>(nn);
  double* tmp = ctx->arena.alloc_n<double>(nn);
  double* Xs = ctx->arena.alloc_n<double>(nn);  // X and Wacc before the last update
  double* Ws = ctx->arena.alloc_n<double>(nn);
  unsigned long long* maxc = ctx->arena.alloc_n<unsigned long long>(3);
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>(((int64_t)nn + 255) / 256, ctx->num_sms * 8));
  bool ok = false;
  double prev = INFINITY;
  int cleanups = 0;
  bool last_cleanup = false;
  for (int it = 0; it <= max_iter; ++it) {
    col_norms<double>(ctx, n, n, X, ldx, S);
    unit_cols_kernel<<<g, 256, 0, ctx->stream>>>(n, X, ldx, S, Xh);
    post_launch(ctx, "unit_cols_kernel");
    gemm<double>(ctx, 't', 'n', n, n, n, 1.0, Xh, n, Xh, n, 0.0, Gh, n);
    LRA_CUDA(cudaMemsetAsync(maxc, 0, 3 * sizeof(unsigned long long), ctx->stream));
    gram_tangent_kernel<<<g, 256, 0, ctx->stream>>>(n, Gh, S, Tm, maxc);
    post_launch(ctx, "gram_tangent_kernel");
    unsigned long long hb[3] = {0, 0, 0};
    LRA_CUDA(cudaMemcpyAsync(hb, maxc, sizeof(hb), cudaMemcpyDeviceToHost, ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    double mc, ma, mt;
    std::memcpy(&mc, &hb[0], sizeof(mc));
    std::memcpy(&ma, &hb[1], sizeof(ma));
    std::memcpy(&mt, &hb[2], sizeof(mt));
    if (trace_on())
      std::fprintf(stderr, "[lra] gram polish n=%lld iteration %d: max cosine %.3e (rotating pairs %.3e)\n",
                   (long long)n, it, mc, ma);
    // progress: a simultaneous update is judged by the pairs it rotates
    // (pairs it leaves out keep their cosine), an exact cleanup by all pairs
    if (!std::isfinite(mc) || (last_cleanup ? mc > prev : ma > prev)) {
      // the last update did not help: back to the state before it
      if (it > 0) {
        copy_matrix(ctx, n, n, Xs, n, X, ldx);
        copy_matrix(ctx, n, n, Ws, n, Wacc, n);
        col_norms<double>(ctx, n, n, X, ldx, S);
      }
      break;
    }
    if (mc <= tol) {
      ok = true;
      break;
    }
    // only pairs of nearly equal norms are left: exact rotations of those
    // pairs when they are few (then the check again), else the pairwise
    // sweeps finish
    if (ma <= tol) {
      if (cleanups < 3 && it < max_iter) {
        prev = mc;
        copy_matrix(ctx, n, n, X, ldx, Xs, n);
        copy_matrix(ctx, n, n, Wacc, n, Ws, n);
        if (rotate_bad_pairs(ctx, n, X, ldx, Wacc, Gh, tol)) {
          ++cleanups;
          last_cleanup = true;
          continue;
        }
      }
      break;
    }
    if (it == max_iter) break;
    prev = ma;
    last_cleanup = false;
    copy_matrix(ctx, n, n, X, ldx, Xs, n);
    copy_matrix(ctx, n, n, Wacc, n, Ws, n);
    gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, Tm, n, Tm, n, 0.0, T2, n);
    gram_rotation_kernel<<<g, 256, 0, ctx->stream>>>(n, Tm, T2, W);
    post_launch(ctx, "gram_rotation_kernel");
    // the orthogonality defect T^4 / 4 matters from |t| ~ 1e-4 on
    const double* WT4 = nullptr;
    if (mt * mt * mt * mt > 4e-16) {
      gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, T2, n, T2, n, 0.0, Tm, n);  // T^4 (T is not needed again)
      gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, W, n, Tm, n, 0.0, Gh, n);   // W T^4
      WT4 = Gh;
    }
    gram_finish_kernel<<<g, 256, 0, ctx->stream>>>(n, WT4, S, W, DW);
    post_launch(ctx, "gram_finish_kernel");
    gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, Xh, n, DW, n, 0.0, tmp, n);
    copy_matrix(ctx, n, n, tmp, n, X, ldx);
    gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, Wacc, n, W, n, 0.0, tmp, n);
    copy_matrix(ctx, n, n, tmp, n, Wacc, n);
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return ok;
}

template <typename T>
void jacobi_svd_fast(lra_ctx* ctx, int64_t n, T* X, int64_t ldx, T* V, int64_t ldv, T* S) {
  if (sizeof(T) != 8 || n < 64) {
    jacobi_svd<T>(ctx, n, X, ldx, V, ldv, S);
    return;
  }
  // The polish runs in double-float on the mixed path when its rtol leaves
  // room for the ~1e-13 orthogonality that gives; there the GEMMs below may
  // use the tensor cores.  Otherwise W must come out orthonormal to FP64
  // rounding and the GEMMs stay in FP64.
  const bool df_polish = sizeof(T) == 8 && ctx->mixed_rtol >= 1e-12;
  const bool saved_tc = ctx->gemm_tc;
  if (!df_polish) ctx->gemm_tc = false;
  struct Restore {
    lra_ctx* c;
    bool v;
    ~Restore() { c->gemm_tc = v; }
  } restore{ctx, saved_tc};
  const ArenaMark mk = ctx->arena.mark();
  // 1. FP32 sweeps on X scaled by a power of two into FP32's range (the
  //    rotations do not depend on the scale)
  double scale = 1.0;
  {
    unsigned long long* mx = ctx->arena.alloc_n<unsigned long long>(1);
    LRA_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), ctx->stream));
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * n + 255) / 256, ctx->num_sms * 4));
    absmax_bits_kernel<T><<<g, 256, 0, ctx->stream>>>(n, n, X, ldx, mx);
    post_launch(ctx, "absmax_bits_kernel");
    unsigned long long hb = 0;
    LRA_CUDA(cudaMemcpyAsync(&hb, mx, sizeof(hb), cudaMemcpyDeviceToHost, ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    double hm;
    std::memcpy(&hm, &hb, sizeof(hm));
    if (!(hm > 0) || !std::isfinite(hm)) {
      // nothing to rotate, or not a finite matrix: the FP64 sweeps handle it
      ctx->arena.release(mk);
      jacobi_svd<T>(ctx, n, X, ldx, V, ldv, S);
      return;
    }
    scale = std::ldexp(1.0, -std::ilogb(hm));
  }
  // leading dimension a multiple of 4 floats: the Jacobi kernels move whole
  // 16-byte vectors of a column
  const int64_t ld32 = (n + 3) & ~(int64_t)3;
  float* X32 = ctx->arena.alloc_n<float>((size_t)ld32 * n);
  float* V32 = ctx->arena.alloc_n<float>((size_t)ld32 * n);
  float* S32 = ctx->arena.alloc_n<float>(n);
  cast<T, float>(ctx, n, n, X, ldx, X32, ld32, scale);
  // the Gram polish converges quadratically from cosines of a few 1e-3 (the
  // FP32 sweeps stop there); the pairwise FP64 sweeps want them near 1e-6
  // (neighbouring singular values of a smooth spectrum of n are ~1/n apart
  // relative to each other, and the simultaneous rotations converge only
  // from cosines below that gap: the start level falls with n)
  const double start = ctx->tuning.gram_start > 0 ? 1e-4 * ctx->tuning.gram_start : std::min(kGramStart, 12.0 / (double)n);
  jacobi_svd<float>(ctx, n, X32, ld32, V32, ld32, S32, true, df_polish ? start : 0.0);
  // 2. the rotation in FP64, re-orthonormalized by two Newton-Schulz steps
  //    W <- W (3 I - W'W) / 2: with |I - W'W| near 1e-6 from the FP32
  //    sweeps the error squares each step, to rounding level after two
  T* W = ctx->arena.alloc_n<T>((size_t)n * n);
  T* G = ctx->arena.alloc_n<T>((size_t)n * n);
  T* W2 = ctx->arena.alloc_n<T>((size_t)n * n);
  cast<float, T>(ctx, n, n, V32, ld32, W, n);
  for (int it = 0; it < 2; ++it) {
    gemm<T>(ctx, 't', 'n', n, n, n, T(1), W, n, W, n, T(0), G, n);
    copy_matrix(ctx, n, n, W, n, W2, n);
    gemm<T>(ctx, 'n', 'n', n, n, n, T(-0.5), W, n, G, n, T(1.5), W2, n);
    std::swap(W, W2);
  }
  // 3. X <- X W, FP64 sweeps, V = W V2
  T* Y = ctx->arena.alloc_n<T>((size_t)n * n);
  gemm<T>(ctx, 'n', 'n', n, n, n, T(1), X, ldx, W, n, T(0), Y, n);
  copy_matrix(ctx, n, n, Y, n, X, ldx);
  // Y <- V2: the Gram polish on the mixed path, pairwise double-float sweeps
  // after it when it did not converge, FP64 sweeps otherwise
  bool done = false;
  if constexpr (sizeof(T) == 8)
    if (df_polish) {
      double* Xd = reinterpret_cast<double*>(X);
      double* Yd = reinterpret_cast<double*>(Y);
      const double tol =
          std::max((double)Real<double>::eps * 2.0 * std::sqrt((double)n), 8.0 * std::ldexp(1.0, -46) * std::sqrt((double)n));
      set_identity(ctx, n, n, Yd, n);
      done = gram_polish(ctx, n, Xd, ldx, Yd, reinterpret_cast<double*>(S), tol, n > 1024 ? 8 : 5);
      if (!done) {
        double* Y2 = reinterpret_cast<double*>(W2);
        done = jacobi_svd_df(ctx, n, Xd, ldx, Y2, n, reinterpret_cast<double*>(S));
        if (!done) jacobi_svd<double>(ctx, n, Xd, ldx, Y2, n, reinterpret_cast<double*>(S), true);
        double* Gd = reinterpret_cast<double*>(G);
        gemm<double>(ctx, 'n', 'n', n, n, n, 1.0, Yd, n, Y2, n, 0.0, Gd, n);
        copy_matrix(ctx, n, n, Gd, n, Yd, n);
        done = true;
      }
    }
  if (!done) jacobi_svd<T>(ctx, n, X, ldx, Y, n, S, true);
  gemm<T>(ctx, 'n', 'n', n, n, n, T(1), W, n, Y, n, T(0), V, ldv);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
}

template void jacobi_svd_fast<float>(lra_ctx*, int64_t, float*, int64_t, float*, int64_t, float*);
template void jacobi_svd_fast<double>(lra_ctx*, int64_t, double*, int64_t, double*, int64_t, double*);

}  // namespace lra
