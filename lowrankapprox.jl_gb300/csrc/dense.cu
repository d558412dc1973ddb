// Small dense factorizations of the post-processing stages, FP64 (input
// precision) on CUDA cores:
//   - one-sided (Hestenes) Jacobi SVD of a square k x k matrix, used for the
//     core SVD of psvdfact (src/psvd.jl:245) after a QR of (R V)^T, and --
//     on the shifted positive semidefinite B + s I -- for the k x k Hermitian
//     eigenproblem of pheigfact (src/pheig.jl:284);
//   - a symmetry test (ishermitian on a dense real matrix).
// One cooperative launch runs all sweeps: each round of the round-robin
// ordering rotates n/2 disjoint column pairs in parallel (one warp per
// pair), separated by bounded grid barriers.

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename T>
struct JacParams {
  int64_t n;
  T* X;
  int64_t ldx;
  T* V;
  int64_t ldv;
  T* S;
  double tol;
  double stop;  // a sweep whose largest rotated cosine is below this is the last
  int max_sweeps;
  double* part;
  GridBar* bar;
  int* sweeps_out;
};

constexpr int JCH = 16;  // rows per lane per register chunk (512 rows)

__device__ __forceinline__ void rr_pair(int64_t r, int64_t s, int64_t nn, int64_t& p, int64_t& q) {
  auto pos = [&](int64_t i) -> int64_t { return i == 0 ? 0 : 1 + (i - 1 + r) % (nn - 1); };
  p = pos(s);
  q = pos(nn - 1 - s);
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) jacobi_kernel(JacParams<T> P) {
  __shared__ double red[32];
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * NW + wid;
  const int64_t W = (int64_t)gridDim.x * NW;
  const int64_t n = P.n;
  const int64_t nn = n + (n & 1);
  int sweep = 0;
  for (; sweep < P.max_sweeps; ++sweep) {
    double off = 0;
    for (int64_t r = 0; r < nn - 1; ++r) {
      for (int64_t s = gw; s < nn / 2; s += W) {
        int64_t p, q;
        rr_pair(r, s, nn, p, q);
        if (p >= n || q >= n) continue;
        if (p > q) {
          const int64_t t = p;
          p = q;
          q = t;
        }
        T* xp = P.X + p * P.ldx;
        T* xq = P.X + q * P.ldx;
        // both columns are pulled into registers with independent loads
        // (one L2 round trip per chunk), reduced, rotated and stored
        T a = 0, b = 0, g = 0;
        T u[JCH], w[JCH];
        const bool one = n <= 32 * JCH;
        for (int64_t b0 = 0; b0 < n; b0 += 32 * JCH) {
#pragma unroll
          for (int t = 0; t < JCH; ++t) {
            const int64_t i = b0 + lane + 32 * t;
            u[t] = i < n ? __ldcg(xp + i) : T(0);
            w[t] = i < n ? __ldcg(xq + i) : T(0);
          }
#pragma unroll
          for (int t = 0; t < JCH; ++t) {
            a = fma(u[t], u[t], a);
            b = fma(w[t], w[t], b);
            g = fma(u[t], w[t], g);
          }
        }
        a = warp_sum(a);
        b = warp_sum(b);
        g = warp_sum(g);
        if (a == 0 || b == 0) continue;
        const T rel = fabs(g) / sqrt(a * b);
        if (!(rel > (T)P.tol)) continue;
        off = fmax(off, (double)rel);
        const T zeta = (b - a) / (T(2) * g);
        const T t = copysign(T(1), zeta) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
        const T c = T(1) / sqrt(T(1) + t * t);
        const T sn = c * t;
        for (int64_t b0 = 0; b0 < n; b0 += 32 * JCH) {
          if (!one) {
#pragma unroll
            for (int tt = 0; tt < JCH; ++tt) {
              const int64_t i = b0 + lane + 32 * tt;
              u[tt] = i < n ? __ldcg(xp + i) : T(0);
              w[tt] = i < n ? __ldcg(xq + i) : T(0);
            }
          }
#pragma unroll
          for (int tt = 0; tt < JCH; ++tt) {
            const int64_t i = b0 + lane + 32 * tt;
            if (i < n) {
              xp[i] = c * u[tt] - sn * w[tt];
              xq[i] = sn * u[tt] + c * w[tt];
            }
          }
        }
        T* vp = P.V + p * P.ldv;
        T* vq = P.V + q * P.ldv;
        for (int64_t b0 = 0; b0 < n; b0 += 32 * JCH) {
#pragma unroll
          for (int tt = 0; tt < JCH; ++tt) {
            const int64_t i = b0 + lane + 32 * tt;
            u[tt] = i < n ? __ldcg(vp + i) : T(0);
            w[tt] = i < n ? __ldcg(vq + i) : T(0);
          }
#pragma unroll
          for (int tt = 0; tt < JCH; ++tt) {
            const int64_t i = b0 + lane + 32 * tt;
            if (i < n) {
              vp[i] = c * u[tt] - sn * w[tt];
              vq[i] = sn * u[tt] + c * w[tt];
            }
          }
        }
      }
      if (!grid_sync(P.bar)) return;
    }
    off = block_max(off, red);
    if (threadIdx.x == 0) P.part[blockIdx.x] = off;
    if (!grid_sync(P.bar)) return;
    double mx = 0;
    for (int b = threadIdx.x; b < gridDim.x; b += NT) mx = fmax(mx, __ldcg(P.part + b));
    mx = block_max(mx, red);
    if (!grid_sync(P.bar)) return;  // everyone read part before it is rewritten
    if (mx <= P.stop) {
      ++sweep;
      break;
    }
  }
  // singular values = column norms
  for (int64_t j = gw; j < n; j += W) {
    const T* x = P.X + j * P.ldx;
    double a = 0;
    for (int64_t i = lane; i < n; i += 32) {
      const double u = __ldcg(x + i);
      a = fma(u, u, a);
    }
    a = warp_sum(a);
    if (lane == 0) P.S[j] = (T)sqrt(a);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.sweeps_out = sweep;
}

// One CTA per column pair for Float64: the rows of the two columns are
// spread over all threads of the CTA (a warp-wide FP64 instruction costs
// tens of cycles on this part, so fewer rows per thread shorten every
// dependent chain), the three dot products are reduced through shared
// memory, and the rotation test g^2 > tol^2 a b needs no division or
// square root.
constexpr int JP_RCH = 8;  // rows per thread per register chunk

template <typename T, int NT>
__global__ void __launch_bounds__(NT) jacobi_pair_kernel(JacParams<T> P) {
  constexpr int NW = NT / 32;
  __shared__ T red[2][NW][3];
  __shared__ int s_flag;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t n = P.n;
  const int64_t nn = n + (n & 1);
  const T tol2 = (T)(P.tol * P.tol), stop2 = (T)(P.stop * P.stop);
  int sweep = 0;
  int buf = 0;
  for (; sweep < P.max_sweeps; ++sweep) {
    int above = 0;  // a pair of this CTA had a cosine above the stopping level
    for (int64_t r = 0; r < nn - 1; ++r) {
      for (int64_t s = blockIdx.x; s < nn / 2; s += gridDim.x) {
        int64_t p, q;
        rr_pair(r, s, nn, p, q);
        if (p >= n || q >= n) continue;
        if (p > q) {
          const int64_t t = p;
          p = q;
          q = t;
        }
        T* xp = P.X + p * P.ldx;
        T* xq = P.X + q * P.ldx;
        T a = 0, b = 0, g = 0;
        T u[JP_RCH], w[JP_RCH];
        const bool one = n <= (int64_t)NT * JP_RCH;
        for (int64_t b0 = 0; b0 < n; b0 += (int64_t)NT * JP_RCH) {
#pragma unroll
          for (int c = 0; c < JP_RCH; ++c) {
            if (b0 + (int64_t)NT * c >= n) break;
            const int64_t i = b0 + threadIdx.x + (int64_t)NT * c;
            u[c] = i < n ? __ldcg(xp + i) : T(0);
            w[c] = i < n ? __ldcg(xq + i) : T(0);
          }
#pragma unroll
          for (int c = 0; c < JP_RCH; ++c) {
            if (b0 + (int64_t)NT * c >= n) break;
            a = fma(u[c], u[c], a);
            b = fma(w[c], w[c], b);
            g = fma(u[c], w[c], g);
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          a += __shfl_xor_sync(0xffffffffu, a, o);
          b += __shfl_xor_sync(0xffffffffu, b, o);
          g += __shfl_xor_sync(0xffffffffu, g, o);
        }
        if (lane == 0) {
          red[buf][wid][0] = a;
          red[buf][wid][1] = b;
          red[buf][wid][2] = g;
        }
        __syncthreads();
        a = red[buf][0][0];
        b = red[buf][0][1];
        g = red[buf][0][2];
#pragma unroll
        for (int k = 1; k < NW; ++k) {
          a += red[buf][k][0];
          b += red[buf][k][1];
          g += red[buf][k][2];
        }
        buf ^= 1;  // the next pair reduces through the other buffer
        if (a == 0 || b == 0) continue;
        const T g2 = g * g, ab = a * b;
        if (!(g2 > tol2 * ab)) continue;
        if (g2 > stop2 * ab) above = 1;
        // t = tan of the rotation angle, the smaller root of t^2 + 2 zeta t - 1
        const T d = b - a;
        const T t = (T(2) * g) / (d + copysign(sqrt(fma(d, d, T(4) * g2)), d));
        const T c = T(1) / sqrt(fma(t, t, T(1)));
        const T sn = c * t;
        for (int64_t b0 = 0; b0 < n; b0 += (int64_t)NT * JP_RCH) {
          if (!one) {
#pragma unroll
            for (int cc = 0; cc < JP_RCH; ++cc) {
              if (b0 + (int64_t)NT * cc >= n) break;
              const int64_t i = b0 + threadIdx.x + (int64_t)NT * cc;
              u[cc] = i < n ? __ldcg(xp + i) : T(0);
              w[cc] = i < n ? __ldcg(xq + i) : T(0);
            }
          }
#pragma unroll
          for (int cc = 0; cc < JP_RCH; ++cc) {
            if (b0 + (int64_t)NT * cc >= n) break;
            const int64_t i = b0 + threadIdx.x + (int64_t)NT * cc;
            if (i < n) {
              xp[i] = c * u[cc] - sn * w[cc];
              xq[i] = sn * u[cc] + c * w[cc];
            }
          }
        }
        T* vp = P.V + p * P.ldv;
        T* vq = P.V + q * P.ldv;
        for (int64_t b0 = 0; b0 < n; b0 += (int64_t)NT * JP_RCH) {
#pragma unroll
          for (int cc = 0; cc < JP_RCH; ++cc) {
            if (b0 + (int64_t)NT * cc >= n) break;
            const int64_t i = b0 + threadIdx.x + (int64_t)NT * cc;
            u[cc] = i < n ? __ldcg(vp + i) : T(0);
            w[cc] = i < n ? __ldcg(vq + i) : T(0);
          }
#pragma unroll
          for (int cc = 0; cc < JP_RCH; ++cc) {
            if (b0 + (int64_t)NT * cc >= n) break;
            const int64_t i = b0 + threadIdx.x + (int64_t)NT * cc;
            if (i < n) {
              vp[i] = c * u[cc] - sn * w[cc];
              vq[i] = sn * u[cc] + c * w[cc];
            }
          }
        }
      }
      if (!grid_sync(P.bar)) return;
    }
    // any CTA above the stopping level keeps the sweeps going
    if (threadIdx.x == 0) P.part[blockIdx.x] = above ? 1.0 : 0.0;
    if (!grid_sync(P.bar)) return;
    if (threadIdx.x == 0) {
      int any = 0;
      for (int k = 0; k < (int)gridDim.x; ++k) any |= __ldcg(P.part + k) != 0.0;
      s_flag = any;
    }
    __syncthreads();
    const int any = s_flag;
    if (!grid_sync(P.bar)) return;  // everyone read part before it is rewritten
    if (!any) {
      ++sweep;
      break;
    }
  }
  // singular values = column norms, a warp per column
  const int64_t gw = (int64_t)blockIdx.x * NW + wid, W = (int64_t)gridDim.x * NW;
  for (int64_t j = gw; j < n; j += W) {
    const T* x = P.X + j * P.ldx;
    double acc = 0;
    for (int64_t i = lane; i < n; i += 32) {
      const double v = __ldcg(x + i);
      acc = fma(v, v, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) P.S[j] = (T)sqrt(acc);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.sweeps_out = sweep;
}

template <typename T>
__global__ void symcheck_kernel(int64_t n, const T* __restrict__ A, int64_t lda, int* bad) {
  const int64_t total = n * n;
  int local = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    if (i < j && A[i + j * lda] != A[j + i * lda]) local = 1;
  }
  if (__syncthreads_or(local) && threadIdx.x == 0) atomicExch(bad, 1);
}

}  // namespace

template <typename T>
void jacobi_svd(lra_ctx* ctx, int64_t n, T* X, int64_t ldx, T* V, int64_t ldv, T* S, bool quadratic_stop) {
  // Float64: a CTA of 128 threads per pair; Float32: a warp per pair
  constexpr bool pair_cta = sizeof(T) == 8;
  constexpr int NT = 128;
  if (n <= 0) return;
  set_identity(ctx, n, n, V, ldv);
  const ArenaMark mk = ctx->arena.mark();
  const void* kern = pair_cta ? (const void*)jacobi_pair_kernel<T, NT> : (const void*)jacobi_kernel<T, NT>;
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NT, 0));
  const int64_t pairs = (n + 1) / 2;
  const int64_t per_cta = pair_cta ? 1 : NT / 32;
  int grid = (int)std::min<int64_t>((pairs + per_cta - 1) / per_cta, (int64_t)ctx->num_sms);
  grid = std::max(1, std::min(grid, ctx->num_sms * std::max(per_sm, 1)));
  JacParams<T> P;
  P.n = n;
  P.X = X;
  P.ldx = ldx;
  P.V = V;
  P.ldv = ldv;
  P.S = S;
  P.tol = (double)Real<T>::eps * 2.0 * std::sqrt((double)n);
  // Started from columns already orthogonal to about 1e-7 (the FP32 sweeps
  // of jacobi_svd_fast), the FP64 sweeps converge quadratically: a sweep
  // whose cosines were all below sqrt(tol)/10 leaves them near tol^2/100
  // times a modest gap factor, so no further sweep is needed.
  P.stop = quadratic_stop ? std::sqrt(P.tol) * 0.1 : P.tol;
  P.max_sweeps = 40;
  P.part = ctx->arena.alloc_n<double>(grid);
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.sweeps_out = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  void* args[] = {&P};
  LRA_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(NT), args, 0, ctx->stream));
  post_launch(ctx, pair_cta ? "jacobi_pair_kernel" : "jacobi_kernel");
  GridBar hb;
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "jacobi: a grid barrier timed out");
}

template <typename T>
bool is_symmetric(lra_ctx* ctx, int64_t n, const T* A, int64_t lda) {
  const ArenaMark mk = ctx->arena.mark();
  int* bad = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * n + 255) / 256, (int64_t)ctx->num_sms * 16));
  symcheck_kernel<T><<<g, 256, 0, ctx->stream>>>(n, A, lda, bad);
  post_launch(ctx, "symcheck_kernel");
  int h = 0;
  LRA_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return h == 0;
}

template void jacobi_svd<float>(lra_ctx*, int64_t, float*, int64_t, float*, int64_t, float*, bool);
template void jacobi_svd<double>(lra_ctx*, int64_t, double*, int64_t, double*, int64_t, double*, bool);
template bool is_symmetric<float>(lra_ctx*, int64_t, const float*, int64_t);
template bool is_symmetric<double>(lra_ctx*, int64_t, const double*, int64_t);

}  // namespace lra

// ---- blocked Cholesky and right triangular solve ----------------------------------
// Used by the sketch-preconditioned Cholesky QR of the post-processing: the
// skeleton columns A[:, sk] times R11^{-1} (R11 from the pivoted QR of the
// sketch) are well conditioned, so their Gram matrix factors stably.

namespace lra {

namespace {

constexpr int CB = 32;  // diagonal block size

// upper Cholesky of the jb x jb diagonal block in place (one CTA); sets *bad
// when the block is not positive definite
template <typename T>
__global__ void potrf_diag_kernel(int jb, T* G, int64_t ldg, int* bad) {
  __shared__ T a[CB][CB + 1];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    a[i][j] = G[i + j * ldg];
  }
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    // a[c][c] <- sqrt(a[c][c] - sum_{r<c} a[r][c]^2); a[c][j] <- (...)/a[c][c]
    if (threadIdx.x == 0) {
      T d = a[c][c];
      for (int r = 0; r < c; ++r) d -= a[r][c] * a[r][c];
      if (!(d > T(0))) {
        atomicExch(bad, 1);
        d = T(1);
      }
      a[c][c] = sqrt(d);
    }
    __syncthreads();
    for (int j = c + 1 + threadIdx.x; j < jb; j += blockDim.x) {
      T s = a[c][j];
      for (int r = 0; r < c; ++r) s -= a[r][c] * a[r][j];
      a[c][j] = s / a[c][c];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    G[i + j * ldg] = i <= j ? a[i][j] : T(0);
  }
}

// panel: R_{b, >b} = R_bb^{-T} G_{b, >b} (jb x nc), one thread per column
template <typename T>
__global__ void potrf_panel_kernel(int jb, int64_t nc, const T* Rbb, int64_t ldr, T* P, int64_t ldp) {
  __shared__ T r[CB][CB + 1];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  __syncthreads();
  for (int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; col < nc; col += (int64_t)gridDim.x * blockDim.x) {
    T* p = P + col * ldp;
    T x[CB];
#pragma unroll
    for (int i = 0; i < CB; ++i)
      if (i < jb) x[i] = p[i];
#pragma unroll
    for (int i = 0; i < CB; ++i) {
      if (i < jb) {
        T s = x[i];
#pragma unroll
        for (int q = 0; q < CB; ++q)
          if (q < i) s -= r[q][i] * x[q];
        x[i] = s / r[i][i];
      }
    }
#pragma unroll
    for (int i = 0; i < CB; ++i)
      if (i < jb) p[i] = x[i];
  }
}

// X_b <- X_b R_bb^{-1} (m x jb), one thread per row
template <typename T>
__global__ void trsm_right_diag_kernel(int64_t m, int jb, const T* Rbb, int64_t ldr, T* X, int64_t ldx) {
  __shared__ T r[CB][CB + 1];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  __syncthreads();
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < m; row += (int64_t)gridDim.x * blockDim.x) {
    T x[CB];
#pragma unroll
    for (int j = 0; j < CB; ++j)
      if (j < jb) x[j] = X[row + j * ldx];
    // x R = b: x_j = (b_j - sum_{i<j} x_i R_ij) / R_jj
#pragma unroll
    for (int j = 0; j < CB; ++j) {
      if (j < jb) {
        T s = x[j];
#pragma unroll
        for (int i = 0; i < CB; ++i)
          if (i < j) s -= x[i] * r[i][j];
        x[j] = s / r[j][j];
      }
    }
#pragma unroll
    for (int j = 0; j < CB; ++j)
      if (j < jb) X[row + j * ldx] = x[j];
  }
}

// X[0:jb, :] <- Rbb^{-1} X[0:jb, :] for an upper-triangular jb x jb block
template <typename T>
__global__ void trsm_left_diag_kernel(int jb, int64_t nrhs, const T* Rbb, int64_t ldr, T* X, int64_t ldx) {
  __shared__ T r[CB][CB + 1];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  __syncthreads();
  for (int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; col < nrhs;
       col += (int64_t)gridDim.x * blockDim.x) {
    T* xc = X + col * ldx;
    T x[CB];
#pragma unroll
    for (int i = 0; i < CB; ++i)
      if (i < jb) x[i] = xc[i];
    // R x = b: x_i = (b_i - sum_{q>i} R_iq x_q) / R_ii, bottom up
#pragma unroll
    for (int i = CB - 1; i >= 0; --i) {
      if (i < jb) {
        T s = x[i];
#pragma unroll
        for (int q = CB - 1; q > i; --q)
          if (q < jb) s -= r[i][q] * x[q];
        x[i] = s / r[i][i];
      }
    }
#pragma unroll
    for (int i = 0; i < CB; ++i)
      if (i < jb) xc[i] = x[i];
  }
}

}  // namespace

template <typename T>
bool potrf_upper(lra_ctx* ctx, int64_t k, T* G, int64_t ldg) {
  if (k <= 0) return true;
  const ArenaMark mk = ctx->arena.mark();
  int* bad = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  for (int64_t j0 = 0; j0 < k; j0 += CB) {
    const int jb = (int)std::min<int64_t>(CB, k - j0);
    T* Gjj = G + j0 + j0 * ldg;
    potrf_diag_kernel<T><<<1, 256, 0, ctx->stream>>>(jb, Gjj, ldg, bad);
    post_launch(ctx, "potrf_diag_kernel");
    const int64_t rest = k - j0 - jb;
    if (rest > 0) {
      T* P = G + j0 + (j0 + jb) * ldg;
      const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((rest + 127) / 128, ctx->num_sms * 4));
      potrf_panel_kernel<T><<<g, 128, 0, ctx->stream>>>(jb, rest, Gjj, ldg, P, ldg);
      post_launch(ctx, "potrf_panel_kernel");
      // trailing: G_{>b,>b} -= P^T P
      T* Gt = G + (j0 + jb) + (j0 + jb) * ldg;
      gemm<T>(ctx, 't', 'n', rest, rest, jb, T(-1), P, ldg, P, ldg, T(1), Gt, ldg);
    }
  }
  zero_lower(ctx, k, k, G, ldg);  // the factor is used as a dense matrix later
  int h = 0;
  LRA_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return h == 0;
}

template <typename T>
void trsm_left_diag(lra_ctx* ctx, int jb, int64_t nrhs, const T* R, int64_t ldr, T* X, int64_t ldx) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nrhs + 127) / 128, ctx->num_sms * 8));
  trsm_left_diag_kernel<T><<<g, 128, 0, ctx->stream>>>(jb, nrhs, R, ldr, X, ldx);
  post_launch(ctx, "trsm_left_diag_kernel");
}

// X <- X triu(R)^{-1}, recursive like trsm_upper: the leading half, a GEMM
// update of the trailing columns, the trailing half
template <typename T>
void trsm_right_upper(lra_ctx* ctx, int64_t m, int64_t k, const T* R, int64_t ldr, T* X, int64_t ldx) {
  if (m <= 0 || k <= 0) return;
  if (k <= CB) {
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 127) / 128, ctx->num_sms * 8));
    trsm_right_diag_kernel<T><<<g, 128, 0, ctx->stream>>>(m, (int)k, R, ldr, X, ldx);
    post_launch(ctx, "trsm_right_diag_kernel");
    return;
  }
  const int64_t k1 = (k / 2 + CB - 1) / CB * CB, k2 = k - k1;
  trsm_right_upper(ctx, m, k1, R, ldr, X, ldx);
  gemm<T>(ctx, 'n', 'n', m, k2, k1, T(-1), X, ldx, R + k1 * ldr, ldr, T(1), X + k1 * ldx, ldx);
  trsm_right_upper(ctx, m, k2, R + k1 + k1 * ldr, ldr, X + k1 * ldx, ldx);
}

template bool potrf_upper<float>(lra_ctx*, int64_t, float*, int64_t);
template bool potrf_upper<double>(lra_ctx*, int64_t, double*, int64_t);
template void trsm_right_upper<float>(lra_ctx*, int64_t, int64_t, const float*, int64_t, float*, int64_t);
template void trsm_right_upper<double>(lra_ctx*, int64_t, int64_t, const double*, int64_t, double*, int64_t);
template void trsm_left_diag<float>(lra_ctx*, int, int64_t, const float*, int64_t, float*, int64_t);
template void trsm_left_diag<double>(lra_ctx*, int, int64_t, const double*, int64_t, double*, int64_t);

}  // namespace lra
