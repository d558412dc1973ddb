// Column-major GEMM on CUDA cores, C = alpha op(A) op(B) + beta C, for the
// input-precision ("native") path.  On GB300 the FP64 rate is the bound of
// this kernel, which a register-tiled SIMT kernel reaches comfortably; the
// split-precision tensor-core path lives in tc_sketch.cu.

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;
constexpr int NT = (BM / TM) * (BN / TN);  // 256

// blockIdx.y selects a K slice of length kchunk; with gridDim.y > 1 each
// slice writes its own partial product to C + y * ldc * N (split-K)
template <typename T, bool TA, bool TB>
__global__ void __launch_bounds__(NT) gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha,
                                                  const T* __restrict__ A, int64_t lda,
                                                  const T* __restrict__ B, int64_t ldb, T beta,
                                                  T* __restrict__ C, int64_t ldc, int64_t kchunk) {
  {
    const int64_t k0 = (int64_t)blockIdx.y * kchunk;
    if (k0 >= K) return;
    K = min(K - k0, kchunk);
    A += TA ? k0 : k0 * lda;
    B += TB ? k0 * ldb : k0;
    C += (int64_t)blockIdx.y * ldc * N;
  }
  __shared__ T As[2][BK][BM + 1];
  __shared__ T Bs[2][BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % (BN / TN), ty = tid / (BN / TN);
  const int64_t tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;

  for (int64_t tile = blockIdx.x; tile < tiles_m * tiles_n; tile += gridDim.x) {
    const int64_t m0 = (tile % tiles_m) * BM, n0 = (tile / tiles_m) * BN;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

    T ra[(BM * BK) / NT], rb[(BN * BK) / NT];
    auto load = [&](int64_t k0) {
#pragma unroll
      for (int r = 0; r < (BM * BK) / NT; ++r) {
        int i, k;
        if (!TA) {
          i = tid % BM;
          k = tid / BM + r * (NT / BM);
        } else {
          k = tid % BK;
          i = tid / BK + r * (NT / BK);
        }
        const int64_t gi = m0 + i, gk = k0 + k;
        T v = T(0);
        if (gi < M && gk < K) v = TA ? A[gk + gi * lda] : A[gi + gk * lda];
        ra[r] = v;
      }
#pragma unroll
      for (int r = 0; r < (BN * BK) / NT; ++r) {
        int j, k;
        if (!TB) {
          k = tid % BK;
          j = tid / BK + r * (NT / BK);
        } else {
          j = tid % BN;
          k = tid / BN + r * (NT / BN);
        }
        const int64_t gj = n0 + j, gk = k0 + k;
        T v = T(0);
        if (gj < N && gk < K) v = TB ? B[gj + gk * ldb] : B[gk + gj * ldb];
        rb[r] = v;
      }
    };
    auto store = [&](int buf) {
#pragma unroll
      for (int r = 0; r < (BM * BK) / NT; ++r) {
        int i, k;
        if (!TA) {
          i = tid % BM;
          k = tid / BM + r * (NT / BM);
        } else {
          k = tid % BK;
          i = tid / BK + r * (NT / BK);
        }
        As[buf][k][i] = ra[r];
      }
#pragma unroll
      for (int r = 0; r < (BN * BK) / NT; ++r) {
        int j, k;
        if (!TB) {
          k = tid % BK;
          j = tid / BK + r * (NT / BK);
        } else {
          j = tid % BN;
          k = tid / BN + r * (NT / BN);
        }
        Bs[buf][k][j] = rb[r];
      }
    };

    int buf = 0;
    load(0);
    store(0);
    __syncthreads();
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
      const bool more = k0 + BK < K;
      if (more) load(k0 + BK);
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][ty + i * (BM / TM)];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[buf][kk][tx + j * (BN / TN)];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
      }
      if (more) {
        store(buf ^ 1);
        __syncthreads();
        buf ^= 1;
      }
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t gi = m0 + ty + i * (BM / TM);
      if (gi >= M) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t gj = n0 + tx + j * (BN / TN);
        if (gj >= N) continue;
        T* c = C + gi + gj * ldc;
        *c = (beta == T(0)) ? alpha * acc[i][j] : alpha * acc[i][j] + beta * *c;
      }
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void splitk_reduce_kernel(int64_t m, int64_t n, int64_t nsplit, const T* __restrict__ W, T alpha, T beta,
                                     T* __restrict__ C, int64_t ldc) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    T s = 0;
    for (int64_t q = 0; q < nsplit; ++q) s += W[q * total + t];
    T* c = C + i + j * ldc;
    *c = (beta == T(0)) ? alpha * s : alpha * s + beta * *c;
  }
}

template <typename T>
__global__ void scale_kernel(int64_t m, int64_t n, T beta, T* C, int64_t ldc) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    C[i + j * ldc] = beta == T(0) ? T(0) : beta * C[i + j * ldc];
  }
}

}  // namespace

template <typename T>
void gemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, T alpha, const T* A,
          int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc) {
  if (m <= 0 || n <= 0) return;
  if (k <= 0) {
    const unsigned g = (unsigned)std::min<int64_t>((m * n + 255) / 256, (int64_t)ctx->num_sms * 8);
    scale_kernel<T><<<std::max(g, 1u), 256, 0, ctx->stream>>>(m, n, beta, C, ldc);
    post_launch(ctx, "scale_kernel");
    return;
  }
  if constexpr (sizeof(T) == 8) {
    if (ctx->gemm_tc && tc_gemm_worthwhile(m, n, k)) {
      tc_gemm(ctx, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
      return;
    }
  }
  const bool TA = (ta == 't' || ta == 'T' || ta == 'c' || ta == 'C');
  const bool TB = (tb == 't' || tb == 'T' || tb == 'c' || tb == 'C');
  const int64_t tiles = ((m + BM - 1) / BM) * ((n + BN - 1) / BN);
  const unsigned g = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 4);
  // split K when the tiles alone leave most SMs idle
  int64_t nsplit = 1;
  if (tiles < ctx->num_sms && k >= 1024)
    nsplit = std::min<int64_t>((2 * ctx->num_sms + tiles - 1) / tiles, k / 256);
  const int64_t kchunk = (k + nsplit - 1) / nsplit;
  nsplit = (k + kchunk - 1) / kchunk;
  T* out = C;
  int64_t ldo = ldc;
  T al = alpha, be = beta;
  const ArenaMark mk = ctx->arena.mark();
  if (nsplit > 1) {
    out = ctx->arena.alloc_n<T>((size_t)nsplit * m * n);
    ldo = m;
    al = T(1);
    be = T(0);
  }
  const dim3 grid(g, (unsigned)nsplit);
  if (!TA && !TB)
    gemm_kernel<T, false, false><<<grid, NT, 0, ctx->stream>>>(m, n, k, al, A, lda, B, ldb, be, out, ldo, kchunk);
  else if (TA && !TB)
    gemm_kernel<T, true, false><<<grid, NT, 0, ctx->stream>>>(m, n, k, al, A, lda, B, ldb, be, out, ldo, kchunk);
  else if (!TA && TB)
    gemm_kernel<T, false, true><<<grid, NT, 0, ctx->stream>>>(m, n, k, al, A, lda, B, ldb, be, out, ldo, kchunk);
  else
    gemm_kernel<T, true, true><<<grid, NT, 0, ctx->stream>>>(m, n, k, al, A, lda, B, ldb, be, out, ldo, kchunk);
  if (nsplit > 1) {
    post_launch(ctx, "gemm_kernel");
    const unsigned gr = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m * n + 255) / 256, ctx->num_sms * 8));
    splitk_reduce_kernel<T><<<gr, 256, 0, ctx->stream>>>(m, n, nsplit, out, alpha, beta, C, ldc);
    ctx->arena.release(mk);  // stream-ordered reuse
    post_launch(ctx, "splitk_reduce_kernel");
    return;
  }
  post_launch(ctx, "gemm_kernel");
}

template void gemm<float>(lra_ctx*, char, char, int64_t, int64_t, int64_t, float, const float*, int64_t,
                          const float*, int64_t, float, float*, int64_t);
template void gemm<double>(lra_ctx*, char, char, int64_t, int64_t, int64_t, double, const double*,
                           int64_t, const double*, int64_t, double, double*, int64_t);

}  // namespace lra
