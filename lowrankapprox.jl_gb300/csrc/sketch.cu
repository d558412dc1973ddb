// Structured sketches of src/sketch.jl, left side, B = S op(A) with op(A)
// the M x N matrix A ('n') or A^T ('c'), real element types:
//   RandomSubset          (src/sketch.jl:248-293)  rows drawn with replacement
//   SparseRandomGaussian  (src/sketch.jl:571-653)  row i of S has fld(M-i,l)+1
//                         Gaussian entries on rows perm[...] of op(A)
//   SRFT                  (src/sketch.jl:396-522)  sampled DFT of d .* x
//
// SRFT output convention, as the reference's srft_apply! produces it for
// real input: slots (1,2), (3,4), ... hold (Re, Im) of DFT(d .* x) at
// frequency idx[1]-1, idx[3]-1, ...; an odd last slot holds Re at idx[l]-1
// (the "purely real" guard at src/sketch.jl:425 compares the function `in`
// with an integer and never fires).  The reference reaches those values
// through an l'-point FFT and a twiddle recurrence; this kernel evaluates
// the same DFT samples directly against an exactly-indexed twiddle table.

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename T>
__device__ __forceinline__ T opA_at(const T* A, int64_t lda, int trans, int64_t r, int64_t c) {
  return trans ? A[c + r * lda] : A[r + c * lda];
}

template <typename T>
__global__ void sub_kernel(int trans, int64_t N, const T* __restrict__ A, int64_t lda,
                           const int64_t* __restrict__ rows, int64_t order, T* __restrict__ B,
                           int64_t ldb) {
  const int64_t total = order * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (trans) {  // read along columns of A (contiguous)
      j = t % N;
      i = t / N;
    } else {
      i = t % order;
      j = t / order;
    }
    B[i + j * ldb] = opA_at(A, lda, trans, rows[i] - 1, j);
  }
}

template <typename T>
__global__ void sprn_kernel(int trans, int64_t N, const T* __restrict__ A, int64_t lda,
                            const int64_t* __restrict__ perm, const T* __restrict__ g,
                            const int64_t* __restrict__ offs, int64_t order, T* __restrict__ B,
                            int64_t ldb) {
  const int64_t total = order * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    int64_t i, j;
    if (trans) {
      j = t % N;
      i = t / N;
    } else {
      i = t % order;
      j = t / order;
    }
    T s = 0;
    for (int64_t l = offs[i]; l < offs[i + 1]; ++l) s += g[l] * opA_at(A, lda, trans, perm[l] - 1, j);
    B[i + j * ldb] = s;
  }
}

// cos / sin of 2 pi t / M for t in [0, M)
__global__ void twiddle_kernel(int64_t M, double* __restrict__ c, double* __restrict__ s) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < M;
       t += (int64_t)gridDim.x * blockDim.x) {
    double sn, cs;
    // 2t/M in [0, 2): sincospi keeps the argument exact for the reduction
    sincospi(2.0 * (double)t / (double)M, &sn, &cs);
    c[t] = cs;
    s[t] = sn;
  }
}

// one warp per (slot pair, column): z = sum_t d_t x_t exp(-2 pi i f t / M)
template <typename T>
__global__ void srft_direct_kernel(int trans, int64_t M, int64_t N, const T* __restrict__ A,
                                   int64_t lda, const T* __restrict__ d,
                                   const int64_t* __restrict__ idx, int64_t order,
                                   const double* __restrict__ tc, const double* __restrict__ ts,
                                   T* __restrict__ B, int64_t ldb) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int64_t npairs = (order + 1) / 2;
  const int64_t total = npairs * N;
  for (int64_t w = (int64_t)blockIdx.x * nw + wid; w < total; w += (int64_t)gridDim.x * nw) {
    const int64_t pr = w % npairs, j = w / npairs;
    const int64_t slot = 2 * pr;
    const int64_t f = idx[slot] - 1;
    double re = 0, im = 0;
    int64_t ph = (f * lane) % M;  // phase index f*t mod M, advanced by 32 f
    const int64_t step = (f * 32) % M;
    for (int64_t t = lane; t < M; t += 32) {
      const double x = (double)d[t] * (double)opA_at(A, lda, trans, t, j);
      re += x * tc[ph];
      im -= x * ts[ph];
      ph += step;
      if (ph >= M) ph -= M;
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) {
      B[slot + j * ldb] = (T)re;
      if (slot + 1 < order) B[slot + 1 + j * ldb] = (T)im;
    }
  }
}

template <typename T>
__global__ void signs_kernel(const double* __restrict__ g, int64_t n, T* __restrict__ d) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    d[t] = g[t] > 0 ? T(1) : T(-1);
}

inline unsigned blocks_for(lra_ctx* ctx, int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)ctx->num_sms * 16));
}

}  // namespace

template <typename T>
void sub_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                const int64_t* rows, int64_t order, T* B, int64_t ldb) {
  (void)M;
  if (order <= 0 || N <= 0) return;
  sub_kernel<T><<<blocks_for(ctx, order * N, 256), 256, 0, ctx->stream>>>(trans == 'c' ? 1 : 0, N, A, lda,
                                                                          rows, order, B, ldb);
  post_launch(ctx, "sub_kernel");
}

template <typename T>
void sprn_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda,
                 const int64_t* perm, const T* g, int64_t order, T* B, int64_t ldb) {
  if (order <= 0 || N <= 0) return;
  // row i (1-based) of S takes fld(M - i, order) + 1 consecutive entries
  std::vector<int64_t> offs(order + 1, 0);
  for (int64_t i = 1; i <= order; ++i) {
    const int64_t q = M - i;
    const int64_t fl = q >= 0 ? q / order : -((-q + order - 1) / order);
    offs[i] = offs[i - 1] + fl + 1;
  }
  const ArenaMark mk = ctx->arena.mark();
  int64_t* doffs = ctx->arena.alloc_n<int64_t>(order + 1);
  LRA_CUDA(cudaMemcpyAsync(doffs, offs.data(), (order + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                           ctx->stream));
  sprn_kernel<T><<<blocks_for(ctx, order * N, 256), 256, 0, ctx->stream>>>(
      trans == 'c' ? 1 : 0, N, A, lda, perm, g, doffs, order, B, ldb);
  post_launch(ctx, "sprn_kernel");
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));  // offs is a stack buffer
  ctx->arena.release(mk);
}

template <typename T>
void srft_sketch(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda, const T* d,
                 const int64_t* idx, int64_t order, T* B, int64_t ldb) {
  if (order <= 0 || N <= 0) return;
  const ArenaMark mk = ctx->arena.mark();
  double* tc = ctx->arena.alloc_n<double>(M);
  double* ts = ctx->arena.alloc_n<double>(M);
  twiddle_kernel<<<blocks_for(ctx, M, 256), 256, 0, ctx->stream>>>(M, tc, ts);
  post_launch(ctx, "twiddle_kernel");
  const int64_t warps_total = ((order + 1) / 2) * N;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((warps_total + 7) / 8, (int64_t)ctx->num_sms * 16));
  srft_direct_kernel<T><<<g, 256, 0, ctx->stream>>>(trans == 'c' ? 1 : 0, M, N, A, lda, d, idx, order, tc,
                                                    ts, B, ldb);
  post_launch(ctx, "srft_direct_kernel");
  ctx->arena.release(mk);
}

template <typename T>
void srft_signs(lra_ctx* ctx, const double* g, int64_t n, T* d) {
  if (n <= 0) return;
  signs_kernel<T><<<blocks_for(ctx, n, 256), 256, 0, ctx->stream>>>(g, n, d);
  post_launch(ctx, "signs_kernel");
}

#define INST(T)                                                                                     \
  template void sub_sketch<T>(lra_ctx*, char, int64_t, int64_t, const T*, int64_t, const int64_t*, \
                              int64_t, T*, int64_t);                                               \
  template void sprn_sketch<T>(lra_ctx*, char, int64_t, int64_t, const T*, int64_t, const int64_t*,\
                               const T*, int64_t, T*, int64_t);                                    \
  template void srft_sketch<T>(lra_ctx*, char, int64_t, int64_t, const T*, int64_t, const T*,      \
                               const int64_t*, int64_t, T*, int64_t);                              \
  template void srft_signs<T>(lra_ctx*, const double*, int64_t, T*);
INST(float)
INST(double)
#undef INST

}  // namespace lra
