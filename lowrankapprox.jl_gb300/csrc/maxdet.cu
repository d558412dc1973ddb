// Determinant-maximizing column swaps of the ID (strong rank-revealing QR,
// Gu & Eisenstat 1996): maxdet_swapcols! / maxdet_update!
// (src/pqr.jl:445-501) on the device: T and the permutation, and R1 when
// an R factor is returned.

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

// findmaxabs (src/util.jl:13-23): largest |x|, ties to the LAST index
template <typename T>
__device__ __forceinline__ void last_max_merge(double& v, int64_t& i, double v2, int64_t i2) {
  if (v2 > v || (v2 == v && i2 > i)) {
    v = v2;
    i = i2;
  }
}

template <typename T>
__global__ void absmax_partial_kernel(int64_t total, const T* __restrict__ x, double* pv, int64_t* pi) {
  __shared__ double sv[32];
  __shared__ int64_t si[32];
  double v = -1;
  int64_t i = -1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    last_max_merge<T>(v, i, fabs((double)x[t]), t);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
    last_max_merge<T>(v, i, v2, i2);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = i;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) last_max_merge<T>(v, i, sv[w], si[w]);
    pv[blockIdx.x] = v;
    pi[blockIdx.x] = i;
  }
}

template <typename T>
__global__ void absmax_final_kernel(int nb, const double* pv, const int64_t* pi, double* outv, int64_t* outi) {
  if (threadIdx.x != 0) return;
  double v = -1;
  int64_t i = -1;
  for (int b = 0; b < nb; ++b) last_max_merge<T>(v, i, pv[b], pi[b]);
  *outv = v;
  *outi = i;
}

// swap, save w1 = T(:, j) - e_i, zero T(:, j) with T(i, j) = 1, save w2 = T(i, :)
template <typename T>
__global__ void maxdet_prep_kernel(int64_t k, int64_t nr, T* Tm, int64_t* jpvt, const int64_t* pidx, T* w1,
                                   T* w2) {
  const int64_t idx = *pidx;
  const int64_t i = idx % k, j = idx / k;
  for (int64_t l = threadIdx.x; l < k; l += blockDim.x) {
    T v = Tm[l + j * k];
    if (l == i) v -= T(1);
    w1[l] = v;
  }
  __syncthreads();
  for (int64_t l = threadIdx.x; l < k; l += blockDim.x) Tm[l + j * k] = (l == i) ? T(1) : T(0);
  __syncthreads();
  for (int64_t l = threadIdx.x; l < nr; l += blockDim.x) w2[l] = Tm[i + l * k];
  if (threadIdx.x == 0) {
    const int64_t t = jpvt[i];
    jpvt[i] = jpvt[k + j];
    jpvt[k + j] = t;
  }
}

// T -= w1 w2^T / (1 + w1[i])  (BLAS ger)
template <typename T>
__global__ void maxdet_ger_kernel(int64_t k, int64_t nr, T* Tm, const int64_t* pidx, const T* w1, const T* w2) {
  const int64_t i = *pidx % k;
  const T alpha = T(-1) / (T(1) + w1[i]);
  const int64_t total = k * nr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % k, c = t / k;
    Tm[t] += alpha * w1[r] * w2[c];
  }
}

// maxdet_update!'s R part (src/pqr.jl:494-499): y = R1 w1 with w1 = T(:, j)
// - e_i as it was before the T update; a thread per row of R1 (k x k)
template <typename T>
__global__ void maxdet_r1_gemv_kernel(int64_t k, const T* __restrict__ R1, int64_t ldr, const T* __restrict__ w1,
                                      T* __restrict__ y) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x) {
    T acc = T(0);
    for (int64_t c = 0; c < k; ++c) acc += R1[l + c * ldr] * w1[c];
    y[l] = acc;
  }
}

// R1(:, i) += y, after every row of y was formed from the old column i
template <typename T>
__global__ void maxdet_r1_add_kernel(int64_t k, T* R1, int64_t ldr, const int64_t* pidx, const T* y) {
  const int64_t i = *pidx % k;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x)
    R1[l + i * ldr] += y[l];
}

}  // namespace

template <typename T>
bool maxdet_step(lra_ctx* ctx, int64_t k, int64_t nr, T* Tm, int64_t* jpvt, double bound, bool update, T* R1,
                 int64_t ldr) {
  const int64_t total = k * nr;
  if (total <= 0) return false;
  const ArenaMark mk = ctx->arena.mark();
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 256));
  double* pv = ctx->arena.alloc_n<double>(nb + 1);
  int64_t* pi = ctx->arena.alloc_n<int64_t>(nb + 1);
  absmax_partial_kernel<T><<<nb, 256, 0, ctx->stream>>>(total, Tm, pv, pi);
  post_launch(ctx, "absmax_partial_kernel");
  absmax_final_kernel<T><<<1, 32, 0, ctx->stream>>>(nb, pv, pi, pv + nb, pi + nb);
  post_launch(ctx, "absmax_final_kernel");
  double hv = 0;
  LRA_CUDA(cudaMemcpyAsync(&hv, pv + nb, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  const bool big = hv > bound;
  if (big && update) {
    T* w1 = ctx->arena.alloc_n<T>(k);
    T* w2 = ctx->arena.alloc_n<T>(nr);
    maxdet_prep_kernel<T><<<1, 256, 0, ctx->stream>>>(k, nr, Tm, jpvt, pi + nb, w1, w2);
    post_launch(ctx, "maxdet_prep_kernel");
    if (R1) {
      T* y = ctx->arena.alloc_n<T>(k);
      const unsigned gk = (unsigned)std::max<int64_t>(1, std::min<int64_t>((k + 127) / 128, (int64_t)ctx->num_sms * 4));
      maxdet_r1_gemv_kernel<T><<<gk, 128, 0, ctx->stream>>>(k, R1, ldr, w1, y);
      post_launch(ctx, "maxdet_r1_gemv_kernel");
      maxdet_r1_add_kernel<T><<<gk, 128, 0, ctx->stream>>>(k, R1, ldr, pi + nb, y);
      post_launch(ctx, "maxdet_r1_add_kernel");
    }
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 8));
    maxdet_ger_kernel<T><<<g, 256, 0, ctx->stream>>>(k, nr, Tm, pi + nb, w1, w2);
    post_launch(ctx, "maxdet_ger_kernel");
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  ctx->arena.release(mk);
  return big;
}

template bool maxdet_step<float>(lra_ctx*, int64_t, int64_t, float*, int64_t*, double, bool, float*, int64_t);
template bool maxdet_step<double>(lra_ctx*, int64_t, int64_t, double*, int64_t*, double, bool, double*, int64_t);

}  // namespace lra
