// Data-movement and elementwise kernels of liblra (gathers, copies, random
// sketch entries, finiteness check, GEMV).

#include <algorithm>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

inline unsigned grid_for(lra_ctx* ctx, int64_t n, int threads, int per_sm = 8) {
  int64_t b = (n + threads - 1) / threads;
  b = std::min<int64_t>(b, (int64_t)ctx->num_sms * per_sm);
  return (unsigned)std::max<int64_t>(b, 1);
}

template <typename T>
__global__ void copy_matrix_kernel(int64_t m, int64_t n, const T* __restrict__ s, int64_t lds,
                                   T* __restrict__ d, int64_t ldd) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    d[i + j * ldd] = s[i + j * lds];
  }
}

// 32 x 32 tiles through shared memory
template <typename T>
__global__ void transpose_kernel(int64_t m, int64_t n, const T* __restrict__ s, int64_t lds,
                                 T* __restrict__ d, int64_t ldd) {
  __shared__ T tile[32][33];
  const int64_t tiles_m = (m + 31) / 32, tiles_n = (n + 31) / 32;
  for (int64_t t = blockIdx.x; t < tiles_m * tiles_n; t += gridDim.x) {
    const int64_t bi = (t % tiles_m) * 32, bj = (t / tiles_m) * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int64_t i = bi + threadIdx.x, j = bj + r;
      if (i < m && j < n) tile[r][threadIdx.x] = s[i + j * lds];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int64_t i = bj + threadIdx.x, j = bi + r;  // d is n x m
      if (i < n && j < m) d[i + j * ldd] = tile[threadIdx.x][r];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void gather_cols_kernel(int64_t m, int64_t k, const T* __restrict__ s, int64_t lds,
                                   const int64_t* __restrict__ idx, T* __restrict__ d, int64_t ldd) {
  const int64_t total = m * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    d[i + j * ldd] = s[i + (idx[j] - 1) * lds];
  }
}

template <typename T>
__global__ void gather_rows_kernel(int64_t k, int64_t n, const T* __restrict__ s, int64_t lds,
                                   const int64_t* __restrict__ idx, T* __restrict__ d, int64_t ldd) {
  const int64_t total = k * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % k, j = t / k;
    d[i + j * ldd] = s[(idx[i] - 1) + j * lds];
  }
}

template <typename T>
__global__ void scatter_cols_kernel(int64_t m, int64_t k, const T* __restrict__ s, int64_t lds,
                                    const int64_t* __restrict__ idx, T* __restrict__ d,
                                    int64_t ldd) {
  const int64_t total = m * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    d[i + (idx[j] - 1) * ldd] = s[i + j * lds];
  }
}

template <typename T>
__global__ void fill_kernel(T* p, int64_t n, T v) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    p[t] = v;
}

template <typename T>
__global__ void identity_kernel(int64_t m, int64_t n, T* A, int64_t lda) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    A[i + j * lda] = (i == j) ? T(1) : T(0);
  }
}

template <typename T>
__global__ void zero_lower_kernel(int64_t m, int64_t n, T* A, int64_t lda) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    if (i > j) A[i + j * lda] = T(0);
  }
}

__device__ __forceinline__ double lattice(double g) {
  double r = rint(g * 32.0);
  r = fmin(127.0, fmax(-127.0, r));
  return r * (1.0 / 32.0);
}

// the same rounding in FP32 (exact: the lattice values are k / 32, |k| <= 127)
__device__ __forceinline__ float lattice_f(float g) {
  const float r = fminf(127.0f, fmaxf(-127.0f, rintf(g * 32.0f)));
  return r * 0.03125f;
}

template <typename T>
__global__ void from_stream_kernel(const double* __restrict__ g, int64_t n, T* __restrict__ out,
                                   int lat) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double v = g[t];
    out[t] = (T)(lat ? lattice(v) : v);
  }
}

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), own implementation.
struct U4 {
  unsigned x, y, z, w;
};
__device__ __forceinline__ U4 philox(U4 c, unsigned k0, unsigned k1) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const unsigned hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

template <typename T>
__global__ void philox_kernel(uint64_t seed, uint64_t base, int64_t n, T* __restrict__ out) {
  const unsigned k0 = (unsigned)seed, k1 = (unsigned)(seed >> 32);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; 2 * t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t ctr = base + (uint64_t)t;
    U4 r = philox(U4{(unsigned)ctr, (unsigned)(ctr >> 32), 0x6c72u, 0x61u}, k0, k1);
    // Box-Muller on two uniforms in (0, 1], in FP32: the draws are rounded
    // to the 1/32 lattice, far coarser than FP32's resolution, and FP64
    // transcendentals are slow on this part
    const float u1 = ((float)r.x + 1.0f) * 2.3283064365386963e-10f;
    const float u2 = ((float)r.y + 0.5f) * 2.3283064365386963e-10f;
    const float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    out[2 * t] = (T)lattice_f(rad * c);
    if (2 * t + 1 < n) out[2 * t + 1] = (T)lattice_f(rad * s);
  }
}

// an all-ones exponent field (Inf / NaN), tested on the bits
__device__ __forceinline__ int nonfinite(double v) {
  return ((unsigned long long)__double_as_longlong(v) >> 52 & 0x7FF) == 0x7FF;
}
__device__ __forceinline__ int nonfinite(float v) { return (__float_as_uint(v) >> 23 & 0xFF) == 0xFF; }

// grid (x: row runs, y: columns); each thread keeps four loads in flight
template <typename T>
__global__ void finite_kernel(int64_t m, int64_t n, const T* __restrict__ A, int64_t lda, int* bad) {
  int local = 0;
  const int64_t rstep = (int64_t)gridDim.x * blockDim.x * 4;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const T* a = A + j * lda;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x * 4 + threadIdx.x; i0 < m; i0 += rstep) {
      T v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t i = i0 + (int64_t)u * blockDim.x;
        v[u] = i < m ? __ldcs(a + i) : T(0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) local |= nonfinite(v[u]);
    }
  }
  if (__syncthreads_or(local) && threadIdx.x == 0) atomicExch(bad, 1);
}

// the same test on 16-byte words of columns whose length and leading
// dimension are multiples of 16 bytes (Float32: 4 values per word, Float64 2)
template <bool F64>
__global__ void finite_vec_kernel(int64_t mv, int64_t n, const uint4* __restrict__ A, int64_t ldv, int* bad) {
  int local = 0;
  const int64_t rstep = (int64_t)gridDim.x * blockDim.x * 4;
  for (int64_t j = blockIdx.y; j < n; j += gridDim.y) {
    const uint4* a = A + j * ldv;
    for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x * 4 + threadIdx.x; i0 < mv; i0 += rstep) {
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t i = i0 + (int64_t)u * blockDim.x;
        v[u] = i < mv ? __ldcs(a + i) : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        if constexpr (F64) {
          local |= ((v[u].y >> 20 & 0x7FF) == 0x7FF) | ((v[u].w >> 20 & 0x7FF) == 0x7FF);
        } else {
          local |= ((v[u].x >> 23 & 0xFF) == 0xFF) | ((v[u].y >> 23 & 0xFF) == 0xFF) |
                   ((v[u].z >> 23 & 0xFF) == 0xFF) | ((v[u].w >> 23 & 0xFF) == 0xFF);
        }
      }
    }
  }
  if (__syncthreads_or(local) && threadIdx.x == 0) atomicExch(bad, 1);
}

// (x: runs of 1024 rows, at most 64; y: columns, so that a block sees at
// least 4096 elements and the grid about eight blocks per SM)
static dim3 finite_grid(lra_ctx* ctx, int64_t m, int64_t n) {
  const int64_t gx = std::max<int64_t>(1, std::min<int64_t>((m + 1023) / 1024, 64));
  const int64_t by_size = (m * n + gx * 4096 - 1) / (gx * 4096);
  const int64_t gy = std::max<int64_t>(1, std::min<int64_t>({(int64_t)ctx->num_sms * 8 / gx + 1, by_size, n, 65535}));
  return dim3((unsigned)gx, (unsigned)gy);
}

// y = alpha A^T x + beta y: one warp per column
template <typename T>
__global__ void gemv_t_kernel(int64_t m, int64_t n, T alpha, const T* __restrict__ A, int64_t lda,
                              const T* __restrict__ x, T beta, T* __restrict__ y) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int64_t j = (int64_t)blockIdx.x * nw + wid; j < n; j += (int64_t)gridDim.x * nw) {
    const T* a = A + j * lda;
    T s = 0;
    for (int64_t i = lane; i < m; i += 32) s += a[i] * x[i];
    s = warp_sum(s);
    if (lane == 0) y[j] = alpha * s + (beta == T(0) ? T(0) : beta * y[j]);
  }
}

// partial[c][i] = sum over the column chunk c of A(i, j) x(j)
template <typename T>
__global__ void gemv_n_partial_kernel(int64_t m, int64_t n, const T* __restrict__ A, int64_t lda,
                                      const T* __restrict__ x, int64_t chunk, T* __restrict__ part) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (i >= m) return;
  const int64_t j0 = c * chunk, j1 = min(n, j0 + chunk);
  T s = 0;
  for (int64_t j = j0; j < j1; ++j) s += A[i + j * lda] * x[j];
  part[c * m + i] = s;
}

template <typename T>
__global__ void gemv_n_reduce_kernel(int64_t m, int64_t nch, const T* __restrict__ part, T alpha,
                                     T beta, T* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x) {
    T s = 0;
    for (int64_t c = 0; c < nch; ++c) s += part[c * m + i];
    y[i] = alpha * s + (beta == T(0) ? T(0) : beta * y[i]);
  }
}

}  // namespace

template <typename T>
void copy_matrix(lra_ctx* ctx, int64_t m, int64_t n, const T* s, int64_t lds, T* d, int64_t ldd) {
  if (m <= 0 || n <= 0) return;
  if (lds == m && ldd == m) {
    LRA_CUDA(cudaMemcpyAsync(d, s, (size_t)m * n * sizeof(T), cudaMemcpyDeviceToDevice, ctx->stream));
    return;
  }
  LRA_CUDA(cudaMemcpy2DAsync(d, ldd * sizeof(T), s, lds * sizeof(T), m * sizeof(T), n,
                             cudaMemcpyDeviceToDevice, ctx->stream));
}

template <typename T>
void transpose(lra_ctx* ctx, int64_t m, int64_t n, const T* s, int64_t lds, T* d, int64_t ldd) {
  if (m <= 0 || n <= 0) return;
  const int64_t tiles = ((m + 31) / 32) * ((n + 31) / 32);
  const unsigned g = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 16);
  transpose_kernel<T><<<g, dim3(32, 8), 0, ctx->stream>>>(m, n, s, lds, d, ldd);
  post_launch(ctx, "transpose_kernel");
}

template <typename T>
void gather_cols(lra_ctx* ctx, int64_t m, int64_t k, const T* s, int64_t lds, const int64_t* idx, T* d,
                 int64_t ldd) {
  if (m <= 0 || k <= 0) return;
  gather_cols_kernel<T><<<grid_for(ctx, m * k, 256), 256, 0, ctx->stream>>>(m, k, s, lds, idx, d, ldd);
  post_launch(ctx, "gather_cols_kernel");
}

template <typename T>
void gather_rows(lra_ctx* ctx, int64_t k, int64_t n, const T* s, int64_t lds, const int64_t* idx, T* d,
                 int64_t ldd) {
  if (k <= 0 || n <= 0) return;
  gather_rows_kernel<T><<<grid_for(ctx, k * n, 256), 256, 0, ctx->stream>>>(k, n, s, lds, idx, d, ldd);
  post_launch(ctx, "gather_rows_kernel");
}

template <typename T>
void scatter_cols(lra_ctx* ctx, int64_t m, int64_t k, const T* s, int64_t lds, const int64_t* idx,
                  T* d, int64_t ldd) {
  if (m <= 0 || k <= 0) return;
  scatter_cols_kernel<T><<<grid_for(ctx, m * k, 256), 256, 0, ctx->stream>>>(m, k, s, lds, idx, d, ldd);
  post_launch(ctx, "scatter_cols_kernel");
}

template <typename T>
void set_zero(lra_ctx* ctx, T* p, int64_t n) {
  if (n <= 0) return;
  LRA_CUDA(cudaMemsetAsync(p, 0, (size_t)n * sizeof(T), ctx->stream));
}

template <typename T>
void set_identity(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda) {
  if (m <= 0 || n <= 0) return;
  identity_kernel<T><<<grid_for(ctx, m * n, 256), 256, 0, ctx->stream>>>(m, n, A, lda);
  post_launch(ctx, "identity_kernel");
}

template <typename T>
void zero_lower(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda) {
  if (m <= 0 || n <= 0) return;
  zero_lower_kernel<T><<<grid_for(ctx, m * n, 256), 256, 0, ctx->stream>>>(m, n, A, lda);
  post_launch(ctx, "zero_lower_kernel");
}

template <typename T>
void sketch_from_stream(lra_ctx* ctx, const double* g, int64_t n, T* out, bool lat) {
  if (n <= 0) return;
  from_stream_kernel<T><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(g, n, out, lat ? 1 : 0);
  post_launch(ctx, "from_stream_kernel");
}

template <typename T>
void sketch_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, T* out) {
  if (n <= 0) return;
  philox_kernel<T><<<grid_for(ctx, (n + 1) / 2, 256), 256, 0, ctx->stream>>>(seed, base, n, out);
  post_launch(ctx, "philox_kernel");
}

// sets *bad (zeroed by the caller) when A has a NaN or Inf entry; no wait
template <typename T>
static void launch_finite(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda, int* bad) {
  constexpr int per = 16 / sizeof(T);
  if (reinterpret_cast<uintptr_t>(A) % 16 == 0 && m % per == 0 && lda % per == 0) {
    finite_vec_kernel<sizeof(T) == 8><<<finite_grid(ctx, m / per, n), 256, 0, ctx->stream>>>(
        m / per, n, reinterpret_cast<const uint4*>(A), lda / per, bad);
    post_launch(ctx, "finite_vec_kernel");
    return;
  }
  finite_kernel<T><<<finite_grid(ctx, m, n), 256, 0, ctx->stream>>>(m, n, A, lda, bad);
  post_launch(ctx, "finite_kernel");
}

template <typename T>
void all_finite_async(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda, int* bad) {
  if (m <= 0 || n <= 0) return;
  launch_finite(ctx, m, n, A, lda, bad);
}

template <typename T>
bool all_finite(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda) {
  if (m <= 0 || n <= 0) return true;
  const ArenaMark mark = ctx->arena.mark();
  int* bad = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  launch_finite(ctx, m, n, A, lda, bad);
  int h = 0;
  LRA_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  return h == 0;
}

template <typename T>
void gemv(lra_ctx* ctx, char trans, int64_t m, int64_t n, T alpha, const T* A, int64_t lda, const T* x,
          T beta, T* y) {
  if (trans == 't' || trans == 'T' || trans == 'c' || trans == 'C') {
    if (n <= 0) return;
    const int warps = 8;
    const unsigned g = (unsigned)std::min<int64_t>((n + warps - 1) / warps, (int64_t)ctx->num_sms * 16);
    gemv_t_kernel<T><<<g, warps * 32, 0, ctx->stream>>>(m, n, alpha, A, lda, x, beta, y);
    post_launch(ctx, "gemv_t_kernel");
    return;
  }
  if (m <= 0) return;
  // split the columns so that about 4 waves of 256-row blocks are in flight
  const int64_t rb = (m + 255) / 256;
  int64_t nch = std::max<int64_t>(1, std::min<int64_t>(n, (int64_t)ctx->num_sms * 8 / std::max<int64_t>(rb, 1)));
  const int64_t chunk = (n + nch - 1) / nch;
  nch = (n + chunk - 1) / chunk;
  const ArenaMark mark = ctx->arena.mark();
  T* part = ctx->arena.alloc_n<T>((size_t)nch * m);
  gemv_n_partial_kernel<T><<<dim3((unsigned)rb, (unsigned)nch), 256, 0, ctx->stream>>>(m, n, A, lda, x,
                                                                                      chunk, part);
  post_launch(ctx, "gemv_n_partial_kernel");
  gemv_n_reduce_kernel<T><<<grid_for(ctx, m, 256), 256, 0, ctx->stream>>>(m, nch, part, alpha, beta, y);
  post_launch(ctx, "gemv_n_reduce_kernel");
  ctx->arena.release(mark);  // stream-ordered: later allocations run after
}

#define INST(T)                                                                                    \
  template void copy_matrix<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*, int64_t);        \
  template void transpose<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*, int64_t);          \
  template void gather_cols<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*,  \
                               int64_t);                                                           \
  template void gather_rows<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*,  \
                               int64_t);                                                           \
  template void scatter_cols<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*, \
                                int64_t);                                                          \
  template void set_zero<T>(lra_ctx*, T*, int64_t);                                                \
  template void set_identity<T>(lra_ctx*, int64_t, int64_t, T*, int64_t);                          \
  template void zero_lower<T>(lra_ctx*, int64_t, int64_t, T*, int64_t);                            \
  template void sketch_from_stream<T>(lra_ctx*, const double*, int64_t, T*, bool);                 \
  template void sketch_philox<T>(lra_ctx*, uint64_t, uint64_t, int64_t, T*);                       \
  template bool all_finite<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t);                      \
  template void all_finite_async<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, int*);          \
  template void gemv<T>(lra_ctx*, char, int64_t, int64_t, T, const T*, int64_t, const T*, T, T*);
INST(float)
INST(double)
#undef INST

// the data movement of complex matrices (the complex drivers)
#define INSTX(T)                                                                                   \
  template void copy_matrix<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*, int64_t);        \
  template void transpose<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*, int64_t);          \
  template void gather_cols<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*,  \
                               int64_t);                                                           \
  template void gather_rows<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*,  \
                               int64_t);                                                           \
  template void scatter_cols<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*, \
                                int64_t);                                                          \
  template void set_zero<T>(lra_ctx*, T*, int64_t);                                                \
  template void set_identity<T>(lra_ctx*, int64_t, int64_t, T*, int64_t);                          \
  template void zero_lower<T>(lra_ctx*, int64_t, int64_t, T*, int64_t);
INSTX(cx<float>)
INSTX(cx<double>)
#undef INSTX

}  // namespace lra

namespace lra {

namespace {

__device__ __forceinline__ unsigned mix32(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void ints_philox_kernel(uint64_t seed, uint64_t base, int64_t n, int64_t hi, int64_t* out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = base + (uint64_t)t;
    const unsigned a = mix32((unsigned)c ^ mix32((unsigned)seed ^ 0x1b873593u));
    const unsigned b = mix32((unsigned)(c >> 32) ^ mix32((unsigned)(seed >> 32) + a));
    const uint64_t r = ((uint64_t)a << 32) | b;
    out[t] = 1 + (int64_t)(r % (uint64_t)hi);
  }
}

// Feistel bijection on [0, 2^(2h)) walked until the value lands in [0, n)
__global__ void perm_kernel(uint64_t seed, uint64_t base, int64_t n, int h, int64_t* out) {
  const uint64_t mask = (h >= 32) ? 0xffffffffull : ((1ull << h) - 1);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    uint64_t x = (uint64_t)t;
    for (int walk = 0; walk < 4096; ++walk) {
      uint64_t L = x >> h, R = x & mask;
      for (int r = 0; r < 4; ++r) {
        const uint64_t F = mix32((unsigned)R ^ mix32((unsigned)(seed + base) + 0x9e3779b9u * (r + 1))) & mask;
        const uint64_t nl = R;
        R = (L ^ F) & mask;
        L = nl;
      }
      x = (L << h) | R;
      if (x < (uint64_t)n) break;
    }
    out[t] = (int64_t)x + 1;
  }
}

template <typename T>
__global__ void symmetrize_kernel(int64_t n, T* B, int64_t ldb) {
  const int64_t total = n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    if (i < j) {
      const T u = T(0.5) * (B[i + j * ldb] + B[j + i * ldb]);
      B[i + j * ldb] = u;
      B[j + i * ldb] = u;
    }
  }
}

template <typename T>
__global__ void add_diag_kernel(int64_t n, T* A, int64_t lda, T s) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    A[t + t * lda] += s;
}

template <typename T>
__global__ void scatter_rows_kernel(int64_t k, int64_t n, const T* __restrict__ s, int64_t lds,
                                    const int64_t* __restrict__ idx, T* __restrict__ d, int64_t ldd) {
  const int64_t total = k * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % k, j = t / k;
    d[(idx[i] - 1) + j * ldd] = s[i + j * lds];
  }
}

template <typename T>
__global__ void scale_vec_kernel(int64_t n, T* x, T s) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    x[t] *= s;
}

template <typename T>
__global__ void div_cols_kernel(int64_t m, int64_t n, T* X, int64_t ldx, const T* s) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    if (s[j] != T(0)) X[i + j * ldx] /= s[j];
  }
}

// one CTA: for each cluster [a, b], v_j -= (v_i . v_j) v_i for a <= i < j <= b
template <typename T>
__global__ void cluster_orth_kernel(int64_t n, T* Z, int64_t ldz, const int64_t* cl, int64_t ncl) {
  __shared__ T red[32];
  for (int64_t c = 0; c < ncl; ++c) {
    const int64_t a = cl[2 * c], b = cl[2 * c + 1];
    for (int64_t i = a; i <= b; ++i) {
      const T* vi = Z + i * ldz;
      for (int64_t j = i + 1; j <= b; ++j) {
        T* vj = Z + j * ldz;
        T s = 0;
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) s += vi[r] * vj[r];
        s = block_sum(s, red);
        for (int64_t r = threadIdx.x; r < n; r += blockDim.x) vj[r] -= s * vi[r];
        __syncthreads();
      }
    }
  }
}

}  // namespace

void ints_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, int64_t hi, int64_t* out) {
  if (n <= 0) return;
  ints_philox_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(seed, base, n, hi, out);
  post_launch(ctx, "ints_philox_kernel");
}

void perm_philox(lra_ctx* ctx, uint64_t seed, uint64_t base, int64_t n, int64_t* out) {
  if (n <= 0) return;
  int bits = 2;
  while ((1ll << bits) < n) bits += 2;
  perm_kernel<<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(seed, base, n, bits / 2, out);
  post_launch(ctx, "perm_kernel");
}

template <typename T>
void symmetrize(lra_ctx* ctx, int64_t n, T* B, int64_t ldb) {
  if (n <= 1) return;
  symmetrize_kernel<T><<<grid_for(ctx, n * n, 256), 256, 0, ctx->stream>>>(n, B, ldb);
  post_launch(ctx, "symmetrize_kernel");
}

template <typename T>
void add_diag(lra_ctx* ctx, int64_t n, T* A, int64_t lda, T s) {
  if (n <= 0) return;
  add_diag_kernel<T><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, A, lda, s);
  post_launch(ctx, "add_diag_kernel");
}

template <typename T>
void scatter_rows(lra_ctx* ctx, int64_t k, int64_t n, const T* s, int64_t lds, const int64_t* idx, T* d,
                  int64_t ldd) {
  if (k <= 0 || n <= 0) return;
  scatter_rows_kernel<T><<<grid_for(ctx, k * n, 256), 256, 0, ctx->stream>>>(k, n, s, lds, idx, d, ldd);
  post_launch(ctx, "scatter_rows_kernel");
}

template <typename T>
void scale_vec(lra_ctx* ctx, int64_t n, T* x, T s) {
  if (n <= 0) return;
  scale_vec_kernel<T><<<grid_for(ctx, n, 256), 256, 0, ctx->stream>>>(n, x, s);
  post_launch(ctx, "scale_vec_kernel");
}

template <typename T>
void div_cols(lra_ctx* ctx, int64_t m, int64_t n, T* X, int64_t ldx, const T* s) {
  if (m <= 0 || n <= 0) return;
  div_cols_kernel<T><<<grid_for(ctx, m * n, 256), 256, 0, ctx->stream>>>(m, n, X, ldx, s);
  post_launch(ctx, "div_cols_kernel");
}

template <typename T>
void cluster_orth(lra_ctx* ctx, int64_t n, int64_t k, T* Z, int64_t ldz, const int64_t* cl, int64_t ncl) {
  (void)k;
  if (ncl <= 0) return;
  cluster_orth_kernel<T><<<1, 256, 0, ctx->stream>>>(n, Z, ldz, cl, ncl);
  post_launch(ctx, "cluster_orth_kernel");
}

#define INST2(T)                                                                                  \
  template void symmetrize<T>(lra_ctx*, int64_t, T*, int64_t);                                   \
  template void add_diag<T>(lra_ctx*, int64_t, T*, int64_t, T);                                  \
  template void scatter_rows<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, const int64_t*, T*, \
                                int64_t);                                                        \
  template void scale_vec<T>(lra_ctx*, int64_t, T*, T);                                           \
  template void div_cols<T>(lra_ctx*, int64_t, int64_t, T*, int64_t, const T*);                   \
  template void cluster_orth<T>(lra_ctx*, int64_t, int64_t, T*, int64_t, const int64_t*, int64_t);
INST2(float)
INST2(double)
#undef INST2

}  // namespace lra
