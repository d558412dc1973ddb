// Shared device helpers of liblra (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>
#include <type_traits>

namespace lra {

constexpr int kWarp = 32;

// Default limit of every device-side wait (ns of %globaltimer).  A wait
// that runs out sets an error status and returns; nothing traps or spins
// forever.
constexpr uint64_t kWaitLimitNs = 4000000000ull;

// The limit in force, one copy per translation unit (no relocatable device
// code): lra_ctx_set_wait_limit writes every copy on the context's device.
// A wait reads it once when it starts.
static __device__ unsigned long long g_wait_limit_ns = kWaitLimitNs;

__device__ __forceinline__ uint64_t wait_limit_ns() {
  return *((volatile const unsigned long long*)&g_wait_limit_ns);
}

// host side: this translation unit's copy (synchronous)
static inline cudaError_t set_unit_wait_limit(uint64_t ns) {
  const unsigned long long v = ns ? ns : kWaitLimitNs;
  return cudaMemcpyToSymbol(g_wait_limit_ns, &v, sizeof v);
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)::"memory");
  return t;
}

template <typename T>
struct Real;
template <>
struct Real<double> {
  static constexpr double eps = DBL_EPSILON * 0.5;  // LAPACK xLAMCH('E')
  static constexpr double safmin = DBL_MIN;         // LAPACK xLAMCH('S')
  static constexpr double big = DBL_MAX;
};
template <>
struct Real<float> {
  static constexpr float eps = FLT_EPSILON * 0.5f;
  static constexpr float safmin = FLT_MIN;
  static constexpr float big = FLT_MAX;
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// (value, index) argmax with LAPACK IxAMAX semantics: the largest value,
// ties resolved to the smallest index.
template <typename T>
__device__ __forceinline__ void argmax_merge(T& v, int64_t& i, T v2, int64_t i2) {
  if (v2 > v || (v2 == v && i2 < i)) {
    v = v2;
    i = i2;
  }
}

template <typename T>
__device__ __forceinline__ void warp_argmax(T& v, int64_t& i) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T v2 = __shfl_xor_sync(0xffffffffu, v, o);
    int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
    argmax_merge(v, i, v2, i2);
  }
}

// Block-wide sum; `red` is shared scratch of >= 32 elements.  All threads
// receive the result.
template <typename T>
__device__ T block_sum(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T r = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
  if (wid == 0) {
    r = warp_sum(r);
    if (lane == 0) red[0] = r;
  }
  __syncthreads();
  r = red[0];
  __syncthreads();
  return r;
}

template <typename T>
__device__ T block_max(T v, T* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T r = (threadIdx.x < nw) ? red[threadIdx.x] : T(0);
  if (wid == 0) {
    r = warp_max(r);
    if (lane == 0) red[0] = r;
  }
  __syncthreads();
  r = red[0];
  __syncthreads();
  return r;
}

// Grid barrier for cooperative launches (all CTAs co-resident).  The wait
// is bounded: on time-out it records LRA_ETIMEDOUT (4) in `err` and every
// CTA leaves; callers return when it yields false.
struct GridBar {
  unsigned int count;
  unsigned int gen;
  int err;
  int pad;
};

__device__ __forceinline__ bool grid_sync(GridBar* gb) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &gb->gen;
    volatile int* verr = &gb->err;
    const unsigned int g = *vgen;
    __threadfence();
    const unsigned int prev = atomicAdd(&gb->count, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      const uint64_t t0 = globaltimer_ns(), lim = wait_limit_ns();
      while (*vgen == g) {
        if (*verr != 0) break;
        if (globaltimer_ns() - t0 > lim) {
          atomicCAS(&gb->err, 0, 4);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *((volatile int*)&gb->err) == 0;
}

}  // namespace lra
