// Gaussian sketch B = S op(A) on tcgen05 tensor cores, FP64-faithful, for
// the mixed-precision path (the sketch of src/sketch.jl:91-98 and
// sketch_randn_ln/lc, src/sketch.jl:129-174).
//
// Exact split products.  S is on the 1/32 lattice: S = sigma / 32 with
// integer |sigma| <= 127, exact in BF16.  Column j of op(A) is written as a
// W-bit fixed-point integer at a per-column power-of-two scale,
//     op(A)(i, j) ~= F_ij 2^(e_j - W),  |op(A)(:, j)| < 2^(e_j),
// (W = 48 for Float64, 24 for Float32) and F is cut into ns = W/8 byte
// slices b_1 (signed, |b_1| <= 256) and b_2..b_ns (0..255), all exact in BF16.
// Every product sigma * b is an integer below 2^15, so the FP32 sum of 512 of
// them is an exact integer below 2^24: the tensor core loses nothing inside
// a 512-long K chunk.  Slices 1..4 (E = min(ns, 4)) get their own TMEM
// accumulators; slices 5..6 are pre-scaled by 2^-8(s-5) and share one FP32
// tail accumulator, whose per-chunk rounding (~half a unit of P5) sits near
// 2^-48 of the result.  All are drained after every chunk into one int64
// per output,
//     X += sum_a P_a 2^(8(E-a)+t) + round(tail 2^(t-8)),
//     B(r, j) = 2^(e_j - 5 - 8E - t) X,
// with t = 8 while |X| stays below 2^62 (K <= 32768), else t = 0.
//
// Kernel: 10 warps; warp 0 issues TMA loads (SW128, K-major) into a 2-stage
// ring, warp 1 allocates TMEM and issues tcgen05.mma from one thread, warps
// 2..9 drain the accumulators and write B.  Tile: 128 columns of op(A) (the
// MMA M dimension, one TMEM lane each) x 96 sketch rows (MMA N; five
// accumulators of 96 columns fit the 512 TMEM columns).  Every mbarrier wait
// is bounded by %globaltimer; a timeout records an error and the kernel runs
// to its end, freeing TMEM.

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstring>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

constexpr int TILE_M = 128;   // columns of op(A) per CTA
// sketch rows per CTA (the MMA N): 32, 64 or 96, picked per element type and
// sketch order by the tuning table; five accumulators of TN columns fit TMEM
constexpr int KBLK = 64;      // K per stage (128 bytes of BF16: one SW128 row)
constexpr int CHUNK_KB = 8;   // K-blocks per exact chunk (512)
constexpr int MAX_NSTAGE = 4;  // ring stages, as many as shared memory holds (at least 2)
constexpr int TILE_BYTES = TILE_M * KBLK * 2;  // 16 KB (one slice tile)
constexpr int NTHREADS = 320;
constexpr int MAX_SLICES = 6;
constexpr int MAX_EXACT = 4;
template <int TN>
struct TcTile {
  static constexpr int S_BYTES = TN * KBLK * 2;  // 4, 8 or 12 KB (1024 multiples)
  static constexpr int COLS = TN / 2;            // sketch rows per drain thread
  static constexpr uint32_t TMEM_COLS = 5 * TN <= 256 ? 256u : 512u;
  static_assert(S_BYTES % 1024 == 0 && COLS % 16 == 0 && TN % 16 == 0, "tile N");
};
constexpr int kNonFinite = 1 << 20;            // exponent of a column holding NaN / Inf

struct TcParams {
  int64_t K;       // sketched dimension (rows of op(A))
  int64_t ncols;   // columns of op(A)
  int64_t L;       // sketch order
  int ns;          // slices
  int tshift;      // t above
  const int* colexp;
  void* B;
  int64_t ldb;
  int out_double;
  int* err;
  // split over K: blockIdx.y takes kc_per 512-long chunks, and the CTAs add
  // their exact partial sums X into W (Lp x ncols int64, zeroed) instead of
  // writing B; null for one split
  int kc_per;
  long long* W;
  int64_t ldw;
  int nstage;  // TMA ring stages (2..MAX_NSTAGE)
};

// ---- PTX helpers -------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; returns false (and records the error) on time-out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns(), lim = wait_limit_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (*((volatile int*)err) != 0) return false;
    if (globaltimer_ns() - t0 > lim) {
      atomicCAS(err, 0, 4);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// tcgen05 shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), version 1, base offset 0 (tiles are 1024-aligned)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);          // start address
  d |= (uint64_t)1 << 16;                           // LBO (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                 // SBO
  d |= (uint64_t)1 << 46;                           // descriptor version
  d |= (uint64_t)2 << 61;                           // SWIZZLE_128B
  return d;
}

// instruction descriptor, kind::f16: BF16 x BF16 -> FP32, K-major A and B
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                        // D format F32
         | (1u << 7)                      // A format BF16
         | (1u << 10)                     // B format BF16
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- the sketch kernel ----------------------------------------------------------
template <int TILE_N>
__global__ void __launch_bounds__(NTHREADS, 1)
    tc_sketch_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmS,
                     TcParams P) {
  constexpr int S_BYTES = TcTile<TILE_N>::S_BYTES;
  constexpr int COLS = TcTile<TILE_N>::COLS;
  constexpr uint32_t TMEM_COLS = TcTile<TILE_N>::TMEM_COLS;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-align the tile area
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int ns = P.ns;
  const int stage_bytes = S_BYTES + ns * TILE_BYTES;
  unsigned char* stages = base;
  const int NSTAGE = P.nstage;
  uint64_t* full = reinterpret_cast<uint64_t*>(base + NSTAGE * stage_bytes);
  uint64_t* empty = full + NSTAGE;
  uint64_t* acc_ready = empty + NSTAGE;
  uint64_t* acc_free = acc_ready + 1;
  uint64_t* mma_done = acc_free + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntl = (P.L + TILE_N - 1) / TILE_N;
  const int64_t n_tile = blockIdx.x / ntl, l_tile = blockIdx.x % ntl;
  // this CTA's K blocks [kb0, kb0 + nkb): whole 512-long chunks, so that
  // every chunk is rounded as without the split
  const int nkb_all = (int)((P.K + KBLK - 1) / KBLK);
  const int kb0 = (int)blockIdx.y * P.kc_per * CHUNK_KB;
  const int nkb = min(nkb_all - kb0, P.kc_per * CHUNK_KB);
  const int nchunks = (nkb + CHUNK_KB - 1) / CHUNK_KB;
  const int n_exact = ns < MAX_EXACT ? ns : MAX_EXACT;
  const bool has_tail = ns > MAX_EXACT;
  const int n_acc = n_exact + (has_tail ? 1 : 0);
  const int t = has_tail ? P.tshift : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
    }
    mbar_init(acc_ready, 1);
    mbar_init(acc_free, 8);  // one arrival per drain warp
    mbar_init(mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int issued = 0;
      for (int kb = 0; kb < nkb; ++kb) {
        const int s = kb % NSTAGE;
        const uint32_t ph = (kb / NSTAGE) & 1;
        if (!mbar_wait(empty + s, ph ^ 1, P.err)) break;
        ++issued;
        unsigned char* st = stages + s * stage_bytes;
        mbar_expect_tx(full + s, (uint32_t)stage_bytes);
        tma_load_2d(st, &tmS, (kb0 + kb) * KBLK, (int)(l_tile * TILE_N), full + s);
        for (int q = 0; q < ns; ++q)
          tma_load_3d(st + S_BYTES + q * TILE_BYTES, &tmA, (kb0 + kb) * KBLK, (int)(n_tile * TILE_M), q, full + s);
      }
      // no copy may still be landing in shared memory when the CTA exits
      int dummy = 0;
      for (int kb = issued - NSTAGE; kb < issued; ++kb)
        if (kb >= 0) mbar_wait(full + kb % NSTAGE, (kb / NSTAGE) & 1, &dummy);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(TILE_M, TILE_N);
      for (int kb = 0; kb < nkb; ++kb) {
        const int chunk = kb / CHUNK_KB;
        const bool chunk_start = (kb % CHUNK_KB) == 0;
        if (chunk_start && chunk > 0) {
          // the drain of the previous chunk must be done before overwriting
          if (!mbar_wait(acc_free, (chunk - 1) & 1, P.err)) break;
          tc_fence_after();
        }
        const int s = kb % NSTAGE;
        const uint32_t ph = (kb / NSTAGE) & 1;
        if (!mbar_wait(full + s, ph, P.err)) break;
        tc_fence_after();
        const uint32_t st = smem_u32(stages + s * stage_bytes);
        for (int q = 0; q < ns; ++q) {
          const int a = q < MAX_EXACT ? q : MAX_EXACT;  // accumulator
          const uint32_t acc = tmem + (uint32_t)(a * TILE_N);
          const uint32_t a_addr = st + (uint32_t)(S_BYTES + q * TILE_BYTES);
#pragma unroll
          for (int k4 = 0; k4 < KBLK / 16; ++k4) {
            const uint64_t ad = sw128_desc(a_addr + k4 * 32);
            const uint64_t bd = sw128_desc(st + k4 * 32);
            // every accumulator restarts at each chunk; the tail slices
            // share one, reset by the first of them
            const bool first = chunk_start && k4 == 0 && q <= MAX_EXACT;
            mma_bf16(acc, ad, bd, idesc, first ? 0u : 1u);
          }
        }
        mma_commit(empty + s);  // frees the stage once these MMAs complete
        if ((kb % CHUNK_KB) == CHUNK_KB - 1 || kb == nkb - 1) mma_commit(acc_ready);
      }
      // every issued MMA has completed before TMEM is released
      mma_commit(mma_done);
      int dummy = 0;
      mbar_wait(mma_done, 0, &dummy);
    }
  } else {
    // ---------------- drain / epilogue: warps 2..9 ----------------
    const int q4 = warp & 3;           // TMEM lane quarter this warp may access
    const int half = (warp - 2) >> 2;  // which COLS of the TILE_N sketch rows
    const uint32_t lane_base = (uint32_t)(32 * q4) << 16;
    long long X[COLS];
#pragma unroll
    for (int c = 0; c < COLS; ++c) X[c] = 0;
    bool ok = true;
    for (int ch = 0; ch < nchunks; ++ch) {
      if (!mbar_wait(acc_ready, ch & 1, P.err)) {
        ok = false;
        break;
      }
      tc_fence_after();
      for (int a = 0; a < n_acc; ++a) {
        const int sh = 8 * (n_exact - 1 - a) + t;
#pragma unroll
        for (int piece = 0; piece < COLS / 16; ++piece) {
          uint32_t r[16];
          tmem_ld16(tmem + lane_base + (uint32_t)(a * TILE_N + half * COLS + piece * 16), r);
          if (a < n_exact) {
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              const int iv = __float2int_rz(__uint_as_float(r[c]));
              X[piece * 16 + c] += (long long)iv << sh;
            }
          } else {
            const float tsc = t ? 1.0f : (1.0f / 256.0f);  // tail weight 2^(t-8)
            // |tail| < 2^25 here: a 32-bit conversion is exact and stays off
            // the FP64 pipe, which runs the 64-bit ones on this part
#pragma unroll
            for (int c = 0; c < 16; ++c)
              X[piece * 16 + c] += (long long)__float2int_rn(__uint_as_float(r[c]) * tsc);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_free);
    }
    // epilogue: scale + store
    const int64_t j = n_tile * TILE_M + 32 * q4 + lane;  // column of op(A) / B
    const int e = (ok && j < P.ncols) ? P.colexp[j] : 0;
    const int sc = e - 5 - 8 * n_exact - t;  // B = 2^(e - 5 - 8E - t) X
    const int64_t r0 = l_tile * TILE_N + half * COLS;
    if (ok && j < P.ncols && P.W) {
      // a part of K: the exact partial sums, added as integers (any order
      // gives the same total)
#pragma unroll
      for (int c = 0; c < COLS; ++c) {
        const int64_t row = r0 + c;
        if (row < P.L)
          atomicAdd(reinterpret_cast<unsigned long long*>(P.W + row + j * P.ldw), (unsigned long long)X[c]);
      }
    } else if (ok && j < P.ncols) {
#pragma unroll
      for (int c = 0; c < COLS; ++c) {
        const int64_t row = r0 + c;
        if (row < P.L) {
          const double v = e >= kNonFinite ? __longlong_as_double(0x7FF8000000000000ll) : ldexp((double)X[c], sc);
          if (P.out_double)
            static_cast<double*>(P.B)[row + j * P.ldb] = v;
          else
            static_cast<float*>(P.B)[row + j * P.ldb] = (float)v;
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// the split-K sketch's sums W (exact int64) scaled into B, as the unsplit
// kernel's epilogue does
__global__ void tc_sketch_finish_kernel(int64_t L, int64_t ncols, const long long* __restrict__ W, int64_t ldw,
                                        const int* __restrict__ colexp, int n_exact, int t, void* B, int64_t ldb,
                                        int out_double) {
  const int64_t total = L * ncols;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = q % L, j = q / L;
    const int e = colexp[j];
    const double v = e >= kNonFinite ? __longlong_as_double(0x7FF8000000000000ll)
                                     : ldexp((double)W[row + j * ldw], e - 5 - 8 * n_exact - t);
    if (out_double)
      static_cast<double*>(B)[row + j * ldb] = v;
    else
      static_cast<float*>(B)[row + j * ldb] = (float)v;
  }
}

// ---- splitting op(A) into byte slices ---------------------------------------------

// per-column exponent e_j with max |op(A)(:, j)| < 2^e_j; a column holding
// a NaN or an infinity gets kNonFinite, and every output it touches is NaN
__device__ __forceinline__ int colexp_of(double mx) {
  if (!(mx <= DBL_MAX)) return kNonFinite;
  return mx > 0 ? ilogb(mx) + 1 : 0;
}

// |x| as an orderable bit pattern (nonnegative floating-point numbers order
// like their bits); NaN and Inf map to +Inf.  Integer operations only: the
// FP64 pipe is narrow on this part.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  return b >= 0x7FF0000000000000ull ? 0x7FF0000000000000ull : b;
}
__device__ __forceinline__ unsigned int abs_bits(float x) {
  const unsigned int b = __float_as_uint(x) & 0x7FFFFFFFu;
  return b >= 0x7F800000u ? 0x7F800000u : b;
}
__device__ __forceinline__ double bits_value(unsigned long long b) { return __longlong_as_double((long long)b); }
__device__ __forceinline__ double bits_value(unsigned int b) { return (double)__uint_as_float(b); }
template <typename K>
__device__ __forceinline__ K warp_max_bits(K v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const K w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}

template <typename T>
__global__ void colexp_n_kernel(int64_t K, int64_t N, const T* __restrict__ A, int64_t lda, int* e) {
  using Key = decltype(abs_bits(T(0)));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int64_t j = (int64_t)blockIdx.x * nw + wid; j < N; j += (int64_t)gridDim.x * nw) {
    Key mx = 0;
    for (int64_t i = lane; i < K; i += 32) {
      const Key a = abs_bits(A[i + j * lda]);
      mx = a > mx ? a : mx;
    }
    mx = warp_max_bits(mx);
    if (lane == 0) e[j] = colexp_of(bits_value(mx));  // NaN and Inf mark the column
  }
}

// op(A) = A^T: column j of op(A) is row j of A.  Tiles of 32 rows of A x
// 256 of its columns: coalesced partial maxima per row, merged with an
// atomic max on the bit patterns of the doubles, then turned into exponents.
template <typename T>
__global__ void rowmax_kernel(int64_t K, int64_t N, const T* __restrict__ A, int64_t lda,
                              unsigned long long* __restrict__ mx) {
  using Key = decltype(abs_bits(T(0)));
  const int64_t tn = (N + 31) / 32, tk = (K + 255) / 256;
  for (int64_t t = blockIdx.x; t < tn * tk; t += gridDim.x) {
    const int64_t j = (t % tn) * 32 + threadIdx.x;
    const int64_t i0 = (t / tn) * 256;
    Key m = 0;
    if (j < N)
      for (int64_t i = i0 + threadIdx.y; i < min(K, i0 + 256); i += blockDim.y) {
        const Key a = abs_bits(A[j + i * lda]);
        m = a > m ? a : m;
      }
    if (j < N && m > 0) atomicMax(mx + j, abs_bits(bits_value(m)));
  }
}

__global__ void rowmax_exp_kernel(int64_t N, const unsigned long long* __restrict__ mx, int* __restrict__ e) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x)
    e[j] = colexp_of(__longlong_as_double((long long)mx[j]));
}

// fixed-point integer of x at scale 2^(e - W) (round half up), from the bits
__device__ __forceinline__ long long fixed_point(double x, int e, int W) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  unsigned long long mant = bits & ((1ull << 52) - 1);
  if ((ex == 0 && mant == 0) || ex == 0x7FF || e >= kNonFinite) return 0;
  if (ex != 0) mant |= 1ull << 52;
  const int e2 = (ex == 0 ? 1 : ex) - 1075;  // x = mant 2^e2
  const int sh = e2 + W - e;                  // F = mant 2^sh, sh < 0 here
  long long F;
  if (sh >= 0) {
    F = (long long)(mant << sh);
  } else if (-sh >= 64) {
    F = 0;
  } else {
    const int r = -sh;
    F = (long long)((mant + (1ull << (r - 1))) >> r);
  }
  return (bits >> 63) ? -F : F;
}

__device__ __forceinline__ long long fixed_point(float x, int e, int W) { return fixed_point((double)x, e, W); }

// exact BF16 of an integer b in [-256, 256], times 2^-8k
__device__ __forceinline__ __nv_bfloat16 bf16_of(int b, int k) {
  float f = __int_as_float(0x4B000000 | (b + 256)) - 8388864.0f;  // exact: 2^23 + 256
  if (k) f *= __int_as_float((127 - 8 * k) << 23);
  return __ushort_as_bfloat16((unsigned short)(__float_as_uint(f) >> 16));
}

// n_exact > 0: slices b_1 (signed) and b_2.. (bytes 0..255) of F, those
// after the first n_exact pre-scaled by 2^-8(s - n_exact - 1) for a shared
// tail accumulator.  n_exact == 0: balanced digits, F = sum_s b_s 2^(W - 8s)
// with every b_s rounded to nearest (|b_1| <= 256, |b_s| <= 128 after), so
// that the products a GEMM drops average to zero instead of piling up.
template <typename T>
__device__ __forceinline__ void write_slices(long long F, int ns, int n_exact, int W, __nv_bfloat16* out,
                                             int64_t plane) {
  if (n_exact == 0) {
#pragma unroll
    for (int s = 1; s <= MAX_SLICES; ++s) {
      if (s > ns) break;
      const int shift = W - 8 * s;
      const long long b = shift > 0 ? (F + (1ll << (shift - 1))) >> shift : F;
      F -= b << shift;
      out[(s - 1) * plane] = bf16_of((int)b, 0);
    }
    return;
  }
#pragma unroll
  for (int s = 1; s <= MAX_SLICES; ++s) {
    if (s > ns) break;
    const int shift = W - 8 * s;
    int b = (s == 1) ? (int)(F >> shift) : (int)((F >> shift) & 255);
    const int k = s > n_exact ? (s - n_exact - 1) : 0;
    out[(s - 1) * plane] = bf16_of(b, k);
  }
}

template <typename T>
__global__ void split_n_kernel(int64_t K, int64_t N, const T* __restrict__ A, int64_t lda, const int* __restrict__ e,
                               int ns, int n_exact, int W, __nv_bfloat16* __restrict__ S, int64_t Kp) {
  const int64_t total = Kp * N;
  const int64_t plane = Kp * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % Kp, j = t / Kp;
    const long long F = i < K ? fixed_point(A[i + j * lda], e[j], W) : 0;
    write_slices<T>(F, ns, n_exact, W, S + i + j * Kp, plane);
  }
}

// op(A) = A^T through 32 x 32 shared-memory tiles
template <typename T>
__global__ void split_c_kernel(int64_t K, int64_t N, const T* __restrict__ A, int64_t lda, const int* __restrict__ e,
                               int ns, int n_exact, int W, __nv_bfloat16* __restrict__ S, int64_t Kp) {
  __shared__ T tile[32][33];
  const int64_t plane = Kp * N;
  const int64_t ti = (Kp + 31) / 32, tj = (N + 31) / 32;
  for (int64_t t = blockIdx.x; t < ti * tj; t += gridDim.x) {
    const int64_t i0 = (t % ti) * 32, j0 = (t / ti) * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int64_t j = j0 + threadIdx.x, i = i0 + r;  // A(j, i) contiguous in j
      tile[r][threadIdx.x] = (i < K && j < N) ? A[j + i * lda] : T(0);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
      const int64_t i = i0 + threadIdx.x, j = j0 + r;
      if (i < Kp && j < N) {
        const long long F = fixed_point(tile[threadIdx.x][r], e[j], W);
        write_slices<T>(F, ns, n_exact, W, S + i + j * Kp, plane);
      }
    }
    __syncthreads();
  }
}

// St (Kp x Lp, K-major: St[i + r Kp]) = 32 S(r, i) in BF16, zero padded
template <typename T>
__global__ void sketch_t_kernel(int64_t L, int64_t K, const T* __restrict__ S, int64_t Lp, int64_t Kp,
                                __nv_bfloat16* __restrict__ St) {
  __shared__ T tile[32][33];
  const int64_t tr = (Lp + 31) / 32, tk = (Kp + 31) / 32;
  for (int64_t t = blockIdx.x; t < tr * tk; t += gridDim.x) {
    const int64_t r0 = (t % tr) * 32, i0 = (t / tr) * 32;
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
      const int64_t r = r0 + threadIdx.x, i = i0 + c;  // S(r, i) contiguous in r
      tile[c][threadIdx.x] = (r < L && i < K) ? S[r + i * L] : T(0);
    }
    __syncthreads();
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
      const int64_t i = i0 + threadIdx.x, r = r0 + c;
      if (i < Kp && r < Lp) St[i + r * Kp] = __float2bfloat16_rn((float)(tile[threadIdx.x][c] * T(32)));
    }
    __syncthreads();
  }
}

// ---- FP64 GEMM from two-sided byte slices -------------------------------------------
//
// C = alpha op(A) op(B) + beta C for Float64.  Row i of op(A) and column j of
// op(B) are 48-bit fixed-point integers at power-of-two scales 2^(ea_i - 48)
// and 2^(eb_j - 48), each cut into six balanced BF16 digits a_1..a_6,
// b_1..b_6 (|a_1|, |b_1| <= 256, the rest <= 128; all exact in BF16).  The
// product is
//     sum_{s,t} a_s b_t 2^(8(12 - s - t)) 2^(ea_i + eb_j - 96),
// kept for s + t <= 7 (21 digit products; the dropped ones weigh below
// 2^-46 of the leading term and, the digits being balanced, average to
// zero).  The products of one diagonal d = s + t - 2 share a TMEM
// accumulator; a digit product is at most 2^16 (2^15, 2^14 for the later
// digits), so the sums of a diagonal over a 128-long K chunk stay within
// 2^24 and the FP32 accumulation is exact.  After every chunk the six
// accumulators are drained, through 32-bit conversions, into one int64
// per output,
//     X += sum_d acc_d 2^(8(5 - d) - t),   C = 2^(ea_i + eb_j - 56 + t) X,
// with t = ceil(log2(K chunks)) + 1 keeping |X| below 2^63.
//
// Same warp roles as the sketch kernel; one 144 KB stage (six 128 x 64 A
// digit tiles, six 64 x 64 B digit tiles), so the loads of block k + 1
// overlap the drain of block k.  blockIdx.y selects a range of K blocks;
// with several, each writes its unscaled partial product to a workspace.
constexpr int G_TILE_M = 128, G_TILE_N = 64, G_NS = 6;
constexpr int G_A_BYTES = G_TILE_M * KBLK * 2;               // 16 KB
constexpr int G_B_BYTES = G_TILE_N * KBLK * 2;               // 8 KB
constexpr int G_STAGE = G_NS * (G_A_BYTES + G_B_BYTES);      // 144 KB
constexpr int G_COLS = G_TILE_N / 2;                         // columns per drain thread
constexpr int G_CHUNK = 2;                                   // K blocks per drain (128)

struct TgParams {
  int64_t M, N;
  int nkb;          // K blocks in all
  int kb_per;       // K blocks per split
  int tshift;
  const int* ea;    // per row of op(A)
  const int* eb;    // per column of op(B)
  double* C;
  int64_t ldc;
  double alpha, beta;
  int to_ws;        // write 2^(...) X to C + y M N (ld M), no alpha / beta
  int* err;
};

__global__ void __launch_bounds__(NTHREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, TgParams P) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* stA = base;
  unsigned char* stB = base + G_NS * G_A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(base + G_STAGE);
  uint64_t* empty = full + 1;
  uint64_t* acc_ready = empty + 1;
  uint64_t* acc_free = acc_ready + 1;
  uint64_t* mma_done = acc_free + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tiles_m = (P.M + G_TILE_M - 1) / G_TILE_M;
  const int64_t m_tile = blockIdx.x % tiles_m, n_tile = blockIdx.x / tiles_m;
  const int kb0 = blockIdx.y * P.kb_per;
  const int nloc = min(P.nkb, kb0 + P.kb_per) - kb0;
  const int t = P.tshift;

  if (threadIdx.x == 0) {
    mbar_init(full, 1);
    mbar_init(empty, 1);
    mbar_init(acc_ready, 1);
    mbar_init(acc_free, 8);
    mbar_init(mma_done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int issued = 0;
      for (int it = 0; it < nloc; ++it) {
        if (!mbar_wait(empty, (it & 1) ^ 1, P.err)) break;
        ++issued;
        const int kx = (kb0 + it) * KBLK;
        mbar_expect_tx(full, (uint32_t)G_STAGE);
        for (int q = 0; q < G_NS; ++q) {
          tma_load_3d(stA + q * G_A_BYTES, &tmA, kx, (int)(m_tile * G_TILE_M), q, full);
          tma_load_3d(stB + q * G_B_BYTES, &tmB, kx, (int)(n_tile * G_TILE_N), q, full);
        }
      }
      int dummy = 0;
      if (issued > 0) mbar_wait(full, (issued - 1) & 1, &dummy);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_bf16(G_TILE_M, G_TILE_N);
      for (int it = 0; it < nloc; ++it) {
        const int ch = it / G_CHUNK;  // drain chunk
        const bool first = (it % G_CHUNK) == 0;
        if (first && ch > 0) {
          if (!mbar_wait(acc_free, (ch - 1) & 1, P.err)) break;
          tc_fence_after();
        }
        if (!mbar_wait(full, it & 1, P.err)) break;
        tc_fence_after();
        const uint32_t a0 = smem_u32(stA), b0 = smem_u32(stB);
        for (int s = 0; s < G_NS; ++s) {
          for (int u = 0; u + s < G_NS; ++u) {
            const uint32_t acc = tmem + (uint32_t)((s + u) * G_TILE_N);
#pragma unroll
            for (int k4 = 0; k4 < KBLK / 16; ++k4) {
              const uint64_t ad = sw128_desc(a0 + s * G_A_BYTES + k4 * 32);
              const uint64_t bd = sw128_desc(b0 + u * G_B_BYTES + k4 * 32);
              // each diagonal restarts with its (1, d + 1) product
              mma_bf16(acc, ad, bd, idesc, (first && s == 0 && k4 == 0) ? 0u : 1u);
            }
          }
        }
        mma_commit(empty);
        if ((it % G_CHUNK) == G_CHUNK - 1 || it == nloc - 1) mma_commit(acc_ready);
      }
      mma_commit(mma_done);
      int dummy = 0;
      mbar_wait(mma_done, 0, &dummy);
    }
  } else {
    const int q4 = warp & 3;
    const int half = (warp - 2) >> 2;
    const uint32_t lane_base = (uint32_t)(32 * q4) << 16;
    long long X[G_COLS];
#pragma unroll
    for (int c = 0; c < G_COLS; ++c) X[c] = 0;
    bool ok = true;
    const int nch = (nloc + G_CHUNK - 1) / G_CHUNK;
    for (int ch = 0; ch < nch; ++ch) {
      if (!mbar_wait(acc_ready, ch & 1, P.err)) {
        ok = false;
        break;
      }
      tc_fence_after();
#pragma unroll 1
      for (int d = 0; d < G_NS; ++d) {
        uint32_t r[32];
        tmem_ld32(tmem + lane_base + (uint32_t)(d * G_TILE_N + half * G_COLS), r);
        const int w = 8 * (G_NS - 1 - d) - t;
        // |acc| <= 2^24: exact through a 32-bit conversion
        if (w >= 0) {
#pragma unroll
          for (int c = 0; c < G_COLS; ++c) X[c] += (long long)__float2int_rn(__uint_as_float(r[c])) << w;
        } else {
#pragma unroll
          for (int c = 0; c < G_COLS; ++c) {
            const long long v = __float2int_rn(__uint_as_float(r[c]));
            X[c] += (v + (1ll << (-w - 1))) >> (-w);  // round half up at weight 2^w
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acc_free);
    }
    const int64_t i = m_tile * G_TILE_M + 32 * q4 + lane;
    if (ok && i < P.M) {
      const int ea = P.ea[i];
      const int64_t j0 = n_tile * G_TILE_N + half * G_COLS;
#pragma unroll
      for (int c = 0; c < G_COLS; ++c) {
        const int64_t j = j0 + c;
        if (j < P.N) {
          const int eb = P.eb[j];
          const double v = (ea >= kNonFinite || eb >= kNonFinite) ? __longlong_as_double(0x7FF8000000000000ll)
                                                                   : ldexp((double)X[c], ea + eb - 56 + t);
          if (P.to_ws) {
            P.C[(int64_t)blockIdx.y * P.M * P.N + i + j * P.M] = v;
          } else {
            double* cp = P.C + i + j * P.ldc;
            *cp = P.beta == 0.0 ? P.alpha * v : P.alpha * v + P.beta * *cp;
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
  }
}

__global__ void tc_gemm_reduce_kernel(int64_t m, int64_t n, int64_t nsplit, const double* __restrict__ W,
                                      double alpha, double beta, double* __restrict__ C, int64_t ldc) {
  const int64_t total = m * n;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = q % m, j = q / m;
    double s = 0;
    for (int64_t z = 0; z < nsplit; ++z) s += W[z * total + q];
    double* c = C + i + j * ldc;
    *c = beta == 0.0 ? alpha * s : alpha * s + beta * *c;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  // looked up once per process, safely under concurrent first calls
  static std::atomic<PFN_cuTensorMapEncodeTiled_v12000> fn{nullptr};
  PFN_cuTensorMapEncodeTiled_v12000 f = fn.load(std::memory_order_acquire);
  if (!f) {
    cudaDriverEntryPointQueryResult q;
    void* p = nullptr;
    check_cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
               "cudaGetDriverEntryPoint(cuTensorMapEncodeTiled)");
    if (q != cudaDriverEntryPointSuccess || !p) fail(LRA_ECUDA, "cuTensorMapEncodeTiled unavailable");
    f = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    fn.store(f, std::memory_order_release);
  }
  return f;
}

void make_map(CUtensorMap* m, void* ptr, int rank, const cuuint64_t* dims, const cuuint64_t* strides,
              const cuuint32_t* box) {
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, ptr, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(LRA_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
}

inline unsigned nblk(lra_ctx* ctx, int64_t n, int t) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, (int64_t)ctx->num_sms * 16));
}

}  // namespace

bool tc_sketch_supported(int64_t order, int64_t M, int64_t N) {
  // K extent and counts kept inside int32 TMA coordinates
  return order > 0 && M > 0 && N > 0 && M < (1ll << 30) && N < (1ll << 30) && order < (1ll << 20);
}

template <typename T>
void tc_split(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda, int ns, TcSplit* out,
              bool balanced) {
  const int W = 8 * ns;
  const int n_exact = balanced ? 0 : std::min(ns, MAX_EXACT);
  const int64_t Kp = (M + 7) / 8 * 8;
  out->K = M;
  out->N = N;
  out->Kp = Kp;
  out->ns = ns;
  out->trans = trans;
  out->colexp = ctx->arena.alloc_n<int>(std::max<int64_t>(N, 1));
  out->slices = ctx->arena.alloc_n<__nv_bfloat16>((size_t)ns * Kp * std::max<int64_t>(N, 1));
  if (trans == 'c') {
    {
      const ArenaMark mk = ctx->arena.mark();
      unsigned long long* mx = ctx->arena.alloc_n<unsigned long long>(std::max<int64_t>(N, 1));
      LRA_CUDA(cudaMemsetAsync(mx, 0, std::max<int64_t>(N, 1) * sizeof(unsigned long long), ctx->stream));
      const int64_t tiles = ((N + 31) / 32) * ((M + 255) / 256);
      rowmax_kernel<T><<<(unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 16), dim3(32, 8), 0,
                         ctx->stream>>>(M, N, A, lda, mx);
      post_launch(ctx, "rowmax_kernel");
      rowmax_exp_kernel<<<nblk(ctx, N, 256), 256, 0, ctx->stream>>>(N, mx, out->colexp);
      post_launch(ctx, "rowmax_exp_kernel");
      ctx->arena.release(mk);  // stream-ordered reuse
    }
    const int64_t tiles = ((Kp + 31) / 32) * ((N + 31) / 32);
    split_c_kernel<T><<<(unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 16), dim3(32, 8), 0,
                        ctx->stream>>>(M, N, A, lda, out->colexp, ns, n_exact, W,
                                       static_cast<__nv_bfloat16*>(out->slices), Kp);
    post_launch(ctx, "split_c_kernel");
  } else {
    colexp_n_kernel<T><<<nblk(ctx, N, 8), 256, 0, ctx->stream>>>(M, N, A, lda, out->colexp);
    post_launch(ctx, "colexp_n_kernel");
    split_n_kernel<T><<<nblk(ctx, Kp * N, 256), 256, 0, ctx->stream>>>(
        M, N, A, lda, out->colexp, ns, n_exact, W, static_cast<__nv_bfloat16*>(out->slices), Kp);
    post_launch(ctx, "split_n_kernel");
  }
}

// the tile N of the tuning table for this element type and sketch order
static int tuned_tile_n(const lra_ctx* ctx, bool f64, int64_t order) {
  int lb = 0;
  while (lb < 15 && ((int64_t)1 << lb) < order) ++lb;
  const int v = ctx->tuning.tc_tile_n[f64 ? 1 : 0][lb];
  return (v == 32 || v == 64) ? v : 96;
}

template <typename T>
void tc_sketch(lra_ctx* ctx, const TcSplit& sp, int64_t order, const T* S, T* B, int64_t ldb, int* err_slot) {
  const int64_t K = sp.K, N = sp.N, Kp = sp.Kp;
  const int ns = sp.ns;
  const int TILE_N = tuned_tile_n(ctx, sizeof(T) == 8, order);
  const int64_t Lp = (order + TILE_N - 1) / TILE_N * TILE_N;
  const ArenaMark mk = ctx->arena.mark();
  __nv_bfloat16* St = ctx->arena.alloc_n<__nv_bfloat16>((size_t)Kp * Lp);
  {
    const int64_t tiles = ((Lp + 31) / 32) * ((Kp + 31) / 32);
    sketch_t_kernel<T><<<(unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 16), dim3(32, 8), 0,
                         ctx->stream>>>(order, K, S, Lp, Kp, St);
    post_launch(ctx, "sketch_t_kernel");
  }
  CUtensorMap tmA, tmS;
  {
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)N, (cuuint64_t)ns};
    cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * N * 2};
    cuuint32_t box[3] = {KBLK, TILE_M, 1};
    make_map(&tmA, sp.slices, 3, dims, strides, box);
  }
  {
    cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)Lp};
    cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
    cuuint32_t box[2] = {KBLK, (cuuint32_t)TILE_N};
    make_map(&tmS, St, 2, dims, strides, box);
  }
  int* err = err_slot;
  if (!err) {
    err = ctx->arena.alloc_n<int>(1);
    LRA_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  }
  TcParams P;
  P.K = K;
  P.ncols = N;
  P.L = order;
  P.ns = ns;
  // |X| < 2^(24 + 8(E-1) + t + log2(chunks)): keep t = 8 while that is < 2^62
  P.tshift = ((K + 511) / 512 <= 64) ? 8 : 0;
  P.colexp = sp.colexp;
  P.B = B;
  P.ldb = ldb;
  P.out_double = sizeof(T) == 8 ? 1 : 0;
  P.err = err;
  // two ring stages when two CTAs fit an SM (their loads interleave), else
  // as many stages as the one CTA's shared memory holds
  const size_t stage_bytes = (size_t)TILE_N * KBLK * 2 + (size_t)ns * TILE_BYTES;
  int smem_optin = 0, smem_sm = 0;
  LRA_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  LRA_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
  const bool two_ctas = 2 * (2 * stage_bytes + 1024 + 256 + 1024) <= (size_t)smem_sm;
  P.nstage = two_ctas ? 2
                      : (int)std::max<size_t>(2, std::min<size_t>(MAX_NSTAGE, ((size_t)smem_optin - 1024 - 256) / stage_bytes));
  const size_t smem = 1024 + (size_t)P.nstage * stage_bytes + 256;
  const int64_t ntiles = ((N + TILE_M - 1) / TILE_M) * (Lp / TILE_N);
  // too few tiles for two CTAs per SM: split K over more CTAs (whole
  // chunks each, at least two), their exact sums added as integers
  const int nkb = (int)((K + KBLK - 1) / KBLK);
  const int nchunks = (nkb + CHUNK_KB - 1) / CHUNK_KB;
  int nsplit = 1;
  if (ntiles < 2 * (int64_t)ctx->num_sms && nchunks >= 4)
    nsplit = (int)std::min<int64_t>((2 * (int64_t)ctx->num_sms + ntiles - 1) / ntiles, nchunks / 2);
  if (ctx->tuning.tc_split > 0) nsplit = std::min(nsplit, ctx->tuning.tc_split);
  P.kc_per = (nchunks + nsplit - 1) / nsplit;
  nsplit = (nchunks + P.kc_per - 1) / P.kc_per;
  P.W = nullptr;
  P.ldw = Lp;
  if (nsplit > 1) {
    P.W = ctx->arena.alloc_n<long long>((size_t)Lp * N);
    LRA_CUDA(cudaMemsetAsync(P.W, 0, (size_t)Lp * N * sizeof(long long), ctx->stream));
  }
  auto launch = [&](auto kern) {
    raise_smem_limit(ctx, (const void*)kern);
    kern<<<dim3((unsigned)ntiles, (unsigned)nsplit), NTHREADS, smem, ctx->stream>>>(tmA, tmS, P);
  };
  if (TILE_N == 32)
    launch(tc_sketch_kernel<32>);
  else if (TILE_N == 64)
    launch(tc_sketch_kernel<64>);
  else
    launch(tc_sketch_kernel<96>);
  post_launch(ctx, "tc_sketch_kernel");
  if (nsplit > 1) {
    const int n_exact = ns < MAX_EXACT ? ns : MAX_EXACT;
    const int t = ns > MAX_EXACT ? P.tshift : 0;
    const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((order * N + 255) / 256, ctx->num_sms * 8));
    tc_sketch_finish_kernel<<<g, 256, 0, ctx->stream>>>(order, N, P.W, Lp, sp.colexp, n_exact, t, B, ldb,
                                                         P.out_double);
    post_launch(ctx, "tc_sketch_finish_kernel");
  }
  // a caller that passes err_slot checks it later (the batch, once per
  // round) and releases the transposed sketch with its own arena mark: the
  // batch issues sketches on several streams, so this memory may not be
  // reused before they have all run
  if (err_slot) return;
  int herr = 0;
  LRA_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  if (herr) fail(LRA_ETIMEDOUT, "tc_sketch: a bounded wait timed out");
}

bool tc_gemm_worthwhile(int64_t m, int64_t n, int64_t k) {
  return m > 0 && n > 0 && k > 0 && (double)m * n * k >= 16.0 * 1024 * 1024 && m < (1ll << 30) &&
         n < (1ll << 30) && k < (1ll << 30);
}

void tc_gemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A,
             int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc) {
  const bool TA = (ta == 't' || ta == 'T' || ta == 'c' || ta == 'C');
  const bool TB = (tb == 't' || tb == 'T' || tb == 'c' || tb == 'C');
  const ArenaMark mk = ctx->arena.mark();
  // X_A = op(A)^T (k x m) and X_B = op(B) (k x n), split by columns
  TcSplit sa, sb;
  tc_split<double>(ctx, TA ? 'n' : 'c', k, m, A, lda, G_NS, &sa, true);
  tc_split<double>(ctx, TB ? 'c' : 'n', k, n, B, ldb, G_NS, &sb, true);
  const int64_t Kp = sa.Kp;
  CUtensorMap tmA, tmB;
  {
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)m, (cuuint64_t)G_NS};
    cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * m * 2};
    cuuint32_t box[3] = {KBLK, G_TILE_M, 1};
    make_map(&tmA, sa.slices, 3, dims, strides, box);
  }
  {
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)n, (cuuint64_t)G_NS};
    cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * n * 2};
    cuuint32_t box[3] = {KBLK, G_TILE_N, 1};
    make_map(&tmB, sb.slices, 3, dims, strides, box);
  }
  const int nkb = (int)((k + KBLK - 1) / KBLK);
  const int64_t tiles = ((m + G_TILE_M - 1) / G_TILE_M) * ((n + G_TILE_N - 1) / G_TILE_N);
  // split K while the tiles alone leave SMs idle (down to one K block each:
  // a k x k product of the post-processing has few tiles and few K blocks,
  // and one CTA per tile would run its K blocks one stage at a time)
  int64_t nsplit = 1;
  if (tiles < ctx->num_sms) nsplit = std::max<int64_t>(1, std::min<int64_t>((ctx->num_sms + tiles - 1) / tiles, nkb));
  const int kb_per = (int)((nkb + nsplit - 1) / nsplit);
  nsplit = (nkb + kb_per - 1) / kb_per;
  // |X| <= chunks * 2^(24 + 40 - t) (1 + 2^-7 + ...): t = ceil(log2(chunks)) + 1
  const int chunks = (kb_per + G_CHUNK - 1) / G_CHUNK;
  int tsh = 1;
  while ((1 << (tsh - 1)) < chunks) ++tsh;
  // a timed-out wait is reported when the library call ends (the context's
  // error word), so that consecutive GEMMs queue without a host round trip
  if (!ctx->dev_err) {
    LRA_CUDA(cudaMalloc(&ctx->dev_err, sizeof(int)));
    LRA_CUDA(cudaMemsetAsync(ctx->dev_err, 0, sizeof(int), ctx->stream));
  }
  ctx->dev_err_armed = true;
  int* err = ctx->dev_err;
  TgParams P;
  P.M = m;
  P.N = n;
  P.nkb = nkb;
  P.kb_per = kb_per;
  P.tshift = tsh;
  P.ea = sa.colexp;
  P.eb = sb.colexp;
  P.alpha = alpha;
  P.beta = beta;
  P.err = err;
  double* ws = nullptr;
  if (nsplit > 1) {
    ws = ctx->arena.alloc_n<double>((size_t)nsplit * m * n);
    P.C = ws;
    P.ldc = m;
    P.to_ws = 1;
  } else {
    P.C = C;
    P.ldc = ldc;
    P.to_ws = 0;
  }
  const size_t smem = 1024 + (size_t)G_STAGE + 256;
  raise_smem_limit(ctx, (const void*)tc_gemm_kernel);
  tc_gemm_kernel<<<dim3((unsigned)tiles, (unsigned)nsplit), NTHREADS, smem, ctx->stream>>>(tmA, tmB, P);
  post_launch(ctx, "tc_gemm_kernel");
  if (nsplit > 1) {
    const unsigned g = nblk(ctx, m * n, 256);
    tc_gemm_reduce_kernel<<<g, 256, 0, ctx->stream>>>(m, n, nsplit, ws, alpha, beta, C, ldc);
    post_launch(ctx, "tc_gemm_reduce_kernel");
  }
  ctx->arena.release(mk);  // stream-ordered reuse
}

template void tc_split<float>(lra_ctx*, char, int64_t, int64_t, const float*, int64_t, int, TcSplit*, bool);
template void tc_split<double>(lra_ctx*, char, int64_t, int64_t, const double*, int64_t, int, TcSplit*, bool);
template void tc_sketch<float>(lra_ctx*, const TcSplit&, int64_t, const float*, float*, int64_t, int*);
template void tc_sketch<double>(lra_ctx*, const TcSplit&, int64_t, const double*, double*, int64_t, int*);

cudaError_t set_wait_limit_tc(uint64_t ns) { return set_unit_wait_limit(ns); }

}  // namespace lra
