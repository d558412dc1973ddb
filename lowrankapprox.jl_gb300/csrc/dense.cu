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
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <mutex>
#include <set>
#include <vector>

#include "common.cuh"
#include "df64.cuh"
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
  // block Jacobi: V stays in global memory (only X's block pair in shared
  // memory), so that longer columns fit 8-column blocks
  int vglobal = 0;
  // LRA_TRACE: CTA 0's time in each phase of the block kernel, summed over
  // its block pairs (ns): load, local rounds, V, write-back, barrier
  unsigned long long* phase_ns = nullptr;
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
  __shared__ T red[2][NT][3];
  __shared__ T rot_c[2], rot_s[2];
  __shared__ int rot_on[2];
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
        // partial dot products to shared memory; warp 0 alone reduces them
        // and computes the rotation (FP64 instructions cost tens of cycles
        // each here, so they are not repeated in every warp)
        red[buf][threadIdx.x][0] = a;
        red[buf][threadIdx.x][1] = b;
        red[buf][threadIdx.x][2] = g;
        __syncthreads();
        if (wid == 0) {
          T ra = 0, rb = 0, rg = 0;
#pragma unroll
          for (int k = 0; k < NW; ++k) {
            ra += red[buf][lane + 32 * k][0];
            rb += red[buf][lane + 32 * k][1];
            rg += red[buf][lane + 32 * k][2];
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            ra += __shfl_xor_sync(0xffffffffu, ra, o);
            rb += __shfl_xor_sync(0xffffffffu, rb, o);
            rg += __shfl_xor_sync(0xffffffffu, rg, o);
          }
          T cs = 1, sn = 0;
          int rot = 0;
          if (ra != 0 && rb != 0) {
            const T g2 = rg * rg, ab = ra * rb;
            if (g2 > tol2 * ab) {
              rot = 1;
              if (g2 > stop2 * ab) above = 1;
              // t = tan of the rotation angle, the smaller root of t^2 + 2 zeta t - 1
              const T d = rb - ra;
              const T t = (T(2) * rg) / (d + copysign(sqrt(fma(d, d, T(4) * g2)), d));
              cs = T(1) / sqrt(fma(t, t, T(1)));
              sn = cs * t;
            }
          }
          if (lane == 0) {
            rot_c[buf] = cs;
            rot_s[buf] = sn;
            rot_on[buf] = rot;
          }
        }
        __syncthreads();
        const int on = rot_on[buf];
        const T c = rot_c[buf], sn = rot_s[buf];
        buf ^= 1;  // the next pair reduces through the other buffer
        if (!on) continue;
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
    // any CTA above the stopping level keeps the sweeps going (warp 0 holds
    // the flag of this CTA)
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

// two FP32 values in one 64-bit register pair, for the packed FP32 pipe
// (fma/mul .f32x2: one instruction for both halves)
typedef unsigned long long f2_t;
__device__ __forceinline__ f2_t f2_pack(float lo, float hi) {
  f2_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ float f2_lo(f2_t v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float f2_hi(f2_t v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// Block one-sided Jacobi for the FP32 sweeps: the columns are grouped in
// blocks of JB; each grid-wide round pairs the blocks round-robin, and the
// CTA holding a block pair loads its 2 JB columns of X and V into shared
// memory and rotates every pair among them there (2 JB - 1 local rounds of
// JB pairs, a warp per pair) before writing them back.  A sweep then costs
// about n / JB grid barriers instead of n, and the local rotations also
// reach the pairs inside each block.  The local rotations are applied to X
// one by one and gathered into a 2 JB x 2 JB orthogonal matrix, which is
// applied to the block's columns of V once, a thread per row, after the
// local rounds.
constexpr int JB = 8;
constexpr int JB_RPL = 16;  // rows per lane in registers (columns up to 512 long)
constexpr int JB_QMAX = 16;  // 16-byte chunks a lane holds in the inter-block steps (columns up to 2048 long)

// 16 bytes, of which the first `bytes` come from src and the rest are zero
__device__ __forceinline__ void cp_async16z(float* dst, const float* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}

template <int JBT>
__global__ void __launch_bounds__(JBT * 32) jacobi_block_kernel(JacParams<float> P) {
  extern __shared__ float jb_smem[];
  __shared__ double red[32];
  __shared__ __align__(16) float Ql[2 * JBT][2 * JBT];  // column k of the block's local rotation at Ql[k][.]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t n = P.n;
  // column stride in shared memory: n rounded up to 16 bytes, the padding
  // rows zero, so that long columns move in 16-byte vectors
  const int64_t ld = (n + 3) & ~(int64_t)3;
  float* Xs = jb_smem;                        // [2 JBT][ld]
  float* Vs = jb_smem + (size_t)2 * JBT * ld;  // [2 JBT][ld], unless V stays in global memory
  const bool vg = P.vglobal != 0;
  // columns that start on 16 bytes move as 16-byte vectors
  const bool vec16 = (P.ldx & 3) == 0 && ((uintptr_t)P.X & 15) == 0 &&
                     (vg || ((P.ldv & 3) == 0 && ((uintptr_t)P.V & 15) == 0));
  const int64_t nblk = (n + JBT - 1) / JBT;
  const int64_t nbb = nblk + (nblk & 1);
  const float tol = (float)P.tol;
  int sweep = 0;
  for (; sweep < P.max_sweeps; ++sweep) {
    float off = 0;
    for (int64_t r = 0; r < nbb - 1; ++r) {
      for (int64_t s = blockIdx.x; s < nbb / 2; s += gridDim.x) {
        const bool stamp = P.phase_ns && blockIdx.x == 0 && threadIdx.x == 0;
        uint64_t t_ph = stamp ? globaltimer_ns() : 0;
        auto phase = [&](int i) {
          if (!stamp) return;
          const uint64_t t = globaltimer_ns();
          P.phase_ns[i] += t - t_ph;
          t_ph = t;
        };
        int64_t b1, b2;
        rr_pair(r, s, nbb, b1, b2);
        // local column k < JBT is column b1 JBT + k, k >= JBT is b2 JBT + k - JBT
        auto gcol = [&](int k) -> int64_t {
          const int64_t b = k < JBT ? b1 : b2;
          if (b >= nblk) return -1;
          const int64_t j = b * JBT + (k % JBT);
          return j < n ? j : -1;
        };
        // all 4 JBT n elements in flight at once (asynchronous copies), in
        // 16-byte vectors when the columns start on 16 bytes (the rows past n
        // zero-filled)
        for (int k = 0; k < 2 * JBT; ++k) {
          const int64_t j = gcol(k);
          if (vec16) {
            for (int64_t i = 4 * (int64_t)threadIdx.x; i < ld; i += 4 * JBT * 32) {
              const int bytes = j >= 0 ? (int)(4 * min((int64_t)4, n - i)) : 0;
              cp_async16z(Xs + k * ld + i, P.X + (j >= 0 ? i + j * P.ldx : 0), bytes);
              if (!vg) cp_async16z(Vs + k * ld + i, P.V + (j >= 0 ? i + j * P.ldv : 0), bytes);
            }
            continue;
          }
          for (int64_t i = threadIdx.x; i < ld; i += JBT * 32) {
            if (j >= 0 && i < n) {
              cp_async4(Xs + k * ld + i, P.X + i + j * P.ldx);
              if (!vg) cp_async4(Vs + k * ld + i, P.V + i + j * P.ldv);
            } else {
              Xs[k * ld + i] = 0.0f;
              if (!vg) Vs[k * ld + i] = 0.0f;
            }
          }
        }
        for (int e = threadIdx.x; e < 4 * JBT * JBT; e += JBT * 32)
          Ql[e / (2 * JBT)][e % (2 * JBT)] = e / (2 * JBT) == e % (2 * JBT) ? 1.0f : 0.0f;
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
        phase(0);
        unsigned long long vmask = 0;  // local columns that exist
#pragma unroll
        for (int k = 0; k < 2 * JBT; ++k) vmask |= (gcol(k) >= 0 ? 1ull : 0ull) << k;
        const int ni = (int)n;
        // Past the first round of a sweep (whose full local sweeps also
        // rotate the pairs inside each block, once a sweep), the block pair
        // of long columns takes inter-block steps only: warp w keeps column w
        // of block b1 in registers and meets column (w + step) mod JBT of
        // block b2, which moves from warp to warp through shared memory --
        // every inter-block pair once, in JBT steps that read and write one
        // column a warp instead of 2 JBT - 1 rounds that read and write all.
        // (registers for up to 2048 rows with 8-column blocks and fewer;
        // larger blocks have too few registers a thread)
        constexpr int QM = JBT <= 8 ? JB_QMAX : 1;
        const bool inter = r > 0 && ni > 32 * JB_RPL && ld <= (int64_t)4 * 32 * QM;
        if (inter) {
          const int p = wid;
          const int nq = (int)(ld / 4);
          const ulonglong2 z2 = make_ulonglong2(0ull, 0ull);
          ulonglong2* tp = reinterpret_cast<ulonglong2*>(Xs + p * ld);
          ulonglong2 top[QM];
#pragma unroll
          for (int c = 0; c < QM; ++c) {
            const int v = lane + 32 * c;
            top[c] = v < nq ? tp[v] : z2;
          }
          const bool pe = (vmask >> p) & 1ull;
          for (int st = 0; st < JBT; ++st) {
            const int q = JBT + (wid + st) % JBT;
            if (pe && ((vmask >> q) & 1ull)) {
              ulonglong2* qp = reinterpret_cast<ulonglong2*>(Xs + q * ld);
              ulonglong2 bot[QM];
#pragma unroll
              for (int c = 0; c < QM; ++c) {
                const int v = lane + 32 * c;
                bot[c] = v < nq ? qp[v] : z2;
              }
              f2_t a2 = 0, b2 = 0, g2 = 0;
#pragma unroll
              for (int c = 0; c < QM; ++c) {
                a2 = f2_fma(top[c].x, top[c].x, a2);
                a2 = f2_fma(top[c].y, top[c].y, a2);
                b2 = f2_fma(bot[c].x, bot[c].x, b2);
                b2 = f2_fma(bot[c].y, bot[c].y, b2);
                g2 = f2_fma(top[c].x, bot[c].x, g2);
                g2 = f2_fma(top[c].y, bot[c].y, g2);
              }
              const float a = warp_sum(f2_lo(a2) + f2_hi(a2));
              const float b = warp_sum(f2_lo(b2) + f2_hi(b2));
              const float g = warp_sum(f2_lo(g2) + f2_hi(g2));
              if (a != 0 && b != 0) {
                const float rel = fabsf(g) * rsqrtf(a * b);
                if (rel > tol) {
                  off = fmaxf(off, rel);
                  const float zeta = (b - a) / (2.0f * g);
                  const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                  const float c = rsqrtf(1.0f + t * t);
                  const float sn = c * t;
                  const f2_t cc = f2_pack(c, c), ss = f2_pack(sn, sn), ns = f2_pack(-sn, -sn);
#pragma unroll
                  for (int k = 0; k < QM; ++k) {
                    const ulonglong2 u = top[k], w = bot[k];
                    top[k].x = f2_fma(ns, w.x, f2_mul(cc, u.x));
                    top[k].y = f2_fma(ns, w.y, f2_mul(cc, u.y));
                    bot[k].x = f2_fma(cc, w.x, f2_mul(ss, u.x));
                    bot[k].y = f2_fma(cc, w.y, f2_mul(ss, u.y));
                    const int v = lane + 32 * k;
                    if (v < nq) qp[v] = bot[k];
                  }
                  for (int l = lane; l < 2 * JBT; l += 32) {
                    const float qu = Ql[p][l], qw = Ql[q][l];
                    Ql[p][l] = c * qu - sn * qw;
                    Ql[q][l] = sn * qu + c * qw;
                  }
                }
              }
            }
            __syncthreads();
          }
#pragma unroll
          for (int c = 0; c < QM; ++c) {
            const int v = lane + 32 * c;
            if (v < nq) tp[v] = top[c];
          }
          __syncthreads();
        } else {
          for (int lr = 0; lr < 2 * JBT - 1; ++lr) {
            // round-robin pair of this warp among the 2 JBT local columns
            auto lpos = [&](int i) { return i == 0 ? 0 : 1 + (i - 1 + lr) % (2 * JBT - 1); };
            int p = lpos(wid), q = lpos(2 * JBT - 1 - wid);
            if (p > q) {
              const int t = p;
              p = q;
              q = t;
            }
            if (((vmask >> p) & 1ull) && ((vmask >> q) & 1ull)) {
              float* xp = Xs + p * ld;
              float* xq = Xs + q * ld;
              float a = 0, b = 0, g = 0;
              if (ni <= 32 * JB_RPL) {
                // both columns in registers for the dots and the update
                float u[JB_RPL], w[JB_RPL];
  #pragma unroll
                for (int t = 0; t < JB_RPL; ++t) {
                  const int i = lane + 32 * t;
                  u[t] = i < ni ? xp[i] : 0.0f;
                  w[t] = i < ni ? xq[i] : 0.0f;
                }
  #pragma unroll
                for (int t = 0; t < JB_RPL; ++t) {
                  a = fmaf(u[t], u[t], a);
                  b = fmaf(w[t], w[t], b);
                  g = fmaf(u[t], w[t], g);
                }
                a = warp_sum(a);
                b = warp_sum(b);
                g = warp_sum(g);
                if (a != 0 && b != 0) {
                  const float rel = fabsf(g) * rsqrtf(a * b);
                  if (rel > tol) {
                    off = fmaxf(off, rel);
                    const float zeta = (b - a) / (2.0f * g);
                    const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                    const float c = rsqrtf(1.0f + t * t);
                    const float sn = c * t;
  #pragma unroll
                    for (int tt = 0; tt < JB_RPL; ++tt) {
                      const int i = lane + 32 * tt;
                      if (i < ni) {
                        xp[i] = c * u[tt] - sn * w[tt];
                        xq[i] = sn * u[tt] + c * w[tt];
                      }
                    }
                    for (int l = lane; l < 2 * JBT; l += 32) {
                      const float qu = Ql[p][l], qw = Ql[q][l];
                      Ql[p][l] = c * qu - sn * qw;
                      Ql[q][l] = sn * qu + c * qw;
                    }
                  }
                }
              } else {
                // long columns: 16-byte vectors (rows 4v .. 4v + 3 in lane v
                // mod 32) and the packed FP32 pipe, two accumulators a value
                const ulonglong2* vp = reinterpret_cast<const ulonglong2*>(xp);
                const ulonglong2* vq = reinterpret_cast<const ulonglong2*>(xq);
                const int nv = (int)(ld / 4);
                f2_t a2 = 0, b2 = 0, g2 = 0;
  #pragma unroll 4
                for (int v = lane; v < nv; v += 32) {
                  const ulonglong2 u = vp[v], w = vq[v];
                  a2 = f2_fma(u.x, u.x, a2);
                  a2 = f2_fma(u.y, u.y, a2);
                  b2 = f2_fma(w.x, w.x, b2);
                  b2 = f2_fma(w.y, w.y, b2);
                  g2 = f2_fma(u.x, w.x, g2);
                  g2 = f2_fma(u.y, w.y, g2);
                }
                a = warp_sum(f2_lo(a2) + f2_hi(a2));
                b = warp_sum(f2_lo(b2) + f2_hi(b2));
                g = warp_sum(f2_lo(g2) + f2_hi(g2));
                if (a != 0 && b != 0) {
                  const float rel = fabsf(g) * rsqrtf(a * b);
                  if (rel > tol) {
                    off = fmaxf(off, rel);
                    const float zeta = (b - a) / (2.0f * g);
                    const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                    const float c = rsqrtf(1.0f + t * t);
                    const float sn = c * t;
                    const f2_t cc = f2_pack(c, c), ss = f2_pack(sn, sn), ns = f2_pack(-sn, -sn);
                    ulonglong2* wp = reinterpret_cast<ulonglong2*>(xp);
                    ulonglong2* wq = reinterpret_cast<ulonglong2*>(xq);
  #pragma unroll 4
                    for (int v = lane; v < nv; v += 32) {
                      const ulonglong2 u = wp[v], w = wq[v];
                      ulonglong2 up, uq;
                      up.x = f2_fma(ns, w.x, f2_mul(cc, u.x));
                      up.y = f2_fma(ns, w.y, f2_mul(cc, u.y));
                      uq.x = f2_fma(cc, w.x, f2_mul(ss, u.x));
                      uq.y = f2_fma(cc, w.y, f2_mul(ss, u.y));
                      wp[v] = up;
                      wq[v] = uq;
                    }
                    for (int l = lane; l < 2 * JBT; l += 32) {
                      const float qu = Ql[p][l], qw = Ql[q][l];
                      Ql[p][l] = c * qu - sn * qw;
                      Ql[q][l] = sn * qu + c * qw;
                    }
                  }
                }
              }
            }
            __syncthreads();
          }
        }
        phase(1);
        // the block's columns of V times the gathered rotation, a thread per
        // row (rows of V read and written in place, coalesced, when V stays
        // in global memory)
        if constexpr (JBT <= 8) {
          // two rows a thread at once: their 4 JBT entries are loaded
          // together (the latencies overlap), and each 16-byte read of the
          // rotation (which the compiler may not hoist out of the row loop)
          // serves both
          constexpr int NT = JBT * 32;
          for (int i = threadIdx.x; i < ni; i += 2 * NT) {
            const int i2 = i + NT;
            const bool two = i2 < ni;
            float v0[2 * JBT], v1[2 * JBT];
#pragma unroll
            for (int j = 0; j < 2 * JBT; ++j) {
              if (vg) {
                const int64_t gj = gcol(j);
                v0[j] = gj >= 0 ? P.V[i + gj * P.ldv] : 0.0f;
                v1[j] = gj >= 0 && two ? P.V[i2 + gj * P.ldv] : 0.0f;
              } else {
                v0[j] = Vs[j * ld + i];
                v1[j] = two ? Vs[j * ld + i2] : 0.0f;
              }
            }
#pragma unroll
            for (int k = 0; k < 2 * JBT; ++k) {
              float s0 = 0.0f, s1 = 0.0f;
#pragma unroll
              for (int j = 0; j < 2 * JBT; j += 4) {
                float4 q;
                asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                             : "=f"(q.x), "=f"(q.y), "=f"(q.z), "=f"(q.w)
                             : "r"((uint32_t)__cvta_generic_to_shared(&Ql[k][j])));
                s0 = fmaf(v0[j], q.x, s0);
                s0 = fmaf(v0[j + 1], q.y, s0);
                s0 = fmaf(v0[j + 2], q.z, s0);
                s0 = fmaf(v0[j + 3], q.w, s0);
                s1 = fmaf(v1[j], q.x, s1);
                s1 = fmaf(v1[j + 1], q.y, s1);
                s1 = fmaf(v1[j + 2], q.z, s1);
                s1 = fmaf(v1[j + 3], q.w, s1);
              }
              if (vg) {
                const int64_t gk = gcol(k);
                if (gk >= 0) {
                  P.V[i + gk * P.ldv] = s0;
                  if (two) P.V[i2 + gk * P.ldv] = s1;
                }
              } else {
                Vs[k * ld + i] = s0;
                if (two) Vs[k * ld + i2] = s1;
              }
            }
          }
        } else {
          for (int i = threadIdx.x; i < ni; i += JBT * 32) {
            float acc[2 * JBT];
#pragma unroll
            for (int k = 0; k < 2 * JBT; ++k) acc[k] = 0.0f;
#pragma unroll 1
            for (int j = 0; j < 2 * JBT; ++j) {  // (not unrolled: Ql would be hoisted into registers)
              float v;
              if (vg) {
                const int64_t gj = gcol(j);
                v = gj >= 0 ? P.V[i + gj * P.ldv] : 0.0f;
              } else {
                v = Vs[j * ld + i];
              }
#pragma unroll
              for (int k = 0; k < 2 * JBT; ++k) acc[k] = fmaf(v, Ql[k][j], acc[k]);
            }
            if (vg) {
#pragma unroll
              for (int k = 0; k < 2 * JBT; ++k) {
                const int64_t gk = gcol(k);
                if (gk >= 0) P.V[i + gk * P.ldv] = acc[k];
              }
            } else {
#pragma unroll
              for (int k = 0; k < 2 * JBT; ++k) Vs[k * ld + i] = acc[k];
            }
          }
        }
        __syncthreads();
        phase(2);
        for (int k = 0; k < 2 * JBT; ++k) {
          const int64_t j = gcol(k);
          if (j < 0) continue;
          if (vec16) {
            // whole vectors up to the last full one, the rest by element
            const int64_t n4 = n & ~(int64_t)3;
            for (int64_t i = 4 * (int64_t)threadIdx.x; i < n4; i += 4 * JBT * 32) {
              *reinterpret_cast<float4*>(P.X + i + j * P.ldx) = *reinterpret_cast<const float4*>(Xs + k * ld + i);
              if (!vg)
                *reinterpret_cast<float4*>(P.V + i + j * P.ldv) = *reinterpret_cast<const float4*>(Vs + k * ld + i);
            }
            for (int64_t i = n4 + threadIdx.x; i < n; i += JBT * 32) {
              P.X[i + j * P.ldx] = Xs[k * ld + i];
              if (!vg) P.V[i + j * P.ldv] = Vs[k * ld + i];
            }
            continue;
          }
          for (int64_t i = threadIdx.x; i < n; i += JBT * 32) {
            P.X[i + j * P.ldx] = Xs[k * ld + i];
            if (!vg) P.V[i + j * P.ldv] = Vs[k * ld + i];
          }
        }
        __syncthreads();
        phase(3);
      }
      {
        const uint64_t t0 = P.phase_ns && blockIdx.x == 0 && threadIdx.x == 0 ? globaltimer_ns() : 0;
        if (!grid_sync(P.bar)) return;
        if (t0) P.phase_ns[4] += globaltimer_ns() - t0;
      }
    }
    const double offd = block_max((double)off, red);
    if (threadIdx.x == 0) P.part[blockIdx.x] = offd;
    if (!grid_sync(P.bar)) return;
    double mx = 0;
    for (int b = threadIdx.x; b < gridDim.x; b += JBT * 32) mx = fmax(mx, __ldcg(P.part + b));
    mx = block_max(mx, red);
    if (!grid_sync(P.bar)) return;
    if (mx <= P.stop) {
      ++sweep;
      break;
    }
  }
  // singular values = column norms, a warp per column
  const int64_t gw = (int64_t)blockIdx.x * JBT + wid, W = (int64_t)gridDim.x * JBT;
  for (int64_t j = gw; j < n; j += W) {
    const float* x = P.X + j * P.ldx;
    double acc = 0;
    for (int64_t i = lane; i < n; i += 32) {
      const double v = __ldcg(x + i);
      acc = fma(v, v, acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) P.S[j] = (float)sqrt(acc);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.sweeps_out = sweep;
}

// ---- FP32 one-sided Jacobi in one thread-block cluster ---------------------------
// Every column pair sits in the registers of one warp (X and V, RPL rows a
// lane), the whole n x n matrix across the CTAs of one cluster.  Each step
// rotates all nn/2 pairs at once; then the columns move one position along
// the round-robin tournament (slot 0 fixed, slot i <- slot i + 1, slot nn - 1
// <- slot 1), which pairs every two columns once in nn - 1 steps and brings
// every column back to its slot at the end of a sweep.  A column moves by the
// sender's stores into the receiver's shared-memory mailbox, double-buffered
// by step parity: within a CTA plain stores and a release arrival on the
// receiver's mbarrier, across CTAs stores into its distributed shared memory
// that count their bytes on that mbarrier (st.async); the receiver waits for
// the mbarrier's phase, with no barrier across the cluster per step.  Warp w owns slots w (top) and nn - 1 - w
// (bottom): its top moves to warp w - 1's top (warp 1's to warp 0's bottom,
// warp 0's stays), its bottom to warp w + 1's bottom (the last warp's to its
// own top).  The rotation of a pair is that of jacobi_block_kernel.
__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// shared::cluster address of the same shared-memory offset in CTA `rank`
__device__ __forceinline__ uint32_t dsmem_addr(const void* local, unsigned rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
               : "=r"(r)
               : "r"((uint32_t)__cvta_generic_to_shared(local)), "r"(rank));
  return r;
}
// 16 / 8 bytes into this CTA's shared memory
__device__ __forceinline__ void mbox_st4(uint32_t a, f2_t x, f2_t y) {
  asm volatile("st.shared.v2.b64 [%0], {%1, %2};" ::"r"(a), "l"(x), "l"(y) : "memory");
}
__device__ __forceinline__ void mbox_st2(uint32_t a, f2_t x) {
  asm volatile("st.shared.b64 [%0], %1;" ::"r"(a), "l"(x) : "memory");
}

// A column in a mailbox: rows lane + 32 t of lane `lane` as 16-byte chunks
// (t = 4q .. 4q + 3 at float offset 4 (32 q + lane)), and when RPL is not a
// multiple of 4 the last two at 4 32 (RPL / 4) + 2 lane.  In registers the
// rows come in pairs: pair p holds t = 2p (low half) and 2p + 1 (high).
template <int RPL>
__device__ __forceinline__ void mbox_send(uint32_t base, int lane, const f2_t (&c)[RPL / 2]) {
#pragma unroll
  for (int q = 0; q < RPL / 4; ++q) mbox_st4(base + (uint32_t)((q * 32 + lane) * 16), c[2 * q], c[2 * q + 1]);
  if constexpr (RPL % 4 == 2) mbox_st2(base + (uint32_t)((RPL / 4) * 512 + lane * 8), c[RPL / 2 - 1]);
}
template <int RPL>
__device__ __forceinline__ void mbox_recv(const float* box, int lane, f2_t (&c)[RPL / 2]) {
  const ulonglong2* b4 = reinterpret_cast<const ulonglong2*>(box);
#pragma unroll
  for (int q = 0; q < RPL / 4; ++q) {
    const ulonglong2 v = b4[q * 32 + lane];
    c[2 * q] = v.x;
    c[2 * q + 1] = v.y;
  }
  if constexpr (RPL % 4 == 2) c[RPL / 2 - 1] = reinterpret_cast<const f2_t*>(box + (RPL / 4) * 128)[lane];
}

// Point-to-point exchange: a remote store that counts its bytes on the
// receiver's mbarrier (st.async ... complete_tx), a release arrival for a
// sender in the receiver's own CTA, and the receiver's bounded wait.
__device__ __forceinline__ void st_async16(uint32_t a, f2_t x, f2_t y, uint32_t mbar) {
  asm volatile(
      "{\n\t.reg .b32 x0, x1, y0, y1;\n\tmov.b64 {x0, x1}, %1;\n\tmov.b64 {y0, y1}, %2;\n\t"
      "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {x0, x1, y0, y1}, [%3];\n}" ::"r"(a),
      "l"(x), "l"(y), "r"(mbar)
      : "memory");
}
__device__ __forceinline__ void st_async8(uint32_t a, f2_t x, uint32_t mbar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(a), "l"(x), "r"(mbar)
               : "memory");
}
template <int RPL>
__device__ __forceinline__ void mbox_send_async(uint32_t base, uint32_t mbar, int lane, const f2_t (&c)[RPL / 2]) {
#pragma unroll
  for (int q = 0; q < RPL / 4; ++q) st_async16(base + (uint32_t)((q * 32 + lane) * 16), c[2 * q], c[2 * q + 1], mbar);
  if constexpr (RPL % 4 == 2) st_async8(base + (uint32_t)((RPL / 4) * 512 + lane * 8), c[RPL / 2 - 1], mbar);
}
__device__ __forceinline__ void jc_mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((uint32_t)__cvta_generic_to_shared(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void jc_arrive_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void jc_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"((uint32_t)__cvta_generic_to_shared(bar))
               : "memory");
}
__device__ __forceinline__ bool jc_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, "
      "p;\n}\n"
      : "=r"(ok)
      : "r"((uint32_t)__cvta_generic_to_shared(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for a phase of `bar`, bounded: a wait that outlasts the limit, or an
// error word already set, sets / keeps the error and gives up.  Returns
// whether the data arrived; the whole warp agrees.
__device__ __forceinline__ bool jc_wait(uint64_t* bar, unsigned parity, int* err) {
  bool ok = true;
  if (*((volatile int*)err) != 0) {
    ok = false;
  } else {
    uint64_t t0 = 0;
    int spins = 0;
    while (!jc_try_wait(bar, parity)) {
      if (++spins < 64) continue;
      spins = 0;
      if (*((volatile int*)err) != 0) {
        ok = false;
        break;
      }
      const uint64_t t = globaltimer_ns();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > wait_limit_ns()) {
        atomicCAS(err, 0, 6);
        ok = false;
        break;
      }
    }
  }
  return __all_sync(0xffffffffu, ok);
}

template <int RPL>
__global__ void __launch_bounds__(512, 1) jacobi_cluster_kernel(JacParams<float> P, int nn) {
  static_assert(RPL % 2 == 0, "rows of a lane go in pairs");
  constexpr int NP = RPL / 2;
  extern __shared__ float4 jc_smem4[];
  float* mbox = reinterpret_cast<float*>(jc_smem4);
  __shared__ unsigned offv[3];  // the sweep's largest cosine (bits of a float >= 0), CTA 0's copy counts
  constexpr int COL = RPL * 32;  // floats of one column in a mailbox
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int NW = blockDim.x >> 5;
  const unsigned rank = cluster_rank();
  const int w = (int)rank * NW + wl;
  const int PW = nn / 2;
  const int n = (int)P.n;
  const float tol = (float)P.tol;
  // mailbox of local warp l, buffer b, slot s (0 top, 1 bottom), X (0) / V (1)
  auto box = [&](int b, int l, int sl, int xv) { return mbox + ((((size_t)b * NW + l) * 2 + sl) * 2 + xv) * COL; };
  f2_t xt[NP], xb[NP], vt[NP], vb[NP];
  {
    const int ct = w, cb = nn - 1 - w;
    auto ld = [&](const float* M, int64_t ldm, int col, int t) -> float {
      const int i = lane + 32 * t;
      return i < n && col < n ? M[i + (int64_t)col * ldm] : 0.0f;
    };
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      xt[p] = f2_pack(ld(P.X, P.ldx, ct, 2 * p), ld(P.X, P.ldx, ct, 2 * p + 1));
      vt[p] = f2_pack(ld(P.V, P.ldv, ct, 2 * p), ld(P.V, P.ldv, ct, 2 * p + 1));
      xb[p] = f2_pack(ld(P.X, P.ldx, cb, 2 * p), ld(P.X, P.ldx, cb, 2 * p + 1));
      vb[p] = f2_pack(ld(P.V, P.ldv, cb, 2 * p), ld(P.V, P.ldv, cb, 2 * p + 1));
    }
  }
  if (threadIdx.x < 3) offv[threadIdx.x] = 0u;
  // destinations of this warp's top and bottom columns
  int dt_w = -1, dt_s = 0;  // warp 0's top stays
  if (w >= 2) {
    dt_w = w - 1;
    dt_s = 0;
  } else if (w == 1) {
    dt_w = 0;
    dt_s = 1;
  }
  const int db_w = w <= PW - 2 ? w + 1 : w, db_s = w <= PW - 2 ? 1 : 0;
  const unsigned dt_r = dt_w >= 0 ? (unsigned)(dt_w / NW) : rank, db_r = (unsigned)(db_w / NW);
  const uint32_t off_remote = dsmem_addr(offv, 0);
  // Point-to-point: full[b][l] completes a phase when the columns of local
  // warp l for a step of parity b have arrived -- its own arrival with the
  // bytes the remote senders store (st.async counts them), plus one release
  // arrival from each sender in this CTA.  A sender never overwrites a
  // buffer before its receiver has read it: every receiver of a warp also
  // sends to it each step, so data of step s + 1 from the receiver means
  // step s was read before step s + 2 reuses the buffer.
  __shared__ __align__(8) uint64_t full[2][16];
  const int ts_w = w == 0 ? -1 : (w == PW - 1 ? w : w + 1);  // sender of this warp's top
  const int bs_w = w >= 1 ? w - 1 : 1;                       // of its bottom
  const bool ts_local = ts_w >= 0 && ts_w / NW == (int)rank, bs_local = bs_w / NW == (int)rank;
  const unsigned remote_bytes = (unsigned)(((ts_w >= 0 && !ts_local) ? 1 : 0) + (bs_local ? 0 : 1)) * 2u * 128u * RPL;
  if (lane == 0) {
    const unsigned cnt = 1u + (ts_local ? 1u : 0u) + (bs_local ? 1u : 0u);
    jc_mbar_init(&full[0][wl], cnt);
    jc_mbar_init(&full[1][wl], cnt);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  cluster_barrier();  // every CTA of the cluster runs (its barriers set up) before any remote store
  int sweep = 0;
  unsigned step_par = 0;
  bool alive = true;  // no wait has given up
  for (; sweep < P.max_sweeps; ++sweep) {
    if (rank == 0 && threadIdx.x == 0) offv[(sweep + 1) % 3] = 0u;
    float off = 0;
    for (int step = 0; step < nn - 1; ++step) {
      if (lane == 0) jc_arrive_tx(&full[step_par & 1u][wl], remote_bytes);
      f2_t a2 = 0, b2 = 0, g2 = 0;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        a2 = f2_fma(xt[p], xt[p], a2);
        b2 = f2_fma(xb[p], xb[p], b2);
        g2 = f2_fma(xt[p], xb[p], g2);
      }
      float a = warp_sum(f2_lo(a2) + f2_hi(a2));
      float b = warp_sum(f2_lo(b2) + f2_hi(b2));
      float g = warp_sum(f2_lo(g2) + f2_hi(g2));
      if (a != 0 && b != 0) {
        const float rel = fabsf(g) * rsqrtf(a * b);
        if (rel > tol) {
          off = fmaxf(off, rel);
          // the angle need not be correctly rounded: (c, s) is a rotation
          // to rounding whatever t is
          const float zeta = __fdividef(b - a, 2.0f * g);
          const float tn = copysignf(__fdividef(1.0f, fabsf(zeta) + sqrtf(fmaf(zeta, zeta, 1.0f))), zeta);
          const float c = rsqrtf(fmaf(tn, tn, 1.0f));
          const float sn = c * tn;
          const f2_t cc = f2_pack(c, c), ss = f2_pack(sn, sn), ns = f2_pack(-sn, -sn);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            const f2_t u = xt[p], v = xb[p];
            xt[p] = f2_fma(ns, v, f2_mul(cc, u));
            xb[p] = f2_fma(cc, v, f2_mul(ss, u));
            const f2_t pu = vt[p], pv = vb[p];
            vt[p] = f2_fma(ns, pv, f2_mul(cc, pu));
            vb[p] = f2_fma(cc, pv, f2_mul(ss, pu));
          }
        }
      }
      if (step == nn - 2 && lane == 0) {
        const uint32_t oa = off_remote + (uint32_t)((sweep % 3) * sizeof(unsigned));
        asm volatile("red.shared::cluster.max.u32 [%0], %1;" ::"r"(oa), "r"(__float_as_uint(off)) : "memory");
      }
      const int buf = (int)(step_par & 1u);
      // a local receiver's arrival releases the whole warp's stores
      if (alive && dt_w >= 0) {
        if (dt_r == rank) {
          mbox_send<RPL>((uint32_t)__cvta_generic_to_shared(box(buf, dt_w % NW, dt_s, 0)), lane, xt);
          mbox_send<RPL>((uint32_t)__cvta_generic_to_shared(box(buf, dt_w % NW, dt_s, 1)), lane, vt);
          __syncwarp();
          if (lane == 0) jc_arrive(&full[buf][dt_w % NW]);
        } else {
          const uint32_t mb = dsmem_addr(&full[buf][dt_w % NW], dt_r);
          mbox_send_async<RPL>(dsmem_addr(box(buf, dt_w % NW, dt_s, 0), dt_r), mb, lane, xt);
          mbox_send_async<RPL>(dsmem_addr(box(buf, dt_w % NW, dt_s, 1), dt_r), mb, lane, vt);
        }
      }
      if (alive) {
        if (db_r == rank) {
          mbox_send<RPL>((uint32_t)__cvta_generic_to_shared(box(buf, db_w % NW, db_s, 0)), lane, xb);
          mbox_send<RPL>((uint32_t)__cvta_generic_to_shared(box(buf, db_w % NW, db_s, 1)), lane, vb);
          __syncwarp();
          if (lane == 0) jc_arrive(&full[buf][db_w % NW]);
        } else {
          const uint32_t mb = dsmem_addr(&full[buf][db_w % NW], db_r);
          mbox_send_async<RPL>(dsmem_addr(box(buf, db_w % NW, db_s, 0), db_r), mb, lane, xb);
          mbox_send_async<RPL>(dsmem_addr(box(buf, db_w % NW, db_s, 1), db_r), mb, lane, vb);
        }
      }
      if (alive) alive = jc_wait(&full[buf][wl], (step_par >> 1) & 1u, &P.bar->err);
      if (w != 0) {
        mbox_recv<RPL>(box(buf, wl, 0, 0), lane, xt);
        mbox_recv<RPL>(box(buf, wl, 0, 1), lane, vt);
      }
      mbox_recv<RPL>(box(buf, wl, 1, 0), lane, xb);
      mbox_recv<RPL>(box(buf, wl, 1, 1), lane, vb);
      ++step_par;
    }
    // a cluster barrier a sweep orders every warp's maximum; a wait that
    // gave up anywhere ends the sweeps everywhere at the same point
    cluster_barrier();
    unsigned mb;
    asm volatile("ld.shared::cluster.u32 %0, [%1];"
                 : "=r"(mb)
                 : "r"(off_remote + (uint32_t)((sweep % 3) * sizeof(unsigned)))
                 : "memory");
    const bool failed = *((volatile int*)&P.bar->err) != 0;
    if ((double)__uint_as_float(mb) <= P.stop || failed) {
      ++sweep;
      break;
    }
  }
  // every column is back in its slot: slot c holds column c
  {
    const int ct = w, cb = nn - 1 - w;
    double st = 0, sb = 0;
#pragma unroll
    for (int t = 0; t < RPL; ++t) {
      const int i = lane + 32 * t;
      const float x0 = t & 1 ? f2_hi(xt[t / 2]) : f2_lo(xt[t / 2]);
      const float x1 = t & 1 ? f2_hi(xb[t / 2]) : f2_lo(xb[t / 2]);
      if (i < n) {
        if (ct < n) {
          P.X[i + (int64_t)ct * P.ldx] = x0;
          P.V[i + (int64_t)ct * P.ldv] = t & 1 ? f2_hi(vt[t / 2]) : f2_lo(vt[t / 2]);
        }
        if (cb < n) {
          P.X[i + (int64_t)cb * P.ldx] = x1;
          P.V[i + (int64_t)cb * P.ldv] = t & 1 ? f2_hi(vb[t / 2]) : f2_lo(vb[t / 2]);
        }
      }
      st = fma((double)x0, (double)x0, st);
      sb = fma((double)x1, (double)x1, sb);
    }
    st = warp_sum(st);
    sb = warp_sum(sb);
    if (lane == 0) {
      if (ct < n) P.S[ct] = (float)sqrt(st);
      if (cb < n) P.S[cb] = (float)sqrt(sb);
    }
  }
  if (rank == 0 && threadIdx.x == 0) *P.sweeps_out = sweep;
  cluster_barrier();  // no CTA leaves while another may still read its shared memory
}

// Double-float block Jacobi: the polish sweeps of the mixed-precision path,
// the same block-pair schedule as jacobi_block_kernel with X and V held as
// float pairs (df64.cuh) and every dot, rotation and update done in
// double-float arithmetic on the FP32 pipes.  Columns are kept orthogonal
// to about 1e-13, ample for the tolerances the mixed path accepts.
struct JacDf {
  int64_t n;
  float* Xh;
  float* Xl;
  float* Vh;
  float* Vl;  // all with leading dimension n
  double* S;
  double tol, stop;
  int max_sweeps;
  double* part;
  GridBar* bar;
  int* sweeps_out;
};

__device__ __forceinline__ bool df_gt(Df x, Df y) { return x.h > y.h || (x.h == y.h && x.l > y.l); }

__device__ __forceinline__ Df df_rot_a(Df c, Df s, Df u, Df w) { return df_add(df_mul(c, u), df_neg(df_mul(s, w))); }
__device__ __forceinline__ Df df_rot_b(Df c, Df s, Df u, Df w) { return df_add(df_mul(s, u), df_mul(c, w)); }

template <int JBT>
__global__ void __launch_bounds__(JBT * 32) jacobi_block_df_kernel(JacDf P) {
  extern __shared__ float jd_smem[];
  __shared__ int s_any;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ni = (int)P.n;
  const size_t plane = (size_t)2 * JBT * ni;
  float* Xh = jd_smem;
  float* Xl = Xh + plane;
  float* Vh = Xl + plane;
  float* Vl = Vh + plane;
  const int nblk = (ni + JBT - 1) / JBT;
  const int nbb = nblk + (nblk & 1);
  const float ftol = (float)P.tol, fstop = (float)P.stop;
  int sweep = 0;
  for (; sweep < P.max_sweeps; ++sweep) {
    int above = 0;
    for (int r = 0; r < nbb - 1; ++r) {
      for (int s = blockIdx.x; s < nbb / 2; s += gridDim.x) {
        auto bpos = [&](int i) { return i == 0 ? 0 : 1 + (i - 1 + r) % (nbb - 1); };
        const int b1 = bpos(s), b2 = bpos(nbb - 1 - s);
        auto gcol = [&](int k) -> int {
          const int b = k < JBT ? b1 : b2;
          if (b >= nblk) return -1;
          const int j = b * JBT + (k % JBT);
          return j < ni ? j : -1;
        };
        for (int k = 0; k < 2 * JBT; ++k) {
          const int j = gcol(k);
          for (int i = threadIdx.x; i < ni; i += JBT * 32) {
            const size_t o = (size_t)k * ni + i;
            if (j >= 0) {
              const size_t g = (size_t)j * ni + i;
              cp_async4(Xh + o, P.Xh + g);
              cp_async4(Xl + o, P.Xl + g);
              cp_async4(Vh + o, P.Vh + g);
              cp_async4(Vl + o, P.Vl + g);
            } else {
              Xh[o] = Xl[o] = Vh[o] = Vl[o] = 0.0f;
            }
          }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncthreads();
        unsigned vmask = 0;
#pragma unroll
        for (int k = 0; k < 2 * JBT; ++k) vmask |= (gcol(k) >= 0 ? 1u : 0u) << k;
        for (int lr = 0; lr < 2 * JBT - 1; ++lr) {
          auto lpos = [&](int i) { return i == 0 ? 0 : 1 + (i - 1 + lr) % (2 * JBT - 1); };
          int p = lpos(wid), q = lpos(2 * JBT - 1 - wid);
          if (p > q) {
            const int t = p;
            p = q;
            q = t;
          }
          if (((vmask >> p) & 1u) && ((vmask >> q) & 1u)) {
            float* xph = Xh + p * ni;
            float* xpl = Xl + p * ni;
            float* xqh = Xh + q * ni;
            float* xql = Xl + q * ni;
            Df u[JB_RPL], w[JB_RPL];
            Df a{0.f, 0.f}, b{0.f, 0.f}, g{0.f, 0.f};
#pragma unroll
            for (int t = 0; t < JB_RPL; ++t) {
              const int i = lane + 32 * t;
              u[t] = i < ni ? Df{xph[i], xpl[i]} : Df{0.f, 0.f};
              w[t] = i < ni ? Df{xqh[i], xql[i]} : Df{0.f, 0.f};
            }
#pragma unroll
            for (int t = 0; t < JB_RPL; ++t) {
              df_fma_acc(a, u[t].h, u[t].l, u[t].h, u[t].l);
              df_fma_acc(b, w[t].h, w[t].l, w[t].h, w[t].l);
              df_fma_acc(g, u[t].h, u[t].l, w[t].h, w[t].l);
            }
            a = quick_two_sum(a.h, a.l);
            b = quick_two_sum(b.h, b.l);
            g = quick_two_sum(g.h, g.l);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
              a = df_add(a, df_shfl_xor(a, o));
              b = df_add(b, df_shfl_xor(b, o));
              g = df_add(g, df_shfl_xor(g, o));
            }
            if (a.h > 0.f && b.h > 0.f) {
              const float rel = fabsf(g.h) * rsqrtf(a.h) * rsqrtf(b.h);
              if (rel > ftol) {
                if (rel > fstop) above = 1;
                // tan of the rotation angle from zeta = (b - a) / (2 g) in
                // double-float; t itself in FP32: a rotation by an angle off
                // by 1e-7 relative still shrinks g by 1e-7, and the rotation
                // matrix below is orthogonal to double-float precision
                const Df zeta = df_div(df_add(b, df_neg(a)), df_mul(Df{2.f, 0.f}, g));
                const float z = zeta.h;
                const float t = copysignf(1.0f, z) / (fabsf(z) + sqrtf(fmaf(z, z, 1.0f)));
                float* vph = Vh + p * ni;
                float* vpl = Vl + p * ni;
                float* vqh = Vh + q * ni;
                float* vql = Vl + q * ni;
                if (fabsf(t) < 9.5367431640625e-07f) {
                  // small angle: x' = x + delta, delta = -eps x -/+ s y in FP32
                  // (c = 1 - eps, eps = t^2 / (r (1 + r)), r = sqrt(1 + t^2))
                  const float r = sqrtf(fmaf(t, t, 1.0f));
                  const float eps = t * t / (r * (1.0f + r));
                  const float sn = t / r;
                  auto bump = [&](Df x, float d) {
                    float hs, e;
                    two_sum(x.h, d, hs, e);
                    return quick_two_sum(hs, x.l + e);
                  };
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    if (i < ni) {
                      const Df x1 = bump(u[tt], fmaf(-sn, w[tt].l, fmaf(-sn, w[tt].h, -eps * u[tt].h)));
                      const Df x2 = bump(w[tt], fmaf(sn, u[tt].l, fmaf(sn, u[tt].h, -eps * w[tt].h)));
                      xph[i] = x1.h;
                      xpl[i] = x1.l;
                      xqh[i] = x2.h;
                      xql[i] = x2.l;
                    }
                  }
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    u[tt] = i < ni ? Df{vph[i], vpl[i]} : Df{0.f, 0.f};
                    w[tt] = i < ni ? Df{vqh[i], vql[i]} : Df{0.f, 0.f};
                  }
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    if (i < ni) {
                      const Df v1 = bump(u[tt], fmaf(-sn, w[tt].l, fmaf(-sn, w[tt].h, -eps * u[tt].h)));
                      const Df v2 = bump(w[tt], fmaf(sn, u[tt].l, fmaf(sn, u[tt].h, -eps * w[tt].h)));
                      vph[i] = v1.h;
                      vpl[i] = v1.l;
                      vqh[i] = v2.h;
                      vql[i] = v2.l;
                    }
                  }
                } else {
                  const Df td{t, 0.f};
                  const Df c = df_div(Df{1.f, 0.f}, df_sqrt(df_add(Df{1.f, 0.f}, df_mul(td, td))));
                  const Df sn = df_mul(c, td);
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    if (i < ni) {
                      const Df x1 = df_rot_a(c, sn, u[tt], w[tt]), x2 = df_rot_b(c, sn, u[tt], w[tt]);
                      xph[i] = x1.h;
                      xpl[i] = x1.l;
                      xqh[i] = x2.h;
                      xql[i] = x2.l;
                    }
                  }
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    u[tt] = i < ni ? Df{vph[i], vpl[i]} : Df{0.f, 0.f};
                    w[tt] = i < ni ? Df{vqh[i], vql[i]} : Df{0.f, 0.f};
                  }
#pragma unroll
                  for (int tt = 0; tt < JB_RPL; ++tt) {
                    const int i = lane + 32 * tt;
                    if (i < ni) {
                      const Df v1 = df_rot_a(c, sn, u[tt], w[tt]), v2 = df_rot_b(c, sn, u[tt], w[tt]);
                      vph[i] = v1.h;
                      vpl[i] = v1.l;
                      vqh[i] = v2.h;
                      vql[i] = v2.l;
                    }
                  }
                }
              }
            }
          }
          __syncthreads();
        }
        for (int k = 0; k < 2 * JBT; ++k) {
          const int j = gcol(k);
          if (j < 0) continue;
          for (int i = threadIdx.x; i < ni; i += JBT * 32) {
            const size_t o = (size_t)k * ni + i, g = (size_t)j * ni + i;
            P.Xh[g] = Xh[o];
            P.Xl[g] = Xl[o];
            P.Vh[g] = Vh[o];
            P.Vl[g] = Vl[o];
          }
        }
        __syncthreads();
      }
      if (!grid_sync(P.bar)) return;
    }
    // any rotation above the stopping level, over the grid
    above = __syncthreads_or(above);
    if (threadIdx.x == 0) P.part[blockIdx.x] = above ? 1.0 : 0.0;
    if (!grid_sync(P.bar)) return;
    if (threadIdx.x == 0) {
      int any = 0;
      for (int k = 0; k < (int)gridDim.x; ++k) any |= __ldcg(P.part + k) != 0.0;
      s_any = any;
    }
    __syncthreads();
    const int any = s_any;
    if (!grid_sync(P.bar)) return;
    if (!any) {
      ++sweep;
      break;
    }
  }
  // singular values = column norms, a warp per column
  const int gw = blockIdx.x * JBT + wid, W = gridDim.x * JBT;
  for (int j = gw; j < ni; j += W) {
    Df acc{0.f, 0.f};
    for (int i = lane; i < ni; i += 32) {
      const float h = __ldcg(P.Xh + (size_t)j * ni + i), l = __ldcg(P.Xl + (size_t)j * ni + i);
      df_fma_acc(acc, h, l, h, l);
    }
    acc = quick_two_sum(acc.h, acc.l);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = df_add(acc, df_shfl_xor(acc, o));
    if (lane == 0) P.S[j] = sqrt(df_val(acc.h, acc.l));
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.sweeps_out = sweep;
}

__global__ void df_from_double_kernel(int64_t m, int64_t n, const double* __restrict__ A, int64_t lda,
                                      float* __restrict__ H, float* __restrict__ L, int identity) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    const double x = identity ? (i == j ? 1.0 : 0.0) : A[i + j * lda];
    const Df d = df_split(x);
    H[t] = d.h;
    L[t] = d.l;
  }
}

__global__ void df_to_double_kernel(int64_t m, int64_t n, const float* __restrict__ H, const float* __restrict__ L,
                                    double* __restrict__ A, int64_t lda) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    A[i + j * lda] = df_val(H[t], L[t]);
  }
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

// LRA_JACOBI_CLUSTER=0 keeps the FP32 sweeps on the block-pair kernel even
// where the matrix fits one cluster (both variants stay testable)
static bool jacobi_cluster_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LRA_JACOBI_CLUSTER");
    return !(e && *e == '0');
  }();
  return on;
}

// The FP32 sweeps in one cluster (jacobi_cluster_kernel) when the columns fit
// the registers of its warps: false when they do not (or no cluster of the
// size needed can be scheduled), the caller then takes the block-pair kernel.
static bool jacobi_cluster(lra_ctx* ctx, JacParams<float>& P) {
  const int64_t n = P.n;
  if (!jacobi_cluster_enabled() || n < 64 || n > 32 * 14) return false;
  const int rpl = n <= 128 ? 4 : n <= 256 ? 8 : 14;
  const void* kern = rpl == 4   ? (const void*)jacobi_cluster_kernel<4>
                     : rpl == 8 ? (const void*)jacobi_cluster_kernel<8>
                                : (const void*)jacobi_cluster_kernel<14>;
  int optin = 0;
  LRA_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
  const size_t per_warp = (size_t)1024 * rpl;  // two buffers x two slots x (X, V) x 32 rpl floats
  const int nw_max = (int)std::min<size_t>(16, ((size_t)optin - 1024) / per_warp);  // static smem below 1 KB
  const int64_t need = (n + 1) / 2;  // column pairs
  raise_smem_limit(ctx, kern);
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> portable_set;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!portable_set.count({kern, ctx->device})) {
      LRA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      portable_set.insert({kern, ctx->device});
    }
  }
  if (ctx->tuning.jacobi_cluster == 1) return false;
  const int c_max = ctx->tuning.jacobi_cluster > 1 ? ctx->tuning.jacobi_cluster : 16;
  for (int c = c_max; c >= 2; --c) {
    const int64_t nw = (need + c - 1) / c;
    if (nw > nw_max || nw < 1) break;  // fewer CTAs only need more warps each
    const int pw = (int)(c * nw);
    if (pw < 2) continue;
    const size_t smem = per_warp * (size_t)nw;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)c);
    cfg.blockDim = dim3((unsigned)(nw * 32));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (clusters < 1) continue;
    int nn = 2 * pw;
    void* args[] = {&P, &nn};
    LRA_CUDA(cudaLaunchKernelExC(&cfg, kern, args));
    post_launch(ctx, "jacobi_cluster_kernel");
    if (trace_on()) std::fprintf(stderr, "[lra] jacobi f32 cluster n=%lld ctas=%d warps=%lld slots=%d\n", (long long)n,
                                 c, (long long)nw, nn);
    return true;
  }
  return false;
}

template <typename T>
void jacobi_svd(lra_ctx* ctx, int64_t n, T* X, int64_t ldx, T* V, int64_t ldv, T* S, bool quadratic_stop,
                double stop) {
  // Float64: a CTA of 128 threads per pair; Float32: block Jacobi with the
  // block pair in shared memory when it fits, else a warp per pair
  constexpr bool pair_cta = sizeof(T) == 8;
  constexpr int NT = 128;
  if (n <= 0) return;
  set_identity(ctx, n, n, V, ldv);
  const ArenaMark mk = ctx->arena.mark();
  // FP32: 8-column blocks (16-column blocks halve the grid barriers but
  // measured slower: the local sweeps become issue-bound on half the SMs);
  // 4-column blocks for the longer columns whose 8-column block pair does
  // not fit shared memory (up to about 3500 rows); a warp per pair beyond
  const size_t blk_cap = 210 * 1024;
  // 8-column blocks with the block pair of X and V in shared memory; for
  // longer columns V stays in global memory (read and written once per block
  // pair), up to about 3400 rows; beyond, a warp per pair
  int jbt = 8;
  const int64_t nld = (n + 3) & ~(int64_t)3;  // the kernel's padded column stride
  bool vglobal = (size_t)4 * jbt * nld * sizeof(float) > blk_cap;
  // the tuning table may ask for another block size (when it fits)
  const int want = ctx->tuning.jacobi_jb;
  if ((want == 4 || want == 8 || want == 16 || want == 32) && (size_t)2 * want * nld * sizeof(float) <= blk_cap) {
    jbt = want;
    vglobal = (size_t)4 * jbt * nld * sizeof(float) > blk_cap;
  }
  const size_t blk_smem = (size_t)(vglobal ? 2 : 4) * jbt * nld * sizeof(float);
  const bool block = !pair_cta && n >= 4 * jbt && blk_smem <= blk_cap;
  const void* kern = pair_cta ? (const void*)jacobi_pair_kernel<T, NT>
                     : !block ? (const void*)jacobi_kernel<T, NT>
                     : jbt == 32 ? (const void*)jacobi_block_kernel<32>
                     : jbt == 16 ? (const void*)jacobi_block_kernel<16>
                     : jbt == 8 ? (const void*)jacobi_block_kernel<8>
                                : (const void*)jacobi_block_kernel<4>;
  const int nt = block ? jbt * 32 : NT;
  const size_t smem = block ? blk_smem : 0;
  if (block) raise_smem_limit(ctx, (const void*)kern);
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem));
  const int64_t pairs = (n + 1) / 2;
  int64_t units = pair_cta ? pairs : (pairs + NT / 32 - 1) / (NT / 32);
  if (block) {
    const int64_t nblk = (n + jbt - 1) / jbt;
    units = (nblk + 1) / 2;
  }
  // the FP64 pairs all at once (up to two CTAs per SM), the rest one CTA per SM
  int grid = (int)std::min<int64_t>(units, (int64_t)ctx->num_sms * (pair_cta ? 2 : 1));
  grid = std::max(1, std::min(grid, ctx->num_sms * std::max(per_sm, 1)));
  JacParams<T> P;
  P.n = n;
  P.X = X;
  P.ldx = ldx;
  P.V = V;
  P.ldv = ldv;
  P.S = S;
  P.vglobal = block && vglobal ? 1 : 0;
  P.tol = (double)Real<T>::eps * 2.0 * std::sqrt((double)n);
  // A sweep whose cosines were all below sqrt(tol)/10 leaves them near
  // tol^2/100 times a modest gap factor (quadratic convergence), so the
  // sweep that would only confirm it is skipped.
  P.stop = stop > 0 ? stop : (quadratic_stop ? std::sqrt(P.tol) * 0.1 : P.tol);
  P.max_sweeps = 40;
  P.part = ctx->arena.alloc_n<double>(grid);
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.sweeps_out = ctx->arena.alloc_n<int>(1);
  if (trace_on() && block) {
    P.phase_ns = ctx->arena.alloc_n<unsigned long long>(5);
    LRA_CUDA(cudaMemsetAsync(P.phase_ns, 0, 5 * sizeof(unsigned long long), ctx->stream));
  }
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  if constexpr (sizeof(T) == 4) {
    if (jacobi_cluster(ctx, P)) {
      int sweeps = 0;
      GridBar hb;
      LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
      if (trace_on())
        LRA_CUDA(cudaMemcpyAsync(&sweeps, P.sweeps_out, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      ctx->arena.release(mk);
      if (hb.err != 0) fail(LRA_ETIMEDOUT, "jacobi: a column exchange between the cluster's CTAs timed out");
      if (trace_on()) std::fprintf(stderr, "[lra] jacobi f32 cluster n=%lld sweeps=%d\n", (long long)n, sweeps);
      return;
    }
  }
  void* args[] = {&P};
  LRA_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(nt), args, smem, ctx->stream));
  post_launch(ctx, pair_cta ? "jacobi_pair_kernel" : (block ? "jacobi_block_kernel" : "jacobi_kernel"));
  GridBar hb;
  int sweeps = 0;
  unsigned long long ph[5] = {0, 0, 0, 0, 0};
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  if (trace_on())
    LRA_CUDA(cudaMemcpyAsync(&sweeps, P.sweeps_out, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (P.phase_ns) LRA_CUDA(cudaMemcpyAsync(ph, P.phase_ns, sizeof(ph), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "jacobi: a grid barrier timed out");
  if (P.phase_ns)
    std::fprintf(stderr, "[lra] jacobi block CTA 0 ms: load %.2f local %.2f V %.2f write %.2f barrier %.2f\n",
                 ph[0] * 1e-6, ph[1] * 1e-6, ph[2] * 1e-6, ph[3] * 1e-6, ph[4] * 1e-6);
  if (trace_on())
    std::fprintf(stderr, "[lra] jacobi %s%s n=%lld sweeps=%d grid=%d\n", sizeof(T) == 8 ? "f64" : "f32",
                 block ? " block" : "", (long long)n, sweeps, grid);
}

bool jacobi_svd_df(lra_ctx* ctx, int64_t n, double* X, int64_t ldx, double* V, int64_t ldv, double* S) {
  // 4-column blocks: the double-float rotations are issue-bound, so the work
  // is spread over as many SMs as the block pairs allow
  constexpr int JDF = 4;
  if (n < 2 || n > 32 * JB_RPL) return false;
  const size_t smem = (size_t)8 * JDF * n * sizeof(float);
  if (smem > 200 * 1024) return false;
  raise_smem_limit(ctx, (const void*)jacobi_block_df_kernel<JDF>);
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, jacobi_block_df_kernel<JDF>, JDF * 32, smem));
  if (per_sm < 1) return false;
  const ArenaMark mk = ctx->arena.mark();
  const int64_t nblk = (n + JDF - 1) / JDF;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nblk + 1) / 2, (int64_t)ctx->num_sms * per_sm));
  JacDf P;
  P.n = n;
  P.Xh = ctx->arena.alloc_n<float>((size_t)n * n);
  P.Xl = ctx->arena.alloc_n<float>((size_t)n * n);
  P.Vh = ctx->arena.alloc_n<float>((size_t)n * n);
  P.Vl = ctx->arena.alloc_n<float>((size_t)n * n);
  P.S = S;
  // double-float resolves cosines down to a few units of 2^-46 sqrt(n)
  P.tol = std::max((double)Real<double>::eps * 2.0 * std::sqrt((double)n), 8.0 * std::ldexp(1.0, -46) * std::sqrt((double)n));
  P.stop = std::sqrt(P.tol) * 0.1;  // quadratic convergence from the FP32 sweeps
  P.max_sweeps = 40;
  P.part = ctx->arena.alloc_n<double>(grid);
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.sweeps_out = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n * n + 255) / 256, ctx->num_sms * 8));
  df_from_double_kernel<<<g, 256, 0, ctx->stream>>>(n, n, X, ldx, P.Xh, P.Xl, 0);
  post_launch(ctx, "df_from_double_kernel");
  df_from_double_kernel<<<g, 256, 0, ctx->stream>>>(n, n, nullptr, n, P.Vh, P.Vl, 1);
  post_launch(ctx, "df_from_double_kernel");
  void* args[] = {&P};
  LRA_CUDA(cudaLaunchCooperativeKernel((const void*)jacobi_block_df_kernel<JDF>, dim3(grid), dim3(JDF * 32), args, smem,
                                       ctx->stream));
  post_launch(ctx, "jacobi_block_df_kernel<JDF>");
  df_to_double_kernel<<<g, 256, 0, ctx->stream>>>(n, n, P.Xh, P.Xl, X, ldx);
  post_launch(ctx, "df_to_double_kernel");
  df_to_double_kernel<<<g, 256, 0, ctx->stream>>>(n, n, P.Vh, P.Vl, V, ldv);
  post_launch(ctx, "df_to_double_kernel");
  GridBar hb;
  int sweeps = 0;
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  if (trace_on())
    LRA_CUDA(cudaMemcpyAsync(&sweeps, P.sweeps_out, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "jacobi: a grid barrier timed out");
  if (trace_on())
    std::fprintf(stderr, "[lra] jacobi df block n=%lld sweeps=%d grid=%d\n", (long long)n, sweeps, grid);
  return true;
}

template <typename T>
bool is_symmetric(lra_ctx* ctx, int64_t n, const T* A, int64_t lda) {
  if (ctx->linop) return ctx->linop->hermitian != 0;  // a HermitianLinearOperator is, by its type
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

template void jacobi_svd<float>(lra_ctx*, int64_t, float*, int64_t, float*, int64_t, float*, bool, double);
template void jacobi_svd<double>(lra_ctx*, int64_t, double*, int64_t, double*, int64_t, double*, bool, double);
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
// Right-looking Cholesky of one jb x jb diagonal block in shared memory, as
// LAPACK xPOTF2 orders it: R(c, c) = sqrt(.), row c scaled by 1 / R(c, c),
// then the trailing block updated in parallel.
template <typename T>
__global__ void potrf_diag_kernel(int jb, T* G, int64_t ldg, int* bad) {
  __shared__ T a[CB][CB + 1];
  __shared__ T s_inv;
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    a[i][j] = G[i + j * ldg];
  }
  __syncthreads();
  for (int c = 0; c < jb; ++c) {
    if (threadIdx.x == 0) {
      T d = a[c][c];
      if (!(d > T(0))) {
        atomicExch(bad, 1);
        d = T(1);
      }
      const T r = sqrt(d);
      a[c][c] = r;
      s_inv = T(1) / r;
    }
    __syncthreads();
    const T inv = s_inv;
    for (int j = c + 1 + threadIdx.x; j < jb; j += blockDim.x) a[c][j] *= inv;
    __syncthreads();
    // a[i][j] -= a[c][i] a[c][j] for c < i <= j < jb
    const int w = jb - c - 1;
    for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
      const int i = c + 1 + t % w, j = c + 1 + t / w;
      if (i <= j) a[i][j] -= a[c][i] * a[c][j];
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    G[i + j * ldg] = i <= j ? a[i][j] : T(0);
  }
}

// The whole blocked right-looking Cholesky in one cooperative launch, of
// one matrix or two independent ones at once (their sequential diagonal
// blocks then overlap): for each 32-wide diagonal block, CTA m factors
// matrix m's block in shared memory (as potrf_diag_kernel), the grid solves
// the block rows with a warp per column (lane i holds x_i; the columns of
// both matrices dealt out over every warp, since the FP64 pipe of one SM
// retires only a few FMAs a clock) and updates the upper trailing
// triangles, with a bounded grid barrier between the phases.
template <typename T>
struct PotrfJobs {
  int n;           // 1 or 2
  int64_t k[2];
  T* G[2];
  int64_t ldg[2];
  int* bad;        // one flag per matrix
};

template <typename T>
__global__ void __launch_bounds__(256) potrf_coop_kernel(PotrfJobs<T> J, GridBar* bar) {
  __shared__ T a[2][CB][CB + 1];
  __shared__ T rinv[2][CB];
  __shared__ T s_inv;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t GT = (int64_t)gridDim.x * blockDim.x;
  const int64_t kmax = J.n > 1 ? max(J.k[0], J.k[1]) : J.k[0];
  for (int64_t j0 = 0; j0 < kmax; j0 += CB) {
    // ---- 1. the diagonal blocks, CTA m for matrix m ----
    for (int m = 0; m < J.n; ++m) {
      if ((int)blockIdx.x != m % (int)gridDim.x || j0 >= J.k[m]) continue;
      const int jb = (int)min((int64_t)CB, J.k[m] - j0);
      const int64_t ldg = J.ldg[m];
      T* Gjj = J.G[m] + j0 + j0 * ldg;
      // every read of G goes around L1: other CTAs wrote it in earlier phases
      for (int t = threadIdx.x; t < jb * jb; t += blockDim.x)
        a[m][t % jb][t / jb] = __ldcg(Gjj + t % jb + (t / jb) * ldg);
      __syncthreads();
      for (int c = 0; c < jb; ++c) {
        if (threadIdx.x == 0) {
          T d = a[m][c][c];
          if (!(d > T(0))) {
            atomicExch(J.bad + m, 1);
            d = T(1);
          }
          const T r = sqrt(d);
          a[m][c][c] = r;
          s_inv = T(1) / r;
        }
        __syncthreads();
        const T inv = s_inv;
        for (int j = c + 1 + threadIdx.x; j < jb; j += blockDim.x) a[m][c][j] *= inv;
        __syncthreads();
        const int w = jb - c - 1;
        for (int t = threadIdx.x; t < w * w; t += blockDim.x) {
          const int i = c + 1 + t % w, j = c + 1 + t / w;
          if (i <= j) a[m][i][j] -= a[m][c][i] * a[m][c][j];
        }
        __syncthreads();
      }
      for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
        const int i = t % jb, j = t / jb;
        if (i <= j) Gjj[i + j * ldg] = a[m][i][j];
      }
    }
    if (!grid_sync(bar)) return;
    int64_t rest[2] = {0, 0};
    int jbm[2] = {0, 0};
    for (int m = 0; m < J.n; ++m) {
      if (j0 >= J.k[m]) continue;
      jbm[m] = (int)min((int64_t)CB, J.k[m] - j0);
      rest[m] = J.k[m] - j0 - jbm[m];
    }
    if (rest[0] + rest[1] <= 0) break;
    // ---- 2. the block rows: R_{b,>b} = R_bb^{-T} G_{b,>b}, a warp per column ----
    for (int m = 0; m < J.n; ++m) {
      if (rest[m] <= 0) continue;
      const int jb = jbm[m];
      const T* Gjj = J.G[m] + j0 + j0 * J.ldg[m];
      for (int t = threadIdx.x; t < jb * jb; t += blockDim.x)
        a[m][t % jb][t / jb] = __ldcg(Gjj + t % jb + (t / jb) * J.ldg[m]);
    }
    __syncthreads();
    for (int m = 0; m < J.n; ++m)
      if (rest[m] > 0 && threadIdx.x < jbm[m]) rinv[m][threadIdx.x] = T(1) / a[m][threadIdx.x][threadIdx.x];
    __syncthreads();
    {
      const int lane = threadIdx.x & 31;
      const int64_t gw = (int64_t)(threadIdx.x >> 5) * gridDim.x + blockIdx.x;
      const int64_t GW = (int64_t)gridDim.x * (blockDim.x >> 5);
      for (int64_t cc = gw; cc < rest[0] + rest[1]; cc += GW) {
        const int m = cc < rest[0] ? 0 : 1;
        const int64_t col = m == 0 ? cc : cc - rest[0];
        const int jb = jbm[m];
        T* p = J.G[m] + j0 + (j0 + jb + col) * J.ldg[m];
        T x = lane < jb ? __ldcg(p + lane) : T(0);
        // x_i = (g_i - sum_{q<i} R_qi x_q) / R_ii, the sums accumulated lane-wise
        for (int i = 0; i < jb; ++i) {
          const T xi = __shfl_sync(0xffffffffu, x, i) * rinv[m][i];
          if (lane == i) x = xi;
          if (lane > i && lane < jb) x -= a[m][i][lane] * xi;
        }
        if (lane < jb) p[lane] = x;
      }
    }
    if (!grid_sync(bar)) return;
    // ---- 3. trailing upper triangles: G(i, j) -= sum_q R(q, i) R(q, j), j0+jb <= i <= j ----
    const int64_t n0 = rest[0] * rest[0];
    for (int64_t t = gt; t < n0 + rest[1] * rest[1]; t += GT) {
      const int m = t < n0 ? 0 : 1;
      const int64_t tt = m == 0 ? t : t - n0, r = rest[m];
      const int64_t i = tt % r, j = tt / r;
      if (i > j) continue;
      const int jb = jbm[m];
      const int64_t ldg = J.ldg[m], o = j0 + jb;
      T* G = J.G[m];
      const T* ri = G + j0 + (o + i) * ldg;
      const T* rj = G + j0 + (o + j) * ldg;
      T s = 0;
#pragma unroll 8
      for (int q = 0; q < jb; ++q) s = fma(__ldcg(ri + q), __ldcg(rj + q), s);
      T* gij = G + (o + i) + (o + j) * ldg;
      *gij = __ldcg(gij) - s;
    }
    if (!grid_sync(bar)) return;
  }
}

// panel: R_{b, >b} = R_bb^{-T} G_{b, >b} (jb x nc), one thread per column
template <typename T>
__global__ void potrf_panel_kernel(int jb, int64_t nc, const T* Rbb, int64_t ldr, T* P, int64_t ldp) {
  __shared__ T r[CB][CB + 1];
  __shared__ T rinv[CB];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  if (threadIdx.x < jb) rinv[threadIdx.x] = T(1) / Rbb[threadIdx.x + threadIdx.x * ldr];
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
        x[i] = s * rinv[i];
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
  __shared__ T rinv[CB];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  if (threadIdx.x < jb) rinv[threadIdx.x] = T(1) / Rbb[threadIdx.x + threadIdx.x * ldr];
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
        x[j] = s * rinv[j];
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
  __shared__ T rinv[CB];
  for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
    const int i = t % jb, j = t / jb;
    r[i][j] = Rbb[i + j * ldr];
  }
  if (threadIdx.x < jb) rinv[threadIdx.x] = T(1) / Rbb[threadIdx.x + threadIdx.x * ldr];
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
        x[i] = s * rinv[i];
      }
    }
#pragma unroll
    for (int i = 0; i < CB; ++i)
      if (i < jb) xc[i] = x[i];
  }
}

}  // namespace

// one or two Cholesky factorizations G_m = R_m^T R_m in place (upper R,
// lower part zeroed) in one cooperative launch; ok[m] false when G_m is not
// numerically positive definite
template <typename T>
void potrf_upper_batch(lra_ctx* ctx, int n, const int64_t* k, T* const* G, const int64_t* ldg, bool* ok);

// Blocked right-looking Cholesky on the tensor-core path for orders past
// kPotrfPanel * 2: per panel of kPotrfPanel columns the diagonal blocks of
// all matrices factored in one cooperative launch, the block rows R12 =
// R11^-T G12 = Dr^-1 (Y^T G12) with Y = R11^-1 Dr (tri_inv_upper), and the
// trailing G22 -= R12^T R12 as a tensor-core GEMM; the cooperative kernel's
// FP64 trailing updates (k^3 / 3 FMAs on the FP64 pipe) are the cost this
// removes.
constexpr int64_t kPotrfPanel = 256;

template <typename T>
void potrf_upper_blocked(lra_ctx* ctx, int n, const int64_t* k, T* const* G, const int64_t* ldg, bool* ok) {
  int64_t kmax = 0;
  for (int m = 0; m < n; ++m) {
    ok[m] = true;
    kmax = std::max(kmax, k[m]);
  }
  for (int64_t j0 = 0; j0 < kmax; j0 += kPotrfPanel) {
    int64_t kb[2] = {0, 0}, lb[2] = {1, 1};
    T* Gb[2] = {nullptr, nullptr};
    bool okb[2] = {true, true};
    int idx[2] = {-1, -1}, nb = 0;
    for (int m = 0; m < n; ++m) {
      if (!ok[m] || j0 >= k[m]) continue;
      idx[nb] = m;
      kb[nb] = std::min(kPotrfPanel, k[m] - j0);
      Gb[nb] = G[m] + j0 + j0 * ldg[m];
      lb[nb] = ldg[m];
      ++nb;
    }
    if (nb == 0) break;
    potrf_upper_batch<T>(ctx, nb, kb, Gb, lb, okb);
    for (int b = 0; b < nb; ++b) {
      const int m = idx[b];
      if (!okb[b]) {
        ok[m] = false;
        continue;
      }
      const int64_t jb = kb[b], rest = k[m] - j0 - jb, ld = ldg[m];
      if (rest <= 0) continue;
      const ArenaMark mk = ctx->arena.mark();
      T* Y = ctx->arena.alloc_n<T>((size_t)jb * jb);
      T* W = ctx->arena.alloc_n<T>((size_t)jb * rest);
      tri_inv_upper<T>(ctx, jb, Gb[b], ld, Y, jb);
      T* G12 = G[m] + j0 + (j0 + jb) * ld;
      gemm<T>(ctx, 't', 'n', jb, rest, jb, T(1), Y, jb, G12, ld, T(0), W, jb);
      div_by_diag<T>(ctx, jb, rest, Gb[b], ld, 'l', W, jb, G12, ld);
      T* G22 = G[m] + (j0 + jb) + (j0 + jb) * ld;
      gemm<T>(ctx, 't', 'n', rest, rest, jb, T(-1), G12, ld, G12, ld, T(1), G22, ld);
      ctx->arena.release(mk);  // stream-ordered reuse
    }
  }
  for (int m = 0; m < n; ++m)
    if (k[m] > 0) zero_lower(ctx, k[m], k[m], G[m], ldg[m]);
}

template <typename T>
void potrf_upper_batch(lra_ctx* ctx, int n, const int64_t* k, T* const* G, const int64_t* ldg, bool* ok) {
  if (sizeof(T) == 8 && ctx->gemm_tc) {
    int64_t kmax = 0;
    for (int m = 0; m < n; ++m) kmax = std::max(kmax, k[m]);
    if (kmax > 2 * kPotrfPanel) {
      potrf_upper_blocked<T>(ctx, n, k, G, ldg, ok);
      return;
    }
  }
  const ArenaMark mk = ctx->arena.mark();
  int* bad = ctx->arena.alloc_n<int>(2);
  LRA_CUDA(cudaMemsetAsync(bad, 0, 2 * sizeof(int), ctx->stream));
  PotrfJobs<T> J{};
  J.n = 0;
  J.bad = bad;
  int slot[2] = {-1, -1};
  for (int m = 0; m < n; ++m) {
    ok[m] = true;
    if (k[m] <= 0) continue;
    slot[m] = J.n;
    J.k[J.n] = k[m];
    J.G[J.n] = G[m];
    J.ldg[J.n] = ldg[m];
    ++J.n;
  }
  if (J.n > 0) {
    int per_sm = 0;
    LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, potrf_coop_kernel<T>, 256, 0));
    const int grid = std::max(J.n, std::min(ctx->num_sms, ctx->num_sms * per_sm));
    GridBar* bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
    LRA_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBar), ctx->stream));
    void* args[] = {&J, &bar};
    LRA_CUDA(cudaLaunchCooperativeKernel((const void*)potrf_coop_kernel<T>, dim3(grid), dim3(256), args, 0,
                                         ctx->stream));
    post_launch(ctx, "potrf_coop_kernel");
    for (int m = 0; m < J.n; ++m) zero_lower(ctx, J.k[m], J.k[m], J.G[m], J.ldg[m]);
    int h[2] = {0, 0};
    GridBar hb;
    LRA_CUDA(cudaMemcpyAsync(h, bad, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    LRA_CUDA(cudaMemcpyAsync(&hb, bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->arena.release(mk);
    if (hb.err != 0) fail(LRA_ETIMEDOUT, "potrf: a grid barrier timed out");
    for (int m = 0; m < n; ++m)
      if (slot[m] >= 0) ok[m] = h[slot[m]] == 0;
    return;
  }
  ctx->arena.release(mk);
}

template <typename T>
bool potrf_upper(lra_ctx* ctx, int64_t k, T* G, int64_t ldg) {
  if (k <= 0) return true;
  if (k > CB) {
    bool ok = true;
    potrf_upper_batch<T>(ctx, 1, &k, &G, &ldg, &ok);
    return ok;
  }
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

namespace {

// Y = R^-1 D with D = diag(R), the inverse of the unit upper triangular
// D^-1 R (k x k, strictly lower part zero), a CTA per column: column j
// solves R y = R_jj e_j by column-oriented back substitution -- y_j = 1,
// then a_i -= R_iq y_q for i < q and y_q = a_q / R_qq from q = j down --
// with the partial sums a_i in the registers of the thread owning row i
// (rows tid + 128 u) and the finished y in shared memory; the column of R a
// step needs is loaded one step ahead, and 1 / R_qq is computed for every q
// first, so that no FP64 division sits on a step's critical path (a product
// with the reciprocal instead, within an ulp of the quotient).  A graded R
// (|R_iq| <= |R_ii|, as a
// pivoted QR leaves it) has an inverse whose rows span its whole diagonal
// range, which a GEMM that scales each row by its largest entry would
// truncate; R^-1 D has entries of order one.
constexpr int kTiNT = 128;
constexpr int kTiRows = 16;   // rows a thread: k up to 2048
constexpr int kTiLeaf = 512;  // larger orders split in two on the tensor-core path

template <typename T>
__global__ void __launch_bounds__(kTiNT) tri_inv_upper_kernel(int64_t k, const T* __restrict__ R, int64_t ldr,
                                                              T* __restrict__ Y, int64_t ldy) {
  extern __shared__ unsigned char ti_smem[];
  T* ys = reinterpret_cast<T*>(ti_smem);  // k
  T* rdi = ys + k;                        // 1 / R_qq, off the per-step critical path
  const int tid = threadIdx.x;
  const int U = (int)((k + kTiNT - 1) / kTiNT);
  for (int64_t q = tid; q < k; q += kTiNT) rdi[q] = T(1) / R[q + q * ldr];
  __syncthreads();
  for (int64_t j = blockIdx.x; j < k; j += gridDim.x) {
    T a[kTiRows], rc[kTiRows];
#pragma unroll
    for (int u = 0; u < kTiRows; ++u) {
      const int64_t i = tid + (int64_t)kTiNT * u;
      a[u] = T(0);
      rc[u] = u < U && i < j ? R[i + j * ldr] : T(0);
    }
    if (tid == 0) ys[j] = T(1);
    __syncthreads();
    for (int64_t q = j; q > 0; --q) {
      const T yq = ys[q];
      const T rqq = rdi[q - 1];
      T rn[kTiRows];
#pragma unroll
      for (int u = 0; u < kTiRows; ++u) {
        const int64_t i = tid + (int64_t)kTiNT * u;
        rn[u] = u < U && i < q - 1 ? R[i + (q - 1) * ldr] : T(0);
      }
#pragma unroll
      for (int u = 0; u < kTiRows; ++u) {
        const int64_t i = tid + (int64_t)kTiNT * u;
        if (u < U && i < q) {
          a[u] = fma(-rc[u], yq, a[u]);
          if (i == q - 1) ys[q - 1] = a[u] * rqq;
        }
        rc[u] = rn[u];
      }
      __syncthreads();
    }
    for (int64_t i = tid; i < k; i += kTiNT) Y[i + j * ldy] = i <= j ? ys[i] : T(0);
    __syncthreads();  // ys is rewritten for the next column
  }
}

// dst = src with row i (side 'l') or column j (side 'r') divided by R's
// diagonal entry, as the substitution divides
template <typename T>
__global__ void div_by_diag_kernel(int64_t m, int64_t n, const T* __restrict__ R, int64_t ldr, bool rows,
                                   const T* __restrict__ src, int64_t lds, T* __restrict__ dst, int64_t ldd) {
  const int64_t total = m * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    const int64_t d = rows ? i : j;
    dst[i + j * ldd] = src[i + j * lds] / R[d + d * ldr];
  }
}

}  // namespace

template <typename T>
void div_by_diag(lra_ctx* ctx, int64_t m, int64_t n, const T* R, int64_t ldr, char side, const T* src, int64_t lds,
                 T* dst, int64_t ldd) {
  if (m <= 0 || n <= 0) return;
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m * n + 255) / 256, ctx->num_sms * 8));
  div_by_diag_kernel<T><<<g, 256, 0, ctx->stream>>>(m, n, R, ldr, side == 'l', src, lds, dst, ldd);
  post_launch(ctx, "div_by_diag_kernel");
}
template void div_by_diag<float>(lra_ctx*, int64_t, int64_t, const float*, int64_t, char, const float*, int64_t,
                                 float*, int64_t);
template void div_by_diag<double>(lra_ctx*, int64_t, int64_t, const double*, int64_t, char, const double*, int64_t,
                                  double*, int64_t);

template <typename T>
bool tri_inv_upper(lra_ctx* ctx, int64_t k, const T* R, int64_t ldr, T* Y, int64_t ldy) {
  if (k <= 0) return true;
  if (k > (int64_t)kTiNT * kTiRows) return false;
  if (sizeof(T) == 8 && ctx->gemm_tc && k > kTiLeaf) {
    // Recursive on the tensor-core path: with R = [A B; 0 C] and D = diag(R),
    // R^-1 D = [Ya, -Ya (Da^-1 B) Yc; 0, Yc] for Ya = A^-1 Da, Yc = C^-1 Dc.
    // Every factor has entries of order one (Da^-1 B because |R_iq| <=
    // |R_ii| in a pivoted QR's R), so the two products are accurate on the
    // tensor cores; the leaves' column substitutions are shorter.
    const int64_t k1 = (k / 2 + 31) / 32 * 32, k2 = k - k1;
    tri_inv_upper<T>(ctx, k1, R, ldr, Y, ldy);
    tri_inv_upper<T>(ctx, k2, R + k1 + k1 * ldr, ldr, Y + k1 + k1 * ldy, ldy);
    const ArenaMark mk = ctx->arena.mark();
    T* W = ctx->arena.alloc_n<T>((size_t)k1 * k2);
    T* W2 = ctx->arena.alloc_n<T>((size_t)k1 * k2);
    div_by_diag<T>(ctx, k1, k2, R, ldr, 'l', R + k1 * ldr, ldr, W, k1);
    gemm<T>(ctx, 'n', 'n', k1, k2, k2, T(1), W, k1, Y + k1 + k1 * ldy, ldy, T(0), W2, k1);
    gemm<T>(ctx, 'n', 'n', k1, k2, k1, T(-1), Y, ldy, W2, k1, T(0), Y + k1 * ldy, ldy);
    zero_lower(ctx, k, k, Y, ldy);  // the block below the diagonal
    ctx->arena.release(mk);  // stream-ordered reuse
    return true;
  }
  const size_t smem = (size_t)2 * k * sizeof(T);
  if (smem > 48 * 1024) raise_smem_limit(ctx, (const void*)tri_inv_upper_kernel<T>);
  tri_inv_upper_kernel<T><<<(unsigned)k, kTiNT, smem, ctx->stream>>>(k, R, ldr, Y, ldy);
  post_launch(ctx, "tri_inv_upper_kernel");
  return true;
}

template bool tri_inv_upper<float>(lra_ctx*, int64_t, const float*, int64_t, float*, int64_t);
template bool tri_inv_upper<double>(lra_ctx*, int64_t, const double*, int64_t, double*, int64_t);

// Whether a triangular solve with a k x k factor and `other` right-hand
// sides should multiply by the explicit inverse instead: on the tensor-core
// path for FP64, where the substitution's diagonal blocks run on the FP64
// pipe (a few FMAs a clock per SM) and the inverse costs one GEMM
template <typename T>
bool trsm_by_inverse(const lra_ctx* ctx, int64_t k, int64_t other) {
  if (sizeof(T) != 8 || !ctx->gemm_tc || ctx->tuning.trsm_inv == 1) return false;
  return k > 2 * CB && k <= (int64_t)kTiNT * kTiRows && tc_gemm_worthwhile(other, k, k);
}
template bool trsm_by_inverse<float>(const lra_ctx*, int64_t, int64_t);
template bool trsm_by_inverse<double>(const lra_ctx*, int64_t, int64_t);

// X <- X triu(R)^{-1}, recursive like trsm_upper: the leading half, a GEMM
// update of the trailing columns, the trailing half; on the tensor-core
// path X times the explicit inverse
template <typename T>
void trsm_right_upper(lra_ctx* ctx, int64_t m, int64_t k, const T* R, int64_t ldr, T* X, int64_t ldx, const T* Yd) {
  if (m <= 0 || k <= 0) return;
  if (trsm_by_inverse<T>(ctx, k, m)) {
    const ArenaMark mk = ctx->arena.mark();
    T* Y = Yd ? nullptr : ctx->arena.alloc_n<T>((size_t)k * k);
    T* W = ctx->arena.alloc_n<T>((size_t)m * k);
    // X R^-1 = (X Y) D^-1 with Y = R^-1 D (Yd when the caller has it)
    if (Y) tri_inv_upper<T>(ctx, k, R, ldr, Y, k);
    gemm<T>(ctx, 'n', 'n', m, k, k, T(1), X, ldx, Yd ? Yd : Y, k, T(0), W, m);
    div_by_diag<T>(ctx, m, k, R, ldr, 'r', W, m, X, ldx);
    ctx->arena.release(mk);  // stream-ordered reuse
    return;
  }
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
template void potrf_upper_batch<float>(lra_ctx*, int, const int64_t*, float* const*, const int64_t*, bool*);
template void potrf_upper_batch<double>(lra_ctx*, int, const int64_t*, double* const*, const int64_t*, bool*);
template void trsm_right_upper<float>(lra_ctx*, int64_t, int64_t, const float*, int64_t, float*, int64_t,
                                      const float*);
template void trsm_right_upper<double>(lra_ctx*, int64_t, int64_t, const double*, int64_t, double*, int64_t,
                                       const double*);
// ---- T = R11^{-1} R12 by back substitution, a thread per right-hand side -------
// The ID's solve (src/id.jl:447, R11 \ R12) for ranks up to kBsMax: row
// i of x is (x_i - sum_{j > i} R_ij x_j) / R_ii, the sum taken from j = i+1
// upwards, from the bottom row.  The batched path runs the same per-column
// loop with a CTA per matrix, so both give the same bits.
template <typename T>
__device__ __forceinline__ void bs_column(int k, const T* __restrict__ R, int64_t ldr, T* __restrict__ x) {
  for (int i = k - 1; i >= 0; --i) {
    T s = x[i];
    const T* r = R + i;
    for (int j = i + 1; j < k; ++j) s = fma(-r[j * ldr], x[j], s);
    x[i] = s / r[i * ldr];
  }
}

template <typename T>
__global__ void trsm_bs_kernel(int k, int64_t nrhs, const T* __restrict__ R, int64_t ldr, T* X, int64_t ldx) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nrhs; c += (int64_t)gridDim.x * blockDim.x)
    bs_column(k, R, ldr, X + c * ldx);
}

template <typename T>
void trsm_bs(lra_ctx* ctx, int64_t k, int64_t nrhs, const T* R, int64_t ldr, T* X, int64_t ldx) {
  if (k <= 0 || nrhs <= 0) return;
  if (k > kBsMax) fail(LRA_EINVAL, "trsm_bs: k > %d", kBsMax);
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((nrhs + 127) / 128, (int64_t)ctx->num_sms * 8));
  trsm_bs_kernel<T><<<g, 128, 0, ctx->stream>>>((int)k, nrhs, R, ldr, X, ldx);
  post_launch(ctx, "trsm_bs_kernel");
}

// one matrix of the batch: T (k x nr, ld k) = R11^{-1} R12, both read from B
struct BsJob {
  int64_t k, nr, ldb;
  const double* B;
  double* T;
};

__global__ void __launch_bounds__(256) trsm_bs_group_kernel(const BsJob* __restrict__ jobs) {
  const BsJob J = jobs[blockIdx.x];
  for (int64_t c = threadIdx.x; c < J.nr; c += blockDim.x) {
    double* x = J.T + c * J.k;
    const double* b = J.B + (J.k + c) * J.ldb;
    for (int64_t i = 0; i < J.k; ++i) x[i] = b[i];
    bs_column((int)J.k, J.B, J.ldb, x);
  }
}

void trsm_bs_batch(lra_ctx* ctx, int64_t count, const BsItem* items) {
  if (count <= 0) return;
  std::vector<BsJob> jobs;
  jobs.reserve((size_t)count);
  for (int64_t i = 0; i < count; ++i) {
    const BsItem& it = items[i];
    if (it.k > kBsMax) fail(LRA_EINVAL, "trsm_bs_batch: k > %d", kBsMax);
    if (it.k > 0 && it.nr > 0) jobs.push_back(BsJob{it.k, it.nr, it.ldb, it.B, it.T});
  }
  if (jobs.empty()) return;
  BsJob* d = ctx->arena.alloc_n<BsJob>(jobs.size());
  LRA_CUDA(cudaMemcpyAsync(d, jobs.data(), jobs.size() * sizeof(BsJob), cudaMemcpyHostToDevice, ctx->stream));
  trsm_bs_group_kernel<<<(unsigned)jobs.size(), 256, 0, ctx->stream>>>(d);
  post_launch(ctx, "trsm_bs_group_kernel");
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
}

__global__ void pack_results_kernel(const PackItem* __restrict__ items, char* __restrict__ out) {
  const PackItem it = items[blockIdx.x];
  int64_t* p = reinterpret_cast<int64_t*>(out + it.off);
  for (int64_t i = threadIdx.x; i < it.n; i += blockDim.x) p[i] = it.jpvt[i];
  double* t = reinterpret_cast<double*>(out + it.off + 8 * (size_t)it.n);
  for (int64_t i = threadIdx.x; i < it.nt; i += blockDim.x) t[i] = it.T[i];
}

void pack_results(lra_ctx* ctx, int64_t count, const PackItem* items, char* out) {
  if (count <= 0) return;
  PackItem* d = ctx->arena.alloc_n<PackItem>((size_t)count);
  LRA_CUDA(cudaMemcpyAsync(d, items, (size_t)count * sizeof(PackItem), cudaMemcpyHostToDevice, ctx->stream));
  pack_results_kernel<<<(unsigned)count, 256, 0, ctx->stream>>>(d, out);
  post_launch(ctx, "pack_results_kernel");
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
}

template void trsm_bs<float>(lra_ctx*, int64_t, int64_t, const float*, int64_t, float*, int64_t);
template void trsm_bs<double>(lra_ctx*, int64_t, int64_t, const double*, int64_t, double*, int64_t);
template void trsm_left_diag<float>(lra_ctx*, int, int64_t, const float*, int64_t, float*, int64_t);
template void trsm_left_diag<double>(lra_ctx*, int, int64_t, const double*, int64_t, double*, int64_t);

cudaError_t set_wait_limit_dense(uint64_t ns) { return set_unit_wait_limit(ns); }

}  // namespace lra
