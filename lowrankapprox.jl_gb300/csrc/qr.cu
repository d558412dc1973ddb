// Rank-adaptive column-pivoted Householder QR (geqp3_adap!), triangular
// solve, Householder application -- CUDA cores, input precision.
//
// geqp3_adap! (src/pqr.jl:348-418) drives LAPACK xLAQPS block by block
// (src/lapack.jl:117-139).  This kernel keeps xLAQPS's observable
// semantics -- IxAMAX pivots (largest partial norm, first index on ties),
// the xLARFG reflector, the partial-norm downdate with the tol3z
// recomputation trigger, the early end of a block when a norm must be
// recomputed, and the reference's rank test on the last diagonal entry of
// each block -- but applies each reflector to the trailing columns at once
// instead of through xLAQPS's F matrix: on the GPU one pass over the
// trailing panel per pivot is the natural unit, and the results agree with
// LAPACK to rounding.
//
// One cooperative launch does the whole factorization.  Every CTA runs the
// same control flow and takes every decision from data made visible by a
// bounded grid barrier, so all CTAs agree without further messages.

#include <cooperative_groups.h>

#include <algorithm>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "df64.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename T>
struct QrParams {
  int64_t m, n, lda;
  T* A;
  int64_t* jpvt;
  T* tau;
  T* vn1;
  T* vn2;
  int* flag;
  T* part_v;
  int64_t* part_i;
  double* part_d;
  int* lsticc;  // [2]
  GridBar* bar;
  int64_t kmax, nb;
  double atol, rtol;
  int pivot;
  int64_t* k_out;
  int64_t vcap;  // reflector rows that fit the dynamic shared memory
  // double-float QR: columns with at most this many rows below the pivot
  // row are summed by one thread each (the tuning table's qr_seq_len)
  int seq_len = 96;
};

constexpr int CH = 16;  // rows per lane held in registers per column chunk

// exact power-of-two scale for a norm computation
__device__ __forceinline__ double pow2_scale_inv(double mx) {
  int e = ilogb(mx);
  return ldexp(1.0, -e);
}

// 2-norm of x[0..len) computed by one warp (all lanes get the result)
template <typename T>
__device__ T warp_nrm2(const T* x, int64_t len, int lane) {
  double mx = 0;
  for (int64_t i = lane; i < len; i += 32) mx = fmax(mx, fabs((double)__ldcg(x + i)));
  mx = warp_max(mx);
  if (mx == 0 || !isfinite(mx)) return (T)mx;
  const double s = pow2_scale_inv(mx);
  double acc = 0;
  for (int64_t i = lane; i < len; i += 32) {
    double t = (double)__ldcg(x + i) * s;
    acc = fma(t, t, acc);
  }
  acc = warp_sum(acc);
  return (T)(sqrt(acc) / s);
}

template <typename T>
__device__ T block_nrm2(const T* x, int64_t len, double* red) {
  double mx = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) mx = fmax(mx, fabs((double)__ldcg(x + i)));
  mx = block_max(mx, red);
  if (mx == 0 || !isfinite(mx)) return (T)mx;
  const double s = pow2_scale_inv(mx);
  double acc = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    double t = (double)__ldcg(x + i) * s;
    acc = fma(t, t, acc);
  }
  acc = block_sum(acc, red);
  return (T)(sqrt(acc) / s);
}

template <typename T>
__device__ __forceinline__ T lapy2(T x, T y) {
  T xa = fabs(x), ya = fabs(y);
  T w = fmax(xa, ya), z = fmin(xa, ya);
  if (z == 0 || w > Real<T>::big) return w;
  T q = z / w;
  return w * sqrt(T(1) + q * q);
}

// block-wide argmax of per-thread candidates; result in (v, i) on all threads
template <typename T>
__device__ void block_argmax(T& v, int64_t& i, T* sv, int64_t* si) {
  warp_argmax(v, i);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = i;
  }
  __syncthreads();
  if (wid == 0) {
    T vv = lane < nw ? sv[lane] : T(-1);
    int64_t ii = lane < nw ? si[lane] : INT64_MAX;
    warp_argmax(vv, ii);
    if (lane == 0) {
      sv[0] = vv;
      si[0] = ii;
    }
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
  __syncthreads();
}

// every CTA reduces the per-CTA partials to the global argmax
template <typename T>
__device__ int64_t reduce_pivot(const QrParams<T>& P, T* sv, int64_t* si) {
  T v = T(-1);
  int64_t i = INT64_MAX;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
    argmax_merge(v, i, __ldcg(P.part_v + b), __ldcg(P.part_i + b));
  block_argmax(v, i, sv, si);
  return i;
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT) geqp3_kernel(QrParams<T> P) {
  __shared__ T sv[32];
  __shared__ int64_t si[32];
  __shared__ double red[32];
  __shared__ T s_tau;
  extern __shared__ unsigned char qr_dyn[];
  T* vs = reinterpret_cast<T*>(qr_dyn);
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * NW + wid;
  const int64_t W = (int64_t)gridDim.x * NW;
  const int64_t m = P.m, n = P.n, lda = P.lda;
  T* __restrict__ A = P.A;
  const T tol3z = sqrt(Real<T>::eps);
  const int64_t lastrk = m < n ? m : n;

  // ---- initial column norms, ptol, first pivot -----------------------------
  double lmax = 0;
  T bv = T(-1);
  int64_t bi = INT64_MAX;
  for (int64_t j = gw; j < n; j += W) {
    T nr = P.pivot ? warp_nrm2(A + j * lda, m, lane) : T(0);
    if (lane == 0) {
      P.vn1[j] = nr;
      P.vn2[j] = nr;
      P.flag[j] = 0;
      P.jpvt[j] = j + 1;
    }
    lmax = fmax(lmax, (double)nr);
    argmax_merge(bv, bi, nr, j);
  }
  lmax = block_max(lmax, red);
  block_argmax(bv, bi, sv, si);
  if (threadIdx.x == 0) {
    P.part_d[blockIdx.x] = lmax;
    P.part_v[blockIdx.x] = bv;
    P.part_i[blockIdx.x] = bi;
  }
  if (!grid_sync(P.bar)) return;
  double maxnrm = 0;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x)
    maxnrm = fmax(maxnrm, __ldcg(P.part_d + b));
  maxnrm = block_max(maxnrm, red);
  const double ptol = fmax(P.atol, P.rtol * maxnrm);
  int64_t pvt = reduce_pivot(P, sv, si);

  int64_t kres = P.kmax;
  int64_t j = 0;
  int par = 0;
  while (j < P.kmax) {
    const int64_t jb = min(P.nb, P.kmax - j);
    int* lst = P.lsticc + par;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.lsticc[par ^ 1] = 0;
    int64_t kk = 0;
    bool stop_block = false;
    while (kk < jb && !stop_block) {
      const int64_t c = j + kk;
      if (!P.pivot) pvt = c;
      // ---- one CTA: pivot swap + reflector -----------------------------------
      if (blockIdx.x == 0) {
        if (pvt != c) {
          T* a1 = A + c * lda;
          T* a2 = A + pvt * lda;
          for (int64_t i = threadIdx.x; i < m; i += NT) {
            T t1 = __ldcg(a1 + i), t2 = __ldcg(a2 + i);
            a1[i] = t2;
            a2[i] = t1;
          }
          if (threadIdx.x == 0) {
            // (every cross-CTA read in this kernel bypasses L1: ld.global.cg)
            const int64_t it = __ldcg(P.jpvt + pvt);
            P.jpvt[pvt] = __ldcg(P.jpvt + c);
            P.jpvt[c] = it;
            P.vn1[pvt] = __ldcg(P.vn1 + c);
            P.vn2[pvt] = __ldcg(P.vn2 + c);
          }
        }
        __syncthreads();
        T* col = A + c * lda;
        T tau = 0;
        if (c < m - 1) {
          T* x = col + c + 1;
          const int64_t len = m - c - 1;
          T xnorm = block_nrm2(x, len, red);
          T alpha = __ldcg(col + c);
          if (xnorm != 0) {
            T beta = -copysign(lapy2(alpha, xnorm), alpha);
            const T safmin = Real<T>::safmin / Real<T>::eps;
            int knt = 0;
            if (fabs(beta) < safmin) {
              const T rsafmn = T(1) / safmin;
              do {
                ++knt;
                for (int64_t i = threadIdx.x; i < len; i += NT) x[i] = __ldcg(x + i) * rsafmn;
                beta *= rsafmn;
                alpha *= rsafmn;
              } while (fabs(beta) < safmin && knt < 20);
              __syncthreads();
              xnorm = block_nrm2(x, len, red);
              beta = -copysign(lapy2(alpha, xnorm), alpha);
            }
            tau = (beta - alpha) / beta;
            const T scal = T(1) / (alpha - beta);
            for (int64_t i = threadIdx.x; i < len; i += NT) x[i] = __ldcg(x + i) * scal;
            for (int q = 0; q < knt; ++q) beta *= safmin;
            __syncthreads();
            if (threadIdx.x == 0) col[c] = beta;
          }
        }
        if (threadIdx.x == 0) P.tau[c] = tau;
      }
      if (!grid_sync(P.bar)) return;

      // ---- all warps: apply H(c) to the trailing columns, downdate norms ------
      // The reflector (rows c+1..m-1) is staged once per CTA in shared memory
      // and each column is pulled into registers with independent loads, so
      // a column costs one L2 round trip instead of one per row.
      if (threadIdx.x == 0) s_tau = __ldcg(P.tau + c);
      const int64_t len = m - c - 1;
      const T* vsrc = A + c * lda + c + 1;
      const bool vsm = len <= P.vcap;
      if (vsm)
        for (int64_t i = threadIdx.x; i < len; i += NT) vs[i] = __ldcg(vsrc + i);
      __syncthreads();
      const T tauc = s_tau;
      bv = T(-1);
      bi = INT64_MAX;
      int myflag = 0;
      int64_t jj = c + 1 + ((gw - (c + 1)) % W + W) % W;
      for (; jj < n; jj += W) {
        T* colj = A + jj * lda;
        T* cj = colj + c + 1;
        T s = 0;
        T x[CH];
        if (len <= 32 * CH) {
#pragma unroll
          for (int t = 0; t < CH; ++t) {
            const int64_t i = lane + 32 * t;
            x[t] = i < len ? __ldcg(cj + i) : T(0);
          }
#pragma unroll
          for (int t = 0; t < CH; ++t) {
            const int64_t i = lane + 32 * t;
            if (i < len) s += (vsm ? vs[i] : __ldcg(vsrc + i)) * x[t];
          }
        } else {
          for (int64_t b0 = 0; b0 < len; b0 += 32 * CH) {
#pragma unroll
            for (int t = 0; t < CH; ++t) {
              const int64_t i = b0 + lane + 32 * t;
              x[t] = i < len ? __ldcg(cj + i) : T(0);
            }
#pragma unroll
            for (int t = 0; t < CH; ++t) {
              const int64_t i = b0 + lane + 32 * t;
              if (i < len) s += (vsm ? vs[i] : __ldcg(vsrc + i)) * x[t];
            }
          }
        }
        s = warp_sum(s);
        const T arc0 = __ldcg(colj + c);
        const T f = tauc * (arc0 + s);
        if (f != 0) {
          if (len <= 32 * CH) {
#pragma unroll
            for (int t = 0; t < CH; ++t) {
              const int64_t i = lane + 32 * t;
              if (i < len) cj[i] = x[t] - f * (vsm ? vs[i] : __ldcg(vsrc + i));
            }
          } else {
            for (int64_t b0 = 0; b0 < len; b0 += 32 * CH) {
#pragma unroll
              for (int t = 0; t < CH; ++t) {
                const int64_t i = b0 + lane + 32 * t;
                x[t] = i < len ? __ldcg(cj + i) : T(0);
              }
#pragma unroll
              for (int t = 0; t < CH; ++t) {
                const int64_t i = b0 + lane + 32 * t;
                if (i < len) cj[i] = x[t] - f * (vsm ? vs[i] : __ldcg(vsrc + i));
              }
            }
          }
        }
        const T arc = arc0 - f;
        if (lane == 0) colj[c] = arc;
        if (P.pivot) {
          T v1 = __ldcg(P.vn1 + jj);
          if (c < lastrk - 1 && v1 != 0) {
            T temp = fabs(arc) / v1;
            temp = fmax(T(0), (T(1) + temp) * (T(1) - temp));
            const T r = v1 / __ldcg(P.vn2 + jj);
            const T temp2 = temp * r * r;
            if (temp2 <= tol3z) {
              myflag = 1;
              if (lane == 0) P.flag[jj] = 1;
            } else {
              v1 = v1 * sqrt(temp);
              if (lane == 0) P.vn1[jj] = v1;
            }
          }
          argmax_merge(bv, bi, v1, jj);
        }
      }
      if (myflag && lane == 0) atomicAdd(lst, 1);
      block_argmax(bv, bi, sv, si);
      if (threadIdx.x == 0) {
        P.part_v[blockIdx.x] = bv;
        P.part_i[blockIdx.x] = bi;
      }
      if (!grid_sync(P.bar)) return;
      stop_block = *((volatile int*)lst) != 0;
      pvt = reduce_pivot(P, sv, si);
      ++kk;
    }
    const int64_t kb = kk;
    const int64_t jn = j + kb;
    if (stop_block) {
      // recompute the flagged partial norms over rows jn..m-1
      bv = T(-1);
      bi = INT64_MAX;
      for (int64_t q = jn + ((gw - jn) % W + W) % W; q < n; q += W) {
        T v1 = __ldcg(P.vn1 + q);
        if (__ldcg(P.flag + q)) {
          v1 = warp_nrm2(A + q * lda + jn, m - jn, lane);
          if (lane == 0) {
            P.vn1[q] = v1;
            P.vn2[q] = v1;
            P.flag[q] = 0;
          }
        }
        argmax_merge(bv, bi, v1, q);
      }
      block_argmax(bv, bi, sv, si);
      if (threadIdx.x == 0) {
        P.part_v[blockIdx.x] = bv;
        P.part_i[blockIdx.x] = bi;
      }
      if (!grid_sync(P.bar)) return;
      pvt = reduce_pivot(P, sv, si);
    }
    // rank test of geqp3_adap_main! (src/pqr.jl:407-415)
    if (fabs((double)__ldcg(A + (jn - 1) + (jn - 1) * lda)) <= ptol) {
      bool found = false;
      for (int64_t i = j; i < jn; ++i) {
        if (fabs((double)__ldcg(A + i + i * lda)) <= ptol) {
          kres = i;
          found = true;
          break;
        }
      }
      if (found) break;
    }
    j = jn;
    par ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.k_out = kres;
}

// ---- geqp3_adap!, one grid barrier per pivot ---------------------------------------
//
// Columns never move during the factorization: pivot c is the physical
// column piv[c], R's row c sits in row c of every column, the reflector of
// pivot c below it in column piv[c].  Every CTA computes the xLARFG
// reflector of the pivot column itself, into its own shared memory, with
// the same block reductions (so the values agree bit for bit); CTA 0 writes
// it back.  Each warp owns the columns gw, gw + W, ... and keeps their partial
// norms in registers, one lane per column.  A pivot thus needs one bounded
// grid barrier, after which every CTA reduces the per-CTA candidates.
// LAPACK's column swaps are replayed afterwards (geqp3_permute) so that A,
// jpvt and the order of the non-pivot columns come out as xLAQPS leaves
// them.  Exactly equal partial norms go to the lowest physical index.

struct QrV2Extra {
  int64_t* piv;     // pivot c -> physical column
  int64_t* nfac;    // number of pivots performed
  long long* part_k;  // per-CTA pivot candidate keys
  double* beta;     // R(c, c) of each pivot, for the rank test
};

// Column state lives in shared memory, one slot per column the CTA owns:
// column j belongs to warp j mod W (W warps in the grid), and its slot in
// the owning CTA is (j div W) * NW + warp-in-CTA.  The dot products and
// updates run a warp per column, two columns at a time so that their load
// and reduction latencies overlap; the norm downdates, which cost two FP64
// divisions and a square root per column, run a thread per slot.  The
// reflector's scalars are computed once per CTA by warp 0, and pivot
// candidates are compared as integer keys (the bit patterns of nonnegative
// floating-point norms order like the norms).
constexpr int QCH = 16;  // rows per lane per register chunk (512 rows)
constexpr int QG = 4;    // rows per lane issued between uniform range checks
constexpr int QRPL = 4;  // rows per lane loaded ahead in the double-float QR's column loops

constexpr int QSEQB = 8;  // rows loaded ahead by a thread that walks a column
constexpr unsigned char ST_LIVE = 1, ST_DONE = 2, ST_FLAG = 4, ST_UPD = 8;

__device__ __forceinline__ long long norm_key(double v) {
  const long long b = __double_as_longlong(v);
  return b < 0 ? -1 : b;
}
__device__ __forceinline__ long long norm_key(float v) {
  const int b = __float_as_int(v);
  return b < 0 ? -1 : (long long)b;
}

__device__ __forceinline__ void key_merge(long long& k, int64_t& i, long long k2, int64_t i2) {
  if (k2 > k || (k2 == k && i2 < i)) {
    k = k2;
    i = i2;
  }
}

// block-wide argmax of (key, index); the index of the winner on all threads
__device__ int64_t block_argmax_key(long long k, int64_t i, long long* sk, int64_t* si) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
    const int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
    key_merge(k, i, k2, i2);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) {
    sk[wid] = k;
    si[wid] = i;
  }
  __syncthreads();
  if (wid == 0) {
    long long kk = lane < nw ? sk[lane] : -2;
    int64_t ii = lane < nw ? si[lane] : INT64_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long k2 = __shfl_xor_sync(0xffffffffu, kk, o);
      const int64_t i2 = __shfl_xor_sync(0xffffffffu, ii, o);
      key_merge(kk, ii, k2, i2);
    }
    if (lane == 0) si[0] = ii;
  }
  __syncthreads();
  const int64_t r = si[0];
  __syncthreads();
  return r;
}

// 2-norm of the reflector tail x[0..len) in shared memory, by one warp:
// an unscaled sum of squares when it is safely inside the exponent range,
// else LAPACK's scaled form
template <typename T>
__device__ T warp_nrm2_smem(const T* x, int64_t len, int lane) {
  double a0 = 0, a1 = 0;
  int64_t i = lane;
  for (; i + 32 < len; i += 64) {
    const double u = (double)x[i], w = (double)x[i + 32];
    a0 = fma(u, u, a0);
    a1 = fma(w, w, a1);
  }
  if (i < len) {
    const double u = (double)x[i];
    a0 = fma(u, u, a0);
  }
  double ssq = warp_sum(a0 + a1);
  if (ssq > 1e-280 && ssq < 1e280) return (T)sqrt(ssq);
  double mx = 0;
  for (int64_t q = lane; q < len; q += 32) mx = fmax(mx, fabs((double)x[q]));
  mx = warp_max(mx);
  if (mx == 0 || !isfinite(mx)) return (T)mx;
  const double s = pow2_scale_inv(mx);
  double acc = 0;
  for (int64_t q = lane; q < len; q += 32) {
    const double t = (double)x[q] * s;
    acc = fma(t, t, acc);
  }
  acc = warp_sum(acc);
  return (T)(sqrt(acc) / s);
}

template <typename T>
struct QrShared {
  long long sk[32];
  int64_t si[32];
  double red[32];
  T alpha, tau, beta, scal;
  int knt;
};

template <typename T, int NT>
__global__ void __launch_bounds__(NT) geqp3_v2_kernel(QrParams<T> P, QrV2Extra X) {
  __shared__ QrShared<T> sh;
  extern __shared__ unsigned char qr_dyn[];
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * NW + wid;
  const int64_t W = (int64_t)gridDim.x * NW;
  const int64_t m = P.m, n = P.n, lda = P.lda;
  T* __restrict__ A = P.A;
  auto ldown = [](const T* p) { return *p; };
  const T tol3z = sqrt(Real<T>::eps);
  const int64_t lastrk = m < n ? m : n;
  const int64_t ncol = gw < n ? (n - 1 - gw) / W + 1 : 0;  // columns of this warp
  const int64_t ncmax = (n + W - 1) / W;
  const int nslot = (int)(ncmax * NW);
  T* vs = reinterpret_cast<T*>(qr_dyn);
  T* s_vn1 = vs + P.vcap;
  T* s_vn2 = s_vn1 + nslot;
  T* s_arc = s_vn2 + nslot;
  unsigned char* s_st = reinterpret_cast<unsigned char*>(s_arc + nslot);
  // slot -> column of this CTA
  auto slot_col = [&](int s) -> int64_t {
    return (int64_t)blockIdx.x * NW + (s % NW) + (int64_t)(s / NW) * W;
  };
  // every CTA reduces the per-CTA candidates to the global pivot
  auto reduce_pivot_key = [&]() -> int64_t {
    long long k = -2;
    int64_t i = INT64_MAX;
    for (int b = threadIdx.x; b < gridDim.x; b += NT) key_merge(k, i, __ldcg(X.part_k + b), __ldcg(P.part_i + b));
    return block_argmax_key(k, i, sh.sk, sh.si);
  };

  // per-CTA winner (key and index) to the grid-wide partials
  auto publish = [&](long long k, int64_t i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
      const int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
      key_merge(k, i, k2, i2);
    }
    __syncthreads();
    if (lane == 0) {
      sh.sk[wid] = k;
      sh.si[wid] = i;
    }
    __syncthreads();
    if (wid == 0) {
      long long k0 = lane < NW ? sh.sk[lane] : -2;
      int64_t i0 = lane < NW ? sh.si[lane] : INT64_MAX;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long k2 = __shfl_xor_sync(0xffffffffu, k0, o);
        const int64_t i2 = __shfl_xor_sync(0xffffffffu, i0, o);
        key_merge(k0, i0, k2, i2);
      }
      if (lane == 0) {
        X.part_k[blockIdx.x] = k0;
        P.part_i[blockIdx.x] = i0;
      }
    }
  };

  // ---- initial column norms, ptol, first pivot -----------------------------
  for (int64_t t = 0; t < ncol; ++t) {
    const int64_t j = gw + t * W;
    const T nr = P.pivot ? warp_nrm2(A + j * lda, m, lane) : T(0);
    if (lane == 0) {
      const int s = (int)(t * NW + wid);
      s_vn1[s] = s_vn2[s] = nr;
    }
  }
  for (int s = threadIdx.x; s < nslot; s += NT) s_st[s] = slot_col(s) < n ? ST_LIVE : 0;
  __syncthreads();
  double lmax = 0;
  long long bk = -2;
  int64_t bi = INT64_MAX;
  for (int s = threadIdx.x; s < nslot; s += NT)
    if (s_st[s] & ST_LIVE) {
      lmax = fmax(lmax, (double)s_vn1[s]);
      key_merge(bk, bi, norm_key(s_vn1[s]), slot_col(s));
    }
  lmax = block_max(lmax, sh.red);
  publish(bk, bi);
  if (threadIdx.x == 0) P.part_d[blockIdx.x] = lmax;
  if (!grid_sync(P.bar)) return;
  double maxnrm = 0;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) maxnrm = fmax(maxnrm, __ldcg(P.part_d + b));
  maxnrm = block_max(maxnrm, sh.red);
  const double ptol = fmax(P.atol, P.rtol * maxnrm);
  int64_t pvt = reduce_pivot_key();

  int64_t kres = P.kmax, nfac = 0;
  int64_t j = 0;
  int par = 0;
  while (j < P.kmax) {
    const int64_t jb = min(P.nb, P.kmax - j);
    int* lst = P.lsticc + par;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.lsticc[par ^ 1] = 0;
    int64_t kk = 0;
    bool stop_block = false;
    while (kk < jb && !stop_block) {
      const int64_t c = j + kk;
      if (!P.pivot) pvt = c;
      // ---- every CTA: the reflector of column pvt, rows c..m-1 ---------------
      const int64_t len = m - c - 1;
      T* pc = A + pvt * lda;
      for (int64_t i = threadIdx.x; i < len; i += NT) vs[i] = __ldcg(pc + c + 1 + i);
      if (threadIdx.x == 0) sh.alpha = __ldcg(pc + c);
      __syncthreads();
      if (wid == 0) {
        // xLARFG: scalars by warp 0, broadcast through shared memory
        T alpha = sh.alpha, tau = 0, beta = alpha, scal = 1;
        int knt = 0;
        if (len > 0) {
          T xnorm = warp_nrm2_smem(vs, len, lane);
          if (xnorm != 0) {
            beta = -copysign(lapy2(alpha, xnorm), alpha);
            const T safmin = Real<T>::safmin / Real<T>::eps;
            if (fabs(beta) < safmin) {
              const T rsafmn = T(1) / safmin;
              do {
                ++knt;
                for (int64_t i = lane; i < len; i += 32) vs[i] *= rsafmn;
                __syncwarp();
                beta *= rsafmn;
                alpha *= rsafmn;
              } while (fabs(beta) < safmin && knt < 20);
              xnorm = warp_nrm2_smem(vs, len, lane);
              beta = -copysign(lapy2(alpha, xnorm), alpha);
            }
            tau = (beta - alpha) / beta;
            scal = T(1) / (alpha - beta);
            for (int q = 0; q < knt; ++q) beta *= safmin;
          }
        }
        if (lane == 0) {
          sh.tau = tau;
          sh.beta = beta;
          sh.scal = scal;
        }
      }
      __syncthreads();
      const T tau = sh.tau;
      if (tau != 0) {
        const T scal = sh.scal;
        for (int64_t i = threadIdx.x; i < len; i += NT) vs[i] *= scal;
      }
      __syncthreads();
      // the reflector goes back into column pvt only after the barrier that
      // ends this step: other CTAs may still be reading the column until then
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.tau[c] = tau;
        X.piv[c] = pvt;
        X.beta[c] = (double)sh.beta;
      }
      // ---- each warp: apply H(c) to its live columns, two at a time -----------
      // (loaded through L1: a warp's columns are written by that warp alone)
      auto dead = [&](int64_t t) {
        return (s_st[t * NW + wid] & ST_DONE) || gw + t * W == pvt;
      };
      int64_t t = 0;
      while (true) {
        while (t < ncol && dead(t)) ++t;
        if (t >= ncol) break;
        const int64_t ta = t++;
        while (t < ncol && dead(t)) ++t;
        const bool two = t < ncol;
        const int64_t tb = two ? t++ : ta;
        T* ca = A + (gw + ta * W) * lda;
        T* cb = A + (gw + tb * W) * lda;
        const T arca0 = ldown(ca + c);
        const T arcb0 = two ? ldown(cb + c) : T(0);
        T* ya = ca + c + 1;
        T* yb = cb + c + 1;
        T sa = 0, sb = 0;
        T xa[QCH], xb[QCH];
        if (tau != 0) {
          for (int64_t b0 = 0; b0 < len; b0 += 32 * QCH) {
            const int64_t rem = len - b0;
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              xa[q] = i < len ? ldown(ya + i) : T(0);
              xb[q] = (two && i < len) ? ldown(yb + i) : T(0);
            }
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              const T v = i < len ? vs[i] : T(0);
              sa = fma(v, xa[q], sa);
              sb = fma(v, xb[q], sb);
            }
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          sa += __shfl_xor_sync(0xffffffffu, sa, o);
          sb += __shfl_xor_sync(0xffffffffu, sb, o);
        }
        const T fa = tau * (arca0 + sa);
        const T fb = two ? tau * (arcb0 + sb) : T(0);
        if (fa != 0 || fb != 0) {
          for (int64_t b0 = 0; b0 < len; b0 += 32 * QCH) {
            const int64_t rem = len - b0;
            if (len > 32 * QCH) {
#pragma unroll
              for (int q = 0; q < QCH; ++q) {
                if (q % QG == 0 && 32 * q >= rem) break;
                const int64_t i = b0 + lane + 32 * q;
                xa[q] = i < len ? ldown(ya + i) : T(0);
                xb[q] = (two && i < len) ? ldown(yb + i) : T(0);
              }
            }
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              if (i < len) {
                const T v = vs[i];
                if (fa != 0) ya[i] = xa[q] - fa * v;
                if (two && fb != 0) yb[i] = xb[q] - fb * v;
              }
            }
          }
        }
        if (lane == 0) {
          const T arca = arca0 - fa;
          ca[c] = arca;
          s_arc[ta * NW + wid] = arca;
          if (two) {
            const T arcb = arcb0 - fb;
            cb[c] = arcb;
            s_arc[tb * NW + wid] = arcb;
          }
        }
      }
      __syncthreads();
      // ---- a thread per slot: norm downdate and the pivot candidate -----------
      bk = -2;
      bi = INT64_MAX;
      int myflag = 0;
      for (int s = threadIdx.x; s < nslot; s += NT) {
        const unsigned char st = s_st[s];
        if (!(st & ST_LIVE) || (st & ST_DONE)) continue;
        const int64_t jj = slot_col(s);
        if (jj == pvt) {
          s_st[s] = st | ST_DONE;
          continue;
        }
        if (!P.pivot) continue;
        T v1 = s_vn1[s];
        if (c < lastrk - 1 && v1 != 0) {
          T temp = fabs(s_arc[s]) / v1;
          temp = fmax(T(0), (T(1) + temp) * (T(1) - temp));
          const T r = v1 / s_vn2[s];
          const T temp2 = temp * r * r;
          if (temp2 <= tol3z) {
            myflag = 1;
            s_st[s] = st | ST_FLAG;
          } else {
            v1 = v1 * sqrt(temp);
            s_vn1[s] = v1;
          }
        }
        key_merge(bk, bi, norm_key(v1), jj);
      }
      if (myflag) atomicAdd(lst, 1);
      publish(bk, bi);
      if (!grid_sync(P.bar)) return;
      if (blockIdx.x == 0) {
        if (tau != 0)
          for (int64_t i = threadIdx.x; i < len; i += NT) pc[c + 1 + i] = vs[i];
        if (threadIdx.x == 0) pc[c] = sh.beta;
      }
      stop_block = *((volatile int*)lst) != 0;
      pvt = reduce_pivot_key();  // its block reduction orders the writes above before vs is reloaded
      ++kk;
    }
    const int64_t kb = kk;
    const int64_t jn = j + kb;
    nfac = jn;
    if (stop_block) {
      // recompute the flagged partial norms over rows jn..m-1
      for (int64_t t = 0; t < ncol; ++t) {
        const int s = (int)(t * NW + wid);
        if (!(s_st[s] & ST_FLAG) || (s_st[s] & ST_DONE)) continue;
        const T v1 = warp_nrm2(A + (gw + t * W) * lda + jn, m - jn, lane);
        __syncwarp();
        if (lane == 0) {
          s_vn1[s] = s_vn2[s] = v1;
          s_st[s] = s_st[s] & (unsigned char)~ST_FLAG;
        }
      }
      __syncthreads();
      bk = -2;
      bi = INT64_MAX;
      for (int s = threadIdx.x; s < nslot; s += NT) {
        const unsigned char st = s_st[s];
        if (!(st & ST_LIVE) || (st & ST_DONE)) continue;
        key_merge(bk, bi, norm_key(s_vn1[s]), slot_col(s));
      }
      publish(bk, bi);
      if (!grid_sync(P.bar)) return;
      pvt = reduce_pivot_key();
    }
    // rank test of geqp3_adap_main! (src/pqr.jl:407-415): R(i, i) lives in
    // row i of the pivot column piv[i]
    auto rdiag = [&](int64_t i) { return fabs(__ldcg(X.beta + i)); };
    if (rdiag(jn - 1) <= ptol) {
      bool found = false;
      for (int64_t i = j; i < jn; ++i) {
        if (rdiag(i) <= ptol) {
          kres = i;
          found = true;
          break;
        }
      }
      if (found) break;
    }
    j = jn;
    par ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *P.k_out = kres;
    *X.nfac = nfac;
  }
}

// ---- double-float variant for the mixed-precision path -----------------------------
// The sketch is held as pairs of floats, x = h + l with |l| <= ulp(h) / 2
// (48 significant bits, the resolution of the tensor-core sketch that
// produced it), at one power-of-two scale for the whole matrix.  The dot
// products and rank-1 updates, which dominate the factorization, run as
// compensated FP32 arithmetic (error-free products by FMA, two-sum
// accumulation) on the FP32 pipes, 64x wider than FP64 on this part; pivot
// decisions, norm downdates and the reflector scalars stay in FP64.

struct QrDf {
  float* Bh;            // high parts, ld = lda of the params
  float* Bl;            // low parts
  const double* vn0;    // initial column norms (scaled)
  const double* scale;  // 2^-E: the factorization sees B * scale
  unsigned long long* stamps;  // LRA_TRACE: %globaltimer at 8 points of each pivot (CTA 0), or null
};


template <int NT>
__global__ void __launch_bounds__(NT) geqp3_df_kernel(QrParams<double> P, QrV2Extra X, QrDf D) {
  __shared__ QrShared<double> sh;
  __shared__ Df s_f;  // reflector scale / tau / beta in df form
  __shared__ Df s_tau;
  __shared__ Df s_beta;
  extern __shared__ unsigned char qr_dyn[];
  constexpr int NW = NT / 32;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t gw = (int64_t)blockIdx.x * NW + wid;
  const int64_t W = (int64_t)gridDim.x * NW;
  const int64_t m = P.m, n = P.n, lda = P.lda;
  auto ldown = [](const float* p) { return *p; };
  auto stamp = [&](int64_t c, int ph) {
    if (D.stamps && blockIdx.x == 0 && threadIdx.x == 0 && c < P.kmax) D.stamps[c * 16 + ph] = globaltimer_ns();
  };
  float* __restrict__ Bh = D.Bh;
  float* __restrict__ Bl = D.Bl;
  const double tol3z = sqrt(Real<double>::eps);
  const int64_t lastrk = m < n ? m : n;
  const int64_t ncol = gw < n ? (n - 1 - gw) / W + 1 : 0;
  const int64_t ncmax = (n + W - 1) / W;
  const int nslot = (int)(ncmax * NW);
  float* vh = reinterpret_cast<float*>(qr_dyn);
  float* vl = vh + P.vcap;
  Df* s_vn1 = reinterpret_cast<Df*>(vl + P.vcap);
  Df* s_vn2 = s_vn1 + nslot;
  Df* s_arc = s_vn2 + nslot;
  unsigned char* s_st = reinterpret_cast<unsigned char*>(s_arc + nslot);
  auto slot_col = [&](int s) -> int64_t {
    return (int64_t)blockIdx.x * NW + (s % NW) + (int64_t)(s / NW) * W;
  };
  // warp 0 alone reduces the per-CTA candidates; one block barrier
  __shared__ int s_lst;
  auto reduce_pivot_key = [&](const int* lstp = nullptr) -> int64_t {
    if (wid == 0) {
      if (lane == 0 && lstp) s_lst = *((const volatile int*)lstp);
      long long k = -2;
      int64_t i = INT64_MAX;
      for (int b = lane; b < gridDim.x; b += 32) key_merge(k, i, __ldcg(X.part_k + b), __ldcg(P.part_i + b));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
        const int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
        key_merge(k, i, k2, i2);
      }
      if (lane == 0) sh.si[0] = i;
    }
    __syncthreads();
    const int64_t r = sh.si[0];
    return r;
  };
  auto publish = [&](long long k, int64_t i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long k2 = __shfl_xor_sync(0xffffffffu, k, o);
      const int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
      key_merge(k, i, k2, i2);
    }
    __syncthreads();
    if (lane == 0) {
      sh.sk[wid] = k;
      sh.si[wid] = i;
    }
    __syncthreads();
    if (wid == 0) {
      long long k0 = lane < NW ? sh.sk[lane] : -2;
      int64_t i0 = lane < NW ? sh.si[lane] : INT64_MAX;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const long long k2 = __shfl_xor_sync(0xffffffffu, k0, o);
        const int64_t i2 = __shfl_xor_sync(0xffffffffu, i0, o);
        key_merge(k0, i0, k2, i2);
      }
      if (lane == 0) {
        X.part_k[blockIdx.x] = k0;
        P.part_i[blockIdx.x] = i0;
      }
    }
  };
  // 2-norm of a column segment held as (h, l), by one warp, in FP64
  auto warp_nrm2_df = [&](const float* h, const float* l, int64_t len) -> double {
    double mx = 0;
    for (int64_t i = lane; i < len; i += 32) mx = fmax(mx, fabs(df_val(__ldcg(h + i), __ldcg(l + i))));
    mx = warp_max(mx);
    if (mx == 0 || !isfinite(mx)) return mx;
    const double sc = pow2_scale_inv(mx);
    double acc = 0;
    for (int64_t i = lane; i < len; i += 32) {
      const double t = df_val(__ldcg(h + i), __ldcg(l + i)) * sc;
      acc = fma(t, t, acc);
    }
    acc = warp_sum(acc);
    return sqrt(acc) / sc;
  };

  // ---- initial column norms (precomputed), ptol, first pivot ---------------
  for (int s = threadIdx.x; s < nslot; s += NT) {
    const int64_t j = slot_col(s);
    s_st[s] = j < n ? ST_LIVE : 0;
    const Df nr = (j < n && P.pivot) ? df_split(D.vn0[j]) : Df{0.f, 0.f};
    s_vn1[s] = s_vn2[s] = nr;
  }
  __syncthreads();
  double lmax = 0;
  long long bk = -2;
  int64_t bi = INT64_MAX;
  for (int s = threadIdx.x; s < nslot; s += NT)
    if (s_st[s] & ST_LIVE) {
      lmax = fmax(lmax, D.vn0[slot_col(s)]);
      key_merge(bk, bi, df_key(s_vn1[s]), slot_col(s));
    }
  lmax = block_max(lmax, sh.red);
  publish(bk, bi);
  if (threadIdx.x == 0) P.part_d[blockIdx.x] = lmax;
  if (!grid_sync(P.bar)) return;
  double maxnrm = 0;
  for (int b = threadIdx.x; b < gridDim.x; b += blockDim.x) maxnrm = fmax(maxnrm, __ldcg(P.part_d + b));
  maxnrm = block_max(maxnrm, sh.red);
  const double ptol = fmax(P.atol * *D.scale, P.rtol * maxnrm);
  int64_t pvt = reduce_pivot_key();

  int64_t kres = P.kmax, nfac = 0;
  int64_t j = 0;
  int par = 0;
  while (j < P.kmax) {
    const int64_t jb = min(P.nb, P.kmax - j);
    int* lst = P.lsticc + par;
    if (blockIdx.x == 0 && threadIdx.x == 0) P.lsticc[par ^ 1] = 0;
    int64_t kk = 0;
    bool stop_block = false;
    while (kk < jb && !stop_block) {
      const int64_t c = j + kk;
      if (!P.pivot) pvt = c;
      stamp(c, 0);
      // ---- every CTA: the reflector of column pvt, rows c..m-1 ---------------
      const int64_t len = m - c - 1;
      const float* ph = Bh + pvt * lda;
      const float* pl = Bl + pvt * lda;
      for (int64_t i = threadIdx.x; i < len; i += NT) {
        vh[i] = __ldcg(ph + c + 1 + i);
        vl[i] = __ldcg(pl + c + 1 + i);
      }
      __shared__ Df s_alpha;
      if (threadIdx.x == 0) s_alpha = Df{__ldcg(ph + c), __ldcg(pl + c)};
      __syncthreads();
      stamp(c, 1);
      if (wid == 0) {
        // xLARFG in double-float: beta = -sign(alpha) sqrt(alpha^2 + |x|^2),
        // tau = (beta - alpha) / beta, x <- x / (alpha - beta).  The matrix
        // is scaled to max |B| < 1, so no intermediate overflows, and the
        // rescaling loop of xLARFG (|beta| < safmin / eps, i.e. entries below
        // 2^-970) cannot arise: a float pair holds nothing below 2^-149.
        const Df alpha = s_alpha;
        Df acc{0.f, 0.f};
        for (int64_t i = lane; i < len; i += 32) df_fma_acc(acc, vh[i], vl[i], vh[i], vl[i]);
        acc = quick_two_sum(acc.h, acc.l);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = df_add(acc, df_shfl_xor(acc, o));
        Df tau{0.f, 0.f}, beta = alpha, scal{1.f, 0.f};
        if (len > 0 && acc.h > 0.f) {
          const Df r = df_sqrt(df_add(df_mul(alpha, alpha), acc));
          beta = alpha.h >= 0.f ? df_neg(r) : r;
          tau = df_div(df_add(beta, df_neg(alpha)), beta);
          scal = df_div(Df{1.f, 0.f}, df_add(alpha, df_neg(beta)));
        }
        if (lane == 0) {
          sh.tau = df_val(tau.h, tau.l);
          sh.beta = df_val(beta.h, beta.l);
          s_f = scal;
          s_tau = tau;
          s_beta = beta;
        }
      }
      __syncthreads();
      stamp(c, 2);
      const double tau = sh.tau;
      if (tau != 0) {
        const Df sc = s_f;
        for (int64_t i = threadIdx.x; i < len; i += NT) {
          const Df y = df_mul(Df{vh[i], vl[i]}, sc);
          vh[i] = y.h;
          vl[i] = y.l;
        }
      }
      __syncthreads();
      // the reflector goes back into column pvt only after the barrier that
      // ends this step: other CTAs may still be reading the column until then
      if (blockIdx.x == 0 && threadIdx.x == 0) {
        P.tau[c] = tau;
        X.piv[c] = pvt;
        X.beta[c] = sh.beta;
      }
      stamp(c, 3);
      const Df tdf = s_tau;
      // ---- each warp: apply H(c) to its live columns, two at a time -----------
      // A warp's columns are read and written by that warp alone, so they
      // are loaded through L1: a CTA's columns fit there for sketches of up
      // to a few hundred rows, and a hit costs tens of cycles, not an L2
      // round trip.  (The pivot column, written by another SM, is read
      // around L1 above.)
      auto dead = [&](int64_t t) {
        return (s_st[t * NW + wid] & ST_DONE) || gw + t * W == pvt;
      };
      int64_t t = 0;
      int pass = 0;
      while (true) {
        while (t < ncol && dead(t)) ++t;
        if (t >= ncol) break;
        const int64_t ta = t++;
        while (t < ncol && dead(t)) ++t;
        const bool two = t < ncol;
        const int64_t tb = two ? t++ : ta;
        const int64_t ja = gw + ta * W, jbb = gw + tb * W;
        float* ah = Bh + ja * lda;
        float* al = Bl + ja * lda;
        float* bh = Bh + jbb * lda;
        float* bl = Bl + jbb * lda;
        const Df arca0{ldown(ah + c), ldown(al + c)};
        const Df arcb0 = two ? Df{ldown(bh + c), ldown(bl + c)} : Df{0.f, 0.f};
        Df sa{0.f, 0.f}, sb{0.f, 0.f};
        float xah[QCH], xal[QCH], xbh[QCH], xbl[QCH];
        const int64_t o = c + 1;
        if (tau != 0) {
          for (int64_t b0 = 0; b0 < len; b0 += 32 * QCH) {
            const int64_t rem = len - b0;
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              const bool in = i < len;
              xah[q] = in ? ldown(ah + o + i) : 0.f;
              xal[q] = in ? ldown(al + o + i) : 0.f;
              xbh[q] = (two && in) ? ldown(bh + o + i) : 0.f;
              xbl[q] = (two && in) ? ldown(bl + o + i) : 0.f;
            }
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              const float wh = i < len ? vh[i] : 0.f, wl = i < len ? vl[i] : 0.f;
              df_fma_acc(sa, wh, wl, xah[q], xal[q]);
              if (two) df_fma_acc(sb, wh, wl, xbh[q], xbl[q]);
            }
          }
        }
        if (pass < 2) stamp(c, 8 + 3 * pass);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          sa = df_add(sa, df_shfl_xor(sa, off));
          sb = df_add(sb, df_shfl_xor(sb, off));
        }
        const Df fa = df_mul(tdf, df_add(arca0, sa));
        const Df fb = two ? df_mul(tdf, df_add(arcb0, sb)) : Df{0.f, 0.f};
        if (pass < 2) stamp(c, 9 + 3 * pass);
        const bool ua = fa.h != 0.f, ub = two && fb.h != 0.f;
        if (ua || ub) {
          for (int64_t b0 = 0; b0 < len; b0 += 32 * QCH) {
            const int64_t rem = len - b0;
            if (len > 32 * QCH) {
#pragma unroll
              for (int q = 0; q < QCH; ++q) {
                if (q % QG == 0 && 32 * q >= rem) break;
                const int64_t i = b0 + lane + 32 * q;
                const bool in = i < len;
                xah[q] = in ? ldown(ah + o + i) : 0.f;
                xal[q] = in ? ldown(al + o + i) : 0.f;
                xbh[q] = (two && in) ? ldown(bh + o + i) : 0.f;
                xbl[q] = (two && in) ? ldown(bl + o + i) : 0.f;
              }
            }
#pragma unroll
            for (int q = 0; q < QCH; ++q) {
              if (q % QG == 0 && 32 * q >= rem) break;
              const int64_t i = b0 + lane + 32 * q;
              if (i < len) {
                const float wh = vh[i], wl = vl[i];
                if (ua) {
                  const Df y = df_axpy_neg(xah[q], xal[q], fa, wh, wl);
                  ah[o + i] = y.h;
                  al[o + i] = y.l;
                }
                if (ub) {
                  const Df y = df_axpy_neg(xbh[q], xbl[q], fb, wh, wl);
                  bh[o + i] = y.h;
                  bl[o + i] = y.l;
                }
              }
            }
          }
        }
        if (pass < 2) stamp(c, 10 + 3 * pass);
        ++pass;
        if (lane == 0) {
          const Df arca = df_add(arca0, Df{-fa.h, -fa.l});
          ah[c] = arca.h;
          al[c] = arca.l;
          s_arc[ta * NW + wid] = arca;
          if (two) {
            const Df arcb = df_add(arcb0, Df{-fb.h, -fb.l});
            bh[c] = arcb.h;
            bl[c] = arcb.l;
            s_arc[tb * NW + wid] = arcb;
          }
        }
      }
      __syncthreads();
      stamp(c, 4);
      // ---- a thread per slot: norm downdate and the pivot candidate -----------
      bk = -2;
      bi = INT64_MAX;
      int myflag = 0;
      for (int s = threadIdx.x; s < nslot; s += NT) {
        const unsigned char st = s_st[s];
        if (!(st & ST_LIVE) || (st & ST_DONE)) continue;
        const int64_t jj = slot_col(s);
        if (jj == pvt) {
          s_st[s] = st | ST_DONE;
          continue;
        }
        if (!P.pivot) continue;
        Df v1 = s_vn1[s];
        if (c < lastrk - 1 && v1.h != 0.f) {
          // LAPACK's partial-norm downdate, in double-float
          const Df a = s_arc[s];
          Df temp = df_div(a.h < 0.f ? df_neg(a) : a, v1);
          temp = df_mul(df_add(Df{1.f, 0.f}, temp), df_add(Df{1.f, 0.f}, df_neg(temp)));
          if (temp.h < 0.f) temp = Df{0.f, 0.f};
          const Df r = df_div(v1, s_vn2[s]);
          const Df temp2 = df_mul(temp, df_mul(r, r));
          if (temp2.h <= (float)tol3z) {
            myflag = 1;
            s_st[s] = st | ST_FLAG;
          } else {
            v1 = df_mul(v1, df_sqrt(temp));
            s_vn1[s] = v1;
          }
        }
        key_merge(bk, bi, df_key(v1), jj);
      }
      if (myflag) atomicAdd(lst, 1);
      stamp(c, 5);
      publish(bk, bi);
      stamp(c, 6);
      if (!grid_sync(P.bar)) return;
      stamp(c, 7);
      if (blockIdx.x == 0) {
        float* wh = Bh + pvt * lda;
        float* wl = Bl + pvt * lda;
        if (tau != 0)
          for (int64_t i = threadIdx.x; i < len; i += NT) {
            wh[c + 1 + i] = vh[i];
            wl[c + 1 + i] = vl[i];
          }
        if (threadIdx.x == 0) {
          wh[c] = s_beta.h;
          wl[c] = s_beta.l;
        }
      }
      pvt = reduce_pivot_key(lst);  // its block barrier also orders the writes above before vs is reloaded
      stop_block = s_lst != 0;
      ++kk;
    }
    const int64_t kb = kk;
    const int64_t jn = j + kb;
    nfac = jn;
    if (stop_block) {
      for (int64_t t = 0; t < ncol; ++t) {
        const int s = (int)(t * NW + wid);
        if (!(s_st[s] & ST_FLAG) || (s_st[s] & ST_DONE)) continue;
        const int64_t jj = gw + t * W;
        const Df v1 = df_split(warp_nrm2_df(Bh + jj * lda + jn, Bl + jj * lda + jn, m - jn));
        __syncwarp();
        if (lane == 0) {
          s_vn1[s] = s_vn2[s] = v1;
          s_st[s] = s_st[s] & (unsigned char)~ST_FLAG;
        }
      }
      __syncthreads();
      bk = -2;
      bi = INT64_MAX;
      for (int s = threadIdx.x; s < nslot; s += NT) {
        const unsigned char st = s_st[s];
        if (!(st & ST_LIVE) || (st & ST_DONE)) continue;
        key_merge(bk, bi, df_key(s_vn1[s]), slot_col(s));
      }
      publish(bk, bi);
      if (!grid_sync(P.bar)) return;
      pvt = reduce_pivot_key();
    }
    auto rdiag = [&](int64_t i) { return fabs(__ldcg(X.beta + i)); };
    if (rdiag(jn - 1) <= ptol) {
      bool found = false;
      for (int64_t i = j; i < jn; ++i) {
        if (rdiag(i) <= ptol) {
          kres = i;
          found = true;
          break;
        }
      }
      if (found) break;
    }
    j = jn;
    par ^= 1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *P.k_out = kres;
    *X.nfac = nfac;
  }
}

// ---- shared-memory-resident double-float variant ------------------------------
// When a CTA's share of the sketch fits in shared memory the columns never
// leave the SM: CTA b owns the contiguous columns [n b / G, n (b + 1) / G),
// held as (h, l) float pairs, and applies every reflector to them there.
// The only traffic between CTAs per pivot is one 64-bit word per CTA and
// the winning candidate's column: each CTA stages its best candidate's
// remaining rows in global memory, then publishes (norm key, column, stop
// flag, sequence bit) as one word.  Readers poll the G words of the
// exchange (one L2 round trip once they are written), take the argmax and
// load the winner's staged rows; this replaces the grid barrier and the
// separate read of the per-CTA partials.  Words and staged columns are
// double-buffered by exchange parity, so a CTA that runs ahead never
// overwrites what a slower CTA still reads, and the sequence bit tells
// this exchange from the one two steps earlier.  The key keeps the 38
// leading bits of the double-float norm (relative resolution 2^-30, far
// below the error of the downdated norms); ties go to the smaller column
// index, as with xLAQPS's idamax.
struct QrSm {
  // the exchange, zeroed before the launch: exchange e's largest word in
  // amax[(e % 4) * 16] and OR of stop flags in astop[(e % 4) * 32] (a 128-byte
  // line each), and one arrival counter (G per exchange)
  unsigned long long* amax;
  unsigned* astop;
  unsigned* arrive;
  void* stage;               // [2][G][m] staged candidate columns (elements of the arithmetic)
  unsigned long long* pubt;  // LRA_TRACE: %globaltimer of each CTA's word per pivot, [kmax][G], or null
  // several adaptive steps factored by one launch: the lowest index of a
  // step whose rank came out below its threshold (k < nt), shared by the
  // launch's steps, or null; a step whose index is higher stops at its next
  // exchange
  int* success = nullptr;
  int job = 0;
  int64_t nt = 0;
};

// the next four live slots s, s + step, ... of a warp (-1: absent); s moves on
__device__ __forceinline__ int live_quad(const unsigned char* st, int nloc, int step, int& s, int (&q)[4]) {
  int cnt = 0;
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    while (s < nloc && (st[s] & ST_DONE)) s += step;
    if (s < nloc) {
      q[g] = s;
      ++cnt;
      s += step;
    } else {
      q[g] = -1;
    }
  }
  return cnt;
}

constexpr unsigned long long XW_IDX = 0xFFFFFFull;  // 24-bit column field, stored as XW_IDX - j
constexpr unsigned long long XW_LOW = (1ull << 62) - 1;
// the word of a CTA that stops a cancelled step: above every candidate's
// (a finite norm's key stays below 2^38 - 1), so every CTA of the step sees
// it at the same exchange
constexpr unsigned long long XW_CANCEL = XW_LOW;

// The arithmetic of the shared-memory pivoted QR.  Float64 sketches are
// held as double-float pairs (the mixed path's sketch has 2^-48
// resolution); Float32 sketches as plain FP32, the precision of xLAQPS for
// Float32.  Both give the step the same operations in the same order.
struct QrArithDf {
  using T = double;
  using E = float2;  // a stored element
  using V = Df;      // a working value
  __device__ static V zero() { return Df{0.f, 0.f}; }
  __device__ static V one() { return Df{1.f, 0.f}; }
  __device__ static E ezero() { return make_float2(0.f, 0.f); }
  __device__ static V ld(E e) { return Df{e.x, e.y}; }
  __device__ static E st(V v) { return make_float2(v.h, v.l); }
  __device__ static float hi(V v) { return v.h; }
  __device__ static float ehi(E e) { return e.x; }
  __device__ static void fma_acc(V& a, E v, E x) { df_fma_acc(a, v.x, v.y, x.x, x.y); }
  __device__ static V norm(V a) { return quick_two_sum(a.h, a.l); }
  __device__ static V add(V a, V b) { return df_add(a, b); }
  __device__ static V mul(V a, V b) { return df_mul(a, b); }
  __device__ static V div(V a, V b) { return df_div(a, b); }
  __device__ static V sqrt_(V a) { return df_sqrt(a); }
  __device__ static V neg(V a) { return df_neg(a); }
  __device__ static V shfl_xor(V a, int o) { return df_shfl_xor(a, o); }
  __device__ static E axpy_neg(E x, V f, E v) {
    const Df y = df_axpy_neg(x.x, x.y, f, v.x, v.y);
    return make_float2(y.h, y.l);
  }
  __device__ static double val(V v) { return df_val(v.h, v.l); }
  __device__ static V split(double x) { return df_split(x); }
  __device__ static E escale(E e, float sc) { return make_float2(e.x * sc, e.y * sc); }
  __device__ static V from_float(float f) { return Df{f, 0.f}; }
  __device__ static V ldexp_(V v, int ex) { return Df{ldexpf(v.h, ex), ldexpf(v.l, ex)}; }
  __device__ static E from_planes(const float* h, const float* l, int64_t i) { return make_float2(h[i], l[i]); }
  __device__ static void to_planes(E y, float* h, float* l, int64_t i) {
    h[i] = y.x;
    l[i] = y.y;
  }
  // 38 bits of the key (df_key < 2^63 for h > 0); zero, negative zero and
  // NaN norms rank lowest
  __device__ static unsigned long long key38(V v) { return v.h > 0.f ? (unsigned long long)df_key(v) >> 25 : 0ull; }
};

struct QrArithF32 {
  using T = float;
  using E = float;
  using V = float;
  __device__ static V zero() { return 0.f; }
  __device__ static V one() { return 1.f; }
  __device__ static E ezero() { return 0.f; }
  __device__ static V ld(E e) { return e; }
  __device__ static E st(V v) { return v; }
  __device__ static float hi(V v) { return v; }
  __device__ static float ehi(E e) { return e; }
  __device__ static void fma_acc(V& a, E v, E x) { a = fmaf(v, x, a); }
  __device__ static V norm(V a) { return a; }
  __device__ static V add(V a, V b) { return a + b; }
  __device__ static V mul(V a, V b) { return a * b; }
  __device__ static V div(V a, V b) { return a / b; }
  __device__ static V sqrt_(V a) { return a > 0.f ? sqrtf(a) : 0.f; }
  __device__ static V neg(V a) { return -a; }
  __device__ static V shfl_xor(V a, int o) { return __shfl_xor_sync(0xffffffffu, a, o); }
  __device__ static E axpy_neg(E x, V f, E v) { return fmaf(-f, v, x); }
  __device__ static double val(V v) { return (double)v; }
  __device__ static V split(double x) { return (float)x; }
  __device__ static E escale(E e, float sc) { return e * sc; }
  __device__ static V from_float(float f) { return f; }
  __device__ static V ldexp_(V v, int ex) { return ldexpf(v, ex); }
  __device__ static E from_planes(const float* h, const float*, int64_t i) { return h[i]; }
  __device__ static void to_planes(E y, float* h, float*, int64_t i) { h[i] = y; }
  // the 31 bits of a positive float, at the place of the double-float
  // key's 38 bits
  __device__ static unsigned long long key38(V v) { return v > 0.f ? (unsigned long long)__float_as_uint(v) << 6 : 0ull; }
};

template <class A>
__device__ __forceinline__ unsigned long long xw_pack(typename A::V v, int64_t j) {
  return (A::key38(v) << 24) | (XW_IDX - (unsigned long long)j);
}


// Warp 0 computes the reflector's scalars while warps 1..NW-1 take the dot
// products of their columns with the (unscaled) reflector tail x; with
// v = [1; scal x] the update of column a is f = tau (a_c + scal (x . a)),
// a_c -= f, a_i -= (f scal) x_i.  A warp takes its columns four at a time:
// one load of x serves four accumulators, and the four dot products are
// reduced together (each butterfly level halves the values a lane holds, so
// the four totals cost about as much as one).  The pivot search needs only
// row c of each column (the norm downdate), so the rank-1 update of rows
// c+1..m-1 is deferred: the CTA updates its candidate column (which it
// stages) and any column whose norm must be recomputed right away, and the
// other columns while warp 0 waits for the exchange.
//
// The same step runs with the columns in global memory for a whole matrix
// per CTA (GCOL): the batched path gives each small matrix one CTA, which
// needs no exchange at all.  Every column sees the same sequence of
// operations in both forms (the dot products' lane order and reduction tree,
// the reflector's partial sums over the same thread-to-row map, the same
// updates), so a matrix factored alone and in a batch gives the same bits.
template <class A, int NT, bool GCOL>
__device__ __forceinline__ void geqp3_df_body(const QrParams<typename A::T>& P, const QrV2Extra& X, const QrDf& D,
                                              const QrSm& S, const int G, const int b, typename A::E* Cg,
                                              const int64_t gcs, const int64_t grs, unsigned char* qr_dyn) {
  using E = typename A::E;
  using V = typename A::V;
  constexpr int NW = NT / 32;
  constexpr int NCW = NW - 1;  // column warps
  __shared__ V s_part[NW];
  __shared__ unsigned long long s_w[NW];
  __shared__ int s_fl[NW];
  __shared__ V s_alpha, s_f, s_tau, s_beta;
  __shared__ double s_red[32];
  __shared__ unsigned long long s_win;
  __shared__ int s_owner, s_stop, s_ok, s_cancel;
  __shared__ double s_taud, s_betad;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t m = P.m, n = P.n, lda = P.lda;
  const int64_t c0 = n * b / G, c1 = n * (b + 1) / G;
  const int nloc = (int)(c1 - c0);
  const int64_t ncap = (n + G - 1) / G;
  E* Vc = reinterpret_cast<E*>(qr_dyn);  // rows c..m-1 of the pivot column
  // the CTA's columns, slot s = column c0 + s: shared memory, or (GCOL) a
  // global m x n workspace
  E* C = GCOL ? Cg : Vc + m;
  // element (row i, slot s) at C[s cs + i rs]: column-major in shared
  // memory; the workspace of GCOL may be row-major (coalesced thread-per-
  // column access)
  const int64_t cs = GCOL ? gcs : m, rs = GCOL ? grs : 1;
  V* s_vn1 = reinterpret_cast<V*>(GCOL ? Vc + m : C + ncap * m);
  V* s_vn2 = s_vn1 + ncap;
  V* s_dot = s_vn2 + ncap;
  V* s_fs = s_dot + ncap;  // f scal of each column for the deferred update
  E* s_x0 = reinterpret_cast<E*>(s_fs + ncap);  // row c of each column
  unsigned char* s_st = reinterpret_cast<unsigned char*>(s_x0 + ncap);
  float* __restrict__ Bh = D.Bh;
  float* __restrict__ Bl = D.Bl;
  const float tol3z = (float)sqrt((double)Real<typename A::T>::eps);
  const int64_t lastrk = m < n ? m : n;
  // LRA_TRACE: a block barrier before each stamp, so that it marks the end
  // of the phase for the whole CTA
  auto stamp = [&](int64_t c, int ph) {
    if (!D.stamps) return;
    __syncthreads();
    if (b == 0 && threadIdx.x == 0 && c < P.kmax) D.stamps[c * 16 + ph] = globaltimer_ns();
  };
  // the CTA's candidate: max of the warps' words (s_w) and OR of their
  // stop flags (s_fl), into s_win / s_stop
  auto cta_word = [&]() {
    __syncthreads();
    if (wid == 0) {
      unsigned long long w0 = lane < NW ? s_w[lane] : 0ull;
      int f0 = lane < NW ? s_fl[lane] : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w2 = __shfl_xor_sync(0xffffffffu, w0, o);
        w0 = w2 > w0 ? w2 : w0;
        f0 |= __shfl_xor_sync(0xffffffffu, f0, o);
      }
      if (lane == 0) {
        s_win = w0;
        s_stop = f0;
      }
    }
    __syncthreads();
  };
  auto warp_word = [&](unsigned long long w, int fl) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long w2 = __shfl_xor_sync(0xffffffffu, w, o);
      w = w2 > w ? w2 : w;
      fl |= __shfl_xor_sync(0xffffffffu, fl, o);
    }
    if (lane == 0) {
      s_w[wid] = w;
      s_fl[wid] = fl;
    }
  };
  // stage the CTA's candidate (rows r0..m-1) and publish its word for
  // exchange e; the candidate's deferred update (upd) is applied on the way.
  // The word goes out after every thread's staged rows.
  auto publish = [&](unsigned e, int64_t r0, bool upd) {
    const bool cancel = !GCOL && s_cancel;
    const unsigned long long w = cancel ? XW_CANCEL : s_win;
    if (!cancel && (w & XW_LOW)) {
      const int sc = (int)((int64_t)(XW_IDX - (w & XW_IDX)) - c0);
      E* col = C + (int64_t)sc * cs;
      E* dst = GCOL ? nullptr : static_cast<E*>(S.stage) + ((size_t)(e & 1) * G + b) * m;
      const V fs = upd ? s_fs[sc] : A::zero();
      if (upd && !(s_st[sc] & ST_UPD) && A::hi(fs) != 0.f) {
        for (int64_t i = r0 + threadIdx.x; i < m; i += NT) {
          const E y = A::axpy_neg(col[i * rs], fs, Vc[i]);
          col[i * rs] = y;
          if (!GCOL) dst[i] = y;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_st[sc] |= ST_UPD;
      } else if (!GCOL) {
        for (int64_t i = r0 + threadIdx.x; i < m; i += NT) dst[i] = col[i];
      }
    }
    __syncthreads();
    if (!GCOL && threadIdx.x == 0) {
      // the word into the exchange's maximum (and the stop flag into its
      // OR), then the arrival, released after the staged rows
      __threadfence();
      if (S.pubt && r0 >= 1 && r0 - 1 < P.kmax) S.pubt[(r0 - 1) * G + b] = globaltimer_ns();
      const unsigned slot = e & 3;
      if (w & XW_LOW) atomicMax(S.amax + slot * 16, w & XW_LOW);
      if (!cancel && s_stop) atomicOr(S.astop + slot * 32, 1u);
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(S.arrive) : "memory");
    }
  };
  // wait for all G arrivals of exchange e (bounded): the winning word, its
  // CTA and the OR of the stop flags, in shared memory
  auto collect = [&](unsigned e) -> bool {
    if (GCOL) {
      // one CTA: its own candidate is the pivot
      if (threadIdx.x == 0) s_owner = 0;
      __syncthreads();
      return true;
    }
    if (threadIdx.x == 0) {
      // a lower step of the launch revealed its rank: this step stops at
      // the next exchange
      const int canc = S.success ? (*((volatile int*)S.success) < S.job ? 1 : 0) : 0;
      // every CTA's arrival at exchange e (the counter grows by G per
      // exchange), bounded
      const unsigned target = (unsigned)G * (e + 1u);
      bool ok = true;
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(S.arrive) : "memory");
      if ((int)(v - target) < 0) {
        const uint64_t t0 = globaltimer_ns(), lim = wait_limit_ns();
        for (unsigned it = 1;; ++it) {
          asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(S.arrive) : "memory");
          if ((int)(v - target) >= 0) break;
          // the error word and the clock every 16th poll
          if (it & 15) continue;
          if (*((volatile int*)&P.bar->err) != 0) {
            ok = false;
            break;
          }
          if (globaltimer_ns() - t0 > lim) {
            atomicCAS(&P.bar->err, 0, 4);
            ok = false;
            break;
          }
        }
      }
      const unsigned slot = e & 3;
      unsigned long long best;
      unsigned fl;
      asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(best) : "l"(S.amax + slot * 16) : "memory");
      asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(fl) : "l"(S.astop + slot * 32) : "memory");
      // every CTA has read exchange e - 1 (each read it before arriving at
      // e): its slot is cleared for exchange e + 3, before this CTA's next
      // arrival releases the clearing
      if (b == 0 && ok) {
        const unsigned prev = (e + 3) & 3;
        asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(S.amax + prev * 16), "l"(0ull) : "memory");
        asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(S.astop + prev * 32), "r"(0u) : "memory");
      }
      // the winner's CTA: the one whose columns [n b / G, n (b + 1) / G)
      // hold the winning column
      const int64_t jw = (int64_t)(XW_IDX - (best & XW_IDX));
      int own = 0;
      if ((best & XW_LOW) != 0 && best != XW_CANCEL) {
        own = (int)(((jw + 1) * (int64_t)G - 1) / n);
        own = own < 0 ? 0 : (own >= G ? G - 1 : own);
      }
      s_win = best;
      s_owner = own;
      s_stop = fl ? 1 : 0;
      s_ok = ok && best != XW_CANCEL ? 1 : 0;
      s_cancel = canc;
    }
    __syncthreads();
    return s_ok != 0;
  };
  auto quad = [&](int& s, int (&q)[4]) { return live_quad(s_st, nloc, NCW, s, q); };

  if (threadIdx.x == 0) s_cancel = 0;
  // ---- the CTA's columns into shared memory (GCOL: the workspace is filled);
  // initial norms, first pivot
  if (!GCOL)
    for (int s = wid; s < nloc; s += NW) {
      const float* ph = Bh + (c0 + s) * lda;
      const float* pl = Bl ? Bl + (c0 + s) * lda : nullptr;
      for (int64_t i = lane; i < m; i += 32) C[s * m + i] = A::from_planes(ph, pl, i);
    }
  double lmax = 0;
  unsigned long long cw = 0;
  for (int s = threadIdx.x; s < nloc; s += NT) {
    s_st[s] = ST_LIVE;
    const double v = D.vn0[c0 + s];
    const V nr = A::split(v);
    s_vn1[s] = s_vn2[s] = nr;
    lmax = fmax(lmax, v);
    const unsigned long long w = xw_pack<A>(nr, c0 + s);
    cw = w > cw ? w : cw;
  }
  lmax = block_max(lmax, s_red);
  if (!GCOL && threadIdx.x == 0) P.part_d[b] = lmax;
  warp_word(cw, 0);
  cta_word();
  unsigned e = 0;
  publish(e, 0, false);
  if (!collect(e)) return;
  double maxnrm = lmax;
  if (!GCOL) {
    maxnrm = 0;
    for (int bb = threadIdx.x; bb < G; bb += NT) maxnrm = fmax(maxnrm, __ldcg(P.part_d + bb));
    maxnrm = block_max(maxnrm, s_red);
  }
  const double ptol = fmax(P.atol * *D.scale, P.rtol * maxnrm);

  int64_t kres = P.kmax, nfac = 0;
  int64_t j = 0;
  while (j < P.kmax) {
    const int64_t jb = min(P.nb, P.kmax - j);
    int64_t kk = 0, first_small = -1;
    bool stop_block = false, last_small = false;
    while (kk < jb && !stop_block) {
      const int64_t c = j + kk;
      const int64_t pvt = (int64_t)(XW_IDX - (s_win & XW_IDX));
      const int owner = s_owner;
      stamp(c, 0);
      // the pivot column is done; the previous step's deferred-update marks
      // are cleared (a thread per slot, so each byte has one writer)
      for (int s = threadIdx.x; s < nloc; s += NT) {
        unsigned char st = (unsigned char)(s_st[s] & ~ST_UPD);
        if (owner == b && s == pvt - c0) st |= ST_DONE;
        s_st[s] = st;
      }
      // ---- the pivot column's rows c..m-1 from the winner's stage, and the
      // per-warp partial sums of squares of rows c+1..m-1
      {
        const E* src = GCOL ? C + (pvt - c0) * cs : static_cast<const E*>(S.stage) + ((size_t)(e & 1) * G + owner) * m;
        V acc = A::zero();
        for (int64_t i = c + threadIdx.x; i < m; i += NT) {
          const E x = GCOL ? src[i * rs] : __ldcg(src + i);
          Vc[i] = x;
          if (i > c) A::fma_acc(acc, x, x);
          else s_alpha = A::ld(x);
        }
        acc = A::norm(acc);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = A::add(acc, A::shfl_xor(acc, o));
        if (lane == 0) s_part[wid] = acc;
      }
      __syncthreads();
      stamp(c, 1);
      const int64_t len = m - c - 1;
      if (wid == 0) {
        // xLARFG in double-float (the matrix is scaled to max |B| < 1, so
        // neither the sum of squares nor beta can overflow, and no entry of
        // a float pair is small enough for xLARFG's rescaling loop)
        V acc = lane < NW ? s_part[lane] : A::zero();
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc = A::add(acc, A::shfl_xor(acc, o));
        const V alpha = s_alpha;
        V tau = A::zero(), beta = alpha, scal = A::one();
        if (len > 0 && A::hi(acc) > 0.f) {
          const V r = A::sqrt_(A::add(A::mul(alpha, alpha), acc));
          beta = A::hi(alpha) >= 0.f ? A::neg(r) : r;
          tau = A::div(A::add(beta, A::neg(alpha)), beta);
          scal = A::div(A::one(), A::add(alpha, A::neg(beta)));
        }
        if (lane == 0) {
          s_taud = A::val(tau);
          s_betad = A::val(beta);
          s_f = scal;
          s_tau = tau;
          s_beta = beta;
          if (b == 0) {
            P.tau[c] = (typename A::T)s_taud;
            X.piv[c] = pvt;
            X.beta[c] = s_betad;
          }
        }
      } else if (len > 0 && len <= P.seq_len) {
        // ---- short columns: a thread per column, the dot product summed
        // row by row (a lane-strided sum and its reduction tree cost more
        // than the products here).  The rule depends on len alone, so both
        // forms of the kernel sum each column the same way.
        for (int s = threadIdx.x - 32; s < nloc; s += NT - 32) {
          if (s_st[s] & ST_DONE) continue;
          const E* col = C + (int64_t)s * cs;
          s_x0[s] = col[c * rs];
          V d = A::zero();
          // QSEQB rows loaded ahead, then added in row order
          for (int64_t i0 = c + 1; i0 < m; i0 += QSEQB) {
            E xb[QSEQB];
#pragma unroll
            for (int r = 0; r < QSEQB; ++r)
              if (i0 + r < m) xb[r] = col[(i0 + r) * rs];
#pragma unroll
            for (int r = 0; r < QSEQB; ++r)
              if (i0 + r < m) A::fma_acc(d, Vc[i0 + r], xb[r]);
          }
          s_dot[s] = A::norm(d);
        }
      } else if (len > 0) {
        // ---- dot products x . a of the warp's live columns, four at a time
        int s = wid - 1;
        int q[4];
        while (quad(s, q)) {
          const E* cg[4];
#pragma unroll
          for (int g = 0; g < 4; ++g) cg[g] = C + (int64_t)(q[g] >= 0 ? q[g] : q[0]) * cs;
          // row c of the column, for the update that follows the dots
          {
            const int g = lane >> 3;
            const int qg = g == 0 ? q[0] : g == 1 ? q[1] : g == 2 ? q[2] : q[3];
            if ((lane & 7) == 0 && qg >= 0) s_x0[qg] = C[(int64_t)qg * cs + c * rs];
          }
          // QRPL rows per lane are loaded before they are used, so that a
          // quad has 4 QRPL loads in flight (the global-memory form waits
          // an L2 round trip per chunk); each lane still adds its rows in
          // increasing order
          V d[4] = {A::zero(), A::zero(), A::zero(), A::zero()};
          for (int64_t b0 = c + 1; b0 < m; b0 += 32 * QRPL) {
            E xv[QRPL], xc[4][QRPL];
#pragma unroll
            for (int r = 0; r < QRPL; ++r) {
              const int64_t i = b0 + lane + 32 * r;
              const bool in = i < m;
              xv[r] = in ? Vc[i] : A::ezero();
#pragma unroll
              for (int g = 0; g < 4; ++g) xc[g][r] = in ? cg[g][i * rs] : A::ezero();
            }
#pragma unroll
            for (int r = 0; r < QRPL; ++r)
              if (b0 + lane + 32 * r < m) {
#pragma unroll
                for (int g = 0; g < 4; ++g) A::fma_acc(d[g], xv[r], xc[g][r]);
              }
          }
#pragma unroll
          for (int g = 0; g < 4; ++g) d[g] = A::norm(d[g]);
          // transposed butterfly: after the 16- and 8-lane levels, lanes
          // 8g..8g+7 hold column g's partial sums
          const bool up = lane & 16;
          const V k0 = up ? d[2] : d[0], k1 = up ? d[3] : d[1];
          const V e0 = A::add(k0, A::shfl_xor(up ? d[0] : d[2], 16));
          const V e1 = A::add(k1, A::shfl_xor(up ? d[1] : d[3], 16));
          const bool hi = lane & 8;
          V t = A::add(hi ? e1 : e0, A::shfl_xor(hi ? e0 : e1, 8));
#pragma unroll
          for (int o = 4; o > 0; o >>= 1) t = A::add(t, A::shfl_xor(t, o));
          const int g = lane >> 3;
          const int qg = g == 0 ? q[0] : g == 1 ? q[1] : g == 2 ? q[2] : q[3];
          if ((lane & 7) == 0 && qg >= 0) s_dot[qg] = t;
        }
      }
      __syncthreads();
      stamp(c, 2);
      const double tau = s_taud;
      const V scal = s_f;
      stamp(c, 3);
      // ---- a thread per column: f, the new row c, the norm downdate and the
      // candidate word
      unsigned long long ww = 0;
      int wfl = 0;
      auto sub = [&](int ph) {
        if (D.stamps && b == 0 && threadIdx.x == 0 && c < P.kmax) D.stamps[c * 16 + ph] = globaltimer_ns();
      };
      sub(8);
      {
        const V tdf = s_tau;
        for (int s = threadIdx.x; s < nloc; s += NT) {
          const unsigned char st = s_st[s];
          if (st & ST_DONE) continue;
          const E x0 = len > 0 ? s_x0[s] : C[(int64_t)s * cs + c * rs];
          V f = A::zero(), fs = A::zero();
          if (tau != 0 && len > 0) {
            f = A::mul(tdf, A::add(A::ld(x0), A::mul(scal, s_dot[s])));
            fs = A::mul(f, scal);
          }
          s_fs[s] = fs;
          const V a = A::add(A::ld(x0), A::neg(f));
          C[(int64_t)s * cs + c * rs] = A::st(a);
          V v1 = s_vn1[s];
          bool flagged = false;
          if (c < lastrk - 1 && A::hi(v1) != 0.f) {
            // LAPACK's partial-norm downdate
            V temp = A::div(A::hi(a) < 0.f ? A::neg(a) : a, v1);
            temp = A::mul(A::add(A::one(), temp), A::add(A::one(), A::neg(temp)));
            if (A::hi(temp) < 0.f) temp = A::zero();
            const V r = A::div(v1, s_vn2[s]);
            const V temp2 = A::mul(temp, A::mul(r, r));
            if (A::hi(temp2) <= tol3z) {
              flagged = true;
            } else {
              v1 = A::mul(v1, A::sqrt_(temp));
              s_vn1[s] = v1;
            }
          }
          if (flagged) {
            // unreliable downdate: xLAQPS would end the block here and
            // recompute the norm before the next pivot, from the updated
            // column; a warp does that below
            s_st[s] = st | ST_FLAG;
            wfl = 1;
            continue;
          }
          const unsigned long long w = xw_pack<A>(v1, c0 + s);
          ww = w > ww ? w : ww;
        }
      }
      sub(9);
      sub(10);
      // ---- the flagged columns, a warp each: the deferred update of rows
      // c+1..m-1 now, then their norm in double-float at a power-of-two
      // scale that puts the largest entry in [1, 2) (lane-strided partial
      // sums and a butterfly, the same tree in both forms of the kernel)
      if (__syncthreads_or(wfl)) {
        sub(11);
        for (int s = wid; s < nloc; s += NW) {
          if (!(s_st[s] & ST_FLAG)) continue;
          E* col = C + (int64_t)s * cs;
          const V fs = s_fs[s];
          const bool upd = A::hi(fs) != 0.f;
          float mx = 0.f;
          for (int64_t i = c + 1 + lane; i < m; i += 32) {
            E y = col[i * rs];
            if (upd) {
              y = A::axpy_neg(y, fs, Vc[i]);
              col[i * rs] = y;
            }
            mx = fmaxf(mx, fabsf(A::ehi(y)));
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
          V nr = A::from_float(mx);
          if (mx > 0.f && isfinite(mx)) {
            const int ex = ilogbf(mx);
            const float sc = ldexpf(1.f, -ex);
            V acc = A::zero();
            for (int64_t i = c + 1 + lane; i < m; i += 32) {
              const E x = A::escale(col[i * rs], sc);
              A::fma_acc(acc, x, x);
            }
            acc = A::norm(acc);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc = A::add(acc, A::shfl_xor(acc, o));
            nr = A::ldexp_(A::sqrt_(acc), ex);
          }
          __syncwarp();
          if (lane == 0) {
            s_vn1[s] = s_vn2[s] = nr;
            s_st[s] = (unsigned char)((s_st[s] & ~ST_FLAG) | ST_UPD);
          }
          const unsigned long long w = xw_pack<A>(nr, c0 + s);
          ww = w > ww ? w : ww;
        }
        wfl = 1;
      } else {
        sub(11);
      }
      sub(12);
      warp_word(ww, wfl);
      sub(13);
      const bool small = fabs(s_betad) <= ptol;
      if (small && first_small < 0) first_small = c;
      last_small = small;
      cta_word();
      stamp(c, 4);
      publish(e + 1, c + 1, true);
      stamp(c, 5);
      ++e;
      // ---- warps 1..NW-1: the deferred updates, and the finished pivot column
      // to global memory (its owner); warp 0 meanwhile waits for the exchange
      if (wid > 0) {
        const int ct = threadIdx.x - 32;
        constexpr int NCT = NT - 32;
        // the finished pivot column (its owner): R's rows above c, beta, the
        // reflector v = scal x below
        if (owner == b) {
          E* col = C + (pvt - c0) * cs;
          const V bt = s_beta;
          for (int64_t i = (GCOL ? c : 0) + ct; i < m; i += NCT) {
            E y;
            if (i < c) {
              y = col[i * rs];
            } else if (i == c) {
              y = A::st(bt);
            } else {
              y = Vc[i];
              if (tau != 0) y = A::st(A::mul(A::ld(y), scal));
            }
            if (GCOL) {
              col[i * rs] = y;
            } else {
              A::to_planes(y, Bh + pvt * lda, Bl ? Bl + pvt * lda : nullptr, i);
            }
          }
        }
        // the rank-1 updates of rows c+1..m-1.  Shared-memory columns: a warp
        // per four columns, QRPL rows per lane in registers.  Global columns
        // (GCOL): a thread per column, whose rows stay in L1 between the
        // dot products and the update.
        if (!GCOL) {
          int s = wid - 1;
          int q[4];
          while (quad(s, q)) {
            V fq[4];
            E* cg[4];
            bool u[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const int qh = q[h] >= 0 ? q[h] : q[0];
              cg[h] = C + (int64_t)qh * cs;
              fq[h] = s_fs[qh];
              u[h] = q[h] >= 0 && A::hi(fq[h]) != 0.f && !(s_st[qh] & ST_UPD);
            }
            if (u[0] || u[1] || u[2] || u[3]) {
              for (int64_t b0 = c + 1; b0 < m; b0 += 32 * QRPL) {
                E xv[QRPL], xc[4][QRPL];
#pragma unroll
                for (int r = 0; r < QRPL; ++r) {
                  const int64_t i = b0 + lane + 32 * r;
                  const bool in = i < m;
                  xv[r] = in ? Vc[i] : A::ezero();
#pragma unroll
                  for (int h = 0; h < 4; ++h) xc[h][r] = (in && u[h]) ? cg[h][i * rs] : A::ezero();
                }
#pragma unroll
                for (int r = 0; r < QRPL; ++r) {
                  const int64_t i = b0 + lane + 32 * r;
                  if (i < m) {
#pragma unroll
                    for (int h = 0; h < 4; ++h)
                      if (u[h]) cg[h][i * rs] = A::axpy_neg(xc[h][r], fq[h], xv[r]);
                  }
                }
              }
            }
          }
        }
        if (GCOL) {
          for (int sl = ct; sl < nloc; sl += NCT) {
            if (s_st[sl] & (ST_DONE | ST_UPD)) continue;
            const V fs = s_fs[sl];
            if (A::hi(fs) == 0.f) continue;
            E* col = C + (int64_t)sl * cs;
            for (int64_t i0 = c + 1; i0 < m; i0 += QSEQB) {
              E xb[QSEQB];
#pragma unroll
              for (int r = 0; r < QSEQB; ++r)
                if (i0 + r < m) xb[r] = col[(i0 + r) * rs];
#pragma unroll
              for (int r = 0; r < QSEQB; ++r)
                if (i0 + r < m) col[(i0 + r) * rs] = A::axpy_neg(xb[r], fs, Vc[i0 + r]);
            }
          }
        }
      }
      if (!collect(e)) return;
      stamp(c, 6);
      stamp(c, 7);
      stop_block = s_stop != 0;
      ++kk;
    }
    const int64_t jn = j + kk;
    nfac = jn;
    // rank test of geqp3_adap_main! (src/pqr.jl:407-415): when R(jn-1, jn-1)
    // is below ptol, the rank is the first i of this block with |R(i, i)| <= ptol
    if (last_small) {
      kres = first_small;
      break;
    }
    j = jn;
  }
  // ---- the columns that were not pivots back to global memory ----------------
  for (int s = wid; s < nloc && !GCOL; s += NW) {
    if (s_st[s] & ST_DONE) continue;
    float* ph = Bh + (c0 + s) * lda;
    float* pl = Bl ? Bl + (c0 + s) * lda : nullptr;
    for (int64_t i = lane; i < m; i += 32) A::to_planes(C[(int64_t)s * m + i], ph, pl, i);
  }
  if (b == 0 && threadIdx.x == 0) {
    *P.k_out = kres;
    *X.nfac = nfac;
    if (S.success && kres < S.nt) atomicMin(S.success, S.job);
  }
}

// one sketch of a shared-memory launch: its parameters and its CTAs
// [off, off + G) of the grid
template <class A>
struct SmJob {
  QrParams<typename A::T> P;
  QrV2Extra X;
  QrDf D;
  QrSm S;
  int G, off;
};
constexpr int kSmJobs = 8;  // sketches per launch
template <class A>
struct SmJobs {
  SmJob<A> j[kSmJobs];
  int n;
};

// the sketches of a launch (one, or several adaptive steps at once), each
// factored by its own CTAs with its own exchange
template <class A, int NT>
__global__ void __launch_bounds__(NT, 1) geqp3_df_smem_kernel(const SmJobs<A> J) {
  extern __shared__ unsigned char qr_dyn[];
  // the CTA's sketch, copied from the parameters to shared memory once
  __shared__ __align__(16) unsigned char s_jb[sizeof(SmJob<A>)];
  int q = 0;
  while (q + 1 < J.n && (int)blockIdx.x >= J.j[q + 1].off) ++q;
  {
    const unsigned* src = reinterpret_cast<const unsigned*>(&J.j[q]);
    unsigned* dst = reinterpret_cast<unsigned*>(s_jb);
    for (int i = threadIdx.x; i < (int)(sizeof(SmJob<A>) / 4); i += NT) dst[i] = src[i];
  }
  __syncthreads();
  const SmJob<A>& job = *reinterpret_cast<const SmJob<A>*>(s_jb);
  geqp3_df_body<A, NT, false>(job.P, job.X, job.D, job.S, job.G, (int)blockIdx.x - job.off, nullptr, 0, 0, qr_dyn);
}

// one matrix of a batch: its parameters and its m x n float2 workspace
struct QrJob {
  QrParams<double> P;
  QrV2Extra X;
  QrDf D;
  float2* work;
  int64_t cs, rs;  // element (i, j) of the workspace at work[j cs + i rs]
};

// persistent grouped pivoted QR: each CTA takes the next matrix (jobs are
// ordered by decreasing work) and factors it alone
template <int NT>
__global__ void __launch_bounds__(NT, 1) geqp3_df_group_kernel(const QrJob* __restrict__ jobs, int njobs, int* next) {
  extern __shared__ unsigned char qr_dyn[];
  __shared__ int s_job;
  const QrSm S{nullptr, nullptr, nullptr};
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_job = atomicAdd(next, 1);
    __syncthreads();
    const int j = s_job;
    if (j >= njobs) return;
    geqp3_df_body<QrArithDf, NT, true>(jobs[j].P, jobs[j].X, jobs[j].D, S, 1, 0, jobs[j].work, jobs[j].cs,
                                       jobs[j].rs, qr_dyn);
  }
}

// ---- the batch's conversions ---------------------------------------------------
// prep: max |B| (its power-of-two scale as df_scale_kernel), the scaled
// float pairs into the workspace and each column's norm as df_split_kernel
// (the same per-warp arithmetic, so the norms agree bit for bit)
struct DfPrepJob {
  int64_t m, n, ldb;
  const double* B;
  float2* work;                // m x n, element (i, j) at work[j cs + i rs]
  int64_t cs, rs;
  double* vn0;                 // n
  double* scale;               // 1
  unsigned long long* maxbits;  // 1, zeroed: max |B| as the bits of a double
};

// CTAs (matrix, part): max |B| of every part's columns into maxbits
__global__ void __launch_bounds__(512) df_prep_max_kernel(const DfPrepJob* __restrict__ jobs) {
  __shared__ double red[32];
  const DfPrepJob J = jobs[blockIdx.x];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double mx = 0;
  for (int64_t j = (int64_t)blockIdx.y * nw + wid; j < J.n; j += (int64_t)gridDim.y * nw)
    for (int64_t i = lane; i < J.m; i += 32) mx = fmax(mx, fabs(J.B[i + j * J.ldb]));
  mx = block_max(mx, red);
  if (threadIdx.x == 0 && mx > 0) atomicMax(J.maxbits, (unsigned long long)__double_as_longlong(mx));
}

// CTAs (matrix, part): the scaled float pairs and each column's norm, a warp
// per column
__global__ void __launch_bounds__(512) df_prep_split_kernel(const DfPrepJob* __restrict__ jobs) {
  const DfPrepJob J = jobs[blockIdx.x];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double mx = __longlong_as_double((long long)*J.maxbits);
  const double sc = mx > 0 ? ldexp(1.0, -(ilogb(mx) + 1)) : 1.0;
  if (blockIdx.y == 0 && threadIdx.x == 0) *J.scale = sc;
  for (int64_t j = (int64_t)blockIdx.y * nw + wid; j < J.n; j += (int64_t)gridDim.y * nw) {
    float2* w = J.work + j * J.cs;
    double cm = 0;
    for (int64_t i = lane; i < J.m; i += 32) {
      const double x = J.B[i + j * J.ldb] * sc;
      const Df d = df_split(x);
      w[i * J.rs] = make_float2(d.h, d.l);
      cm = fmax(cm, fabs(x));
    }
    cm = warp_max(cm);
    double acc = 0;
    if (cm > 0) {
      const double s2 = pow2_scale_inv(cm);
      for (int64_t i = lane; i < J.m; i += 32) {
        const Df d = df_split(J.B[i + j * J.ldb] * sc);
        const double t = df_val(d.h, d.l) * s2;
        acc = fma(t, t, acc);
      }
      acc = sqrt(warp_sum(acc)) / s2;
    }
    if (lane == 0) J.vn0[j] = acc;
  }
}

// finish: xLAQPS's swaps replayed into the column order, jpvt (1-based), and
// B = (h + l) / scale in that order (df_join_kernel, then the gather)
struct DfFinishJob {
  int64_t m, n, ldb;
  double* B;
  const float2* work;
  int64_t cs, rs;
  const double* scale;
  const int64_t* piv;
  const int64_t* nfac;
  int64_t* jpvt;
};

__global__ void __launch_bounds__(512) df_finish_group_kernel(const DfFinishJob* __restrict__ jobs) {
  extern __shared__ int fin_smem[];
  const DfFinishJob J = jobs[blockIdx.x];
  int* ca = fin_smem;        // column at position
  int* ps = fin_smem + J.n;  // position of column
  for (int64_t i = threadIdx.x; i < J.n; i += blockDim.x) ca[i] = ps[i] = (int)i;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int64_t nf = *J.nfac;
    for (int64_t c = 0; c < nf; ++c) {
      const int pc = (int)J.piv[c];
      const int p = ps[pc];
      const int other = ca[c];
      ca[p] = other;
      ps[other] = p;
      ca[c] = pc;
      ps[pc] = (int)c;
    }
  }
  __syncthreads();
  const double inv = 1.0 / *J.scale;
  for (int64_t j = threadIdx.x; j < J.n; j += blockDim.x) J.jpvt[j] = ca[j] + 1;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t j = wid; j < J.n; j += nw) {
    const float2* w = J.work + (int64_t)ca[j] * J.cs;
    for (int64_t i = lane; i < J.m; i += 32) J.B[i + j * J.ldb] = df_val(w[i * J.rs].x, w[i * J.rs].y) * inv;
  }
}

// max |B| as the bit pattern of a nonnegative double
__global__ void df_absmax_kernel(int64_t m, int64_t n, const double* __restrict__ B, int64_t ldb,
                                 unsigned long long* __restrict__ out) {
  double mx = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, fabs(B[t % m + (t / m) * ldb]));
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

// scale = 2^-E with max |B| in [2^(E-1), 2^E)
__global__ void df_scale_kernel(const unsigned long long* mx, double* scale) {
  const double m = __longlong_as_double((long long)*mx);
  *scale = m > 0 ? ldexp(1.0, -(ilogb(m) + 1)) : 1.0;
}

// (h, l) = split(B * scale); a warp per column also writes its norm
__global__ void df_split_kernel(int64_t m, int64_t n, const double* __restrict__ B, int64_t ldb,
                                const double* __restrict__ scale, float* __restrict__ Bh, float* __restrict__ Bl,
                                int64_t ldh, double* __restrict__ vn0) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double sc = *scale;
  for (int64_t j = w0; j < n; j += nw) {
    double mx = 0;
    for (int64_t i = lane; i < m; i += 32) {
      const double x = B[i + j * ldb] * sc;
      const Df d = df_split(x);
      Bh[i + j * ldh] = d.h;
      Bl[i + j * ldh] = d.l;
      mx = fmax(mx, fabs(x));
    }
    mx = warp_max(mx);
    double acc = 0;
    if (mx > 0) {
      const double s = pow2_scale_inv(mx);
      for (int64_t i = lane; i < m; i += 32) {
        const double t = df_val(Bh[i + j * ldh], Bl[i + j * ldh]) * s;
        acc = fma(t, t, acc);
      }
      acc = sqrt(warp_sum(acc)) / s;
    }
    if (lane == 0) vn0[j] = acc;
  }
}

// the step at which each column became a pivot (n when it did not):
// step_of[piv[c]] = c for c < nfac
__global__ void qr_step_of_kernel(int64_t n, const int64_t* __restrict__ piv, const int64_t* __restrict__ nfac_p,
                                  int64_t* __restrict__ step_of) {
  const int64_t nfac = *nfac_p;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    step_of[t] = n;
  __syncthreads();
  if (blockIdx.x == 0)
    for (int64_t c = threadIdx.x; c < nfac; c += blockDim.x) step_of[piv[c]] = c;
}

// B = (h + l) / scale, except the Householder vectors below the diagonal of
// the pivot columns (rows below the step of column j), which carry no scale
__global__ void df_join_kernel(int64_t m, int64_t n, const float* __restrict__ Bh, const float* __restrict__ Bl,
                               int64_t ldh, const double* __restrict__ scale, double* __restrict__ B, int64_t ldb,
                               const int64_t* __restrict__ step_of) {
  const double inv = 1.0 / *scale;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    const double v = df_val(Bh[i + j * ldh], Bl[i + j * ldh]);
    B[i + j * ldb] = i > step_of[j] ? v : v * inv;
  }
}

// the Float32 sketch's conversions for the shared-memory QR: max |B| (as
// the bits of a double, for df_scale_kernel), B * scale (exact: a power of
// two) with each column's norm, and back
__global__ void f32_absmax_kernel(int64_t m, int64_t n, const float* __restrict__ B, int64_t ldb,
                                  unsigned long long* __restrict__ out) {
  double mx = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x)
    mx = fmax(mx, (double)fabsf(B[t % m + (t / m) * ldb]));
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, (unsigned long long)__double_as_longlong(mx));
}

__global__ void f32_split_kernel(int64_t m, int64_t n, const float* __restrict__ B, int64_t ldb,
                                 const double* __restrict__ scale, float* __restrict__ Bs, int64_t lds,
                                 double* __restrict__ vn0) {
  const int lane = threadIdx.x & 31;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float sc = (float)*scale;
  for (int64_t j = w0; j < n; j += nw) {
    double mx = 0;
    for (int64_t i = lane; i < m; i += 32) {
      const float x = B[i + j * ldb] * sc;
      Bs[i + j * lds] = x;
      mx = fmax(mx, (double)fabsf(x));
    }
    mx = warp_max(mx);
    double acc = 0;
    if (mx > 0) {
      const double s = pow2_scale_inv(mx);
      for (int64_t i = lane; i < m; i += 32) {
        const double t = (double)Bs[i + j * lds] * s;
        acc = fma(t, t, acc);
      }
      acc = sqrt(warp_sum(acc)) / s;
    }
    if (lane == 0) vn0[j] = acc;
  }
}

__global__ void f32_join_kernel(int64_t m, int64_t n, const float* __restrict__ Bs, int64_t lds,
                                const double* __restrict__ scale, float* __restrict__ B, int64_t ldb,
                                const int64_t* __restrict__ step_of) {
  const float inv = (float)(1.0 / *scale);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % m, j = t / m;
    const float v = Bs[i + j * lds];
    B[i + j * ldb] = i > step_of[j] ? v : v * inv;
  }
}

// LAPACK's column order after pivots piv[0..nfac): replay the swaps of
// position c with the position holding piv[c] (one thread; nfac is small)
__global__ void geqp3_replay_kernel(int64_t n, const int64_t* piv, const int64_t* nfac_p, int64_t* col_at,
                                    int64_t* pos) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int64_t nfac = *nfac_p;
  for (int64_t c = 0; c < nfac; ++c) {
    const int64_t pc = piv[c];
    const int64_t p = pos[pc];
    const int64_t other = col_at[c];
    col_at[p] = other;
    pos[other] = p;
    col_at[c] = pc;
    pos[pc] = c;
  }
}

// the same replay with the permutation in shared memory (n <= 24576):
// the swaps are a chain of dependent reads, which shared memory serves in
// tens of cycles instead of an L2 round trip each
__global__ void __launch_bounds__(1024) geqp3_replay_smem_kernel(int64_t n, const int64_t* piv, const int64_t* nfac_p,
                                                                 int64_t* col_at) {
  extern __shared__ int rp_smem[];
  int* ca = rp_smem;      // column at position
  int* ps = rp_smem + n;  // position of column
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) ca[i] = ps[i] = (int)i;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int64_t nfac = *nfac_p;
    for (int64_t c = 0; c < nfac; ++c) {
      const int pc = (int)piv[c];
      const int p = ps[pc];
      const int other = ca[c];
      ca[p] = other;
      ps[other] = p;
      ca[c] = pc;
      ps[pc] = (int)c;
    }
  }
  __syncthreads();
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) col_at[i] = ca[i];
}

__global__ void iota_kernel(int64_t n, int64_t* a, int64_t* b) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    a[t] = b[t] = t;
}

__global__ void jpvt_kernel(int64_t n, const int64_t* col_at, int64_t* jpvt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    jpvt[t] = col_at[t] + 1;
}

__global__ void jpvt_identity_kernel(int64_t n, int64_t* jpvt) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    jpvt[t] = t + 1;
}

// ---- Householder application, one warp per column of X ----------------------
template <typename T>
__global__ void apply_q_kernel(int trans, int64_t m, int64_t k, const T* __restrict__ V, int64_t ldv,
                               const T* __restrict__ tau, T* __restrict__ X, int64_t ldx, int64_t nc) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int64_t col = (int64_t)blockIdx.x * nw + wid; col < nc; col += (int64_t)gridDim.x * nw) {
    T* x = X + col * ldx;
    for (int64_t t = 0; t < k; ++t) {
      const int64_t i = trans ? t : (k - 1 - t);
      const T ti = tau[i];
      if (ti == 0) continue;
      const T* v = V + i * ldv;
      T s = 0;
      for (int64_t r = i + 1 + lane; r < m; r += 32) s += v[r] * x[r];
      s = warp_sum(s);
      const T f = ti * (x[i] + s);
      __syncwarp();
      for (int64_t r = i + 1 + lane; r < m; r += 32) x[r] -= f * v[r];
      if (lane == 0) x[i] -= f;
      __syncwarp();
    }
  }
}

template <typename T>
__global__ void col_norms_kernel(int64_t m, int64_t n, const T* __restrict__ A, int64_t lda,
                                 T* __restrict__ out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  for (int64_t j = (int64_t)blockIdx.x * nw + wid; j < n; j += (int64_t)gridDim.x * nw) {
    T r = warp_nrm2(A + j * lda, m, lane);
    if (lane == 0) out[j] = r;
  }
}

}  // namespace

// LRA_QR_SMEM=0 keeps the double-float QR's columns in global memory
// even where they would fit shared memory (both variants stay testable)
static bool qr_smem_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("LRA_QR_SMEM");
    return !(e && *e == '0');
  }();
  return on;
}

// LRA_TRACE: the mean time per pivot of each phase of the double-float QR
// (CTA 0's %globaltimer stamps, 16 per pivot)
static void print_qr_trace(lra_ctx* ctx, const unsigned long long* stamps, int64_t kmax, int64_t m, int64_t n,
                           const char* kname, bool smem, const unsigned long long* pubt, int G) {
  std::vector<unsigned long long> h((size_t)16 * kmax), pt;
  LRA_CUDA(cudaMemcpyAsync(h.data(), stamps, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  if (pubt) {
    pt.resize((size_t)G * kmax);
    LRA_CUDA(cudaMemcpyAsync(pt.data(), pubt, pt.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  if (pubt) {
    // spread of the CTAs' word times per pivot, and CTA 0's wait after the last
    double spread = 0, after = 0;
    int64_t cnt = 0;
    for (int64_t c = 0; c < kmax; ++c) {
      const unsigned long long* p = pt.data() + (size_t)c * G;
      unsigned long long lo = ~0ull, hi = 0;
      for (int q = 0; q < G; ++q) {
        lo = std::min(lo, p[q]);
        hi = std::max(hi, p[q]);
      }
      if (!lo || !h[16 * c + 6]) continue;
      spread += (double)(hi - lo);
      after += (double)h[16 * c + 6] - (double)hi;
      ++cnt;
    }
    if (cnt)
      std::fprintf(stderr, "[lra] %s exchange: word spread %.2f us, last word to CTA 0 done %.2f us\n", kname,
                   spread / cnt / 1e3, after / cnt / 1e3);
  }
  static const char* const glob[8] = {"vs-load", "reflector", "scale", "columns", "downdate", "publish", "barrier",
                                      "write-back+pivot"};
  static const char* const sm[8] = {"stage-load", "dots+reflector", "-", "f+downdate+word",
                                    "stage+word", "deferred-update||exchange", "-", "rest"};
  const char* const* lab = smem ? sm : glob;
  double ph[7] = {0}, cyc = 0, sub[6] = {0};
  int64_t cnt = 0, nsub = 0, nflag = 0;
  for (int64_t c = 0; c + 1 < kmax; ++c) {
    const unsigned long long* t = h.data() + 16 * c;
    if (!t[0] || !t[7] || !h[16 * (c + 1)]) continue;
    for (int q = 0; q < 7; ++q) ph[q] += (double)(t[q + 1] - t[q]);
    cyc += (double)(h[16 * (c + 1)] - t[0]);
    ++cnt;
    if (t[8] && t[9] && t[10] && t[11] && t[12] && t[13]) {
      sub[0] += (double)t[8] - (double)t[3];
      for (int q = 1; q < 6; ++q) sub[q] += (double)(t[8 + q] - t[7 + q]);
      if (t[12] - t[11] > 300) ++nflag;
      ++nsub;
    }
  }
  if (nsub && smem)
    std::fprintf(stderr,
                 "[lra] %s warp 1 (us): to start %.2f f %.2f - %.2f downdate %.2f recompute %.2f "
                 "word %.2f; flagged steps %lld\n",
                 kname, sub[0] / nsub / 1e3, sub[1] / nsub / 1e3, sub[2] / nsub / 1e3, sub[3] / nsub / 1e3,
                 sub[4] / nsub / 1e3, sub[5] / nsub / 1e3, (long long)nflag);
  else if (nsub)
    std::fprintf(stderr,
                 "[lra] %s warp-0 passes (us): load+dots %.2f reduce+f %.2f update %.2f | load+dots %.2f "
                 "reduce+f %.2f update %.2f\n",
                 kname, sub[0] / nsub / 1e3, sub[1] / nsub / 1e3, sub[2] / nsub / 1e3, sub[3] / nsub / 1e3,
                 sub[4] / nsub / 1e3, sub[5] / nsub / 1e3);
  if (cnt) {
    std::fprintf(stderr, "[lra] %s m=%lld n=%lld pivots=%lld us/pivot %.2f:", kname, (long long)m, (long long)n,
                 (long long)cnt, cyc / cnt / 1e3);
    double rest = cyc;
    for (int q = 0; q < 7; ++q) {
      std::fprintf(stderr, " %s %.2f", lab[q], ph[q] / cnt / 1e3);
      rest -= ph[q];
    }
    std::fprintf(stderr, " %s %.2f\n", lab[7], rest / cnt / 1e3);
  }
}

// The mixed path's pivoted QR of many small sketches at once: one grouped
// launch each for the conversion, the factorization (a CTA per matrix,
// largest first) and the replay into column order.  Each matrix comes out
// as geqp3_adap leaves it when its shared-memory kernel runs, bit for bit.
bool geqp3_df_batch_fits(lra_ctx* ctx, int64_t m, int64_t n) {
  constexpr int NTG = 512;
  if (m < 1 || n < 1 || n >= (int64_t)XW_IDX || m > 20480) return false;
  const size_t smem = (size_t)m * sizeof(float2) + (size_t)n * (5 * 8 + 1);
  static size_t cap = [&] {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, geqp3_df_group_kernel<NTG>) != cudaSuccess) {
      cudaGetLastError();
      return (size_t)0;
    }
    return (size_t)(optin - (int)fa.sharedSizeBytes);
  }();
  return smem <= cap && (size_t)2 * n * sizeof(int) <= 200 * 1024;
}

void geqp3_df_batch(lra_ctx* ctx, int64_t count, const DfBatchItem* items, int64_t nb, double atol, double rtol,
                    int64_t* k_dev) {
  constexpr int NTG = 512;
  if (count <= 0) return;
  // largest factorizations first, so that the last wave is short
  std::vector<int64_t> ord((size_t)count);
  for (int64_t i = 0; i < count; ++i) ord[(size_t)i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) {
    const DfBatchItem &x = items[a], &y = items[b];
    return x.m * x.n * std::min(x.kmax, x.m) > y.m * y.n * std::min(y.kmax, y.m);
  });
  std::vector<DfPrepJob> prep((size_t)count);
  std::vector<QrJob> qr((size_t)count);
  std::vector<DfFinishJob> fin((size_t)count);
  size_t smem_qr = 0, smem_fin = 0;
  unsigned long long* maxbits = ctx->arena.alloc_n<unsigned long long>((size_t)count);
  LRA_CUDA(cudaMemsetAsync(maxbits, 0, (size_t)count * sizeof(unsigned long long), ctx->stream));
  int64_t nmax = 1;
  for (int64_t i = 0; i < count; ++i) nmax = std::max(nmax, items[i].n);
  for (int64_t t = 0; t < count; ++t) {
    const int64_t i = ord[(size_t)t];
    const DfBatchItem& it = items[i];
    const int64_t m = it.m, n = it.n;
    if (!geqp3_df_batch_fits(ctx, m, n)) fail(LRA_EINVAL, "geqp3_df_batch: a sketch does not fit");
    float2* work = ctx->arena.alloc_n<float2>((size_t)m * n);
    double* vn0 = ctx->arena.alloc_n<double>(n);
    double* scale = ctx->arena.alloc_n<double>(1);
    // row-major when every step sums its columns row by row (a thread per
    // column reads a row of the workspace coalesced), else column-major
    const bool rowmaj = m - 1 <= ctx->tuning.qr_seq_len;
    const int64_t cs = rowmaj ? 1 : m, rs = rowmaj ? n : 1;
    prep[(size_t)t] = DfPrepJob{m, n, it.ldb, it.B, work, cs, rs, vn0, scale, maxbits + t};
    QrJob& J = qr[(size_t)t];
    std::memset(&J, 0, sizeof J);
    J.P.m = m;
    J.P.n = n;
    J.P.lda = m;
    J.P.tau = it.tau;
    J.P.kmax = std::min<int64_t>(it.kmax, std::min(m, n));
    J.P.nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(J.P.kmax, 1)));
    J.P.atol = atol;
    J.P.rtol = rtol;
    J.P.pivot = 1;
    J.P.seq_len = ctx->tuning.qr_seq_len;
    J.P.k_out = k_dev + i;
    J.X.piv = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(J.P.kmax, 1));
    J.X.nfac = ctx->arena.alloc_n<int64_t>(1);
    J.X.beta = ctx->arena.alloc_n<double>(std::max<int64_t>(J.P.kmax, 1));
    J.D.vn0 = vn0;
    J.D.scale = scale;
    J.work = work;
    J.cs = cs;
    J.rs = rs;
    fin[(size_t)t] = DfFinishJob{m, n, it.ldb, it.B, work, cs, rs, scale, J.X.piv, J.X.nfac, it.jpvt};
    smem_qr = std::max(smem_qr, (size_t)m * sizeof(float2) + (size_t)n * (5 * 8 + 1));
    smem_fin = std::max(smem_fin, (size_t)2 * n * sizeof(int));
  }
  // LRA_TRACE: the phase stamps of the largest factorization
  unsigned long long* stamps = nullptr;
  if (trace_on()) {
    const int64_t km = std::max<int64_t>(qr[0].P.kmax, 1);
    stamps = ctx->arena.alloc_n<unsigned long long>((size_t)16 * km);
    LRA_CUDA(cudaMemsetAsync(stamps, 0, (size_t)16 * km * 8, ctx->stream));
    qr[0].D.stamps = stamps;
  }
  DfPrepJob* dprep = ctx->arena.alloc_n<DfPrepJob>((size_t)count);
  QrJob* dqr = ctx->arena.alloc_n<QrJob>((size_t)count);
  DfFinishJob* dfin = ctx->arena.alloc_n<DfFinishJob>((size_t)count);
  int* next = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemcpyAsync(dprep, prep.data(), prep.size() * sizeof(DfPrepJob), cudaMemcpyHostToDevice, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(dqr, qr.data(), qr.size() * sizeof(QrJob), cudaMemcpyHostToDevice, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(dfin, fin.data(), fin.size() * sizeof(DfFinishJob), cudaMemcpyHostToDevice, ctx->stream));
  LRA_CUDA(cudaMemsetAsync(next, 0, sizeof(int), ctx->stream));
  cudaEvent_t ev[4];
  const bool tr = trace_on();
  if (tr)
    for (auto& e : ev) LRA_CUDA(cudaEventCreate(&e));
  if (tr) LRA_CUDA(cudaEventRecord(ev[0], ctx->stream));
  {
    const unsigned parts = (unsigned)std::min<int64_t>(16, (nmax + 15) / 16);
    df_prep_max_kernel<<<dim3((unsigned)count, parts), 512, 0, ctx->stream>>>(dprep);
    post_launch(ctx, "df_prep_max_kernel");
    df_prep_split_kernel<<<dim3((unsigned)count, parts), 512, 0, ctx->stream>>>(dprep);
    post_launch(ctx, "df_prep_split_kernel");
  }
  if (tr) LRA_CUDA(cudaEventRecord(ev[1], ctx->stream));
  raise_smem_limit(ctx, (const void*)geqp3_df_group_kernel<NTG>);
  const int grid = (int)std::min<int64_t>(count, ctx->num_sms);
  geqp3_df_group_kernel<NTG><<<grid, NTG, smem_qr, ctx->stream>>>(dqr, (int)count, next);
  post_launch(ctx, "geqp3_df_group_kernel");
  if (tr) LRA_CUDA(cudaEventRecord(ev[2], ctx->stream));
  raise_smem_limit(ctx, (const void*)df_finish_group_kernel);
  df_finish_group_kernel<<<(unsigned)count, 512, smem_fin, ctx->stream>>>(dfin);
  post_launch(ctx, "df_finish_group_kernel");
  if (tr) {
    LRA_CUDA(cudaEventRecord(ev[3], ctx->stream));
    LRA_CUDA(cudaEventSynchronize(ev[3]));
    float a = 0, b = 0, c = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    cudaEventElapsedTime(&c, ev[2], ev[3]);
    int64_t piv = 0, mn = 0;
    for (const DfBatchItem* it = items; it < items + count; ++it) {
      piv += std::min(it->kmax, std::min(it->m, it->n));
      mn += it->m * it->n;
    }
    std::fprintf(stderr, "[lra] geqp3_df_batch %lld sketches (%.1f MB, <= %lld pivots): prep %.3f ms qr %.3f ms finish %.3f ms\n",
                 (long long)count, 8e-6 * (double)mn, (long long)piv, a, b, c);
    print_qr_trace(ctx, stamps, qr[0].P.kmax, qr[0].P.m, qr[0].P.n, "geqp3_df_group_kernel", true, nullptr, 1);
    for (auto& e : ev) cudaEventDestroy(e);
  }
  // the host copies of the job lists must outlive the asynchronous uploads
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
}

// ---- the shared-memory pivoted QR in phases ---------------------------------------
// prepare (buffers; the sketch converted to the kernel's arithmetic, its
// column norms), launch (one sketch, or several adaptive steps' sketches on
// CTAs of their own), finish (the factors joined back, xLAQPS's swaps
// replayed, the columns permuted), so that a launch can hold several steps.

template <typename T>
using SmA = typename std::conditional<sizeof(T) == 8, QrArithDf, QrArithF32>::type;
constexpr int kSmNT = 512;  // warp 0 for the reflector, 15 column warps

// dynamic shared memory of a CTA holding ncap columns of m rows: the pivot
// column, the columns, four values, a stored element and a state byte per
// column
template <class A>
size_t sm_smem(int64_t m, int64_t ncap) {
  using E = typename A::E;
  using V = typename A::V;
  return (size_t)(m + ncap * m) * sizeof(E) + (size_t)ncap * (4 * sizeof(V) + sizeof(E) + 1);
}

template <class A>
size_t sm_capacity(lra_ctx* ctx) {
  raise_smem_limit(ctx, (const void*)geqp3_df_smem_kernel<A, kSmNT>);
  cudaFuncAttributes fa;
  LRA_CUDA(cudaFuncGetAttributes(&fa, geqp3_df_smem_kernel<A, kSmNT>));
  return (size_t)fa.maxDynamicSharedSizeBytes;
}

template <class A>
bool sm_resident(lra_ctx* ctx, size_t smem) {
  int per = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, geqp3_df_smem_kernel<A, kSmNT>, kSmNT, smem));
  return per >= 1;
}

// the SMs a pivoted-QR launch of this context may take (the tuning's
// qr_sms cap, else all)
static int qr_sm_cap(const lra_ctx* ctx) {
  const int c = ctx->tuning.qr_sms;
  return c > 0 ? std::min(c, ctx->num_sms) : ctx->num_sms;
}

// a sketch factored alone: every SM it may take, at least one column per
// column warp
static int sm_natural_ctas(lra_ctx* ctx, int64_t n) {
  return (int)std::min<int64_t>(std::min(qr_sm_cap(ctx), 256),
                                std::max<int64_t>(1, (n + kSmNT / 32 - 2) / (kSmNT / 32 - 1)));
}

// the fewest CTAs whose shared memory holds an m x n sketch (0: not one column)
template <class A>
int sm_min_ctas(size_t cap, int64_t m, int64_t n) {
  using E = typename A::E;
  using V = typename A::V;
  const size_t fixed = (size_t)m * sizeof(E);
  const size_t per = (size_t)m * sizeof(E) + 4 * sizeof(V) + sizeof(E) + 1;
  if (cap < fixed + per) return 0;
  const int64_t ncap = (int64_t)((cap - fixed) / per);
  return (int)((n + ncap - 1) / ncap);
}

template <typename T>
struct SmQr {
  int64_t m = 0, n = 0, lda = 0;
  T* A = nullptr;
  int64_t* jpvt = nullptr;
  int G = 0;
  size_t smem = 0;
  SmJob<SmA<T>> job;
  int64_t* col_at = nullptr;
  int64_t* pos = nullptr;
  double* scale = nullptr;
  unsigned gm = 1;
};

template <typename T>
void sm_prepare(lra_ctx* ctx, SmQr<T>& q, int64_t m, int64_t n, T* A, int64_t lda, int64_t* jpvt, T* tau,
                int64_t kmax, int64_t nb, double atol, double rtol, int G) {
  using Ar = SmA<T>;
  using E = typename Ar::E;
  q.m = m;
  q.n = n;
  q.A = A;
  q.lda = lda;
  q.jpvt = jpvt;
  q.G = G;
  q.smem = sm_smem<Ar>(m, (n + G - 1) / G);
  QrParams<T>& P = q.job.P;
  P = QrParams<T>{};
  P.m = m;
  P.n = n;
  P.lda = m;  // the converted sketch's leading dimension
  P.A = A;
  P.jpvt = jpvt;
  P.tau = tau;
  P.part_d = ctx->arena.alloc_n<double>(G);
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.kmax = std::min<int64_t>(kmax, std::min(m, n));
  P.nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(P.kmax, 1)));
  P.atol = atol;
  P.rtol = rtol;
  P.pivot = 1;
  P.k_out = ctx->arena.alloc_n<int64_t>(1);
  P.seq_len = ctx->tuning.qr_seq_len;
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  LRA_CUDA(cudaMemsetAsync(P.k_out, 0, sizeof(int64_t), ctx->stream));
  QrV2Extra& X = q.job.X;
  X.piv = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(P.kmax, 1));
  X.nfac = ctx->arena.alloc_n<int64_t>(1);
  X.part_k = ctx->arena.alloc_n<long long>(G);
  X.beta = ctx->arena.alloc_n<double>(std::max<int64_t>(P.kmax, 1));
  LRA_CUDA(cudaMemsetAsync(X.nfac, 0, sizeof(int64_t), ctx->stream));
  q.col_at = ctx->arena.alloc_n<int64_t>(n);
  q.pos = ctx->arena.alloc_n<int64_t>(n);
  const unsigned gi = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->num_sms * 4));
  iota_kernel<<<gi, 256, 0, ctx->stream>>>(n, q.col_at, q.pos);
  post_launch(ctx, "iota_kernel");
  // the sketch at a power-of-two scale in the kernel's arithmetic
  double* vn0 = ctx->arena.alloc_n<double>(n);
  q.scale = ctx->arena.alloc_n<double>(1);
  unsigned long long* mx = ctx->arena.alloc_n<unsigned long long>(1);
  LRA_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), ctx->stream));
  q.gm = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m * n + 255) / 256, ctx->num_sms * 8));
  const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 7) / 8, ctx->num_sms * 8));
  QrDf& D = q.job.D;
  D = QrDf{nullptr, nullptr, vn0, q.scale, nullptr};
  if constexpr (sizeof(T) == 8) {
    const double* Bd = reinterpret_cast<const double*>(A);
    df_absmax_kernel<<<q.gm, 256, 0, ctx->stream>>>(m, n, Bd, lda, mx);
    post_launch(ctx, "df_absmax_kernel");
    df_scale_kernel<<<1, 1, 0, ctx->stream>>>(mx, q.scale);
    post_launch(ctx, "df_scale_kernel");
    D.Bh = ctx->arena.alloc_n<float>((size_t)m * n);
    D.Bl = ctx->arena.alloc_n<float>((size_t)m * n);
    df_split_kernel<<<gs, 256, 0, ctx->stream>>>(m, n, Bd, lda, q.scale, D.Bh, D.Bl, m, vn0);
    post_launch(ctx, "df_split_kernel");
  } else {
    const float* Bf = reinterpret_cast<const float*>(A);
    f32_absmax_kernel<<<q.gm, 256, 0, ctx->stream>>>(m, n, Bf, lda, mx);
    post_launch(ctx, "f32_absmax_kernel");
    df_scale_kernel<<<1, 1, 0, ctx->stream>>>(mx, q.scale);
    post_launch(ctx, "df_scale_kernel");
    D.Bh = ctx->arena.alloc_n<float>((size_t)m * n);
    f32_split_kernel<<<gs, 256, 0, ctx->stream>>>(m, n, Bf, lda, q.scale, D.Bh, m, vn0);
    post_launch(ctx, "f32_split_kernel");
  }
  QrSm& S = q.job.S;
  S = QrSm{nullptr, nullptr, nullptr};
  if (trace_on()) {
    const int64_t km = std::max<int64_t>(P.kmax, 1);
    D.stamps = ctx->arena.alloc_n<unsigned long long>((size_t)16 * km);
    LRA_CUDA(cudaMemsetAsync(D.stamps, 0, (size_t)16 * km * 8, ctx->stream));
    S.pubt = ctx->arena.alloc_n<unsigned long long>((size_t)G * km);
    LRA_CUDA(cudaMemsetAsync(S.pubt, 0, (size_t)G * km * 8, ctx->stream));
  }
  // the exchange: 4 max words and 4 stop words a 128-byte line apart, and
  // the arrival counter on a line of its own
  unsigned char* xb = static_cast<unsigned char*>(ctx->arena.alloc(1152));
  S.amax = reinterpret_cast<unsigned long long*>(xb);
  S.astop = reinterpret_cast<unsigned*>(xb + 512);
  S.arrive = reinterpret_cast<unsigned*>(xb + 1024);
  S.stage = ctx->arena.alloc_n<E>((size_t)2 * G * m);
  LRA_CUDA(cudaMemsetAsync(xb, 0, 1152, ctx->stream));
  q.job.G = G;
  q.job.off = 0;
}

// one cooperative launch for nq prepared sketches (CTAs laid out in order)
template <typename T>
void sm_launch(lra_ctx* ctx, SmQr<T>* const* qs, int nq) {
  using Ar = SmA<T>;
  SmJobs<Ar> J;
  J.n = nq;
  int off = 0;
  size_t smem = 0;
  for (int i = 0; i < nq; ++i) {
    J.j[i] = qs[i]->job;
    J.j[i].G = qs[i]->G;
    J.j[i].off = off;
    off += qs[i]->G;
    smem = std::max(smem, qs[i]->smem);
  }
  void* args[] = {&J};
  LRA_CUDA(cudaLaunchCooperativeKernel((const void*)geqp3_df_smem_kernel<Ar, kSmNT>, dim3(off), dim3(kSmNT), args,
                                       smem, ctx->stream));
  post_launch(ctx, sizeof(T) == 8 ? "geqp3_df_smem_kernel" : "geqp3_f32_smem_kernel");
}

// the factors back into the sketch: R and the reflectors, xLAQPS's column
// swaps replayed into jpvt, the columns in pivot order
template <typename T>
void sm_finish(lra_ctx* ctx, SmQr<T>& q) {
  const int64_t m = q.m, n = q.n;
  const QrV2Extra& X = q.job.X;
  const QrDf& D = q.job.D;
  if (D.stamps)
    print_qr_trace(ctx, D.stamps, q.job.P.kmax, m, n, sizeof(T) == 8 ? "geqp3_df_smem_kernel" : "geqp3_f32_smem_kernel",
                   true, q.job.S.pubt, q.G);
  int64_t* step_of = ctx->arena.alloc_n<int64_t>(n);
  qr_step_of_kernel<<<1, 1024, 0, ctx->stream>>>(n, X.piv, X.nfac, step_of);
  post_launch(ctx, "qr_step_of_kernel");
  if constexpr (sizeof(T) == 8) {
    df_join_kernel<<<q.gm, 256, 0, ctx->stream>>>(m, n, D.Bh, D.Bl, m, q.scale, reinterpret_cast<double*>(q.A), q.lda,
                                                  step_of);
    post_launch(ctx, "df_join_kernel");
  } else {
    f32_join_kernel<<<q.gm, 256, 0, ctx->stream>>>(m, n, D.Bh, m, q.scale, reinterpret_cast<float*>(q.A), q.lda,
                                                   step_of);
    post_launch(ctx, "f32_join_kernel");
  }
  if (n <= 24576) {
    const size_t rs = (size_t)2 * n * sizeof(int);
    raise_smem_limit(ctx, (const void*)geqp3_replay_smem_kernel);
    geqp3_replay_smem_kernel<<<1, 1024, rs, ctx->stream>>>(n, X.piv, X.nfac, q.col_at);
    post_launch(ctx, "geqp3_replay_smem_kernel");
  } else {
    geqp3_replay_kernel<<<1, 32, 0, ctx->stream>>>(n, X.piv, X.nfac, q.col_at, q.pos);
    post_launch(ctx, "geqp3_replay_kernel");
  }
  const unsigned gi = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->num_sms * 4));
  jpvt_kernel<<<gi, 256, 0, ctx->stream>>>(n, q.col_at, q.jpvt);
  post_launch(ctx, "jpvt_kernel");
  T* tmp = ctx->arena.alloc_n<T>((size_t)m * n);
  gather_cols(ctx, m, n, q.A, q.lda, q.jpvt, tmp, m);
  copy_matrix(ctx, m, n, tmp, m, q.A, q.lda);
}

// the shared-memory kernel applies to an m x n sketch of this type (the
// mixed path's double-float for Float64, FP32 for Float32)
template <typename T>
static bool sm_applies(lra_ctx* ctx, int64_t m, int64_t n) {
  if (!qr_smem_enabled() || n >= (int64_t)XW_IDX || m <= 0 || n <= 0) return false;
  if (sizeof(T) == 8 && !ctx->gemm_tc) return false;
  // the rows a CTA stages per column (the single-step form's reflector bound)
  const int64_t vcap = std::min<int64_t>(m, (int64_t)(160 * 1024 / sizeof(T)));
  return m - 1 <= vcap;
}

template <typename T>
int geqp3_steps_fit(lra_ctx* ctx, int count, const int64_t* m, int64_t n) {
  using Ar = SmA<T>;
  const size_t cap = sm_capacity<Ar>(ctx);
  int total = 0, fit = 0;
  for (int i = 0; i < count && i < kSmJobs; ++i) {
    if (!sm_applies<T>(ctx, m[i], n)) break;
    const int g = sm_min_ctas<Ar>(cap, m[i], n);
    if (g <= 0 || g > sm_natural_ctas(ctx, n) || total + g > qr_sm_cap(ctx)) break;
    total += g;
    fit = i + 1;
  }
  return fit;
}

template <typename T>
int geqp3_adap_steps(lra_ctx* ctx, int count, const QrStep<T>* st, int64_t nb, double atol, double rtol,
                     int64_t* k) {
  using Ar = SmA<T>;
  if (count < 1 || count > kSmJobs) fail(LRA_EINVAL, "geqp3_adap_steps: %d steps", count);
  std::vector<int64_t> ms(count);
  for (int i = 0; i < count; ++i) {
    ms[i] = st[i].m;
    if (st[i].n != st[0].n) fail(LRA_EINVAL, "geqp3_adap_steps: the steps' column counts differ");
  }
  if (geqp3_steps_fit<T>(ctx, count, ms.data(), st[0].n) < count) fail(LRA_EINVAL, "geqp3_adap_steps: no fit");
  const ArenaMark mark = ctx->arena.mark();
  const size_t cap = sm_capacity<Ar>(ctx);
  // each step on the fewest CTAs that hold it; the rest to the last (the
  // largest, with the most pivots)
  std::vector<int> G(count);
  int used = 0;
  for (int i = 0; i < count; ++i) used += G[i] = sm_min_ctas<Ar>(cap, st[i].m, st[i].n);
  G[count - 1] = std::min(sm_natural_ctas(ctx, st[count - 1].n), G[count - 1] + (qr_sm_cap(ctx) - used));
  int* success = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(success, 0x7f, sizeof(int), ctx->stream));
  std::vector<SmQr<T>> q(count);
  std::vector<SmQr<T>*> qp(count);
  size_t smem = 0;
  for (int i = 0; i < count; ++i) {
    sm_prepare<T>(ctx, q[i], st[i].m, st[i].n, st[i].A, st[i].lda, st[i].jpvt, st[i].tau, st[i].kmax, nb, atol,
                  rtol, G[i]);
    q[i].job.S.success = success;
    q[i].job.S.job = i;
    q[i].job.S.nt = st[i].nt;
    qp[i] = &q[i];
    smem = std::max(smem, q[i].smem);
  }
  if (smem > cap || !sm_resident<Ar>(ctx, smem)) fail(LRA_ECUDA, "geqp3_adap_steps: the launch cannot be resident");
  sm_launch<T>(ctx, qp.data(), count);
  std::vector<int64_t> kk(count);
  std::vector<GridBar> hb(count);
  int win = 0x7f7f7f7f;
  for (int i = 0; i < count; ++i) {
    LRA_CUDA(cudaMemcpyAsync(&kk[i], q[i].job.P.k_out, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    LRA_CUDA(cudaMemcpyAsync(&hb[i], q[i].job.P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  }
  LRA_CUDA(cudaMemcpyAsync(&win, success, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < count; ++i)
    if (hb[i].err != 0) {
      ctx->arena.release(mark);
      fail(LRA_ETIMEDOUT, "geqp3: a wait between CTAs timed out");
    }
  const int c = win >= 0 && win < count ? win : -1;
  for (int i = 0; i < count; ++i) k[i] = (c >= 0 && i > c) ? -1 : kk[i];
  if (c >= 0) sm_finish<T>(ctx, q[c]);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  return c;
}

template <typename T>
int64_t geqp3_adap(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda, int64_t* jpvt, T* tau,
                   int64_t kmax, int64_t nb, double atol, double rtol, bool pivot) {
  constexpr int NT = 512;
  if (n <= 0) return 0;
  const ArenaMark mark = ctx->arena.mark();
  // the reflector of each pivot is staged in shared memory when it fits
  const int64_t vcap = std::min<int64_t>(m, (int64_t)(160 * 1024 / sizeof(T)));
  const size_t dyn_smem = (size_t)vcap * sizeof(T);
  raise_smem_limit(ctx, (const void*)geqp3_kernel<T, NT>);
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, geqp3_kernel<T, NT>, NT, dyn_smem));
  if (per_sm < 1) fail(LRA_ECUDA, "geqp3 kernel cannot be resident");
  const int64_t want = (n + (NT / 32) - 1) / (NT / 32);
  int grid = (int)std::min<int64_t>((int64_t)qr_sm_cap(ctx) * std::min(per_sm, 1), want);
  grid = std::max(grid, 1);

  QrParams<T> P;
  P.m = m;
  P.n = n;
  P.lda = lda;
  P.A = A;
  P.jpvt = jpvt;
  P.tau = tau;
  P.vn1 = ctx->arena.alloc_n<T>(n);
  P.vn2 = ctx->arena.alloc_n<T>(n);
  P.flag = ctx->arena.alloc_n<int>(n);
  P.part_v = ctx->arena.alloc_n<T>(grid);
  P.part_i = ctx->arena.alloc_n<int64_t>(grid);
  P.part_d = ctx->arena.alloc_n<double>(grid);
  int* small = ctx->arena.alloc_n<int>(8);
  P.lsticc = small;
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.kmax = std::min<int64_t>(kmax, std::min(m, n));
  P.nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(P.kmax, 1)));
  P.atol = atol;
  P.rtol = rtol;
  P.pivot = pivot ? 1 : 0;
  P.k_out = ctx->arena.alloc_n<int64_t>(1);
  P.vcap = vcap;
  P.seq_len = ctx->tuning.qr_seq_len;
  LRA_CUDA(cudaMemsetAsync(small, 0, 8 * sizeof(int), ctx->stream));
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  if (P.kmax <= 0) {
    // nothing to factor: identity permutation
    std::vector<int64_t> id(n);
    for (int64_t i = 0; i < n; ++i) id[i] = i + 1;
    LRA_CUDA(cudaMemcpyAsync(jpvt, id.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice,
                             ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->arena.release(mark);
    return 0;
  }
  // one barrier per pivot when the reflector and the per-column state of
  // each CTA fit shared memory
  const int64_t nwarps = (int64_t)grid * (NT / 32);
  const int64_t nslot = (n + nwarps - 1) / nwarps * (NT / 32);
  const size_t smem2 = dyn_smem + (size_t)nslot * (3 * sizeof(T) + 1);
  const bool v2 = (m - 1) <= vcap && smem2 <= 200 * 1024;
  if (v2 && pivot && sm_applies<T>(ctx, m, n)) {
    // the shared-memory kernels (Float32 in FP32, the mixed path's Float64 in
    // double-float) when each CTA's share of the columns fits there
    using Ar = SmA<T>;
    // the CTAs it may take, or the fewest that hold the sketch when those
    // are more
    const int G = std::min(std::max(sm_natural_ctas(ctx, n), sm_min_ctas<Ar>(sm_capacity<Ar>(ctx), m, n)),
                           std::min(ctx->num_sms, 256));
    const size_t need = sm_smem<Ar>(m, (n + G - 1) / G);
    if (need <= sm_capacity<Ar>(ctx) && sm_resident<Ar>(ctx, need)) {
      SmQr<T> q;
      sm_prepare<T>(ctx, q, m, n, A, lda, jpvt, tau, P.kmax, nb, atol, rtol, G);
      SmQr<T>* qp = &q;
      sm_launch<T>(ctx, &qp, 1);
      sm_finish<T>(ctx, q);
      int64_t k = 0;
      GridBar hb;
      LRA_CUDA(cudaMemcpyAsync(&k, q.job.P.k_out, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaMemcpyAsync(&hb, q.job.P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
      LRA_CUDA(cudaStreamSynchronize(ctx->stream));
      ctx->arena.release(mark);
      if (hb.err != 0) fail(LRA_ETIMEDOUT, "geqp3: a wait between CTAs timed out");
      return k;
    }
  }
  if (v2) {
    raise_smem_limit(ctx, (const void*)geqp3_v2_kernel<T, NT>);
    LRA_CUDA(cudaFuncSetAttribute(geqp3_v2_kernel<T, NT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxL1));
    int per_sm2 = 0;
    LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, geqp3_v2_kernel<T, NT>, NT, smem2));
    if (per_sm2 < 1) fail(LRA_ECUDA, "geqp3 kernel cannot be resident");
    QrV2Extra X;
    X.piv = ctx->arena.alloc_n<int64_t>(std::max<int64_t>(P.kmax, 1));
    X.nfac = ctx->arena.alloc_n<int64_t>(1);
    X.part_k = ctx->arena.alloc_n<long long>(grid);
    X.beta = ctx->arena.alloc_n<double>(std::max<int64_t>(P.kmax, 1));
    int64_t* col_at = ctx->arena.alloc_n<int64_t>(n);
    int64_t* pos = ctx->arena.alloc_n<int64_t>(n);
    const unsigned gi = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->num_sms * 4));
    iota_kernel<<<gi, 256, 0, ctx->stream>>>(n, col_at, pos);
    post_launch(ctx, "iota_kernel");
    // the mixed-precision path factors Float64 sketches in double-float
    const bool dfq = sizeof(T) == 8 && ctx->gemm_tc && pivot;
    if (dfq) {
      float* Bh = ctx->arena.alloc_n<float>((size_t)m * n);
      float* Bl = ctx->arena.alloc_n<float>((size_t)m * n);
      double* vn0 = ctx->arena.alloc_n<double>(n);
      double* scale = ctx->arena.alloc_n<double>(1);
      unsigned long long* mx = ctx->arena.alloc_n<unsigned long long>(1);
      LRA_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), ctx->stream));
      const double* Bd = reinterpret_cast<const double*>(A);
      const unsigned gm = (unsigned)std::max<int64_t>(1, std::min<int64_t>((m * n + 255) / 256, ctx->num_sms * 8));
      df_absmax_kernel<<<gm, 256, 0, ctx->stream>>>(m, n, Bd, lda, mx);
      post_launch(ctx, "df_absmax_kernel");
      df_scale_kernel<<<1, 1, 0, ctx->stream>>>(mx, scale);
      post_launch(ctx, "df_scale_kernel");
      const unsigned gs = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 7) / 8, ctx->num_sms * 8));
      df_split_kernel<<<gs, 256, 0, ctx->stream>>>(m, n, Bd, lda, scale, Bh, Bl, m, vn0);
      post_launch(ctx, "df_split_kernel");
      QrDf D{Bh, Bl, vn0, scale, nullptr};
      if (trace_on()) {
        D.stamps = ctx->arena.alloc_n<unsigned long long>((size_t)16 * std::max<int64_t>(P.kmax, 1));
        LRA_CUDA(cudaMemsetAsync(D.stamps, 0, (size_t)16 * std::max<int64_t>(P.kmax, 1) * 8, ctx->stream));
      }
      QrParams<double> Pd;
      std::memcpy(&Pd, &P, sizeof(Pd));
      Pd.lda = m;
      // the columns stay in global memory (a CTA's share does not fit shared
      // memory)
      const char* kname = "geqp3_df_kernel";
      {
        raise_smem_limit(ctx, (const void*)geqp3_df_kernel<NT>);
        // as much L1 as the shared memory leaves: the warps' columns live there
        LRA_CUDA(cudaFuncSetAttribute(geqp3_df_kernel<NT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxL1));
        int per_df = 0;
        LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_df, geqp3_df_kernel<NT>, NT, smem2));
        if (per_df < 1) fail(LRA_ECUDA, "geqp3 kernel cannot be resident");
        void* args[] = {&Pd, &X, &D};
        LRA_CUDA(cudaLaunchCooperativeKernel((const void*)geqp3_df_kernel<NT>, dim3(grid), dim3(NT), args, smem2,
                                             ctx->stream));
      }
      post_launch(ctx, kname);
      if (D.stamps) print_qr_trace(ctx, D.stamps, P.kmax, m, n, kname, false, nullptr, 1);
      int64_t* step_of = ctx->arena.alloc_n<int64_t>(n);
      qr_step_of_kernel<<<1, 1024, 0, ctx->stream>>>(n, X.piv, X.nfac, step_of);
      post_launch(ctx, "qr_step_of_kernel");
      df_join_kernel<<<gm, 256, 0, ctx->stream>>>(m, n, Bh, Bl, m, scale, reinterpret_cast<double*>(A), lda,
                                                  step_of);
      post_launch(ctx, "df_join_kernel");
    } else {
      void* args[] = {&P, &X};
      LRA_CUDA(cudaLaunchCooperativeKernel((const void*)geqp3_v2_kernel<T, NT>, dim3(grid), dim3(NT), args,
                                           smem2, ctx->stream));
      post_launch(ctx, "geqp3_v2_kernel");
    }
    if (pivot) {
      // xLAQPS's swaps, replayed: jpvt and the column order of A
      if (n <= 24576) {
        const size_t rs = (size_t)2 * n * sizeof(int);
        raise_smem_limit(ctx, (const void*)geqp3_replay_smem_kernel);
        geqp3_replay_smem_kernel<<<1, 1024, rs, ctx->stream>>>(n, X.piv, X.nfac, col_at);
        post_launch(ctx, "geqp3_replay_smem_kernel");
      } else {
        geqp3_replay_kernel<<<1, 32, 0, ctx->stream>>>(n, X.piv, X.nfac, col_at, pos);
        post_launch(ctx, "geqp3_replay_kernel");
      }
    }
    jpvt_kernel<<<gi, 256, 0, ctx->stream>>>(n, col_at, jpvt);
    post_launch(ctx, "jpvt_kernel");
    if (pivot) {
      T* tmp = ctx->arena.alloc_n<T>((size_t)m * n);
      gather_cols(ctx, m, n, A, lda, jpvt, tmp, m);
      copy_matrix(ctx, m, n, tmp, m, A, lda);
    }
  } else {
    void* args[] = {&P};
    LRA_CUDA(cudaLaunchCooperativeKernel((const void*)geqp3_kernel<T, NT>, dim3(grid), dim3(NT), args,
                                         dyn_smem, ctx->stream));
    post_launch(ctx, "geqp3_kernel");
  }
  int64_t k = 0;
  GridBar hb;
  LRA_CUDA(cudaMemcpyAsync(&k, P.k_out, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "geqp3: a grid barrier timed out");
  return k;
}

// X <- triu(R)^{-1} X, recursive: the solve with the trailing half, a GEMM
// update of the leading rows, the solve with the leading half; blocks of at
// most 32 rows are solved by trsm_left_diag_kernel (a thread per right-hand
// side, back substitution in registers)
template <typename T>
void trsm_upper(lra_ctx* ctx, int64_t k, int64_t nrhs, const T* R, int64_t ldr, T* X, int64_t ldx, const T* Yd) {
  if (k <= 0 || nrhs <= 0) return;
  if (trsm_by_inverse<T>(ctx, k, nrhs)) {
    // R^-1 X = Y (D^-1 X) with Y = R^-1 D (entries of order one; Yd when the
    // caller has it already), a tensor-core GEMM
    const ArenaMark mk = ctx->arena.mark();
    T* Y = Yd ? nullptr : ctx->arena.alloc_n<T>((size_t)k * k);
    T* W = ctx->arena.alloc_n<T>((size_t)k * nrhs);
    if (Y) tri_inv_upper<T>(ctx, k, R, ldr, Y, k);
    const T* Yu = Yd ? Yd : Y;
    div_by_diag<T>(ctx, k, nrhs, R, ldr, 'l', X, ldx, W, k);
    gemm<T>(ctx, 'n', 'n', k, nrhs, k, T(1), Yu, k, W, k, T(0), X, ldx);
    ctx->arena.release(mk);
    return;
  }
  if (k <= 32) {
    trsm_left_diag(ctx, (int)k, nrhs, R, ldr, X, ldx);
    return;
  }
  const int64_t k1 = (k / 2 + 31) / 32 * 32, k2 = k - k1;
  trsm_upper(ctx, k2, nrhs, R + k1 + k1 * ldr, ldr, X + k1, ldx);
  gemm<T>(ctx, 'n', 'n', k1, nrhs, k2, T(-1), R + k1 * ldr, ldr, X + k1, ldx, T(1), X, ldx);
  trsm_upper(ctx, k1, nrhs, R, ldr, X, ldx);
}

template <typename T>
void apply_q(lra_ctx* ctx, char trans, int64_t m, int64_t k, const T* V, int64_t ldv, const T* tau,
             T* X, int64_t ldx, int64_t nc) {
  if (k <= 0 || nc <= 0) return;
  const int warps = 4;
  const int64_t blocks = std::min<int64_t>((nc + warps - 1) / warps, (int64_t)ctx->num_sms * 16);
  apply_q_kernel<T><<<(unsigned)blocks, warps * 32, 0, ctx->stream>>>(
      (trans == 't' || trans == 'T' || trans == 'c' || trans == 'C') ? 1 : 0, m, k, V, ldv, tau, X,
      ldx, nc);
  post_launch(ctx, "apply_q_kernel");
}

template <typename T>
void orgqr(lra_ctx* ctx, int64_t m, int64_t k, T* V, int64_t ldv, const T* tau) {
  // Q = H(0) ... H(k-1) [I; 0] built in a separate buffer, then copied back
  const ArenaMark mark = ctx->arena.mark();
  T* Q = ctx->arena.alloc_n<T>((size_t)m * k);
  set_identity(ctx, m, k, Q, m);
  apply_q(ctx, 'n', m, k, V, ldv, tau, Q, m, k);
  copy_matrix(ctx, m, k, Q, m, V, ldv);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
}

template <typename T>
void col_norms(lra_ctx* ctx, int64_t m, int64_t n, const T* A, int64_t lda, T* out) {
  if (n <= 0) return;
  const int warps = 8;
  const int64_t blocks = std::min<int64_t>((n + warps - 1) / warps, (int64_t)ctx->num_sms * 8);
  col_norms_kernel<T><<<(unsigned)blocks, warps * 32, 0, ctx->stream>>>(m, n, A, lda, out);
  post_launch(ctx, "col_norms_kernel");
}

// ---- bounded waits: the limit in force, and a self-test ----------------------------

cudaError_t set_wait_limit_qr(uint64_t ns) { return set_unit_wait_limit(ns); }

namespace {

// Two CTAs meet at a grid barrier whose arrival count starts at the grid
// size, so that no arrival completes it: both wait until the limit runs
// out, the barrier records the time-out and every CTA returns.
__global__ void probe_wait_kernel(GridBar* gb, int* returned) {
  if (!grid_sync(gb)) {
    if (threadIdx.x == 0) atomicAdd(returned, 1);
    return;
  }
  if (threadIdx.x == 0) atomicAdd(returned, 1000);  // the barrier completed: not expected
}

}  // namespace

int probe_grid_wait(lra_ctx* ctx, int* returned) {
  const ArenaMark mark = ctx->arena.mark();
  GridBar* gb = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  int* ret = ctx->arena.alloc_n<int>(1);
  static const GridBar init{2u, 0u, 0, 0};
  LRA_CUDA(cudaMemcpyAsync(gb, &init, sizeof init, cudaMemcpyHostToDevice, ctx->stream));
  LRA_CUDA(cudaMemsetAsync(ret, 0, sizeof(int), ctx->stream));
  void* args[] = {&gb, &ret};
  LRA_CUDA(cudaLaunchCooperativeKernel((const void*)probe_wait_kernel, dim3(2), dim3(32), args, 0, ctx->stream));
  post_launch(ctx, "probe_wait_kernel");
  GridBar hb;
  int hr = 0;
  LRA_CUDA(cudaMemcpyAsync(&hb, gb, sizeof hb, cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(&hr, ret, sizeof hr, cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  *returned = hr;
  return hb.err;
}

// ---- pivoted QR without any device allocation --------------------------------------
//
// Some callers cannot allocate device memory while they factor: a serving
// loop that has reserved all of its device memory up front and must not
// grow, or a host framework that owns the device allocator (a Julia or
// Python memory pool) and does not let a library call cudaMalloc behind its
// back.  For them the pivoted
// QR's scratch -- the partial column norms, the per-CTA pivot candidates,
// the block-stop counters and the grid barrier -- lives in one fixed device
// array of this file, sized for at most kNoAllocMaxCols columns.  Every GPU
// that loads the library keeps the array until the process exits.
//
// The array's host-side name is not a device address; its address is taken
// once per device with cudaGetSymbolAddress, with that device current, on
// the first call that runs on the device, and cached by device ordinal.  So
// the entry point supports the device's primary context (the runtime API's
// context) only: a caller that makes another driver-API context current on
// the same device would be handed the primary context's address.  All calls
// on a device share the array: calls that overlap on the GPU (different
// streams, threads or contexts) race on it and must be serialized by the
// caller.  Each call synchronizes its stream and reads the rank back.

constexpr int64_t kNoAllocMaxCols = 32768;
constexpr int kNoAllocMaxGrid = 1024;
constexpr size_t kNoAllocBytes = 1u << 20;  // 1 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[128] = {};

// device address of the scratch array on the current device (set up once)
void* noalloc_scratch(int device) {
  if (device < 0 || device >= 128) fail(LRA_EINVAL, "device index %d out of range", device);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
    if (!p) fail(LRA_ECUDA, "no-alloc scratch has no device address");
    g_noalloc_ptr[device] = p;
  }
  return g_noalloc_ptr[device];
}

inline unsigned char* carve(unsigned char*& cur, size_t bytes) {
  unsigned char* p = cur;
  cur += (bytes + 255) / 256 * 256;
  return p;
}

}  // namespace

int64_t noalloc_max_cols() { return kNoAllocMaxCols; }

template <typename T>
int64_t geqp3_adap_noalloc(lra_ctx* ctx, int64_t m, int64_t n, T* A, int64_t lda, int64_t* jpvt, T* tau,
                           int64_t kmax, int64_t nb, double atol, double rtol) {
  constexpr int NT = 512;
  if (n <= 0) return 0;
  if (n > kNoAllocMaxCols)
    fail(LRA_EINVAL, "lra_geqp3_adap_noalloc: n = %lld exceeds its limit of %lld columns", (long long)n,
         (long long)kNoAllocMaxCols);
  unsigned char* base = static_cast<unsigned char*>(noalloc_scratch(ctx->device));
  const int64_t vcap = std::min<int64_t>(m, (int64_t)(160 * 1024 / sizeof(T)));
  const size_t dyn_smem = (size_t)vcap * sizeof(T);
  raise_smem_limit(ctx, (const void*)geqp3_kernel<T, NT>);
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, geqp3_kernel<T, NT>, NT, dyn_smem));
  if (per_sm < 1) fail(LRA_ECUDA, "geqp3 kernel cannot be resident");
  const int64_t want = (n + (NT / 32) - 1) / (NT / 32);
  int grid = (int)std::min<int64_t>(std::min<int64_t>((int64_t)ctx->num_sms, want), kNoAllocMaxGrid);
  grid = std::max(grid, 1);

  unsigned char* cur = base;
  QrParams<T> P;
  P.m = m;
  P.n = n;
  P.lda = lda;
  P.A = A;
  P.jpvt = jpvt;
  P.tau = tau;
  P.vn1 = reinterpret_cast<T*>(carve(cur, n * sizeof(T)));
  P.vn2 = reinterpret_cast<T*>(carve(cur, n * sizeof(T)));
  P.flag = reinterpret_cast<int*>(carve(cur, n * sizeof(int)));
  P.part_v = reinterpret_cast<T*>(carve(cur, grid * sizeof(T)));
  P.part_i = reinterpret_cast<int64_t*>(carve(cur, grid * sizeof(int64_t)));
  P.part_d = reinterpret_cast<double*>(carve(cur, grid * sizeof(double)));
  int* small = reinterpret_cast<int*>(carve(cur, 8 * sizeof(int)));
  P.lsticc = small;
  P.bar = reinterpret_cast<GridBar*>(carve(cur, sizeof(GridBar)));
  P.k_out = reinterpret_cast<int64_t*>(carve(cur, sizeof(int64_t)));
  if ((size_t)(cur - base) > kNoAllocBytes) fail(LRA_EINVAL, "no-alloc scratch overflow");
  P.kmax = std::min<int64_t>(kmax, std::min(m, n));
  P.nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(P.kmax, 1)));
  P.atol = atol;
  P.rtol = rtol;
  P.pivot = 1;
  P.vcap = vcap;
  // the array keeps the previous call's contents: clear the counters and
  // the barrier, which must start at zero (the kernel initializes the rest)
  LRA_CUDA(cudaMemsetAsync(small, 0, 8 * sizeof(int), ctx->stream));
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  if (P.kmax <= 0) {
    // nothing to factor (rank 0): the identity permutation, as lra_geqp3_adap
    const unsigned gi = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->num_sms * 4));
    jpvt_identity_kernel<<<gi, 256, 0, ctx->stream>>>(n, jpvt);
    post_launch(ctx, "jpvt_identity_kernel");
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    return 0;
  }
  void* args[] = {&P};
  LRA_CUDA(cudaLaunchCooperativeKernel((const void*)geqp3_kernel<T, NT>, dim3(grid), dim3(NT), args,
                                       dyn_smem, ctx->stream));
  post_launch(ctx, "geqp3_kernel");
  int64_t k = 0;
  GridBar hb;
  LRA_CUDA(cudaMemcpyAsync(&k, P.k_out, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "geqp3: a grid barrier timed out");
  return k;
}

template int64_t geqp3_adap_noalloc<float>(lra_ctx*, int64_t, int64_t, float*, int64_t, int64_t*, float*, int64_t,
                                           int64_t, double, double);
template int64_t geqp3_adap_noalloc<double>(lra_ctx*, int64_t, int64_t, double*, int64_t, int64_t*, double*,
                                            int64_t, int64_t, double, double);

#define INST(T)                                                                                   \
  template int64_t geqp3_adap<T>(lra_ctx*, int64_t, int64_t, T*, int64_t, int64_t*, T*, int64_t,  \
                                 int64_t, double, double, bool);                                 \
  template void trsm_upper<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*, int64_t, const T*); \
  template void apply_q<T>(lra_ctx*, char, int64_t, int64_t, const T*, int64_t, const T*, T*,    \
                           int64_t, int64_t);                                                    \
  template void orgqr<T>(lra_ctx*, int64_t, int64_t, T*, int64_t, const T*);                      \
  template void col_norms<T>(lra_ctx*, int64_t, int64_t, const T*, int64_t, T*);                  \
  template int geqp3_steps_fit<T>(lra_ctx*, int, const int64_t*, int64_t);                        \
  template int geqp3_adap_steps<T>(lra_ctx*, int, const QrStep<T>*, int64_t, double, double, int64_t*);
INST(float)
INST(double)
#undef INST

}  // namespace lra
