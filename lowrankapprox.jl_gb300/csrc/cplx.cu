// Complex element types (ComplexF32 / ComplexF64) on the native path: the
// kernels behind the complex drivers of api.cpp.  They follow the same
// reference functions as the real kernels, with the complex rules of LAPACK:
// the pivoted QR keeps xLAQPS's pivot order, downdate and recompute trigger
// and early block exit for ZLAQPS / CLAQPS (src/lapack.jl:117-139), its
// reflectors are xLARFG's complex ones (beta real, tau complex), and every
// transpose of the reference's A' is a conjugate transpose.  These are
// straightforward SIMT kernels: the complex paths are correct and
// complete, not tuned like the real ones.

#include <algorithm>
#include <cfloat>
#include <vector>

#include "common.cuh"
#include "cplx.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename R>
using C = cx<R>;

inline unsigned grid_for_c(lra_ctx* ctx, int64_t n, int t) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, (int64_t)ctx->num_sms * 8));
}

// ---- GEMM: C = alpha op(A) op(B) + beta C, op 0 = n, 1 = t, 2 = c ------------------
template <typename R, int OA, int OB>
__global__ void __launch_bounds__(256) cgemm_kernel(int64_t M, int64_t N, int64_t K, C<R> alpha,
                                                    const C<R>* __restrict__ A, int64_t lda,
                                                    const C<R>* __restrict__ B, int64_t ldb, C<R> beta,
                                                    C<R>* __restrict__ Cm, int64_t ldc) {
  constexpr int BM = 32, BN = 32, BK = 8;
  __shared__ C<R> As[BK][BM + 1];
  __shared__ C<R> Bs[BK][BN + 1];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int64_t tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
  const bool zero_beta = beta.re == R(0) && beta.im == R(0);
  for (int64_t tile = blockIdx.x; tile < tiles_m * tiles_n; tile += gridDim.x) {
    const int64_t m0 = (tile % tiles_m) * BM, n0 = (tile / tiles_m) * BN;
    C<R> acc[2][2] = {{C<R>(0), C<R>(0)}, {C<R>(0), C<R>(0)}};
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
      {
        const int i = tid % BM, k = tid / BM;
        const int64_t gi = m0 + i, gk = k0 + k;
        C<R> v(0);
        if (gi < M && gk < K) v = OA == 0 ? A[gi + gk * lda] : A[gk + gi * lda];
        if (OA == 2) v = conj(v);
        As[k][i] = v;
      }
      {
        const int k = tid % BK, j = tid / BK;
        const int64_t gj = n0 + j, gk = k0 + k;
        C<R> v(0);
        if (gj < N && gk < K) v = OB == 0 ? B[gk + gj * ldb] : B[gj + gk * ldb];
        if (OB == 2) v = conj(v);
        Bs[k][j] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        const C<R> a0 = As[kk][ty], a1 = As[kk][ty + 16], b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
        acc[0][0] += a0 * b0;
        acc[0][1] += a0 * b1;
        acc[1][0] += a1 * b0;
        acc[1][1] += a1 * b1;
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int64_t gi = m0 + ty + 16 * i, gj = n0 + tx + 16 * j;
        if (gi < M && gj < N) {
          C<R>* c = Cm + gi + gj * ldc;
          *c = zero_beta ? alpha * acc[i][j] : alpha * acc[i][j] + beta * *c;
        }
      }
  }
}

template <typename R>
__global__ void cconj_kernel(int64_t m, int64_t n, C<R>* A, int64_t lda) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m * n; t += (int64_t)gridDim.x * blockDim.x) {
    C<R>& a = A[t % m + (t / m) * lda];
    a.im = -a.im;
  }
}

// ---- norms ------------------------------------------------------------------------
// ||x|| of a complex vector by one warp, at a power-of-two scale set by the
// largest component (no overflow or underflow of the squares)
template <typename R>
__device__ R warp_cnrm2(const C<R>* x, int64_t len, int lane) {
  R mx = 0;
  for (int64_t i = lane; i < len; i += 32) mx = fmax(mx, fmax(fabs(x[i].re), fabs(x[i].im)));
  mx = warp_max(mx);
  if (!(mx > R(0)) || !(mx <= Real<R>::big)) return mx;
  const int e = ilogb(mx);
  const R sc = scalbn(R(1), -e);
  R s = 0;
  for (int64_t i = lane; i < len; i += 32) {
    const R a = x[i].re * sc, b = x[i].im * sc;
    s += a * a + b * b;
  }
  s = warp_sum(s);
  return scalbn(sqrt(s), e);
}

template <typename R>
__device__ R block_cnrm2(const C<R>* x, int64_t len, R* red) {
  R mx = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) mx = fmax(mx, fmax(fabs(x[i].re), fabs(x[i].im)));
  mx = block_max(mx, red);
  if (!(mx > R(0)) || !(mx <= Real<R>::big)) return mx;
  const int e = ilogb(mx);
  const R sc = scalbn(R(1), -e);
  R s = 0;
  for (int64_t i = threadIdx.x; i < len; i += blockDim.x) {
    const R a = x[i].re * sc, b = x[i].im * sc;
    s += a * a + b * b;
  }
  s = block_sum(s, red);
  return scalbn(sqrt(s), e);
}

template <typename R>
__global__ void ccol_norms_kernel(int64_t m, int64_t n, const C<R>* A, int64_t lda, R* out) {
  const int lane = threadIdx.x & 31, w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w; j < n; j += nw) {
    const R v = warp_cnrm2(A + j * lda, m, lane);
    if (lane == 0) out[j] = v;
  }
}

// sqrt(x^2 + y^2 + z^2) without overflow (LAPACK's xLAPY3 rule)
template <typename R>
__device__ __forceinline__ R lapy3(R x, R y, R z) {
  x = fabs(x);
  y = fabs(y);
  z = fabs(z);
  const R w = fmax(x, fmax(y, z));
  if (w == R(0)) return x + y + z;
  const R a = x / w, b = y / w, c = z / w;
  return w * sqrt(a * a + b * b + c * c);
}

// The complex reflector of xLARFG: H^H [alpha; x] = [beta; 0] with
// H = I - tau v v^H, v = [1; scal x], beta real.  Returns tau, beta, scal.
template <typename R>
__device__ void clarfg(C<R> alpha, R xnorm, C<R>& tau, R& beta, C<R>& scal) {
  R alphr = alpha.re, alphi = alpha.im;
  if (xnorm == R(0) && alphi == R(0)) {
    tau = C<R>(0);
    beta = alphr;
    scal = C<R>(1);
    return;
  }
  beta = -copysign(lapy3(alphr, alphi, xnorm), alphr);
  const R safmin = Real<R>::safmin / Real<R>::eps, rsafmn = R(1) / safmin;
  int knt = 0;
  R xs = xnorm;
  R mul = 1;
  if (fabs(beta) < safmin) {
    do {
      ++knt;
      xs *= rsafmn;
      beta *= rsafmn;
      alphi *= rsafmn;
      alphr *= rsafmn;
      mul *= rsafmn;
    } while (fabs(beta) < safmin && knt < 20);
    beta = -copysign(lapy3(alphr, alphi, xs), alphr);
  }
  tau = C<R>((beta - alphr) / beta, -alphi / beta);
  scal = mul * cdiv(C<R>(1), C<R>(alphr - beta, alphi));
  for (int j = 0; j < knt; ++j) beta *= safmin;
}

// ---- pivoted QR (xLAQPS for complex types, column by column) -------------------------
//
// One cooperative launch.  Per pivot c: the CTAs' argmax partials of the
// partial norms (ties: the smaller column, IxAMAX), one grid barrier; the
// swap of the pivot column into place, one grid barrier; every CTA then
// forms the reflector of column c itself (the same arithmetic in each CTA)
// and applies H^H to its own trailing columns, a warp per column, with the
// norm downdate of xLAQPS.  A column whose downdate is unreliable
// (tol3z) has its norm recomputed from the updated column at once and ends
// the block, as xLAQPS ends the block there and recomputes it; the rank
// test of geqp3_adap_main! (src/pqr.jl:407-415) runs at each block end.
// Column c is finalized (beta, scal x) by CTA 0 after the next barrier,
// when no CTA reads it any more.
template <typename R>
struct CQrParams {
  int64_t m, n, lda;
  C<R>* A;
  int64_t* jpvt;
  C<R>* tau;
  R* vn1;
  R* vn2;
  R* part_v;
  int64_t* part_i;
  int* part_f;
  GridBar* bar;
  int64_t kmax, nb;
  double atol, rtol;
  int pivot;
  int64_t* k_out;
};

template <typename R, int NT>
__global__ void __launch_bounds__(NT) cgeqp3_kernel(CQrParams<R> P) {
  constexpr int NW = NT / 32;
  __shared__ R s_red[32];
  __shared__ int64_t s_ri[32];
  __shared__ int64_t s_pvt;
  __shared__ int s_flag, s_anyflag;
  __shared__ C<R> s_tau, s_scal;
  __shared__ R s_beta;
  const int G = gridDim.x, b = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t m = P.m, n = P.n, lda = P.lda;
  const int64_t c0 = n * b / G, c1 = n * (b + 1) / G;
  const int64_t lastrk = m < n ? m : n;
  const R tol3z = sqrt(Real<R>::eps);
  C<R>* A = P.A;

  // initial norms of the CTA's columns (and the identity permutation)
  for (int64_t j = c0 + wid; j < c1; j += NW) {
    const R v = warp_cnrm2(A + j * lda, m, lane);
    if (lane == 0) {
      P.vn1[j] = P.vn2[j] = v;
      P.jpvt[j] = j + 1;
    }
  }
  __syncthreads();
  R lmax = 0;
  for (int64_t j = c0 + threadIdx.x; j < c1; j += NT) lmax = fmax(lmax, P.vn1[j]);
  lmax = block_max(lmax, s_red);
  if (threadIdx.x == 0) P.part_v[b] = lmax;
  if (!grid_sync(P.bar)) return;
  R maxnrm = 0;
  for (int bb = threadIdx.x; bb < G; bb += NT) maxnrm = fmax(maxnrm, *((volatile R*)(P.part_v + bb)));
  maxnrm = block_max(maxnrm, s_red);
  const R ptol = (R)fmax(P.atol, P.rtol * (double)maxnrm);
  if (!grid_sync(P.bar)) return;  // everyone read part_v before it is reused

  // the argmax partial of this CTA over positions >= from, and its flag
  auto publish = [&](int64_t from, int flag) {
    R v = -1;
    int64_t i = n;
    for (int64_t j = (from > c0 ? from : c0) + threadIdx.x; j < c1; j += NT) argmax_merge(v, i, P.vn1[j], j);
    warp_argmax(v, i);
    if (lane == 0) {
      s_red[wid] = v;
      s_ri[wid] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < NW; ++w) argmax_merge(v, i, s_red[w], s_ri[w]);
      P.part_v[b] = v;
      P.part_i[b] = i;
      P.part_f[b] = flag;
    }
    __syncthreads();
  };
  // after the barrier: the global pivot and the OR of the flags
  auto collect = [&]() {
    if (threadIdx.x == 0) {
      R v = -1;
      int64_t i = n;
      int f = 0;
      for (int bb = 0; bb < G; ++bb) {
        argmax_merge(v, i, *((volatile R*)(P.part_v + bb)), *((volatile int64_t*)(P.part_i + bb)));
        f |= *((volatile int*)(P.part_f + bb));
      }
      s_pvt = i;
      s_anyflag = f;
    }
    __syncthreads();
  };

  publish(0, 0);
  if (!grid_sync(P.bar)) return;
  collect();
  int64_t kres = P.kmax;
  int64_t c = 0;
  C<R> fin_scal(1);
  R fin_beta = 0;
  int64_t fin_col = -1;
  while (c < P.kmax) {
    const int64_t jb = min(P.nb, P.kmax - c);
    int64_t kk = 0, first_small = -1;
    bool last_small = false, block_end = false;
    while (kk < jb && !block_end) {
      if (P.pivot) {
        const int64_t pvt = s_pvt;
        if (pvt != c && pvt < n) {
          for (int64_t i = (int64_t)b * NT + threadIdx.x; i < m; i += (int64_t)G * NT) {
            const C<R> t = A[i + c * lda];
            A[i + c * lda] = A[i + pvt * lda];
            A[i + pvt * lda] = t;
          }
          if (b == 0 && threadIdx.x == 0) {
            const int64_t t = P.jpvt[c];
            P.jpvt[c] = P.jpvt[pvt];
            P.jpvt[pvt] = t;
            P.vn1[pvt] = P.vn1[c];
            P.vn2[pvt] = P.vn2[c];
          }
        }
        if (!grid_sync(P.bar)) return;
      }
      // the reflector of column c (rows c..m-1), in every CTA
      const C<R>* col = A + c * lda;
      const R xnorm = c + 1 < m ? block_cnrm2(col + c + 1, m - c - 1, s_red) : R(0);
      if (threadIdx.x == 0) {
        C<R> t, sc;
        R bt;
        clarfg(col[c], xnorm, t, bt, sc);
        s_tau = t;
        s_scal = sc;
        s_beta = bt;
        s_flag = 0;
        if (b == 0) P.tau[c] = t;
      }
      __syncthreads();
      const C<R> tau = s_tau, scal = s_scal;
      const C<R> ctau = conj(tau);
      // H^H applied to the CTA's trailing columns, a warp per column
      int flag = 0;
      for (int64_t j = (c + 1 > c0 ? c + 1 : c0) + wid; j < c1; j += NW) {
        C<R>* a = A + j * lda;
        if (tau.re != R(0) || tau.im != R(0)) {
          // w = v^H a, v = [1; scal x]
          C<R> w(0);
          for (int64_t i = c + 1 + lane; i < m; i += 32) w += cmulc(scal * col[i], a[i]);
          w.re = warp_sum(w.re);
          w.im = warp_sum(w.im);
          w += a[c];
          const C<R> f = ctau * w;
          for (int64_t i = c + 1 + lane; i < m; i += 32) a[i] -= f * (scal * col[i]);
          if (lane == 0) a[c] -= f;
        }
        __syncwarp();
        if (P.pivot && c < lastrk - 1) {
          R v1 = P.vn1[j];
          bool recompute = false;
          if (v1 != R(0)) {
            R temp = cabs(a[c]) / v1;
            temp = fmax(R(0), (R(1) + temp) * (R(1) - temp));
            const R r = v1 / P.vn2[j];
            const R temp2 = temp * r * r;
            if (temp2 <= tol3z)
              recompute = true;
            else if (lane == 0)
              P.vn1[j] = v1 * sqrt(temp);
          }
          if (recompute) {
            const R nr = warp_cnrm2(a + c + 1, m - c - 1, lane);
            if (lane == 0) P.vn1[j] = P.vn2[j] = nr;
            flag = 1;
          }
        }
        __syncwarp();
      }
      if (flag && lane == 0) atomicOr(&s_flag, 1);
      const R beta = s_beta;
      const bool small = fabs(beta) <= ptol;
      if (small && first_small < 0) first_small = c;
      last_small = small;
      fin_scal = scal;
      fin_beta = beta;
      fin_col = c;
      __syncthreads();
      ++c;
      ++kk;
      publish(c, s_flag);
      if (!grid_sync(P.bar)) return;
      collect();
      // column c - 1 is read by no one now: CTA 0 writes beta and v below it
      if (b == 0 && fin_col >= 0) {
        C<R>* fc = A + fin_col * lda;
        for (int64_t i = fin_col + 1 + threadIdx.x; i < m; i += NT) fc[i] = fin_scal * fc[i];
        if (threadIdx.x == 0) fc[fin_col] = C<R>(fin_beta, R(0));
      }
      block_end = P.pivot && s_anyflag;
    }
    if (P.pivot && last_small) {
      kres = first_small;
      break;
    }
  }
  if (b == 0 && threadIdx.x == 0) *P.k_out = kres;
}

// ---- Householder application, a warp per column of X ------------------------------
// trans 0: X <- Q X = H_0 H_1 ... H_{k-1} X; trans 1: X <- Q^H X
template <typename R>
__global__ void capply_q_kernel(int trans, int64_t m, int64_t k, const C<R>* __restrict__ V, int64_t ldv,
                                const C<R>* __restrict__ tau, C<R>* __restrict__ X, int64_t ldx, int64_t nc) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = w; j < nc; j += nw) {
    C<R>* x = X + j * ldx;
    for (int64_t s = 0; s < k; ++s) {
      const int64_t i0 = trans ? s : k - 1 - s;
      const C<R> t = trans ? conj(tau[i0]) : tau[i0];
      if (t.re == R(0) && t.im == R(0)) continue;
      const C<R>* v = V + i0 * ldv;
      C<R> d(0);
      for (int64_t i = i0 + 1 + lane; i < m; i += 32) d += cmulc(v[i], x[i]);
      d.re = warp_sum(d.re);
      d.im = warp_sum(d.im);
      d += x[i0];
      const C<R> f = t * d;
      for (int64_t i = i0 + 1 + lane; i < m; i += 32) x[i] -= f * v[i];
      if (lane == 0) x[i0] -= f;
      __syncwarp();
    }
  }
}

// ---- X <- triu(R)^{-1} X by back substitution, a thread per column --------------------
template <typename R>
__global__ void ctrsm_kernel(int64_t k, int64_t nrhs, const C<R>* __restrict__ Rm, int64_t ldr, C<R>* X,
                             int64_t ldx) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nrhs; j += (int64_t)gridDim.x * blockDim.x) {
    C<R>* x = X + j * ldx;
    for (int64_t i = k - 1; i >= 0; --i) {
      C<R> s = x[i];
      for (int64_t l = i + 1; l < k; ++l) s -= Rm[i + l * ldr] * x[l];
      x[i] = cdiv(s, Rm[i + i * ldr]);
    }
  }
}

// ---- one-sided Jacobi SVD of a k x k matrix, one CTA --------------------------------
// X = U diag(S) V^H: the columns of X are rotated pairwise until orthogonal
// (round-robin order, a warp per pair of a round); S are the column norms
// and X ends as U.  Each rotation J = D R with D = diag(1, e^{-i phi}),
// gamma = x_p^H x_q = |gamma| e^{i phi}, R the real Jacobi rotation of
// [[alpha, |gamma|], [|gamma|, beta]].
template <typename R>
__global__ void __launch_bounds__(1024) cjacobi_kernel(int k, C<R>* X, int64_t ldx, C<R>* V, int64_t ldv, R* S,
                                                       int maxsweep, R tol) {
  __shared__ int s_rot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  for (int64_t t = threadIdx.x; t < (int64_t)k * k; t += blockDim.x) {
    const int r = (int)(t % k), c = (int)(t / k);
    V[r + c * ldv] = C<R>(r == c ? R(1) : R(0));
  }
  __syncthreads();
  const int kk = k + (k & 1);
  for (int sweep = 0; sweep < maxsweep; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    for (int round = 0; round < kk - 1; ++round) {
      for (int pr = wid; pr < kk / 2; pr += nwarp) {
        int p, q;
        if (pr == 0) {
          p = round;
          q = kk - 1;
        } else {
          p = (round + pr) % (kk - 1);
          q = (round - pr + (kk - 1)) % (kk - 1);
        }
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        if (q >= k) continue;
        C<R>* xp = X + (int64_t)p * ldx;
        C<R>* xq = X + (int64_t)q * ldx;
        R al = 0, be = 0;
        C<R> ga(0);
        for (int i = lane; i < k; i += 32) {
          al += abs2(xp[i]);
          be += abs2(xq[i]);
          ga += cmulc(xp[i], xq[i]);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga.re = warp_sum(ga.re);
        ga.im = warp_sum(ga.im);
        const R g = cabs(ga);
        if (!(al > R(0)) || !(be > R(0)) || !(g > tol * sqrt(al) * sqrt(be))) continue;
        const R zeta = (be - al) / (R(2) * g);
        const R t = (zeta >= R(0) ? R(1) : R(-1)) / (fabs(zeta) + sqrt(R(1) + zeta * zeta));
        const R cs = R(1) / sqrt(R(1) + t * t), sn = cs * t;
        const C<R> e = C<R>(ga.re / g, -ga.im / g);  // e^{-i phi}
        for (int i = lane; i < k; i += 32) {
          const C<R> a = xp[i], bq = e * xq[i];
          xp[i] = cs * a - sn * bq;
          xq[i] = sn * a + cs * bq;
        }
        C<R>* vp = V + (int64_t)p * ldv;
        C<R>* vq = V + (int64_t)q * ldv;
        for (int i = lane; i < k; i += 32) {
          const C<R> a = vp[i], bq = e * vq[i];
          vp[i] = cs * a - sn * bq;
          vq[i] = sn * a + cs * bq;
        }
        if (lane == 0) s_rot = 1;
      }
      __syncthreads();
    }
    if (!s_rot) break;
  }
  // singular values, and U = X diag(1 / S)
  for (int j = wid; j < k; j += nwarp) {
    C<R>* x = X + (int64_t)j * ldx;
    const R s = warp_cnrm2(x, k, lane);
    if (lane == 0) S[j] = s;
    if (s > R(0))
      for (int i = lane; i < k; i += 32) x[i] = (R(1) / s) * x[i];
  }
}

// ---- Hermitian test: A == A^H exactly (the reference's ishermitian) -------------------
template <typename R>
__global__ void cherm_kernel(int64_t n, const C<R>* A, int64_t lda, int* bad) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    if (i > j) continue;
    const C<R> a = A[i + j * lda], b = A[j + i * lda];
    if (a.re != b.re || a.im != -b.im) *bad = 1;
  }
}

// B <- (B + B^H) / 2 (hermitianize!, src/util.jl:31-45, both triangles)
template <typename R>
__global__ void chermitianize_kernel(int64_t n, C<R>* B, int64_t ldb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, j = t / n;
    if (i > j) continue;
    const C<R> a = B[i + j * ldb], b = B[j + i * ldb];
    const C<R> h = R(0.5) * (a + conj(b));
    B[i + j * ldb] = h;
    B[j + i * ldb] = conj(h);
  }
}

template <typename R>
__global__ void cadd_diag_kernel(int64_t n, C<R>* A, int64_t lda, R s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    A[i + i * lda].re += s;
}

// ---- sketches ---------------------------------------------------------------------
// unit phases d_t = g_t / |g_t| from pairs of Gaussians (srft_rand for
// complex types, src/sketch.jl:345-351)
template <typename R>
__global__ void cphase_kernel(int64_t n, const double* __restrict__ g, C<R>* d) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const C<R> z((R)g[2 * t], (R)g[2 * t + 1]);
    const R a = cabs(z);
    d[t] = a > R(0) ? C<R>(z.re / a, z.im / a) : C<R>(1);
  }
}

// B(i, col) = sum_t d_t op(A)(t, col) e^{-2 pi i f_i t / M}, f_i = idx_i - 1:
// the SRFT of complex types samples the DFT of d .* x at the frequencies
// idx (srft_apply!, src/sketch.jl:452-472); the phase is reduced exactly
// as (f t) mod M
// the operand accessor of the gather-type sketches: element (t, col) is
// A(col, t) when mode & 1 (transposed) else A(t, col), conjugated when mode & 2
template <typename R>
__device__ __forceinline__ C<R> opel(int mode, const C<R>* A, int64_t lda, int64_t t, int64_t col) {
  const C<R> a = (mode & 1) ? A[col + t * lda] : A[t + col * lda];
  return (mode & 2) ? conj(a) : a;
}

template <typename R>
__global__ void csrft_direct_kernel(int mode, int64_t M, int64_t N, const C<R>* __restrict__ A, int64_t lda,
                                    const C<R>* __restrict__ d, const int64_t* __restrict__ idx, int64_t order,
                                    C<R>* B, int64_t ldb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < order * N;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % order, col = t / order;
    const int64_t f = idx[i] - 1;
    C<R> acc(0);
    for (int64_t s = 0; s < M; ++s) {
      const C<R> a = opel(mode, A, lda, s, col);
      const int64_t r = (f * s) % M;  // f, s < M < 2^31
      R sn, cs;
      if constexpr (sizeof(R) == 8)
        sincospi(-2.0 * (double)r / (double)M, &sn, &cs);
      else
        sincospif(-2.0f * (float)((double)r / (double)M), &sn, &cs);
      acc += C<R>(cs, sn) * (d[s] * a);
    }
    B[i + col * ldb] = acc;
  }
}

// B(i, :) = sum over the rows r of group i of g_r op(A)(perm_r, :)
// (SparseRandomGaussian, src/sketch.jl:571-653), groups of fld(M - i, l) + 1
template <typename R>
__global__ void csprn_kernel(int mode, int64_t M, int64_t N, const C<R>* __restrict__ A, int64_t lda,
                             const int64_t* __restrict__ perm, const C<R>* __restrict__ g,
                             const int64_t* __restrict__ start, int64_t order, C<R>* B, int64_t ldb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < order * N;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % order, col = t / order;
    C<R> acc(0);
    for (int64_t l = start[i]; l < start[i + 1]; ++l) {
      const C<R> a = opel(mode, A, lda, perm[l] - 1, col);
      acc += g[l] * a;
    }
    B[i + col * ldb] = acc;
  }
}

// B(i, :) = op(A)(rows_i, :) (RandomSubset, src/sketch.jl:248-293)
template <typename R>
__global__ void csub_kernel(int mode, int64_t N, const C<R>* __restrict__ A, int64_t lda,
                            const int64_t* __restrict__ rows, int64_t order, C<R>* B, int64_t ldb) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < order * N;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % order, col = t / order;
    B[i + col * ldb] = opel(mode, A, lda, rows[i] - 1, col);
  }
}

// ---- maxdet on complex T: max |T| (ties: the last index), the swap and the
// Sherman-Morrison update T -= w1 T(i, :) / (1 + w1_i) (maxdet_update!,
// src/pqr.jl:479-501; BLAS.ger! conjugates its second vector, which holds
// conj(T(i, :)))
template <typename R>
__global__ void cabsmax_kernel(int64_t total, const C<R>* T, double* outv, int64_t* outi) {
  __shared__ double sv[32];
  __shared__ int64_t si[32];
  double v = -1;
  int64_t i = -1;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x) {
    const double a = (double)cabs(T[t]);
    if (a > v || (a == v && t > i)) {
      v = a;
      i = t;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
    const int64_t i2 = __shfl_xor_sync(0xffffffffu, i, o);
    if (v2 > v || (v2 == v && i2 > i)) {
      v = v2;
      i = i2;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = i;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (sv[w] > v || (sv[w] == v && si[w] > i)) {
        v = sv[w];
        i = si[w];
      }
    *outv = v;
    *outi = i;
  }
}

template <typename R>
__global__ void cmaxdet_prep_kernel(int64_t k, int64_t nr, C<R>* T, int64_t* jpvt, const int64_t* pidx, C<R>* w1,
                                    C<R>* w2) {
  const int64_t idx = *pidx, i = idx % k, j = idx / k;
  for (int64_t l = threadIdx.x; l < k; l += blockDim.x) {
    C<R> v = T[l + j * k];
    if (l == i) v -= C<R>(1);
    w1[l] = v;
  }
  __syncthreads();
  for (int64_t l = threadIdx.x; l < k; l += blockDim.x) T[l + j * k] = C<R>(l == i ? R(1) : R(0));
  __syncthreads();
  for (int64_t l = threadIdx.x; l < nr; l += blockDim.x) w2[l] = T[i + l * k];
  if (threadIdx.x == 0) {
    const int64_t t = jpvt[i];
    jpvt[i] = jpvt[k + j];
    jpvt[k + j] = t;
  }
}

template <typename R>
__global__ void cmaxdet_ger_kernel(int64_t k, int64_t nr, C<R>* T, const int64_t* pidx, const C<R>* w1,
                                   const C<R>* w2) {
  const int64_t i = *pidx % k;
  const C<R> alpha = cdiv(C<R>(-1), C<R>(1) + w1[i]);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < k * nr; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % k, c = t / k;
    T[t] += alpha * (w1[r] * w2[c]);
  }
}

// R1(:, i) += R1 w1 (maxdet_update!'s R part), a thread per row, then the add
template <typename R>
__global__ void cmaxdet_r1_gemv_kernel(int64_t k, const C<R>* R1, int64_t ldr, const C<R>* w1, C<R>* y) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x) {
    C<R> acc(0);
    for (int64_t c = 0; c < k; ++c) acc += R1[l + c * ldr] * w1[c];
    y[l] = acc;
  }
}
template <typename R>
__global__ void cmaxdet_r1_add_kernel(int64_t k, C<R>* R1, int64_t ldr, const int64_t* pidx, const C<R>* y) {
  const int64_t i = *pidx % k;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < k; l += (int64_t)gridDim.x * blockDim.x)
    R1[l + i * ldr] += y[l];
}

// pheigorth! (src/pheig.jl:342-364): v_j -= (v_i^H v_j) v_i inside each
// cluster [cl[2c], cl[2c+1]), one CTA per cluster, pairs in order
template <typename R>
__global__ void ccluster_orth_kernel(int64_t n, C<R>* Z, int64_t ldz, const int64_t* cl) {
  __shared__ R red[32];
  const int64_t a = cl[2 * blockIdx.x], e = cl[2 * blockIdx.x + 1];
  for (int64_t i = a; i < e; ++i)
    for (int64_t j = i + 1; j < e; ++j) {
      const C<R>* vi = Z + i * ldz;
      C<R>* vj = Z + j * ldz;
      C<R> d(0);
      for (int64_t r = threadIdx.x; r < n; r += blockDim.x) d += cmulc(vi[r], vj[r]);
      d.re = block_sum(d.re, red);
      d.im = block_sum(d.im, red);
      for (int64_t r = threadIdx.x; r < n; r += blockDim.x) vj[r] -= d * vi[r];
      __syncthreads();
    }
}

}  // namespace

// ---- launchers ----------------------------------------------------------------------

// the accessor mode of a sketch operand: 'n' A(t, col); 'c' conj(A(col, t));
// 't' A(col, t); 'j' conj(A(t, col))
inline int cmode(char m) { return m == 'n' ? 0 : m == 'c' ? 3 : m == 't' ? 1 : 2; }

template <typename R>
void cgemm(lra_ctx* ctx, char ta, char tb, int64_t m, int64_t n, int64_t k, cx<R> alpha, const cx<R>* A,
           int64_t lda, const cx<R>* B, int64_t ldb, cx<R> beta, cx<R>* Cm, int64_t ldc) {
  if (m <= 0 || n <= 0) return;
  const int oa = ta == 'n' ? 0 : (ta == 't' ? 1 : 2), ob = tb == 'n' ? 0 : (tb == 't' ? 1 : 2);
  const int64_t tiles = ((m + 31) / 32) * ((n + 31) / 32);
  const unsigned g = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->num_sms * 8);
#define CG(OA, OB)                                                                                             \
  if (oa == OA && ob == OB) {                                                                                  \
    cgemm_kernel<R, OA, OB><<<g, 256, 0, ctx->stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc);        \
    post_launch(ctx, "cgemm_kernel");                                                                          \
    return;                                                                                                    \
  }
  CG(0, 0) CG(0, 1) CG(0, 2) CG(1, 0) CG(1, 1) CG(1, 2) CG(2, 0) CG(2, 1) CG(2, 2)
#undef CG
}

template <typename R>
void cadjoint(lra_ctx* ctx, int64_t m, int64_t n, const cx<R>* src, int64_t lds, cx<R>* dst, int64_t ldd) {
  if (m <= 0 || n <= 0) return;
  transpose<cx<R>>(ctx, m, n, src, lds, dst, ldd);
  cconj_kernel<R><<<grid_for_c(ctx, m * n, 256), 256, 0, ctx->stream>>>(n, m, dst, ldd);
  post_launch(ctx, "cconj_kernel");
}

template <typename R>
void cconj(lra_ctx* ctx, int64_t m, int64_t n, cx<R>* A, int64_t lda) {
  if (m <= 0 || n <= 0) return;
  cconj_kernel<R><<<grid_for_c(ctx, m * n, 256), 256, 0, ctx->stream>>>(m, n, A, lda);
  post_launch(ctx, "cconj_kernel");
}

template <typename R>
void ccol_norms(lra_ctx* ctx, int64_t m, int64_t n, const cx<R>* A, int64_t lda, R* out) {
  if (n <= 0) return;
  ccol_norms_kernel<R><<<grid_for_c(ctx, n, 8), 256, 0, ctx->stream>>>(m, n, A, lda, out);
  post_launch(ctx, "ccol_norms_kernel");
}

template <typename R>
int64_t cgeqp3(lra_ctx* ctx, int64_t m, int64_t n, cx<R>* A, int64_t lda, int64_t* jpvt, cx<R>* tau, int64_t kmax,
               int64_t nb, double atol, double rtol, bool pivot) {
  constexpr int NT = 256;
  if (n <= 0) return 0;
  const ArenaMark mark = ctx->arena.mark();
  const int64_t want = (n + (NT / 32) - 1) / (NT / 32);
  int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms, want));
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cgeqp3_kernel<R, NT>, NT, 0));
  if (per_sm < 1) fail(LRA_ECUDA, "complex QR kernel cannot be resident");
  CQrParams<R> P;
  P.m = m;
  P.n = n;
  P.lda = lda;
  P.A = A;
  P.jpvt = jpvt;
  P.tau = tau;
  P.vn1 = ctx->arena.alloc_n<R>(n);
  P.vn2 = ctx->arena.alloc_n<R>(n);
  P.part_v = ctx->arena.alloc_n<R>(grid);
  P.part_i = ctx->arena.alloc_n<int64_t>(grid);
  P.part_f = ctx->arena.alloc_n<int>(grid);
  P.bar = reinterpret_cast<GridBar*>(ctx->arena.alloc(sizeof(GridBar)));
  P.kmax = std::min<int64_t>(kmax, std::min(m, n));
  P.nb = std::max<int64_t>(1, std::min<int64_t>(nb, std::max<int64_t>(P.kmax, 1)));
  P.atol = atol;
  P.rtol = rtol;
  P.pivot = pivot ? 1 : 0;
  P.k_out = ctx->arena.alloc_n<int64_t>(1);
  LRA_CUDA(cudaMemsetAsync(P.bar, 0, sizeof(GridBar), ctx->stream));
  if (P.kmax <= 0) {
    std::vector<int64_t> id(n);
    for (int64_t i = 0; i < n; ++i) id[i] = i + 1;
    if (pivot)
      LRA_CUDA(cudaMemcpyAsync(jpvt, id.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->stream));
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->arena.release(mark);
    return 0;
  }
  if (!pivot) P.jpvt = ctx->arena.alloc_n<int64_t>(n);
  void* args[] = {&P};
  LRA_CUDA(cudaLaunchCooperativeKernel((const void*)cgeqp3_kernel<R, NT>, dim3(grid), dim3(NT), args, 0,
                                       ctx->stream));
  post_launch(ctx, "cgeqp3_kernel");
  int64_t k = 0;
  GridBar hb;
  LRA_CUDA(cudaMemcpyAsync(&k, P.k_out, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaMemcpyAsync(&hb, P.bar, sizeof(GridBar), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  if (hb.err != 0) fail(LRA_ETIMEDOUT, "complex geqp3: a grid barrier timed out");
  return k;
}

template <typename R>
void capply_q(lra_ctx* ctx, char trans, int64_t m, int64_t k, const cx<R>* V, int64_t ldv, const cx<R>* tau,
              cx<R>* X, int64_t ldx, int64_t nc) {
  if (k <= 0 || nc <= 0) return;
  capply_q_kernel<R><<<grid_for_c(ctx, nc, 4), 128, 0, ctx->stream>>>(trans == 'n' ? 0 : 1, m, k, V, ldv, tau, X,
                                                                     ldx, nc);
  post_launch(ctx, "capply_q_kernel");
}

template <typename R>
void corgqr(lra_ctx* ctx, int64_t m, int64_t k, cx<R>* V, int64_t ldv, const cx<R>* tau) {
  if (k <= 0 || m <= 0) return;
  const ArenaMark mark = ctx->arena.mark();
  cx<R>* Q = ctx->arena.alloc_n<cx<R>>((size_t)m * k);
  set_identity<cx<R>>(ctx, m, k, Q, m);
  capply_q<R>(ctx, 'n', m, k, V, ldv, tau, Q, m, k);
  copy_matrix<cx<R>>(ctx, m, k, Q, m, V, ldv);
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
}

template <typename R>
void ctrsm_upper(lra_ctx* ctx, int64_t k, int64_t nrhs, const cx<R>* Rm, int64_t ldr, cx<R>* X, int64_t ldx) {
  if (k <= 0 || nrhs <= 0) return;
  ctrsm_kernel<R><<<grid_for_c(ctx, nrhs, 128), 128, 0, ctx->stream>>>(k, nrhs, Rm, ldr, X, ldx);
  post_launch(ctx, "ctrsm_kernel");
}

template <typename R>
void cjacobi_svd(lra_ctx* ctx, int64_t k, cx<R>* X, int64_t ldx, cx<R>* V, int64_t ldv, R* S) {
  if (k <= 0) return;
  const R tol = Real<R>::eps * (R)std::max<int64_t>(k, 4);
  cjacobi_kernel<R><<<1, 1024, 0, ctx->stream>>>((int)k, X, ldx, V, ldv, S, 60, tol);
  post_launch(ctx, "cjacobi_kernel");
}

template <typename R>
bool cis_hermitian(lra_ctx* ctx, int64_t n, const cx<R>* A, int64_t lda) {
  if (n <= 0) return true;
  const ArenaMark mark = ctx->arena.mark();
  int* bad = ctx->arena.alloc_n<int>(1);
  LRA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  cherm_kernel<R><<<grid_for_c(ctx, n * n, 256), 256, 0, ctx->stream>>>(n, A, lda, bad);
  post_launch(ctx, "cherm_kernel");
  int h = 0;
  LRA_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mark);
  return h == 0;
}

template <typename R>
void chermitianize(lra_ctx* ctx, int64_t n, cx<R>* B, int64_t ldb) {
  if (n <= 0) return;
  chermitianize_kernel<R><<<grid_for_c(ctx, n * n, 256), 256, 0, ctx->stream>>>(n, B, ldb);
  post_launch(ctx, "chermitianize_kernel");
}

template <typename R>
void cadd_diag(lra_ctx* ctx, int64_t n, cx<R>* A, int64_t lda, R s) {
  if (n <= 0) return;
  cadd_diag_kernel<R><<<grid_for_c(ctx, n, 256), 256, 0, ctx->stream>>>(n, A, lda, s);
  post_launch(ctx, "cadd_diag_kernel");
}

template <typename R>
void cphases(lra_ctx* ctx, const double* g, int64_t n, cx<R>* d) {
  if (n <= 0) return;
  cphase_kernel<R><<<grid_for_c(ctx, n, 256), 256, 0, ctx->stream>>>(n, g, d);
  post_launch(ctx, "cphase_kernel");
}

template <typename R>
void csrft_direct(lra_ctx* ctx, char trans, int64_t M, int64_t N, const cx<R>* A, int64_t lda, const cx<R>* d,
                  const int64_t* idx, int64_t order, cx<R>* B, int64_t ldb) {
  if (order <= 0 || N <= 0) return;
  csrft_direct_kernel<R><<<grid_for_c(ctx, order * N, 128), 128, 0, ctx->stream>>>(cmode(trans), M, N, A,
                                                                                 lda, d, idx, order, B, ldb);
  post_launch(ctx, "csrft_direct_kernel");
}

template <typename R>
void csprn(lra_ctx* ctx, char trans, int64_t M, int64_t N, const cx<R>* A, int64_t lda, const int64_t* perm,
           const cx<R>* g, const int64_t* start, int64_t order, cx<R>* B, int64_t ldb) {
  if (order <= 0 || N <= 0) return;
  csprn_kernel<R><<<grid_for_c(ctx, order * N, 128), 128, 0, ctx->stream>>>(cmode(trans), M, N, A, lda, perm,
                                                                          g, start, order, B, ldb);
  post_launch(ctx, "csprn_kernel");
}

template <typename R>
void csub(lra_ctx* ctx, char trans, int64_t N, const cx<R>* A, int64_t lda, const int64_t* rows, int64_t order,
          cx<R>* B, int64_t ldb) {
  if (order <= 0 || N <= 0) return;
  csub_kernel<R><<<grid_for_c(ctx, order * N, 256), 256, 0, ctx->stream>>>(cmode(trans), N, A, lda, rows,
                                                                          order, B, ldb);
  post_launch(ctx, "csub_kernel");
}

template <typename R>
bool cmaxdet_step(lra_ctx* ctx, int64_t k, int64_t nr, cx<R>* T, int64_t* jpvt, double bound, bool update, cx<R>* R1,
                  int64_t ldr) {
  const int64_t total = k * nr;
  if (total <= 0) return false;
  const ArenaMark mk = ctx->arena.mark();
  double* pv = ctx->arena.alloc_n<double>(1);
  int64_t* pi = ctx->arena.alloc_n<int64_t>(1);
  cabsmax_kernel<R><<<1, 1024, 0, ctx->stream>>>(total, T, pv, pi);
  post_launch(ctx, "cabsmax_kernel");
  double hv = 0;
  LRA_CUDA(cudaMemcpyAsync(&hv, pv, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  const bool big = hv > bound;
  if (big && update) {
    cx<R>* w1 = ctx->arena.alloc_n<cx<R>>(k);
    cx<R>* w2 = ctx->arena.alloc_n<cx<R>>(nr);
    cmaxdet_prep_kernel<R><<<1, 256, 0, ctx->stream>>>(k, nr, T, jpvt, pi, w1, w2);
    post_launch(ctx, "cmaxdet_prep_kernel");
    if (R1) {
      cx<R>* y = ctx->arena.alloc_n<cx<R>>(k);
      cmaxdet_r1_gemv_kernel<R><<<grid_for_c(ctx, k, 128), 128, 0, ctx->stream>>>(k, R1, ldr, w1, y);
      post_launch(ctx, "cmaxdet_r1_gemv_kernel");
      cmaxdet_r1_add_kernel<R><<<grid_for_c(ctx, k, 128), 128, 0, ctx->stream>>>(k, R1, ldr, pi, y);
      post_launch(ctx, "cmaxdet_r1_add_kernel");
    }
    cmaxdet_ger_kernel<R><<<grid_for_c(ctx, total, 256), 256, 0, ctx->stream>>>(k, nr, T, pi, w1, w2);
    post_launch(ctx, "cmaxdet_ger_kernel");
    LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  ctx->arena.release(mk);
  return big;
}

template <typename R>
void ccluster_orth(lra_ctx* ctx, int64_t n, int64_t k, cx<R>* Z, int64_t ldz, const int64_t* cl, int64_t ncl) {
  if (ncl <= 0 || n <= 0 || k <= 0) return;
  ccluster_orth_kernel<R><<<(unsigned)ncl, 256, 0, ctx->stream>>>(n, Z, ldz, cl);
  post_launch(ctx, "ccluster_orth_kernel");
}

#define INSTC(R)                                                                                               \
  template void cgemm<R>(lra_ctx*, char, char, int64_t, int64_t, int64_t, cx<R>, const cx<R>*, int64_t,        \
                         const cx<R>*, int64_t, cx<R>, cx<R>*, int64_t);                                       \
  template void cadjoint<R>(lra_ctx*, int64_t, int64_t, const cx<R>*, int64_t, cx<R>*, int64_t);              \
  template void cconj<R>(lra_ctx*, int64_t, int64_t, cx<R>*, int64_t);                                         \
  template void ccol_norms<R>(lra_ctx*, int64_t, int64_t, const cx<R>*, int64_t, R*);                          \
  template int64_t cgeqp3<R>(lra_ctx*, int64_t, int64_t, cx<R>*, int64_t, int64_t*, cx<R>*, int64_t, int64_t,  \
                             double, double, bool);                                                            \
  template void capply_q<R>(lra_ctx*, char, int64_t, int64_t, const cx<R>*, int64_t, const cx<R>*, cx<R>*,     \
                            int64_t, int64_t);                                                                 \
  template void corgqr<R>(lra_ctx*, int64_t, int64_t, cx<R>*, int64_t, const cx<R>*);                          \
  template void ctrsm_upper<R>(lra_ctx*, int64_t, int64_t, const cx<R>*, int64_t, cx<R>*, int64_t);            \
  template void cjacobi_svd<R>(lra_ctx*, int64_t, cx<R>*, int64_t, cx<R>*, int64_t, R*);                       \
  template bool cis_hermitian<R>(lra_ctx*, int64_t, const cx<R>*, int64_t);                                    \
  template void chermitianize<R>(lra_ctx*, int64_t, cx<R>*, int64_t);                                          \
  template void cadd_diag<R>(lra_ctx*, int64_t, cx<R>*, int64_t, R);                                           \
  template void cphases<R>(lra_ctx*, const double*, int64_t, cx<R>*);                                          \
  template void csrft_direct<R>(lra_ctx*, char, int64_t, int64_t, const cx<R>*, int64_t, const cx<R>*,         \
                                const int64_t*, int64_t, cx<R>*, int64_t);                                     \
  template void csprn<R>(lra_ctx*, char, int64_t, int64_t, const cx<R>*, int64_t, const int64_t*, const cx<R>*, \
                         const int64_t*, int64_t, cx<R>*, int64_t);                                            \
  template void csub<R>(lra_ctx*, char, int64_t, const cx<R>*, int64_t, const int64_t*, int64_t, cx<R>*,       \
                        int64_t);                                                                              \
  template bool cmaxdet_step<R>(lra_ctx*, int64_t, int64_t, cx<R>*, int64_t*, double, bool, cx<R>*, int64_t);   \
  template void ccluster_orth<R>(lra_ctx*, int64_t, int64_t, cx<R>*, int64_t, const int64_t*, int64_t);
INSTC(float)
INSTC(double)
#undef INSTC

}  // namespace lra
