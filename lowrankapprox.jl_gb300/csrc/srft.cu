// SRFT sketch through FFTs, one pass over op(A) (HBM-bound).
//
// The reference (srft_init / srft_reshape! / srft_apply!, src/sketch.jl:353-450)
// fills, for every column x of op(A), an l x m2 matrix X[jj, kk] = d[i] x[i]
// (i = jj m2 + kk, row-major; l the largest divisor of M not above the sketch
// order, m2 = M / l), takes l-point FFTs along jj and evaluates, for each
// sampled frequency f = idx - 1 = R l + C, the sum over kk of Y[C, kk] w^kk
// with w = exp(-2 pi i f / M).  That sum is DFT(d .* x)[f]; real input yields
// (Re, Im) pairs in consecutive output slots (the guard at src/sketch.jl:425
// never fires), an odd last slot only the real part.
//
// Here one CTA handles one column: chunks of the m2 axis are staged in shared
// memory (two real chunk columns packed into one complex sequence), each
// l-point FFT runs in place (radix 2, bit-reversed load), and the twiddled
// sums for the sampled frequencies accumulate in registers, with the phase
// exp(-2 pi i f kk / M) read from an exact table indexed by f kk mod M.
// Used when l is a power of two (always for power-of-two M); otherwise the
// direct evaluation in sketch.cu runs.

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename T>
struct Cx {
  T re, im;
};

template <typename T>
__global__ void cis_table_kernel(int64_t n, Cx<T>* tab) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)n, &s, &c);
    tab[t] = Cx<T>{(T)c, (T)-s};  // exp(-2 pi i t / n)
  }
}

__device__ __forceinline__ unsigned bitrev(unsigned x, int bits) { return __brev(x) >> (32 - bits); }

// exp(-2 pi i t / M): Float32 evaluates it in registers (the table is read
// at random and its loads, not the arithmetic, bound the sampled sums);
// Float64 keeps the table (FP64 sin/cos would cost more than the loads)
__device__ __forceinline__ Cx<float> twiddle(const Cx<float>* tab, int64_t t, int64_t M) {
  float s, c;
  sincospif(2.0f * ((float)t / (float)M), &s, &c);
  return Cx<float>{c, -s};
}
__device__ __forceinline__ Cx<double> twiddle(const Cx<double>* tab, int64_t t, int64_t) { return tab[t]; }

constexpr int SRFT_NT = 256;
constexpr int MAX_PAIRS_PER_THREAD = 8;  // sampled frequencies per thread

// grid: one CTA per column of op(A) (A column-major M x N here)
template <typename T>
__global__ void __launch_bounds__(SRFT_NT) srft_fft_kernel(int64_t M, int64_t N, const T* __restrict__ A, int64_t lda,
                                                           const T* __restrict__ d, const int64_t* __restrict__ idx,
                                                           int64_t order, int lbits, int kcp,
                                                           const Cx<T>* __restrict__ tw_l,
                                                           const Cx<T>* __restrict__ tw_M, T* __restrict__ B,
                                                           int64_t ldb) {
  extern __shared__ unsigned char srft_smem[];
  Cx<T>* Z = reinterpret_cast<Cx<T>*>(srft_smem);  // [l][kcp]
  const int64_t l = (int64_t)1 << lbits;
  const int64_t m2 = M / l;
  const int64_t npairs = (order + 1) / 2;
  for (int64_t col = blockIdx.x; col < N; col += gridDim.x) {
    const T* x = A + col * lda;
    // accumulators of the sampled frequencies owned by this thread
    T zr[MAX_PAIRS_PER_THREAD], zi[MAX_PAIRS_PER_THREAD];
#pragma unroll
    for (int q = 0; q < MAX_PAIRS_PER_THREAD; ++q) zr[q] = zi[q] = T(0);
    for (int64_t kk0 = 0; kk0 < m2; kk0 += 2 * kcp) {
      // load: Z[bitrev(jj)][p] = X[jj, kk0 + 2p] + i X[jj, kk0 + 2p + 1]
      // (32-bit index arithmetic: l kcp < 2^31)
      const int k2 = 2 * kcp;
      for (int t = threadIdx.x; t < (int)l * k2; t += SRFT_NT) {
        const int jj = t / k2, r = t - jj * k2;
        const int64_t kk = kk0 + r;
        T v = T(0);
        if (kk < m2) {
          const int64_t i = jj * m2 + kk;
          v = d[i] * x[i];
        }
        Cx<T>* z = Z + (int64_t)bitrev((unsigned)jj, lbits) * kcp + (r >> 1);
        if (r & 1)
          z->im = v;
        else
          z->re = v;
      }
      __syncthreads();
      // in-place radix-2 decimation-in-time FFTs of length l, kcp of them
      for (int s = 1; s <= lbits; ++s) {
        const int64_t half = (int64_t)1 << (s - 1);
        const int64_t stride = l >> s;  // twiddle index step
        for (int t = threadIdx.x; t < (int)(l / 2) * kcp; t += SRFT_NT) {
          const int bf = t / kcp, p = t - bf * kcp;
          const int grp = bf >> (s - 1), pos = bf & (int)(half - 1);
          const int i0 = grp * 2 * (int)half + pos, i1 = i0 + (int)half;
          const Cx<T> w = tw_l[pos * stride];
          Cx<T>* a = Z + i0 * kcp + p;
          Cx<T>* b = Z + i1 * kcp + p;
          const T br = b->re * w.re - b->im * w.im, bi = b->re * w.im + b->im * w.re;
          const T ar = a->re, ai = a->im;
          a->re = ar + br;
          a->im = ai + bi;
          b->re = ar - br;
          b->im = ai - bi;
        }
        __syncthreads();
      }
      // twiddled sums for the sampled frequencies
#pragma unroll
      for (int q = 0; q < MAX_PAIRS_PER_THREAD; ++q) {
        const int64_t pr = threadIdx.x + (int64_t)q * SRFT_NT;
        if (pr < npairs) {
          const int64_t f = idx[2 * pr] - 1;
          const int64_t C = f & (l - 1), Cm = (l - C) & (l - 1);
          // the phase index f kk mod M, stepped by f per kk (exact, no division)
          int64_t ph = (f * kk0) % M;
          for (int p = 0; p < kcp; ++p) {
            const int64_t kka = kk0 + 2 * p;
            if (kka >= m2) break;
            // unpack the two real sequences from the packed FFT
            const Cx<T> z1 = Z[C * kcp + p], z2 = Z[Cm * kcp + p];
            const T yar = T(0.5) * (z1.re + z2.re), yai = T(0.5) * (z1.im - z2.im);  // sequence a
            const T ybr = T(0.5) * (z1.im + z2.im), ybi = T(0.5) * (z2.re - z1.re);  // sequence b
            const Cx<T> wa = twiddle(tw_M, ph, M);
            zr[q] += yar * wa.re - yai * wa.im;
            zi[q] += yar * wa.im + yai * wa.re;
            ph += f;
            if (ph >= M) ph -= M;
            if (kka + 1 < m2) {
              const Cx<T> wb = twiddle(tw_M, ph, M);
              zr[q] += ybr * wb.re - ybi * wb.im;
              zi[q] += ybr * wb.im + ybi * wb.re;
            }
            ph += f;
            if (ph >= M) ph -= M;
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < MAX_PAIRS_PER_THREAD; ++q) {
      const int64_t pr = threadIdx.x + (int64_t)q * SRFT_NT;
      if (pr < npairs) {
        const int64_t slot = 2 * pr;
        B[slot + col * ldb] = zr[q];
        if (slot + 1 < order) B[slot + 1 + col * ldb] = zi[q];
      }
    }
  }
}

}  // namespace

// true when the FFT path ran; false when the shape needs the direct kernel
template <typename T>
bool srft_sketch_fft(lra_ctx* ctx, char trans, int64_t M, int64_t N, const T* A, int64_t lda, const T* d,
                     const int64_t* idx, int64_t order, T* B, int64_t ldb) {
  if (order <= 0 || N <= 0 || M <= 0) return true;
  int64_t l = std::min(order, M);
  while (M % l) --l;
  if (l < 2 || (l & (l - 1))) return false;
  const int64_t npairs = (order + 1) / 2;
  if (npairs > (int64_t)MAX_PAIRS_PER_THREAD * SRFT_NT) return false;
  int lbits = 0;
  while (((int64_t)1 << lbits) < l) ++lbits;
  const int64_t m2 = M / l;
  const size_t per = (size_t)l * sizeof(Cx<T>);
  // at most 48 KB of shared memory per CTA, so that several CTAs (and their
  // loads) share an SM
  int64_t kcp = std::min<int64_t>(16, (int64_t)((48 * 1024) / per));
  kcp = std::min<int64_t>(kcp, (m2 + 1) / 2);
  if (kcp < 1) return false;
  const ArenaMark mk = ctx->arena.mark();
  const T* X = A;
  int64_t ldx = lda;
  if (trans == 'c') {  // columns of op(A) = rows of A: make them contiguous first
    T* At = ctx->arena.alloc_n<T>((size_t)M * N);
    transpose(ctx, N, M, A, lda, At, M);
    X = At;
    ldx = M;
  }
  Cx<T>* tw_l = ctx->arena.alloc_n<Cx<T>>(l);
  Cx<T>* tw_M = ctx->arena.alloc_n<Cx<T>>(M);
  const unsigned g1 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((M + 255) / 256, ctx->num_sms * 8));
  cis_table_kernel<T><<<g1, 256, 0, ctx->stream>>>(l, tw_l);
  post_launch(ctx, "cis_table_kernel");
  cis_table_kernel<T><<<g1, 256, 0, ctx->stream>>>(M, tw_M);
  post_launch(ctx, "cis_table_kernel");
  const size_t smem = per * kcp;
  raise_smem_limit(ctx, (const void*)srft_fft_kernel<T>);
  const unsigned grid = (unsigned)std::min<int64_t>(N, (int64_t)ctx->num_sms * 8);
  srft_fft_kernel<T><<<grid, SRFT_NT, smem, ctx->stream>>>(M, N, X, ldx, d, idx, order, lbits, (int)kcp, tw_l,
                                                           tw_M, B, ldb);
  post_launch(ctx, "srft_fft_kernel");
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return true;
}

template bool srft_sketch_fft<float>(lra_ctx*, char, int64_t, int64_t, const float*, int64_t, const float*,
                                     const int64_t*, int64_t, float*, int64_t);
template bool srft_sketch_fft<double>(lra_ctx*, char, int64_t, int64_t, const double*, int64_t, const double*,
                                      const int64_t*, int64_t, double*, int64_t);

}  // namespace lra
