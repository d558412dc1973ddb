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
// Main kernel (srft_dif_kernel): one CTA per column.  The m2 axis is cut
// into chunks of PC complex columns (two real columns kk = 2p, 2p + 1 packed
// into one complex sequence, so one l-point FFT serves both).  The l-point
// FFTs are mixed-radix decimation in frequency (radix 2..16 in registers,
// one to three passes), in place in shared memory, so each pass needs one
// barrier and a thread keeps one group of R values at a time.  Two forms:
// 256 threads with rows padded by one element (any chunk width), and, for
// Float32 with l = 128 .. 1024, 512 threads with 8192-value chunks whose
// unpadded rows are swizzled so that the passes are free of bank conflicts
// (SkCfg below).  The first pass takes its inputs straight from HBM
// with coalesced 8- or 16-byte loads (lanes along p) and the signs d = +-1
// as bits.  The output rows are in digit-reversed order, which the sampled
// sums read through a per-frequency index.  The sums unpack the two real
// sequences and accumulate exp(-2 pi i f kk / M) Y with the phase factor
// stepped by a complex recurrence, reseeded from the exact integer phase
// every 16 steps.  Shapes outside its range (l above 1024, odd m2, unaligned
// columns, more than 1024 sampled pairs) take srft_fft_kernel (radix 2 in
// shared memory), and l not a power of two the direct evaluation in
// sketch.cu.

#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "internal.hpp"

namespace lra {

namespace {

template <typename T>
struct alignas(2 * sizeof(T)) Cx {
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

// ---------------------------------------------------------------------------
// decimation-in-frequency kernel

constexpr int SK_NT = 256;
constexpr int SK_PAIRS_MAX = 1024;  // sampled frequency pairs (item state in shared memory)
constexpr int SK_RUN = 16;  // recurrence steps of the phase between exact reseeds

// complex values per chunk (32 KB): 16 per thread
template <typename T>
constexpr int sk_chunk() {
  return 32768 / (2 * (int)sizeof(T));
}
constexpr int sk_passes(int lb) { return (lb + 3) / 4; }

// a kernel configuration: NT threads, and either a run-time chunk width PC
// (PCF = 0: rows padded to PC + 1 elements) or the compile-time width PCF
// >= 8 with unpadded rows whose elements are permuted by p ^ (row & 15)
// (p ^ (row & 7) for PCF = 8): a row of 16 or more then spans all 32 banks,
// so every pass reads and writes whole rows without conflicts, and the
// random rows of the sampled sums still spread over the banks
template <typename T, int LB, int NTT, int PCF>
struct SkCfg {
  static constexpr int NT = NTT;
  static constexpr int CHUNK = PCF ? (PCF << LB) : sk_chunk<T>();
  static constexpr int PCFB = PCF >= 256 ? 8 : PCF >= 128 ? 7 : PCF >= 64 ? 6 : PCF >= 32 ? 5 : PCF >= 16 ? 4 : PCF >= 8 ? 3 : 0;
  static constexpr int SWM = PCF >= 16 ? 15 : PCF >= 8 ? 7 : 0;
};
// log2 of the radix of pass q (radices 2..16, as even as the passes allow)
constexpr int sk_bits(int lb, int q) { return lb / sk_passes(lb) + (q < lb % sk_passes(lb) ? 1 : 0); }
// log2 of the sub-transform length before pass q
constexpr int sk_ns_bits(int lb, int q) {
  int s = 0;
  for (int i = 0; i < q; ++i) s += sk_bits(lb, i);
  return s;
}

// cos(2 pi k / 16) from the exact values of cos(pi/8), cos(pi/4), cos(3 pi/8)
__host__ __device__ constexpr double cos16(int k) {
  k &= 15;
  if (k > 8) k = 16 - k;
  const bool neg = k > 4;
  if (neg) k = 8 - k;
  const double c = k == 0   ? 1.0
                   : k == 1 ? 0.92387953251128675613
                   : k == 2 ? 0.70710678118654752440
                   : k == 3 ? 0.38268343236508977173
                            : 0.0;
  return neg ? -c : c;
}

template <typename T>
__device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
  return Cx<T>{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}

// a exp(-2 pi i e / 16); e is a constant once the callers are unrolled
template <typename T>
__device__ __forceinline__ Cx<T> mul_root16(Cx<T> a, int e) {
  e &= 15;
  if (e == 0) return a;
  if (e == 4) return Cx<T>{a.im, -a.re};
  if (e == 8) return Cx<T>{-a.re, -a.im};
  if (e == 12) return Cx<T>{-a.im, a.re};
  const T c = (T)cos16(e), s = -(T)cos16(e - 4);
  return Cx<T>{a.re * c - a.im * s, a.re * s + a.im * c};
}

// in-register DFT of length R (natural order in and out): bit reversal, then
// radix-2 decimation-in-time stages with constant roots
template <int R, typename T>
__device__ __forceinline__ void dft_reg(Cx<T> (&v)[R]) {
  constexpr int RB = R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : 4;
  static_assert((1 << RB) == R, "radix");
#pragma unroll
  for (int i = 0; i < R; ++i) {
    int j = 0;
#pragma unroll
    for (int b = 0; b < RB; ++b) j |= ((i >> b) & 1) << (RB - 1 - b);
    if (j > i) {
      const Cx<T> t = v[i];
      v[i] = v[j];
      v[j] = t;
    }
  }
#pragma unroll
  for (int h = 1; h < R; h <<= 1) {
#pragma unroll
    for (int g = 0; g < R; g += 2 * h) {
#pragma unroll
      for (int q = 0; q < h; ++q) {
        const Cx<T> b = mul_root16(v[g + q + h], q * (8 / h));  // exp(-2 pi i q / (2h))
        const Cx<T> a = v[g + q];
        v[g + q] = Cx<T>{a.re + b.re, a.im + b.im};
        v[g + q + h] = Cx<T>{a.re - b.re, a.im - b.im};
      }
    }
  }
}

__device__ __forceinline__ Cx<float> ld_stream(const float* p) {
  const float2 t = __ldcs(reinterpret_cast<const float2*>(p));
  return Cx<float>{t.x, t.y};
}
__device__ __forceinline__ Cx<double> ld_stream(const double* p) {
  const double2 t = __ldcs(reinterpret_cast<const double2*>(p));
  return Cx<double>{t.x, t.y};
}
// dbits[w] bit b set where d[32 w + b] < 0 (d = +-1)
template <typename T>
__global__ void sign_bits_kernel(int64_t n, const T* __restrict__ d, unsigned* __restrict__ dbits) {
  const int64_t nw = (n + 31) / 32;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < nw;
       w += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t i = w * 32 + (threadIdx.x & 31);
    const unsigned b = __ballot_sync(0xffffffffu, i < n && d[i] < T(0));
    if ((threadIdx.x & 31) == 0) dbits[w] = b;
  }
}

__host__ __device__ constexpr size_t sk_align16(size_t b) { return (b + 15) & ~(size_t)15; }

// log2 of the block length before pass q of the decimation-in-frequency FFT
constexpr int sk_block_bits(int lb, int q) { return lb - sk_ns_bits(lb, q); }

// per-pass twiddle tables: pass q (all but the last) keeps
// w^(n1 k2) = exp(-2 pi i n1 k2 / 2^NB) at [(k2 - 1) 2^NPB + n1], so that the
// lanes of a warp (consecutive n1) read consecutive entries
constexpr int sk_tw_len(int lb, int q) {
  return ((1 << sk_bits(lb, q)) - 1) << (sk_block_bits(lb, q) - sk_bits(lb, q));
}
constexpr int sk_tw_off(int lb, int q) {
  int o = 0;
  for (int i = 0; i < q; ++i)
    if (i + 1 < sk_passes(lb)) o += sk_tw_len(lb, i);
  return o;
}
constexpr int sk_tw_size(int lb) { return sk_tw_off(lb, sk_passes(lb)); }

// position in Z of frequency k after all passes (digits of k in the pass
// radices, reversed)
template <int LB>
__device__ __forceinline__ int sk_pos(int k) {
  int pos = 0;
#pragma unroll
  for (int q = 0; q < sk_passes(LB); ++q) {
    pos += (k & ((1 << sk_bits(LB, q)) - 1)) << (sk_block_bits(LB, q) - sk_bits(LB, q));
    k >>= sk_bits(LB, q);
  }
  return pos;
}

// one group of pass q, in place: v[k2] = w^(n1 k2) sum over n2 of
// v[n2] exp(-2 pi i n2 k2 / R), w = exp(-2 pi i / 2^NB)
template <typename T, int LB, int Q, int R>
__device__ __forceinline__ void sk_butterfly(Cx<T> (&v)[R], int n1, const Cx<T>* tw) {
  constexpr int NB = sk_block_bits(LB, Q), NPB = NB - sk_bits(LB, Q);
  dft_reg<R>(v);
  if constexpr (NPB > 0) {
    const Cx<T>* tq = tw + sk_tw_off(LB, Q) + n1;
#pragma unroll
    for (int k2 = 1; k2 < R; ++k2) v[k2] = cmul(v[k2], tq[(k2 - 1) << NPB]);
  }
}

// x with its sign flipped where bit 0 (flip0) or bit 1 (flip1) of w is set
__device__ __forceinline__ float flip0(float x, unsigned w) { return __int_as_float(__float_as_int(x) ^ (w << 31)); }
__device__ __forceinline__ float flip1(float x, unsigned w) {
  return __int_as_float(__float_as_int(x) ^ ((w << 30) & 0x80000000u));
}
__device__ __forceinline__ double flip0(double x, unsigned w) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)(w << 31) << 32));
}
__device__ __forceinline__ double flip1(double x, unsigned w) {
  return __longlong_as_double(__double_as_longlong(x) ^ ((unsigned long long)((w << 30) & 0x80000000u) << 32));
}

// the inputs of pass 0 for one chunk, held in registers from their loads
// (issued while the previous chunk's sums run) to their use
template <typename T, int LB, class CF>
struct SkIn {
  static constexpr int R = 1 << sk_bits(LB, 0);
  static constexpr int NG = (CF::CHUNK / R + CF::NT - 1) / CF::NT;
  Cx<T> x[NG][R];
  unsigned w[NG][R];
};

// loads of pass 0: z[jj][p] = d x at (jj, kk0 + 2p) + i d x at (jj, kk0 + 2p + 1)
// for the rows jj = n1 + n2 l / R of each group; the signs d = +-1 come as
// bits (bit i of dbits set where d[i] = -1)
template <typename T, int LB, class CF>
__device__ __forceinline__ void sk_load(SkIn<T, LB, CF>& in, const T* __restrict__ x,
                                        const unsigned* __restrict__ dbits, int m2, int kk0, int pcb) {
  constexpr int R = SkIn<T, LB, CF>::R, NG = SkIn<T, LB, CF>::NG, NP = (1 << LB) / R;
  const int groups = NP << pcb;
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    const int g = threadIdx.x + k * CF::NT;
    if (g < groups) {
      const int n1 = g >> pcb, p = g & ((1 << pcb) - 1);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = (n1 + r * NP) * m2 + kk0 + 2 * p;
        in.x[k][r] = ld_stream(x + i);
        in.w[k][r] = __ldg(dbits + (i >> 5)) >> (i & 31);  // i even: both bits in this word
      }
    }
  }
}

// pass 0: signs applied, transformed, written to Z
template <typename T, int LB, class CF>
__device__ __forceinline__ void sk_first(const SkIn<T, LB, CF>& in, Cx<T>* Z, const Cx<T>* tab, int pcb, int pcp) {
  constexpr int R = SkIn<T, LB, CF>::R, NG = SkIn<T, LB, CF>::NG, NP = (1 << LB) / R;
  const int groups = NP << pcb;
  __syncthreads();  // the previous chunk's sums have read Z
#pragma unroll
  for (int k = 0; k < NG; ++k) {
    const int g = threadIdx.x + k * CF::NT;
    if (g < groups) {
      const int n1 = g >> pcb, p = (g & ((1 << pcb) - 1)) ^ (n1 & CF::SWM);
      Cx<T> v[R];
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = Cx<T>{flip0(in.x[k][r].re, in.w[k][r]), flip1(in.x[k][r].im, in.w[k][r])};
      sk_butterfly<T, LB, 0, R>(v, n1, tab);
      // rows n1 + r NP with n1 < NP: the row's swizzle splits into n1's and r NP's
#pragma unroll
      for (int r = 0; r < R; ++r) Z[(n1 + r * NP) * pcp + (p ^ ((r * NP) & CF::SWM))] = v[r];
    }
  }
  __syncthreads();
}

// passes Q >= 1, each in place in shared memory (a thread reads and writes
// the same R rows of its groups), one barrier per pass
template <typename T, int LB, class CF, int Q>
__device__ __forceinline__ void sk_rest(Cx<T>* Z, const Cx<T>* tab, int pcb, int pcp) {
  if constexpr (Q < sk_passes(LB)) {
    constexpr int RB = sk_bits(LB, Q), R = 1 << RB, NB = sk_block_bits(LB, Q), NPB = NB - RB;
    constexpr int NG = (CF::CHUNK / R + CF::NT - 1) / CF::NT;
    const int groups = ((1 << LB) / R) << pcb;
#pragma unroll
    for (int k = 0; k < NG; ++k) {
      const int g = threadIdx.x + k * CF::NT;
      if (g < groups) {
        const int gi = g >> pcb;
        const int n1 = gi & ((1 << NPB) - 1);
        const int base = ((gi >> NPB) << NB) + n1;  // rows base + (r << NPB), disjoint bits
        const int p = (g & ((1 << pcb) - 1)) ^ (base & CF::SWM);
        Cx<T>* z = Z + base * pcp;
        Cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = z[(r << NPB) * pcp + (p ^ ((r << NPB) & CF::SWM))];
        sk_butterfly<T, LB, Q, R>(v, n1, tab);
#pragma unroll
        for (int r = 0; r < R; ++r) z[(r << NPB) * pcp + (p ^ ((r << NPB) & CF::SWM))] = v[r];
      }
    }
    __syncthreads();
    sk_rest<T, LB, CF, Q + 1>(Z, tab, pcb, pcp);
  }
}

// a sampled frequency f (pair of output slots): v = -i exp(-2 pi i f / M)
// unpacks the two real sequences; step = exp(-2 pi i 2 NS f / M) advances
// the phase factor by NS complex columns, dph16 = 16 (2 NS f) mod M the
// integer phase by SK_RUN of those steps
template <typename T>
struct SkPair {
  Cx<T> v, step;
  int f, cc, dph16;  // cc = pos(C) | pos(l - C mod l) << 16
};

// CTAs per SM the register budget aims at: three (80 registers) for l up to
// 128, two (128 registers, no spills) for the three-pass transforms and the
// radix-16 pairs, where spilled values cost more than the third CTA gains
constexpr int sk_min_ctas(int lb, int nt) { return nt > 256 ? 1 : lb >= 8 ? 2 : 3; }

// grid: columns of op(A) (column-major M x N); a CTA takes the chunks of its
// columns in turn, loading the next chunk while it sums the current one
template <typename T, int LB, class CF>
__global__ void __launch_bounds__(CF::NT, sk_min_ctas(LB, CF::NT)) srft_dif_kernel(int M, int64_t N, const T* __restrict__ A, int64_t lda,
                                                            const unsigned* __restrict__ dbits,
                                                            const int64_t* __restrict__ idx, int order, int pcb,
                                                            int nsl, const Cx<T>* __restrict__ tw_l,
                                                            const Cx<T>* __restrict__ tw_M, T* __restrict__ B,
                                                            int64_t ldb) {
  extern __shared__ __align__(16) unsigned char sk_smem[];
  constexpr int L = 1 << LB;
  if (CF::PCFB) pcb = CF::PCFB;
  const int PC = 1 << pcb, pcp = CF::SWM ? PC : PC + 1, NS = 1 << nsl;
  const int npairs = (order + 1) / 2, items = npairs << nsl;
  const int m2 = M >> LB, per_chunk = PC >> nsl, nchunks = m2 / (2 * PC);
  const int run = per_chunk < SK_RUN ? per_chunk : SK_RUN;
  // shared memory: the item states (sums, phase factors, integer phases at
  // the next reseed), the pairs, the l-point twiddles, then Z
  Cx<T>* st_acc = reinterpret_cast<Cx<T>*>(sk_smem);
  Cx<T>* st_cur = st_acc + items;
  int* st_ph = reinterpret_cast<int*>(st_cur + items);
  SkPair<T>* pairs = reinterpret_cast<SkPair<T>*>(sk_smem + sk_align16((size_t)items * (2 * sizeof(Cx<T>) + 4)));
  Cx<T>* tab = reinterpret_cast<Cx<T>*>(reinterpret_cast<unsigned char*>(pairs) +
                                        sk_align16((size_t)npairs * sizeof(SkPair<T>)));
  Cx<T>* Z = tab + sk_tw_size(LB);  // [l][PC + 1], rows in digit-reversed frequency order after the passes
#pragma unroll
  for (int q = 0; q + 1 < sk_passes(LB); ++q) {
    const int npb = sk_block_bits(LB, q) - sk_bits(LB, q), len = sk_tw_len(LB, q);
    for (int e = threadIdx.x; e < len; e += CF::NT) {
      const int k2 = (e >> npb) + 1, n1 = e & ((1 << npb) - 1);
      tab[sk_tw_off(LB, q) + e] = tw_l[(n1 * k2) << (LB - sk_block_bits(LB, q))];
    }
  }
  for (int pr = threadIdx.x; pr < npairs; pr += CF::NT) {
    const int f = (int)(idx[2 * pr] - 1);
    const int C = f & (L - 1);
    const Cx<T> w = twiddle(tw_M, f, M);
    SkPair<T> P;
    P.v = Cx<T>{w.im, -w.re};
    P.step = twiddle(tw_M, (int)(((int64_t)2 * NS * f) % M), M);
    P.f = f;
    P.cc = sk_pos<LB>(C) | (sk_pos<LB>((L - C) & (L - 1)) << 16);
    P.dph16 = (int)(((int64_t)(2 * SK_RUN) * NS * f) % M);
    pairs[pr] = P;
  }
  __syncthreads();
  // item (pair pr, split s) visits kk = 2 s, 2 s + 2 NS, ...: the factor
  // exp(-2 pi i f kk / M) by recurrence, reseeded every SK_RUN steps from the
  // exact integer phase f kk mod M; the item's own thread is the only one
  // to touch its state
  auto start_column = [&]() {
    for (int it = threadIdx.x; it < items; it += CF::NT) {
      st_acc[it] = Cx<T>{T(0), T(0)};
      st_ph[it] = (int)(((int64_t)pairs[it >> nsl].f * (2 * (it & (NS - 1)))) % M);
    }
  };
  int64_t col = blockIdx.x;
  int ch = 0;
  SkIn<T, LB, CF> in;
  if (col < N) {
    start_column();
    sk_load<T, LB, CF>(in, A + col * lda, dbits, m2, 0, pcb);
  }
  while (col < N) {
    sk_first<T, LB, CF>(in, Z, tab, pcb, pcp);
    sk_rest<T, LB, CF, 1>(Z, tab, pcb, pcp);
    int64_t ncol = col;
    int nch = ch + 1;
    if (nch == nchunks) {
      ncol = col + gridDim.x;
      nch = 0;
    }
    if (ncol < N) sk_load<T, LB, CF>(in, A + ncol * lda, dbits, m2, nch * 2 * PC, pcb);
    const int t0 = ch * per_chunk;  // steps taken so far in this column
    for (int it = threadIdx.x; it < items; it += CF::NT) {
      const SkPair<T> P = pairs[it >> nsl];
      const int s = it & (NS - 1);
      const int row1 = P.cc & 0xffff, row2 = P.cc >> 16;
      const int sw1 = row1 & CF::SWM, sw2 = row2 & CF::SWM;
      const Cx<T>* z1p = Z + row1 * pcp;
      const Cx<T>* z2p = Z + row2 * pcp;
      Cx<T> a = st_acc[it], c = st_cur[it];
      int h = st_ph[it];
      for (int i0 = 0; i0 < per_chunk; i0 += run) {
        if (((t0 + i0) & (SK_RUN - 1)) == 0) {
          c = twiddle(tw_M, h, M);
          h += P.dph16;
          if (h >= M) h -= M;
        }
#pragma unroll 4
        for (int i = 0; i < run; ++i) {
          const int pp = s + ((i0 + i) << nsl);
          const Cx<T> z1 = z1p[pp ^ sw1], z2 = z2p[pp ^ sw2];
          // t = (z1 + conj z2) + v (z1 - conj z2) = 2 (Y_a + Y_b w^f)
          const T sr = z1.re + z2.re, si = z1.im - z2.im, dr = z1.re - z2.re, di = z1.im + z2.im;
          const T tr = sr + P.v.re * dr - P.v.im * di, ti = si + P.v.re * di + P.v.im * dr;
          a.re += c.re * tr - c.im * ti;
          a.im += c.re * ti + c.im * tr;
          c = cmul(c, P.step);
        }
      }
      st_acc[it] = a;
      st_cur[it] = c;
      st_ph[it] = h;
    }
    if (ch + 1 == nchunks) {
      // combine the NS splits of each pair (consecutive lanes) and store
      for (int it0 = 0; it0 < items; it0 += CF::NT) {
        const int it = it0 + threadIdx.x;
        Cx<T> a = it < items ? st_acc[it] : Cx<T>{T(0), T(0)};
        for (int o = NS >> 1; o > 0; o >>= 1) {
          a.re += __shfl_xor_sync(0xffffffffu, a.re, o);
          a.im += __shfl_xor_sync(0xffffffffu, a.im, o);
        }
        if (it < items && (it & (NS - 1)) == 0) {
          const int64_t slot = 2 * (int64_t)(it >> nsl);
          B[slot + col * ldb] = T(0.5) * a.re;
          if (slot + 1 < order) B[slot + 1 + col * ldb] = T(0.5) * a.im;
        }
      }
      if (ncol < N) start_column();
    }
    col = ncol;
    ch = nch;
  }
}

template <typename T, int LB, class CF>
void launch_dif(lra_ctx* ctx, int M, int64_t N, const T* A, int64_t lda, const unsigned* d,
                const int64_t* idx, int order, int pcb, int nsl, const Cx<T>* tw_l, const Cx<T>* tw_M, T* B,
                int64_t ldb, size_t smem) {
  auto* kern = srft_dif_kernel<T, LB, CF>;
  raise_smem_limit(ctx, (const void*)kern);
  int per_sm = 0;
  LRA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, CF::NT, smem));
  if (per_sm < 1) per_sm = 1;
  const unsigned grid = (unsigned)std::min<int64_t>(N, (int64_t)ctx->num_sms * per_sm);
  kern<<<grid, CF::NT, smem, ctx->stream>>>(M, N, A, lda, d, idx, order, pcb, nsl, tw_l, tw_M, B, ldb);
  post_launch(ctx, "srft_dif_kernel");
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
  const ArenaMark mk = ctx->arena.mark();
  const T* X = A;
  int64_t ldx = lda;
  if (trans == 'c') {  // columns of op(A) = rows of A: make them contiguous first
    T* At = ctx->arena.alloc_n<T>((size_t)M * N);
    transpose(ctx, N, M, A, lda, At, M);
    X = At;
    ldx = M;
  }
  const unsigned g1 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((M + 255) / 256, ctx->num_sms * 8));
  Cx<T>* tw_l = ctx->arena.alloc_n<Cx<T>>(l);
  cis_table_kernel<T><<<g1, 256, 0, ctx->stream>>>(l, tw_l);
  post_launch(ctx, "cis_table_kernel");
  // Float32 evaluates exp(-2 pi i t / M) in registers; Float64 reads a table
  Cx<T>* tw_M = nullptr;
  if (sizeof(T) == 8) {
    tw_M = ctx->arena.alloc_n<Cx<T>>(M);
    cis_table_kernel<T><<<g1, 256, 0, ctx->stream>>>(M, tw_M);
    post_launch(ctx, "cis_table_kernel");
  }
  const int64_t pair_align = 2 * (int64_t)sizeof(T);
  bool dif = lbits <= 10 && m2 % 2 == 0 && M < ((int64_t)1 << 31) && npairs <= (int64_t)SK_PAIRS_MAX &&
             ldx % 2 == 0 && reinterpret_cast<uintptr_t>(X) % pair_align == 0;
  bool wide = false;
  int pcb = 0, nsl = 0;
  size_t smem = 0;
  if (dif) {
    // Float32 with l' = 128 .. 1024 and m2 / 2 a multiple of PC = 8192 / l':
    // 512 threads and swizzled rows PC wide (chunks of 8192 complex values;
    // measured 2%, 4%, 19% and 17% faster than the padded form at 128, 256,
    // 512 and 1024, and 3% slower at 64); otherwise 256 threads and padded
    // rows of a chunk width PC, a power of two dividing m2 / 2, at most the
    // kernel's
    const int wide_pcb = 13 - lbits;
    wide = sizeof(T) == 4 && lbits >= 7 && lbits <= 10 && (m2 / 2) % (1 << wide_pcb) == 0 &&
           ctx->tuning.srft_wide[lbits] != 0;
    const int nt = wide ? 512 : SK_NT;
    if (wide) {
      pcb = wide_pcb;
    } else {
      const int64_t pc_max = std::max<int64_t>(1, (int64_t)sk_chunk<T>() >> lbits);
      while (((int64_t)2 << pcb) <= pc_max && (m2 / 2) % ((int64_t)2 << pcb) == 0) ++pcb;
    }
    // splits of each pair's sum: as many as idle threads allow, within a warp
    while ((2 << nsl) <= (1 << pcb) && (2 << nsl) <= 32 && ((int64_t)2 << nsl) * npairs <= nt) ++nsl;
    const size_t items = (size_t)npairs << nsl;
    smem = sk_align16(items * (2 * sizeof(Cx<T>) + 4)) + sk_align16((size_t)npairs * sizeof(SkPair<T>)) +
           ((size_t)sk_tw_size(lbits) + (size_t)l * (size_t)((wide ? 0 : 1) + (1 << pcb))) * sizeof(Cx<T>);
    int optin = 0;
    LRA_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    dif = smem + 1024 <= (size_t)optin;  // (the kernel's static shared memory is a few bytes)
  }
  if (dif) {
    unsigned* dbits = ctx->arena.alloc_n<unsigned>((size_t)(M + 31) / 32);
    sign_bits_kernel<T><<<g1, 256, 0, ctx->stream>>>(M, d, dbits);
    post_launch(ctx, "sign_bits_kernel");
    const int Mi = (int)M, oi = (int)order;
    if constexpr (sizeof(T) == 4) {
      if (wide) {
        switch (lbits) {
#define SK_WIDE(LB)                                                                                             \
  case LB:                                                                                                      \
    launch_dif<T, LB, SkCfg<T, LB, 512, (1 << (13 - LB))>>(ctx, Mi, N, X, ldx, dbits, idx, oi, pcb, nsl, tw_l, \
                                                           tw_M, B, ldb, smem);                               \
    break;
          SK_WIDE(7) SK_WIDE(8) SK_WIDE(9) SK_WIDE(10)
#undef SK_WIDE
        }
      }
    }
    if (!wide) {
      switch (lbits) {
#define SK_CASE(LB)                                                                                          \
  case LB:                                                                                                   \
    launch_dif<T, LB, SkCfg<T, LB, SK_NT, 0>>(ctx, Mi, N, X, ldx, dbits, idx, oi, pcb, nsl, tw_l, tw_M, B, ldb, \
                                             smem);                                                          \
    break;
        SK_CASE(1) SK_CASE(2) SK_CASE(3) SK_CASE(4) SK_CASE(5)
        SK_CASE(6) SK_CASE(7) SK_CASE(8) SK_CASE(9) SK_CASE(10)
#undef SK_CASE
      }
    }
  } else {
    const size_t per = (size_t)l * sizeof(Cx<T>);
    // at most 48 KB of shared memory per CTA, so that several CTAs (and
    // their loads) share an SM
    int64_t kcp = std::min<int64_t>(16, (int64_t)((48 * 1024) / per));
    kcp = std::min<int64_t>(kcp, (m2 + 1) / 2);
    if (kcp < 1) kcp = 1;
    const size_t smem = per * kcp;
    raise_smem_limit(ctx, (const void*)srft_fft_kernel<T>);
    const unsigned grid = (unsigned)std::min<int64_t>(N, (int64_t)ctx->num_sms * 8);
    srft_fft_kernel<T><<<grid, SRFT_NT, smem, ctx->stream>>>(M, N, X, ldx, d, idx, order, lbits, (int)kcp, tw_l,
                                                             tw_M, B, ldb);
    post_launch(ctx, "srft_fft_kernel");
  }
  LRA_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->arena.release(mk);
  return true;
}

template bool srft_sketch_fft<float>(lra_ctx*, char, int64_t, int64_t, const float*, int64_t, const float*,
                                     const int64_t*, int64_t, float*, int64_t);
template bool srft_sketch_fft<double>(lra_ctx*, char, int64_t, int64_t, const double*, int64_t, const double*,
                                      const int64_t*, int64_t, double*, int64_t);

}  // namespace lra
