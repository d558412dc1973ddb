// Double-float ("df64") arithmetic on the FP32 pipes: x = h + l with
// |l| <= ulp(h) / 2, about 48 significant bits.  Products are split exactly
// with an FMA (p = a b, e = fma(a, b, -p)), sums with Knuth's two-sum; the
// results are accurate to a few units of 2^-46.  On GB300 the FP32 pipes
// issue 64 lanes for every FP64 lane, so these sequences of 3-20 FP32
// operations are several times faster than one FP64 operation.
#pragma once

namespace lra {

struct Df {
  float h, l;
};

static __device__ __forceinline__ double df_val(float h, float l) { return (double)h + (double)l; }

static __device__ __forceinline__ Df df_split(double x) {
  const float h = (float)x;
  return Df{h, (float)(x - (double)h)};
}

static __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

static __device__ __forceinline__ Df quick_two_sum(float a, float b) {
  const float s = a + b;
  return Df{s, b - (s - a)};
}

static __device__ __forceinline__ Df df_add(Df a, Df b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e += a.l + b.l;
  return quick_two_sum(s, e);
}

static __device__ __forceinline__ Df df_mul(Df a, Df b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
  return quick_two_sum(p, e);
}

// acc += v x, the high parts by two-sum, every lower-order term into acc.l
static __device__ __forceinline__ void df_fma_acc(Df& acc, float vh, float vl, float xh, float xl) {
  const float p = vh * xh;
  float pe = fmaf(vh, xh, -p);
  pe = fmaf(vh, xl, fmaf(vl, xh, pe));
  float s, e;
  two_sum(acc.h, p, s, e);
  acc.h = s;
  acc.l += e + pe;
}

// y = x - f v
static __device__ __forceinline__ Df df_axpy_neg(float xh, float xl, Df f, float vh, float vl) {
  const float p = f.h * vh;
  float pe = fmaf(f.h, vh, -p);
  pe = fmaf(f.h, vl, fmaf(f.l, vh, pe));
  float s, e;
  two_sum(xh, -p, s, e);
  return quick_two_sum(s, (xl - pe) + e);
}

static __device__ __forceinline__ Df df_shfl_xor(Df a, int o) {
  return Df{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
}

static __device__ __forceinline__ Df df_neg(Df a) { return Df{-a.h, -a.l}; }

static __device__ __forceinline__ Df df_div(Df a, Df b) {
  const float q1 = a.h / b.h;
  const Df r = df_add(a, df_neg(df_mul(Df{q1, 0.f}, b)));
  const float q2 = r.h / b.h;
  return quick_two_sum(q1, q2);
}

static __device__ __forceinline__ Df df_sqrt(Df a) {
  if (!(a.h > 0.f)) return Df{0.f, 0.f};
  const float y = sqrtf(a.h);
  const float p = y * y;
  const float pe = fmaf(y, y, -p);
  const float d = ((a.h - p) - pe) + a.l;
  return quick_two_sum(y, d / (2.f * y));
}

// orderable key of a nonnegative double-float (h >= 0, |l| <= ulp(h) / 2):
// h's bits, then l mapped to an unsigned order
static __device__ __forceinline__ long long df_key(Df a) {
  if (a.h < 0.f) return -1;
  const unsigned int lb = __float_as_uint(a.l);
  const unsigned int lo = (lb & 0x80000000u) ? ~lb : (lb | 0x80000000u);
  return (long long)(((unsigned long long)__float_as_uint(a.h) << 32) | lo);
}

}  // namespace lra
