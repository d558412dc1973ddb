// Complex element types (ComplexF32 / ComplexF64) of liblra: the number
// type, its arithmetic and the LAPACK scalar rules the complex kernels use.
// Storage is two reals (re, im) in a row, the layout of Julia's Complex{T}
// arrays, so caller buffers are used as they are.
#pragma once

#include <cuda_runtime.h>

#include <cmath>

namespace lra {

template <typename R>
struct __align__(2 * sizeof(R)) cx {
  R re, im;
  cx() = default;
  __host__ __device__ constexpr cx(R r, R i = R(0)) : re(r), im(i) {}
};

template <typename R>
__host__ __device__ __forceinline__ cx<R> operator+(cx<R> a, cx<R> b) {
  return {a.re + b.re, a.im + b.im};
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator-(cx<R> a, cx<R> b) {
  return {a.re - b.re, a.im - b.im};
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator-(cx<R> a) {
  return {-a.re, -a.im};
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(cx<R> a, cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> operator*(R s, cx<R> a) {
  return {s * a.re, s * a.im};
}
template <typename R>
__host__ __device__ __forceinline__ cx<R>& operator+=(cx<R>& a, cx<R> b) {
  a.re += b.re;
  a.im += b.im;
  return a;
}
template <typename R>
__host__ __device__ __forceinline__ cx<R>& operator-=(cx<R>& a, cx<R> b) {
  a.re -= b.re;
  a.im -= b.im;
  return a;
}
template <typename R>
__host__ __device__ __forceinline__ cx<R> conj(cx<R> a) {
  return {a.re, -a.im};
}
// conj(a) * b, the term of a dot product a^H b
template <typename R>
__host__ __device__ __forceinline__ cx<R> cmulc(cx<R> a, cx<R> b) {
  return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}
template <typename R>
__host__ __device__ __forceinline__ R abs2(cx<R> a) {
  return a.re * a.re + a.im * a.im;
}
// |a| without overflow or underflow of the squares (LAPACK's xLAPY2 rule)
template <typename R>
__host__ __device__ __forceinline__ R cabs(cx<R> a) {
  const R x = fabs(a.re), y = fabs(a.im);
  const R w = x > y ? x : y, z = x > y ? y : x;
  if (z == R(0) || w != w) return w + z;
  const R q = z / w;
  return w * sqrt(R(1) + q * q);
}
// a / b by Smith's scaling (the rule of LAPACK's xLADIV in spirit)
template <typename R>
__host__ __device__ __forceinline__ cx<R> cdiv(cx<R> a, cx<R> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const R r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  const R r = b.re / b.im, d = b.im + b.re * r;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

}  // namespace lra
