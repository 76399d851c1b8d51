// Core types shared by every kernel of libkhp: complex scalars, status codes, and the "team"
// abstraction the dense algorithms are written against.
//
// A Team is the group of threads that cooperates on one problem (one CTA on the GPU).  The
// algorithms are __host__ __device__ templates over the Team type: on the GPU TeamCta maps to
// threadIdx/blockDim/__syncthreads; the serial TeamSerial (one thread, no-op barrier) lets the
// same algorithm source be compiled by g++ and checked on a machine without a GPU.
#pragma once

#include <cstdint>
#include <cmath>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

#define KHP_HD __host__ __device__ __forceinline__

namespace khp {

#ifndef __CUDACC__
using std::copysign;
using std::cos;
using std::exp;
using std::fabs;
using std::fma;
using std::hypot;
using std::isfinite;
using std::sin;
using std::sqrt;
#endif

// ---- status codes (per call); the same values as the public C header defines -------------
#ifndef KHP_OK
#define KHP_OK 0
#define KHP_ERR_INVALID_ARG 1
#define KHP_ERR_WORKSPACE 2
#define KHP_ERR_CUDA 3
#define KHP_ERR_SINGULAR 4
#define KHP_ERR_NOT_CONVERGED 5
#define KHP_ERR_NONFINITE 6
#define KHP_ERR_TOO_LARGE 7
#endif

// Per-problem status words are OR-ed bit flags so that several conditions can be recorded.
enum StatusBit : int {
  KHP_BIT_SINGULAR = 1,
  KHP_BIT_NOT_CONVERGED = 2,
  KHP_BIT_NONFINITE = 4,
  KHP_BIT_REFINE = 8,      // mixed-precision iterative refinement did not converge: re-solve in FP64
  KHP_BIT_BAD_INPUT = 16,  // a per-problem input outside its range (e.g. a map index)
  KHP_BIT_MODES = 32,      // mixed-precision eigen-refinement left a residual above 1e-8: re-solve in FP64
};

// ---- complex scalar with the memory layout of numpy/torch complex64 / complex128 ----------
template <typename T>
struct alignas(2 * sizeof(T)) cplx {
  T re, im;
};

template <typename T> KHP_HD cplx<T> mk(T r, T i = T(0)) { cplx<T> z; z.re = r; z.im = i; return z; }
template <typename T> KHP_HD cplx<T> operator+(cplx<T> a, cplx<T> b) { return mk(a.re + b.re, a.im + b.im); }
template <typename T> KHP_HD cplx<T> operator-(cplx<T> a, cplx<T> b) { return mk(a.re - b.re, a.im - b.im); }
template <typename T> KHP_HD cplx<T> operator-(cplx<T> a) { return mk(-a.re, -a.im); }
template <typename T> KHP_HD cplx<T> operator*(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> KHP_HD cplx<T> operator*(T s, cplx<T> a) { return mk(s * a.re, s * a.im); }
template <typename T> KHP_HD cplx<T> operator*(cplx<T> a, T s) { return mk(s * a.re, s * a.im); }
template <typename T> KHP_HD cplx<T>& operator+=(cplx<T>& a, cplx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <typename T> KHP_HD cplx<T>& operator-=(cplx<T>& a, cplx<T> b) { a.re -= b.re; a.im -= b.im; return a; }
template <typename T> KHP_HD cplx<T> conj(cplx<T> a) { return mk(a.re, -a.im); }
template <typename T> KHP_HD T norm2(cplx<T> a) { return a.re * a.re + a.im * a.im; }
template <typename T> KHP_HD T abs1(cplx<T> a) { return fabs(a.re) + fabs(a.im); }
template <typename T> KHP_HD T cabs(cplx<T> a) { return hypot(a.re, a.im); }
// a * conj(b) and conj(a) * b without forming the conjugate
template <typename T> KHP_HD cplx<T> mul_conj(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
}
template <typename T> KHP_HD cplx<T> conj_mul(cplx<T> a, cplx<T> b) {
  return mk(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
// acc += a * b (fused where the compiler can)
template <typename T> KHP_HD void fma_acc(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(a.re, b.re, acc.re); acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im); acc.im = fma(a.im, b.re, acc.im);
}
template <typename T> KHP_HD void fms_acc(cplx<T>& acc, cplx<T> a, cplx<T> b) {
  acc.re = fma(-a.re, b.re, acc.re); acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(-a.re, b.im, acc.im); acc.im = fma(-a.im, b.re, acc.im);
}
// Robust complex division a / b (Smith's algorithm).
template <typename T> KHP_HD cplx<T> cdiv(cplx<T> a, cplx<T> b) {
  if (fabs(b.re) >= fabs(b.im)) {
    if (b.re == T(0) && b.im == T(0)) return mk(a.re / b.re, a.im / b.re);
    T r = b.im / b.re, d = b.re + b.im * r;
    return mk((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  }
  T r = b.re / b.im, d = b.im + b.re * r;
  return mk((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
// Principal square root (branch cut on the negative real axis, Re >= 0; sqrt(-x + 0i) = +i sqrt(x),
// sqrt(-x - 0i) = -i sqrt(x), matching numpy's complex sqrt with signed zeros).
template <typename T> KHP_HD cplx<T> csqrt(cplx<T> z) {
  T x = z.re, y = z.im;
  if (x == T(0) && y == T(0)) return mk(T(0), y);
  T r = hypot(x, y);
  if (x >= T(0)) {
    T t = sqrt(T(0.5) * (r + x));
    return mk(t, y / (T(2) * t));
  }
  T t = sqrt(T(0.5) * (r - x));
  return mk(fabs(y) / (T(2) * t), copysign(t, y));
}
template <typename T> KHP_HD cplx<T> cexp(cplx<T> z) {
  T e = exp(z.re);
  return mk(e * cos(z.im), e * sin(z.im));
}
template <typename T> KHP_HD bool cfinite(cplx<T> z) { return isfinite(z.re) && isfinite(z.im); }

template <typename T> struct Eps;
template <> struct Eps<double> {
  static constexpr double ulp = 2.220446049250313e-16;
  static constexpr double safemin = 2.2250738585072014e-308;
};
template <> struct Eps<float> {
  static constexpr float ulp = 1.1920929e-07f;
  static constexpr float safemin = 1.17549435e-38f;
};

// ---- teams -----------------------------------------------------------------------------------
struct TeamSerial {
  KHP_HD int tid() const { return 0; }
  KHP_HD int size() const { return 1; }
  KHP_HD void sync() const {}
  KHP_HD void warp_sync() const {}
};

#ifdef __CUDACC__
struct TeamCta {
  __device__ __forceinline__ int tid() const { return threadIdx.x; }
  __device__ __forceinline__ int size() const { return blockDim.x; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  // barrier among the 32 lanes of the calling warp (used by warp-0-only phases)
  __device__ __forceinline__ void warp_sync() const { __syncwarp(); }
};
#endif

// Shared scratch every team algorithm receives (one per CTA, in shared memory on the GPU):
// per-warp reduction partials and a few broadcast slots for scalars chosen by thread 0.
struct TeamShared {
  double rv[32];
  int ri[32];
  double bd[16];
  int bi[16];
};

// Sum of one value per thread, returned to every thread (fixed summation order: deterministic).
template <typename T> KHP_HD T team_sum(const TeamSerial&, T v, TeamShared*) { return v; }
// Largest v over the team with its index (ties -> smallest index), returned to every thread.
template <typename T> KHP_HD void team_argmax(const TeamSerial&, T& v, int& idx, TeamShared*) {}

// Sum of a complex value over the 32 lanes of a warp, returned to every lane (TeamSerial: itself).
template <typename T> KHP_HD cplx<T> warp_sum(const TeamSerial&, cplx<T> v) { return v; }

#ifdef __CUDACC__
template <typename T> __device__ __forceinline__ cplx<T> warp_sum(const TeamCta&, cplx<T> v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return v;
}
template <typename T> __device__ __forceinline__ T team_sum(const TeamCta&, T v, TeamShared* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();  // earlier readers of sh->rv are done
  if ((threadIdx.x & 31) == 0) sh->rv[w] = (double)v;
  __syncthreads();
  double s = 0.0;
  for (int k = 0; k < nw; ++k) s += sh->rv[k];
  return (T)s;
}
template <typename T> __device__ __forceinline__ void team_argmax(const TeamCta&, T& v, int& idx, TeamShared* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    T ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { sh->rv[w] = (double)v; sh->ri[w] = idx; }
  __syncthreads();
  double bv = sh->rv[0];
  int bi = sh->ri[0];
  for (int k = 1; k < nw; ++k) {
    if (sh->rv[k] > bv || (sh->rv[k] == bv && sh->ri[k] < bi)) { bv = sh->rv[k]; bi = sh->ri[k]; }
  }
  v = (T)bv;
  idx = bi;
}
#endif

// Strided view of a batch of row-major matrices: element (b, i, j) at base + b*bs + i*ld + j.
template <typename T>
struct MatB {
  cplx<T>* p;
  int64_t ld;
  int64_t bs;
  KHP_HD cplx<T>* at(int64_t b) const { return p + b * bs; }
};

}  // namespace khp
