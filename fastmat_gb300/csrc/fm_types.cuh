// Element types, arithmetic and dtype conversion for the matvec kernels.
//
// The engine computes in one of five element types: float, double (real
// operators such as Hadamard/Diag on real data), float2, double2 (complex,
// stored interleaved exactly like numpy complex64/complex128) and long long
// (integer-only operator trees; results are narrowed to the fastmat output
// type on store, which reproduces fastmat's wrap-around integer arithmetic
// because wrapping is a ring homomorphism).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fmgpu.h"

namespace fmk {

typedef long long i64;

// ---------------------------------------------------------------- traits
template <class E> struct Tr;
template <> struct Tr<float> {
  static constexpr bool cplx = false;
  static constexpr int code = FM_F32;
  typedef float R;
};
template <> struct Tr<double> {
  static constexpr bool cplx = false;
  static constexpr int code = FM_F64;
  typedef double R;
};
template <> struct Tr<float2> {
  static constexpr bool cplx = true;
  static constexpr int code = FM_C64;
  typedef float R;
};
template <> struct Tr<double2> {
  static constexpr bool cplx = true;
  static constexpr int code = FM_C128;
  typedef double R;
};
template <> struct Tr<i64> {
  static constexpr bool cplx = false;
  static constexpr int code = FM_I64;
  typedef i64 R;
};

// shared-memory padding: one spare element per 128 bytes keeps strided
// butterfly accesses spread over all banks.
template <class E> struct PadShift;
template <> struct PadShift<float> { static constexpr int v = 5; };
template <> struct PadShift<double> { static constexpr int v = 4; };
template <> struct PadShift<i64> { static constexpr int v = 4; };
template <> struct PadShift<float2> { static constexpr int v = 4; };
template <> struct PadShift<double2> { static constexpr int v = 3; };

template <class E> __host__ __device__ __forceinline__ int pidx(int i) {
  return i + (i >> PadShift<E>::v);
}

// ---------------------------------------------------------------- arithmetic
__device__ __forceinline__ float2 operator+(float2 a, float2 b) {
  return make_float2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float2 operator-(float2 a, float2 b) {
  return make_float2(a.x - b.x, a.y - b.y);
}
__device__ __forceinline__ double2 operator+(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ double2 operator-(double2 a, double2 b) {
  return make_double2(a.x - b.x, a.y - b.y);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}

// generic multiply for all element types (conj applies to b)
__device__ __forceinline__ float mulv(float a, float b, bool) { return a * b; }
__device__ __forceinline__ double mulv(double a, double b, bool) {
  return a * b;
}
__device__ __forceinline__ i64 mulv(i64 a, i64 b, bool) { return a * b; }
__device__ __forceinline__ float2 mulv(float2 a, float2 b, bool c) {
  return c ? cmulc(a, b) : cmul(a, b);
}
__device__ __forceinline__ double2 mulv(double2 a, double2 b, bool c) {
  return c ? cmulc(a, b) : cmul(a, b);
}

__device__ __forceinline__ float conjv(float a) { return a; }
__device__ __forceinline__ double conjv(double a) { return a; }
__device__ __forceinline__ i64 conjv(i64 a) { return a; }
__device__ __forceinline__ float2 conjv(float2 a) {
  return make_float2(a.x, -a.y);
}
__device__ __forceinline__ double2 conjv(double2 a) {
  return make_double2(a.x, -a.y);
}

template <class E> __device__ __forceinline__ E zero();
template <> __device__ __forceinline__ float zero<float>() { return 0.f; }
template <> __device__ __forceinline__ double zero<double>() { return 0.; }
template <> __device__ __forceinline__ i64 zero<i64>() { return 0; }
template <> __device__ __forceinline__ float2 zero<float2>() {
  return make_float2(0.f, 0.f);
}
template <> __device__ __forceinline__ double2 zero<double2>() {
  return make_double2(0., 0.);
}

__device__ __forceinline__ float addv(float a, float b) { return a + b; }
__device__ __forceinline__ double addv(double a, double b) { return a + b; }
__device__ __forceinline__ i64 addv(i64 a, i64 b) { return a + b; }
__device__ __forceinline__ float2 addv(float2 a, float2 b) { return a + b; }
__device__ __forceinline__ double2 addv(double2 a, double2 b) { return a + b; }
__device__ __forceinline__ float subv(float a, float b) { return a - b; }
__device__ __forceinline__ double subv(double a, double b) { return a - b; }
__device__ __forceinline__ i64 subv(i64 a, i64 b) { return a - b; }
__device__ __forceinline__ float2 subv(float2 a, float2 b) { return a - b; }
__device__ __forceinline__ double2 subv(double2 a, double2 b) { return a - b; }

// scale by a (possibly complex) scalar given in double precision
__device__ __forceinline__ float scalev(float a, double sr, double) {
  return a * (float)sr;
}
__device__ __forceinline__ double scalev(double a, double sr, double) {
  return a * sr;
}
__device__ __forceinline__ i64 scalev(i64 a, double sr, double) {
  return a * (i64)sr;
}
__device__ __forceinline__ float2 scalev(float2 a, double sr, double si) {
  return cmul(a, make_float2((float)sr, (float)si));
}
__device__ __forceinline__ double2 scalev(double2 a, double sr, double si) {
  return cmul(a, make_double2(sr, si));
}

// ---------------------------------------------------------------- conversion
// A loaded source element, widened to (re, im) doubles or an integer.
struct Wide {
  double re, im;
  i64 iv;
  bool is_int;
};

__device__ __forceinline__ Wide load_wide(const void *p, int type, i64 idx) {
  Wide w;
  w.im = 0.;
  w.is_int = false;
  w.iv = 0;
  switch (type) {
    case FM_I8: w.iv = ((const int8_t *)p)[idx]; w.is_int = true; break;
    case FM_I16: w.iv = ((const int16_t *)p)[idx]; w.is_int = true; break;
    case FM_I32: w.iv = ((const int32_t *)p)[idx]; w.is_int = true; break;
    case FM_I64: w.iv = ((const i64 *)p)[idx]; w.is_int = true; break;
    case FM_F32: w.re = ((const float *)p)[idx]; break;
    case FM_F64: w.re = ((const double *)p)[idx]; break;
    case FM_C64: {
      float2 v = ((const float2 *)p)[idx];
      w.re = v.x;
      w.im = v.y;
      break;
    }
    default: {
      double2 v = ((const double2 *)p)[idx];
      w.re = v.x;
      w.im = v.y;
      break;
    }
  }
  if (w.is_int) w.re = (double)w.iv;
  return w;
}

template <class E> __device__ __forceinline__ E from_wide(const Wide &w);
template <> __device__ __forceinline__ float from_wide<float>(const Wide &w) {
  return (float)w.re;
}
template <> __device__ __forceinline__ double from_wide<double>(const Wide &w) {
  return w.re;
}
template <> __device__ __forceinline__ i64 from_wide<i64>(const Wide &w) {
  return w.is_int ? w.iv : (i64)w.re;
}
template <> __device__ __forceinline__ float2 from_wide<float2>(const Wide &w) {
  return make_float2((float)w.re, (float)w.im);
}
template <>
__device__ __forceinline__ double2 from_wide<double2>(const Wide &w) {
  return make_double2(w.re, w.im);
}

// Load element idx of a buffer of element type `type` as E.  The common case
// (buffer already in the compute type) is a single typed load.
template <class E>
__device__ __forceinline__ E load_as(const void *p, int type, i64 idx) {
  if (type == Tr<E>::code) return ((const E *)p)[idx];
  return from_wide<E>(load_wide(p, type, idx));
}

__device__ __forceinline__ void split(float v, double &re, double &im) {
  re = v;
  im = 0.;
}
__device__ __forceinline__ void split(double v, double &re, double &im) {
  re = v;
  im = 0.;
}
__device__ __forceinline__ void split(i64 v, double &re, double &im) {
  re = (double)v;
  im = 0.;
}
__device__ __forceinline__ void split(float2 v, double &re, double &im) {
  re = v.x;
  im = v.y;
}
__device__ __forceinline__ void split(double2 v, double &re, double &im) {
  re = v.x;
  im = v.y;
}

// Store v (compute type E) into a buffer of element type `type`, optionally
// adding to what is there.
template <class E>
__device__ __forceinline__ void store_as(void *p, int type, i64 idx, E v,
                                         bool acc) {
  if (type == Tr<E>::code) {
    E *q = (E *)p + idx;
    *q = acc ? addv(*q, v) : v;
    return;
  }
  if constexpr (Tr<E>::code == FM_I64) {
    // integer compute narrowed to the output integer type (wraps like
    // fastmat's typed integer loops)
    const i64 iv = v;
    switch (type) {
      case FM_I8: {
        int8_t *q = (int8_t *)p + idx;
        *q = (int8_t)(acc ? (i64)*q + iv : iv);
        return;
      }
      case FM_I16: {
        int16_t *q = (int16_t *)p + idx;
        *q = (int16_t)(acc ? (i64)*q + iv : iv);
        return;
      }
      case FM_I32: {
        int32_t *q = (int32_t *)p + idx;
        *q = (int32_t)(acc ? (i64)*q + iv : iv);
        return;
      }
      default: break;
    }
  }
  double re, im;
  split(v, re, im);
  switch (type) {
    case FM_F32: {
      float *q = (float *)p + idx;
      *q = acc ? *q + (float)re : (float)re;
      return;
    }
    case FM_F64: {
      double *q = (double *)p + idx;
      *q = acc ? *q + re : re;
      return;
    }
    case FM_C64: {
      float2 *q = (float2 *)p + idx;
      float2 n = make_float2((float)re, (float)im);
      *q = acc ? *q + n : n;
      return;
    }
    case FM_C128: {
      double2 *q = (double2 *)p + idx;
      double2 n = make_double2(re, im);
      *q = acc ? *q + n : n;
      return;
    }
    case FM_I64: {
      i64 *q = (i64 *)p + idx;
      i64 n = (i64)re;
      *q = acc ? *q + n : n;
      return;
    }
    default: return;
  }
}

}  // namespace fmk
