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

// ---------------------------------------------------------------- double-float
// A double-float number is an unevaluated sum h + l of two floats with
// |l| <= ulp(h) / 2, carrying a 48-bit significand (relative precision about
// 2^-48) on the FP32 pipes.  Sums use Knuth's TwoSum, products Dekker's
// TwoProduct through the fused multiply-add (both error-free
// transformations), each followed by a renormalisation (Fast2Sum).  The
// sum is the "sloppy" variant: its error is bounded by 2^-46 (|a| + |b|),
// the norm-wise bound an FFT error analysis needs.
struct df {
  float h, l;
  df() = default;
  __host__ __device__ constexpr df(float h_, float l_) : h(h_), l(l_) {}
  // compile-time constants: split a double literal into two floats
  __host__ __device__ constexpr df(double d)
      : h((float)d), l((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr df(int i) : h((float)i), l(0.f) {}
};
struct dfc {
  df x, y;  // real, imaginary
};

__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = a + b;
  return df(s, b - (s - a));
}
__device__ __forceinline__ df operator+(df a, df b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb) + (a.l + b.l);
  return fast_two_sum(s, e);
}
__device__ __forceinline__ df operator-(df a) { return df(-a.h, -a.l); }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return fast_two_sum(p, e);
}
// sign * x for sign = +1 / -1
__device__ __forceinline__ df operator*(int s, df a) { return s < 0 ? -a : a; }
__device__ __forceinline__ float smul(int s, float a) { return s < 0 ? -a : a; }
__device__ __forceinline__ double smul(int s, double a) {
  return s < 0 ? -a : a;
}
__device__ __forceinline__ df smul(int s, df a) { return s < 0 ? -a : a; }

__device__ __forceinline__ dfc operator+(dfc a, dfc b) {
  return dfc{a.x + b.x, a.y + b.y};
}
__device__ __forceinline__ dfc operator-(dfc a, dfc b) {
  return dfc{a.x - b.x, a.y - b.y};
}
__device__ __forceinline__ dfc cmul(dfc a, dfc b) {
  return dfc{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ dfc cmulc(dfc a, dfc b) {
  return dfc{a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};
}

// Unnormalised double-float, for the additions inside one butterfly: the
// head is the rounded sum of the heads (TwoSum keeps its rounding error
// exactly) and the tail collects tails and errors without renormalising,
// 8 FP32 operations per addition instead of 11; a product skips the final
// renormalisation too (4 instead of 7).  Tails stay a few units of 2^-24
// of the magnitudes that entered the chain, so a chain of k operations
// keeps the norm-wise error bound of about k 2^-48 times the sum of those
// magnitudes (the bound an FFT error analysis uses).  Values are
// renormalised (Fast2Sum) when they leave the butterfly.
struct dfu {
  float h, l;
  dfu() = default;
  __host__ __device__ constexpr dfu(float h_, float l_) : h(h_), l(l_) {}
  __host__ __device__ constexpr dfu(double d)
      : h((float)d), l((float)(d - (double)(float)d)) {}
};
struct dfcu {
  dfu x, y;
};
__device__ __forceinline__ dfu operator+(dfu a, dfu b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb);
  return dfu(s, (a.l + b.l) + e);
}
__device__ __forceinline__ dfu operator-(dfu a) { return dfu(-a.h, -a.l); }
__device__ __forceinline__ dfu operator-(dfu a, dfu b) { return a + (-b); }
__device__ __forceinline__ dfu operator*(dfu a, dfu b) {
  const float p = a.h * b.h;
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return dfu(p, e);
}
__device__ __forceinline__ dfu smul(int s, dfu a) { return s < 0 ? -a : a; }
__device__ __forceinline__ dfcu operator+(dfcu a, dfcu b) {
  return dfcu{a.x + b.x, a.y + b.y};
}
__device__ __forceinline__ dfcu operator-(dfcu a, dfcu b) {
  return dfcu{a.x - b.x, a.y - b.y};
}

// double -> double-float with integer operations only (the FP64 pipe of
// this GPU is slow): h is d rounded to 24 bits, l the float nearest to the
// exact remainder d - h.  Zeros, subnormals and values outside the float
// exponent range map to (0, 0) / (+-inf, 0).
__device__ __forceinline__ df d2df(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sgn = (unsigned)(b >> 63) << 31;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return df(0.f, 0.f);
  int e = ex - 1023;
  if (ex == 0x7FF || e > 127)
    return df(__int_as_float((int)(sgn | 0x7F800000u)), 0.f);
  if (e < -126) return df(0.f, 0.f);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned long long mh = m >> 29;  // 24 bits
  const unsigned long long rem = m & 0x1FFFFFFFull;
  const unsigned long long half = 1ull << 28;
  if (rem > half || (rem == half && (mh & 1))) ++mh;
  // remainder relative to the rounded head: m - mh * 2^29 (|.| <= 2^28)
  const long long r = (long long)m - (long long)(mh << 29);
  if (mh == (1ull << 24)) {  // rounding carried into the next binade
    mh >>= 1;
    ++e;
    if (e > 127) return df(__int_as_float((int)(sgn | 0x7F800000u)), 0.f);
  }
  const float h = __int_as_float(
      (int)(sgn | ((unsigned)(e + 127) << 23) | (unsigned)(mh & 0x7FFFFF)));
  // l = r * 2^(e0 - 52) with e0 the exponent before any carry
  const int el = ex - 1023 - 52;
  float l = (float)(int)r;  // |r| <= 2^28: rounds to 24 bits
  if (el >= -126) {
    l *= __int_as_float((el + 127) << 23);
  } else if (el >= -126 - 23) {
    l *= __int_as_float((el + 127 + 24) << 23);
    l *= __int_as_float((127 - 24) << 23);
  } else {
    l = 0.f;
  }
  if (sgn) l = -l;
  return df(h, l);
}

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
// double-float types hold (complex) float64 data: their buffers in global
// memory are float64 / complex128, converted on load and store (emu)
template <> struct Tr<df> {
  static constexpr bool cplx = false;
  static constexpr int code = FM_F64;
  typedef df R;
};
template <> struct Tr<dfc> {
  static constexpr bool cplx = true;
  static constexpr int code = FM_C128;
  typedef df R;
};
template <> struct Tr<dfu> {
  static constexpr bool cplx = false;
  static constexpr int code = FM_F64;
  typedef dfu R;
};
template <> struct Tr<dfcu> {
  static constexpr bool cplx = true;
  static constexpr int code = FM_C128;
  typedef dfu R;
};
// the type a butterfly computes in: unnormalised for double-float
template <class C> struct Lazy { typedef C type; };
template <> struct Lazy<df> { typedef dfu type; };
template <> struct Lazy<dfc> { typedef dfcu type; };
template <class C> __device__ __forceinline__ C to_lazy(C a) { return a; }
template <class C> __device__ __forceinline__ C from_lazy(C a) { return a; }
__device__ __forceinline__ dfu to_lazy(df a) { return dfu(a.h, a.l); }
__device__ __forceinline__ dfcu to_lazy(dfc a) {
  return dfcu{dfu(a.x.h, a.x.l), dfu(a.y.h, a.y.l)};
}
__device__ __forceinline__ df from_lazy(dfu a) {
  return fast_two_sum(a.h, a.l);
}
__device__ __forceinline__ dfc from_lazy(dfcu a) {
  return dfc{fast_two_sum(a.x.h, a.x.l), fast_two_sum(a.y.h, a.y.l)};
}
template <class E> struct Emu { static constexpr bool v = false; };
template <> struct Emu<df> { static constexpr bool v = true; };
template <> struct Emu<dfc> { static constexpr bool v = true; };

// shared-memory padding: one spare 16-byte granule per 128 bytes keeps
// strided butterfly accesses spread over the banks while every 128-byte
// chunk of a vector stays 16-byte aligned (a bulk-copy destination)
template <class E> struct PadShift {
  static constexpr int v = sizeof(E) == 4 ? 5 : (sizeof(E) == 8 ? 4 : 3);
  static constexpr int mul = 16 / (int)sizeof(E);
};

template <class E> __host__ __device__ __forceinline__ int pidx(int i) {
  return i + PadShift<E>::mul * (i >> PadShift<E>::v);
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

__device__ __forceinline__ df mulv(df a, df b, bool) { return a * b; }
__device__ __forceinline__ dfc mulv(dfc a, dfc b, bool c) {
  return c ? cmulc(a, b) : cmul(a, b);
}
__device__ __forceinline__ df conjv(df a) { return a; }
__device__ __forceinline__ dfc conjv(dfc a) { return dfc{a.x, -a.y}; }
__device__ __forceinline__ df addv(df a, df b) { return a + b; }
__device__ __forceinline__ dfc addv(dfc a, dfc b) { return a + b; }
__device__ __forceinline__ df subv(df a, df b) { return a - b; }
__device__ __forceinline__ dfc subv(dfc a, dfc b) { return a - b; }
__device__ __forceinline__ dfu addv(dfu a, dfu b) { return a + b; }
__device__ __forceinline__ dfcu addv(dfcu a, dfcu b) { return a + b; }
__device__ __forceinline__ dfu subv(dfu a, dfu b) { return a - b; }
__device__ __forceinline__ dfcu subv(dfcu a, dfcu b) { return a - b; }

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
template <> __device__ __forceinline__ df zero<df>() { return df(0.f, 0.f); }
template <> __device__ __forceinline__ dfc zero<dfc>() {
  return dfc{df(0.f, 0.f), df(0.f, 0.f)};
}

// a (complex) scalar given in double precision, in the element type E;
// for double-float types this is the host-free integer split
template <class E> __device__ __forceinline__ E scalar_of(double re, double im);
template <> __device__ __forceinline__ float scalar_of<float>(double re, double) {
  return (float)re;
}
template <> __device__ __forceinline__ double scalar_of<double>(double re, double) {
  return re;
}
template <> __device__ __forceinline__ i64 scalar_of<i64>(double re, double) {
  return (i64)re;
}
template <> __device__ __forceinline__ float2 scalar_of<float2>(double re, double im) {
  return make_float2((float)re, (float)im);
}
template <> __device__ __forceinline__ double2 scalar_of<double2>(double re, double im) {
  return make_double2(re, im);
}
template <> __device__ __forceinline__ df scalar_of<df>(double re, double) {
  return d2df(re);
}
template <> __device__ __forceinline__ dfc scalar_of<dfc>(double re, double im) {
  return dfc{d2df(re), d2df(im)};
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

template <> __device__ __forceinline__ df from_wide<df>(const Wide &w) {
  return d2df(w.re);
}
template <> __device__ __forceinline__ dfc from_wide<dfc>(const Wide &w) {
  return dfc{d2df(w.re), d2df(w.im)};
}

// Load element idx of a buffer of element type `type` as E.  The common case
// (buffer already in the compute type) is a single typed load.
template <class E>
__device__ __forceinline__ E load_as(const void *p, int type, i64 idx) {
  if constexpr (Emu<E>::v) {
    return from_wide<E>(load_wide(p, type, idx));
  } else {
    if (type == Tr<E>::code) return ((const E *)p)[idx];
    return from_wide<E>(load_wide(p, type, idx));
  }
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
// exponent field of a double (0 for zero / subnormal)
__device__ __forceinline__ int dexp(double d) {
  return (int)(((unsigned long long)__double_as_longlong(d) >> 52) & 0x7FF);
}
// in-place conversions of a double-float tile element and its float64 /
// complex128 bit pattern (same size)
// (s: power-of-two scale of the vector, removed on load, restored on store)
__device__ __forceinline__ int raw_exp(df raw) {
  return dexp(*reinterpret_cast<const double *>(&raw));
}
__device__ __forceinline__ int raw_exp(dfc raw) {
  const double2 d = *reinterpret_cast<const double2 *>(&raw);
  const int a = dexp(d.x), b = dexp(d.y);
  return a > b ? a : b;
}
// Tile conversions, branch-free (they run once per element on every load
// and store of the double-float kernels).
// float64 d times 2^-s -> double-float: h keeps the leading 24 significand
// bits (truncated), l is the other 29 bits rounded to a float, so h + l is
// within 2^-48 |d|.  s is the vector's largest exponent minus the bias (so
// every element's rebased float exponent is at most 127): elements more
// than 2^126 below that flush to zero, their l more than 2^74 below it;
// Inf and NaN stay Inf and NaN.
__device__ __forceinline__ df d2df_scaled(double d, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned sg = hi & 0x80000000u;
  const int ex = (int)((hi >> 20) & 0x7FFu);
  const int ef = ex - s - 896;  // biased float exponent of h
  const unsigned mh = __funnelshift_l(lo, hi, 3) & 0x7FFFFFu;
  float h = __int_as_float((int)(sg | ((unsigned)ef << 23) | mh));
  // the remaining bits weigh 2^(ef - 127 - 52) each
  float l = (float)(lo & 0x1FFFFFFFu) * __int_as_float((ef - 52) << 23);
  l = __int_as_float(__float_as_int(l) | (int)sg);
  if (ef < 53) l = 0.f;
  if (ef < 1) h = 0.f;
  if (ex == 0x7FF) {
    h = __int_as_float((int)(sg | (((hi & 0xFFFFFu) | lo) ? 0x7FC00000u
                                                           : 0x7F800000u)));
    l = 0.f;
  }
  return df(h, l);
}
// float -> float64, exact for normal floats; zero and subnormal floats give
// a signed zero, Inf and NaN stay Inf and NaN
__device__ __forceinline__ double f2d_fast(float f) {
  const unsigned u = (unsigned)__float_as_int(f);
  const unsigned ex = (u >> 23) & 0xFFu;
  // exponent rebased by 1023 - 127 = 896 (0x38000000 = 896 << 20)
  unsigned hi = (u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + 0x38000000u);
  unsigned lo = u << 29;
  if (ex == 0) {
    hi = u & 0x80000000u;
    lo = 0u;
  }
  if (ex == 0xFFu) hi |= 0x7FF00000u;
  return __hiloint2double((int)hi, (int)lo);
}
// d * 2^s by exponent arithmetic: zero, Inf and NaN unchanged, results
// beyond the float64 range saturate to Inf or flush to a signed zero
__device__ __forceinline__ double dscale_fast(double d, int s) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int ex = (int)((hi >> 20) & 0x7FFu);
  const int ne = ex + s;
  const unsigned sg = hi & 0x80000000u;
  unsigned nhi = hi + ((unsigned)s << 20), nlo = lo;
  if (ne <= 0) {
    nhi = sg;
    nlo = 0u;
  }
  if (ne >= 0x7FF) {
    nhi = sg | 0x7FF00000u;
    nlo = 0u;
  }
  if (ex == 0 || ex == 0x7FF) {
    nhi = hi;
    nlo = lo;
  }
  return __hiloint2double((int)nhi, (int)nlo);
}
__device__ __forceinline__ double df2d_scaled(df v, int s) {
  return dscale_fast(f2d_fast(v.h) + f2d_fast(v.l), s);
}

// (double-float values carry their vector's power-of-two scale s)
__device__ __forceinline__ void split(df v, double &re, double &im,
                                      int s = 0) {
  re = df2d_scaled(v, s);
  im = 0.;
}
__device__ __forceinline__ void split(dfc v, double &re, double &im,
                                      int s = 0) {
  re = df2d_scaled(v.x, s);
  im = df2d_scaled(v.y, s);
}

__device__ __forceinline__ df from_bits(df raw, int s) {
  return d2df_scaled(*reinterpret_cast<const double *>(&raw), s);
}
__device__ __forceinline__ dfc from_bits(dfc raw, int s) {
  const double2 d = *reinterpret_cast<const double2 *>(&raw);
  return dfc{d2df_scaled(d.x, s), d2df_scaled(d.y, s)};
}
__device__ __forceinline__ df to_bits(df v, int s) {
  const double d = df2d_scaled(v, s);
  return *reinterpret_cast<const df *>(&d);
}
__device__ __forceinline__ dfc to_bits(dfc v, int s) {
  const double2 d = make_double2(df2d_scaled(v.x, s), df2d_scaled(v.y, s));
  return *reinterpret_cast<const dfc *>(&d);
}

// Store v (compute type E) into a buffer of element type `type`, optionally
// adding to what is there.
template <class E>
__device__ __forceinline__ void store_as(void *p, int type, i64 idx, E v,
                                         bool acc, int scale = 0) {
  if (!Emu<E>::v && type == Tr<E>::code) {
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
  if constexpr (Emu<E>::v) split(v, re, im, scale);
  else split(v, re, im);
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
