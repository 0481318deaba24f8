// Column reductions for the gradients of the differentiable matvec path.
//
// fm_reduce_mulconj computes, for a column-major array viewed per column as
// a 3-D block (A, n, Cc) (row r = (a * n + j) * Cc + c, the same view the
// vector-program kernels use for one Kron mode),
//
//     out[j] = scale * sum_{a, c, column k} u[r, k] * conj(v[r, k])
//
// which is the parameter gradient of a diagonal factor (u = upstream
// gradient, v = the factor's input) and, with u and v in the Fourier domain,
// the spectrum of the circular cross-correlation that gives the gradient of
// a circulant or Toeplitz defining vector.  Optionally the same pass writes
// w[r, k] = conj(d[j]) * u[r, k], the adjoint of that diagonal factor
// (fastmat's Diag backward, fastmat/Diag.pyx:149-167), so a Diag at the
// input of a chain yields both of its gradients from one read of u.
//
// Two passes, deterministic: pass 1 writes per-slice partial sums
// (slices split the summed indices so that the grid covers the GPU), pass 2
// adds the slices of every j.  Both are streaming kernels bound by HBM.

#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"

namespace {

using i64 = long long;

__device__ __forceinline__ float mulconj(float u, float v) { return u * v; }
__device__ __forceinline__ double mulconj(double u, double v) {
  return u * v;
}
__device__ __forceinline__ float2 mulconj(float2 u, float2 v) {
  return make_float2(fmaf(u.x, v.x, u.y * v.y), fmaf(u.y, v.x, -u.x * v.y));
}
__device__ __forceinline__ double2 mulconj(double2 u, double2 v) {
  return make_double2(fma(u.x, v.x, u.y * v.y), fma(u.y, v.x, -u.x * v.y));
}
// conj(d) * u
__device__ __forceinline__ float conjmul(float d, float u) { return d * u; }
__device__ __forceinline__ double conjmul(double d, double u) {
  return d * u;
}
__device__ __forceinline__ float2 conjmul(float2 d, float2 u) {
  return make_float2(fmaf(d.x, u.x, d.y * u.y), fmaf(d.x, u.y, -d.y * u.x));
}
__device__ __forceinline__ double2 conjmul(double2 d, double2 u) {
  return make_double2(fma(d.x, u.x, d.y * u.y), fma(d.x, u.y, -d.y * u.x));
}

__device__ __forceinline__ void acc_add(float &a, float b) { a += b; }
__device__ __forceinline__ void acc_add(double &a, double b) { a += b; }
__device__ __forceinline__ void acc_add(float2 &a, float2 b) {
  a.x += b.x;
  a.y += b.y;
}
__device__ __forceinline__ void acc_add(double2 &a, double2 b) {
  a.x += b.x;
  a.y += b.y;
}
template <typename T> __device__ __forceinline__ T acc_zero() { return T{}; }

__device__ __forceinline__ float shfl_down(float v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ double shfl_down(double v, int o) {
  return __shfl_down_sync(0xffffffffu, v, o);
}
__device__ __forceinline__ float2 shfl_down(float2 v, int o) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, o),
                     __shfl_down_sync(0xffffffffu, v.y, o));
}
__device__ __forceinline__ double2 shfl_down(double2 v, int o) {
  return make_double2(__shfl_down_sync(0xffffffffu, v.x, o),
                      __shfl_down_sync(0xffffffffu, v.y, o));
}

__device__ __forceinline__ float scaled(float v, double s) {
  return (float)((double)v * s);
}
__device__ __forceinline__ double scaled(double v, double s) { return v * s; }
__device__ __forceinline__ float2 scaled(float2 v, double s) {
  return make_float2((float)((double)v.x * s), (float)((double)v.y * s));
}
__device__ __forceinline__ double2 scaled(double2 v, double s) {
  return make_double2(v.x * s, v.y * s);
}

constexpr int kThreads = 256;

// Pass 1, Cc == 1: consecutive threads take consecutive j (coalesced along
// the column); slice s sums pairs p = k * A + a in [p0, p1).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_reduce_rows(i64 A, i64 n, const T *__restrict__ u, i64 ldu,
              const T *__restrict__ v, i64 ldv, const T *__restrict__ d,
              T *__restrict__ w, i64 ldw, i64 P, i64 per,
              T *__restrict__ part) {
  const i64 j = (i64)blockIdx.x * kThreads + threadIdx.x;
  if (j >= n) return;
  const i64 s = blockIdx.y;
  const i64 p0 = s * per, p1 = min(P, p0 + per);
  T acc = acc_zero<T>();
  const T dj = d ? d[j] : acc_zero<T>();
  i64 a = p0 % A, k = p0 / A;
  for (i64 p = p0; p < p1; ++p) {
    const i64 r = a * n + j;
    const T uu = u[r + k * ldu];
    acc_add(acc, mulconj(uu, v[r + k * ldv]));
    if (w) w[r + k * ldw] = conjmul(dj, uu);
    if (++a == A) {
      a = 0;
      ++k;
    }
  }
  part[s * n + j] = acc;
}

// Pass 1, Cc > 1: one block per (j, slice); consecutive threads take
// consecutive c (coalesced inside each run of Cc elements).
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_reduce_runs(i64 A, i64 n, i64 Cc, const T *__restrict__ u, i64 ldu,
              const T *__restrict__ v, i64 ldv, const T *__restrict__ d,
              T *__restrict__ w, i64 ldw, i64 E, i64 per,
              T *__restrict__ part) {
  const i64 j = blockIdx.x;
  const i64 s = blockIdx.y;
  const i64 e0 = s * per, e1 = min(E, e0 + per);
  T acc = acc_zero<T>();
  const T dj = d ? d[j] : acc_zero<T>();
  for (i64 e = e0 + threadIdx.x; e < e1; e += kThreads) {
    const i64 c = e % Cc, p = e / Cc;
    const i64 a = p % A, k = p / A;
    const i64 r = (a * n + j) * Cc + c;
    const T uu = u[r + k * ldu];
    acc_add(acc, mulconj(uu, v[r + k * ldv]));
    if (w) w[r + k * ldw] = conjmul(dj, uu);
  }
  __shared__ T red[kThreads / 32];
  for (int o = 16; o > 0; o >>= 1) acc_add(acc, shfl_down(acc, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : acc_zero<T>();
    for (int o = 16; o > 0; o >>= 1) acc_add(acc, shfl_down(acc, o));
    if (threadIdx.x == 0) part[s * n + j] = acc;
  }
}

// Pass 2: out[j] = scale * sum over slices.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_reduce_slices(i64 n, i64 S, const T *__restrict__ part, double scale,
                T *__restrict__ out) {
  const i64 j = (i64)blockIdx.x * kThreads + threadIdx.x;
  if (j >= n) return;
  T acc = acc_zero<T>();
  for (i64 s = 0; s < S; ++s) acc_add(acc, part[s * n + j]);
  out[j] = scaled(acc, scale);
}

struct Fail {
  int code;
  std::string msg;
};

int sms_of_device() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 132;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
      cudaSuccess)
    return 132;
  return sms > 0 ? sms : 132;
}

template <typename T>
void run(i64 A, i64 n, i64 Cc, i64 cols, const void *u, i64 ldu,
         const void *v, i64 ldv, void *out, double scale, const void *d,
         void *w, i64 ldw, cudaStream_t st) {
  const i64 target = (i64)sms_of_device() * 16;  // blocks to cover the GPU
  const i64 P = A * cols;                         // (a, column) pairs per j
  i64 S, per;
  if (Cc == 1) {
    const i64 jb = (n + kThreads - 1) / kThreads;
    S = std::max<i64>(1, std::min<i64>(P, (target + jb - 1) / jb));
    S = std::min<i64>(S, 65535);
    per = (P + S - 1) / S;
    S = (P + per - 1) / per;
  } else {
    const i64 E = P * Cc;
    S = std::max<i64>(1, std::min<i64>((target + n - 1) / n,
                                       (E + 4 * kThreads - 1) /
                                           (4 * kThreads)));
    S = std::min<i64>(S, 65535);
    per = (E + S - 1) / S;
    S = (E + per - 1) / per;
  }
  if (n > 2147483647LL && Cc > 1) throw Fail{FM_ERR_VALUE, "n too large"};
  T *part = nullptr;
  cudaError_t e =
      cudaMallocAsync((void **)&part, sizeof(T) * (size_t)(S * n), st);
  if (e != cudaSuccess)
    throw Fail{e == cudaErrorMemoryAllocation ? FM_ERR_NOMEM : FM_ERR_CUDA,
               std::string("cudaMallocAsync: ") + cudaGetErrorString(e)};
  if (Cc == 1) {
    dim3 grid((unsigned)((n + kThreads - 1) / kThreads), (unsigned)S);
    k_reduce_rows<T><<<grid, kThreads, 0, st>>>(
        A, n, (const T *)u, ldu, (const T *)v, ldv, (const T *)d, (T *)w,
        ldw, P, per, part);
  } else {
    dim3 grid((unsigned)n, (unsigned)S);
    k_reduce_runs<T><<<grid, kThreads, 0, st>>>(
        A, n, Cc, (const T *)u, ldu, (const T *)v, ldv, (const T *)d, (T *)w,
        ldw, P * Cc, per, part);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_reduce_slices<T><<<(unsigned)((n + kThreads - 1) / kThreads), kThreads,
                         0, st>>>(n, S, part, scale, (T *)out);
    e = cudaGetLastError();
  }
  cudaFreeAsync(part, st);
  if (e != cudaSuccess)
    throw Fail{FM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e)};
}

int elem_size(int t) {
  switch (t) {
    case FM_F32: return 4;
    case FM_F64: return 8;
    case FM_C64: return 8;
    case FM_C128: return 16;
    default: return 0;
  }
}

}  // namespace

extern "C" int fm_reduce_mulconj(int64_t A, int64_t n, int64_t Cc,
                                 int64_t num_cols, int32_t type,
                                 const void *u, int64_t ld_u, const void *v,
                                 int64_t ld_v, void *out, double scale,
                                 const void *d, void *w, int64_t ld_w,
                                 void *stream) {
  try {
    const int es = elem_size(type);
    if (!es) throw Fail{FM_ERR_TYPE, "fm_reduce_mulconj: type must be "
                                     "FM_F32, FM_F64, FM_C64 or FM_C128"};
    if (A < 0 || n < 0 || Cc < 0 || num_cols < 0)
      throw Fail{FM_ERR_VALUE, "fm_reduce_mulconj: negative size"};
    if (n == 0) return FM_OK;
    if (!out) throw Fail{FM_ERR_VALUE, "fm_reduce_mulconj: out is NULL"};
    cudaStream_t st = (cudaStream_t)stream;
    const i64 rows = A * n * Cc;
    if (A == 0 || Cc == 0 || num_cols == 0) {
      cudaError_t e = cudaMemsetAsync(out, 0, (size_t)n * es, st);
      if (e != cudaSuccess)
        throw Fail{FM_ERR_CUDA, std::string("cudaMemsetAsync: ") +
                                    cudaGetErrorString(e)};
      return FM_OK;
    }
    if (!u || !v)
      throw Fail{FM_ERR_VALUE, "fm_reduce_mulconj: u or v is NULL"};
    if ((d == nullptr) != (w == nullptr))
      throw Fail{FM_ERR_VALUE, "fm_reduce_mulconj: d and w go together"};
    if (num_cols > 1 && (ld_u < rows || ld_v < rows || (w && ld_w < rows)))
      throw Fail{FM_ERR_VALUE, "fm_reduce_mulconj: leading dimension "
                               "smaller than A * n * Cc"};
    switch (type) {
      case FM_F32:
        run<float>(A, n, Cc, num_cols, u, ld_u, v, ld_v, out, scale, d, w,
                   ld_w, st);
        break;
      case FM_F64:
        run<double>(A, n, Cc, num_cols, u, ld_u, v, ld_v, out, scale, d, w,
                    ld_w, st);
        break;
      case FM_C64:
        run<float2>(A, n, Cc, num_cols, u, ld_u, v, ld_v, out, scale, d, w,
                    ld_w, st);
        break;
      default:
        run<double2>(A, n, Cc, num_cols, u, ld_u, v, ld_v, out, scale, d, w,
                     ld_w, st);
        break;
    }
    return FM_OK;
  } catch (const Fail &f) {
    fmk::set_last_error(f.msg.c_str());
    return f.code;
  }
}
