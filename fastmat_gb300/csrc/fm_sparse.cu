// Sparse (CSR) matrix times a block of columns: the launch behind fastmat's
// Sparse operator (fastmat/Sparse.pyx:25-185, forward S x and backward
// S^H x, both CSR products in scipy).
//
// A group of G lanes (G a power of two up to a warp, picked from the mean
// row length) owns one (row, column) pair of the output: the lanes stride
// over the row's nonzeros, gather x at the column indices, multiply in the
// compute type and reduce by shuffles within the group; the group's first
// lane converts and stores the result.  Groups walk the pairs column by
// column so that consecutive groups write consecutive rows.  The adjoint is
// a second CSR (the conjugate transpose) built when the plan is created, so
// both directions are row-parallel with no atomics and results are
// deterministic.  Bound by the gathers from x (HBM / L2).

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>

#include "fm_launch.cuh"

namespace fmk {
namespace {

// shuffle of any element type by its 32-bit words
template <class E>
__device__ __forceinline__ E shfl_down_e(unsigned mask, E v, int o, int w) {
  static_assert(sizeof(E) % 4 == 0, "element size");
  constexpr int K = sizeof(E) / 4;
  int a[K];
  memcpy(a, &v, sizeof(E));
#pragma unroll
  for (int i = 0; i < K; ++i) a[i] = __shfl_down_sync(mask, a[i], o, w);
  E r;
  memcpy(&r, a, sizeof(E));
  return r;
}

template <class E, int G>
__global__ void __launch_bounds__(256)
    spmv_kernel(const __grid_constant__ SpStep p) {
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = (int)(threadIdx.x & (G - 1));
  // lanes of one group share w, so they leave the loop together
  const unsigned mask =
      G == 32 ? 0xFFFFFFFFu
              : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  const i64 stride = (i64)gridDim.x * blockDim.x / G;
  const i64 total = p.rows * p.num_cols;
  const E *val = (const E *)p.val;
  for (i64 w = t / G; w < total; w += stride) {
    const i64 m = w / p.rows, r = w - m * p.rows;
    const i64 b = p.ptr[r], e = p.ptr[r + 1];
    const i64 xc = m * p.ld_src;
    E acc = zero<E>();
    for (i64 k = b + lane; k < e; k += G)
      acc = addv(acc, mulv(val[k], load_as<E>(p.src, p.src_type,
                                                xc + p.idx[k]),
                           false));
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
      acc = addv(acc, shfl_down_e(mask, acc, o, G));
    if (lane == 0)
      store_as<E>(p.dst, p.dst_type, m * p.ld_dst + r, acc, false);
  }
}

template <class E>
cudaError_t launch_group(const SpStep &p, int group, cudaStream_t s) {
  const int threads = 256;
  const i64 lanes = p.rows * p.num_cols * (i64)group;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const i64 want = (lanes + threads - 1) / threads;
  const int grid = (int)std::max<i64>(
      1, std::min<i64>(want, (i64)std::max(sms, 1) * 16));
  switch (group) {
    case 1: spmv_kernel<E, 1><<<grid, threads, 0, s>>>(p); break;
    case 2: spmv_kernel<E, 2><<<grid, threads, 0, s>>>(p); break;
    case 4: spmv_kernel<E, 4><<<grid, threads, 0, s>>>(p); break;
    case 8: spmv_kernel<E, 8><<<grid, threads, 0, s>>>(p); break;
    case 16: spmv_kernel<E, 16><<<grid, threads, 0, s>>>(p); break;
    default: spmv_kernel<E, 32><<<grid, threads, 0, s>>>(p); break;
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_spmv(int ctype, const SpStep &p, int group,
                        cudaStream_t s) {
  if (p.rows <= 0 || p.num_cols <= 0) return cudaSuccess;
  switch (ctype) {
    case FM_F32:
    case FM_F32_TC: return launch_group<float>(p, group, s);
    case FM_F64: return launch_group<double>(p, group, s);
    case FM_C64: return launch_group<float2>(p, group, s);
    case FM_C128: return launch_group<double2>(p, group, s);
    case FM_I64: return launch_group<i64>(p, group, s);
    case FM_F64_DF: return launch_group<df>(p, group, s);
    case FM_C128_DF: return launch_group<dfc>(p, group, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace fmk
