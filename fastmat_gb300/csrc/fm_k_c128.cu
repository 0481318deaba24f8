// Instantiations of the vector-program kernel for element type double2.
#include "fm_launch.cuh"

namespace fmk {

template <class K> static cudaError_t cfg(K kernel) {
  return cudaFuncSetAttribute(kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kMaxSmem);
}

cudaError_t launch_c128(const Step &st, int cls, int threads, size_t smem,
                       i64 grid, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e;
    if ((e = cfg(vprog_kernel<double2, 0>)) != cudaSuccess) return e;
    if ((e = cfg(vprog_kernel<double2, 1>)) != cudaSuccess) return e;
    if ((e = cfg(vprog_kernel<double2, 2>)) != cudaSuccess) return e;
    if ((e = cfg(vprog_kernel<double2, 3>)) != cudaSuccess) return e;
    configured = true;
  }
  switch (cls) {
    case 1:
      vprog_kernel<double2, 1><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
    case 2:
      vprog_kernel<double2, 2><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
    case 3:
      vprog_kernel<double2, 3><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
    default:
      vprog_kernel<double2, 0><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
  }
  return cudaGetLastError();
}

}  // namespace fmk
