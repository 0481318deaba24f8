// Instantiations of the vector-program kernel for element type float.
#include "fm_launch.cuh"

namespace fmk {

template <class K> static cudaError_t cfg(K kernel) {
  return cudaFuncSetAttribute(kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kMaxSmem);
}

cudaError_t launch_f32(const Step &st, int cls, int threads, size_t smem,
                       i64 grid, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e;
    if ((e = cfg(vprog_kernel<float, 0>)) != cudaSuccess) return e;
    if ((e = cfg(vprog_kernel<float, 3>)) != cudaSuccess) return e;
    configured = true;
  }
  switch (cls) {
    case 3:
      vprog_kernel<float, 3><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
    default:
      vprog_kernel<float, 0><<<(unsigned)grid, threads, smem, s>>>(st);
      break;
  }
  return cudaGetLastError();
}

}  // namespace fmk
