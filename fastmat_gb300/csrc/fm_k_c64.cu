// Instantiations of the vector-program kernel for element type float2.
#include <map>
#include <mutex>
#include <tuple>

#include "fm_launch.cuh"

namespace fmk {

template <class K> static cudaError_t cfg(K kernel) {
  return cudaFuncSetAttribute(kernel,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kMaxSmem);
}

template <class K>
static cudaError_t occ(K kernel, int threads, size_t smem, int *n) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, kernel, threads,
                                                       smem);
}

// cls: op subset, lay: tile layout (instantiated pairs only; others run the
// general vector-major kernel)
cudaError_t launch_c64(const Step &st, int cls, int lay, int threads,
                       size_t smem, i64 grid, cudaStream_t s) {
  static std::mutex mu;
  static bool configured = false;
  static int sms = 0;
  static std::map<std::tuple<int, int, size_t>, int> resident;
  const int key2 = cls * 2 + lay;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    cudaError_t e;
    if (!configured) {
      if ((e = cfg(vprog_kernel<float2, 0, 0>)) != cudaSuccess) return e;
      if ((e = cfg(vprog_kernel<float2, 1, 0>)) != cudaSuccess) return e;
      if ((e = cfg(vprog_kernel<float2, 2, 0>)) != cudaSuccess) return e;
      if ((e = cfg(vprog_kernel<float2, 3, 0>)) != cudaSuccess) return e;
      if ((e = cfg(vprog_kernel<float2, 1, 1>)) != cudaSuccess) return e;
      if ((e = cfg(vprog_kernel<float2, 3, 1>)) != cudaSuccess) return e;
      int dev = 0;
      if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
      if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                                      dev)) != cudaSuccess)
        return e;
      configured = true;
    }
    const auto key = std::make_tuple(key2, threads, smem);
    auto it = resident.find(key);
    if (it == resident.end()) {
      int n = 0;
      switch (key2) {
        case 2: e = occ(vprog_kernel<float2, 1, 0>, threads, smem, &n); break;
        case 4: e = occ(vprog_kernel<float2, 2, 0>, threads, smem, &n); break;
        case 6: e = occ(vprog_kernel<float2, 3, 0>, threads, smem, &n); break;
        case 3: e = occ(vprog_kernel<float2, 1, 1>, threads, smem, &n); break;
        case 7: e = occ(vprog_kernel<float2, 3, 1>, threads, smem, &n); break;
        default: e = occ(vprog_kernel<float2, 0, 0>, threads, smem, &n); break;
      }
      if (e != cudaSuccess) return e;
      it = resident.emplace(key, n < 1 ? 1 : n).first;
    }
    per_sm = it->second;
  }
  // persistent CTAs: at most as many as fit on the device at once
  const i64 cap = (i64)per_sm * sms;
  const i64 g = grid < cap ? grid : cap;
  switch (key2) {
    case 2:
      vprog_kernel<float2, 1, 0><<<(unsigned)g, threads, smem, s>>>(st);
      break;
    case 4:
      vprog_kernel<float2, 2, 0><<<(unsigned)g, threads, smem, s>>>(st);
      break;
    case 6:
      vprog_kernel<float2, 3, 0><<<(unsigned)g, threads, smem, s>>>(st);
      break;
    case 3:
      vprog_kernel<float2, 1, 1><<<(unsigned)g, threads, smem, s>>>(st);
      break;
    case 7:
      vprog_kernel<float2, 3, 1><<<(unsigned)g, threads, smem, s>>>(st);
      break;
    default:
      vprog_kernel<float2, 0, 0><<<(unsigned)g, threads, smem, s>>>(st);
      break;
  }
  return cudaGetLastError();
}

}  // namespace fmk

#if FM_PHASE_TIMING
extern "C" int fm_debug_phase_cycles(unsigned long long *out, int reset) {
  if (cudaMemcpyFromSymbol(out, fmk::g_phase_cycles, 8 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  if (reset) {
    unsigned long long z[8] = {0};
    cudaMemcpyToSymbol(fmk::g_phase_cycles, z, sizeof(z));
  }
  return 0;
}
#endif
