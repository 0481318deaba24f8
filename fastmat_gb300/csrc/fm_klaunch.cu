// Shared launch path of the vector-program kernel instantiations.
#include <map>
#include <mutex>
#include <set>
#include <tuple>

#include "fm_klaunch.cuh"

namespace fmk {

cudaError_t launch_kfn(KFn fn, const Step &st, int threads, size_t smem,
                       i64 grid, cudaStream_t s) {
  static std::mutex mu;
  static std::set<KFn> configured;
  static std::map<std::tuple<KFn, int, size_t>, int> resident;
  static int sms = 0;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    cudaError_t e;
    if (!sms) {
      int dev = 0;
      if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
      if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount,
                                      dev)) != cudaSuccess)
        return e;
    }
    if (!configured.count(fn)) {
      if ((e = cudaFuncSetAttribute((const void *)fn,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMaxSmem)) != cudaSuccess)
        return e;
      configured.insert(fn);
    }
    const auto key = std::make_tuple(fn, threads, smem);
    auto it = resident.find(key);
    if (it == resident.end()) {
      int n = 0;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
               &n, (const void *)fn, threads, smem)) != cudaSuccess)
        return e;
      it = resident.emplace(key, n < 1 ? 1 : n).first;
    }
    per_sm = it->second;
  }
  const i64 cap = (i64)per_sm * sms;
  const i64 g = grid < cap ? grid : cap;
  void *args[] = {const_cast<Step *>(&st)};
  return cudaLaunchKernel((const void *)fn, dim3((unsigned)g),
                          dim3(threads), args, smem, s);
}

}  // namespace fmk
