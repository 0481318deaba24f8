// Instantiations and launcher of the fused circulant + Hadamard Kron modes
// (fm_rpair.cuh): complex64, a circulant mode of 128 or 256 points followed
// by a Hadamard mode of 128 or 256 points.
#include <map>
#include <mutex>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"
#include "fm_rpair.cuh"

namespace fmk {

namespace {

template <class E, int L1, int L2>
cudaError_t launch_one(const RchPair &p, cudaStream_t s) {
  auto *fn = rkch_kernel<E, L1, L2>;
  constexpr size_t smem = RchShape<E, L1, L2>::bytes;
  static std::mutex mu;
  static std::map<int, int> resident;  // device -> CTAs per SM x SMs
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int cap = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = resident.find(dev);
    if (it == resident.end()) {
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, sms = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &per_sm, fn, FM_RCH_THREADS, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      it = resident.emplace(dev, per_sm * sms).first;
    }
    cap = it->second;
  }
  if (cap < 1) return cudaErrorInvalidConfiguration;
  RchPair q = p;
  q.lag = 2 * cap / (p.n1 + p.n2) + 1;
  // every CTA resident at once (cooperative): the waits rely on it
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cap);
  cfg.blockDim = dim3(FM_RCH_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, q);
}

template <class E, int L1, int L2>
bool fits(i64 block_rows, i64 real_per_block) {
  typedef RchShape<E, L1, L2> Sh;
  return block_rows % L1 == 0 && (block_rows / L1) % Sh::VPC == 0 &&
         real_per_block % Sh::NV2 == 0;
}

}  // namespace

// the items of a block: convolution vectors (complex rows / L1) and real
// FWHT vectors (real_per_block) in whole items
bool rkch_supported(int ctype, int L1, int L2, i64 block_rows,
                    i64 real_per_block, int *n1, int *n2) {
  auto set = [&](int vpc, int nv2) {
    *n1 = (int)(block_rows / L1 / vpc);
    *n2 = (int)(real_per_block / nv2);
    return true;
  };
  if ((L1 != 128 && L1 != 256) || (L2 != 128 && L2 != 256)) return false;
#define FM_RCH_CASE(E, A, B)                                              \
  if (L1 == A && L2 == B)                                                 \
    return fits<E, A, B>(block_rows, real_per_block) &&                   \
           set(RchShape<E, A, B>::VPC, RchShape<E, A, B>::NV2);
  if (ctype == FM_C64) {
    FM_RCH_CASE(float2, 128, 128)
    FM_RCH_CASE(float2, 128, 256)
    FM_RCH_CASE(float2, 256, 128)
    FM_RCH_CASE(float2, 256, 256)
  }
#undef FM_RCH_CASE
  return false;
}

cudaError_t launch_rkch(int ctype, const RchPair &p, cudaStream_t s) {
  const int L1 = p.c.L, L2 = p.h.L;
#define FM_RCH_LAUNCH(E, A, B) \
  if (L1 == A && L2 == B) return launch_one<E, A, B>(p, s);
  if (ctype == FM_C64) {
    FM_RCH_LAUNCH(float2, 128, 128)
    FM_RCH_LAUNCH(float2, 128, 256)
    FM_RCH_LAUNCH(float2, 256, 128)
    FM_RCH_LAUNCH(float2, 256, 256)
  }
#undef FM_RCH_LAUNCH
  return cudaErrorInvalidConfiguration;
}

}  // namespace fmk
