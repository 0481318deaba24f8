// Instantiations and launcher of the register-resident convolution kernel
// (fm_rconv.cuh): complex64 and double-float complex128, power-of-two
// lengths up to one warp's registers.
#include <map>
#include <mutex>
#include <utility>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"
#include "fm_rconv.cuh"

namespace fmk {

namespace {

template <class E, int L>
cudaError_t launch_one(const RcStep &p, cudaStream_t s) {
  auto *fn = rconv_kernel<E, L>;
  constexpr size_t smem = rc_smem<E, L>();
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
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn,
                                                        FM_RC_THREADS, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      it = resident.emplace(dev, (per_sm < 1 ? 1 : per_sm) * sms).first;
    }
    cap = it->second;
  }
  constexpr int VPC = (FM_RC_THREADS / 32) * (32 / (L / RcLane<E>::P));
  const long long nv = (long long)p.A * p.num_cols;
  long long grid = (nv + VPC - 1) / VPC;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  fn<<<(unsigned)grid, FM_RC_THREADS, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

int rconv_max_len(int ctype) {
  return ctype == FM_C64 ? 512 : ctype == FM_C128_DF ? 256 : 0;
}
int rconv_min_len(int ctype) {
  return ctype == FM_C64 ? RcLane<float2>::P
         : ctype == FM_C128_DF ? RcLane<dfc>::P
                               : 0;
}
int rconv_lane_points(int ctype) { return rconv_min_len(ctype); }

cudaError_t launch_rconv(int ctype, const RcStep &p, cudaStream_t s) {
  if (ctype == FM_C64) {
    switch (p.L) {
      case 16: return launch_one<float2, 16>(p, s);
      case 32: return launch_one<float2, 32>(p, s);
      case 64: return launch_one<float2, 64>(p, s);
      case 128: return launch_one<float2, 128>(p, s);
      case 256: return launch_one<float2, 256>(p, s);
      case 512: return launch_one<float2, 512>(p, s);
      default: break;
    }
  } else if (ctype == FM_C128_DF) {
    switch (p.L) {
      case 8: return launch_one<dfc, 8>(p, s);
      case 16: return launch_one<dfc, 16>(p, s);
      case 32: return launch_one<dfc, 32>(p, s);
      case 64: return launch_one<dfc, 64>(p, s);
      case 128: return launch_one<dfc, 128>(p, s);
      case 256: return launch_one<dfc, 256>(p, s);
      default: break;
    }
  }
  return cudaErrorInvalidConfiguration;
}

}  // namespace fmk
