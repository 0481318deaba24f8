// Instantiations and launcher of the register FFT of strided vectors
// (fm_rsfft.cuh): complex64 vectors of 32..512 points, double-float complex
// of 16..256, both transform signs.
#include <map>
#include <mutex>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"
#include "fm_rsfft.cuh"

namespace fmk {

namespace {

template <class E, int L, int SG>
cudaError_t launch_one(const RsfStep &p, cudaStream_t s) {
  auto *fn = rsfft_kernel<E, L, SG>;
  constexpr size_t smem = rsf_smem<E, L>();
  constexpr int T = RsfShape<E, L>::T, NV = RsfShape<E, L>::NV;
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
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, T, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      it = resident.emplace(dev, (per_sm < 1 ? 1 : per_sm) * sms).first;
    }
    cap = it->second;
  }
  const long long nb = (long long)p.A * p.num_cols / NV;
  long long grid = nb;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  fn<<<(unsigned)grid, T, smem, s>>>(p);
  return cudaGetLastError();
}

template <class E, int L>
cudaError_t launch_signed(const RsfStep &p, cudaStream_t s) {
  return p.sign < 0 ? launch_one<E, L, -1>(p, s) : launch_one<E, L, +1>(p, s);
}

}  // namespace

int rsfft_min_len(int ctype) {
  return ctype == FM_C64 ? 32 : ctype == FM_C128_DF ? 16 : 0;
}
int rsfft_max_len(int ctype) {
  return ctype == FM_C64 ? 512 : ctype == FM_C128_DF ? 256 : 0;
}

cudaError_t launch_rsfft(int ctype, const RsfStep &p, cudaStream_t s) {
  if (ctype == FM_C64) {
    switch (p.L) {
      case 32: return launch_signed<float2, 32>(p, s);
      case 64: return launch_signed<float2, 64>(p, s);
      case 128: return launch_signed<float2, 128>(p, s);
      case 256: return launch_signed<float2, 256>(p, s);
      case 512: return launch_signed<float2, 512>(p, s);
      default: break;
    }
  } else if (ctype == FM_C128_DF) {
    switch (p.L) {
      case 16: return launch_signed<dfc, 16>(p, s);
      case 32: return launch_signed<dfc, 32>(p, s);
      case 64: return launch_signed<dfc, 64>(p, s);
      case 128: return launch_signed<dfc, 128>(p, s);
      case 256: return launch_signed<dfc, 256>(p, s);
      default: break;
    }
  }
  return cudaErrorInvalidConfiguration;
}

}  // namespace fmk
