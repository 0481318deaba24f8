// Instantiations and launchers of the register-resident FWHT kernels
// (fm_rfwht.cuh): float32 and double-float real data, contiguous vectors of
// 1024..8192 (float32) or 256..8192 (double-float) points, strided vectors
// of 64..2048 (float32) or 32..1024 (double-float) points.
#include <map>
#include <mutex>
#include <tuple>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"
#include "fm_rfwht.cuh"

namespace fmk {

namespace {

template <class E, int L>
cudaError_t launch_one(const RfStep &p, cudaStream_t s) {
  auto *fn = rfwht_kernel<E, L>;
  constexpr size_t smem = rf_smem<E, L>();
  constexpr int T = RfShape<E, L>::T, VPC = RfShape<E, L>::VPC;
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
  const long long nv = (long long)p.A * p.num_cols;
  long long grid = (nv + VPC - 1) / VPC;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  fn<<<(unsigned)grid, T, smem, s>>>(p);
  return cudaGetLastError();
}

template <class E, int L>
cudaError_t launch_strided(const RfStep &p, cudaStream_t s) {
  auto *fn = rsfwht_kernel<E, L>;
  constexpr size_t smem = rs_smem<E, L>();
  constexpr int T = RsShape<E, L>::T;
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
  const long long nb = (long long)p.A * p.num_cols / RsShape<E, L>::NV;
  long long grid = nb;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  fn<<<(unsigned)grid, T, smem, s>>>(p);
  return cudaGetLastError();
}

template <class E, int L1, int L2>
cudaError_t launch_pair(const RfPair &p, cudaStream_t s) {
  auto *fn = rfwht2_kernel<E, L1, L2>;
  constexpr size_t smem = rf2_smem<E, L1, L2>();
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
          &per_sm, fn, FM_RF2_THREADS, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      it = resident.emplace(dev, per_sm * sms).first;
    }
    cap = it->second;
  }
  if (cap < 1) return cudaErrorInvalidConfiguration;
  // every CTA resident at once (cooperative): the waits of the second pass
  // rely on it
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cap);
  cfg.blockDim = dim3(FM_RF2_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, p);
}

}  // namespace

bool rfwht2_supported(int ctype, int L1, int L2) {
  if (ctype == FM_F32)
    return L1 == 8192 && (L2 == 64 || L2 == 128 || L2 == 256 || L2 == 512);
  if (ctype == FM_F64_DF)
    return L1 == 4096 && L2 >= 32 && L2 <= 1024 && (L2 & (L2 - 1)) == 0;
  return false;
}

cudaError_t launch_rfwht2(int ctype, const RfPair &p, cudaStream_t s) {
  if (ctype == FM_F32 && p.a.L == 8192) {
    switch (p.b.L) {
      case 64: return launch_pair<float, 8192, 64>(p, s);
      case 128: return launch_pair<float, 8192, 128>(p, s);
      case 256: return launch_pair<float, 8192, 256>(p, s);
      case 512: return launch_pair<float, 8192, 512>(p, s);
      default: break;
    }
  } else if (ctype == FM_F64_DF && p.a.L == 4096) {
    switch (p.b.L) {
      case 32: return launch_pair<df, 4096, 32>(p, s);
      case 64: return launch_pair<df, 4096, 64>(p, s);
      case 128: return launch_pair<df, 4096, 128>(p, s);
      case 256: return launch_pair<df, 4096, 256>(p, s);
      case 512: return launch_pair<df, 4096, 512>(p, s);
      case 1024: return launch_pair<df, 4096, 1024>(p, s);
      default: break;
    }
  }
  return cudaErrorInvalidConfiguration;
}

int rsfwht_min_len(int ctype) {
  return ctype == FM_F32 ? 64 : ctype == FM_F64_DF ? 32 : 0;
}
int rsfwht_max_len(int ctype) {
  return ctype == FM_F32 ? 2048 : ctype == FM_F64_DF ? 1024 : 0;
}

int rfwht_min_len(int ctype) {
  return ctype == FM_F32 ? 1024 : ctype == FM_F64_DF ? 256 : 0;
}
int rfwht_max_len(int ctype) {
  return ctype == FM_F32 || ctype == FM_F64_DF ? 8192 : 0;
}

cudaError_t launch_rfwht(int ctype, const RfStep &p, cudaStream_t s) {
  if (p.es > 1) {
    if (ctype == FM_F32) {
      switch (p.L) {
        case 64: return launch_strided<float, 64>(p, s);
        case 128: return launch_strided<float, 128>(p, s);
        case 256: return launch_strided<float, 256>(p, s);
        case 512: return launch_strided<float, 512>(p, s);
        case 1024: return launch_strided<float, 1024>(p, s);
        case 2048: return launch_strided<float, 2048>(p, s);
        default: break;
      }
    } else if (ctype == FM_F64_DF) {
      switch (p.L) {
        case 32: return launch_strided<df, 32>(p, s);
        case 64: return launch_strided<df, 64>(p, s);
        case 128: return launch_strided<df, 128>(p, s);
        case 256: return launch_strided<df, 256>(p, s);
        case 512: return launch_strided<df, 512>(p, s);
        case 1024: return launch_strided<df, 1024>(p, s);
        default: break;
      }
    }
    return cudaErrorInvalidConfiguration;
  }
  if (ctype == FM_F32) {
    switch (p.L) {
      case 1024: return launch_one<float, 1024>(p, s);
      case 2048: return launch_one<float, 2048>(p, s);
      case 4096: return launch_one<float, 4096>(p, s);
      case 8192: return launch_one<float, 8192>(p, s);
      default: break;
    }
  } else if (ctype == FM_F64_DF) {
    switch (p.L) {
      case 256: return launch_one<df, 256>(p, s);
      case 512: return launch_one<df, 512>(p, s);
      case 1024: return launch_one<df, 1024>(p, s);
      case 2048: return launch_one<df, 2048>(p, s);
      case 4096: return launch_one<df, 4096>(p, s);
      case 8192: return launch_one<df, 8192>(p, s);
      default: break;
    }
  }
  return cudaErrorInvalidConfiguration;
}

}  // namespace fmk
