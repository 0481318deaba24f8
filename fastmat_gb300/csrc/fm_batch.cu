// Instantiations and launcher of the batched persistent kernel (many
// operators in one cooperative launch; see batch_kernel).

#include <cuda_runtime.h>

#include "../../include/fmgpu.h"
#include "fm_launch.cuh"

namespace fmk {

namespace {

template <class E, int CLS>
cudaError_t launch_one(const BatchLaunch &b, cudaStream_t s) {
  auto *fn = batch_kernel<E, CLS>;
  cudaError_t e = cudaFuncSetAttribute(
      fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b.smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0, dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn,
                                                    FM_MAX_THREADS, b.smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  // every CTA must be resident at once for the grid barriers
  long long grid = (long long)per_sm * sms;
  if (b.max_level_tiles < grid) grid = b.max_level_tiles;
  if (grid < 1) grid = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(FM_MAX_THREADS);
  cfg.dynamicSmemBytes = b.smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, fn, b.steps, b.start, b.level, b.nlev,
                            b.bar, b.err, b.max_B, b.max_tile, b.wait_limit);
}

}  // namespace

cudaError_t launch_batch(const BatchLaunch &b, cudaStream_t s) {
  switch (b.ctype) {
    case FM_C64:
      switch (b.cls) {
        case 1: return launch_one<float2, 1>(b, s);
        case 2: return launch_one<float2, 2>(b, s);
        default: return launch_one<float2, 0>(b, s);
      }
    case FM_C128_DF: return launch_one<dfc, 0>(b, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace fmk
