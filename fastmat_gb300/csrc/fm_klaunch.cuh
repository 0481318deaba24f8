// Shared launch path of the vector-program kernel instantiations.
#pragma once

#include "fm_launch.cuh"

namespace fmk {

using KFn = void (*)(Step);

// Launches one instantiation as a persistent grid: the dynamic shared
// memory limit is raised once per kernel, the CTAs a multiprocessor can
// hold are looked up once per (kernel, threads, shared memory) and the grid
// is capped at that many per multiprocessor.
cudaError_t launch_kfn(KFn fn, const Step &st, int threads, size_t smem,
                       i64 grid, cudaStream_t s);

}  // namespace fmk
