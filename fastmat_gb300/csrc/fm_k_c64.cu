// Instantiations of the vector-program kernel for element type float2:
// padded vector-major (layout 0) and element-major (layout 1) tiles; the
// dense vector-major ones (layout 2) live in fm_k_c64_d.cu so that the two
// halves compile in parallel.
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_c64_dense(int cls);

namespace {
KFn pick_main(int cls, int lay) {
  switch (cls * 3 + lay) {
    case 0: return vprog_kernel<float2, 0, 0>;
    case 3: return vprog_kernel<float2, 1, 0>;
    case 6: return vprog_kernel<float2, 2, 0>;
    case 9: return vprog_kernel<float2, 3, 0>;
    case 4: return vprog_kernel<float2, 1, 1>;
    case 10: return vprog_kernel<float2, 3, 1>;
    case 15: return vprog_kernel<float2, 5, 0>;
    case 16: return vprog_kernel<float2, 5, 1>;
    default: return nullptr;
  }
}
}  // namespace

cudaError_t launch_c64(const Step &st, int cls, int lay, int threads,
                      size_t smem, i64 grid, cudaStream_t s) {
  const KFn fn = lay == 2 ? pick_c64_dense(cls) : pick_main(cls, lay);
  // no fallback to another layout: the planner only picks instantiated ones
  if (!fn) return cudaErrorInvalidConfiguration;
  return launch_kfn(fn, st, threads, smem, grid, s);
}

}  // namespace fmk
