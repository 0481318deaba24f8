// Instantiations of the vector-program kernel for element type float:
// padded vector-major (layout 0) and element-major (layout 1) tiles; the
// dense vector-major ones (layout 2) live in fm_k_f32_d.cu so that the two
// halves compile in parallel.
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_f32_dense(int cls);

namespace {
KFn pick_main(int cls, int lay) {
  switch (cls * 3 + lay) {
    case 0: return vprog_kernel<float, 0, 0>;
    case 9: return vprog_kernel<float, 3, 0>;
    case 10: return vprog_kernel<float, 3, 1>;
    case 12: return vprog_kernel<float, 4, 0>;
    case 13: return vprog_kernel<float, 4, 1>;
    case 18: return vprog_kernel<float, 6, 0>;
    case 19: return vprog_kernel<float, 6, 1>;
    default: return nullptr;
  }
}
}  // namespace

cudaError_t launch_f32(const Step &st, int cls, int lay, int threads,
                      size_t smem, i64 grid, cudaStream_t s) {
  const KFn fn = lay == 2 ? pick_f32_dense(cls) : pick_main(cls, lay);
  // no fallback to another layout: the planner only picks instantiated ones
  if (!fn) return cudaErrorInvalidConfiguration;
  return launch_kfn(fn, st, threads, smem, grid, s);
}

}  // namespace fmk
