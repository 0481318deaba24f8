// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type float2 (see fm_k_c64.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_c64_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<float2, 0, 2>;
    case 1: return vprog_kernel<float2, 1, 2>;
    case 2: return vprog_kernel<float2, 2, 2>;
    case 3: return vprog_kernel<float2, 3, 2>;
    case 5: return vprog_kernel<float2, 5, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
