// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type float (see fm_k_f32.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_f32_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<float, 0, 2>;
    case 3: return vprog_kernel<float, 3, 2>;
    case 4: return vprog_kernel<float, 4, 2>;
    case 6: return vprog_kernel<float, 6, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
