// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type double2 (see fm_k_c128.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_c128_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<double2, 0, 2>;
    case 1: return vprog_kernel<double2, 1, 2>;
    case 2: return vprog_kernel<double2, 2, 2>;
    case 3: return vprog_kernel<double2, 3, 2>;
    case 5: return vprog_kernel<double2, 5, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
