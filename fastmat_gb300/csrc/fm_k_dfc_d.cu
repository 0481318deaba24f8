// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type dfc (see fm_k_dfc.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_dfc_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<dfc, 0, 2>;
    case 1: return vprog_kernel<dfc, 1, 2>;
    case 2: return vprog_kernel<dfc, 2, 2>;
    case 3: return vprog_kernel<dfc, 3, 2>;
    case 5: return vprog_kernel<dfc, 5, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
