// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type double (see fm_k_f64.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_f64_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<double, 0, 2>;
    case 3: return vprog_kernel<double, 3, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
