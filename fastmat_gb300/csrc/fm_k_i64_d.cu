// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type i64 (see fm_k_i64.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_i64_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<i64, 0, 2>;
    case 3: return vprog_kernel<i64, 3, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
