// Dense vector-major (layout 2) instantiations of the vector-program
// kernel for element type df (see fm_k_df.cu).
#include "fm_klaunch.cuh"

namespace fmk {

KFn pick_df_dense(int cls) {
  switch (cls) {
    case 0: return vprog_kernel<df, 0, 2>;
    case 3: return vprog_kernel<df, 3, 2>;
    default: return nullptr;
  }
}

}  // namespace fmk
