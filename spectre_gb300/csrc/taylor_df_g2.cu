// taylor_df_g2.cu -- launches of the Taylor-step kernels (taylor_df.cuh) for
// gamma2 != 0: the forward step only (the transposed operator is built for
// gamma2 = 0).  A translation unit of its own, so that the kernels compile
// in parallel with those of taylor_df.cu.
#include "taylor_df.cuh"

namespace dgsw {

cudaError_t launch_taylor_df_g2(const TaylorLaunch& L, cudaStream_t s) {
  return launch_any<true>(L, s);
}

}  // namespace dgsw
