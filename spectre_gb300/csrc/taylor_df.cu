// taylor_df.cu -- launches of the Taylor-step kernels (taylor_df.cuh) for
// gamma2 = 0, forward and transposed; gamma2 != 0 (forward only) is compiled
// in taylor_df_g2.cu.
#include "taylor_df.cuh"

namespace dgsw {

cudaError_t launch_taylor_df(const TaylorLaunch& L, cudaStream_t s) {
  if (L.gamma2 != 0.0) return launch_taylor_df_g2(L, s);
  return launch_any<false>(L, s);
}

}  // namespace dgsw
