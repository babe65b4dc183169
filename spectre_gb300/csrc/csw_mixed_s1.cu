// csw_mixed_s1.cu -- launch shape 1 of the mixed-precision CurvedScalarWave
// stage (csw_mixed.cuh), in its own translation unit so that the shapes
// compile in parallel.
#include "csw_mixed.cuh"

namespace dgsw {
namespace csw_mixed {
cudaError_t launch_shape1(const CswMixedLaunch& L, cudaStream_t s) { return launch_shape<1>(L, s); }
}  // namespace csw_mixed
}  // namespace dgsw
