// csw_mixed.cu -- launch shape 0 of the mixed-precision CurvedScalarWave
// stage (csw_mixed.cuh) and the entry point that picks the shape.
#include "csw_mixed.cuh"

namespace dgsw {
namespace csw_mixed {
cudaError_t launch_shape0(const CswMixedLaunch& L, cudaStream_t s) { return launch_shape<0>(L, s); }
}  // namespace csw_mixed

int csw_mixed_shapes() { return csw_mixed::kShapes; }

cudaError_t launch_csw_mixed(const CswMixedLaunch& L, cudaStream_t s) {
  if ((L.x64 == nullptr) == (L.x32 == nullptr)) return cudaErrorInvalidValue;
  switch (L.variant) {
    case 0: return csw_mixed::launch_shape0(L, s);
    case 1: return csw_mixed::launch_shape1(L, s);
    case 2: return csw_mixed::launch_shape2(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
