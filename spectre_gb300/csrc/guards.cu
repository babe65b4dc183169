// guards.cu -- the state check behind DGSW_ERR_NOT_FINITE: the first element
// whose block holds a NaN or an Inf.  One block per element, the element's
// values read once (an HBM-bound pass over the state).
#include "common.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

__global__ void finite_check_kernel(const double* __restrict__ u, const int64_t* __restrict__ offset,
                                    int64_t n_elem, unsigned long long* first) {
  const int64_t e = blockIdx.x;
  if (e >= n_elem) return;
  const int64_t a = offset[e], b = offset[e + 1];
  bool bad = false;
  for (int64_t i = a + threadIdx.x; i < b; i += blockDim.x) bad |= !isfinite(u[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicMin(first, (unsigned long long)e);
}

}  // namespace

cudaError_t launch_finite_check(const double* u, const int64_t* offset, int64_t n_elem,
                                unsigned long long* first, cudaStream_t s) {
  if (n_elem <= 0) return cudaSuccess;
  finite_check_kernel<<<(unsigned)n_elem, 128, 0, s>>>(u, offset, n_elem, first);
  return cudaGetLastError();
}

}  // namespace dgsw
