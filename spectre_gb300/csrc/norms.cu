// norms.cu -- Events::ObserveNorms of the evolved variables on the device
// (ParallelAlgorithms/Events/ObserveNorms.cpp:33-105, ObserveNorms.hpp:47-80,
// 145-171): for each of Psi, Pi, Phi_x, Phi_y, Phi_z, "Individual":
//   Max, Min, L2Norm = sqrt(sum u^2 / points),
//   L2IntegralNorm = sqrt(int u^2 dV / V), VolumeIntegral = int u dV,
// where the integrals are definite_integral (the LGL weights of every axis)
// times det(Jacobian), and V = int 1 dV.  The reference reduces per element
// and then over elements (Parallel::ReductionData); here one block per element
// writes its partial sums, and one block folds the partials in a fixed order,
// so the result does not depend on scheduling.  FP64 throughout.
#include <cmath>

#include "common.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

constexpr int kThreads = 256;
constexpr int kPart = 26;  // 5 x (max, min, sum u^2, int u^2, int u) + volume

__global__ void __launch_bounds__(kThreads) norms_partial_kernel(NormsLaunch L) {
  __shared__ double red[kThreads];
  const int64_t e = blockIdx.x;
  const int n = L.uniform_n ? L.uniform_n : L.elem_n[e];
  const int np = n * n * n;
  const int64_t off = L.offset ? L.offset[e] : e * (int64_t)(kVars * np);
  const double* w1 = L.lgl_w + n * kMaxN;
  double flat_det = 0.0;
  if (L.width) flat_det = 0.125 * L.width[3 * e] * L.width[3 * e + 1] * L.width[3 * e + 2];
  double acc[kPart];
  for (int v = 0; v < 5; ++v) {
    acc[5 * v + 0] = -INFINITY;
    acc[5 * v + 1] = INFINITY;
    acc[5 * v + 2] = acc[5 * v + 3] = acc[5 * v + 4] = 0.0;
  }
  acc[25] = 0.0;
  for (int p = threadIdx.x; p < np; p += kThreads) {
    const int i = p % n, j = (p / n) % n, k = p / (n * n);
    double dj = flat_det;
    if (!L.width) {
      const double* J = L.ij + e * 9 * (int64_t)np + p;
      double m[9];
      for (int c = 0; c < 9; ++c) m[c] = J[c * np];
      const double det = m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                         m[2] * (m[3] * m[7] - m[4] * m[6]);
      dj = 1.0 / det;
    }
    const double w = w1[i] * w1[j] * w1[k] * dj;
    acc[25] += w;
    for (int v = 0; v < 5; ++v) {
      double x = L.u[off + v * np + p];
      if (L.subtract) x -= L.subtract[off + v * np + p];
      acc[5 * v + 0] = fmax(acc[5 * v + 0], x);
      acc[5 * v + 1] = fmin(acc[5 * v + 1], x);
      acc[5 * v + 2] = fma(x, x, acc[5 * v + 2]);
      acc[5 * v + 3] = fma(w * x, x, acc[5 * v + 3]);
      acc[5 * v + 4] = fma(w, x, acc[5 * v + 4]);
    }
  }
  // fixed-order tree reduction of each quantity over the block
  for (int c = 0; c < kPart; ++c) {
    const int m = c < 25 ? c % 5 : 2;  // 0 max, 1 min, else sum
    red[threadIdx.x] = acc[c];
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        const double a = red[threadIdx.x], b = red[threadIdx.x + s];
        red[threadIdx.x] = m == 0 ? fmax(a, b) : (m == 1 ? fmin(a, b) : a + b);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) L.partial[e * kPart + c] = red[0];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) norms_final_kernel(NormsLaunch L, int64_t n_elem) {
  __shared__ double red[kThreads];
  for (int c = 0; c < kPart; ++c) {
    const int m = c < 25 ? c % 5 : 2;
    double a = m == 0 ? -INFINITY : (m == 1 ? INFINITY : 0.0);
    for (int64_t e = threadIdx.x; e < n_elem; e += kThreads) {
      const double b = L.partial[e * kPart + c];
      a = m == 0 ? fmax(a, b) : (m == 1 ? fmin(a, b) : a + b);
    }
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = kThreads / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        const double x = red[threadIdx.x], y = red[threadIdx.x + s];
        red[threadIdx.x] = m == 0 ? fmax(x, y) : (m == 1 ? fmin(x, y) : x + y);
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) L.result[c] = red[0];
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_norms(const NormsLaunch& L, cudaStream_t s) {
  if (L.n_elem <= 0) return cudaSuccess;
  norms_partial_kernel<<<(unsigned)L.n_elem, kThreads, 0, s>>>(L);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  norms_final_kernel<<<1, kThreads, 0, s>>>(L, L.n_elem);
  return cudaGetLastError();
}

}  // namespace dgsw
