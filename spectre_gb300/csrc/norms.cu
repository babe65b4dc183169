// norms.cu -- Events::ObserveNorms of the evolved variables on the device
// (ParallelAlgorithms/Events/ObserveNorms.cpp:33-105, ObserveNorms.hpp:47-80,
// 145-171): for each of Psi, Pi, Phi_x, Phi_y, Phi_z, "Individual":
//   Max, Min, L2Norm = sqrt(sum u^2 / points),
//   L2IntegralNorm = sqrt(int u^2 dV / V), VolumeIntegral = int u dV,
// where the integrals are definite_integral (the LGL weights of every axis)
// times det(Jacobian), and V = int 1 dV.  The reference reduces per element
// and then over elements (Parallel::ReductionData).  Here one warp per element
// forms its 26 partial quantities (butterfly shuffles), kNormsBlocks blocks
// each fold a fixed contiguous range of elements, and one block folds those:
// every reduction has a fixed order, so the result does not depend on
// scheduling.  FP64 throughout.
#include <cmath>

#include "common.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kPart = 26;  // 5 x (max, min, sum u^2, int u^2, int u) + volume

// 0: max, 1: min, 2: sum -- the fold of quantity c
__device__ __forceinline__ int fold_kind(int c) { return c < 25 ? (c % 5 < 2 ? c % 5 : 2) : 2; }
__device__ __forceinline__ double fold(int m, double a, double b) {
  return m == 0 ? fmax(a, b) : (m == 1 ? fmin(a, b) : a + b);
}
__device__ __forceinline__ double fold_identity(int m) {
  return m == 0 ? -INFINITY : (m == 1 ? INFINITY : 0.0);
}
// butterfly over the warp: every lane ends with the same value, combined in
// a fixed order
__device__ __forceinline__ double warp_fold(int m, double a) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) a = fold(m, a, __shfl_xor_sync(0xffffffffu, a, off));
  return a;
}
// the block's fold of one value per thread (fixed order: within the warps,
// then the warps' results in warp order); every thread gets the result
__device__ __forceinline__ double block_fold(int m, double a, double* red) {
  a = warp_fold(m, a);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) red[warp] = a;
  __syncthreads();
  double r = fold_identity(m);
  for (int w = 0; w < kWarps; ++w) r = fold(m, r, red[w]);
  __syncthreads();
  return r;
}

// one warp per element: partial[c * n_elem + e]
__global__ void __launch_bounds__(kThreads) norms_partial_kernel(NormsLaunch L) {
  const int lane = threadIdx.x % 32;
  const int64_t e = (int64_t)blockIdx.x * kWarps + threadIdx.x / 32;
  if (e >= L.n_elem) return;  // whole warps leave; no block barrier follows
  const int n = L.uniform_n ? L.uniform_n : L.elem_n[e];
  const int np = n * n * n;
  const int64_t off = L.offset ? L.offset[e] : e * (int64_t)(kVars * np);
  const double* w1 = L.lgl_w + n * kMaxN;
  double flat_det = 0.0;
  if (L.width) flat_det = 0.125 * L.width[3 * e] * L.width[3 * e + 1] * L.width[3 * e + 2];
  double acc[kPart];
#pragma unroll
  for (int c = 0; c < kPart; ++c) acc[c] = fold_identity(fold_kind(c));
  for (int p = lane; p < np; p += 32) {
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
#pragma unroll
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
#pragma unroll
  for (int c = 0; c < kPart; ++c) {
    const double r = warp_fold(fold_kind(c), acc[c]);
    if (lane == 0) L.partial[c * L.n_elem + e] = r;
  }
}

// block b folds elements [b * chunk, (b + 1) * chunk) of every quantity into
// stage[c * kNormsBlocks + b]
__global__ void __launch_bounds__(kThreads) norms_range_kernel(NormsLaunch L, double* stage) {
  __shared__ double red[kWarps];
  const int64_t chunk = (L.n_elem + kNormsBlocks - 1) / kNormsBlocks;
  const int64_t lo = (int64_t)blockIdx.x * chunk;
  const int64_t hi = lo + chunk < L.n_elem ? lo + chunk : L.n_elem;
  for (int c = 0; c < kPart; ++c) {
    const int m = fold_kind(c);
    double a = fold_identity(m);
    for (int64_t e = lo + threadIdx.x; e < hi; e += kThreads)
      a = fold(m, a, L.partial[c * L.n_elem + e]);
    a = block_fold(m, a, red);
    if (threadIdx.x == 0) stage[c * kNormsBlocks + blockIdx.x] = a;
  }
}

__global__ void __launch_bounds__(kThreads) norms_final_kernel(NormsLaunch L, const double* stage) {
  __shared__ double red[kWarps];
  for (int c = 0; c < kPart; ++c) {
    const int m = fold_kind(c);
    double a = fold_identity(m);
    for (int b = threadIdx.x; b < kNormsBlocks; b += kThreads) a = fold(m, a, stage[c * kNormsBlocks + b]);
    a = block_fold(m, a, red);
    if (threadIdx.x == 0) L.result[c] = a;
  }
}

}  // namespace

cudaError_t launch_norms(const NormsLaunch& L, cudaStream_t s) {
  if (L.n_elem <= 0) return cudaSuccess;
  const int64_t blocks = (L.n_elem + kWarps - 1) / kWarps;
  norms_partial_kernel<<<(unsigned)blocks, kThreads, 0, s>>>(L);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double* stage = L.partial + (size_t)kPart * L.n_elem;
  norms_range_kernel<<<kNormsBlocks, kThreads, 0, s>>>(L, stage);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  norms_final_kernel<<<1, kThreads, 0, s>>>(L, stage);
  return cudaGetLastError();
}

}  // namespace dgsw
