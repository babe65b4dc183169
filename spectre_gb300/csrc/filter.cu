// filter.cu -- the exponential filter applied to every element's evolved
// variables after a substep: dg::Actions::Filter<Filters::Exponential>
// (ParallelAlgorithms/Actions/FilterAction.hpp:109-180), i.e. apply_matrices
// with the 1D filter matrix F (Spectral/Filtering.cpp:18-31) along each of
// the three logical axes, in place, FP64.
//
// One block per element: the five variables are staged in shared memory,
// then three passes (one per axis) apply F to every line, ping-ponging
// between two shared buffers, and the result is written back.  The filter is
// an element-local N^3 x N^3 tensor-product operator: it reads and writes the
// state once (80 B per point) and costs 3 N FP64 FMAs per value.
#include "common.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

constexpr int kThreads = 256;

template <int N>
__global__ void __launch_bounds__(kThreads) filter_kernel(FilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N;
  extern __shared__ double fbuf[];
  double* A = fbuf;
  double* B = fbuf + 5 * NP;
  double* F = B + 5 * NP;
  const int64_t e = L.tasks ? (int64_t)L.tasks[blockIdx.x] : (int64_t)blockIdx.x;
  const int64_t off = L.offset ? L.offset[e] : e * (int64_t)(kVars * NP);
  double* u = L.u + off;
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads) A[q] = u[q];
  for (int q = threadIdx.x; q < NN; q += kThreads) F[q] = L.F[q];
  __syncthreads();
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    const double* src = (a == 1) ? B : A;
    double* dst = (a == 1) ? A : B;
    for (int task = threadIdx.x; task < 5 * NN; task += kThreads) {
      const int v = task / NN, line = task - v * NN;
      const int ta = line % N, tb = line / N;
      int base, stride;
      if (a == 0) {
        base = N * ta + NN * tb;
        stride = 1;
      } else if (a == 1) {
        base = ta + NN * tb;
        stride = N;
      } else {
        base = ta + N * tb;
        stride = NN;
      }
      double x[N];
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = src[v * NP + base + i * stride];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        double s = F[i * N] * x[0];
#pragma unroll
        for (int j = 1; j < N; ++j) s = fma(F[i * N + j], x[j], s);
        dst[v * NP + base + i * stride] = s;
      }
    }
    __syncthreads();
  }
  // three passes: A -> B -> A -> B
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads) u[q] = B[q];
}

template <int N>
cudaError_t launch_n(const FilterLaunch& L, cudaStream_t s) {
  const size_t smem = (size_t)(10 * N * N * N + N * N) * sizeof(double);
  auto k = filter_kernel<N>;
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  if (L.n_tasks <= 0) return cudaSuccess;
  k<<<(unsigned)L.n_tasks, kThreads, smem, s>>>(L);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_n<2>(L, s);
    case 3: return launch_n<3>(L, s);
    case 4: return launch_n<4>(L, s);
    case 5: return launch_n<5>(L, s);
    case 6: return launch_n<6>(L, s);
    case 7: return launch_n<7>(L, s);
    case 8: return launch_n<8>(L, s);
    case 9: return launch_n<9>(L, s);
    case 10: return launch_n<10>(L, s);
    case 11: return launch_n<11>(L, s);
    case 12: return launch_n<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
