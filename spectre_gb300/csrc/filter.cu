// filter.cu -- the exponential filter applied to every element's evolved
// variables after a substep: dg::Actions::Filter<Filters::Exponential>
// (ParallelAlgorithms/Actions/FilterAction.hpp:109-180), i.e. apply_matrices
// with the 1D filter matrix F (Spectral/Filtering.cpp:18-31) along each of
// the three logical axes, in place, FP64.
//
// One block per (element, variable), one thread per line: the variable's
// N^3 block is staged in shared memory, then three passes (one per axis)
// each read every thread's line into registers, synchronise, and write F
// times the line back in place; the result is written back to the state.
// F's mirror symmetry halves the multiply-adds (filter_line.cuh): the filter
// reads and writes the state once (80 B per point) and costs about 3 N / 2
// FP64 FMAs per value, which bind it on GB300.
#include "common.cuh"
#include "filter_line.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

template <int N>
__global__ void __launch_bounds__(filt::line_threads<N>()) filter_kernel(FilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N, TS = filt::SymTab<N>::SIZE;
  constexpr int T = filt::line_threads<N>();
  __shared__ double S[NP];
  __shared__ double tab[TS];
  const int64_t slot = blockIdx.x / kVars;
  const int v = (int)(blockIdx.x - slot * kVars);
  const int64_t e = L.tasks ? (int64_t)L.tasks[slot] : slot;
  const int64_t off = (L.offset ? L.offset[e] : e * (int64_t)(kVars * NP)) + (int64_t)v * NP;
  double* u = L.u + off;
  const int tid = threadIdx.x;
  for (int q = tid; q < NP; q += T) S[q] = u[q];
  for (int q = tid; q < TS; q += T) tab[q] = filt::sym_entry<N>(L.F, q);
  __syncthreads();
  const bool has = tid < NN;
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    int base = 0, stride = 0;
    double x[N], y[N];
    if (has) {
      filt::axis_line<N>(a, tid, base, stride);
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = S[base + i * stride];
    }
    __syncthreads();  // every line read before any is overwritten
    if (has) {
      filt::sym_line<N, double>(x, y, tab);
#pragma unroll
      for (int i = 0; i < N; ++i) S[base + i * stride] = y[i];
    }
    __syncthreads();
  }
  for (int q = tid; q < NP; q += T) u[q] = S[q];
}

template <int N>
cudaError_t launch_n(const FilterLaunch& L, cudaStream_t s) {
  if (L.n_tasks <= 0) return cudaSuccess;
  filter_kernel<N><<<(unsigned)(L.n_tasks * kVars), filt::line_threads<N>(), 0, s>>>(L);
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
