// filter_mixed.cu -- the exponential filter after every substep
// (dg::Actions::Filter, ParallelAlgorithms/Actions/FilterAction.hpp:109-180,
// matrix Spectral/Filtering.cpp:18-31) on the mixed-precision path.
//
// The mixed path keeps the FP64 state u0 and FP32 increments.  With the
// filter F (linear, applied along each axis) after every substep, SSP-RK3
// (Rk3HesthavenSsp.cpp:63-80) becomes, with R = (F - I) u0,
//   W1 = dt L u0,           D1 = t1 - u0 = R + F W1,
//   W2 = dt L D1,           D2 = t2 - u0 = 3/4 R + 1/4 D1 + 1/4 F(D1 + W2),
//   W3 = dt L D2,           u  = u0 + 1/3 R + 2/3 D1 + 2/3 F(D2 + W3),
// so every filter application acts on FP32 increments except R, which is
// formed from the FP64 state in double-float arithmetic (hi + lo FP32
// values and tables, compensated products and sums) and rounded once.
//
// Both kernels run one block per (element, variable) and one thread per
// line, with F's mirror symmetry (filter_line.cuh); each axis pass reads every
// thread's line into registers, synchronises and writes the result in place.
// filter_residual_kernel: R = (F u) - u, u split into (hi, lo) FP32 pairs,
// three compensated sweeps with the hi + lo split tables, rounded once.
// filter_combine_kernel: out = ar R + ad D + b F(X + Y), X + Y staged, three
// FP32 sweeps, written as FP32 and / or added to an FP64 base.
#include "common.cuh"
#include "dg_device.cuh"
#include "filter_line.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

using dev::split_df;
using dev::two_sum;
using dev::widen;

template <int N>
__global__ void __launch_bounds__(filt::line_threads<N>())
    filter_residual_kernel(MixedFilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N, TS = filt::SymTab<N>::SIZE;
  constexpr int T = filt::line_threads<N>();
  __shared__ float Sh[NP], Sl[NP];
  __shared__ float th[TS], tl[TS];
  const int64_t slot = blockIdx.x / kVars;
  const int v = (int)(blockIdx.x - slot * kVars);
  const int64_t e = L.tasks ? (int64_t)L.tasks[slot] : slot;
  const int64_t off = (L.offset ? L.offset[e] : e * (int64_t)(kVars * NP)) + (int64_t)v * NP;
  const double* u = L.u64 + off;
  const int tid = threadIdx.x;
  for (int q = tid; q < NP; q += T) split_df(u[q], Sh[q], Sl[q]);
  for (int q = tid; q < TS; q += T) {
    const double t = filt::sym_entry<N>(L.F, q);
    const float hi = __double2float_rn(t);
    th[q] = hi;
    tl[q] = __double2float_rn(t - (double)hi);
  }
  __syncthreads();
  const bool has = tid < NN;
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    int base = 0, stride = 0;
    float xh[N], xl[N], yh[N], yl[N];
    if (has) {
      filt::axis_line<N>(a, tid, base, stride);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        xh[i] = Sh[base + i * stride];
        xl[i] = Sl[base + i * stride];
      }
    }
    __syncthreads();  // every line read before any is overwritten
    if (has) {
      filt::sym_line_df<N>(xh, xl, yh, yl, th, tl);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Sh[base + i * stride] = yh[i];
        Sl[base + i * stride] = yl[i];
      }
    }
    __syncthreads();
  }
  // R = (F u) - u, rounded once; with out64 the filtered state u + R itself
  for (int q = tid; q < NP; q += T) {
    float uh, ul, s, t;
    const double uq = u[q];
    split_df(uq, uh, ul);
    two_sum(Sh[q], -uh, s, t);
    const float r = s + (t + (Sl[q] - ul));
    if (L.out64)
      L.out64[off + q] = uq + widen(r);
    else
      L.r32[off + q] = r;
  }
}

template <int N>
__global__ void __launch_bounds__(filt::line_threads<N>())
    filter_combine_kernel(MixedFilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N, TS = filt::SymTab<N>::SIZE;
  constexpr int T = filt::line_threads<N>();
  __shared__ float S[NP];
  __shared__ float tab[TS];
  const int64_t slot = blockIdx.x / kVars;
  const int v = (int)(blockIdx.x - slot * kVars);
  const int64_t e = L.tasks ? (int64_t)L.tasks[slot] : slot;
  const int64_t off = (L.offset ? L.offset[e] : e * (int64_t)(kVars * NP)) + (int64_t)v * NP;
  const int tid = threadIdx.x;
  for (int q = tid; q < NP; q += T) S[q] = L.x32[off + q] + (L.y32 ? L.y32[off + q] : 0.0f);
  for (int q = tid; q < TS; q += T) tab[q] = (float)filt::sym_entry<N>(L.F, q);
  __syncthreads();
  const bool has = tid < NN;
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    int base = 0, stride = 0;
    float x[N], y[N];
    if (has) {
      filt::axis_line<N>(a, tid, base, stride);
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = S[base + i * stride];
    }
    __syncthreads();  // every line read before any is overwritten
    if (has) {
      filt::sym_line<N, float>(x, y, tab);
#pragma unroll
      for (int i = 0; i < N; ++i) S[base + i * stride] = y[i];
    }
    __syncthreads();
  }
  const float ar = (float)L.ar, ad = (float)L.ad, b = (float)L.b;
  for (int q = tid; q < NP; q += T) {
    float w = b * S[q];
    if (L.r32) w = fmaf(ar, L.r32[off + q], w);
    if (L.d32) w = fmaf(ad, L.d32[off + q], w);
    if (L.w32) L.w32[off + q] = w;
    if (L.out64) L.out64[off + q] = L.base64[off + q] + widen(w);
  }
}

template <int N>
cudaError_t launch_n(const MixedFilterLaunch& L, bool residual, cudaStream_t s) {
  if (L.n_tasks <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)(L.n_tasks * kVars);
  if (residual)
    filter_residual_kernel<N><<<blocks, filt::line_threads<N>(), 0, s>>>(L);
  else
    filter_combine_kernel<N><<<blocks, filt::line_threads<N>(), 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_any(const MixedFilterLaunch& L, bool residual, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_n<2>(L, residual, s);
    case 3: return launch_n<3>(L, residual, s);
    case 4: return launch_n<4>(L, residual, s);
    case 5: return launch_n<5>(L, residual, s);
    case 6: return launch_n<6>(L, residual, s);
    case 7: return launch_n<7>(L, residual, s);
    case 8: return launch_n<8>(L, residual, s);
    case 9: return launch_n<9>(L, residual, s);
    case 10: return launch_n<10>(L, residual, s);
    case 11: return launch_n<11>(L, residual, s);
    case 12: return launch_n<12>(L, residual, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_filter_residual(const MixedFilterLaunch& L, cudaStream_t s) {
  if (!L.u64 || (!L.r32 && !L.out64) || !L.F) return cudaErrorInvalidValue;
  return launch_any(L, true, s);
}

cudaError_t launch_filter_combine(const MixedFilterLaunch& L, cudaStream_t s) {
  if (!L.x32 || !L.F || (!L.w32 && !L.out64) || (L.out64 && !L.base64)) return cudaErrorInvalidValue;
  return launch_any(L, false, s);
}

}  // namespace dgsw
