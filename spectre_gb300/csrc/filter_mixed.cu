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
// filter_residual_kernel: R for one element per block: u split into (hi, lo)
// pairs in shared memory, three sweeps of F, then (F u) - u.
// filter_combine_kernel: out = ar R + ad D + b F(X + Y) for one element per
// block (X + Y staged in shared memory, three FP32 sweeps), written as FP32
// and / or added to an FP64 base.
#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

using dev::dot2_first;
using dev::dot2_term;
using dev::split_df;
using dev::two_sum;
using dev::widen;

constexpr int kThreads = 256;

__device__ __forceinline__ void line_of(int N, int a, int line, int* base, int* stride) {
  const int NN = N * N, ta = line % N, tb = line / N;
  if (a == 0) {
    *base = N * ta + NN * tb;
    *stride = 1;
  } else if (a == 1) {
    *base = ta + NN * tb;
    *stride = N;
  } else {
    *base = ta + N * tb;
    *stride = NN;
  }
}

template <int N>
__global__ void __launch_bounds__(kThreads) filter_residual_kernel(MixedFilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N;
  extern __shared__ float2 rbuf[];
  float2* A = rbuf;
  float2* B = rbuf + 5 * NP;
  float* Fh = reinterpret_cast<float*>(B + 5 * NP);
  float* Fl = Fh + NN;
  const int64_t e = L.tasks ? (int64_t)L.tasks[blockIdx.x] : (int64_t)blockIdx.x;
  const int64_t off = L.offset ? L.offset[e] : e * (int64_t)(kVars * NP);
  const double* u = L.u64 + off;
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads) {
    float hi, lo;
    split_df(u[q], hi, lo);
    A[q] = make_float2(hi, lo);
  }
  for (int q = threadIdx.x; q < NN; q += kThreads) {
    Fh[q] = L.Fh[q];
    Fl[q] = L.Fl[q];
  }
  __syncthreads();
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    const float2* src = (a == 1) ? B : A;
    float2* dst = (a == 1) ? A : B;
    for (int task = threadIdx.x; task < 5 * NN; task += kThreads) {
      const int v = task / NN, line = task - v * NN;
      int base, stride;
      line_of(N, a, line, &base, &stride);
      float xh[N], xl[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float2 x = src[v * NP + base + i * stride];
        xh[i] = x.x;
        xl[i] = x.y;
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        float s, c;
        dot2_first(Fh[i * N], Fl[i * N], xh[0], xl[0], s, c);
#pragma unroll
        for (int j = 1; j < N; ++j) dot2_term(Fh[i * N + j], Fl[i * N + j], xh[j], xl[j], s, c);
        float h, l;
        two_sum(s, c, h, l);
        dst[v * NP + base + i * stride] = make_float2(h, l);
      }
    }
    __syncthreads();
  }
  // three sweeps: A -> B -> A -> B; R = (F u) - u, rounded once
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads) {
    float uh, ul, s, t;
    split_df(u[q], uh, ul);
    const float2 f = B[q];
    two_sum(f.x, -uh, s, t);
    L.r32[off + q] = s + (t + (f.y - ul));
  }
}

template <int N>
__global__ void __launch_bounds__(kThreads) filter_combine_kernel(MixedFilterLaunch L) {
  constexpr int NN = N * N, NP = N * N * N;
  extern __shared__ float cbuf[];
  float* A = cbuf;
  float* B = cbuf + 5 * NP;
  float* F = B + 5 * NP;
  const int64_t e = L.tasks ? (int64_t)L.tasks[blockIdx.x] : (int64_t)blockIdx.x;
  const int64_t off = L.offset ? L.offset[e] : e * (int64_t)(kVars * NP);
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads)
    A[q] = L.x32[off + q] + (L.y32 ? L.y32[off + q] : 0.0f);
  for (int q = threadIdx.x; q < NN; q += kThreads) F[q] = L.Fh[q];
  __syncthreads();
#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    const float* src = (a == 1) ? B : A;
    float* dst = (a == 1) ? A : B;
    for (int task = threadIdx.x; task < 5 * NN; task += kThreads) {
      const int v = task / NN, line = task - v * NN;
      int base, stride;
      line_of(N, a, line, &base, &stride);
      float x[N];
#pragma unroll
      for (int i = 0; i < N; ++i) x[i] = src[v * NP + base + i * stride];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        float s = F[i * N] * x[0];
#pragma unroll
        for (int j = 1; j < N; ++j) s = fmaf(F[i * N + j], x[j], s);
        dst[v * NP + base + i * stride] = s;
      }
    }
    __syncthreads();
  }
  const float ar = (float)L.ar, ad = (float)L.ad, b = (float)L.b;
  for (int q = threadIdx.x; q < 5 * NP; q += kThreads) {
    float w = b * B[q];
    if (L.r32) w = fmaf(ar, L.r32[off + q], w);
    if (L.d32) w = fmaf(ad, L.d32[off + q], w);
    if (L.w32) L.w32[off + q] = w;
    if (L.out64) L.out64[off + q] = L.base64[off + q] + widen(w);
  }
}

template <int N>
cudaError_t launch_n(const MixedFilterLaunch& L, bool residual, cudaStream_t s) {
  if (L.n_tasks <= 0) return cudaSuccess;
  constexpr int NP = N * N * N, NN = N * N;
  if (residual) {
    const size_t smem = (size_t)10 * NP * sizeof(float2) + 2 * NN * sizeof(float);
    auto k = filter_residual_kernel<N>;
    cudaError_t err = set_kernel_smem<filter_residual_kernel<N>>((int)smem, false);
    if (err != cudaSuccess) return err;
    k<<<(unsigned)L.n_tasks, kThreads, smem, s>>>(L);
  } else {
    const size_t smem = (size_t)(10 * NP + NN) * sizeof(float);
    auto k = filter_combine_kernel<N>;
    cudaError_t err = set_kernel_smem<filter_combine_kernel<N>>((int)smem, false);
    if (err != cudaSuccess) return err;
    k<<<(unsigned)L.n_tasks, kThreads, smem, s>>>(L);
  }
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
  if (!L.u64 || !L.r32 || !L.Fh || !L.Fl) return cudaErrorInvalidValue;
  return launch_any(L, true, s);
}

cudaError_t launch_filter_combine(const MixedFilterLaunch& L, cudaStream_t s) {
  if (!L.x32 || !L.Fh || (!L.w32 && !L.out64) || (L.out64 && !L.base64)) return cudaErrorInvalidValue;
  return launch_any(L, false, s);
}

}  // namespace dgsw
