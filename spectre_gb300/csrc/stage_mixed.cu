// stage_mixed.cu -- mixed-precision fused DG right-hand side + SSP-RK3 stage
// (uniform LGL extent N, conforming mortars, affine mesh).
//
// The DG operator L of ScalarWave::TimeDerivative + UpwindPenalty + lift is
// linear in (Psi, Pi, Phi) for a static mesh (fixed normals, fixed char
// speeds (0, +1, -1)).  With u1 = u0 + d1 and d1 = dt L(u0), the SSP-RK3
// stages of Rk3HesthavenSsp.cpp:63-80 become
//   d1 = dt L(u0)
//   s2 = u2 - u0 = d1/2 + dt/4 L(d1)
//   u3 = u0 + 2/3 (s2 + d1) + 2dt/3 L(s2)
// so only the first stage differentiates the full FP64 state; the other two
// differentiate small increments whose FP32 rounding is far below the
// step's truncation error.  The first stage is done in FP32 "double-float"
// arithmetic: the state is split exactly into hi + lo FP32 parts (integer bit
// operations, no FP64 instruction), the scaled even/odd D tables are split
// into hi + lo FP32 parts, and every dot product is compensated (TwoProd via
// FMA, TwoSum), so L(u0) is accurate to far better than FP32 before its
// final rounding.  The FP64 state is updated once per step, u0 + (double)inc,
// with one FP64 add per value.
//
// One kernel template serves every stage:
//   W = alpha X + beta Y + c L(X)
// X: fields read with faces (FP64 and compensated when COMP, else FP32),
// Y: optional FP32 pointwise input.  Outputs (each optional):
//   w32[p]   = W                  (FP32 increment buffer)
//   out64[p] = base64[p] + W      (FP64; out64 may alias base64)
//   out64[p] = W                  (when base64 is null: the RHS itself)
#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

template <int N>
struct MShape {
  static constexpr int h = N / 2;
  static constexpr int odd = N % 2;
  static constexpr int H = h + odd;
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = 2 * H * h + H;
};

using dev::eo_line;
using dev::eo_line_df;
using dev::split_df;
using dev::two_sum;
using dev::widen;

// plain FP32 (scaled D) x line with the even/odd split
template <int N>
__device__ __forceinline__ void eo_line_f(const float (&x)[N], float (&out)[N],
                                          const float* __restrict__ th) {
  eo_line<N, float>(x, out, th);
}

template <int N, int EPB, bool COMP>
struct MSmem {
  using S = MShape<N>;
  // per element: fields (COMP: hi and lo of Pi, Phi_x, Phi_y, Phi_z; else the
  // four FP32 fields), the dt Pi accumulator, 3 scaled tables (hi [+ lo])
  static constexpr int kFieldFloats = (COMP ? 8 : 4) * S::NP;
  static constexpr int kTabFloats = (COMP ? 2 : 1) * 3 * S::TAB;
  static constexpr int kSlot = kFieldFloats + S::NP + kTabFloats;
  static constexpr size_t kBytes = (size_t)EPB * kSlot * sizeof(float);
};

template <int N, int EPB, bool COMP>
__global__ void __launch_bounds__(N * N * EPB, COMP ? 1 : 2)
    stage_mixed_kernel(MixedLaunch L) {
  using S = MShape<N>;
  using SM = MSmem<N, EPB, COMP>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB, h = S::h, H = S::H;
  constexpr int64_t VS = (int64_t)kVars * NP;  // values per element
  extern __shared__ float fsm[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  const int64_t e = (int64_t)blockIdx.x * EPB + slot;
  const bool active = e < L.n_elem;
  float* F = fsm + slot * SM::kSlot;
  float* Sacc = F + SM::kFieldFloats;
  float* T = Sacc + NP;  // COMP: [hi tables 3*TAB][lo tables 3*TAB]
  const int64_t off = e * VS;
  const float cf = (float)L.c;

  double jd[3] = {0.0, 0.0, 0.0};
  if (active) {
    jd[0] = L.jac[3 * e];
    jd[1] = L.jac[3 * e + 1];
    jd[2] = L.jac[3 * e + 2];
    if (COMP) {
      const double* src = L.x64 + off + NP;
      for (int q = t; q < 4 * NP; q += NN) {
        float hi, lo;
        split_df(src[q], hi, lo);
        F[q] = hi;
        F[4 * NP + q] = lo;
      }
    } else {
      const float* src = L.x32 + off + NP;
      for (int q = t; q < 4 * NP; q += NN) F[q] = src[q];
    }
    for (int q = t; q < 3 * TAB; q += NN) {
      const int d = q / TAB, r = q - d * TAB;
      double v;
      if (r < H * h)
        v = L.eo.A[r / h][r % h];
      else if (r < 2 * H * h)
        v = L.eo.B[(r - H * h) / h][(r - H * h) % h];
      else
        v = L.eo.M[r - 2 * H * h];
      const double sv = (-L.c * jd[d]) * v;
      const float hi = __double2float_rn(sv);
      T[q] = hi;
      if (COMP) T[3 * TAB + q] = __double2float_rn(sv - (double)hi);
    }
  }
  __syncthreads();

  const int ta = t % N, tb = t / N;
  const float alpha = (float)L.alpha, beta = (float)L.beta;
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    if (active) {
      int base, stride;
      if (d == 0) {
        base = N * ta + NN * tb;
        stride = 1;
      } else if (d == 1) {
        base = ta + NN * tb;
        stride = N;
      } else {
        base = ta + N * tb;
        stride = NN;
      }
      const float* th = T + d * TAB;
      const float* tl = T + 3 * TAB + d * TAB;
      float dF[N], dP[N];
      // fields of this line: Pi (index 0) and Phi_d (index 1 + d)
      float pih[N], pil[N], fh[N], fl[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        pih[i] = F[base + i * stride];
        fh[i] = F[(1 + d) * NP + base + i * stride];
        if (COMP) {
          pil[i] = F[4 * NP + base + i * stride];
          fl[i] = F[4 * NP + (1 + d) * NP + base + i * stride];
        } else {
          pil[i] = 0.0f;
          fl[i] = 0.0f;
        }
      }
      if (COMP) {
        eo_line_df<N>(fh, fl, dF, th, tl);
        eo_line_df<N>(pih, pil, dP, th, tl);
      } else {
        eo_line_f<N>(fh, dF, th);
        eo_line_f<N>(pih, dP, th);
      }
      // UpwindPenalty face corrections at both ends of the line (flat unit
      // normal s e_d, char speeds (0, +1, -1)): D_Pi = (w_int - w_ext)/2,
      // D_Phi_d = -s D_Pi, w = Pi - s Phi_d; lifted and scaled:
      // G = -c N(N-1) J_d / 4.
      const float G = (float)(-0.25 * L.c * (double)(N * (N - 1)) * jd[d]);
      const int64_t nlo = (int64_t)L.nbr[6 * e + 2 * d] * VS;
      const int64_t nhi = (int64_t)L.nbr[6 * e + 2 * d + 1] * VS;
      const int lo_pt = base + (N - 1) * stride;
      const int hi_pt = base;
      float dw_lo, dw_hi;
      if (COMP) {
        // w in double-float; the jump is the small difference of two O(u)
        // numbers, so it is formed before rounding to FP32
        float ph, pl, qh, ql;
        split_df(L.x64[nlo + NP + lo_pt], ph, pl);
        split_df(L.x64[nlo + (2 + d) * NP + lo_pt], qh, ql);
        // s = -1: w = Pi + Phi_d
        float wih, wil, weh, wel, t1;
        two_sum(pih[0], fh[0], wih, t1);
        wil = t1 + (pil[0] + fl[0]);
        two_sum(ph, qh, weh, t1);
        wel = t1 + (pl + ql);
        float dh;
        two_sum(wih, -weh, dh, t1);
        dw_lo = dh + (t1 + (wil - wel));
        split_df(L.x64[nhi + NP + hi_pt], ph, pl);
        split_df(L.x64[nhi + (2 + d) * NP + hi_pt], qh, ql);
        // s = +1: w = Pi - Phi_d
        two_sum(pih[N - 1], -fh[N - 1], wih, t1);
        wil = t1 + (pil[N - 1] - fl[N - 1]);
        two_sum(ph, -qh, weh, t1);
        wel = t1 + (pl - ql);
        two_sum(wih, -weh, dh, t1);
        dw_hi = dh + (t1 + (wil - wel));
      } else {
        const float we_lo = L.x32[nlo + NP + lo_pt] + L.x32[nlo + (2 + d) * NP + lo_pt];
        const float we_hi = L.x32[nhi + NP + hi_pt] - L.x32[nhi + (2 + d) * NP + hi_pt];
        dw_lo = (pih[0] + fh[0]) - we_lo;
        dw_hi = (pih[N - 1] - fh[N - 1]) - we_hi;
      }
      dF[0] = fmaf(G, dw_lo, dF[0]);
      dP[0] = fmaf(G, dw_lo, dP[0]);
      dF[N - 1] = fmaf(G, dw_hi, dF[N - 1]);
      dP[N - 1] = fmaf(-G, dw_hi, dP[N - 1]);

      // Phi_d: W = alpha X + beta Y + c L
      {
        const int64_t vo = off + (2 + d) * NP + base;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float w = dP[i];
          if (!COMP) {
            w = fmaf(alpha, fh[i], w);
            if (L.y32) w = fmaf(beta, L.y32[vo + i * stride], w);
          }
          if (L.w32) L.w32[vo + i * stride] = w;
          if (L.out64) {
            if (L.base64)
              L.out64[vo + i * stride] = L.base64[vo + i * stride] + widen(w);
            else
              L.out64[vo + i * stride] = widen(w);
          }
        }
      }
      if (d < 2) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (d == 0)
            Sacc[base + i * stride] = dF[i];
          else
            Sacc[base + i * stride] += dF[i];
        }
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int p = base + i * stride;
          float wpi = Sacc[p] + dF[i];
          // dt Psi = -Pi (TimeDerivative.cpp:38)
          float wpsi = COMP ? fmaf(-cf, pih[i], -cf * pil[i]) : -cf * pih[i];
          if (!COMP) {
            wpi = fmaf(alpha, pih[i], wpi);
            wpsi = fmaf(alpha, L.x32[off + p], wpsi);
            if (L.y32) {
              wpi = fmaf(beta, L.y32[off + NP + p], wpi);
              wpsi = fmaf(beta, L.y32[off + p], wpsi);
            }
          }
          if (L.w32) {
            L.w32[off + NP + p] = wpi;
            L.w32[off + p] = wpsi;
          }
          if (L.out64) {
            if (L.base64) {
              L.out64[off + NP + p] = L.base64[off + NP + p] + widen(wpi);
              L.out64[off + p] = L.base64[off + p] + widen(wpsi);
            } else {
              L.out64[off + NP + p] = widen(wpi);
              L.out64[off + p] = widen(wpsi);
            }
          }
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

template <int N>
constexpr int mixed_epb() {
  return N <= 4 ? 16 : (N <= 6 ? 8 : (N <= 8 ? 4 : 2));
}

template <int N, bool COMP>
cudaError_t launch_mixed_n(const MixedLaunch& L, cudaStream_t s) {
  constexpr int EPB = mixed_epb<N>();
  using SM = MSmem<N, EPB, COMP>;
  auto k = stage_mixed_kernel<N, EPB, COMP>;
  cudaError_t err =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SM::kBytes);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  const int64_t blocks = (L.n_elem + EPB - 1) / EPB;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, N * N * EPB, SM::kBytes, s>>>(L);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_mixed_comp(const MixedLaunch& L, cudaStream_t s) {
  return L.x64 ? launch_mixed_n<N, true>(L, s) : launch_mixed_n<N, false>(L, s);
}

}  // namespace

cudaError_t launch_stage_mixed(const MixedLaunch& L, cudaStream_t s) {
  if ((L.x64 == nullptr) == (L.x32 == nullptr)) return cudaErrorInvalidValue;
  switch (L.n) {
    case 2: return launch_mixed_comp<2>(L, s);
    case 3: return launch_mixed_comp<3>(L, s);
    case 4: return launch_mixed_comp<4>(L, s);
    case 5: return launch_mixed_comp<5>(L, s);
    case 6: return launch_mixed_comp<6>(L, s);
    case 7: return launch_mixed_comp<7>(L, s);
    case 8: return launch_mixed_comp<8>(L, s);
    case 9: return launch_mixed_comp<9>(L, s);
    case 10: return launch_mixed_comp<10>(L, s);
    case 11: return launch_mixed_comp<11>(L, s);
    case 12: return launch_mixed_comp<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

// out[i] = base[i] + (double)w[i]: the FP64 update of the last incremental
// stage, as its own stream (pairs of values per thread when both arrays
// allow 16- and 8-byte vector access).
__global__ void accumulate_kernel(double* out, const double* base, const float* w, int64_t n) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(base)) & 15u) == 0 &&
                   (reinterpret_cast<uintptr_t>(w) & 7u) == 0;
  if (vec) {
    const int64_t n2 = n / 2;
    for (int64_t i = i0; i < n2; i += stride) {
      const double2 b = reinterpret_cast<const double2*>(base)[i];
      const float2 x = reinterpret_cast<const float2*>(w)[i];
      reinterpret_cast<double2*>(out)[i] = make_double2(b.x + dev::widen(x.x), b.y + dev::widen(x.y));
    }
    if (i0 == 0 && (n & 1)) out[n - 1] = base[n - 1] + dev::widen(w[n - 1]);
  } else {
    for (int64_t i = i0; i < n; i += stride) out[i] = base[i] + dev::widen(w[i]);
  }
}

cudaError_t launch_accumulate(double* out, const double* base, const float* w, int64_t n,
                              cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int64_t want = (n / 2 + 255) / 256;
  const int64_t grid = want < (int64_t)sms * 8 ? (want > 0 ? want : 1) : (int64_t)sms * 8;
  accumulate_kernel<<<(unsigned)grid, 256, 0, s>>>(out, base, w, n);
  return cudaGetLastError();
}

}  // namespace dgsw
