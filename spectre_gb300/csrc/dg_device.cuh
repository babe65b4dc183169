// dg_device.cuh -- device helpers shared by the DG stage kernels: the even/odd
// line operators of the split differentiation matrix (FP64, FP32, FP32
// double-float), exact FP64 <-> FP32 conversions by integer operations, and
// error-free FP32 transformations.
#pragma once

#include <cstdint>
#include <type_traits>

#include "common.cuh"

namespace dgsw {
namespace dev {

template <int N>
struct Eo {
  static constexpr int h = N / 2;
  static constexpr int odd = N % 2;
  static constexpr int H = h + odd;          // rows formed by the split
  static constexpr int TAB = 2 * H * h + H;  // entries of one table (A, B, M)
};

// (scaled D) u along one line with the even/odd split, FP64.  tab holds the
// scaled A (H x h), B (H x h) and M (H) tables of an EoTable.
// kReload reads every table entry from shared memory where it is used
// (volatile loads), instead of letting the compiler keep the table in
// registers across calls: fewer registers per thread for a few more shared
// loads, which the FP64 pipe's rate hides.
template <int N, typename T, bool kReload = false>
__device__ __forceinline__ void eo_line(const T (&u)[N], T (&out)[N], const T* __restrict__ tab) {
  constexpr int h = Eo<N>::h, H = Eo<N>::H, odd = Eo<N>::odd;
  using Tab = typename std::conditional<kReload, const volatile T*, const T*>::type;
  const Tab A = tab;
  const Tab B = tab + H * h;
  const Tab M = tab + 2 * H * h;
  T e[h], o[h];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    e[j] = u[j] + u[N - 1 - j];
    o[j] = u[j] - u[N - 1 - j];
  }
#pragma unroll
  for (int i = 0; i < h; ++i) {
    T P = A[i * h] * e[0];
#pragma unroll
    for (int j = 1; j < h; ++j) P = fma(A[i * h + j], e[j], P);
    if (odd) P = fma(M[i], u[h], P);
    T Q = B[i * h] * o[0];
#pragma unroll
    for (int j = 1; j < h; ++j) Q = fma(B[i * h + j], o[j], Q);
    out[i] = P + Q;
    out[N - 1 - i] = Q - P;
  }
  if (odd) {
    T Q = B[h * h] * o[0];
#pragma unroll
    for (int j = 1; j < h; ++j) Q = fma(B[h * h + j], o[j], Q);
    out[h] = Q;
  }
}

// ---- exact FP64 -> (hi, lo) FP32 split with integer operations -----------
// hi = u truncated to 24 significant bits, lo = the next 23 bits (u - hi to
// 2^-47 relative).  |u| < 2^-126 flushes to (0, 0); the lo part flushes below
// 2^-103.  Non-finite u gives (u as float, 0).
__device__ __forceinline__ void split_df(double u, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  const unsigned int top = (unsigned int)(b >> 32);
  const unsigned int sign = top & 0x80000000u;
  const int e = (int)((top >> 20) & 0x7ffu);
  if (e >= 1023 + 128) {
    hi = __double2float_rn(u);
    lo = 0.0f;
    return;
  }
  if (e < 1023 - 126) {
    hi = 0.0f;
    lo = 0.0f;
    return;
  }
  const unsigned int mhi = (unsigned int)((b >> 29) & 0x7fffffu);
  hi = __int_as_float((int)(sign | ((unsigned int)(e - 1023 + 127) << 23) | mhi));
  const unsigned int mlo = (unsigned int)(b & 0x1fffffffu);
  if (e < 920 || mlo == 0u) {
    lo = 0.0f;
    return;
  }
  // (1 + m 2^-23) - 1 is exact; m = mlo >> 6 keeps the top 23 of the 29 bits
  const float f = __int_as_float((int)(0x3f800000u | (mlo >> 6))) - 1.0f;
  const float scale = __int_as_float((e - 919) << 23);  // 2^(e - 1046)
  lo = __int_as_float(__float_as_int(f * scale) | (int)sign);
}

// exact FP32 -> FP64 widening with integer operations (normal floats; zero
// and subnormals widen to signed zero)
__device__ __forceinline__ double widen(float f) {
  const unsigned int b = (unsigned int)__float_as_int(f);
  const unsigned int e = (b >> 23) & 0xffu;
  if (e == 0u)
    return __longlong_as_double((long long)((unsigned long long)(b & 0x80000000u) << 32));
  if (e == 0xffu) return (double)f;
  const unsigned int hiw = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
  return __hiloint2double((int)hiw, (int)((b & 0x7u) << 29));
}

// ---- error-free FP32 transformations --------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t) {
  s = a + b;
  const float bb = s - a;
  t = (a - (s - bb)) + (b - bb);
}

// compensated accumulation of (ah + al)(xh + xl) into (s, c)
__device__ __forceinline__ void dot2_term(float ah, float al, float xh, float xl, float& s,
                                          float& c) {
  const float p = ah * xh;
  const float pe = fmaf(ah, xh, -p);
  float t;
  two_sum(s, p, s, t);
  c += t + pe;
  c = fmaf(al, xh, c);
  c = fmaf(ah, xl, c);
}

__device__ __forceinline__ void dot2_first(float ah, float al, float xh, float xl, float& s,
                                           float& c) {
  s = ah * xh;
  c = fmaf(ah, xh, -s);
  c = fmaf(al, xh, c);
  c = fmaf(ah, xl, c);
}

// w - gamma2 Psi in double-float: (wh, wl) -= (gh + gl)(ph + pl), gamma2 =
// gh + gl and Psi = ph + pl split into FP32 pairs
__device__ __forceinline__ void sub_g2psi(float& wh, float& wl, float gh, float gl, float ph,
                                          float pl) {
  float qh, qc, t;
  dot2_first(gh, gl, ph, pl, qh, qc);
  two_sum(wh, -qh, wh, t);
  wl = wl + (t - qc);
}

// compensated (scaled D) x line in double-float, FP32 result (odd N allowed)
template <int N>
__device__ __forceinline__ void eo_line_df(const float (&xh)[N], const float (&xl)[N],
                                           float (&out)[N], const float* __restrict__ th,
                                           const float* __restrict__ tl) {
  constexpr int h = Eo<N>::h, H = Eo<N>::H, odd = Eo<N>::odd;
  float eh[h], el[h], oh[h], ol[h];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    float t;
    two_sum(xh[j], xh[N - 1 - j], eh[j], t);
    el[j] = t + (xl[j] + xl[N - 1 - j]);
    two_sum(xh[j], -xh[N - 1 - j], oh[j], t);
    ol[j] = t + (xl[j] - xl[N - 1 - j]);
  }
  const float* Ah = th;
  const float* Al = tl;
  const float* Bh = th + H * h;
  const float* Bl = tl + H * h;
  const float* Mh = th + 2 * H * h;
  const float* Ml = tl + 2 * H * h;
#pragma unroll
  for (int i = 0; i < h; ++i) {
    float ps, pc, qs, qc;
    dot2_first(Ah[i * h], Al[i * h], eh[0], el[0], ps, pc);
#pragma unroll
    for (int j = 1; j < h; ++j) dot2_term(Ah[i * h + j], Al[i * h + j], eh[j], el[j], ps, pc);
    if (odd) dot2_term(Mh[i], Ml[i], xh[h], xl[h], ps, pc);
    dot2_first(Bh[i * h], Bl[i * h], oh[0], ol[0], qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j) dot2_term(Bh[i * h + j], Bl[i * h + j], oh[j], ol[j], qs, qc);
    out[i] = (ps + qs) + (pc + qc);
    out[N - 1 - i] = (qs - ps) + (qc - pc);
  }
  if (odd) {
    float qs, qc;
    dot2_first(Bh[h * h], Bl[h * h], oh[0], ol[0], qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j) dot2_term(Bh[h * h + j], Bl[h * h + j], oh[j], ol[j], qs, qc);
    out[h] = qs + qc;
  }
}

}  // namespace dev
}  // namespace dgsw
