// filter_line.cuh -- the 1D exponential filter matrix F applied to one line,
// with its mirror symmetry.
//
// F = V diag(sigma) V^-1 on the LGL nodes (Spectral/Filtering.cpp:18-31).
// The nodes are symmetric about 0 and Legendre polynomials have parity, so F
// commutes with the reflection of the line: F[N-1-i][N-1-j] = F[i][j].  With
// e_j = x_j + x_{N-1-j} and o_j = x_j - x_{N-1-j} (j < h = N/2),
//   P_i = sum_j A_ij e_j (+ F[i][h] x_h for odd N),  Q_i = sum_j B_ij o_j,
//   out_i = P_i + Q_i,  out_{N-1-i} = P_i - Q_i,
//   A_ij = (F[i][j] + F[i][N-1-j]) / 2,  B_ij = (F[i][j] - F[i][N-1-j]) / 2,
// and for odd N the middle row out_h = sum_j R_j e_j + F[h][h] x_h with
// R_j = (F[h][j] + F[h][N-1-j]) / 2: N^2 / 2 + O(N) multiply-adds per line
// instead of N^2.
//
// Table layout (SymTab<N>::SIZE entries): A (h x h), B (h x h), M (h: the
// middle column F[i][h]), R (h), and F[h][h]; M, R and the last entry are
// used for odd N only.
#pragma once

#include "dg_device.cuh"

namespace dgsw {
namespace filt {

template <int N>
struct SymTab {
  static constexpr int h = N / 2;
  static constexpr int odd = N % 2;
  static constexpr int A = 0, B = h * h, M = 2 * h * h, R = 2 * h * h + h, C = 2 * h * h + 2 * h;
  static constexpr int SIZE = 2 * h * h + 2 * h + 1;
};

// entry q of the split tables from the FP64 matrix F (row-major N x N)
template <int N>
__device__ __forceinline__ double sym_entry(const double* F, int q) {
  using T = SymTab<N>;
  constexpr int h = T::h;
  if (q < T::B) {
    const int i = q / h, j = q - (q / h) * h;
    return 0.5 * (F[i * N + j] + F[i * N + N - 1 - j]);
  }
  if (q < T::M) {
    const int r = q - T::B, i = r / h, j = r - (r / h) * h;
    return 0.5 * (F[i * N + j] - F[i * N + N - 1 - j]);
  }
  if (!T::odd) return 0.0;
  if (q < T::R) return F[(q - T::M) * N + h];
  if (q < T::C) {
    const int j = q - T::R;
    return 0.5 * (F[h * N + j] + F[h * N + N - 1 - j]);
  }
  return F[h * N + h];
}

// out = F x, plain arithmetic of type Tv (FP64 or FP32)
template <int N, typename Tv>
__device__ __forceinline__ void sym_line(const Tv (&x)[N], Tv (&out)[N], const Tv* __restrict__ t) {
  using T = SymTab<N>;
  constexpr int h = T::h;
  Tv e[h > 0 ? h : 1], o[h > 0 ? h : 1];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    e[j] = x[j] + x[N - 1 - j];
    o[j] = x[j] - x[N - 1 - j];
  }
#pragma unroll
  for (int i = 0; i < h; ++i) {
    Tv P = t[T::A + i * h] * e[0];
#pragma unroll
    for (int j = 1; j < h; ++j) P = fma(t[T::A + i * h + j], e[j], P);
    if (T::odd) P = fma(t[T::M + i], x[h], P);
    Tv Q = t[T::B + i * h] * o[0];
#pragma unroll
    for (int j = 1; j < h; ++j) Q = fma(t[T::B + i * h + j], o[j], Q);
    out[i] = P + Q;
    out[N - 1 - i] = P - Q;
  }
  if (T::odd) {
    Tv P = t[T::C] * x[h];
#pragma unroll
    for (int j = 0; j < h; ++j) P = fma(t[T::R + j], e[j], P);
    out[h] = P;
  }
}

// out = F x in double-float: x = xh + xl, tables th + tl; each result as an
// (oh, ol) pair with oh = fl(oh + ol)
template <int N>
__device__ __forceinline__ void sym_line_df(const float (&xh)[N], const float (&xl)[N],
                                            float (&oh)[N], float (&ol)[N],
                                            const float* __restrict__ th,
                                            const float* __restrict__ tl) {
  using T = SymTab<N>;
  constexpr int h = T::h;
  float eh[h > 0 ? h : 1], el[h > 0 ? h : 1], qh[h > 0 ? h : 1], ql[h > 0 ? h : 1];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    float t;
    dev::two_sum(xh[j], xh[N - 1 - j], eh[j], t);
    el[j] = t + (xl[j] + xl[N - 1 - j]);
    dev::two_sum(xh[j], -xh[N - 1 - j], qh[j], t);
    ql[j] = t + (xl[j] - xl[N - 1 - j]);
  }
#pragma unroll
  for (int i = 0; i < h; ++i) {
    float ps, pc, qs, qc, s, t;
    dev::dot2_first(th[T::A + i * h], tl[T::A + i * h], eh[0], el[0], ps, pc);
#pragma unroll
    for (int j = 1; j < h; ++j)
      dev::dot2_term(th[T::A + i * h + j], tl[T::A + i * h + j], eh[j], el[j], ps, pc);
    if (T::odd) dev::dot2_term(th[T::M + i], tl[T::M + i], xh[h], xl[h], ps, pc);
    dev::dot2_first(th[T::B + i * h], tl[T::B + i * h], qh[0], ql[0], qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j)
      dev::dot2_term(th[T::B + i * h + j], tl[T::B + i * h + j], qh[j], ql[j], qs, qc);
    dev::two_sum(ps, qs, s, t);
    dev::two_sum(s, t + (pc + qc), oh[i], ol[i]);
    dev::two_sum(ps, -qs, s, t);
    dev::two_sum(s, t + (pc - qc), oh[N - 1 - i], ol[N - 1 - i]);
  }
  if (T::odd) {
    float ps, pc;
    dev::dot2_first(th[T::C], tl[T::C], xh[h], xl[h], ps, pc);
#pragma unroll
    for (int j = 0; j < h; ++j) dev::dot2_term(th[T::R + j], tl[T::R + j], eh[j], el[j], ps, pc);
    dev::two_sum(ps, pc, oh[h], ol[h]);
  }
}

// the (base, stride) of line `line` along axis a of an N^3 block
template <int N>
__device__ __forceinline__ void axis_line(int a, int line, int& base, int& stride) {
  const int ta = line % N, tb = line / N;
  if (a == 0) {
    base = N * ta + N * N * tb;
    stride = 1;
  } else if (a == 1) {
    base = ta + N * N * tb;
    stride = N;
  } else {
    base = ta + N * tb;
    stride = N * N;
  }
}

// threads of a block that owns one variable of one element: one per line
template <int N>
constexpr int line_threads() {
  return (N * N + 31) / 32 * 32;
}

}  // namespace filt
}  // namespace dgsw
