// eo_packed.cuh -- even/odd split contractions of one line with Blackwell's
// packed FP32 instructions (FFMA2 / FADD2 / FMUL2): the even part P and the
// odd part Q of each output pair in the two lanes.  Any extent N (odd N adds
// the middle point's column and the middle row).
#pragma once

#include "dg_device.cuh"
#include "pipe.cuh"

namespace dgsw {
namespace pipe {

// Table layout of the even/odd split of D (h = N/2): pairs (A_ij, B_ij),
// i, j < h, as float2 [h*h], then for odd N the middle-point column M_i
// (i < h) and the middle row B_hj (j < h).
__host__ __device__ constexpr int tab_stride(int n) {
  return 2 * (n / 2) * (n / 2) + ((n & 1) ? 2 * (n / 2) : 0);
}

// packed plain contraction (lanes: x = even part P, y = odd part Q)
template <int N>
__device__ __forceinline__ void eo_line_pg(const float (&x)[N], float (&out)[N],
                                           const float* __restrict__ tab) {
  constexpr int h = N / 2, odd = N & 1;
  const float2* pr = reinterpret_cast<const float2*>(tab);
  float2 eo[h];
#pragma unroll
  for (int j = 0; j < h; ++j) eo[j] = make_float2(x[j] + x[N - 1 - j], x[j] - x[N - 1 - j]);
#pragma unroll
  for (int i = 0; i < h; ++i) {
    float2 acc = mul2(pr[i * h], eo[0]);
#pragma unroll
    for (int j = 1; j < h; ++j) acc = fma2(pr[i * h + j], eo[j], acc);
    float P = acc.x;
    if (odd) P = fmaf(tab[2 * h * h + i], x[h], P);
    out[i] = P + acc.y;
    out[N - 1 - i] = acc.y - P;
  }
  if (odd) {
    const float* bm = tab + 2 * h * h + h;
    float Q = bm[0] * eo[0].y;
#pragma unroll
    for (int j = 1; j < h; ++j) Q = fmaf(bm[j], eo[j].y, Q);
    out[h] = Q;
  }
}

// packed compensated contraction of a double-float line (hi + lo tables)
template <int N>
__device__ __forceinline__ void eo_line_pdfg(const float (&xh)[N], const float (&xl)[N],
                                             float (&out)[N], const float* __restrict__ th,
                                             const float* __restrict__ tl) {
  constexpr int h = N / 2, odd = N & 1;
  const float2* ph = reinterpret_cast<const float2*>(th);
  const float2* pl = reinterpret_cast<const float2*>(tl);
  float2 eoh[h], eol[h];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    float2 s, t;
    two_sum2(make_float2(xh[j], xh[j]), make_float2(xh[N - 1 - j], -xh[N - 1 - j]), s, t);
    eoh[j] = s;
    eol[j] = add2(t, make_float2(xl[j] + xl[N - 1 - j], xl[j] - xl[N - 1 - j]));
  }
#pragma unroll
  for (int i = 0; i < h; ++i) {
    // s: the running sum of the products' high parts; the corrections are
    // three independent sums (rounding errors of s and of the products; the
    // table's low parts; the data's low parts), added at the end
    float2 s = mul2(ph[i * h], eoh[0]);
    float2 c1 = fma2(ph[i * h], eoh[0], neg2(s));
    float2 c2 = mul2(pl[i * h], eoh[0]);
    float2 c3 = mul2(ph[i * h], eol[0]);
#pragma unroll
    for (int j = 1; j < h; ++j) {
      const float2 a = ph[i * h + j];
      const float2 p = mul2(a, eoh[j]);
      const float2 pe = fma2(a, eoh[j], neg2(p));
      float2 t;
      two_sum2(s, p, s, t);
      c1 = add2(c1, add2(t, pe));
      c2 = fma2(pl[i * h + j], eoh[j], c2);
      c3 = fma2(a, eol[j], c3);
    }
    float2 c = add2(c1, add2(c2, c3));
    if (odd) dev::dot2_term(th[2 * h * h + i], tl[2 * h * h + i], xh[h], xl[h], s.x, c.x);
    out[i] = (s.x + s.y) + (c.x + c.y);
    out[N - 1 - i] = (s.y - s.x) + (c.y - c.x);
  }
  if (odd) {
    const float* bh = th + 2 * h * h + h;
    const float* bl = tl + 2 * h * h + h;
    float qs, qc;
    dev::dot2_first(bh[0], bl[0], eoh[0].y, eol[0].y, qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j) dev::dot2_term(bh[j], bl[j], eoh[j].y, eol[j].y, qs, qc);
    out[h] = qs + qc;
  }
}

}  // namespace pipe
}  // namespace dgsw
