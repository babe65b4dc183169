// taylor_df.cuh -- the plain DG step and its discrete adjoint with FP64
// states and double-float increments formed with FP32 arithmetic: the step of
// DGSW_PRECISION_DOUBLE_FLOAT handles, and both sweeps of the misfit gradient
// on mixed-precision and double-float handles.
//
// The operator L of the flat ScalarWave system with gamma2 = 0 is linear and
// does not change in time, so one Rk3HesthavenSsp step (Rk3HesthavenSsp.cpp:
// 63-80) is the third-order Taylor polynomial u <- (1 + dt L + (dt L)^2 / 2 +
// (dt L)^3 / 6) u:
//   W1 = dt L u,  W2 = dt L W1,  W3 = dt L W2,  u <- u + (W1 + W2/2 + W3/6),
// and the step's adjoint is the same with L^T in place of L.  (Expanding the
// reverse stages m2 = 2/3 (l + dt L^T l), m1 = 1/4 (m2 + dt L^T m2),
// l <- m1 + dt L^T m1 + 3/4 m2 + 1/3 l of adjoint_fp64.cu gives the same
// polynomial.)
//
// Every increment is a double-float value, a (hi, lo) pair of FP32 numbers
// (8 bytes, like FP64), formed with FP32 arithmetic only: the FP64 state
// split into pairs, the split tables of D (or D^T) in hi + lo FP32,
// compensated products and sums.  The misfit gradient needs the forward
// residuals (sample - target, ~1e-2 of the field) and the rough adjoint field
// (driven by point injections) to ~1e-8 over thousands of steps, which
// FP32-rounded increments do not keep (they lost ~2e-6 of the gradient over
// 2000 steps).  The step's sum W1 + W2/2 + W3/6 is formed in double-float and
// added to the FP64 state once per step (two FP64 adds per value: the FP64
// pipe does nothing else).
//
// Forward: (L u)_Psi = -Pi, (L u)_Pi = -sum_d J_d D_d Phi_d + B_Pi,
// (L u)_Phi_d = -J_d D_d Pi + B_Phi_d (stage_fp64.cu), nothing reads Psi.
// Adjoint: (L^T l)_Psi = 0, so the adjoint increments' Psi parts are zero and
// are neither written nor read; only W1's Pi part takes -dt l_Psi.
//
// Work split: one element per block and 3 N^2 threads, one per (axis, line),
// as in the split variants of stage_fp64.cu and adjoint_fp64.cu; each axis
// leaves its share of the Pi sum in shared memory and the block adds the
// three after a barrier.
#pragma once

#include <cstdint>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

using dev::Eo;
using dev::split_df;
using dev::two_sum;
using dev::widen;

template <int N>
struct MShape {
  static constexpr int NN = N * N, NP = N * N * N;
  static constexpr int TAB = Eo<N>::TAB;
  // floats: X (Pi, Phi as hi and lo), three axis sums as (hi, lo), tables hi,
  // lo; rounded to 16 bytes
  static constexpr int SIZE = (8 * NP + 6 * NP + 2 * TAB + 3) / 4 * 4;
  // the last launch's prefetch regions (floats): the state block (FP64), W1
  // and W2's Psi (pairs)
  static constexpr int PF_EXTRA = 10 * NP + 10 * NP + 2 * NP;
  static constexpr bool PF_FITS = (SIZE + PF_EXTRA) * 4 <= 200 * 1024;
};

// 8-byte asynchronous global -> shared copies (cp.async), and the wait for
// all of this thread's
__device__ __forceinline__ void cp_async8(void* smem_dst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// double-float helpers: (h, l) with |l| <= ulp(h) / 2
__device__ __forceinline__ void quick_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
__device__ __forceinline__ void df_add(float ah, float al, float bh, float bl, float& sh,
                                       float& sl) {
  float s, t;
  two_sum(ah, bh, s, t);
  quick_two_sum(s, t + (al + bl), sh, sl);
}
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph,
                                       float& pl) {
  const float p = ah * bh;
  const float e = fmaf(ah, bh, -p);
  quick_two_sum(p, fmaf(ah, bl, fmaf(al, bh, e)), ph, pl);
}

// D x (or D^T x) along one line in double-float with every result kept as a
// (hi, lo) pair: both have large corner entries (D_00 = -N(N-1)/4; D^T =
// B M^-1 - M D M^-1 with |B M^-1| = N(N-1)/2 at the ends) which the lifted
// face terms cancel, so the ends stay unrounded until those are added.
template <int N>
__device__ __forceinline__ void eo_line_pairs(const float (&xh)[N], const float (&xl)[N],
                                              float (&oh)[N], float (&ol)[N],
                                              const float* __restrict__ th,
                                              const float* __restrict__ tl) {
  using dev::dot2_first;
  using dev::dot2_term;
  constexpr int h = Eo<N>::h, H = Eo<N>::H, odd = Eo<N>::odd;
  float eh[h], el[h], qh[h], ql[h];
#pragma unroll
  for (int j = 0; j < h; ++j) {
    float t;
    two_sum(xh[j], xh[N - 1 - j], eh[j], t);
    el[j] = t + (xl[j] + xl[N - 1 - j]);
    two_sum(xh[j], -xh[N - 1 - j], qh[j], t);
    ql[j] = t + (xl[j] - xl[N - 1 - j]);
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
    dot2_first(Bh[i * h], Bl[i * h], qh[0], ql[0], qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j) dot2_term(Bh[i * h + j], Bl[i * h + j], qh[j], ql[j], qs, qc);
    df_add(ps, pc, qs, qc, oh[i], ol[i]);
    df_add(qs, qc, -ps, -pc, oh[N - 1 - i], ol[N - 1 - i]);
  }
  if (odd) {
    float qs, qc;
    dot2_first(Bh[h * h], Bl[h * h], qh[0], ql[0], qs, qc);
#pragma unroll
    for (int j = 1; j < h; ++j) dot2_term(Bh[h * h + j], Bl[h * h + j], qh[j], ql[j], qs, qc);
    quick_two_sum(qs, qc, oh[h], ol[h]);
  }
}

// (wh, wl) -= (gh, gl) (ph, pl) in double-float: the gamma2 Psi of w
__device__ __forceinline__ void sub_g2psi_df(float& wh, float& wl, float gh, float gl, float ph,
                                             float pl) {
  float qh, ql;
  df_mul(gh, gl, ph, pl, qh, ql);
  df_add(wh, wl, -qh, -ql, wh, wl);
}

// (vh, vl) += k (dh, dl), k a small integer or half-integer (exact in FP32)
__device__ __forceinline__ void df_axpy(float& vh, float& vl, float k, float dh, float dl) {
  const float p = k * dh;
  const float pe = fmaf(k, dh, -p);
  float s, t;
  two_sum(vh, p, s, t);
  quick_two_sum(s, t + (vl + fmaf(k, dl, pe)), vh, vl);
}

// Value q of the input as a (hi, lo) pair: the FP64 l split, or a stored pair
template <bool FIRST>
__device__ __forceinline__ void load_pair(const TaylorLaunch& L, int64_t q, float& h,
                                          float& l) {
  if (FIRST) {
    split_df(L.x64[q], h, l);
  } else {
    const float2 v = L.xp[q];
    h = v.x;
    l = v.y;
  }
}

// A contiguous row of N floats (an x line) moved 16 or 8 bytes at a time
template <int N>
__device__ __forceinline__ void load_row(const float* p, float (&x)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int k = 0; k < N / 4; ++k) {
      const float4 v = reinterpret_cast<const float4*>(p)[k];
      x[4 * k] = v.x;
      x[4 * k + 1] = v.y;
      x[4 * k + 2] = v.z;
      x[4 * k + 3] = v.w;
    }
  } else if constexpr (N % 2 == 0) {
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      const float2 v = reinterpret_cast<const float2*>(p)[k];
      x[2 * k] = v.x;
      x[2 * k + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) x[i] = p[i];
  }
}
template <int N>
__device__ __forceinline__ void store_row(float* p, const float (&x)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int k = 0; k < N / 4; ++k)
      reinterpret_cast<float4*>(p)[k] = make_float4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
  } else if constexpr (N % 2 == 0) {
#pragma unroll
    for (int k = 0; k < N / 2; ++k) reinterpret_cast<float2*>(p)[k] = make_float2(x[2 * k], x[2 * k + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = x[i];
  }
}
// a row of N (hi, lo) pairs, two pairs per 16-byte store (even N)
template <int N>
__device__ __forceinline__ void store_row_pairs(float2* p, const float (&h)[N], const float (&l)[N]) {
  if constexpr (N % 2 == 0) {
#pragma unroll
    for (int k = 0; k < N / 2; ++k)
      reinterpret_cast<float4*>(p)[k] = make_float4(h[2 * k], l[2 * k], h[2 * k + 1], l[2 * k + 1]);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) p[i] = make_float2(h[i], l[i]);
  }
}

// W1 + W2/2 + W3/6 of one value in double-float, W3 = (w3h, w3l), widened
__device__ __forceinline__ double step_inc(const TaylorLaunch& L, float2 w1, float2 w2, float w3h,
                                           float w3l) {
  float sh, sl, uh, ul;
  df_mul(w3h, w3l, L.sixth_h, L.sixth_l, uh, ul);        // W3 / 6
  df_add(w1.x, w1.y, 0.5f * w2.x, 0.5f * w2.y, sh, sl);  // W1 + W2 / 2
  df_add(sh, sl, uh, ul, sh, sl);
  return widen(sh) + widen(sl);
}

// state[q] += W1 + W2/2 + W3/6 at value q
__device__ __forceinline__ void step_sum(const TaylorLaunch& L, int64_t q, float w3h, float w3l) {
  const double v = L.l64[q];
  L.l64[q] = v + step_inc(L, L.w1[q], L.xp[q], w3h, w3l);
}

// TR: L^T (else L).  FIRST: x = the FP64 state; otherwise x = W1 or W2
// (pairs).  FINAL: W3 = dt L W2 stays in registers and the state takes
// W1 + W2/2 + W3/6; otherwise out = dt L x.  LW (final launch): the state
// is not prefetched, so that the block's shared memory allows one more
// resident block; its loads are issued in batches in the epilogue.
template <int N, bool TR, bool FIRST, bool FINAL, int MINB, bool LW = false, bool G2 = false>
__global__ void __launch_bounds__(3 * N * N, MINB) taylor_df_kernel(TaylorLaunch L) {
  using S = MShape<N>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB;
  constexpr int h = Eo<N>::h, H = Eo<N>::H;
  extern __shared__ float msm_[];
  float* Xh = msm_;                 // Pi, Phi_x, Phi_y, Phi_z: hi
  float* Xl = msm_ + 4 * NP;        // and lo
  float2* Sd = reinterpret_cast<float2*>(msm_ + 8 * NP);  // each axis's share of the Pi sum
  float* th = msm_ + 14 * NP;       // split tables of D (D^T), hi
  float* tl = th + TAB;             // and lo
  constexpr int NT = 3 * NN;  // threads
  const int d = threadIdx.x / NN;
  const int t = threadIdx.x - d * NN;
  const int64_t e = L.elem_begin + blockIdx.x;  // the grid covers the range exactly
  const int64_t off = e * (int64_t)(kVars * NP);
  const double c = L.dt;
  const int ta = t % N, tb = t / N;
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
  // G2 (forward, gamma2 != 0): the input's Psi as (hi, lo) pairs, for
  // d_d Psi and the w = Pi - s Phi_d - gamma2 Psi of the faces
  static_assert(!(G2 && TR), "the transposed step is built for gamma2 = 0");
  constexpr int B0 = S::SIZE + (G2 ? 2 * NP : 0);
  float* Ph = msm_ + S::SIZE;  // Psi hi (G2)
  float* Pl = Ph + NP;         // and lo
  float g2h = 0.0f, g2l = 0.0f;
  if (G2) split_df(L.gamma2, g2h, g2l);
  // The last launch (where it fits): the values its update reads -- the
  // state, W1 and (forward) W2's Psi -- copied to shared memory in the
  // background while the block computes W3 (W2's Pi and Phi are staged
  // below).
  constexpr bool PF = FINAL && S::PF_FITS;
  constexpr bool PFU = PF && !LW;  // the state prefetched too
  double* Us = reinterpret_cast<double*>(msm_ + B0);
  float2* W1s = reinterpret_cast<float2*>(msm_ + B0 + (PFU ? 10 * NP : 0));
  float2* W2ps = reinterpret_cast<float2*>(msm_ + B0 + (PFU ? 20 * NP : 10 * NP));
  if (PF) {
    // the adjoint leaves l_Psi unchanged (its increments' Psi is 0)
    for (int q = TR ? NP + threadIdx.x : threadIdx.x; q < kVars * NP; q += NT) {
      if (PFU) cp_async8(Us + q, L.l64 + off + q);
      cp_async8(W1s + q, L.w1 + off + q);
    }
    if (!TR)
      for (int q = threadIdx.x; q < NP; q += NT) cp_async8(W2ps + q, L.xp + off + q);
  }
  // the neighbours' values at this line's two face points, loaded first so
  // that their latency overlaps the staging below
  float nbh[G2 ? 6 : 4], nbl[G2 ? 6 : 4];
  {
    const int64_t nlo = (int64_t)L.nbr[6 * e + 2 * d] * (kVars * NP);
    const int64_t nhi = (int64_t)L.nbr[6 * e + 2 * d + 1] * (kVars * NP);
    const int64_t lo_pt = base + (N - 1) * stride;  // lower neighbour's upper face
    const int64_t hi_pt = base;                     // upper neighbour's lower face
    load_pair<FIRST>(L, nlo + NP + lo_pt, nbh[0], nbl[0]);
    load_pair<FIRST>(L, nlo + (2 + d) * NP + lo_pt, nbh[1], nbl[1]);
    load_pair<FIRST>(L, nhi + NP + hi_pt, nbh[2], nbl[2]);
    load_pair<FIRST>(L, nhi + (2 + d) * NP + hi_pt, nbh[3], nbl[3]);
    if (G2) {
      load_pair<FIRST>(L, nlo + lo_pt, nbh[G2 ? 4 : 0], nbl[G2 ? 4 : 0]);
      load_pair<FIRST>(L, nhi + hi_pt, nbh[G2 ? 5 : 0], nbl[G2 ? 5 : 0]);
    }
  }
  {
    // the element's Pi and Phi, all of a thread's loads issued before any
    // is used
    constexpr int QPT = (4 * NP + NT - 1) / NT;
    float vh[QPT], vl[QPT];
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
      const int q = threadIdx.x + k * NT;
      if (q < 4 * NP) load_pair<FIRST>(L, off + NP + q, vh[k], vl[k]);
    }
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
      const int q = threadIdx.x + k * NT;
      if (q < 4 * NP) {
        Xh[q] = vh[k];
        Xl[q] = vl[k];
      }
    }
  }
  if (G2)
    for (int q = threadIdx.x; q < NP; q += NT) load_pair<FIRST>(L, off + q, Ph[q], Pl[q]);
  for (int q = threadIdx.x; q < TAB; q += NT) {
    double v;
    if (q < H * h)
      v = L.eo.A[q / h][q % h];
    else if (q < 2 * H * h)
      v = L.eo.B[(q - H * h) / h][(q - H * h) % h];
    else
      v = L.eo.M[q - 2 * H * h];
    const float vh = __double2float_rn(v);
    th[q] = vh;
    tl[q] = __double2float_rn(v - (double)vh);
  }
  const double fd = -c * L.jac[3 * e + d];  // the line's scale -c (d xi_d/dx_d)
  const float Fh = __double2float_rn(fd), Fl = __double2float_rn(fd - (double)Fh);
  __syncthreads();
  {
    // UpwindPenalty at both ends of the line, lifted with G = fd K, K =
    // N(N-1)/4: the sums are formed unscaled, then scaled.  Forward
    // (stage_fp64.cu): dw = w_int - w_ext, w = Pi - s Phi_d, dPi += G dw,
    // dPhi_d += -s G dw.  Transposed (adjoint_fp64.cu): q = G (l_Pi - s
    // l_Phi_d) of this element, q' = G (l_Pi,nbr + s l_Phi_d,nbr) of the
    // neighbour; dPi += q - q', dPhi_d += -s (q + q').  The Phi_d line is
    // differentiated first and its result leaves registers (into Sd) before
    // the Pi line's: fewer live registers, more resident blocks.
    constexpr float K = 0.25f * (float)(N * (N - 1));
    float e0h, e0l, e1h, e1l;  // the dF face terms: a - b at both ends
    float g0h, g0l, g1h, g1l;  // the dP face terms (a - b forward, a + b transposed)
    float ph[N], pl[N];
    {
      float fh[N], fl[N];
      if (d == 0) {
        // x lines are contiguous rows N floats apart: vector accesses keep
        // the shared-memory banks from serialising them
        load_row<N>(Xh + base, ph);
        load_row<N>(Xl + base, pl);
        load_row<N>(Xh + NP + base, fh);
        load_row<N>(Xl + NP + base, fl);
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          ph[i] = Xh[base + i * stride];
          pl[i] = Xl[base + i * stride];
          fh[i] = Xh[(1 + d) * NP + base + i * stride];
          fl[i] = Xl[(1 + d) * NP + base + i * stride];
        }
      }
      {
        float ah, al, bh, bl;
        // s = -1: a = Pi + Phi_d here; b = the neighbour's Pi -+ Phi_d
        df_add(ph[0], pl[0], fh[0], fl[0], ah, al);
        df_add(nbh[0], nbl[0], TR ? -nbh[1] : nbh[1], TR ? -nbl[1] : nbl[1], bh, bl);
        if (G2) {
          // w = Pi - s Phi_d - gamma2 Psi on both sides
          sub_g2psi_df(ah, al, g2h, g2l, Ph[base], Pl[base]);
          sub_g2psi_df(bh, bl, g2h, g2l, nbh[G2 ? 4 : 0], nbl[G2 ? 4 : 0]);
        }
        df_add(ah, al, -bh, -bl, e0h, e0l);
        if (TR) {
          df_add(ah, al, bh, bl, g0h, g0l);
        } else {
          g0h = e0h;
          g0l = e0l;
        }
        // s = +1: a = Pi - Phi_d here; b = the neighbour's Pi +- Phi_d
        df_add(ph[N - 1], pl[N - 1], -fh[N - 1], -fl[N - 1], ah, al);
        df_add(nbh[2], nbl[2], TR ? nbh[3] : -nbh[3], TR ? nbl[3] : -nbl[3], bh, bl);
        if (G2) {
          sub_g2psi_df(ah, al, g2h, g2l, Ph[base + (N - 1) * stride], Pl[base + (N - 1) * stride]);
          sub_g2psi_df(bh, bl, g2h, g2l, nbh[G2 ? 5 : 0], nbl[G2 ? 5 : 0]);
        }
        df_add(ah, al, -bh, -bl, e1h, e1l);
        if (TR) {
          df_add(ah, al, bh, bl, g1h, g1l);
        } else {
          g1h = e1h;
          g1l = e1l;
        }
      }
      float dFh[N], dFl[N];
      eo_line_pairs<N>(fh, fl, dFh, dFl, th, tl);  // D Phi_d : into Pi
      df_axpy(dFh[0], dFl[0], K, e0h, e0l);
      df_axpy(dFh[N - 1], dFl[N - 1], K, e1h, e1l);
#pragma unroll
      for (int i = 0; i < N; ++i) df_mul(dFh[i], dFl[i], Fh, Fl, dFh[i], dFl[i]);
      // this axis's share of the Pi sum (Sd is read after the last barrier)
      if (d == 0) {
        store_row_pairs<N>(Sd + base, dFh, dFl);
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) Sd[d * NP + base + i * stride] = make_float2(dFh[i], dFl[i]);
      }
    }
    float dPh[N], dPl[N];
    eo_line_pairs<N>(ph, pl, dPh, dPl, th, tl);  // D Pi : into Phi_d
    df_axpy(dPh[0], dPl[0], K, g0h, g0l);
    df_axpy(dPh[N - 1], dPl[N - 1], -K, g1h, g1l);
#pragma unroll
    for (int i = 0; i < N; ++i) df_mul(dPh[i], dPl[i], Fh, Fl, dPh[i], dPl[i]);
    if (G2) {
      // the gamma2 (d_d Psi - Phi_d) term of dt Phi_d (TimeDerivative.cpp:
      // 42-43): dP -= gamma2 (fd D Psi + c Phi_d), fd = -c (d xi_d/dx_d)
      float sh[N], sl[N], qh[N], ql[N];
      if (d == 0) {
        load_row<N>(Ph + base, sh);
        load_row<N>(Pl + base, sl);
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          sh[i] = Ph[base + i * stride];
          sl[i] = Pl[base + i * stride];
        }
      }
      eo_line_pairs<N>(sh, sl, qh, ql, th, tl);  // D Psi
      float ch, cl;
      split_df(c, ch, cl);
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int q = (1 + d) * NP + base + i * stride;
        float ah, al, bh, bl;
        df_mul(qh[i], ql[i], Fh, Fl, ah, al);  // fd D Psi
        df_mul(ch, cl, Xh[q], Xl[q], bh, bl);  // c Phi_d
        df_add(ah, al, bh, bl, ah, al);
        sub_g2psi_df(dPh[i], dPl[i], g2h, g2l, ah, al);
      }
    }
    // every line read: the Phi_d results replace Phi_d in shared memory (the
    // last launch: the step's sum W1 + W2/2 + W3/6 on the line replaces W2),
    // and the block writes all results out with coalesced accesses below
    if (PF) cp_async_wait_all();
    __syncthreads();
    if (PF) {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int q = (1 + d) * NP + base + i * stride;
        float sh, sl, uh, ul;
        const float2 w1 = W1s[NP + q];
        df_mul(dPh[i], dPl[i], L.sixth_h, L.sixth_l, uh, ul);          // W3 / 6
        df_add(w1.x, w1.y, 0.5f * Xh[q], 0.5f * Xl[q], sh, sl);        // W1 + W2 / 2
        df_add(sh, sl, uh, ul, dPh[i], dPl[i]);
      }
    }
    if (d == 0) {
      store_row<N>(Xh + NP + base, dPh);
      store_row<N>(Xl + NP + base, dPl);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) {
        Xh[(1 + d) * NP + base + i * stride] = dPh[i];
        Xl[(1 + d) * NP + base + i * stride] = dPl[i];
      }
    }
  }
  __syncthreads();
  // Phi: the increments, or (last launch) the step's sums into the state,
  // with all of a thread's global loads issued before any is used
  if (PFU) {
    for (int q = NP + threadIdx.x; q < 4 * NP; q += NT)
      L.l64[off + NP + q] = Us[NP + q] + (widen(Xh[q]) + widen(Xl[q]));
  } else if (PF) {
    constexpr int QPT = (3 * NP + NT - 1) / NT;
    constexpr int KB = 4;  // loads in flight per thread
#pragma unroll
    for (int k0 = 0; k0 < QPT; k0 += KB) {
      double lv[KB];
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        const int q = NP + threadIdx.x + (k0 + k) * NT;
        if (k0 + k < QPT && q < 4 * NP) lv[k] = L.l64[off + NP + q];
      }
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        const int q = NP + threadIdx.x + (k0 + k) * NT;
        if (k0 + k < QPT && q < 4 * NP)
          L.l64[off + NP + q] = lv[k] + (widen(Xh[q]) + widen(Xl[q]));
      }
    }
  } else if (FINAL) {
    constexpr int QPT = (3 * NP + NT - 1) / NT;
    constexpr int KB = 4;  // loads in flight per thread
#pragma unroll
    for (int k0 = 0; k0 < QPT; k0 += KB) {
      float2 a1[KB], a2[KB];
      double lv[KB];
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        const int q = NP + threadIdx.x + (k0 + k) * NT;
        if (k0 + k < QPT && q < 4 * NP) {
          a1[k] = L.w1[off + NP + q];
          a2[k] = L.xp[off + NP + q];
          lv[k] = L.l64[off + NP + q];
        }
      }
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        const int q = NP + threadIdx.x + (k0 + k) * NT;
        if (k0 + k < QPT && q < 4 * NP)
          L.l64[off + NP + q] = lv[k] + step_inc(L, a1[k], a2[k], Xh[q], Xl[q]);
      }
    }
  } else {
    for (int q = NP + threadIdx.x; q < 4 * NP; q += NT)
      L.outp[off + NP + q] = make_float2(Xh[q], Xl[q]);
  }
  for (int p = threadIdx.x; p < NP; p += NT) {
    const float2 s0 = Sd[p], s1 = Sd[NP + p], s2 = Sd[2 * NP + p];
    float wh, wl;
    df_add(s0.x, s0.y, s1.x, s1.y, wh, wl);
    df_add(wh, wl, s2.x, s2.y, wh, wl);
    float ch, cl;
    split_df(-c, ch, cl);
    if (TR && FIRST) {
      // (L^T l)_Pi gets -l_Psi from (L u)_Psi = -Pi; the increments' Psi is 0
      float xh, xl, yh, yl;
      split_df(L.x64[off + p], xh, xl);
      df_mul(ch, cl, xh, xl, yh, yl);
      df_add(wh, wl, yh, yl, wh, wl);
    }
    const int64_t q = off + NP + p;
    // forward: the Psi increment -c Pi of the input
    float sh = 0.0f, sl = 0.0f;
    if (!TR) df_mul(ch, cl, Xh[p], Xl[p], sh, sl);
    if (PF) {
      const double u1 = PFU ? Us[NP + p] : L.l64[q];
      L.l64[q] = u1 + step_inc(L, W1s[NP + p], make_float2(Xh[p], Xl[p]), wh, wl);
      if (!TR) {
        const double u0 = PFU ? Us[p] : L.l64[off + p];
        L.l64[off + p] = u0 + step_inc(L, W1s[p], W2ps[p], sh, sl);
      }
    } else if (FINAL) {
      step_sum(L, q, wh, wl);
      if (!TR) step_sum(L, off + p, sh, sl);
    } else {
      L.outp[q] = make_float2(wh, wl);
      if (!TR) L.outp[off + p] = make_float2(sh, sl);
    }
  }
}

// resident blocks per SM asked of the register allocator
// (N = 8: with the Phi_d line finished before the Pi line, the non-final
// kinds fit 80 registers without a spill (4 blocks per SM) or 64 with a
// 28-44 byte spill (5 blocks per SM: 1.80 against 1.90 ms per double-float
// step at 32^3); the final kind, whose shared-memory prefetch allows 3
// blocks, 91-93.  N = 9: 80 registers; 10:
// 96; 11: 80 with a 72-92 byte spill; 12: ~120.)
template <int N, bool FINAL>
constexpr int mixed_minb() {
  return N <= 4 ? 8
                : (N <= 6 ? 4
                          : (N == 7 ? 3
                                    : (N == 8 ? (FINAL ? 3 : 5)
                                              : (N == 9 ? 3 : (N <= 11 ? 2 : 1)))));
}

template <int N, bool TR, bool FIRST, bool FINAL, bool LW = false, bool G2 = false>
cudaError_t launch_k(const TaylorLaunch& L, cudaStream_t s) {
  using S = MShape<N>;
  constexpr int pf = FINAL && S::PF_FITS ? (LW ? S::PF_EXTRA - 10 * S::NP : S::PF_EXTRA) : 0;
  constexpr size_t smem = (size_t)(S::SIZE + (G2 ? 2 * S::NP : 0) + pf) * sizeof(float);
  // LW at N = 8: 53 KB of shared memory and 80 registers, 4 blocks per SM
  constexpr int minb = LW && N == 8 ? 4 : mixed_minb<N, FINAL>();
  constexpr auto k = taylor_df_kernel<N, TR, FIRST, FINAL, minb, LW, G2>;
  cudaError_t err = set_kernel_smem<k>((int)smem, true);
  if (err != cudaSuccess) return err;
  TaylorLaunch A = L;
  // 1/6 as a (hi, lo) pair
  A.sixth_h = (float)(1.0 / 6.0);
  A.sixth_l = (float)(1.0 / 6.0 - (double)A.sixth_h);
  k<<<(unsigned)L.n_elem, 3 * N * N, smem, s>>>(A);
  return cudaGetLastError();
}

template <int N, bool TR, bool G2 = false>
cudaError_t launch_kind(const TaylorLaunch& L, cudaStream_t s) {
  switch (L.kind) {
    case 0: return launch_k<N, TR, true, false, false, G2>(L, s);
    case 1: return launch_k<N, TR, false, false, false, G2>(L, s);
    case 2:
      // N = 8: the final launch without the state's prefetch (4 blocks per
      // SM) measured faster on both the 512-element and the 32^3 grid
      if constexpr (N == 8) return launch_k<N, TR, false, true, true, G2>(L, s);
      return launch_k<N, TR, false, true, false, G2>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

template <int N>
cudaError_t launch_n(const TaylorLaunch& L, cudaStream_t s) {
  return L.transpose ? launch_kind<N, true>(L, s) : launch_kind<N, false>(L, s);
}

// the launch checks and the switch over N, for one gamma2 case
template <bool G2>
cudaError_t launch_any(const TaylorLaunch& L, cudaStream_t s) {
  if (L.n_elem <= 0) return cudaSuccess;
  const bool ok = L.kind == 0 ? (L.x64 && L.outp)
                              : (L.xp && (L.kind == 1 ? L.outp != nullptr : (L.l64 && L.w1)));
  if (!ok || !L.nbr || !L.jac || (G2 && L.transpose)) return cudaErrorInvalidValue;
  switch (L.n) {
#define DGSW_TAYLOR_CASE(n)                         \
  case n:                                           \
    if constexpr (G2) return launch_kind<n, false, true>(L, s); \
    else return launch_n<n>(L, s);
    DGSW_TAYLOR_CASE(2)
    DGSW_TAYLOR_CASE(3)
    DGSW_TAYLOR_CASE(4)
    DGSW_TAYLOR_CASE(5)
    DGSW_TAYLOR_CASE(6)
    DGSW_TAYLOR_CASE(7)
    DGSW_TAYLOR_CASE(8)
    DGSW_TAYLOR_CASE(9)
    DGSW_TAYLOR_CASE(10)
    DGSW_TAYLOR_CASE(11)
    DGSW_TAYLOR_CASE(12)
#undef DGSW_TAYLOR_CASE
    default: return cudaErrorInvalidValue;
  }
}


}  // namespace
}  // namespace dgsw
