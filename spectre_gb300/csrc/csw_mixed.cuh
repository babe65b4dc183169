// csw_mixed.cuh -- mixed-precision CurvedScalarWave stage on the shell.
//
// The curved operator L (TimeDerivative + UpwindPenalty + lift + the
// radiation condition on the outer sphere) is linear in (Psi, Pi, Phi) on a
// static background and mesh, so SSP-RK3 (Rk3HesthavenSsp.cpp:63-80) takes
// the incremental form
//   d1 = dt L(u0),  s2 = d1/2 + dt/4 L(d1),  u3 = u0 + 2/3 (s2 + d1) + 2dt/3 L(s2)
// and only the first stage differentiates the full FP64 state.  One kernel
// serves every stage:  W = alpha X + beta Y + c L(X), with
//  - X FP64 (first stage): split exactly into hi + lo FP32 parts; the
//    logical derivatives are compensated double-float dot products with the
//    hi + lo split of D, and the jumps across faces are formed from the
//    hi + lo parts, so no cancellation loses more than FP32 rounding of the
//    result;
//  - X FP32 (increments): plain FP32.
// The background/geometry coefficients are the FP64 set-up tables rounded to
// FP32 (formed once from the FP64 inverse Jacobian and FP64 background); the
// FP64 state is touched only by the first stage's read and the last stage's
// u0 + W.  Outputs: w32 = W, and/or out64 = base64 + W (out64 = W without a
// base).  The work split is the FP64 kernel's (csw_fp64.cu): one element
// per block, one round per logical axis.  Each launch shape is instantiated
// in its own translation unit (csw_mixed.cu, csw_mixed_s1.cu, csw_mixed_s2.cu),
// compiled in parallel.
#pragma once

#include "common.cuh"
#include "dg_device.cuh"
#include "eo_packed.cuh"
#include "launch.hpp"
#include "pipe.cuh"

namespace dgsw {
namespace csw_mixed {

template <int N, bool COMP, int kThreads>
struct CmShape {
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = pipe::tab_stride(N);  // packed split of D (eo_packed.cuh)
  static constexpr int PTS = (NP + kThreads - 1) / kThreads;
  // floats: hi state, lo state (COMP), one axis of derivatives, outer-layer
  // derivatives, the internal-face corrections [6][5][N^2], then (at a
  // 16-byte boundary) the hi and lo tables
  static constexpr int TAB0 =
      (5 * NP + (COMP ? 5 * NP : 0) + 5 * NP + 12 * NN + 30 * NN + 3) / 4 * 4;
  static constexpr int SMEM = TAB0 + 2 * ((TAB + 3) / 4 * 4);
};

template <int N>
__device__ __forceinline__ void line_geometry(int a, int line, int& base, int& stride) {
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

// Launch shapes (threads per block, resident blocks per SM asked of the
// register allocator), timed by the handle's launch tuner:
//  0: 256 threads; three resident blocks for the plain FP32 stages, whose
//     split tables are read from shared memory where used (fewer
//     registers), two for the compensated stage.  Extents 11 and 12 ask one
//     fewer: with three (two) their lines spill 150-230 (110-160) bytes
//     (ptxas), at two (one) nothing;
//  1: 256 threads, one more resident block than shape 0 (fewer registers);
//  2: 512 threads (fewer points per thread), one fewer resident block than
//     shape 0, at least one.
constexpr int kShapes = 3;
template <int V>
constexpr int shape_threads() {
  return V == 2 ? 512 : 256;
}
template <int N, bool COMP, int V>
constexpr int shape_min_blocks() {
  constexpr int base = (COMP ? 2 : 3) - (N >= 11 ? 1 : 0);
  return V == 1 ? base + 1 : (V == 2 ? (base > 1 ? base - 1 : 1) : base);
}

template <int N, bool COMP, int kThreads, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) csw_stage_mixed_kernel(CswMixedLaunch L) {
  using S = CmShape<N, COMP, kThreads>;
  constexpr int NN = S::NN, NP = S::NP, PTS = S::PTS, TAB = S::TAB;
  extern __shared__ float fsm[];
  float* Uh = fsm;
  float* Ul = Uh + 5 * NP;  // COMP only
  float* Ga = Ul + (COMP ? 5 * NP : 0);
  float* Go = Ga + 5 * NP;
  float* Cf = Go + 12 * NN;
  float* th = fsm + S::TAB0;
  float* tl = th + (TAB + 3) / 4 * 4;
  const int64_t e = L.list ? (int64_t)L.list[blockIdx.x] : (int64_t)blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t off = e * (int64_t)(kVars * NP);
  if (L.frec && COMP) {
    // AdamsBashforth record: the element's FP64 face values as they are
    for (int fp = tid; fp < 6 * NN; fp += kThreads) {
      const int dir = fp / NN, q = fp - (fp / NN) * NN, d = dir >> 1;
      const int sl = (dir & 1) ? N - 1 : 0, fa = q % N, fb = q / N;
      const int p = d == 0 ? sl + N * (fa + N * fb)
                           : (d == 1 ? fa + N * (sl + N * fb) : fa + N * (fb + N * sl));
#pragma unroll
      for (int v = 0; v < 5; ++v)
        L.frec[e * 30 * NN + (dir * 5 + v) * NN + q] = L.x64[off + (int64_t)v * NP + p];
    }
  }
  const bool outer = L.nbr[6 * e + 5] == -2;
  if (tid == 0) {
    // L2 prefetch of what the element reads after its derivative rounds --
    // the coefficient rows of the pointwise terms, its face table and the
    // pointwise inputs -- so that those loads meet L2, not DRAM
    pipe::prefetch_l2(L.T + (e * (int64_t)kCswT + kTK) * NP,
                      (size_t)(kCswT - kTK) * NP * sizeof(float));
    pipe::prefetch_l2(L.F + e * 6 * (int64_t)kCswF * NN, (size_t)6 * kCswF * NN * sizeof(float));
    if (L.y32) pipe::prefetch_l2(L.y32 + off, (size_t)kVars * NP * sizeof(float));
    if (L.base64) pipe::prefetch_l2(L.base64 + off, (size_t)kVars * NP * sizeof(double));
  }
  // state of the element: vector loads when every element block starts on a
  // 16-byte boundary (even N and an aligned base pointer), else scalar loads
  if (COMP) {
    if (NP % 2 == 0 && (reinterpret_cast<uintptr_t>(L.x64) & 15u) == 0) {
      const double2* src = reinterpret_cast<const double2*>(L.x64 + off);
      constexpr int Q = 5 * NP / 2, KQ = (Q + kThreads - 1) / kThreads, KB = 8;
      // batches of KB loads in flight per thread before their splits
#pragma unroll
      for (int k0 = 0; k0 < KQ; k0 += KB) {
        double2 v[KB];
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          const int q = tid + (k0 + k) * kThreads;
          if (k0 + k < KQ && q < Q) v[k] = __ldg(src + q);
        }
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          const int q = tid + (k0 + k) * kThreads;
          if (k0 + k < KQ && q < Q) {
            float h0, l0, h1, l1;
            dev::split_df(v[k].x, h0, l0);
            dev::split_df(v[k].y, h1, l1);
            Uh[2 * q] = h0;
            Ul[2 * q] = l0;
            Uh[2 * q + 1] = h1;
            Ul[2 * q + 1] = l1;
          }
        }
      }
    } else {
      for (int q = tid; q < 5 * NP; q += kThreads) {
        float hi, lo;
        dev::split_df(L.x64[off + q], hi, lo);
        Uh[q] = hi;
        Ul[q] = lo;
      }
    }
  } else {
    if (NP % 4 == 0 && (reinterpret_cast<uintptr_t>(L.x32) & 15u) == 0) {
      const float4* src = reinterpret_cast<const float4*>(L.x32 + off);
      float4* dst = reinterpret_cast<float4*>(Uh);
      constexpr int Q = 5 * NP / 4, KQ = (Q + kThreads - 1) / kThreads, KB = 8;
#pragma unroll
      for (int k0 = 0; k0 < KQ; k0 += KB) {
        float4 v[KB];
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          const int q = tid + (k0 + k) * kThreads;
          if (k0 + k < KQ && q < Q) v[k] = __ldg(src + q);
        }
#pragma unroll
        for (int k = 0; k < KB; ++k) {
          const int q = tid + (k0 + k) * kThreads;
          if (k0 + k < KQ && q < Q) dst[q] = v[k];
        }
      }
    } else {
      for (int q = tid; q < 5 * NP; q += kThreads) Uh[q] = L.x32[off + q];
    }
  }
  // the unscaled split of D in the packed layout: (A, B) pairs, then for odd
  // N the middle column and the middle row; hi and lo FP32 parts
  for (int q = tid; q < TAB; q += kThreads) {
    constexpr int h = N / 2;
    double v;
    if (q < 2 * h * h) {
      const int pr = q >> 1, i = pr / h, j = pr - (pr / h) * h;
      v = (q & 1) ? L.eo.B[i][j] : L.eo.A[i][j];
    } else if (q < 2 * h * h + h) {
      v = L.eo.M[q - 2 * h * h];
    } else {
      v = L.eo.B[h][q - 2 * h * h - h];
    }
    const float hv = (float)v;
    th[q] = hv;
    tl[q] = (float)(v - (double)hv);
  }
  const float* T = L.T + e * (int64_t)kCswT * NP;
  const float g1 = L.gamma1, g2 = L.gamma2;
  __syncthreads();

  // UpwindPenalty corrections of the internal faces, one thread per face
  // point: they need only the jumps of the state across the face, so their
  // gathers of the exterior values are issued here, all at once, rather than
  // point by point after the derivative rounds
  for (int fp = tid; fp < (L.internal ? 6 * NN : 0); fp += kThreads) {
    const int dir = fp / NN, q = fp - (fp / NN) * NN, d = dir >> 1;
    const int sl = (dir & 1) ? N - 1 : 0, fa = q % N, fb = q / N;
    const int p = d == 0 ? sl + N * (fa + N * fb)
                         : (d == 1 ? fa + N * (sl + N * fb) : fa + N * (fb + N * sl));
    const int64_t ef = e * 6 + dir;
    const int32_t x = L.X[ef * NN + q];
    float corr[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (x >= 0) {
      const float* f = L.F + ef * kCswF * NN + q;
      // jumps d = exterior - interior
      float dv[5];
#pragma unroll
      for (int v = 0; v < 5; ++v) {
        if (COMP) {
          float eh, el;
          dev::split_df(L.x64[x + (int64_t)v * NP], eh, el);
          dv[v] = (eh - Uh[v * NP + p]) + (el - Ul[v * NP + p]);
        } else {
          dv[v] = L.x32[x + (int64_t)v * NP] - Uh[v * NP + p];
        }
      }
      float ndp = 0.0f;
#pragma unroll
      for (int c = 0; c < 3; ++c) ndp = fmaf(f[(kFv + c) * NN], dv[2 + c], ndp);
      const float m0 = f[(kFm + 0) * NN], m1 = f[(kFm + 1) * NN];
      const float m2 = f[(kFm + 2) * NN], m3 = f[(kFm + 3) * NN];
      const float g2p = g2 * dv[0];
      const float t1 = m3 * (dv[1] - ndp - g2p);
      const float t2 = -m2 * (dv[1] + ndp - g2p);
      const float cpsi = m0 * dv[0];
      corr[0] = cpsi;
      corr[1] = fmaf(g2, cpsi, 0.5f * (t1 - t2));
      const float hh = -0.5f * (t1 + t2);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float nc = f[(kFn + c) * NN];
        corr[2 + c] = fmaf(hh, nc, m1 * fmaf(-nc, ndp, dv[2 + c]));
      }
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) Cf[(dir * 5 + v) * NN + q] = corr[v];
  }

  float acc[PTS][5];
#pragma unroll
  for (int r = 0; r < PTS; ++r)
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[r][v] = 0.0f;

#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    // this round's coefficients (B^a, G^a., A_a.) for the owned points are
    // loaded before the derivative work, which then hides their latency
    float cf[PTS][7];
#pragma unroll
    for (int r = 0; r < PTS; ++r) {
      const int p = tid + r * kThreads;
      if (p < NP) {
        cf[r][0] = __ldg(T + (kTB + a) * NP + p);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          cf[r][1 + j] = __ldg(T + (kTG + 3 * a + j) * NP + p);
          cf[r][4 + j] = __ldg(T + (kTA + 3 * a + j) * NP + p);
        }
      }
    }
    __syncthreads();
    for (int task = tid; task < 5 * NN; task += kThreads) {
      const int v = task / NN, line = task - v * NN;
      int base, stride;
      line_geometry<N>(a, line, base, stride);
      float uh[N], du[N];
#pragma unroll
      for (int i = 0; i < N; ++i) uh[i] = Uh[v * NP + base + i * stride];
      if (COMP) {
        float ul[N];
#pragma unroll
        for (int i = 0; i < N; ++i) ul[i] = Ul[v * NP + base + i * stride];
        pipe::eo_line_pdfg<N>(uh, ul, du, th, tl);
      } else {
        pipe::eo_line_pg<N>(uh, du, th);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) Ga[v * NP + base + i * stride] = du[i];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PTS; ++r) {
      const int p = tid + r * kThreads;
      if (p < NP) {
        const float gpsi = Ga[p], gpi = Ga[NP + p];
        const float gf[3] = {Ga[2 * NP + p], Ga[3 * NP + p], Ga[4 * NP + p]};
        const float B = cf[r][0];
        acc[r][0] = fmaf(B, gpsi, acc[r][0]);
        float s = B * fmaf(g1 * g2, gpsi, gpi);
#pragma unroll
        for (int j = 0; j < 3; ++j) s = fmaf(-cf[r][1 + j], gf[j], s);
        acc[r][1] += s;
        const float hh = fmaf(g2, gpsi, -gpi);
#pragma unroll
        for (int i = 0; i < 3; ++i)
          acc[r][2 + i] = fmaf(cf[r][4 + i], hh, fmaf(B, gf[i], acc[r][2 + i]));
        if (outer && p >= NP - NN) {
          const int q = p - (NP - NN);
          Go[(4 * a + 0) * NN + q] = gpsi;
#pragma unroll
          for (int j = 0; j < 3; ++j) Go[(4 * a + 1 + j) * NN + q] = gf[j];
        }
      }
    }
  }
  __syncthreads();

#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int p = tid + r * kThreads;
    if (p >= NP) continue;
    float ui[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) ui[v] = COMP ? Uh[v * NP + p] + Ul[v * NP + p] : Uh[v * NP + p];
    const float psi = ui[0], pi = ui[1];
    const float phi[3] = {ui[2], ui[3], ui[4]};
    const float lapse = T[kTLapse * NP + p];
    float dt[5];
    float bphi = 0.0f;
    if (g1 != 0.0f)
      for (int i = 0; i < 3; ++i) bphi = fmaf(T[(kTBeta + i) * NP + p], phi[i], bphi);
    dt[0] = fmaf(-g1, bphi, fmaf(1.0f + g1, acc[r][0], -lapse * pi));
    float s = fmaf(T[kTK * NP + p], pi, acc[r][1]);
    for (int i = 0; i < 3; ++i) s = fmaf(T[(kTC + i) * NP + p], phi[i], s);
    dt[1] = fmaf(-g1 * g2, bphi, s);
    for (int i = 0; i < 3; ++i) {
      float v = fmaf(-g2 * lapse, phi[i], acc[r][2 + i]);
      v = fmaf(-pi, T[(kTDl + i) * NP + p], v);
      for (int j = 0; j < 3; ++j) v = fmaf(T[(kTDs + 3 * i + j) * NP + p], phi[j], v);
      dt[2 + i] = v;
    }
    const int i = p % N, j = (p / N) % N, k = p / NN;
    float corr[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const int dirs[6] = {i == 0 ? 0 : -1, i == N - 1 ? 1 : -1, j == 0 ? 2 : -1,
                         j == N - 1 ? 3 : -1, k == 0 ? 4 : -1, k == N - 1 ? 5 : -1};
    const int fq[3] = {j + N * k, i + N * k, i + N * j};
#pragma unroll
    for (int s6 = 0; s6 < 6; ++s6) {
      const int dir = dirs[s6];
      if (dir < 0) continue;
      const int q = fq[dir >> 1];
      const int64_t ef = e * 6 + dir;
      if (L.internal) {
#pragma unroll
        for (int v = 0; v < 5; ++v) corr[v] += Cf[(dir * 5 + v) * NN + q];
      }
      if (dir == 5 && outer) {
        // ConstraintPreservingSphericalRadiation from the volume dt
        const float* f = L.F + ef * kCswF * NN + q;
        const double* J = L.ij + e * 9 * (int64_t)NP + p;
        float dpsi[3], dphi[3][3];
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) {
          float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const float Jai = (float)J[(3 * a + ii) * NP];
            s0 = fmaf(Jai, Go[(4 * a + 0) * NN + q], s0);
            s1 = fmaf(Jai, Go[(4 * a + 1) * NN + q], s1);
            s2 = fmaf(Jai, Go[(4 * a + 2) * NN + q], s2);
            s3 = fmaf(Jai, Go[(4 * a + 3) * NN + q], s3);
          }
          dpsi[ii] = s0;
          dphi[ii][0] = s1;
          dphi[ii][1] = s2;
          dphi[ii][2] = s3;
        }
        const double* X3 = L.xyz + e * 3 * (int64_t)NP + p;
        const float rr = (float)sqrt(X3[0] * X3[0] + X3[NP] * X3[NP] + X3[2 * NP] * X3[2 * NP]);
        const float ir = 1.0f / rr;
        float nv[3], nc[3], beta[3], bn = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          nv[c] = f[(kFv + c) * NN];
          nc[c] = f[(kFn + c) * NN];
          beta[c] = T[(kTBeta + c) * NP + p];
          bn = fmaf(beta[c], nc[c], bn);
        }
        const float l0 = fminf(-(1.0f + g1) * bn, 0.0f), l1 = fminf(-bn, 0.0f);
        float cpsi = 0.0f;
#pragma unroll
        for (int c = 0; c < 3; ++c) cpsi = fmaf(nv[c], dpsi[c] - phi[c], cpsi);
        cpsi *= l0;
        corr[0] += cpsi;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float v = 0.0f;
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) v = fmaf(nv[jj], dphi[jj][c] - dphi[c][jj], v);
          corr[2 + c] += l1 * v;
        }
        float cpi = fmaf(2.0f * ir, psi, 4.0f * dt[0]) * ir;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          cpi = fmaf(nv[c], fmaf(2.0f, dt[2 + c], 4.0f * ir * phi[c]), cpi);
          cpi = fmaf(beta[c], dt[2 + c], cpi);
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) cpi = fmaf(nv[c] * nv[jj], dphi[c][jj], cpi);
        }
        cpi /= lapse;
        corr[1] += fmaf(g2, cpsi, cpi - dt[1]);
      }
    }
    const float al = (float)L.alpha, be = (float)L.beta, cc = (float)L.c;
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const int64_t o = off + v * NP + p;
      float w = cc * (dt[v] + corr[v]);
      if (L.alpha != 0.0) w = fmaf(al, ui[v], w);
      if (L.y32) w = fmaf(be, L.y32[o], w);
      if (L.w32) L.w32[o] = w;
      if (L.out64) L.out64[o] = L.base64 ? L.base64[o] + dev::widen(w) : dev::widen(w);
    }
  }
}

template <int N, bool COMP, int V>
cudaError_t launch_shape_n(const CswMixedLaunch& L, cudaStream_t s) {
  constexpr int T = shape_threads<V>();
  const size_t smem = (size_t)CmShape<N, COMP, T>::SMEM * sizeof(float);
  auto k = csw_stage_mixed_kernel<N, COMP, T, shape_min_blocks<N, COMP, V>()>;
  cudaError_t err =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  const int64_t blocks = L.list ? L.list_count : L.n_elem;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, T, smem, s>>>(L);
  return cudaGetLastError();
}

// every extent of one launch shape (instantiated once per translation unit)
template <int V>
cudaError_t launch_shape(const CswMixedLaunch& L, cudaStream_t s) {
  const bool c = L.x64 != nullptr;
  switch (L.n) {
#define DGSW_CSW_MIXED_CASE(n) \
  case n: return c ? launch_shape_n<n, true, V>(L, s) : launch_shape_n<n, false, V>(L, s);
    DGSW_CSW_MIXED_CASE(2)
    DGSW_CSW_MIXED_CASE(3)
    DGSW_CSW_MIXED_CASE(4)
    DGSW_CSW_MIXED_CASE(5)
    DGSW_CSW_MIXED_CASE(6)
    DGSW_CSW_MIXED_CASE(7)
    DGSW_CSW_MIXED_CASE(8)
    DGSW_CSW_MIXED_CASE(9)
    DGSW_CSW_MIXED_CASE(10)
    DGSW_CSW_MIXED_CASE(11)
    DGSW_CSW_MIXED_CASE(12)
#undef DGSW_CSW_MIXED_CASE
    default: return cudaErrorInvalidValue;
  }
}

// defined in the shape's translation unit
cudaError_t launch_shape0(const CswMixedLaunch& L, cudaStream_t s);
cudaError_t launch_shape1(const CswMixedLaunch& L, cudaStream_t s);
cudaError_t launch_shape2(const CswMixedLaunch& L, cudaStream_t s);

}  // namespace csw_mixed
}  // namespace dgsw
