// stage_mixed_pipe.cu -- persistent, TMA-pipelined mixed-precision DG stage
// for even LGL extents N (element blocks are multiples of 16 bytes).
//
// Same arithmetic as stage_mixed.cu (W = alpha X + beta Y + c L(X), see the
// header comment there for the incremental SSP-RK3 form and the double-float
// first stage), restructured so that HBM latency is hidden:
//  - a persistent grid; each CTA walks groups of EPB elements;
//  - each element's contiguous blocks (X, and Y / base64 when present) are
//    staged into shared memory by TMA bulk copies (cp.async.bulk, completion
//    on an mbarrier), double-buffered: the next group's copies are in flight
//    while the current group computes;
//  - the 12 neighbour face values each thread needs are prefetched for the
//    next group with cp.async into the same double buffer;
//  - the contractions use Blackwell's packed FP32 instructions (FFMA2 /
//    FADD2 / FMUL2), the even and odd halves of the split D in the two lanes.
// Every mbarrier wait is bounded by a wall-clock limit; on timeout the
// kernel records an error word the host reads and returns.
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"
#include "pipe.cuh"

namespace dgsw {
namespace {

using namespace pipe;

using dev::split_df;
using dev::two_sum;
using dev::widen;

// ---------------------------------------------------------------- geometry
template <int N>
struct P {
  static constexpr int h = N / 2;
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB2 = h * h;  // float2 (A, B) pairs per direction
};

constexpr int round128(int b) { return (b + 127) / 128 * 128; }

// Shared-memory layout of one element slot (bytes).  Every region starts on a
// 128-byte boundary (TMA destinations must be 16-byte aligned).
template <int N, bool COMP, bool HAS_Y, bool HAS_B>
struct Lay {
  using S = P<N>;
  static constexpr int kX = round128(COMP ? 4 * S::NP * 8 : 5 * S::NP * 4);  // staged X
  static constexpr int kY = HAS_Y ? round128(5 * S::NP * 4) : 0;
  static constexpr int kB = HAS_B ? round128(5 * S::NP * 8) : 0;
  static constexpr int kFace = round128(12 * S::NN * (COMP ? 8 : 4));  // 3 dirs x 2 sides x 2
  static constexpr int kBuf = kX + kY + kB + kFace;  // one pipeline buffer
  static constexpr int kHiLo = 0;  // the double-float split is done as values are read
  static constexpr int kS = round128(S::NP * 4);
  static constexpr int kTab = 128;  // per axis: lift factor G and derivative scale F
  static constexpr int kSlot = 2 * kBuf + kHiLo + kS + kTab;  // two pipeline buffers
  static constexpr int kSlot1 = kBuf + kHiLo + kS + kTab;     // one
  // bytes the TMA copies of one element move (unpadded)
  static constexpr uint32_t kXBytes = COMP ? 4 * S::NP * 8 : 5 * S::NP * 4;
  static constexpr uint32_t kYBytes = HAS_Y ? 5 * S::NP * 4 : 0;
  static constexpr uint32_t kBBytes = HAS_B ? 5 * S::NP * 8 : 0;
};

// A contiguous row of N floats (an x line; N even, the row 8-byte aligned,
// 16-byte aligned when N % 4 == 0) moved with the widest vector accesses:
// neighbouring threads' x lines are N floats apart, so scalar accesses
// would conflict on the shared-memory banks N-fold.
template <int N, typename P>
__device__ __forceinline__ void load_row(const P* p, float (&x)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int k = 0; k < N / 4; ++k) {
      const float4 v = reinterpret_cast<const float4*>(p)[k];
      x[4 * k] = v.x;
      x[4 * k + 1] = v.y;
      x[4 * k + 2] = v.z;
      x[4 * k + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < N / 2; ++k) {
      const float2 v = reinterpret_cast<const float2*>(p)[k];
      x[2 * k] = v.x;
      x[2 * k + 1] = v.y;
    }
  }
}
template <int N, typename P>
__device__ __forceinline__ void store_row(P* p, const float (&x)[N]) {
  if constexpr (N % 4 == 0) {
#pragma unroll
    for (int k = 0; k < N / 4; ++k)
      reinterpret_cast<float4*>(p)[k] = make_float4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < N / 2; ++k) reinterpret_cast<float2*>(p)[k] = make_float2(x[2 * k], x[2 * k + 1]);
  }
}
// a contiguous row of N (hi, lo) pairs, two pairs per 16-byte access
template <int N>
__device__ __forceinline__ void load_row2(const float2* p, float (&h)[N], float (&l)[N]) {
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    const float4 v = reinterpret_cast<const float4*>(p)[k];
    h[2 * k] = v.x;
    l[2 * k] = v.y;
    h[2 * k + 1] = v.z;
    l[2 * k + 1] = v.w;
  }
}

// packed even/odd contraction, plain FP32 (lanes: x = even part P, y = odd Q)
template <int N>
__device__ __forceinline__ void eo_line_p(const float (&x)[N], float (&out)[N],
                                          const float2* __restrict__ tab) {
  constexpr int h = N / 2;
  float2 eo[h];
#pragma unroll
  for (int j = 0; j < h; ++j) eo[j] = make_float2(x[j] + x[N - 1 - j], x[j] - x[N - 1 - j]);
#pragma unroll
  for (int i = 0; i < h; ++i) {
    float2 acc = mul2(tab[i * h], eo[0]);
#pragma unroll
    for (int j = 1; j < h; ++j) acc = fma2(tab[i * h + j], eo[j], acc);
    out[i] = acc.x + acc.y;
    out[N - 1 - i] = acc.y - acc.x;
  }
}

// packed compensated contraction of a double-float line
template <int N>
__device__ __forceinline__ void eo_line_pdf(const float (&xh)[N], const float (&xl)[N],
                                            float (&out)[N], const float2* __restrict__ th,
                                            const float2* __restrict__ tl) {
  constexpr int h = N / 2;
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
    // s: running sum of the products' high parts; the corrections are three
    // independent sums (rounding errors of s and of the products; the
    // table's low parts; the data's low parts), added at the end
    float2 s = mul2(th[i * h], eoh[0]);
    float2 c1 = fma2(th[i * h], eoh[0], neg2(s));
    float2 c2 = mul2(tl[i * h], eoh[0]);
    float2 c3 = mul2(th[i * h], eol[0]);
#pragma unroll
    for (int j = 1; j < h; ++j) {
      const float2 a = th[i * h + j];
      const float2 p = mul2(a, eoh[j]);
      const float2 pe = fma2(a, eoh[j], neg2(p));
      float2 t;
      two_sum2(s, p, s, t);
      c1 = add2(c1, add2(t, pe));
      c2 = fma2(tl[i * h + j], eoh[j], c2);
      c3 = fma2(a, eol[j], c3);
    }
    const float2 c = add2(c1, add2(c2, c3));
    // lanes: x = P_i (even part), y = Q_i (odd part)
    out[i] = (s.x + s.y) + (c.x + c.y);
    out[N - 1 - i] = (s.y - s.x) + (c.y - c.x);
  }
}

// STAGES pipeline buffers per element slot (2: the next group's copies land
// while this one computes; 1: they are issued when this one is done, and the
// other resident CTAs -- MINB asked of the register allocator -- cover the
// wait).
// ACC (FP32 stages with Y, no staged base): W is written in place into the
// staged X (each line's values are read into registers before its outputs
// land, and the pointwise reads of X and Y at a point precede its write),
// then one coalesced pass over the element's contiguous block forms
// out64 = base64 + W in FP64 with 16-byte loads and stores.
template <int N, int EPB, bool COMP, bool HAS_Y, bool HAS_B, int STAGES, int MINB,
          bool ACC = false>
__global__ void __launch_bounds__(N * N * EPB, MINB)
    stage_mixed_pipe_kernel(MixedLaunch L, int64_t n_groups) {
  static_assert(!ACC || (!COMP && HAS_Y && !HAS_B), "the fused accumulate is the last stage's");
  using S = P<N>;
  using Y = Lay<N, COMP, HAS_Y, HAS_B>;
  constexpr int NN = S::NN, NP = S::NP, h = S::h, TAB2 = S::TAB2;
  constexpr int64_t VS = (int64_t)kVars * NP;
  using FT = typename std::conditional<COMP, double, float>::type;  // staged field type

  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ uint64_t bars[2];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  constexpr int kSlotBytes = STAGES == 2 ? Y::kSlot : Y::kSlot1;
  unsigned char* slot_base = smem_raw + (size_t)slot * kSlotBytes;
  unsigned char* bufs[2] = {slot_base, slot_base + (STAGES - 1) * Y::kBuf};
  float* Sacc = reinterpret_cast<float*>(slot_base + STAGES * Y::kBuf + Y::kHiLo);
  float* GF = reinterpret_cast<float*>(slot_base + STAGES * Y::kBuf + Y::kHiLo + Y::kS);
  // the unscaled split of D as (A, B) pairs, hi then lo, once per CTA; each
  // element's -c dxi/dx scales the contractions' results per axis
  __shared__ float2 s_tab[2 * TAB2];
  const int ta = t % N, tb = t / N;
  const uint64_t kLimitNs = 2000000000ull;  // 2 s per wait

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  for (int q = threadIdx.x; q < TAB2; q += blockDim.x) {
    const int i = q / h, j = q - (q / h) * h;
    const double va = L.eo.A[i][j], vb = L.eo.B[i][j];
    const float ah = __double2float_rn(va), bh = __double2float_rn(vb);
    s_tab[q] = make_float2(ah, bh);
    s_tab[TAB2 + q] =
        make_float2(__double2float_rn(va - (double)ah), __double2float_rn(vb - (double)bh));
  }
  __syncthreads();

  // issue the TMA copies of group g into buffer b (one thread)
  auto issue_group = [&](int64_t g, int b) {
    uint32_t bytes = 0;
    for (int s = 0; s < EPB; ++s) {
      const int64_t e = g * EPB + s;
      if (e >= L.n_elem) break;
      bytes += Y::kXBytes + Y::kYBytes + Y::kBBytes;
    }
    if (bytes == 0) return;
    fence_proxy_async_smem();
    mbar_arrive_expect_tx(&bars[b], bytes);
    for (int s = 0; s < EPB; ++s) {
      const int64_t e = g * EPB + s;
      if (e >= L.n_elem) break;
      unsigned char* dst = smem_raw + (size_t)s * kSlotBytes + (size_t)b * Y::kBuf;
      if (COMP)
        bulk_g2s(dst, L.x64 + e * VS + NP, Y::kXBytes, &bars[b]);
      else
        bulk_g2s(dst, L.x32 + e * VS, Y::kXBytes, &bars[b]);
      if (HAS_Y) bulk_g2s(dst + Y::kX, L.y32 + e * VS, Y::kYBytes, &bars[b]);
      if (HAS_B) bulk_g2s(dst + Y::kX + Y::kY, L.base64 + e * VS, Y::kBBytes, &bars[b]);
    }
  };
  // prefetch this thread's 12 neighbour face values of element e into buffer b
  auto issue_faces = [&](int64_t e, int b) {
    if (e >= L.n_elem) return;
    FT* face = reinterpret_cast<FT*>(bufs[b] + Y::kX + Y::kY + Y::kB);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
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
      const int64_t nlo = (int64_t)L.nbr[6 * e + 2 * d] * VS;
      const int64_t nhi = (int64_t)L.nbr[6 * e + 2 * d + 1] * VS;
      const int lo_pt = base + (N - 1) * stride, hi_pt = base;
      const FT* src = COMP ? reinterpret_cast<const FT*>(L.x64) : reinterpret_cast<const FT*>(L.x32);
      FT* f = face + (4 * d) * NN + t;
      cp_async<sizeof(FT)>(f, src + nlo + NP + lo_pt);
      cp_async<sizeof(FT)>(f + NN, src + nlo + (2 + d) * NP + lo_pt);
      cp_async<sizeof(FT)>(f + 2 * NN, src + nhi + NP + hi_pt);
      cp_async<sizeof(FT)>(f + 3 * NN, src + nhi + (2 + d) * NP + hi_pt);
    }
  };

  const int64_t G = gridDim.x;
  int64_t g = blockIdx.x;
  if (g < n_groups) {
    if (threadIdx.x == 0) issue_group(g, 0);
    issue_faces(g * EPB + slot, 0);
    cp_async_commit();
  }
  const float alpha = (float)L.alpha, beta = (float)L.beta, cf = (float)L.c;
  for (int k = 0; g < n_groups; ++k, g += G) {
    const int b = STAGES == 2 ? (k & 1) : 0;
    const uint32_t parity = STAGES == 2 ? (uint32_t)((k >> 1) & 1) : (uint32_t)(k & 1);
    const int64_t gn = g + G;
    const int64_t e = g * EPB + slot;
    const bool active = e < L.n_elem;
    if (STAGES == 2 && threadIdx.x == 0 && gn < n_groups) issue_group(gn, b ^ 1);
    // the element's lift factors and derivative scales per axis
    if (active && t < 3) {
      const double jd = L.jac[3 * e + t];
      GF[t] = (float)(-0.25 * L.c * (double)(N * (N - 1)) * jd);
      GF[3 + t] = (float)(-L.c * jd);
    }
    const bool landed = mbar_wait(&bars[b], parity, kLimitNs);
    cp_async_wait_all();
    if (__syncthreads_or(!landed)) {
      // a copy did not land in time: record it, give copies still in flight
      // one more bounded wait, and leave together
      if (threadIdx.x == 0 && L.err) atomicExch(L.err, 1);
      if (!landed) mbar_wait(&bars[b], parity, kLimitNs);
      if (STAGES == 2 && threadIdx.x == 0 && gn < n_groups)
        mbar_wait(&bars[b ^ 1], (uint32_t)(((k + 1) >> 1) & 1), kLimitNs);
      return;
    }
    const unsigned char* buf = bufs[b];
    float* Xw = reinterpret_cast<float*>(bufs[b]);  // W in place (ACC)
    if (COMP) {
      // each FP64 value of the staged X becomes its (hi, lo) FP32 pair in
      // place, so that the passes split each value once
      if (active) {
        double* Xs = reinterpret_cast<double*>(bufs[b]);
        for (int q = t; q < 4 * NP; q += NN) {
          float hi, lo;
          split_df(Xs[q], hi, lo);
          reinterpret_cast<float2*>(Xs)[q] = make_float2(hi, lo);
        }
      }
      __syncthreads();
    }
    const FT* X = reinterpret_cast<const FT*>(buf);
    const float2* X2 = reinterpret_cast<const float2*>(buf);
    const float* Yb = reinterpret_cast<const float*>(buf + Y::kX);
    const double* Bb = reinterpret_cast<const double*>(buf + Y::kX + Y::kY);
    const FT* face = reinterpret_cast<const FT*>(buf + Y::kX + Y::kY + Y::kB);

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
        const float2* th = s_tab;
        const float2* tl = s_tab + TAB2;
        const float Fd = GF[3 + d];
        float dF[N], dP[N], pih[N], fh[N];
        float pil[N], fl[N];
        if (COMP) {
          // X holds Pi, Phi_x, Phi_y, Phi_z as (hi, lo) FP32 pairs
          if (d == 0) {
            load_row2<N>(X2 + base, pih, pil);
            load_row2<N>(X2 + NP + base, fh, fl);
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const float2 vp = X2[base + i * stride], vf = X2[(1 + d) * NP + base + i * stride];
              pih[i] = vp.x;
              pil[i] = vp.y;
              fh[i] = vf.x;
              fl[i] = vf.y;
            }
          }
          eo_line_pdf<N>(fh, fl, dF, th, tl);
          eo_line_pdf<N>(pih, pil, dP, th, tl);
#pragma unroll
          for (int i = 0; i < N; ++i) {
            dF[i] *= Fd;
            dP[i] *= Fd;
          }
        } else {
          if (d == 0) {
            load_row<N>(X + NP + base, pih);
            load_row<N>(X + 2 * NP + base, fh);
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              pih[i] = X[NP + base + i * stride];
              fh[i] = X[(2 + d) * NP + base + i * stride];
            }
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            pil[i] = 0.0f;
            fl[i] = 0.0f;
          }
          eo_line_p<N>(fh, dF, th);
          eo_line_p<N>(pih, dP, th);
#pragma unroll
          for (int i = 0; i < N; ++i) {
            dF[i] *= Fd;
            dP[i] *= Fd;
          }
        }
        // UpwindPenalty corrections at both ends of the line (see stage_mixed.cu)
        const float G2 = GF[d];
        const FT* fc = face + (4 * d) * NN + t;
        float dw_lo, dw_hi;
        if (COMP) {
          float ph, pl, qh, ql, wih, wil, weh, wel, t1, dh;
          split_df((double)fc[0], ph, pl);
          split_df((double)fc[NN], qh, ql);
          two_sum(pih[0], fh[0], wih, t1);
          wil = t1 + (pil[0] + fl[0]);
          two_sum(ph, qh, weh, t1);
          wel = t1 + (pl + ql);
          two_sum(wih, -weh, dh, t1);
          dw_lo = dh + (t1 + (wil - wel));
          split_df((double)fc[2 * NN], ph, pl);
          split_df((double)fc[3 * NN], qh, ql);
          two_sum(pih[N - 1], -fh[N - 1], wih, t1);
          wil = t1 + (pil[N - 1] - fl[N - 1]);
          two_sum(ph, -qh, weh, t1);
          wel = t1 + (pl - ql);
          two_sum(wih, -weh, dh, t1);
          dw_hi = dh + (t1 + (wil - wel));
        } else {
          dw_lo = (pih[0] + fh[0]) - ((float)fc[0] + (float)fc[NN]);
          dw_hi = (pih[N - 1] - fh[N - 1]) - ((float)fc[2 * NN] - (float)fc[3 * NN]);
        }
        dF[0] = fmaf(G2, dw_lo, dF[0]);
        dP[0] = fmaf(G2, dw_lo, dP[0]);
        dF[N - 1] = fmaf(G2, dw_hi, dF[N - 1]);
        dP[N - 1] = fmaf(-G2, dw_hi, dP[N - 1]);
        // Phi_d output
        const int64_t vo = e * VS + (2 + d) * NP + base;
        float yv[N];
        if (!COMP && HAS_Y) {
          if (d == 0) {
            load_row<N>(Yb + 2 * NP + base, yv);
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) yv[i] = Yb[(2 + d) * NP + base + i * stride];
          }
        }
        float wv[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float w = dP[i];
          if (!COMP) {
            w = fmaf(alpha, fh[i], w);
            if (HAS_Y) w = fmaf(beta, yv[i], w);
          }
          wv[i] = w;
        }
        if (ACC) {
          if (d == 0) {
            store_row<N>(Xw + 2 * NP + base, wv);
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) Xw[(2 + d) * NP + base + i * stride] = wv[i];
          }
        } else {
          if (L.w32) {
            if (d == 0) {
              store_row<N>(L.w32 + vo, wv);
            } else {
#pragma unroll
              for (int i = 0; i < N; ++i) L.w32[vo + i * stride] = wv[i];
            }
          }
          if (L.out64) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              if (HAS_B)
                L.out64[vo + i * stride] = Bb[(2 + d) * NP + base + i * stride] + widen(wv[i]);
              else
                L.out64[vo + i * stride] = widen(wv[i]);
            }
          }
        }
        if (d < 2) {
          if (d == 0) {
            store_row<N>(Sacc + base, dF);
          } else {
#pragma unroll
            for (int i = 0; i < N; ++i) Sacc[base + i * stride] += dF[i];
          }
        } else {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int p = base + i * stride;
            float wpi = Sacc[p] + dF[i];
            float wpsi = COMP ? fmaf(-cf, pih[i], -cf * pil[i]) : -cf * pih[i];
            if (!COMP) {
              wpi = fmaf(alpha, pih[i], wpi);
              wpsi = fmaf(alpha, X[p], wpsi);
              if (HAS_Y) {
                wpi = fmaf(beta, Yb[NP + p], wpi);
                wpsi = fmaf(beta, Yb[p], wpsi);
              }
            }
            if (ACC) {
              Xw[NP + p] = wpi;
              Xw[p] = wpsi;
              continue;
            }
            if (L.w32) {
              L.w32[e * VS + NP + p] = wpi;
              L.w32[e * VS + p] = wpsi;
            }
            if (L.out64) {
              if (HAS_B) {
                L.out64[e * VS + NP + p] = Bb[NP + p] + widen(wpi);
                L.out64[e * VS + p] = Bb[p] + widen(wpsi);
              } else {
                L.out64[e * VS + NP + p] = widen(wpi);
                L.out64[e * VS + p] = widen(wpsi);
              }
            }
          }
        }
      }
      if (d < 2) __syncthreads();
    }
    if (ACC) {
      // out64 = base64 + W over the element's contiguous block: 4 values per
      // thread and step, KB steps' loads issued before their stores (out64
      // may alias base64; every value is read and written by one thread)
      __syncthreads();
      if (active) {
        constexpr int Q4 = kVars * NP / 4, KB = N == 8 ? 5 : 3;
        const float4* W4 = reinterpret_cast<const float4*>(bufs[b]);
        const double2* B2 = reinterpret_cast<const double2*>(L.base64 + e * VS);
        double2* O2 = reinterpret_cast<double2*>(L.out64 + e * VS);
#pragma unroll 1
        for (int q0 = t; q0 < Q4; q0 += KB * NN) {
          double2 lo[KB], hi[KB];
#pragma unroll
          for (int k2 = 0; k2 < KB; ++k2) {
            const int q = q0 + k2 * NN;
            if (q < Q4) {
              lo[k2] = B2[2 * q];
              hi[k2] = B2[2 * q + 1];
            }
          }
#pragma unroll
          for (int k2 = 0; k2 < KB; ++k2) {
            const int q = q0 + k2 * NN;
            if (q < Q4) {
              const float4 w = W4[q];
              O2[2 * q] = make_double2(lo[k2].x + widen(w.x), lo[k2].y + widen(w.y));
              O2[2 * q + 1] = make_double2(hi[k2].x + widen(w.z), hi[k2].y + widen(w.w));
            }
          }
        }
      }
    }
    // neighbour faces of the next group, then release this buffer (the
    // in-place split wrote it: order those generic writes before the next
    // TMA writes into it)
    if (STAGES == 2) {
      if (gn < n_groups) issue_faces(gn * EPB + slot, b ^ 1);
      cp_async_commit();
    }
    if (COMP || ACC) fence_proxy_async_smem();
    __syncthreads();
    if (STAGES == 1 && gn < n_groups) {
      if (threadIdx.x == 0) issue_group(gn, 0);
      issue_faces(gn * EPB + slot, 0);
      cp_async_commit();
    }
  }
  cp_async_wait_all();
}

template <int N>
constexpr int pipe_epb_target() {
  return N <= 4 ? 8 : (N <= 6 ? 4 : 2);
}

// Elements per CTA: the target, reduced until the double-buffered slots fit
// the 227 KB of shared memory a CTA may use; 0 when one slot does not fit.
constexpr int kSmemLimit = 227 * 1024;
template <int N, bool COMP, bool HAS_Y, bool HAS_B>
constexpr int pipe_epb() {
  constexpr int slot = Lay<N, COMP, HAS_Y, HAS_B>::kSlot;
  constexpr int fit = kSmemLimit / slot;
  return fit < pipe_epb_target<N>() ? fit : pipe_epb_target<N>();
}

// Launch shapes: 0 two pipeline buffers, 1 one buffer and MINB = 4 resident
// CTAs asked of the register allocator (the FP32 stages ask for 6).
template <int N, bool COMP, bool HAS_Y, bool HAS_B, int V, bool ACC = false>
cudaError_t launch_pipe_v(const MixedLaunch& L, cudaStream_t s);

template <int N, bool COMP, bool HAS_Y, bool HAS_B>
cudaError_t launch_pipe(const MixedLaunch& L, cudaStream_t s) {
  // the single-buffered shape is compiled for the step's three stages only
  if constexpr (!HAS_B) {
    if (L.variant == 1) return launch_pipe_v<N, COMP, HAS_Y, HAS_B, 1>(L, s);
  }
  return launch_pipe_v<N, COMP, HAS_Y, HAS_B, 0>(L, s);
}

template <int N, bool COMP, bool HAS_Y, bool HAS_B, int V, bool ACC>
cudaError_t launch_pipe_v(const MixedLaunch& L, cudaStream_t s) {
  constexpr int EPB_FIT = pipe_epb<N, COMP, HAS_Y, HAS_B>();
  if (EPB_FIT < 1) return launch_stage_mixed(L, s);  // too large to double-buffer
  constexpr int EPB = EPB_FIT < 1 ? 1 : EPB_FIT;
  constexpr int STAGES = V == 1 ? 1 : 2;
  constexpr int MINB = V == 1 ? (COMP ? 4 : 6) : 1;
  using Y = Lay<N, COMP, HAS_Y, HAS_B>;
  const size_t smem = (size_t)EPB * (STAGES == 2 ? Y::kSlot : Y::kSlot1);
  auto k = stage_mixed_pipe_kernel<N, EPB, COMP, HAS_Y, HAS_B, STAGES, MINB, ACC>;
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0, per_sm = 0;
  if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
  if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return err;
  if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, N * N * EPB, smem)) !=
      cudaSuccess)
    return err;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int64_t groups = (L.n_elem + EPB - 1) / EPB;
  if (groups <= 0) return cudaSuccess;
  int64_t grid = (int64_t)sms * per_sm;
  if (grid > groups) grid = groups;
  k<<<(unsigned)grid, N * N * EPB, smem, s>>>(L, groups);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_pipe_n(const MixedLaunch& L, cudaStream_t s) {
  const bool y = L.y32 != nullptr, bb = L.base64 != nullptr && L.out64 != nullptr;
  if (L.fuse_acc) {
    // the last stage with u0 + W formed in its epilogue
    if (L.x64 || !y || !bb || L.w32) return cudaErrorInvalidValue;
    return L.variant == 1 ? launch_pipe_v<N, false, true, false, 1, true>(L, s)
                          : launch_pipe_v<N, false, true, false, 0, true>(L, s);
  }
  if (L.x64) {
    if (y) return cudaErrorInvalidValue;
    return bb ? launch_pipe<N, true, false, true>(L, s) : launch_pipe<N, true, false, false>(L, s);
  }
  if (y) return bb ? launch_pipe<N, false, true, true>(L, s) : launch_pipe<N, false, true, false>(L, s);
  return bb ? launch_pipe<N, false, false, true>(L, s) : launch_pipe<N, false, false, false>(L, s);
}

}  // namespace

namespace {
// The bounded wait of the pipeline on an mbarrier whose transaction never
// arrives: the wait gives up after limit_ns, the kernel records the error
// word and returns, exactly as the stage kernel does when a copy does not
// land.  Nothing faults and nothing spins without a bound.
__global__ void bounded_wait_check_kernel(int* err, uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool landed = mbar_wait(&bar, 0u, limit_ns);
  if (__syncthreads_or(!landed)) {
    if (threadIdx.x == 0) atomicExch(err, 1);
  }
}
}  // namespace

cudaError_t launch_bounded_wait_check(int* err, uint64_t limit_ns, cudaStream_t s) {
  bounded_wait_check_kernel<<<1, 64, 0, s>>>(err, limit_ns);
  return cudaGetLastError();
}

bool mixed_pipe_supported(int n) { return n % 2 == 0 && n >= 2 && n <= kMaxN; }

cudaError_t launch_stage_mixed_pipe(const MixedLaunch& L, cudaStream_t s) {
  if ((L.x64 == nullptr) == (L.x32 == nullptr)) return cudaErrorInvalidValue;
  switch (L.n) {
    case 2: return launch_pipe_n<2>(L, s);
    case 4: return launch_pipe_n<4>(L, s);
    case 6: return launch_pipe_n<6>(L, s);
    case 8: return launch_pipe_n<8>(L, s);
    case 10: return launch_pipe_n<10>(L, s);
    case 12: return launch_pipe_n<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
