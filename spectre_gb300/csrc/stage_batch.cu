// stage_batch.cu -- one persistent, TMA-pipelined launch per mixed-precision
// SSP-RK3 stage over elements of any LGL extents (many independent
// evolutions with p-nonconforming mortars in one launch).
//
// The operator is the same as in stage_general.cu: the ScalarWave time
// derivative (ScalarWave/TimeDerivative.cpp:37-44) with the UpwindPenalty
// correction (UpwindPenalty.cpp:35-205) lifted onto GLL faces
// (LiftFlux.hpp:41-62).  With char speeds (0, +1, -1) the reference's mortar
// round trip (project both sides to the mortar, dg_boundary_terms, project
// back: ApplyBoundaryCorrections.hpp:880-937, Projection.cpp:56-375) equals
//   D_Pi = (w_int - T w_ext)/2,  D_Phi = -n D_Pi,  w = Pi - n.Phi,
// with T = R_{mortar->face} P_{nbr face->mortar} applied along both face
// dimensions.
//
// Work and data flow (mixed precision, incremental SSP-RK3 of
// stage_mixed.cu: W1 = dt L(u0), W2 = W1/2 + dt/4 L(W1),
// u = u0 + 2/3 (W2 + W1) + 2dt/3 L(W2)):
//  - Tasks: a host-built list of (extent N, g elements of that extent), at
//    most (threads per CTA) / N^2 elements so that one thread owns one grid
//    line of one element in each axis pass.  The launch is persistent: CTA b
//    takes tasks b, b + grid, ...; every extent class runs in the same launch.
//  - Exterior face values are not gathered from the neighbours' volume data.
//    Each stage writes, for every face of every element, the w of its output
//    already mapped by T onto the neighbour's face points, into the
//    neighbour's slot of a compact face buffer ([element][6][N^2], each
//    element's block contiguous).  The next stage then reads an element's six
//    exterior faces as one contiguous block.  For the FP64 state u the face
//    buffer holds double-float (hi, lo) values: it is formed from u by
//    batch_faces_kernel and then kept current by the last stage of every step
//    (faces of u + W = faces of u + T w(W), T linear).
//  - Each task's element blocks (X and the face block) are staged into
//    shared memory by TMA bulk copies completing on an mbarrier; with two
//    pipeline buffers the next task's copies land while the current task
//    computes, with one the other resident CTAs cover the wait.  Element
//    blocks of odd extent start on 8- or 4-byte boundaries; the copy starts at
//    the 16-byte boundary below and reads up to 15 bytes past the block
//    (every buffer the kernel reads is allocated with padding).
//  - The three axis passes write the stage's output W to the FP32 output
//    and in place over X in shared memory (each value is read and
//    overwritten by the one thread that owns its line in that pass); the
//    warps then form the next stage's face values from it.  The FP64 state
//    is updated once per step by a streaming kernel (u0 + W3 + 2/3 W1, FP64
//    add), which also adds the last stage's face values to the state's.
//  - Arithmetic: FP32 with the even/odd split of D in the two lanes of packed
//    FFMA2; the first stage differentiates the FP64 state as double-float
//    (hi + lo FP32 pairs formed once per value in shared memory, compensated
//    products and sums).
// Every mbarrier wait is bounded (2 s of wall clock); a wait that gives up
// sets the device error word and the CTA returns.
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "dg_device.cuh"
#include "host_setup.hpp"
#include "launch.hpp"
#include "eo_packed.cuh"
#include "pipe.cuh"

namespace dgsw {
namespace {

using namespace pipe;
using dev::dot2_first;
using dev::dot2_term;
using dev::split_df;
using dev::sub_g2psi;
using dev::two_sum;
using dev::widen;

constexpr uint64_t kLimitNs = 2000000000ull;  // 2 s per bounded wait

// ------------------------------------------------------------ split tables
// The unscaled split tables of every extent 2..12, one after another (the
// hi parts, then the lo parts at kTabTotal): held once per CTA in shared
// memory; the element's -c dxi/dx of each axis scales the contraction's
// result instead.
__host__ __device__ constexpr int tab_offset(int n) {
  int o = 0;
  for (int k = kMinN; k < n; ++k) o += tab_stride(k);
  return o;
}
constexpr int kTabTotal = tab_offset(kMaxN + 1);

// --------------------------------------------------------- buffer layout
// Bytes of one element's X block, its face block, and their shared-memory
// slots (room for the 16-byte alignment shift of the copy).
// (COMP stages X's FP64 Pi and Phi -- and Psi too when gamma2 != 0, G2)
__host__ __device__ constexpr int x_bytes(int n, bool comp, bool g2 = false) {
  return comp ? (g2 ? 5 : 4) * 8 * n * n * n : 5 * 4 * n * n * n;
}
__host__ __device__ constexpr int f_bytes(int n, bool comp) {
  return comp ? 6 * 8 * n * n : (6 * 4 * n * n + 15) / 16 * 16;
}
__host__ __device__ constexpr int round128(int b) { return (b + 127) / 128 * 128; }
__host__ __device__ constexpr int x_slot(int n, bool comp, bool g2 = false) {
  return round128(x_bytes(n, comp, g2) + 32);
}
__host__ __device__ constexpr int f_slot(int n, bool comp) { return round128(f_bytes(n, comp) + 32); }
// elements per task of extent n with bt threads per CTA (one per grid line)
__host__ __device__ constexpr int task_g(int n, int bt) { return bt / (n * n); }

// face coordinates (a, b) of face direction dir -> volume index of extent n
__device__ __forceinline__ int face_point(int n, int d, int slice, int a, int b) {
  return d == 0 ? slice + n * (a + n * b) : (d == 1 ? a + n * (slice + n * b) : a + n * (b + n * slice));
}

// copy source of element e's X block
template <bool COMP, bool G2>
__device__ __forceinline__ const unsigned char* x_src(const BatchLaunch& L, int64_t off, int np) {
  return COMP ? reinterpret_cast<const unsigned char*>(L.x64 + off + (G2 ? 0 : np))
              : reinterpret_cast<const unsigned char*>(L.x32 + off);
}

// issue the TMA copies of task tk into buffer buf (one thread)
template <bool COMP, bool G2>
__device__ void issue_task(const BatchLaunch& L, int2 tk, unsigned char* buf, uint64_t* bar) {
  const int n = tk.x & 0xff, g = tk.x >> 8;
  const int np = n * n * n;
  const int xs = x_slot(n, COMP, G2), fb = f_bytes(n, COMP);
  uint32_t total = 0;
  for (int s = 0; s < g; ++s) {
    const int64_t e = L.task_elems[tk.y + s];
    const uintptr_t src = reinterpret_cast<uintptr_t>(x_src<COMP, G2>(L, L.offset[e], np));
    const uintptr_t a0 = src & ~(uintptr_t)15;
    const uintptr_t a1 = (src + (uintptr_t)x_bytes(n, COMP, G2) + 15) & ~(uintptr_t)15;
    total += (uint32_t)(a1 - a0) + (uint32_t)fb;
  }
  mbar_arrive_expect_tx(bar, total);
  for (int s = 0; s < g; ++s) {
    const int64_t e = L.task_elems[tk.y + s];
    const uintptr_t src = reinterpret_cast<uintptr_t>(x_src<COMP, G2>(L, L.offset[e], np));
    const uintptr_t a0 = src & ~(uintptr_t)15;
    const uintptr_t a1 = (src + (uintptr_t)x_bytes(n, COMP, G2) + 15) & ~(uintptr_t)15;
    bulk_g2s(buf + s * xs, reinterpret_cast<const void*>(a0), (uint32_t)(a1 - a0), bar);
    const unsigned char* fsrc = COMP ? reinterpret_cast<const unsigned char*>(L.fx2 + L.foff[e])
                                     : reinterpret_cast<const unsigned char*>(L.fx32 + L.foff[e]);
    bulk_g2s(buf + g * xs + s * f_slot(n, COMP), fsrc, (uint32_t)fb, bar);
  }
}

// Where the element in slot s of the current task sits in shared memory.
template <bool COMP, bool G2>
struct TaskView {
  unsigned char* buf;   // the task's pipeline buffer
  const int64_t* offs;  // value offset of each slot's element (shared memory)
  const BatchLaunch* L;
  int n, g;
  __device__ __forceinline__ unsigned char* x(int s) const {
    const uintptr_t src = reinterpret_cast<uintptr_t>(x_src<COMP, G2>(*L, offs[s], n * n * n));
    return buf + s * x_slot(n, COMP, G2) + (int)(src & 15);
  }
  __device__ __forceinline__ const unsigned char* f(int s) const {
    return buf + g * x_slot(n, COMP, G2) + s * f_slot(n, COMP);
  }
};

// ------------------------------------------------------------- one task
// W of slot s, field f (Psi, Pi, Phi_x, Phi_y, Phi_z), point p: where the
// passes leave it inside the X block.  F32: in place of X.  COMP (X holds
// Pi, Phi_x, Phi_y, Phi_z -- preceded by Psi when G2 -- as (hi, lo) FP32
// pairs): each field in the first word of its pair, except Psi without G2,
// in the second word of X's Pi pair.
template <bool COMP, bool G2>
__device__ __forceinline__ int w_index(int f, int p, int np) {
  if (!COMP) return f * np + p;
  if (G2) return 2 * (f * np + p);
  return f <= 1 ? 2 * p + (f == 0 ? 1 : 0) : 2 * ((f - 1) * np + p);
}


template <int N, bool COMP, bool G2>
__device__ __forceinline__ void task_passes(const BatchLaunch& L, const TaskView<COMP, G2>& V,
                                            float* S, const float* tabs, const int g,
                                            const float cf, const float* G, const float* F) {
  constexpr int NN = N * N, NP = NN * N;
  // pair index of Pi and of Phi_x in the COMP block
  constexpr int PI0 = (COMP && G2) ? NP : 0, PHI0 = (COMP && G2) ? 2 * NP : NP;
  const float g2 = (float)L.gamma2;
  const float g2h = g2, g2l = (float)(L.gamma2 - (double)g2);
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  const bool active = slot < g;
  const int ta = t % N, tb = t / N;
  const float alpha = (float)L.alpha;
  unsigned char* xb = active ? V.x(slot) : nullptr;
  const unsigned char* fbk = active ? V.f(slot) : nullptr;
  float* Sl = S + slot * NP;
  const float* th = tabs + tab_offset(N);
  const float* tl = tabs + kTabTotal + tab_offset(N);
  const int64_t off = active ? V.offs[slot] : 0;
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
      const int fidx = ta + N * tb;
      const float Gd = G[slot * 3 + d];
      const float Fd = F[slot * 3 + d];  // -c dxi/dx along this axis
      // the two lines one after the other (fewer live registers): Phi_d,
      // keeping its end values, then Pi
      float dF[N], dP[N], pih[N], pil[N];
      float dw_lo, dw_hi;
      if (COMP) {
        // X holds each FP64 value as its (hi, lo) FP32 pair (split_x)
        const float2* X = reinterpret_cast<const float2*>(xb);
        float f0h, f0l, f1h, f1l;
        float ps0h = 0.0f, ps0l = 0.0f, ps1h = 0.0f, ps1l = 0.0f;
        {
          float fh[N], fl[N];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const float2 v = X[PHI0 + d * NP + base + i * stride];
            fh[i] = v.x;
            fl[i] = v.y;
          }
          eo_line_pdfg<N>(fh, fl, dF, th, tl);
#pragma unroll
          for (int i = 0; i < N; ++i) dF[i] *= Fd;
          f0h = fh[0];
          f0l = fl[0];
          f1h = fh[N - 1];
          f1l = fl[N - 1];
          if (G2) {
            // the gamma2 (d_d Psi - Phi_d) term of the Phi_d output
            float psh[N], psl[N], dps[N];
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const float2 v = X[base + i * stride];
              psh[i] = v.x;
              psl[i] = v.y;
            }
            eo_line_pdfg<N>(psh, psl, dps, th, tl);
#pragma unroll
            for (int i = 0; i < N; ++i) dP[i] = -g2 * fmaf(Fd, dps[i], cf * (fh[i] + fl[i]));
            ps0h = psh[0];
            ps0l = psl[0];
            ps1h = psh[N - 1];
            ps1l = psl[N - 1];
          }
        }
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const float2 v = X[PI0 + base + i * stride];
          pih[i] = v.x;
          pil[i] = v.y;
        }
        {
          float dd[N];
          eo_line_pdfg<N>(pih, pil, dd, th, tl);
#pragma unroll
          for (int i = 0; i < N; ++i) dP[i] = G2 ? fmaf(Fd, dd[i], dP[i]) : Fd * dd[i];
        }
        const float2* ext = reinterpret_cast<const float2*>(fbk);
        const float2 elo = ext[(2 * d) * NN + fidx], ehi = ext[(2 * d + 1) * NN + fidx];
        float wh, wl, t0, dh;
        two_sum(pih[0], f0h, wh, t0);
        wl = t0 + (pil[0] + f0l);
        if (G2) sub_g2psi(wh, wl, g2h, g2l, ps0h, ps0l);
        two_sum(wh, -elo.x, dh, t0);
        dw_lo = dh + (t0 + (wl - elo.y));
        two_sum(pih[N - 1], -f1h, wh, t0);
        wl = t0 + (pil[N - 1] - f1l);
        if (G2) sub_g2psi(wh, wl, g2h, g2l, ps1h, ps1l);
        two_sum(wh, -ehi.x, dh, t0);
        dw_hi = dh + (t0 + (wl - ehi.y));
      } else {
        const float* X = reinterpret_cast<const float*>(xb);
        float f0h, f1h, ps0 = 0.0f, ps1 = 0.0f;
        {
          float fh[N];
#pragma unroll
          for (int i = 0; i < N; ++i) fh[i] = X[(2 + d) * NP + base + i * stride];
          eo_line_pg<N>(fh, dF, th);
#pragma unroll
          for (int i = 0; i < N; ++i) dF[i] *= Fd;
          f0h = fh[0];
          f1h = fh[N - 1];
          // alpha X_Phi_d enters the Phi_d output
#pragma unroll
          for (int i = 0; i < N; ++i) dP[i] = alpha * fh[i];
          if (G2) {
            // the gamma2 (d_d Psi - Phi_d) term of the Phi_d output
            float ps[N], dps[N];
#pragma unroll
            for (int i = 0; i < N; ++i) ps[i] = X[base + i * stride];
            eo_line_pg<N>(ps, dps, th);
#pragma unroll
            for (int i = 0; i < N; ++i) dP[i] = fmaf(-g2, fmaf(Fd, dps[i], cf * fh[i]), dP[i]);
            ps0 = ps[0];
            ps1 = ps[N - 1];
          }
        }
#pragma unroll
        for (int i = 0; i < N; ++i) {
          pih[i] = X[NP + base + i * stride];
          pil[i] = 0.0f;
        }
        {
          float dd[N];
          eo_line_pg<N>(pih, dd, th);
#pragma unroll
          for (int i = 0; i < N; ++i) dP[i] = fmaf(Fd, dd[i], dP[i]);
        }
        const float* ext = reinterpret_cast<const float*>(fbk);
        float wi_lo = pih[0] + f0h, wi_hi = pih[N - 1] - f1h;
        if (G2) {
          wi_lo = fmaf(-g2, ps0, wi_lo);
          wi_hi = fmaf(-g2, ps1, wi_hi);
        }
        dw_lo = wi_lo - ext[(2 * d) * NN + fidx];
        dw_hi = wi_hi - ext[(2 * d + 1) * NN + fidx];
      }
      dF[0] = fmaf(Gd, dw_lo, dF[0]);
      dP[0] = fmaf(Gd, dw_lo, dP[0]);
      dF[N - 1] = fmaf(Gd, dw_hi, dF[N - 1]);
      dP[N - 1] = fmaf(-Gd, dw_hi, dP[N - 1]);
      float* W = reinterpret_cast<float*>(xb);
      float* Wg = L.w32 + off;  // this element's block of the FP32 output
      // Phi_d output: to the output and, in place, for the face maps
#pragma unroll
      for (int i = 0; i < N; ++i) {
        W[w_index<COMP, G2>(2 + d, base + i * stride, NP)] = dP[i];
        Wg[(2 + d) * NP + base + i * stride] = dP[i];
      }
      if (d < 2) {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (d == 0)
            Sl[base + i * stride] = dF[i];
          else
            Sl[base + i * stride] += dF[i];
        }
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int p = base + i * stride;
          float wpi = Sl[p] + dF[i];
          float wpsi = COMP ? fmaf(-cf, pih[i], -cf * pil[i]) : -cf * pih[i];
          if (!COMP) {
            wpi = fmaf(alpha, pih[i], wpi);
            wpsi = fmaf(alpha, reinterpret_cast<const float*>(xb)[p], wpsi);
          }
          W[w_index<COMP, G2>(1, p, NP)] = wpi;
          W[w_index<COMP, G2>(0, p, NP)] = wpsi;
          Wg[NP + p] = wpi;
          Wg[p] = wpsi;
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

// COMP: each FP64 value of the staged X becomes its (hi, lo) FP32 pair in
// place (the same 8 bytes), so that the passes split each value once.
template <int N, bool G2>
__device__ __forceinline__ void split_x(const TaskView<true, G2>& V, int g, int bt) {
  constexpr int NP4 = (G2 ? 5 : 4) * N * N * N;
  for (int s = 0; s < g; ++s) {
    double* X = reinterpret_cast<double*>(V.x(s));
    for (int q = threadIdx.x; q < NP4; q += bt) {
      float hi, lo;
      split_df(X[q], hi, lo);
      reinterpret_cast<float2*>(X)[q] = make_float2(hi, lo);
    }
  }
}

// The face values of W in the element's own resolution: for each face dir,
// w = Pi + s_e Phi_d - gamma2 Psi (s_e = +1 upper, -1 lower) at its N^2
// points, into the
// element's own slots of the raw face buffer (coalesced); the face-map
// kernel then maps them onto the neighbours' points.
template <int n, bool COMP, bool G2, int BT>
__device__ __forceinline__ void task_raw_faces(const BatchLaunch& L, const TaskView<COMP, G2>& V,
                                               const int32_t* elems) {
  constexpr int nn = n * n, np = nn * n, F6 = 6 * nn;
  const float g2 = (float)L.gamma2;
  for (int s = 0; s < V.g; ++s) {
    const float* W = reinterpret_cast<const float*>(V.x(s));
    float* dst = L.raw32 + L.foff[elems[s]];
    for (int q = threadIdx.x; q < F6; q += BT) {
      const int dir = q / nn, r = q - dir * nn, d = dir >> 1;
      const bool upper = dir & 1;
      const int p = face_point(n, d, upper ? n - 1 : 0, r % n, r / n);
      const float pi = W[w_index<COMP, G2>(1, p, np)], ph = W[w_index<COMP, G2>(2 + d, p, np)];
      float w = upper ? pi + ph : pi - ph;
      if (G2) w = fmaf(-g2, W[w_index<COMP, G2>(0, p, np)], w);
      dst[q] = w;
    }
  }
}

template <int N, bool COMP, int BT, bool G2>
__device__ __forceinline__ void run_task(const BatchLaunch& L, const TaskView<COMP, G2>& V,
                                         float* S, const float* tabs, const float* G,
                                         const float* F, const int32_t* elems) {
  if constexpr (COMP) {
    split_x<N, G2>(V, V.g, BT);
    __syncthreads();
  }
  task_passes<N, COMP, G2>(L, V, S, tabs, V.g, (float)L.c, G, F);
  if (L.raw32 != nullptr) {
    __syncthreads();
    task_raw_faces<N, COMP, G2, BT>(L, V, elems);
  }
}

template <bool COMP, int BT, int NMAX, bool G2>
__device__ __forceinline__ void dispatch_task(const BatchLaunch& L, const TaskView<COMP, G2>& V,
                                              float* S, const float* tabs, const float* G,
                                              const float* F, const int32_t* elems) {
  switch (V.n) {
    case 2: run_task<2, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 3: run_task<3, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 4: run_task<4, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 5: run_task<5, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 6: run_task<6, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 7: run_task<7, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 8: run_task<8, COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 9: if (NMAX >= 9) run_task<(NMAX >= 9 ? 9 : 2), COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 10: if (NMAX >= 10) run_task<(NMAX >= 10 ? 10 : 2), COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 11: if (NMAX >= 11) run_task<(NMAX >= 11 ? 11 : 2), COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    case 12: if (NMAX >= 12) run_task<(NMAX >= 12 ? 12 : 2), COMP, BT, G2>(L, V, S, tabs, G, F, elems); break;
    default: break;
  }
}

// One stage over every task.  BT threads per CTA (one per grid line of the
// task's elements), MINB resident CTAs per SM asked of the register
// allocator, extents up to NMAX compiled in, STAGES pipeline buffers (2:
// the next task's copies land while this one computes; 1: they are issued
// when this one is done, and other resident CTAs cover the wait).
template <bool COMP, int BT, int MINB, int NMAX, int STAGES, bool G2>
__global__ void __launch_bounds__(BT, MINB) stage_batch_kernel(BatchLaunch L) {
  constexpr int kMaxG = BT / (kMinN * kMinN);  // elements per task at most (N = 2)
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bars[2];
  __shared__ int32_t s_elems[kMaxG];
  __shared__ int64_t s_offs[kMaxG];
  __shared__ float s_G[3 * kMaxG];
  __shared__ float s_F[3 * kMaxG];
  __shared__ __align__(16) float s_tab[2 * kTabTotal];
  unsigned char* bufs[2] = {smem, smem + (STAGES - 1) * L.buf_bytes};
  unsigned char* rest = smem + STAGES * L.buf_bytes;
  float* S = reinterpret_cast<float*>(rest);
  for (int q = threadIdx.x; q < 2 * kTabTotal; q += BT) s_tab[q] = L.dtab[q];

  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int64_t Gd = gridDim.x;
  int64_t task = blockIdx.x;
  if (task < L.n_tasks && threadIdx.x == 0) issue_task<COMP, G2>(L, L.tasks[task], bufs[0], &bars[0]);
  const double c = L.c;
  for (int k = 0; task < L.n_tasks; ++k, task += Gd) {
    const int b = STAGES == 2 ? (k & 1) : 0;
    const uint32_t parity = STAGES == 2 ? (uint32_t)((k >> 1) & 1) : (uint32_t)(k & 1);
    const int64_t next = task + Gd;
    if (STAGES == 2 && threadIdx.x == 0 && next < L.n_tasks)
      issue_task<COMP, G2>(L, L.tasks[next], bufs[b ^ 1], &bars[b ^ 1]);
    const int2 tk = L.tasks[task];
    const int n = tk.x & 0xff, g = tk.x >> 8;
    // per-element data (overlaps the copies)
    if (threadIdx.x < g) {
      const int32_t e = L.task_elems[tk.y + threadIdx.x];
      s_elems[threadIdx.x] = e;
      s_offs[threadIdx.x] = L.offset[e];
      for (int d = 0; d < 3; ++d) {
        const double jd = L.jac[3 * (int64_t)e + d];
        s_G[3 * threadIdx.x + d] = (float)(-0.25 * c * (double)(n * (n - 1)) * jd);
        s_F[3 * threadIdx.x + d] = (float)(-c * jd);
      }
    }
    const bool landed = mbar_wait(&bars[b], parity, kLimitNs);
    if (__syncthreads_or(!landed)) {
      // a copy did not land in time: record it, give the copies still in
      // flight one more bounded wait, and leave together
      if (threadIdx.x == 0 && L.err) atomicExch(L.err, 1);
      if (!landed) mbar_wait(&bars[b], parity, kLimitNs);
      if (STAGES == 2 && threadIdx.x == 0 && next < L.n_tasks)
        mbar_wait(&bars[b ^ 1], (uint32_t)(((k + 1) >> 1) & 1), kLimitNs);
      return;
    }
    TaskView<COMP, G2> V;
    V.buf = bufs[b];
    V.offs = s_offs;
    V.L = &L;
    V.n = n;
    V.g = g;
    dispatch_task<COMP, BT, NMAX, G2>(L, V, S, s_tab, s_G, s_F, s_elems);
    // generic-proxy accesses of this buffer before the next TMA writes into it
    fence_proxy_async_smem();
    __syncthreads();
    if (STAGES == 1 && threadIdx.x == 0 && next < L.n_tasks)
      issue_task<COMP, G2>(L, L.tasks[next], bufs[0], &bars[0]);
  }
}

// The step's update of the FP64 state and of its face values, as streams:
// u = u + (W + beta Y) for every value (FP64 add), and every face value
// fu += fw + beta fy in double-float.
__global__ void __launch_bounds__(256) accumulate_step_kernel(double* u, const float* w,
                                                              const float* y, float beta, int64_t n,
                                                              float2* fu, const float* fw,
                                                              const float* fy, int64_t nf) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  // four values per thread and iteration: one 16-byte load of W and of Y,
  // two of u, streamed past the caches
  const int64_t n4 = n / 4;
  const float4* w4 = reinterpret_cast<const float4*>(w);
  const float4* y4 = reinterpret_cast<const float4*>(y);
  double2* u2 = reinterpret_cast<double2*>(u);
  for (int64_t i = i0; i < n4; i += stride) {
    const float4 x = __ldcs(w4 + i);
    const float4 v = __ldcs(y4 + i);
    const double2 a = __ldcs(u2 + 2 * i);
    const double2 b = __ldcs(u2 + 2 * i + 1);
    __stcs(u2 + 2 * i, make_double2(a.x + widen(fmaf(beta, v.x, x.x)), a.y + widen(fmaf(beta, v.y, x.y))));
    __stcs(u2 + 2 * i + 1,
           make_double2(b.x + widen(fmaf(beta, v.z, x.z)), b.y + widen(fmaf(beta, v.w, x.w))));
  }
  for (int64_t i = 4 * n4 + i0; i < n; i += stride) u[i] = u[i] + widen(fmaf(beta, y[i], w[i]));
  for (int64_t i = i0; i < nf; i += stride) {
    const float v = fmaf(beta, fy[i], fw[i]);
    const float2 o = fu[i];
    float sh, st;
    two_sum(o.x, v, sh, st);
    st += o.y;
    const float hi = sh + st;
    fu[i] = make_float2(hi, st - (hi - sh));
  }
}

// ---------------------------------------------------------------- faces of u
// Double-float exterior values of an FP64 state: one warp per (element,
// face): w = Pi + s_e Phi_d - gamma2 Psi split into hi + lo, mapped by T (compensated
// products and sums, hi + lo tables) onto the neighbour's face points.
constexpr int kFaceWarps = 4;

__global__ void __launch_bounds__(32 * kFaceWarps) batch_faces_kernel(BatchFaceLaunch L) {
  __shared__ float2 sw[kFaceWarps][kMaxN * kMaxN];
  __shared__ float2 st[kFaceWarps][kMaxN * kMaxN];
  __shared__ float2 sT[kFaceWarps][kMaxN * kMaxN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t fc = (int64_t)blockIdx.x * kFaceWarps + warp;
  if (fc >= 6 * L.n_elem) return;  // whole warps leave; only warp barriers follow
  const int64_t e = fc / 6;
  const int dir = (int)(fc - 6 * e), d = dir >> 1;
  const bool upper = dir & 1;
  const int n = L.elem_n[e], nn = n * n, np = nn * n;
  const int slice = upper ? n - 1 : 0;
  const int64_t off = L.offset[e];
  const int64_t nb = L.nbr[fc];
  const int m = L.elem_n[nb];
  const int64_t dst = L.foff[nb] + (int64_t)(dir ^ 1) * m * m;
  float2* wv = sw[warp];
  float2* tv = st[warp];
  float2* T = sT[warp];
  if (m != n) {
    const int oo = L.op_off[m * (kMaxN + 1) + n];
    for (int q = lane; q < m * n; q += 32) T[q] = make_float2(L.op_hi[oo + q], L.op_lo[oo + q]);
  }
  const float g2h = (float)L.gamma2, g2l = (float)(L.gamma2 - (double)g2h);
  for (int q = lane; q < nn; q += 32) {
    const int p = face_point(n, d, slice, q % n, q / n);
    float ph, pl, qh, ql, wh, t0;
    split_df(L.x64[off + np + p], ph, pl);
    split_df(L.x64[off + (2 + d) * np + p], qh, ql);
    if (upper) {
      two_sum(ph, qh, wh, t0);
      t0 += pl + ql;
    } else {
      two_sum(ph, -qh, wh, t0);
      t0 += pl - ql;
    }
    if (L.gamma2 != 0.0) {
      float sh, sl;
      split_df(L.x64[off + p], sh, sl);
      sub_g2psi(wh, t0, g2h, g2l, sh, sl);
    }
    float hi, lo;
    two_sum(wh, t0, hi, lo);
    wv[q] = make_float2(hi, lo);
  }
  __syncwarp();
  if (m == n) {
    for (int q = lane; q < nn; q += 32) L.fu2[dst + q] = wv[q];
    return;
  }
  for (int q = lane; q < n * m; q += 32) {
    const int pp = q % n, b = q / n;
    float sh, sc;
    dot2_first(T[b * n].x, T[b * n].y, wv[pp].x, wv[pp].y, sh, sc);
    for (int k = 1; k < n; ++k)
      dot2_term(T[b * n + k].x, T[b * n + k].y, wv[pp + n * k].x, wv[pp + n * k].y, sh, sc);
    float r, rt;
    two_sum(sh, sc, r, rt);
    tv[q] = make_float2(r, rt);
  }
  __syncwarp();
  for (int q = lane; q < m * m; q += 32) {
    const int a = q % m, b = q / m;
    float sh, sc;
    dot2_first(T[a * n].x, T[a * n].y, tv[n * b].x, tv[n * b].y, sh, sc);
    for (int k = 1; k < n; ++k)
      dot2_term(T[a * n + k].x, T[a * n + k].y, tv[k + n * b].x, tv[k + n * b].y, sh, sc);
    float r, rt;
    two_sum(sh, sc, r, rt);
    L.fu2[dst + q] = make_float2(r, rt);
  }
}

// ---------------------------------------------------------------- face maps
// The next stage's exterior values: every producer face (element e, face
// dir) of the raw face buffer mapped by T (m x n, m the neighbour's extent;
// a copy when m = n) onto the neighbour's points, into its slot opposite
// dir.  The faces are sorted by (n, m) and cut into chunks of at most
// kMapFaces faces of one pair; a CTA takes one chunk, holds its T and all of
// its faces' values in shared memory, and each warp maps one face at a time:
// the first sweep into the warp's scratch, the second straight to the
// output.
constexpr int kMapWarps = 8;

constexpr int kMapFaces = kBatchMapFaces;

template <int n>
__device__ __forceinline__ void map_chunk(const FaceMapLaunch& L, int4 ch, float* Ts,
                                          float (*wall)[kMaxN * kMaxN], float* tv,
                                          int64_t* s_src, int64_t* s_dst) {
  constexpr int nn = n * n;
  const int m = (ch.x >> 8) & 0xff;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < ch.z) {
    s_src[threadIdx.x] = L.face_src[ch.y + threadIdx.x];
    s_dst[threadIdx.x] = L.face_dst[ch.y + threadIdx.x];
  }
  if (m != n) {
    const float* T = L.op_hi + L.op_off[m * (kMaxN + 1) + n];  // m x n, row-major
    for (int q = threadIdx.x; q < m * n; q += 32 * kMapWarps) Ts[q] = T[q];
  }
  __syncthreads();
  // every face of the chunk into shared memory at once (one load latency)
  for (int q = threadIdx.x; q < ch.z * nn; q += 32 * kMapWarps) {
    const int f = q / nn, r = q - f * nn;
    wall[f][r] = L.raw[s_src[f] + r];
  }
  __syncthreads();
  for (int f = warp; f < ch.z; f += kMapWarps) {
    const float* wv = wall[f];
    const int64_t dst = s_dst[f];
    if (m == n) {
      for (int q = lane; q < nn; q += 32) L.out[dst + q] = wv[q];
      continue;
    }
    // tv[pp + n b] = sum_k T(b, k) wv[pp + n k], b < m
    for (int q = lane; q < n * m; q += 32) {
      const int pp = q % n, b = q / n;
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < n; ++k) acc = fmaf(Ts[b * n + k], wv[pp + n * k], acc);
      tv[q] = acc;
    }
    __syncwarp();
    // out[a + m b] = sum_k T(a, k) tv[k + n b]
    for (int q = lane; q < m * m; q += 32) {
      const int b = (q * ((65536 + m - 1) / m)) >> 16, a = q - b * m;  // q / m, exact here
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < n; ++k) acc = fmaf(Ts[a * n + k], tv[k + n * b], acc);
      L.out[dst + q] = acc;
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(32 * kMapWarps) face_map_kernel(FaceMapLaunch L) {
  __shared__ float Ts[kMaxN * kMaxN];
  __shared__ float wall[kMapFaces][kMaxN * kMaxN];
  __shared__ float tv[kMapWarps][kMaxN * kMaxN];
  __shared__ int64_t s_src[kMapFaces], s_dst[kMapFaces];
  const int4 ch = L.chunks[blockIdx.x];
  const int n = ch.x & 0xff, warp = threadIdx.x >> 5;
  switch (n) {
    case 2: map_chunk<2>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 3: map_chunk<3>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 4: map_chunk<4>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 5: map_chunk<5>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 6: map_chunk<6>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 7: map_chunk<7>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 8: map_chunk<8>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 9: map_chunk<9>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 10: map_chunk<10>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 11: map_chunk<11>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    case 12: map_chunk<12>(L, ch, Ts, wall, tv[warp], s_src, s_dst); break;
    default: break;
  }
}

// The compiled launch shapes (variants): threads per CTA, resident CTAs
// asked of the register allocator for the FP64-input and the FP32 stages,
// largest extent, pipeline buffers.
struct ShapeSpec {
  int bt, minb_comp, minb_f32, nmax, stages;
};
constexpr ShapeSpec kShapes[] = {
    {128, 2, 3, 11, 2},  // 0
    {256, 1, 2, 12, 2},  // 1
    {128, 2, 4, 10, 2},  // 2
    {128, 4, 6, 10, 1},  // 3
    {128, 3, 5, 10, 1},  // 4
};
constexpr int kNumShapes = sizeof(kShapes) / sizeof(kShapes[0]);

template <bool COMP, int V, bool G2>
constexpr auto kernel_of() {
  constexpr ShapeSpec S = kShapes[V];
  return stage_batch_kernel<COMP, S.bt, COMP ? S.minb_comp : S.minb_f32, S.nmax, S.stages, G2>;
}

template <bool COMP, int V, bool G2>
cudaError_t launch_v(const BatchLaunch& L, size_t smem, cudaStream_t s) {
  constexpr auto k = kernel_of<COMP, V, G2>();
  cudaError_t e = set_kernel_smem<k>((int)smem, true);
  if (e != cudaSuccess) return e;
  k<<<(unsigned)L.grid, kShapes[V].bt, smem, s>>>(L);
  return cudaGetLastError();
}

template <bool COMP, int V, bool G2>
cudaError_t grid_v(size_t smem, int* per_sm) {
  constexpr auto k = kernel_of<COMP, V, G2>();
  cudaError_t e = set_kernel_smem<k>((int)smem, true);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, kShapes[V].bt, smem);
}

template <int V, bool G2>
cudaError_t launch_g(bool comp, const BatchLaunch& L, size_t smem, cudaStream_t s) {
  return comp ? launch_v<true, V, G2>(L, smem, s) : launch_v<false, V, G2>(L, smem, s);
}

template <int V>
cudaError_t launch_any(bool comp, bool g2, const BatchLaunch& L, size_t smem, cudaStream_t s) {
  if (L.variant == V) return g2 ? launch_g<V, true>(comp, L, smem, s) : launch_g<V, false>(comp, L, smem, s);
  if constexpr (V + 1 < kNumShapes) return launch_any<V + 1>(comp, g2, L, smem, s);
  return cudaErrorInvalidValue;
}

template <int V>
cudaError_t grid_any(bool comp, bool g2, int variant, size_t smem, int* per_sm) {
  if (variant == V) {
    if (g2) return comp ? grid_v<true, V, true>(smem, per_sm) : grid_v<false, V, true>(smem, per_sm);
    return comp ? grid_v<true, V, false>(smem, per_sm) : grid_v<false, V, false>(smem, per_sm);
  }
  if constexpr (V + 1 < kNumShapes) return grid_any<V + 1>(comp, g2, variant, smem, per_sm);
  return cudaErrorInvalidValue;
}

}  // namespace

int batch_variants() { return kNumShapes; }

int batch_threads(int variant) { return kShapes[variant].bt; }

int batch_max_extent(int variant) { return kShapes[variant].nmax; }

int batch_task_elements(int n, int variant) { return task_g(n, batch_threads(variant)); }

void batch_smem_bytes(int n, bool comp, bool g2, int variant, size_t* buf, size_t* s) {
  const int g = task_g(n, batch_threads(variant));
  *buf = (size_t)g * (x_slot(n, comp, g2) + f_slot(n, comp));
  *s = (size_t)round128(g * n * n * n * 4);
}

size_t batch_smem_total(int variant, size_t buf, size_t s) {
  return (size_t)kShapes[variant].stages * buf + s;
}

void batch_split_tables(std::vector<float>* out) {
  out->assign(2 * kTabTotal, 0.0f);
  for (int n = kMinN; n <= kMaxN; ++n) {
    EoTable eo;
    lgl_eo_table(n, &eo);
    const int h = n / 2, ts = tab_stride(n), o = tab_offset(n);
    for (int rr = 0; rr < ts; ++rr) {
      double v;
      if (rr < 2 * h * h) {
        const int pi = rr >> 1, i = pi / h, j = pi - i * h;
        v = (rr & 1) ? eo.B[i][j] : eo.A[i][j];
      } else if (rr < 2 * h * h + h) {
        v = eo.M[rr - 2 * h * h];
      } else {
        v = eo.B[h][rr - 2 * h * h - h];
      }
      const float hi = (float)v;
      (*out)[o + rr] = hi;
      (*out)[kTabTotal + o + rr] = (float)(v - (double)hi);
    }
  }
}

cudaError_t launch_stage_batch(const BatchLaunch& L, cudaStream_t s) {
  if (L.n_tasks <= 0) return cudaSuccess;
  const bool comp = L.prec == kPrecComp;
  if (comp ? (L.x64 == nullptr || L.fx2 == nullptr) : (L.x32 == nullptr || L.fx32 == nullptr))
    return cudaErrorInvalidValue;
  if (L.w32 == nullptr) return cudaErrorInvalidValue;
  if (L.variant < 0 || L.variant >= kNumShapes) return cudaErrorInvalidValue;
  const size_t smem = batch_smem_total(L.variant, L.buf_bytes, L.s_bytes);
  return launch_any<0>(comp, L.gamma2 != 0.0, L, smem, s);
}

cudaError_t batch_grid(bool comp, bool g2, int variant, size_t smem, int* grid) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  if (variant < 0 || variant >= kNumShapes) return cudaErrorInvalidValue;
  if ((e = grid_any<0>(comp, g2, variant, smem, &per_sm)) != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  *grid = sms * per_sm;
  return cudaSuccess;
}

cudaError_t launch_batch_faces(const BatchFaceLaunch& L, cudaStream_t s) {
  const int64_t faces = 6 * L.n_elem;
  if (faces <= 0) return cudaSuccess;
  const int64_t blocks = (faces + kFaceWarps - 1) / kFaceWarps;
  batch_faces_kernel<<<(unsigned)blocks, 32 * kFaceWarps, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_face_map(const FaceMapLaunch& L, cudaStream_t s) {
  if (L.n_chunks <= 0) return cudaSuccess;
  face_map_kernel<<<(unsigned)L.n_chunks, 32 * kMapWarps, 0, s>>>(L);
  return cudaGetLastError();
}

cudaError_t launch_accumulate_step(double* u, const float* w, const float* y, double beta,
                                   int64_t n, float2* fu, const float* fw, const float* fy,
                                   int64_t nf, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(w) |
        reinterpret_cast<uintptr_t>(y)) & 15u) != 0)
    return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int64_t want = (n / 4 + 255) / 256;
  const int64_t grid = want < (int64_t)sms * 16 ? (want > 0 ? want : 1) : (int64_t)sms * 16;
  accumulate_step_kernel<<<(unsigned)grid, 256, 0, s>>>(u, w, y, (float)beta, n, fu, fw, fy, nf);
  return cudaGetLastError();
}

}  // namespace dgsw
