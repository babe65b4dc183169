// stage_general.cu -- fused DG right-hand side + SSP-RK3 stage for elements of
// differing LGL extents (p-nonconforming mortars), one launch per extent class.
//
// Same operator as stage_fp64.cu / stage_mixed.cu, generalised to a face
// whose neighbour has a different extent Nn.  The reference projects both
// sides' packaged data onto the mortar (extent max(N, Nn): interpolation,
// Projection.cpp:310-330), evaluates UpwindPenalty there, projects the
// correction back to the face (Legendre modal truncation, Projection.cpp:97-130)
// and lifts it (ApplyBoundaryCorrections.hpp:880-937).  With char speeds
// (0, +1, -1) the correction is linear in the packaged fields
// (D_Pi = (w_int - w_ext)/2, D_Phi = -n D_Pi, w = Pi - n.Phi - gamma2 Psi),
// and restriction after interpolation is the identity, so the whole mortar
// round trip equals
//   D_Pi = (w_int - T w_ext)/2,   T = R_{mortar->face} P_{nbr face->mortar},
// a separable N x Nn operator applied along both face dimensions: the
// interpolation matrix when Nn < N, the restriction when Nn > N.
//
// Each element: stage X (Pi, Phi) in shared memory; map every face's
// exterior w onto this face's points (T applied in two sweeps); then the
// three line passes of the uniform kernels reading the mapped exterior
// values.  Arithmetic classes:
//   PREC_F64  FP64 throughout (the plain path),
//   PREC_COMP FP64 input, double-float FP32 arithmetic, FP32 result
//             (first mixed stage; the face maps are compensated too),
//   PREC_F32  FP32 input and arithmetic (mixed increments).
// Result: W = alpha X + beta Y + c L(X); outputs as in stage_mixed.cu, with
// Y and the FP64 output in FP64 for PREC_F64.
#include <cstdint>
#include <type_traits>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

using dev::dot2_first;
using dev::dot2_term;
using dev::Eo;
using dev::eo_line;
using dev::eo_line_df;
using dev::split_df;
using dev::sub_g2psi;
using dev::two_sum;
using dev::widen;

constexpr int kNmax = kMaxN;

constexpr int round16(int b) { return (b + 15) / 16 * 16; }

// Shared-memory layout of one element slot.  Every region size is rounded to
// 16 bytes so that each region starts aligned for its widest access (double
// or float2), whatever N.
template <int N, int PREC>
struct GLay {
  using FT = typename std::conditional<PREC == kPrecF32, float, double>::type;
  static constexpr int NN = N * N, NP = N * N * N;
  static constexpr int TAB = Eo<N>::TAB;
  // bytes of each region
  static constexpr int kF = round16(4 * NP * (int)sizeof(FT));         // X: Pi, Phi
  static constexpr int kS = round16(NP * (PREC == kPrecF64 ? 8 : 4));  // dt Pi accumulator
  static constexpr int kTab = round16(3 * TAB * (PREC == kPrecF32 ? 4 : 8));
  // face maps: temp1 [6][Nmax^2], temp2 [6][Nmax*N], ext [6][N^2]; double or
  // double-float (two floats: same bytes) for F64 / COMP, float for F32
  static constexpr int kVal = PREC == kPrecF32 ? 4 : 8;
  static constexpr int kT1 = round16(6 * kNmax * kNmax * kVal);
  static constexpr int kT2 = round16(6 * kNmax * N * kVal);
  static constexpr int kExt = round16(6 * NN * kVal);
  static constexpr int kSlot = kF + kS + kTab + kT1 + kT2 + kExt;
};

template <int N>
constexpr int general_epb() {
  return N <= 4 ? 8 : (N <= 6 ? 4 : (N <= 8 ? 2 : 1));
}

// face coordinates (a, b) of face direction dir -> volume index of extent n
__device__ __forceinline__ int face_point(int n, int d, int slice, int a, int b) {
  return d == 0 ? slice + n * (a + n * b) : (d == 1 ? a + n * (slice + n * b) : a + n * (b + n * slice));
}

template <int N, int EPB, int PREC>
__global__ void __launch_bounds__(N * N * EPB) stage_general_kernel(GeneralLaunch L) {
  using Y = GLay<N, PREC>;
  using FT = typename Y::FT;
  constexpr int NN = N * N, NP = N * N * N, TAB = Y::TAB;
  constexpr int h = Eo<N>::h, H = Eo<N>::H;
  constexpr bool kF64 = PREC == kPrecF64, kComp = PREC == kPrecComp, kF32 = PREC == kPrecF32;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  const int64_t task = (int64_t)blockIdx.x * EPB + slot;
  const bool active = task < L.n_tasks;
  unsigned char* base_ptr = gsm + (size_t)slot * Y::kSlot;
  FT* F = reinterpret_cast<FT*>(base_ptr);
  unsigned char* p = base_ptr + Y::kF;
  double* S64 = reinterpret_cast<double*>(p);
  float* S32 = reinterpret_cast<float*>(p);
  p += Y::kS;
  double* T64 = reinterpret_cast<double*>(p);
  float* T32 = reinterpret_cast<float*>(p);  // COMP: hi [3 TAB] then lo [3 TAB]
  p += Y::kTab;
  unsigned char* t1 = p;
  unsigned char* t2 = p + Y::kT1;
  unsigned char* ex = p + Y::kT1 + Y::kT2;

  const int64_t e = active ? (int64_t)L.tasks[task] : 0;
  const int64_t off = active ? L.offset[e] : 0;
  double jd[3] = {0.0, 0.0, 0.0};
  const double c = L.c;

  // ---- stage X and the scaled split tables -------------------------------
  if (active) {
    jd[0] = L.jac[3 * e];
    jd[1] = L.jac[3 * e + 1];
    jd[2] = L.jac[3 * e + 2];
    if (kF32) {
      const float* src = L.x32 + off + NP;
      for (int q = t; q < 4 * NP; q += NN) F[q] = (FT)src[q];
    } else {
      const double* src = L.x64 + off + NP;
      for (int q = t; q < 4 * NP; q += NN) F[q] = (FT)src[q];
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
      const double sv = (-c * jd[d]) * v;
      if (kF64) {
        T64[q] = sv;
      } else {
        const float hi = __double2float_rn(sv);
        T32[q] = hi;
        if (kComp) T32[3 * TAB + q] = __double2float_rn(sv - (double)hi);
      }
    }
  }

  // ---- exterior w of every face, mapped onto this face's points ----------
  // step 1: w_ext at the neighbour's own face points (temp1), or straight
  // into ext when the extents match
  if (active) {
    for (int dir = 0; dir < 6; ++dir) {
      const int d = dir >> 1;
      const bool upper = dir & 1;
      const int64_t nb = L.nbr[6 * e + dir];
      const int nn = L.elem_n[nb];
      const int64_t noff = L.offset[nb];
      const int npts = nn * nn;
      const int nslice = upper ? 0 : nn - 1;
      const double s = upper ? 1.0 : -1.0;
      for (int q = t; q < npts; q += NN) {
        const int a = q % nn, b = q / nn;
        const int v = face_point(nn, d, nslice, a, b);
        const int64_t np_n = (int64_t)nn * nn * nn;
        if (kF32) {
          float w = L.x32[noff + np_n + v] - (float)s * L.x32[noff + (2 + d) * np_n + v];
          if (L.gamma2 != 0.0) w = fmaf(-(float)L.gamma2, L.x32[noff + v], w);
          float* dst = reinterpret_cast<float*>(nn == N ? ex : t1) + (nn == N ? dir * NN : dir * kNmax * kNmax);
          dst[q] = w;
        } else if (kF64) {
          double w = L.x64[noff + np_n + v] - s * L.x64[noff + (2 + d) * np_n + v];
          if (L.gamma2 != 0.0) w = fma(-L.gamma2, L.x64[noff + v], w);
          double* dst = reinterpret_cast<double*>(nn == N ? ex : t1) + (nn == N ? dir * NN : dir * kNmax * kNmax);
          dst[q] = w;
        } else {
          float ph, pl, qh, ql, wh, t0;
          split_df(L.x64[noff + np_n + v], ph, pl);
          split_df(L.x64[noff + (2 + d) * np_n + v], qh, ql);
          if (upper) {
            two_sum(ph, -qh, wh, t0);
            t0 += pl - ql;
          } else {
            two_sum(ph, qh, wh, t0);
            t0 += pl + ql;
          }
          if (L.gamma2 != 0.0) {
            float sh, sl;
            split_df(L.x64[noff + v], sh, sl);
            const float gh = (float)L.gamma2;
            sub_g2psi(wh, t0, gh, (float)(L.gamma2 - (double)gh), sh, sl);
          }
          float2* dst = reinterpret_cast<float2*>(nn == N ? ex : t1) + (nn == N ? dir * NN : dir * kNmax * kNmax);
          dst[q] = make_float2(wh, t0);
        }
      }
    }
  }
  __syncthreads();
  // step 2: temp2[dir][p + nn*b] = sum_q T(b, q) temp1[dir][p + nn*q]
  if (active) {
    for (int dir = 0; dir < 6; ++dir) {
      const int nn = L.elem_n[L.nbr[6 * e + dir]];
      if (nn == N) continue;
      const int oo = L.op_off[N * (kNmax + 1) + nn];
      for (int q = t; q < nn * N; q += NN) {
        const int pp = q % nn, b = q / nn;
        if (kF64) {
          const double* src = reinterpret_cast<const double*>(t1) + dir * kNmax * kNmax;
          double acc = 0.0;
          for (int k = 0; k < nn; ++k) acc = fma(L.op64[oo + b * nn + k], src[pp + nn * k], acc);
          reinterpret_cast<double*>(t2)[dir * kNmax * N + q] = acc;
        } else if (kF32) {
          const float* src = reinterpret_cast<const float*>(t1) + dir * kNmax * kNmax;
          float acc = 0.0f;
          for (int k = 0; k < nn; ++k) acc = fmaf(L.op_hi[oo + b * nn + k], src[pp + nn * k], acc);
          reinterpret_cast<float*>(t2)[dir * kNmax * N + q] = acc;
        } else {
          const float2* src = reinterpret_cast<const float2*>(t1) + dir * kNmax * kNmax;
          float sh, sc;
          dot2_first(L.op_hi[oo + b * nn], L.op_lo[oo + b * nn], src[pp].x, src[pp].y, sh, sc);
          for (int k = 1; k < nn; ++k)
            dot2_term(L.op_hi[oo + b * nn + k], L.op_lo[oo + b * nn + k], src[pp + nn * k].x,
                      src[pp + nn * k].y, sh, sc);
          float r, rt;
          two_sum(sh, sc, r, rt);
          reinterpret_cast<float2*>(t2)[dir * kNmax * N + q] = make_float2(r, rt);
        }
      }
    }
  }
  __syncthreads();
  // step 3: ext[dir][a + N b] = sum_p T(a, p) temp2[dir][p + nn*b]
  if (active) {
    for (int dir = 0; dir < 6; ++dir) {
      const int nn = L.elem_n[L.nbr[6 * e + dir]];
      if (nn == N) continue;
      const int oo = L.op_off[N * (kNmax + 1) + nn];
      for (int q = t; q < NN; q += NN) {
        const int a = q % N, b = q / N;
        if (kF64) {
          const double* src = reinterpret_cast<const double*>(t2) + dir * kNmax * N;
          double acc = 0.0;
          for (int k = 0; k < nn; ++k) acc = fma(L.op64[oo + a * nn + k], src[k + nn * b], acc);
          reinterpret_cast<double*>(ex)[dir * NN + q] = acc;
        } else if (kF32) {
          const float* src = reinterpret_cast<const float*>(t2) + dir * kNmax * N;
          float acc = 0.0f;
          for (int k = 0; k < nn; ++k) acc = fmaf(L.op_hi[oo + a * nn + k], src[k + nn * b], acc);
          reinterpret_cast<float*>(ex)[dir * NN + q] = acc;
        } else {
          const float2* src = reinterpret_cast<const float2*>(t2) + dir * kNmax * N;
          float sh, sc;
          dot2_first(L.op_hi[oo + a * nn], L.op_lo[oo + a * nn], src[nn * b].x, src[nn * b].y, sh, sc);
          for (int k = 1; k < nn; ++k)
            dot2_term(L.op_hi[oo + a * nn + k], L.op_lo[oo + a * nn + k], src[k + nn * b].x,
                      src[k + nn * b].y, sh, sc);
          float r, rt;
          two_sum(sh, sc, r, rt);
          reinterpret_cast<float2*>(ex)[dir * NN + q] = make_float2(r, rt);
        }
      }
    }
  }
  __syncthreads();

  // ---- three line passes ----------------------------------------------------
  const int ta = t % N, tb = t / N;
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
      const int fidx = ta + N * tb;  // this line's point on faces normal to d
      // pointwise inputs of this pass, loaded before any store
      double y64v[N], b64v[N];
      float y32v[N];
      const int64_t vo = off + (2 + d) * NP + base;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        y64v[i] = (kF64 && L.y64) ? L.y64[vo + i * stride] : 0.0;
        y32v[i] = (!kF64 && L.y32) ? L.y32[vo + i * stride] : 0.0f;
        b64v[i] = (!kF64 && L.base64 && L.out64) ? L.base64[vo + i * stride] : 0.0;
      }
      if (kF64) {
        double up[N], uf[N], dF[N], dP[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          up[i] = F[base + i * stride];
          uf[i] = F[(1 + d) * NP + base + i * stride];
        }
        const double* tab = T64 + d * TAB;
        eo_line<N, double>(uf, dF, tab);
        eo_line<N, double>(up, dP, tab);
        if (L.boundary) {
          const double G = -0.25 * c * (double)(N * (N - 1)) * jd[d];
          const double* ext = reinterpret_cast<const double*>(ex);
          double wi_lo = up[0] + uf[0];
          double wi_hi = up[N - 1] - uf[N - 1];
          if (L.gamma2 != 0.0) {
            wi_lo = fma(-L.gamma2, L.x64[off + base], wi_lo);
            wi_hi = fma(-L.gamma2, L.x64[off + base + (N - 1) * stride], wi_hi);
          }
          const double dw_lo = wi_lo - ext[(2 * d) * NN + fidx];
          const double dw_hi = wi_hi - ext[(2 * d + 1) * NN + fidx];
          dF[0] = fma(G, dw_lo, dF[0]);
          dP[0] = fma(G, dw_lo, dP[0]);
          dF[N - 1] = fma(G, dw_hi, dF[N - 1]);
          dP[N - 1] = fma(-G, dw_hi, dP[N - 1]);
        }
        if (L.gamma2 != 0.0) {
          double ups[N], dpsi[N];
#pragma unroll
          for (int i = 0; i < N; ++i) ups[i] = L.x64[off + base + i * stride];
          eo_line<N, double>(ups, dpsi, tab);
#pragma unroll
          for (int i = 0; i < N; ++i) dP[i] = fma(-L.gamma2, dpsi[i] + c * uf[i], dP[i]);
        }
#pragma unroll
        for (int i = 0; i < N; ++i)
          L.out64[vo + i * stride] = fma(L.beta, y64v[i], fma(L.alpha, uf[i], dP[i]));
        if (d < 2) {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            if (d == 0)
              S64[base + i * stride] = dF[i];
            else
              S64[base + i * stride] += dF[i];
          }
        } else {
          double ypi[N], ypsi[N], xpsi[N];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int pt = base + i * stride;
            ypi[i] = L.y64 ? L.y64[off + NP + pt] : 0.0;
            ypsi[i] = L.y64 ? L.y64[off + pt] : 0.0;
            xpsi[i] = L.x64[off + pt];
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int pt = base + i * stride;
            const double sp = S64[pt] + dF[i];
            L.out64[off + NP + pt] = fma(L.beta, ypi[i], fma(L.alpha, up[i], sp));
            L.out64[off + pt] = fma(L.beta, ypsi[i], fma(L.alpha, xpsi[i], -c * up[i]));
          }
        }
      } else {
        // FP32 arithmetic (double-float for COMP)
        float pih[N], pil[N], fh[N], fl[N], dF[N], dP[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          if (kComp) {
            split_df((double)F[base + i * stride], pih[i], pil[i]);
            split_df((double)F[(1 + d) * NP + base + i * stride], fh[i], fl[i]);
          } else {
            pih[i] = (float)F[base + i * stride];
            fh[i] = (float)F[(1 + d) * NP + base + i * stride];
            pil[i] = 0.0f;
            fl[i] = 0.0f;
          }
        }
        const float* th = T32 + d * TAB;
        // Psi at the line's ends, for the gamma2 Psi part of w
        float ps0h = 0.0f, ps0l = 0.0f, ps1h = 0.0f, ps1l = 0.0f;
        if (kComp) {
          const float* tl = T32 + 3 * TAB + d * TAB;
          eo_line_df<N>(fh, fl, dF, th, tl);
          eo_line_df<N>(pih, pil, dP, th, tl);
          if (L.gamma2 != 0.0) {
            // the gamma2 (d_d Psi - Phi_d) term of the Phi_d output
            float psh[N], psl[N], dps[N];
#pragma unroll
            for (int i = 0; i < N; ++i) split_df(L.x64[off + base + i * stride], psh[i], psl[i]);
            eo_line_df<N>(psh, psl, dps, th, tl);
            const float g2 = (float)L.gamma2, cc = (float)c;
#pragma unroll
            for (int i = 0; i < N; ++i) dP[i] = fmaf(-g2, dps[i] + cc * (fh[i] + fl[i]), dP[i]);
            ps0h = psh[0];
            ps0l = psl[0];
            ps1h = psh[N - 1];
            ps1l = psl[N - 1];
          }
        } else {
          eo_line<N, float>(fh, dF, th);
          eo_line<N, float>(pih, dP, th);
          if (L.gamma2 != 0.0) {
            float ps[N], dps[N];
#pragma unroll
            for (int i = 0; i < N; ++i) ps[i] = L.x32[off + base + i * stride];
            eo_line<N, float>(ps, dps, th);
            const float g2 = (float)L.gamma2, cc = (float)c;
#pragma unroll
            for (int i = 0; i < N; ++i) dP[i] = fmaf(-g2, dps[i] + cc * fh[i], dP[i]);
            ps0h = ps[0];
            ps1h = ps[N - 1];
          }
        }
        if (L.boundary) {
          const float G = (float)(-0.25 * c * (double)(N * (N - 1)) * jd[d]);
          float dw_lo, dw_hi;
          if (kComp) {
            const float2* ext = reinterpret_cast<const float2*>(ex);
            const float2 elo = ext[(2 * d) * NN + fidx], ehi = ext[(2 * d + 1) * NN + fidx];
            float wh, wl, t0, dh;
            const float gh = (float)L.gamma2, gl = (float)(L.gamma2 - (double)gh);
            two_sum(pih[0], fh[0], wh, t0);
            wl = t0 + (pil[0] + fl[0]);
            if (L.gamma2 != 0.0) sub_g2psi(wh, wl, gh, gl, ps0h, ps0l);
            two_sum(wh, -elo.x, dh, t0);
            dw_lo = dh + (t0 + (wl - elo.y));
            two_sum(pih[N - 1], -fh[N - 1], wh, t0);
            wl = t0 + (pil[N - 1] - fl[N - 1]);
            if (L.gamma2 != 0.0) sub_g2psi(wh, wl, gh, gl, ps1h, ps1l);
            two_sum(wh, -ehi.x, dh, t0);
            dw_hi = dh + (t0 + (wl - ehi.y));
          } else {
            const float* ext = reinterpret_cast<const float*>(ex);
            const float g2 = (float)L.gamma2;
            dw_lo = fmaf(-g2, ps0h, pih[0] + fh[0]) - ext[(2 * d) * NN + fidx];
            dw_hi = fmaf(-g2, ps1h, pih[N - 1] - fh[N - 1]) - ext[(2 * d + 1) * NN + fidx];
          }
          dF[0] = fmaf(G, dw_lo, dF[0]);
          dP[0] = fmaf(G, dw_lo, dP[0]);
          dF[N - 1] = fmaf(G, dw_hi, dF[N - 1]);
          dP[N - 1] = fmaf(-G, dw_hi, dP[N - 1]);
        }
        const float alpha = (float)L.alpha, beta = (float)L.beta, cf = (float)c;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float w = dP[i];
          if (kF32) w = fmaf(alpha, fh[i], w);
          if (L.y32) w = fmaf(beta, y32v[i], w);
          if (L.w32) L.w32[vo + i * stride] = w;
          if (L.out64) L.out64[vo + i * stride] = (L.base64 ? b64v[i] : 0.0) + widen(w);
        }
        if (d < 2) {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            if (d == 0)
              S32[base + i * stride] = dF[i];
            else
              S32[base + i * stride] += dF[i];
          }
        } else {
          float ypi[N], ypsi[N], xpsi[N];
          double bpi[N], bpsi[N];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int pt = base + i * stride;
            ypi[i] = L.y32 ? L.y32[off + NP + pt] : 0.0f;
            ypsi[i] = L.y32 ? L.y32[off + pt] : 0.0f;
            xpsi[i] = kF32 ? L.x32[off + pt] : 0.0f;
            bpi[i] = (L.base64 && L.out64) ? L.base64[off + NP + pt] : 0.0;
            bpsi[i] = (L.base64 && L.out64) ? L.base64[off + pt] : 0.0;
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int pt = base + i * stride;
            float wpi = S32[pt] + dF[i];
            float wpsi = kComp ? fmaf(-cf, pih[i], -cf * pil[i]) : -cf * pih[i];
            if (kF32) {
              wpi = fmaf(alpha, pih[i], wpi);
              wpsi = fmaf(alpha, xpsi[i], wpsi);
            }
            if (L.y32) {
              wpi = fmaf(beta, ypi[i], wpi);
              wpsi = fmaf(beta, ypsi[i], wpsi);
            }
            if (L.w32) {
              L.w32[off + NP + pt] = wpi;
              L.w32[off + pt] = wpsi;
            }
            if (L.out64) {
              L.out64[off + NP + pt] = (L.base64 ? bpi[i] : 0.0) + widen(wpi);
              L.out64[off + pt] = (L.base64 ? bpsi[i] : 0.0) + widen(wpsi);
            }
          }
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

template <int N, int PREC>
cudaError_t launch_general_np(const GeneralLaunch& L, cudaStream_t s) {
  constexpr int EPB = general_epb<N>();
  const size_t smem = (size_t)EPB * GLay<N, PREC>::kSlot;
  auto k = stage_general_kernel<N, EPB, PREC>;
  cudaError_t err = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  const int64_t blocks = (L.n_tasks + EPB - 1) / EPB;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, N * N * EPB, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_general_n(const GeneralLaunch& L, cudaStream_t s) {
  switch (L.prec) {
    case kPrecF64: return launch_general_np<N, kPrecF64>(L, s);
    case kPrecComp: return launch_general_np<N, kPrecComp>(L, s);
    case kPrecF32: return launch_general_np<N, kPrecF32>(L, s);
    default: return cudaErrorInvalidValue;
  }
}


// ---- exterior w of the faces whose neighbour has another extent ------------
// For the FP64 path the stage kernel of uniform meshes (stage_fp64.cu) runs
// each extent class over its task list and reads, on these faces, the
// exterior w mapped onto its own face points from a record written here
// before the stage: ext = (T x T) w_nbr, T = R_{mortar->face} P_{nbr->mortar}
// (N x nn), w = Pi - s Phi_d - gamma2 Psi of the neighbour's face points with
// this face's sign s.  One warp per record; w_nbr and the first sweep sit in
// the warp's shared memory.
constexpr int kPncWarps = 4;

template <int N>
__global__ void __launch_bounds__(32 * kPncWarps) pnc_faces_kernel(PncFaceLaunch L) {
  constexpr int NN = N * N;
  __shared__ double sw[kPncWarps][kNmax * kNmax];
  __shared__ double s2[kPncWarps][kNmax * N];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int64_t r = (int64_t)blockIdx.x * kPncWarps + warp;
  if (r >= L.n_rec) return;  // whole warps leave; only warp barriers follow
  const int64_t face = L.rec_face[r];
  const int64_t e = face / 6;
  const int dir = (int)(face - 6 * e), d = dir >> 1;
  const bool upper = dir & 1;
  const int64_t nb = L.nbr[face];
  const int nn = L.elem_n[nb];
  const int64_t noff = L.offset[nb], np_n = (int64_t)nn * nn * nn;
  const int nslice = upper ? 0 : nn - 1;
  const double sgn = upper ? 1.0 : -1.0;
  double* w = sw[warp];
  double* t2 = s2[warp];
  for (int q = lane; q < nn * nn; q += 32) {
    const int v = face_point(nn, d, nslice, q % nn, q / nn);
    double x = L.x[noff + np_n + v] - sgn * L.x[noff + (2 + d) * np_n + v];
    if (L.gamma2 != 0.0) x = fma(-L.gamma2, L.x[noff + v], x);
    w[q] = x;
  }
  __syncwarp();
  const double* T = L.op64 + L.op_off[N * (kNmax + 1) + nn];  // N x nn, row-major
  for (int q = lane; q < nn * N; q += 32) {
    const int pp = q % nn, b = q / nn;
    double acc = 0.0;
    for (int k = 0; k < nn; ++k) acc = fma(T[b * nn + k], w[pp + nn * k], acc);
    t2[q] = acc;
  }
  __syncwarp();
  for (int q = lane; q < NN; q += 32) {
    const int a = q % N, b = q / N;
    double acc = 0.0;
    for (int k = 0; k < nn; ++k) acc = fma(T[a * nn + k], t2[k + nn * b], acc);
    L.wext[r * NN + q] = acc;
  }
}

template <int N>
cudaError_t launch_pnc_n(const PncFaceLaunch& L, cudaStream_t s) {
  const int64_t blocks = (L.n_rec + kPncWarps - 1) / kPncWarps;
  if (blocks <= 0) return cudaSuccess;
  pnc_faces_kernel<N><<<(unsigned)blocks, 32 * kPncWarps, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_pnc_faces(const PncFaceLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_pnc_n<2>(L, s);
    case 3: return launch_pnc_n<3>(L, s);
    case 4: return launch_pnc_n<4>(L, s);
    case 5: return launch_pnc_n<5>(L, s);
    case 6: return launch_pnc_n<6>(L, s);
    case 7: return launch_pnc_n<7>(L, s);
    case 8: return launch_pnc_n<8>(L, s);
    case 9: return launch_pnc_n<9>(L, s);
    case 10: return launch_pnc_n<10>(L, s);
    case 11: return launch_pnc_n<11>(L, s);
    case 12: return launch_pnc_n<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_stage_general(const GeneralLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_general_n<2>(L, s);
    case 3: return launch_general_n<3>(L, s);
    case 4: return launch_general_n<4>(L, s);
    case 5: return launch_general_n<5>(L, s);
    case 6: return launch_general_n<6>(L, s);
    case 7: return launch_general_n<7>(L, s);
    case 8: return launch_general_n<8>(L, s);
    case 9: return launch_general_n<9>(L, s);
    case 10: return launch_general_n<10>(L, s);
    case 11: return launch_general_n<11>(L, s);
    case 12: return launch_general_n<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
