// stage_gauss.cu -- plain FP64 fused DG right-hand side + SSP-RK3 substep of
// the flat scalar wave on Legendre-Gauss points (Spectral::Quadrature::Gauss),
// uniform extent N, conforming periodic bricks.
//
// With Gauss points the faces are not volume points.  The volume terms are
// those of stage_fp64.cu with the Gauss differentiation matrix (also
// centro-antisymmetric, so the even/odd split applies).  For the boundary,
// each side interpolates its own data to the shared face with the rows
// l_j(-1), l_j(+1) (Spectral::boundary_interpolation_matrices), the
// UpwindPenalty correction is formed there, and it is lifted into every
// point of the line normal to the face by lift_boundary_terms_gauss_points
// (LiftFromBoundary.cpp:20-140, ApplyBoundaryCorrections.hpp:938-987):
//   dt u(point i of the line) -= |n| (l_i(+-1) / w_i) correction.
// On an affine element det(inverse Jacobian) x det(Jacobian on the face) = 1,
// so only |n| = 2 / width remains.
//
// Flat UpwindPenalty in closed form (char speeds 0, +1, -1, unit normal
// n = s e_d): D_Psi = 0, D_Pi = (w_int - w_ext) / 2, D_Phi_d = -s D_Pi with
// w = Pi - s Phi_d - gamma2 Psi.  Since w is linear in the fields, each side's
// face value is the interpolation of w along the line.
//
// Work split: N*N threads per element, one line per thread per axis, the
// three axes in turn (as stage_fp64.cu); a thread reads the two neighbours'
// lines along its axis straight from their volume data to interpolate their
// face values.  unext = a u0 + b ucur + c L(ucur).
#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

template <int N>
struct GShape {
  static constexpr int h = N / 2;
  static constexpr int H = h + N % 2;
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = 2 * H * h + H;
  static constexpr int SLOT = 5 * NP + 3 * TAB;  // Pi, Phi (4 NP), Sacc, tables
};

template <int N>
constexpr int gauss_epb() {
  return N <= 4 ? 8 : (N <= 6 ? 4 : (N <= 10 ? 2 : 1));
}

template <int N, int EPB, bool kBoundary>
__global__ void __launch_bounds__(N * N * EPB) stage_gauss_kernel(GaussLaunch L) {
  using S = GShape<N>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB, h = S::h, H = S::H;
  extern __shared__ double smem[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  const int64_t e = (int64_t)blockIdx.x * EPB + slot;
  const bool active = e < L.n_elem;
  double* F = smem + slot * S::SLOT;  // Pi, Phi_x, Phi_y, Phi_z of ucur
  double* Sacc = F + 4 * NP;         // running c * (dt Pi)
  double* T = Sacc + NP;             // three scaled split tables
  const int64_t off = e * (int64_t)(kVars * NP);
  const double c = L.c, g2 = L.gamma2;
  const double* u = L.ucur;

  double jd[3] = {0.0, 0.0, 0.0};
  if (active) {
    for (int d = 0; d < 3; ++d) jd[d] = L.jac[3 * e + d];
    for (int q = t; q < 4 * NP; q += NN) F[q] = u[off + NP + q];
    for (int q = t; q < 3 * TAB; q += NN) {
      const int d = q / TAB, r = q - d * TAB;
      double v;
      if (r < H * h)
        v = L.eo.A[r / h][r % h];
      else if (r < 2 * H * h)
        v = L.eo.B[(r - H * h) / h][(r - H * h) % h];
      else
        v = L.eo.M[r - 2 * H * h];
      T[q] = (-c * jd[d]) * v;
    }
  }
  __syncthreads();

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
      double up[N], uf[N], dF[N], dP[N], ps[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        up[i] = F[base + i * stride];
        uf[i] = F[(1 + d) * NP + base + i * stride];
        ps[i] = g2 != 0.0 ? u[off + base + i * stride] : 0.0;
      }
      const double* tab = T + d * TAB;
      dev::eo_line<N, double>(uf, dF, tab);  // -c J_d D Phi_d : part of c dt Pi
      dev::eo_line<N, double>(up, dP, tab);  // -c J_d D Pi    : c dt Phi_d
      if (kBoundary) {
        const int64_t nlo = (int64_t)L.nbr[6 * e + 2 * d] * (kVars * NP) + base;
        const int64_t nhi = (int64_t)L.nbr[6 * e + 2 * d + 1] * (kVars * NP) + base;
        double wi_lo = 0.0, wi_hi = 0.0, we_lo = 0.0, we_hi = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int64_t o = (int64_t)i * stride;
          // s = -1 on the lower face, +1 on the upper one (this element's s
          // for both sides of each face)
          wi_lo = fma(L.lo[i], up[i] + uf[i] - g2 * ps[i], wi_lo);
          wi_hi = fma(L.hi[i], up[i] - uf[i] - g2 * ps[i], wi_hi);
          double ep = u[nlo + NP + o], ef = u[nlo + (2 + d) * NP + o];
          double es = g2 != 0.0 ? u[nlo + o] : 0.0;
          we_lo = fma(L.hi[i], ep + ef - g2 * es, we_lo);
          ep = u[nhi + NP + o];
          ef = u[nhi + (2 + d) * NP + o];
          es = g2 != 0.0 ? u[nhi + o] : 0.0;
          we_hi = fma(L.lo[i], ep - ef - g2 * es, we_hi);
        }
        // lifted: c dt += -c |n| lift_i D, |n| = J_d; D_Pi = dw / 2,
        // D_Phi_d = -s D_Pi
        const double Gg = -0.5 * c * jd[d];
        const double dw_lo = wi_lo - we_lo, dw_hi = wi_hi - we_hi;
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const double lo = Gg * L.lift_lo[i] * dw_lo, hi = Gg * L.lift_hi[i] * dw_hi;
          dF[i] += lo + hi;
          dP[i] += lo - hi;
        }
      }
      if (g2 != 0.0) {
        // gamma2 (d_d Psi - Phi_d) of dt Phi_d (TimeDerivative.cpp:42-43)
        double dpsi[N];
        dev::eo_line<N, double>(ps, dpsi, tab);  // -c J_d D Psi
#pragma unroll
        for (int i = 0; i < N; ++i) dP[i] = fma(-g2, dpsi[i] + c * uf[i], dP[i]);
      }
      const int64_t vo = off + (2 + d) * NP + base;
#pragma unroll
      for (int i = 0; i < N; ++i) {
        double v = fma(L.b, uf[i], dP[i]);
        if (L.a != 0.0) v = fma(L.a, L.u0[vo + i * stride], v);
        L.unext[vo + i * stride] = v;
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
          const int64_t p = base + i * stride;
          const double sp = Sacc[p] + dF[i];
          double vpi = fma(L.b, up[i], sp);
          double vpsi = fma(L.b, u[off + p], -c * up[i]);
          if (L.a != 0.0) {
            vpi = fma(L.a, L.u0[off + NP + p], vpi);
            vpsi = fma(L.a, L.u0[off + p], vpsi);
          }
          L.unext[off + NP + p] = vpi;
          L.unext[off + p] = vpsi;
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

template <int N, bool kBoundary>
cudaError_t launch_n(const GaussLaunch& L, cudaStream_t s) {
  constexpr int EPB = gauss_epb<N>();
  const size_t smem = (size_t)EPB * GShape<N>::SLOT * sizeof(double);
  auto k = stage_gauss_kernel<N, EPB, kBoundary>;
  cudaError_t err =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  const int64_t blocks = (L.n_elem + EPB - 1) / EPB;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, N * N * EPB, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_b(const GaussLaunch& L, cudaStream_t s) {
  return L.boundary ? launch_n<N, true>(L, s) : launch_n<N, false>(L, s);
}

}  // namespace

cudaError_t launch_stage_gauss(const GaussLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_b<2>(L, s);
    case 3: return launch_b<3>(L, s);
    case 4: return launch_b<4>(L, s);
    case 5: return launch_b<5>(L, s);
    case 6: return launch_b<6>(L, s);
    case 7: return launch_b<7>(L, s);
    case 8: return launch_b<8>(L, s);
    case 9: return launch_b<9>(L, s);
    case 10: return launch_b<10>(L, s);
    case 11: return launch_b<11>(L, s);
    case 12: return launch_b<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
