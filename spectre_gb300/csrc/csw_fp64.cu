// csw_fp64.cu -- CurvedScalarWave on a static curved mesh: set-up kernels
// (Kerr-Schild background, per-point operator tables, face geometry, the
// excision check, initial data) and the plain FP64 fused right-hand side +
// SSP-RK3 substep.
//
// The right-hand side is CurvedScalarWave::TimeDerivative<3>
// (Evolution/Systems/CurvedScalarWave/TimeDerivative.cpp:47-68) applied to
// the partial derivatives d_i u = (d xi^a / d x^i) d_a u of the five fields
// (PartialDerivatives.tpp:315-363), plus the UpwindPenalty correction of every
// internal mortar (CurvedScalarWave/BoundaryCorrections/UpwindPenalty.cpp:
// 35-146) lifted onto the GLL face (LiftFlux.hpp:57-61), plus the
// ConstraintPreservingSphericalRadiation time-derivative correction on the
// outer sphere (ConstraintPreservingSphericalRadiation.cpp:40-156; it is
// added to dt u without lifting, from the volume time derivative, as
// BoundaryConditionsImpl.hpp:398 does).  The inner sphere's
// DemandOutgoingCharSpeeds adds nothing; its check depends only on the static
// background and the normal, so it runs once, at set-up.
//
// The background is static (CalculateGrVars is skipped for time-independent
// blocks), so every background- and geometry-dependent coefficient of the
// right-hand side is formed once per point in FP64 at set-up.  With
// g_{v,a} = d_a u_v the logical derivatives and
//   B^a = (d xi^a/d x^i) beta^i,  A_{ai} = alpha d xi^a/d x^i,
//   G^{aj} = alpha gamma^{ij} d xi^a/d x^i,
//   C^i = alpha Gamma^i - gamma^{ij} d_j alpha,
// the time derivative is
//   dt Psi   = (1+g1) B^a g_{Psi,a} - alpha Pi - g1 beta.Phi
//   dt Pi    = B^a (g_{Pi,a} + g1 g2 g_{Psi,a}) - G^{aj} g_{Phi_j,a}
//              + alpha K Pi + C^i Phi_i - g1 g2 beta.Phi
//   dt Phi_i = A_{ai} (g2 g_{Psi,a} - g_{Pi,a}) + B^a g_{Phi_i,a}
//              - g2 alpha Phi_i - Pi d_i alpha + (d_i beta^j) Phi_j
// which is the reference's expression with the sums regrouped.
//
// Work split (plain FP64): one block of 256 threads per element.  The state
// of the element sits in shared memory; three rounds follow, one per logical
// axis a.  In round a the block forms the five derivatives along a with the
// even/odd split of D (one line per task) into shared memory, then every
// thread folds them into the running dt of the points it owns.  The last
// phase adds the non-derivative terms, the face corrections (the neighbour's
// face values are read from its volume data through a precomputed point
// index, which carries the orientation of the wedge interface) and the
// radiation condition, and writes u_next = a u0 + b ucur + c L(ucur).
#include <cmath>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------- set-up --

// Schwarzschild in Kerr-Schild coordinates (gr::Solutions::KerrSchild with
// zero spin at the origin), the spatial quantities CalculateGrVars asks for.
// The closed forms are those Test_KerrSchild.cpp:55-232 checks:
//   alpha = (1 + 2M/r)^-1/2, beta^i = 2M x^i / r^2 alpha^2,
//   d_i alpha = M x_i / r^3 alpha^3,
//   d_i beta^j = 2M/r^2 alpha^2 delta_ij - 4M x_i x_j / r^4 alpha^2 (1 - M alpha^2 / r),
//   gamma^ij = delta^ij - 2M x^i x^j / (r^2 (r + 2M)),
//   Gamma^i = M (8M + 3r) x^i / ((2M + r)^2 r^2),  K = 2M (3M + r) ((2M + r) r)^-3/2.
__global__ void csw_background_kernel(const double* __restrict__ xyz, double mass,
                                      double* __restrict__ bg, int64_t n_elem, int np) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_elem * np) return;
  const int64_t e = idx / np;
  const int64_t p = idx - e * np;
  const double* X = xyz + e * 3 * np + p;
  double* out = bg + e * kBgFields * np + p;
  const double x[3] = {X[0], X[np], X[2 * np]};
  const double M = mass;
  const double r2 = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
  const double r = sqrt(r2);
  const double l2 = 1.0 / (1.0 + 2.0 * M / r);
  const double lapse = sqrt(l2);
  out[0] = lapse;
  for (int i = 0; i < 3; ++i) out[(1 + i) * np] = 2.0 * M * x[i] / r2 * l2;
  for (int i = 0; i < 3; ++i) out[(4 + i) * np] = M * x[i] / (r2 * r) * l2 * lapse;
  const double diag = 2.0 * M / r2 * l2;
  const double off = 4.0 * M / (r2 * r2) * l2 * (1.0 - M / r * l2);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out[(7 + 3 * i + j) * np] = (i == j ? diag : 0.0) - off * x[i] * x[j];
  const double g = 2.0 * M / (r2 * (r + 2.0 * M));
  const int pi_[6] = {0, 0, 0, 1, 1, 2}, pj_[6] = {0, 1, 2, 1, 2, 2};
  for (int q = 0; q < 6; ++q)
    out[(16 + q) * np] = (pi_[q] == pj_[q] ? 1.0 : 0.0) - g * x[pi_[q]] * x[pj_[q]];
  const double f = M * (8.0 * M + 3.0 * r) / ((2.0 * M + r) * (2.0 * M + r) * r2);
  for (int i = 0; i < 3; ++i) out[(22 + i) * np] = f * x[i];
  const double s = (2.0 * M + r) * r;
  out[25 * np] = 2.0 * M * (3.0 * M + r) / (s * sqrt(s));
}

__device__ __forceinline__ double inv_metric(const double* b, int np, int i, int j) {
  const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  return b[(16 + idx[i][j]) * np];
}

// Per-point coefficient table (kCswT entries, layout in launch.hpp).
__global__ void csw_table_kernel(const double* __restrict__ ij, const double* __restrict__ bg,
                                 double* __restrict__ T, float* __restrict__ T32,
                                 int64_t n_elem, int np) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_elem * np) return;
  const int64_t e = idx / np;
  const int64_t p = idx - e * np;
  const double* J = ij + e * 9 * np + p;
  const double* b = bg + e * kBgFields * np + p;
  double* out = T + e * kCswT * np + p;
  double v[kCswT];
  const double lapse = b[0];
  double shift[3], dl[3];
  for (int i = 0; i < 3; ++i) {
    shift[i] = b[(1 + i) * np];
    dl[i] = b[(4 + i) * np];
  }
  for (int a = 0; a < 3; ++a) {
    double s = 0.0;
    for (int i = 0; i < 3; ++i) s = fma(J[(3 * a + i) * np], shift[i], s);
    v[kTB + a] = s;
    for (int i = 0; i < 3; ++i) v[kTA + 3 * a + i] = lapse * J[(3 * a + i) * np];
    for (int j = 0; j < 3; ++j) {
      double g = 0.0;
      for (int i = 0; i < 3; ++i) g = fma(inv_metric(b, np, i, j), J[(3 * a + i) * np], g);
      v[kTG + 3 * a + j] = lapse * g;
    }
  }
  v[kTK] = lapse * b[25 * np];
  for (int i = 0; i < 3; ++i) {
    double c = lapse * b[(22 + i) * np];
    for (int j = 0; j < 3; ++j) c = fma(-inv_metric(b, np, i, j), dl[j], c);
    v[kTC + i] = c;
    v[kTDl + i] = dl[i];
    for (int j = 0; j < 3; ++j) v[kTDs + 3 * i + j] = b[(7 + 3 * i + j) * np];
    v[kTBeta + i] = shift[i];
  }
  v[kTLapse] = lapse;
  for (int c = 0; c < kCswT; ++c) {
    out[c * np] = v[c];
    if (T32) T32[e * kCswT * np + c * np + p] = (float)v[c];
  }
}

// Face geometry per face point (kCswF entries, layout in launch.hpp): the
// unit normal covector n_i = s (d xi^d/d x^i) / |.|, the vector n^i =
// gamma^ij n_j and |.| = sqrt(gamma^ij (d xi^d/d x^i)(d xi^d/d x^j))
// (NormalCovectorAndMagnitude.hpp:57-84), and the four upwind weights
// min(lambda_k, 0) times the lift factor -N(N-1)/2 |.| (LiftFlux.hpp:57-61)
// for the characteristic speeds lambda = (-(1+g1) beta.n, -beta.n,
// -beta.n + alpha, -beta.n - alpha) (Characteristics.cpp:20-50).  On the
// inner sphere every speed must be outgoing (DemandOutgoingCharSpeeds.cpp:
// 40-77); a violation sets *excision.
__global__ void csw_face_kernel(const double* __restrict__ ij, const double* __restrict__ bg,
                                const int32_t* __restrict__ nbr, int n, double gamma1,
                                double* __restrict__ F, float* __restrict__ F32,
                                int* __restrict__ excision, int64_t n_elem) {
  const int nn = n * n, np = nn * n;
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_elem * 6 * nn) return;
  const int64_t ef = idx / nn;  // e * 6 + dir
  const int q = (int)(idx - ef * nn);
  const int64_t e = ef / 6;
  const int dir = (int)(ef - e * 6);
  const int d = dir >> 1;
  const int fa = q % n, fb = q / n;
  const int sl = (dir & 1) ? n - 1 : 0;
  const int p = d == 0 ? sl + n * (fa + n * fb) : (d == 1 ? fa + n * (sl + n * fb) : fa + n * (fb + n * sl));
  const double* J = ij + e * 9 * np + p;
  const double* b = bg + e * kBgFields * np + p;
  const double sgn = (dir & 1) ? 1.0 : -1.0;
  double un[3], vec[3];
  for (int i = 0; i < 3; ++i) un[i] = sgn * J[(3 * d + i) * np];
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int j = 0; j < 3; ++j) s = fma(inv_metric(b, np, i, j), un[j], s);
    vec[i] = s;
  }
  const double mag = sqrt(un[0] * vec[0] + un[1] * vec[1] + un[2] * vec[2]);
  double v[kCswF];
  double bn = 0.0;
  for (int i = 0; i < 3; ++i) {
    v[kFn + i] = un[i] / mag;
    v[kFv + i] = vec[i] / mag;
    bn = fma(b[(1 + i) * np], v[kFn + i], bn);
  }
  const double lapse = b[0];
  const double lam[4] = {-(1.0 + gamma1) * bn, -bn, -bn + lapse, -bn - lapse};
  const double fac = -0.5 * (double)(n * (n - 1)) * mag;
  for (int k = 0; k < 4; ++k) v[kFm + k] = fac * fmin(lam[k], 0.0);
  double* out = F + ef * kCswF * nn + q;
  for (int c = 0; c < kCswF; ++c) {
    out[c * nn] = v[c];
    if (F32) F32[ef * kCswF * nn + c * nn + q] = (float)v[c];
  }
  if (nbr[ef] == -1 && (lam[0] < 0.0 || lam[1] < 0.0 || lam[2] < 0.0 || lam[3] < 0.0))
    atomicOr(excision, 1);
}

// Spherical Gaussian shell psi = A exp(-(r - r0)^2 / w^2), Pi = 0, Phi = grad psi.
__global__ void csw_initial_kernel(const double* __restrict__ xyz, double A, double r0, double w,
                                   double* __restrict__ u, int64_t n_elem, int np) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n_elem * np) return;
  const int64_t e = idx / np;
  const int64_t p = idx - e * np;
  const double* X = xyz + e * 3 * np + p;
  const double x[3] = {X[0], X[np], X[2 * np]};
  const double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
  const double z = (r - r0) / w;
  const double psi = A * exp(-z * z);
  double* U = u + e * kVars * np + p;
  U[0] = psi;
  U[np] = 0.0;
  const double f = -2.0 * z / w * psi / r;
  for (int i = 0; i < 3; ++i) U[(2 + i) * np] = f * x[i];
}

// ------------------------------------------------------------ FP64 stage --

template <int N>
struct CswShape {
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = 2 * dev::Eo<N>::H * dev::Eo<N>::h + dev::Eo<N>::H;
  static constexpr int PTS = (NP + kThreads - 1) / kThreads;  // points per thread
  // shared doubles: state, one axis of derivatives (afterwards the
  // internal-face corrections [6][5][N^2]), the outer layer's logical
  // derivatives of Psi and Phi (for the radiation condition), table
  static constexpr int GA = 5 * NP > 30 * NN ? 5 * NP : 30 * NN;
  static constexpr int SMEM = 5 * NP + GA + 12 * NN + TAB;
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

// UpwindPenalty correction (already lifted) at one internal face point, in
// closed form for an exterior side that shares the point, the background
// and the (negated) normal: with d = exterior - interior,
//   Psi:  m0 d_Psi
//   Pi:   (t1 - t2)/2 + g2 m0 d_Psi
//   Phi:  -(t1 + t2)/2 n_i + m1 (d_Phi_i - n_i n^j d_Phi_j)
//   t1 = m3 (d_Pi - n^j d_Phi_j - g2 d_Psi),  t2 = -m2 (d_Pi + n^j d_Phi_j - g2 d_Psi)
// (UpwindPenalty.cpp:77-127 with the exterior speeds -lambda of the interior
// ones; m_k are the lifted weights of csw_face_kernel).
template <typename T>
__device__ __forceinline__ void upwind_face(const T (&ui)[5], const T (&ue)[5], const T* f,
                                            int nn, T gamma2, T (&acc)[5]) {
  const T dpsi = ue[0] - ui[0];
  const T dpi = ue[1] - ui[1];
  T dphi[3];
  T ndp = 0;
  for (int i = 0; i < 3; ++i) {
    dphi[i] = ue[2 + i] - ui[2 + i];
    ndp = fma(f[(kFv + i) * nn], dphi[i], ndp);
  }
  const T m0 = f[(kFm + 0) * nn], m1 = f[(kFm + 1) * nn];
  const T m2 = f[(kFm + 2) * nn], m3 = f[(kFm + 3) * nn];
  const T g2p = gamma2 * dpsi;
  const T t1 = m3 * (dpi - ndp - g2p);
  const T t2 = -m2 * (dpi + ndp - g2p);
  const T cpsi = m0 * dpsi;
  acc[0] += cpsi;
  acc[1] += fma(gamma2, cpsi, T(0.5) * (t1 - t2));
  const T h = T(-0.5) * (t1 + t2);
  for (int i = 0; i < 3; ++i) {
    const T ni = f[(kFn + i) * nn];
    acc[2 + i] += fma(h, ni, m1 * fma(-ni, ndp, dphi[i]));
  }
}

template <int N, bool kBoundary>
__global__ void __launch_bounds__(kThreads, CswShape<N>::SMEM * 8 <= 113 * 1024 ? 2 : 1)
    csw_stage_fp64_kernel(CswLaunch L) {
  using S = CswShape<N>;
  constexpr int NN = S::NN, NP = S::NP, PTS = S::PTS;
  extern __shared__ double smem[];
  double* U = smem;          // 5 * NP: ucur of this element
  double* Ga = U + 5 * NP;   // 5 * NP: d_a of the five fields, one axis at a time
  double* Go = Ga + S::GA;   // 12 * NN: outer layer d_a Psi, d_a Phi_j ([a][4][NN])
  double* tab = Go + 12 * NN;
  const int64_t e = L.list ? (int64_t)L.list[blockIdx.x] : (int64_t)blockIdx.x;
  const int tid = threadIdx.x;
  const int64_t off = e * (int64_t)(kVars * NP);
  const bool outer = kBoundary && L.nbr[6 * e + 5] == -2;
  for (int q = tid; q < 5 * NP; q += kThreads) U[q] = L.ucur[off + q];
  for (int q = tid; q < S::TAB; q += kThreads) {
    constexpr int h = dev::Eo<N>::h, H = dev::Eo<N>::H;
    double v;
    if (q < H * h)
      v = L.eo.A[q / h][q % h];
    else if (q < 2 * H * h)
      v = L.eo.B[(q - H * h) / h][(q - H * h) % h];
    else
      v = L.eo.M[q - 2 * H * h];
    tab[q] = v;
  }
  const double* T = L.T + e * (int64_t)kCswT * NP;
  const double g1 = L.gamma1, g2 = L.gamma2;
  if (L.frec) {
    // AdamsBashforth record: the element's face values, [6][5][N^2]
    __syncthreads();  // U staged
    for (int fp = tid; fp < 6 * NN; fp += kThreads) {
      const int dir = fp / NN, q = fp - (fp / NN) * NN, d = dir >> 1;
      const int sl = (dir & 1) ? N - 1 : 0, fa = q % N, fb = q / N;
      const int p = d == 0 ? sl + N * (fa + N * fb)
                           : (d == 1 ? fa + N * (sl + N * fb) : fa + N * (fb + N * sl));
#pragma unroll
      for (int v = 0; v < 5; ++v) L.frec[e * 30 * NN + (dir * 5 + v) * NN + q] = U[v * NP + p];
    }
  }

  double acc[PTS][5];
#pragma unroll
  for (int r = 0; r < PTS; ++r)
#pragma unroll
    for (int v = 0; v < 5; ++v) acc[r][v] = 0.0;

#pragma unroll 1
  for (int a = 0; a < 3; ++a) {
    __syncthreads();  // U ready (a = 0); previous round's Ga consumed
    for (int task = tid; task < 5 * NN; task += kThreads) {
      const int v = task / NN, line = task - v * NN;
      int base, stride;
      line_geometry<N>(a, line, base, stride);
      double u[N], du[N];
#pragma unroll
      for (int i = 0; i < N; ++i) u[i] = U[v * NP + base + i * stride];
      dev::eo_line<N, double>(u, du, tab);
#pragma unroll
      for (int i = 0; i < N; ++i) Ga[v * NP + base + i * stride] = du[i];
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < PTS; ++r) {
      const int p = tid + r * kThreads;
      if (p < NP) {
        const double gpsi = Ga[p], gpi = Ga[NP + p];
        const double gf[3] = {Ga[2 * NP + p], Ga[3 * NP + p], Ga[4 * NP + p]};
        const double B = T[(kTB + a) * NP + p];
        acc[r][0] = fma(B, gpsi, acc[r][0]);
        double s = fma(g1 * g2, gpsi, gpi);
        s = B * s;
#pragma unroll
        for (int j = 0; j < 3; ++j) s = fma(-T[(kTG + 3 * a + j) * NP + p], gf[j], s);
        acc[r][1] += s;
        const double hh = fma(g2, gpsi, -gpi);
#pragma unroll
        for (int i = 0; i < 3; ++i)
          acc[r][2 + i] = fma(T[(kTA + 3 * a + i) * NP + p], hh, fma(B, gf[i], acc[r][2 + i]));
        if (outer && p >= NP - NN) {
          const int q = p - (NP - NN);
          Go[(4 * a + 0) * NN + q] = gpsi;
#pragma unroll
          for (int j = 0; j < 3; ++j) Go[(4 * a + 1 + j) * NN + q] = gf[j];
        }
      }
    }
  }
  __syncthreads();  // Go complete, Ga free

  // UpwindPenalty corrections of the internal faces, one thread per face
  // point, into Ga ([dir][var][N^2]): every exterior gather of the element
  // issued together rather than point by point
  double* Cf = Ga;
  const bool internal = kBoundary && L.internal;
  if (internal) {
    for (int fp = tid; fp < 6 * NN; fp += kThreads) {
      const int dir = fp / NN, q = fp - (fp / NN) * NN, d = dir >> 1;
      const int sl = (dir & 1) ? N - 1 : 0, fa = q % N, fb = q / N;
      const int p = d == 0 ? sl + N * (fa + N * fb)
                           : (d == 1 ? fa + N * (sl + N * fb) : fa + N * (fb + N * sl));
      const int64_t ef = e * 6 + dir;
      const int32_t x = L.X[ef * NN + q];
      double c[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      if (x >= 0) {
        double ui[5], ue[5];
#pragma unroll
        for (int v = 0; v < 5; ++v) {
          ui[v] = U[v * NP + p];
          ue[v] = L.ucur[x + (int64_t)v * NP];
        }
        upwind_face<double>(ui, ue, L.F + ef * kCswF * NN + q, NN, g2, c);
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) Cf[(dir * 5 + v) * NN + q] = c[v];
    }
    __syncthreads();
  }

#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int p = tid + r * kThreads;
    if (p >= NP) continue;
    const double psi = U[p], pi = U[NP + p];
    const double phi[3] = {U[2 * NP + p], U[3 * NP + p], U[4 * NP + p]};
    const double lapse = T[kTLapse * NP + p];
    double dt[5];
    double bphi = 0.0;
    if (g1 != 0.0)
      for (int i = 0; i < 3; ++i) bphi = fma(T[(kTBeta + i) * NP + p], phi[i], bphi);
    dt[0] = fma(-g1, bphi, fma(1.0 + g1, acc[r][0], -lapse * pi));
    double s = fma(T[kTK * NP + p], pi, acc[r][1]);
    for (int i = 0; i < 3; ++i) s = fma(T[(kTC + i) * NP + p], phi[i], s);
    dt[1] = fma(-g1 * g2, bphi, s);
    for (int i = 0; i < 3; ++i) {
      double v = fma(-g2 * lapse, phi[i], acc[r][2 + i]);
      v = fma(-pi, T[(kTDl + i) * NP + p], v);
      for (int j = 0; j < 3; ++j) v = fma(T[(kTDs + 3 * i + j) * NP + p], phi[j], v);
      dt[2 + i] = v;
    }
    if (kBoundary) {
      const int i = p % N, j = (p / N) % N, k = p / NN;
      double corr[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      const int dirs[6] = {i == 0 ? 0 : -1, i == N - 1 ? 1 : -1, j == 0 ? 2 : -1,
                           j == N - 1 ? 3 : -1, k == 0 ? 4 : -1, k == N - 1 ? 5 : -1};
      const int fq[3] = {j + N * k, i + N * k, i + N * j};
#pragma unroll
      for (int s6 = 0; s6 < 6; ++s6) {
        const int dir = dirs[s6];
        if (dir < 0) continue;
        const int q = fq[dir >> 1];
        const int64_t ef = e * 6 + dir;
        const double* f = L.F + ef * kCswF * NN + q;
        if (internal) {
#pragma unroll
          for (int v = 0; v < 5; ++v) corr[v] += Cf[(dir * 5 + v) * NN + q];
        }
        if (dir == 5 && outer) {
          // ConstraintPreservingSphericalRadiation::dg_time_derivative from
          // the volume dt (only zeta-upper faces lie on the outer sphere)
          const double* J = L.ij + e * 9 * (int64_t)NP + p;
          double dpsi[3], dphi[3][3];  // d_i Psi, d_i Phi_j
#pragma unroll
          for (int ii = 0; ii < 3; ++ii) {
            double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
              const double Jai = J[(3 * a + ii) * NP];
              s0 = fma(Jai, Go[(4 * a + 0) * NN + q], s0);
              s1 = fma(Jai, Go[(4 * a + 1) * NN + q], s1);
              s2 = fma(Jai, Go[(4 * a + 2) * NN + q], s2);
              s3 = fma(Jai, Go[(4 * a + 3) * NN + q], s3);
            }
            dpsi[ii] = s0;
            dphi[ii][0] = s1;
            dphi[ii][1] = s2;
            dphi[ii][2] = s3;
          }
          const double* X3 = L.xyz + e * 3 * (int64_t)NP + p;
          const double rr = sqrt(X3[0] * X3[0] + X3[NP] * X3[NP] + X3[2 * NP] * X3[2 * NP]);
          const double ir = 1.0 / rr;
          double nv[3], nc[3], beta[3], bn = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            nv[c] = f[(kFv + c) * NN];
            nc[c] = f[(kFn + c) * NN];
            beta[c] = T[(kTBeta + c) * NP + p];
            bn = fma(beta[c], nc[c], bn);
          }
          const double l0 = fmin(-(1.0 + g1) * bn, 0.0), l1 = fmin(-bn, 0.0);
          double cpsi = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c) cpsi = fma(nv[c], dpsi[c] - phi[c], cpsi);
          cpsi *= l0;
          corr[0] += cpsi;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            double v = 0.0;
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) v = fma(nv[jj], dphi[jj][c] - dphi[c][jj], v);
            corr[2 + c] += l1 * v;
          }
          double cpi = fma(2.0 * ir, psi, 4.0 * dt[0]) * ir;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            cpi = fma(nv[c], fma(2.0, dt[2 + c], 4.0 * ir * phi[c]), cpi);
            cpi = fma(beta[c], dt[2 + c], cpi);
#pragma unroll
            for (int jj = 0; jj < 3; ++jj) cpi = fma(nv[c] * nv[jj], dphi[c][jj], cpi);
          }
          cpi /= lapse;
          corr[1] += fma(g2, cpsi, cpi - dt[1]);
        }
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) dt[v] += corr[v];
    }
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      const double uc = (v == 0) ? psi : (v == 1 ? pi : phi[v - 2]);
      double o = fma(L.b, uc, L.c * dt[v]);
      if (L.a != 0.0) o = fma(L.a, L.u0[off + v * NP + p], o);
      L.unext[off + v * NP + p] = o;
    }
  }
}

// AdamsBashforth on the shell, one element per block: u (or the initial
// values on a self-start reset) plus sum_j c_j F_j, plus on every internal
// face point the curved UpwindPenalty of the marginal-weighted records.
// The correction is linear in the exterior-minus-interior jump with static
// weights (csw_face_kernel), so sum_{l,r} c_lr C(L_l, R_r) =
// C(sum_l a_l L_l, sum_r b_r R_r).  The records hold each element's face
// values ([6][5][N^2]); the exterior record point is the offset X of the
// neighbour's matching face point in the same ring slot.
template <int N>
__global__ void __launch_bounds__(kThreads) csw_ab_update_kernel(const __grid_constant__ CswAbArgs A) {
  constexpr int NN = N * N, NP = NN * N;
  int64_t g = blockIdx.x;
  int j = -1;
  for (int q = 0; q < A.L.n_jobs; ++q) {
    if (g < A.L.job[q].count) {
      j = q;
      break;
    }
    g -= A.L.job[q].count;
  }
  if (j < 0) return;  // uniform over the block, before its one barrier
  const AbLevelJob& J = A.L.job[j];
  const int64_t e = A.list[J.begin + g];
  const int64_t per = (int64_t)kVars * NP, E = A.n_elem;
  const int64_t off = e * per;
  const bool update = J.update && !J.reset;
  if (!update && !J.reset) return;
  const double* src = J.reset ? A.u0 : A.u;
  // the boundary delta of every internal face point first, one thread per
  // face point, into shared memory ([dir][var][N^2]): the record gathers of
  // the whole element issued together
  __shared__ double Cf[6 * 5 * NN];
  if (update) {
    for (int fp = threadIdx.x; fp < 6 * NN; fp += kThreads) {
      const int dir = fp / NN, q = fp - (fp / NN) * NN;
      const int64_t ef = e * 6 + dir;
      const int32_t x = A.X[ef * NN + q];
      double corr[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      if (x >= 0) {  // external faces: their condition is in the time derivative
        const int64_t rs = E * 30 * (int64_t)NN;  // one ring slot of face records
        const AbFaceTable& f = J.face[A.level[x / (30 * NN)]];
        double ui[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, ue[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int i = 0; i < f.n_loc; ++i) {
          const double* Ul = A.U + (int64_t)f.loc_slot[i] * rs + e * 30 * NN + dir * 5 * NN + q;
#pragma unroll
          for (int v = 0; v < 5; ++v) ui[v] = fma(f.loc_c[i], Ul[v * NN], ui[v]);
        }
        for (int i = 0; i < f.n_rem; ++i) {
          const double* Ur = A.U + (int64_t)f.rem_slot[i] * rs + x;
#pragma unroll
          for (int v = 0; v < 5; ++v) ue[v] = fma(f.rem_c[i], Ur[v * NN], ue[v]);
        }
        if (A.Fc32) {
          // mixed precision: the jumps rounded to FP32 once, the correction
          // in FP32 with the FP32 face table
          float z[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f}, dv[5], c32[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
          for (int v = 0; v < 5; ++v) dv[v] = (float)(ue[v] - ui[v]);
          upwind_face<float>(z, dv, A.Fc32 + ef * kCswF * NN + q, NN, (float)A.gamma2, c32);
#pragma unroll
          for (int v = 0; v < 5; ++v) corr[v] = c32[v];
        } else {
          upwind_face<double>(ui, ue, A.Fc + ef * kCswF * NN + q, NN, A.gamma2, corr);
        }
      }
#pragma unroll
      for (int v = 0; v < 5; ++v) Cf[(dir * 5 + v) * NN + q] = corr[v];
    }
    __syncthreads();  // update is uniform over the block
  }
  // every point of this thread at once: the state loads, then each
  // record's loads, issued together (the stores alias the state)
  constexpr int PTS = (NP + kThreads - 1) / kThreads;
  double val[PTS][5];
#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int p = threadIdx.x + r * kThreads;
    if (p < NP)
#pragma unroll
      for (int v = 0; v < 5; ++v) val[r][v] = src[off + v * NP + p];
  }
  if (update) {
    // the 0-3 face corrections of point p, summed in a fixed order
    auto face_sum = [&](int p, double (&corr)[5]) {
      const int i0 = p % N, j0 = (p / N) % N, k0 = p / NN;
      const int dirs[6] = {i0 == 0 ? 0 : -1, i0 == N - 1 ? 1 : -1, j0 == 0 ? 2 : -1,
                           j0 == N - 1 ? 3 : -1, k0 == 0 ? 4 : -1, k0 == N - 1 ? 5 : -1};
      const int fq[3] = {j0 + N * k0, i0 + N * k0, i0 + N * j0};
#pragma unroll
      for (int v = 0; v < 5; ++v) corr[v] = 0.0;
#pragma unroll
      for (int s6 = 0; s6 < 6; ++s6) {
        const int dir = dirs[s6];
        if (dir < 0) continue;
        const int q = fq[dir >> 1];
#pragma unroll
        for (int v = 0; v < 5; ++v) corr[v] += Cf[(dir * 5 + v) * NN + q];
      }
    };
    if (A.F32) {
      // mixed precision: the increment sum_j c_j F_j and the face
      // corrections in FP32 (the records' own precision), added to the FP64
      // state once
      float inc[PTS][5];
#pragma unroll
      for (int r = 0; r < PTS; ++r)
#pragma unroll
        for (int v = 0; v < 5; ++v) inc[r][v] = 0.0f;
      for (int i = 0; i < J.n_vol; ++i) {
        const float c = (float)J.vol_c[i];
        const int64_t fo = ((int64_t)J.vol_slot[i] * E + e) * per;
#pragma unroll
        for (int r = 0; r < PTS; ++r) {
          const int p = threadIdx.x + r * kThreads;
          if (p >= NP) continue;
#pragma unroll
          for (int v = 0; v < 5; ++v) inc[r][v] = fmaf(c, A.F32[fo + v * NP + p], inc[r][v]);
        }
      }
#pragma unroll
      for (int r = 0; r < PTS; ++r) {
        const int p = threadIdx.x + r * kThreads;
        if (p >= NP) continue;
        double corr[5];
        face_sum(p, corr);  // FP32 values: their sums below are FP32 sums
#pragma unroll
        for (int v = 0; v < 5; ++v) val[r][v] += dev::widen(inc[r][v] + (float)corr[v]);
      }
    } else {
      for (int i = 0; i < J.n_vol; ++i) {
        const double c = J.vol_c[i];
        const int64_t fo = ((int64_t)J.vol_slot[i] * E + e) * per;
#pragma unroll
        for (int r = 0; r < PTS; ++r) {
          const int p = threadIdx.x + r * kThreads;
          if (p >= NP) continue;
#pragma unroll
          for (int v = 0; v < 5; ++v) val[r][v] = fma(c, A.F[fo + v * NP + p], val[r][v]);
        }
      }
#pragma unroll
      for (int r = 0; r < PTS; ++r) {
        const int p = threadIdx.x + r * kThreads;
        if (p >= NP) continue;
        double corr[5];
        face_sum(p, corr);
#pragma unroll
        for (int v = 0; v < 5; ++v) val[r][v] += corr[v];
      }
    }
  }
#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int p = threadIdx.x + r * kThreads;
    if (p < NP)
#pragma unroll
      for (int v = 0; v < 5; ++v) A.u[off + v * NP + p] = val[r][v];
  }
}

template <int N, bool kBoundary>
cudaError_t launch_fp64_n(const CswLaunch& L, cudaStream_t s) {
  const size_t smem = (size_t)CswShape<N>::SMEM * sizeof(double);
  auto k = csw_stage_fp64_kernel<N, kBoundary>;
  cudaError_t err =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  err = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  const int64_t blocks = L.list ? L.list_count : L.n_elem;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, kThreads, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_fp64_mode(const CswLaunch& L, cudaStream_t s) {
  return L.boundary ? launch_fp64_n<N, true>(L, s) : launch_fp64_n<N, false>(L, s);
}

unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

cudaError_t launch_csw_fp64(const CswLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_fp64_mode<2>(L, s);
    case 3: return launch_fp64_mode<3>(L, s);
    case 4: return launch_fp64_mode<4>(L, s);
    case 5: return launch_fp64_mode<5>(L, s);
    case 6: return launch_fp64_mode<6>(L, s);
    case 7: return launch_fp64_mode<7>(L, s);
    case 8: return launch_fp64_mode<8>(L, s);
    case 9: return launch_fp64_mode<9>(L, s);
    case 10: return launch_fp64_mode<10>(L, s);
    case 11: return launch_fp64_mode<11>(L, s);
    case 12: return launch_fp64_mode<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_csw_ab_update(const CswAbArgs& A, cudaStream_t s) {
  int64_t total = 0;
  for (int q = 0; q < A.L.n_jobs; ++q) total += A.L.job[q].count;
  if (total <= 0) return cudaSuccess;
  switch (A.n) {
#define DGSW_CSW_AB(NV) \
  case NV: csw_ab_update_kernel<NV><<<(unsigned)total, kThreads, 0, s>>>(A); break;
    DGSW_CSW_AB(2) DGSW_CSW_AB(3) DGSW_CSW_AB(4) DGSW_CSW_AB(5) DGSW_CSW_AB(6) DGSW_CSW_AB(7)
    DGSW_CSW_AB(8) DGSW_CSW_AB(9) DGSW_CSW_AB(10) DGSW_CSW_AB(11) DGSW_CSW_AB(12)
#undef DGSW_CSW_AB
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_csw_setup(const CswSetup& S, cudaStream_t s) {
  const int np = S.n * S.n * S.n, nn = S.n * S.n;
  const int th = 256;
  if (S.n_elem <= 0) return cudaSuccess;
  csw_background_kernel<<<blocks_for(S.n_elem * np, th), th, 0, s>>>(S.xyz, S.mass, S.bg,
                                                                       S.n_elem, np);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  csw_table_kernel<<<blocks_for(S.n_elem * np, th), th, 0, s>>>(S.ij, S.bg, S.T, S.T32,
                                                                  S.n_elem, np);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  csw_face_kernel<<<blocks_for(S.n_elem * 6 * nn, th), th, 0, s>>>(
      S.ij, S.bg, S.nbr, S.n, S.gamma1, S.F, S.F32, S.excision, S.n_elem);
  return cudaGetLastError();
}

cudaError_t launch_csw_initial(const double* xyz, int n, int64_t n_elem, double A, double r0,
                               double w, double* u, cudaStream_t s) {
  const int np = n * n * n;
  if (n_elem <= 0) return cudaSuccess;
  csw_initial_kernel<<<blocks_for(n_elem * np, 256), 256, 0, s>>>(xyz, A, r0, w, u, n_elem, np);
  return cudaGetLastError();
}

}  // namespace dgsw
