// adjoint_fp64.cu -- discrete adjoint of the plain FP64 DG operator (uniform
// extent N, conforming mortars, affine mesh, gamma2 = 0) and the point
// sampler used by the misfit objective.
//
// The semi-discrete operator of stage_fp64.cu,
//   (L u)_Psi = -Pi,  (L u)_Pi = -sum_d J_d D_d Phi_d + B_Pi,
//   (L u)_Phi_d = -J_d D_d Pi + B_Phi_d,
// is linear.  Its exact transpose is
//   (L^T l)_Psi = 0,
//   (L^T l)_Pi = -l_Psi - sum_d J_d D_d^T l_Phi_d + B^T_Pi,
//   (L^T l)_Phi_d = -J_d D_d^T l_Pi + B^T_Phi_d,
// where D^T is again centro-antisymmetric (so the even/odd split applies)
// and the face part B (UpwindPenalty lifted with G = -c N(N-1) J_d / 4:
// dPi += G (w_int - w_ext), dPhi_d += -s G (w_int - w_ext), w = Pi - s Phi_d)
// transposes, at each face point shared with a neighbour, to
//   q  = G (l_Pi - s l_Phi_d)            (this element's own face term)
//   q' = G (l_Pi,nbr + s l_Phi_d,nbr)    (the neighbour's face term, whose
//                                         exterior is this element)
//   dPi += q - q',   dPhi_d += -s (q + q').
// One launch computes out = alpha X + beta Y + c L^T X and, optionally, a
// second pointwise combination out2 = alpha2 X + beta2 Y, which is what one
// step of the adjoint of Rk3HesthavenSsp needs (three launches per step).
// Two work splits give the same bits (AdjointLaunch::variant): N^2 threads
// per element and the three axes in turn, or 3 N^2 threads per element and
// the axes at once (more threads for the same work, for small grids).
#include <cstdint>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

using dev::Eo;

template <int N>
struct AShape {
  static constexpr int NN = N * N, NP = N * N * N;
  static constexpr int TAB = Eo<N>::TAB;
  static constexpr int SLOT = 5 * NP + 3 * TAB;   // doubles: X (Pi, Phi), S, tables
  static constexpr int SLOT3 = 7 * NP + 3 * TAB;  // split: X, three axis sums, tables
};

// X's Pi and Phi into shared memory and the three split tables of D^T scaled
// by -c (d xi_d/dx_d)
template <int N>
__device__ __forceinline__ void adj_prologue(const AdjointLaunch& L, int64_t off,
                                             const double (&jd)[3], double* F, double* T, int tid,
                                             int nthreads) {
  using S = AShape<N>;
  constexpr int NP = S::NP, TAB = S::TAB;
  constexpr int h = Eo<N>::h, H = Eo<N>::H;
  const double* src = L.x + off + NP;
  for (int q = tid; q < 4 * NP; q += nthreads) F[q] = src[q];
  for (int q = tid; q < 3 * TAB; q += nthreads) {
    const int d = q / TAB, r = q - d * TAB;
    double v;
    if (r < H * h)
      v = L.eoT.A[r / h][r % h];
    else if (r < 2 * H * h)
      v = L.eoT.B[(r - H * h) / h][(r - H * h) % h];
    else
      v = L.eoT.M[r - 2 * H * h];
    T[q] = (-L.c * jd[d]) * v;
  }
}

// One thread's line along axis d (line index t): the D^T contractions, the
// transposed face terms at both ends and the Phi_d outputs; dF is the line's
// share of (L^T l)_Pi's derivative sum, and (base, stride) its place.
template <int N>
__device__ __forceinline__ void adj_axis_pass(const AdjointLaunch& L, int d, int t, int64_t e,
                                              int64_t off, double jd, const double* F,
                                              const double* T, double (&dF)[N], int& base,
                                              int& stride) {
  using S = AShape<N>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB;
  const double c = L.c;
  const int ta = t % N, tb = t / N;
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
  double lp[N], lf[N], dP[N], yv[N];
  const int64_t vo = off + (2 + d) * NP + base;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    lp[i] = F[base + i * stride];
    lf[i] = F[(1 + d) * NP + base + i * stride];
    yv[i] = L.y ? L.y[vo + i * stride] : 0.0;
  }
  const double* tab = T + d * TAB;
  dev::eo_line<N, double>(lf, dF, tab);  // -c J_d D^T l_Phi_d : into Pi
  dev::eo_line<N, double>(lp, dP, tab);  // -c J_d D^T l_Pi    : into Phi_d
  {
    const double G = -0.25 * c * (double)(N * (N - 1)) * jd;
    const int64_t nlo = (int64_t)L.nbr[6 * e + 2 * d] * (kVars * NP);
    const int64_t nhi = (int64_t)L.nbr[6 * e + 2 * d + 1] * (kVars * NP);
    const int64_t lo_pt = base + (N - 1) * stride;  // lower neighbour's upper face
    const int64_t hi_pt = base;                     // upper neighbour's lower face
    // lower end, s = -1
    const double q_lo = G * (lp[0] + lf[0]);
    const double qn_lo = G * (L.x[nlo + NP + lo_pt] - L.x[nlo + (2 + d) * NP + lo_pt]);
    dF[0] += q_lo - qn_lo;
    dP[0] += q_lo + qn_lo;
    // upper end, s = +1
    const double q_hi = G * (lp[N - 1] - lf[N - 1]);
    const double qn_hi = G * (L.x[nhi + NP + hi_pt] + L.x[nhi + (2 + d) * NP + hi_pt]);
    dF[N - 1] += q_hi - qn_hi;
    dP[N - 1] -= q_hi + qn_hi;
  }
#pragma unroll
  for (int i = 0; i < N; ++i) {
    L.out[vo + i * stride] = fma(L.beta, yv[i], fma(L.alpha, lf[i], dP[i]));
    if (L.out2) L.out2[vo + i * stride] = fma(L.beta2, yv[i], L.alpha2 * lf[i]);
  }
}

// The Pi and Psi outputs at point p from the summed derivative part sd
__device__ __forceinline__ void adj_pi_psi(const AdjointLaunch& L, int64_t off, int NP, int p,
                                           double lpi, double sd) {
  const double ypi = L.y ? L.y[off + NP + p] : 0.0;
  const double ypsi = L.y ? L.y[off + p] : 0.0;
  const double xpsi = L.x[off + p];
  // (L^T l)_Pi gets -l_Psi from (L u)_Psi = -Pi
  const double sp = fma(-L.c, xpsi, sd);
  L.out[off + NP + p] = fma(L.beta, ypi, fma(L.alpha, lpi, sp));
  L.out[off + p] = fma(L.beta, ypsi, L.alpha * xpsi);
  if (L.out2) {
    L.out2[off + NP + p] = fma(L.beta2, ypi, L.alpha2 * lpi);
    L.out2[off + p] = fma(L.beta2, ypsi, L.alpha2 * xpsi);
  }
}

// Variant 0: EPB elements per block, N*N threads per element and three
// sequential axis passes with the running sum in shared memory.
template <int N, int EPB, int MINB>
__global__ void __launch_bounds__(N * N * EPB, MINB) adjoint_fp64_kernel(AdjointLaunch L) {
  using S = AShape<N>;
  constexpr int NN = S::NN, NP = S::NP;
  extern __shared__ double asm_[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  const int64_t e = (int64_t)blockIdx.x * EPB + slot;
  const bool active = e < L.n_elem;
  double* F = asm_ + slot * S::SLOT;
  double* Sacc = F + 4 * NP;
  double* T = Sacc + NP;
  const int64_t off = e * (int64_t)(kVars * NP);
  double jd[3] = {0.0, 0.0, 0.0};
  if (active) {
    jd[0] = L.jac[3 * e];
    jd[1] = L.jac[3 * e + 1];
    jd[2] = L.jac[3 * e + 2];
    adj_prologue<N>(L, off, jd, F, T, t, NN);
  }
  __syncthreads();
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    if (active) {
      double dF[N];
      int base, stride;
      adj_axis_pass<N>(L, d, t, e, off, jd[d], F, T, dF, base, stride);
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
          const int p = base + i * stride;
          adj_pi_psi(L, off, NP, p, F[p], Sacc[p] + dF[i]);
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

// Variant 1: one element per block and 3 N^2 threads, one per (axis, line),
// the three axis passes at once; the per-axis sums are added in the order of
// variant 0, (x + y) + z, so both give the same bits.
template <int N, int MINB>
__global__ void __launch_bounds__(3 * N * N, MINB) adjoint_fp64_split_kernel(AdjointLaunch L) {
  using S = AShape<N>;
  constexpr int NN = S::NN, NP = S::NP;
  extern __shared__ double asm_[];
  const int d = threadIdx.x / NN;
  const int t = threadIdx.x - d * NN;
  const int64_t e = blockIdx.x;  // one block per element
  double* F = asm_;
  double* Sd = F + 4 * NP;
  double* T = Sd + 3 * NP;
  const int64_t off = e * (int64_t)(kVars * NP);
  const double jd[3] = {L.jac[3 * e], L.jac[3 * e + 1], L.jac[3 * e + 2]};
  adj_prologue<N>(L, off, jd, F, T, threadIdx.x, 3 * NN);
  __syncthreads();
  {
    double dF[N];
    int base, stride;
    adj_axis_pass<N>(L, d, t, e, off, jd[d], F, T, dF, base, stride);
#pragma unroll
    for (int i = 0; i < N; ++i) Sd[d * NP + base + i * stride] = dF[i];
  }
  __syncthreads();
  for (int p = threadIdx.x; p < NP; p += 3 * NN)
    adj_pi_psi(L, off, NP, p, F[p], (Sd[p] + Sd[NP + p]) + Sd[2 * NP + p]);
}

template <int N>
constexpr int adj_epb() {
  return N <= 4 ? 16 : (N <= 6 ? 8 : (N == 7 ? 4 : (N <= 11 ? 2 : 1)));
}
template <int N>
constexpr int adj_minb() {
  return N <= 5 ? 2 : 1;
}
template <int N>
constexpr int adj_split_minb() {
  return N <= 4 ? 8 : (N == 5 ? 6 : (N == 6 ? 4 : (N <= 8 ? 3 : (N <= 10 ? 2 : 1))));
}

template <int N>
cudaError_t launch_adjoint_n(const AdjointLaunch& L, cudaStream_t s) {
  if (L.n_elem <= 0) return cudaSuccess;
  if (L.variant == 1) {
    const size_t smem = (size_t)AShape<N>::SLOT3 * sizeof(double);
    constexpr auto k = adjoint_fp64_split_kernel<N, adj_split_minb<N>()>;
    cudaError_t err = set_kernel_smem<k>((int)smem, true);
    if (err != cudaSuccess) return err;
    k<<<(unsigned)L.n_elem, 3 * N * N, smem, s>>>(L);
    return cudaGetLastError();
  }
  constexpr int EPB = adj_epb<N>();
  const size_t smem = (size_t)EPB * AShape<N>::SLOT * sizeof(double);
  constexpr auto k = adjoint_fp64_kernel<N, EPB, adj_minb<N>()>;
  cudaError_t err = set_kernel_smem<k>((int)smem, true);
  if (err != cudaSuccess) return err;
  const int64_t blocks = (L.n_elem + EPB - 1) / EPB;
  k<<<(unsigned)blocks, N * N * EPB, smem, s>>>(L);
  return cudaGetLastError();
}

// ---- point sampler ------------------------------------------------------------
// One warp per sample point: value = sum_{ijk} wx_i wy_j wz_k Psi_ijk of its
// element (barycentric Lagrange weights on the LGL nodes, computed on the host).
__global__ void sample_kernel(const double* __restrict__ u, int n_samples, int n,
                              const int64_t* __restrict__ elem_off,
                              const double* __restrict__ w, const double* __restrict__ target,
                              double* __restrict__ out) {
  const int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (s >= n_samples) return;
  const double* ws = w + (size_t)s * 3 * n;
  const double* psi = u + elem_off[s];
  double acc = 0.0;
  const int np = n * n * n;
  for (int p = lane; p < np; p += 32) {
    const int i = p % n, j = (p / n) % n, k = p / (n * n);
    acc = fma(ws[i] * ws[n + j] * ws[2 * n + k], psi[p], acc);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) out[s] = target ? acc - target[s] : acc;
}

// lambda_Psi += scale * r_s * weights (adjoint of the sampler)
__global__ void sample_scatter_kernel(double* __restrict__ lam, int n_samples, int n,
                                      const int64_t* __restrict__ elem_off,
                                      const double* __restrict__ w,
                                      const double* __restrict__ r, double scale) {
  const int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (s >= n_samples) return;
  const double* ws = w + (size_t)s * 3 * n;
  double* psi = lam + elem_off[s];
  const double a = scale * r[s];
  const int np = n * n * n;
  for (int p = lane; p < np; p += 32) {
    const int i = p % n, j = (p / n) % n, k = p / (n * n);
    atomicAdd(psi + p, a * (ws[i] * ws[n + j] * ws[2 * n + k]));
  }
}

}  // namespace

cudaError_t launch_adjoint_fp64(const AdjointLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_adjoint_n<2>(L, s);
    case 3: return launch_adjoint_n<3>(L, s);
    case 4: return launch_adjoint_n<4>(L, s);
    case 5: return launch_adjoint_n<5>(L, s);
    case 6: return launch_adjoint_n<6>(L, s);
    case 7: return launch_adjoint_n<7>(L, s);
    case 8: return launch_adjoint_n<8>(L, s);
    case 9: return launch_adjoint_n<9>(L, s);
    case 10: return launch_adjoint_n<10>(L, s);
    case 11: return launch_adjoint_n<11>(L, s);
    case 12: return launch_adjoint_n<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_sample(const double* u, int n_samples, int n, const int64_t* elem_off,
                          const double* w, const double* target, double* out, cudaStream_t s) {
  if (n_samples <= 0) return cudaSuccess;
  const int warps = 4;
  sample_kernel<<<(n_samples + warps - 1) / warps, 32 * warps, 0, s>>>(u, n_samples, n, elem_off,
                                                                       w, target, out);
  return cudaGetLastError();
}

cudaError_t launch_sample_scatter(double* lam, int n_samples, int n, const int64_t* elem_off,
                                  const double* w, const double* r, double scale, cudaStream_t s) {
  if (n_samples <= 0) return cudaSuccess;
  const int warps = 4;
  sample_scatter_kernel<<<(n_samples + warps - 1) / warps, 32 * warps, 0, s>>>(
      lam, n_samples, n, elem_off, w, r, scale);
  return cudaGetLastError();
}

}  // namespace dgsw
