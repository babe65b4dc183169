// adams_step.cu -- one tick position of AdamsBashforth with local time
// stepping for the flat scalar wave (uniform LGL extent N, conforming
// periodic bricks, FP64).
//
// A launch runs the jobs of the levels whose step ends at this position
// (AdamsSchedule, adams_schedule.cpp).  Per element of such a level:
//  1. finish the step (job.update):
//       u += sum_j c_j F_j                      AdamsBashforth::update_u
//                                               (AdamsBashforth.cpp:131-200)
//     with F_j the element's recorded volume time derivatives, then on every
//     face the boundary delta (add_boundary_delta, AdamsBashforth.cpp:264-281;
//     lifted and added to the face slice, ApplyBoundaryCorrections.hpp:
//     990-1011).  The flat UpwindPenalty correction is linear: with
//     w = Pi - s Phi_d - gamma2 Psi (s the face's outward sign), D_Pi =
//     (w_int - w_ext) / 2, D_Phi_d = -s D_Pi, D_Psi = 0, lifted by
//     -N(N-1)/2 |n| (LiftFlux.hpp:57-61).  The pairwise LTS sum therefore
//     collapses to marginal weights: W_int = sum_l a_l w_int(l),
//     W_ext = sum_r b_r w_ext(r), and
//       Pi_face += g (W_int - W_ext),  Phi_d,face += -s g (W_int - W_ext),
//     g = -N(N-1) J_d / 4 (J_d = d xi / d x).
//  2. optionally restore the initial values (self-start resets),
//  3. record the new state: its volume time derivative
//     (TimeDerivative.cpp:37-44, no boundary terms) into ring slot rec_slot
//     of F, and per face point, with P = Pi - gamma2 Psi, Q = Phi_d and s
//     the face's sign, the pair (P - s Q, P + s Q) into the same slot of B:
//     the first is this element's w on the face, the second the w the
//     neighbour across the face forms with its own (opposite) sign.
// The new record's slot is never one this launch reads (the schedule keeps
// it out), so elements of one launch do not race.
//
// Work split as stage_fp64.cu: N*N threads per element, one line per thread
// in each of the three axis passes; the element's state is staged in shared
// memory.
//
// Elements of differing extents (GEN): one launch per extent class; each
// element's blocks sit at its own offsets in the state, the F ring and the B
// ring.  The reference couples a p-nonconforming face on the mortar at the
// larger extent for every (local, remote) record pair and projects the
// correction back (ApplyBoundaryCorrections.hpp:816-937); the coupling is
// linear and restriction after interpolation is the identity, so the sum of
// pairs equals (W_int - T W_ext) / 2 with W_ext the neighbour's weighted
// records on its own grid and T = R P the separable face map (as
// stage_general.cu).  ab_pnc_faces_kernel forms T W_ext per such face before
// the class launches.
#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

template <int N>
struct AbShape {
  static constexpr int h = N / 2;
  static constexpr int H = h + N % 2;
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = 2 * H * h + H;
  static constexpr int SLOT = 6 * NP + 3 * TAB;  // state (5 NP), dt Pi sum, tables
};

template <int N>
constexpr int ab_epb() {
  return N <= 4 ? 8 : (N <= 6 ? 4 : (N <= 10 ? 2 : 1));
}

// an element's face record (B at its block) for face dir at point t: side 0
// is the element's own w there, side 1 the w of the neighbour's sign
__device__ __forceinline__ double face_w(const double* __restrict__ B, int dir, int t, int NN,
                                         int side) {
  return __ldg(B + (int64_t)(dir * 2 + side) * NN + t);
}

// resident blocks per SM asked of the register allocator: the FP64 pipe binds
// this kernel, and more resident elements overlap one element's loads with
// another's arithmetic (at N = 8, four blocks measured 1.14x faster than
// three despite a few spilled registers)
template <int N>
constexpr int ab_min_blocks() {
  return N == 8 ? 4 : 1;
}

template <int N, int EPB, bool GEN>
__global__ void __launch_bounds__(N * N * EPB, ab_min_blocks<N>())
    ab_step_kernel(const __grid_constant__ AbArgs A) {
  using S = AbShape<N>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB, h = S::h, H = S::H;
  extern __shared__ double smem[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  int64_t g = (int64_t)blockIdx.x * EPB + slot;
  int j = -1;
  for (int q = 0; q < A.L.n_jobs; ++q) {
    if (g < A.L.job[q].count) {
      j = q;
      break;
    }
    g -= A.L.job[q].count;
  }
  const bool active = j >= 0;
  const AbLevelJob& J = A.L.job[active ? j : 0];
  const int64_t e = active ? (int64_t)A.list[J.begin + g] : 0;
  const bool update = active && J.update && !J.reset;
  double* U = smem + slot * S::SLOT;  // Psi, Pi, Phi_x, Phi_y, Phi_z
  double* Sacc = U + 5 * NP;          // running dt Pi
  double* T = Sacc + NP;              // three scaled split tables
  const int64_t off = GEN ? A.offset[e] : e * (int64_t)(kVars * NP);
  const int64_t E = A.n_elem;
  const double g2 = A.gamma2;
  // element el's volume record in slot s of F, and its face records in slot
  // s of B
  auto frec = [&](int s) -> int64_t {
    return GEN ? (int64_t)s * A.total + off : ((int64_t)s * E + e) * (kVars * NP);
  };
  auto brec = [&](int s, int64_t el) -> int64_t {
    return GEN ? (int64_t)s * A.total_b + A.boff[el] : ((int64_t)s * E + el) * 12 * (int64_t)NN;
  };

  double jd[3] = {0.0, 0.0, 0.0};
  if (active)
    for (int d = 0; d < 3; ++d) jd[d] = A.jac[3 * e + d];

  const int ta = t % N, tb = t / N;
  auto line = [&](int d, int& base, int& stride) {
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
  };

  // 1a. boundary delta of this thread's six face points (the ends of its
  // line along each axis).  The loops run to the job's own term counts
  // (uniform in a warp): no issue slots are spent on absent terms.
  double dwf[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (update) {
#pragma unroll
    for (int dir = 0; dir < 6; ++dir) {
      const int64_t nb = A.nbr[6 * e + dir];
      const AbFaceTable& f = J.face[A.level[nb]];
      double wi = 0.0, we = 0.0;
      for (int i = 0; i < f.n_loc; ++i)
        wi = fma(f.loc_c[i], face_w(A.B + brec(f.loc_slot[i], e), dir, t, NN, 0), wi);
      const int32_t pr = GEN ? A.face_idx[6 * e + dir] : -1;
      if (pr >= 0) {
        we = __ldg(A.wext + (int64_t)pr * NN + t);
      } else {
        for (int i = 0; i < f.n_rem; ++i)
          we = fma(f.rem_c[i], face_w(A.B + brec(f.rem_slot[i], nb), dir ^ 1, t, NN, 1), we);
      }
      dwf[dir] = -0.25 * (double)(N * (N - 1)) * jd[dir >> 1] * (wi - we);
    }
  }

  // 1b. state (the initial values on a reset) plus the volume part of the
  // step, u + sum_j c_j F_j, accumulated in shared memory one record at a
  // time (each thread updates only its own points: no barrier in between)
  if (active) {
    const double* src = (J.reset ? A.u0 : A.u) + off;
    for (int q = t; q < 5 * NP; q += NN) U[q] = src[q];
    if (update)
      for (int i = 0; i < J.n_vol; ++i) {
        const double c = J.vol_c[i];
        const double* Fi = A.F + frec(J.vol_slot[i]);
        for (int q = t; q < 5 * NP; q += NN) U[q] = fma(c, __ldg(Fi + q), U[q]);
      }
    for (int q = t; q < 3 * TAB; q += NN) {
      const int d = q / TAB, r = q - d * TAB;
      double v;
      if (r < H * h)
        v = A.eo.A[r / h][r % h];
      else if (r < 2 * H * h)
        v = A.eo.B[(r - H * h) / h][(r - H * h) % h];
      else
        v = A.eo.M[r - 2 * H * h];
      T[q] = -jd[d] * v;
    }
  }
  __syncthreads();

  // 1c. the boundary delta added to the face points, one axis at a time
  // (edge points belong to faces of two axes)
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (update) {
      int base, stride;
      line(d, base, stride);
      const int p0 = base, p1 = base + (N - 1) * stride;
      U[NP + p0] += dwf[2 * d];
      U[(2 + d) * NP + p0] += dwf[2 * d];         // -s dw, s = -1
      U[NP + p1] += dwf[2 * d + 1];
      U[(2 + d) * NP + p1] -= dwf[2 * d + 1];     // -s dw, s = +1
    }
    __syncthreads();
  }

  if (active && (update || J.reset))
    for (int q = t; q < 5 * NP; q += NN) A.u[off + q] = U[q];

  // 3. record: volume time derivative and face data of the new state
  double* Fo = A.F + frec(active ? J.rec_slot : 0);
  double* Bo = A.B + brec(active ? J.rec_slot : 0, e);
#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    if (active) {
      int base, stride;
      line(d, base, stride);
      double up[N], uf[N], dF[N], dP[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        up[i] = U[NP + base + i * stride];
        uf[i] = U[(2 + d) * NP + base + i * stride];
      }
      const double* tab = T + d * TAB;
      dev::eo_line<N, double>(uf, dF, tab);  // -J_d D Phi_d: part of dt Pi
      dev::eo_line<N, double>(up, dP, tab);  // -J_d D Pi = dt Phi_d (gamma2 = 0)
      const double psi_lo = U[base], psi_hi = U[base + (N - 1) * stride];
      if (g2 != 0.0) {
        // gamma2 (d_d Psi - Phi_d) of dt Phi_d (TimeDerivative.cpp:42-43)
        double ps[N], dpsi[N];
#pragma unroll
        for (int i = 0; i < N; ++i) ps[i] = U[base + i * stride];
        dev::eo_line<N, double>(ps, dpsi, tab);
#pragma unroll
        for (int i = 0; i < N; ++i) dP[i] = fma(-g2, dpsi[i] + uf[i], dP[i]);
      }
#pragma unroll
      for (int i = 0; i < N; ++i) Fo[(2 + d) * NP + base + i * stride] = dP[i];
        // lower face (s = -1): own w = P + Q, the neighbour's P - Q; upper
      // face (s = +1): own P - Q, the neighbour's P + Q
      double* b_lo = Bo + (2 * d) * 2 * NN;
      double* b_hi = Bo + (2 * d + 1) * 2 * NN;
      const double p_lo = fma(-g2, psi_lo, up[0]), p_hi = fma(-g2, psi_hi, up[N - 1]);
      b_lo[t] = p_lo + uf[0];
      b_lo[NN + t] = p_lo - uf[0];
      b_hi[t] = p_hi - uf[N - 1];
      b_hi[NN + t] = p_hi + uf[N - 1];
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
          Fo[NP + p] = Sacc[p] + dF[i];
          Fo[p] = -up[i];
        }
      }
    }
    // Sacc points of pass d are touched by other threads in pass d + 1
    if (d < 2) __syncthreads();
  }
}

template <int N, bool GEN>
cudaError_t launch_nv(const AbArgs& A, cudaStream_t s) {
  constexpr int EPB = ab_epb<N>();
  const size_t smem = (size_t)EPB * AbShape<N>::SLOT * sizeof(double);
  constexpr auto k = ab_step_kernel<N, EPB, GEN>;
  cudaError_t err = set_kernel_smem<k>((int)smem, false);
  if (err != cudaSuccess) return err;
  int64_t total = 0;
  for (int q = 0; q < A.L.n_jobs; ++q) total += A.L.job[q].count;
  const int64_t blocks = (total + EPB - 1) / EPB;
  if (blocks <= 0) return cudaSuccess;
  k<<<(unsigned)blocks, N * N * EPB, smem, s>>>(A);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_n(const AbArgs& A, cudaStream_t s) {
  if (A.offset) {
    if (!A.boff || !A.face_idx || A.total <= 0 || A.total_b <= 0) return cudaErrorInvalidValue;
    return launch_nv<N, true>(A, s);
  }
  return launch_nv<N, false>(A, s);
}

// One warp per face record: the neighbour's weighted records (its own grid)
// in shared memory, then T along the face's second axis and its first, as
// pnc_faces_kernel (stage_general.cu) maps a state's exterior w.
constexpr int kAbPncWarps = 4;

template <int N>
__global__ void __launch_bounds__(32 * kAbPncWarps)
    ab_pnc_faces_kernel(const __grid_constant__ AbPncLaunch P) {
  constexpr int NN = N * N;
  __shared__ double sw[kAbPncWarps][kMaxN * kMaxN];
  __shared__ double s2[kAbPncWarps][kMaxN * N];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int64_t r = (int64_t)blockIdx.x * kAbPncWarps + warp;
  if (r >= P.n_rec) return;  // whole warps leave; only warp barriers follow
  const int64_t face = P.rec_face[r];
  const int64_t e = face / 6;
  const int dir = (int)(face - 6 * e);
  // the job of e's level, if it finishes a step in this launch
  const int l = P.level[e];
  int j = -1;
  for (int q = 0; q < P.L.n_jobs; ++q)
    if (P.L.job[q].level == l) {
      j = q;
      break;
    }
  if (j < 0) return;
  const AbLevelJob& J = P.L.job[j];
  if (!J.update || J.reset) return;
  const int64_t nb = P.nbr[face];
  const int nn = P.elem_n[nb], mm = nn * nn;
  const AbFaceTable& f = J.face[P.level[nb]];
  // side 1 of the neighbour's record of its face dir ^ 1: the w this face
  // forms from the neighbour's data, on the neighbour's face points
  const int64_t side = P.boff[nb] + (int64_t)((dir ^ 1) * 2 + 1) * mm;
  double* w = sw[warp];
  double* t2 = s2[warp];
  for (int q = lane; q < mm; q += 32) {
    double acc = 0.0;
    for (int i = 0; i < f.n_rem; ++i)
      acc = fma(f.rem_c[i], __ldg(P.B + (int64_t)f.rem_slot[i] * P.total_b + side + q), acc);
    w[q] = acc;
  }
  __syncwarp();
  const double* T = P.op64 + P.op_off[N * (kMaxN + 1) + nn];  // N x nn, row-major
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
    P.wext[r * NN + q] = acc;
  }
}

template <int N>
cudaError_t launch_pnc_n(const AbPncLaunch& P, cudaStream_t s) {
  const int64_t blocks = (P.n_rec + kAbPncWarps - 1) / kAbPncWarps;
  if (blocks <= 0) return cudaSuccess;
  ab_pnc_faces_kernel<N><<<(unsigned)blocks, 32 * kAbPncWarps, 0, s>>>(P);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_adams_step(const AbArgs& A, int n, cudaStream_t s) {
  switch (n) {
    case 2: return launch_n<2>(A, s);
    case 3: return launch_n<3>(A, s);
    case 4: return launch_n<4>(A, s);
    case 5: return launch_n<5>(A, s);
    case 6: return launch_n<6>(A, s);
    case 7: return launch_n<7>(A, s);
    case 8: return launch_n<8>(A, s);
    case 9: return launch_n<9>(A, s);
    case 10: return launch_n<10>(A, s);
    case 11: return launch_n<11>(A, s);
    case 12: return launch_n<12>(A, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_adams_pnc_faces(const AbPncLaunch& P, cudaStream_t s) {
  if (!P.rec_face || !P.elem_n || !P.nbr || !P.level || !P.boff || !P.B || !P.op64 || !P.op_off ||
      !P.wext || P.total_b <= 0)
    return cudaErrorInvalidValue;
  switch (P.n) {
    case 2: return launch_pnc_n<2>(P, s);
    case 3: return launch_pnc_n<3>(P, s);
    case 4: return launch_pnc_n<4>(P, s);
    case 5: return launch_pnc_n<5>(P, s);
    case 6: return launch_pnc_n<6>(P, s);
    case 7: return launch_pnc_n<7>(P, s);
    case 8: return launch_pnc_n<8>(P, s);
    case 9: return launch_pnc_n<9>(P, s);
    case 10: return launch_pnc_n<10>(P, s);
    case 11: return launch_pnc_n<11>(P, s);
    case 12: return launch_pnc_n<12>(P, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
