// stage_fp64.cu -- plain FP64 fused DG right-hand side + SSP-RK3 substep for
// elements of one uniform LGL extent N with conforming (aligned, equal-N)
// mortars on an affine (rectilinear) mesh.
//
// One launch computes, for every element, L(u) of ScalarWave::TimeDerivative
// (TimeDerivative.cpp:37-44) from the logical derivatives along each axis
// (PartialDerivatives.tpp:315-363) times the diagonal inverse Jacobian, adds
// the UpwindPenalty boundary correction (UpwindPenalty.cpp:35-205) of each of
// the six mortars lifted onto the GLL face (LiftFlux.hpp:57-61,
// ApplyBoundaryCorrections.hpp:934-1043), and writes
//   u_next = a * u0 + b * ucur + c * L(ucur)
// which is Rk3HesthavenSsp::update_u_impl (Rk3HesthavenSsp.cpp:63-80) for the
// stage coefficients (0,1,dt), (3/4,1/4,dt/4), (1/3,2/3,2dt/3).
//
// Work split: one group of N*N threads per element.  The four differentiated
// fields (Pi, Phi_x, Phi_y, Phi_z) are staged in shared memory; three passes
// follow, one per logical axis d.  In pass d each thread owns one line along
// d: it differentiates Phi_d (into the running sum for dt Pi) and Pi (giving
// dt Phi_d), adds the two face corrections at the ends of its line (the
// neighbour's face value is read straight from its volume data: GLL faces are
// volume points), and writes Phi_d's update.  The z pass completes dt Pi and
// writes the Pi and Psi updates.
//
// Arithmetic: every operation on field values is FP64.  The FP64 pipe, not
// HBM, binds this kernel on GB300, so the contraction uses the even/odd split
// of the centro-antisymmetric D (N^2/2 + N fused multiply-adds per line
// instead of N^2), only the six derivatives the system needs are formed
// (d_i Phi_i and d_i Pi; d Psi enters only through gamma2), and the scalars
// -c * (d xi/dx) are folded into the split tables once per element.
#include <cstdio>

#include "common.cuh"
#include "dg_device.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

template <int N>
struct Shape {
  static constexpr int h = N / 2;          // even/odd pairs
  static constexpr int odd = N % 2;
  static constexpr int H = h + odd;        // rows formed by the split
  static constexpr int NN = N * N;
  static constexpr int NP = N * N * N;
  static constexpr int TAB = 2 * H * h + H;  // doubles of one scaled table
  // smem doubles per element, even so that every slot starts 16-byte aligned
  static constexpr int SLOT = (5 * NP + 3 * TAB + 1) / 2 * 2;
};

// A contiguous row of N doubles (an x line; even N, 16-byte aligned) moved
// two at a time: neighbouring threads' x lines are N doubles apart, so scalar
// accesses would conflict on the shared-memory banks.
template <int N>
__device__ __forceinline__ void load_row(const double* p, double (&x)[N]) {
#pragma unroll
  for (int k = 0; k < N / 2; ++k) {
    const double2 v = reinterpret_cast<const double2*>(p)[k];
    x[2 * k] = v.x;
    x[2 * k + 1] = v.y;
  }
}
template <int N>
__device__ __forceinline__ void store_row(double* p, const double (&x)[N]) {
#pragma unroll
  for (int k = 0; k < N / 2; ++k)
    reinterpret_cast<double2*>(p)[k] = make_double2(x[2 * k], x[2 * k + 1]);
}

template <int N>
__device__ __forceinline__ void eo_line(const double (&u)[N], double (&out)[N],
                                        const double* __restrict__ tab) {
  dev::eo_line<N, double, true>(u, out, tab);  // table reloaded: registers for occupancy
}

// The kernel arguments shared by both work splits.
struct StageArgs {
  const double* ucur;
  const double* u0;
  double* unext;
  const int32_t* __restrict__ nbr;
  StageCoef coef;
  double gamma2;
  const int32_t* __restrict__ face_idx;
  const double* __restrict__ wext;
  const int64_t* __restrict__ offset;
};

// The element's fields and the scaled split tables into shared memory:
// F <- Pi, Phi_x, Phi_y, Phi_z; T[d] <- -c (d xi_d/dx_d) times the split of D.
template <int N>
__device__ __forceinline__ void stage_prologue(const StageArgs& a, int64_t off, const double (&jd)[3],
                                               const EoTable& eo, double* F, double* T, int tid,
                                               int nthreads) {
  using S = Shape<N>;
  constexpr int NP = S::NP, TAB = S::TAB, h = S::h, H = S::H;
  const double* src = a.ucur + off + NP;
  for (int q = tid; q < 4 * NP; q += nthreads) F[q] = src[q];
  for (int q = tid; q < 3 * TAB; q += nthreads) {
    const int d = q / TAB, r = q - d * TAB;
    double v;
    if (r < H * h)
      v = eo.A[r / h][r % h];
    else if (r < 2 * H * h)
      v = eo.B[(r - H * h) / h][(r - H * h) % h];
    else
      v = eo.M[r - 2 * H * h];
    T[q] = (-a.coef.c * jd[d]) * v;
  }
}

// One thread's line along axis d (line index t): differentiates Phi_d (into
// dF, its share of c * (dt Pi)) and Pi (giving c * (dt Phi_d)), adds the two
// face corrections at the ends of the line (the neighbour's face value is read
// straight from its volume data: GLL faces are volume points) and writes
// Phi_d's update.  Returns the line's Pi values in up and its place in the
// element block as (base, stride).
template <int N, int MODE>
__device__ __forceinline__ void axis_pass(const StageArgs& a, int d, int t, int64_t e, int64_t off,
                                          double jd, const double* F, const double* T,
                                          double (&up)[N], double (&dF)[N], int& base,
                                          int& stride) {
  using S = Shape<N>;
  constexpr int NN = S::NN, NP = S::NP, TAB = S::TAB;
  constexpr bool kBoundary = MODE != kModeVolume;
  const double c = a.coef.c;
  const double gamma2 = a.gamma2;
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
  double uf[N], dP[N];
  if (N % 2 == 0 && d == 0) {
    load_row<N>(F + base, up);
    load_row<N>(F + NP + base, uf);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      up[i] = F[base + i * stride];
      uf[i] = F[(1 + d) * NP + base + i * stride];
    }
  }
  const double* tab = T + d * TAB;
  eo_line<N>(uf, dF, tab);  // -c J_d D Phi_d : c * (dt Pi) part
  eo_line<N>(up, dP, tab);  // -c J_d D Pi    : c * (dt Phi_d)
  if (kBoundary) {
    // UpwindPenalty with char speeds (0, +1, -1) and a flat unit normal
    // n = s e_d: D_Psi = 0, D_Pi = (w_int - w_ext)/2 and D_Phi_d = -s D_Pi
    // with w = Pi - s Phi_d - gamma2 Psi (the exterior w uses the
    // neighbour's fields and this element's s).  Lifted with
    // -N(N-1)/2 |n| and scaled by c: G = -c N(N-1) J_d / 4.
    const double G = -0.25 * c * (double)(N * (N - 1)) * jd;
    double wi_lo = up[0] + uf[0];          // s = -1
    double wi_hi = up[N - 1] - uf[N - 1];  // s = +1
    if (gamma2 != 0.0) {
      wi_lo = fma(-gamma2, a.ucur[off + base], wi_lo);
      wi_hi = fma(-gamma2, a.ucur[off + base + (N - 1) * stride], wi_hi);
    }
    // Faces with a record (2:1 faces of refined lattices, faces whose
    // neighbour has another extent) take the exterior w on this face's
    // points from it (face point index = line index t); the others read
    // the neighbour's volume, which then has this element's extent.
    const int32_t flo = a.face_idx ? a.face_idx[6 * e + 2 * d] : -1;
    const int32_t fhi = a.face_idx ? a.face_idx[6 * e + 2 * d + 1] : -1;
    double we_lo, we_hi;
    if (flo >= 0) {
      we_lo = a.wext[(int64_t)flo * NN + t];
    } else {
      const int32_t nb = a.nbr[6 * e + 2 * d];
      const int64_t nlo = a.offset ? a.offset[nb] : (int64_t)nb * (kVars * NP);
      const int64_t lo_pt = base + (N - 1) * stride;  // neighbour's upper face
      we_lo = a.ucur[nlo + NP + lo_pt] + a.ucur[nlo + (2 + d) * NP + lo_pt];
      if (gamma2 != 0.0) we_lo = fma(-gamma2, a.ucur[nlo + lo_pt], we_lo);
    }
    if (fhi >= 0) {
      we_hi = a.wext[(int64_t)fhi * NN + t];
    } else {
      const int32_t nb = a.nbr[6 * e + 2 * d + 1];
      const int64_t nhi = a.offset ? a.offset[nb] : (int64_t)nb * (kVars * NP);
      const int64_t hi_pt = base;  // neighbour's lower face
      we_hi = a.ucur[nhi + NP + hi_pt] - a.ucur[nhi + (2 + d) * NP + hi_pt];
      if (gamma2 != 0.0) we_hi = fma(-gamma2, a.ucur[nhi + hi_pt], we_hi);
    }
    const double dw_lo = wi_lo - we_lo;
    const double dw_hi = wi_hi - we_hi;
    dF[0] = fma(G, dw_lo, dF[0]);
    dP[0] = fma(G, dw_lo, dP[0]);
    dF[N - 1] = fma(G, dw_hi, dF[N - 1]);
    dP[N - 1] = fma(-G, dw_hi, dP[N - 1]);
  }
  if (gamma2 != 0.0) {
    // gamma2 (d_d Psi - Phi_d) term of dt Phi_d (TimeDerivative.cpp:42-43)
    // needs d_d Psi: one more line contraction along d.
    double ups[N], dpsi[N];
#pragma unroll
    for (int i = 0; i < N; ++i) ups[i] = a.ucur[off + base + i * stride];
    eo_line<N>(ups, dpsi, tab);  // -c J_d D Psi
#pragma unroll
    for (int i = 0; i < N; ++i) dP[i] = fma(-gamma2, dpsi[i] + c * uf[i], dP[i]);
  }
  // Phi_d update (x lines: contiguous, moved two doubles at a time when
  // the element blocks are 16-byte aligned)
  double* outF = a.unext + off + (2 + d) * NP + base;
  const bool row = N % 2 == 0 && d == 0 && (reinterpret_cast<uintptr_t>(outF) & 15u) == 0;
  double ua[N];
  if (MODE == kModeStage) {
    if (N % 2 == 0 && d == 0 &&
        (reinterpret_cast<uintptr_t>(a.u0 + off + 2 * NP + base) & 15u) == 0) {
      load_row<N>(a.u0 + off + 2 * NP + base, ua);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) ua[i] = a.u0[off + (2 + d) * NP + base + i * stride];
    }
  }
  double ov[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    if (MODE == kModeRhs || MODE == kModeVolume) {
      ov[i] = dP[i];
    } else if (MODE == kModeStageFirst) {
      ov[i] = uf[i] + dP[i];
    } else {
      ov[i] = fma(a.coef.a, ua[i], fma(a.coef.b, uf[i], dP[i]));
    }
  }
  if (row) {
    store_row<N>(outF, ov);
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) outF[i * stride] = ov[i];
  }
}

// Pi and Psi updates at point p from Pi there (upi) and c * (dt Pi) (sp)
template <int MODE>
__device__ __forceinline__ void pi_psi_update(const StageArgs& a, int64_t off, int NP, int64_t p,
                                              double upi, double sp) {
  const double c = a.coef.c;
  double vpi, vpsi;
  if (MODE == kModeRhs || MODE == kModeVolume) {
    vpi = sp;
    vpsi = -upi;
  } else if (MODE == kModeStageFirst) {
    vpi = upi + sp;
    vpsi = fma(-c, upi, a.ucur[off + p]);
  } else {
    vpi = fma(a.coef.a, a.u0[off + NP + p], fma(a.coef.b, upi, sp));
    vpsi = fma(a.coef.a, a.u0[off + p], fma(a.coef.b, a.ucur[off + p], -c * upi));
  }
  a.unext[off + NP + p] = vpi;
  a.unext[off + p] = vpsi;
}

// Work split of variants 0 and 1: EPB elements per block, N*N threads per
// element, three passes over the axes with the running sum of c * (dt Pi) in
// shared memory; the z pass completes it and writes the Pi and Psi updates.
template <int N, int EPB, int MINB, int MODE>
__global__ void __launch_bounds__(N * N * EPB, MINB)
    stage_fp64_kernel(StageArgs a, const double* __restrict__ jac, EoTable eo,
                      int64_t elem_begin, int64_t elem_end, const int32_t* __restrict__ tasks) {
  using S = Shape<N>;
  constexpr int NN = S::NN, NP = S::NP;
  extern __shared__ double smem[];
  const int slot = threadIdx.x / NN;
  const int t = threadIdx.x - slot * NN;
  // task i: element tasks[i] of a class list, or element i; its values at
  // offset[e] (elements of differing extents) or e * 5 N^3
  const int64_t i_task = elem_begin + (int64_t)blockIdx.x * EPB + slot;
  const bool active = i_task < elem_end;
  const int64_t e = tasks ? (active ? (int64_t)tasks[i_task] : 0) : i_task;
  double* F = smem + slot * S::SLOT;  // Pi, Phi_x, Phi_y, Phi_z of ucur
  double* Sacc = F + 4 * NP;         // running c * (dt Pi)
  double* T = Sacc + NP;             // three scaled split tables
  const int64_t off = a.offset ? (active ? a.offset[e] : 0) : e * (int64_t)(kVars * NP);

  double jd[3] = {0.0, 0.0, 0.0};
  if (active) {
    jd[0] = jac[3 * e];
    jd[1] = jac[3 * e + 1];
    jd[2] = jac[3 * e + 2];
    stage_prologue<N>(a, off, jd, eo, F, T, t, NN);
  }
  __syncthreads();

#pragma unroll 1
  for (int d = 0; d < 3; ++d) {
    if (active) {
      double up[N], dF[N];
      int base, stride;
      axis_pass<N, MODE>(a, d, t, e, off, jd[d], F, T, up, dF, base, stride);
      if (d < 2) {
        if (N % 2 == 0 && d == 0) {
          store_row<N>(Sacc + base, dF);
        } else {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            if (d == 0)
              Sacc[base + i * stride] = dF[i];
            else
              Sacc[base + i * stride] += dF[i];
          }
        }
      } else {
        // z pass: dt Pi complete on this line; Pi and Psi updates
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int p = base + i * stride;
          pi_psi_update<MODE>(a, off, NP, p, up[i], Sacc[p] + dF[i]);
        }
      }
    }
    if (d < 2) __syncthreads();
  }
}

// Work split of variant 2: one element per block and 3 N^2 threads, one per
// (axis, line), so that the three axis passes run at once -- three times the
// threads of the other split for the same work, which pays where the grid is
// too small to fill the GPU.  Each axis leaves its share of c * (dt Pi) in a
// buffer of its own; after a barrier the block sums them in the order of the
// other split, (x + y) + z, so both splits give the same bits.
template <int N, int MINB, int MODE>
__global__ void __launch_bounds__(3 * N * N, MINB)
    stage_fp64_split_kernel(StageArgs a, const double* __restrict__ jac, EoTable eo,
                            int64_t elem_begin, const int32_t* __restrict__ tasks) {
  using S = Shape<N>;
  constexpr int NN = S::NN, NP = S::NP;
  extern __shared__ double smem[];
  const int d = threadIdx.x / NN;
  const int t = threadIdx.x - d * NN;
  const int64_t i_task = elem_begin + (int64_t)blockIdx.x;  // the grid covers the range exactly
  const int64_t e = tasks ? (int64_t)tasks[i_task] : i_task;
  double* F = smem;         // Pi, Phi_x, Phi_y, Phi_z of ucur
  double* Sd = F + 4 * NP;  // each axis's share of c * (dt Pi)
  double* T = Sd + 3 * NP;  // three scaled split tables
  const int64_t off = a.offset ? a.offset[e] : e * (int64_t)(kVars * NP);
  const double jd[3] = {jac[3 * e], jac[3 * e + 1], jac[3 * e + 2]};
  stage_prologue<N>(a, off, jd, eo, F, T, threadIdx.x, 3 * NN);
  __syncthreads();
  {
    double up[N], dF[N];
    int base, stride;
    axis_pass<N, MODE>(a, d, t, e, off, jd[d], F, T, up, dF, base, stride);
    double* out = Sd + d * NP + base;
    if (N % 2 == 0 && d == 0) {
      store_row<N>(out, dF);
    } else {
#pragma unroll
      for (int i = 0; i < N; ++i) out[i * stride] = dF[i];
    }
  }
  __syncthreads();
  for (int p = threadIdx.x; p < NP; p += 3 * NN)
    pi_psi_update<MODE>(a, off, NP, p, F[p], (Sd[p] + Sd[NP + p]) + Sd[2 * NP + p]);
}

// Elements per block and the minimum resident blocks per SM asked of the
// register allocator: chosen per N so that no variant spills and several
// blocks share an SM (one block's global loads and barriers overlap another
// block's FP64 work).
//
// Variant 1, a candidate of the launch autotuner (StageLaunch::variant, timed
// on the handle's own data by dgsw_autotune), halves the elements per block
// and doubles the resident blocks asked for.  Variants 2 and 3 are the split
// of stage_fp64_split_kernel (one element and 3 N^2 threads per block), 3 with
// one more resident block asked for than 2.
template <int N, int V>
constexpr int elems_per_block() {
  constexpr int e = N <= 4 ? 16 : (N <= 6 ? 8 : (N == 7 ? 4 : (N <= 11 ? 2 : 1)));
  return V >= 2 ? 1 : (V == 0 ? e : (e > 1 ? e / 2 : 1));
}
template <int N, int V>
constexpr int min_blocks() {
  constexpr int m = N <= 5 ? 2 : (N == 8 ? 3 : (N == 9 || N == 10 ? 2 : 1));
  constexpr int m2 = N <= 4 ? 8 : (N == 5 ? 6 : (N == 6 ? 4 : (N <= 8 ? 3 : (N <= 10 ? 2 : 1))));
  return V == 3 ? m2 + 1 : (V == 2 ? m2 : (V == 0 ? m : (2 * m > 8 ? 8 : 2 * m)));
}
template <int N, int V>
constexpr int block_threads() {
  return V >= 2 ? 3 * N * N : N * N * elems_per_block<N, V>();
}
template <int N, int V>
constexpr size_t block_smem() {
  // variants 2, 3: the fields, three axis buffers and the tables of one element
  return V >= 2 ? (size_t)((7 * Shape<N>::NP + 3 * Shape<N>::TAB + 1) / 2 * 2) * sizeof(double)
                : (size_t)elems_per_block<N, V>() * Shape<N>::SLOT * sizeof(double);
}
template <int N, int MODE, int V>
constexpr auto stage_kernel() {
  if constexpr (V >= 2)
    return stage_fp64_split_kernel<N, min_blocks<N, V>(), MODE>;
  else
    return stage_fp64_kernel<N, elems_per_block<N, V>(), min_blocks<N, V>(), MODE>;
}

template <int N, int MODE, int V = 0>
cudaError_t launch_n(const StageLaunch& L, cudaStream_t s) {
  constexpr int EPB = elems_per_block<N, V>();
  constexpr size_t smem = block_smem<N, V>();
  constexpr auto k = stage_kernel<N, MODE, V>();
  // several resident blocks per SM overlap one block's loads and barriers
  // with another's FP64 work: the largest carveout
  cudaError_t err = set_kernel_smem<k>((int)smem, true);
  if (err != cudaSuccess) return err;
  const int64_t count = L.elem_count < 0 ? L.n_elem - L.elem_begin : L.elem_count;
  const int64_t blocks = (count + EPB - 1) / EPB;
  if (blocks <= 0) return cudaSuccess;
  const StageArgs a{L.ucur, L.u0, L.unext, L.nbr, L.coef, L.gamma2, L.face_idx, L.wext, L.offset};
  if constexpr (V >= 2)
    k<<<(unsigned)blocks, block_threads<N, V>(), smem, s>>>(a, L.jac, L.eo, L.elem_begin, L.tasks);
  else
    k<<<(unsigned)blocks, block_threads<N, V>(), smem, s>>>(a, L.jac, L.eo, L.elem_begin,
                                                            L.elem_begin + count, L.tasks);
  return cudaGetLastError();
}

template <int N, int MODE>
cudaError_t launch_v(const StageLaunch& L, cudaStream_t s) {
  switch (L.variant) {
    case 1: return launch_n<N, MODE, 1>(L, s);
    case 2: return launch_n<N, MODE, 2>(L, s);
    case 3: return launch_n<N, MODE, 3>(L, s);
    default: return launch_n<N, MODE, 0>(L, s);
  }
}

template <int N>
cudaError_t launch_mode(const StageLaunch& L, cudaStream_t s) {
  switch (L.mode) {
    case kModeRhs: return launch_n<N, kModeRhs>(L, s);
    case kModeVolume: return launch_n<N, kModeVolume>(L, s);
    case kModeStageFirst: return launch_v<N, kModeStageFirst>(L, s);
    case kModeStage: return launch_v<N, kModeStage>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

// elements one full wave of the FP64 stage kernel (mode kModeStage) holds on
// the current device
template <int N, int V>
int64_t wave_n() {
  constexpr auto k = stage_kernel<N, kModeStage, V>();
  constexpr size_t smem = block_smem<N, V>();
  if (set_kernel_smem<k>((int)smem, true) != cudaSuccess) return 0;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, block_threads<N, V>(), smem) !=
          cudaSuccess)
    return 0;
  return (int64_t)per_sm * sms * elems_per_block<N, V>();
}

template <int N>
int64_t wave_v(int variant) {
  switch (variant) {
    case 1: return wave_n<N, 1>();
    case 2: return wave_n<N, 2>();
    case 3: return wave_n<N, 3>();
    default: return wave_n<N, 0>();
  }
}

}  // namespace

int64_t stage_fp64_wave_elements(int n, int variant) {
  switch (n) {
    case 2: return wave_v<2>(variant);
    case 3: return wave_v<3>(variant);
    case 4: return wave_v<4>(variant);
    case 5: return wave_v<5>(variant);
    case 6: return wave_v<6>(variant);
    case 7: return wave_v<7>(variant);
    case 8: return wave_v<8>(variant);
    case 9: return wave_v<9>(variant);
    case 10: return wave_v<10>(variant);
    case 11: return wave_v<11>(variant);
    case 12: return wave_v<12>(variant);
    default: return 0;
  }
}

cudaError_t launch_stage_fp64(const StageLaunch& L, cudaStream_t s) {
  switch (L.n) {
    case 2: return launch_mode<2>(L, s);
    case 3: return launch_mode<3>(L, s);
    case 4: return launch_mode<4>(L, s);
    case 5: return launch_mode<5>(L, s);
    case 6: return launch_mode<6>(L, s);
    case 7: return launch_mode<7>(L, s);
    case 8: return launch_mode<8>(L, s);
    case 9: return launch_mode<9>(L, s);
    case 10: return launch_mode<10>(L, s);
    case 11: return launch_mode<11>(L, s);
    case 12: return launch_mode<12>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace dgsw
