// common.cuh -- shared device-side definitions of the DG scalar-wave kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace dgsw {

constexpr int kVars = 5;    // Psi, Pi, Phi_x, Phi_y, Phi_z
constexpr int kPkg = 16;    // UpwindPenalty packaged doubles per face point
constexpr int kMinN = 2;
constexpr int kMaxN = 12;   // largest LGL extent compiled into the kernels

// Even/odd split of a centro-antisymmetric LGL differentiation matrix
// (D_{N-1-i,N-1-j} = -D_{ij}): for rows i < H = ceil(N/2),
//   P_i = sum_{j<N/2} A_ij (u_j + u_{N-1-j})  [+ M_i u_mid when N is odd]
//   Q_i = sum_{j<N/2} B_ij (u_j - u_{N-1-j})
//   (D u)_i = P_i + Q_i,  (D u)_{N-1-i} = Q_i - P_i  (i < N/2),
//   (D u)_mid = Q_mid  (N odd).
// A_ij = (D_ij + D_{i,N-1-j}) / 2, B_ij = (D_ij - D_{i,N-1-j}) / 2.
struct EoTable {
  double A[kMaxN / 2 + 1][kMaxN / 2];
  double B[kMaxN / 2 + 1][kMaxN / 2];
  double M[kMaxN / 2 + 1];
};

// CurvedScalarWave static per-point data.
// Background (26 per point): lapse, shift[3], d_i lapse[3], d_i shift^j[9] at
// 7 + 3i + j, inverse spatial metric[6] (xx xy xz yy yz zz), Gamma^i[3], K.
constexpr int kBgFields = 26;
// Operator coefficient table (41 per point), see csw_fp64.cu:
//   B^a[3], A_ai[9] (3a+i), G^aj[9] (3a+j), alpha K, C^i[3], d_i alpha[3],
//   d_i beta^j[9] (3i+j), alpha, beta^i[3]
enum : int {
  kTB = 0, kTA = 3, kTG = 12, kTK = 21, kTC = 22, kTDl = 25, kTDs = 28, kTLapse = 37,
  kTBeta = 38, kCswT = 41
};
// Face table (10 per face point): n_i[3], n^i[3], lifted upwind weights[4].
enum : int { kFn = 0, kFv = 3, kFm = 6, kCswF = 10 };

// Per-stage update u_next = a * u0 + b * ucur + c * L(ucur).
struct StageCoef {
  double a, b, c;
};

// Kernel modes.
enum : int {
  kModeRhs = 0,        // out = L(ucur), volume + boundary
  kModeVolume = 1,     // out = volume terms only
  kModeStageFirst = 2, // out = ucur + c L(ucur)            (a = 0, b = 1)
  kModeStage = 3       // out = a u0 + b ucur + c L(ucur)
};

// Arithmetic classes of the general (mixed-extent) kernel.
enum : int {
  kPrecF64 = 0,   // FP64 throughout
  kPrecComp = 1,  // FP64 input, compensated double-float FP32 arithmetic
  kPrecF32 = 2    // FP32 input and arithmetic
};

}  // namespace dgsw
