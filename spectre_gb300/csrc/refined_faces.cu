// refined_faces.cu -- the exterior side of every 2:1 (h-nonconforming) face
// of a refined block lattice, assembled before each stage.
//
// The flat UpwindPenalty correction is linear in the jump of
// w = Pi - s Phi_d - gamma2 Psi (s: the face's outward sign, the correction
// D_Pi = (w_int - w_ext) / 2, D_Phi_d = -s D_Pi, D_Psi = 0), and its char
// speeds are constant, so the reference's mortar round trip
// (ApplyBoundaryCorrections.hpp:723-1050 with MortarSize halves) reduces to
// an exterior w on this element's own face points:
//  - fine side (one Full mortar = this face): the coarse neighbour's face w
//    interpolated to this face's half (projection_matrix_parent_to_child);
//  - coarse side (four half mortars): sum over the four fine faces of their w
//    restricted to this face (projection_matrix_child_to_parent), since the
//    restrictions of the prolonged interior sum to the identity.
// One block per 2:1 face, one thread per face point, FP64; the stage kernel
// then uses these values in place of the neighbour's volume data.
#include "common.cuh"
#include "launch.hpp"

namespace dgsw {
namespace {

__device__ __forceinline__ int face_volume_index(int n, int d, int slice, int a, int b) {
  return d == 0 ? slice + n * (a + n * b) : (d == 1 ? a + n * (slice + n * b) : a + n * (b + n * slice));
}

__global__ void refined_faces_kernel(RefinedFaceLaunch L) {
  extern __shared__ double wsm[];  // 4 x n^2 neighbour w
  const int n = L.n, nn = n * n, np = nn * n;
  const int32_t* rec = L.faces + 9 * (int64_t)blockIdx.x;
  const int dir = rec[1], coarse = rec[2];
  const int d = dir >> 1;
  const double s = (dir & 1) ? 1.0 : -1.0;
  const int slice = (dir & 1) ? 0 : n - 1;  // the neighbour's face, dir ^ 1
  const int q = threadIdx.x;
  const int a = q % n, b = q / n;
  const int nsrc = coarse ? 4 : 1;
  if (q < nn)
    for (int c = 0; c < nsrc; ++c) {
      const int64_t base = (int64_t)rec[3 + c] * (kVars * np);
      const int vi = face_volume_index(n, d, slice, a, b);
      double w = L.u[base + np + vi] - s * L.u[base + (2 + d) * np + vi];
      if (L.gamma2 != 0.0) w = fma(-L.gamma2, L.u[base + vi], w);
      wsm[c * nn + q] = w;
    }
  __syncthreads();
  if (q >= nn) return;
  double acc = 0.0;
  if (coarse) {
    for (int c = 0; c < 4; ++c) {
      const double* R0 = L.R + (c & 1) * nn;
      const double* R1 = L.R + (c >> 1) * nn;
      for (int bp = 0; bp < n; ++bp) {
        double row = 0.0;
        for (int ap = 0; ap < n; ++ap) row = fma(R0[a * n + ap], wsm[c * nn + ap + n * bp], row);
        acc = fma(R1[b * n + bp], row, acc);
      }
    }
  } else {
    const double* P0 = L.P + rec[7] * nn;
    const double* P1 = L.P + rec[8] * nn;
    for (int bp = 0; bp < n; ++bp) {
      double row = 0.0;
      for (int ap = 0; ap < n; ++ap) row = fma(P0[a * n + ap], wsm[ap + n * bp], row);
      acc = fma(P1[b * n + bp], row, acc);
    }
  }
  L.wext[(int64_t)blockIdx.x * nn + q] = acc;
}

}  // namespace

cudaError_t launch_refined_faces(const RefinedFaceLaunch& L, cudaStream_t s) {
  if (L.n_faces <= 0) return cudaSuccess;
  const int nn = L.n * L.n;
  const int threads = (nn + 31) / 32 * 32;
  refined_faces_kernel<<<(unsigned)L.n_faces, threads, 4 * nn * sizeof(double), s>>>(L);
  return cudaGetLastError();
}

}  // namespace dgsw
