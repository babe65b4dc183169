// amr.cu -- AMR projection of element data on the device:
// amr::projectors::ProjectVariables (ParallelAlgorithms/Amr/Projectors/
// Variables.hpp:25-99).  Target block k is the source block src[k] with the
// 1D matrices of its three dimensions applied in turn:
//  - p-refinement (Full): Spectral::p_projection_matrices
//    (Projection.cpp:401-421), the identity when the extent is unchanged,
//    interpolation when the target is finer, the Legendre modal truncation
//    when it is coarser;
//  - h-refinement (LowerHalf / UpperHalf): projection_matrix_parent_to_child
//    (Projection.cpp:291-372), interpolation from the parent's points to the
//    child's points mapped into the half interval, (x -/+ 1) / 2, which needs
//    at least as many points in the child.
// The reference leaves h-coarsening unimplemented (an ERROR), and so does
// this file.
#include <algorithm>
#include <cstdint>
#include <map>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "host_setup.hpp"
#include "launch.hpp"

namespace dgsw {

bool amr_matrix(int src, int dst, int child, double* M) {
  if (src < 2 || dst < 2 || src > kMaxN || dst > kMaxN || child < 0 || child > 2) return false;
  if (child == 0) {
    if (dst == src) {
      for (int i = 0; i < dst; ++i)
        for (int j = 0; j < src; ++j) M[i * src + j] = i == j ? 1.0 : 0.0;
      return true;
    }
    // finer: interpolation (dst x src); coarser: the restriction of the
    // src-point polynomial onto dst points (dst x src)
    return dst > src ? lgl_mortar_projections(src, dst, M, nullptr)
                     : lgl_mortar_projections(dst, src, nullptr, M);
  }
  if (dst < src) return false;
  double xs[kMaxN], ws[kMaxN], xd[kMaxN], wd[kMaxN], t[kMaxN];
  if (!lgl_nodes_weights(src, xs, ws) || !lgl_nodes_weights(dst, xd, wd)) return false;
  const double shift = child == 2 ? 1.0 : -1.0;
  for (int i = 0; i < dst; ++i) t[i] = 0.5 * (xd[i] + shift);
  return lgl_interp_matrix(src, dst, t, M);
}

namespace {

constexpr int kAmrThreads = 256;
constexpr int kAmrMax = kMaxN * kMaxN * kMaxN;

// One block per target element; each variable is staged in shared memory
// and swept along x, y and z (ping-pong between two buffers).
__global__ void __launch_bounds__(kAmrThreads) amr_project_kernel(AmrLaunch L) {
  __shared__ double A[kAmrMax], B[kAmrMax];
  __shared__ double Mx[kMaxN * kMaxN], My[kMaxN * kMaxN], Mz[kMaxN * kMaxN];
  const int64_t k = blockIdx.x;
  if (k >= L.n_out) return;
  const int32_t* se = L.src_ext + 3 * k;
  const int32_t* de = L.dst_ext + 3 * k;
  const int sx = se[0], sy = se[1], sz = se[2], dx = de[0], dy = de[1], dz = de[2];
  const int64_t s_np = (int64_t)sx * sy * sz, d_np = (int64_t)dx * dy * dz;
  const double* Gx = L.mats + L.mat_off[3 * k];
  const double* Gy = L.mats + L.mat_off[3 * k + 1];
  const double* Gz = L.mats + L.mat_off[3 * k + 2];
  for (int q = threadIdx.x; q < dx * sx; q += blockDim.x) Mx[q] = Gx[q];
  for (int q = threadIdx.x; q < dy * sy; q += blockDim.x) My[q] = Gy[q];
  for (int q = threadIdx.x; q < dz * sz; q += blockDim.x) Mz[q] = Gz[q];
  const double* in = L.in + L.in_off[L.src[k]];
  double* out = L.out + L.out_off[k];
  for (int v = 0; v < L.n_vars; ++v) {
    __syncthreads();  // matrices loaded; the previous variable's sweeps done
    for (int64_t q = threadIdx.x; q < s_np; q += blockDim.x) A[q] = in[v * s_np + q];
    __syncthreads();
    // x: B[i + dx (j + sy l)] = sum_a Mx[i][a] A[a + sx (j + sy l)]
    for (int q = threadIdx.x; q < dx * sy * sz; q += blockDim.x) {
      const int i = q % dx, r = q / dx;
      double acc = 0.0;
      for (int a = 0; a < sx; ++a) acc = fma(Mx[i * sx + a], A[a + sx * r], acc);
      B[q] = acc;
    }
    __syncthreads();
    // y: A[i + dx (j + dy l)] = sum_b My[j][b] B[i + dx (b + sy l)]
    for (int q = threadIdx.x; q < dx * dy * sz; q += blockDim.x) {
      const int i = q % dx, j = (q / dx) % dy, l = q / (dx * dy);
      double acc = 0.0;
      for (int b = 0; b < sy; ++b) acc = fma(My[j * sy + b], B[i + dx * (b + sy * l)], acc);
      A[q] = acc;
    }
    __syncthreads();
    // z: out[i + dx (j + dy m)] = sum_c Mz[m][c] A[i + dx (j + dy c)]
    for (int64_t q = threadIdx.x; q < d_np; q += blockDim.x) {
      const int ij = (int)(q % (dx * dy)), m = (int)(q / (dx * dy));
      double acc = 0.0;
      for (int c = 0; c < sz; ++c) acc = fma(Mz[m * sz + c], A[ij + dx * dy * c], acc);
      out[v * d_np + q] = acc;
    }
  }
}

}  // namespace

cudaError_t launch_amr_project(const AmrLaunch& L, cudaStream_t s) {
  if (L.n_out <= 0) return cudaSuccess;
  amr_project_kernel<<<(unsigned)L.n_out, kAmrThreads, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace dgsw
