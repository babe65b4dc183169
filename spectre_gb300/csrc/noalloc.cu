// noalloc.cu -- dgsw_step_noalloc: SSP-RK3 steps of one periodic brick that
// allocate nothing.
//
// Some callers cannot allocate device memory while they step: a host
// framework that owns a fixed device-memory budget and hands plug-ins only
// the buffers it has placed, or a caller enqueueing work where the implicit
// device-wide synchronisation of cudaMalloc/cudaFree is not allowed.  This
// entry point runs the same plain FP64 stage kernel as dgsw_step, but every
// scratch buffer it needs -- the two Runge-Kutta stage states and the
// per-element neighbour and inverse-Jacobian tables -- lives in one
// file-scope device array of fixed size, g_noalloc_scratch (32 MiB), which
// every GPU that loads this library holds until the process exits.  The
// caller passes the state (input and output) and the domain; no cudaMalloc,
// cudaFree or other allocating routine is called, on the host or the device.
//
// Set-up: every call looks up the device address of the array on the current
// device with cudaGetSymbolAddress (no allocation; a cached address could go
// stale after cudaDeviceReset reloads the module).  The first call on a device
// may load the library's device code there, so make that first call before
// any stream capture.  All calls share the array and
// it keeps the last call's contents; every word a call reads is written by
// the same call first (tables, then stage 1 before stage 2 reads it, ...), so
// nothing needs clearing.  Calls that overlap on the GPU (different streams,
// or other host threads) race on the array and must be serialised by the
// caller.
#include <cmath>

#include "../../include/dgsw.h"
#include "common.cuh"
#include "host_setup.hpp"
#include "launch.hpp"

namespace dgsw {
namespace {

constexpr size_t kScratchDoubles = (size_t)4 * 1024 * 1024;  // 32 MiB
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct BrickTables {
  int32_t elements[3];
  int32_t blocks[3];
  int32_t level[3];
  double jac[3];
  int64_t n_elem;
};

// Neighbour and inverse-Jacobian tables of one periodic brick, in the element
// order of the handle-based entry points (blocks x fastest, then x-outer /
// z-inner segments inside a block).
__global__ void fill_brick_tables(BrickTables B, int32_t* nbr, double* jac) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= B.n_elem) return;
  const int64_t per_block = (int64_t)1 << (B.level[0] + B.level[1] + B.level[2]);
  const int64_t bid = e / per_block;
  const int64_t within = e % per_block;
  int seg[3], blk[3], q[3];
  seg[2] = (int)(within & ((1 << B.level[2]) - 1));
  seg[1] = (int)((within >> B.level[2]) & ((1 << B.level[1]) - 1));
  seg[0] = (int)(within >> (B.level[1] + B.level[2]));
  blk[0] = (int)(bid % B.blocks[0]);
  blk[1] = (int)((bid / B.blocks[0]) % B.blocks[1]);
  blk[2] = (int)(bid / ((int64_t)B.blocks[0] * B.blocks[1]));
  for (int d = 0; d < 3; ++d) q[d] = (blk[d] << B.level[d]) + seg[d];
  for (int dir = 0; dir < 6; ++dir) {
    const int d = dir >> 1;
    int r[3] = {q[0], q[1], q[2]};
    const int n = B.elements[d];
    r[d] = (dir & 1) ? (r[d] + 1 == n ? 0 : r[d] + 1) : (r[d] == 0 ? n - 1 : r[d] - 1);
    int64_t rb[3], rs[3];
    for (int a = 0; a < 3; ++a) {
      rb[a] = r[a] >> B.level[a];
      rs[a] = r[a] & ((1 << B.level[a]) - 1);
    }
    const int64_t rbid = rb[0] + B.blocks[0] * (rb[1] + (int64_t)B.blocks[1] * rb[2]);
    nbr[6 * e + dir] = (int32_t)(rbid * per_block +
                                 ((rs[0] << (B.level[1] + B.level[2])) | (rs[1] << B.level[2]) | rs[2]));
  }
  for (int d = 0; d < 3; ++d) jac[3 * e + d] = B.jac[d];
}

// messages are string literals, so even the error path allocates nothing
thread_local const char* g_noalloc_error = "";

int noalloc_fail(int code, const char* msg) {
  g_noalloc_error = msg;
  return code;
}

// Device address of g_noalloc_scratch on the current device.  Looked up on
// every call: the lookup allocates nothing, and an address cached across calls
// would be stale after cudaDeviceReset reloads the module.
cudaError_t scratch_address(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

}  // namespace
}  // namespace dgsw

using namespace dgsw;

extern "C" {

size_t dgsw_noalloc_scratch_bytes(void) { return kScratchDoubles * sizeof(double); }

const char* dgsw_noalloc_last_error(void) { return g_noalloc_error; }

int dgsw_step_noalloc(const DgswBrick* brick, int points, double gamma2, double* dev_u,
                      int n_steps, double dt, void* stream) {
  if (!brick || !dev_u) return noalloc_fail(DGSW_ERR_ARGUMENT, "null argument");
  if (points < kMinN || points > kMaxN)
    return noalloc_fail(DGSW_ERR_ARGUMENT, "points per dimension must be in [2, 12]");
  if (n_steps < 0 || !std::isfinite(dt) || !std::isfinite(gamma2))
    return noalloc_fail(DGSW_ERR_ARGUMENT, "bad step arguments");
  BrickTables B;
  int64_t n_elem = 1;
  for (int d = 0; d < 3; ++d) {
    const int n = brick->elements[d];
    if (n < 1 || n > 4096) return noalloc_fail(DGSW_ERR_ARGUMENT, "elements per axis must be in [1, 4096]");
    if (!(brick->upper[d] > brick->lower[d]) || !std::isfinite(brick->upper[d]) ||
        !std::isfinite(brick->lower[d]))
      return noalloc_fail(DGSW_ERR_ARGUMENT, "brick bounds must satisfy lower < upper");
    int m = n, L = 0;
    while ((m & 1) == 0) {
      m >>= 1;
      ++L;
    }
    B.elements[d] = n;
    B.blocks[d] = m;
    B.level[d] = L;
    B.jac[d] = 2.0 / ((brick->upper[d] - brick->lower[d]) / n);
    n_elem *= n;
  }
  B.n_elem = n_elem;
  // scratch layout: stage state 1 | stage state 2 | neighbours (int32) | jac
  const int64_t np = (int64_t)points * points * points;
  const int64_t state = n_elem * kVars * np;
  const int64_t nbr_doubles = (6 * n_elem + 1) / 2;
  const int64_t need = 2 * state + nbr_doubles + 3 * n_elem;
  if (need > (int64_t)kScratchDoubles)
    return noalloc_fail(DGSW_ERR_ARGUMENT,
                        "brick too large for the fixed 32 MiB scratch array: need "
                        "2 * elements * 5 * points^3 + 6 * elements doubles <= 4194304");
  if (n_steps == 0) return DGSW_OK;
  cudaPointerAttributes attr;
  cudaError_t e = cudaPointerGetAttributes(&attr, dev_u);
  if (e != cudaSuccess || (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged))
    return noalloc_fail(DGSW_ERR_ARGUMENT, "dev_u must be device memory");
  // the scratch array used is the current device's: device memory of another
  // GPU would mix two devices' pointers in one launch
  int cur = 0;
  if ((e = cudaGetDevice(&cur)) != cudaSuccess) return noalloc_fail(DGSW_ERR_CUDA, cudaGetErrorString(e));
  if (attr.type == cudaMemoryTypeDevice && attr.device != cur)
    return noalloc_fail(DGSW_ERR_ARGUMENT, "dev_u is not on the current device");
  double* scratch = nullptr;
  e = scratch_address(&scratch);
  if (e != cudaSuccess) return noalloc_fail(DGSW_ERR_CUDA, cudaGetErrorString(e));
  double* t1 = scratch;
  double* t2 = scratch + state;
  int32_t* nbr = reinterpret_cast<int32_t*>(scratch + 2 * state);
  double* jac = scratch + 2 * state + nbr_doubles;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  fill_brick_tables<<<(unsigned)((n_elem + 127) / 128), 128, 0, s>>>(B, nbr, jac);
  if ((e = cudaGetLastError()) != cudaSuccess) return noalloc_fail(DGSW_ERR_CUDA, cudaGetErrorString(e));

  StageLaunch L;
  L.n = points;
  L.nbr = nbr;
  L.jac = jac;
  L.n_elem = n_elem;
  L.gamma2 = gamma2;
  lgl_eo_table(points, &L.eo);
  for (int step = 0; step < n_steps; ++step) {
    L.mode = kModeStageFirst;
    L.ucur = dev_u;
    L.u0 = dev_u;
    L.unext = t1;
    L.coef = {0.0, 1.0, dt};
    if ((e = launch_stage_fp64(L, s)) != cudaSuccess) break;
    L.mode = kModeStage;
    L.ucur = t1;
    L.u0 = dev_u;
    L.unext = t2;
    L.coef = {0.75, 0.25, 0.25 * dt};
    if ((e = launch_stage_fp64(L, s)) != cudaSuccess) break;
    L.ucur = t2;
    L.u0 = dev_u;
    L.unext = dev_u;
    L.coef = {1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt};
    if ((e = launch_stage_fp64(L, s)) != cudaSuccess) break;
  }
  if (e != cudaSuccess) return noalloc_fail(DGSW_ERR_CUDA, cudaGetErrorString(e));
  return DGSW_OK;
}

}  // extern "C"
