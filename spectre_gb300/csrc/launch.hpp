// launch.hpp -- host-side launch descriptors shared by the kernel translation
// units and the C-ABI layer.
#pragma once

#include <atomic>
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "adams.hpp"
#include "common.cuh"

namespace dgsw {

// Dynamic shared memory size (and, optionally, the largest shared-memory
// carveout) of a kernel, set once per device: the attributes persist for the
// process, and setting them on every launch costs host time that a chain of
// small launches notices.
template <auto Kernel>
cudaError_t set_kernel_smem(int smem, bool max_carveout) {
  static std::atomic<uint64_t> done{0};
  static std::atomic<int> done_smem[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const bool tracked = dev >= 0 && dev < 64;
  if (tracked && ((done.load() >> dev) & 1) && done_smem[dev].load() >= smem) return cudaSuccess;
  e = cudaFuncSetAttribute(Kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e == cudaSuccess && max_carveout)
    e = cudaFuncSetAttribute(Kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess && tracked) {
    done_smem[dev].store(smem);
    done.fetch_or(uint64_t(1) << dev);
  }
  return e;
}

// One fused RHS / RK-substep launch over elements of a uniform extent n.
struct StageLaunch {
  int n = 0;       // LGL points per dimension
  int mode = 0;    // kModeRhs, kModeVolume, kModeStageFirst, kModeStage
  const double* ucur = nullptr;
  const double* u0 = nullptr;
  double* unext = nullptr;
  const int32_t* nbr = nullptr;  // 6 per element
  const double* jac = nullptr;   // 3 per element (diagonal inverse Jacobian)
  int64_t n_elem = 0;
  StageCoef coef{0.0, 0.0, 1.0};
  double gamma2 = 0.0;
  EoTable eo{};
  // refined lattices: per element face the index of its 2:1 record (-1
  // conforming) and the exterior w assembled for each record
  const int32_t* face_idx = nullptr;
  const double* wext = nullptr;
  int variant = 0;  // launch-configuration candidate of the stage modes (0 or 1)
  // the elements [elem_begin, elem_begin + elem_count) only (count < 0: to
  // the end); neighbours are read wherever they are
  int64_t elem_begin = 0;
  int64_t elem_count = -1;
  // elements of differing extents: the range runs over tasks (element
  // indices of one extent class) and element e's values start at offset[e];
  // faces whose neighbour has another extent have face_idx records
  const int32_t* tasks = nullptr;
  const int64_t* offset = nullptr;
};

cudaError_t launch_stage_fp64(const StageLaunch& L, cudaStream_t s);
// Lowers *first to the smallest element index whose block of u holds a NaN
// or an Inf (guards.cu).
cudaError_t launch_finite_check(const double* u, const int64_t* offset, int64_t n_elem,
                                unsigned long long* first, cudaStream_t s);
// Elements that one full wave of the FP64 stage kernel (extent n, launch
// variant) holds on the current device; 0 if unknown.
int64_t stage_fp64_wave_elements(int n, int variant);

// One tick position of AdamsBashforth with local time stepping
// (adams_step.cu): the coefficient tables of the levels stepping there, by
// value in the kernel's parameter space.
struct AbArgs {
  double* u = nullptr;         // state, updated in place
  const double* u0 = nullptr;  // initial values (self-start resets)
  double* F = nullptr;         // ring slots x elements x 5 N^3 volume time derivatives
  double* B = nullptr;         // ring slots x elements x 6 faces x (own w, neighbour w) x N^2
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  const int32_t* list = nullptr;  // element ids sorted by level
  const int8_t* level = nullptr;  // per element
  int64_t n_elem = 0;
  double gamma2 = 0.0;
  EoTable eo{};
  AbLaunch L{};
  // elements of differing extents (offset non-null): the launch covers the
  // elements of extent n in the jobs' ranges; offset / boff give each
  // element's block in the state (and in a ring slot of F, total values per
  // slot) and in a ring slot of B (total_b values per slot); faces whose
  // neighbour has another extent (face_idx >= 0) read their exterior w,
  // already weighted over the records and mapped onto this face, from wext
  const int64_t* offset = nullptr;
  const int64_t* boff = nullptr;
  int64_t total = 0, total_b = 0;
  const int32_t* face_idx = nullptr;
  const double* wext = nullptr;
};
cudaError_t launch_adams_step(const AbArgs& A, int n, cudaStream_t s);

// The exterior w of the faces (records rec_face, 6 e + dir, of elements of
// extent n) whose neighbour has another extent, for the elements that finish
// a step in launch L: sum_r b_r of the neighbour's recorded w (its own grid),
// mapped onto this face by T = R P (op64 / op_off as PncFaceLaunch); wext
// gets n^2 values per record (adams_step.cu).
struct AbPncLaunch {
  int n = 0;
  int64_t n_rec = 0;
  const int32_t* rec_face = nullptr;
  const int32_t* elem_n = nullptr;
  const int32_t* nbr = nullptr;
  const int8_t* level = nullptr;
  const int64_t* boff = nullptr;
  int64_t total_b = 0;
  const double* B = nullptr;
  const double* op64 = nullptr;
  const int32_t* op_off = nullptr;
  double* wext = nullptr;
  AbLaunch L{};
};
cudaError_t launch_adams_pnc_faces(const AbPncLaunch& P, cudaStream_t s);

// Exterior w = Pi - s Phi_d - gamma2 Psi of every 2:1 face of a refined
// lattice (refined_faces.cu): the coarse neighbour's face interpolated to this
// fine face, or the four fine faces restricted to this coarse face.
// faces: 9 int32 per record (element, dir, coarse, nb[4], child[2]);
// P, R: [2][n*n] half-interval prolongation and restriction.
struct RefinedFaceLaunch {
  int n = 0;
  int64_t n_faces = 0;
  const int32_t* faces = nullptr;
  const double* P = nullptr;
  const double* R = nullptr;
  const double* u = nullptr;
  double gamma2 = 0.0;
  double* wext = nullptr;
};
cudaError_t launch_refined_faces(const RefinedFaceLaunch& L, cudaStream_t s);

// One mixed-precision stage: W = alpha X + beta Y + c L(X) (stage_mixed.cu).
// Exactly one of x64 (FP64 input, compensated double-float arithmetic) and
// x32 (FP32 increment input) is set.
struct MixedLaunch {
  int n = 0;
  int64_t n_elem = 0;
  const double* x64 = nullptr;
  const float* x32 = nullptr;
  const float* y32 = nullptr;   // optional pointwise input
  float* w32 = nullptr;         // optional FP32 output
  double* out64 = nullptr;      // optional FP64 output
  const double* base64 = nullptr;  // out64 = base64 + W when set, else W
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  double alpha = 0.0, beta = 0.0, c = 1.0;
  EoTable eo{};
  int* err = nullptr;  // device error word (bounded waits that timed out)
  int variant = 0;     // launch shape of the pipelined kernel (0 or 1)
  // pipelined kernel, FP32 stage with y32, out64 and base64: out64 = base64
  // + W formed in the kernel's epilogue (no w32)
  bool fuse_acc = false;
};

cudaError_t launch_stage_mixed(const MixedLaunch& L, cudaStream_t s);
// out = base + (double)w elementwise (n values; out may alias base).
cudaError_t launch_accumulate(double* out, const double* base, const float* w, int64_t n,
                              cudaStream_t s);
// Persistent TMA-pipelined variant for even extents (stage_mixed_pipe.cu).
bool mixed_pipe_supported(int n);
// Exercises the pipeline's bounded mbarrier wait on a barrier nothing
// completes: sets *err after limit_ns and returns (stage_mixed_pipe.cu).
cudaError_t launch_bounded_wait_check(int* err, uint64_t limit_ns, cudaStream_t s);
cudaError_t launch_stage_mixed_pipe(const MixedLaunch& L, cudaStream_t s);

// One mixed-precision stage over every element of a batch of any extents in
// one persistent launch (stage_batch.cu): W = alpha X + c L(X) with the
// exterior face values of X read from a compact face buffer, and the face
// values of W written for the next stage.
struct BatchLaunch {
  int variant = 0;                  // compiled launch shape (batch_threads, ...)
  int prec = kPrecComp;             // kPrecComp (FP64 X) or kPrecF32
  const int2* tasks = nullptr;      // (n | g << 8, first index into task_elems)
  int64_t n_tasks = 0;
  const int32_t* task_elems = nullptr;
  const int64_t* offset = nullptr;  // per element, values of the state layout
  const int64_t* foff = nullptr;    // per element, values of the face buffers
  const int32_t* elem_n = nullptr;
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  const float* dtab = nullptr;      // device: unscaled split tables of every extent
                                    // (batch_split_tables), hi then lo
  const float* op_hi = nullptr;     // face operators T (n x nn) at op_off[n (kMaxN+1) + nn]
  const int32_t* op_off = nullptr;
  const double* x64 = nullptr;      // X (kPrecComp): FP64 state
  const float* x32 = nullptr;       // X (kPrecF32): FP32 increment
  const float2* fx2 = nullptr;      // exterior face values of X (kPrecComp, double-float)
  const float* fx32 = nullptr;      // exterior face values of X (kPrecF32)
  float* w32 = nullptr;             // FP32 output W (may be X's own buffer)
  float* raw32 = nullptr;           // optional: W's face values in the element's own
                                    // resolution, at its face-buffer offsets
  double alpha = 0.0, c = 1.0;
  double gamma2 = 0.0;              // ScalarWave's constraint damping (Psi staged too when != 0)
  int* err = nullptr;               // device error word (bounded waits that timed out)
  int buf_bytes = 0, s_bytes = 0;   // shared-memory regions
  int grid = 0;
};
cudaError_t launch_stage_batch(const BatchLaunch& L, cudaStream_t s);
// The compiled launch shapes (variants): threads per CTA and largest extent;
// elements per task of extent n; the shared-memory regions a launch whose
// tasks have extent n needs (*buf pipeline buffer, *s accumulator).
int batch_variants();
int batch_threads(int variant);
int batch_max_extent(int variant);
int batch_task_elements(int n, int variant);
void batch_smem_bytes(int n, bool comp, bool g2, int variant, size_t* buf, size_t* s);
// the launch's dynamic shared memory for the given region sizes (pipeline
// buffers, accumulator and the face maps' scratch)
size_t batch_smem_total(int variant, size_t buf, size_t s);
// The split tables the batch kernels read (BatchLaunch.dtab): for every
// extent 2..12 the even/odd split of the LGL D as FP32 hi parts, then the lo
// parts; its length in floats.
void batch_split_tables(std::vector<float>* out);
// resident grid of the batch kernel with smem bytes of shared memory
cudaError_t batch_grid(bool comp, bool g2, int variant, size_t smem, int* grid);
// The step's update of the FP64 state u (n values) by (double)(w + beta y),
// and of its double-float face values fu (nf values) by fw + beta fy.
cudaError_t launch_accumulate_step(double* u, const float* w, const float* y, double beta,
                                   int64_t n, float2* fu, const float* fw, const float* fy,
                                   int64_t nf, cudaStream_t s);
// The next stage's exterior face values from the raw face values of a stage:
// each producer face mapped onto its neighbour's points (stage_batch.cu).
// chunks: (n | m << 8, first face, faces, 0), one (n, m) pair per chunk;
// face_src / face_dst: per face, offsets into raw / out.
constexpr int kBatchMapFaces = 32;  // faces per chunk at most
struct FaceMapLaunch {
  const int4* chunks = nullptr;
  int64_t n_chunks = 0;
  const int64_t* face_src = nullptr;
  const int64_t* face_dst = nullptr;
  const float* op_hi = nullptr;
  const int32_t* op_off = nullptr;
  const float* raw = nullptr;
  float* out = nullptr;
};
cudaError_t launch_face_map(const FaceMapLaunch& L, cudaStream_t s);
// Double-float exterior face values of an FP64 state for the first stage.
struct BatchFaceLaunch {
  int64_t n_elem = 0;
  const int32_t* elem_n = nullptr;
  const int64_t* offset = nullptr;
  const int64_t* foff = nullptr;
  const int32_t* nbr = nullptr;
  const float* op_hi = nullptr;
  const float* op_lo = nullptr;
  const int32_t* op_off = nullptr;
  const double* x64 = nullptr;
  float2* fu2 = nullptr;
  double gamma2 = 0.0;
};
cudaError_t launch_batch_faces(const BatchFaceLaunch& L, cudaStream_t s);

// One class of elements of extent n with neighbours of any extent
// (stage_general.cu): W = alpha X + beta Y + c L(X).
struct GeneralLaunch {
  int n = 0;
  int prec = kPrecF64;             // kPrecF64, kPrecComp, kPrecF32
  const int32_t* tasks = nullptr;  // element indices of this class
  int64_t n_tasks = 0;
  const int64_t* offset = nullptr; // per element, in values
  const int32_t* elem_n = nullptr;
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  // face operators T (n x nn, row-major) at op_off[n * (kMaxN + 1) + nn]
  const double* op64 = nullptr;
  const float* op_hi = nullptr;
  const float* op_lo = nullptr;
  const int32_t* op_off = nullptr;
  EoTable eo{};
  double gamma2 = 0.0;
  int boundary = 1;                // 0: volume terms only
  const double* x64 = nullptr;     // X (kPrecF64, kPrecComp)
  const float* x32 = nullptr;      // X (kPrecF32)
  const double* y64 = nullptr;     // Y (kPrecF64)
  const float* y32 = nullptr;      // Y (kPrecComp, kPrecF32)
  float* w32 = nullptr;            // FP32 output
  double* out64 = nullptr;         // FP64 output (= W, or base64 + W)
  const double* base64 = nullptr;
  double alpha = 0.0, beta = 0.0, c = 1.0;
};

cudaError_t launch_stage_general(const GeneralLaunch& L, cudaStream_t s);

// Exterior w of the faces of one extent class n whose neighbour has another
// extent (stage_general.cu): record r is face rec_face[r] = 6 e + dir of an
// element e of the class; wext[r n^2 + a + n b] is the neighbour's
// w = Pi - s Phi_d - gamma2 Psi mapped onto e's face points by
// T = R_{mortar->face} P_{nbr->mortar} in both face dimensions.
struct PncFaceLaunch {
  int n = 0;
  int64_t n_rec = 0;
  const int32_t* rec_face = nullptr;
  const int64_t* offset = nullptr;
  const int32_t* elem_n = nullptr;
  const int32_t* nbr = nullptr;
  const double* op64 = nullptr;
  const int32_t* op_off = nullptr;
  double gamma2 = 0.0;
  const double* x = nullptr;
  double* wext = nullptr;
};

cudaError_t launch_pnc_faces(const PncFaceLaunch& L, cudaStream_t s);

// AMR projection of element data (amr.cu): target block k (n_vars
// components, x fastest, at out + out_off[k]) from source block src[k] (at
// in + in_off[src[k]]) with extents src_ext[3k..] -> dst_ext[3k..] by the
// dst x src matrices at mats + mat_off[3k + d].
struct AmrLaunch {
  int n_vars = 0;
  int64_t n_out = 0;
  const int32_t* src = nullptr;
  const int32_t* src_ext = nullptr;
  const int32_t* dst_ext = nullptr;
  const int64_t* mat_off = nullptr;
  const double* mats = nullptr;
  const double* in = nullptr;
  const int64_t* in_off = nullptr;
  double* out = nullptr;
  const int64_t* out_off = nullptr;
};

cudaError_t launch_amr_project(const AmrLaunch& L, cudaStream_t s);

// Transposed operator (adjoint_fp64.cu): out = alpha X + beta Y + c L^T X,
// out2 = alpha2 X + beta2 Y (optional, pointwise).
struct AdjointLaunch {
  int n = 0;
  int64_t n_elem = 0;
  const double* x = nullptr;
  const double* y = nullptr;
  double* out = nullptr;
  double* out2 = nullptr;
  double alpha = 0.0, beta = 0.0, c = 1.0, alpha2 = 0.0, beta2 = 0.0;
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  EoTable eoT{};  // even/odd split of D^T
  int variant = 0;  // 0: N^2 threads per element, axes in turn; 1: 3 N^2, axes at once
};
cudaError_t launch_adjoint_fp64(const AdjointLaunch& L, cudaStream_t s);
// One launch of the mixed-precision Taylor step (taylor_df.cu) of the plain
// operator L or (transpose) of L^T, increments as double-float (hi, lo) FP32
// pairs in the state's layout: W1 = dt L u (kind 0, x64 = the FP64 state,
// outp = W1), W2 = dt L W1 (kind 1, xp = W1, outp = W2), and kind 2:
// W3 = dt L W2 (xp = W2) with state l64 += W1 + W2/2 + W3/6 (w1 = W1).  eo:
// the split tables of D (forward) or D^T (transpose).
struct TaylorLaunch {
  int n = 0;
  int kind = 0;
  bool transpose = false;
  int64_t n_elem = 0;
  double dt = 0.0;
  const double* x64 = nullptr;
  const float2* xp = nullptr;
  float2* outp = nullptr;
  double* l64 = nullptr;
  const float2* w1 = nullptr;
  float sixth_h = 0.0f, sixth_l = 0.0f;  // 1/6 as a pair (set by the launcher)
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;
  EoTable eo{};
  double gamma2 = 0.0;  // forward only: ScalarWave's constraint damping
  // the elements [elem_begin, elem_begin + n_elem) only (neighbours are read
  // wherever they are)
  int64_t elem_begin = 0;
};
cudaError_t launch_taylor_df(const TaylorLaunch& L, cudaStream_t s);
// the gamma2 != 0 kernels (taylor_df_g2.cu); launch_taylor_df calls it
cudaError_t launch_taylor_df_g2(const TaylorLaunch& L, cudaStream_t s);
// Psi at sample points: out[s] = sample - target[s] (target may be null).
cudaError_t launch_sample(const double* u, int n_samples, int n, const int64_t* elem_off,
                          const double* w, const double* target, double* out, cudaStream_t s);
// lam_Psi += scale * r[s] * weights of sample s
cudaError_t launch_sample_scatter(double* lam, int n_samples, int n, const int64_t* elem_off,
                                  const double* w, const double* r, double scale,
                                  cudaStream_t s);

// CurvedScalarWave on the shell (csw_fp64.cu, csw_mixed.cu).
// Static data, per element: T [kCswT][N^3] coefficients, F [6][kCswF][N^2]
// face geometry, X [6][N^2] the neighbour's value offset of each face point
// (element * 5 N^3 + point; -1 inner sphere, -2 outer sphere), ij [9][N^3]
// inverse Jacobian, xyz [3][N^3] coordinates.
struct CswLaunch {
  int n = 0;
  int64_t n_elem = 0;
  int boundary = 1;  // 0: volume terms only
  const double* ucur = nullptr;
  const double* u0 = nullptr;
  double* unext = nullptr;  // unext = a u0 + b ucur + c L(ucur)
  double a = 0.0, b = 0.0, c = 1.0;
  const double* T = nullptr;
  const double* F = nullptr;
  const int32_t* X = nullptr;
  const double* ij = nullptr;
  const double* xyz = nullptr;
  const int32_t* nbr = nullptr;
  double gamma1 = 0.0, gamma2 = 0.0;
  EoTable eo{};
  // AdamsBashforth records: only the listed elements (list non-null), no
  // internal mortar terms (internal = 0), and ucur's face values written to
  // frec ([6][5][N^2] per element at e * 30 N^2)
  const int32_t* list = nullptr;
  int64_t list_count = 0;
  int internal = 1;
  double* frec = nullptr;
};
cudaError_t launch_csw_fp64(const CswLaunch& L, cudaStream_t s);

// One tick position of AdamsBashforth with local time stepping on the shell:
// the volume update and the boundary delta of the listed levels' elements
// (csw_fp64.cu); the records follow with launch_csw_fp64 in record mode.
struct CswAbArgs {
  double* u = nullptr;
  const double* u0 = nullptr;
  const double* F = nullptr;  // ring slots x elements x 5 N^3 time derivatives
  const float* F32 = nullptr; // the same in FP32 (mixed precision; F null)
  const double* U = nullptr;  // ring slots x elements x [6][5][N^2] recorded face values
  const double* Fc = nullptr; // face table (kCswF per face point)
  const float* Fc32 = nullptr; // its FP32 copy (mixed precision: FP32 face corrections)
  const int32_t* X = nullptr; // per face point: the exterior point's offset in a
                              // slot of U ((nb 6 + nd) 5 N^2 + point), < 0 external
  const int32_t* list = nullptr;
  const int8_t* level = nullptr;
  int n = 0;
  int64_t n_elem = 0;
  double gamma2 = 0.0;
  AbLaunch L{};
};
cudaError_t launch_csw_ab_update(const CswAbArgs& A, cudaStream_t s);

// Mixed-precision stage on the shell: W = alpha X + beta Y + c L(X) in FP32
// arithmetic, with X either FP64 (compensated double-float derivatives) or
// an FP32 increment; out64 = base64 + W when set.
struct CswMixedLaunch {
  int n = 0;
  int64_t n_elem = 0;
  const double* x64 = nullptr;
  const float* x32 = nullptr;
  const float* y32 = nullptr;
  float* w32 = nullptr;
  double* out64 = nullptr;
  const double* base64 = nullptr;
  double alpha = 0.0, beta = 0.0, c = 1.0;
  const float* T = nullptr;   // FP32 copies of the tables
  const float* F = nullptr;
  const int32_t* X = nullptr;
  const double* ij = nullptr;
  const double* xyz = nullptr;
  const int32_t* nbr = nullptr;
  float gamma1 = 0.0f, gamma2 = 0.0f;
  EoTable eo{};
  int variant = 0;  // launch shape (csw_mixed.cuh), < csw_mixed_shapes()
  // AdamsBashforth records: only the listed elements (list non-null), no
  // internal mortar terms (internal = 0), and the FP64 x64's face values
  // written to frec ([6][5][N^2] per element at e * 30 N^2)
  const int32_t* list = nullptr;
  int64_t list_count = 0;
  int internal = 1;
  double* frec = nullptr;
};
cudaError_t launch_csw_mixed(const CswMixedLaunch& L, cudaStream_t s);
int csw_mixed_shapes();

struct CswSetup {
  int n = 0;
  int64_t n_elem = 0;
  const double* xyz = nullptr;
  const double* ij = nullptr;
  const int32_t* nbr = nullptr;
  double mass = 1.0, gamma1 = 0.0;
  double* bg = nullptr;   // [kBgFields][N^3] per element
  double* T = nullptr;
  float* T32 = nullptr;   // optional
  double* F = nullptr;
  float* F32 = nullptr;   // optional
  int* excision = nullptr;  // set to 1 if a speed on the inner sphere is incoming
};
cudaError_t launch_csw_setup(const CswSetup& S, cudaStream_t s);
cudaError_t launch_csw_initial(const double* xyz, int n, int64_t n_elem, double A, double r0,
                               double w, double* u, cudaStream_t s);

// Flat ScalarWave on Legendre-Gauss points (stage_gauss.cu): uniform extent
// n, conforming periodic bricks, FP64.  unext = a u0 + b ucur + c L(ucur).
struct GaussLaunch {
  int n = 0;
  int64_t n_elem = 0;
  int boundary = 1;  // 0: volume terms only
  const double* ucur = nullptr;
  const double* u0 = nullptr;
  double* unext = nullptr;
  double a = 0.0, b = 0.0, c = 1.0;
  const int32_t* nbr = nullptr;
  const double* jac = nullptr;  // 3 per element
  double gamma2 = 0.0;
  EoTable eo{};                 // split of the Gauss D
  double lo[kMaxN] = {}, hi[kMaxN] = {};            // interpolation to -1, +1
  double lift_lo[kMaxN] = {}, lift_hi[kMaxN] = {};  // boundary lifting terms
};
cudaError_t launch_stage_gauss(const GaussLaunch& L, cudaStream_t s);

// Exponential filter of every element's variables, in place (filter.cu).
// tasks / offset null: elements 0..n_tasks-1 of extent n, packed; else the
// listed elements at their value offsets.  F: n x n row-major, device.
struct FilterLaunch {
  int n = 0;
  int64_t n_tasks = 0;
  const int32_t* tasks = nullptr;
  const int64_t* offset = nullptr;
  double* u = nullptr;
  const double* F = nullptr;
};
cudaError_t launch_filter(const FilterLaunch& L, cudaStream_t s);

// The exponential filter on the mixed-precision path (filter_mixed.cu).
// residual: r32 = (F - I) u64, compensated (or, with out64, out64 = u64 +
// that residual: the filtered state); combine: out = ar r32 + ad d32 +
// b F(x32 + y32), to w32 and / or out64 = base64 + out.  tasks / offset null:
// elements 0..n_tasks-1 of extent n, packed; else the listed elements at
// their value offsets.  F: the n x n filter matrix (FP64, row-major).
struct MixedFilterLaunch {
  int n = 0;
  int64_t n_tasks = 0;
  const int32_t* tasks = nullptr;
  const int64_t* offset = nullptr;
  const double* F = nullptr;
  const double* u64 = nullptr;
  float* r32 = nullptr;          // residual output / combine input
  const float* x32 = nullptr;
  const float* y32 = nullptr;
  const float* d32 = nullptr;
  double ar = 0.0, ad = 0.0, b = 1.0;
  float* w32 = nullptr;
  double* out64 = nullptr;
  const double* base64 = nullptr;
};
cudaError_t launch_filter_residual(const MixedFilterLaunch& L, cudaStream_t s);
cudaError_t launch_filter_combine(const MixedFilterLaunch& L, cudaStream_t s);

// ObserveNorms partial sums per element and their fixed-order total
// (norms.cu).  Flat elements: width (3 per element) gives det J; curved:
// ij (9 x N^3 per element) gives det J = 1 / det(inverse Jacobian).
struct NormsLaunch {
  int64_t n_elem = 0;
  int uniform_n = 0;                // extent of every element, or 0: elem_n
  const int32_t* elem_n = nullptr;
  const int64_t* offset = nullptr;  // null: uniform packing
  const double* width = nullptr;
  const double* ij = nullptr;
  const double* lgl_w = nullptr;    // [kMaxN + 1][kMaxN] LGL weights
  const double* u = nullptr;
  const double* subtract = nullptr;
  double* partial = nullptr;        // 26 x n_elem, then 26 x kNormsBlocks scratch
  double* result = nullptr;         // 26
};
constexpr int kNormsBlocks = 256;  // blocks of the second reduction level
cudaError_t launch_norms(const NormsLaunch& L, cudaStream_t s);

// UpwindPenalty pointwise kernels (face_kernels.cu).
cudaError_t launch_package_data(int64_t npts, const double* psi, const double* pi,
                                const double* phi, const double* gamma2,
                                const double* normal, const double* ndotv,
                                double* packaged, cudaStream_t s);
cudaError_t launch_boundary_terms(int64_t npts, const double* pkg_int,
                                  const double* pkg_ext, double* out, cudaStream_t s);

// Analytic initial data (init_kernels.cu).
struct InitLaunch {
  int kind = 0;
  int64_t n_elem = 0;
  const int32_t* elem_n = nullptr;
  const int64_t* offset = nullptr;
  const int32_t* instance = nullptr;
  const double* lower = nullptr;
  const double* width = nullptr;
  const double* params = nullptr;  // device copy
  const double* lgl_x = nullptr;   // [kMaxN+1][kMaxN] nodes table
  double t = 0.0;
  double* u = nullptr;
};
cudaError_t launch_initial_data(const InitLaunch& L, cudaStream_t s);

}  // namespace dgsw
