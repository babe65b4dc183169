// dgsw_api.cu -- the C ABI (include/dgsw.h): handle lifecycle, state
// transfer, RHS / substep / step launches and host-only setup queries.
//
// Ownership follows the reference's DG element: the caller owns the state it
// passes in (Variables of Psi, Pi, Phi), the handle owns every device buffer.
// dgsw_step allocates nothing: the three stage launches of one SSP-RK3 step
// (Rk3HesthavenSsp.cpp:63-80) are captured once into a CUDA graph per
// (dt, steps-per-graph) and replayed.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <type_traits>
#include <mutex>
#include <new>
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/dgsw.h"
#include "adams.hpp"
#include "common.cuh"
#include "host_setup.hpp"
#include "launch.hpp"

using namespace dgsw;

struct DgswHandle_ {
  DgswConfig cfg{};
  Domain dom;
  int device = 0;
  cudaStream_t stream = nullptr;
  // device buffers
  double* state = nullptr;  // u^n (Variables of all elements)
  double* t1 = nullptr;     // stage buffers
  double* t2 = nullptr;
  double* u0s = nullptr;    // step-start copy for dgsw_substep
  float* w1 = nullptr;      // mixed precision: d1 = dt L(u0)
  float* w2 = nullptr;      // mixed precision: s2 = u2 - u0
  int* dev_err = nullptr;   // error word written by bounded device waits
  int32_t* nbr = nullptr;
  double* jac = nullptr;
  double* lower = nullptr;
  double* width = nullptr;
  int32_t* elem_n = nullptr;
  int64_t* offset = nullptr;
  int32_t* instance = nullptr;
  double* lgl_x = nullptr;
  double* params = nullptr;  // initial-data parameters
  size_t params_cap = 0;
  EoTable eo{};
  // elements of differing extents: one task list per extent, the face
  // operators T(n, nn) and a split-table per extent
  bool general = false;
  int32_t* class_tasks[kMaxN + 1] = {};
  int64_t class_count[kMaxN + 1] = {};
  EoTable class_eo[kMaxN + 1] = {};
  double* op64 = nullptr;
  float* op_hi = nullptr;
  float* op_lo = nullptr;
  int32_t* op_off = nullptr;
  // FP64 path: per element face the index of its record within the
  // element's class (-1: the neighbour has the same extent), and per class
  // the records' faces (6 e + dir) and their exterior w (n^2 per record)
  int32_t* pnc_face_idx = nullptr;
  int32_t* pnc_rec[kMaxN + 1] = {};
  int64_t pnc_count[kMaxN + 1] = {};
  double* pnc_wext[kMaxN + 1] = {};
  // mixed precision in one persistent launch per stage over every extent
  // (stage_batch.cu): the task list, the compact face buffers of the state
  // (double-float) and of the two increments, and the launch shapes
  bool batch = false;
  int bt_variant = 0;               // launch shape in use
  int2* bt_tasks[2] = {};           // task lists for 128 and 256 threads per CTA
  int64_t bt_ntasks[2] = {};
  int32_t* bt_elems[2] = {};
  int bt_nmax = 0;                  // largest extent of the domain
  int64_t* bt_foff = nullptr;
  int64_t bt_fsize = 0;
  float2* bt_fu = nullptr;
  float* bt_fw1 = nullptr;
  float* bt_fw2 = nullptr;
  float* bt_fw3 = nullptr;
  float* bt_raw = nullptr;           // a stage's face values in each element's own resolution
  int4* bt_chunks = nullptr;         // face-map chunks, one (n, m) pair each
  int64_t bt_nchunks = 0;
  int64_t* bt_face_src = nullptr;    // per producer face, sorted by (n, m)
  int64_t* bt_face_dst = nullptr;
  float* bt_dtab = nullptr;
  // per variant and precision (0: FP64 input, 1: FP32): shared-memory regions
  // and resident grid
  static constexpr int kBtVariants = 8;
  int bt_buf[kBtVariants][2] = {}, bt_s[kBtVariants][2] = {}, bt_grid[kBtVariants][2] = {};
  double bt_tune_ms[kBtVariants] = {};
  bool bt_tuned = false;
  // launch shape of the uniform-extent pipelined mixed kernel (stage_mixed_pipe.cu)
  int pipe_variant = 0;
  bool pipe_tuned = false;
  double pipe_tune_ms[4] = {0.0, 0.0, 0.0, 0.0};
  int csw_variant = 0;  // launch shape of the mixed curved stage kernel
  bool csw_tuned = false;
  double csw_tune_ms[DGSW_TUNE_MAX_VARIANTS] = {};
  int bt_fu_age = 0;  // steps since the state's face values were formed from it
  // misfit objective and discrete adjoint (uniform FP64 path)
  EoTable eoT{};
  int n_samples = 0;
  int64_t* samp_off = nullptr;
  double* samp_w = nullptr;
  double* adj = nullptr;   // adjoint state
  double* adjz = nullptr;  // adjoint stage combination
  float2* adj32 = nullptr;  // mixed precision: the increments W1, W2 (double-float pairs)
  double* targets = nullptr;
  double* residuals = nullptr;
  int64_t record_cap = 0;  // windows x samples the two buffers above hold
  int rec_windows = 0, rec_steps = 0;
  double rec_dt = 0.0;
  cudaGraphExec_t graph_adj = nullptr;
  int graph_adj_steps = 0;
  cudaGraphExec_t graph_tf = nullptr;  // mixed precision: the misfit forward's window of steps
  int graph_tf_steps = 0;
  double graph_tf_dt = std::nan("");
  // the adjoint kernel's work split (AdjointLaunch::variant), timed on first use
  bool adj_tuned = false;
  int adj_variant = 0;
  double adj_tune_ms[2] = {0.0, 0.0};
  double graph_adj_dt = std::nan("");
  // CurvedScalarWave on the shell: static tables (csw_fp64.cu)
  bool curved = false;
  DgswShell shell{};
  double* c_xyz = nullptr;
  double* c_ij = nullptr;
  double* c_T = nullptr;
  double* c_F = nullptr;
  float* c_T32 = nullptr;
  float* c_F32 = nullptr;
  int32_t* c_X = nullptr;
  int32_t* c_Xf = nullptr;  // per face point: the exterior point in the face records
  // launch autotuner: the FP64 stage's launch-configuration variant
  bool tuned = false;
  int stage_variant = 0;
  double tune_ms[DGSW_STAGE_VARIANTS] = {};
  // refined block lattice (h-nonconforming 2:1 faces)
  bool refined = false;
  DgswRefinedBrick rbrick{};
  std::vector<int32_t> rlevels;
  int64_t r_nfaces = 0;
  int32_t* r_faces = nullptr;     // 9 per 2:1 face record
  int32_t* r_face_idx = nullptr;  // per element face
  double* r_PR = nullptr;         // [P lower, P upper, R lower, R upper], n*n each
  double* r_wext = nullptr;       // n*n per record
  // guards of dgsw_step (dgsw_set_guards)
  double guard_cfl = 0.0;
  bool guard_finite = false;
  std::vector<double> cfl_e;            // Cfl step per element
  unsigned long long* dev_first = nullptr;
  // AdamsBashforth with local time stepping (adams_schedule.cpp, adams_step.cu)
  bool adams = false;
  std::vector<int8_t> ab_level_host;
  AdamsSchedule ab;
  int64_t ab_count[kAbMaxLevels] = {};
  int32_t* ab_list = nullptr;   // element ids sorted by step level
  int8_t* ab_level = nullptr;   // step level per element
  double* ab_F = nullptr;       // ring of volume time derivatives
  float* ab_F32 = nullptr;      // the same in FP32 (mixed precision on the shell)
  double* ab_B = nullptr;       // ring of face data
  int64_t ab_points[kAbMaxLevels] = {};  // grid points of each level's elements
  // elements of differing extents: the level list is sorted by (level,
  // extent); each (level, extent) range, every element's block in a slot of
  // the face-data ring and that slot's length
  int32_t ab_cls_begin[kAbMaxLevels][kMaxN + 1] = {};
  int32_t ab_cls_count[kAbMaxLevels][kMaxN + 1] = {};
  int64_t* ab_boff = nullptr;
  int64_t ab_total_b = 0;
  double ab_slab = std::nan("");
  // steps of a host-resident state with the copies overlapped (dgsw_step_host)
  cudaStream_t pipe_in = nullptr, pipe_out = nullptr;
  std::vector<cudaStream_t> pipe_aux;          // compute streams besides the handle's
  cudaStream_t pipe_seam = nullptr;            // the launches the last copy-in holds back
  std::vector<char> pipe_seam_set;             // per stage launch (3 c + stage)
  std::vector<cudaEvent_t> pipe_ev;            // per chunk: in, stage 1, 2, 3; plus 2
  std::vector<int64_t> chunk_begin;            // chunks + 1 element offsets
  std::vector<std::vector<int>> chunk_deps;    // chunks holding a chunk's neighbours
  std::vector<int> pipe_order[2];              // stage launches (3 c + stage) in issue
                                               // order, without / with copies in
  int pipe_streams = 4;                        // compute streams
  int pipe_edge_chunks = 3;                    // thin chunks at each end of the order
  double pipe_link_gbs = 160.0;                // host link rate of the model
  double pipe_stage_ns = 0.0;                  // stage time per element of the model
                                               // (0: the autotuner's, else per point)
  // graphs of pipelined steps on pinned host buffers: copies in and out, in
  // only, out only; each for one host pointer and dt
  cudaGraphExec_t pipe_graph[3] = {nullptr, nullptr, nullptr};
  const double* pipe_graph_ptr[3] = {nullptr, nullptr, nullptr};
  double pipe_graph_dt[3] = {0.0, 0.0, 0.0};
  // Legendre-Gauss quadrature (flat, uniform, FP64)
  bool gauss = false;
  GaussTables gt{};
  // ObserveNorms scratch
  double* lgl_w = nullptr;
  double* norm_partial = nullptr;
  // exponential filter after every substep (dg::Actions::Filter)
  bool filter_on = false;
  double filter_alpha = 0.0;
  int filter_half_power = 0;
  double* filt = nullptr;  // [kMaxN + 1][kMaxN * kMaxN], matrix of extent n at n
  float* fr32 = nullptr;    // mixed precision with the filter: R = (F - I) u0
  float* fw3 = nullptr;     //   and the third stage's dt L(D2)
  // graphs of whole steps
  cudaGraphExec_t graph_one = nullptr;
  cudaGraphExec_t graph_many = nullptr;
  int graph_many_steps = 0;
  double graph_dt = std::nan("");
  std::string err;
};

namespace {

thread_local std::string g_last_error;

int fail(DgswHandle h, int code, const std::string& msg) {
  if (h) h->err = msg;
  g_last_error = msg;
  return code;
}

int cuda_fail(DgswHandle h, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  return fail(h, DGSW_ERR_CUDA, m);
}

#define DGSW_CUDA(h, call)                          \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call); \
  } while (0)

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& v) {
  cudaError_t e = cudaMalloc(dst, v.size() * sizeof(T) + 16);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

int select_device(DgswHandle h) {
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaSetDevice");
  return DGSW_OK;
}

void destroy_graphs(DgswHandle h) {
  for (cudaGraphExec_t& g : h->pipe_graph) {
    if (g) cudaGraphExecDestroy(g);
    g = nullptr;
  }
  if (h->graph_one) cudaGraphExecDestroy(h->graph_one);
  if (h->graph_many) cudaGraphExecDestroy(h->graph_many);
  h->graph_one = h->graph_many = nullptr;
  h->graph_many_steps = 0;
  h->graph_dt = std::nan("");
}

StageLaunch base_launch(DgswHandle h) {
  StageLaunch L;
  L.n = h->dom.elem_n.empty() ? 0 : h->dom.elem_n[0];
  L.nbr = h->nbr;
  L.jac = h->jac;
  L.n_elem = h->dom.n_elem;
  L.gamma2 = h->cfg.gamma2;
  L.eo = h->eo;
  if (h->refined && h->r_nfaces > 0) {
    L.face_idx = h->r_face_idx;
    L.wext = h->r_wext;
  }
  L.variant = h->stage_variant;
  return L;
}

// On a refined lattice the exterior w of every 2:1 face is assembled from
// the stage input first (refined_faces.cu).
cudaError_t launch_stage(DgswHandle h, const StageLaunch& L) {
  if (h->refined && h->r_nfaces > 0 && L.mode != kModeVolume) {
    const int n = L.n;
    RefinedFaceLaunch R;
    R.n = n;
    R.n_faces = h->r_nfaces;
    R.faces = h->r_faces;
    R.P = h->r_PR;
    R.R = h->r_PR + 2 * n * n;
    R.u = L.ucur;
    R.gamma2 = h->cfg.gamma2;
    R.wext = h->r_wext;
    cudaError_t e = launch_refined_faces(R, h->stream);
    if (e != cudaSuccess) return e;
  }
  return launch_stage_fp64(L, h->stream);
}

bool mixed(DgswHandle h) { return h->cfg.precision == DGSW_PRECISION_MIXED; }
// double-float arithmetic on an FP64 state (taylor_df.cu)
bool dfloat(DgswHandle h) { return h->cfg.precision == DGSW_PRECISION_DOUBLE_FLOAT; }

MixedLaunch base_mixed(DgswHandle h) {
  MixedLaunch L;
  L.n = h->dom.elem_n.empty() ? 0 : h->dom.elem_n[0];
  L.n_elem = h->dom.n_elem;
  L.nbr = h->nbr;
  L.jac = h->jac;
  L.eo = h->eo;
  L.err = h->dev_err;
  L.variant = h->pipe_variant & 1;
  return L;
}

cudaError_t launch_mixed(DgswHandle h, const MixedLaunch& L) {
  if (mixed_pipe_supported(L.n)) return launch_stage_mixed_pipe(L, h->stream);
  return launch_stage_mixed(L, h->stream);
}

GeneralLaunch base_general(DgswHandle h) {
  GeneralLaunch G;
  G.offset = h->offset;
  G.elem_n = h->elem_n;
  G.nbr = h->nbr;
  G.jac = h->jac;
  G.op64 = h->op64;
  G.op_hi = h->op_hi;
  G.op_lo = h->op_lo;
  G.op_off = h->op_off;
  G.gamma2 = h->cfg.gamma2;
  return G;
}

BatchLaunch base_batch(DgswHandle h, bool comp) {
  BatchLaunch B;
  const int v = h->bt_variant, lst = batch_threads(v) == 256 ? 1 : 0;
  B.variant = v;
  B.prec = comp ? kPrecComp : kPrecF32;
  B.tasks = h->bt_tasks[lst];
  B.n_tasks = h->bt_ntasks[lst];
  B.task_elems = h->bt_elems[lst];
  B.offset = h->offset;
  B.foff = h->bt_foff;
  B.elem_n = h->elem_n;
  B.nbr = h->nbr;
  B.jac = h->jac;
  B.dtab = h->bt_dtab;
  B.op_hi = h->op_hi;
  B.op_off = h->op_off;
  B.err = h->dev_err;
  B.gamma2 = h->cfg.gamma2;
  const int i = comp ? 0 : 1;
  B.buf_bytes = h->bt_buf[v][i];
  B.s_bytes = h->bt_s[v][i];
  B.grid = h->bt_grid[v][i];
  return B;
}

// The exterior face values of the next stage from the raw face values.
cudaError_t batch_face_map(DgswHandle h, float* out) {
  FaceMapLaunch M;
  M.chunks = h->bt_chunks;
  M.n_chunks = h->bt_nchunks;
  M.face_src = h->bt_face_src;
  M.face_dst = h->bt_face_dst;
  M.op_hi = h->op_hi;
  M.op_off = h->op_off;
  M.raw = h->bt_raw;
  M.out = out;
  return launch_face_map(M, h->stream);
}

// The double-float face values of the state, formed from it.
cudaError_t batch_state_faces(DgswHandle h) {
  BatchFaceLaunch F;
  F.n_elem = h->dom.n_elem;
  F.elem_n = h->elem_n;
  F.offset = h->offset;
  F.foff = h->bt_foff;
  F.nbr = h->nbr;
  F.op_hi = h->op_hi;
  F.op_lo = h->op_lo;
  F.op_off = h->op_off;
  F.x64 = h->state;
  F.fu2 = h->bt_fu;
  F.gamma2 = h->cfg.gamma2;
  return launch_batch_faces(F, h->stream);
}

// One mixed-precision SSP-RK3 step in three persistent launches (incremental
// form of Rk3HesthavenSsp, see enqueue_mixed_stage); the last stage updates
// the state in place and adds the faces of its increment to the state's.
cudaError_t enqueue_batch_step(DgswHandle h, double dt) {
  BatchLaunch A = base_batch(h, true);
  A.x64 = h->state;
  A.fx2 = h->bt_fu;
  A.w32 = h->w1;
  A.raw32 = h->bt_raw;
  A.c = dt;
  cudaError_t e = launch_stage_batch(A, h->stream);
  if (e == cudaSuccess) e = batch_face_map(h, h->bt_fw1);
  if (e != cudaSuccess) return e;
  BatchLaunch B = base_batch(h, false);
  B.x32 = h->w1;
  B.fx32 = h->bt_fw1;
  B.w32 = h->w2;
  B.raw32 = h->bt_raw;
  B.alpha = 0.5;
  B.c = 0.25 * dt;
  if ((e = launch_stage_batch(B, h->stream)) != cudaSuccess) return e;
  if ((e = batch_face_map(h, h->bt_fw2)) != cudaSuccess) return e;
  // W3 = 2/3 W2 + 2dt/3 L(W2) in place of W2 (each element's block is read
  // only by the CTA that overwrites it) with its face values, then in one
  // stream u = u0 + W3 + 2/3 W1 and the state's face values += those of
  // W3 + 2/3 W1 (T linear)
  BatchLaunch C = base_batch(h, false);
  C.x32 = h->w2;
  C.fx32 = h->bt_fw2;
  C.w32 = h->w2;
  C.raw32 = h->bt_raw;
  C.alpha = 2.0 / 3.0;
  C.c = (2.0 / 3.0) * dt;
  if ((e = launch_stage_batch(C, h->stream)) != cudaSuccess) return e;
  if ((e = batch_face_map(h, h->bt_fw3)) != cudaSuccess) return e;
  return launch_accumulate_step(h->state, h->w2, h->w1, 2.0 / 3.0, h->dom.offset.back(), h->bt_fu,
                                h->bt_fw3, h->bt_fw1, h->bt_fsize, h->stream);
}

// One launch per extent class present in the domain.
cudaError_t launch_general_classes(DgswHandle h, GeneralLaunch G) {
  for (int n = kMinN; n <= kMaxN; ++n) {
    if (h->class_count[n] == 0) continue;
    G.n = n;
    G.tasks = h->class_tasks[n];
    G.n_tasks = h->class_count[n];
    G.eo = h->class_eo[n];
    cudaError_t e = launch_stage_general(G, h->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// FP64 stage on the general path: out = alpha x + beta y + c L(x).  The
// forms of the SSP-RK3 stages, the right-hand side and the volume terms run
// the stage kernel of uniform meshes per extent class (stage_fp64.cu), after
// the exterior w of the class's faces with neighbours of another extent is
// mapped onto them (launch_pnc_faces); other forms run stage_general.cu.
cudaError_t general_f64(DgswHandle h, const double* x, const double* y, double* out, double alpha,
                        double beta, double c, int boundary = 1) {
  int mode = -1;
  if (y) mode = boundary ? kModeStage : -1;
  else if (alpha == 1.0 && beta == 0.0) mode = boundary ? kModeStageFirst : -1;
  else if (alpha == 0.0 && beta == 0.0 && c == 1.0) mode = boundary ? kModeRhs : kModeVolume;
  if (mode >= 0) {
    for (int n = kMinN; n <= kMaxN; ++n) {
      if (h->class_count[n] == 0) continue;
      if (mode != kModeVolume && h->pnc_count[n] > 0) {
        PncFaceLaunch P;
        P.n = n;
        P.n_rec = h->pnc_count[n];
        P.rec_face = h->pnc_rec[n];
        P.offset = h->offset;
        P.elem_n = h->elem_n;
        P.nbr = h->nbr;
        P.op64 = h->op64;
        P.op_off = h->op_off;
        P.gamma2 = h->cfg.gamma2;
        P.x = x;
        P.wext = h->pnc_wext[n];
        cudaError_t e = launch_pnc_faces(P, h->stream);
        if (e != cudaSuccess) return e;
      }
      StageLaunch L = base_launch(h);
      L.n = n;
      L.mode = mode;
      L.ucur = x;
      L.u0 = y ? y : x;
      L.unext = out;
      L.coef = {beta, alpha, c};
      L.eo = h->class_eo[n];
      // the launch configuration with half the elements per block: at the
      // 256-instance batch it measured 7.44 against 8.02 ms per step (for
      // N >= 7 a block's barriers then overlap another resident block's work)
      L.variant = 1;
      L.face_idx = h->pnc_face_idx;
      L.wext = h->pnc_wext[n];
      L.tasks = h->class_tasks[n];
      L.offset = h->offset;
      L.elem_begin = 0;
      L.elem_count = h->class_count[n];
      cudaError_t e = launch_stage_fp64(L, h->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  GeneralLaunch G = base_general(h);
  G.prec = kPrecF64;
  G.x64 = x;
  G.y64 = y;
  G.out64 = out;
  G.alpha = alpha;
  G.beta = beta;
  G.c = c;
  G.boundary = boundary;
  return launch_general_classes(h, G);
}

// FP64 stage on Gauss points: out = a u0 + b x + c L(x)
cudaError_t gauss_f64(DgswHandle h, const double* x, const double* u0, double* out, double a,
                      double b, double c, int boundary = 1) {
  GaussLaunch G;
  G.n = h->dom.elem_n[0];
  G.n_elem = h->dom.n_elem;
  G.boundary = boundary;
  G.ucur = x;
  G.u0 = u0;
  G.unext = out;
  G.a = a;
  G.b = b;
  G.c = c;
  G.nbr = h->nbr;
  G.jac = h->jac;
  G.gamma2 = h->cfg.gamma2;
  G.eo = h->eo;
  for (int i = 0; i < G.n; ++i) {
    G.lo[i] = h->gt.lo[i];
    G.hi[i] = h->gt.hi[i];
    G.lift_lo[i] = h->gt.lift_lo[i];
    G.lift_hi[i] = h->gt.lift_hi[i];
  }
  return launch_stage_gauss(G, h->stream);
}

// ---- CurvedScalarWave ------------------------------------------------------

CswLaunch base_csw(DgswHandle h) {
  CswLaunch L;
  L.n = h->dom.elem_n.empty() ? 0 : h->dom.elem_n[0];
  L.n_elem = h->dom.n_elem;
  L.T = h->c_T;
  L.F = h->c_F;
  L.X = h->c_X;
  L.ij = h->c_ij;
  L.xyz = h->c_xyz;
  L.nbr = h->nbr;
  L.gamma1 = h->shell.gamma1;
  L.gamma2 = h->cfg.gamma2;
  L.eo = h->eo;
  return L;
}

// FP64 curved stage: out = a u0 + b x + c L(x)
cudaError_t csw_f64(DgswHandle h, const double* x, const double* u0, double* out, double a,
                    double b, double c, int boundary = 1) {
  CswLaunch L = base_csw(h);
  L.ucur = x;
  L.u0 = u0;
  L.unext = out;
  L.a = a;
  L.b = b;
  L.c = c;
  L.boundary = boundary;
  return launch_csw_fp64(L, h->stream);
}

CswMixedLaunch base_csw_mixed(DgswHandle h) {
  CswMixedLaunch L;
  L.n = h->dom.elem_n.empty() ? 0 : h->dom.elem_n[0];
  L.n_elem = h->dom.n_elem;
  L.T = h->c_T32;
  L.F = h->c_F32;
  L.X = h->c_X;
  L.ij = h->c_ij;
  L.xyz = h->c_xyz;
  L.nbr = h->nbr;
  L.gamma1 = (float)h->shell.gamma1;
  L.gamma2 = (float)h->cfg.gamma2;
  L.eo = h->eo;
  L.variant = h->csw_variant % csw_mixed_shapes();
  return L;
}

// The neighbour's value offset of every face point (element * 5 N^3 + its
// volume point) from the shell's face permutations; -1 / -2 on the inner /
// outer sphere.
std::vector<int32_t> shell_face_offsets(const Domain& dom, const ShellGeometry& geo) {
  const int n = geo.n, nn = n * n, np = nn * n;
  std::vector<int32_t> X(6 * (size_t)nn * dom.n_elem);
  for (int64_t e = 0; e < dom.n_elem; ++e)
    for (int dir = 0; dir < 6; ++dir) {
      const int32_t nb = dom.neighbor[6 * e + dir];
      int32_t* out = &X[(6 * e + dir) * (size_t)nn];
      if (nb < 0) {
        for (int q = 0; q < nn; ++q) out[q] = nb;
        continue;
      }
      const int nd = geo.back_dir[6 * e + dir];
      const int d = nd >> 1, sl = (nd & 1) ? n - 1 : 0;
      for (int q = 0; q < nn; ++q) {
        const int t = geo.face_perm[(6 * e + dir) * (size_t)nn + q];
        const int a = t % n, b = t / n;
        const int p = d == 0 ? sl + n * (a + n * b) : (d == 1 ? a + n * (sl + n * b) : a + n * (b + n * sl));
        out[q] = nb * kVars * np + p;
      }
    }
  return X;
}

// The same exterior points in the AdamsBashforth face records ([6][5][N^2]
// values per element): (nb 6 + nd) 5 N^2 + the neighbour's face point.
std::vector<int32_t> shell_face_record_offsets(const Domain& dom, const ShellGeometry& geo) {
  const int n = geo.n, nn = n * n;
  std::vector<int32_t> X(6 * (size_t)nn * dom.n_elem);
  for (int64_t e = 0; e < dom.n_elem; ++e)
    for (int dir = 0; dir < 6; ++dir) {
      const int32_t nb = dom.neighbor[6 * e + dir];
      int32_t* out = &X[(6 * e + dir) * (size_t)nn];
      if (nb < 0) {
        for (int q = 0; q < nn; ++q) out[q] = nb;
        continue;
      }
      const int nd = geo.back_dir[6 * e + dir];
      for (int q = 0; q < nn; ++q)
        out[q] = (int32_t)(((int64_t)nb * 6 + nd) * 5 * nn + geo.face_perm[(6 * e + dir) * (size_t)nn + q]);
    }
  return X;
}

// Uploads the shell geometry and forms the background, the operator tables
// and the face geometry on the device (FP64).  Fails if a characteristic
// speed on the inner (excision) sphere is incoming.
int csw_init(DgswHandle h, const ShellGeometry& geo) {
  const int64_t E = h->dom.n_elem;
  const int n = geo.n;
  const int64_t np = (int64_t)n * n * n, nn = (int64_t)n * n;
  cudaError_t e;
  if ((e = upload(&h->c_xyz, geo.xyz)) != cudaSuccess) return cuda_fail(h, e, "upload coordinates");
  if ((e = upload(&h->c_ij, geo.inv_jac)) != cudaSuccess)
    return cuda_fail(h, e, "upload inverse Jacobian");
  if ((e = upload(&h->c_X, shell_face_offsets(h->dom, geo))) != cudaSuccess)
    return cuda_fail(h, e, "upload face offsets");
  if (E * 30 * nn >= ((int64_t)1 << 31))
    return fail(h, DGSW_ERR_ARGUMENT, "shell too large for 32-bit face record offsets");
  if ((e = upload(&h->c_Xf, shell_face_record_offsets(h->dom, geo))) != cudaSuccess)
    return cuda_fail(h, e, "upload face record offsets");
  DGSW_CUDA(h, cudaMalloc(&h->c_T, (size_t)E * kCswT * np * sizeof(double)));
  DGSW_CUDA(h, cudaMalloc(&h->c_F, (size_t)E * 6 * kCswF * nn * sizeof(double)));
  if (mixed(h)) {
    DGSW_CUDA(h, cudaMalloc(&h->c_T32, (size_t)E * kCswT * np * sizeof(float)));
    DGSW_CUDA(h, cudaMalloc(&h->c_F32, (size_t)E * 6 * kCswF * nn * sizeof(float)));
  }
  double* bg = nullptr;
  DGSW_CUDA(h, cudaMalloc(&bg, (size_t)E * kBgFields * np * sizeof(double)));
  CswSetup S;
  S.n = n;
  S.n_elem = E;
  S.xyz = h->c_xyz;
  S.ij = h->c_ij;
  S.nbr = h->nbr;
  S.mass = h->shell.mass;
  S.gamma1 = h->shell.gamma1;
  S.bg = bg;
  S.T = h->c_T;
  S.T32 = h->c_T32;
  S.F = h->c_F;
  S.F32 = h->c_F32;
  S.excision = h->dev_err;
  e = launch_csw_setup(S, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(bg);
  if (e != cudaSuccess) return cuda_fail(h, e, "shell set-up kernels");
  int flag = 0;
  DGSW_CUDA(h, cudaMemcpy(&flag, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
  DGSW_CUDA(h, cudaMemset(h->dev_err, 0, sizeof(int)));
  if (flag)
    return fail(h, DGSW_ERR_ARGUMENT,
                "DemandOutgoingCharSpeeds: a characteristic speed on the inner sphere is "
                "incoming; the excision surface must lie inside the horizon");
  return DGSW_OK;
}

// The exponential filter on a state of this handle's layout (no-op when off).
cudaError_t apply_filter(DgswHandle h, double* u) {
  if (!h->filter_on) return cudaSuccess;
  FilterLaunch F;
  F.u = u;
  if (h->general) {
    F.offset = h->offset;
    for (int n = kMinN; n <= kMaxN; ++n) {
      if (h->class_count[n] == 0) continue;
      F.n = n;
      F.tasks = h->class_tasks[n];
      F.n_tasks = h->class_count[n];
      F.F = h->filt + (size_t)n * kMaxN * kMaxN;
      cudaError_t e = launch_filter(F, h->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  F.n = h->dom.elem_n[0];
  F.n_tasks = h->dom.n_elem;
  F.F = h->filt + (size_t)F.n * kMaxN * kMaxN;
  return launch_filter(F, h->stream);
}

// W = c L(X) on the handle's mixed-precision kernels: X the FP64 state
// (x64, compensated double-float arithmetic) or an FP32 increment (x32).
cudaError_t mixed_apply_L(DgswHandle h, const double* x64, const float* x32, double c, float* w32) {
  if (h->curved) {
    CswMixedLaunch L = base_csw_mixed(h);
    L.x64 = x64;
    L.x32 = x32;
    L.c = c;
    L.w32 = w32;
    return launch_csw_mixed(L, h->stream);
  }
  if (h->general) {
    GeneralLaunch G = base_general(h);
    G.prec = x64 ? kPrecComp : kPrecF32;
    G.x64 = x64;
    G.x32 = x32;
    G.c = c;
    G.w32 = w32;
    return launch_general_classes(h, G);
  }
  MixedLaunch L = base_mixed(h);
  L.x64 = x64;
  L.x32 = x32;
  L.c = c;
  L.w32 = w32;
  return launch_mixed(h, L);
}

// A filter launch (residual or combine) over every element of the handle.
template <typename Launch>
cudaError_t mixed_filter_all(DgswHandle h, MixedFilterLaunch F, Launch launch) {
  const size_t stride = (size_t)kMaxN * kMaxN;
  if (h->general) {
    F.offset = h->offset;
    for (int n = kMinN; n <= kMaxN; ++n) {
      if (h->class_count[n] == 0) continue;
      F.n = n;
      F.tasks = h->class_tasks[n];
      F.n_tasks = h->class_count[n];
      F.F = h->filt + (size_t)n * stride;
      cudaError_t e = launch(F, h->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  F.n = h->dom.elem_n[0];
  F.n_tasks = h->dom.n_elem;
  F.F = h->filt + (size_t)F.n * stride;
  return launch(F, h->stream);
}

// Substep k of the mixed-precision SSP-RK3 step with the filter after every
// substep (filter_mixed.cu): with R = (F - I) u0,
//   k = 0: W1 = dt L u0,  D1 = R + F W1                       (w1)
//   k = 1: W2 = dt L D1,  D2 = 3/4 R + 1/4 D1 + 1/4 F(D1 + W2) (w2)
//   k = 2: W3 = dt L D2,  u = u0 + 1/3 R + 2/3 D1 + 2/3 F(D2 + W3)
// out (k < 2, optional) receives u0 + D_k; k = 2 writes out.
cudaError_t mixed_filtered_stage(DgswHandle h, int k, double dt, const double* u0, double* out) {
  cudaError_t e = cudaSuccess;
  MixedFilterLaunch F;
  F.r32 = h->fr32;
  if (k == 0) {
    if ((e = mixed_apply_L(h, u0, nullptr, dt, h->w1)) != cudaSuccess) return e;
    MixedFilterLaunch R;
    R.u64 = u0;
    R.r32 = h->fr32;
    if ((e = mixed_filter_all(h, R, launch_filter_residual)) != cudaSuccess) return e;
    F.x32 = h->w1;
    F.ar = 1.0;
    F.b = 1.0;
    F.w32 = h->w1;
  } else if (k == 1) {
    if ((e = mixed_apply_L(h, nullptr, h->w1, dt, h->w2)) != cudaSuccess) return e;
    F.x32 = h->w1;
    F.y32 = h->w2;
    F.d32 = h->w1;
    F.ar = 0.75;
    F.ad = 0.25;
    F.b = 0.25;
    F.w32 = h->w2;
  } else {
    if ((e = mixed_apply_L(h, nullptr, h->w2, dt, h->fw3)) != cudaSuccess) return e;
    F.x32 = h->w2;
    F.y32 = h->fw3;
    F.d32 = h->w1;
    F.ar = 1.0 / 3.0;
    F.ad = 2.0 / 3.0;
    F.b = 2.0 / 3.0;
  }
  if (out) {
    F.out64 = out;
    F.base64 = u0;
  }
  return mixed_filter_all(h, F, launch_filter_combine);
}

// ---- launch autotuner ------------------------------------------------------
// The FP64 stage kernel is compiled in DGSW_STAGE_VARIANTS launch
// configurations per N (elements per block and resident blocks asked of the
// register allocator; variants 2 and 3 run the three axis passes at once, for
// grids too small to fill the GPU).  Before the first step the handle times each on its own data
// (the stage input copied to t1, output to t2: the state is untouched) and
// keeps the fastest; the choice is cached per (N, elements) for later
// handles.
bool tunable(DgswHandle h) {
  return !mixed(h) && !dfloat(h) && !h->curved && !h->gauss && !h->general;
}

std::mutex g_tune_mu;
std::map<std::pair<int, int64_t>, int> g_tuned;

int autotune(DgswHandle h, bool force) {
  if (!tunable(h) || (h->tuned && !force)) return DGSW_OK;
  const std::pair<int, int64_t> key(h->dom.elem_n[0], h->dom.n_elem);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      h->stage_variant = it->second;
      h->tuned = true;
      return DGSW_OK;
    }
  }
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
  cudaEvent_t e0, e1;
  DGSW_CUDA(h, cudaEventCreate(&e0));
  DGSW_CUDA(h, cudaEventCreate(&e1));
  float best = -1.0f;
  int choice = 0;
  cudaError_t err = cudaSuccess;
  for (int v = 0; v < DGSW_STAGE_VARIANTS && err == cudaSuccess; ++v) {
    StageLaunch L = base_launch(h);
    L.variant = v;
    L.mode = kModeStage;
    L.ucur = h->t1;
    L.u0 = h->state;
    L.unext = h->t2;
    L.coef = {0.75, 0.25, 1e-4};
    err = launch_stage(h, L);  // warm-up (attributes, caches)
    if (err == cudaSuccess) err = cudaEventRecord(e0, h->stream);
    for (int r = 0; r < 3 && err == cudaSuccess; ++r) err = launch_stage(h, L);
    if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    h->tune_ms[v] = ms / 3.0;
    if (err == cudaSuccess && (best < 0.0f || ms < best)) {
      best = ms;
      choice = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return cuda_fail(h, err, "autotune");
  h->stage_variant = choice;
  h->tuned = true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key] = choice;
  return DGSW_OK;
}

cudaError_t enqueue_step(DgswHandle h, double dt);

// Times whole steps of each launch shape v < nv for which select(v) (which
// also puts the shape in place) is true, on the handle's own state: the
// state is saved first and restored after each candidate.  ms[v] is 0 for
// shapes not timed; *best is the fastest (-1 if none).
template <typename Select>
cudaError_t time_step_shapes(DgswHandle h, int nv, Select select, double* ms, int* best) {
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  cudaError_t err = cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream);
  if (err != cudaSuccess) return err;
  cudaEvent_t e0, e1;
  if ((err = cudaEventCreate(&e0)) != cudaSuccess) return err;
  if ((err = cudaEventCreate(&e1)) != cudaSuccess) {
    cudaEventDestroy(e0);
    return err;
  }
  const double dt = 1e-9;  // the state is restored: any step will do
  double fastest = 0.0;
  *best = -1;
  for (int v = 0; v < nv && err == cudaSuccess; ++v) {
    ms[v] = 0.0;
    if (!select(v)) continue;
    if (h->batch) err = batch_state_faces(h);  // warm-up step (attributes, caches)
    if (err == cudaSuccess) err = enqueue_step(h, dt);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(h->state, h->u0s, bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (err == cudaSuccess && h->batch) err = batch_state_faces(h);
    if (err == cudaSuccess) err = cudaEventRecord(e0, h->stream);
    for (int r = 0; r < 2 && err == cudaSuccess; ++r) err = enqueue_step(h, dt);
    if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(h->state, h->u0s, bytes, cudaMemcpyDeviceToDevice, h->stream);
    ms[v] = t / 2.0;
    if (err == cudaSuccess && (*best < 0 || ms[v] < fastest)) {
      fastest = ms[v];
      *best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err == cudaSuccess) err = cudaStreamSynchronize(h->stream);
  return err;
}

// Launch autotuner of the mixed-precision batch path: every compiled launch
// shape valid for the domain (threads per CTA, resident CTAs, pipeline
// buffers, largest extent) is timed over whole steps on the handle's own
// state; the fastest is kept for the handle and for handles of the same
// shape in this process.
std::map<std::tuple<int64_t, int64_t, int>, int> g_batch_tuned;

int batch_autotune(DgswHandle h, bool force) {
  if (!h->batch || (h->bt_tuned && !force)) return DGSW_OK;
  const std::tuple<int64_t, int64_t, int> key(h->dom.n_elem, h->dom.offset.back(), h->bt_nmax);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_batch_tuned.find(key);
    if (it != g_batch_tuned.end()) {
      h->bt_variant = it->second;
      h->bt_tuned = true;
      return DGSW_OK;
    }
  }
  const int keep = h->bt_variant;
  int best = -1;
  cudaError_t err = time_step_shapes(
      h, batch_variants(),
      [&](int v) {
        if (h->bt_nmax > batch_max_extent(v) || h->bt_grid[v][0] <= 0 || h->bt_grid[v][1] <= 0)
          return false;
        h->bt_variant = v;
        return true;
      },
      h->bt_tune_ms, &best);
  if (err != cudaSuccess) {
    h->bt_variant = keep;
    return cuda_fail(h, err, "batch autotune");
  }
  h->bt_variant = best >= 0 ? best : keep;
  h->bt_tuned = true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_batch_tuned[key] = h->bt_variant;
  return DGSW_OK;
}

// The uniform-extent mixed path on the pipelined kernel (even extents): four
// candidates timed the same way, cached per (extent, elements).  Bit 0: two
// pipeline buffers, or one with more resident CTAs; bit 1: the last stage
// writes W for a separate FP64 accumulate stream, or forms u0 + W in its own
// epilogue.
bool pipe_tunable(DgswHandle h) {
  return mixed(h) && !h->batch && !h->curved && !h->general && !h->gauss && !h->refined &&
         !h->adams && mixed_pipe_supported(h->dom.elem_n[0]);
}

std::map<std::pair<int, int64_t>, int> g_pipe_tuned;

// The mixed curved path: the stage kernel's launch shapes (threads per
// block, resident blocks asked of the register allocator), each with the
// step's FP64 update in the last stage's epilogue or as a separate stream,
// timed the same way, cached per (extent, elements).
bool csw_tunable(DgswHandle h) { return mixed(h) && h->curved && !h->adams; }

std::map<std::pair<int, int64_t>, int> g_csw_tuned;

int csw_autotune(DgswHandle h, bool force) {
  if (!csw_tunable(h) || (h->csw_tuned && !force)) return DGSW_OK;
  const std::pair<int, int64_t> key(h->dom.elem_n[0], h->dom.n_elem);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_csw_tuned.find(key);
    if (it != g_csw_tuned.end()) {
      h->csw_variant = it->second;
      h->csw_tuned = true;
      return DGSW_OK;
    }
  }
  const int keep = h->csw_variant;
  int best = -1;
  cudaError_t err = time_step_shapes(
      h, 2 * csw_mixed_shapes(),
      [&](int v) {
        h->csw_variant = v;
        return true;
      },
      h->csw_tune_ms, &best);
  if (err != cudaSuccess) {
    h->csw_variant = keep;
    return cuda_fail(h, err, "curved launch autotune");
  }
  h->csw_variant = best >= 0 ? best : keep;
  h->csw_tuned = true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_csw_tuned[key] = h->csw_variant;
  return DGSW_OK;
}

int pipe_autotune(DgswHandle h, bool force) {
  if (!pipe_tunable(h) || (h->pipe_tuned && !force)) return DGSW_OK;
  const std::pair<int, int64_t> key(h->dom.elem_n[0], h->dom.n_elem);
  if (!force) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_pipe_tuned.find(key);
    if (it != g_pipe_tuned.end()) {
      h->pipe_variant = it->second;
      h->pipe_tuned = true;
      return DGSW_OK;
    }
  }
  const int keep = h->pipe_variant;
  int best = -1;
  cudaError_t err = time_step_shapes(
      h, 4,
      [&](int v) {
        h->pipe_variant = v;
        return true;
      },
      h->pipe_tune_ms, &best);
  if (err != cudaSuccess) {
    h->pipe_variant = keep;
    return cuda_fail(h, err, "pipeline autotune");
  }
  h->pipe_variant = best >= 0 ? best : keep;
  h->pipe_tuned = true;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_pipe_tuned[key] = h->pipe_variant;
  return DGSW_OK;
}

// Reads and clears the device error word; DGSW_ERR_DEVICE_TIMEOUT when set.
int check_device_error(DgswHandle h) {
  if (!h->dev_err) return DGSW_OK;
  int v = 0;
  cudaError_t e = cudaMemcpy(&v, h->dev_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(h, e, "read device error word");
  if (v) {
    cudaMemset(h->dev_err, 0, sizeof(int));
    return fail(h, DGSW_ERR_DEVICE_TIMEOUT,
                "a device-side wait for staged element data timed out; results are invalid");
  }
  return DGSW_OK;
}

// The three mixed-precision stages (incremental form of Rk3HesthavenSsp):
//   A: w1 = dt L(u0)                         [base/out: u0 + w1 for substeps]
//   B: w2 = w1/2 + dt/4 L(w1)                [u0 + w2]
//   C: u  = u0 + 2/3 (w2 + w1) + 2dt/3 L(w2)
cudaError_t enqueue_mixed_stage(DgswHandle h, int k, double dt, const double* u0, double* out) {
  if (h->curved) {
    CswMixedLaunch L = base_csw_mixed(h);
    if (k == 0) {
      L.x64 = u0;
      L.c = dt;
      L.w32 = h->w1;
    } else if (k == 1) {
      L.x32 = h->w1;
      L.alpha = 0.5;
      L.c = 0.25 * dt;
      L.w32 = h->w2;
    } else {
      L.x32 = h->w2;
      L.y32 = h->w1;
      L.alpha = 2.0 / 3.0;
      L.beta = 2.0 / 3.0;
      L.c = (2.0 / 3.0) * dt;
      if (out && h->csw_variant >= csw_mixed_shapes()) {
        // tuning candidates of the second half: W in place into d1 (each
        // point's d1 is read only by the thread that overwrites it), then
        // u0 + W as one FP64 stream, so that the stage's epilogue waits on no
        // FP64 loads
        L.w32 = h->w1;
        cudaError_t e = launch_csw_mixed(L, h->stream);
        if (e != cudaSuccess) return e;
        return launch_accumulate(out, u0, h->w1, h->dom.offset.back(), h->stream);
      }
    }
    if (out) {
      L.out64 = out;
      L.base64 = u0;
    }
    return launch_csw_mixed(L, h->stream);
  }
  if (h->general) {
    GeneralLaunch G = base_general(h);
    if (k == 0) {
      G.prec = kPrecComp;
      G.x64 = u0;
      G.c = dt;
      G.w32 = h->w1;
    } else if (k == 1) {
      G.prec = kPrecF32;
      G.x32 = h->w1;
      G.alpha = 0.5;
      G.c = 0.25 * dt;
      G.w32 = h->w2;
    } else {
      G.prec = kPrecF32;
      G.x32 = h->w2;
      G.y32 = h->w1;
      G.alpha = 2.0 / 3.0;
      G.beta = 2.0 / 3.0;
      G.c = (2.0 / 3.0) * dt;
      if (out) {
        // as on the uniform path: W in place into d1 (each point's d1 is
        // read only by the thread that overwrites it), then u0 + W in one
        // FP64 stream; reading u0 pointwise inside the stage measured slower
        G.w32 = h->w1;
        cudaError_t e = launch_general_classes(h, G);
        if (e != cudaSuccess) return e;
        return launch_accumulate(out, u0, h->w1, h->dom.offset.back(), h->stream);
      }
    }
    if (out) {
      G.out64 = out;
      G.base64 = u0;
    }
    return launch_general_classes(h, G);
  }
  MixedLaunch L = base_mixed(h);
  if (k == 0) {
    L.x64 = u0;
    L.c = dt;
    L.w32 = h->w1;
  } else if (k == 1) {
    L.x32 = h->w1;
    L.alpha = 0.5;
    L.c = 0.25 * dt;
    L.w32 = h->w2;
  } else {
    L.x32 = h->w2;
    L.y32 = h->w1;
    L.alpha = 2.0 / 3.0;
    L.beta = 2.0 / 3.0;
    L.c = (2.0 / 3.0) * dt;
    if (out && mixed_pipe_supported(L.n) && (h->pipe_variant & 2)) {
      // u0 + W formed in the stage's epilogue, one coalesced pass over each
      // element's block after its W is complete in shared memory
      L.out64 = out;
      L.base64 = u0;
      L.fuse_acc = true;
      return launch_mixed(h, L);
    }
    if (out) {
      // W lands in d1 (each point's d1 is read only by the thread that
      // overwrites it), then one stream forms u0 + W in FP64: the stage then
      // stages no FP64 data and keeps twice the blocks per SM
      L.w32 = h->w1;
      cudaError_t e = launch_mixed(h, L);
      if (e != cudaSuccess) return e;
      return launch_accumulate(out, u0, h->w1, h->dom.offset.back(), h->stream);
    }
  }
  if (out) {
    L.out64 = out;
    L.base64 = u0;
  }
  return launch_mixed(h, L);
}

// Enqueue the three substeps of one SSP-RK3 step on the handle's stream:
//   t1 = u + dt L(u); t2 = 3/4 u + 1/4 t1 + dt/4 L(t1);
//   u  = 1/3 u + 2/3 t2 + 2dt/3 L(t2)   (in place: each element reads only
//   its own u, neighbours' faces come from t2).
cudaError_t enqueue_taylor_step(DgswHandle h, double dt, bool transpose);

cudaError_t enqueue_step(DgswHandle h, double dt) {
  if (dfloat(h)) return enqueue_taylor_step(h, dt, false);
  if (mixed(h) && h->filter_on) {
    cudaError_t e = mixed_filtered_stage(h, 0, dt, h->state, nullptr);
    if (e == cudaSuccess) e = mixed_filtered_stage(h, 1, dt, h->state, nullptr);
    if (e == cudaSuccess) e = mixed_filtered_stage(h, 2, dt, h->state, h->state);
    return e;
  }
  if (h->batch) return enqueue_batch_step(h, dt);
  if (mixed(h)) {
    cudaError_t e = enqueue_mixed_stage(h, 0, dt, h->state, nullptr);
    if (e != cudaSuccess) return e;
    e = enqueue_mixed_stage(h, 1, dt, h->state, nullptr);
    if (e != cudaSuccess) return e;
    return enqueue_mixed_stage(h, 2, dt, h->state, h->state);
  }
  // each substep's result is filtered when the filter is on, as
  // dg::Actions::Filter follows UpdateU in the reference's step actions
  if (h->gauss) {
    cudaError_t e = gauss_f64(h, h->state, nullptr, h->t1, 0.0, 1.0, dt);
    if (e == cudaSuccess) e = gauss_f64(h, h->t1, h->state, h->t2, 0.75, 0.25, 0.25 * dt);
    if (e == cudaSuccess)
      e = gauss_f64(h, h->t2, h->state, h->state, 1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt);
    return e;
  }
  if (h->curved) {
    cudaError_t e = csw_f64(h, h->state, nullptr, h->t1, 0.0, 1.0, dt);
    if (e == cudaSuccess) e = apply_filter(h, h->t1);
    if (e == cudaSuccess) e = csw_f64(h, h->t1, h->state, h->t2, 0.75, 0.25, 0.25 * dt);
    if (e == cudaSuccess) e = apply_filter(h, h->t2);
    if (e == cudaSuccess)
      e = csw_f64(h, h->t2, h->state, h->state, 1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt);
    if (e == cudaSuccess) e = apply_filter(h, h->state);
    return e;
  }
  if (h->general) {
    cudaError_t e = general_f64(h, h->state, nullptr, h->t1, 1.0, 0.0, dt);
    if (e == cudaSuccess) e = apply_filter(h, h->t1);
    if (e == cudaSuccess) e = general_f64(h, h->t1, h->state, h->t2, 0.25, 0.75, 0.25 * dt);
    if (e == cudaSuccess) e = apply_filter(h, h->t2);
    if (e == cudaSuccess)
      e = general_f64(h, h->t2, h->state, h->state, 2.0 / 3.0, 1.0 / 3.0, (2.0 / 3.0) * dt);
    if (e == cudaSuccess) e = apply_filter(h, h->state);
    return e;
  }
  StageLaunch L = base_launch(h);
  L.mode = kModeStageFirst;
  L.ucur = h->state;
  L.u0 = h->state;
  L.unext = h->t1;
  L.coef = {0.0, 1.0, dt};
  cudaError_t e = launch_stage(h, L);
  if (e == cudaSuccess) e = apply_filter(h, h->t1);
  if (e != cudaSuccess) return e;
  L.mode = kModeStage;
  L.ucur = h->t1;
  L.u0 = h->state;
  L.unext = h->t2;
  L.coef = {0.75, 0.25, 0.25 * dt};
  e = launch_stage(h, L);
  if (e == cudaSuccess) e = apply_filter(h, h->t2);
  if (e != cudaSuccess) return e;
  L.ucur = h->t2;
  L.u0 = h->state;
  L.unext = h->state;
  L.coef = {1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt};
  e = launch_stage(h, L);
  if (e == cudaSuccess) e = apply_filter(h, h->state);
  return e;
}

AdjointLaunch base_adjoint(DgswHandle h) {
  AdjointLaunch A;
  A.n = h->dom.elem_n.empty() ? 0 : h->dom.elem_n[0];
  A.n_elem = h->dom.n_elem;
  A.nbr = h->nbr;
  A.jac = h->jac;
  A.eoT = h->eoT;
  A.variant = h->adj_variant;
  return A;
}

// Times both work splits of the adjoint kernel on the handle's state (read
// only; the output goes to t1) and keeps the faster.  Both give the same bits.
cudaError_t adjoint_autotune(DgswHandle h) {
  cudaEvent_t e0, e1;
  cudaError_t err = cudaEventCreate(&e0);
  if (err != cudaSuccess) return err;
  err = cudaEventCreate(&e1);
  if (err != cudaSuccess) {
    cudaEventDestroy(e0);
    return err;
  }
  float best = -1.0f;
  int choice = 0;
  for (int v = 0; v < 2 && err == cudaSuccess; ++v) {
    AdjointLaunch A = base_adjoint(h);
    A.variant = v;
    A.x = h->state;
    A.out = h->t1;
    A.alpha = 1.0;
    A.c = 1e-4;
    err = launch_adjoint_fp64(A, h->stream);  // warm-up
    if (err == cudaSuccess) err = cudaEventRecord(e0, h->stream);
    for (int r = 0; r < 5 && err == cudaSuccess; ++r) err = launch_adjoint_fp64(A, h->stream);
    if (err == cudaSuccess) err = cudaEventRecord(e1, h->stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    h->adj_tune_ms[v] = ms / 5.0;
    if (err == cudaSuccess && (best < 0.0f || ms < best)) {
      best = ms;
      choice = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err == cudaSuccess) {
    h->adj_variant = choice;
    h->adj_tuned = true;
  }
  return err;
}

// One step of the discrete adjoint of Rk3HesthavenSsp (Rk3HesthavenSsp.cpp:63-80)
// on h->adj.  Reverse of u1 = u0 + dt L u0, u2 = 3/4 u0 + 1/4 (u1 + dt L u1),
// u3 = 1/3 u0 + 2/3 (u2 + dt L u2):
//   m2 = 2/3 (l + dt L^T l);  m1 = 1/4 (m2 + dt L^T m2);
//   l <- m1 + dt L^T m1 + 3/4 m2 + 1/3 l.
cudaError_t enqueue_adjoint_step(DgswHandle h, double dt) {
  AdjointLaunch A = base_adjoint(h);
  A.x = h->adj;
  A.out = h->t1;
  A.alpha = 2.0 / 3.0;
  A.c = (2.0 / 3.0) * dt;
  cudaError_t e = launch_adjoint_fp64(A, h->stream);
  if (e != cudaSuccess) return e;
  A = base_adjoint(h);
  A.x = h->t1;
  A.y = h->adj;
  A.out = h->t2;
  A.alpha = 0.25;
  A.c = 0.25 * dt;
  A.out2 = h->adjz;
  A.alpha2 = 0.75;
  A.beta2 = 1.0 / 3.0;
  e = launch_adjoint_fp64(A, h->stream);
  if (e != cudaSuccess) return e;
  A = base_adjoint(h);
  A.x = h->t2;
  A.y = h->adjz;
  A.out = h->adj;
  A.alpha = 1.0;
  A.beta = 1.0;
  A.c = dt;
  return launch_adjoint_fp64(A, h->stream);
}

// One mixed-precision step of the plain operator (taylor_df.cu) or of its
// adjoint: the step map is the Taylor polynomial 1 + dt L + (dt L)^2/2 +
// (dt L)^3/6, so
//   W1 = dt L u,  W2 = dt L W1,  W3 = dt L W2,  u += W1 + W2/2 + W3/6
// (L^T and the adjoint state for the adjoint), with double-float increments
// formed in FP32 arithmetic.  The misfit forward of a mixed-precision handle
// steps with it (its residuals must hold ~1e-8 of themselves over thousands
// of steps), on the state; the adjoint on h->adj.
// One launch (kind 0, 1, 2) of the Taylor step over the elements
// [begin, begin + count), on stream s.
cudaError_t taylor_launch(DgswHandle h, double dt, bool transpose, int kind, int64_t begin,
                          int64_t count, cudaStream_t s) {
  const int64_t size = h->dom.offset.back();
  float2* w1 = h->adj32;
  float2* w2 = h->adj32 + size;
  double* u = transpose ? h->adj : h->state;
  TaylorLaunch A;
  A.n = h->dom.elem_n[0];
  A.n_elem = count;
  A.elem_begin = begin;
  A.transpose = transpose;
  A.dt = dt;
  A.nbr = h->nbr;
  A.jac = h->jac;
  A.eo = transpose ? h->eoT : h->eo;
  A.gamma2 = transpose ? 0.0 : h->cfg.gamma2;
  A.kind = kind;
  if (kind == 0) {
    A.x64 = u;
    A.outp = w1;
  } else if (kind == 1) {
    A.xp = w1;
    A.outp = w2;
  } else {
    A.xp = w2;
    A.l64 = u;
    A.w1 = w1;
  }
  return launch_taylor_df(A, s);
}

cudaError_t enqueue_taylor_step(DgswHandle h, double dt, bool transpose) {
  const int64_t size = h->dom.offset.back();
  float2* w1 = h->adj32;
  float2* w2 = h->adj32 + size;
  double* u = transpose ? h->adj : h->state;
  TaylorLaunch A;
  A.n = h->dom.elem_n[0];
  A.n_elem = h->dom.n_elem;
  A.transpose = transpose;
  A.dt = dt;
  A.nbr = h->nbr;
  A.jac = h->jac;
  A.eo = transpose ? h->eoT : h->eo;
  A.gamma2 = transpose ? 0.0 : h->cfg.gamma2;
  A.kind = 0;
  A.x64 = u;
  A.outp = w1;
  cudaError_t e = launch_taylor_df(A, h->stream);
  if (e != cudaSuccess) return e;
  A.kind = 1;
  A.x64 = nullptr;
  A.xp = w1;
  A.outp = w2;
  e = launch_taylor_df(A, h->stream);
  if (e != cudaSuccess) return e;
  A.kind = 2;
  A.xp = w2;
  A.outp = nullptr;
  A.l64 = u;
  A.w1 = w1;
  return launch_taylor_df(A, h->stream);
}

cudaError_t capture_adjoint_steps(DgswHandle h, double dt, int steps, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = cudaSuccess;
  for (int s = 0; s < steps && le == cudaSuccess; ++s)
    le = mixed(h) || dfloat(h) ? enqueue_taylor_step(h, dt, true) : enqueue_adjoint_step(h, dt);
  e = cudaStreamEndCapture(h->stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return le;
  }
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// the two increment blocks of the mixed-precision Taylor step
int taylor_buffers(DgswHandle h) {
  if (h->adj32) return DGSW_OK;
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  DGSW_CUDA(h, cudaMalloc(&h->adj32, 2 * h->dom.offset.back() * sizeof(float2)));
  return DGSW_OK;
}

// steps mixed-precision Taylor steps of the state (the misfit forward of a
// mixed-precision handle)
cudaError_t capture_taylor_steps(DgswHandle h, double dt, int steps, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = cudaSuccess;
  for (int s = 0; s < steps && le == cudaSuccess; ++s) le = enqueue_taylor_step(h, dt, false);
  e = cudaStreamEndCapture(h->stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return le;
  }
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

cudaError_t capture_steps(DgswHandle h, double dt, int steps, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t le = cudaSuccess;
  for (int s = 0; s < steps && le == cudaSuccess; ++s) le = enqueue_step(h, dt);
  e = cudaStreamEndCapture(h->stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return le;
  }
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

// AdamsBashforth handle set-up: step levels, the level-sorted element list,
// the schedule (whose dry run sizes the history rings) and the rings.
int adams_init(DgswHandle h, const DgswConfig& cfg) {
  if (h->refined || h->gauss || (mixed(h) && !h->curved) || (!h->dom.uniform && h->curved))
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "AdamsBashforth: Gauss-Lobatto, conforming elements (of any extents on bricks), FP64 "
                "(mixed precision on the shell)");
  const int64_t E = h->dom.n_elem;
  std::vector<int8_t> level(E, 0);
  for (int64_t e = 0; e < E; ++e) {
    const int l = cfg.step_levels ? cfg.step_levels[e] : 0;
    if (l < 0 || l >= kAbMaxLevels) return fail(h, DGSW_ERR_ARGUMENT, "step levels must be in [0, 3]");
    level[e] = (int8_t)l;
  }
  bool adj[kAbMaxLevels][kAbMaxLevels] = {};
  for (int64_t e = 0; e < E; ++e) {
    ++h->ab_count[level[e]];
    for (int f = 0; f < 6; ++f) {
      const int32_t nb = h->dom.neighbor[6 * e + f];
      if (nb >= 0) adj[level[e]][level[nb]] = true;  // < 0: the shell's boundary spheres
    }
  }
  // the level list, each level's elements grouped by extent
  std::vector<int32_t> list;
  list.reserve(E);
  for (int l = 0; l < kAbMaxLevels; ++l)
    for (int n = kMinN; n <= kMaxN; ++n) {
      h->ab_cls_begin[l][n] = (int32_t)list.size();
      for (int64_t e = 0; e < E; ++e)
        if (level[e] == l && h->dom.elem_n[e] == n) {
          list.push_back((int32_t)e);
          h->ab_points[l] += (int64_t)n * n * n;
        }
      h->ab_cls_count[l][n] = (int32_t)list.size() - h->ab_cls_begin[l][n];
    }
  std::string err;
  const int order = cfg.stepper_order ? cfg.stepper_order : 3;
  if (!h->ab.init(order, adj, h->ab_count, &err)) return fail(h, DGSW_ERR_ARGUMENT, err);
  cudaError_t e;
  if ((e = upload(&h->ab_list, list)) != cudaSuccess) return cuda_fail(h, e, "upload level list");
  if ((e = upload(&h->ab_level, level)) != cudaSuccess) return cuda_fail(h, e, "upload levels");
  h->ab_level_host = level;
  const int n = h->dom.elem_n[0];
  const size_t slots = (size_t)h->ab.ring_slots();
  if (mixed(h)) {
    if ((e = cudaMalloc(&h->ab_F32, slots * h->dom.offset.back() * sizeof(float))) != cudaSuccess)
      return cuda_fail(h, e, "cudaMalloc time-derivative ring");
  } else if ((e = cudaMalloc(&h->ab_F, slots * h->dom.offset.back() * sizeof(double))) !=
             cudaSuccess) {
    return cuda_fail(h, e, "cudaMalloc time-derivative ring");
  }
  // the shell records the whole state (its exterior points are reached
  // through the face offsets of the volume layout); bricks record the face w's
  // (12 n^2 per element: 6 faces x (own w, the neighbour's w))
  if (h->curved) {
    h->ab_total_b = E * 30 * (int64_t)n * n;  // face records, [6][5][N^2] per element
  } else {
    std::vector<int64_t> boff(E + 1, 0);
    for (int64_t el = 0; el < E; ++el)
      boff[el + 1] = boff[el] + 12 * (int64_t)h->dom.elem_n[el] * h->dom.elem_n[el];
    h->ab_total_b = boff[E];
    if (h->general && (e = upload(&h->ab_boff, boff)) != cudaSuccess)
      return cuda_fail(h, e, "upload face-record offsets");
  }
  if ((e = cudaMalloc(&h->ab_B, slots * h->ab_total_b * sizeof(double))) != cudaSuccess)
    return cuda_fail(h, e, "cudaMalloc face-data ring");
  h->adams = true;
  return DGSW_OK;
}

// n_steps slabs of duration dt: the schedule's launches, one per tick
// position (the first slab after a restart begins with the self-start).
int adams_step(DgswHandle h, int n_steps, double dt) {
  if (!(dt > 0.0)) return fail(h, DGSW_ERR_ARGUMENT, "the slab duration must be positive");
  if (h->ab.started() && !(dt == h->ab_slab))
    return fail(h, DGSW_ERR_ARGUMENT,
                "AdamsBashforth steps slabs of one duration; set the state again to change it");
  h->ab.set_slab(dt);
  h->ab_slab = dt;
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  AbArgs A;
  A.u = h->state;
  A.u0 = h->t1;
  A.F = h->ab_F;
  A.B = h->ab_B;
  A.nbr = h->nbr;
  A.jac = h->jac;
  A.list = h->ab_list;
  A.level = h->ab_level;
  A.n_elem = h->dom.n_elem;
  A.gamma2 = h->cfg.gamma2;
  A.eo = h->eo;
  const int n = h->dom.elem_n[0];
  const int64_t per = (int64_t)kVars * n * n * n;
  if (h->filter_on && !h->curved)
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "AdamsBashforth applies the exponential filter on the curved shell only (the "
                "flat 3D scalar-wave executable does not filter)");
  std::vector<AbLaunch> launches;
  std::string err;
  for (int s = 0; s < n_steps; ++s) {
    if (!h->ab.started())  // initial values for the self-start resets
      DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (!h->ab.slab(&launches, &err)) return fail(h, DGSW_ERR_ARGUMENT, err);
    for (const AbLaunch& L : launches) {
      if (!h->curved && !h->general) {
        A.L = L;
        DGSW_CUDA(h, launch_adams_step(A, n, h->stream));
        continue;
      }
      if (!h->curved) {
        // elements of differing extents: the exterior w of the faces whose
        // neighbour has another extent, then one launch per extent class
        for (int c = kMinN; c <= kMaxN; ++c) {
          if (h->class_count[c] == 0 || h->pnc_count[c] == 0) continue;
          AbPncLaunch P;
          P.n = c;
          P.n_rec = h->pnc_count[c];
          P.rec_face = h->pnc_rec[c];
          P.elem_n = h->elem_n;
          P.nbr = h->nbr;
          P.level = h->ab_level;
          P.boff = h->ab_boff;
          P.total_b = h->ab_total_b;
          P.B = h->ab_B;
          P.op64 = h->op64;
          P.op_off = h->op_off;
          P.wext = h->pnc_wext[c];
          P.L = L;
          DGSW_CUDA(h, launch_adams_pnc_faces(P, h->stream));
        }
        for (int c = kMinN; c <= kMaxN; ++c) {
          if (h->class_count[c] == 0) continue;
          AbArgs G = A;
          G.L = L;
          int64_t total = 0;
          for (int j = 0; j < L.n_jobs; ++j) {
            const int l = L.job[j].level;
            G.L.job[j].begin = h->ab_cls_begin[l][c];
            G.L.job[j].count = h->ab_cls_count[l][c];
            total += G.L.job[j].count;
          }
          if (total == 0) continue;
          G.eo = h->class_eo[c];
          G.offset = h->offset;
          G.boff = h->ab_boff;
          G.total = h->dom.offset.back();
          G.total_b = h->ab_total_b;
          G.face_idx = h->pnc_face_idx;
          G.wext = h->pnc_wext[c];
          DGSW_CUDA(h, launch_adams_step(G, c, h->stream));
        }
        continue;
      }
      // shell: update (volume part and boundary delta), then the records
      // (time derivative with the radiation condition, and the state)
      CswAbArgs C;
      C.u = h->state;
      C.u0 = h->t1;
      C.F = h->ab_F;
      C.F32 = h->ab_F32;
      C.Fc32 = mixed(h) ? h->c_F32 : nullptr;
      C.U = h->ab_B;
      C.Fc = h->c_F;
      C.X = h->c_Xf;
      C.list = h->ab_list;
      C.level = h->ab_level;
      C.n = n;
      C.n_elem = h->dom.n_elem;
      C.gamma2 = h->cfg.gamma2;
      C.L = L;
      DGSW_CUDA(h, launch_csw_ab_update(C, h->stream));
      if (h->filter_on) {
        // dg::Actions::Filter after the step of every element that finished
        // one (the curved executable's step actions end with it), before
        // its new state is recorded
        for (int j = 0; j < L.n_jobs; ++j) {
          const AbLevelJob& J = L.job[j];
          if (!J.update || J.reset || J.count == 0) continue;
          if (mixed(h)) {
            // u + (F - I) u with the residual in double-float FP32
            MixedFilterLaunch R;
            R.n = n;
            R.n_tasks = J.count;
            R.tasks = h->ab_list + J.begin;
            R.F = h->filt + (size_t)n * kMaxN * kMaxN;
            R.u64 = h->state;
            R.out64 = h->state;
            DGSW_CUDA(h, launch_filter_residual(R, h->stream));
            continue;
          }
          FilterLaunch F;
          F.n = n;
          F.n_tasks = J.count;
          F.tasks = h->ab_list + J.begin;
          F.u = h->state;
          F.F = h->filt + (size_t)n * kMaxN * kMaxN;
          DGSW_CUDA(h, launch_filter(F, h->stream));
        }
      }
      for (int j = 0; j < L.n_jobs; ++j) {
        const AbLevelJob& J = L.job[j];
        if (mixed(h)) {
          // the record in mixed precision: dt u = L(u) by the compensated
          // double-float stage (FP32 result), the state copied as it is
          CswMixedLaunch M = base_csw_mixed(h);
          M.x64 = h->state;
          M.alpha = 0.0;
          M.c = 1.0;
          M.w32 = h->ab_F32 + (int64_t)J.rec_slot * h->dom.n_elem * per;
          M.frec = h->ab_B + (int64_t)J.rec_slot * h->ab_total_b;
          M.internal = 0;
          M.list = h->ab_list + J.begin;
          M.list_count = J.count;
          DGSW_CUDA(h, launch_csw_mixed(M, h->stream));
          continue;
        }
        CswLaunch R = base_csw(h);
        R.ucur = h->state;
        R.unext = h->ab_F + (int64_t)J.rec_slot * h->dom.n_elem * per;
        R.frec = h->ab_B + (int64_t)J.rec_slot * h->ab_total_b;
        R.a = 0.0;
        R.b = 0.0;
        R.c = 1.0;
        R.internal = 0;
        R.list = h->ab_list + J.begin;
        R.list_count = J.count;
        DGSW_CUDA(h, launch_csw_fp64(R, h->stream));
      }
    }
  }
  return DGSW_OK;
}

// ---- steps of a host-resident state ---------------------------------------
// The elements are cut into contiguous chunks.  Copy-in of chunk c, the
// three stages of chunk c and the copy-out of chunk c are separate
// operations; a stage of chunk c waits only for the previous stage (or the
// copy-in) of the chunks holding c's face neighbours.  The stage launches are
// issued in the order of a list schedule (plan_pipe) over several compute
// streams, so that launches that do not depend on each other fill each
// other's tails, and the copies of some chunks overlap the stages of others
// (the host link carries both directions at once).
bool pipelinable(DgswHandle h) {
  return !mixed(h) && !h->curved && !h->gauss && !h->general && !h->refined && !h->adams &&
         !h->filter_on && h->dom.n_elem >= 4096;
}

// The issue order of the 3 C stage launches (3 c + stage).  The model: the
// copies in land one after another in element order at the host link's rate
// (copy_s per element; all at time 0 without copies in), and the GPU runs one
// launch at a time, a stage of chunk c taking its elements times stage_s.
// Whenever the modelled GPU is free it takes, among the launches whose
// inputs are complete, one of the latest stage (its chunk's copy-out can
// start sooner); ties go to the lower chunk.
std::vector<int> plan_pipe(const std::vector<int64_t>& begin,
                           const std::vector<std::vector<int>>& deps, bool copy_in,
                           double copy_s, double stage_s) {
  const int C = (int)begin.size() - 1;
  std::vector<double> t_in(C, 0.0), done(3 * C, 0.0);
  double t = 0.0;
  if (copy_in)
    for (int c = 0; c < C; ++c) t_in[c] = (t += (begin[c + 1] - begin[c]) * copy_s);
  std::vector<int> level(C, 0), order;
  t = 0.0;
  while ((int)order.size() < 3 * C) {
    int best = -1;
    double next_ready = INFINITY;
    for (int c = 0; c < C; ++c) {
      const int st = level[c];
      if (st == 3) continue;
      bool ok = true;
      double ready = 0.0;
      for (int d : deps[c]) {
        if (st > 0 && level[d] < st) ok = false;
        else ready = std::max(ready, st == 0 ? t_in[d] : done[3 * d + st - 1]);
      }
      if (!ok) continue;
      if (ready > t) {
        next_ready = std::min(next_ready, ready);
        continue;
      }
      if (best < 0 || st > level[best]) best = c;
    }
    if (best < 0) {
      if (!(next_ready < INFINITY)) break;  // a dependency cycle: cannot happen
      t = next_ready;
      continue;
    }
    const int st = level[best]++;
    t += (begin[best + 1] - begin[best]) * stage_s;
    done[3 * best + st] = t;
    order.push_back(3 * best + st);
  }
  return order;
}

int pipe_init(DgswHandle h) {
  if (h->pipe_in) return DGSW_OK;
  const int64_t E = h->dom.n_elem;
  // Chunks of whole waves of the stage kernel in the middle of the element
  // order and thin ones at both ends.  On a periodic brick the chunks are
  // slabs on a ring, and the last chunk copied in holds back the stage
  // chains of the chunks around it (the last few and the first few), which
  // then form the tail of the step.  The thin chunks are as wide as the
  // neighbour reach (the largest distance around the ring of element indices
  // between an element and a face neighbour), so that the work held back is
  // whole neighbour layers.
  int64_t reach = 1;
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < 6; ++f) {
      const int64_t d = std::llabs(h->dom.neighbor[6 * e + f] - e);
      reach = std::max(reach, std::min(d, E - d));
    }
  // The middle chunks are the fewest whole waves that span the neighbour
  // reach (at 32^3 x 8^3: 2 x 912 elements with 6 resident blocks per SM,
  // 1 x 1216 with 8).
  const int64_t wave = stage_fp64_wave_elements(h->dom.elem_n[0], h->stage_variant);
  const int64_t thick = std::max<int64_t>(
      512, wave > 0 && E >= 24 * wave ? wave * ((reach + wave - 1) / wave) : E / 16);
  const int64_t thin = std::min(thick, std::max<int64_t>(256, reach));
  const int n_edge = std::max(1, h->pipe_edge_chunks);
  h->chunk_begin.assign(1, 0);
  for (int k = 0; k < n_edge && h->chunk_begin.back() + thin < E; ++k)
    h->chunk_begin.push_back(h->chunk_begin.back() + thin);
  const int64_t tail_start = std::max(h->chunk_begin.back(), E - n_edge * thin);
  while (h->chunk_begin.back() + thick <= tail_start)
    h->chunk_begin.push_back(h->chunk_begin.back() + thick);
  if (h->chunk_begin.back() < tail_start) h->chunk_begin.push_back(tail_start);
  while (h->chunk_begin.back() + thin < E) h->chunk_begin.push_back(h->chunk_begin.back() + thin);
  h->chunk_begin.push_back(E);
  const int C = (int)h->chunk_begin.size() - 1;
  std::vector<int> chunk_of(E);
  for (int c = 0; c < C; ++c)
    for (int64_t e = h->chunk_begin[c]; e < h->chunk_begin[c + 1]; ++e) chunk_of[e] = c;
  h->chunk_deps.assign(C, {});
  for (int c = 0; c < C; ++c) {
    std::vector<char> need(C, 0);
    need[c] = 1;
    for (int64_t e = h->chunk_begin[c]; e < h->chunk_begin[c + 1]; ++e)
      for (int f = 0; f < 6; ++f) need[chunk_of[h->dom.neighbor[6 * e + f]]] = 1;
    for (int d = 0; d < C; ++d)
      if (need[d]) h->chunk_deps[c].push_back(d);
  }
  // the model's rates: the host link at pipe_link_gbs (each direction's
  // share with both busy; a faster link in the model issues launches that
  // wait on copies too early, where they hold up their stream); a stage at
  // pipe_stage_ns per element if set, else at the launch time the autotuner
  // measured on the whole state, else at 0.1 ns per point
  const int64_t pts = (int64_t)h->dom.elem_n[0] * h->dom.elem_n[0] * h->dom.elem_n[0];
  const double copy_s = kVars * pts * sizeof(double) / (h->pipe_link_gbs * 1e9);
  const double tuned_ms = h->tuned ? h->tune_ms[h->stage_variant] : 0.0;
  // (double-float launches: ~3.6e-11 s per point, measured at 32^3 x 8^3)
  const double stage_s = h->pipe_stage_ns > 0.0 ? h->pipe_stage_ns * 1e-9
                         : tuned_ms > 0.0       ? tuned_ms * 1e-3 / E
                         : dfloat(h)            ? pts * 3.6e-11
                                                : pts * 1e-10;
  const int n_streams = std::max(1, h->pipe_streams);
  for (int k = 0; k < 2; ++k) {
    h->pipe_order[k] = plan_pipe(h->chunk_begin, h->chunk_deps, k == 1, copy_s, stage_s);
    if ((int)h->pipe_order[k].size() != 3 * C)
      return fail(h, DGSW_ERR_ARGUMENT, "chunk schedule did not complete");
  }
  // The launches that need the last chunk copied in, directly or through an
  // earlier stage (the ring's seam), go to a stream of their own with the
  // highest priority: they wait there for the copy without holding up other
  // launches, and no other launch needs them.  They start as soon as the
  // copy lands.
  h->pipe_seam_set.assign(3 * C, 0);
  for (int st = 0; st < 3; ++st)
    for (int c = 0; c < C; ++c)
      for (int d : h->chunk_deps[c])
        if (st == 0 ? d == C - 1 : h->pipe_seam_set[3 * d + st - 1] != 0) h->pipe_seam_set[3 * c + st] = 1;
  int least = 0, greatest = 0;
  DGSW_CUDA(h, cudaDeviceGetStreamPriorityRange(&least, &greatest));
  DGSW_CUDA(h, cudaStreamCreateWithPriority(&h->pipe_seam, cudaStreamNonBlocking, greatest));
  DGSW_CUDA(h, cudaStreamCreateWithFlags(&h->pipe_in, cudaStreamNonBlocking));
  DGSW_CUDA(h, cudaStreamCreateWithFlags(&h->pipe_out, cudaStreamNonBlocking));
  h->pipe_aux.assign(n_streams - 1, nullptr);
  for (cudaStream_t& s : h->pipe_aux)
    DGSW_CUDA(h, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  h->pipe_ev.assign(4 * C + 2, nullptr);
  for (cudaEvent_t& ev : h->pipe_ev)
    DGSW_CUDA(h, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  return DGSW_OK;
}

// One SSP-RK3 step of the device state, chunked; with copy_in the chunks are
// first copied from host_u, with copy_out copied back as they finish.
int pipelined_step(DgswHandle h, double* host_u, double dt, bool copy_in, bool copy_out) {
  const int C = (int)h->chunk_begin.size() - 1;
  const int64_t per = kVars * (int64_t)h->dom.elem_n[0] * h->dom.elem_n[0] * h->dom.elem_n[0];
  auto ev = [&](int kind, int c) { return h->pipe_ev[4 * c + kind]; };  // 0 in, 1-3 stages
  cudaEvent_t start = h->pipe_ev[4 * C], done = h->pipe_ev[4 * C + 1];
  std::vector<cudaStream_t> cs(1, h->stream);
  cs.insert(cs.end(), h->pipe_aux.begin(), h->pipe_aux.end());
  const int S = (int)cs.size();
  cs.push_back(h->pipe_seam);  // index S: the seam's launches when copying in
  // everything already queued on the handle's stream comes first
  DGSW_CUDA(h, cudaEventRecord(start, h->stream));
  for (int s = 1; s <= S; ++s) DGSW_CUDA(h, cudaStreamWaitEvent(cs[s], start, 0));
  if (copy_in) {
    DGSW_CUDA(h, cudaStreamWaitEvent(h->pipe_in, start, 0));
    for (int c = 0; c < C; ++c) {
      const int64_t off = h->chunk_begin[c] * per, n = (h->chunk_begin[c + 1] - h->chunk_begin[c]) * per;
      DGSW_CUDA(h, cudaMemcpyAsync(h->state + off, host_u + off, n * sizeof(double),
                                   cudaMemcpyHostToDevice, h->pipe_in));
      DGSW_CUDA(h, cudaEventRecord(ev(0, c), h->pipe_in));
    }
  }
  if (copy_out) DGSW_CUDA(h, cudaStreamWaitEvent(h->pipe_out, start, 0));
  const StageCoef coef[3] = {{0.0, 1.0, dt}, {0.75, 0.25, 0.25 * dt},
                             {1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt}};
  const double* in[3] = {h->state, h->t1, h->t2};
  double* out[3] = {h->t1, h->t2, h->state};
  // the launches go round-robin to the streams in issue order (the seam's to
  // its own stream); each waits on the launches (or copies) it needs that
  // went to other streams
  std::vector<int> stream_of(3 * C, -1);
  const std::vector<int>& order = h->pipe_order[copy_in ? 1 : 0];
  int rr = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    const int c = order[i] / 3, st = order[i] % 3;
    const int s = copy_in && h->pipe_seam_set[order[i]] ? S : (rr++ % S);
    cudaStream_t q = cs[s];
    for (int d : h->chunk_deps[c]) {
      if (st == 0) {
        if (copy_in) DGSW_CUDA(h, cudaStreamWaitEvent(q, ev(0, d), 0));
      } else {
        const int src = stream_of[3 * d + st - 1];
        if (src < 0) return fail(h, DGSW_ERR_ARGUMENT, "chunk schedule out of order");
        if (src != s) DGSW_CUDA(h, cudaStreamWaitEvent(q, ev(st, d), 0));
      }
    }
    if (dfloat(h)) {
      // the Taylor step's three launches take the stages' places: W1 from
      // the state, W2 from W1, W3 with the state's update in place (its
      // readers, the W1 launches of the neighbouring chunks, precede it
      // through the W2 launches it waits for)
      DGSW_CUDA(h, taylor_launch(h, dt, false, st, h->chunk_begin[c],
                                 h->chunk_begin[c + 1] - h->chunk_begin[c], q));
    } else {
      StageLaunch L = base_launch(h);
      L.mode = st == 0 ? kModeStageFirst : kModeStage;
      L.ucur = in[st];
      L.u0 = h->state;
      L.unext = out[st];
      L.coef = coef[st];
      L.elem_begin = h->chunk_begin[c];
      L.elem_count = h->chunk_begin[c + 1] - h->chunk_begin[c];
      DGSW_CUDA(h, launch_stage_fp64(L, q));
    }
    DGSW_CUDA(h, cudaEventRecord(ev(st + 1, c), q));
    stream_of[3 * c + st] = s;
    if (st == 2 && copy_out) {
      const int64_t off = h->chunk_begin[c] * per;
      const int64_t n = (h->chunk_begin[c + 1] - h->chunk_begin[c]) * per;
      DGSW_CUDA(h, cudaStreamWaitEvent(h->pipe_out, ev(3, c), 0));
      DGSW_CUDA(h, cudaMemcpyAsync(host_u + off, h->state + off, n * sizeof(double),
                                   cudaMemcpyDeviceToHost, h->pipe_out));
    }
  }
  // the handle's stream resumes after every chunk's last stage (and copy)
  for (int s = 1; s <= S; ++s) {
    DGSW_CUDA(h, cudaEventRecord(done, cs[s]));
    DGSW_CUDA(h, cudaStreamWaitEvent(h->stream, done, 0));
  }
  if (copy_out) {
    DGSW_CUDA(h, cudaEventRecord(done, h->pipe_out));
    DGSW_CUDA(h, cudaStreamWaitEvent(h->stream, done, 0));
  }
  return DGSW_OK;
}

// pipelined_step replayed from a graph when host_u is pinned (the graph's
// copy nodes need page-locked memory); pageable buffers are issued directly
int run_pipelined(DgswHandle h, double* host_u, double dt, bool copy_in, bool copy_out) {
  cudaPointerAttributes attr;
  const bool pinned =
      cudaPointerGetAttributes(&attr, host_u) == cudaSuccess && attr.type == cudaMemoryTypeHost;
  cudaGetLastError();  // pageable pointers may leave an error on some runtimes
  if (!pinned) return pipelined_step(h, host_u, dt, copy_in, copy_out);
  const int kind = copy_in && copy_out ? 0 : (copy_in ? 1 : 2);
  cudaGraphExec_t& exec = h->pipe_graph[kind];
  if (!exec || h->pipe_graph_ptr[kind] != host_u || !(h->pipe_graph_dt[kind] == dt)) {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    DGSW_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = pipelined_step(h, host_u, dt, copy_in, copy_out);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "capture of the pipelined step");
    const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      exec = nullptr;
      return cuda_fail(h, ei, "instantiate the pipelined step");
    }
    h->pipe_graph_ptr[kind] = host_u;
    h->pipe_graph_dt[kind] = dt;
  }
  DGSW_CUDA(h, cudaGraphLaunch(exec, h->stream));
  return DGSW_OK;
}

}  // namespace

extern "C" {

int dgsw_step_host(DgswHandle h, double* host_u, int n_steps, double dt) {
  if (!h || !host_u) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (n_steps < 1 || !std::isfinite(dt)) return fail(h, DGSW_ERR_ARGUMENT, "bad step arguments");
  if (int rc = select_device(h)) return rc;
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  if (!pipelinable(h)) {
    // the same device steps, with whole-state copies around them
    DGSW_CUDA(h, cudaMemcpyAsync(h->state, host_u, bytes, cudaMemcpyHostToDevice, h->stream));
    if (h->adams) h->ab.restart();
    if (int rc = dgsw_step(h, n_steps, dt)) return rc;
    DGSW_CUDA(h, cudaMemcpyAsync(host_u, h->state, bytes, cudaMemcpyDeviceToHost, h->stream));
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    return check_device_error(h);
  }
  if (!h->tuned && tunable(h)) {
    destroy_graphs(h);
    if (int rc = autotune(h, false)) return rc;
  }
  if (int rc = pipe_init(h)) return rc;
  if (int rc = run_pipelined(h, host_u, dt, true, n_steps == 1)) return rc;
  if (n_steps > 2)
    if (int rc = dgsw_step(h, n_steps - 2, dt)) return rc;
  if (n_steps > 1)
    if (int rc = run_pipelined(h, host_u, dt, false, true)) return rc;
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int dgsw_adams_info(DgswHandle h, int* ring_slots, int64_t* ticks_per_slab,
                    int64_t* rhs_points_per_slab, int* launches_per_slab) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (!h->adams) return fail(h, DGSW_ERR_UNSUPPORTED, "not an AdamsBashforth handle");
  int64_t pts = 0;
  int finest = 0;
  for (int l = 0; l < kAbMaxLevels; ++l)
    if (h->ab_count[l]) {
      pts += h->ab_points[l] * h->ab.steps_per_slab(l);
      finest = l;
    }
  if (ring_slots) *ring_slots = h->ab.ring_slots();
  if (ticks_per_slab) *ticks_per_slab = h->ab.ticks_per_slab();
  if (rhs_points_per_slab) *rhs_points_per_slab = pts;
  if (launches_per_slab) *launches_per_slab = 1 << finest;
  return DGSW_OK;
}

int dgsw_abi_version(void) { return DGSW_ABI_VERSION; }

const char* dgsw_last_error(DgswHandle h) {
  if (h) return h->err.c_str();
  return g_last_error.c_str();
}

// Builds the host maps of either system.
bool any_domain(const DgswConfig& cfg, Domain* dom, ShellGeometry* geo, std::string* err,
                RefinedMaps* rmaps = nullptr) {
  if (cfg.refined) {
    RefinedMaps local;
    return build_refined_domain(cfg, dom, rmaps ? rmaps : &local, err);
  }
  if (cfg.system == DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D) return build_shell_domain(cfg, dom, geo, err);
  return build_domain(cfg, dom, err);
}

int dgsw_count_elements(const DgswConfig* cfg, int64_t* n_elements, int64_t* state_doubles) {
  if (!cfg) return fail(nullptr, DGSW_ERR_ARGUMENT, "null config");
  Domain dom;
  ShellGeometry geo;
  std::string err;
  if (!any_domain(*cfg, &dom, &geo, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  if (n_elements) *n_elements = dom.n_elem;
  if (state_doubles) *state_doubles = dom.offset.back();
  return DGSW_OK;
}

int dgsw_index_maps(const DgswConfig* cfg, uint64_t* ids, int32_t* nbr, int32_t* mortar) {
  if (!cfg) return fail(nullptr, DGSW_ERR_ARGUMENT, "null config");
  Domain dom;
  ShellGeometry geo;
  std::string err;
  if (!any_domain(*cfg, &dom, &geo, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  if (ids) std::memcpy(ids, dom.element_id.data(), dom.n_elem * sizeof(uint64_t));
  if (nbr) std::memcpy(nbr, dom.neighbor.data(), 6 * dom.n_elem * sizeof(int32_t));
  if (mortar)
    for (int64_t e = 0; e < dom.n_elem; ++e)
      for (int dir = 0; dir < 6; ++dir) {
        const int32_t nb = dom.neighbor[6 * e + dir];
        if (nb < 0) {
          mortar[6 * e + dir] = 0;
          continue;
        }
        const int a = dom.elem_n[e], b = dom.elem_n[nb];
        mortar[6 * e + dir] = a > b ? a : b;
      }
  if (!dom.block_ids_fit)
    return fail(nullptr, DGSW_ERR_UNSUPPORTED, "a block id does not fit in 8 bits");
  return DGSW_OK;
}

int dgsw_shell_geometry(const DgswConfig* cfg, double* xyz, double* inv_jac, int32_t* perm) {
  if (!cfg) return fail(nullptr, DGSW_ERR_ARGUMENT, "null config");
  if (cfg->system != DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D)
    return fail(nullptr, DGSW_ERR_ARGUMENT, "not a curved (shell) configuration");
  Domain dom;
  ShellGeometry geo;
  std::string err;
  if (!build_shell_domain(*cfg, &dom, &geo, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  if (xyz) std::memcpy(xyz, geo.xyz.data(), geo.xyz.size() * sizeof(double));
  if (inv_jac) std::memcpy(inv_jac, geo.inv_jac.data(), geo.inv_jac.size() * sizeof(double));
  if (perm) std::memcpy(perm, geo.face_perm.data(), geo.face_perm.size() * sizeof(int32_t));
  return DGSW_OK;
}

int dgsw_refined_mortars(const DgswConfig* cfg, int32_t* slots, int32_t* sizes) {
  if (!cfg || !cfg->refined) return fail(nullptr, DGSW_ERR_ARGUMENT, "not a refined lattice");
  Domain dom;
  RefinedMaps rm;
  std::string err;
  if (!build_refined_domain(*cfg, &dom, &rm, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  if (slots) std::memcpy(slots, rm.slots.data(), rm.slots.size() * sizeof(int32_t));
  if (sizes) std::memcpy(sizes, rm.sizes.data(), rm.sizes.size() * sizeof(int32_t));
  return DGSW_OK;
}

int dgsw_amr_matrix(int src_extent, int dst_extent, int child, double* M) {
  if (!M) return fail(nullptr, DGSW_ERR_ARGUMENT, "null argument");
  if (!amr_matrix(src_extent, dst_extent, child, M))
    return fail(nullptr, DGSW_ERR_ARGUMENT,
                "need extents in [2, 12], child 0 (Full), 1 (LowerHalf) or 2 (UpperHalf), and "
                "a half-interval target at least as fine as its source");
  return DGSW_OK;
}

int dgsw_amr_project_device(DgswHandle h, int n_vars, int64_t n_in, const int64_t* in_offset,
                            const double* dev_in, int64_t n_out, const int32_t* src,
                            const int32_t* src_extents, const int32_t* dst_extents,
                            const int8_t* child, const int64_t* out_offset, double* dev_out) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (n_out < 0 || n_vars < 1 || n_in < 1) return fail(h, DGSW_ERR_ARGUMENT, "bad sizes");
  if (n_out == 0) return DGSW_OK;
  if (!in_offset || !dev_in || !src || !src_extents || !dst_extents || !child || !out_offset ||
      !dev_out)
    return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (dev_in == dev_out) return fail(h, DGSW_ERR_ARGUMENT, "input and output must differ");
  if (n_out > INT32_MAX) return fail(h, DGSW_ERR_ARGUMENT, "too many target blocks");
  // one matrix per distinct (source extent, target extent, child size)
  std::map<std::tuple<int, int, int>, int64_t> mat_at;
  std::vector<double> mats;
  std::vector<int64_t> mat_off(3 * n_out);
  double M[kMaxN * kMaxN];
  for (int64_t k = 0; k < n_out; ++k) {
    if (src[k] < 0 || src[k] >= n_in)
      return fail(h, DGSW_ERR_ARGUMENT, "source block index out of range");
    for (int d = 0; d < 3; ++d) {
      const int se = src_extents[3 * k + d], de = dst_extents[3 * k + d], c = child[3 * k + d];
      const auto key = std::make_tuple(se, de, c);
      auto it = mat_at.find(key);
      if (it == mat_at.end()) {
        if (!amr_matrix(se, de, c, M))
          return fail(h, DGSW_ERR_ARGUMENT,
                      "bad projection: extents in [2, 12], child 0, 1 or 2, and a half-interval "
                      "target at least as fine as its source");
        it = mat_at.emplace(key, (int64_t)mats.size()).first;
        mats.insert(mats.end(), M, M + de * se);
      }
      mat_off[3 * k + d] = it->second;
    }
  }
  if (int rc = select_device(h)) return rc;
  // the tables live for this call only
  struct Temp {
    std::vector<void*> p;
    ~Temp() {
      for (void* q : p) cudaFree(q);
    }
  } tmp;
  AmrLaunch L;
  L.n_vars = n_vars;
  L.n_out = n_out;
  auto up = [&](auto** dst, const auto* host, size_t n) {
    using T = typename std::remove_const<typename std::remove_pointer<decltype(host)>::type>::type;
    std::vector<T> v(host, host + n);
    T* d = nullptr;
    const cudaError_t e = upload(&d, v);
    if (d) tmp.p.push_back(d);
    *dst = d;
    return e;
  };
  DGSW_CUDA(h, up(&L.src, src, n_out));
  DGSW_CUDA(h, up(&L.src_ext, src_extents, 3 * n_out));
  DGSW_CUDA(h, up(&L.dst_ext, dst_extents, 3 * n_out));
  DGSW_CUDA(h, up(&L.mat_off, mat_off.data(), mat_off.size()));
  DGSW_CUDA(h, up(&L.mats, mats.data(), mats.size()));
  DGSW_CUDA(h, up(&L.in_off, in_offset, n_in));
  DGSW_CUDA(h, up(&L.out_off, out_offset, n_out));
  L.in = dev_in;
  L.out = dev_out;
  DGSW_CUDA(h, launch_amr_project(L, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return DGSW_OK;
}

int dgsw_half_projections(int n, int upper, double* P, double* R) {
  if (!half_projections(n, upper, P, R))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "n must be in [2, 12]");
  return DGSW_OK;
}

int dgsw_gauss_spectral(int n, double* x, double* w, double* D, double* ilo, double* ihi,
                        double* llo, double* lhi) {
  GaussTables g;
  if (!lg_spectral(n, &g)) return fail(nullptr, DGSW_ERR_ARGUMENT, "n must be in [2, 20]");
  for (int i = 0; i < n; ++i) {
    if (x) x[i] = g.x[i];
    if (w) w[i] = g.w[i];
    if (ilo) ilo[i] = g.lo[i];
    if (ihi) ihi[i] = g.hi[i];
    if (llo) llo[i] = g.lift_lo[i];
    if (lhi) lhi[i] = g.lift_hi[i];
  }
  if (D) std::memcpy(D, g.D, sizeof(double) * n * n);
  return DGSW_OK;
}

int dgsw_lgl_points_weights(int n, double* x, double* w) {
  if (!lgl_nodes_weights(n, x, w)) return fail(nullptr, DGSW_ERR_ARGUMENT, "n must be in [2, 20]");
  return DGSW_OK;
}

int dgsw_adams_coefficients(int n, const int64_t* ticks, int64_t start, int64_t end, double slab,
                            int64_t ticks_per_slab, double* out) {
  if (!adams_step_coefficients(n, ticks, start, end, slab, ticks_per_slab, out))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "need 0 <= n <= 8 and ticks_per_slab >= 1");
  return DGSW_OK;
}

int dgsw_lts_coefficients(int n_local, const int64_t* local_slab, const int64_t* local_tick,
                          int n_remote, const int64_t* remote_slab, const int64_t* remote_tick,
                          int64_t start, int64_t end, double slab, int64_t ticks_per_slab,
                          int local_order, int remote_order, int small_order, int max_out,
                          int32_t* out_local, int32_t* out_remote, double* out_coef) {
  if (n_local < 0 || n_remote < 0 || max_out < 0 || ticks_per_slab < 1 ||
      (n_local && (!local_slab || !local_tick)) || (n_remote && (!remote_slab || !remote_tick)) ||
      (max_out && (!out_local || !out_remote || !out_coef)))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "bad history or output arguments");
  std::vector<AbId> l(n_local), r(n_remote);
  for (int i = 0; i < n_local; ++i) l[i] = {local_slab[i], local_tick[i]};
  for (int i = 0; i < n_remote; ++i) r[i] = {remote_slab[i], remote_tick[i]};
  std::vector<AbTerm> terms;
  if (adams_lts_terms(l, r, start, end, local_order, remote_order, small_order, slab,
                      ticks_per_slab, &terms))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "the histories lack the data of the step");
  if ((int)terms.size() > max_out) return fail(nullptr, DGSW_ERR_ARGUMENT, "max_out too small");
  for (size_t i = 0; i < terms.size(); ++i) {
    out_local[i] = terms[i].local;
    out_remote[i] = terms[i].remote;
    out_coef[i] = terms[i].coef;
  }
  return (int)terms.size();
}

int dgsw_adams_schedule(int order, const int64_t* level_counts, const int32_t* adjacency,
                        double slab, int n_slabs, int max_jobs, DgswAdamsJob* jobs, int* n_jobs,
                        int64_t* ticks_per_slab, int* ring_slots) {
  if (!level_counts || !adjacency || n_slabs < 0 || max_jobs < 0 || (max_jobs && !jobs) ||
      !(slab > 0.0))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "bad schedule arguments");
  bool adj[kAbMaxLevels][kAbMaxLevels];
  int64_t cnt[kAbMaxLevels];
  for (int l = 0; l < kAbMaxLevels; ++l) {
    cnt[l] = level_counts[l];
    for (int m = 0; m < kAbMaxLevels; ++m) adj[l][m] = adjacency[kAbMaxLevels * l + m] != 0;
  }
  AdamsSchedule sched;
  std::string err;
  if (!sched.init(order, adj, cnt, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  sched.set_slab(slab);
  int count = 0, launch_index = 0;
  for (int s = 0; s < n_slabs; ++s) {
    std::vector<AbLaunch> launches;
    if (!sched.slab(&launches, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
    for (const AbLaunch& L : launches) {
      for (int j = 0; j < L.n_jobs; ++j) {
        if (count >= max_jobs) return fail(nullptr, DGSW_ERR_ARGUMENT, "max_jobs too small");
        const AbLevelJob& a = L.job[j];
        DgswAdamsJob& o = jobs[count++];
        std::memset(&o, 0, sizeof(o));
        o.launch = launch_index;
        o.level = a.level;
        o.update = a.update;
        o.reset = a.reset;
        o.rec_slot = a.rec_slot;
        o.n_vol = a.n_vol;
        for (int i = 0; i < a.n_vol; ++i) {
          o.vol_slot[i] = a.vol_slot[i];
          o.vol_c[i] = a.vol_c[i];
        }
        for (int m = 0; m < kAbMaxLevels; ++m) {
          const AbFaceTable& f = a.face[m];
          o.n_loc[m] = f.n_loc;
          o.n_rem[m] = f.n_rem;
          for (int i = 0; i < f.n_loc; ++i) {
            o.loc_slot[m][i] = f.loc_slot[i];
            o.loc_c[m][i] = f.loc_c[i];
          }
          for (int i = 0; i < f.n_rem; ++i) {
            o.rem_slot[m][i] = f.rem_slot[i];
            o.rem_c[m][i] = f.rem_c[i];
          }
        }
      }
      ++launch_index;
    }
  }
  if (n_jobs) *n_jobs = count;
  if (ticks_per_slab) *ticks_per_slab = sched.ticks_per_slab();
  if (ring_slots) *ring_slots = sched.ring_slots();
  return DGSW_OK;
}

int dgsw_differentiation_matrix(int n, double* D) {
  if (!lgl_diff_matrix(n, D)) return fail(nullptr, DGSW_ERR_ARGUMENT, "n must be in [2, 20]");
  return DGSW_OK;
}

int dgsw_mortar_projections(int ne, int nm, double* to_m, double* from_m) {
  if (!lgl_mortar_projections(ne, nm, to_m, from_m))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "need 2 <= ne <= nm <= 20");
  return DGSW_OK;
}

// Set-up of the mixed-precision batch path (stage_batch.cu): per element
// face-buffer offsets (6 N^2 values, rounded up to 4 so that every element's
// block starts 16-byte aligned), the three face buffers, the split tables of
// every extent, the task list and the launch shapes.  Tasks: the elements in
// windows of 256 consecutive elements, grouped by extent within a window
// (largest first) into tasks of at most batch_task_elements(n).
int batch_init(DgswHandle h) {
  const int64_t E = h->dom.n_elem;
  std::vector<int64_t> foff(E + 1, 0);
  for (int64_t e = 0; e < E; ++e) {
    const int64_t n = h->dom.elem_n[e];
    foff[e + 1] = foff[e] + (6 * n * n + 3) / 4 * 4;
  }
  h->bt_fsize = foff[E];
  cudaError_t e = upload(&h->bt_foff, foff);
  if (e != cudaSuccess) return cuda_fail(h, e, "upload face offsets");
  const size_t pad = 64;
  if ((e = cudaMalloc(&h->bt_fu, h->bt_fsize * sizeof(float2) + pad)) != cudaSuccess ||
      (e = cudaMalloc(&h->bt_fw1, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMalloc(&h->bt_fw2, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMalloc(&h->bt_fw3, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMalloc(&h->bt_raw, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess)
    return cuda_fail(h, e, "allocate face buffers");
  // the rounding pads are read by the copies: keep them finite
  if ((e = cudaMemset(h->bt_fu, 0, h->bt_fsize * sizeof(float2) + pad)) != cudaSuccess ||
      (e = cudaMemset(h->bt_fw1, 0, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMemset(h->bt_fw2, 0, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMemset(h->bt_fw3, 0, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess ||
      (e = cudaMemset(h->bt_raw, 0, h->bt_fsize * sizeof(float) + pad)) != cudaSuccess)
    return cuda_fail(h, e, "clear face buffers");
  // the producer faces sorted by (own extent, neighbour's extent), cut into
  // chunks of at most kBatchMapFaces faces of one pair
  {
    constexpr int kFacesPerChunk = kBatchMapFaces;
    std::vector<std::vector<std::pair<int64_t, int64_t>>> by_pair((kMaxN + 1) * (kMaxN + 1));
    for (int64_t el = 0; el < E; ++el) {
      const int n = h->dom.elem_n[el];
      for (int dir = 0; dir < 6; ++dir) {
        const int64_t nb = h->dom.neighbor[6 * el + dir];
        const int m = h->dom.elem_n[nb];
        by_pair[n * (kMaxN + 1) + m].emplace_back(foff[el] + (int64_t)dir * n * n,
                                                  foff[nb] + (int64_t)(dir ^ 1) * m * m);
      }
    }
    std::vector<int4> chunks;
    std::vector<int64_t> src, dst;
    src.reserve(6 * E);
    dst.reserve(6 * E);
    for (int n = kMinN; n <= kMaxN; ++n)
      for (int m = kMinN; m <= kMaxN; ++m) {
        const auto& fl = by_pair[n * (kMaxN + 1) + m];
        for (size_t i = 0; i < fl.size(); i += kFacesPerChunk) {
          const int cnt = (int)std::min<size_t>(kFacesPerChunk, fl.size() - i);
          chunks.push_back(make_int4(n | (m << 8), (int)src.size(), cnt, 0));
          for (int k = 0; k < cnt; ++k) {
            src.push_back(fl[i + k].first);
            dst.push_back(fl[i + k].second);
          }
        }
      }
    h->bt_nchunks = (int64_t)chunks.size();
    if ((e = upload(&h->bt_chunks, chunks)) != cudaSuccess ||
        (e = upload(&h->bt_face_src, src)) != cudaSuccess ||
        (e = upload(&h->bt_face_dst, dst)) != cudaSuccess)
      return cuda_fail(h, e, "upload face maps");
  }
  std::vector<float> dtab;
  batch_split_tables(&dtab);
  if ((e = upload(&h->bt_dtab, dtab)) != cudaSuccess) return cuda_fail(h, e, "upload split tables");
  constexpr int64_t kWindow = 256;
  bool present[kMaxN + 1] = {};
  for (int64_t el = 0; el < E; ++el) present[h->dom.elem_n[el]] = true;
  for (int n = kMinN; n <= kMaxN; ++n)
    if (present[n]) h->bt_nmax = n;
  for (int lst = 0; lst < 2; ++lst) {
    const int variant = lst == 0 ? 0 : 1;  // 128 / 256 threads per CTA
    if (h->bt_nmax > batch_max_extent(variant)) continue;
    std::vector<int2> tasks;
    std::vector<int32_t> elems;
    elems.reserve(E);
    for (int64_t w0 = 0; w0 < E; w0 += kWindow) {
      std::vector<int32_t> bucket[kMaxN + 1];
      for (int64_t el = w0; el < std::min(E, w0 + kWindow); ++el)
        bucket[h->dom.elem_n[el]].push_back((int32_t)el);
      for (int n = kMaxN; n >= kMinN; --n) {
        if (bucket[n].empty()) continue;
        const int gmax = batch_task_elements(n, variant);  // >= 1: n <= batch_max_extent
        for (size_t i = 0; i < bucket[n].size(); i += gmax) {
          const int g = (int)std::min<size_t>(gmax, bucket[n].size() - i);
          tasks.push_back(make_int2(n | (g << 8), (int)elems.size()));
          elems.insert(elems.end(), bucket[n].begin() + i, bucket[n].begin() + i + g);
        }
      }
    }
    h->bt_ntasks[lst] = (int64_t)tasks.size();
    if ((e = upload(&h->bt_tasks[lst], tasks)) != cudaSuccess) return cuda_fail(h, e, "upload tasks");
    if ((e = upload(&h->bt_elems[lst], elems)) != cudaSuccess) return cuda_fail(h, e, "upload tasks");
  }
  if (batch_variants() > DgswHandle_::kBtVariants)
    return fail(h, DGSW_ERR_UNSUPPORTED, "batch stage: more launch shapes than the handle holds");
  for (int v = 0; v < batch_variants(); ++v) {
    if (h->bt_nmax > batch_max_extent(v)) continue;
    for (int i = 0; i < 2; ++i) {
      size_t buf = 0, sb = 0;
      for (int n = kMinN; n <= kMaxN; ++n) {
        if (!present[n]) continue;
        size_t b1, s1;
        batch_smem_bytes(n, i == 0, h->cfg.gamma2 != 0.0, v, &b1, &s1);
        buf = std::max(buf, b1);
        sb = std::max(sb, s1);
      }
      const size_t total = batch_smem_total(v, buf, sb);
      if (total > 227 * 1024)
        return fail(h, DGSW_ERR_UNSUPPORTED, "batch stage: shared memory of a task exceeds 227 KB");
      h->bt_buf[v][i] = (int)buf;
      h->bt_s[v][i] = (int)sb;
      if ((e = batch_grid(i == 0, h->cfg.gamma2 != 0.0, v, total, &h->bt_grid[v][i])) != cudaSuccess)
        return cuda_fail(h, e, "batch stage occupancy");
    }
  }
  // the shape compiled for the domain's largest extent, 128 threads per CTA
  // where an element fits, single-buffered where extents are at most 10
  h->bt_variant = h->bt_nmax <= batch_max_extent(3) ? 3 : (h->bt_nmax <= batch_max_extent(0) ? 0 : 1);
  const char* env = std::getenv("DGSW_BATCH_VARIANT");
  if (env) {
    const int v = std::atoi(env);
    if (v >= 0 && v < batch_variants() && h->bt_nmax <= batch_max_extent(v)) h->bt_variant = v;
  }
  h->batch = true;
  return DGSW_OK;
}

int dgsw_create(const DgswConfig* cfg, DgswHandle* out) {
  if (!cfg || !out) return fail(nullptr, DGSW_ERR_ARGUMENT, "null argument");
  *out = nullptr;
  DgswHandle h = new (std::nothrow) DgswHandle_;
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "out of host memory");
  h->cfg = *cfg;
  std::string err;
  ShellGeometry geo;
  h->curved = cfg->system == DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D;
  h->refined = cfg->refined != nullptr;
  RefinedMaps rmaps;
  if (!any_domain(*cfg, &h->dom, &geo, &err, &rmaps)) {
    delete h;
    return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  }
  h->cfg.bricks = nullptr;  // copies live in h->dom
  h->cfg.points_per_element = nullptr;
  if (h->curved) h->shell = *cfg->shell;
  if (h->refined) {
    h->rbrick = *cfg->refined;
    const int nb = cfg->refined->blocks[0] * cfg->refined->blocks[1] * cfg->refined->blocks[2];
    h->rlevels.assign(cfg->refined->levels, cfg->refined->levels + nb);
    h->rbrick.levels = h->rlevels.data();
  }
  h->cfg.refined = h->refined ? &h->rbrick : nullptr;
  h->cfg.shell = h->curved ? &h->shell : nullptr;
  h->gauss = cfg->quadrature == DGSW_QUADRATURE_GAUSS;
  if (cfg->quadrature != DGSW_QUADRATURE_GAUSS_LOBATTO && !h->gauss) {
    delete h;
    return fail(nullptr, DGSW_ERR_ARGUMENT, "unknown quadrature");
  }
  if (h->gauss && (h->curved || !h->dom.uniform || cfg->precision != DGSW_PRECISION_FP64)) {
    delete h;
    return fail(nullptr, DGSW_ERR_UNSUPPORTED,
                "Gauss quadrature: flat system, one extent for every element, FP64 precision");
  }
  if (cfg->precision == DGSW_PRECISION_DOUBLE_FLOAT &&
      (h->curved || h->refined || h->gauss || !h->dom.uniform ||
       cfg->time_stepper != DGSW_STEPPER_RK3_HESTHAVEN_SSP)) {
    delete h;
    return fail(nullptr, DGSW_ERR_UNSUPPORTED,
                "double-float precision: flat system, one extent, Rk3HesthavenSsp");
  }

  if (cfg->time_stepper == DGSW_STEPPER_ADAMS_BASHFORTH) {
    // checked before any device work, so that a bad request fails the same
    // way with or without a GPU
    int code = DGSW_OK;
    const char* why = nullptr;
    if (h->refined || h->gauss || (!h->dom.uniform && h->curved) ||
        (cfg->precision != DGSW_PRECISION_FP64 && !h->curved)) {
      code = DGSW_ERR_UNSUPPORTED;
      why = "AdamsBashforth: Gauss-Lobatto, conforming elements (of any extents on bricks), FP64 "
            "(mixed precision on the shell)";
    } else if (cfg->stepper_order < 0 || cfg->stepper_order > kAbMaxOrder) {
      code = DGSW_ERR_ARGUMENT;
      why = "AdamsBashforth order must be in [1, 8] (0: 3)";
    } else if (cfg->step_levels) {
      for (int64_t e = 0; e < h->dom.n_elem && !why; ++e)
        if (cfg->step_levels[e] < 0 || cfg->step_levels[e] >= kAbMaxLevels) {
          code = DGSW_ERR_ARGUMENT;
          why = "step levels must be in [0, 3]";
        }
    }
    if (why) {
      delete h;
      return fail(nullptr, code, why);
    }
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= cfg->device || cfg->device < 0) {
    delete h;
    return fail(nullptr, DGSW_ERR_NO_DEVICE, "no CUDA device with that ordinal");
  }
  h->device = cfg->device;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess || prop.major != 10) {
    delete h;
    return fail(nullptr, DGSW_ERR_NO_DEVICE, "device is not a Blackwell (sm_10x) GPU");
  }
  int rc = select_device(h);
  if (rc) {
    delete h;
    return rc;
  }
  auto bail = [&](cudaError_t e, const char* where) {
    int code = cuda_fail(nullptr, e, where);
    dgsw_destroy(h);
    return code;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return bail(e, "cudaStreamCreate");
  const size_t bytes = (size_t)h->dom.offset.back() * sizeof(double);
  // 64 bytes of padding past each state-sized buffer: the batch stage's bulk
  // copies of odd-extent blocks round their end up to 16 bytes
  const size_t pad = 64;
  if ((e = cudaMalloc(&h->state, bytes + pad)) != cudaSuccess) return bail(e, "cudaMalloc state");
  if ((e = cudaMalloc(&h->t1, bytes + pad)) != cudaSuccess) return bail(e, "cudaMalloc stage 1");
  if ((e = cudaMalloc(&h->t2, bytes + pad)) != cudaSuccess) return bail(e, "cudaMalloc stage 2");
  if ((e = cudaMalloc(&h->u0s, bytes + pad)) != cudaSuccess) return bail(e, "cudaMalloc step start");
  if ((e = cudaMemset(h->state, 0, bytes + pad)) != cudaSuccess) return bail(e, "cudaMemset");
  if ((e = cudaMalloc(&h->dev_err, sizeof(int))) != cudaSuccess) return bail(e, "cudaMalloc err");
  if ((e = cudaMemset(h->dev_err, 0, sizeof(int))) != cudaSuccess) return bail(e, "cudaMemset err");
  if (cfg->precision == DGSW_PRECISION_DOUBLE_FLOAT) {
    // the Taylor step's increments W1, W2 as double-float pairs
    if ((e = cudaMalloc(&h->adj32, 2 * h->dom.offset.back() * sizeof(float2))) != cudaSuccess)
      return bail(e, "cudaMalloc increments");
  }
  if (cfg->precision == DGSW_PRECISION_MIXED) {
    if ((e = cudaMalloc(&h->w1, bytes / 2 + pad)) != cudaSuccess) return bail(e, "cudaMalloc w1");
    if ((e = cudaMalloc(&h->w2, bytes / 2 + pad)) != cudaSuccess) return bail(e, "cudaMalloc w2");
    if ((e = cudaMemset(h->w1, 0, bytes / 2 + pad)) != cudaSuccess) return bail(e, "cudaMemset w1");
    if ((e = cudaMemset(h->w2, 0, bytes / 2 + pad)) != cudaSuccess) return bail(e, "cudaMemset w2");
  }
  std::vector<double> jac(3 * h->dom.n_elem, 0.0);
  if (!h->curved)
    for (int64_t i = 0; i < 3 * h->dom.n_elem; ++i) jac[i] = 2.0 / h->dom.width[i];
  if ((e = upload(&h->nbr, h->dom.neighbor)) != cudaSuccess) return bail(e, "upload neighbors");
  if ((e = upload(&h->jac, jac)) != cudaSuccess) return bail(e, "upload jacobian");
  if ((e = upload(&h->lower, h->dom.lower)) != cudaSuccess) return bail(e, "upload lower");
  if ((e = upload(&h->width, h->dom.width)) != cudaSuccess) return bail(e, "upload width");
  if ((e = upload(&h->elem_n, h->dom.elem_n)) != cudaSuccess) return bail(e, "upload extents");
  if ((e = upload(&h->offset, h->dom.offset)) != cudaSuccess) return bail(e, "upload offsets");
  if ((e = upload(&h->instance, h->dom.instance)) != cudaSuccess) return bail(e, "upload instance");
  if (h->refined && !rmaps.faces.empty()) {
    const int n = h->dom.elem_n[0];
    h->r_nfaces = (int64_t)rmaps.faces.size();
    std::vector<int32_t> rec;
    rec.reserve(9 * rmaps.faces.size());
    for (const RefinedFace& f : rmaps.faces) {
      const int32_t r9[9] = {f.element, f.dir, f.coarse, f.nb[0], f.nb[1],
                             f.nb[2], f.nb[3], f.child[0], f.child[1]};
      rec.insert(rec.end(), r9, r9 + 9);
    }
    std::vector<double> PR(4 * (size_t)n * n);
    half_projections(n, 0, &PR[0], &PR[2 * (size_t)n * n]);
    half_projections(n, 1, &PR[(size_t)n * n], &PR[3 * (size_t)n * n]);
    if ((e = upload(&h->r_faces, rec)) != cudaSuccess) return bail(e, "upload 2:1 faces");
    if ((e = upload(&h->r_face_idx, rmaps.face_index)) != cudaSuccess)
      return bail(e, "upload 2:1 face index");
    if ((e = upload(&h->r_PR, PR)) != cudaSuccess) return bail(e, "upload half projections");
    if ((e = cudaMalloc(&h->r_wext, (size_t)h->r_nfaces * n * n * sizeof(double))) != cudaSuccess)
      return bail(e, "cudaMalloc 2:1 exterior values");
  }
  std::vector<double> nodes((kMaxN + 1) * kMaxN, 0.0);
  for (int n = kMinN; n <= kMaxN; ++n) {
    double w[kMaxN];
    if (h->gauss) {
      GaussTables g;
      lg_spectral(n, &g);
      for (int i = 0; i < n; ++i) nodes[n * kMaxN + i] = g.x[i];
    } else {
      lgl_nodes_weights(n, &nodes[n * kMaxN], w);
    }
  }
  if ((e = upload(&h->lgl_x, nodes)) != cudaSuccess) return bail(e, "upload nodes");
  lgl_eo_table(h->dom.elem_n[0], &h->eo);
  lgl_eo_table_transposed(h->dom.elem_n[0], &h->eoT);
  if (h->gauss) {
    lg_spectral(h->dom.elem_n[0], &h->gt);
    lg_eo_table(h->dom.elem_n[0], &h->eo);
  }
  if (h->curved) {
    int rc = csw_init(h, geo);
    if (rc) {
      const std::string msg = h->err;
      dgsw_destroy(h);
      return fail(nullptr, rc, msg);
    }
  }
  // mixed precision with gamma2 != 0 runs the kernels of differing extents
  // (their gamma2 terms) on uniform meshes too
  if (!h->dom.uniform || (mixed(h) && !h->curved && h->cfg.gamma2 != 0.0)) {
    h->general = true;
    std::vector<int32_t> lists[kMaxN + 1];
    for (int64_t el = 0; el < h->dom.n_elem; ++el) lists[h->dom.elem_n[el]].push_back((int32_t)el);
    for (int n = kMinN; n <= kMaxN; ++n) {
      h->class_count[n] = (int64_t)lists[n].size();
      lgl_eo_table(n, &h->class_eo[n]);
      if (!lists[n].empty() && (e = upload(&h->class_tasks[n], lists[n])) != cudaSuccess)
        return bail(e, "upload task list");
    }
    // face operators: interpolation (nn < n) or modal restriction (nn > n)
    std::vector<double> ops;
    std::vector<int32_t> op_off((kMaxN + 1) * (kMaxN + 1), -1);
    double buf[kMaxN * kMaxN];
    for (int n = kMinN; n <= kMaxN; ++n)
      for (int nn = kMinN; nn <= kMaxN; ++nn) {
        if (nn == n) continue;
        if (nn < n)
          lgl_mortar_projections(nn, n, buf, nullptr);  // n x nn
        else
          lgl_mortar_projections(n, nn, nullptr, buf);  // n x nn
        op_off[n * (kMaxN + 1) + nn] = (int32_t)ops.size();
        ops.insert(ops.end(), buf, buf + n * nn);
      }
    std::vector<float> hi(ops.size()), lo(ops.size());
    for (size_t i = 0; i < ops.size(); ++i) {
      hi[i] = (float)ops[i];
      lo[i] = (float)(ops[i] - (double)hi[i]);
    }
    if ((e = upload(&h->op64, ops)) != cudaSuccess) return bail(e, "upload face operators");
    if ((e = upload(&h->op_hi, hi)) != cudaSuccess) return bail(e, "upload face operators");
    if ((e = upload(&h->op_lo, lo)) != cudaSuccess) return bail(e, "upload face operators");
    if ((e = upload(&h->op_off, op_off)) != cudaSuccess) return bail(e, "upload face operators");
    // records of the faces whose neighbour has another extent
    std::vector<int32_t> face_idx(6 * h->dom.n_elem, -1), recs[kMaxN + 1];
    for (int64_t el = 0; el < h->dom.n_elem; ++el) {
      const int n = h->dom.elem_n[el];
      for (int dir = 0; dir < 6; ++dir)
        if (h->dom.elem_n[h->dom.neighbor[6 * el + dir]] != n) {
          face_idx[6 * el + dir] = (int32_t)recs[n].size();
          recs[n].push_back((int32_t)(6 * el + dir));
        }
    }
    if ((e = upload(&h->pnc_face_idx, face_idx)) != cudaSuccess) return bail(e, "upload face records");
    for (int n = kMinN; n <= kMaxN; ++n) {
      h->pnc_count[n] = (int64_t)recs[n].size();
      if (recs[n].empty()) continue;
      if ((e = upload(&h->pnc_rec[n], recs[n])) != cudaSuccess) return bail(e, "upload face records");
      if ((e = cudaMalloc(&h->pnc_wext[n], recs[n].size() * n * n * sizeof(double))) != cudaSuccess)
        return bail(e, "allocate face records");
    }
  }
  if (mixed(h) && !h->curved && !h->gauss && !h->refined) {
    // the batch kernels take every mixed-extent mixed-precision handle; on
    // uniform meshes DGSW_MIXED_KERNEL=batch selects them in place of the
    // even-extent pipeline kernel
    const char* env = std::getenv("DGSW_MIXED_KERNEL");
    const bool want = h->general ? !(env && std::string(env) == "general")
                                 : (env && std::string(env) == "batch");
    if (want) {
      int rc = batch_init(h);
      if (rc) {
        const std::string msg = h->err;
        dgsw_destroy(h);
        return fail(nullptr, rc, msg);
      }
    }
  }
  if (cfg->time_stepper == DGSW_STEPPER_ADAMS_BASHFORTH) {
    int rc = adams_init(h, *cfg);
    if (rc) {
      const std::string msg = h->err;
      dgsw_destroy(h);
      return fail(nullptr, rc, msg);
    }
  }
  *out = h;
  return DGSW_OK;
}

int dgsw_destroy(DgswHandle h) {
  if (!h) return DGSW_OK;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  destroy_graphs(h);
  double* dbl[] = {h->state, h->t1, h->t2, h->u0s, h->jac, h->lower, h->width, h->lgl_x, h->params};
  for (double* p : dbl)
    if (p) cudaFree(p);
  if (h->graph_adj) cudaGraphExecDestroy(h->graph_adj);
  if (h->graph_tf) cudaGraphExecDestroy(h->graph_tf);
  double* adjbufs[] = {h->samp_w, h->adj, h->adjz, h->targets, h->residuals};
  for (double* p : adjbufs)
    if (p) cudaFree(p);
  if (h->adj32) cudaFree(h->adj32);
  if (h->samp_off) cudaFree(h->samp_off);
  double* cdbl[] = {h->c_xyz, h->c_ij, h->c_T, h->c_F};
  for (double* p : cdbl)
    if (p) cudaFree(p);
  if (h->c_T32) cudaFree(h->c_T32);
  if (h->c_F32) cudaFree(h->c_F32);
  if (h->c_X) cudaFree(h->c_X);
  if (h->c_Xf) cudaFree(h->c_Xf);
  if (h->filt) cudaFree(h->filt);
  if (h->fr32) cudaFree(h->fr32);
  if (h->fw3) cudaFree(h->fw3);
  if (h->lgl_w) cudaFree(h->lgl_w);
  if (h->norm_partial) cudaFree(h->norm_partial);
  if (h->r_faces) cudaFree(h->r_faces);
  if (h->r_face_idx) cudaFree(h->r_face_idx);
  if (h->r_PR) cudaFree(h->r_PR);
  if (h->r_wext) cudaFree(h->r_wext);
  if (h->dev_err) cudaFree(h->dev_err);
  for (cudaEvent_t ev : h->pipe_ev)
    if (ev) cudaEventDestroy(ev);
  if (h->pipe_in) cudaStreamDestroy(h->pipe_in);
  if (h->pipe_out) cudaStreamDestroy(h->pipe_out);
  for (cudaStream_t s : h->pipe_aux)
    if (s) cudaStreamDestroy(s);
  if (h->pipe_seam) cudaStreamDestroy(h->pipe_seam);
  if (h->dev_first) cudaFree(h->dev_first);
  if (h->ab_list) cudaFree(h->ab_list);
  if (h->ab_level) cudaFree(h->ab_level);
  if (h->ab_F) cudaFree(h->ab_F);
  if (h->ab_B) cudaFree(h->ab_B);
  if (h->ab_F32) cudaFree(h->ab_F32);
  if (h->ab_boff) cudaFree(h->ab_boff);
  for (int n = 0; n <= kMaxN; ++n) {
    if (h->class_tasks[n]) cudaFree(h->class_tasks[n]);
    if (h->pnc_rec[n]) cudaFree(h->pnc_rec[n]);
    if (h->pnc_wext[n]) cudaFree(h->pnc_wext[n]);
  }
  if (h->pnc_face_idx) cudaFree(h->pnc_face_idx);
  void* bt[] = {h->bt_tasks[0], h->bt_tasks[1], h->bt_elems[0], h->bt_elems[1], h->bt_foff,
                h->bt_fu, h->bt_fw1, h->bt_fw2, h->bt_fw3, h->bt_dtab, h->bt_raw,
                h->bt_chunks, h->bt_face_src, h->bt_face_dst};
  for (void* p : bt)
    if (p) cudaFree(p);
  if (h->op64) cudaFree(h->op64);
  if (h->op_hi) cudaFree(h->op_hi);
  if (h->op_lo) cudaFree(h->op_lo);
  if (h->op_off) cudaFree(h->op_off);
  if (h->w1) cudaFree(h->w1);
  if (h->w2) cudaFree(h->w2);
  if (h->nbr) cudaFree(h->nbr);
  if (h->elem_n) cudaFree(h->elem_n);
  if (h->offset) cudaFree(h->offset);
  if (h->instance) cudaFree(h->instance);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return DGSW_OK;
}

int dgsw_sizes(DgswHandle h, int64_t* n_elements, int64_t* state_doubles, int64_t* grid_points) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (n_elements) *n_elements = h->dom.n_elem;
  if (state_doubles) *state_doubles = h->dom.offset.back();
  if (grid_points) *grid_points = h->dom.n_points;
  return DGSW_OK;
}

void* dgsw_stream(DgswHandle h) { return h ? (void*)h->stream : nullptr; }

int dgsw_synchronize(DgswHandle h) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int dgsw_set_state(DgswHandle h, const double* host_u) {
  if (!h || !host_u) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->adams) h->ab.restart();  // new initial values: self-start again
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, cudaMemcpyAsync(h->state, host_u, h->dom.offset.back() * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
  return DGSW_OK;
}

int dgsw_get_state(DgswHandle h, double* host_u) {
  if (!h || !host_u) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, cudaMemcpyAsync(host_u, h->state, h->dom.offset.back() * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int dgsw_set_state_device(DgswHandle h, const double* dev_u) {
  if (!h || !dev_u) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->adams) h->ab.restart();  // new initial values: self-start again
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, cudaMemcpyAsync(h->state, dev_u, h->dom.offset.back() * sizeof(double),
                               cudaMemcpyDeviceToDevice, h->stream));
  return DGSW_OK;
}

int dgsw_get_state_device(DgswHandle h, double* dev_u) {
  if (!h || !dev_u) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, cudaMemcpyAsync(dev_u, h->state, h->dom.offset.back() * sizeof(double),
                               cudaMemcpyDeviceToDevice, h->stream));
  return DGSW_OK;
}

int dgsw_set_initial_data(DgswHandle h, int kind, const double* params, double t) {
  if (!h || !params) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->adams) h->ab.restart();  // new initial values: self-start again
  if (h->curved) {
    if (kind != 2) return fail(h, DGSW_ERR_ARGUMENT, "the shell takes initial data kind 2");
    if (!std::isfinite(params[0]) || !std::isfinite(params[1]) || !(params[2] > 0.0) ||
        !std::isfinite(params[2]))
      return fail(h, DGSW_ERR_ARGUMENT, "need finite A, r0 and a positive width");
    if (int rc = select_device(h)) return rc;
    DGSW_CUDA(h, launch_csw_initial(h->c_xyz, h->dom.elem_n[0], h->dom.n_elem, params[0],
                                    params[1], params[2], h->state, h->stream));
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    return DGSW_OK;
  }
  if (kind != 0 && kind != 1) return fail(h, DGSW_ERR_ARGUMENT, "unknown initial data kind");
  if (int rc = select_device(h)) return rc;
  // one Gaussian per instance; a refined lattice is one instance (its
  // elements' instance index is 0) and keeps no brick list
  const size_t n_inst = h->dom.bricks.empty() ? 1 : h->dom.bricks.size();
  const size_t count = kind == 0 ? 3 : 5 * n_inst;
  for (size_t i = 0; i < count; ++i)
    if (!std::isfinite(params[i])) return fail(h, DGSW_ERR_ARGUMENT, "non-finite parameter");
  if (kind == 1)
    for (size_t i = 0; i < n_inst; ++i)
      if (!(params[5 * i + 1] > 0.0)) return fail(h, DGSW_ERR_ARGUMENT, "width must be positive");
  if (count > h->params_cap) {
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->params) cudaFree(h->params);
    h->params = nullptr;
    DGSW_CUDA(h, cudaMalloc(&h->params, count * sizeof(double)));
    h->params_cap = count;
  }
  DGSW_CUDA(h, cudaMemcpyAsync(h->params, params, count * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream));
  InitLaunch L;
  L.kind = kind;
  L.n_elem = h->dom.n_elem;
  L.elem_n = h->elem_n;
  L.offset = h->offset;
  L.instance = h->instance;
  L.lower = h->lower;
  L.width = h->width;
  L.params = h->params;
  L.lgl_x = h->lgl_x;
  L.t = t;
  L.u = h->state;
  DGSW_CUDA(h, launch_initial_data(L, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return DGSW_OK;
}

int dgsw_rhs_device(DgswHandle h, const double* dev_u, double* dev_dudt) {
  if (!h || !dev_u || !dev_dudt) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (dev_u == dev_dudt) return fail(h, DGSW_ERR_ARGUMENT, "input and output must differ");
  if (int rc = select_device(h)) return rc;
  if (h->curved) {
    if (mixed(h)) {
      CswMixedLaunch M = base_csw_mixed(h);
      M.x64 = dev_u;
      M.c = 1.0;
      M.out64 = dev_dudt;
      DGSW_CUDA(h, launch_csw_mixed(M, h->stream));
      return DGSW_OK;
    }
    DGSW_CUDA(h, csw_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0));
    return DGSW_OK;
  }
  if (h->gauss) {
    DGSW_CUDA(h, gauss_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0));
    return DGSW_OK;
  }
  if (mixed(h)) {
    if (h->general) {
      GeneralLaunch G = base_general(h);
      G.prec = kPrecComp;
      G.x64 = dev_u;
      G.c = 1.0;
      G.out64 = dev_dudt;
      DGSW_CUDA(h, launch_general_classes(h, G));
      return DGSW_OK;
    }
    MixedLaunch M = base_mixed(h);
    M.x64 = dev_u;
    M.c = 1.0;
    M.out64 = dev_dudt;
    DGSW_CUDA(h, launch_mixed(h, M));
    return DGSW_OK;
  }
  if (h->general) {
    DGSW_CUDA(h, general_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0));
    return DGSW_OK;
  }
  StageLaunch L = base_launch(h);
  L.mode = kModeRhs;
  L.ucur = dev_u;
  L.u0 = dev_u;
  L.unext = dev_dudt;
  L.coef = {0.0, 0.0, 1.0};
  DGSW_CUDA(h, launch_stage(h, L));
  return DGSW_OK;
}

int dgsw_volume_rhs_device(DgswHandle h, const double* dev_u, double* dev_dudt) {
  if (!h || !dev_u || !dev_dudt) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (dev_u == dev_dudt) return fail(h, DGSW_ERR_ARGUMENT, "input and output must differ");
  if (int rc = select_device(h)) return rc;
  if (h->curved) {
    DGSW_CUDA(h, csw_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0, 0));
    return DGSW_OK;
  }
  if (h->gauss) {
    DGSW_CUDA(h, gauss_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0, 0));
    return DGSW_OK;
  }
  if (h->general) {
    DGSW_CUDA(h, general_f64(h, dev_u, nullptr, dev_dudt, 0.0, 0.0, 1.0, 0));
    return DGSW_OK;
  }
  StageLaunch L = base_launch(h);
  L.mode = kModeVolume;
  L.ucur = dev_u;
  L.u0 = dev_u;
  L.unext = dev_dudt;
  L.coef = {0.0, 0.0, 1.0};
  DGSW_CUDA(h, launch_stage(h, L));
  return DGSW_OK;
}

int dgsw_rhs(DgswHandle h, const double* host_u, double* host_dudt) {
  if (!h || !host_u || !host_dudt) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (int rc = select_device(h)) return rc;
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  // t1/t2 hold only intermediate stage values between launches, so they
  // double as staging buffers here.
  DGSW_CUDA(h, cudaMemcpyAsync(h->t1, host_u, bytes, cudaMemcpyHostToDevice, h->stream));
  if (int rc = dgsw_rhs_device(h, h->t1, h->t2)) return rc;
  DGSW_CUDA(h, cudaMemcpyAsync(host_dudt, h->t2, bytes, cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return DGSW_OK;
}

int dgsw_package_data_device(int64_t npts, const double* psi, const double* pi, const double* phi,
                             const double* gamma2, const double* normal, const double* ndotv,
                             double* packaged, void* stream) {
  if (npts < 0 || (npts > 0 && (!psi || !pi || !phi || !gamma2 || !normal || !packaged)))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "null argument");
  cudaError_t e = launch_package_data(npts, psi, pi, phi, gamma2, normal, ndotv, packaged,
                                      (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "package_data");
  return DGSW_OK;
}

int dgsw_boundary_terms_device(int64_t npts, const double* pkg_int, const double* pkg_ext,
                               double* out, void* stream) {
  if (npts < 0 || (npts > 0 && (!pkg_int || !pkg_ext || !out)))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "null argument");
  cudaError_t e = launch_boundary_terms(npts, pkg_int, pkg_ext, out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "boundary_terms");
  return DGSW_OK;
}

int dgsw_substep(DgswHandle h, int k, double dt) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (h->adams)
    return fail(h, DGSW_ERR_UNSUPPORTED, "AdamsBashforth has no substeps; use dgsw_step");
  if (k < 0 || k > 2 || !std::isfinite(dt)) return fail(h, DGSW_ERR_ARGUMENT, "bad substep");
  if (dfloat(h))
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "double-float precision steps the Taylor form, which has no substeps");
  if (int rc = select_device(h)) return rc;
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  if (mixed(h)) {
    if (k == 0)
      DGSW_CUDA(h, cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (h->filter_on)
      DGSW_CUDA(h, mixed_filtered_stage(h, k, dt, h->u0s, h->state));
    else
      DGSW_CUDA(h, enqueue_mixed_stage(h, k, dt, h->u0s, h->state));
    return DGSW_OK;
  }
  if (h->gauss) {
    if (k == 0) {
      DGSW_CUDA(h, cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      DGSW_CUDA(h, gauss_f64(h, h->u0s, nullptr, h->state, 0.0, 1.0, dt));
    } else {
      DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      if (k == 1)
        DGSW_CUDA(h, gauss_f64(h, h->t1, h->u0s, h->state, 0.75, 0.25, 0.25 * dt));
      else
        DGSW_CUDA(h, gauss_f64(h, h->t1, h->u0s, h->state, 1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt));
    }
    return DGSW_OK;
  }
  if (h->curved) {
    if (k == 0) {
      DGSW_CUDA(h, cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      DGSW_CUDA(h, csw_f64(h, h->u0s, nullptr, h->state, 0.0, 1.0, dt));
    } else {
      DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      if (k == 1)
        DGSW_CUDA(h, csw_f64(h, h->t1, h->u0s, h->state, 0.75, 0.25, 0.25 * dt));
      else
        DGSW_CUDA(h, csw_f64(h, h->t1, h->u0s, h->state, 1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt));
    }
    DGSW_CUDA(h, apply_filter(h, h->state));
    return DGSW_OK;
  }
  if (h->general) {
    if (k == 0) {
      DGSW_CUDA(h, cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      DGSW_CUDA(h, general_f64(h, h->u0s, nullptr, h->state, 1.0, 0.0, dt));
    } else {
      DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
      if (k == 1)
        DGSW_CUDA(h, general_f64(h, h->t1, h->u0s, h->state, 0.25, 0.75, 0.25 * dt));
      else
        DGSW_CUDA(h, general_f64(h, h->t1, h->u0s, h->state, 2.0 / 3.0, 1.0 / 3.0, (2.0 / 3.0) * dt));
    }
    DGSW_CUDA(h, apply_filter(h, h->state));
    return DGSW_OK;
  }
  StageLaunch L = base_launch(h);
  if (k == 0) {
    DGSW_CUDA(h, cudaMemcpyAsync(h->u0s, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
    L.mode = kModeStageFirst;
    L.ucur = h->u0s;
    L.u0 = h->u0s;
    L.unext = h->state;
    L.coef = {0.0, 1.0, dt};
  } else {
    DGSW_CUDA(h, cudaMemcpyAsync(h->t1, h->state, bytes, cudaMemcpyDeviceToDevice, h->stream));
    L.mode = kModeStage;
    L.ucur = h->t1;
    L.u0 = h->u0s;
    L.unext = h->state;
    L.coef = k == 1 ? StageCoef{0.75, 0.25, 0.25 * dt}
                    : StageCoef{1.0 / 3.0, 2.0 / 3.0, (2.0 / 3.0) * dt};
  }
  DGSW_CUDA(h, launch_stage(h, L));
  DGSW_CUDA(h, apply_filter(h, h->state));
  return DGSW_OK;
}

// ObserveNorms of u (or u - subtract) into out[27] (see dgsw.h).
static int observe_norms(DgswHandle h, const double* dev_u, const double* dev_sub, double* out) {
  const int64_t E = h->dom.n_elem;
  if (!h->norm_partial) {
    std::vector<double> w((kMaxN + 1) * kMaxN, 0.0);
    for (int n = kMinN; n <= kMaxN; ++n) {
      double x[kMaxN];
      if (h->gauss) {
        GaussTables g;
        lg_spectral(n, &g);
        for (int i = 0; i < n; ++i) w[n * kMaxN + i] = g.w[i];
      } else {
        lgl_nodes_weights(n, x, &w[n * kMaxN]);
      }
    }
    DGSW_CUDA(h, upload(&h->lgl_w, w));
    DGSW_CUDA(h, cudaMalloc(&h->norm_partial,
                            ((size_t)(E + kNormsBlocks) * 26 + 32) * sizeof(double)));
  }
  NormsLaunch L;
  L.n_elem = E;
  L.uniform_n = h->dom.uniform ? h->dom.elem_n[0] : 0;
  L.elem_n = h->elem_n;
  L.offset = h->dom.uniform ? nullptr : h->offset;
  if (h->curved)
    L.ij = h->c_ij;
  else
    L.width = h->width;
  L.lgl_w = h->lgl_w;
  L.u = dev_u ? dev_u : h->state;
  L.subtract = dev_sub;
  L.partial = h->norm_partial;
  L.result = h->norm_partial + (size_t)(E + kNormsBlocks) * 26;
  DGSW_CUDA(h, launch_norms(L, h->stream));
  double r[26];
  DGSW_CUDA(h, cudaMemcpyAsync(r, L.result, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  const double pts = (double)h->dom.n_points, vol = r[25];
  for (int v = 0; v < 5; ++v) {
    out[5 * v + 0] = r[5 * v + 0];
    out[5 * v + 1] = r[5 * v + 1];
    out[5 * v + 2] = std::sqrt(r[5 * v + 2] / pts);
    out[5 * v + 3] = std::sqrt(r[5 * v + 3] / vol);
    out[5 * v + 4] = r[5 * v + 4];
  }
  out[25] = pts;
  out[26] = vol;
  return DGSW_OK;
}

int dgsw_observe_norms(DgswHandle h, const double* dev_u, const double* dev_subtract,
                       double* out) {
  if (!h || !out) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (int rc = select_device(h)) return rc;
  return observe_norms(h, dev_u, dev_subtract, out);
}

int dgsw_observe_plane_wave_errors(DgswHandle h, const double* k, double t, double* out) {
  if (!h || !k || !out) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->curved) return fail(h, DGSW_ERR_UNSUPPORTED, "the plane wave is a flat-space solution");
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(k[i])) return fail(h, DGSW_ERR_ARGUMENT, "non-finite wave vector");
  if (!std::isfinite(t)) return fail(h, DGSW_ERR_ARGUMENT, "non-finite time");
  if (int rc = select_device(h)) return rc;
  // the analytic solution at t goes to the stage buffer t1 (free between steps)
  if (3 > h->params_cap) {
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->params) cudaFree(h->params);
    h->params = nullptr;
    DGSW_CUDA(h, cudaMalloc(&h->params, 3 * sizeof(double)));
    h->params_cap = 3;
  }
  DGSW_CUDA(h, cudaMemcpyAsync(h->params, k, 3 * sizeof(double), cudaMemcpyHostToDevice,
                               h->stream));
  InitLaunch L;
  L.kind = 0;
  L.n_elem = h->dom.n_elem;
  L.elem_n = h->elem_n;
  L.offset = h->offset;
  L.instance = h->instance;
  L.lower = h->lower;
  L.width = h->width;
  L.params = h->params;
  L.lgl_x = h->lgl_x;
  L.t = t;
  L.u = h->t1;
  DGSW_CUDA(h, launch_initial_data(L, h->stream));
  return observe_norms(h, h->state, h->t1, out);
}

int dgsw_autotune(DgswHandle h, int force_variant, int* variant, double* ms_per_launch) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (force_variant < -1 || force_variant >= DGSW_STAGE_VARIANTS)
    return fail(h, DGSW_ERR_ARGUMENT, "force_variant must be -1 or a variant index");
  if (int rc = select_device(h)) return rc;
  if (tunable(h)) {
    destroy_graphs(h);
    if (int rc = autotune(h, true)) return rc;
    if (force_variant >= 0) h->stage_variant = force_variant;
  }
  if (variant) *variant = h->stage_variant;
  if (ms_per_launch)
    for (int v = 0; v < DGSW_STAGE_VARIANTS; ++v) ms_per_launch[v] = h->tune_ms[v];
  return DGSW_OK;
}

int dgsw_tune(DgswHandle h, int force_variant, int* family, int* n_variants, int* variant,
              double* ms_per_step) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (int rc = select_device(h)) return rc;
  int fam = DGSW_TUNE_NONE, nv = 0, v = 0;
  double ms[DGSW_TUNE_MAX_VARIANTS] = {};
  if (h->batch) {
    fam = DGSW_TUNE_MIXED_BATCH;
    nv = batch_variants();
    if (force_variant >= nv || force_variant < -1)
      return fail(h, DGSW_ERR_ARGUMENT, "force_variant out of range");
    if (force_variant >= 0 && h->bt_nmax > batch_max_extent(force_variant))
      return fail(h, DGSW_ERR_ARGUMENT, "that launch shape does not hold the domain's extents");
    destroy_graphs(h);
    if (int rc = batch_autotune(h, true)) return rc;
    if (force_variant >= 0) h->bt_variant = force_variant;
    v = h->bt_variant;
    for (int i = 0; i < nv && i < DGSW_TUNE_MAX_VARIANTS; ++i) ms[i] = h->bt_tune_ms[i];
  } else if (csw_tunable(h)) {
    fam = DGSW_TUNE_MIXED_CURVED;
    nv = 2 * csw_mixed_shapes();
    if (force_variant >= nv || force_variant < -1)
      return fail(h, DGSW_ERR_ARGUMENT, "force_variant out of range");
    destroy_graphs(h);
    if (int rc = csw_autotune(h, true)) return rc;
    if (force_variant >= 0) h->csw_variant = force_variant;
    v = h->csw_variant;
    for (int i = 0; i < nv; ++i) ms[i] = h->csw_tune_ms[i];
  } else if (pipe_tunable(h)) {
    fam = DGSW_TUNE_MIXED_PIPE;
    nv = 4;
    if (force_variant >= nv || force_variant < -1)
      return fail(h, DGSW_ERR_ARGUMENT, "force_variant out of range");
    destroy_graphs(h);
    if (int rc = pipe_autotune(h, true)) return rc;
    if (force_variant >= 0) h->pipe_variant = force_variant;
    v = h->pipe_variant;
    for (int i = 0; i < nv; ++i) ms[i] = h->pipe_tune_ms[i];
  } else if (tunable(h)) {
    fam = DGSW_TUNE_FP64_STAGE;
    nv = DGSW_STAGE_VARIANTS;
    if (force_variant >= nv || force_variant < -1)
      return fail(h, DGSW_ERR_ARGUMENT, "force_variant out of range");
    destroy_graphs(h);
    if (int rc = autotune(h, true)) return rc;
    if (force_variant >= 0) h->stage_variant = force_variant;
    v = h->stage_variant;
    for (int i = 0; i < nv; ++i) ms[i] = 3.0 * h->tune_ms[i];
  }
  if (family) *family = fam;
  if (n_variants) *n_variants = nv;
  if (variant) *variant = v;
  if (ms_per_step)
    for (int i = 0; i < DGSW_TUNE_MAX_VARIANTS; ++i) ms_per_step[i] = ms[i];
  return DGSW_OK;
}

int dgsw_check_device_timeout(DgswHandle h, double limit_seconds) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (!(limit_seconds > 0.0) || limit_seconds > 10.0)
    return fail(h, DGSW_ERR_ARGUMENT, "the wait limit must be in (0, 10] s");
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, launch_bounded_wait_check(h->dev_err, (uint64_t)(limit_seconds * 1e9),
                                         h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

int dgsw_set_exponential_filter(DgswHandle h, double alpha, int half_power, int enable) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (!enable) {
    if (h->filter_on) destroy_graphs(h);
    h->filter_on = false;
    return DGSW_OK;
  }
  if (!std::isfinite(alpha) || alpha < 0.0 || half_power < 0 || half_power > 64)
    return fail(h, DGSW_ERR_ARGUMENT, "need a finite alpha >= 0 and half_power in [0, 64]");
  if (h->gauss)
    return fail(h, DGSW_ERR_UNSUPPORTED, "the filter is built for Gauss-Lobatto meshes");
  if (dfloat(h))
    return fail(h, DGSW_ERR_UNSUPPORTED, "the filter is not built for double-float precision");
  if (int rc = select_device(h)) return rc;
  std::vector<double> mats((size_t)(kMaxN + 1) * kMaxN * kMaxN, 0.0);
  for (int n = kMinN; n <= kMaxN; ++n)
    lgl_exponential_filter(n, alpha, half_power, &mats[(size_t)n * kMaxN * kMaxN]);
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  if (!h->filt) DGSW_CUDA(h, cudaMalloc(&h->filt, mats.size() * sizeof(double)));
  DGSW_CUDA(h, cudaMemcpy(h->filt, mats.data(), mats.size() * sizeof(double),
                          cudaMemcpyHostToDevice));
  if (mixed(h)) {
    // the residual and third-stage buffers (the kernels split the FP64
    // matrices themselves)
    const size_t b32 = (size_t)h->dom.offset.back() * sizeof(float) + 64;
    if (!h->fr32) DGSW_CUDA(h, cudaMalloc(&h->fr32, b32));
    if (!h->fw3) DGSW_CUDA(h, cudaMalloc(&h->fw3, b32));
  }
  destroy_graphs(h);
  h->filter_on = true;
  h->filter_alpha = alpha;
  h->filter_half_power = half_power;
  return DGSW_OK;
}

int dgsw_exponential_filter_matrix(int n, double alpha, int half_power, double* F) {
  if (!lgl_exponential_filter(n, alpha, half_power, F))
    return fail(nullptr, DGSW_ERR_ARGUMENT, "need 2 <= n <= 20, finite alpha, half_power >= 0");
  return DGSW_OK;
}

static int step_impl(DgswHandle h, int n_steps, double dt);

// the first element whose block holds a NaN or an Inf, -1 if none
static int first_non_finite(DgswHandle h, int64_t* first) {
  if (!h->dev_first) DGSW_CUDA(h, cudaMalloc(&h->dev_first, sizeof(unsigned long long)));
  DGSW_CUDA(h, cudaMemsetAsync(h->dev_first, 0xff, sizeof(unsigned long long), h->stream));
  DGSW_CUDA(h, launch_finite_check(h->state, h->offset, h->dom.n_elem, h->dev_first, h->stream));
  unsigned long long v = 0;
  DGSW_CUDA(h, cudaMemcpyAsync(&v, h->dev_first, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  *first = v == ~0ull ? -1 : (int64_t)v;
  return DGSW_OK;
}

int dgsw_step(DgswHandle h, int n_steps, double dt) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (n_steps < 0 || !std::isfinite(dt)) return fail(h, DGSW_ERR_ARGUMENT, "bad step arguments");
  if (n_steps == 0) return DGSW_OK;
  if (h->guard_cfl > 0.0) {
    // StepChoosers::Cfl rejects a step longer than the element's Cfl step
    for (int64_t e = 0; e < h->dom.n_elem; ++e) {
      const double step = h->adams ? std::ldexp(std::abs(dt), -(int)h->ab_level_host[e]) : std::abs(dt);
      if (step > h->cfl_e[e])
        return fail(h, DGSW_ERR_CFL,
                    "the step " + std::to_string(step) + " of element " + std::to_string(e) +
                        " exceeds its Cfl step " + std::to_string(h->cfl_e[e]));
    }
  }
  const int rc = step_impl(h, n_steps, dt);
  if (rc || !h->guard_finite) return rc;
  int64_t first = -1;
  if (int r = first_non_finite(h, &first)) return r;
  if (first >= 0)
    return fail(h, DGSW_ERR_NOT_FINITE,
                "NaN or Inf in the state after the step, first in element " + std::to_string(first));
  return DGSW_OK;
}

int dgsw_set_guards(DgswHandle h, double cfl_safety_factor, int check_finite) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (!std::isfinite(cfl_safety_factor) || cfl_safety_factor < 0.0)
    return fail(h, DGSW_ERR_ARGUMENT, "the Cfl safety factor must be >= 0 (0: off)");
  if (cfl_safety_factor > 0.0) {
    std::string err;
    ShellGeometry geo;
    Domain dom;
    const Domain* d = &h->dom;
    if (h->curved) {  // the shell's inertial coordinates, rebuilt on the host
      if (!build_shell_domain(h->cfg, &dom, &geo, &err)) return fail(h, DGSW_ERR_ARGUMENT, err);
      d = &dom;
    }
    if (!cfl_steps(h->cfg, *d, h->curved ? &geo : nullptr, cfl_safety_factor, &h->cfl_e, &err))
      return fail(h, DGSW_ERR_ARGUMENT, err);
  }
  h->guard_cfl = cfl_safety_factor;
  h->guard_finite = check_finite != 0;
  return DGSW_OK;
}

int dgsw_check_finite(DgswHandle h, int64_t* first_element) {
  if (!h || !first_element) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (int rc = select_device(h)) return rc;
  return first_non_finite(h, first_element);
}

int dgsw_cfl_steps(const DgswConfig* cfg, double safety_factor, double* element_steps,
                   double* min_step) {
  if (!cfg) return fail(nullptr, DGSW_ERR_ARGUMENT, "null config");
  Domain dom;
  ShellGeometry geo;
  std::string err;
  if (!any_domain(*cfg, &dom, &geo, &err)) return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  std::vector<double> steps;
  const bool curved = cfg->system == DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D;
  if (!cfl_steps(*cfg, dom, curved ? &geo : nullptr, safety_factor, &steps, &err))
    return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  if (element_steps) std::memcpy(element_steps, steps.data(), steps.size() * sizeof(double));
  if (min_step) *min_step = steps.empty() ? 0.0 : *std::min_element(steps.begin(), steps.end());
  return DGSW_OK;
}

int dgsw_time_step_id(int time_runs_forward, int64_t slab_number, double slab_start,
                      double slab_end, int32_t num, int32_t den, DgswTimeStepId* out) {
  if (!out) return fail(nullptr, DGSW_ERR_ARGUMENT, "null output");
  std::string err;
  if (!make_time_step_id(time_runs_forward, slab_number, slab_start, slab_end, num, den, out, &err))
    return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  return DGSW_OK;
}

int dgsw_next_time_id(int time_stepper, const DgswTimeStepId* current, int32_t size_num,
                      int32_t size_den, DgswTimeStepId* next) {
  if (!current || !next) return fail(nullptr, DGSW_ERR_ARGUMENT, "null argument");
  std::string err;
  if (!next_time_id(time_stepper, *current, size_num, size_den, next, &err))
    return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  return DGSW_OK;
}

int dgsw_substep_time_fraction(int time_stepper, int substep, double* fraction) {
  if (!fraction) return fail(nullptr, DGSW_ERR_ARGUMENT, "null output");
  std::string err;
  if (!substep_fraction(time_stepper, substep, fraction, &err))
    return fail(nullptr, DGSW_ERR_ARGUMENT, err);
  return DGSW_OK;
}

static int step_impl(DgswHandle h, int n_steps, double dt) {
  if (int rc = select_device(h)) return rc;
  if (h->adams) return adams_step(h, n_steps, dt);
  if (!h->tuned && tunable(h)) {
    destroy_graphs(h);
    if (int rc = autotune(h, false)) return rc;
  }
  if (h->batch && !h->bt_tuned) {
    destroy_graphs(h);
    if (int rc = batch_autotune(h, false)) return rc;
  }
  if (pipe_tunable(h) && !h->pipe_tuned) {
    destroy_graphs(h);
    if (int rc = pipe_autotune(h, false)) return rc;
  }
  if (csw_tunable(h) && !h->csw_tuned) {
    destroy_graphs(h);
    if (int rc = csw_autotune(h, false)) return rc;
  }
  if (!(h->graph_dt == dt)) {
    destroy_graphs(h);
    DGSW_CUDA(h, capture_steps(h, dt, 1, &h->graph_one));
    h->graph_dt = dt;
  }
  // replay chunks of up to 16 steps per graph launch to amortise launch cost
  constexpr int kChunk = 16;
  if (n_steps >= kChunk && !h->graph_many) {
    DGSW_CUDA(h, capture_steps(h, dt, kChunk, &h->graph_many));
    h->graph_many_steps = kChunk;
  }
  // batch handles: the state's face values are formed from the state at the
  // start of every call (whatever changed it since) and again every kChunk
  // steps; in between each step's last stage keeps them current
  if (h->batch) {
    DGSW_CUDA(h, batch_state_faces(h));
    h->bt_fu_age = 0;
  }
  auto resync = [&]() -> cudaError_t {
    if (!h->batch || h->bt_fu_age < kChunk) return cudaSuccess;
    h->bt_fu_age = 0;
    return batch_state_faces(h);
  };
  int left = n_steps;
  while (h->graph_many && left >= h->graph_many_steps) {
    DGSW_CUDA(h, resync());
    DGSW_CUDA(h, cudaGraphLaunch(h->graph_many, h->stream));
    left -= h->graph_many_steps;
    h->bt_fu_age += h->graph_many_steps;
  }
  for (; left > 0; --left) {
    DGSW_CUDA(h, resync());
    DGSW_CUDA(h, cudaGraphLaunch(h->graph_one, h->stream));
    ++h->bt_fu_age;
  }
  return DGSW_OK;
}

int dgsw_adjoint_rhs_device(DgswHandle h, const double* dev_lambda, double* dev_out) {
  if (!h || !dev_lambda || !dev_out) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (dev_lambda == dev_out) return fail(h, DGSW_ERR_ARGUMENT, "input and output must differ");
  if (h->general || h->curved || h->gauss || h->refined || h->cfg.gamma2 != 0.0)
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "the adjoint needs the flat system, uniform extents and gamma2 = 0");
  if (int rc = select_device(h)) return rc;
  AdjointLaunch A = base_adjoint(h);
  A.x = dev_lambda;
  A.out = dev_out;
  DGSW_CUDA(h, launch_adjoint_fp64(A, h->stream));
  return DGSW_OK;
}

int dgsw_set_samples(DgswHandle h, int n_samples, const double* xyz) {
  if (!h || n_samples < 1 || !xyz) return fail(h, DGSW_ERR_ARGUMENT, "need sample points");
  if (h->general || h->gauss || h->dom.bricks.size() != 1 || h->cfg.gamma2 != 0.0)
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "samples and the adjoint need one brick of uniform extent and gamma2 = 0");
  if (int rc = select_device(h)) return rc;
  const int n = h->dom.elem_n[0];
  std::vector<int64_t> off(n_samples);
  std::vector<double> w((size_t)n_samples * 3 * n);
  if (!sample_weights(h->dom, n, n_samples, xyz, off.data(), w.data()))
    return fail(h, DGSW_ERR_ARGUMENT, "a sample point lies outside the brick");
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->samp_off) cudaFree(h->samp_off);
  if (h->samp_w) cudaFree(h->samp_w);
  h->samp_off = nullptr;
  h->samp_w = nullptr;
  DGSW_CUDA(h, upload(&h->samp_off, off));
  DGSW_CUDA(h, upload(&h->samp_w, w));
  h->n_samples = n_samples;
  if (!h->adj) {
    const size_t bytes = h->dom.offset.back() * sizeof(double);
    DGSW_CUDA(h, cudaMalloc(&h->adj, bytes));
    DGSW_CUDA(h, cudaMalloc(&h->adjz, bytes));
  }
  return DGSW_OK;
}

int dgsw_sample_psi(DgswHandle h, double* host_out) {
  if (!h || !host_out) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->n_samples < 1) return fail(h, DGSW_ERR_ARGUMENT, "no sample points set");
  if (int rc = select_device(h)) return rc;
  if (h->record_cap < h->n_samples) {
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->residuals) cudaFree(h->residuals);
    if (h->targets) cudaFree(h->targets);
    h->residuals = h->targets = nullptr;
    DGSW_CUDA(h, cudaMalloc(&h->residuals, h->n_samples * sizeof(double)));
    DGSW_CUDA(h, cudaMalloc(&h->targets, h->n_samples * sizeof(double)));
    h->record_cap = h->n_samples;
  }
  const int n = h->dom.elem_n[0];
  DGSW_CUDA(h, launch_sample(h->state, h->n_samples, n, h->samp_off, h->samp_w, nullptr,
                             h->residuals, h->stream));
  DGSW_CUDA(h, cudaMemcpyAsync(host_out, h->residuals, h->n_samples * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return DGSW_OK;
}

int dgsw_misfit_forward(DgswHandle h, int n_windows, int steps_per_window, double dt,
                        const double* host_targets, double* J) {
  if (!h || !host_targets || !J) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (n_windows < 1 || steps_per_window < 1 || !std::isfinite(dt))
    return fail(h, DGSW_ERR_ARGUMENT, "bad window arguments");
  if (h->n_samples < 1) return fail(h, DGSW_ERR_ARGUMENT, "no sample points set");
  if (h->curved || h->refined || h->filter_on ||
      h->cfg.time_stepper != DGSW_STEPPER_RK3_HESTHAVEN_SSP)
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "the misfit adjoint needs the flat system, Rk3HesthavenSsp and no filter");
  if (int rc = select_device(h)) return rc;
  const int64_t need = (int64_t)n_windows * h->n_samples;
  if (h->record_cap < need) {
    DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
    if (h->residuals) cudaFree(h->residuals);
    if (h->targets) cudaFree(h->targets);
    h->residuals = h->targets = nullptr;
    DGSW_CUDA(h, cudaMalloc(&h->residuals, need * sizeof(double)));
    DGSW_CUDA(h, cudaMalloc(&h->targets, need * sizeof(double)));
    h->record_cap = need;
  }
  DGSW_CUDA(h, cudaMemcpyAsync(h->targets, host_targets, need * sizeof(double),
                               cudaMemcpyHostToDevice, h->stream));
  const int n = h->dom.elem_n[0];
  if (mixed(h)) {
    if (int rc = taylor_buffers(h)) return rc;
    if (!(h->graph_tf_dt == dt) || h->graph_tf_steps != steps_per_window) {
      if (h->graph_tf) cudaGraphExecDestroy(h->graph_tf);
      h->graph_tf = nullptr;
      DGSW_CUDA(h, capture_taylor_steps(h, dt, steps_per_window, &h->graph_tf));
      h->graph_tf_dt = dt;
      h->graph_tf_steps = steps_per_window;
    }
  }
  for (int m = 0; m < n_windows; ++m) {
    if (mixed(h)) {
      DGSW_CUDA(h, cudaGraphLaunch(h->graph_tf, h->stream));
    } else if (int rc = dgsw_step(h, steps_per_window, dt)) {
      return rc;
    }
    DGSW_CUDA(h, launch_sample(h->state, h->n_samples, n, h->samp_off, h->samp_w,
                               h->targets + (int64_t)m * h->n_samples,
                               h->residuals + (int64_t)m * h->n_samples, h->stream));
  }
  std::vector<double> r(need);
  DGSW_CUDA(h, cudaMemcpyAsync(r.data(), h->residuals, need * sizeof(double),
                               cudaMemcpyDeviceToHost, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  double acc = 0.0;
  for (double v : r) acc += v * v;
  *J = acc;
  h->rec_windows = n_windows;
  h->rec_steps = steps_per_window;
  h->rec_dt = dt;
  return check_device_error(h);
}

int dgsw_adjoint_autotune(DgswHandle h, int force_variant, int* variant, double* ms_per_launch) {
  if (!h) return fail(nullptr, DGSW_ERR_ARGUMENT, "null handle");
  if (force_variant < -1 || force_variant > 1)
    return fail(h, DGSW_ERR_ARGUMENT, "force_variant must be -1, 0 or 1");
  if (h->general || h->curved || h->gauss || h->refined || mixed(h) || dfloat(h) ||
      h->cfg.gamma2 != 0.0)
    return fail(h, DGSW_ERR_UNSUPPORTED,
                "the FP64 adjoint needs the flat FP64 system, uniform extents and gamma2 = 0");
  if (int rc = select_device(h)) return rc;
  DGSW_CUDA(h, adjoint_autotune(h));
  if (force_variant >= 0) h->adj_variant = force_variant;
  // the captured sweep holds the old split
  if (h->graph_adj) cudaGraphExecDestroy(h->graph_adj);
  h->graph_adj = nullptr;
  h->graph_adj_steps = 0;
  if (variant) *variant = h->adj_variant;
  if (ms_per_launch) {
    ms_per_launch[0] = h->adj_tune_ms[0];
    ms_per_launch[1] = h->adj_tune_ms[1];
  }
  return DGSW_OK;
}

int dgsw_misfit_adjoint(DgswHandle h, double* dev_grad) {
  if (!h || !dev_grad) return fail(h, DGSW_ERR_ARGUMENT, "null argument");
  if (h->rec_windows < 1) return fail(h, DGSW_ERR_ARGUMENT, "no recorded misfit run");
  if (int rc = select_device(h)) return rc;
  const size_t bytes = h->dom.offset.back() * sizeof(double);
  if (mixed(h) || dfloat(h))
    if (int rc = taylor_buffers(h)) return rc;
  const int K = h->rec_steps;
  const double dt = h->rec_dt;
  if (!h->adj_tuned && !mixed(h) && !dfloat(h)) DGSW_CUDA(h, adjoint_autotune(h));
  if (!(h->graph_adj_dt == dt) || h->graph_adj_steps != K) {
    if (h->graph_adj) cudaGraphExecDestroy(h->graph_adj);
    h->graph_adj = nullptr;
    DGSW_CUDA(h, capture_adjoint_steps(h, dt, K, &h->graph_adj));
    h->graph_adj_dt = dt;
    h->graph_adj_steps = K;
  }
  const int n = h->dom.elem_n[0];
  DGSW_CUDA(h, cudaMemsetAsync(h->adj, 0, bytes, h->stream));
  for (int m = h->rec_windows - 1; m >= 0; --m) {
    // dJ/d(sample) = 2 r, injected at the window's time, then K steps back
    DGSW_CUDA(h, launch_sample_scatter(h->adj, h->n_samples, n, h->samp_off, h->samp_w,
                                       h->residuals + (int64_t)m * h->n_samples, 2.0, h->stream));
    DGSW_CUDA(h, cudaGraphLaunch(h->graph_adj, h->stream));
  }
  DGSW_CUDA(h, cudaMemcpyAsync(dev_grad, h->adj, bytes, cudaMemcpyDeviceToDevice, h->stream));
  DGSW_CUDA(h, cudaStreamSynchronize(h->stream));
  return check_device_error(h);
}

}  // extern "C"
