// host_setup.hpp -- host-side (FP64) spectral tables and domain index maps.
//
// Setup work that runs once per handle on the CPU: Legendre-Gauss-Lobatto
// nodes and weights, the differentiation matrix, mortar projection matrices
// and the integer element/neighbour/mortar maps of a periodic brick lattice.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dgsw.h"
#include "common.cuh"

namespace dgsw {

// Spectral::collocation_points/quadrature_weights<Legendre, GaussLobatto>,
// Legendre.cpp:186-239.  Nodes are the roots of q = L_{p+1} - L_{p-1}
// found by Newton's method with q' = (2p+1) L_p.
bool lgl_nodes_weights(int n, double* x, double* w);
// Barycentric differentiation matrix with negative-sum diagonal,
// Spectral.cpp:84-111,431-444.  Row-major.
bool lgl_diff_matrix(int n, double* D);
// Interpolation from n LGL points to m targets, Spectral.cpp:625-670.
bool lgl_interp_matrix(int n, int m, const double* targets, double* M);
// Face -> mortar (nm x ne, interpolation) and mortar -> face (ne x nm,
// Legendre modal truncation), Projection.cpp:56-375, ChildSize::Full.
bool lgl_mortar_projections(int ne, int nm, double* to_mortar, double* from_mortar);
// Legendre-Gauss spectral tables on n points: nodes, weights, the
// barycentric differentiation matrix, interpolation rows to xi = -1 / +1
// (boundary_interpolation_matrices) and those rows over the weights
// (boundary_lifting_term), Spectral.cpp:676-790.
struct GaussTables {
  int n = 0;
  double x[20], w[20], D[400], lo[20], hi[20], lift_lo[20], lift_hi[20];
};
bool lg_spectral(int n, GaussTables* g);
bool lg_eo_table(int n, EoTable* t);

// Exponential filter V diag(exp(-alpha (k/(n-1))^(2 half_power))) V^-1 on n
// LGL points (Spectral::filtering::exponential_filter, Filtering.cpp:18-31),
// row-major.
bool lgl_exponential_filter(int n, double alpha, int half_power, double* F);
// Even/odd split tables of the differentiation matrix (see EoTable), and of
// its transpose (also centro-antisymmetric), used by the adjoint.
bool lgl_eo_table(int n, EoTable* t);
bool lgl_eo_table_transposed(int n, EoTable* t);

struct BrickLayout {
  int blocks[3];  // odd part of each per-axis element count
  int level[3];   // refinement level: count = blocks * 2^level
  int64_t first;  // global index of the instance's first element
  int64_t count;
};

struct Domain {
  std::vector<DgswBrick> bricks;
  std::vector<BrickLayout> layout;
  std::vector<int32_t> elem_n;     // LGL extent per element
  std::vector<int64_t> offset;     // doubles, n_elem + 1 entries
  std::vector<int32_t> neighbor;   // 6 per element
  std::vector<int32_t> instance;   // per element
  std::vector<double> lower;       // 3 per element
  std::vector<double> width;       // 3 per element
  std::vector<uint64_t> element_id;
  int64_t n_elem = 0;
  int64_t n_points = 0;
  bool block_ids_fit = true;       // every block id < 256
  bool uniform = true;             // every element has the same extent
  int max_n = 0;
};

// Element and barycentric interpolation weights (3 x n per point) of points
// inside a single-instance uniform-extent domain; false if a point lies
// outside the brick.
bool sample_weights(const Domain& dom, int n, int n_samples, const double* xyz,
                    int64_t* elem_off, double* weights);

// Geometry of the curved shell (shell_setup.cpp), per element: coordinates
// 3*N^3, inverse Jacobian 9*N^3 (component 3a+i = d xi^a / d x^i), and per
// face (6) the neighbour's face direction and, per face point, the
// neighbour's face-point index of the same physical point.
struct ShellGeometry {
  int n = 0;
  std::vector<double> xyz;
  std::vector<double> inv_jac;
  std::vector<int32_t> face_perm;
  std::vector<int32_t> back_dir;
};

// StepChoosers::Cfl per element (cfl.cpp): safety * stable_step * minimum
// grid spacing / (largest characteristic speed * 3).
double time_stepper_stable_step(const DgswConfig& cfg);
// TimeStepId and the time steppers' next_time_id (time_step_id.cpp).
bool make_time_step_id(int forward, int64_t slab_number, double slab_start, double slab_end,
                       int32_t num, int32_t den, DgswTimeStepId* out, std::string* err);
bool substep_fraction(int time_stepper, int substep, double* fraction, std::string* err);
bool next_time_id(int time_stepper, const DgswTimeStepId& cur, int32_t size_num, int32_t size_den,
                  DgswTimeStepId* next, std::string* err);
bool cfl_steps(const DgswConfig& cfg, const Domain& dom, const struct ShellGeometry* geo,
               double safety, std::vector<double>* steps, std::string* err);

// Builds the shell's element maps (Domain fields: element ids, neighbours
// with -1 / -2 on the inner / outer sphere, offsets) and its geometry.
bool build_shell_domain(const DgswConfig& cfg, Domain* dom, ShellGeometry* geo,
                        std::string* err);

// h-nonconforming refined lattice (refined_setup.cpp).  One record per
// 2:1 face: coarse = 1 for the coarse side (four fine neighbours nb[c],
// c = c0 + 2 c1 the half in each transverse dimension), coarse = 0 for a fine
// side (nb[0] the coarse neighbour, child[t] which half of its face).
struct RefinedFace {
  int32_t element, dir, coarse;
  int32_t nb[4];
  int32_t child[2];
};
struct RefinedMaps {
  std::vector<int32_t> level;       // per element
  std::vector<int32_t> slots;       // 4 per element face
  std::vector<int32_t> sizes;       // 2 per slot: 0 Full, 1 LowerHalf, 2 UpperHalf
  std::vector<int32_t> face_index;  // per element face: record index or -1
  std::vector<RefinedFace> faces;
};
bool build_refined_domain(const DgswConfig& cfg, Domain* dom, RefinedMaps* rm,
                          std::string* err);
// Half-interval projections on n LGL points (n x n, row-major), parent ->
// child interpolation and child -> parent L2 restriction, Projection.cpp.
bool half_projections(int n, int upper, double* parent_to_child, double* child_to_parent);
// The 1D matrix (dst x src, row-major) of amr::projectors::ProjectVariables
// along one dimension: child 0 (ChildSize::Full) is p-projection (identity,
// interpolation to a finer or truncation to a coarser extent), child 1 / 2
// (LowerHalf / UpperHalf) interpolation into that half, dst >= src (amr.cu).
bool amr_matrix(int src, int dst, int child, double* M);

// Validates a configuration and builds every host-side map.  On failure
// returns false with a message in *err.
bool build_domain(const DgswConfig& cfg, Domain* dom, std::string* err);

}  // namespace dgsw
