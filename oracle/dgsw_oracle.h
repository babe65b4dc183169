/*
 * dgsw_oracle.h -- CPU FP64 restatement of SpECTRE's DG scalar-wave evolution
 * step (test infrastructure only).
 *
 * This library is the correctness checker for the CUDA path in
 * spectre_gb300/.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product library never links it.
 *
 * It follows the reference's own algorithms (file:line relative to the
 * SpECTRE source tree, release 2024.09.29):
 *   LGL nodes/weights   src/NumericalAlgorithms/Spectral/Legendre.cpp:160-239
 *   barycentric weights src/NumericalAlgorithms/Spectral/Spectral.cpp:84-101
 *   D-matrix            src/NumericalAlgorithms/Spectral/Spectral.cpp:431-444
 *   Vandermonde         src/NumericalAlgorithms/Spectral/Spectral.cpp:499-523
 *   interpolation       src/NumericalAlgorithms/Spectral/Spectral.cpp:625-670
 *   mortar projections  src/NumericalAlgorithms/Spectral/Projection.cpp:56-375
 *   partial derivatives src/NumericalAlgorithms/LinearOperators/PartialDerivatives.tpp:56-110,315-363
 *   time derivative     src/Evolution/Systems/ScalarWave/TimeDerivative.cpp:13-45
 *   UpwindPenalty       src/Evolution/Systems/ScalarWave/BoundaryCorrections/UpwindPenalty.cpp:35-205
 *   face normals        src/Evolution/DiscontinuousGalerkin/Actions/NormalCovectorAndMagnitude.hpp:48-101
 *   lift_flux           src/NumericalAlgorithms/DiscontinuousGalerkin/LiftFlux.hpp:41-62
 *   SSP-RK3             src/Time/TimeSteppers/Rk3HesthavenSsp.cpp:55-81
 *   ElementId layout    src/Domain/Structure/ElementId.hpp:55-90,138-147
 *   element ordering    src/Domain/Structure/InitialElementIds.cpp:45-96
 *   multi-block lattice src/Domain/DomainHelpers.cpp:1187-1201 (blocks x fastest)
 *   mortar mesh         src/NumericalAlgorithms/DiscontinuousGalerkin/MortarHelpers.cpp:21-47
 *
 * All arrays are caller-owned host memory.  Every function returns 0 on
 * success and a negative code on bad arguments.
 */
#ifndef DGSW_ORACLE_H
#define DGSW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- spectral (a1, a7) ---------------- */
int orc_lgl(int n, double* x, double* w);
int orc_barycentric_weights(int n, double* bw);
/* D[i*n + j] = d l_j / d xi at x_i (row-major) */
int orc_diff_matrix(int n, double* D);
/* V[i*n + k] = P_k(x_i) */
int orc_vandermonde(int n, double* V);
int orc_inv_vandermonde(int n, double* Vinv);
/* M[k*n + j]: value at targets[k] of the j-th Lagrange polynomial on n LGL pts */
int orc_interp_matrix(int n, int m, const double* targets, double* M);
/* face (ne pts) -> mortar (nm >= ne pts): P[i*ne + j], i < nm (interpolation) */
int orc_proj_face_to_mortar(int ne, int nm, double* P);
/* mortar (nm pts) -> face (ne <= nm pts): P[i*nm + j], i < ne (modal truncation) */
int orc_proj_mortar_to_face(int ne, int nm, double* P);
/* amr::projectors::ProjectVariables: the 1D matrix (dst x src) for child 0
 * (p-projection), 1 (LowerHalf) or 2 (UpperHalf), and the projection of
 * n_out target blocks from source blocks src[k] (extents 3 per block) */
int orc_amr_matrix(int src, int dst, int child, double* M);
int orc_amr_project(int n_vars, int64_t n_out, const int32_t* src, const int32_t* src_ext,
                    const int32_t* dst_ext, const int8_t* child, const double* in,
                    const int64_t* in_off, double* out, const int64_t* out_off);

/* ---------------- domain (a13, a14) ---------------- */
/* One periodic brick evolution: [lo, hi]^3 with n[d] elements along axis d.
 * n[d] = b * 2^L with b odd is laid out as b blocks of refinement L. */
typedef struct {
  double lo[3];
  double hi[3];
  int32_t n[3];
} OrcBrick;

/* number of elements over all instances */
int64_t orc_num_elements(int n_inst, const OrcBrick* bricks);
/* elem_id: packed 64-bit ElementId; nbr: 6 per element in Direction order
 * (lower_xi, upper_xi, lower_eta, upper_eta, lower_zeta, upper_zeta), global
 * element index; ijk: 3 global lattice coordinates per element; inst: owner. */
int orc_index_maps(int n_inst, const OrcBrick* bricks, uint64_t* elem_id,
                   int32_t* nbr, int32_t* ijk, int32_t* inst);

/* Offsets (in doubles) of each element's 5*N^3 block; off has n_elem+1 entries. */
int orc_offsets(int64_t n_elem, const int32_t* elem_n, int64_t* off);

/* Inertial coordinates, 3*N^3 per element (x, y, z component-major). */
int orc_coords(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
               double* xyz);

/* ---------------- initial data ---------------- */
/* kind 0: plane wave psi = sin(k.x - |k| t), params = {kx, ky, kz}
 * kind 1: gaussian pulse psi = A exp(-|x-c|^2 / w^2), Pi = 0,
 *         params per instance = {A, w, cx, cy, cz} (5 * n_inst values) */
int orc_initial_data(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
                     int kind, const double* params, double t, double* u);

/* ---------------- UpwindPenalty (a6, a8) ---------------- */
/* packaged: 16*npts component-major in dg_package_field_tags order:
 *   v_psi, v_zero[3], v_plus, v_minus, n*v_plus[3], n*v_minus[3],
 *   gamma2*v_psi, char_speeds[3]
 * phi, normal: 3*npts component-major.  ndotv may be NULL (no mesh velocity). */
int orc_package(int npts, const double* psi, const double* pi,
                const double* phi, const double* gamma2, const double* normal,
                const double* ndotv, double* packaged, double* max_speed);
/* out: 5*npts (psi, pi, phi_x, phi_y, phi_z boundary corrections) */
int orc_boundary_terms(int npts, const double* pkg_int, const double* pkg_ext,
                       double* out);

/* ---------------- DG right-hand side and stepping (a2-a12) ---------------- */
/* dudt = strong-form DG time derivative with UpwindPenalty corrections lifted
 * at GLL faces; u, dudt laid out per element [var][k][j][i]. gamma2 constant. */
int orc_rhs(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
            double gamma2, const double* u, double* dudt, int n_threads);
/* volume terms only (TimeDerivative::apply after partial_derivatives) */
int orc_volume_rhs(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
                   double gamma2, const double* u, double* dudt, int n_threads);
/* one SSP-RK3 substep k (0,1,2) given u0 (step start) and the current stage
 * value ucur: writes unext. */
int orc_rk3_substep(int64_t n, int k, double dt, const double* u0,
                    const double* ucur, const double* dudt, double* unext);
/* n_steps full SSP-RK3 steps in place */
int orc_evolve(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
               double gamma2, double dt, int n_steps, double* u, int n_threads);


/* ---------------- Legendre-Gauss quadrature ----------------
 * collocation points/weights <Legendre, Gauss> (Legendre.cpp:106-149),
 * differentiation_matrix on those nodes, boundary_interpolation_matrices
 * (rows to xi = -1, +1) and boundary_lifting_term (rows / weights),
 * Spectral.cpp:676-790. */
int orc_lg(int n, double* x, double* w);
int orc_lg_diff_matrix(int n, double* D);
int orc_lg_boundary(int n, double* lo, double* hi, double* lift_lo, double* lift_hi);
/* Flat ScalarWave on Gauss points, uniform extent n, periodic bricks:
 * volume terms with the Gauss D; faces interpolated to the boundary, packaged
 * and corrected by UpwindPenalty; the correction lifted into the whole
 * element by lift_boundary_terms_gauss_points (LiftFromBoundary.cpp:20-140,
 * called from ApplyBoundaryCorrections.hpp:938-987). */
int orc_coords_gauss(int n_inst, const OrcBrick* bricks, int n, double* xyz);
int orc_rhs_gauss(int n_inst, const OrcBrick* bricks, int n, double gamma2, const double* u,
                  double* dudt, int n_threads);
int orc_evolve_gauss(int n_inst, const OrcBrick* bricks, int n, double gamma2, double dt,
                     int n_steps, double* u, int n_threads);

/* ---------------- h-nonconforming refined bricks ----------------
 * A periodic lattice of blocks on [lo, hi]^3 (blocks x fastest), each block
 * with its own isotropic refinement level (2^level elements per axis);
 * neighbouring blocks differ by at most one level (2:1).  Faces between a
 * coarse and a fine block carry one mortar per fine element, of
 * Spectral::MortarSize LowerHalf / UpperHalf in each transverse dimension
 * on the coarse side (MortarHelpers.cpp:49-75); data go face -> mortar by
 * projection_matrix_parent_to_child and back by projection_matrix_child_to_parent
 * (Projection.cpp:56-375). */
typedef struct {
  double lo[3], hi[3];
  int32_t blocks[3];
  const int32_t* level;  /* blocks[0]*blocks[1]*blocks[2] levels */
} OrcRefinedBrick;
int64_t orc_refined_num_elements(const OrcRefinedBrick* b);
/* ids: packed ElementId; nbr: 4 slots per element face ((6e + dir) * 4 + k,
 * -1 unused); msize: 2 per slot (transverse dims ascending), 0 Full,
 * 1 LowerHalf, 2 UpperHalf, as mortar_size(self, neighbour).  Returns -2 if
 * two neighbouring blocks differ by more than one level. */
int orc_refined_index_maps(const OrcRefinedBrick* b, uint64_t* ids, int32_t* nbr,
                           int32_t* msize);
int orc_refined_coords(const OrcRefinedBrick* b, int n, double* xyz);
int orc_refined_rhs(const OrcRefinedBrick* b, int n, double gamma2, const double* u,
                    double* dudt, int n_threads);
int orc_refined_evolve(const OrcRefinedBrick* b, int n, double gamma2, double dt, int n_steps,
                       double* u, int n_threads);
/* n x n matrices, row-major: parent (element face) -> child half (mortar)
 * interpolation and child half -> parent L2 restriction; upper = 1 for
 * UpperHalf, 0 for LowerHalf */
int orc_proj_half(int n, int upper, double* parent_to_child, double* child_to_parent);

/* ---------------- exponential filter ----------------
 * Spectral::filtering::exponential_filter (NumericalAlgorithms/Spectral/
 * Filtering.cpp:18-31): F = V diag(exp(-alpha (k/(n-1))^(2 half_power))) V^-1
 * with V the Legendre Vandermonde on the LGL nodes; F[i*n + j] row-major. */
int orc_exponential_filter(int n, double alpha, int half_power, double* F);
/* dg::Actions::Filter (ParallelAlgorithms/Actions/FilterAction.hpp:109-180):
 * every element's five variables filtered along each axis (apply_matrices
 * with F in every dimension), in place.  elem_n: extent per element. */
int orc_filter_elements(int64_t n_elem, const int32_t* elem_n, double alpha,
                        int half_power, double* u);

/* ---------------- ObserveNorms ----------------
 * Events::ObserveNorms (ParallelAlgorithms/Events/ObserveNorms.cpp:33-105,
 * ObserveNorms.hpp:47-80,145-171) of the five evolved components, each
 * "Individual", reduced over all elements.  out[5*v + m] for variable v and
 * m = Max, Min, L2Norm = sqrt(sum u^2 / points), L2IntegralNorm =
 * sqrt(int u^2 dV / V), VolumeIntegral = int u dV; out[25] = points,
 * out[26] = V.  The integrals are definite_integral on the LGL mesh times
 * det(Jacobian).  subtract (may be NULL): a state-sized array subtracted
 * first (errors against an analytic solution). */
int orc_observe_norms(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
                      const double* u, const double* subtract, double* out);
int orc_shell_observe_norms_impl(int64_t n_elem, int n, const double* det_jac,
                                 const double* u, const double* subtract, double* out);

/* ---------------- CurvedScalarWave (configuration 5) ----------------
 * Follows (paths relative to the SpECTRE tree):
 *   TimeDerivative       src/Evolution/Systems/CurvedScalarWave/TimeDerivative.cpp:19-69
 *   characteristics      src/Evolution/Systems/CurvedScalarWave/Characteristics.cpp:20-137
 *   UpwindPenalty        src/Evolution/Systems/CurvedScalarWave/BoundaryCorrections/UpwindPenalty.cpp:35-146
 *   CPSR boundary        src/Evolution/Systems/CurvedScalarWave/BoundaryConditions/
 *                        ConstraintPreservingSphericalRadiation.cpp:40-156
 *   Schwarzschild in Kerr-Schild coordinates: the closed forms checked by
 *   tests/Unit/PointwiseFunctions/AnalyticSolutions/GeneralRelativity/Test_KerrSchild.cpp:55-232
 * Per point, component-major arrays of npts each. */

/* background out (26 per point): lapse, shift[3], d_lapse[3],
 * d_shift[9] (d_i shift^j at 3*i+j), inv_metric[6] (xx xy xz yy yz zz),
 * trace_christoffel[3], trace_K */
int orc_ks_background(int npts, double mass, const double* xyz, double* bg);
/* dt (5*npts) from d_psi[3], d_pi[3], d_phi[9] (d_i Phi_j at 3*i+j), pi,
 * phi[3], background (26*npts), gamma1, gamma2 */
int orc_csw_time_derivative(int npts, const double* d_psi, const double* d_pi,
                            const double* d_phi, const double* pi,
                            const double* phi, const double* bg, double gamma1,
                            double gamma2, double* dt);
/* packaged 14*npts: v_psi, v_zero[3], v_plus, v_minus, gamma2, normal[3],
 * char_speeds[4]; returns the max char speed. ndotv may be NULL. */
int orc_csw_package(int npts, const double* psi, const double* pi,
                    const double* phi, const double* lapse, const double* shift,
                    const double* gamma1, const double* gamma2,
                    const double* normal, const double* normal_vector,
                    const double* ndotv, double* packaged, double* max_speed);
int orc_csw_boundary_terms(int npts, const double* pkg_int, const double* pkg_ext,
                           double* out);
/* CPSR dt corrections (5*npts) */
int orc_csw_cpsr(int npts, const double* psi, const double* pi,
                 const double* phi, const double* lapse, const double* shift,
                 const double* gamma1, const double* gamma2, const double* normal,
                 const double* normal_vector, const double* xyz,
                 const double* d_psi, const double* d_pi, const double* d_phi,
                 const double* dt_psi, const double* dt_pi, const double* dt_phi,
                 double* out);

/* ---------------- spherical shell of 6 wedges (configuration 5) ----------------
 * Domain/Creators/Sphere.cpp (shell, no interior), Domain/CoordinateMaps/Wedge.cpp:476-536
 * (sphericity 1 inside and out, equiangular, logarithmic radial distribution),
 * block orientations DomainHelpers.cpp:553-578 (+z, -z, +y, -y, +x, -x),
 * refinement (ref_ang, ref_ang, ref_rad) per block, elements in
 * initial_element_ids order.  Neighbours across blocks are found by matching
 * face centres; face points are matched by their coordinates (the role of
 * orient_variables_on_slice, OrientationMapHelpers.hpp:63-120). */
typedef struct {
  double r_inner, r_outer;
  int32_t ref_ang, ref_rad;
  int32_t n;        /* LGL points per dimension */
  double mass;      /* Kerr-Schild mass (spin 0) */
  double gamma1, gamma2;
} OrcShell;
int64_t orc_shell_num_elements(const OrcShell* s);
/* coordinates (3*N^3) and inverse Jacobian (9*N^3, d xi^a / d x^i at 3a+i)
 * per element, component-major within the element */
int orc_shell_geometry(const OrcShell* s, double* xyz, double* inv_jac);
/* nbr: 6 per element, -1 inner boundary, -2 outer boundary; perm: 6*N^2 per
 * element, the neighbour's face-point index of each of this face's points;
 * element_ids: packed ElementId bits */
int orc_shell_connectivity(const OrcShell* s, int32_t* nbr, int32_t* perm,
                           uint64_t* element_ids);
/* Gaussian shell psi = exp(-(r - r0)^2 / w^2), Pi = 0, Phi = grad psi */
int orc_shell_initial_data(const OrcShell* s, double r0, double w, double* u);
/* curved DG time derivative with UpwindPenalty, excision check at the inner
 * sphere (returns 1 if a char speed is incoming) and CPSR at the outer one */
int orc_shell_rhs(const OrcShell* s, const double* u, double* dudt, int n_threads);
int orc_shell_evolve(const OrcShell* s, double dt, int n_steps, double* u, int n_threads);
/* AdamsBashforth(order) with local time stepping on the shell (self-start,
 * then n_slabs slabs; element e steps slab / 2^levels[e], levels may be
 * NULL), the outer radiation condition in dt u, UpwindPenalty across wedges
 * through the boundary histories (adams_oracle.cpp) */
int orc_shell_evolve_adams(const OrcShell* s, int order, const int32_t* levels, double slab,
                           int n_slabs, double* u, int n_threads);
/* The same with dg::Actions::Filter (the exponential filter of
 * orc_filter_elements) applied to each element after every one of its
 * steps, as the curved executable's step actions end. */
int orc_shell_evolve_adams_filtered(const OrcShell* s, int order, const int32_t* levels,
                                    double slab, int n_slabs, double alpha, int half_power,
                                    double* u, int n_threads);
/* ObserveNorms (as orc_observe_norms) of a shell state */
int orc_shell_observe_norms(const OrcShell* s, const double* u, double* out);

/* ---------------- Adams-Bashforth, local time stepping (f5) ---------------- */
/* adams_oracle.cpp.  Times are integer ticks, ticks_per_slab to a slab of
 * duration `slab` (exact, as the reference's Time).
 * variable_coefficients: AdamsCoefficients.cpp:73-117 (n <= 8) */
int orc_variable_coefficients(int n, const double* control_times, double step_start,
                              double step_end, double* out);
/* adams_coefficients::coefficients, AdamsCoefficients.hpp:29-67 */
int orc_adams_coefficients(int n, const int64_t* control_ticks, int64_t step_start,
                           int64_t step_end, double slab, int64_t ticks_per_slab, double* out);
/* adams_lts::lts_coefficients for explicit schemes (AdamsLts.cpp:301-415) of
 * orders local_order, remote_order and small_order.  Histories are (slab
 * number, tick) ids in insertion order; the output terms index them.
 * Returns the number of terms, or < 0. */
int orc_lts_coefficients(int n_local, const int64_t* local_slab, const int64_t* local_tick,
                         int n_remote, const int64_t* remote_slab, const int64_t* remote_tick,
                         int64_t step_start, int64_t step_end, double slab, int64_t ticks_per_slab,
                         int local_order, int remote_order, int small_order, int max_out,
                         int32_t* out_local, int32_t* out_remote, double* out_coef);
/* Self-start, then n_slabs slabs of AdamsBashforth(order) with local time
 * stepping on conforming bricks of uniform extent n: element e steps
 * slab / 2^levels[e] (levels may be NULL: global stepping), after the first
 * steps at the finest step.  u in place. */
int orc_evolve_adams(int n_inst, const OrcBrick* bricks, int n, double gamma2, int order,
                     const int32_t* levels, double slab, int n_slabs, double* u, int n_threads);
/* The same on bricks whose elements have their own extents elem_n[e]
 * (p-nonconforming faces through mortars at the larger extent); u in the
 * layout of orc_offsets. */
int orc_evolve_adams_extents(int n_inst, const OrcBrick* bricks, const int32_t* elem_n,
                             double gamma2, int order, const int32_t* levels, double slab,
                             int n_slabs, double* u, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
