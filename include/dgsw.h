/*
 * dgsw.h -- C ABI of the GB300-native DG scalar-wave evolution hot path.
 *
 * This library replaces, for one GPU, the per-element DG evolution step of
 * SpECTRE's first-order scalar wave (reference release 2024.09.29):
 *   ScalarWave::System<3>            src/Evolution/Systems/ScalarWave/System.hpp:39-57
 *   ScalarWave::TimeDerivative<3>    src/Evolution/Systems/ScalarWave/TimeDerivative.cpp:13-45
 *     (called from evolution::dg::Actions::detail::volume_terms,
 *      src/Evolution/DiscontinuousGalerkin/Actions/VolumeTermsImpl.tpp:76-295,
 *      after partial_derivatives, src/NumericalAlgorithms/LinearOperators/PartialDerivatives.tpp:191-241)
 *   ScalarWave::BoundaryCorrections::UpwindPenalty<3>
 *                                    src/Evolution/Systems/ScalarWave/BoundaryCorrections/UpwindPenalty.cpp:35-205
 *   dg::lift_flux + add_slice_to_data
 *                                    src/NumericalAlgorithms/DiscontinuousGalerkin/LiftFlux.hpp:41-62,
 *                                    src/Evolution/DiscontinuousGalerkin/Actions/ApplyBoundaryCorrections.hpp:723-1050
 *   TimeSteppers::Rk3HesthavenSsp    src/Time/TimeSteppers/Rk3HesthavenSsp.cpp:21-81
 *     (TimeStepper::update_u, src/Time/TimeSteppers/TimeStepper.hpp:56-101,
 *      driven by Actions::UpdateU, src/Time/Actions/UpdateU.hpp:45-154)
 *
 * Conventions
 *  - Every function returns an int status: DGSW_OK (0) or a negative
 *    DgswStatus.  Nothing aborts.  dgsw_last_error() gives the message of the
 *    most recent failure on that handle (or of the last handle-less call).
 *  - State layout is the reference's Variables layout, one contiguous block
 *    per element, elements in initial_element_ids order: per element
 *    [var][k][j][i] with i (xi) fastest, vars = Psi, Pi, Phi_x, Phi_y, Phi_z.
 *  - Host pointers are borrowed for the duration of a call.  Device buffers
 *    are owned by the handle.  "_device" entry points take device pointers.
 *  - One CUDA stream per handle; a handle is not thread-safe.
 *  - Functions with no handle argument are host-only and need no GPU.
 */
#ifndef DGSW_H
#define DGSW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGSW_ABI_VERSION 9

typedef enum {
  DGSW_OK = 0,
  DGSW_ERR_ARGUMENT = -1,     /* bad configuration or argument */
  DGSW_ERR_CUDA = -2,         /* CUDA runtime error */
  DGSW_ERR_UNSUPPORTED = -3,  /* valid request this build does not support */
  DGSW_ERR_NOT_FINITE = -4,   /* NaN or Inf detected in the state */
  DGSW_ERR_NO_DEVICE = -5,    /* no usable GB300-class device */
  DGSW_ERR_DEVICE_TIMEOUT = -6, /* a bounded device-side wait gave up */
  DGSW_ERR_CFL = -7             /* a step longer than the Cfl step (dgsw_set_guards) */
} DgswStatus;

/* System::variables_tag, ScalarWave/System.hpp:39-57 and
 * CurvedScalarWave/System.hpp:24-62 (same Psi, Pi, Phi variables). */
typedef enum {
  DGSW_SYSTEM_SCALAR_WAVE_3D = 0,
  DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D = 1
} DgswSystem;
/* BoundaryCorrection creatable classes, ScalarWave/BoundaryCorrections/Factory.hpp */
typedef enum { DGSW_CORRECTION_UPWIND_PENALTY = 0 } DgswBoundaryCorrection;
/* TimeStepper creatable classes, Time/TimeSteppers/Factory.hpp */
typedef enum {
  DGSW_STEPPER_RK3_HESTHAVEN_SSP = 0,
  /* TimeSteppers::AdamsBashforth (AdamsBashforth.cpp:51-339) with local time
   * stepping (AdamsLts.cpp:301-415); see dgsw_step */
  DGSW_STEPPER_ADAMS_BASHFORTH = 1
} DgswTimeStepper;
/* Arithmetic of the derivative/flux/lift work.  FP64: everything in FP64.
 * MIXED: FP32 contractions with the D-matrix split into hi+lo FP32 parts,
 * FP64 state and FP64 accumulation of each time step.  DOUBLE_FLOAT: FP64
 * state; every operation on field values in double-float arithmetic (each
 * value a hi + lo pair of FP32 numbers, ~44 bits: compensated products with
 * the hi + lo split of D and compensated sums, FP32 pipes only), the step
 * taken as its Taylor polynomial (identical to Rk3HesthavenSsp for this
 * linear, time-independent operator) and added to the FP64 state once per
 * step; results agree with FP64 to ~1e-14 relative.  Flat system, one brick
 * set of one extent (gamma2 general), Rk3HesthavenSsp, no filter;
 * dgsw_substep is not available (the Taylor form has no substeps). */
typedef enum {
  DGSW_PRECISION_FP64 = 0,
  DGSW_PRECISION_MIXED = 1,
  DGSW_PRECISION_DOUBLE_FLOAT = 2
} DgswPrecision;
/* Spectral::Quadrature of the element meshes.  GAUSS_LOBATTO: faces are
 * volume points and corrections are lifted onto them (lift_flux).  GAUSS:
 * faces are interpolated (boundary_interpolation_matrices) and corrections
 * lifted into the whole element (lift_boundary_terms_gauss_points,
 * NumericalAlgorithms/DiscontinuousGalerkin/LiftFromBoundary.cpp:20-140);
 * flat system, one extent for every element, FP64 precision. */
typedef enum { DGSW_QUADRATURE_GAUSS_LOBATTO = 0, DGSW_QUADRATURE_GAUSS = 1 } DgswQuadrature;

/* One periodic rectilinear evolution domain [lower, upper]^3 with
 * elements[d] elements along axis d.  A count n = b * 2^L (b odd) is laid out
 * as b aligned blocks of refinement level L (Domain/Creators/AlignedLattice,
 * blocks numbered x fastest, Domain/DomainHelpers.cpp:1187-1201). */
typedef struct {
  double lower[3];
  double upper[3];
  int32_t elements[3];
} DgswBrick;

/* A periodic lattice of blocks[0] x blocks[1] x blocks[2] equal blocks on
 * [lower, upper]^3 (blocks x fastest), block k split into 2^levels[k]
 * elements per axis (isotropic initial refinement per block, as
 * Domain/Creators/AlignedLattice's refined regions give).  Blocks that share
 * a face differ by at most one level: the 2:1 faces carry h-nonconforming
 * mortars (Spectral::MortarSize LowerHalf / UpperHalf,
 * NumericalAlgorithms/DiscontinuousGalerkin/MortarHelpers.cpp:49-75).  Flat
 * system, Gauss-Lobatto, one extent for every element, FP64. */
typedef struct {
  double lower[3];
  double upper[3];
  int32_t blocks[3];
  const int32_t* levels;
} DgswRefinedBrick;

/* CurvedScalarWave domain: a spherical shell of six cubed-sphere wedges
 * (Domain/Creators/Sphere.cpp, shell without interior cube; Wedge<3>,
 * Domain/CoordinateMaps/Wedge.cpp:476-536, equiangular, sphericity 1 inside
 * and out; blocks +z, -z, +y, -y, +x, -x, Domain/DomainHelpers.cpp:553-578),
 * initial refinement (ang, ang, rad) per wedge, on the analytic Schwarzschild
 * background in Kerr-Schild coordinates (gr::Solutions::KerrSchild with zero
 * spin and centre, PointwiseFunctions/AnalyticSolutions/GeneralRelativity/
 * KerrSchild.cpp).  Inner sphere: DemandOutgoingCharSpeeds (excision,
 * CurvedScalarWave/BoundaryConditions/DemandOutgoingCharSpeeds.cpp:40-77);
 * outer sphere: ConstraintPreservingSphericalRadiation
 * (.../ConstraintPreservingSphericalRadiation.cpp:40-156). */
typedef enum {
  DGSW_RADIAL_LINEAR = 0,      /* Domain::CoordinateMaps::Distribution::Linear */
  DGSW_RADIAL_LOGARITHMIC = 1  /* Distribution::Logarithmic */
} DgswRadialDistribution;

typedef struct {
  double inner_radius;
  double outer_radius;
  int32_t refinement_angular;  /* elements per wedge along xi and eta: 2^ang */
  int32_t refinement_radial;   /* elements per wedge along zeta: 2^rad */
  int32_t radial_distribution; /* DgswRadialDistribution */
  double mass;                 /* Kerr-Schild mass */
  double gamma1;               /* CurvedScalarWave constraint damping gamma1 */
} DgswShell;

typedef struct {
  int32_t system;              /* DgswSystem */
  int32_t boundary_correction; /* DgswBoundaryCorrection */
  int32_t time_stepper;        /* DgswTimeStepper */
  int32_t precision;           /* DgswPrecision */
  int32_t n_instances;         /* independent evolutions in this handle */
  const DgswBrick* bricks;     /* n_instances domains */
  /* Legendre-Gauss-Lobatto points per dimension, per element (isotropic),
   * in global element order.  NULL: every element has uniform_points. */
  const int32_t* points_per_element;
  int32_t uniform_points;
  double gamma2;               /* constraint damping, ScalarWave/Initialize.hpp:33-56 */
  int32_t device;              /* CUDA device ordinal */
  /* DGSW_SYSTEM_CURVED_SCALAR_WAVE_3D: the shell domain (n_instances = 1,
   * bricks ignored, uniform_points per element); NULL for the flat system. */
  const DgswShell* shell;
  int32_t quadrature;          /* DgswQuadrature (0 = Gauss-Lobatto) */
  /* non-NULL: the domain is this refined block lattice (n_instances = 1,
   * bricks ignored) */
  const DgswRefinedBrick* refined;
  /* DGSW_STEPPER_ADAMS_BASHFORTH: order 1..8 (0 means 3) and, per element,
   * its step level 0..3 (the element steps slab / 2^level; NULL: all 0,
   * global time stepping). */
  int32_t stepper_order;
  const int32_t* step_levels;
} DgswConfig;

typedef struct DgswHandle_* DgswHandle;

/* ---- handle lifecycle ---------------------------------------------------- */
int dgsw_create(const DgswConfig* config, DgswHandle* out);
int dgsw_destroy(DgswHandle h);
const char* dgsw_last_error(DgswHandle h); /* h may be NULL */
int dgsw_abi_version(void);

/* Sizes: elements over all instances; doubles in one state vector. */
int dgsw_sizes(DgswHandle h, int64_t* n_elements, int64_t* state_doubles,
               int64_t* grid_points);
/* The handle's CUDA stream (a cudaStream_t), for interop. */
void* dgsw_stream(DgswHandle h);
int dgsw_synchronize(DgswHandle h);

/* ---- state transfer (Variables<tmpl::list<Psi, Pi, Phi>>) ---------------- */
int dgsw_set_state(DgswHandle h, const double* host_u);
int dgsw_get_state(DgswHandle h, double* host_u);
int dgsw_set_state_device(DgswHandle h, const double* dev_u);
int dgsw_get_state_device(DgswHandle h, double* dev_u);
/* Analytic initial data evaluated on the device at time t.
 * kind 0: PlaneWave (PointwiseFunctions/AnalyticSolutions/WaveEquation/
 *         PlaneWave.cpp:56-80) psi = sin(k.x - |k| t), params = {kx, ky, kz}.
 * kind 1: Gaussian pulse psi = A exp(-|x-c|^2 / w^2), Pi = 0, Phi = grad psi;
 *         params = {A, w, cx, cy, cz} per instance (5 * n_instances values).
 * kind 2: spherical Gaussian shell psi = A exp(-(r - r0)^2 / w^2), Pi = 0,
 *         Phi = grad psi; params = {A, r0, w} (curved system). */
int dgsw_set_initial_data(DgswHandle h, int kind, const double* params,
                          double t);

/* ---- TimeDerivative / BoundaryCorrection ---------------------------------
 * dgsw_rhs: the full semi-discrete DG time derivative du/dt of the state u:
 * volume terms (partial_derivatives + TimeDerivative::apply) plus the
 * UpwindPenalty correction of every mortar lifted onto the GLL faces
 * (ComputeTimeDerivative.hpp:388-650 + ApplyBoundaryCorrections.hpp:723-1050).
 * The handle's precision selects FP64 or mixed arithmetic. */
int dgsw_rhs(DgswHandle h, const double* host_u, double* host_dudt);
int dgsw_rhs_device(DgswHandle h, const double* dev_u, double* dev_dudt);
/* Volume terms only (TimeDerivative::apply after partial_derivatives). */
int dgsw_volume_rhs_device(DgswHandle h, const double* dev_u, double* dev_dudt);

/* UpwindPenalty<3>::dg_package_data (UpwindPenalty.cpp:35-108) on npts face
 * points, device pointers, component-major.  packaged: 16*npts doubles in
 * dg_package_field_tags order (VPsi, VZero[3], VPlus, VMinus,
 * NormalTimesVPlus[3], NormalTimesVMinus[3], Gamma2VPsi, CharSpeeds[3]).
 * normal_dot_mesh_velocity may be NULL.  stream: a cudaStream_t or NULL. */
int dgsw_package_data_device(int64_t npts, const double* psi, const double* pi,
                             const double* phi, const double* gamma2,
                             const double* normal,
                             const double* normal_dot_mesh_velocity,
                             double* packaged, void* stream);
/* UpwindPenalty<3>::dg_boundary_terms (UpwindPenalty.cpp:110-205):
 * out = 5*npts (Psi, Pi, Phi_x, Phi_y, Phi_z corrections). */
int dgsw_boundary_terms_device(int64_t npts, const double* packaged_int,
                               const double* packaged_ext, double* out,
                               void* stream);

/* ---- TimeStepper (Rk3HesthavenSsp) ---------------------------------------
 * dgsw_step: n_steps full SSP-RK3 steps of size dt on the handle's state, each
 * step one fused launch per substep, replayed from a CUDA graph.
 * dgsw_substep: substep k (0, 1, 2) of the step that starts from the state
 * saved by the last dgsw_substep(k=0); for stepping parity with
 * TimeStepper::update_u one substep at a time. */
int dgsw_step(DgswHandle h, int n_steps, double dt);
int dgsw_substep(DgswHandle h, int k, double dt);
/* n_steps of dgsw_step on a state that lives in host memory: host_u is read,
 * stepped on the device and written back in place before the call returns
 * (the handle's device state ends equal to it).  On the plain FP64 path of
 * handles with at least 4096 elements the copies are cut into element chunks
 * overlapped with the stages of the first and the last step (a stage of a
 * chunk waits only for the chunks holding its face neighbours); otherwise
 * the whole state is copied around the steps.  host_u should be pinned
 * (cudaHostAlloc / cudaHostRegister) for full link bandwidth.  As with
 * dgsw_set_state, an AdamsBashforth handle takes the host values as new
 * initial values (self-start). */
int dgsw_step_host(DgswHandle h, double* host_u, int n_steps, double dt);

/* ---- TimeStepper (AdamsBashforth, local time stepping) -------------------
 * Handles with time_stepper DGSW_STEPPER_ADAMS_BASHFORTH: Gauss-Lobatto;
 * the flat system (FP64) on conforming bricks of one extent or of
 * per-element extents (p-nonconforming faces coupled on the mortar at the
 * larger extent for every pair of records, ApplyBoundaryCorrections.hpp:
 * 816-937), or the curved shell of one extent in FP64 or mixed precision
 * (each record dt u in compensated FP32 arithmetic, FP64 state), with the
 * exponential filter after each element step when it is set.  dgsw_step
 * advances n_steps slabs of duration dt (the same dt on every call); within a
 * slab an element of step level l takes 2^l steps, and the UpwindPenalty
 * coupling across faces between levels is integrated by
 * AdamsBashforth::add_boundary_delta.  The first call (and the first after
 * dgsw_set_state or dgsw_set_initial_data) runs the reference's self-start
 * procedure (SelfStartActions.hpp:136-482) at steps of slab / (order 2^L),
 * L the finest level; every element then steps slab / 2^L until the first
 * slab boundary after which no self-start value remains in any history,
 * and from there slab / 2^level.  dgsw_substep returns
 * DGSW_ERR_UNSUPPORTED. */
/* Device history of AdamsBashforth handles: ring slots per element, ticks
 * per slab, grid-point time derivatives evaluated per slab after the
 * start-up, and device launches per slab. */
int dgsw_adams_info(DgswHandle h, int* ring_slots, int64_t* ticks_per_slab,
                    int64_t* rhs_points_per_slab, int* launches_per_slab);

/* Host-only restatements used by the schedule (no GPU needed).  Times are
 * integer ticks, ticks_per_slab to a slab of duration `slab`.
 * adams_coefficients::coefficients (AdamsCoefficients.hpp:29-67), n <= 8: */
int dgsw_adams_coefficients(int n, const int64_t* control_ticks, int64_t step_start,
                            int64_t step_end, double slab, int64_t ticks_per_slab,
                            double* out);
/* adams_lts::lts_coefficients for explicit schemes (AdamsLts.cpp:301-415) of
 * orders local_order, remote_order, small_order.  Histories are (slab
 * number, tick) time ids in insertion order; output terms index them, one
 * per (local id, remote id), sorted by ids.  Returns the number of terms
 * (<= max_out) or a negative status. */
int dgsw_lts_coefficients(int n_local, const int64_t* local_slab, const int64_t* local_tick,
                          int n_remote, const int64_t* remote_slab, const int64_t* remote_tick,
                          int64_t step_start, int64_t step_end, double slab,
                          int64_t ticks_per_slab, int local_order, int remote_order,
                          int small_order, int max_out, int32_t* out_local,
                          int32_t* out_remote, double* out_coef);
/* One level's work in one device launch of the schedule (the coefficient
 * tables the kernel applies; marginals of the lts_coefficients terms). */
typedef struct {
  int32_t launch;   /* index of the device launch */
  int32_t level;
  int32_t update;   /* finish the step: volume update and boundary delta */
  int32_t reset;    /* restore the initial values (self-start) */
  int32_t rec_slot; /* ring slot of the record of the new state */
  int32_t n_vol;
  int32_t vol_slot[8];
  double vol_c[8];
  int32_t n_loc[4]; /* per neighbour level */
  int32_t loc_slot[4][8];
  double loc_c[4][8];
  int32_t n_rem[4];
  int32_t rem_slot[4][16];
  double rem_c[4][16];
} DgswAdamsJob;
/* The schedule of n_slabs slabs (the first includes the self-start) for
 * level_counts[l] elements of level l and adjacency[4*l + m] != 0 when a
 * level-l element has a level-m face neighbour.  Writes up to max_jobs jobs
 * and their number, the ticks per slab and the ring slots needed. */
int dgsw_adams_schedule(int order, const int64_t* level_counts, const int32_t* adjacency,
                        double slab, int n_slabs, int max_jobs, DgswAdamsJob* jobs,
                        int* n_jobs, int64_t* ticks_per_slab, int* ring_slots);

/* ---- time bookkeeping: TimeStepId and next_time_id --------------------------
 * TimeStepId (src/Time/TimeStepId.hpp:26-70, TimeStepId.cpp:19-98) with the
 * step start as an exact fraction of its slab (Time, src/Time/Time.cpp:96-98:
 * value = (1 - f) start + f end; Slab::advance / retreat, Slab.cpp:31-33),
 * and the time steppers' next_time_id: Rk3HesthavenSsp
 * (src/Time/TimeSteppers/Rk3HesthavenSsp.cpp:36-48: substep 0 -> 1 at
 * fraction 1 of the step, 1 -> 2 at 1/2, 2 -> the next step) and
 * AdamsBashforth (one substep: the next step).  Host-only.  The substeps of
 * dgsw_step evaluate the right-hand side at these times; nothing on this
 * path depends on time explicitly, so they are bookkeeping for callers. */
typedef struct DgswTimeStepId {
  int64_t slab_number;
  double slab_start, slab_end; /* the slab of the step's start */
  int32_t step_num, step_den;  /* step start = step_num/step_den of the slab (reduced) */
  int32_t substep;
  int32_t size_num, size_den;  /* step size as a slab fraction; +-1/1 (time's
                                  direction) at substep 0 */
  double substep_time;         /* time of this substep */
} DgswTimeStepId;
/* The id at the start of a step at fraction num/den of the slab
 * [slab_start, slab_end] (the TimeStepId(bool, int64_t, const Time&)
 * constructor: a time at the slab's end moves into the next slab). */
int dgsw_time_step_id(int time_runs_forward, int64_t slab_number, double slab_start,
                      double slab_end, int32_t num, int32_t den, DgswTimeStepId* out);
/* TimeStepper::next_time_id for time_stepper (DgswTimeStepper) with the step
 * size size_num/size_den of the slab.  DGSW_ERR_ARGUMENT where the reference
 * ERRORs or ASSERTs (bad substep, a step leaving its slab, a step size that
 * changes within a step, 32-bit fraction overflow). */
int dgsw_next_time_id(int time_stepper, const DgswTimeStepId* current, int32_t size_num,
                      int32_t size_den, DgswTimeStepId* next);
/* The fraction of the step at which substep k evaluates the right-hand side
 * (Rk3HesthavenSsp: 0, 1, 1/2; AdamsBashforth: 0). */
int dgsw_substep_time_fraction(int time_stepper, int substep, double* fraction);

/* ---- step size and state guards ---------------------------------------------
 * dgsw_cfl_steps: StepChoosers::Cfl (src/Time/StepChoosers/Cfl.hpp:55-67) for
 * every element of a configuration: safety_factor * stable_step of the
 * configured time stepper (Rk3HesthavenSsp.cpp:23-26, AdamsBashforth.cpp:
 * 66-82) * the element's minimum grid spacing (src/Domain/
 * MinimumGridSpacing.cpp) / (its largest characteristic speed * 3)
 * (ScalarWave: 1; CurvedScalarWave: Characteristics.cpp:202-212).  Host-only;
 * element_steps (one per element) and min_step may be NULL.
 * dgsw_set_guards: with cfl_safety_factor > 0, dgsw_step refuses, before any
 * work, a step longer than an element's Cfl step (for AdamsBashforth: the
 * slab / 2^level of any element) with DGSW_ERR_CFL, as the Cfl chooser
 * rejects it; with check_finite, dgsw_step checks the state afterwards and
 * reports a NaN or Inf with DGSW_ERR_NOT_FINITE (the message names the first
 * element).  Both off at creation.
 * dgsw_check_finite: the first element whose values hold a NaN or an Inf,
 * -1 when all are finite. */
int dgsw_cfl_steps(const DgswConfig* config, double safety_factor, double* element_steps,
                   double* min_step);
int dgsw_set_guards(DgswHandle h, double cfl_safety_factor, int check_finite);
int dgsw_check_finite(DgswHandle h, int64_t* first_element);

/* ---- launch autotuner -------------------------------------------------------
 * The plain FP64 stage kernel exists in DGSW_STAGE_VARIANTS launch
 * configurations per N: two of elements per block and resident blocks per SM
 * (0, 1), and two that run the three axis passes of one element at once (2, 3:
 * three times the threads for the same work, for grids too small to fill the
 * GPU; 3 asks for one more resident block per SM than 2).
 * All give the same bits.  The first dgsw_step of a handle times each on the
 * handle's own data (without touching its state), keeps the fastest and
 * reuses the choice for handles of the same shape.  dgsw_autotune re-runs
 * the timing now and returns the chosen variant and the measured ms per
 * stage launch of each (ms_per_launch holds DGSW_STAGE_VARIANTS values; zeros
 * where nothing is tuned: mixed, curved, Gauss and mixed-extent handles use
 * fixed configurations); force_variant >= 0 then imposes that variant (-1
 * keeps the fastest).  No counterpart in the reference. */
#define DGSW_STAGE_VARIANTS 4
int dgsw_autotune(DgswHandle h, int force_variant, int* variant, double* ms_per_launch);

/* The launch autotuner of whichever step kernels the handle runs.
 * family: DGSW_TUNE_FP64_STAGE (the plain FP64 stage kernel's
 * configurations, as dgsw_autotune), DGSW_TUNE_MIXED_BATCH (mixed precision
 * on elements of differing extents: the persistent batch kernels' compiled
 * launch shapes -- threads per CTA, resident CTAs per SM, pipeline buffers,
 * largest extent), DGSW_TUNE_MIXED_PIPE (mixed precision on one even extent:
 * four candidates, the pipelined kernel with two pipeline buffers or one
 * buffer and more resident CTAs (bit 0), each with the step's FP64 update
 * u0 + W as a separate stream or in the last stage's epilogue (bit 1)),
 * DGSW_TUNE_MIXED_CURVED (mixed precision on the curved shell: the stage
 * kernel at 256 threads per block with its default or one more resident
 * block per SM, or at 512 threads (candidates 0-2), each with the step's
 * FP64 update in the last stage's epilogue or as a separate stream (3-5)),
 * or DGSW_TUNE_NONE (fixed
 * configurations).  Re-times every
 * candidate now on the handle's own state (saved and restored), keeps the
 * fastest (force_variant >= 0 imposes one instead) and returns the number of
 * candidates, the choice and ms per step of each (ms_per_step holds
 * DGSW_TUNE_MAX_VARIANTS values; 0 for candidates that cannot hold the
 * domain).  The first dgsw_step of a handle runs the same timing when its
 * shape has not been tuned in this process.  No counterpart in the
 * reference. */
enum {
  DGSW_TUNE_NONE = 0,
  DGSW_TUNE_FP64_STAGE = 1,
  DGSW_TUNE_MIXED_BATCH = 2,
  DGSW_TUNE_MIXED_PIPE = 3,
  DGSW_TUNE_MIXED_CURVED = 4
};
#define DGSW_TUNE_MAX_VARIANTS 8
int dgsw_tune(DgswHandle h, int force_variant, int* family, int* n_variants, int* variant,
              double* ms_per_step);

/* ---- diagnostics -------------------------------------------------------------
 * dgsw_check_device_timeout: runs the mixed-precision pipeline's bounded
 * device-side wait on an mbarrier that no copy ever completes, with the given
 * limit (at most 10 s).  The kernel gives up, records the handle's error word
 * and returns; the call then reports DGSW_ERR_DEVICE_TIMEOUT exactly as a
 * stage whose staged copy never landed would, and the handle stays usable.
 * No counterpart in the reference (its runtime has no device-side waits). */
int dgsw_check_device_timeout(DgswHandle h, double limit_seconds);

/* ---- observation ------------------------------------------------------------
 * Events::ObserveNorms (ParallelAlgorithms/Events/ObserveNorms.cpp:33-105,
 * ObserveNorms.hpp:47-80,145-171) of Psi, Pi, Phi_x, Phi_y, Phi_z, each
 * "Individual", over every element of the handle, on the device in FP64:
 * out[5*v + m], m = 0 Max, 1 Min, 2 L2Norm = sqrt(sum u^2 / points),
 * 3 L2IntegralNorm = sqrt(int u^2 dV / V), 4 VolumeIntegral = int u dV;
 * out[25] = points, out[26] = V (definite_integral on the LGL mesh times
 * det(Jacobian)).  dev_u: device state (NULL: the handle's state);
 * dev_subtract (may be NULL) is subtracted first.
 * dgsw_observe_plane_wave_errors: the same norms of the state minus
 * PlaneWave(k, t) (PointwiseFunctions/AnalyticSolutions/WaveEquation/
 * PlaneWave.cpp:56-80), the Error(...) norms of ObserveNorms; flat system. */
int dgsw_observe_norms(DgswHandle h, const double* dev_u, const double* dev_subtract,
                       double* out);
int dgsw_observe_plane_wave_errors(DgswHandle h, const double* k, double t, double* out);

/* ---- exponential filter ----------------------------------------------------
 * Filters::Exponential (NumericalAlgorithms/LinearOperators/
 * ExponentialFilter.cpp:23-80) applied by dg::Actions::Filter
 * (ParallelAlgorithms/Actions/FilterAction.hpp:109-180) to Psi, Pi and Phi
 * after every substep's update, as the curved executable's step actions do
 * (Evolution/Executables/CurvedScalarWave/EvolveCurvedScalarWave.hpp:237-266):
 * per axis F = V diag(exp(-alpha (k/(N-1))^(2 half_power))) V^-1
 * (Spectral/Filtering.cpp:18-31).  enable = 0 switches it off.  FP64
 * precision only (DGSW_ERR_UNSUPPORTED for mixed handles).
 * dgsw_exponential_filter_matrix: the 1D matrix, row-major (host only). */
int dgsw_set_exponential_filter(DgswHandle h, double alpha, int half_power, int enable);
int dgsw_exponential_filter_matrix(int n, double alpha, int half_power, double* F);

/* ---- AMR projection of element data ----------------------------------------
 * amr::projectors::ProjectVariables (ParallelAlgorithms/Amr/Projectors/
 * Variables.hpp:25-99) on the device.  Per dimension d of target block k,
 * child[3k + d] selects the 1D matrix from source extent src_extents[3k + d]
 * to target extent dst_extents[3k + d]:
 *   0  p-refinement (ChildSize::Full, Spectral::p_projection_matrices,
 *      Projection.cpp:401-421): identity for equal extents, interpolation to
 *      a finer extent, Legendre modal truncation to a coarser one;
 *   1, 2  h-refinement to the lower / upper half
 *      (projection_matrix_parent_to_child, Projection.cpp:291-372):
 *      interpolation to the child's points mapped into that half; the target
 *      needs at least as many points as the source.
 * dgsw_amr_matrix: that matrix, dst x src row-major (host only).
 * dgsw_amr_project_device: target block k (n_vars components, x fastest, as
 * in Variables) is written at dev_out + out_offset[k] from source block
 * src[k] at dev_in + in_offset[src[k]] (offsets in doubles, host arrays;
 * device pointers for the data; dev_in != dev_out).  Uses h's device and
 * stream and returns when the projection is done.  h-coarsening is not
 * provided (the reference ERRORs on it too). */
int dgsw_amr_matrix(int src_extent, int dst_extent, int child, double* M);
int dgsw_amr_project_device(DgswHandle h, int n_vars, int64_t n_in, const int64_t* in_offset,
                            const double* dev_in, int64_t n_out, const int32_t* src,
                            const int32_t* src_extents, const int32_t* dst_extents,
                            const int8_t* child, const int64_t* out_offset, double* dev_out);

/* ---- discrete adjoint and the misfit objective -----------------------------
 * One brick of uniform extent, gamma2 = 0, Rk3HesthavenSsp, no filter.  The
 * step map of this path is linear (fixed normals and char speeds), so the
 * reverse sweep needs only the recorded residuals, not the forward states.
 * FP64 handles run dgsw_step forward and the FP64 adjoint (three L^T
 * launches per step, the reverse stages of Rk3HesthavenSsp).  Mixed-precision
 * and double-float handles run both sweeps as the step's Taylor polynomial
 * 1 + dt L + (dt L)^2/2 + (dt L)^3/6 (the same map): W1 = dt L u,
 * W2 = dt L W1, W3 = dt L W2, u += W1 + W2/2 + W3/6 (L^T and the adjoint
 * state backwards), with FP64 states and double-float increments formed in
 * FP32 arithmetic (on mixed-precision handles not the FP32 increments of
 * dgsw_step: the residuals and the rough adjoint field need ~1e-8 of
 * themselves over thousands of steps).
 * dgsw_adjoint_rhs_device: lambda -> L^T lambda (FP64), the exact transpose
 * of the operator dgsw_rhs_device applies.
 * dgsw_set_samples: points (x, y, z per point) where Psi is sampled by
 * barycentric Lagrange interpolation on the element's LGL nodes
 * (Spectral.cpp:625-670 weights; the role of IrregularInterpolant,
 * NumericalAlgorithms/Interpolation/IrregularInterpolant.cpp:257-319).
 * dgsw_sample_psi: Psi of the current state at the sample points (host).
 * dgsw_misfit_forward: advances the state by n_windows x steps_per_window
 * steps, sampling after each window; J = sum (sample - target)^2, targets
 * n_windows x n_samples (host, window-major).
 * dgsw_misfit_adjoint: dJ/du at the start of the last dgsw_misfit_forward,
 * state-sized, into dev_grad (device); the adjoint of Rk3HesthavenSsp run
 * backwards with 2 (sample - target) injected at each window. */
int dgsw_adjoint_rhs_device(DgswHandle h, const double* dev_lambda, double* dev_out);
int dgsw_set_samples(DgswHandle h, int n_samples, const double* xyz);
int dgsw_sample_psi(DgswHandle h, double* host_out);
int dgsw_misfit_forward(DgswHandle h, int n_windows, int steps_per_window, double dt,
                        const double* host_targets, double* J);
int dgsw_misfit_adjoint(DgswHandle h, double* dev_grad);
/* The adjoint kernel's two work splits (N^2 threads per element with the
 * three axes in turn, or 3 N^2 threads with the axes at once; the same bits).
 * The first dgsw_misfit_adjoint times both on the handle's state and keeps the
 * faster; dgsw_adjoint_autotune re-times them now and returns the choice and
 * ms per L^T launch of each (ms_per_launch: 2 values); force_variant 0 or 1
 * imposes a split afterwards (-1 keeps the faster).  No counterpart in the
 * reference. */
int dgsw_adjoint_autotune(DgswHandle h, int force_variant, int* variant, double* ms_per_launch);

/* ---- host-only setup (no GPU) ---------------------------------------------
 * Spectral::collocation_points / quadrature_weights <Legendre, GaussLobatto>
 * (NumericalAlgorithms/Spectral/Legendre.cpp:186-239) */
int dgsw_lgl_points_weights(int n, double* x, double* w);
/* Legendre-Gauss tables (Spectral.cpp, Quadrature::Gauss): nodes x and
 * weights w (Legendre.cpp:106-149), D row-major, the interpolation rows to
 * xi = -1 and +1 (boundary_interpolation_matrices, Spectral.cpp:676-697) and
 * the boundary_lifting_term rows (Spectral.cpp:753-781).  Any output may be
 * NULL; each holds n (D: n*n) doubles. */
int dgsw_gauss_spectral(int n, double* x, double* w, double* D, double* interp_lower,
                        double* interp_upper, double* lift_lower, double* lift_upper);
/* Spectral::differentiation_matrix, row-major D[i*n+j]
 * (NumericalAlgorithms/Spectral/Spectral.cpp:113-447) */
int dgsw_differentiation_matrix(int n, double* D);
/* Spectral::projection_matrix_parent_to_child (face -> mortar, nm x ne) and
 * projection_matrix_child_to_parent (mortar -> face, ne x nm), ChildSize::Full
 * (NumericalAlgorithms/Spectral/Projection.cpp:56-375) */
int dgsw_mortar_projections(int ne, int nm, double* face_to_mortar,
                            double* mortar_to_face);
/* Element / neighbour index maps of a configuration (Domain/Structure):
 * element_ids: packed ElementId<3> bits (ElementId.hpp:138-147), n_elements;
 * neighbors: 6 per element in Direction<3>::all_directions() order
 *            (Direction.hpp:186-193), global element index;
 * mortar_points: 6 per element, mortar_mesh extent (MortarHelpers.cpp:21-47);
 * Curved shell: neighbours -1 on the inner sphere and -2 on the outer one,
 * where mortar_points is 0 (external boundaries carry no mortar).
 * Any output may be NULL.  Returns DGSW_ERR_UNSUPPORTED when a block id does
 * not fit the reference's 8 block-id bits (the other outputs are still set). */
int dgsw_index_maps(const DgswConfig* config, uint64_t* element_ids,
                    int32_t* neighbors, int32_t* mortar_points);
int dgsw_count_elements(const DgswConfig* config, int64_t* n_elements,
                        int64_t* state_doubles);
/* Mortars of a refined block lattice: 4 neighbour slots per element face
 * (slot (6e + dir) * 4 + k; -1 unused) and, per slot, the mortar size in the
 * face's two transverse dimensions (ascending): 0 Full, 1 LowerHalf,
 * 2 UpperHalf, as mortar_size(self, neighbour) (MortarHelpers.cpp:49-75).
 * DGSW_ERR_ARGUMENT when neighbouring blocks differ by more than one level. */
int dgsw_refined_mortars(const DgswConfig* config, int32_t* neighbor_slots,
                         int32_t* mortar_sizes);
/* Half-interval projections on n LGL points, n x n row-major:
 * projection_matrix_parent_to_child (interpolation to the half) and
 * projection_matrix_child_to_parent (L2 restriction from the half),
 * ChildSize LowerHalf (upper = 0) or UpperHalf (upper = 1),
 * NumericalAlgorithms/Spectral/Projection.cpp:56-375. */
int dgsw_half_projections(int n, int upper, double* parent_to_child,
                          double* child_to_parent);
/* Shell geometry of a curved configuration (host, FP64): per element the
 * inertial coordinates (3*N^3, component-major), the inverse Jacobian
 * d xi^a / d x^i (9*N^3, component 3a+i; ElementMap::inv_jacobian of the
 * element's affine map composed with Wedge<3>), and for each of the 6 faces
 * and each face point (a + N*b over the two remaining axes, ascending) the
 * neighbour's face-point index of the same physical point: the permutation
 * that orient_variables_on_slice (Domain/Structure/OrientationMapHelpers.cpp)
 * applies between wedges (6*N^2 per element; -1 on the shell's boundary).
 * Any output may be NULL. */
int dgsw_shell_geometry(const DgswConfig* config, double* xyz, double* inverse_jacobian,
                        int32_t* face_permutation);

/* ---- stepping without any allocation ---------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory while they step (a host framework that owns a fixed device-memory
 * budget, or a caller that must not trigger the device-wide synchronisation
 * of cudaMalloc/cudaFree): n_steps plain-FP64 SSP-RK3 steps of one periodic
 * brick, in place on the caller's device state dev_u (layout as
 * dgsw_set_state), on `stream` (a cudaStream_t or NULL).  Creates no handle
 * and calls no allocating routine: the stage states and element tables live
 * in one fixed 32 MiB device array inside the library, held by every GPU that
 * loads it until the process exits.  The limit is
 *   2 * elements * 5 * points^3 + 6 * elements <= 4,194,304 doubles
 * (e.g. 8^3 elements at 8 points, 12^3 elements at 5 points); larger bricks
 * return DGSW_ERR_ARGUMENT, and so does a dev_u that is not memory of the
 * current device.  Every call looks up the array's address on the current
 * device; the first call on a device may load the library's device code
 * there, so make it before any stream capture.  Calls share the array and
 * it keeps the last call's contents: calls that overlap on the GPU race, and
 * the caller must serialise them.  Errors: dgsw_noalloc_last_error(). */
int dgsw_step_noalloc(const DgswBrick* brick, int points, double gamma2,
                      double* dev_u, int n_steps, double dt, void* stream);
size_t dgsw_noalloc_scratch_bytes(void);
const char* dgsw_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* DGSW_H */
