/*
 * sse_gb300.h -- C-ABI of the GB300 (sm_103a) semi-discrete residual library.
 *
 * Drop-in for the right-hand side that StableSpectralElements.jl's
 * `semidiscretize(...)` hands to OrdinaryDiffEq:
 *
 *   semi_discrete_residual!(dudt, u, solver, t)   src/Solvers/Solvers.jl:474-514
 *     -> nodal_values!(u, solver, k)              standard_form_first_order.jl:1-14,
 *                                                 flux_differencing_form.jl:253-292
 *     -> time_derivative!(dudt, solver, k)        standard_form_first_order.jl:16-63,
 *                                                 flux_differencing_form.jl:294-347
 *
 * A Julia `Solver{..., GB300}` owns one handle; the operator and geometry
 * arrays are the fields of `solver.operators` / `solver.mass_solver` and
 * `solver.connectivity`, passed by pointer in the reference's own
 * column-major layouts (no transposition).  All arithmetic of the plain form
 * is FP64, as in the reference.
 *
 * Threading: one handle = one CUDA stream.  Calls on one handle must be
 * serialised by the caller (OrdinaryDiffEq calls the RHS from one thread);
 * distinct handles are independent.  No function throws; every function
 * returns an sse_status and leaves a message for sse_last_error().
 */
#ifndef SSE_GB300_H
#define SSE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SSE_ABI_VERSION 1

typedef enum sse_status {
  SSE_OK = 0,
  SSE_ERR_INVALID_ARGUMENT = 1, /* null pointer, size mismatch, bad index */
  SSE_ERR_UNSUPPORTED = 2,      /* combination the library does not implement */
  SSE_ERR_CUDA = 3,             /* CUDA runtime error (message in sse_last_error) */
  SSE_ERR_NONPHYSICAL = 4,      /* non-finite result or non-positive density/pressure */
  SSE_ERR_OUT_OF_MEMORY = 5
} sse_status;

/* Residual form: StandardForm / FluxDifferencingForm (Solvers.jl:90-115). */
enum sse_form { SSE_STANDARD_FORM = 0, SSE_FLUX_DIFFERENCING_FORM = 1 };
/* Conservation law (ConservationLaws.jl:192-204). */
enum sse_law { SSE_LINEAR_ADVECTION = 0, SSE_EULER = 1 };
/* Interface numerical flux (ConservationLaws.jl:52-62). */
enum sse_numerical_flux {
  SSE_LAX_FRIEDRICHS = 0,        /* LaxFriedrichsNumericalFlux(λ): halfλ = λ/2 */
  SSE_CENTRAL = 1,               /* CentralNumericalFlux */
  SSE_ENTROPY_CONSERVATIVE = 2   /* EntropyConservativeNumericalFlux */
};
/* Two-point flux (ConservationLaws.jl:70-73): ConservativeFlux,
 * EntropyConservativeFlux (Ranocha's, euler_navierstokes.jl:171-195), and
 * Chandrashekar's entropy-conservative, kinetic-energy-preserving flux
 * (Chandrashekar 2013; an extra option with no reference counterpart). */
enum sse_two_point_flux { SSE_CONSERVATIVE_FLUX = 0, SSE_EC_FLUX = 1, SSE_CHANDRASHEKAR_FLUX = 2 };
/* Mass-matrix solver (mass_matrix.jl:1-17). */
enum sse_mass_solver { SSE_WEIGHT_ADJUSTED = 0, SSE_DIAGONAL = 1 };
/* Arithmetic of the bulk flux/operator work. */
enum sse_precision { SSE_FP64 = 0, SSE_MIXED = 1 };
/* Where the caller's state buffers live. */
enum sse_memory { SSE_HOST = 0, SSE_DEVICE = 1 };
/* Time integrators (OrdinaryDiffEq algorithms the reference's tests use). */
enum sse_rk_scheme { SSE_CARPENTER_KENNEDY_2N54 = 0, SSE_RK4 = 1 };

typedef struct sse_config {
  int32_t d;              /* spatial dimension: 2 (Tri) or 3 (Tet) */
  int32_t n_p;            /* solution coefficients per element (size(V, 2)) */
  int32_t n_q;            /* volume quadrature nodes (size(V, 1)) */
  int32_t n_f;            /* facet quadrature nodes (size(R, 1)) */
  int32_t n_c;            /* conservative variables */
  int32_t n_e;            /* elements */
  int32_t num_faces;      /* 3 (Tri) or 4 (Tet) */
  int32_t nodes_per_face; /* FluxDifferencingOperators.nodes_per_face */
  int32_t form;           /* enum sse_form */
  int32_t law;            /* enum sse_law */
  int32_t numerical_flux; /* enum sse_numerical_flux */
  int32_t two_point_flux; /* enum sse_two_point_flux (FluxDifferencingForm) */
  int32_t mass_solver;    /* enum sse_mass_solver */
  int32_t reserved;
  double half_lambda;     /* LaxFriedrichsNumericalFlux.halfλ */
  double gamma;           /* EulerEquations.γ */
  double a[3];            /* LinearAdvectionEquation.a */
} sse_config;

/* SparseArrays.SparseMatrixCSC{Float64,Int64} fields, 1-based as in Julia. */
typedef struct sse_csc {
  int64_t m, n;
  const int64_t *colptr; /* n + 1 entries */
  const int64_t *rowval; /* nnz entries */
  const double *nzval;   /* nnz entries */
} sse_csc;

typedef struct sse_operators {
  /* V: WarpedTensorProductMap2D/3D factors (warped_product_2d.jl:2-23,
   * warped_product_3d.jl:2-36), all NULL when V is the identity
   * (NodalTensor's UniformScalingMap). */
  int32_t vdm_p;             /* polynomial degree p */
  int32_t vdm_m[3];          /* M1, M2, M3: 1-D quadrature sizes */
  const double *vdm_A;       /* M1 x (p+1) */
  const double *vdm_B;       /* M2 x (p+1) x (p+1) */
  const double *vdm_C;       /* M3 x (p+1) x (p+1) x (p+1), Tet only */
  const int64_t *vdm_sigma_in; /* (p+1)^d modal index, 1-based, 0 if unused */
  /* R: volume -> facet interpolation, sparse(Matrix(R)), N_f x N_q */
  sse_csc R;
  /* StandardForm (ReferenceOperators.D, operators.jl:25): N_q x N_q each */
  sse_csc D[3];
  /* FluxDifferencingForm (FluxDifferencingOperators.S, C; operators.jl:192-200) */
  sse_csc S[3];              /* N_q x N_q each */
  sse_csc C;                 /* N_q x N_f; nnz = 0 means no facet correction */
  /* Dense V, N_q x N_p: Matrix(V) of the multidimensional ModalMulti
   * approximation (OctavianMap(VDM), multidimensional.jl:1-41), with vdm_*
   * NULL; NULL for the tensor-product and nodal approximations. */
  const double *V_dense;
} sse_operators;

typedef struct sse_geometry {
  /* both forms */
  const double *BJf;         /* N_f x N_e        : B .* J_f */
  const double *n_f;         /* d x N_f x N_e    : nJf ./ J_f */
  const int64_t *mapP;       /* N_f x N_e        : 1-based linear index into (N_f, N_e) */
  /* StandardForm: ReferenceOperators.halfWΛ packed as N_q x d x d x N_e */
  const double *halfWLambda;
  /* FluxDifferencingForm */
  const double *WJ;          /* N_q x N_e        : W .* J_q */
  const double *Lambda_q;    /* N_q x d x d x N_e */
  const double *halfnJf;     /* d x N_f x N_e */
  const double *halfnJq;     /* d x num_faces x N_q x N_e */
  /* mass solver */
  const double *JinvW;       /* N_q x N_e : WeightAdjustedSolver.J⁻¹W (W ./ J_q) */
  const double *WJinv;       /* N_q x N_e : DiagonalSolver.WJ⁻¹ (1 ./ (W .* J_q)) */
} sse_geometry;

typedef struct sse_solver sse_solver;

/* Library ABI version (SSE_ABI_VERSION). */
int32_t sse_abi_version(void);

/* Build a handle: validates sizes and indices, deep-copies operators and
 * geometry to the current CUDA device and allocates the per-element scratch
 * (u_q, u_f) that Solver.preallocated_arrays holds in the reference
 * (Solvers.jl:183-209).  With a weight-adjusted mass solver it also builds
 * each element's mass operator V' diag(J^-1 W) V (N_p x N_p doubles per
 * element) when they take at most a quarter of the free device memory; the
 * mass solves are then dense products, otherwise two sum-factorised
 * applications of V.  Replaces Solver(...) + the Threaded/Serial parallelism
 * tag (Solvers.jl:287-333, 429-452). */
int32_t sse_create(const sse_config *cfg, const sse_operators *ops,
                   const sse_geometry *geo, sse_solver **out);
int32_t sse_destroy(sse_solver *s);

/* dudt <- R(u): semi_discrete_residual!(dudt, u, solver, t), Solvers.jl:474-514.
 * u and dudt are N_p x N_c x N_e column-major FP64, host or device memory.
 * SSE_HOST buffers that are page-locked and mapped into the device's address
 * space (cudaHostAlloc, cudaHostRegister with mapping) are read and written
 * in place by the kernels over the host link; other host buffers go through
 * the handle's device buffers with one copy each way.  dudt may be u. */
int32_t sse_residual(sse_solver *s, const double *u, double *dudt, double t,
                     int32_t memory);

/* Capacity of the fixed device buffer used by sse_residual_static_scratch:
 * 32 MiB, i.e. room for (n_q + n_f) * n_c * n_e nodal values up to 4,194,304
 * doubles in the FP64 form (for example 8192 Euler triangles at p = 4, not
 * the 24,576-tet mesh) or 8,388,608 floats in the mixed form. */
#define SSE_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)

/* dudt <- R(u) exactly like sse_residual on the same handle, in the handle's
 * precision (SSE_FP64 or SSE_MIXED), for callers that cannot allocate GPU
 * memory while they run: code that must not call cudaMalloc inside its time
 * loop (a real-time or latency-bound step whose memory is fixed up front, a
 * host framework that owns the device memory pool and forbids raw
 * allocation), after the handle was created (and its precision set) at
 * set-up.  This call allocates nothing: the element nodal states that the
 * residual's two kernels hand to each other (FP64 states, or the mixed
 * form's FP32 perturbation states) live in one file-scope device array of
 * SSE_STATIC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits; u_dev and dudt_dev are device pointers supplied by the
 * caller.  Meshes whose nodal states exceed that size are rejected with
 * SSE_ERR_INVALID_ARGUMENT.  The first call on each device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  On an SSE_MIXED handle
 * whose reference state is not yet chosen, the call chooses it first (a
 * reduction over u and one FP64 evaluation, in buffers sse_set_precision
 * allocated).  Every call synchronises the handle's stream before it
 * returns, to read the non-physical-state flag.  All calls share the one
 * array: calls that overlap on the GPU (other handles, other streams, other
 * threads) race and must be serialised by the caller.  Each call rewrites
 * the whole part of the array it reads, so nothing needs clearing between
 * calls.  On a handle running the one-kernel StandardForm path
 * (sse_kernel_path) the residual keeps no nodal states: the call uses
 * neither the array nor its size limit.  No counterpart in the reference,
 * which has no device memory. */
int32_t sse_residual_static_scratch(sse_solver *s, const double *u_dev, double *dudt_dev);

/* Phase A alone: nodal_values! for every element (standard_form_first_order.jl:
 * 1-14, flux_differencing_form.jl:253-292).  u_q is N_q x N_c x N_e and u_f is
 * N_f x N_e x N_c, the reference's PreAllocatedArraysFirstOrder layouts. */
int32_t sse_nodal_values(sse_solver *s, const double *u, double *u_q, double *u_f,
                         int32_t memory);

/* n_steps fixed-step time steps of OrdinaryDiffEq's CarpenterKennedy2N54 or
 * RK4 (solve(ode, alg; dt, adaptive=false)), entirely on the device; u is
 * advanced in place and *t by n_steps*dt. */
int32_t sse_rk_steps(sse_solver *s, double *u, int32_t n_steps, double dt,
                     int32_t scheme, double *t, int32_t memory);

/* Discrete adjoint of the FP64 residual: mu <- (dR/du)^T lam at the state u
 * (all three N_p x N_c x N_e, host or device).  Covers every configuration
 * sse_create accepts: StandardForm and FluxDifferencingForm (entropy-
 * conservative or conservative two-point flux), Euler and linear advection,
 * any of the three interface fluxes.  With
 * the handle in SSE_MIXED the product is that of the mixed form (FP32
 * transposes of its reduced fluxes and projection arithmetic, ModalTensor
 * bases).  The vector-Jacobian product of semi_discrete_residual!; no
 * counterpart in the reference, whose residual is typed Float64 throughout
 * and has no AD or adjoint code (Solvers.jl:474-514). */
int32_t sse_residual_vjp(sse_solver *s, const double *u, const double *lam, double *mu,
                         int32_t memory);

/* sse_rk_steps that also records the trajectory for sse_rk_adjoint: the
 * state at every checkpoint_every-th step (and the compensation term in
 * SSE_MIXED) plus the stage data of the last segment are kept in device
 * memory owned by the handle, replacing the previous recording (the memory
 * is reused when it suffices).  checkpoint_every = 0 picks the longest
 * segments whose recording fits in 3/4 of the free device memory less
 * 512 MiB, i.e. the fewest segments to recompute (none when the whole
 * trajectory fits).  Fails with SSE_ERR_OUT_OF_MEMORY (nothing advanced)
 * when the recording does not fit.  The forward half of the stepper's
 * rrule; no counterpart in the reference. */
int32_t sse_rk_record(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme,
                      int32_t checkpoint_every, double *t, int32_t memory);

/* sse_rk_steps that records the trajectory for sse_rk_adjoint on the
 * binomial ("revolve") schedule of Griewank & Walther (ACM TOMS 26, 2000),
 * for horizons whose uniform recording does not fit: only n_checkpoints
 * states (0: as many as fit in 3/4 of the free device memory less 512 MiB,
 * at most n_steps - 1) plus the stage data of one step are kept, and the
 * reverse sweep recomputes the fewest forward steps any schedule with that
 * many checkpoints can (optimal split table for up to 2048 steps, fewer
 * when the checkpoints are many, halving beyond).  The gradient is bitwise that of sse_rk_record.  Fails with
 * SSE_ERR_OUT_OF_MEMORY when even that does not fit.  No counterpart in the
 * reference. */
int32_t sse_rk_record_binomial(sse_solver *s, double *u, int32_t n_steps, double dt,
                               int32_t scheme, int32_t n_checkpoints, double *t,
                               int32_t memory);

/* Extra forward steps (beyond the n_steps recorded ones) of the optimal
 * binomial schedule for n_steps steps and n_checkpoints checkpoints, and the
 * first step at which it places a checkpoint (0 when it places none).  Host
 * arithmetic only, no device work. */
int32_t sse_binomial_schedule(int32_t n_steps, int32_t n_checkpoints, int64_t *extra_steps,
                              int32_t *first_split);

/* Reverse sweep of the last sse_rk_record or sse_rk_record_binomial:
 * lam_0 <- (du(T)/du(0))^T lam_T, the gradient of J(u(T)) w.r.t. the
 * initial state when lam_T = dJ/du(T) (both N_p x N_c x N_e, host or
 * device).  Uniform recording: each checkpoint segment is recomputed once,
 * in the precision it was recorded in, storing its RK stage states; the
 * segment whose stage data is still held (the last one, after
 * sse_rk_record) is not recomputed.  Binomial recording: the schedule's
 * steps are recomputed from its checkpoints, one step's stage data at a
 * time.  The stage adjoints use sse_residual_vjp's kernels at the stage
 * states, in the recorded precision.  The recording stays valid for
 * further calls.  out_info, if not NULL, receives {segments (binomial:
 * checkpoint slots including the initial state), checkpoint_every
 * (binomial: -1), recording bytes, segments (binomial: forward steps)
 * recomputed by this call}.  The pullback half of the stepper's rrule; no
 * counterpart in the reference. */
int32_t sse_rk_adjoint(sse_solver *s, const double *lam_T, double *lam_0, double *out_info,
                       int32_t memory);

/* sse_rk_steps with the snapshot hook of the reference's save_callback /
 * save_solution (File/save.jl:44-89): after every `every`-th step the state
 * is copied to snapshots[i] and, when residuals is not NULL, its residual
 * R(u) (the saved "du") to residuals[i], i = 0 .. n_steps/every - 1, each
 * N_p x N_c x N_e, in the memory kind of u (copies are ordered on the
 * handle's stream; the call returns after the last one).  The state at
 * snapshot i belongs to t0 + (i + 1) every dt. */
int32_t sse_rk_steps_snapshots(sse_solver *s, double *u, int32_t n_steps, double dt,
                               int32_t scheme, int32_t every, double *snapshots,
                               double *residuals, double *t, int32_t memory);

/* FP64 reductions of Analysis/conservation.jl:145-189 for one (u, dudt):
 * out[0..N_c-1] = sum_k 1' WJ V dudt[:, e, k]       (PrimaryConservationAnalysis)
 * out[N_c]      = sum_k (P w)' M dudt               (EntropyConservationAnalysis,
 *                 :177-189; P = M^-1 V' WJ, so this is w_q' WJ V dudt for any
 *                 mass solver; for linear advection w = u, the entropy u^2/2).
 * EnergyConservationAnalysis (:161-175, u' M dudt with the mass solver's own
 * mass matrix) is sse_energy_residual. */
int32_t sse_conservation_residual(sse_solver *s, const double *u, const double *dudt,
                                  double *out, int32_t memory);

/* EnergyConservationAnalysis residual (Analysis/conservation.jl:161-175):
 * out[e] = sum_k u[:, e, k]' M_k dudt[:, e, k], e = 0 .. N_c-1, with the mass
 * solver's own mass matrix (mass_matrix.jl:150-158): inv(V' diag(J^-1 W) V)
 * for WeightAdjustedSolver (applied through a Cholesky solve per element),
 * diag(W J) for DiagonalSolver.  FP64. */
int32_t sse_energy_residual(sse_solver *s, const double *u, const double *dudt, double *out,
                            int32_t memory);

/* SSE_FP64 (default, the drop-in) or SSE_MIXED (FP32 fluxes, operator
 * arithmetic and entropy-variable maps on perturbations from a constant
 * reference state; FP64 geometry, RK accumulation and reductions). */
int32_t sse_set_precision(sse_solver *s, int32_t precision);

/* Run this handle's work on the caller's CUDA stream (a cudaStream_t; NULL
 * selects the legacy default stream) instead of its own.  No counterpart in
 * the reference, which has no device. */
int32_t sse_set_stream(sse_solver *s, void *stream);

/* Average device time in milliseconds of each residual phase over n_iter
 * evaluations at the device state u_dev, timed with CUDA events on the
 * handle's stream: out[0] nodal values (phase A), out[1] time derivative
 * (phase B), out[2] one Runge-Kutta stage update.  On the one-kernel
 * StandardForm path out[0] is 0 and out[1] times that kernel.  No
 * counterpart in the reference; mirrors the "nodal values" / "time deriv."
 * TimerOutputs sections of Solvers.jl:474-489. */
int32_t sse_phase_timings(sse_solver *s, const double *u_dev, int32_t n_iter, double *out);

/* Which kernels evaluate the residual.  SSE_PATH_TWO_PHASE: phase A
 * (nodal_values!) then phase B (time_derivative!), the element nodal states
 * handed over through device memory.  SSE_PATH_ONE_KERNEL: StandardForm on
 * elements with at most 32 volume, facet and modal nodes, each face meeting
 * one neighbour element, with a weight-adjusted mass solver whose dense
 * per-element operators fit in device memory or a diagonal one: one kernel
 * per residual (and per Runge-Kutta stage in sse_rk_steps, with the stage
 * update applied by the same kernel), one warp per element, the facet traces
 * R V u evaluated from the modal coefficients of the element and of its
 * neighbours.  Handles start on the one-kernel path where it applies.
 * sse_residual_vjp, sse_nodal_values and the recordings of sse_rk_record /
 * sse_rk_record_binomial always take the two-phase kernels.  Both paths
 * restate the same reference algorithm; their results differ by round-off
 * (the traces are (R V) u instead of R (V u), and the contracted fluxes are
 * summed before the D_m^T product).  No counterpart in the reference. */
enum sse_kernel_path_kind { SSE_PATH_TWO_PHASE = 0, SSE_PATH_ONE_KERNEL = 1 };
/* returns SSE_PATH_TWO_PHASE or SSE_PATH_ONE_KERNEL (negative: error) */
int32_t sse_kernel_path(const sse_solver *s);
/* SSE_ERR_UNSUPPORTED when SSE_PATH_ONE_KERNEL is asked for a configuration
 * outside its scope; the handle's path is then unchanged. */
int32_t sse_set_kernel_path(sse_solver *s, int32_t path);

/* ---- Geometric factors on the device -------------------------------------
 *
 * Drop-in for the constructor GeometricFactors(mesh, reference_element,
 * metric_type) (src/SpatialDiscretizations/mesh.jl:229-282 ExactMetrics,
 * :284-339 ConservativeCurlMetrics on Tri, :410-506 on Tet) followed by
 * project_jacobian! (SpatialDiscretizations.jl:310-317), which
 * SpatialDiscretization(...) calls (SpatialDiscretizations.jl:333-392).  All
 * arithmetic is FP64; each element's metric terms come from its own
 * mapping-node coordinates, one CTA per element. */
enum sse_metrics { SSE_EXACT_METRICS = 0, SSE_CONSERVATIVE_CURL_METRICS = 1 };

/* Reference-element matrices, column-major (Julia Matrix{Float64}). */
typedef struct sse_metric_operators {
  int32_t d;                /* 2 (Tri) or 3 (Tet) */
  int32_t metrics;          /* enum sse_metrics (ChanWilcoxMetrics = curl) */
  int32_t n_map;            /* mapping nodes per element: size(mesh.xyz[1], 1) */
  int32_t n_q;              /* size(reference_element.Vq, 1) */
  int32_t n_f;              /* size(reference_element.Vf, 1) */
  int32_t num_faces;        /* 3 (Tri) or 4 (Tet) */
  int32_t n_curl;           /* Tet curl: nodes of the degree N+1 basis; else 0 */
  int32_t project_jacobian; /* 1: J_q <- project J_q (exact metrics only) */
  const double *Drst[3];    /* reference_element.Dr, Ds, Dt: n_map x n_map */
  const double *Vq;         /* reference_element.Vq: n_q x n_map */
  const double *Vf;         /* reference_element.Vf: n_f x n_map */
  const double *nrstJ[3];   /* reference_element.nrstJ: n_f each */
  /* Tet with ConservativeCurlMetrics (mesh.jl:410-464) */
  const double *N_to_Nplus1;     /* n_curl x n_map */
  const double *Drst_Nplus1[3];  /* Vr_Nplus1 / V_Nplus1, ...: n_curl x n_curl */
  const double *Vq_Nplus1;       /* reference_element.Vq * Nplus1_to_N: n_q x n_curl */
  const double *Vf_Nplus1;       /* reference_element.Vf * Nplus1_to_N: n_f x n_curl */
  /* project_jacobian!: VDM inv(VDM' W VDM) VDM' W, n_q x n_q */
  const double *project;
} sse_metric_operators;

/* GeometricFactors fields (SpatialDiscretizations.jl:283-289), written in
 * the reference's layouts. */
typedef struct sse_geometric_factors_out {
  double *J_q;      /* n_q x N_e */
  double *Lambda_q; /* n_q x d x d x N_e : Λ_q[i, m, n, k] = J ∂ξ_m/∂x_n */
  double *J_f;      /* n_f x N_e */
  double *nJf;      /* d x n_f x N_e */
  double *nJq;      /* d x num_faces x n_q x N_e */
} sse_geometric_factors_out;

/* Compute the geometric factors of n_e elements from the mapping-node
 * coordinates xyz[m] (mesh.xyz[m], n_map x n_e each).  memory = SSE_HOST:
 * xyz and the outputs are host arrays (staged through temporary device
 * buffers); SSE_DEVICE: all are device pointers.  The operator matrices are
 * host arrays in both cases.  Errors leave their message for
 * sse_create_error(). */
int32_t sse_geometric_factors(const sse_metric_operators *ops, int64_t n_e,
                              const double *const *xyz,
                              const sse_geometric_factors_out *out, int32_t memory);

/* ---- L2 projection of initial data ---------------------------------------
 *
 * project_function (src/Solvers/Solvers.jl:396-418) behind initialize
 * (Solvers.jl:421-427) for a modal basis: for every element
 *   u0[:, :, k] = M_k \ (VDM' diag(W .* J_q[:, k]) u_q[:, :, k]),
 *   M_k = VDM' diag(W .* J_q[:, k]) VDM,
 * with M_k factorised by Cholesky as the reference does (a non-SPD M_k is an
 * error, SSE_ERR_NONPHYSICAL).  VDM is Matrix(V) (n_q x n_p), W the volume
 * weights (n_q), J_q (n_q x n_e), u_q the initial data at the volume nodes
 * (n_q x n_c x n_e, the layout of evaluate(initial_data, xyzq, 0)), u0 the
 * modal coefficients (n_p x n_c x n_e).  memory = SSE_HOST: J_q, u_q, u0 are
 * host arrays; SSE_DEVICE: device pointers.  VDM and W are host arrays in both
 * cases.  FP64, one CTA per element; errors leave their message for
 * sse_create_error(). */
int32_t sse_project_function(int32_t n_p, int32_t n_q, int32_t n_c, int64_t n_e,
                             const double *VDM, const double *W, const double *J_q,
                             const double *u_q, double *u0, int32_t memory);

/* Measured FMA throughput of the current device in TFLOP/s (2 flops per
 * FMA): out[0] FP64, out[1] FP32 CUDA-core pipes.  The roofline
 * denominators of the residual kernels; no counterpart in the reference. */
int32_t sse_measure_fma_peaks(double *out);

/* sizeof(sse_config), sizeof(sse_csc), sizeof(sse_operators),
 * sizeof(sse_geometry), sizeof(sse_metric_operators),
 * sizeof(sse_geometric_factors_out) into out[0..5], for checking foreign
 * bindings; returns the count. */
int32_t sse_struct_sizes(int32_t *out);

/* Message of the last failing call on this handle ("" if none). */
const char *sse_last_error(const sse_solver *s);
/* Message of the last failing sse_create (no handle exists then). */
const char *sse_create_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SSE_GB300_H */
