/*
 * trixiatmo_gpu.h — C ABI of libtrixiatmo_gpu.so, the GB300 (sm_103a) DGSEM
 * right-hand side and Runge-Kutta stage engine that stands in for Trixi.jl's
 * `rhs!` as TrixiAtmo.jl drives it.
 *
 * All entry points are `extern "C"`, take plain pointers and sizes and return
 * an int status (TAG_OK = 0).  Arrays cross the boundary in Julia's
 * column-major layout (first index fastest), exactly as Trixi stores them:
 *   u, du                  u[v, i, j, element]            (Trixi `wrap_array(u_ode, semi)`)
 *   contravariant_vectors  [component, direction, i, j, element]
 *   inverse_jacobian       [i, j, element]
 *   node_coordinates       [component, i, j, element]
 *   derivative_split       [i, ii]  (dg.basis.derivative_split)
 *   weights                [i]      (dg.basis.weights)
 * Element, face and interface indices are 0-based.  Faces: 0 = xi-, 1 = xi+,
 * 2 = eta-, 3 = eta+ (Trixi directions 1..4) and, in 3D, 4 = zeta-, 5 = zeta+.
 * 3D arrays: u[v, i, j, k, element], contravariant_vectors[c, d, i, j, k, element],
 * inverse_jacobian[i, j, k, element]; face-local node indices (l1, l2) are
 * (j, k), (i, k), (i, j) on xi, eta, zeta faces.
 *
 * Interface orientation (interface_flip): 2D — 1 if the secondary face's node
 * order runs backward.  3D — a code o in 0..7 mapping the primary's (l1, l2)
 * to the secondary's (s1, s2): swap the two when o & 1, then s1 = n-1-s1 when
 * o & 2 and s2 = n-1-s2 when o & 4 (covers every face-to-face orientation of a
 * conforming hexahedral mesh such as the cubed-sphere shell).
 *
 * Ownership: the caller owns every host array and keeps it alive for the
 * duration of the call (Julia: GC.@preserve).  The library copies what it
 * needs to device memory in tag_create and owns all device buffers.
 * Threading: one host thread per handle; work is ordered on the handle's own
 * CUDA stream; calls on one handle are not re-entrant.
 */
#ifndef TRIXIATMO_GPU_H
#define TRIXIATMO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TAG_OK 0
#define TAG_E_INVALID 1        /* bad argument / unsupported configuration     */
#define TAG_E_CUDA 2           /* a CUDA runtime call failed                   */
#define TAG_E_NO_DEVICE 3      /* no CUDA device visible                       */
#define TAG_E_STATE 4          /* device status word has an error bit set      */
#define TAG_E_IO 5             /* a file could not be written                  */

/* ---- device status word bits (tag_status) ------------------------------ */
#define TAG_S_NAN 0x1u         /* non-finite value met in a kernel             */
#define TAG_S_NEG_DENSITY 0x2u /* rho <= 0 met                                 */
#define TAG_S_NEG_PRESSURE 0x4u/* p <= 0 met                                   */
#define TAG_S_NEWTON_MAXIT 0x8u/* Newton limiter hit max_iterations (warning)  */

/* ---- equation systems, fluxes, boundary kinds --------------------------- */
#define TAG_EQ_EULER_ENERGY_2D 1 /* CompressibleEulerEnergyEquationsWithGravity2D */
#define TAG_EQ_EULER_ENERGY_3D 2 /* CompressibleEulerEnergyEquationsWithGravity3D + source_terms_coriolis */
#define TAG_EQ_RAINY_2D 3        /* CompressibleRainyEulerEquations2D (+ Newton stage limiter) */
#define TAG_EQ_MOIST_EULER_2D 4  /* CompressibleMoistEulerEquations2D                             */
#define TAG_EQ_COVARIANT_SWE 5   /* (Split)CovariantShallowWaterEquations2D on a 2D manifold     */
#define TAG_EQ_POTENTIAL_TEMPERATURE_2D 6 /* CompressibleEulerPotentialTemperatureEquationsWithGravity2D */
#define TAG_EQ_POTENTIAL_TEMPERATURE_3D 7 /* CompressibleEulerPotentialTemperatureEquationsWithGravity3D + source_terms_coriolis */
#define TAG_EQ_INTERNAL_ENERGY_2D 8 /* CompressibleEulerInternalEnergyEquationsWithGravity2D */

#define TAG_VF_RANOCHA_WARUSZEWSKI 1 /* (flux_ranocha, flux_nonconservative_waruszewski_etal) */
#define TAG_VF_EC_RAIN 2             /* VolumeIntegralFluxDifferencing(flux_ec_rain)    */
#define TAG_VF_WEAK_FORM 3           /* VolumeIntegralWeakForm (physical flux)          */
#define TAG_VF_CHANDRASHEKAR 4       /* VolumeIntegralFluxDifferencing(flux_chandrashekar), moist */
#define TAG_VF_COV_CENTRAL 5         /* covariant: flux differencing with flux_central  */
#define TAG_VF_COV_EC 6              /* covariant: flux differencing with flux_ec (split form) */
#define TAG_VF_PT_TEC 7              /* potential temperature: (flux_tec, nonconservative gravity term) */
#define TAG_VF_PT_EC 8               /* potential temperature: (flux_ec, nonconservative gravity term)  */
#define TAG_VF_PT_ETEC 9             /* potential temperature: (flux_etec, nonconservative gravity term) */
#define TAG_VF_IE_ETEC 10            /* internal energy: (flux_conservative_etec, flux_nonconservative_etec) */
#define TAG_VF_PT_KG 11              /* potential temperature 3D: (flux_kennedy_gruber, a nonconservative gravity term) */
#define TAG_SF_LMARS 1               /* (FluxLMARS(c), flux_zero)                       */
#define TAG_SF_LAX_FRIEDRICHS 2      /* flux_lax_friedrichs (max_abs_speed_naive)       */
#define TAG_SF_CHANDRASHEKAR 3       /* flux_chandrashekar as surface flux (moist)      */
#define TAG_SF_COV_EC 4              /* covariant: flux_ec                              */
#define TAG_SF_COV_EC_LLF 5          /* covariant: FluxPlusDissipation(flux_ec, DissipationLocalLaxFriedrichs()) */
#define TAG_SF_COV_CENTRAL 6         /* covariant: flux_central (no dissipation)        */
#define TAG_SF_IE_ES 7               /* internal energy: (flux_conservative_es, flux_nonconservative_es) */
#define TAG_SF_PT_EC 8               /* potential temperature 2D: (flux_ec, params[7]: 0 flux_zero,
                                        1 waruszewski, 2 artiano, 3 souza gravity term) */

#define TAG_SRC_RAINY 1              /* source_terms_rainy (microphysics + gravity)     */
#define TAG_SRC_RAINY_CONVERGENCE 2  /* manufactured source of the rainy convergence test */
#define TAG_SRC_GEOPOTENTIAL 3       /* source_terms_geopotential (moist)               */
#define TAG_SRC_MOIST_BUBBLE 4       /* source_terms_moist_bubble: geopotential + phase change */
#define TAG_SRC_MOIST_CONVERGENCE_DRY 5 /* source_terms_convergence_test_dry (moist equations) */
#define TAG_SRC_MOIST_CONVERGENCE 6  /* source_terms_convergence_test_moist            */
#define TAG_SRC_MOIST_GRAVITY_WAVE 7 /* geopotential + phase change +
                                        source_terms_nonhydrostatic_rayleigh_sponge     */
#define TAG_SRC_RAINY_NO_PHASE_CHANGE 8 /* source_terms_no_phase_change (rainy: gravity only) */
#define TAG_SRC_MOUNTAIN_WAVE 9      /* MountainWaveSetup as source terms (potential temperature
                                        2D), set by tag_set_source                          */

#define TAG_BC_SLIP_WALL_STRUCTURED 1 /* boundary_condition_slip_wall reached from a StructuredMesh */
#define TAG_BC_SLIP_WALL_NORMAL 2     /* boundary_condition_slip_wall reached from a P4estMesh      */
#define TAG_BC_SIMPLE_SLIP_WALL 3     /* boundary_condition_simple_slip_wall (rainy, StructuredMesh) */
#define TAG_BC_DIRICHLET 4            /* BoundaryConditionDirichlet reached from a P4estMesh: the
                                         surface flux of the inner and a given state, the states
                                         set by tag_set_boundary_values (2D equations)          */

typedef struct tag_handle_s* tag_handle;

/* Semidiscretization description: what Trixi's `SemidiscretizationHyperbolic`
 * holds in (equations, solver, cache) for this path. */
typedef struct {
  int32_t equations;      /* TAG_EQ_*                                         */
  int32_t volume_flux;    /* TAG_VF_*                                         */
  int32_t surface_flux;   /* TAG_SF_*                                         */
  int32_t polydeg;        /* N; nodes per direction n = N + 1                 */
  int32_t nelements;
  int32_t ninterfaces;
  int32_t nboundaries;    /* boundary faces                                   */
  int32_t nmembers;       /* ensemble members (0 or 1: a single mesh)         */
  const double* derivative_split;      /* [n, n]                               */
  const double* weights;               /* [n]                                  */
  const double* contravariant_vectors; /* [2, 2, n, n, E]                      */
  const double* inverse_jacobian;      /* [n, n, E]                            */
  const double* node_coordinates;      /* [2, n, n, E]                         */
  const int32_t* interface_elements;   /* [2, I]: primary, secondary element   */
  const int32_t* interface_faces;      /* [2, I]: primary, secondary face      */
  const int32_t* interface_flip;       /* [I]: 1 if the secondary face runs backward */
  const int32_t* boundary_elements;    /* [B]                                  */
  const int32_t* boundary_faces;       /* [B]                                  */
  const int32_t* boundary_kinds;       /* [B]: TAG_BC_*                        */
  const int32_t* element_member;       /* [E]: ensemble member of each element
                                          (null when nmembers <= 1).  Members are
                                          independent meshes (no interface joins
                                          two members); each has its own t, dt and
                                          CFL reduction.                         */
  double params[8];  /* EULER_ENERGY_2D: c_p, c_v, gravity, LMARS speed of sound;
                        EULER_ENERGY_3D: the same, then the Coriolis angular
                        velocity (0 disables the source);
                        RAINY_2D: params[0] = TAG_SRC_* source kind (surface flux
                        TAG_SF_LAX_FRIEDRICHS or TAG_SF_LMARS = flux_LMARS, c = 360);
                        MOIST_EULER_2D: c_pd, c_vd, c_pv, c_vv, gravity, LMARS
                        speed of sound, TAG_SRC_* source kind (0: none);
                        POTENTIAL_TEMPERATURE_2D: c_p, c_v, gravity, LMARS speed
                        of sound, nonconservative gravity term (0
                        flux_nonconservative_waruszewski_etal, 1 _artiano_etal,
                        2 _souza_etal);
                        COVARIANT_SWE: gravity, rotation rate, split form (0/1),
                        volume nonconservative flux (0 none, 1
                        flux_nonconservative_ec), surface nonconservative flux
                        (0 none, 1 flux_nonconservative_ec, 2
                        flux_nonconservative_surface_simplified); the surface
                        flux TAG_SF_LAX_FRIEDRICHS is flux_central + local
                        Lax-Friedrichs dissipation; source_terms_geometric_coriolis
                        is always applied */
  const double* aux_node_vars;  /* COVARIANT_SWE: [26, n, n, E], the reference's
                                   cache.auxiliary_variables.aux_node_vars
                                   (src/equations/equations.jl:139-215);
                                   node_coordinates is then [3, n, n, E];
                                   contravariant_vectors / inverse_jacobian are
                                   not used */
} tag_config;

/* Creates a handle on the current CUDA device.  Replaces the cache build of
 * Trixi.SemidiscretizationHyperbolic (reference: src/semidiscretization/
 * semidiscretization_hyperbolic_2d_manifold_in_3d.jl:78-111, create_cache in
 * src/solvers/dgsem_p4est/dg.jl:5-32): geometry and connectivity are uploaded once. */
int tag_create(const tag_config* cfg, tag_handle* out);

/* One handle for many independent members (COVARIANT_SWE), each its own mesh,
 * polynomial degree, geometry and initial state: an uneven ensemble.  The
 * solution is the members' u concatenated in the given order; each member has
 * its own t, dt and CFL reduction; every stage is one interface launch and one
 * element launch over all members (elements grouped by degree).  No counterpart
 * in the reference, which runs one semidiscretization per process. */
int tag_create_ensemble(const tag_config* members, int32_t nmembers, tag_handle* out);
int tag_destroy(tag_handle h);

/* Number of solution entries nv * n^2 * E (length of Trixi's u_ode). */
int64_t tag_ndofs_total(tag_handle h);

/* du = rhs(u, t): Trixi.rhs_hyperbolic!(du_ode, u_ode, semi, t) as called by
 * test/test_2d_rainy_euler.jl:38 and overridden in
 * src/solvers/dgsem_p4est/dg_2d_manifold_in_3d_covariant.jl:8-71.
 * u and du are host pointers when on_device == 0, device pointers otherwise. */
int tag_rhs(tag_handle h, const double* u, double* du, double t, int32_t on_device);

/* Load / read back the handle's resident solution (the ODE state u_ode). */
int tag_set_state(tag_handle h, const double* u_host);
int tag_get_state(tag_handle h, double* u_host);
/* Device pointer of the resident state (for callers that keep data on the GPU). */
int tag_state_device_ptr(tag_handle h, double** u_dev);

/* Trixi.max_dt(u, t, mesh, constant_speed = False(), equations, dg, cache) on
 * the resident state (the minimum over members for an ensemble); reference
 * pattern src/callbacks_step/stepsize_dg2d.jl:5-44. */
int tag_max_dt(tag_handle h, double* out);

/* Advances the resident state by `nsteps` steps of the handle's time
 * integrator (CarpenterKennedy2N54 unless tag_set_time_integrator chose an
 * SSP scheme).  With
 * fixed_dt > 0 every step uses it, otherwise dt = cfl * max_dt(u) before each
 * step (StepsizeCallback), per ensemble member.  t points to nmembers doubles
 * (one when there is a single mesh): the members' times, read and updated.
 * Each step is one CUDA-graph replay of a dt kernel and one
 * (interface kernel + element kernel) pair per stage (5, 4 or 3 stages). */
int tag_rk_steps(tag_handle h, int32_t nsteps, double cfl, double fixed_dt, double* t);

typedef struct tag_adaptive_stats {
  int64_t accepted;  /* steps taken                                   */
  int64_t rejected;  /* steps repeated with a smaller dt               */
  double dt_first;   /* the initial step size                          */
  double dt_last;    /* the last accepted step (shortened at t_end)    */
} tag_adaptive_stats;

/* Error-controlled SSPRK43 from *t to t_end on a single mesh: what the
 * reference's elixirs get from `solve(ode, SSPRK43(); abstol, reltol,
 * callback = ...)` without a StepsizeCallback (e.g.
 * examples/euler/dry_air/mountain_flow/elixir_potential_temperature_linear_hydrostatic.jl:83-86,
 * examples/euler/dry_air/global_circulation/elixir_potential_temperature_baroclinic_instability.jl:62-66;
 * OrdinaryDiffEq's integrator, an external dependency).  The handle's scheme
 * must be SSPRK43 (tag_set_time_integrator).  Each step runs the four stages
 * on the device (and the stage limiter after each, for the rainy equations)
 * and one error kernel; the error estimate is the difference to the embedded
 * second-order solution with weights (1/4, 1/4, 1/4, 1/4), in the
 * root-mean-square norm of e / (abstol + max(|u_prev|, |u_new|) reltol) over
 * every state entry.  The step size follows the PI controller with beta1 =
 * 7/30, beta2 = 2/15, gamma = 0.9, qmin = 0.2, qmax = 10 (a rejected step is
 * repeated from its starting state); the first step follows Hairer, Norsett
 * and Wanner's starting-step algorithm.  A step never passes the next of the
 * increasing `stops` (the times of a SaveSolutionCallback(dt)) or t_end.
 * *t is updated to the time reached; TAG_E_INVALID after max_steps attempts. */
int tag_rk_adaptive(tag_handle h, double* t, double t_end, double abstol, double reltol,
                    const double* stops, int32_t nstops, int64_t max_steps,
                    tag_adaptive_stats* stats);

/* Time integrator of tag_rk_steps.  The reference picks it by the algorithm
 * passed to `solve(ode, alg; dt, callback = StepsizeCallback(cfl))`:
 *   TAG_RK_CK2N54   CarpenterKennedy2N54(williamson_condition = false), the default
 *                   (e.g. examples/euler/moist_air/buoyancy/elixir_gemein_bubble.jl)
 *   TAG_RK_SSPRK43  SSPRK43() with the step size of the StepsizeCallback,
 *                   adaptive = false (examples/euler/dry_air/buoyancy/
 *                   elixir_energy_inertia_gravity_waves.jl,
 *                   elixir_potential_temperature_inertia_gravity_waves.jl)
 *   TAG_RK_SSPRK33  SSPRK33() (elixir_gemein_nonhydrostatic_gravity_waves.jl)
 * Applies to the following tag_rk_steps calls (the captured step graph is
 * rebuilt); stage limiters run after every stage of any scheme. */
#define TAG_RK_CK2N54 0
#define TAG_RK_SSPRK43 1
#define TAG_RK_SSPRK33 2
int tag_set_time_integrator(tag_handle h, int32_t scheme);

/* States [B, n, nv] of the boundary faces of kind TAG_BC_DIRICHLET (entries of
 * other faces are ignored): the values of Trixi's
 * BoundaryConditionDirichlet(boundary_value_function) at the face nodes
 * (reference: BoundaryConditionDirichlet(setup) in
 * examples/euler/dry_air/mountain_flow/elixir_potential_temperature_linear_hydrostatic.jl:26-31).
 * Required before the first rhs or step of a mesh with such faces; the states
 * may be replaced between steps (time-dependent data). */
int tag_set_boundary_values(tag_handle h, const double* values);

/* Source terms that need more constants than tag_config.params holds:
 *   POTENTIAL_TEMPERATURE_2D, TAG_SRC_MOUNTAIN_WAVE, 8 params (theta_0, u0,
 *   Brunt-Vaisala frequency, z_damping_start, z_damping_end, x_damping_start,
 *   x_damping_end, damping_rate): MountainWaveSetup passed as source_terms
 *   (src/equations/initial_condition_compressible_euler_2d.jl:174-200). */
int tag_set_source(tag_handle h, int32_t kind, const double* params, int32_t nparams);

/* ---- analysis of the resident state (AnalysisCallback) ------------------ */
/* Integrals over each member's domain, computed on the device in a fixed
 * summation order (repeated calls return the same bits):
 *   TAG_AQ_STATE          every conserved variable (nv values; the basis of
 *                         :conservation_error, Trixi `integrate(u_ode, semi)`)
 *   TAG_AQ_ENTROPY        the equations' `entropy` (extra_analysis_integrals =
 *                         (entropy,)); not defined for the rainy equations
 *   TAG_AQ_ENERGY_TOTAL   `energy_total` (energy, moist and potential-
 *                         temperature equations)
 *   TAG_AQ_ENTROPY_TIMEDERIVATIVE  the integral of cons2entropy(u) . du/dt with
 *                         du/dt = rhs(u, t) evaluated on the device (the
 *                         AnalysisCallback's default `entropy_timederivative`)
 * Quadrature: LGL weights times |J| (Cartesian meshes: 1/inverse_jacobian;
 * covariant equations: the area element of aux_node_vars, reference
 * src/callbacks_step/analysis_covariant.jl:53-105).  out: nmembers x values
 * doubles, divided by the member's volume when normalize != 0 (Trixi's
 * default).  Members of an ensemble must occupy contiguous element ranges. */
#define TAG_AQ_STATE 0
#define TAG_AQ_ENTROPY 1
#define TAG_AQ_ENERGY_TOTAL 2
#define TAG_AQ_ENTROPY_TIMEDERIVATIVE 3
int tag_analyze_integral(tag_handle h, int32_t quantity, int32_t normalize, double t, double* out);

/* Analysis nodes for tag_analyze_errors.  Cartesian meshes: *m = 2N + 1
 * nodes per direction (the LGL nodes of degree 2N, Trixi's default analysis
 * polydeg); x (may be null) receives their coordinates [E][m^d][d],
 * interpolated from node_coordinates (which tag_create must have been given).
 * Covariant equations: *m = 0, the analysis nodes are the solution nodes and
 * x receives their Cartesian coordinates [nodes][3]. */
int tag_analysis_nodes(tag_handle h, int32_t* m, double* x);

/* l2 and linf errors of the resident state against u_exact (host array, the
 * caller's initial_condition(x, t) at the analysis nodes: [E][m^d][nv] on
 * Cartesian meshes, [nodes][nv] for covariant equations in the contravariant
 * components).  l2 = sqrt(sum wJ d^2 / sum wJ), linf = max |d| per variable,
 * d = u_exact - u, with the solution and J interpolated to the analysis nodes
 * on Cartesian meshes (Trixi's calc_error_norms; covariant
 * src/callbacks_step/analysis_covariant.jl:143-189).  l2, linf: nmembers x nv. */
int tag_analyze_errors(tag_handle h, const double* u_exact, double* l2, double* linf);

/* Covariant metric terms of a cubed-sphere mesh, computed on the device
 * (the reference's cache construction, init_auxiliary_node_variables!,
 * src/solvers/dgsem_p4est/containers_2d_manifold_in_3d_covariant.jl:232-489,
 * with the element-local mapping of src/meshes/p4est_cubed_sphere.jl).
 * vertices [E][4][3]: each element's corners (counter-clockwise, outward
 * normal); nodes [n]: dg.basis.nodes; derivative_matrix [n, n] column-major
 * (dg.basis.derivative_matrix, needed when collocation != 0).  spherical != 0:
 * GlobalSphericalCoordinates, else GlobalCartesianCoordinates; collocation
 * != 0: ChristoffelSymbolsCollocationDerivative, else the exact derivatives
 * (ChristoffelSymbolsAutodiff).  Outputs (host): aux [E][n][n][26] in the
 * aux_node_vars order with the bottom topography (slot 19) set to 0 for the
 * caller to fill, and the node coordinates xyz [E][n][n][3].  Returns
 * TAG_E_INVALID when a metric term is not finite (spherical components at a
 * pole). */
int tag_cov_metric_terms(const double* vertices, int32_t nelements, int32_t polydeg, double radius,
                         int32_t spherical, int32_t collocation, const double* nodes,
                         const double* derivative_matrix, double* aux, double* xyz);

/* Legendre-Gauss-Lobatto nodes and weights of degree polydeg on [-1, 1]
 * (Trixi's LobattoLegendreBasis(polydeg).nodes / .weights); host only. */
int tag_lgl_basis(int32_t polydeg, double* nodes, double* weights);

/* Per-member max_dt of the resident state (out: nmembers doubles). */
int tag_max_dt_members(tag_handle h, double* out);

/* Times `reps` launches of each stage kernel on the handle's stream with CUDA
 * events (after a warm-up) and returns the mean milliseconds per launch of the
 * interface kernel and of the element kernel (stage mode). The resident state
 * is advanced by the timed stages. */
int tag_time_kernels(tag_handle h, int32_t reps, double* ms_interface, double* ms_element);

/* ---- rainy Euler: saturation Newton solve (stage limiter) ---------------- */
/* Settings of the Newton stage limiter that tag_rk_steps applies after every
 * stage of a TAG_EQ_RAINY_2D handle (reference: NonlinearSolveDG,
 * src/callbacks_stage/nonlinear_solve_dg.jl:18-44; defaults tolerance 1e-9,
 * max_iterations 20).  mode 0: the reference's criterion max|residual| < tol;
 * mode 1: relative, |res_1| < tol |E_internal| and |res_2|, |res_3| <=
 * tol 1e7 rho_moist.  polish (canonical finish, not in the reference; 0 = off):
 * a converged iterate is snapped to a grid fixed by the node's state (vapour
 * and cloud to 2^-24 of the power of two above rho_moist, temperature to
 * 2^-18 K) and this many Newton updates are taken from there, so that solves
 * converged from different starts return the same bits. */
int tag_set_newton(tag_handle h, int32_t mode, double tol, int32_t max_iterations,
                   int32_t polish);

/* Start of the Newton solve inside tag_rk_steps' stage limiter (no counterpart
 * in the reference, whose NonlinearSolveDG always starts from the previous
 * values of slots 7-9): 0 that warm start (default); 1 the learned guess (the
 * closed-form unsaturated equilibrium where it is valid, else the MLP set by
 * tag_set_mlp); 2 the closed-form branch alone, with the warm start on
 * saturated nodes; 3 the closed-form branch, and on saturated nodes whichever
 * of the MLP guess and the warm start has the smaller residual (needs
 * tag_set_mlp).  A guessed start not converged after 8 updates falls back
 * to the warm start; with the canonical finish (tag_set_newton polish = 1) all
 * four starts give the same bits. */
int tag_set_newton_start(tag_handle h, int32_t start);

/* Newton work of the stage limiter summed over tag_rk_steps calls:
 * out[0] updates, out[1] fallbacks to the warm start, out[2] node solves that
 * missed the tolerance, out[3] node solves (nodes x stages); reset != 0 zeroes
 * the sums after reading. */
int tag_newton_counters(tag_handle h, int64_t* out, int32_t reset);

typedef struct {
  int64_t nodes;            /* nodes solved                                    */
  int64_t updates;          /* Newton updates until convergence, summed        */
  int64_t fallbacks;        /* learned guesses that failed within 8 updates    */
  int64_t not_converged;    /* nodes that never met the tolerance              */
} tag_newton_stats;

/* One Newton solve of the saturation system on every node of the resident
 * state (the stage limiter's work once, nonlinear_solve_dg2d.jl:6-44).
 * use_learned 1 starts from the learned guess, 2 from its closed-form branch
 * alone (the warm start on saturated nodes), 3 from the closed-form branch and
 * on saturated nodes from the smaller-residual one of the MLP guess and the
 * warm start; all three fall back to the warm
 * start (slots 7-9) when not converged after 8 updates; 0 starts warm.  The learned
 * guess is the closed-form unsaturated equilibrium T_unsat = (e_int - rho_m L)
 * / (c_vd rho_d + c_vv rho_m + c_l rho_r) where e_s(T_unsat)/(R_v T_unsat) >=
 * rho_m (exact there), else T_unsat plus the offset predicted by the MLP set
 * with tag_set_mlp (inputs rho_d, rho_m, rho_r, e_int, T_unsat).
 * iters (host, may be null): per-node update counts. */
int tag_newton_solve(tag_handle h, int32_t use_learned, int32_t* iters, tag_newton_stats* stats);

/* The same solve on n host states u[n][9] (slots 7-9 updated in place); mlp
 * (host, 1293 floats, may be null) selects the learned initial guess. */
int tag_newton_solve_states(double* u, int64_t n, int32_t mode, double tol, int32_t max_iterations,
                            int32_t polish, const float* mlp, int32_t* iters,
                            tag_newton_stats* stats);

/* Uploads the FP32 MLP parameters (1293 floats: W1[32][5], b1[32], W2[32][32],
 * b2[32], W3[32], b3, in_mean[5], in_scale[5], out_mean, out_scale). */
int tag_set_mlp(tag_handle h, const float* params);

/* MLP utilities on the current device (host arrays): forward pass; mean
 * squared error of the normalised output and its gradient w.r.t. the 1281
 * trainable parameters; Adam training over shuffled mini-batches. */
int tag_mlp_forward(const float* params, const float* x, int64_t n, float* y);
int tag_mlp_loss_grad(const float* params, const float* x, const float* t, int64_t n,
                      float* grad, float* loss);
int tag_mlp_train(float* params, const float* x, const float* t, int64_t n, int32_t epochs,
                  int32_t batch, float lr, uint64_t seed, float* loss_per_epoch);

/* Reads (and clears when clear != 0) the device status word (TAG_S_* bits). */
int tag_status(tag_handle h, uint32_t* flags, int32_t clear);

/* The handle's CUDA stream (cudaStream_t as void*), for callers that order
 * their own work against the library's. */
void* tag_stream(tag_handle h);

/* Tuning knob: elements per CTA of the element kernel (0 = autotune).  The
 * autotuner, run on the first step or rhs call, times the element kernel for
 * elements per CTA in {1, 2, 3, 4, 6, 8, 12, 16} (the shared-memory tile: each
 * element's state, metric terms and accumulators staged once) and, for each,
 * one or two work items per thread and phase (the CTA width), and keeps the
 * fastest; setting a value here fixes the tile with one item per thread. */
int tag_set_elements_per_block(tag_handle h, int32_t epb);
int tag_get_elements_per_block(tag_handle h, int32_t* epb);
/* Fixes the tile: epb elements per CTA, 1 or 2 work items per thread and phase. */
int tag_set_tile(tag_handle h, int32_t epb, int32_t items_per_thread);
/* Threads per CTA of the element kernel for the current tile (measurement). */
int tag_get_cta_threads(tag_handle h, int32_t* threads);

/* Geometry of the cubed-sphere shell built on the device: what TrixiAtmo's
 * P4estMeshCubedSphereTopography(trees, layers, inner_radius, thickness;
 * polydeg) and Trixi's curved P4estMesh{3} cache hold
 * (src/meshes/p4est_cubed_sphere_topography.jl:596-670): node coordinates of
 * the equiangular cubed-sphere map, the contravariant vectors in the
 * invariant curl form (Kopriva 2006) from collocation derivatives, and the
 * inverse Jacobian.  nodes / derivative_matrix: the LGL basis (host);
 * ground_height (host, may be null): [E, n, n] heights of each element's
 * column nodes (j, i) above the sphere, spread over the column by Gal-Chen
 * (vertical 0) or Sleve(eta_H, s) (vertical 1).  Elements
 * e = cz + layers (cx + trees (cy + trees face)); outputs (host)
 * xyz[3, n, n, n, E], Ja[3, 3, n, n, n, E], invJ[n, n, n, E] column-major. */
int tag_shell_geometry(int32_t trees, int32_t layers, double inner_radius, double thickness,
                       int32_t polydeg, const double* nodes, const double* derivative_matrix,
                       const double* ground_height, int32_t vertical, double sleve_eta_h,
                       double sleve_s, double* xyz, double* Ja, double* invJ);

/* FP64 FMA throughput probe (FLOP/s, FMA = 2) on the current device; the
 * denominator of the FP64 roofline. */
int tag_fp64_peak(double* flops_per_s);

/* Diagnostics, no counterpart in the reference (whose ln_mean, inv_ln_mean
 * and stolarsky_mean come from Trixi, imported at src/TrixiAtmo.jl:37):
 * evaluates the device forms of those means on n host value pairs (x[q],
 * y[q]) in one kernel.  kind 0: the 2D kernels' pair form (six-coefficient
 * polynomials, logarithms beyond f2 = 1e-2); 1: the same with per-node
 * logarithms and the four-term form below f2 = 1e-4; 2: the 3D energy
 * kernel's halved form (polynomials up to f2 = 0.09); 3: the single means;
 * 4: the potential-temperature kernels' Stolarsky mean with gamma = cp / cv;
 * 5 and 6: the halved form of kind 2 with one mean's pair (x[q], y[q]) and
 * the other's (1, 1), so that the two means take different forms
 * (5: ln_mean of the pair in out1; 6: inv_ln_mean of the pair in out2).
 * out1 = ln_mean (kind 4: the Stolarsky mean), out2 = inv_ln_mean. */
int tag_eval_means(int32_t kind, int64_t n, double cp, double cv, const double* x,
                   const double* y, double* out1, double* out2);

/* tag_rhs_noalloc — no counterpart in the reference.
 * du = rhs(u) for TAG_EQ_EULER_ENERGY_2D (TAG_VF_RANOCHA_WARUSZEWSKI,
 * TAG_SF_LMARS) on one mesh, with no source terms and no time-dependent data,
 * for callers that cannot allocate device memory (a program whose device
 * memory belongs to an arena or pool it alone manages, a Julia GPU allocator
 * that owns every buffer).  It allocates nothing: the caller passes every
 * buffer it owns as DEVICE pointers — u, du and, inside cfg,
 * contravariant_vectors, inverse_jacobian and the interface / boundary arrays
 * (derivative_split and weights stay host pointers) — and the surface-flux
 * scratch comes from a fixed 8 MiB device array of the library, so
 * nelements * 4 * (polydeg + 1) * 4 must not exceed 1048576 (larger meshes
 * are rejected with TAG_E_INVALID).  Boundary faces must be slip walls
 * (TAG_BC_SLIP_WALL_STRUCTURED or TAG_BC_SLIP_WALL_NORMAL); any other kind,
 * TAG_BC_DIRICHLET included, is rejected with TAG_E_INVALID before a kernel
 * runs.  The first call on each device looks up that array's device address
 * (cudaGetSymbolAddress) with the device current and keeps it: make that first
 * call before any stream capture, call only under the device's primary
 * context (the CUDA runtime's), and not after cudaDeviceReset.  Every call on
 * a device shares the array and clears it first; calls whose kernels overlap
 * on the same GPU race on it.  Index arrays are not range-checked (they are
 * device memory).  Work runs on `stream` (a cudaStream_t, or null for the
 * default stream) and the call returns after it finished; *status (may be
 * null) receives the TAG_S_* bits of this call. */
int tag_rhs_noalloc(const tag_config* cfg, const double* u, double* du, void* stream,
                    uint32_t* status);

/* Registers (u_host) or clears (null) a state sink: while it is registered,
 * the last kernel of every tag_rk_steps step (the element kernel's last stage,
 * or for the rainy equations the Newton stage limiter after it) also stores
 * the step's new state into u_host, so that the copy to the host overlaps the
 * step's work; when tag_rk_steps returns, u_host holds what tag_get_state
 * would copy (every ensemble member, Trixi's layout).  u_host must be pinned
 * host memory mapped for the device (cudaHostAlloc / cudaHostRegister under
 * unified addressing) of tag_ndofs_total doubles; the caller keeps it alive
 * while registered.  tag_rk_adaptive, tag_rhs and the other entry points do
 * not write it.  TAG_E_INVALID for an unmapped pointer.  No counterpart in the
 * reference (Julia keeps u_ode on the host); the end-to-end path of a step
 * that returns its state. */
int tag_set_state_sink(tag_handle h, double* u_host);

/* ---- solution output (SaveSolutionCallback) ---------------------------- */
/* Trixi's `solution_variables` functions for tag_solution_variables. */
#define TAG_SOLVAR_CONS2CONS 0               /* the conservative variables, every equation system */
#define TAG_SOLVAR_CONS2PRIM 1               /* covariant SWE: (H, vcon1, vcon2)                 */
#define TAG_SOLVAR_CONTRAVARIANT2GLOBAL 2    /* covariant SWE: (h, h_v1, h_v2, h_v3)             */
#define TAG_SOLVAR_CONS2PRIM_AND_VORTICITY 3 /* covariant SWE: (H, v1, v2, v3, b, vorticity)     */

/* The solution variables of the handle's current state, computed on the
 * device, in the layout Trixi writes them: data[v * nnodes + q] is variable v
 * at node q = i + n (j + n element) (3D: i + n (j + n (k + n element))), so
 * that each row is `vec(data[v, .., :])` of the reference.  member selects
 * one member of an ensemble (0 .. nmembers-1; -1 = every element of the
 * handle).  *nvars and *nnodes receive the sizes; data may be null to query
 * them.  Replaces convert_variables (src/callbacks_step/
 * save_solution_covariant.jl:5-33 with cons2prim_and_vorticity :64-74 and
 * calc_vorticity_node :93-118; cons2prim / contravariant2global of
 * src/equations/covariant_shallow_water.jl:113-145); cons2cons is the
 * transposed state (save_solution_2d_manifold_in_3d_cartesian.jl:66-68). */
int tag_solution_variables(tag_handle h, int32_t solution_variables, int32_t member,
                           int32_t* nvars, int64_t* nnodes, double* data);

/* A scalar attribute of tag_h5_write. */
#define TAG_H5_INT64 0
#define TAG_H5_FLOAT64 1
#define TAG_H5_STRING 2
typedef struct tag_h5_attribute {
  const char* name;   /* at most 1024 bytes */
  int32_t type;       /* TAG_H5_INT64 (i), TAG_H5_FLOAT64 (d) or TAG_H5_STRING (s, UTF-8) */
  int64_t i;
  double d;
  const char* s;      /* at most 60000 bytes; null = "" */
} tag_h5_attribute;

/* A one-dimensional float64 dataset of tag_h5_write with an optional string
 * attribute "name" (the variable's name in Trixi's files). */
typedef struct tag_h5_dataset {
  const char* name;       /* link name in the root group: no '/', at most 1024 bytes */
  const double* data;     /* count doubles (host memory) */
  int64_t count;
  const char* var_name;   /* value of the "name" attribute, or null for none */
} tag_h5_dataset;

/* Writes an HDF5 file (clobbering `path`) whose root group holds the scalar
 * attributes and up to 256 datasets: the layout of Trixi's solution files
 * (src/callbacks_step/save_solution_2d_manifold_in_3d_cartesian.jl:72-116:
 * attributes ndims, equations, polydeg, n_vars, n_elements, mesh_type,
 * mesh_file, time, dt, timestep; datasets variables_1 .. variables_n with
 * their names), readable by any HDF5 library and so by Trixi2Vtk.  Host
 * only: no device work, no CUDA call.  Returns TAG_E_IO when the file cannot
 * be written. */
int tag_h5_write(const char* path, const tag_h5_attribute* attrs, int32_t nattrs,
                 const tag_h5_dataset* sets, int32_t nsets);

/* Last error message of this thread (static storage). */
const char* tag_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* TRIXIATMO_GPU_H */
