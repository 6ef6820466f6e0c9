/*
 * gbdycore: C ABI of the GB300 (sm_103a) dry dynamical-core IMEX step.
 *
 * The library replaces the hot path of ClimaAtmos.jl's dry dynamical core:
 * the hooks that ClimaTimeSteppers calls through the ClimaODEFunction built in
 * src/simulation/integrator.jl:189-225, plus a fused, graph-captured ARS343
 * step.  Every entry point returns GB_OK (0) or a negative gb_status; no C++
 * exception crosses the ABI.  Device work is queued on the context's stream
 * (gb_set_stream) and is asynchronous unless stated otherwise.  A context is
 * not thread-safe (one host thread drives it, as in the reference).
 *
 * State layout (a FieldVector with fields c and f, precision set by
 * gb_config.ft_bytes; ClimaCore's VIJFH order with Nq = 4, i fastest in a slab):
 *   c : [Nh][4][16][Nv]   components (rho, u_1, u_2, rho e_tot); u_h covariant
 *   f : [Nh][16][Nv + 1]  covariant u_3
 * with node n = i + 4 j and elements ordered panel-major, row-major within a
 * panel, unless gb_config.elem_map / elem_orient give the caller's own order and
 * element frames (gb_match_elements derives them from node positions).
 * All pointers in gb_fieldvec are device pointers (e.g. CuArray / torch
 * tensors), 16-byte aligned.
 */
#ifndef GBDYCORE_H
#define GBDYCORE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_ctx gb_ctx;

enum gb_status {
  GB_OK = 0,
  GB_ERR_ARG = -1,        /* invalid argument or configuration */
  GB_ERR_CUDA = -2,       /* a CUDA runtime call failed */
  GB_ERR_NOMEM = -3,      /* device allocation failed */
  GB_ERR_NONFINITE = -4,  /* a NaN/Inf was detected in the Newton residual */
  GB_ERR_TIMEOUT = -5,    /* a bounded device wait gave up */
  GB_ERR_STATE = -6       /* call out of order (e.g. ldiv before update_jacobian) */
};

typedef struct {
  int h_elem;        /* elements per cubed-sphere panel edge (SphereGrid h_elem) */
  int z_elem;        /* vertical levels (centres) */
  int ft_bytes;      /* 4 = Float32, 8 = Float64 */
  int z_stretch;     /* 0 uniform, 1 hyperbolic-tangent stretching (grids.jl:356) */
  double z_max, dz_bottom;
  double dt;         /* model time step: van Leer Courant factor (implicit_tendency.jl:131-139) */
  double nu_v, nu_s; /* hyperdiffusivities nu_4_vorticity, nu_4_scalar (hyperdiffusion.jl:21-28) */
  double div_damp;   /* divergence_damping_factor */
  double sponge_zd, alpha_uh, alpha_w; /* Rayleigh sponge (rayleigh_sponge.jl:7-57); alpha = 0: off */
  int upwinding;     /* energy_q_tot_upwinding: 0 none, 1 van Leer (types.jl:1916) */
  /* physical constants (ClimaParams names) */
  double grav, omega, R_d, cp_d, cv_d, T_0, p_ref, T_min_ref, T_surf_ref, T_min_sgs, radius;
  /* Held-Suarez forcing of the explicit tendency (rad: held_suarez; held_suarez.jl): 0 off, 1 on
     (flat surface: sigma = p / MSLP); day length, boundary-layer top sigma_b, equator-to-pole
     contrast Delta T_y, equatorial surface temperature, static stability Delta theta_z, the
     equilibrium floor T_min, the potential-temperature reference pressure and MSLP */
  int held_suarez;
  double hs_day, hs_sigma_b, hs_dT_y, hs_T_equator, hs_dtheta_z, hs_T_min, hs_p_ref_theta, hs_MSLP;
  /* The caller's element layout (both NULL: the library's own order, see above).  ClimaCore
     numbers the elements along a space-filling curve (Topology2D(..., spacefillingcurve(mesh)),
     src/simulation/grids.jl:74-75) and each element has its own local (xi^1, xi^2) frame.
     elem_map[e] is the library element (panel-major, row-major) that the caller's element e
     is; elem_orient[e] in 0..3 says by how many quarter turns the caller's frame is rotated
     against the library's: the caller's node (i, j) is the library's node
       0: (i, j)   1: (3 - j, i)   2: (3 - i, 3 - j)   3: (j, 3 - i)
     (i fastest, n = i + 4 j), and its covariant u_1, u_2 are components on its own basis.
     Every geometry table, the DSS plan and every kernel then work in the caller's layout
     directly (no permutation of the state).  gb_match_elements derives both arrays from the
     caller's node positions.  Read by gb_sizes, gb_geometry_export and gb_ctx_create only. */
  const int *elem_map;
  const int *elem_orient;
  /* test_dycore_consistency (src/utils/debug_utils.jl:58-70, called from
     remaining_tendency.jl:52 and implicit_tendency.jl:37): 1 fills every library scratch
     buffer (Laplacians, stage state, explicit and implicit tendencies, Jacobian, residual
     slots) with NaN before each tendency evaluation and each step, so that a read of a
     quantity not recomputed first shows up as NaN in the result.  0 off. */
  int test_dycore_consistency;
  /* Terrain-following levels (topography: src/topography/topography.jl with the hypsography of
     the extruded space, src/simulation/grids.jl).  z_surface is the surface elevation in m at
     every node, in the caller's element and node order ([Nh][16], FP64), the collocated copies
     of a node holding the same value; NULL is a flat surface.  The face heights are
     z = zeta + z_s b(zeta) over the flat faces zeta (the centres midway between warped faces):
     warp 0 decays the terrain linearly to zero at z_max (LinearWarp), b = 1 - zeta / z_max;
     warp 1 is the one-scale SLEVE coordinate (SLEVEWarp) with eta_h = sleve_eta and
     s = sleve_s, b = sinh((eta_h - eta) / (s eta_h)) / sinh(1 / s) for eta = zeta / z_max
     <= eta_h, else 0.  The metric of every point (J, g^ij, g_ij with their vertical cross
     terms) follows from z_s, its spectral derivatives in each element and b; the kernels
     compute it where they use it.  Supported by gb_step, every hook (gb_set_precomputed_quantities
     applies u_3 = -u_h^3 / g^33 on the bottom and top faces; gb_update_jacobian adds the
     (rho, u_h) and (rho e_tot, u_h) blocks that gb_ldiv applies to R's u_h part),
     gb_global_sums and gb_time_kernel; gb_jacobian_solve_noalloc, the reverse-mode entries and
     the Held-Suarez forcing return GB_ERR_ARG for a terrain context. */
  const double *z_surface;
  int warp;
  double sleve_eta, sleve_s;
  /* Moist 0M (microphysics_model: EquilibriumMicrophysics0M): moist = 1 adds the prognostic
     rho q_tot as a fifth centre component, so the centre block is [Nh][5][16][Nv] with
     rho q_tot last (ClimaCore's Y.c field order rho, u_h, rho e_tot, rho q_tot).  The
     precomputed temperature then comes from the saturation adjustment of (rho, e_int,
     max(0, q_tot)) (precomputed_quantities.jl:734-747), the pressure is rho R_m T and
     theta_v = T R_m / (Pi R_d); the implicit tendency transports q_tot centrally
     (implicit_tendency.jl:211-215); gb_update_jacobian forms kappa_m = R_m / cv_m and the
     (u_3, rho q_tot) and (rho q_tot, u_3) blocks (manual_sparse_jacobian.jl:646-685, 770-831),
     and gb_ldiv solves the Schur complement onto u_3 with the rho q_tot row (the reference's
     ApproximateBlockArrowheadIterativeSolve, exact here because with 0M and no diffusion the
     scalar blocks are -I); gb_correct_implicit_advection_tendency corrects rho q_tot as well.
     The moist thermodynamic constants carry the Thermodynamics.jl parameter names (the
     liquid fraction ramps from 0 at T_icenuc to 1 at T_freeze with exponent pow_icenuc);
     sa_iters (>= 1) Newton iterations solve the saturation adjustment.  A moist context
     supports gb_set_precomputed_quantities, gb_implicit_tendency, gb_update_jacobian,
     gb_ldiv, gb_correct_implicit_advection_tendency, gb_jacobian_solve_noalloc, gb_dss (rho
     q_tot averaged as a scalar)
     and the conservation sums (gb_global_sums, gb_conservation_sums with the water integral);
     every other state entry point returns GB_ERR_ARG, as does moist = 1 with a surface or the
     Held-Suarez forcing. */
  int moist;
  double R_v, cp_v, cp_l, cp_i, LH_v0, LH_s0, T_triple, press_triple, T_freeze, T_icenuc, pow_icenuc;
  int sa_iters;
} gb_config;

typedef struct {
  void *c; /* centre block, see above */
  void *f; /* face block */
} gb_fieldvec;

/* Host-side geometry export (no GPU needed); any pointer may be NULL. */
typedef struct {
  double *xyz;   /* [Nh*16*3] unit-sphere node positions */
  double *ecov;  /* [Nh*16*2*3] covariant basis dX/dxi^i at radius R, Cartesian */
  double *Jh;    /* [Nh*16] horizontal Jacobian at radius R */
  double *gup;   /* [Nh*16*3] g^11, g^12, g^22 at radius R */
  double *fh0;   /* [Nh*16*2] contravariant 2*Omega*cos(lat)*north at radius R */
  double *zf;    /* [Nv+1] face heights */
  int *dss_off;  /* [ngroups+1] */
  int *dss_copy; /* [ncopies] element*16 + node, in the library's element order within a group
                    (ascending without elem_map) */
  double *econ;  /* [Nh*16*2*3] contravariant basis at radius R, Cartesian */
  double *dss_w; /* [ncopies] the J-weight of each copy in its group */
} gb_geometry_host;

/* Sizes for a configuration (no GPU needed). */
int gb_sizes(const gb_config *cfg, size_t *n_center, size_t *n_face, int *n_dss_groups, int *n_dss_copies);
int gb_geometry_export(const gb_config *cfg, gb_geometry_host *out);
/* The caller's element layout from its node positions (no GPU needed): xyz holds, for each of
 * the caller's 6 h_elem^2 elements and its 16 nodes (n = i + 4 j), the node's position
 * (any radius; FP64, [Nh][16][3]).  Fills elem_map[Nh] and elem_orient[Nh] for gb_config.
 * Fails with GB_ERR_ARG when an element is not one of the equiangular cubed sphere's at
 * h_elem, its nodes are not the GLL nodes in a rotated (i, j) frame (a mirrored frame is
 * refused), or two elements are the same one.  The replacement for the layout a ClimaCore
 * SpectralElementSpace2D takes from its topology (src/simulation/grids.jl:74-75). */
int gb_match_elements(const gb_config *cfg, const double *xyz, int *elem_map, int *elem_orient);

/* Context lifetime.  Replaces the library-owned parts of AtmosCache
 * (src/cache/cache.jl:165-305: geometry, Coriolis, DSS buffers, scratch) and
 * the Jacobian cache (manual_sparse_jacobian.jl:603). */
int gb_ctx_create(const gb_config *cfg, gb_ctx **out);
int gb_ctx_destroy(gb_ctx *ctx);
int gb_set_stream(gb_ctx *ctx, void *cuda_stream);
/* Copies the last error message; returns the last gb_status. */
int gb_last_error(gb_ctx *ctx, char *buf, size_t len);

/* set_precomputed_quantities!(Y, p, t)  src/cache/precomputed_quantities.jl:928
 * Applies the impenetrable-boundary filter to Y.f (u^3 = 0 at the bottom and
 * top faces); the other precomputed quantities are recomputed inside each
 * kernel from Y. */
int gb_set_precomputed_quantities(gb_ctx *ctx, gb_fieldvec Y, double t);

/* remaining_tendency!(Yt, Yt_lim, Y, p, t)  src/prognostic_equations/remaining_tendency.jl:48
 * (Yt_lim is empty for the dry model). */
int gb_remaining_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t);

/* implicit_tendency!(Yt, Y, p, t)  src/prognostic_equations/implicit/implicit_tendency.jl:36 */
int gb_implicit_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t);

/* update_jacobian!(jacobian, Y, p, dtgamma, t)  src/prognostic_equations/implicit/jacobian.jl:74
 * -> manual_sparse_jacobian.jl:713-870; the blocks are kept in the context. */
int gb_update_jacobian(gb_ctx *ctx, gb_fieldvec Y, double dtgamma, double t);

/* LinearAlgebra.ldiv!(dY, jacobian, R)  src/prognostic_equations/implicit/jacobian.jl:78-82
 * (BlockArrowheadSolve, manual_sparse_jacobian.jl:580-583). */
int gb_ldiv(gb_ctx *ctx, gb_fieldvec dY, gb_fieldvec R);

/* correct_implicit_advection_tendency!(Yt, Y, p, t)  implicit_tendency.jl:322-339 */
int gb_correct_implicit_advection_tendency(gb_ctx *ctx, gb_fieldvec Yt, gb_fieldvec Y, double t);

/* dss!(Y, p, t)  src/prognostic_equations/constrain_state.jl:59-64 */
int gb_dss(gb_ctx *ctx, gb_fieldvec Y);

/* One or more fused ARS343 steps with one Newton iteration per implicit stage
 * (the ClimaTimeSteppers stage loop driven by solve_atmos!,
 * src/simulation/solve.jl:57-63).  use_graph = 1 replays a captured CUDA
 * graph of the whole step. */
int gb_step(gb_ctx *ctx, gb_fieldvec Y, double t, double dt, int nsteps, int use_graph);

/* Global integrals of rho and rho e_tot (sum of value * WJ), compensated FP64,
 * as check_conservation does (src/simulation/solve.jl:216-265).  Synchronous. */
int gb_global_sums(gb_ctx *ctx, gb_fieldvec Y, double out[2]);

/* The three integrals check_conservation compares (src/simulation/solve.jl:216-265): out[0]
 * of rho, out[1] of rho e_tot and out[2] of rho q_tot (the water; 0 for a dry context, whose
 * water_conservation the reference sets to zero), compensated FP64.  Synchronous. */
int gb_conservation_sums(gb_ctx *ctx, gb_fieldvec Y, double out[3]);

/* FP64 sums of squares of the Newton residual of the last gb_step (rho,
 * rho e_tot, u_3 parts, summed over stages); synchronous. */
int gb_newton_residual(gb_ctx *ctx, double out[3]);

/* Failure-detection self-test (no counterpart in the reference, whose failure
 * detection is the host-side NaN scan).  Every wait of this library's kernels
 * on an asynchronous copy is bounded: when it runs out, the kernel sets a bit
 * in the context's device status word, waits once more with the same limit for
 * its own copies and leaves, and the next synchronous entry returns
 * GB_ERR_TIMEOUT.  This entry runs that path on purpose: one warp waits, with a
 * limit of limit_s seconds (0 < limit_s <= 1), on an mbarrier whose announced
 * transfer is never issued.  Returns GB_ERR_TIMEOUT (the status is then
 * cleared and the context stays usable); GB_OK would mean the wait did not run
 * out.  Synchronous. */
int gb_selftest_bounded_wait(gb_ctx *ctx, double limit_s);

/* Allocation-free Jacobian update + solve.  No counterpart in the reference.
 * It is for callers that cannot let a library allocate device memory while
 * they run: a host model whose runtime owns all device memory through its own
 * pool or a pre-sized arena (a cudaMalloc behind its back fails or breaks its
 * accounting), or a Newton loop that must not take the device-wide
 * synchronisation of a first cudaMalloc.  gb_update_jacobian allocates its
 * block storage with cudaMalloc on first use; this entry instead builds the
 * Jacobian at Y (with dtgamma) in a file-scope static device array of
 * GB_NOALLOC_SCRATCH_BYTES and solves W dY = R with it, allocating nothing.
 * Limit: (6 h_elem^2 * 16 columns) * (z_elem + 1) * nq * ft_bytes, nq = 15
 * (19 for a moist 0M context, whose Jacobian carries the rho q_tot blocks), must
 * not exceed GB_NOALLOC_SCRATCH_BYTES (else GB_ERR_ARG).  A terrain context
 * returns GB_ERR_ARG.  The array is held by
 * every GPU that loads the library until the process exits.  The first call on
 * a device, with that device current, resolves the array's device address
 * (cudaGetSymbolAddress) and keeps it for the process: make that first call
 * before any stream capture, and do not reset the device while the library is
 * loaded (a reset invalidates the kept address, as it does every context).
 * Every call overwrites the whole block storage it uses before reading it, so
 * nothing needs to start at zero; all calls share the one array, so calls that
 * overlap on the GPU race.  Asynchronous on the context stream. */
#define GB_NOALLOC_SCRATCH_BYTES (64u << 20)
int gb_jacobian_solve_noalloc(gb_ctx *ctx, gb_fieldvec dY, gb_fieldvec Y, gb_fieldvec R, double dtgamma);

/* Measurement support (no counterpart in the reference): launches one of the
 * step's kernels `reps` times on the context stream between CUDA events and
 * returns the mean time per launch in milliseconds.  kernel: 0 pass A
 * (Laplacians), 1 pass B (explicit tendency), 2 column stage (stage 4: five
 * sources), 3 state DSS, 4 the unfolded final combination (run by gb_step only
 * for a tableau that is not stiffly accurate), 9 the last stage's pass B with
 * the final combination folded in (what gb_step runs for ARS343).  Y is read (and, for 3, written);
 * synchronous. */
enum gb_kernel_id {
  GB_K_PASSA = 0, GB_K_PASSB = 1, GB_K_COLUMN = 2, GB_K_DSS = 3, GB_K_FINAL = 4,
  /* reverse mode: pass A^T, pass B^T, the implicit column stage VJP, DSS^T */
  GB_K_PASSA_VJP = 5, GB_K_PASSB_VJP = 6, GB_K_COLUMN_VJP = 7, GB_K_DSS_T = 8,
  GB_K_PASSB_FINAL = 9
};
int gb_time_kernel(gb_ctx *ctx, int kernel, gb_fieldvec Y, int reps, double *ms_per_launch);

/* ---------------------------------------------------------------------------
 * Reverse mode (adjoint) of the step, for gradients with respect to the state
 * and to two scalars: nu (nu_4_vorticity, with nu_4_scalar = nu / Prandtl
 * following it) and the Rayleigh sponge rate alpha (alpha_uh = alpha_w =
 * alpha, beta(z) = alpha s(z) above sponge_zd).  Julia AD reaches them
 * through a ChainRulesCore rule: these entries are the forward and pullback
 * halves of ChainRulesCore.rrule(solve, Y0, (nu, rate), p, dt, n), which the
 * Julia shim defines on gb_adjoint_forward / gb_adjoint_reverse.  Every *_vjp entry ACCUMULATES into its cotangent
 * outputs (+=) and into dparams[0] (d/dnu) and dparams[1] (d/dalpha); each
 * is the exact reverse of the corresponding forward computation in this
 * library.  Synchronous.  The reverse slab kernels keep an element's state,
 * Laplacians and tendency cotangent in shared memory: FP64 contexts support
 * z_elem up to ~50, FP32 up to 127 (else GB_ERR_ARG).
 * ------------------------------------------------------------------------- */

/* Transpose of gb_dss (in place). */
int gb_dss_transpose(gb_ctx *ctx, gb_fieldvec X);
/* Reverse of gb_remaining_tendency: Ybar += (dT/dY)^T Tbar (Tbar is not modified). */
int gb_remaining_tendency_vjp(gb_ctx *ctx, gb_fieldvec Ybar, gb_fieldvec Tbar, gb_fieldvec Y, double t,
                              double dparams[2]);
/* One fused implicit stage on a given U^: one Newton iteration of the stage
 * equation, the impenetrable filter and the van Leer post-Newton correction
 * (as inside gb_step); writes U and T_imp = (U - U^)/dtgamma, the latter in
 * the reduced layout c: [Nh][2][16][Nv] (rho, rho e_tot), f: faces. */
int gb_implicit_stage(gb_ctx *ctx, gb_fieldvec U, gb_fieldvec Timp, gb_fieldvec Uhat, double dtgamma);
/* Reverse of gb_implicit_stage, including the dependence of the Jacobian on
 * the state: Uhat_bar += (dU/dU^)^T Ubar + (dT_imp/dU^)^T Timp_bar. */
int gb_implicit_stage_vjp(gb_ctx *ctx, gb_fieldvec Uhat_bar, gb_fieldvec Ubar, gb_fieldvec Timp_bar, gb_fieldvec Uhat,
                          double dtgamma, double dparams[2]);
/* Reverse of one gb_step from u_n = Y (not modified): Ybar holds the cotangent
 * of u_{n+1} on entry and that of u_n on return. */
int gb_step_vjp(gb_ctx *ctx, gb_fieldvec Ybar, gb_fieldvec Y, double t, double dt, double dparams[2]);
/* Forward half of the trajectory gradient: Y advances nsteps steps (as
 * gb_step) and a copy of the state is kept every checkpoint_every steps. */
int gb_adjoint_forward(gb_ctx *ctx, gb_fieldvec Y, double t0, double dt, int nsteps, int checkpoint_every);
/* Pullback of the last gb_adjoint_forward: Ybar holds dJ/du_N on entry and
 * dJ/du_0 on return; dparams receives (dJ/dnu, dJ/dalpha) (overwritten).
 * Each segment between checkpoints is recomputed from its checkpoint with its
 * stage data kept, then reversed.  peak_bytes (may be NULL) receives the
 * device bytes the library held during the pass. */
int gb_adjoint_reverse(gb_ctx *ctx, gb_fieldvec Ybar, double dparams[2], size_t *peak_bytes);
/* Memory against recomputation in the checkpointed adjoint (no counterpart in the reference,
 * which leaves checkpointing to the AD tool): the forward half keeps the stage data of the
 * last `segments` checkpoint segments (default 1), so the reverse pass recomputes only the
 * segments before them.  Each kept step holds about 13 states (its stage states, Laplacians
 * and tendencies).  segments >= 1; it applies from the next gb_adjoint_forward. */
int gb_adjoint_set_record_segments(gb_ctx *ctx, int segments);

/* ---------------------------------------------------------------------------
 * Batched standalone columns of uneven height.
 *
 * A batch of independent dry columns, each a ColumnGrid of its own z_elem
 * (src/simulation/grids.jl:93-127: flat column metric, faces uniform or
 * tanh-stretched as gb_config.z_stretch / dz_bottom / z_max say), solved by
 * NewtonsMethod(max_iters = newton_iters, update_j =
 * UpdateEvery(NewNewtonIteration)) (integrator.jl:63-120) on the implicit
 * stage equation U = U^ + dtgamma T_imp(U): each iteration is
 * implicit_tendency! (implicit_tendency.jl:185-298) for the residual,
 * update_jacobian! (manual_sparse_jacobian.jl:713-870) and ldiv! with
 * BlockArrowheadSolve (:580-583), with the impenetrable filter on u_3
 * (precomputed_quantities.jl:486-553).  Columns do not interact.
 *
 * Layout (C_c = sum over d < c of z_elem_d, C = C_ncols):
 *   c : [4][C]          (rho, u_1, u_2, rho e_tot), column c at C_c .. C_c + z_elem_c - 1
 *   f : [C + ncols]     u_3, column c at C_c + c .. C_c + c + z_elem_c
 * Precision and constants come from gb_config (h_elem, dt, hyperdiffusion,
 * upwinding and the radius are unused; the column metric is flat).
 *
 * Modes of gb_columns_solve:
 *   GB_COLUMNS_GRAPH       one persistent launch (warps take groups of
 *                          columns of one height class from a work counter,
 *                          tallest first), captured with its reset and the
 *                          residual reduction as one CUDA graph and replayed;
 *   GB_COLUMNS_PERSISTENT  the same launch sequence without the graph;
 *   GB_COLUMNS_PER_HEIGHT  the plain form: one launch per distinct z_elem.
 * The persistent kernel variant (columns per block, levels per lane) is the
 * one gb_columns_autotune chose, else a default.
 * ------------------------------------------------------------------------- */
typedef struct gb_columns gb_columns;
enum gb_columns_mode { GB_COLUMNS_GRAPH = 0, GB_COLUMNS_PERSISTENT = 1, GB_COLUMNS_PER_HEIGHT = 2 };
#define GB_COLUMNS_VARIANTS 5

/* z_elem[c] in [2, 127].  Builds the per-height level tables and the work
 * lists; allocates device memory. */
int gb_columns_create(const gb_config *cfg, int ncols, const int *z_elem, gb_columns **out);
int gb_columns_destroy(gb_columns *cols);
int gb_columns_set_stream(gb_columns *cols, void *cuda_stream);
/* Total centres C (the component stride of the centre block). */
int gb_columns_size(const gb_columns *cols, long long *centres, long long *faces);
/* U: the initial iterate on entry (normally a copy of Uhat), the iterate after
 * newton_iters iterations on return (u_h set to Uhat's, u_3 filtered).  rnorm, if
 * not NULL, receives newton_iters x 3 FP64 sums over the batch of the squared
 * residual (rho, rho e_tot, u_3) of each iteration, and the call synchronizes;
 * otherwise it is asynchronous.  newton_iters in [1, 8]. */
int gb_columns_solve(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uhat, double dtgamma, int newton_iters, int mode,
                     double *rnorm);
/* Times every persistent kernel variant (each from the same initial iterate U,
 * which is left unchanged) and keeps the fastest for later solves.  ms, if not
 * NULL, receives GB_COLUMNS_VARIANTS mean times (negative: variant not
 * applicable); *choice the chosen variant.  Synchronous. */
int gb_columns_autotune(gb_columns *cols, gb_fieldvec U, gb_fieldvec Uhat, double dtgamma, int newton_iters,
                        int reps, int *choice, double *ms);
/* Sets the persistent kernel variant (0 .. GB_COLUMNS_VARIANTS - 1) directly. */
int gb_columns_set_variant(gb_columns *cols, int variant);
int gb_columns_last_error(const gb_columns *cols, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif
