/*
 * sfgpu.h -- C ABI of the GB300 (sm_103a) library that replaces the two grid solves of a SimFerrofluid
 * substep: the ghost-fluid pressure projection and the FDM magnetostatic potential solve.
 *
 * Every entry point takes plain pointers and sizes.  Arrays use the reference's layout (core/Grid.h:28):
 *   cell (i,j,k)            -> k + nz*(j + ny*i)                  (nx*ny*nz doubles)
 *   face (i,j,k) of axis a  -> same formula on the face grid of size res + e_a (core/StaggeredGrid.h:16-20)
 * Face arrays are passed as `const double *x[3]` (x, y, z face grids).  `_dev` variants take device
 * pointers (cudaMalloc'ed or managed, on the context's device) and run without host<->device copies.
 *
 * Thread safety: one context per host thread; calls on one context are serialised by the caller.  A context
 * owns a CUDA stream (or borrows one) and all device workspaces; the solvers' warm-start state (the last
 * pressure for Reproject, the last potential for the magnetic warm start) lives in the context, like the
 * members m_RdP (core/Pressure.h:49) and m_Sol (core/MagneticField.h:66) of the reference classes.
 */
#ifndef SFGPU_H
#define SFGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFGPU_ABI_VERSION 2

#if defined(__GNUC__)
#define SF_EXPORT __attribute__((visibility("default")))
#else
#define SF_EXPORT
#endif

typedef enum {
    SF_OK = 0,
    SF_NOT_CONVERGED = 1,   /* iteration cap reached; outputs hold the last iterate */
    SF_BAD_ARG = 2,         /* null pointer, non-positive size, unknown option value */
    SF_CUDA_ERROR = 3,      /* a CUDA call failed; sf_last_error() has the message */
    SF_NO_DEVICE = 4,       /* no CUDA device, or the device is not sm_103 */
    SF_OUT_OF_MEMORY = 5,
    SF_STALLED_FALLBACK = 6, /* learned solve: the network stalled (a step removed less than 10% of the residual,
                                or was not finite); the plain MGPCG finished the solve (not an error) */
    SF_NOT_READY = 7,       /* Reproject called before any Project on this context / grid */
    SF_TOO_LARGE = 8        /* grid exceeds the fixed scratch of sf_magnetic_residual_noalloc */
} sf_status;

typedef enum {
    SF_PREC_FP64 = 0,   /* plain method: FP64 MGPCG */
    SF_PREC_MIXED = 1,  /* FP32 V-cycle, FP16 coarse coefficients, inner FP32 FCG, FP64 iterative refinement */
    SF_PREC_LEARNED = 2 /* mixed form with learned correction steps: at the start of every inner flexible-CG
                           solve of the refinement (the first from r = b), the attached U-Net's prediction y of
                           A^-1 r, scaled by gamma = (y,r)/(y,Ay) (never a larger A-norm error than no step), is
                           the first step, and the flexible CG continues from the remaining residual.  A step
                           that removes less than 10% of ||r|| stalls the network: the rest of the solve is the
                           plain MGPCG iteration (SF_STALLED_FALLBACK); the FP64 residual judges the result. */
} sf_precision;

/* Cell grid of a staggered grid: resolution, spacing and corner (StaggeredGrid ctor,
 * core/StaggeredGrid.h:8-21: origin = center - res*h/2). */
typedef struct {
    int nx, ny, nz;
    double h;
    double origin[3];
} sf_grid;

typedef struct {
    int precision;       /* sf_precision */
    double tol;          /* stop when ||b - A x|| <= tol * ||b|| (the reference's amgcl criterion) */
    int max_iters;       /* PCG iterations (FP64) or total inner iterations (mixed) */
    int pre_smooth;      /* red-black Gauss-Seidel sweeps before restriction */
    int post_smooth;     /* ... after prolongation */
    int coarse_sweeps;   /* symmetric sweep pairs on the coarsest level (default 8 pressure, 48 potential) */
    int max_levels;      /* 0 = coarsen until every dimension is <= coarse_dim */
    int coarse_dim;      /* default 8 */
    int warm_start;      /* magnetic: start from the context's last potential (reference behaviour, default 1);
                            pressure Project always starts from zero (core/Pressure.cpp:122) */
    int use_graph;       /* capture one PCG iteration in a CUDA graph (default 1) */
    int check_every;     /* read the residual norm back every k iterations (default 1) */
    int report_ref_residual; /* also compute the residual on the reference's own operator (default 1) */
    double inner_tol;    /* mixed: floor of the inner relative reduction (default 1e-3: the FP32 inner flexible CG
                            stagnates near 1e-4 on large grids, and an earlier FP64 refinement step restarts it) */
    int profile;         /* time every finest-level smoother launch with CUDA events (disables graphs) */
    int smoother;        /* 0: two in-place colour passes, 1: fused one-pass red-black sweep (TMA-staged at the
                            finest FP32 level), 2: as 0, and in the mixed form the finest level's smoother reads
                            an FP16 copy of the operator (residuals and the CG operator stay FP32), 3 (default):
                            as 2, with the mixed form's finest-level FP32 vectors and operator copies stored
                            colour by colour (each half sweep streams one colour); needs nz % 8 == 0 and two or
                            more levels, else runs as 2.  FP64 solves run 2 and 3 as 0. */
    int coarse_pre;      /* pre- / post-smoothing sweeps on levels 2 and coarser (0: as pre_smooth / post_smooth) */
    int coarse_post;
    int coarse_tail;     /* mixed form, levels of at most 65,536 cells: 0 (default) one launch of a thread-block
                            cluster of 16 CTAs where the device runs it, else 8; 8 or 16 that cluster size; 1 separate
                            kernels.  All give the same results. */
    int full_sweeps;     /* FP64 form: 1 smooths and iterates over every row of the grid; 0 (default) skips the rows
                            without an active cell (air in the pressure system) on every level, as the mixed form
                            does.  Both give the same answer. */
    int reserved[2];
} sf_solve_opts;

typedef struct {
    int iters;               /* PCG iterations (FP64) or inner FCG iterations summed over outer steps */
    int outer_iters;         /* mixed: iterative-refinement steps; FP64: 0 */
    int levels;              /* multigrid levels used */
    int converged;
    long long unknowns;      /* liquid cells (pressure) or all cells (magnetic) */
    double rel_residual;     /* ||b - A x|| / ||b|| of the solved system, FP64, recomputed after the solve */
    double rel_residual_ref; /* same on the reference's operator (pinned row 0 for the potential) */
    double ms_build, ms_solve, ms_post, ms_total; /* device time per phase (CUDA events), ms_total = wall */
    long long h2d_bytes, d2h_bytes;
    int status_detail;       /* 1: Krylov breakdown (non-positive curvature) */
    int smooth_launches;     /* profile: finest-level smoother launches timed */
    double smooth_ms;        /* profile: their summed device time */
    long long kernel_launches; /* kernels this call launched (graph nodes counted per replay) */
    double smooth_bytes;     /* profile: algorithmic bytes of the timed smoother launches */
    double guess_rel_residual; /* learned form: ||b - A x0|| / ||b|| after the first learned step x0 = gamma y
                                  (-1: none) */
    double guess_energy_ratio; /* learned form: ||x* - x0||_A^2 / ||x*||_A^2 of that step (-1: none) */
    int learned_steps;         /* learned form: correction steps applied */
    int reserved_stats;
} sf_solve_stats;

/* ----- context ------------------------------------------------------------------------------------------- */
SF_EXPORT sf_status sf_create(int device, void *cuda_stream /* NULL = own non-blocking stream */, void **ctx_out);
SF_EXPORT void sf_destroy(void *ctx);
SF_EXPORT const char *sf_status_string(int status);
SF_EXPORT const char *sf_last_error(void *ctx);
SF_EXPORT int sf_abi_version(void);
/* which: 0 = pressure defaults (tol 1e-8, amgcl's default), 1 = magnetic defaults (tol 1e-6,
 * core/MagneticField.cpp:93). */
SF_EXPORT void sf_default_opts(sf_solve_opts *opts, int which);
/* Device bytes the context holds right now. */
SF_EXPORT long long sf_device_bytes(void *ctx);

/* ----- pressure projection ------------------------------------------------------------------------------
 * Replaces Pressure::Project (core/Pressure.cpp:17-26): SetUnKnowns (:104-123), BuildProjectionMatrix
 * (:38-78), SolveLinearSystem (:125-135, amgcl SA+SPAI0 BiCGStab there, MGPCG here) and ApplyProjection
 * (:137-166).
 *   vel[3]      in/out MAC velocity (face arrays)
 *   phi         level set on cells; liquid where phi <= 0 (NULL: the level set of sf_levelset_upload)
 *   frac[3]     collider solid fraction per face (Collider::GetFraction, 1 = solid); frac == NULL: the collider of
 *               sf_collider_upload
 *   solid_vel[3] collider velocity per face (Collider::Velocity), or NULL = 0
 *   jump[3]     per-face value of the pressure-jump callback J(axis, face, theta) = p_liquid - p_air
 *               (core/Pressure.h:20-22), read on liquid-air faces only, or NULL = no callback.  The shipped
 *               callback ignores theta (core/Simulation.cpp:216-235); a theta-dependent callback cannot be
 *               expressed as an array.
 *   vol_error   volume-correction source added to every liquid row (core/Pressure.cpp:75)
 *   p_out       optional (nx*ny*nz) pressure on cells, 0 in air
 * Faces on the outer boundary of the grid are treated as closed walls (the reference reads outside its
 * arrays there if they are open). */
SF_EXPORT sf_status sf_pressure_project(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                              const double *const frac[3], const double *const solid_vel[3],
                              const double *const jump[3], double vol_error, double *p_out,
                              const sf_solve_opts *opts, sf_solve_stats *stats);
SF_EXPORT sf_status sf_pressure_project_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                  const double *const frac[3], const double *const solid_vel[3],
                                  const double *const jump[3], double vol_error, double *p_out,
                                  const sf_solve_opts *opts, sf_solve_stats *stats);
/* Replaces Pressure::Reproject (core/Pressure.cpp:28-36): keeps the unknowns and matrix of the last
 * Project on this context, rebuilds only the right-hand side (SetRightHandSide, :80-102, no jump terms),
 * starts from the last pressure and applies the projection with `jump`. */
SF_EXPORT sf_status sf_pressure_reproject(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                const double *const frac[3], const double *const solid_vel[3],
                                const double *const jump[3], double vol_error, double *p_out,
                                const sf_solve_opts *opts, sf_solve_stats *stats);
SF_EXPORT sf_status sf_pressure_reproject_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                    const double *const frac[3], const double *const solid_vel[3],
                                    const double *const jump[3], double vol_error, double *p_out,
                                    const sf_solve_opts *opts, sf_solve_stats *stats);

/* ----- magnetic potential -------------------------------------------------------------------------------
 * Replaces MagneticField::Solve (core/MagneticField.cpp:29-35): mu on faces from the smoothed Heaviside of
 * phi (BuildMatrix :51-60, Heaviside core/MagneticField.h:44-54), the full-grid variable-coefficient
 * Laplacian with homogeneous Neumann walls and psi[0] = 0 (:62-90), the right-hand side (AssembleRHS
 * :97-118), the solve (amgcl SA+SPAI0 CG there, MGPCG here) and AssignTotalField (:125-143).
 *   phi          level set on the simulation's cell grid (NULL: the level set of sf_levelset_upload)
 *   chi          susceptibility (SetSusceptibility), band_width the Heaviside half-width (SetBandWidth)
 *   hext[3]      applied field on faces (NULL: the field of sf_applied_field_prefetch)
 *   psi_out      optional (nx*ny*nz) potential, psi[0] = 0
 *   H_out[3]     optional total field H = Hext - grad psi on faces (m_TotalField)
 * The solve starts from the context's last potential on the same grid when opts->warm_start (m_Sol). */
SF_EXPORT sf_status sf_magnetic_solve(void *ctx, const sf_grid *g, const double *phi, double chi, double band_width,
                            const double *const hext[3], double *psi_out, double *const H_out[3],
                            const sf_solve_opts *opts, sf_solve_stats *stats);
SF_EXPORT sf_status sf_magnetic_solve_dev(void *ctx, const sf_grid *g, const double *phi, double chi, double band_width,
                                const double *const hext[3], double *psi_out, double *const H_out[3],
                                const sf_solve_opts *opts, sf_solve_stats *stats);
/* ----- collider inputs ----------------------------------------------------------------------------------
 * Solid fractions of the pressure solve (host code, run once per scene).
 * sf_collider_box_fractions replaces Collider(sgrid) + Collider::Finish for the domain-box walls
 * (core/Collider.cpp:8-19,21-45): node level set -0.01 h - sdf_box, FastMarching::Solve(LevelSet, -1)
 * (core/FastMarching.cpp:25-62), then CalcFaceFraction (core/Collider.cpp:47-73) on every face.
 * boundary_width is the staggered grid's boundary width (the box spans origin + bw h .. origin + (res-bw) h).
 * node_ls_out (optional) receives the (nx+1)(ny+1)(nz+1) redistanced node level set.
 * sf_collider_face_fractions runs CalcFaceFraction alone on a caller-supplied node level set. */
SF_EXPORT sf_status sf_collider_box_fractions(const sf_grid *g, int boundary_width, double *const frac_out[3],
                                              double *node_ls_out);
SF_EXPORT sf_status sf_collider_face_fractions(const sf_grid *g, const double *node_ls, double *const frac_out[3]);

/* ----- learned form: the 3D U-Net (no counterpart in the reference) --------------------------------------
 * 4 levels, 16/32/64/64 channels, 3x3x3 convolutions, BF16 weights and activations, FP32 accumulation on the
 * tensor cores.  Input: 16 feature channels per cell (BF16, channels last); output: one FP32 value per cell.
 * Parameters: a flat FP32 vector, layer by layer, weights [tap][cout][cin] then bias [cout].  All pointers in
 * the _dev calls are device pointers on the context's device. */
SF_EXPORT sf_status sf_unet_create(void *ctx, void **net_out);
SF_EXPORT void sf_unet_destroy(void *net);
SF_EXPORT long long sf_unet_num_params(void *net);
SF_EXPORT sf_status sf_unet_set_params(void *net, const float *host_params, long long n);
SF_EXPORT sf_status sf_unet_get_params(void *net, float *host_params, long long n);
SF_EXPORT sf_status sf_unet_forward_dev(void *net, const sf_grid *g, const void *features_bf16, float *out);
/* gradients of sum(dout * net(features)) w.r.t. the parameters, copied to grads_host (nullable) */
SF_EXPORT sf_status sf_unet_backward_dev(void *net, const sf_grid *g, const void *features_bf16, const float *dout,
                                         float *grads_host);
/* one Adam step (lr) on the scale-invariant loss 1 - (o.t)^2 / (|o|^2 |t|^2); *loss receives the loss */
SF_EXPORT sf_status sf_unet_train_step_dev(void *net, const sf_grid *g, const void *features_bf16,
                                           const float *target, float lr, double *loss);
/* convolution kernels: 0 = warp-level tensor-core MMA (mma.sync), 1 (default) = tcgen05 tensor cores with TMA
 * staging and TMEM accumulators for the forward, input-gradient and weight-gradient convolutions (layers whose grid
 * holds one brick: 32 x 4 for the forward and input gradient, 128 x 6 x 4 for the 16-channel line kernel, 32 x 4 x 2
 * for the weight gradient; others use mode 0), 2 = tcgen05 for the weight gradient alone.  sf_unet_tc_launches
 * counts the tcgen05 convolutions launched so far. */
SF_EXPORT sf_status sf_unet_set_mode(void *net, int mode);
SF_EXPORT long long sf_unet_tc_launches(void *net);
/* attach (or detach with NULL) the network used by SF_PREC_LEARNED solves on this context */
SF_EXPORT sf_status sf_set_network(void *ctx, void *net);
/* features of the last assembled pressure (which = 0) or potential (1) system and its solution (FP32) */
SF_EXPORT sf_status sf_system_features_dev(void *ctx, int which, void *features_bf16, float *solution);
/* Read back the finest-level operator and right-hand side of the last assembled pressure (which = 0) or
 * potential (1) system on this context into host arrays of nx*ny*nz doubles (any pointer may be NULL): the
 * diagonal, the couplings on each cell's lower x / y / z face (the off-diagonal entry is minus the coupling)
 * and b.  Pressure rows of air cells are all zero; the potential keeps row 0 in its unpinned (Neumann) form.
 * For checking the assembly against the reference's matrices (core/Pressure.cpp:38-78,
 * core/MagneticField.cpp:62-118).  Synchronises the context's stream. */
SF_EXPORT sf_status sf_system_operator(void *ctx, int which, double *diag, double *const lower[3], double *rhs);

/* ----- velocity pipeline after the projection (core/Simulation.cpp:236-241) -------------------------------------
 * Extrapolation::Solve (core/Extrapolation.cpp:4-30) of the projected velocity over max_steps layers, with the
 * simulation's validity predicate (core/Simulation.cpp:237-240: fraction < 1 and an adjacent cell liquid);
 * faces left without a valid neighbour take clear_val.  vel is updated in place. */
SF_EXPORT sf_status sf_extrapolate_velocity(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                            const double *const frac[3], double clear_val, int max_steps);
SF_EXPORT sf_status sf_extrapolate_velocity_dev(void *ctx, const sf_grid *g, double *const vel[3], const double *phi,
                                                const double *const frac[3], double clear_val, int max_steps);
/* Collider::Enforce (core/Collider.cpp:75-86): on faces with fraction 1 the velocity becomes the trilinearly
 * interpolated old velocity minus its normal component relative to the solid velocity (solid_vel NULL: zero).
 * normal: the collider's face normals (sf_collider_face_normals). */
SF_EXPORT sf_status sf_collider_enforce(void *ctx, const sf_grid *g, double *const vel[3], const double *const frac[3],
                                        const double *const normal[3], const double *const solid_vel[3]);
SF_EXPORT sf_status sf_collider_enforce_dev(void *ctx, const sf_grid *g, double *const vel[3],
                                            const double *const frac[3], const double *const normal[3],
                                            const double *const solid_vel[3]);
/* Collider::Finish normals (core/Collider.cpp:30-44) from the node level set (host). */
SF_EXPORT sf_status sf_collider_face_normals(const sf_grid *g, const double *node_ls, double *const normal[3]);

/* ----- interface coupling (core/Simulation.cpp:204-235) ----------------------------------------------------------
 * MagneticField::CalculateVertexPressures (core/MagneticField.cpp:37-48): p_m at each surface-mesh vertex from the
 * total field H (the H_out of sf_magnetic_solve): H trilinear at the vertex, p = mu0/2 chi (|H|^2 +
 * chi^2/(4chi+4) (H.n)^2).  positions, normals: nverts x 3 doubles (SurfaceMesh::Positions / Normals). */
SF_EXPORT sf_status sf_magnetic_vertex_pressures(void *ctx, const sf_grid *g, double chi, const double *const H[3],
                                                 const double *positions, const double *normals, long long nverts,
                                                 double *pressures);
SF_EXPORT sf_status sf_magnetic_vertex_pressures_dev(void *ctx, const sf_grid *g, double chi, const double *const H[3],
                                                     const double *positions, const double *normals,
                                                     long long nverts, double *pressures);
/* The pressure jump J(axis, face) of the simulation's callback (core/Simulation.cpp:216-235) on every face, for
 * sf_pressure_project's jump argument: with v = Contour::VertexIndexOf(axis, face - e_axis) (edge_mark[a]: int32
 * per edge of the cell grid along a, size res - e_a, -1 = no vertex), J = curvature[v] st_coeff / density / h dt
 * (if curvature) - mag_pressure[v] / density / h dt (if mag_pressure); 0 where there is no vertex. */
SF_EXPORT sf_status sf_pressure_jump(void *ctx, const sf_grid *g, const int32_t *const edge_mark[3],
                                     const double *curvature, const double *mag_pressure, long long nverts,
                                     double st_coeff, double density, double dt, double *const jump[3]);
SF_EXPORT sf_status sf_pressure_jump_dev(void *ctx, const sf_grid *g, const int32_t *const edge_mark[3],
                                         const double *curvature, const double *mag_pressure, long long nverts,
                                         double st_coeff, double density, double dt, double *const jump[3]);

/* ----- level-set neighbours (core/Simulation.cpp:164-165, 265) --------------------------------------------------
 * Advection::Solve<2> (core/Advection.h:33-59): semi-Lagrangian advection over dt with the TVD RK2 trace through
 * the velocity (trilinear per face grid); the level set is interpolated tricubically (TriCuInterp), the velocity
 * (advected by itself) trilinearly.  Reinitialization::Solve (core/Reinitialization.cpp:36-76): max_steps TVD-RK3
 * steps of the reinitialisation equation with WENO5 derivatives, dt = h/2.  All update their arrays in place. */
SF_EXPORT sf_status sf_advect_levelset(void *ctx, const sf_grid *g, double *phi, const double *const vel[3], double dt);
SF_EXPORT sf_status sf_advect_levelset_dev(void *ctx, const sf_grid *g, double *phi, const double *const vel[3],
                                           double dt);
SF_EXPORT sf_status sf_advect_velocity(void *ctx, const sf_grid *g, double *const vel[3], double dt);
SF_EXPORT sf_status sf_advect_velocity_dev(void *ctx, const sf_grid *g, double *const vel[3], double dt);
SF_EXPORT sf_status sf_reinitialize(void *ctx, const sf_grid *g, double *phi, int max_steps);
SF_EXPORT sf_status sf_reinitialize_dev(void *ctx, const sf_grid *g, double *phi, int max_steps);

/* Forget the magnetic warm start (MagneticField ctor zeroes m_Sol, core/MagneticField.cpp:26). */
SF_EXPORT sf_status sf_magnetic_reset(void *ctx);

/* ----- self-test of the bounded waits (no counterpart in the reference) ------------------------------------
 * The TMA-staged kernels wait on mbarriers with a time limit, after which they record an error and return instead
 * of hanging.  This runs that wait where it cannot succeed: one CTA arms an mbarrier for bytes that no copy
 * delivers (nothing is in flight) and waits at most limit_ms (0 < limit_ms <= 10000); *timed_out = 1 when the
 * wait gave up, *waited_ms (nullable) the time it waited.  The context stays usable afterwards. */
SF_EXPORT sf_status sf_selftest_bounded_wait(void *ctx, double limit_ms, int *timed_out, double *waited_ms);

/* ----- resident inputs --------------------------------------------------------------------------------------
 * The reference's simulation keeps its collider and level set in memory across calls: the collider's face
 * fractions and velocity are computed once per scene (Collider::Finish, core/Collider.cpp:21-45; Velocity is a
 * public member, core/Collider.h:27-28) and both solves of a substep read the same level set m_LevelSet
 * (core/Simulation.cpp:204-226).  These calls keep device copies of them on the context, so that the host entry
 * points need not copy them again on every call:
 *   sf_collider_upload   fractions (and the collider velocity, or NULL = 0) of grid g; a pressure call with
 *                        frac == NULL reads them, and with frac == NULL and solid_vel == NULL also the uploaded
 *                        velocity;
 *   sf_levelset_upload   a cell level set of grid g; a pressure or magnetic call with phi == NULL reads it.
 * Pointers may be host or device memory.  Each call copies on the context's stream and returns once the copy has
 * finished; the copy stays until the next upload or sf_destroy.  A call that passes NULL on a grid of other
 * dimensions, or before any upload, returns SF_NOT_READY. */
SF_EXPORT sf_status sf_collider_upload(void *ctx, const sf_grid *g, const double *const frac[3],
                                       const double *const solid_vel[3]);
SF_EXPORT sf_status sf_levelset_upload(void *ctx, const sf_grid *g, const double *phi);
/* sf_applied_field_prefetch: the applied field hext[3] (host or device face arrays of grid g) of a later magnetic
 * call, copied asynchronously into buffers of the context: the copy starts on a side stream when the next pressure
 * call has enqueued its input copies (so it runs under that solve), or else in the magnetic call; a magnetic call
 * with hext == NULL waits for it and reads it, and so do later ones until the next prefetch.  The arrays must stay
 * unchanged until the first magnetic call that reads them returns.  No counterpart in the reference, whose
 * applied field lives in host memory; this lets its host-pointer callers overlap the copy with the pressure solve.
 * A magnetic call with hext == NULL and no prefetch of its grid returns SF_NOT_READY. */
SF_EXPORT sf_status sf_applied_field_prefetch(void *ctx, const sf_grid *g, const double *const hext[3]);

/* ----- allocation-free residual check ------------------------------------------------------------------------
 * No counterpart in the reference: its solvers allocate freely and report only the residual of their own
 * iterate.  This entry point measures any potential psi (from this library, from the reference's amgcl path, a
 * warm start, ...) against the reference's pinned FDM system (core/MagneticField.cpp:62-118; row 0 is psi_0 = 0,
 * b_0 = 0) and writes, on `stream`, result[0] = ||b - A psi|| / ||b|| (||r|| when b = 0) and result[1] = ||b||.
 * mu and b are formed on the fly from phi, chi, band_width and hext as sf_magnetic_solve forms them.
 *
 * It allocates nothing: no cudaMalloc/cudaFree, no context, no staging copies.  It is for callers that cannot
 * allocate -- a step loop whose device memory is fully reserved by its own pool (an allocation could fail), code
 * that must not stall its other streams (cudaFree synchronises the device, cudaMalloc may), and the reference's
 * own FDM step checking its potential without creating a context (sf_create allocates the solver workspaces).
 * The reduction's scratch is a file-scope device array of about 130 KB per device.
 *
 * All pointers are device pointers on the calling thread's current device; `stream` (NULL = default stream)
 * belongs to that device.  The call is asynchronous: result is valid once the stream reaches it.
 * Limit: ceil(ny/8) * ceil(nz/32) <= SF_NOALLOC_MAX_BLOCKS tiles per x-plane (e.g. ny, nz <= 1024, or ny = 2048
 * with nz = 1024); nx is free.  Larger grids return SF_TOO_LARGE without touching the device.
 * Every call looks up the scratch's address in the current context (cudaGetSymbolAddress, a host-side query), so
 * it stays valid across cudaDeviceReset and context switches.  With lazy module loading (the CUDA default) the
 * first call in a context loads the module that holds the scratch, which needs device memory and is not allowed
 * inside a stream capture: make that first call before the caller reserves its memory pool and before any
 * capture.  Calls that overlap on the GPU (in flight on two streams at once, or from two threads) share the
 * scratch and race: order them on one stream. */
#define SF_NOALLOC_MAX_BLOCKS 8192
SF_EXPORT sf_status sf_magnetic_residual_noalloc(void *stream, const sf_grid *g, const double *phi, double chi,
                                                 double band_width, const double *const hext[3], const double *psi,
                                                 double *result);

#ifdef __cplusplus
}
#endif
#endif /* SFGPU_H */
