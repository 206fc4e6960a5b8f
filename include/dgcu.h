/*
 * dgcu.h -- C ABI of the GB300-native 2D nodal-DG hot path (libdgcu.so).
 *
 * Drop-in boundary for HopeFOAM's DG Euler right-hand side and SIPG pressure
 * solve.  Every entry point returns an int status (DG_OK or a DG_ERR_* code);
 * no C++ exception crosses this boundary.  A context is used by one host
 * thread at a time and issues all of its GPU work on one CUDA stream.
 *
 * Reference layouts kept at this boundary (paths relative to HopeFOAM-0.1/src/DG):
 *  - state: the conserved fields rho, rhoU (x, y), Ener of
 *    GeometricDofField (fields/GeometricDofField/GeometricDofField.H:301-341),
 *    each K*Np doubles, element-contiguous (dofStart = k*Np), nodes in the
 *    reference order of triangleBaseFunction::initDofLocation
 *    (element/baseFunctions/straightBaseFunctions/triangleBaseFunction/
 *    triangleBaseFunction.C:122-186).  Host arrays are packed as
 *    q[v*K*Np + k*Np + i], v = 0 rho, 1 rhoU.x, 2 rhoU.y, 3 Ener.
 *  - boundary traces: fixed values at the owner's face nodes in
 *    faceToCellIndex order (triangleBaseFunction.C:75-94), as the
 *    fixed-value patch data consumed by dgGaussField::initField
 *    (fields/dgGaussField/dgGaussField.C:240-266).
 */
#ifndef DGCU_H
#define DGCU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
enum {
    DG_OK = 0,
    DG_ERR_ARG = 1,           /* invalid argument or mesh */
    DG_ERR_CUDA = 2,          /* a CUDA call failed */
    DG_ERR_TIMEOUT = 3,       /* a bounded device wait gave up */
    DG_ERR_NOT_CONVERGED = 4, /* iterative solve hit its iteration limit */
    DG_ERR_NONFINITE = 5,     /* NaN/Inf detected */
    DG_ERR_UNSUPPORTED = 6,   /* order / option not built */
    DG_ERR_NOMEM = 7          /* device allocation failed */
};

/* numerical flux (DG/godunovFlux/fluxSchemes/scheme/RoeFlux/RoeFlux.C:46-191
 * for Roe; Lax-Friedrichs/Rusanov for Euler has no reference counterpart) */
enum { DG_FLUX_LF = 0, DG_FLUX_ROE = 1 };

/* arithmetic of the right-hand side */
enum {
    DG_PREC_FP64 = 0,  /* plain FP64 everywhere */
    DG_PREC_SPLIT = 1  /* split-precision tensor-core volume/lift, FP64 state */
};

/* boundary kind per element face */
enum { DG_BC_INTERIOR = 0, DG_BC_FIXED = 1 };

/* preconditioners for dg_pcg_solve */
enum {
    DG_PC_NONE = 0,
    DG_PC_BLOCK_JACOBI = 1,
    DG_PC_LEARNED = 2,
    DG_PC_LEARNED_ONLY = 3,
    DG_PC_MULTILEVEL = 4,
    DG_PC_LEARNED_MULTILEVEL = 5
};

typedef struct dg_ctx dg_ctx;

/* Triangle mesh.  Faces of element k are (v0,v1), (v1,v2), (v2,v0) of its
 * counter-clockwise vertices (dgMesh/dgPolyMesh.C:486-506, :601-613). */
typedef struct dg_mesh_desc {
    int32_t K;             /* number of triangles */
    const int32_t* EToV;   /* K*3 global vertex ids (periodic images share ids) */
    const double* VXY;     /* K*3*2 element vertex coordinates */
    const int32_t* EToE;   /* K*3 neighbour element, -1 on a boundary */
    const int32_t* EToF;   /* K*3 neighbour's local face */
    const int32_t* ROT;    /* K*3 face rotation (firstPointIndex, dgPolyMesh.C:866-893); NULL: from EToV */
    const int32_t* BC;     /* K*3 DG_BC_* kind; NULL: DG_BC_FIXED exactly where EToE < 0 */
} dg_mesh_desc;

typedef struct dg_opts {
    int32_t order;           /* polynomial order N, 1..7 */
    const double* cubature;  /* n_cubature x 3 (r, s, w): triangle rule of strength 3(N+1),
                                (gaussIntegration.C:66, gaussTriangleIntegration.C:48-63) */
    int32_t n_cubature;
    double gamma;            /* ratio of specific heats (transportProperties) */
    void* stream;            /* cudaStream_t to use; NULL: the context creates one */
} dg_opts;

typedef struct dg_info {
    int32_t K, order, Np, Ng, Nfp, Nfq, n_bfaces;
    void* stream;            /* the context's cudaStream_t */
    size_t device_bytes;     /* device memory held by the context */
} dg_info;

typedef struct dg_solve_stats {
    int32_t iterations;
    double rel_residual;     /* final ||b - A x|| / ||b|| */
    double ms;               /* device time of the solve */
} dg_solve_stats;

/* Builds the per-order reference operators and the per-element geometry and
 * connectivity on the device.  Replaces dgMesh::dgMesh (dgMesh/dgMesh.C:71-116)
 * and physicalElementData::initElements
 * (element/physicalElementData/physicalElementData.C:60-161, :228-263). */
int dg_ctx_create(const dg_mesh_desc* mesh, const dg_opts* opts, dg_ctx** out);
int dg_ctx_destroy(dg_ctx* ctx);
int dg_get_info(const dg_ctx* ctx, dg_info* info);
/* Message of the last error on this context (static storage of the context). */
const char* dg_last_error(const dg_ctx* ctx);

/* State transfer (host arrays, reference layout above).  Replaces the
 * GeometricDofField internal fields read/written by the solver loop. */
int dg_upload_state(dg_ctx* ctx, const double* q_host);
int dg_download_state(dg_ctx* ctx, double* q_host);
/* Same with device pointers (reference layout), stream-ordered. */
int dg_upload_state_device(dg_ctx* ctx, const double* q_dev);
int dg_download_state_device(dg_ctx* ctx, double* q_dev);

/* Fixed-value boundary traces, n_bfaces x 4 x Nfp doubles; boundary faces
 * ordered by (k, f).  Replaces setBoundaryValues / fixedValue patch data
 * (tutorials/DG/2D/isentropicVortex/dgEulerFoam/setBoundaryValues.H). */
int dg_set_boundary_traces(dg_ctx* ctx, const double* traces_host);

/* R(q) = M^-1 [ volume(dgc::div + dgc::grad) - surface lift(flux) ] of the
 * current state into rhs_host (reference layout).  Replaces one
 * Equation::evaluate of the three solveEquation calls of dgEulerFoam.C:86-90
 * without the ddt part: Equation/Equation.C:39-75,
 * DG/convectionSchemes/defaultConvectionScheme/defaultConvectionScheme.C:48-129,
 * DG/gradSchemes/defaultGrad/defaultGrad.C:87-166,
 * DG/divSchemes/defaultDivScheme/defaultDivScheme.C:85-166. */
int dg_euler_rhs(dg_ctx* ctx, int flux, int precision, double* rhs_host);

/* Device-pointer, stream-ordered form of dg_euler_rhs: R(q) of the context's
 * state into rhs_dev (4*K*Np doubles on the context's device, reference
 * layout), queued on the context's stream; returns without synchronising.
 * A bounded-wait timeout of the split-precision kernel is reported by the
 * next dg_sync (or stepping call) on the context.  Wall and zero-gradient
 * boundary slots take their traces from the state, as in every stage. */
int dg_euler_rhs_device(dg_ctx* ctx, int flux, int precision, double* rhs_dev);

/* One forward-Euler stage q <- q + dt M^-1 R_weak(q) of the context's state
 * on the device, stream-ordered, no host synchronisation: the work of one
 * dg::solveEquation(dgm::ddt(q) + dgc::div(...)) of the reference's three
 * conserved equations together (Equation/Equation.C:39-75,
 * DG/ddtSchemes/EulerDdtScheme/EulerDdtScheme.C:118-144). */
int dg_forward_euler_stage(dg_ctx* ctx, double dt, int flux, int precision);

/* Waits for the context's queued work; reports a bounded-wait timeout of a
 * split-precision kernel queued by a stream-ordered call (DG_ERR_TIMEOUT). */
int dg_sync(dg_ctx* ctx);

/* nsteps low-storage RK4 steps (5 stages each, coefficients of
 * tutorials/DG/2D/isentropicVortex/dgEulerFoam/createFields.H:119-138). */
int dg_lserk4_step(dg_ctx* ctx, double dt, int nsteps, int flux, int precision);

/* nsteps SSP-RK2 steps exactly as the reference solver's time loop
 * (tutorials/DG/2D/isentropicVortex/dgEulerFoam/dgEulerFoam.C:64-131): each
 * stage is dg::solveEquation(dgm::ddt(q) + R(q)) = q + dt M^-1 R_weak
 * (DG/ddtSchemes/EulerDdtScheme/EulerDdtScheme.C:118-144). */
int dg_ssprk2_step(dg_ctx* ctx, double dt, int nsteps, int flux, int precision);

/* Largest stable time step by the build's CFL rule:
 * dt = cfl * min_k h_k / ((N+1)^2 * max_nodes(|u| + c)), h_k = 2 area / longest edge
 * (the reference uses a fixed dt, controlDict). */
int dg_cfl_dt(dg_ctx* ctx, double cfl, double* dt);

/* Per-element time-step factors: after this call the step of element k in
 * dg_lserk4_step / dg_ssprk2_step / dg_batch_run is dt * dtk_host[k] (K
 * positive values); NULL restores the uniform dt.  Lets one context hold many
 * independent cases (disjoint meshes) that each keep their own CFL step.  No
 * counterpart in the reference (one case per process, fixed deltaT). */
int dg_set_element_dt(dg_ctx* ctx, const double* dtk_host);

/* Batched Euler cases.  A batch holds groups (contexts, typically one per
 * order, each over the disjoint meshes of its cases); dg_batch_run advances
 * every group nsteps LSERK4 steps in one CUDA-graph launch (captured on the
 * first run with these arguments, replayed after).  dg_batch_tune measures
 * launch shapes on the live state (restored afterwards): CTAs per SM of the
 * split kernel where two fit, and three schedules: the groups one after
 * another on the whole GPU, side by side on streams with SM shares
 * proportional to their measured cost, or (split precision, orders <= 6, up
 * to 8 groups) every stage of every group in one persistent mixed-order
 * launch, each group on its SM share; the fastest is kept.  No counterpart in the reference.  The groups must not
 * be used on their own streams while a dg_batch_run is in flight. */
typedef struct dg_batch dg_batch;
typedef struct dg_batch_tuning {
    int32_t concurrent;      /* schedule kept: 0 groups one after another, 1 side by side on streams,
                                2 one mixed-order launch per stage */
    double ms_sequential;    /* per step */
    double ms_concurrent;    /* per step */
    double ms_fused;         /* per step (0: schedule 2 not possible for this batch) */
} dg_batch_tuning;
int dg_batch_create(dg_ctx* const* groups, int n_groups, dg_batch** out);
int dg_batch_destroy(dg_batch* batch);
const char* dg_batch_last_error(const dg_batch* batch);
int dg_batch_tune(dg_batch* batch, double dt, int flux, int precision, int steps_per_trial, dg_batch_tuning* result);
int dg_batch_get_shape(const dg_batch* batch, int group, int* ctas_per_sm, int* sm_budget, int* concurrent);
/* Fixes the schedule (0, 1 or 2 as in dg_batch_tuning.concurrent) without
 * measuring; SM shares from the last tuning, else in proportion to each
 * group's element nodes.  DG_ERR_UNSUPPORTED when schedule 2 is not possible. */
int dg_batch_set_schedule(dg_batch* batch, int schedule, int precision);
int dg_batch_run(dg_batch* batch, double dt, int nsteps, int flux, int precision, double* ms);

/* Symmetric interior-penalty Laplacian of the pressure equation on the
 * context's mesh, penalty tau = tau_coef (N+1)^2 max(sJ/J) per face
 * (tau_coef = 20 is the reference's value,
 * DG/laplacianSchemes/defaultLaplacianScheme/defaultLaplacianScheme.C:114);
 * boundary faces are homogeneous Dirichlet (fixesValue, :157-209).  Builds
 * the reference stiffness parts and the block-Jacobi inverse on the device.
 * Replaces the per-element assembly of laplacianFunc (:63-288) and
 * dgMatrix::assembleMatrix (dgMatrices/dgMatrix/dgMatrix.C:383-438). */
int dg_ipdg_setup(dg_ctx* ctx, double tau_coef);

/* Boundary types of the operator per boundary slot (the context's boundary
 * faces in element, face order): 0 fixesValue (the SIPG penalty and
 * consistency terms, defaultLaplacianScheme.C:157-209), 1 fixesGradient and
 * 2 neither (no operator terms on the face; data enter the right-hand side,
 * :210-220).  Default after dg_ipdg_setup: all 0.  Rebuilds the block-Jacobi
 * inverse. */
int dg_ipdg_set_boundary_types(dg_ctx* ctx, const int* btype);

/* S <- S + alpha M (Helmholtz form of the viscous step, dgChorinFoam.C:92-96:
 * dgm::Sp(U) * g0/(dt nu) == laplacian(U) + ...); alpha = 0 restores the
 * Laplacian.  Rebuilds the block-Jacobi inverse. */
int dg_ipdg_set_mass(dg_ctx* ctx, double alpha);

/* y = S x with S = -A (SPD sign of the reference operator A), matrix-free,
 * FP64; x, y host arrays of K*Np doubles in the reference node order. */
int dg_ipdg_apply(dg_ctx* ctx, const double* x_host, double* y_host);
/* Same on device vectors (K*Np doubles each, reference node order, on the
 * context's device), stream-ordered: queued on the context's stream, no host
 * synchronisation.  The matrix-free apply that replaces the assembled
 * dgLduMatrix / PETSc MatMult of the pressure operator
 * (defaultLaplacianScheme.C:63-288, dgMatrix.C:383-438). */
int dg_ipdg_apply_device(dg_ctx* ctx, const double* x_dev, double* y_dev);

/* Solves S x = b to ||b - S x|| <= rtol ||b|| with preconditioned CG
 * (replaces dgMatrix::solve -> KSPSolve, dgMatrices/dgMatrix/dgMatrix.C:162-283,
 * dgMatrixSolve.C:91-213).  x_host holds the initial guess and receives the
 * solution.  pc: DG_PC_BLOCK_JACOBI, DG_PC_LEARNED (after dg_lpc_*; falls back
 * to block Jacobi), DG_PC_LEARNED_ONLY (no fallback: reports the learned
 * solve's own outcome) or DG_PC_MULTILEVEL (block Jacobi plus a coarse-space
 * correction: continuous piecewise-linear functions on the mesh vertices with
 * the Galerkin operator, one V-cycle over aggregated levels per application;
 * built on first use from the mesh's vertex ids, rebuilt after
 * dg_ipdg_set_boundary_types / dg_ipdg_set_mass; the reference has no
 * counterpart, its solver options are PETSc's) or DG_PC_LEARNED_MULTILEVEL
 * (after dg_lpc_*: the learned local preconditioner in place of block Jacobi,
 * plus the same coarse-space correction).
 * precision DG_PREC_FP64: FP64 operator in every iteration; DG_PREC_SPLIT:
 * FP32-arithmetic operator inside CG with FP64 vectors, dot products and
 * recurrences, the recurrence residual replaced by the true FP64 residual
 * b - S x every 64 iterations.  Either way a convergence claim of the
 * recurrence is confirmed against the true FP64 residual.  The returned
 * rel_residual is the true FP64 residual.  DG_ERR_NOT_CONVERGED when maxit is
 * reached (x_host still receives the last iterate). */
int dg_pcg_solve(dg_ctx* ctx, const double* b_host, double* x_host, double rtol, int maxit, int pc, int precision,
                 dg_solve_stats* stats);
/* Same on device vectors (K*Np doubles each, reference node order, on the
 * context's device): b_dev is read, x_dev holds the initial guess and
 * receives the solution, with no host staging.  The iteration count is not
 * known in advance, so the call synchronises the context's stream between
 * batches of iterations to test convergence (as KSPSolve returns only once
 * converged, dgMatrixSolve.C:114-207), and once at the end. */
int dg_pcg_solve_device(dg_ctx* ctx, const double* b_dev, double* x_dev, double rtol, int maxit, int pc, int precision,
                        dg_solve_stats* stats);

/* Learned element-block preconditioner for dg_pcg_solve (DG_PC_LEARNED).  No
 * counterpart in the reference (its KSP uses jacobi / LU, dgMatrix.C:199-222).
 * z = M(r) = P r + s W2 relu(W1 x / s): P the block-Jacobi inverse, x the
 * block-Jacobi outputs of the element and its three neighbours (neighbours
 * rotated so the shared face is their face 0) and four scaled metrics, s
 * their RMS; W1 (hidden x F), W2 (Np x hidden), F = 4 Np + 4, BF16 for the
 * kernels, FP32 master copies.  The solve is flexible CG; a learned solve
 * whose best residual has not halved within 256 iterations stops early, and
 * when a learned solve does not reach rtol dg_pcg_solve (DG_PC_LEARNED)
 * repeats it with block Jacobi from the same initial guess and reports
 * negative iterations (the block-Jacobi count) and the time of both attempts.
 *   dg_lpc_setup: after dg_ipdg_setup; capacity = training residual vectors
 *     kept on the device; form DG_LPC_SCHWARZ (recommended): the learned
 *     additive-Schwarz preconditioner M r = P r + sum_m G_m^T W^T W G_m r, G_m
 *     the residual on element m and its rotated neighbours, W (hidden x 4 Np,
 *     hidden 32 or 64, N <= 6), SPD by construction (plain CG); the tensor
 *     cores run its local stage at hidden 32.  DG_LPC_SCHWARZ_MLP: the same
 *     gather with a two-layer network of tied weights between, M r = P r +
 *     sum_m G_m^T W^T relu(W G_m r), W (128 x 4 Np, N <= 6) in BF16; every
 *     term is >= 0 against r (r.M(r) > 0), M is not linear, and the solve
 *     uses the flexible beta; its local stage and its training gradient run
 *     as BF16 tensor-core (tcgen05) kernels.  DG_LPC_RELU (the network above)
 *     or DG_LPC_LINEAR (identity activation, no metric features) correct the
 *     block-Jacobi output instead; they are not SPD.  For the two Schwarz
 *     forms the weights are W1 = W only (W2 / gW2 arguments may be NULL);
 *     DG_PC_LEARNED_MULTILEVEL takes DG_LPC_SCHWARZ only.
 *   dg_lpc_add_residual: one residual r = b - S x of the method's own PCG
 *     (host array, reference node order), stored scaled to r.P r = 1.
 *   dg_lpc_train: Adam epochs, one step per stored residual, minimising the
 *     energy loss L(r) = -(r.z)^2 / (z.S z), z = M(r) (the S-norm error
 *     decrease of one optimally scaled step along z, negated, times 2), with
 *     the hand-written BF16 forward/backward kernels (FP32 accumulation).
 *     final_loss / final_loss_bj: mean L over the stored residuals with the
 *     network and with block Jacobi alone (more negative is better).
 *   dg_lpc_loss: L(r) for one host residual, with and without the network.
 *   dg_lpc_energy_gradients: dL/dW1, dL/dW2 and L for one host residual.
 *   dg_lpc_get/set_weights: FP32 W1 (hidden x F), W2 (Np x hidden) row-major
 *     (set also resets the Adam moments).
 *   dg_lpc_gradients: gradients of the mean-squared loss
 *     sum_b 0.5 ||W2 h_b - t_b||^2 / B of the network alone on a host batch
 *     (X: B x F, T: B x Np; X rounded to BF16 on the device; loss reported
 *     per output), a direct check of the backward kernels.
 *   dg_lpc_apply: z = M(r) once (host arrays of K*Np doubles, reference node
 *     order). */
enum { DG_LPC_RELU = 0, DG_LPC_LINEAR = 1, DG_LPC_SCHWARZ = 2, DG_LPC_SCHWARZ_MLP = 3 };
int dg_lpc_setup(dg_ctx* ctx, int hidden, unsigned long long seed, int capacity, int form);
/* Activation of DG_LPC_SCHWARZ_MLP: max(h, slope h), slope in [0, 1]
 * (default 0, relu; 1 makes M linear and symmetric). */
int dg_lpc_set_slope(dg_ctx* ctx, double slope);
/* Training objective of DG_LPC_SCHWARZ: on != 0 trains the local stage for
 * DG_PC_LEARNED_MULTILEVEL (the loss takes z = the learned local stage plus
 * the coarse-space correction of DG_PC_MULTILEVEL, which is built here if
 * needed); 0 (default) for the learned stage alone. */
int dg_lpc_set_coarse(dg_ctx* ctx, int on);
int dg_lpc_add_residual(dg_ctx* ctx, const double* r_host);
int dg_lpc_train(dg_ctx* ctx, int epochs, double lr, unsigned long long seed, double* final_loss,
                 double* final_loss_bj);
int dg_lpc_loss(dg_ctx* ctx, const double* r_host, double* loss, double* loss_bj);
int dg_lpc_energy_gradients(dg_ctx* ctx, const double* r_host, float* gW1, float* gW2, double* loss);
int dg_lpc_get_weights(dg_ctx* ctx, float* W1, float* W2);
int dg_lpc_set_weights(dg_ctx* ctx, const float* W1, const float* W2);
int dg_lpc_gradients(dg_ctx* ctx, const float* X_host, const float* T_host, int B, float* gW1, float* gW2,
                     double* loss);
int dg_lpc_apply(dg_ctx* ctx, const double* r_host, double* z_host);

/* Allocation-free right-hand side.  No counterpart in the reference: it is an
 * addition for callers that must not allocate device memory while they run
 * (inside a CUDA stream capture, under an application-owned memory pool, or
 * in a loop with a real-time budget).  Same result as dg_euler_rhs with
 * DG_PREC_FP64 for the state q_dev, but state and output are device arrays in
 * the reference layout (q_dev, rhs_dev: 4*K*Np doubles each, on the context's
 * device, which must be current: DG_ERR_ARG otherwise).  Boundary traces:
 * fixed-value slots use the traces set on the context; wall and zero-gradient
 * slots are recomputed from q_dev into the context's trace buffer (as
 * dg_euler_rhs does from the context's state).  The call makes no allocation:
 * its scratch is a fixed
 * array in device global memory, 2 x DG_NOALLOC_MAX_VALUES doubles (8 MiB),
 * kept by every GPU that loads the library until the process exits.  Sizes
 * with 4*K*Np > DG_NOALLOC_MAX_VALUES are rejected with DG_ERR_ARG.  The
 * first call on a device looks up the scratch address; make that first call
 * before any stream capture starts.  Work is queued on the context's stream
 * and the call returns without synchronising.  All calls share the scratch
 * array, which keeps the last call's contents; calls whose GPU work overlaps
 * in time (other streams, other contexts on the same device) race on it. */
#define DG_NOALLOC_MAX_VALUES 524288
int dg_euler_rhs_noalloc(dg_ctx* ctx, const double* q_dev, double* rhs_dev, int flux);

/* ---------------------------------------------------------------------------
 * Slope limiter and the limited SSP-RK2 step of the reference's Euler solver
 * for flows with shocks (DG/DG/godunovFlux/limiteSchemes/scheme/Trianglelimite/
 * Trianglelimite.C:61-861 via godunovScheme::limite;
 * tutorials/DG/2D/doubleMach/dgEulerFoam/dgEulerFoam.C:50-101).
 *
 * dg_set_boundary_kinds: per boundary slot 0 fixed value, 1 reflective wall
 * (the boundary value mirrors the interior trace's momentum,
 * reflectiveDgPatchField.C:79-111; the limiter's ghost cell removes the normal
 * momentum), 2 other (the boundary value stays as set; the limiter's ghost
 * cell copies the owner), 3 zero gradient (the boundary value is the interior
 * trace, re-evaluated with the walls'; the ghost cell copies the owner); gref (may be
 * NULL = itself) per slot: the slot whose first boundary value a fixed-value
 * ghost cell takes (the reference uses the first value of the slot's patch).
 * dg_limit: the limiter on the current state with the current boundary traces.
 * dg_reflect_boundary_traces: the reflective and zero-gradient slots' traces
 * from the state.  Once kinds are set, dg_lserk4_step and dg_ssprk2_step also
 * take those slots' traces from each stage's input state (the reference
 * corrects its boundary conditions after every equation solve,
 * dgMatrixSolve.C:209); fixed-value and other slots keep the traces as set.
 * dg_limited_ssprk2_step: one step (stage, walls, limiter, stage, walls,
 * average with the boundary values, limiter, walls); bdata [nb][4][Nfp] holds
 * this step's values of the fixed-value slots (setBoundaryValues.H).
 * dg_set_node_locations: node locations x, y ([K][Np] each, reference node
 * order) for the code that reads them (the limiter's cell geometry), as the
 * nodes next to curved arc patches are moved after the element metrics are
 * built (physicalElementData.C:186-224); the operators keep the straight
 * element's metrics, as the reference's do.  Default: the straight element's
 * nodes. */
int dg_set_node_locations(dg_ctx* ctx, const double* x, const double* y);
int dg_set_boundary_kinds(dg_ctx* ctx, const int* kinds, const int* gref);
int dg_limit(dg_ctx* ctx);
int dg_reflect_boundary_traces(dg_ctx* ctx);
int dg_limited_ssprk2_step(dg_ctx* ctx, double dt, const double* bdata, int flux, int precision);

/* ---------------------------------------------------------------------------
 * Incompressible Navier-Stokes: the velocity-correction (Chorin) step of
 * tutorials/DG/2D/pearsonVortex/dgChorinFoam/dgChorinFoam.C:63-109, FP64 on
 * the device (one step = convection, pressure Poisson solve, velocity
 * correction, Helmholtz solve per velocity component; BDF1/EXT1 on the first
 * step after dg_ins_set_state, BDF2/EXT2 after).
 *
 * Boundary slots are the mesh's boundary faces in element, face order.  Per
 * slot u_kind: 0 fixedValue, 1 fixedGradient; p_kind: 0 fixedValue,
 * 2 zeroGradient.  The pressure Neumann data of pEqnCorrect.H apply on the
 * u_kind 0 slots.  State arrays: U as 2 x K x Np (x then y component), p as
 * K x Np, reference node order. */
typedef struct dg_ins dg_ins;

/* Boundary data of one step, host arrays per slot in face-node order
 * (the order of dg_set_boundary_traces): u_value [nb][2][Nfp] (read on u_kind
 * 0 slots), u_gradient [nb][2][Nfp] (n.grad U, u_kind 1), p_value [nb][Nfp]
 * (p_kind 0), p_neumann_extra [nb][Nfp] (added to n.(N + nu curl curl U) in
 * the pressure Neumann data, u_kind 0: the reference case's n.dU/dt term);
 * p_data_scale / u_data_scale multiply the Laplacians' boundary-data terms
 * (the reference case's paraT3 / paraT4 of bCorrectEquation.H). */
typedef struct {
    const double* u_value;
    const double* u_gradient;
    const double* p_value;
    const double* p_neumann_extra;
    double p_data_scale;
    double u_data_scale;
} dg_ins_bdata;

typedef struct {
    int iterations_p;
    int iterations_u[2];
    double rel_residual_p;
    double rel_residual_u;
    double ms;  /* device time of the step */
} dg_ins_stats;

int dg_ins_create(const dg_mesh_desc* mesh, const dg_opts* opts, const int* u_kind, const int* p_kind, double nu,
                  double dt, double tau_coef, dg_ins** out);
int dg_ins_destroy(dg_ins* ins);
const char* dg_ins_last_error(const dg_ins* ins);
int dg_ins_set_state(dg_ins* ins, const double* U_host, const double* p_host);
int dg_ins_get_state(dg_ins* ins, double* U_host, double* p_host);
/* one step; the linear solves stop at rtol (relative residual) */
int dg_ins_step(dg_ins* ins, const dg_ins_bdata* bd, double rtol, int maxit, dg_ins_stats* stats);
/* arithmetic of the step's linear solves: DG_PREC_FP64 (default) or
 * DG_PREC_SPLIT (FP32 operator on FP64 element offsets, FP64 vectors and
 * recurrences, the same rtol on the true FP64 residual) */
int dg_ins_set_precision(dg_ins* ins, int precision);
/* one operator of the step alone (parity tests): op 0 div(U (x) U) with the
 * u_value of bd on u_kind 0 slots, 1 div U, 2 grad p, 3 curl curl U */
int dg_ins_operator(dg_ins* ins, int op, const dg_ins_bdata* bd, const double* in_host, double* out_host);

/* Host-only (no GPU needed): the reference-element operators this library
 * builds for order N from a cubature rule, in the reference node order.
 * Arrays are caller-allocated: r, s [Np]; Dr, Ds, Mref [Np*Np] (row-major);
 * Vg [Ng*Np]; If [Nfq*Nfp]; any may be NULL.  Replaces the operator set of
 * triangleBaseFunction (triangleBaseFunction.C:46-71, :236-246) and
 * gaussTriangleIntegration (gaussTriangleIntegration.C:45-97). */
int dg_reference_operators(int order, const double* cubature, int n_cubature, double* r, double* s, double* Dr,
                           double* Ds, double* Vg, double* If, double* Mref);

#ifdef __cplusplus
}
#endif

#endif /* DGCU_H */
