/*
 * amaru_gpu.h -- C ABI of the GB300 (sm_103a) library for Amaru's mechanical
 * hot path: solid-element stiffness and internal-force integration with the
 * constitutive update, global sparse assembly of K and the RHS, and the
 * linear solve K*dU = dR inside the staged Newton loop.
 *
 * Conventions
 *  - Plain C types only; every call returns an int status (AMR_OK == 0,
 *    negative on failure) and never throws across the ABI.  The message of the
 *    last failure on a handle is available from amr_last_error().
 *  - Indices are 0-based int64 (the Julia binding subtracts 1).  Nodal arrays
 *    are node-major with 3 slots per node (x, y, z) even in 2-D.
 *  - The caller owns every host buffer; the library copies inputs in and
 *    results out and keeps no host pointer after a call returns.  Each handle
 *    owns its device memory and one CUDA stream; amr_model_destroy frees both.
 *  - A handle is used by one host thread at a time; different handles may be
 *    used concurrently from different threads.
 *
 * Each entry point names the reference function (Amaru.jl source path:line)
 * whose behaviour it replaces.
 */
#ifndef AMARU_GPU_H
#define AMARU_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes: mirror ReturnStatus (src/tools/returnstatus.jl:1-13) ---- */
#define AMR_OK 0
#define AMR_EINVAL -1       /* bad argument or call order */
#define AMR_ECUDA -2        /* CUDA runtime error */
#define AMR_ENEGJAC -3      /* detJ <= 0 (src/mech/elem/mech-solid.jl:150) */
#define AMR_ERETMAP -4      /* return-mapping failure (src/mech/mat/von-mises.jl:146) */
#define AMR_ENAN -5         /* NaN in K or internal forces (src/mech/mech-solver.jl:142, src/solver.jl:60) */
#define AMR_ESINGULAR -6    /* |U1|max > 1e8 (src/solver.jl:68-71) */
#define AMR_ENOCONV -7      /* Krylov solver did not reach its tolerance / broke down */
#define AMR_ETIMEOUT -8     /* a bounded device wait gave up */
#define AMR_ENOMEM -9       /* device allocation failed or admission refused */
#define AMR_EUNSUPPORTED -10 /* element/material/stress model not on the GPU path */
#define AMR_ESTAGE -11      /* staged Newton loop did not converge (src/mech/mech-solver.jl:478-483) */

/* ---- cell shapes (src/shape/*.jl) ---- */
enum {
    AMR_LIN2 = 1, AMR_LIN3 = 2, AMR_TRI3 = 3, AMR_TRI6 = 4, AMR_QUAD4 = 5, AMR_QUAD8 = 6,
    AMR_QUAD9 = 7, AMR_TET4 = 8, AMR_TET10 = 9, AMR_HEX8 = 10, AMR_HEX20 = 11
};

/* ---- stress models (src/mech/mech-solver.jl:9) ---- */
enum { AMR_D3 = 0, AMR_PLANESTRAIN = 1, AMR_PLANESTRESS = 2, AMR_AXISYMMETRIC = 3 };

/* ---- materials: parameters are 8 doubles per element ----
 * LinearElastic  (src/mech/mat/linear-elastic.jl:12-20):  E, nu
 * VonMises       (src/mech/mat/von-mises.jl:14-27):       E, nu, fy, H
 * DruckerPrager  (src/mech/mat/drucker-prager.jl:15-33):  E, nu, alpha, kappa, H */
enum { AMR_LINEAR_ELASTIC = 0, AMR_VON_MISES = 1, AMR_DRUCKER_PRAGER = 2 };

typedef struct amr_model amr_model;

/* Model description: nodes, MechSolid elements and their materials.
 * Mirrors FEModel(mesh, "tag" => MechSolid => Mat => params, MechContext)
 * (src/fe-model.jl:66-255). */
typedef struct {
    int32_t ndim;            /* 2 or 3 (MechContext.ndim) */
    int32_t stressmodel;     /* AMR_D3, AMR_PLANESTRAIN, AMR_PLANESTRESS */
    double thickness;        /* FEModel thickness (2-D) */
    int64_t nnodes;
    const double *coords;    /* nnodes x 3 */
    int64_t nelems;
    const int32_t *shape;    /* nelems: AMR_* shape code */
    const int32_t *nips;     /* nelems: quadrature key, 0 = shape default (src/element.jl:119-166) */
    const int64_t *conn_ptr; /* nelems + 1 */
    const int64_t *conn;     /* node indices in Amaru's local node order */
    const int32_t *mat_type; /* nelems: AMR_LINEAR_ELASTIC ... */
    const double *mat_params;/* nelems x 8 */
} amr_model_desc;

/* Distributed natural load on facets or element bodies, with its value an
 * affine function of the evaluation point: v = c[0] + c[1] x + c[2] y + c[3] z + c[4] t.
 * Replaces mech_boundary_forces (src/mech/elem/distributed.jl:76-152) and
 * mech_solid_body_forces (:157-217) as called by compute_bc_vals!
 * (src/bc.jl:116-136,175-194). */
enum { AMR_LOAD_FACET = 0, AMR_LOAD_BODY = 1 };
typedef struct {
    int32_t kind;            /* AMR_LOAD_FACET or AMR_LOAD_BODY */
    int32_t dir;             /* 0,1,2 = x,y,z component; 3 = facet normal (tn/qn) */
    int32_t edge_key;        /* 1 for q* keys on edges (thickness 1), 0 for t* / w* keys */
    int32_t facet_shape;     /* facet cell shape (FACET kind) */
    int64_t nitems;          /* number of facets or elements */
    const int64_t *items;    /* FACET: nitems x npoints(facet_shape) node ids; BODY: element ids */
    double coef[5];
} amr_load;

/* Linear-solver options for the Newton corrector solve. */
enum { AMR_SOLVER_MIXED = 0, AMR_SOLVER_FP64 = 1, AMR_SOLVER_AMG = 2, AMR_SOLVER_AMG_FP64 = 3 };
typedef struct {
    int32_t method;          /* AMR_SOLVER_MIXED: FP32 block-Jacobi PCG in FP64 iterative refinement
                                AMR_SOLVER_FP64:  the same block-Jacobi PCG all in FP64 (FP64 matrix,
                                                  block inverses and vectors): MIXED's comparator
                                AMR_SOLVER_AMG:   as MIXED with an aggregation-multigrid V-cycle
                                                  (rigid-body coarse spaces, Chebyshev/block-Jacobi
                                                  smoothing) in place of block-Jacobi
                                AMR_SOLVER_AMG_FP64: the same multigrid PCG all in FP64 (the
                                                  hierarchy built and applied in FP64): AMG's
                                                  comparator */
    double rtol;             /* relative residual ||b - K u|| / ||b|| to reach (default 1e-8) */
    int32_t max_iters;       /* cap on inner Krylov iterations (default 20000) */
    int32_t refine_every;    /* FP64 true-residual refresh interval in inner iterations (default 32) */
} amr_solve_opts;

typedef struct {
    int32_t iterations;      /* Krylov iterations */
    int32_t refinements;     /* FP64 residual refreshes */
    double rel_residual;     /* final ||b - K u|| / ||b|| in FP64 */
    double seconds;          /* device time of the solve */
} amr_solve_stats;

/* Newton solver parameters: mech_solver_params (src/mech/mech-solver.jl:155-168). */
enum { AMR_SCHEME_FE = 0, AMR_SCHEME_ME = 1, AMR_SCHEME_BE = 2, AMR_SCHEME_RALSTON = 3 };
typedef struct {
    double tol, rtol, rspan, dT0, dTmin, dTmax;
    int32_t scheme, maxits, autoinc, nincs, nouts;
    amr_solve_opts linear;
} amr_stage_params;

typedef struct {
    int32_t status;          /* AMR_OK or the failure code */
    int32_t increments;      /* converged increments */
    int32_t iterations;      /* Newton iterations, all increments */
    int32_t krylov_iterations;
    double residue;          /* last Newton residue ||R||inf */
    double T;                /* pseudo-time reached */
    double seconds;          /* device time of the stage (CUDA events on the handle's stream) */
    double solve_seconds;    /* device time spent in the linear solves */
} amr_stage_stats;

/* ---- lifecycle ---- */

/* FEModel construction (src/fe-model.jl:66-255): uploads nodes and elements,
 * sorts elements by (shape, quadrature) for the element kernels and builds
 * the node-block sparsity pattern, the element-entry -> nonzero contribution
 * map and the IP state arrays on the device. */
int amr_model_create(const amr_model_desc *desc, amr_model **out);
int amr_model_destroy(amr_model *m);
/* Copies the last error message of the handle (NUL-terminated). */
int amr_last_error(const amr_model *m, char *buf, size_t n);
/* Message of a failure in amr_model_create (no handle yet). */
const char *amr_create_error(void);

/* DOF numbering from configure_dofs! (src/bc.jl:198-233): eq_id is nnodes x 3
 * (only the first ndim used), -1 for nodes without DOFs; unknown DOFs are
 * numbered 0..nu-1, prescribed ones nu..ndofs-1. */
int amr_set_dofs(amr_model *m, const int64_t *eq_id, int64_t ndofs, int64_t nu);

/* Overrides Young's modulus per element (e.g. a random field). */
int amr_set_youngs(amr_model *m, const double *E);

/* ---- element / assembly operations (the drop-in for mount_K) ---- */

/* Element-stiffness arithmetic of amr_assemble_K.
 * AMR_ASSEMBLY_FAST (default): per node pair, K_ab = lambda T + mu T^T + mu tr(T) I - P
 *   with FMA accumulation; the form the Newton loop uses.
 * AMR_ASSEMBLY_REFERENCE: B^T (D B) in the operation order of elem_stiffness
 *   (src/mech/elem/mech-solid.jl:142-158) without FMA contraction, so entries that
 *   are zero only by cancellation fall under the |Ke_ij| >= eps() rule as the
 *   reference's own arithmetic decides; used to export K in the reference layout. */
enum { AMR_ASSEMBLY_FAST = 0, AMR_ASSEMBLY_REFERENCE = 1 };
int amr_set_assembly(amr_model *m, int32_t mode);

/* Prolongators of the multigrid preconditioner (AMR_SOLVER_AMG, AMR_SOLVER_AMG_FP64).
 * 1 (default): smoothed aggregation, P = (I - 4/(3 lambda) D^-1 A) T on every level but the
 *   coarsest, T the rigid-body tentative prolongator, D the node-block diagonal and lambda the
 *   power-iteration estimate of the largest eigenvalue of D^-1 A; coarse operator P' A P.
 * 0: the tentative prolongators themselves (unsmoothed aggregation); coarse operator T' A T.
 * A change rebuilds the hierarchy at the next multigrid solve. */
int amr_set_amg_smoothing(amr_model *m, int32_t on);

/* mount_K (src/mech/mech-solver.jl:78-110): element stiffness
 * (src/mech/elem/mech-solid.jl:124-166) with the tangent of each IP's current
 * state, deterministic assembly into the device pattern. */
int amr_assemble_K(amr_model *m);
/* Number of stored entries of K in the reference's SparseMatrixCSC after its
 * |Ke_ij| >= eps() drop rule (src/mech/mech-solver.jl:90). */
int amr_get_K_nnz(amr_model *m, int64_t *nnz);
/* K in the reference's layout: CSC over eq_id order (colptr ndofs+1, rowval/nzval nnz). */
int amr_get_K_csc(amr_model *m, int64_t *colptr, int64_t *rowval, double *nzval);

/* update_state!(elems, dU, t) (src/mech/mech-solver.jl:124-144 and
 * update_elem!, src/mech/elem/mech-solid.jl:243-279): trial IP states from the
 * committed ones and dU (ndofs, eq_id order); returns dFin (ndofs). */
int amr_update_state(amr_model *m, const double *dU, double *dFin);
/* StateBk <- State and State <- StateBk (src/mech/mech-solver.jl:333,391,461). */
int amr_state_commit(amr_model *m);
int amr_state_restore(amr_model *m);
/* IP states out (nip_total x 16: sigma[6], eps[6], epa, dlambda, 0, 0) in the
 * caller's element order and IP order; nip_total via amr_get_sizes. */
int amr_get_state(amr_model *m, double *state);
/* IP states in, same layout (copyto! of the IpState arrays, src/ip.jl:22-57): a
 * checkpoint restored, or states set by the caller. */
int amr_set_state(amr_model *m, const double *state);
/* The number of IPs of each element, in the caller's element order: its rows in the state layout
 * above.  A host that moves states between handles over different element sets (a stage's
 * toactivate, src/mech/mech-solver.jl:216-220) locates an element's rows with it. */
int amr_get_elem_nips(const amr_model *m, int32_t *nips);
int amr_get_sizes(const amr_model *m, int64_t *nnodes, int64_t *nelems, int64_t *nip_total, int64_t *nblocks);

/* Distributed loads (compute_bc_vals!, src/bc.jl:116-136,175-194):
 * F (ndofs, eq_id order) += the integrated facet / body forces at time t. */
int amr_assemble_loads(amr_model *m, const amr_load *loads, int32_t nloads, double t, double *F);

/* solve_system!(K, U, F, nu) (src/solver.jl:5-79) on the last assembled K:
 * in: U[nu:] prescribed values, F[:nu] natural values; out: U[:nu] and the
 * reactions F[nu:] = K21 U1 + K22 U2. */
int amr_solve(amr_model *m, double *U, double *F, const amr_solve_opts *opts, amr_solve_stats *stats);

/* mech_stage_solver! (src/mech/mech-solver.jl:186-492) on the device for one
 * stage: Uex / Fex are the stage's essential values and natural loads from
 * get_bc_vals (ndofs, eq_id order).  On return U and F (ndofs) hold the
 * stage's accumulated displacements and internal forces (dof.vals updates,
 * :394-397), IP states are committed. */
int amr_stage_run(amr_model *m, const double *Uex, const double *Fex, const amr_stage_params *p, double *U,
                  double *F, amr_stage_stats *stats);

/* One record per Newton iteration of the last whole-model static stage (amr_stage_run,
 * amr_stage_run_dev), as the reference logs them (mech_stage_solver!, "inc" at
 * src/mech/mech-solver.jl:293-297, "it ... residue" at :352): iterations that end in a
 * system error before their residue is computed are not logged, as there. */
typedef struct {
    int32_t increment;         /* the reference's inc counter: 1-based; a failed increment's number is reused */
    int32_t iteration;         /* Newton iteration within the increment, 1-based */
    int32_t krylov_iterations; /* inner Krylov iterations of this Newton iteration */
    int32_t converged;         /* 1 on the iteration that ended its increment converged */
    double T;                  /* pseudo-time at the start of the increment */
    double dT;                 /* the increment's size */
    double residue;            /* ||R||inf after the iteration */
} amr_iteration_record;
/* Copies min(cap, n) records into rec (may be null with cap 0) and sets *n to the count. */
int amr_get_stage_log(const amr_model *m, amr_iteration_record *rec, int32_t cap, int32_t *n);

/* Hook of the whole-model static stage after every converged increment, where the reference calls
 * update_records!(ana, checkpoint=checkpoint) (src/mech/mech-solver.jl:410-424) to write its output
 * files at checkpoints (nouts) and to update its loggers and monitors.  U and F (ndofs, eq_id order)
 * are the stage's accumulated displacements and internal forces so far (the increments of dof.vals,
 * :394-397), in host memory the library owns for the duration of the call; the handle's IP states
 * are the committed ones and may be read with amr_get_state.  A nonzero return stops the stage with
 * AMR_ESTAGE, as a failed update_records! ends the reference's loop (:421-424).  fn = null clears it.
 * No kernels of the handle are in flight during the call. */
typedef struct {
    double T;                  /* the stage's pseudo-time after this increment */
    int32_t increment;         /* the reference's inc counter */
    int32_t checkpoint;        /* 1 if this increment reached an output time (T > Tcheck - dTmin) */
    int64_t ndofs;
    const double *U, *F;
} amr_increment_info;
typedef int (*amr_increment_fn)(void *user, const amr_increment_info *info);
int amr_set_increment_callback(amr_model *m, amr_increment_fn fn, void *user);

/* amr_solve for callers that cannot allocate GPU memory while they solve (a host
 * application that gives the library a fixed memory budget up front, a real-time
 * loop that must stay out of the CUDA allocator, a memory pool that may not grow).
 * No counterpart in the reference: Amaru allocates freely in solve_system!.
 * Same semantics as amr_solve on the last assembled K of a single model (not a
 * batch of parts: AMR_EUNSUPPORTED), mixed-precision solver only, but d_U and d_F
 * are caller-owned DEVICE buffers of ndofs doubles (eq_id order):
 * in: d_U[nu:] prescribed values, d_F[:nu] natural values; out: d_U[:nu] and the
 * reactions d_F[nu:].  The call allocates nothing: all scratch lives in one static
 * device array of about 11.5 MB, which limits the model to nnodes x ndim <= 262 144
 * (larger models get AMR_EINVAL; use amr_solve).  The array is reserved on a device
 * when the library's solver module is first loaded there (with CUDA's lazy module
 * loading that can be this call's first use) and is held until the process exits:
 * make one warm-up call, or any solve, before entering a region that may not
 * allocate.  The first call on each device also looks up that array's device
 * address (cudaGetSymbolAddress), so make it before any stream capture.  All calls
 * share the one array: calls whose work overlaps on the GPU (other handles, other
 * streams, other threads) race and must be serialized. */
int amr_solve_noalloc(amr_model *m, double *d_U, double *d_F, const amr_solve_opts *opts, amr_solve_stats *stats);

/* amr_stage_run with device-resident vectors: d_Uex, d_Fex, d_U, d_F are device
 * pointers to ndofs doubles in eq_id order (for callers that keep their loads
 * and results on the GPU across stages). */
int amr_stage_run_dev(amr_model *m, const double *d_Uex, const double *d_Fex, const amr_stage_params *p,
                      double *d_U, double *d_F, amr_stage_stats *stats);

/* ---- batches of independent models ----
 * Many independent FE models (each one a call of mech_stage_solver!,
 * src/mech/mech-solver.jl:186-492, on its own FEModel) joined into one handle:
 * part i owns the nodes node_ptr[i] .. node_ptr[i+1]-1 and no element joins two
 * parts.  With parts set, amr_solve runs one persistent kernel in which each
 * part's mixed-precision solve is done by one CTA (relative residual per part),
 * and amr_stage_run / amr_stage_run_dev run each part's own Newton loop and
 * increment control on the device, one Newton iteration of all parts per CUDA
 * graph launch; assembly and internal forces stay one launch for all parts.  A
 * part's result does not depend on the other parts in the batch.
 * nparts = 0 clears the parts. */
int amr_set_parts(amr_model *m, int64_t nparts, const int64_t *node_ptr);
/* Per-part outcome of the last batched stage (nparts entries). */
int amr_get_part_stats(const amr_model *m, int64_t nparts, amr_stage_stats *stats);

/* ---- serving (no counterpart in the reference: Amaru runs one analysis per call) ----
 * A request is one mech_stage_solver! stage (src/mech/mech-solver.jl:186-492) of
 * its own model: the model description, the DOF numbering of configure_dofs!,
 * the stage's essential values and natural loads (get_bc_vals, src/bc.jl:237-249,
 * with distributed loads as amr_load items evaluated at t = 0) and the stage
 * parameters.  The server copies it at submit.  max_active worker slots run
 * admitted requests concurrently, each on its own CUDA stream; requests are
 * admitted in arrival order once a slot is free and amr_estimate_bytes of the
 * request fits in hbm_budget_bytes beside the running ones (continuous
 * batching).  A request's pattern, K, IP states and solution stay on the device
 * across all increments of its stage.  Its result is the one it gets alone. */
typedef struct amr_server amr_server;
typedef struct {
    double hbm_budget_bytes;  /* device memory the admitted requests may hold together */
    int32_t max_active;       /* worker slots: requests on the device at once */
    int32_t pad;
} amr_server_config;
typedef struct {
    amr_model_desc model;
    const int64_t *eq_id;     /* nnodes x 3, as amr_set_dofs */
    int64_t ndofs, nu;
    const double *Uex, *Fex;  /* ndofs each, eq_id order */
    const amr_load *loads;    /* distributed loads added to Fex on the device */
    int32_t nloads, pad;
    amr_stage_params stage;
} amr_request;
typedef struct {
    int32_t status;           /* AMR_OK, AMR_ESTAGE or the error of the request */
    int32_t active_at_admit;  /* requests on the device right after this one was admitted */
    int64_t bytes;            /* admitted footprint (amr_estimate_bytes) */
    double t_submit, t_admit, t_done;  /* seconds since the server was created */
    amr_stage_stats stage;
    double t_stage;           /* host set-up done (model created, DOFs set, loads assembled), stage starts */
    double dev_start, dev_end;/* the stage's span on the request's stream, seconds on the device clock
                                 since the server was created (CUDA events): requests whose spans
                                 intersect ran on the GPU at the same time */
} amr_request_result;
typedef struct {
    int64_t queued, active, peak_active, completed, active_bytes, peak_bytes;
    double seconds;           /* since the server was created */
} amr_server_info;
/* Upper bound of the device bytes one model and one stage of it (mixed-precision
 * solver) allocate. */
int amr_estimate_bytes(const amr_model_desc *desc, int64_t *bytes);
int amr_server_create(const amr_server_config *cfg, amr_server **out);
/* Queues a request (copied); AMR_ENOMEM if it can never fit the budget. */
int amr_server_submit(amr_server *s, const amr_request *req, int64_t *id);
/* Blocks until request id has finished; U, F (ndofs, eq_id order) receive the
 * stage's results as amr_stage_run's; err (may be null) its error message.
 * Returns the request's status.  Each id is waited for once. */
int amr_server_wait(amr_server *s, int64_t id, double *U, double *F, amr_request_result *res, char *err,
                    size_t nerr);
int amr_server_stats(amr_server *s, amr_server_info *st);
/* Finishes the queued and running requests, then stops the slots. */
int amr_server_destroy(amr_server *s);

/* Launch shapes picked by amr_autotune (no counterpart in the reference). */
#define AMR_MAX_TUNED_GROUPS 8
typedef struct {
    int32_t ngroups;                            /* element groups (shape, quadrature) */
    int32_t shape[AMR_MAX_TUNED_GROUPS];
    int32_t stiffness_epb[AMR_MAX_TUNED_GROUPS];  /* elements per CTA, element stiffness */
    int32_t internal_epb[AMR_MAX_TUNED_GROUPS];   /* elements per CTA, internal forces */
    int32_t batch_threads;                      /* threads per CTA of the batched solve */
    int32_t batch_ctas_per_sm;                  /* resident CTAs per SM of the batched solve */
    double stiffness_seconds;                   /* best time of one assembly, all groups */
    double internal_seconds;                    /* best time of one internal-force pass */
} amr_tuning;
/* Times the candidate launch shapes of the element kernels on this model (and of
 * the batched solve when parts are set) and keeps the fastest.  Needs the DOFs
 * set; leaves K, the IP states and the results of earlier calls unchanged. */
int amr_autotune(amr_model *m, amr_tuning *out);

/* ---- diagnostics (no counterpart in the reference) ---- */
/* Average device time of one launch of a hot kernel over `reps` launches,
 * timed with CUDA events on the handle's stream, and its algorithmic bytes
 * per launch.  Needs a preceding amr_assemble_K (and a solve for the SpMV). */
enum { AMR_KERNEL_SPMV32 = 0, AMR_KERNEL_RESIDUAL64 = 1,
       AMR_KERNEL_STIFFNESS = 2 /* the fast element-stiffness kernels (no gather); bytes_per_launch returns their
                                   FP64 operations per assembly instead of bytes */,
       AMR_KERNEL_GATHER = 3,
       AMR_KERNEL_INTERNAL = 4, AMR_KERNEL_AMG_RESIDUAL = 5 /* the multigrid cycle's fine residual; after an AMG solve */,
       AMR_KERNEL_DYN_RHS = 6 /* base + M x + C y of the dynamic Newton loop; after amr_assemble_M */,
       AMR_KERNEL_SPMV64 = 7 /* the all-FP64 PCG's q = K64 p; after an AMR_SOLVER_FP64 solve */,
       AMR_KERNEL_AMG_RESIDUAL64 = 8 /* the FP64 cycle's fine residual; after an AMR_SOLVER_AMG_FP64 solve */ };
int amr_time_kernel(amr_model *m, int32_t kernel, int32_t reps, double *avg_seconds, double *bytes_per_launch);
/* Measured arithmetic peak of the current GPU, the denominator of FP-pipe-bound kernels' rooflines:
 * TFLOP/s of fused multiply-adds in a register-resident kernel (8 independent chains per thread, every
 * SM full), timed with CUDA events.  No counterpart in the reference. */
enum { AMR_PEAK_FP64_FMA = 0, AMR_PEAK_FP32_FMA = 1 };
int amr_measure_peak(int32_t which, double *tflops);
/* Number of kernels this handle has launched since it was created. */
int amr_launch_count(const amr_model *m, int64_t *count);
/* Number of device allocations and frees (cudaMalloc / cudaFree) the library has
 * made in this process, all handles together. */
int amr_alloc_count(int64_t *count);

/* ---- dynamics ----
 * Element density (MechSolid props rho, src/mech/elem/mech-solid.jl:6-29), nelems values in the
 * caller's element order. */
int amr_set_density(amr_model *m, const double *rho);
/* mount_M (src/mech/dyn-solver.jl:71-104) over elem_mass (src/mech/elem/mech-solid.jl:169-205):
 * |M_ij| >= eps() entries summed in element order, on K's block pattern.  Needs amr_set_dofs. */
int amr_assemble_M(amr_model *m);
/* M as CSC (0-based, rows sorted): *nnz always; colptr/rowval/nzval filled when colptr is non-null. */
int amr_get_M_csc(amr_model *m, int64_t *nnz, int64_t *colptr, int64_t *rowval, double *nzval);

/* dyn_solver_params (src/mech/dyn-solver.jl:166-186) and the stage's tspan. */
typedef struct {
    double tol, dTmin, dTmax, rspan;
    double alpha, beta;      /* Rayleigh damping C = alpha M + beta K */
    double tspan;            /* time span of the stage (Stage.tspan), > 0 */
    int32_t maxits, autoinc, nincs, nouts;
    amr_solve_opts linear;   /* the Krylov solve of each Newton iteration */
    /* Seismic input (the sism keywords of dyn_solver_params, src/mech/dyn-solver.jl:182-186, applied as
     * sismic_force, :106-157, at :271-287 and :348-352): while tss <= t <= tss + tds the force M (a(t) e_dir)
     * is added to Fex(t), a(t) linear between the record's samples, spread uniformly over tds after an
     * initial 0.  The reference binds tss, tds, sism_file and sism_dir only as keywords, not in its stage
     * function, which stops there with an undefined-variable error; this is the evident intent. */
    int32_t sism;            /* 1: seismic input on */
    int32_t sism_dir;        /* 0, 1, 2: the x, y, z component (sism_dir "fx"/"ux", "fy", "fz") */
    double tss, tds;         /* start time and duration of the record */
    const double *sism_acc;  /* the record's accelerations in file order, row by row, in model units
                                (the reference multiplies the file's values by 9.81) */
    int64_t sism_n;          /* number of samples */
} amr_dyn_params;

/* dyn_stage_solver! (src/mech/dyn-solver.jl:203-534) of a first stage: M A0 = Fex(0), then
 * Newmark's average-acceleration rule with the reference's Newton loop and increment control.
 * Boundary values at time t: Uex(t) = Uex0 + t Uex1, Fex(t) = Fex0 + t Fex1 (eq_id order, ndofs each;
 * get_bc_vals of affine time functions).  Out (eq_id order, ndofs each, may be null): U (the stage's
 * displacements), V, A, F (TFin, dof.vals[fs]).  AMR_ESTAGE when an increment fails without autoinc
 * or below dTmin with it. */
int amr_dyn_stage_run(amr_model *m, const double *Uex0, const double *Uex1, const double *Fex0, const double *Fex1,
                      const amr_dyn_params *p, double *U, double *V, double *A, double *F, amr_stage_stats *stats);
/* (The stage leaves the pseudo-stiffness in the handle's K storage: amr_assemble_K is needed again
 * before amr_get_K_csc or amr_solve.) */
void amr_default_dyn_params(amr_dyn_params *p);

/* ---- modal analysis ----
 * mech_modal_solver! (src/mech/mech-modal-solver.jl:72-235): the nmodes eigenpairs of smallest
 * magnitude of P = K11 ./ sum(M11, dims=1) (K11, M11 on the unknown DOFs), as Arpack's
 * eigs(P, which=:SM) returns them after the reference's filter: omega = sqrt(lambda) ascending and P's
 * eigenvectors, unit 2-norm, the largest entry positive.  Solved as the symmetric-definite pencil
 * diag(L) phi = (1/lambda) K11 phi by LOBPCG with the multigrid V-cycle as preconditioner.
 * Needs amr_set_dofs and amr_set_density (every element rho > 0). */
typedef struct {
    int32_t nmodes;          /* default 5, at most 42 (a LOBPCG block of at most 64 vectors) */
    int32_t max_iters;       /* LOBPCG iterations (default 1000) */
    double tol;              /* relative residual of every wanted pair (default 1e-7) */
} amr_modal_params;
typedef struct {
    int32_t iterations, block;
    double max_residual, seconds;
} amr_modal_stats;
/* omega: nmodes values; modes: nu x nmodes, column-major, in eq_id order (may be null).  stats are
 * written also when LOBPCG stops without converging (AMR_ENOCONV): its iterations and residual. */
int amr_modal_run(amr_model *m, const amr_modal_params *p, double *omega, double *modes, amr_modal_stats *stats);
void amr_default_modal_params(amr_modal_params *p);

/* ---- VTU output ----
 * save(model, "file.vtu") -> save_vtu (src/mesh/io.jl:167-274, ascii) with the XML writer of
 * src/tools/xml.jl:250-318, byte for byte: the model's points and cells, then the point and cell
 * arrays in the caller's order (update_output_data!'s node_data / elem_data).  The tag columns
 * save_vtu adds for tagged elements (tag-s1, tag-s2, tag) are cell arrays the caller passes. */
enum { AMR_VTU_FLOAT64 = 0, AMR_VTU_INT32 = 1, AMR_VTU_INT64 = 2, AMR_VTU_UINT64 = 3 };
typedef struct {
    const char *name;        /* DataArray Name */
    int32_t type;            /* AMR_VTU_*: element type of data and the DataArray type */
    int32_t ncomp;           /* NumberOfComponents */
    int32_t on_device;       /* data is a device pointer */
    int32_t pad;
    const void *data;        /* nrows x ncomp, column-major (component c of row i at c * nrows + i);
                                nrows = nnodes for point arrays, nelems (caller order) for cell arrays */
} amr_vtu_array;
/* nthreads host threads format the arrays (0: all cores). */
int amr_write_vtu(amr_model *m, const char *path, const amr_vtu_array *point_data, int32_t npoint,
                  const amr_vtu_array *cell_data, int32_t ncell, int32_t nthreads);
/* save_vtu(...; compress=true) (src/mesh/io.jl:119-135,167-274): the same document with every array
 * appended as a zlib block (level 4) in <AppendedData encoding="raw">, blocks compressed by nthreads
 * host threads.  Needs the system zlib (libz.so.1); AMR_EUNSUPPORTED without it. */
int amr_write_vtu_compressed(amr_model *m, const char *path, const amr_vtu_array *point_data, int32_t npoint,
                             const amr_vtu_array *cell_data, int32_t ncell, int32_t nthreads);

/* ---- output recovery ----
 * Nodal values of the IP fields: replaces nodal_patch_recovery (src/fe-model.jl:504-702)
 * as called by update_output_data! (:341-427) and get_node_and_elem_vals (:430-485).
 * Field codes name the keys of ip_state_vals (src/tools/tensors.jl:162-215,
 * src/mech/mat/von-mises.jl:159-168,330-341, src/mech/mat/drucker-prager.jl:152-163):
 * σxx σyy σzz σyz σxz σxy σvm σ1 σ2 σ3 εxx εyy εzz εyz εxz εxy ep epa j1 srj2d.  In an axisymmetric
 * analysis the codes SXX SZZ SXY EXX EZZ EXY carry the keys σrr σtt σry εrr εtt εry. */
enum {
    AMR_FIELD_SXX = 0, AMR_FIELD_SYY = 1, AMR_FIELD_SZZ = 2, AMR_FIELD_SYZ = 3, AMR_FIELD_SXZ = 4,
    AMR_FIELD_SXY = 5, AMR_FIELD_SVM = 6, AMR_FIELD_S1 = 7, AMR_FIELD_S2 = 8, AMR_FIELD_S3 = 9,
    AMR_FIELD_EXX = 10, AMR_FIELD_EYY = 11, AMR_FIELD_EZZ = 12, AMR_FIELD_EYZ = 13, AMR_FIELD_EXZ = 14,
    AMR_FIELD_EXY = 15, AMR_FIELD_EP = 16, AMR_FIELD_EPA = 17, AMR_FIELD_J1 = 18, AMR_FIELD_SRJ2D = 19,
    AMR_NFIELD_CODES = 20
};
/* The recovered fields in the reference's column order (first appearance over the
 * elements): codes[0 .. min(cap, n)) and *nfields = n.  The first call builds the
 * patch structure (outer facets, corner patches, the boundary-patch fallback). */
int amr_recovery_fields(amr_model *m, int32_t *codes, int32_t cap, int32_t *nfields);
/* V (nnodes x nfields, column-major as the reference's V_rec[:, i]) from the handle's
 * current IP states; host buffer. */
int amr_recover_nodal(amr_model *m, double *V);
/* The same into a device buffer, on the handle's stream (synchronised on return). */
int amr_recover_nodal_dev(amr_model *m, double *d_V);
/* Average device time of the patch-fit kernel over reps launches (CUDA events), its
 * algorithmic FP64 operations per launch and the patches that took the SVD path. */
int amr_time_recovery(amr_model *m, int32_t reps, double *avg_seconds, double *flops_per_launch,
                      int64_t *svd_patches);

/* ---- coupled mounts ----
 * hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) for HMSolid elements with a linear
 * elastic skeleton and constant isotropic permeability (LinearElasticSeep), and tm_mount_global_matrices
 * (src/thermomech/thermomech-solver.jl:80-170) for TMSolid elements with a linear elastic skeleton and
 * constant conductivity: G = [K, C; s C', dt H + Cap] with every element entry pushed (no eps() drop) and
 * duplicates summed in the reference's order, and RHS = -dt H phi (+ dt Q for the hydraulic mount).  The
 * handle's elements give the geometry and E, nu (LinearElastic); the scalar field lives on the basic (corner)
 * nodes. */
enum { AMR_COUPLED_HYDRO = 0, AMR_COUPLED_THERMO = 1 };
typedef struct {
    int32_t kind;            /* AMR_COUPLED_HYDRO or AMR_COUPLED_THERMO */
    int32_t pad;
    double gammaw;           /* HYDRO: the analysis' water unit weight (HydromechAnalysis gammaw) */
    double T0;               /* THERMO: the reference temperature T0 in degrees C; C' is scaled by T0 + 273.15 */
    const double *params;    /* nelems x 3, caller's element order.  HYDRO: Biot's alpha, permeability k,
                                storativity S.  THERMO: thermal expansion alpha, conductivity k, rho cv */
} amr_coupled_desc;
/* eq4: nnodes x 4 DOF numbers (ux, uy, uz, and the scalar uw / ut; -1 where a node has none), as
 * configure_dofs! numbers them; phi: ndofs current DOF values (eq order), of which the scalar ones are read
 * (dof.vals[:uw] / dof.vals[:ut]).  *nnz always; with colptr non-null also G in CSC (colptr ndofs+1, rowval /
 * nzval nnz, rows sorted) and rhs (ndofs). */
int amr_coupled_mount(amr_model *m, const amr_coupled_desc *d, const int64_t *eq4, int64_t ndofs, double dt,
                      const double *phi, int64_t *nnz, int64_t *colptr, int64_t *rowval, double *nzval,
                      double *rhs);

/* Default parameter blocks (the reference's KwArgInfo defaults). */
void amr_default_solve_opts(amr_solve_opts *o);
void amr_default_stage_params(amr_stage_params *p);

#ifdef __cplusplus
}
#endif
#endif
