// Internal declarations of the GB300 mechanical-path library (not part of the ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "amaru_gpu.h"

#define AMR_MAXN 20     // largest element (HEX20)
#define AMR_MAXIP 27    // largest quadrature (HEX 3x3x3)
#define AMR_NST 14      // IP state fields: sigma[6] eps[6] epa dlambda
#define AMR_ST_SIG 0
#define AMR_ST_EPS 6
#define AMR_ST_EPA 12
#define AMR_ST_DL 13

// Host shape library (shapes.cpp): the library's own statement of Amaru's
// shape functions and Gauss tables, used to build per-shape device tables.
namespace amr {
int shape_npoints(int shape);
int shape_ndim(int shape);
int shape_facet_shape(int shape);
void shape_func(int shape, const double *R, double *N);
void shape_deriv(int shape, const double *R, double *D);  // D[i*ndim+k]
int quadrature(int shape, int nips, double *R, double *w);  // returns count or -1
}  // namespace amr

struct AmrGroup {             // elements sharing (shape, quadrature)
    int shape = 0, nen = 0, nip = 0;
    int64_t first = 0, count = 0;  // range in the sorted element order
    double *tab = nullptr;    // device: [nip][nen*ndim] dN/dR, then [nip] w, then [nip][nen] N
    int epb = 1;              // elements per CTA for the stiffness kernel (autotuned)
    int epb_int = 0;          // elements per CTA for the internal-force kernel (0: by quadrature size)
    // 3-D geometry cache, the same at every assembly (coordinates are fixed): dN/dX as
    // [element][node * 3 + component][IP] and w = detJ * weight * thickness as [element][IP] (FP64)
    double *geo_g = nullptr, *geo_w = nullptr;
};

struct AmrSolveWork;          // solver workspace (solver.cu)
struct AmrBatch;              // independent parts solved together (batch.cu)
struct AmrAmg;                // aggregation multigrid preconditioner (amg.cu)
struct AmrRecovery;           // nodal patch recovery of the IP fields (recovery.cu)

struct amr_model {
    int ndim = 3, B = 3, BB = 9, stressmodel = 0;
    double thickness = 1.0;
    int64_t nnodes = 0, nelems = 0, nip_total = 0;
    std::vector<AmrGroup> groups;
    // host-side copies (sorted element order)
    std::vector<int64_t> perm;      // sorted -> caller element id
    std::vector<int64_t> inv_perm;  // caller element id -> sorted
    std::vector<int64_t> h_conn_ptr, h_ip_ptr, h_kel_ptr;
    std::vector<int32_t> h_conn, h_shape, h_nips;
    std::vector<double> h_coords;
    // device model
    double *coords = nullptr;       // nnodes x 3
    int32_t *conn = nullptr;        // sorted elements, flat
    int64_t *conn_ptr = nullptr;    // nelems+1
    int32_t *mat_type = nullptr;    // sorted
    double *mat_par = nullptr;      // sorted, nelems x 8
    int64_t *ip_ptr = nullptr;      // nelems+1
    int64_t *kel_ptr = nullptr;     // nelems+1 (in blocks: sum nen^2)
    int64_t kel_blocks = 0;
    // node -> (element, local node) incidence, ordered by caller element id
    int64_t *inc_ptr = nullptr;     // nnodes+1
    int64_t *inc = nullptr;         // (sorted elem << 8) | local
    int64_t ninc = 0;
    // node-block sparsity pattern
    int64_t nblocks = 0;
    // component stride of the SoA K64 / K32 (and the cycle's FP16) arrays and length of bcol: nblocks
    // rounded up to a multiple of 8, plus 8, so every component starts on 16 bytes and whole 16-byte
    // groups of 8 blocks (FP16 values, column indices) stay inside
    int64_t bstride = 0;
    int64_t *brow_ptr = nullptr;    // nnodes+1
    int32_t *bcol = nullptr;        // nblocks
    int64_t *contrib_ptr = nullptr; // nblocks+1
    int64_t *contrib = nullptr;     // element block slots, element order
    int64_t ncontrib = 0;
    // the gather's block order: blocks grouped by their number of contributions (ascending, stable), so
    // a warp's lanes loop over equal counts; and the row of each block
    int32_t *gorder = nullptr;      // nblocks
    int32_t *grow = nullptr;        // nblocks
    std::vector<int64_t> h_brow_ptr;
    std::vector<int32_t> h_bcol;
    // values
    double *Kel = nullptr;          // kel_blocks x BB element blocks (staging)
    double *K64 = nullptr;          // SoA [BB][nblocks]
    float *K32 = nullptr;           // SoA [BB][nblocks], Dirichlet-masked
    uint16_t *keep = nullptr;       // nblocks: bit (c*B+d) set if some |Ke| >= eps
    float *Minv32 = nullptr;        // nnodes x BB block-Jacobi inverse (masked)
    double *Minv64 = nullptr;       // nnodes x BB (FP64 block-Jacobi, comparator path)
    bool K_valid = false;
    bool geo_valid = false;         // the groups' geometry caches are built (and no element is inverted)
    bool geo_tried = false;         // a build was attempted (not again after an inverted element)
    // dofs
    int64_t ndofs = 0, nu = 0;
    std::vector<int64_t> h_eq_id;   // nnodes x 3
    int64_t *eq_id = nullptr;       // device nnodes x 3
    uint8_t *free_mask = nullptr;   // nnodes x B : 1 free, 0 prescribed or absent
    int64_t *dof_node = nullptr;    // ndofs: node*B + comp for each eq_id
    bool dofs_set = false;
    // IP states, SoA [AMR_NST][nip_total]
    double *st = nullptr, *stbk = nullptr;
    // element force staging and vectors
    double *Fel = nullptr;          // sum nen*B per element
    int64_t *fel_ptr = nullptr;     // nelems+1 (in doubles)
    // device status: [0] code, [1] first failing element (sorted)
    int32_t *d_status = nullptr;
    int32_t *h_status = nullptr;    // pinned
    // scratch
    double *vtmp[8] = {nullptr};    // node-major FP64 vectors (nnodes*B)
    AmrSolveWork *sw = nullptr;
    AmrBatch *batch = nullptr;
    AmrAmg *amg = nullptr;
    AmrRecovery *rec = nullptr;
    // dynamics: element density (sorted order), the mass matrix on K's pattern and its keep bits
    double *rho = nullptr;
    double *M64 = nullptr;
    uint16_t *Mkeep = nullptr;
    int64_t dofs_version = 0;       // bumped by every amr_set_dofs
    // per-part masks read by the element kernels while a batched stage runs (null otherwise)
    const int32_t *bp_elem_part = nullptr;  // sorted element -> part
    const int32_t *bp_node_part = nullptr;  // node -> part
    const uint8_t *bp_active = nullptr;     // part -> takes part in this Newton iteration
    int32_t *bp_err = nullptr;              // part -> first error code of this iteration
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    bool any_plastic = false;
    int assembly_mode = AMR_ASSEMBLY_FAST;
    int amg_smooth = 1;  // multigrid prolongators: smoothed (1) or the tentative ones (0)
    // the last whole-model static stage's Newton iterations, and the hook after each converged increment
    std::vector<amr_iteration_record> stage_log;
    amr_increment_fn inc_fn = nullptr;
    void *inc_user = nullptr;
};

// helpers
// process-wide count of kernel launches by this library (reported by amr_launch_count)
extern std::atomic<long long> amr_g_launches;
// process-wide count of device allocations and frees by this library (reported by amr_alloc_count)
extern std::atomic<long long> amr_g_allocs;
#define AMR_COUNT(n) amr_g_launches.fetch_add((n), std::memory_order_relaxed)
#define AMR_CUDA(call)                                                                 \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            throw AmrError(AMR_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                              \
    } while (0)

struct AmrError {
    int code;
    std::string msg;
    AmrError(int c, std::string m) : code(c), msg(std::move(m)) {}
};

// Two timing events owned for one scope: destroyed on every exit, an exception included.
struct AmrEventPair {
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    AmrEventPair() {
        const cudaError_t e0 = cudaEventCreate(&t0);
        const cudaError_t e1 = e0 == cudaSuccess ? cudaEventCreate(&t1) : e0;
        if (e1 != cudaSuccess) {
            release();
            throw AmrError(AMR_ECUDA, std::string("cudaEventCreate: ") + cudaGetErrorString(e1));
        }
    }
    ~AmrEventPair() { release(); }
    AmrEventPair(const AmrEventPair &) = delete;
    AmrEventPair &operator=(const AmrEventPair &) = delete;
    void release() {
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        t0 = t1 = nullptr;
    }
};

// Device memory of the library.  Inside a call on a handle (AmrStreamScope, set by every entry point)
// allocations and frees are stream-ordered on that handle's stream, from a library pool per device that
// keeps freed memory for reuse and never makes one stream wait for another's frees: a handle that
// allocates or frees does not synchronise the device, so concurrent handles (served requests) overlap.
// Outside a call, or while the stream is being captured into a graph, they are plain cudaMalloc /
// cudaFree.  Copies between host and library memory are ordered on the handle's stream too (amr_h2d,
// amr_d2h).
extern thread_local cudaStream_t amr_tl_stream;
struct AmrStreamScope {
    cudaStream_t prev;
    explicit AmrStreamScope(cudaStream_t s) : prev(amr_tl_stream) { amr_tl_stream = s; }
    ~AmrStreamScope() { amr_tl_stream = prev; }
    AmrStreamScope(const AmrStreamScope &) = delete;
    AmrStreamScope &operator=(const AmrStreamScope &) = delete;
};
void *amr_raw_alloc(size_t bytes);  // throws AmrError(AMR_ENOMEM)
void amr_raw_free(void *p);
void amr_trim_pool();               // returns the pool's unused memory of the current device

template <class T>
inline void amr_alloc(T **p, size_t n) {
    if (n == 0) n = 1;
    amr_g_allocs.fetch_add(1, std::memory_order_relaxed);
    *p = nullptr;  // a failed allocation leaves nothing for the caller's cleanup to free
    *p = (T *)amr_raw_alloc(n * sizeof(T));
}
template <class T>
inline void amr_free(T *&p) {
    if (p) {
        amr_g_allocs.fetch_add(1, std::memory_order_relaxed);
        amr_raw_free((void *)p);
    }
    p = nullptr;
}
// small pinned host buffers (status and control-block reads), from slabs kept for the process: freeing
// one never synchronises the device
void *amr_pinned_alloc(size_t bytes);
void amr_pinned_free(void *p);
// host <-> library device memory, ordered on the handle's stream; both return once the host side may be
// reused (amr_d2h synchronises the stream)
void amr_h2d(amr_model *m, void *d, const void *h, size_t bytes);
void amr_d2h(amr_model *m, void *h, const void *d, size_t bytes);

// pattern.cu
void amr_build_pattern(amr_model *m);
void amr_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s);  // exclusive, out has n+1
// element.cu
void amr_stiffness(amr_model *m);                       // Kel + gather into K64/K32/Minv
void amr_stiffness_elements(amr_model *m);              // Kel only (element kernels)
void amr_combine_K(amr_model *m, double a1, const double *Ks, double a2);  // K64 = a1 Ks + a2 K64, K32, Minv
void amr_mass(amr_model *m);                            // mount_M: element masses gathered into M64 / Mkeep
// K64 = Ks + s1 M + s2 (alpha M + beta Ks) (Ks may be null: K = 0), then K32, Minv
void amr_dyn_combine(amr_model *m, const double *Ks, double s1, double s2, double alpha, double beta);
void amr_update_elements(amr_model *m, const double *dU_nm, double *dFin_nm);  // node-major device vectors
void amr_apply_dofs(amr_model *m);                      // masks after amr_set_dofs
void amr_loads(amr_model *m, const amr_load *loads, int nloads, double t, double *F_nm);  // F_nm += (device)
int amr_check_status(amr_model *m);                     // reads d_status, resets, returns code
// solver.cu
struct AmrSolveResult {
    int status;
    int iterations, refinements;
    double rel_residual, seconds;
};
// Solves K11 x1 = b1 - K12 x2 on node-major device vectors: x (in: prescribed values at
// prescribed slots; out: free slots), b (free slots), reac (out: K x at prescribed slots).
AmrSolveResult amr_solve_device(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o);
void amr_solver_free(amr_model *m);
// vector helpers (solver.cu)
double amr_norm_inf(amr_model *m, const double *v, const uint8_t *mask_or_null);
void amr_eq_to_nm(amr_model *m, const double *d_eq, double *d_nm);  // scatter eq_id-ordered -> node-major (0 elsewhere)
void amr_nm_to_eq(amr_model *m, const double *d_nm, double *d_eq);
// amg.cu: multigrid preconditioner (structure per DOF numbering, values per assembly)
// CTAs of `threads` threads that `kernel` keeps resident on the current device at once, at most cap_per_sm per
// SM: the grid of a grid-stride kernel, so that its rows are spread over one wave (a partial last wave leaves
// SMs idle).  Cached per kernel and device.
unsigned amr_resident_grid(const void *kernel, int threads, int cap_per_sm);
void amr_amg_prepare(amr_model *m);
void amr_amg_vcycle(amr_model *m, const float *r, float *z);
// rows of the fine level the FP32 cycle skips (bytes per node, 0 = skip; null: none): a batch's finished parts
void amr_amg_set_gate(amr_model *m, const uint8_t *gate);
void amr_amg_set_halt(amr_model *m, const int32_t *halt);
void amr_amg_prepare64(amr_model *m);                           // the same hierarchy in FP64
void amr_amg_vcycle64(amr_model *m, const double *r, double *z);
void amr_amg_invalidate(amr_model *m);
double amr_amg_time_residual(amr_model *m, int reps, bool fp64, double *bytes);
void amr_amg_free(amr_model *m);
// recovery.cu: nodal_patch_recovery (structure once per model, values per call)
void amr_recovery_prepare(amr_model *m);
const std::vector<int32_t> &amr_recovery_codes(amr_model *m);
void amr_recover(amr_model *m, double *d_V);  // device, nnodes x nfields column-major
double amr_recovery_time_fit(amr_model *m, int reps, double *flops, int64_t *n_svd);
void amr_recovery_free(amr_model *m);
// batch.cu: independent parts (contiguous node ranges, no element spanning two)
void amr_batch_set(amr_model *m, int64_t nparts, const int64_t *node_ptr);
void amr_batch_free(amr_model *m);
AmrSolveResult amr_batch_solve(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o);
int amr_batch_stage(amr_model *m, const double *Uex_nm, const double *Fex_nm, const amr_stage_params &p, double *U_nm,
                    double *F_nm, amr_stage_stats *stats);
void amr_batch_part_stats(const amr_model *m, int64_t nparts, amr_stage_stats *out);
void amr_autotune_model(amr_model *m, amr_tuning *out);
// dyn.cu: dyn_stage_solver! on node-major device vectors; boundary values at time t are U0 + t U1, F0 + t F1
int amr_dyn_stage_device(amr_model *m, const double *U0, const double *U1, const double *F0, const double *F1,
                         const amr_dyn_params &p, double *U, double *V, double *A, double *F, amr_stage_stats *stats);
double amr_dyn_time_rhs(amr_model *m, int reps, double *bytes);
// modal.cu: omega (host, nmodes) and P's eigenvectors (device, node-major columns, not normalised)
int amr_modal_device(amr_model *m, const amr_modal_params &p, double *omega, double *d_modes_nm, amr_modal_stats *stats);
// vtu.cpp: save_vtu of the model with the caller's arrays
void amr_vtu_write(amr_model *m, const char *path, const amr_vtu_array *pd, int npd, const amr_vtu_array *cd,
                   int ncd, int nthreads, bool compress);
// stage.cpp-equivalent (capi.cu)
int amr_stage_device(amr_model *m, const double *Uex_nm, const double *Fex_nm, const amr_stage_params &p,
                     double *U_nm, double *F_nm, amr_stage_stats *stats);
