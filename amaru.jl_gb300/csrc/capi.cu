// C ABI of the library (include/amaru_gpu.h): model lifecycle, DOFs, assembly,
// parity export, state update, linear solve, loads and the staged Newton
// driver (mech_stage_solver!, src/mech/mech-solver.jl:186-492) whose vectors
// all stay on the device.
#include <algorithm>
#include <map>
#include <mutex>
#include <unordered_set>
#include <cmath>
#include <cstring>
#include <numeric>
#include <optional>
#include <stdexcept>

#include "amr_internal.h"

std::atomic<long long> amr_g_launches{0};
std::atomic<long long> amr_g_allocs{0};
thread_local cudaStream_t amr_tl_stream = nullptr;

// ---------------------------------------------------------------------------
// device memory: stream-ordered allocation from a library pool per device
// ---------------------------------------------------------------------------
namespace {
std::mutex g_mem_mu;
std::map<int, cudaMemPool_t> g_pools;          // device -> the library's pool
std::unordered_set<void *> g_pool_ptrs;        // live allocations taken from a pool

cudaMemPool_t library_pool() {
    int dev = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mem_mu);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) return it->second;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    AMR_CUDA(cudaMemPoolCreate(&pool, &props));
    // keep freed memory for the next allocation; never let a stream wait on another stream's frees
    uint64_t keep = UINT64_MAX;
    int no = 0;
    AMR_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    AMR_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no));
    g_pools[dev] = pool;
    return pool;
}
}  // namespace

void *amr_raw_alloc(size_t bytes) {
    void *p = nullptr;
    cudaError_t e;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (amr_tl_stream && cudaStreamIsCapturing(amr_tl_stream, &cap) == cudaSuccess &&
        cap == cudaStreamCaptureStatusNone) {
        e = cudaMallocFromPoolAsync(&p, bytes, library_pool(), amr_tl_stream);
        if (e == cudaSuccess) {
            std::lock_guard<std::mutex> lk(g_mem_mu);
            g_pool_ptrs.insert(p);
        }
    } else {
        e = cudaMalloc(&p, bytes);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw AmrError(AMR_ENOMEM, std::string("device allocation of ") + std::to_string(bytes) + " bytes: " +
                                       cudaGetErrorString(e));
    }
    return p;
}

void amr_raw_free(void *p) {
    bool pooled;
    {
        std::lock_guard<std::mutex> lk(g_mem_mu);
        pooled = g_pool_ptrs.erase(p) > 0;
    }
    if (!pooled) {
        cudaFree(p);
        return;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (amr_tl_stream && cudaStreamIsCapturing(amr_tl_stream, &cap) == cudaSuccess &&
        cap == cudaStreamCaptureStatusNone) {
        cudaFreeAsync(p, amr_tl_stream);
    } else {  // no stream to order the free on: wait for the device, then free
        cudaDeviceSynchronize();
        cudaFreeAsync(p, 0);
        cudaStreamSynchronize(0);
    }
}

void amr_trim_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    std::lock_guard<std::mutex> lk(g_mem_mu);
    auto it = g_pools.find(dev);
    if (it != g_pools.end()) cudaMemPoolTrimTo(it->second, 0);
}

namespace {
constexpr size_t kPinnedSlot = 256, kPinnedSlab = 256;  // slot bytes, slots per slab
std::vector<void *> g_pinned_free;
}  // namespace

void *amr_pinned_alloc(size_t bytes) {
    if (bytes > kPinnedSlot) throw AmrError(AMR_EINVAL, "pinned buffer larger than a slot");
    std::lock_guard<std::mutex> lk(g_mem_mu);
    if (g_pinned_free.empty()) {
        void *slab = nullptr;
        AMR_CUDA(cudaMallocHost(&slab, kPinnedSlot * kPinnedSlab));
        for (size_t i = 0; i < kPinnedSlab; i++) g_pinned_free.push_back((char *)slab + i * kPinnedSlot);
    }
    void *p = g_pinned_free.back();
    g_pinned_free.pop_back();
    return p;
}

void amr_pinned_free(void *p) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_mem_mu);
    g_pinned_free.push_back(p);
}

void amr_h2d(amr_model *m, void *d, const void *h, size_t bytes) {
    if (!bytes) return;
    AMR_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, m->stream));
    AMR_CUDA(cudaStreamSynchronize(m->stream));
}

void amr_d2h(amr_model *m, void *h, const void *d, size_t bytes) {
    if (!bytes) return;
    AMR_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, m->stream));
    AMR_CUDA(cudaStreamSynchronize(m->stream));
}
double amr_time_solver_kernel(amr_model *m, int which, int reps);

namespace {

thread_local std::string g_create_error;

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// elementwise ops on node-major vectors
enum VecOp {
    V_SET_AXPBY = 0,   // o = a x + b y
    V_MASK_FREE = 1,   // o = x at free slots, 0 at prescribed
    V_MASK_PRESC = 2,  // o = x at prescribed slots, 0 at free
    V_PRESC_AX = 3,    // o = a x at prescribed slots, 0 at free
};

__global__ void k_vec(int64_t n, int op, double a, const double *x, double b, const double *y, double *o,
                      const uint8_t *fm) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    switch (op) {
    case V_SET_AXPBY: o[i] = a * x[i] + (y ? b * y[i] : 0.0); break;
    case V_MASK_FREE: o[i] = fm[i] ? x[i] : 0.0; break;
    case V_MASK_PRESC: o[i] = fm[i] ? 0.0 : x[i]; break;
    case V_PRESC_AX: o[i] = fm[i] ? 0.0 : a * x[i]; break;
    }
}

__global__ void k_free_mask(int64_t nnodes, int B, const int64_t *eq_id, int64_t nu, uint8_t *fm) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * B) return;
    int64_t e = eq_id[(t / B) * 3 + t % B];
    fm[t] = (e >= 0 && e < nu) ? 1 : 0;
}

void vec(amr_model *m, int op, double a, const double *x, double b, const double *y, double *o) {
    int64_t n = m->nnodes * m->B;
    k_vec<<<nblk(n, 256), 256, 0, m->stream>>>(n, op, a, x, b, y, o, m->free_mask);
    AMR_COUNT(1);
}

void upload(void *d, const void *h, size_t bytes, cudaStream_t s) {
    AMR_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
}

void check_dofs(amr_model *m) {
    if (!m->dofs_set) throw AmrError(AMR_EINVAL, "amr_set_dofs must be called first");
}

int fail(amr_model *m, const AmrError &e) {
    if (m) m->err = e.msg;
    return e.code;
}

template <class F>
int guarded(amr_model *m, F f) {
    if (!m) return AMR_EINVAL;
    AmrStreamScope scope(m->stream);  // the call's allocations and frees are ordered on the handle's stream
    try {
        m->err.clear();
        return f();
    } catch (const AmrError &e) {
        return fail(m, e);
    } catch (const std::exception &e) {
        return fail(m, AmrError(AMR_EINVAL, e.what()));
    }
}

// eq_id-ordered host array -> node-major device vector (0 where no DOF)
void eq_host_to_nm(amr_model *m, const double *h, double *d_nm) {
    double *d_eq;
    amr_alloc(&d_eq, m->ndofs);
    upload(d_eq, h, m->ndofs * sizeof(double), m->stream);
    amr_eq_to_nm(m, d_eq, d_nm);
    AMR_CUDA(cudaStreamSynchronize(m->stream));
    amr_free(d_eq);
}

void nm_to_eq_host(amr_model *m, const double *d_nm, double *h) {
    double *d_eq;
    amr_alloc(&d_eq, m->ndofs);
    amr_nm_to_eq(m, d_nm, d_eq);
    AMR_CUDA(cudaMemcpyAsync(h, d_eq, m->ndofs * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    AMR_CUDA(cudaStreamSynchronize(m->stream));
    amr_free(d_eq);
}

void assemble(amr_model *m) {
    check_dofs(m);
    amr_stiffness(m);
    int rc = amr_check_status(m);
    if (rc == AMR_ENEGJAC) throw AmrError(rc, "Negative Jacobian determinant in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
    if (rc == AMR_ENAN) throw AmrError(rc, "NaN values in coefficients matrix");
    if (rc) throw AmrError(rc, "assembly failed");
    m->K_valid = true;
}

double round_sig3(double x) {
    if (x == 0.0 || !std::isfinite(x)) return x;
    double e = std::floor(std::log10(std::fabs(x)));
    double sc = std::pow(10.0, 2.0 - e);
    return std::round(x * sc) / sc;
}

}  // namespace

// ---------------------------------------------------------------------------
unsigned amr_resident_grid(const void *kernel, int threads, int cap_per_sm) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int64_t>, unsigned> cache;
    int dev = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    const int64_t key = ((int64_t)dev << 32) | ((int64_t)threads << 8) | (int64_t)(cap_per_sm & 0xff);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find({kernel, key});
    if (it != cache.end()) return it->second;
    int sms = 0, per = 0;
    AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    AMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0));
    const unsigned g = (unsigned)sms * (unsigned)std::max(1, std::min(per, cap_per_sm));
    cache[{kernel, key}] = g;
    return g;
}

extern "C" {

const char *amr_create_error(void) { return g_create_error.c_str(); }

void amr_default_solve_opts(amr_solve_opts *o) {
    o->method = AMR_SOLVER_MIXED;
    o->rtol = 1e-8;
    o->max_iters = 20000;
    o->refine_every = 32;
}

void amr_default_stage_params(amr_stage_params *p) {
    p->tol = 0.01; p->rtol = 0.01; p->rspan = 0.01; p->dT0 = 0.01; p->dTmin = 1e-7; p->dTmax = 0.1;
    p->scheme = AMR_SCHEME_FE; p->maxits = 5; p->autoinc = 0; p->nincs = 1; p->nouts = 0;
    amr_default_solve_opts(&p->linear);
}

int amr_model_create(const amr_model_desc *d, amr_model **out) {
    g_create_error.clear();
    if (!d || !out) { g_create_error = "null argument"; return AMR_EINVAL; }
    *out = nullptr;
    amr_model *m = new amr_model();
    std::optional<AmrStreamScope> scope;  // set once the handle's stream exists
    try {
        if (d->ndim != 2 && d->ndim != 3) throw AmrError(AMR_EINVAL, "ndim must be 2 or 3");
        if (d->stressmodel < 0 || d->stressmodel > 3) throw AmrError(AMR_EINVAL, "bad stress model");
        if (d->ndim == 3 && d->stressmodel != AMR_D3) throw AmrError(AMR_EINVAL, "3-D analyses use the d3 stress model");
        if (d->nnodes <= 0 || d->nelems <= 0) throw AmrError(AMR_EINVAL, "empty model");
        if (d->nnodes >= INT32_MAX) throw AmrError(AMR_EUNSUPPORTED, "more than 2^31 nodes");
        if (!d->coords || !d->shape || !d->nips || !d->conn_ptr || !d->conn || !d->mat_type || !d->mat_params)
            throw AmrError(AMR_EINVAL, "null array in the model description");
        // 2-D analyses need thickness > 0: the condition the reference's analysis argument tables state
        // (src/hydromech/hydromech-solver.jl:8; the mechanical one is commented out, src/mech/dyn-solver.jl:8)
        if (d->ndim == 2 && !(d->thickness > 0.0)) throw AmrError(AMR_EINVAL, "thickness must be > 0");
        m->ndim = d->ndim; m->B = d->ndim; m->BB = d->ndim * d->ndim;
        m->stressmodel = d->stressmodel; m->thickness = d->thickness;
        m->nnodes = d->nnodes; m->nelems = d->nelems;
        // validate elements and group them by (shape, quadrature), stable; no device call before the
        // description is known to be valid, so that a refused description touches no GPU
        std::vector<int> nq(d->nelems);
        for (int64_t e = 0; e < d->nelems; e++) {
            int sh = d->shape[e];
            int np = amr::shape_npoints(sh);
            if (np <= 0 || amr::shape_ndim(sh) != d->ndim) throw AmrError(AMR_EUNSUPPORTED, "element " + std::to_string(e) + ": shape not a bulk cell of this dimension");
            if (d->conn_ptr[e + 1] - d->conn_ptr[e] != np) throw AmrError(AMR_EINVAL, "element " + std::to_string(e) + ": wrong node count");
            for (int64_t p = d->conn_ptr[e]; p < d->conn_ptr[e + 1]; p++)
                if (d->conn[p] < 0 || d->conn[p] >= d->nnodes) throw AmrError(AMR_EINVAL, "element " + std::to_string(e) + ": node index out of range");
            double R[64 * 3], w[64];
            nq[e] = amr::quadrature(sh, d->nips[e], R, w);
            if (nq[e] <= 0) throw AmrError(AMR_EINVAL, "element " + std::to_string(e) + ": unsupported number of integration points");
            int mt = d->mat_type[e];
            if (mt < 0 || mt > 2) throw AmrError(AMR_EUNSUPPORTED, "unsupported material");
            if (mt != AMR_LINEAR_ELASTIC) m->any_plastic = true;
            const double *p = d->mat_params + 8 * e;
            if (!(p[0] > 0.0) || !(p[1] >= 0.0 && p[1] < 0.5)) throw AmrError(AMR_EINVAL, "element " + std::to_string(e) + ": E > 0 and 0 <= nu < 0.5 required");
        }
        m->perm.resize(d->nelems);
        std::iota(m->perm.begin(), m->perm.end(), 0);
        std::stable_sort(m->perm.begin(), m->perm.end(), [&](int64_t a, int64_t b) {
            if (d->shape[a] != d->shape[b]) return d->shape[a] < d->shape[b];
            return nq[a] < nq[b];
        });
        m->inv_perm.resize(d->nelems);
        for (int64_t s = 0; s < d->nelems; s++) m->inv_perm[m->perm[s]] = s;
        m->h_conn_ptr.resize(d->nelems + 1);
        m->h_ip_ptr.resize(d->nelems + 1);
        m->h_kel_ptr.resize(d->nelems + 1);
        std::vector<int64_t> fel(d->nelems + 1);
        m->h_shape.resize(d->nelems);
        m->h_nips.resize(d->nelems);
        std::vector<int32_t> mt(d->nelems);
        std::vector<double> mp(8 * d->nelems);
        m->h_conn_ptr[0] = m->h_ip_ptr[0] = m->h_kel_ptr[0] = fel[0] = 0;
        m->h_conn.clear();
        for (int64_t s = 0; s < d->nelems; s++) {
            int64_t e = m->perm[s];
            int np = amr::shape_npoints(d->shape[e]);
            for (int64_t p = d->conn_ptr[e]; p < d->conn_ptr[e + 1]; p++) m->h_conn.push_back((int32_t)d->conn[p]);
            m->h_conn_ptr[s + 1] = m->h_conn_ptr[s] + np;
            m->h_ip_ptr[s + 1] = m->h_ip_ptr[s] + nq[e];
            m->h_kel_ptr[s + 1] = m->h_kel_ptr[s] + (int64_t)np * np;
            fel[s + 1] = fel[s] + (int64_t)np * d->ndim;
            m->h_shape[s] = d->shape[e];
            m->h_nips[s] = nq[e];
            mt[s] = d->mat_type[e];
            std::memcpy(&mp[8 * s], d->mat_params + 8 * e, 8 * sizeof(double));
            if (s == 0 || m->groups.back().shape != d->shape[e] || m->groups.back().nip != nq[e]) {
                AmrGroup g;
                g.shape = d->shape[e]; g.nen = np; g.nip = nq[e]; g.first = s; g.count = 0;
                g.epb = (np >= 20) ? 1 : (np >= 10 ? 4 : 6);
                m->groups.push_back(g);
            }
            m->groups.back().count++;
        }
        m->nip_total = m->h_ip_ptr.back();
        m->kel_blocks = m->h_kel_ptr.back();
        AMR_CUDA(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
        AMR_CUDA(cudaEventCreate(&m->ev0));
        AMR_CUDA(cudaEventCreate(&m->ev1));
        cudaStream_t s = m->stream;
        scope.emplace(s);
        m->h_coords.assign(d->coords, d->coords + 3 * d->nnodes);
        amr_alloc(&m->coords, 3 * d->nnodes);
        upload(m->coords, d->coords, 3 * d->nnodes * sizeof(double), s);
        amr_alloc(&m->conn, m->h_conn.size());
        upload(m->conn, m->h_conn.data(), m->h_conn.size() * sizeof(int32_t), s);
        amr_alloc(&m->conn_ptr, d->nelems + 1);
        upload(m->conn_ptr, m->h_conn_ptr.data(), (d->nelems + 1) * sizeof(int64_t), s);
        amr_alloc(&m->ip_ptr, d->nelems + 1);
        upload(m->ip_ptr, m->h_ip_ptr.data(), (d->nelems + 1) * sizeof(int64_t), s);
        amr_alloc(&m->kel_ptr, d->nelems + 1);
        upload(m->kel_ptr, m->h_kel_ptr.data(), (d->nelems + 1) * sizeof(int64_t), s);
        amr_alloc(&m->fel_ptr, d->nelems + 1);
        upload(m->fel_ptr, fel.data(), (d->nelems + 1) * sizeof(int64_t), s);
        amr_alloc(&m->mat_type, d->nelems);
        upload(m->mat_type, mt.data(), d->nelems * sizeof(int32_t), s);
        amr_alloc(&m->mat_par, 8 * d->nelems);
        upload(m->mat_par, mp.data(), 8 * d->nelems * sizeof(double), s);
        // per-group tables: dN/dR at the IPs, weights, N
        for (AmrGroup &g : m->groups) {
            double R[64 * 3], w[64];
            amr::quadrature(g.shape, d->nips[m->perm[g.first]], R, w);
            std::vector<double> tab((size_t)g.nip * g.nen * m->ndim + g.nip + (size_t)g.nip * g.nen);
            for (int q = 0; q < g.nip; q++) {
                amr::shape_deriv(g.shape, R + 3 * q, tab.data() + (size_t)q * g.nen * m->ndim);
                tab[(size_t)g.nip * g.nen * m->ndim + q] = w[q];
                amr::shape_func(g.shape, R + 3 * q, tab.data() + (size_t)g.nip * g.nen * m->ndim + g.nip + (size_t)q * g.nen);
            }
            amr_alloc(&g.tab, tab.size());
            upload(g.tab, tab.data(), tab.size() * sizeof(double), s);
            AMR_CUDA(cudaStreamSynchronize(s));
        }
        // pattern and contribution map
        amr_build_pattern(m);
        // values and states
        amr_alloc(&m->Kel, (size_t)m->kel_blocks * m->BB);
        amr_alloc(&m->K64, (size_t)m->bstride * m->BB);
        amr_alloc(&m->K32, (size_t)m->bstride * m->BB);
        amr_alloc(&m->keep, m->nblocks);
        amr_alloc(&m->Minv32, (size_t)m->nnodes * m->BB);
        amr_alloc(&m->Minv64, (size_t)m->nnodes * m->BB);
        amr_alloc(&m->st, (size_t)AMR_NST * m->nip_total);
        amr_alloc(&m->stbk, (size_t)AMR_NST * m->nip_total);
        // nodes that no element uses have no diagonal block: their block-Jacobi inverse stays 0
        AMR_CUDA(cudaMemsetAsync(m->Minv32, 0, (size_t)m->nnodes * m->BB * sizeof(float), s));
        AMR_CUDA(cudaMemsetAsync(m->Minv64, 0, (size_t)m->nnodes * m->BB * sizeof(double), s));
        AMR_CUDA(cudaMemsetAsync(m->st, 0, (size_t)AMR_NST * m->nip_total * sizeof(double), s));
        AMR_CUDA(cudaMemsetAsync(m->stbk, 0, (size_t)AMR_NST * m->nip_total * sizeof(double), s));
        amr_alloc(&m->Fel, fel.back());
        amr_alloc(&m->d_status, 2);
        int32_t init[2] = {0, INT32_MAX};
        upload(m->d_status, init, sizeof init, s);
        m->h_status = (int32_t *)amr_pinned_alloc(2 * sizeof(int32_t));
        for (int i = 0; i < 8; i++) amr_alloc(&m->vtmp[i], m->nnodes * m->B);
        amr_alloc(&m->eq_id, 3 * m->nnodes);
        amr_alloc(&m->free_mask, m->nnodes * m->B);
        AMR_CUDA(cudaStreamSynchronize(s));
    } catch (const AmrError &e) {
        g_create_error = e.msg;
        amr_model_destroy(m);
        return e.code;
    } catch (const std::exception &e) {
        g_create_error = e.what();
        amr_model_destroy(m);
        return AMR_EINVAL;
    }
    *out = m;
    return AMR_OK;
}

int amr_model_destroy(amr_model *m) {
    if (!m) return AMR_OK;
    AmrStreamScope scope(m->stream);  // the frees are ordered on the handle's stream, destroyed last
    if (m->stream) cudaStreamSynchronize(m->stream);
    amr_solver_free(m);
    amr_batch_free(m);
    amr_amg_free(m);
    amr_recovery_free(m);
    for (AmrGroup &g : m->groups) {
        amr_free(g.tab); amr_free(g.geo_g); amr_free(g.geo_w);
    }
    amr_free(m->coords); amr_free(m->conn); amr_free(m->conn_ptr); amr_free(m->mat_type); amr_free(m->mat_par);
    amr_free(m->ip_ptr); amr_free(m->kel_ptr); amr_free(m->inc_ptr); amr_free(m->inc); amr_free(m->brow_ptr);
    amr_free(m->bcol); amr_free(m->contrib_ptr); amr_free(m->contrib); amr_free(m->gorder); amr_free(m->grow);
    amr_free(m->Kel); amr_free(m->K64);
    amr_free(m->K32); amr_free(m->keep); amr_free(m->Minv32); amr_free(m->Minv64); amr_free(m->eq_id);
    amr_free(m->free_mask); amr_free(m->dof_node); amr_free(m->st); amr_free(m->stbk); amr_free(m->Fel);
    amr_free(m->fel_ptr); amr_free(m->d_status); amr_free(m->rho); amr_free(m->M64); amr_free(m->Mkeep);
    for (int i = 0; i < 8; i++) amr_free(m->vtmp[i]);
    amr_pinned_free(m->h_status);
    if (m->ev0) cudaEventDestroy(m->ev0);
    if (m->ev1) cudaEventDestroy(m->ev1);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return AMR_OK;
}

int amr_last_error(const amr_model *m, char *buf, size_t n) {
    if (!m || !buf || n == 0) return AMR_EINVAL;
    std::snprintf(buf, n, "%s", m->err.c_str());
    return AMR_OK;
}

int amr_get_sizes(const amr_model *m, int64_t *nnodes, int64_t *nelems, int64_t *nip_total, int64_t *nblocks) {
    if (!m) return AMR_EINVAL;
    if (nnodes) *nnodes = m->nnodes;
    if (nelems) *nelems = m->nelems;
    if (nip_total) *nip_total = m->nip_total;
    if (nblocks) *nblocks = m->nblocks;
    return AMR_OK;
}

int amr_set_dofs(amr_model *m, const int64_t *eq_id, int64_t ndofs, int64_t nu) {
    return guarded(m, [&] {
        if (!eq_id || ndofs < 0 || nu < 0 || nu > ndofs) throw AmrError(AMR_EINVAL, "bad dof numbering");
        std::vector<uint8_t> seen(ndofs, 0);
        for (int64_t n = 0; n < m->nnodes; n++)
            for (int c = 0; c < 3; c++) {
                int64_t e = eq_id[3 * n + c];
                if (c >= m->ndim) {
                    if (e >= 0) throw AmrError(AMR_EINVAL, "eq_id set for a component beyond ndim");
                    continue;
                }
                if (e < -1 || e >= ndofs) throw AmrError(AMR_EINVAL, "eq_id out of range");
                if (e >= 0) {
                    if (seen[e]) throw AmrError(AMR_EINVAL, "eq_id used twice");
                    seen[e] = 1;
                }
            }
        for (int64_t i = 0; i < ndofs; i++)
            if (!seen[i]) throw AmrError(AMR_EINVAL, "eq_id numbering has gaps");
        // every element node must carry all its DOFs
        for (int32_t v : m->h_conn)
            for (int c = 0; c < m->ndim; c++)
                if (eq_id[3 * (int64_t)v + c] < 0) throw AmrError(AMR_EINVAL, "an element node has no DOF");
        m->h_eq_id.assign(eq_id, eq_id + 3 * m->nnodes);
        m->ndofs = ndofs;
        m->nu = nu;
        upload(m->eq_id, eq_id, 3 * m->nnodes * sizeof(int64_t), m->stream);
        int64_t nt = m->nnodes * m->B;
        k_free_mask<<<nblk(nt, 256), 256, 0, m->stream>>>(m->nnodes, m->B, m->eq_id, nu, m->free_mask);
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        m->dofs_version++;
        m->dofs_set = true;
        m->K_valid = false;
        if (m->sw) amr_solver_free(m);  // the comparator CSR depends on the numbering
        return AMR_OK;
    });
}

int amr_set_youngs(amr_model *m, const double *E) {
    return guarded(m, [&] {
        std::vector<double> mp(8 * m->nelems);
        amr_d2h(m, mp.data(), m->mat_par, mp.size() * sizeof(double));
        for (int64_t s = 0; s < m->nelems; s++) {
            double v = E[m->perm[s]];
            if (!(v > 0.0)) throw AmrError(AMR_EINVAL, "E must be > 0");
            mp[8 * s] = v;
        }
        amr_h2d(m, m->mat_par, mp.data(), mp.size() * sizeof(double));
        m->K_valid = false;
        return AMR_OK;
    });
}

int amr_set_assembly(amr_model *m, int32_t mode) {
    return guarded(m, [&] {
        if (mode != AMR_ASSEMBLY_FAST && mode != AMR_ASSEMBLY_REFERENCE) throw AmrError(AMR_EINVAL, "bad assembly mode");
        m->assembly_mode = mode;  // applies to the next assembly; the current K stays valid
        return AMR_OK;
    });
}

int amr_set_amg_smoothing(amr_model *m, int32_t on) {
    return guarded(m, [&] {
        if (on != 0 && on != 1) throw AmrError(AMR_EINVAL, "smoothing is 0 or 1");
        if (m->amg_smooth != on) {
            m->amg_smooth = on;
            amr_amg_free(m);  // the hierarchy is rebuilt at the next multigrid solve
        }
        return AMR_OK;
    });
}

int amr_assemble_K(amr_model *m) {
    return guarded(m, [&] {
        assemble(m);
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        return AMR_OK;
    });
}

// Host export of K in the reference layout (CSC over eq_id order, eps drop rule)
// CSC of the block matrix vals (SoA, K's pattern) with the scalar entries its keep bits mark
static void export_csc(amr_model *m, int64_t *nnz_out, int64_t *colptr, int64_t *rowval, double *nzval,
                       const uint16_t *d_keep, const double *d_vals) {
    int B = m->B, BB = m->BB;
    std::vector<uint16_t> keep(m->nblocks);
    amr_d2h(m, keep.data(), d_keep, m->nblocks * sizeof(uint16_t));
    std::vector<double> K;
    if (nzval) {
        K.resize((size_t)m->bstride * BB);
        amr_d2h(m, K.data(), d_vals, K.size() * sizeof(double));
    }
    const std::vector<int64_t> &eq = m->h_eq_id;
    // count per column (= per row of the symmetric pattern walk)
    std::vector<int64_t> cnt(m->ndofs + 1, 0);
    for (int64_t n = 0; n < m->nnodes; n++)
        for (int64_t k = m->h_brow_ptr[n]; k < m->h_brow_ptr[n + 1]; k++) {
            int64_t j = m->h_bcol[k];
            for (int c = 0; c < B; c++) {
                int64_t r = eq[3 * n + c];
                if (r < 0) continue;
                for (int d = 0; d < B; d++) {
                    int64_t col = eq[3 * j + d];
                    if (col < 0 || !(keep[k] >> (c * B + d) & 1)) continue;
                    cnt[col + 1]++;
                }
            }
        }
    for (int64_t i = 0; i < m->ndofs; i++) cnt[i + 1] += cnt[i];
    *nnz_out = cnt[m->ndofs];
    if (!colptr) return;
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (int64_t n = 0; n < m->nnodes; n++)
        for (int64_t k = m->h_brow_ptr[n]; k < m->h_brow_ptr[n + 1]; k++) {
            int64_t j = m->h_bcol[k];
            for (int c = 0; c < B; c++) {
                int64_t r = eq[3 * n + c];
                if (r < 0) continue;
                for (int d = 0; d < B; d++) {
                    int64_t col = eq[3 * j + d];
                    if (col < 0 || !(keep[k] >> (c * B + d) & 1)) continue;
                    int64_t p = pos[col]++;
                    rowval[p] = r;
                    if (nzval) nzval[p] = K[(size_t)(c * B + d) * m->bstride + k];
                }
            }
        }
    for (int64_t i = 0; i <= m->ndofs; i++) colptr[i] = cnt[i];
    // sort rows within each column
    std::vector<std::pair<int64_t, double>> tmp;
    for (int64_t col = 0; col < m->ndofs; col++) {
        int64_t a = cnt[col], b = cnt[col + 1];
        tmp.resize(b - a);
        for (int64_t p = a; p < b; p++) tmp[p - a] = {rowval[p], nzval ? nzval[p] : 0.0};
        std::sort(tmp.begin(), tmp.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
        for (int64_t p = a; p < b; p++) {
            rowval[p] = tmp[p - a].first;
            if (nzval) nzval[p] = tmp[p - a].second;
        }
    }
}

int amr_get_K_nnz(amr_model *m, int64_t *nnz) {
    return guarded(m, [&] {
        if (!m->K_valid) throw AmrError(AMR_EINVAL, "K has not been assembled");
        export_csc(m, nnz, nullptr, nullptr, nullptr, m->keep, m->K64);
        return AMR_OK;
    });
}

int amr_get_K_csc(amr_model *m, int64_t *colptr, int64_t *rowval, double *nzval) {
    return guarded(m, [&] {
        int64_t nnz = 0;
        if (!m->K_valid) throw AmrError(AMR_EINVAL, "K has not been assembled");
        export_csc(m, &nnz, colptr, rowval, nzval, m->keep, m->K64);
        return AMR_OK;
    });
}

int amr_set_density(amr_model *m, const double *rho) {
    return guarded(m, [&] {
        if (!rho) throw AmrError(AMR_EINVAL, "null argument");
        std::vector<double> r(m->nelems);
        for (int64_t e = 0; e < m->nelems; e++) {
            if (!(rho[e] >= 0.0)) throw AmrError(AMR_EINVAL, "element " + std::to_string(e) + ": rho >= 0 required");
            r[m->inv_perm[e]] = rho[e];
        }
        if (!m->rho) amr_alloc(&m->rho, m->nelems);
        upload(m->rho, r.data(), m->nelems * sizeof(double), m->stream);
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        return AMR_OK;
    });
}

int amr_assemble_M(amr_model *m) {
    return guarded(m, [&] {
        check_dofs(m);
        amr_mass(m);
        int rc = amr_check_status(m);
        if (rc == AMR_ENEGJAC) throw AmrError(rc, "Negative Jacobian determinant in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
        if (rc) throw AmrError(rc, "mass assembly failed");
        return AMR_OK;
    });
}

int amr_get_M_csc(amr_model *m, int64_t *nnz, int64_t *colptr, int64_t *rowval, double *nzval) {
    return guarded(m, [&] {
        if (!nnz) throw AmrError(AMR_EINVAL, "null argument");
        if (!m->M64) throw AmrError(AMR_EINVAL, "M has not been assembled");
        export_csc(m, nnz, colptr, rowval, nzval, m->Mkeep, m->M64);
        return AMR_OK;
    });
}

int amr_update_state(amr_model *m, const double *dU, double *dFin) {
    return guarded(m, [&] {
        check_dofs(m);
        double *u = m->vtmp[0], *f = m->vtmp[1];
        eq_host_to_nm(m, dU, u);
        amr_update_elements(m, u, f);
        int rc = amr_check_status(m);
        if (rc == AMR_ERETMAP) throw AmrError(rc, "VonMises: return mapping failed in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
        if (rc == AMR_ENAN) throw AmrError(rc, "solve_system!: NaN values in internal forces vector");
        if (rc) throw AmrError(rc, "update_state failed");
        nm_to_eq_host(m, f, dFin);
        return AMR_OK;
    });
}

int amr_state_commit(amr_model *m) {
    return guarded(m, [&] {
        AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, (size_t)AMR_NST * m->nip_total * sizeof(double),
                                 cudaMemcpyDeviceToDevice, m->stream));
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        return AMR_OK;
    });
}

int amr_state_restore(amr_model *m) {
    return guarded(m, [&] {
        AMR_CUDA(cudaMemcpyAsync(m->st, m->stbk, (size_t)AMR_NST * m->nip_total * sizeof(double),
                                 cudaMemcpyDeviceToDevice, m->stream));
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        if (m->any_plastic) m->K_valid = false;
        return AMR_OK;
    });
}

int amr_get_state(amr_model *m, double *state) {
    return guarded(m, [&] {
        std::vector<double> st((size_t)AMR_NST * m->nip_total);
        amr_d2h(m, st.data(), m->st, st.size() * sizeof(double));
        int64_t o = 0;
        for (int64_t e = 0; e < m->nelems; e++) {
            int64_t s = m->inv_perm[e];
            for (int64_t g = m->h_ip_ptr[s]; g < m->h_ip_ptr[s + 1]; g++, o++) {
                for (int f = 0; f < 16; f++) state[16 * o + f] = f < AMR_NST ? st[(size_t)f * m->nip_total + g] : 0.0;
            }
        }
        return AMR_OK;
    });
}

int amr_get_elem_nips(const amr_model *m, int32_t *nips) {
    return guarded(const_cast<amr_model *>(m), [&] {
        if (!nips) throw AmrError(AMR_EINVAL, "null argument");
        for (int64_t e = 0; e < m->nelems; e++) nips[e] = m->h_nips[m->inv_perm[e]];
        return AMR_OK;
    });
}

int amr_set_state(amr_model *m, const double *state) {
    return guarded(m, [&] {
        if (!state) throw AmrError(AMR_EINVAL, "null argument");
        std::vector<double> st((size_t)AMR_NST * m->nip_total);
        int64_t o = 0;
        for (int64_t e = 0; e < m->nelems; e++) {
            int64_t s = m->inv_perm[e];
            for (int64_t g = m->h_ip_ptr[s]; g < m->h_ip_ptr[s + 1]; g++, o++)
                for (int f = 0; f < AMR_NST; f++) st[(size_t)f * m->nip_total + g] = state[16 * o + f];
        }
        AMR_CUDA(cudaMemcpyAsync(m->st, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice, m->stream));
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        return AMR_OK;
    });
}

int amr_assemble_loads(amr_model *m, const amr_load *loads, int32_t nloads, double t, double *F) {
    return guarded(m, [&] {
        check_dofs(m);
        double *f = m->vtmp[0];
        eq_host_to_nm(m, F, f);
        amr_loads(m, loads, nloads, t, f);
        nm_to_eq_host(m, f, F);
        return AMR_OK;
    });
}

int amr_solve(amr_model *m, double *U, double *F, const amr_solve_opts *opts, amr_solve_stats *stats) {
    return guarded(m, [&] {
        check_dofs(m);
        if (!m->K_valid) throw AmrError(AMR_EINVAL, "K has not been assembled");
        amr_solve_opts o;
        amr_default_solve_opts(&o);
        if (opts) o = *opts;
        double *x = m->vtmp[0], *b = m->vtmp[1], *reac = m->vtmp[2];
        eq_host_to_nm(m, U, x);
        vec(m, V_MASK_PRESC, 1.0, x, 0.0, nullptr, x);  // free slots start at 0
        eq_host_to_nm(m, F, b);
        AMR_CUDA(cudaMemsetAsync(reac, 0, m->nnodes * m->B * sizeof(double), m->stream));
        AmrSolveResult r = amr_solve_device(m, x, b, reac, o);
        if (stats) {
            stats->iterations = r.iterations;
            stats->refinements = r.refinements;
            stats->rel_residual = r.rel_residual;
            stats->seconds = r.seconds;
        }
        if (r.status) throw AmrError(r.status, "solve_system!: Krylov solver did not converge (relative residual " + std::to_string(r.rel_residual) + ")");
        double umax = amr_norm_inf(m, x, m->free_mask);
        if (std::isnan(umax) || std::isinf(umax)) throw AmrError(AMR_ENAN, "solve_system!: NaN values in the solution");
        if (umax > 1e8) throw AmrError(AMR_ESINGULAR, "solve_system!: Possible syngular matrix");
        std::vector<double> xs(m->ndofs), rs(m->ndofs);
        nm_to_eq_host(m, x, xs.data());
        nm_to_eq_host(m, reac, rs.data());
        for (int64_t i = 0; i < m->nu; i++) U[i] = xs[i];
        for (int64_t i = m->nu; i < m->ndofs; i++) F[i] = rs[i];
        return AMR_OK;
    });
}

int amr_stage_run(amr_model *m, const double *Uex, const double *Fex, const amr_stage_params *p, double *U, double *F,
                  amr_stage_stats *stats) {
    return guarded(m, [&] {
        check_dofs(m);
        amr_stage_params prm;
        amr_default_stage_params(&prm);
        if (p) prm = *p;
        int64_t n = m->nnodes * m->B;
        double *uex = nullptr, *fex = nullptr, *u = nullptr, *f = nullptr;
        int rc;
        try {
            amr_alloc(&uex, n); amr_alloc(&fex, n); amr_alloc(&u, n); amr_alloc(&f, n);
            eq_host_to_nm(m, Uex, uex);
            eq_host_to_nm(m, Fex, fex);
            rc = amr_stage_device(m, uex, fex, prm, u, f, stats);
            if (rc == AMR_OK || rc == AMR_ESTAGE) {
                nm_to_eq_host(m, u, U);
                nm_to_eq_host(m, f, F);
            }
        } catch (...) {
            amr_free(uex); amr_free(fex); amr_free(u); amr_free(f);
            throw;
        }
        amr_free(uex); amr_free(fex); amr_free(u); amr_free(f);
        return rc;
    });
}

void amr_default_dyn_params(amr_dyn_params *p) {
    p->tol = 0.01; p->dTmin = 1e-7; p->dTmax = 0.1; p->rspan = 0.01;
    p->alpha = 0.0; p->beta = 0.0; p->tspan = 0.0;
    p->maxits = 5; p->autoinc = 0; p->nincs = 1; p->nouts = 0;
    amr_default_solve_opts(&p->linear);
    p->sism = 0; p->sism_dir = 0; p->tss = 0.0; p->tds = 0.0; p->sism_acc = nullptr; p->sism_n = 0;
}

int amr_dyn_stage_run(amr_model *m, const double *Uex0, const double *Uex1, const double *Fex0, const double *Fex1,
                      const amr_dyn_params *p, double *U, double *V, double *A, double *F, amr_stage_stats *stats) {
    return guarded(m, [&] {
        check_dofs(m);
        if (!p || !Uex0 || !Uex1 || !Fex0 || !Fex1) throw AmrError(AMR_EINVAL, "null argument");
        const int64_t n = m->nnodes * m->B;
        std::vector<double *> d(8, nullptr);
        auto release = [&]() {
            for (auto &x : d) amr_free(x);
        };
        int rc;
        try {
            for (auto &x : d) amr_alloc(&x, n);
            eq_host_to_nm(m, Uex0, d[0]);
            eq_host_to_nm(m, Uex1, d[1]);
            eq_host_to_nm(m, Fex0, d[2]);
            eq_host_to_nm(m, Fex1, d[3]);
            rc = amr_dyn_stage_device(m, d[0], d[1], d[2], d[3], *p, d[4], d[5], d[6], d[7], stats);
            if (rc == AMR_OK || rc == AMR_ESTAGE) {
                double *outs[4] = {U, V, A, F};
                for (int i = 0; i < 4; i++)
                    if (outs[i]) nm_to_eq_host(m, d[4 + i], outs[i]);
            }
        } catch (...) {
            release();
            throw;
        }
        release();
        return rc;
    });
}

int amr_write_vtu(amr_model *m, const char *path, const amr_vtu_array *point_data, int32_t npoint,
                  const amr_vtu_array *cell_data, int32_t ncell, int32_t nthreads) {
    return guarded(m, [&] {
        if (npoint < 0 || ncell < 0 || (npoint && !point_data) || (ncell && !cell_data))
            throw AmrError(AMR_EINVAL, "bad array lists");
        amr_vtu_write(m, path, point_data, npoint, cell_data, ncell, nthreads, false);
        return AMR_OK;
    });
}

int amr_write_vtu_compressed(amr_model *m, const char *path, const amr_vtu_array *point_data, int32_t npoint,
                             const amr_vtu_array *cell_data, int32_t ncell, int32_t nthreads) {
    return guarded(m, [&] {
        if (npoint < 0 || ncell < 0 || (npoint && !point_data) || (ncell && !cell_data))
            throw AmrError(AMR_EINVAL, "bad array lists");
        amr_vtu_write(m, path, point_data, npoint, cell_data, ncell, nthreads, true);
        return AMR_OK;
    });
}

void amr_default_modal_params(amr_modal_params *p) {
    p->nmodes = 5;
    p->max_iters = 1000;
    p->tol = 1e-7;
}

int amr_modal_run(amr_model *m, const amr_modal_params *p, double *omega, double *modes, amr_modal_stats *stats) {
    return guarded(m, [&] {
        check_dofs(m);
        if (!p || !omega) throw AmrError(AMR_EINVAL, "null argument");
        const int nm = p->nmodes;
        const int64_t n = m->nnodes * m->B;
        double *d = nullptr;
        amr_alloc(&d, (size_t)n * std::max(1, nm));
        int rc;
        try {
            rc = amr_modal_device(m, *p, omega, d, stats);
            if (modes) {
                std::vector<double> eq(m->ndofs);
                for (int c = 0; c < nm; c++) {
                    nm_to_eq_host(m, d + (size_t)c * n, eq.data());
                    double nrm = 0.0, big = 0.0;
                    for (int64_t i = 0; i < m->nu; i++) {
                        nrm += eq[i] * eq[i];
                        if (std::fabs(eq[i]) > std::fabs(big)) big = eq[i];
                    }
                    const double sc = (big < 0 ? -1.0 : 1.0) / std::sqrt(nrm);
                    for (int64_t i = 0; i < m->nu; i++) modes[(size_t)c * m->nu + i] = eq[i] * sc;
                }
            }
        } catch (...) {
            amr_free(d);
            throw;
        }
        amr_free(d);
        return rc;
    });
}

int amr_stage_run_dev(amr_model *m, const double *d_Uex, const double *d_Fex, const amr_stage_params *p,
                      double *d_U, double *d_F, amr_stage_stats *stats) {
    return guarded(m, [&] {
        check_dofs(m);
        amr_stage_params prm;
        amr_default_stage_params(&prm);
        if (p) prm = *p;
        double *uex = m->vtmp[2], *fex = m->vtmp[3], *u = m->vtmp[4], *f = m->vtmp[5];
        amr_eq_to_nm(m, d_Uex, uex);
        amr_eq_to_nm(m, d_Fex, fex);
        int rc = amr_stage_device(m, uex, fex, prm, u, f, stats);
        if (rc == AMR_OK || rc == AMR_ESTAGE) {
            amr_nm_to_eq(m, u, d_U);
            amr_nm_to_eq(m, f, d_F);
            AMR_CUDA(cudaStreamSynchronize(m->stream));
        }
        return rc;
    });
}

int amr_set_parts(amr_model *m, int64_t nparts, const int64_t *node_ptr) {
    return guarded(m, [&] {
        if (nparts == 0) amr_batch_free(m);
        else amr_batch_set(m, nparts, node_ptr);
        return AMR_OK;
    });
}

int amr_get_part_stats(const amr_model *m, int64_t nparts, amr_stage_stats *stats) {
    if (!stats) return AMR_EINVAL;
    return guarded(const_cast<amr_model *>(m), [&] {
        amr_batch_part_stats(m, nparts, stats);
        return AMR_OK;
    });
}

int amr_autotune(amr_model *m, amr_tuning *out) {
    return guarded(m, [&] {
        amr_autotune_model(m, out);
        return AMR_OK;
    });
}

int amr_recovery_fields(amr_model *m, int32_t *codes, int32_t cap, int32_t *nfields) {
    return guarded(m, [&] {
        if (!nfields || (cap > 0 && !codes)) throw AmrError(AMR_EINVAL, "null argument");
        const std::vector<int32_t> &c = amr_recovery_codes(m);
        for (int32_t i = 0; i < cap && i < (int32_t)c.size(); i++) codes[i] = c[i];
        *nfields = (int32_t)c.size();
        return AMR_OK;
    });
}

int amr_recover_nodal_dev(amr_model *m, double *d_V) {
    return guarded(m, [&] {
        if (!d_V) throw AmrError(AMR_EINVAL, "null argument");
        amr_recover(m, d_V);
        AMR_CUDA(cudaStreamSynchronize(m->stream));
        return AMR_OK;
    });
}

int amr_recover_nodal(amr_model *m, double *V) {
    return guarded(m, [&] {
        if (!V) throw AmrError(AMR_EINVAL, "null argument");
        const size_t n = (size_t)m->nnodes * amr_recovery_codes(m).size();
        if (!n) return AMR_OK;
        double *d_V;
        amr_alloc(&d_V, n);
        try {
            amr_recover(m, d_V);
            AMR_CUDA(cudaMemcpyAsync(V, d_V, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
            AMR_CUDA(cudaStreamSynchronize(m->stream));
        } catch (...) {
            amr_free(d_V);
            throw;
        }
        amr_free(d_V);
        return AMR_OK;
    });
}

int amr_time_recovery(amr_model *m, int32_t reps, double *avg_seconds, double *flops_per_launch,
                      int64_t *svd_patches) {
    return guarded(m, [&] {
        if (reps < 1 || !avg_seconds) throw AmrError(AMR_EINVAL, "reps >= 1 and avg_seconds required");
        *avg_seconds = amr_recovery_time_fit(m, reps, flops_per_launch, svd_patches);
        return AMR_OK;
    });
}

int amr_launch_count(const amr_model *m, int64_t *count) {
    if (!count) return AMR_EINVAL;
    (void)m;
    *count = amr_g_launches.load();
    return AMR_OK;
}

int amr_get_stage_log(const amr_model *m, amr_iteration_record *rec, int32_t cap, int32_t *n) {
    if (!m || !n || cap < 0 || (cap > 0 && !rec)) return AMR_EINVAL;
    const size_t k = std::min(m->stage_log.size(), (size_t)cap);
    std::copy(m->stage_log.begin(), m->stage_log.begin() + k, rec);
    *n = (int32_t)m->stage_log.size();
    return AMR_OK;
}

int amr_set_increment_callback(amr_model *m, amr_increment_fn fn, void *user) {
    if (!m) return AMR_EINVAL;
    m->inc_fn = fn;
    m->inc_user = fn ? user : nullptr;
    return AMR_OK;
}

int amr_alloc_count(int64_t *count) {
    if (!count) return AMR_EINVAL;
    *count = amr_g_allocs.load();
    return AMR_OK;
}

int amr_time_kernel(amr_model *m, int32_t kernel, int32_t reps, double *avg_seconds, double *bytes_per_launch) {
    return guarded(m, [&] {
        // the dynamic right-hand side reads M and a K-shaped operand only
        if (!m->K_valid && kernel != AMR_KERNEL_DYN_RHS) throw AmrError(AMR_EINVAL, "assemble K first");
        if (reps < 1) throw AmrError(AMR_EINVAL, "reps must be >= 1");
        const double nb = (double)m->nblocks, nn = (double)m->nnodes, B = m->B, BB = m->BB;
        double t = 0.0, bytes = 0.0;
        switch (kernel) {
        case AMR_KERNEL_SPMV32:  // K32 blocks + block columns + row pointers; p (padded) read once, q written
            t = amr_time_solver_kernel(m, AMR_KERNEL_SPMV32, reps);
            bytes = nb * (4.0 * BB + 4.0) + (nn + 1) * 8.0 + 4.0 * nn * ((B == 3 ? 4.0 : 2.0) + B);
            break;
        case AMR_KERNEL_RESIDUAL64:  // K64 blocks + columns + row pointers; u, b read; r32, z written; Minv read
            t = amr_time_solver_kernel(m, AMR_KERNEL_RESIDUAL64, reps);
            bytes = nb * (8.0 * BB + 4.0) + (nn + 1) * 8.0 + nn * B * (8.0 + 8.0 + 4.0 + 4.0 + 1.0) + nn * BB * 4.0;
            break;
        case AMR_KERNEL_AMG_RESIDUAL:  // the FP16 copy's blocks, row pointers, b, r, the scale and xt per node
            t = amr_amg_time_residual(m, reps, false, &bytes);
            break;
        case AMR_KERNEL_SPMV64:  // K64 blocks + columns + row pointers; p read once, q written, row mask
            t = amr_time_solver_kernel(m, AMR_KERNEL_SPMV64, reps);
            bytes = nb * (8.0 * BB + 4.0) + (nn + 1) * 8.0 + nn * B * (8.0 * 2.0 + 1.0);
            break;
        case AMR_KERNEL_AMG_RESIDUAL64:  // as SPMV64, plus b read
            t = amr_amg_time_residual(m, reps, true, &bytes);
            break;
        case AMR_KERNEL_DYN_RHS:
            t = amr_dyn_time_rhs(m, reps, &bytes);
            break;
        case AMR_KERNEL_STIFFNESS: {  // the fast element kernels alone; the second output is their FP64 operations
            if (m->assembly_mode != AMR_ASSEMBLY_FAST) throw AmrError(AMR_EINVAL, "time the fast assembly");
            const int D = m->ndim;
            for (const AmrGroup &g : m->groups) {
                const double nen = g.nen, nip = g.nip, np = nen * (nen + 1) / 2;
                // per IP: J and dN/dX (2 nen D^2 each), det and inverse (about 30), w g (nen D); per node pair:
                // T_ab (an FMA per component per IP) and the lambda / mu combination (about 4 D^2)
                const double per_elem = nip * (4.0 * nen * D * D + nen * D + 30.0) + np * (2.0 * D * D * nip + 4.0 * D * D);
                bytes += per_elem * (double)g.count;
            }
            amr_stiffness_elements(m);  // warm-up
            AMR_CUDA(cudaEventRecord(m->ev0, m->stream));
            for (int i = 0; i < reps; i++) amr_stiffness_elements(m);
            AMR_CUDA(cudaEventRecord(m->ev1, m->stream));
            AMR_CUDA(cudaEventSynchronize(m->ev1));
            float ms = 0.f;
            AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
            t = ms * 1e-3 / reps;
            if (int rc = amr_check_status(m)) throw AmrError(rc, "assembly failed");
            break;
        }
        default:
            throw AmrError(AMR_EINVAL, "kernel not timed by this entry point");
        }
        if (avg_seconds) *avg_seconds = t;
        if (bytes_per_launch) *bytes_per_launch = bytes;
        return AMR_OK;
    });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// mech_stage_solver! (src/mech/mech-solver.jl:186-492), device vectors
// ---------------------------------------------------------------------------
int amr_stage_device(amr_model *m, const double *Uex, const double *Fex, const amr_stage_params &p, double *U,
                     double *F, amr_stage_stats *stats) {
    if (m->batch) return amr_batch_stage(m, Uex, Fex, p, U, F, stats);  // each part its own stage
    int64_t n = m->nnodes * m->B;
    cudaStream_t s = m->stream;
    // predictor-corrector schemes (mech-solver.jl:280-288)
    double p1 = 1.0, q11 = 1.0, a1 = 0.0, a2 = 0.0;
    switch (p.scheme) {
    case AMR_SCHEME_FE: break;
    case AMR_SCHEME_ME: a1 = 0.5; a2 = 0.5; break;
    case AMR_SCHEME_BE: a1 = 0.0; a2 = 1.0; break;
    case AMR_SCHEME_RALSTON: p1 = 2.0 / 3.0; q11 = 2.0 / 3.0; a1 = 0.25; a2 = 0.75; break;
    default: throw AmrError(AMR_EINVAL, "unknown scheme");
    }
    const bool corrector = p.scheme != AMR_SCHEME_FE;
    if (p.maxits < 1 || p.nincs < 1) throw AmrError(AMR_EINVAL, "bad stage parameters");
    AmrEventPair ev;  // destroyed on every exit
    cudaEvent_t t0 = ev.t0, t1 = ev.t1;
    std::vector<double *> v(10, nullptr);
    double *Ks = nullptr;  // the predictor's tangent, kept for the weighted corrector tangent
    auto release = [&]() {
        for (auto &x : v) amr_free(x);
        amr_free(Ks);
    };
    try {
        for (auto &x : v) amr_alloc(&x, n);
        if (corrector) amr_alloc(&Ks, (size_t)m->bstride * m->BB);
    } catch (...) {
        release();
        throw;
    }
    double *R = v[0], *dUa = v[1], *dUi = v[2], *Rc = v[3], *dFin = v[4], *dFex = v[5], *dUitr = v[6], *Rtr = v[7],
           *reac = v[8], *dUt = v[9];
    int status = AMR_OK;
    amr_stage_stats st{};
    m->stage_log.clear();
    std::vector<double> hU, hF;  // the hook's host copies
    try {
        AMR_CUDA(cudaEventRecord(t0, s));
        for (double *x : {U, F, R, dUa, dUi, Rc, dFin}) AMR_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        double tol = p.tol, rtol = p.rtol, dTmin = p.dTmin;
        bool autoinc = p.autoinc != 0;
        bool saveouts = p.nouts > 0;
        int nincs = p.nincs;
        if (saveouts && !autoinc) {  // src/solver.jl:128-140
            if (p.nouts > nincs) nincs = p.nouts;
            if (nincs % p.nouts != 0) nincs = nincs - (nincs % p.nouts) + p.nouts;
        }
        double dTcheck = saveouts ? 1.0 / p.nouts : 1.0, Tcheck = dTcheck;
        double T = 0.0, dT = 1.0 / nincs, dTbk = 0.0;
        if (autoinc) dT = std::min({dT, p.dTmax, dTcheck, p.dT0});
        // every stage mounts K at least once (the reference mounts it at every iteration;
        // a state-independent K is reused across the iterations of the stage only)
        m->K_valid = false;
        // committed states = current states at stage start
        AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, (size_t)AMR_NST * m->nip_total * sizeof(double),
                                 cudaMemcpyDeviceToDevice, s));
        const double eps = 2.220446049250313e-16;
        int inc = 0;  // the reference's increment counter (a failed increment's number is reused)
        while (T < 1.0 - dTmin) {
            inc++;
            // dUex, dFex (+ carried residue)
            double dTcr = std::min(p.rspan, 1 - T);
            double acr = std::min(dT / dTcr, 1.0);
            vec(m, V_SET_AXPBY, dT, Fex, (T < 1 - p.rspan) ? acr : 0.0, Rc, dFex);
            AMR_CUDA(cudaMemcpyAsync(R, dFex, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            AMR_CUDA(cudaMemsetAsync(dUa, 0, n * sizeof(double), s));
            vec(m, V_SET_AXPBY, dT, Uex, 0.0, nullptr, dUi);
            double res = 0.0, res1 = 0.0, err = 0.0;
            bool converged = false, syserror = false;
            std::string sysmsg;
            int nits = 0;
            for (int it = 1; it <= p.maxits; it++) {
                nits++;
                const int kry0 = st.krylov_iterations;
                if (it > 1) AMR_CUDA(cudaMemsetAsync(dUi, 0, n * sizeof(double), s));
                double lastres = res;
                if (m->any_plastic || !m->K_valid) assemble(m);
                // predictor solve: x = p1 dUi at prescribed slots, b = q11 R
                vec(m, V_PRESC_AX, p1, dUi, 0.0, nullptr, dUitr);
                vec(m, V_SET_AXPBY, q11, R, 0.0, nullptr, Rtr);
                AmrSolveResult sr = amr_solve_device(m, dUitr, Rtr, reac, p.linear);
                st.krylov_iterations += sr.iterations;
                st.solve_seconds += sr.seconds;
                if (sr.status) { syserror = true; sysmsg = "solve_system!: Krylov solver did not converge"; break; }
                double umax = amr_norm_inf(m, dUitr, m->free_mask);
                if (!(umax <= 1e8)) { syserror = true; sysmsg = "solve_system!: Possible syngular matrix"; break; }
                // restore states (update reads the committed copy) and update
                vec(m, V_SET_AXPBY, 1.0, dUa, 1.0, dUitr, dUt);
                amr_update_elements(m, dUt, dFin);
                int rc = amr_check_status(m);
                if (rc) { syserror = true; sysmsg = rc == AMR_ERETMAP ? "return mapping failed" : "NaN values in internal forces vector"; break; }
                if (!corrector) {
                    AMR_CUDA(cudaMemcpyAsync(dUi, dUitr, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                } else {
                    // corrector (mech-solver.jl:341-348): K = a1 K + a2 K2 with K2 the tangent of the
                    // predictor's trial states, solve for dUi, update the states again from the committed ones
                    AMR_CUDA(cudaMemcpyAsync(Ks, m->K64, (size_t)m->bstride * m->BB * sizeof(double),
                                             cudaMemcpyDeviceToDevice, s));
                    if (m->any_plastic) assemble(m);  // a state-independent K2 equals K
                    amr_combine_K(m, a1, Ks, a2);
                    m->K_valid = false;  // the next iteration mounts the plain tangent again
                    vec(m, V_MASK_PRESC, 1.0, dUi, 0.0, nullptr, dUi);
                    vec(m, V_SET_AXPBY, 1.0, R, 0.0, nullptr, Rtr);
                    AmrSolveResult sc = amr_solve_device(m, dUi, Rtr, reac, p.linear);
                    st.krylov_iterations += sc.iterations;
                    st.solve_seconds += sc.seconds;
                    if (sc.status) { syserror = true; sysmsg = "solve_system!: Krylov solver did not converge"; break; }
                    double um = amr_norm_inf(m, dUi, m->free_mask);
                    if (!(um <= 1e8)) { syserror = true; sysmsg = "solve_system!: Possible syngular matrix"; break; }
                    vec(m, V_SET_AXPBY, 1.0, dUa, 1.0, dUi, dUt);
                    amr_update_elements(m, dUt, dFin);
                    int rc2 = amr_check_status(m);
                    if (rc2) { syserror = true; sysmsg = rc2 == AMR_ERETMAP ? "return mapping failed" : "NaN values in internal forces vector"; break; }
                }
                vec(m, V_SET_AXPBY, 1.0, dUa, 1.0, dUi, dUa);
                vec(m, V_SET_AXPBY, 1.0, dFex, -1.0, dFin, R);
                vec(m, V_MASK_FREE, 1.0, R, 0.0, nullptr, R);
                res = amr_norm_inf(m, R, nullptr);
                double nui = amr_norm_inf(m, dUi, nullptr), nua = amr_norm_inf(m, dUa, nullptr);
                err = nui / nua;
                st.iterations++;
                m->stage_log.push_back(amr_iteration_record{inc, it, st.krylov_iterations - kry0, 0, T, dT, res});
                if (it == 1) res1 = res;
                if (res < tol) { converged = true; m->stage_log.back().converged = 1; break; }
                if (err < rtol) { converged = true; m->stage_log.back().converged = 1; break; }
                if (std::isnan(res)) break;
                if (it > 1 && res > lastres) break;
            }
            if (syserror) converged = false;
            st.residue = res;
            if (converged) {
                vec(m, V_SET_AXPBY, 1.0, U, 1.0, dUa, U);
                vec(m, V_SET_AXPBY, 1.0, F, 1.0, dFin, F);
                vec(m, V_SET_AXPBY, 1.0 - acr, Rc, 1.0, R, Rc);
                AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, (size_t)AMR_NST * m->nip_total * sizeof(double),
                                         cudaMemcpyDeviceToDevice, s));
                T += dT;
                st.increments++;
                bool checkpoint = T > Tcheck - dTmin;
                if (checkpoint) Tcheck += dTcheck;
                if (m->inc_fn) {  // update_records!(ana, checkpoint=checkpoint)
                    hU.resize(m->ndofs);
                    hF.resize(m->ndofs);
                    nm_to_eq_host(m, U, hU.data());
                    nm_to_eq_host(m, F, hF.data());
                    const amr_increment_info info{T, inc, checkpoint ? 1 : 0, m->ndofs, hU.data(), hF.data()};
                    if (m->inc_fn(m->inc_user, &info) != 0) {
                        status = AMR_ESTAGE;
                        m->err = "the increment callback stopped the stage";
                        break;
                    }
                }
                if (autoinc) {
                    if (dTbk > 0.0) {
                        dT = std::min(dTbk, Tcheck - T);
                        dTbk = 0.0;
                    } else {
                        double q = 1 + std::tanh(std::log10(tol / (res1 + eps)));
                        q = std::max(q, 1.1);
                        double dTtr = std::min({q * dT, p.dTmax, 1 - T});
                        if (T + dTtr > Tcheck - dTmin) {
                            dTbk = dT;
                            dT = Tcheck - T;
                        } else {
                            dT = dTtr;
                            dTbk = 0.0;
                        }
                    }
                }
            } else {
                inc--;
                AMR_CUDA(cudaMemcpyAsync(m->st, m->stbk, (size_t)AMR_NST * m->nip_total * sizeof(double),
                                         cudaMemcpyDeviceToDevice, s));
                if (m->any_plastic) m->K_valid = false;
                if (autoinc) {
                    double q = 1 + std::tanh(std::log10(tol / (res1 + eps)));
                    q = std::min(std::max(q, 0.2), 0.9);
                    if (syserror) q = 0.7;
                    dT = round_sig3(q * dT);
                    if (dT < dTmin) { status = AMR_ESTAGE; m->err = "Solver did not converge."; break; }
                } else {
                    status = AMR_ESTAGE;
                    m->err = syserror ? sysmsg : "Solver did not converge. Try `autoinc=true`. ";
                    break;
                }
            }
        }
        st.T = T;
        st.status = status;
        AMR_CUDA(cudaEventRecord(t1, s));
        AMR_CUDA(cudaEventSynchronize(t1));
        float ms = 0.f;
        AMR_CUDA(cudaEventElapsedTime(&ms, t0, t1));
        st.seconds = ms * 1e-3;
    } catch (...) {
        release();
        throw;
    }
    release();
    if (stats) *stats = st;
    return status;
}
