// A request loop over the staged solver: independent analyses (a model, its
// DOFs, its stage loads and parameters) are submitted as they arrive and run
// with continuous batching.  A fixed set of worker slots each runs one request
// at a time on its own CUDA stream, so the work of the requests on the device
// overlaps.  A request is admitted, in arrival order, as soon as a slot is
// free and its device footprint fits the HBM budget beside the requests
// already running.  While it runs, its pattern, K, IP states and solution stay
// on the device across all load increments of its stage (one amr_stage_run).
// Each request's result is the one it gets alone: every kernel is
// deterministic and its launch shape depends on the request's own model only.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "amr_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

// Upper bound of the device bytes amr_model_create, amr_set_dofs and one
// amr_stage_run allocate for a model, from its description (fp64: with the
// all-FP64 comparator's CSR copy of K11 and its vectors).
int64_t model_bytes(const amr_model_desc *d, int method) {
    if (!d || d->nnodes <= 0 || d->nelems <= 0 || !d->shape || !d->nips) return -1;
    const int64_t N = d->nnodes, E = d->nelems, B = d->ndim, BB = B * B;
    int64_t S = 0, C = 0, Q = 0, G = 0;
    double R[64 * 3], w[64];
    for (int64_t e = 0; e < E; e++) {
        const int np = amr::shape_npoints(d->shape[e]);
        const int nq = amr::quadrature(d->shape[e], d->nips[e], R, w);
        if (np <= 0 || nq <= 0) return -1;
        S += (int64_t)np * np;
        C += np;
        Q += nq;
        if (B == 3) G += (int64_t)nq * (3 * np + 1);  // the 3-D geometry cache: dN/dX and w per IP
    }
    const int64_t NB = std::min<int64_t>(S, N * N);  // node blocks of the pattern
    int64_t b = 0;
    b += 24 * N + 4 * C + 32 * (E + 1) + 4 * E + 64 * E;         // coords, conn, pointers, materials
    b += 8 * BB * S + 8 * S + 8 * C + 16 * (N + 1) + 8 * E * 2;  // staging Kel, contributions, incidence
    b += 12 * BB * NB + 2 * NB + 4 * NB + 8 * (NB + 1) + 8 * NB; // K64, K32, keep, columns, contrib ptr, build temp
    b += 12 * BB * N + 2 * 8 * AMR_NST * Q + 8 * C * B;          // block-Jacobi, IP states, element forces
    b += 8 * 8 * N * B + 24 * N + N * B;                         // work vectors, eq_id, masks
    b += 7 * 4 * N * B + ((int64_t)1 << 20);                     // FP32 Krylov vectors, reduction scratch
    if (method == AMR_SOLVER_FP64 || method == AMR_SOLVER_AMG_FP64) b += 4 * 8 * N * B;  // FP64 Krylov vectors
    if (method == AMR_SOLVER_AMG_FP64) b += 80 * N * B;          // FP64 cycle vectors and prolongator
    b += 14 * 8 * N * B;                                         // stage vectors (host-buffer stage)
    b += 8 * G;                                                  // 3-D geometry cache (FP64)
    b += (int64_t)64 << 20;                                      // allocation granularity and tables
    return b;
}

struct Request {
    int64_t id = 0;
    // deep copies of the caller's arrays
    std::vector<double> coords, mat_params, Uex, Fex;
    std::vector<int32_t> shape, nips, mat_type;
    std::vector<int64_t> conn_ptr, conn, eq_id;
    std::vector<std::vector<int64_t>> load_items;
    std::vector<amr_load> loads;
    amr_model_desc desc{};
    int64_t ndofs = 0, nu = 0;
    amr_stage_params stage{};
    int64_t bytes = 0;
    // outcome
    std::vector<double> U, F;
    amr_request_result res{};
    std::string err;
    bool done = false, taken = false;
};

}  // namespace

struct amr_server {
    amr_server_config cfg{};
    int device = 0;
    Clock::time_point t0;
    cudaEvent_t ev_ref = nullptr;  // recorded at creation: the origin of the requests' device timeline
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> queue;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    int64_t next_id = 1, active_bytes = 0, peak_bytes = 0, completed = 0;
    int active = 0, peak_active = 0;
    bool stop = false;
    std::vector<std::thread> workers;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    void run(Request *r) {
        cudaSetDevice(device);
        amr_model *m = nullptr;
        int rc = amr_model_create(&r->desc, &m);
        if (rc) {
            r->err = amr_create_error();
        } else {
            rc = amr_set_dofs(m, r->eq_id.data(), r->ndofs, r->nu);
            if (!rc && !r->loads.empty())
                rc = amr_assemble_loads(m, r->loads.data(), (int32_t)r->loads.size(), 0.0, r->Fex.data());
            r->U.assign(r->ndofs, 0.0);
            r->F.assign(r->ndofs, 0.0);
            r->res.t_stage = now();
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            const bool timed = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
            if (timed) cudaEventRecord(e0, m->stream);
            if (!rc) rc = amr_stage_run(m, r->Uex.data(), r->Fex.data(), &r->stage, r->U.data(), r->F.data(),
                                        &r->res.stage);
            if (timed) {
                cudaEventRecord(e1, m->stream);
                float a = 0.f, b = 0.f;
                if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&a, ev_ref, e0) == cudaSuccess &&
                    cudaEventElapsedTime(&b, ev_ref, e1) == cudaSuccess) {
                    r->res.dev_start = a * 1e-3;
                    r->res.dev_end = b * 1e-3;
                }
            }
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
            cudaGetLastError();
            if (rc) {
                char buf[512];
                amr_last_error(m, buf, sizeof buf);
                r->err = buf;
            }
            amr_model_destroy(m);
        }
        r->res.status = rc;
    }

    void worker() {
        for (;;) {
            Request *r = nullptr;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] {
                    return stop || (!queue.empty() && active < cfg.max_active &&
                                    active_bytes + queue.front()->bytes <= (int64_t)cfg.hbm_budget_bytes);
                });
                if (stop) return;
                r = queue.front();
                queue.pop_front();
                active++;
                active_bytes += r->bytes;
                peak_active = std::max(peak_active, active);
                peak_bytes = std::max(peak_bytes, active_bytes);
                r->res.t_admit = now();
                r->res.active_at_admit = active;
            }
            cv_work.notify_all();  // another slot may take the next request as well
            run(r);
            {
                std::lock_guard<std::mutex> lk(mu);
                active--;
                active_bytes -= r->bytes;
                r->res.t_done = now();
                r->done = true;
                completed++;
            }
            cv_work.notify_all();
            cv_done.notify_all();
        }
    }
};

extern "C" {

int amr_estimate_bytes(const amr_model_desc *desc, int64_t *bytes) {
    if (!bytes) return AMR_EINVAL;
    const int64_t b = model_bytes(desc, AMR_SOLVER_MIXED);
    if (b < 0) return AMR_EINVAL;
    *bytes = b;
    return AMR_OK;
}

int amr_server_create(const amr_server_config *cfg, amr_server **out) {
    if (!cfg || !out || cfg->max_active < 1 || !(cfg->hbm_budget_bytes > 0)) return AMR_EINVAL;
    amr_server *s = new amr_server();
    s->cfg = *cfg;
    s->t0 = Clock::now();
    if (cudaGetDevice(&s->device) != cudaSuccess || cudaEventCreate(&s->ev_ref) != cudaSuccess ||
        cudaEventRecord(s->ev_ref, 0) != cudaSuccess || cudaEventSynchronize(s->ev_ref) != cudaSuccess) {
        cudaGetLastError();
        if (s->ev_ref) cudaEventDestroy(s->ev_ref);
        delete s;
        return AMR_ECUDA;
    }
    for (int i = 0; i < cfg->max_active; i++) s->workers.emplace_back([s] { s->worker(); });
    *out = s;
    return AMR_OK;
}

int amr_server_submit(amr_server *s, const amr_request *q, int64_t *id) {
    if (!s || !q || !id) return AMR_EINVAL;
    const amr_model_desc &d = q->model;
    if (!d.coords || !d.shape || !d.nips || !d.conn_ptr || !d.conn || !d.mat_type || !d.mat_params || !q->eq_id ||
        q->ndofs < 0 || q->nu < 0 || q->nu > q->ndofs || (q->ndofs > 0 && (!q->Uex || !q->Fex)) || q->nloads < 0 ||
        (q->nloads > 0 && !q->loads))
        return AMR_EINVAL;
    const int64_t bytes = model_bytes(&d, q->stage.linear.method);
    if (bytes < 0) return AMR_EINVAL;
    if (bytes > (int64_t)s->cfg.hbm_budget_bytes) return AMR_ENOMEM;  // could never be admitted
    auto r = std::make_unique<Request>();
    r->coords.assign(d.coords, d.coords + 3 * d.nnodes);
    r->shape.assign(d.shape, d.shape + d.nelems);
    r->nips.assign(d.nips, d.nips + d.nelems);
    r->conn_ptr.assign(d.conn_ptr, d.conn_ptr + d.nelems + 1);
    r->conn.assign(d.conn, d.conn + r->conn_ptr.back());
    r->mat_type.assign(d.mat_type, d.mat_type + d.nelems);
    r->mat_params.assign(d.mat_params, d.mat_params + 8 * d.nelems);
    r->desc = d;
    r->desc.coords = r->coords.data();
    r->desc.shape = r->shape.data();
    r->desc.nips = r->nips.data();
    r->desc.conn_ptr = r->conn_ptr.data();
    r->desc.conn = r->conn.data();
    r->desc.mat_type = r->mat_type.data();
    r->desc.mat_params = r->mat_params.data();
    r->eq_id.assign(q->eq_id, q->eq_id + 3 * d.nnodes);
    r->ndofs = q->ndofs;
    r->nu = q->nu;
    r->Uex.assign(q->Uex, q->Uex + q->ndofs);
    r->Fex.assign(q->Fex, q->Fex + q->ndofs);
    for (int32_t i = 0; i < q->nloads; i++) {
        const amr_load &L = q->loads[i];
        const int np = L.kind == AMR_LOAD_FACET ? amr::shape_npoints(L.facet_shape) : 1;
        if (np <= 0 || L.nitems < 0 || (L.nitems > 0 && !L.items)) return AMR_EINVAL;
        r->load_items.emplace_back(L.items, L.items + L.nitems * np);
        r->loads.push_back(L);
    }
    for (size_t i = 0; i < r->loads.size(); i++) r->loads[i].items = r->load_items[i].data();
    amr_default_stage_params(&r->stage);
    r->stage = q->stage;
    r->bytes = bytes;
    r->res.bytes = bytes;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->res.t_submit = s->now();
        *id = r->id;
        s->queue.push_back(r.get());
        s->reqs[r->id] = std::move(r);
    }
    s->cv_work.notify_all();
    return AMR_OK;
}

int amr_server_wait(amr_server *s, int64_t id, double *U, double *F, amr_request_result *res, char *err,
                    size_t nerr) {
    if (!s) return AMR_EINVAL;
    std::unique_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(id);
        if (it == s->reqs.end() || it->second->taken) return AMR_EINVAL;
        Request *p = it->second.get();
        p->taken = true;
        s->cv_done.wait(lk, [&] { return p->done; });
        r = std::move(it->second);
        s->reqs.erase(it);
    }
    if (U && !r->U.empty()) std::memcpy(U, r->U.data(), r->ndofs * sizeof(double));
    if (F && !r->F.empty()) std::memcpy(F, r->F.data(), r->ndofs * sizeof(double));
    if (res) *res = r->res;
    if (err && nerr) {
        std::strncpy(err, r->err.c_str(), nerr - 1);
        err[nerr - 1] = 0;
    }
    return r->res.status;
}

int amr_server_stats(amr_server *s, amr_server_info *st) {
    if (!s || !st) return AMR_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    st->queued = (int64_t)s->queue.size();
    st->active = s->active;
    st->peak_active = s->peak_active;
    st->completed = s->completed;
    st->active_bytes = s->active_bytes;
    st->peak_bytes = s->peak_bytes;
    st->seconds = s->now();
    return AMR_OK;
}

int amr_server_destroy(amr_server *s) {
    if (!s) return AMR_OK;
    {
        // finish what was admitted or queued, then stop the slots
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait(lk, [&] { return s->queue.empty() && s->active == 0; });
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    cudaEventDestroy(s->ev_ref);
    amr_trim_pool();  // the finished requests' memory goes back to the device
    delete s;
    return AMR_OK;
}

}  // extern "C"
