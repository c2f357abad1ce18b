// Coupled mounts: hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) and
// tm_mount_global_matrices (src/thermomech/thermomech-solver.jl:80-170) for solid elements with a linear
// elastic skeleton and a scalar field on the basic (corner) nodes -- the pore pressure uw of HMSolid
// (src/hydromech/elem/hydromech-solid.jl) with a constant isotropic permeability, or the temperature ut of
// TMSolid (src/thermomech/elem/thermomech-solid.jl) with a constant conductivity.
//
// G = [ K        C         ]   K the elastic stiffness, C = -c int Bu' m Nw' (c: Biot's alpha, or the
//     [ s C'     dt H + Cap ]   thermal stress modulus), H = -h int Bw' Bw, Cap = -cap int Nw Nw', s = 1 or
//                               T0 + 273.15 (the thermal mount scales the transposed coupling)
// RHS = -dt H phi (+ dt Q, Q = k int Bw' e_last, hydraulic only), phi the current nodal values.
//
// The reference pushes every entry of every element matrix (no eps() drop), K, C and C' interleaved, dt H
// and Cap, element by element, and sparse() sums duplicates in that order.  Here every node pair (a, b) of an
// element stages its (ndim+1) x (ndim+1) block with dt H and Cap kept apart; the deterministic gather sums
// the element blocks of each node block in element order through the model's contribution map; the RHS is
// gathered per node over its incidences in element order.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "amr_internal.h"

namespace {

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int basic_shape(int shape) {
    switch (shape) {
    case AMR_HEX8: case AMR_HEX20: return AMR_HEX8;
    case AMR_TET4: case AMR_TET10: return AMR_TET4;
    case AMR_QUAD4: case AMR_QUAD8: case AMR_QUAD9: return AMR_QUAD4;
    case AMR_TRI3: case AMR_TRI6: return AMR_TRI3;
    default: return -1;
    }
}

struct CoupledArgs {
    int ndim, ps, kind;
    double th, dt, s, gammaw;
    const double *coords;
    const int32_t *conn;
    const int64_t *conn_ptr, *kel_ptr;
    const double *mat_par;  // sorted elements x 8 (E, nu)
    const double *prm;      // sorted elements x 3
    const double *phiN;     // nodal scalar values (0 without the DOF)
    double *Gst;            // staging: kel_blocks x (B*B + 1)
    double *Rst;            // per sorted element, per basic node: dt H phi, dt Q
    int32_t *status;
};

// one CTA per element: the IP geometry in shared memory, then a thread per node pair
template <int DIM, int NEN, int NB>
__global__ void __launch_bounds__(256) k_coupled_elem(CoupledArgs A, int64_t first, const double *tab,
                                                      const double *btab, int nip, int64_t rst_stride) {
    constexpr int B = DIM + 1, SB = B * B + 1;
    const int64_t e = first + blockIdx.x;
    __shared__ double sG[AMR_MAXIP][NEN * DIM], sGw[AMR_MAXIP][NB * DIM], sNw[AMR_MAXIP][NB], sDv[AMR_MAXIP];
    __shared__ double sX[NEN * DIM];
    const int32_t *nodes = A.conn + A.conn_ptr[e];
    for (int t = threadIdx.x; t < NEN * DIM; t += blockDim.x) sX[t] = A.coords[(int64_t)nodes[t / DIM] * 3 + t % DIM];
    __syncthreads();
    // tab: [nip][NEN*DIM] dN/dR, [nip] w, [nip][NEN] N (the element's shape); btab: [nip][NB*DIM] dNw/dR, [nip][NB] Nw
    for (int ip = threadIdx.x; ip < nip; ip += blockDim.x) {
        const double *D = tab + (size_t)ip * NEN * DIM;
        double J[DIM * DIM];
        for (int a = 0; a < DIM; a++)
            for (int b = 0; b < DIM; b++) {
                double s = 0.0;
                for (int i = 0; i < NEN; i++) s += sX[i * DIM + a] * D[i * DIM + b];
                J[a * DIM + b] = s;
            }
        double det, Ji[DIM * DIM];
        if (DIM == 2) {
            det = J[0] * J[3] - J[1] * J[2];
            Ji[0] = J[3] / det; Ji[1] = -J[1] / det; Ji[2] = -J[2] / det; Ji[3] = J[0] / det;
        } else {
            const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[3] * J[8] - J[5] * J[6], c2 = J[3] * J[7] - J[4] * J[6];
            det = J[0] * c0 - J[1] * c1 + J[2] * c2;
            Ji[0] = c0 / det; Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det; Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
            Ji[3] = -c1 / det; Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det; Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
            Ji[6] = c2 / det; Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det; Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
        }
        if (!(det > 0.0)) {
            atomicCAS(&A.status[0], 0, AMR_ENEGJAC);
            atomicMin(&A.status[1], (int32_t)e);
        }
        for (int i = 0; i < NEN; i++)
            for (int b = 0; b < DIM; b++) {
                double s = 0.0;
                for (int a = 0; a < DIM; a++) s += D[i * DIM + a] * Ji[a * DIM + b];
                sG[ip][i * DIM + b] = s;
            }
        const double *Dw = btab + (size_t)ip * NB * DIM;
        for (int i = 0; i < NB; i++) {
            for (int b = 0; b < DIM; b++) {
                double s = 0.0;
                for (int a = 0; a < DIM; a++) s += Dw[i * DIM + a] * Ji[a * DIM + b];
                sGw[ip][i * DIM + b] = s;
            }
            sNw[ip][i] = btab[(size_t)nip * NB * DIM + (size_t)ip * NB + i];
        }
        sDv[ip] = det * tab[(size_t)nip * NEN * DIM + ip] * A.th;
    }
    __syncthreads();
    const double *par = A.mat_par + e * 8;
    const double E = par[0], nu = par[1];
    const double mu = E / (2.0 * (1.0 + nu));
    const double lam = A.ps ? E * nu / (1.0 - nu * nu) : E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    const double alpha = A.prm[e * 3 + 0], kc = A.prm[e * 3 + 1], cap = A.prm[e * 3 + 2];
    // coupling factor: Biot's alpha, or the thermal stress modulus E alpha / (1 - 2 nu) (1 - nu in plane stress)
    const double cc = A.kind == AMR_COUPLED_HYDRO ? alpha : (A.ps ? E * alpha / (1.0 - nu) : E * alpha / (1.0 - 2.0 * nu));
    const double ch = A.kind == AMR_COUPLED_HYDRO ? kc / A.gammaw : kc;  // conductivity factor of H
    const int64_t base = A.kel_ptr[e];
    for (int t = threadIdx.x; t < NEN * NEN; t += blockDim.x) {
        const int a = t / NEN, b = t % NEN;
        double T[DIM * DIM], Cab[DIM], Cba[DIM], Hs = 0.0, Ms = 0.0;
        for (int q = 0; q < DIM * DIM; q++) T[q] = 0.0;
        for (int c = 0; c < DIM; c++) Cab[c] = Cba[c] = 0.0;
        for (int ip = 0; ip < nip; ip++) {
            const double dv = sDv[ip];
            const double *ga = sG[ip] + a * DIM, *gb = sG[ip] + b * DIM;
            for (int c = 0; c < DIM; c++) {
                const double wg = dv * ga[c];
                for (int d = 0; d < DIM; d++) T[c * DIM + d] += wg * gb[d];
            }
            if (b < NB)
                for (int c = 0; c < DIM; c++) Cab[c] += dv * ga[c] * sNw[ip][b];
            if (a < NB)
                for (int d = 0; d < DIM; d++) Cba[d] += dv * gb[d] * sNw[ip][a];
            if (a < NB && b < NB) {
                double gg = 0.0;
                for (int c = 0; c < DIM; c++) gg += sGw[ip][a * DIM + c] * sGw[ip][b * DIM + c];
                Hs += dv * gg;
                Ms += dv * sNw[ip][a] * sNw[ip][b];
            }
        }
        double *o = A.Gst + (base + (int64_t)a * NEN + b) * SB;
        double tr = 0.0;
        for (int c = 0; c < DIM; c++) tr += T[c * DIM + c];
        for (int c = 0; c < DIM; c++)
            for (int d = 0; d < DIM; d++)
                o[c * B + d] = lam * T[c * DIM + d] + mu * T[d * DIM + c] + (c == d ? mu * tr : 0.0);
        for (int c = 0; c < DIM; c++) o[c * B + DIM] = b < NB ? -cc * Cab[c] : 0.0;
        for (int d = 0; d < DIM; d++) o[DIM * B + d] = a < NB ? A.s * (-cc * Cba[d]) : 0.0;
        const bool ww = a < NB && b < NB;
        o[DIM * B + DIM] = ww ? A.dt * (-ch * Hs) : 0.0;  // alpha dt H with alpha = 1
        o[SB - 1] = ww ? -cap * Ms : 0.0;
    }
    // the element's right-hand side at its basic nodes: dt (H phi)_a and dt Q_a
    for (int a = threadIdx.x; a < NB; a += blockDim.x) {
        double hp = 0.0, qa = 0.0;
        for (int b = 0; b < NB; b++) {
            double h = 0.0;
            for (int ip = 0; ip < nip; ip++) {
                double gg = 0.0;
                for (int c = 0; c < DIM; c++) gg += sGw[ip][a * DIM + c] * sGw[ip][b * DIM + c];
                h += sDv[ip] * gg;
            }
            hp += (-ch * h) * A.phiN[nodes[b]];
        }
        for (int ip = 0; ip < nip; ip++) qa += sDv[ip] * kc * sGw[ip][a * DIM + DIM - 1];
        A.Rst[(e * rst_stride + a) * 2 + 0] = A.dt * hp;
        A.Rst[(e * rst_stride + a) * 2 + 1] = A.kind == AMR_COUPLED_HYDRO ? A.dt * qa : 0.0;
    }
}

// G blocks: the element blocks of each node block summed in element order (the w-w entry: dt H, then Cap)
template <int B>
__global__ void k_coupled_gather(int64_t nnodes, int64_t nbs, const int64_t *rp, const int64_t *contrib_ptr,
                                 const int64_t *contrib, const double *Gst, double *G) {
    constexpr int SB = B * B + 1;
    const int lane = threadIdx.x & 31;
    const int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (n >= nnodes) return;
    for (int64_t k = rp[n] + lane; k < rp[n + 1]; k += 32) {
        double v[B * B];
        for (int q = 0; q < B * B; q++) v[q] = 0.0;
        for (int64_t c = contrib_ptr[k]; c < contrib_ptr[k + 1]; c++) {
            const double *src = Gst + contrib[c] * SB;
            for (int q = 0; q < B * B; q++) v[q] += src[q];
            v[B * B - 1] += src[SB - 1];
        }
        for (int q = 0; q < B * B; q++) G[(int64_t)q * nbs + k] = v[q];
    }
}

// RHS at each node's scalar DOF: over its incidences in element order, RHS - dt H phi + dt Q
__global__ void k_coupled_rhs(int64_t nnodes, const int64_t *inc_ptr, const int64_t *inc, const int32_t *nb_of,
                              const double *Rst, int64_t rst_stride, double *out) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes) return;
    double r = 0.0;
    for (int64_t q = inc_ptr[n]; q < inc_ptr[n + 1]; q++) {
        const int64_t e = inc[q] >> 8;
        const int a = (int)(inc[q] & 0xff);
        if (a >= nb_of[e]) continue;
        r = r - Rst[(e * rst_stride + a) * 2 + 0];
        r = r + Rst[(e * rst_stride + a) * 2 + 1];
    }
    out[n] = r;
}

template <int DIM, int NEN, int NB>
void launch_elem(amr_model *m, const CoupledArgs &a, const AmrGroup &g, const double *btab, int64_t rst_stride) {
    k_coupled_elem<DIM, NEN, NB><<<(unsigned)g.count, 256, 0, m->stream>>>(a, g.first, g.tab, btab, g.nip,
                                                                             rst_stride);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

void launch_group(amr_model *m, const CoupledArgs &a, const AmrGroup &g, const double *btab, int64_t rst_stride) {
    switch (g.shape) {
    case AMR_HEX8: launch_elem<3, 8, 8>(m, a, g, btab, rst_stride); break;
    case AMR_HEX20: launch_elem<3, 20, 8>(m, a, g, btab, rst_stride); break;
    case AMR_TET4: launch_elem<3, 4, 4>(m, a, g, btab, rst_stride); break;
    case AMR_TET10: launch_elem<3, 10, 4>(m, a, g, btab, rst_stride); break;
    case AMR_QUAD4: launch_elem<2, 4, 4>(m, a, g, btab, rst_stride); break;
    case AMR_QUAD8: launch_elem<2, 8, 4>(m, a, g, btab, rst_stride); break;
    case AMR_QUAD9: launch_elem<2, 9, 4>(m, a, g, btab, rst_stride); break;
    case AMR_TRI3: launch_elem<2, 3, 3>(m, a, g, btab, rst_stride); break;
    case AMR_TRI6: launch_elem<2, 6, 3>(m, a, g, btab, rst_stride); break;
    default: throw AmrError(AMR_EUNSUPPORTED, "shape without a basic shape on the coupled path");
    }
}

// column-major walk of the structural pattern: every scalar entry whose row and column DOFs exist
template <class F>
void walk(const amr_model *m, const int64_t *eq4, F f) {
    const int ndim = m->ndim, B = ndim + 1;
    for (int64_t n = 0; n < m->nnodes; n++)
        for (int64_t k = m->h_brow_ptr[n]; k < m->h_brow_ptr[n + 1]; k++) {
            const int64_t j = m->h_bcol[k];
            for (int c = 0; c < B; c++) {
                const int64_t r = eq4[4 * n + (c < ndim ? c : 3)];
                if (r < 0) continue;
                for (int d = 0; d < B; d++) {
                    const int64_t col = eq4[4 * j + (d < ndim ? d : 3)];
                    if (col >= 0) f(r, col, k, c * B + d);
                }
            }
        }
}

}  // namespace

extern "C" int amr_coupled_mount(amr_model *m, const amr_coupled_desc *d, const int64_t *eq4, int64_t ndofs,
                                 double dt, const double *phi, int64_t *nnz, int64_t *colptr, int64_t *rowval,
                                 double *nzval, double *rhs) {
    if (!m) return AMR_EINVAL;
    AmrStreamScope scope(m->stream);
    try {
        m->err.clear();
        if (!d || !eq4 || !nnz || ndofs < 0) throw AmrError(AMR_EINVAL, "null argument");
        if (d->kind != AMR_COUPLED_HYDRO && d->kind != AMR_COUPLED_THERMO) throw AmrError(AMR_EINVAL, "unknown kind");
        if (m->stressmodel == AMR_AXISYMMETRIC) throw AmrError(AMR_EUNSUPPORTED, "axisymmetric coupled mounts");
        if (m->batch) throw AmrError(AMR_EUNSUPPORTED, "coupled mounts of batched parts are not supported");
        if (d->kind == AMR_COUPLED_HYDRO && !(d->gammaw > 0.0)) throw AmrError(AMR_EINVAL, "gammaw must be > 0");
        for (int64_t i = 0; i < 4 * m->nnodes; i++)
            if (eq4[i] >= ndofs) throw AmrError(AMR_EINVAL, "DOF number beyond ndofs");
        for (const AmrGroup &g : m->groups)
            if (basic_shape(g.shape) < 0) throw AmrError(AMR_EUNSUPPORTED, "shape without a basic shape");
        // the structural pattern's size
        int64_t count = 0;
        walk(m, eq4, [&](int64_t, int64_t, int64_t, int) { count++; });
        *nnz = count;
        if (!colptr) return AMR_OK;
        if (!rowval || !nzval || !rhs || !d->params || (!phi && ndofs > 0)) throw AmrError(AMR_EINVAL, "null buffer");
        std::vector<int32_t> mt(m->nelems);
        amr_d2h(m, mt.data(), m->mat_type, m->nelems * sizeof(int32_t));
        for (int32_t t : mt)
            if (t != AMR_LINEAR_ELASTIC) throw AmrError(AMR_EUNSUPPORTED, "the coupled skeleton must be linear elastic");
        const int ndim = m->ndim, B = ndim + 1, SB = B * B + 1;
        const int64_t nn = m->nnodes, ne = m->nelems;
        cudaStream_t s = m->stream;
        // per sorted element: the coupled parameters and the basic-node count; nodal values of the scalar
        std::vector<double> prm(3 * ne), phiN(nn, 0.0);
        std::vector<int32_t> nb_of(ne);
        for (int64_t e = 0; e < ne; e++) {
            const int64_t c = m->perm[e];
            for (int q = 0; q < 3; q++) prm[3 * e + q] = d->params[3 * c + q];
            nb_of[e] = amr::shape_npoints(basic_shape(m->h_shape[e]));
        }
        for (int64_t n = 0; n < nn; n++)
            if (eq4[4 * n + 3] >= 0) phiN[n] = phi[eq4[4 * n + 3]];
        std::vector<void *> bufs;
        struct Free {
            std::vector<void *> &b;
            ~Free() {
                for (void *&p : b) amr_free(p);
            }
        } free_bufs{bufs};
        auto dalloc = [&](size_t bytes) {
            unsigned char *p = nullptr;
            amr_alloc(&p, bytes);
            bufs.push_back(p);
            return (void *)p;
        };
        double *d_prm = (double *)dalloc(prm.size() * sizeof(double));
        double *d_phi = (double *)dalloc(nn * sizeof(double));
        int32_t *d_nb = (int32_t *)dalloc(ne * sizeof(int32_t));
        AMR_CUDA(cudaMemcpyAsync(d_prm, prm.data(), prm.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        AMR_CUDA(cudaMemcpyAsync(d_phi, phiN.data(), nn * sizeof(double), cudaMemcpyHostToDevice, s));
        AMR_CUDA(cudaMemcpyAsync(d_nb, nb_of.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        const int64_t rst_stride = 8;  // basic nodes per element at most
        double *Gst = (double *)dalloc((size_t)m->kel_blocks * SB * sizeof(double));
        double *Rst = (double *)dalloc((size_t)ne * rst_stride * 2 * sizeof(double));
        double *G = (double *)dalloc((size_t)m->bstride * B * B * sizeof(double));
        double *R = (double *)dalloc(nn * sizeof(double));
        CoupledArgs a;
        a.ndim = ndim; a.ps = m->stressmodel == AMR_PLANESTRESS; a.kind = d->kind;
        a.th = m->thickness; a.dt = dt; a.s = d->kind == AMR_COUPLED_HYDRO ? 1.0 : d->T0 + 273.15; a.gammaw = d->gammaw;
        a.coords = m->coords; a.conn = m->conn; a.conn_ptr = m->conn_ptr; a.kel_ptr = m->kel_ptr;
        a.mat_par = m->mat_par; a.prm = d_prm; a.phiN = d_phi; a.Gst = Gst; a.Rst = Rst; a.status = m->d_status;
        for (const AmrGroup &g : m->groups) {
            // the basic shape's derivatives and functions at the group's IPs
            double R3[64 * 3], w[64];
            const int bs = basic_shape(g.shape), nb = amr::shape_npoints(bs);
            const int nq = amr::quadrature(g.shape, m->h_nips[g.first], R3, w);
            if (nq != g.nip) throw AmrError(AMR_EINVAL, "quadrature of a group");
            std::vector<double> bt((size_t)g.nip * nb * ndim + (size_t)g.nip * nb);
            for (int q = 0; q < g.nip; q++) {
                amr::shape_deriv(bs, R3 + 3 * q, bt.data() + (size_t)q * nb * ndim);
                amr::shape_func(bs, R3 + 3 * q, bt.data() + (size_t)g.nip * nb * ndim + (size_t)q * nb);
            }
            double *d_bt = (double *)dalloc(bt.size() * sizeof(double));
            AMR_CUDA(cudaMemcpyAsync(d_bt, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice, s));
            launch_group(m, a, g, d_bt, rst_stride);
            AMR_CUDA(cudaStreamSynchronize(s));  // the host table goes out of scope
        }
        if (int rc = amr_check_status(m)) {
            if (rc == AMR_ENEGJAC)
                throw AmrError(rc, "Negative Jacobian determinant in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
            throw AmrError(rc, "coupled element matrices failed");
        }
        if (ndim == 3)
            k_coupled_gather<4><<<nblk(nn * 32, 256), 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->contrib_ptr,
                                                                   m->contrib, Gst, G);
        else
            k_coupled_gather<3><<<nblk(nn * 32, 256), 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->contrib_ptr,
                                                                   m->contrib, Gst, G);
        k_coupled_rhs<<<nblk(nn, 256), 256, 0, s>>>(nn, m->inc_ptr, m->inc, d_nb, Rst, rst_stride, R);
        AMR_COUNT(2);
        AMR_CUDA(cudaGetLastError());
        std::vector<double> hG((size_t)m->bstride * B * B), hR(nn);
        amr_d2h(m, hG.data(), G, hG.size() * sizeof(double));
        amr_d2h(m, hR.data(), R, nn * sizeof(double));
        // RHS at the scalar DOFs, zero elsewhere
        std::fill(rhs, rhs + ndofs, 0.0);
        for (int64_t n = 0; n < nn; n++)
            if (eq4[4 * n + 3] >= 0) rhs[eq4[4 * n + 3]] = hR[n];
        // CSC in the reference's layout: rows sorted within each column
        std::vector<int64_t> cnt(ndofs + 1, 0);
        walk(m, eq4, [&](int64_t, int64_t col, int64_t, int) { cnt[col + 1]++; });
        for (int64_t i = 0; i < ndofs; i++) cnt[i + 1] += cnt[i];
        std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
        walk(m, eq4, [&](int64_t r, int64_t col, int64_t k, int q) {
            const int64_t p = pos[col]++;
            rowval[p] = r;
            nzval[p] = hG[(size_t)q * m->bstride + k];
        });
        std::vector<std::pair<int64_t, double>> tmp;
        for (int64_t col = 0; col < ndofs; col++) {
            const int64_t lo = cnt[col], hi = cnt[col + 1];
            tmp.resize(hi - lo);
            for (int64_t p = lo; p < hi; p++) tmp[p - lo] = {rowval[p], nzval[p]};
            std::sort(tmp.begin(), tmp.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
            for (int64_t p = lo; p < hi; p++) {
                rowval[p] = tmp[p - lo].first;
                nzval[p] = tmp[p - lo].second;
            }
        }
        for (int64_t i = 0; i <= ndofs; i++) colptr[i] = cnt[i];
        return AMR_OK;
    } catch (const AmrError &e) {
        m->err = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        m->err = e.what();
        return AMR_EINVAL;
    }
}
