// Dynamic mechanical stage on the device: dyn_stage_solver! (src/mech/dyn-solver.jl:203-534).
//
// Newmark's average-acceleration rule with Rayleigh damping C = alpha M + beta K.  Every Newton
// iteration solves Kp dUi = dFp with the pseudo-stiffness Kp = K + 4/dt^2 M + 2/dt C and
//   dFp  = Fex - Fina + M (A + 4 V/dt - 4 dUa/dt^2) + C (V - 2 dUa/dt),
// updates the IP states from the committed ones with dUt = dUa + dUi, and checks the residue of
//   TFin = Fina + C Va + M Aa,  Va = -V + 2 dUt/dt,  Aa = -A + 4 (dUt - V dt)/dt^2
// over the unknown DOFs.  The first stage starts from M A0 = Fex(0) (:270-296); the reference defines
// V and A only there, so a dynamic analysis is one stage.
//
// Device layout: node-major FP64 vectors (nnodes x B) as in the static stage; M64 on K's block
// pattern; K kept in Ks while K64 holds Kp for the solver.  C is never stored: the SpMV forms
// C y = alpha (M y) + beta (K y).  For state-independent K
// (no plastic material) K is mounted once per stage and Kp only when dt changes: the reference mounts
// both at every iteration, with the same values.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "amr_internal.h"

namespace {

constexpr int kThreads = 256;

// out = base + M x + C y with C = alpha M + beta K (K may be null); warp per node row.  Every block of
// M is m_ab I (elem_mass has no entry between components, and the three diagonal components of a block
// sum the same contributions in the same order), so the kernel reads component (0,0) of M only and forms
// C y as alpha (M y) + beta (K y) per row; with beta = 0 it reads no K.
constexpr int kRowLanes = 4;  // lanes per block row; the warp's rows share the reduction steps
template <int B>
__global__ void __launch_bounds__(kThreads) k_dyn_rhs(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                      const int32_t *__restrict__ cj, const double *__restrict__ M,
                                                      const double *__restrict__ K, double alpha, double beta,
                                                      const double *__restrict__ base, const double *__restrict__ x,
                                                      const double *__restrict__ y, double *__restrict__ out) {
    constexpr int RPW = 32 / kRowLanes;
    const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool useK = K && beta != 0.0;
    for (int64_t n0 = warp * RPW; n0 < nn; n0 += nw * RPW) {  // whole warps: every lane reaches the shuffles
        const int64_t n = n0 + lane / kRowLanes;
        const bool valid = n < nn;
        double mx[B], my[B], ky[B];
#pragma unroll
        for (int c = 0; c < B; c++) mx[c] = my[c] = ky[c] = 0.0;
        if (valid)
            for (int64_t k = rp[n] + sub; k < rp[n + 1]; k += kRowLanes) {
                const int64_t j = cj[k];
                const double m = M[k];
                double yj[B];
#pragma unroll
                for (int d = 0; d < B; d++) {
                    yj[d] = y[j * B + d];
                    mx[d] = fma(m, x[j * B + d], mx[d]);
                    my[d] = fma(m, yj[d], my[d]);
                }
                if (useK)
#pragma unroll
                    for (int c = 0; c < B; c++)
#pragma unroll
                        for (int d = 0; d < B; d++) ky[c] = fma(K[(int64_t)(c * B + d) * nb + k], yj[d], ky[c]);
            }
#pragma unroll
        for (int c = 0; c < B; c++)
#pragma unroll
            for (int o = kRowLanes / 2; o > 0; o >>= 1) {
                mx[c] += __shfl_xor_sync(0xffffffffu, mx[c], o);
                my[c] += __shfl_xor_sync(0xffffffffu, my[c], o);
                if (useK) ky[c] += __shfl_xor_sync(0xffffffffu, ky[c], o);
            }
        if (valid && sub == 0)
#pragma unroll
            for (int c = 0; c < B; c++)
                out[n * B + c] = base[n * B + c] + (mx[c] + (alpha * my[c] + beta * ky[c]));
    }
}

// x1 = A + 4 V/dt - 4 dUa/dt^2 and y1 = V - 2 dUa/dt, in the reference's operation order
__global__ void k_dyn_prep(int64_t n, double dt, const double *A, const double *V, const double *dUa, double *x1,
                           double *y1) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt2 = __dmul_rn(dt, dt);
    x1[i] = __dsub_rn(__dadd_rn(A[i], __ddiv_rn(__dmul_rn(4.0, V[i]), dt)), __ddiv_rn(__dmul_rn(4.0, dUa[i]), dt2));
    y1[i] = __dsub_rn(V[i], __ddiv_rn(__dmul_rn(2.0, dUa[i]), dt));
}

// dUt = dUa + dUi; Fina = Fin + dFin; Va = -V + 2 dUt/dt; Aa = -A + 4 (dUt - V dt)/dt^2
__global__ void k_dyn_post(int64_t n, double dt, const double *dUa, const double *dUi, const double *Fin,
                           const double *dFin, const double *V, const double *A, double *dUt, double *Fina,
                           double *Va, double *Aa) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double u = __dadd_rn(dUa[i], dUi[i]);
    dUt[i] = u;
    Fina[i] = __dadd_rn(Fin[i], dFin[i]);
    Va[i] = __dadd_rn(-V[i], __ddiv_rn(__dmul_rn(2.0, u), dt));
    Aa[i] = __dadd_rn(-A[i], __ddiv_rn(__dmul_rn(4.0, __dsub_rn(u, __dmul_rn(V[i], dt))), __dmul_rn(dt, dt)));
}

// R = (Fex - TFin) at free slots; dUa += dUi; FexFin = (Fex - Fina) at free slots, 0 elsewhere
__global__ void k_dyn_after(int64_t n, const uint8_t *fm, const double *Fex, const double *TFin, const double *Fina,
                            const double *dUi, double *R, double *dUa, double *FexFin) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    R[i] = fm[i] ? __dsub_rn(Fex[i], TFin[i]) : 0.0;
    dUa[i] = __dadd_rn(dUa[i], dUi[i]);
    FexFin[i] = fm[i] ? __dsub_rn(Fex[i], Fina[i]) : 0.0;
}

// o = x at free slots, y at the others (solve_system!'s F with the reactions at prescribed DOFs)
__global__ void k_dyn_merge(int64_t n, const uint8_t *fm, const double *x, const double *y, double *o) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    o[i] = fm[i] ? x[i] : y[i];
}

// o = a x + b y (y may be null), elementwise
__global__ void k_dyn_axpby(int64_t n, double a, const double *x, double b, const double *y, double *o) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    o[i] = y ? __dadd_rn(__dmul_rn(a, x[i]), __dmul_rn(b, y[i])) : __dmul_rn(a, x[i]);
}

// M e_dir: the row sums of the mass blocks' scalar (every block is m I), in component dir
__global__ void k_mass_rowsum(int64_t nnodes, int B, int dir, const int64_t *rp, const double *M, double *me) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nnodes) return;
    double acc = 0.0;
    for (int64_t k = rp[i]; k < rp[i + 1]; k++) acc += M[k];  // component (0,0) of block k
    for (int c = 0; c < B; c++) me[i * B + c] = c == dir ? acc : 0.0;
}

}  // namespace

namespace {

unsigned blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

void assemble_K(amr_model *m) {
    amr_stiffness(m);
    const int rc = amr_check_status(m);
    if (rc == AMR_ENEGJAC)
        throw AmrError(rc, "Negative Jacobian determinant in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
    if (rc == AMR_ENAN) throw AmrError(rc, "NaN values in coefficients matrix");
    if (rc) throw AmrError(rc, "assembly failed");
    m->K_valid = true;
}

void rhs(amr_model *m, const double *Ks, double alpha, double beta, const double *base, const double *x,
         const double *y, double *out) {
    int dev = 0, sms = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const unsigned g = (unsigned)std::min<int64_t>((m->nnodes * 32 + kThreads - 1) / kThreads, (int64_t)sms * 8);
    if (m->B == 3)
        k_dyn_rhs<3><<<std::max(1u, g), kThreads, 0, m->stream>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol,
                                                                   m->M64, Ks, alpha, beta, base, x, y, out);
    else
        k_dyn_rhs<2><<<std::max(1u, g), kThreads, 0, m->stream>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol,
                                                                   m->M64, Ks, alpha, beta, base, x, y, out);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

void axpby(amr_model *m, double a, const double *x, double b, const double *y, double *o) {
    const int64_t n = m->nnodes * m->B;
    k_dyn_axpby<<<blocks(n), kThreads, 0, m->stream>>>(n, a, x, b, y, o);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

// The acceleration of sismic_force (src/mech/dyn-solver.jl:110-146) at t: the record preceded by 0 at
// times i tds / n, linear between samples, from the last interval that holds t (the reference's search
// never stops early); beyond the record the reference fails, and so does this.
double seismic_acceleration(const amr_dyn_params &p, double t) {
    const int64_t n = p.sism_n;
    auto at = [&](int64_t i) { return i == 0 ? 0.0 : p.sism_acc[i - 1]; };
    auto ts = [&](int64_t i) { return (double)i * p.tds / (double)n; };
    int64_t ini = -1;
    for (int64_t i = 0; i < n; i++)
        if (ts(i) <= t && t <= ts(i + 1)) ini = i;
    if (ini < 0) throw AmrError(AMR_EINVAL, "the seismic record does not cover t = " + std::to_string(t));
    const double m = (at(ini + 1) - at(ini)) / (ts(ini + 1) - ts(ini));
    return at(ini) + m * (t - ts(ini));
}

double round_sig3(double x) {
    if (x == 0.0 || !std::isfinite(x)) return x;
    const double e = std::floor(std::log10(std::fabs(x)));
    const double sc = std::pow(10.0, 2.0 - e);
    return std::round(x * sc) / sc;
}

}  // namespace

int amr_dyn_stage_device(amr_model *m, const double *U0, const double *U1, const double *F0, const double *F1,
                         const amr_dyn_params &p, double *U, double *V, double *A, double *F,
                         amr_stage_stats *stats) {
    if (m->batch) throw AmrError(AMR_EUNSUPPORTED, "dynamic stages of batched parts are not supported");
    if (p.maxits < 1 || p.nincs < 1 || !(p.tspan > 0.0)) throw AmrError(AMR_EINVAL, "bad dynamic stage parameters");
    if (p.sism && (!p.sism_acc || p.sism_n < 1 || !(p.tds > 0.0) || p.sism_dir < 0 || p.sism_dir >= m->ndim))
        throw AmrError(AMR_EINVAL, "seismic input needs a record, tds > 0 and a direction of the model");
    const int64_t n = m->nnodes * m->B;
    cudaStream_t s = m->stream;
    const size_t nK = (size_t)m->bstride * m->BB;
    const size_t nst = (size_t)AMR_NST * m->nip_total * sizeof(double);
    AmrEventPair ev;  // destroyed on every exit
    cudaEvent_t t0 = ev.t0, t1 = ev.t1;
    std::vector<double *> v(17, nullptr);
    double *Ks = nullptr;
    auto release = [&]() {
        for (auto &x : v) amr_free(x);
        amr_free(Ks);
    };
    try {
        for (auto &x : v) amr_alloc(&x, n);
        amr_alloc(&Ks, nK);
    } catch (...) {
        release();
        throw;
    }
    double *Fex = v[0], *Uex = v[1], *Fin = v[2], *Fina = v[3], *FexFin = v[4], *dUa = v[5], *dUi = v[6],
           *dUt = v[7], *dFin = v[8], *Va = v[9], *Aa = v[10], *x1 = v[11], *y1 = v[12], *dFp = v[13], *R = v[14],
           *reac = v[15], *Me = v[16];
    int status = AMR_OK;
    amr_stage_stats st{};
    try {
        AMR_CUDA(cudaEventRecord(t0, s));
        for (double *x : {U, V, A, F, Fin, Fina, dUa, dUi, Va, Aa})
            AMR_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
        // initial accelerations: K and M mounted, M A = Fex(0) (dyn-solver.jl:276-296); F keeps Fex(0)
        // with the reactions M21 A1 at the prescribed DOFs, as dof.vals[fs]
        assemble_K(m);
        AMR_CUDA(cudaMemcpyAsync(Ks, m->K64, nK * sizeof(double), cudaMemcpyDeviceToDevice, s));
        amr_mass(m);
        if (int rc = amr_check_status(m)) throw AmrError(rc, "mass assembly failed");
        axpby(m, 1.0, F0, 0.0, F1, Fex);
        if (p.sism) {  // M e_dir once: M does not change in the stage (the reference mounts it again)
            k_mass_rowsum<<<blocks(m->nnodes), kThreads, 0, s>>>(m->nnodes, m->B, p.sism_dir, m->brow_ptr, m->M64, Me);
            AMR_COUNT(1);
            if (p.tss <= 0.0) axpby(m, 1.0, Fex, seismic_acceleration(p, 0.0), Me, Fex);
        }
        amr_dyn_combine(m, nullptr, 1.0, 0.0, 0.0, 0.0);  // K64 = M
        AMR_CUDA(cudaMemsetAsync(reac, 0, n * sizeof(double), s));
        {
            AmrSolveResult sr = amr_solve_device(m, A, Fex, reac, p.linear);
            st.krylov_iterations += sr.iterations;
            st.solve_seconds += sr.seconds;
            if (sr.status) throw AmrError(AMR_ENOCONV, "initial accelerations: Krylov solver did not converge");
        }
        k_dyn_merge<<<blocks(n), kThreads, 0, s>>>(n, m->free_mask, Fex, reac, F);
        AMR_COUNT(1);
        AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, nst, cudaMemcpyDeviceToDevice, s));
        const bool saveouts = p.nouts > 0;
        const double dTmin = p.dTmin, tol = p.tol;
        const double dTcheck = saveouts ? 1.0 / p.nouts : 1.0;
        double Tcheck = dTcheck, T = 0.0, dT = 1.0 / p.nincs, dTbk = 0.0, t = 0.0;
        if (p.autoinc) dT = std::min({dT, p.dTmax, dTcheck});
        double kp_dt = -1.0;  // dt of the Kp in K64 (state-independent K only)
        while (T < 1.0 - dTmin) {
            const double dt = p.tspan * dT;
            const double s1 = 4.0 / (dt * dt), s2 = 2.0 / dt;
            axpby(m, 1.0, U0, t + dt, U1, Uex);
            axpby(m, 1.0, F0, t + dt, F1, Fex);
            if (p.sism && p.tss <= t + dt && p.tds + p.tss >= t + dt)
                axpby(m, 1.0, Fex, seismic_acceleration(p, t + dt), Me, Fex);
            axpby(m, 1.0, Fex, -1.0, Fina, FexFin);
            AMR_CUDA(cudaMemsetAsync(dUa, 0, n * sizeof(double), s));
            AMR_CUDA(cudaMemcpyAsync(dUi, Uex, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            double res = 0.0, res1 = 0.0;
            const int maxfails = 3;
            int nfails = 0;
            const int nits = 0;  // the reference never counts it (dyn-solver.jl:363,491)
            bool converged = false;
            for (int it = 1; it <= p.maxits; it++) {
                if (it > 1) AMR_CUDA(cudaMemsetAsync(dUi, 0, n * sizeof(double), s));
                const double lastres = res;
                if (m->any_plastic) {
                    assemble_K(m);
                    AMR_CUDA(cudaMemcpyAsync(Ks, m->K64, nK * sizeof(double), cudaMemcpyDeviceToDevice, s));
                    kp_dt = -1.0;
                }
                if (kp_dt != dt) {
                    amr_dyn_combine(m, Ks, s1, s2, p.alpha, p.beta);
                    if (int rc = amr_check_status(m)) throw AmrError(rc, "NaN values in the pseudo-stiffness matrix");
                    kp_dt = dt;
                }
                // dFp = Fex - Fina + M x1 + C y1; solve Kp dUi = dFp (prescribed slots of dUi: Uex, then 0)
                k_dyn_prep<<<blocks(n), kThreads, 0, s>>>(n, dt, A, V, dUa, x1, y1);
                AMR_COUNT(1);
                rhs(m, Ks, p.alpha, p.beta, FexFin, x1, y1, dFp);
                AmrSolveResult sr = amr_solve_device(m, dUi, dFp, reac, p.linear);
                st.krylov_iterations += sr.iterations;
                st.solve_seconds += sr.seconds;
                st.iterations++;
                if (sr.status) { res = NAN; break; }
                // states from the committed ones with dUt = dUa + dUi
                axpby(m, 1.0, dUa, 1.0, dUi, dUt);
                amr_update_elements(m, dUt, dFin);
                if (amr_check_status(m)) { res = NAN; break; }
                k_dyn_post<<<blocks(n), kThreads, 0, s>>>(n, dt, dUa, dUi, Fin, dFin, V, A, dUt, Fina, Va, Aa);
                AMR_COUNT(1);
                // TFin = Fina + C Va + M Aa (in F); residue over the unknowns
                rhs(m, Ks, p.alpha, p.beta, Fina, Aa, Va, F);
                k_dyn_after<<<blocks(n), kThreads, 0, s>>>(n, m->free_mask, Fex, F, Fina, dUi, R, dUa, FexFin);
                AMR_COUNT(1);
                res = amr_norm_inf(m, R, m->free_mask);
                if (it == 1) res1 = res;
                if (res > tol) axpby(m, 1.0, Fina, -1.0, dFin, Fina);
                if (res < tol) { converged = true; break; }
                if (std::isnan(res)) break;
                if (it > 1 && res > lastres) break;
                if (res > 0.9 * lastres) nfails++;
                if (nfails == maxfails) break;
            }
            st.residue = res;
            if (converged) {
                AMR_CUDA(cudaMemcpyAsync(Fin, Fina, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                axpby(m, 1.0, U, 1.0, dUa, U);
                AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, nst, cudaMemcpyDeviceToDevice, s));
                AMR_CUDA(cudaMemcpyAsync(A, Aa, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                AMR_CUDA(cudaMemcpyAsync(V, Va, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
                T += dT;
                t += dt;
                st.increments++;
                if (T > Tcheck - dTmin) Tcheck += dTcheck;
                if (p.autoinc) {
                    if (dTbk > 0.0) {
                        dT = std::min(dTbk, Tcheck - T);
                        dTbk = 0.0;
                    } else {
                        const double q = nits == 1 ? 1 + std::tanh(std::log10(tol / res1)) : 1.0;
                        const double dTtr = std::min({q * dT, 1.0 / p.nincs, 1 - T});
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
                AMR_CUDA(cudaMemcpyAsync(m->st, m->stbk, nst, cudaMemcpyDeviceToDevice, s));
                if (p.autoinc) {
                    double q = 1 + std::tanh(std::log10(tol / res1));
                    q = std::min(std::max(q, 0.2), 0.9);
                    dT = round_sig3(q * dT);
                    if (dT < dTmin) { status = AMR_ESTAGE; m->err = "solver did not converge"; break; }
                } else {
                    status = AMR_ESTAGE;
                    m->err = "solver did not converge";
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

// Average device time of k_dyn_rhs with both matrices read (beta != 0, K64 as the K operand) and its
// algorithmic bytes: per block the (0,0) component of M, the 9 (4) components of K and the column index;
// per node the row pointer and x, y, base read and out written once.
double amr_dyn_time_rhs(amr_model *m, int reps, double *bytes) {
    if (!m->M64) throw AmrError(AMR_EINVAL, "assemble M first");
    const int64_t n = m->nnodes * m->B;
    std::vector<double *> v(4, nullptr);
    auto release = [&]() {
        for (auto &x : v) amr_free(x);
    };
    double sec = 0.0;
    try {
        for (auto &x : v) {
            amr_alloc(&x, n);
            AMR_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), m->stream));
        }
        rhs(m, m->K64, 0.5, 1e-4, v[0], v[1], v[2], v[3]);
        AMR_CUDA(cudaEventRecord(m->ev0, m->stream));
        for (int r = 0; r < reps; r++) rhs(m, m->K64, 0.5, 1e-4, v[0], v[1], v[2], v[3]);
        AMR_CUDA(cudaEventRecord(m->ev1, m->stream));
        AMR_CUDA(cudaEventSynchronize(m->ev1));
        float ms = 0.f;
        AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
        sec = ms * 1e-3 / std::max(1, reps);
    } catch (...) {
        release();
        throw;
    }
    release();
    if (bytes)
        *bytes = (double)m->nblocks * (8.0 + 8.0 * m->BB + 4.0) + (double)(m->nnodes + 1) * 8.0 +
                 4.0 * 8.0 * (double)n;
    return sec;
}
