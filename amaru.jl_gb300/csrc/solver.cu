// Linear solve of the Newton corrector, K11 U1 = F1 - K12 U2 (solve_system!,
// src/solver.jl:5-79), on the device.
//
// AMR_SOLVER_MIXED: preconditioned CG whose SpMV, block-Jacobi preconditioner
//   and vector updates run in FP32 over the node-block (BSR) matrix K32 with
//   Dirichlet rows/columns masked; every `refine_every` iterations the FP64
//   true residual r = b - K64 u is recomputed from the FP64 matrix, the FP32
//   correction is folded into the FP64 solution and the recursive residual is
//   replaced (iterative refinement by reliable updates; the search direction
//   is kept).  Convergence is decided on the FP64 true residual only.
// AMR_SOLVER_FP64 / AMR_SOLVER_AMG_FP64: the all-FP64 comparators of MIXED and
//   AMG: the same Krylov method and the same preconditioner, with the FP64 matrix
//   K64, FP64 block inverses (and an FP64 multigrid hierarchy) and FP64 vectors.
//
// Scalars (alpha, beta, norms) live in a device control block; each kernel's
// last CTA reduces the per-CTA partials in a fixed order, so results are
// bitwise reproducible run to run.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <mutex>

#include "amr_internal.h"

namespace {

struct Ctl {
    double rz, pq, alpha, beta, rr, rr_true, bnorm2, gold, aold;
    int32_t stop, converged, breakdown, iters, first, pad;
    unsigned int ticket[4];
};

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sum of up to 2 values, fixed order; result valid in thread 0
template <int NV>
__device__ void block_sum(double (&v)[NV], double (*sh)[kThreads / 32]) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        double x = warp_sum(v[i]);
        if (lane == 0) sh[i][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int i = 0; i < NV; i++) {
            double x = (lane < (int)(blockDim.x >> 5)) ? sh[i][lane] : 0.0;
            v[i] = warp_sum(x);
        }
    }
    __syncthreads();
}

// Writes this CTA's partials; returns true in the last CTA to finish, which then
// holds the fixed-order totals in tot[] (all threads).
template <int NV>
__device__ bool grid_sum(double (&v)[NV], double *partials, unsigned int *ticket, double (&tot)[NV]) {
    __shared__ double sh[NV][kThreads / 32];
    __shared__ bool last;
    block_sum<NV>(v, sh);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) partials[i * gridDim.x + blockIdx.x] = v[i];
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) {
        acc[i] = 0.0;
        for (unsigned j = threadIdx.x; j < gridDim.x; j += blockDim.x)
            acc[i] += ((volatile double *)partials)[i * gridDim.x + j];
    }
    block_sum<NV>(acc, sh);
    __shared__ double res[NV];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) res[i] = acc[i];
        *ticket = 0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; i++) tot[i] = res[i];
    return true;
}

// As grid_sum, for FP32 per-thread values: the CTA-level tree runs in FP32 (the FP64 pipe of
// this GPU is narrow enough that a per-CTA FP64 shuffle tree shows in a bandwidth-bound
// kernel); each CTA's partial is widened once and the last CTA adds them in FP64.
template <int NV>
__device__ bool grid_sumf(float (&v)[NV], double *partials, unsigned int *ticket, double (&tot)[NV]) {
    __shared__ float shf[NV][kThreads / 32];
    __shared__ double sh[NV][kThreads / 32];
    __shared__ bool last;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        float x = warp_sumf(v[i]);
        if (lane == 0) shf[i][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int i = 0; i < NV; i++) {
            float x = (lane < (int)(blockDim.x >> 5)) ? shf[i][lane] : 0.0f;
            x = warp_sumf(x);
            if (lane == 0) partials[i * gridDim.x + blockIdx.x] = (double)x;
        }
        if (lane == 0) {
            __threadfence();
            unsigned int t = atomicAdd(ticket, 1u);
            last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int i = 0; i < NV; i++) {
        acc[i] = 0.0;
        for (unsigned j = threadIdx.x; j < gridDim.x; j += blockDim.x)
            acc[i] += ((volatile double *)partials)[i * gridDim.x + j];
    }
    block_sum<NV>(acc, sh);
    __shared__ double res[NV];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < NV; i++) res[i] = acc[i];
        *ticket = 0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; i++) tot[i] = res[i];
    return true;
}

// ---------------------------------------------------------------------------
// Mixed path kernels (BSR, B x B blocks, SoA values [BB][nblocks]).
// Preconditioned CG in three launches per iteration: p = z + beta p, then
// q = K32 p with pq = p.q and alpha = gamma / pq, then the vector updates
// with gamma = r.z and beta.  Keeping the direction update out of the SpMV
// lets the SpMV gather a single vector.
// ---------------------------------------------------------------------------
template <int B>
__global__ void k_pupdate32(int64_t n, const float *__restrict__ z, float *__restrict__ p, const Ctl *ctl) {
    if (ctl->stop) return;
    const float beta = ctl->first ? 0.0f : (float)ctl->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * B; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fmaf(beta, p[i], z[i]);
}

// q = K32 p ; pq = p.q ; alpha = gamma / pq
template <int B>
__global__ void __launch_bounds__(kThreads) k_spmv32(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                     const int32_t *__restrict__ cj, const float *__restrict__ A,
                                                     const float *__restrict__ z, float *__restrict__ sv, Ctl *ctl,
                                                     double *partials) {
    if (ctl->stop) return;
    // a half-warp per block row, two blocks per lane in flight; the matrix streams (evict-first).
    // Shuffles are masked to the half-warp, so the two halves of a warp may run different row counts.
    constexpr int G = 16, U = 2;
    const int lane = threadIdx.x % G;
    const unsigned hmask = 0xffffu << (16 * ((threadIdx.x >> 4) & 1));
    const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    // FP32 partial dot per thread: per-row FP64 arithmetic would saturate this GPU's narrow FP64 pipe
    float dot = 0.0f;
    for (int64_t n = grp; n < nn; n += ng) {
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0f;
        const int64_t k0 = rp[n], k1 = rp[n + 1];
        for (int64_t kb = k0 + lane; kb < k1; kb += G * U) {
            int32_t j[U];
            float a[U][B * B];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int64_t k = kb + u * G;
                const bool ok = k < k1;
                j[u] = ok ? __ldcs(cj + k) : 0;
#pragma unroll
                for (int q = 0; q < B * B; q++) a[u][q] = ok ? __ldcs(A + (int64_t)q * nb + k) : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                float xv[B];
#pragma unroll
                for (int d = 0; d < B; d++) xv[d] = __ldg(z + (int64_t)B * j[u] + d);
#pragma unroll
                for (int c = 0; c < B; c++)
#pragma unroll
                    for (int d = B - 1; d >= 0; d--) acc[c] = fmaf(a[u][c * B + d], xv[d], acc[c]);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < B; c++) acc[c] += __shfl_down_sync(hmask, acc[c], o, G);
        if (lane == 0) {
#pragma unroll
            for (int c = 0; c < B; c++) {
                sv[n * B + c] = acc[c];
                dot = fmaf(z[n * B + c], acc[c], dot);
            }
        }
    }
    float v[1] = {dot};
    double tot[1];
    if (grid_sumf<1>(v, partials, &ctl->ticket[0], tot) && threadIdx.x == 0) {
        ctl->pq = tot[0];
        if (!(tot[0] > 0.0)) { ctl->breakdown = 1; ctl->stop = 1; }
        else { ctl->alpha = ctl->rz / tot[0]; ctl->first = 0; }
    }
}

// The PCG direction in a padded layout, one aligned vector per node (float4 in 3-D, float2 in 2-D), so
// that the SpMV gathers it with one load per block.
template <int B>
struct DirVec;
template <>
struct DirVec<3> {
    using T = float4;
    static constexpr int S = 4;
    __device__ static void get(const T &t, float *v) { v[0] = t.x; v[1] = t.y; v[2] = t.z; }
    __device__ static T make(const float *v) { return make_float4(v[0], v[1], v[2], 0.0f); }
};
template <>
struct DirVec<2> {
    using T = float2;
    static constexpr int S = 2;
    __device__ static void get(const T &t, float *v) { v[0] = t.x; v[1] = t.y; }
    __device__ static T make(const float *v) { return make_float2(v[0], v[1]); }
};

// p = z + beta p on the padded direction
template <int B>
__global__ void k_pupdate32v(int64_t nn, const float *__restrict__ z, typename DirVec<B>::T *__restrict__ p,
                             const Ctl *ctl) {
    if (ctl->stop) return;
    const float beta = ctl->first ? 0.0f : (float)ctl->beta;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        float v[B];
        DirVec<B>::get(p[n], v);
#pragma unroll
        for (int c = 0; c < B; c++) v[c] = fmaf(beta, v[c], z[n * B + c]);
        p[n] = DirVec<B>::make(v);
    }
}

// q = K32 p ; pq = p.q ; alpha = gamma / pq, with the padded direction: 8 lanes per block row, each lane 4
// consecutive blocks per step (one 16-byte load per component and one of column indices, from the row's
// start rounded down to 4), one gather of p per block.  The matrix streams (evict-first).
template <int B>
__global__ void __launch_bounds__(kThreads) k_spmv32v(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                      const int32_t *__restrict__ cj, const float *__restrict__ A,
                                                      const typename DirVec<B>::T *__restrict__ p,
                                                      float *__restrict__ q, Ctl *ctl, double *partials) {
    if (ctl->stop) return;
    constexpr int G = 8;
    const int lane = threadIdx.x % G;
    const unsigned gmask = 0xffu << (G * ((threadIdx.x & 31) / G));
    const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    float dot = 0.0f;
    for (int64_t n = grp; n < nn; n += ng) {
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0f;
        const int64_t k0 = rp[n], k1 = rp[n + 1];
        for (int64_t kc = (k0 & ~int64_t(3)) + 4 * lane; kc < k1; kc += 4 * G) {
            const int4 jj = __ldcs(reinterpret_cast<const int4 *>(cj + kc));
            float4 a[B * B];
#pragma unroll
            for (int q4 = 0; q4 < B * B; q4++) a[q4] = __ldcs(reinterpret_cast<const float4 *>(A + (int64_t)q4 * nb + kc));
            const int js[4] = {jj.x, jj.y, jj.z, jj.w};
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int64_t k = kc + u;
                if (k < k0 || k >= k1) continue;
                float xv[B];
                DirVec<B>::get(__ldg(p + js[u]), xv);
#pragma unroll
                for (int c = 0; c < B; c++)
#pragma unroll
                    for (int d = B - 1; d >= 0; d--) {
                        const float4 &t = a[c * B + d];
                        const float av = u == 0 ? t.x : u == 1 ? t.y : u == 2 ? t.z : t.w;
                        acc[c] = fmaf(av, xv[d], acc[c]);
                    }
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < B; c++) acc[c] += __shfl_down_sync(gmask, acc[c], o, G);
        if (lane == 0) {
            float pv[B];
            DirVec<B>::get(p[n], pv);
#pragma unroll
            for (int c = 0; c < B; c++) {
                q[n * B + c] = acc[c];
                dot = fmaf(pv[c], acc[c], dot);
            }
        }
    }
    float v[1] = {dot};
    double tot[1];
    if (grid_sumf<1>(v, partials, &ctl->ticket[0], tot) && threadIdx.x == 0) {
        ctl->pq = tot[0];
        if (!(tot[0] > 0.0)) { ctl->breakdown = 1; ctl->stop = 1; }
        else { ctl->alpha = ctl->rz / tot[0]; ctl->first = 0; }
    }
}

// x += alpha p ; r -= alpha q ; z = Minv r ; gamma = r.z, |r|^2 ; beta = gamma / gamma_old
// (PS: floats per node of p, B or the padded direction's 4)
template <int B, int PS = B>
__global__ void __launch_bounds__(kThreads) k_update32(int64_t nn, const float *__restrict__ Minv,
                                                       const float *__restrict__ p, const float *__restrict__ q,
                                                       float *__restrict__ x, float *__restrict__ r,
                                                       float *__restrict__ z, Ctl *ctl, double *partials,
                                                       double stop_rr, double delta2) {
    if (ctl->stop) return;
    const float alpha = (float)ctl->alpha;
    float rz = 0.0f, rr = 0.0f;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        float rv[B];
#pragma unroll
        for (int c = 0; c < B; c++) {
            const int64_t i = n * B + c;
            x[i] = fmaf(alpha, p[n * PS + c], x[i]);
            rv[c] = fmaf(-alpha, q[i], r[i]);
            r[i] = rv[c];
        }
#pragma unroll
        for (int c = 0; c < B; c++) {
            float zz = 0.0f;
#pragma unroll
            for (int d = 0; d < B; d++) zz = fmaf(Minv[n * B * B + c * B + d], rv[d], zz);
            z[n * B + c] = zz;
            rz = fmaf(rv[c], zz, rz);
            rr = fmaf(rv[c], rv[c], rr);
        }
    }
    float v[2] = {rz, rr};
    double tot[2];
    if (grid_sumf<2>(v, partials, &ctl->ticket[1], tot) && threadIdx.x == 0) {
        ctl->beta = tot[0] / ctl->rz;
        ctl->rz = tot[0];
        ctl->rr = tot[1];
        ctl->iters += 1;
        // reliable update: refresh the FP64 true residual once the recursive one has dropped by delta
        // since the last refresh, or looks converged (or is NaN)
        if (!(tot[1] > stop_rr) || tot[1] <= delta2 * ctl->rr_true) ctl->stop = 1;
    }
}

// Multigrid-preconditioned variant of the update: x += alpha p ; r -= alpha q (z = M r comes after)
template <int B, int PS = B>
__global__ void k_update32a(int64_t nn, const float *__restrict__ p, const float *__restrict__ q,
                            float *__restrict__ x, float *__restrict__ r, const Ctl *ctl) {
    if (ctl->stop) return;
    const float alpha = (float)ctl->alpha;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn * B; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = fmaf(alpha, p[(i / B) * PS + i % B], x[i]);
        r[i] = fmaf(-alpha, q[i], r[i]);
    }
}

// gamma = r.z and |r|^2 once z = M r.  mode 0, an iteration: beta, the counters and the refresh
// criteria of k_update32; mode 1, after a refresh: gamma only.
template <int B>
__global__ void __launch_bounds__(kThreads) k_rz32(int64_t nn, const float *__restrict__ r,
                                                   const float *__restrict__ z, Ctl *ctl, double *partials,
                                                   double stop_rr, double delta2, int mode) {
    if (mode == 0 && ctl->stop) return;
    float rz = 0.0f, rr = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn * B; i += (int64_t)gridDim.x * blockDim.x) {
        rz = fmaf(r[i], z[i], rz);
        rr = fmaf(r[i], r[i], rr);
    }
    float v[2] = {rz, rr};
    double tot[2];
    if (grid_sumf<2>(v, partials, &ctl->ticket[1], tot) && threadIdx.x == 0) {
        if (mode == 0) {
            ctl->beta = tot[0] / ctl->rz;
            ctl->rz = tot[0];
            ctl->rr = tot[1];
            ctl->iters += 1;
            if (!(tot[1] > stop_rr) || tot[1] <= delta2 * ctl->rr_true) ctl->stop = 1;
        } else {
            ctl->rz = tot[0];
        }
    }
}

// FP64 true residual: u64 += x32 (free slots), x32 = 0; r64 = mask(b - K64 u64);
// reac = (K64 u64) at prescribed slots; r32 = r64; z = Minv r32 ; rz, |r64|^2.
// kRowLanes lanes per block row, 32 / kRowLanes rows per warp: the FP64 pipe, not HBM, bounds this
// kernel on GB300, and a row's three sums reduce in log2(kRowLanes) shuffle steps shared by the
// warp's rows.  The row loop advances whole warps so every lane reaches the shuffles.
// R is the type of the Krylov vectors r, z and of the block inverses: float for the mixed path, double for
// the all-FP64 comparator.
constexpr int kRowLanes = 4;
template <int B, typename R = float>
__global__ void __launch_bounds__(kThreads) k_refine(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                     const int32_t *__restrict__ cj, const double *__restrict__ A,
                                                     const uint8_t *__restrict__ fmask, const double *__restrict__ b,
                                                     const double *__restrict__ u64, double *__restrict__ reac,
                                                     R *__restrict__ r32, R *__restrict__ z,
                                                     const R *__restrict__ Minv, Ctl *ctl, double *partials,
                                                     int first, double tol2) {
    constexpr int RPW = 32 / kRowLanes;
    const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double rz = 0.0, rr = 0.0;
    for (int64_t n0 = warp * RPW; n0 < nn; n0 += nw * RPW) {
        const int64_t n = n0 + lane / kRowLanes;
        const bool valid = n < nn;
        double acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0;
        if (valid)
            for (int64_t k = rp[n] + sub; k < rp[n + 1]; k += kRowLanes) {
                const int64_t j = __ldg(cj + k);
                double xv[B];
#pragma unroll
                for (int d = 0; d < B; d++) xv[d] = __ldg(u64 + j * B + d);
#pragma unroll
                for (int c = 0; c < B; c++)
#pragma unroll
                    for (int d = 0; d < B; d++) acc[c] = fma(__ldg(A + (int64_t)(c * B + d) * nb + k), xv[d], acc[c]);
            }
#pragma unroll
        for (int c = 0; c < B; c++)
#pragma unroll
            for (int o = kRowLanes / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (valid && sub == 0) {
            R rv[B];
#pragma unroll
            for (int c = 0; c < B; c++) {
                double res = 0.0;
                if (fmask[n * B + c]) res = b[n * B + c] - acc[c];
                else if (reac) reac[n * B + c] = acc[c];
                rv[c] = (R)res;
                r32[n * B + c] = rv[c];
                rr += res * res;
            }
#pragma unroll
            for (int c = 0; c < B; c++) {
                R s = 0;
#pragma unroll
                for (int d = 0; d < B; d++) s = fma(Minv[n * B * B + c * B + d], rv[d], s);
                z[n * B + c] = s;
                rz += (double)rv[c] * (double)s;
            }
        }
    }
    double v[2] = {rz, rr}, tot[2];
    if (grid_sum<2>(v, partials, &ctl->ticket[2], tot) && threadIdx.x == 0) {
        ctl->rz = tot[0];
        ctl->rr_true = tot[1];
        ctl->rr = tot[1];
        if (first) ctl->bnorm2 = tot[1];
        double ref = first ? tot[1] : ctl->bnorm2;
        ctl->converged = (tot[1] <= tol2 * ref) ? 1 : 0;
        ctl->stop = ctl->converged;
        if (isnan(tot[1])) { ctl->breakdown = 1; ctl->stop = 1; }
    }
}

// u64 += x32 at free slots; x32 = 0
template <int B>
__global__ void k_fold(int64_t n, const uint8_t *fmask, float *x32, double *u64) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * B) return;
    if (fmask[i]) u64[i] += (double)x32[i];
    x32[i] = 0.0f;
}

// ---------------------------------------------------------------------------
// All-FP64 comparator: the mixed path's block-Jacobi PCG with every operand in FP64.  The matrix is
// K64 itself, not a masked copy: p and z are zero at prescribed slots (the block inverses are those of
// the masked diagonal blocks), so K64 p equals the masked product at free rows, and prescribed rows
// are written as zero.  kRowLanes lanes per block row: the FP64 pipe bounds these kernels on GB300,
// and a row's sums reduce in two shuffle steps.
// ---------------------------------------------------------------------------
template <int B>
__global__ void k_pupdate64(int64_t n, const double *__restrict__ z, double *__restrict__ p, const Ctl *ctl) {
    if (ctl->stop) return;
    const double beta = ctl->first ? 0.0 : ctl->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * B; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = fma(beta, p[i], z[i]);
}

// q = mask(K64 p) ; pq = p.q ; alpha = gamma / pq
template <int B>
__global__ void __launch_bounds__(kThreads) k_spmv64(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                     const int32_t *__restrict__ cj, const double *__restrict__ A,
                                                     const uint8_t *__restrict__ fmask, const double *__restrict__ p,
                                                     double *__restrict__ q, Ctl *ctl, double *partials) {
    if (ctl->stop) return;
    constexpr int RPW = 32 / kRowLanes;
    const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double dot = 0.0;
    for (int64_t n0 = warp * RPW; n0 < nn; n0 += nw * RPW) {
        const int64_t n = n0 + lane / kRowLanes;
        const bool valid = n < nn;
        double acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0;
        if (valid)
            for (int64_t k = rp[n] + sub; k < rp[n + 1]; k += kRowLanes) {
                // the read-only path for the matrix too: measured faster than evict-first loads here, where
                // the FP64 pipe and not HBM is the bound
                const int64_t j = __ldg(cj + k);
                double xv[B];
#pragma unroll
                for (int d = 0; d < B; d++) xv[d] = __ldg(p + j * B + d);
#pragma unroll
                for (int c = 0; c < B; c++)
#pragma unroll
                    for (int d = 0; d < B; d++) acc[c] = fma(__ldg(A + (int64_t)(c * B + d) * nb + k), xv[d], acc[c]);
            }
#pragma unroll
        for (int c = 0; c < B; c++)
#pragma unroll
            for (int o = kRowLanes / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (valid && sub == 0)
#pragma unroll
            for (int c = 0; c < B; c++) {
                const double v = fmask[n * B + c] ? acc[c] : 0.0;
                q[n * B + c] = v;
                dot = fma(p[n * B + c], v, dot);
            }
    }
    double v[1] = {dot}, tot[1];
    if (grid_sum<1>(v, partials, &ctl->ticket[0], tot) && threadIdx.x == 0) {
        ctl->pq = tot[0];
        if (!(tot[0] > 0.0)) { ctl->breakdown = 1; ctl->stop = 1; }
        else { ctl->alpha = ctl->rz / tot[0]; ctl->first = 0; }
    }
}

// u += alpha p ; r -= alpha q ; z = Minv r ; gamma = r.z, |r|^2 ; beta.  Stops for a true-residual check
// once the recursive residual looks converged (or is NaN).
template <int B>
__global__ void __launch_bounds__(kThreads) k_update64(int64_t nn, const double *__restrict__ Minv,
                                                       const double *__restrict__ p, const double *__restrict__ q,
                                                       double *__restrict__ u, double *__restrict__ r,
                                                       double *__restrict__ z, Ctl *ctl, double *partials,
                                                       double stop_rr) {
    if (ctl->stop) return;
    const double alpha = ctl->alpha;
    double rz = 0.0, rr = 0.0;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += (int64_t)gridDim.x * blockDim.x) {
        double rv[B];
#pragma unroll
        for (int c = 0; c < B; c++) {
            const int64_t i = n * B + c;
            u[i] = fma(alpha, p[i], u[i]);
            rv[c] = fma(-alpha, q[i], r[i]);
            r[i] = rv[c];
        }
#pragma unroll
        for (int c = 0; c < B; c++) {
            double zz = 0.0;
#pragma unroll
            for (int d = 0; d < B; d++) zz = fma(Minv[n * B * B + c * B + d], rv[d], zz);
            z[n * B + c] = zz;
            rz = fma(rv[c], zz, rz);
            rr = fma(rv[c], rv[c], rr);
        }
    }
    double v[2] = {rz, rr}, tot[2];
    if (grid_sum<2>(v, partials, &ctl->ticket[1], tot) && threadIdx.x == 0) {
        ctl->beta = tot[0] / ctl->rz;
        ctl->rz = tot[0];
        ctl->rr = tot[1];
        ctl->iters += 1;
        if (!(tot[1] > stop_rr)) ctl->stop = 1;
    }
}

// Multigrid-preconditioned FP64 update: u += alpha p ; r -= alpha q (z = M r comes after)
template <int B>
__global__ void k_update64a(int64_t nn, const double *__restrict__ p, const double *__restrict__ q,
                            double *__restrict__ u, double *__restrict__ r, const Ctl *ctl) {
    if (ctl->stop) return;
    const double alpha = ctl->alpha;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn * B; i += (int64_t)gridDim.x * blockDim.x) {
        u[i] = fma(alpha, p[i], u[i]);
        r[i] = fma(-alpha, q[i], r[i]);
    }
}

// gamma = r.z and |r|^2 once z = M r, in FP64.  mode 0, an iteration: beta, the counter and the stop
// for a true-residual check; mode 1, after a true-residual check: gamma only.
template <int B>
__global__ void __launch_bounds__(kThreads) k_rz64(int64_t nn, const double *__restrict__ r,
                                                   const double *__restrict__ z, Ctl *ctl, double *partials,
                                                   double stop_rr, int mode) {
    if (mode == 0 && ctl->stop) return;
    double rz = 0.0, rr = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nn * B; i += (int64_t)gridDim.x * blockDim.x) {
        rz = fma(r[i], z[i], rz);
        rr = fma(r[i], r[i], rr);
    }
    double v[2] = {rz, rr}, tot[2];
    if (grid_sum<2>(v, partials, &ctl->ticket[1], tot) && threadIdx.x == 0) {
        if (mode == 0) {
            ctl->beta = tot[0] / ctl->rz;
            ctl->rz = tot[0];
            ctl->rr = tot[1];
            ctl->iters += 1;
            if (!(tot[1] > stop_rr)) ctl->stop = 1;
        } else {
            ctl->rz = tot[0];
        }
    }
}

// r = b - K12 u2 on the free eq rows, from the BSR FP64 matrix (u = prescribed part only)
__global__ void k_scatter_eq(int64_t nnodes, int B, const int64_t *eq_id, int64_t nu, double *nm, double *eq,
                             int to_eq) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * B) return;
    int64_t n = t / B;
    int c = (int)(t % B);
    int64_t e = eq_id[n * 3 + c];
    if (e < 0 || e >= nu) return;
    if (to_eq) eq[e] = nm[t];
    else nm[t] = eq[e];
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace


struct AmrSolveWork {
    int64_t n = 0;               // nnodes * B
    float *x32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32[2] = {nullptr, nullptr}, *q32 = nullptr,
          *s32 = nullptr;
    double *partials = nullptr;
    Ctl *ctl = nullptr;
    Ctl *h_ctl = nullptr;        // pinned
    int grid = 0, grid_spmv = 0;
    // all-FP64 comparators: Krylov vectors (allocated on their first use)
    double *r64 = nullptr, *z64 = nullptr, *p64 = nullptr, *q64 = nullptr;
};

static AmrSolveWork *work(amr_model *m) {
    if (!m->sw) m->sw = new AmrSolveWork();
    AmrSolveWork *w = m->sw;
    int64_t n = m->nnodes * m->B;
    if (w->n != n) {
        w->n = n;
        amr_free(w->x32); amr_free(w->r32); amr_free(w->z32); amr_free(w->p32[0]); amr_free(w->p32[1]);
        amr_free(w->q32);
        amr_free(w->s32);
        amr_free(w->r64); amr_free(w->z64); amr_free(w->p64); amr_free(w->q64);
        amr_alloc(&w->s32, n);
        amr_alloc(&w->x32, n); amr_alloc(&w->r32, n); amr_alloc(&w->z32, n);
        amr_alloc(&w->p32[0], (size_t)m->nnodes * (m->B == 3 ? 4 : 2));  // the padded direction
        amr_alloc(&w->p32[1], n); amr_alloc(&w->q32, n);
        int dev = 0, sms = 148;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        w->grid = sms * 8;
        w->grid_spmv = sms * 8;
        amr_free(w->partials);
        amr_alloc(&w->partials, (size_t)std::max(4 * w->grid, w->grid_spmv) + 8);
        if (!w->ctl) {
            amr_alloc(&w->ctl, 1);
            AMR_CUDA(cudaMemsetAsync(w->ctl, 0, sizeof(Ctl), m->stream));
            w->h_ctl = (Ctl *)amr_pinned_alloc(sizeof(Ctl));
        }
    }
    return w;
}

void amr_solver_free(amr_model *m) {
    AmrSolveWork *w = m->sw;
    if (!w) return;
    amr_free(w->x32); amr_free(w->r32); amr_free(w->z32); amr_free(w->p32[0]); amr_free(w->p32[1]); amr_free(w->q32);
    amr_free(w->s32);
    amr_free(w->partials); amr_free(w->ctl);
    amr_pinned_free(w->h_ctl);
    amr_free(w->r64); amr_free(w->z64); amr_free(w->p64); amr_free(w->q64);
    delete w;
    m->sw = nullptr;
}

// the grid of a grid-stride kernel of kThreads threads: the CTAs it keeps resident (at most 8 per SM).  The FP64
// SpMV (FP64-pipe bound, 3 CTAs per SM) measured faster in one resident wave than in 8 CTAs per SM; the
// HBM-bound FP32 and FP16 kernels measured slower, and keep 8 CTAs per SM.
template <class K>
static unsigned grid_of(K kernel) {
    return amr_resident_grid((const void *)kernel, kThreads, 8);
}

template <int B>
static void launch_spmv32(amr_model *m, AmrSolveWork *w, const float *p, float *q) {
    using PT = typename DirVec<B>::T;
    k_spmv32v<B><<<(unsigned)w->grid_spmv, kThreads, 0, m->stream>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol,
                                                                      m->K32, reinterpret_cast<const PT *>(p), q,
                                                                      w->ctl, w->partials);
    AMR_COUNT(1);
}
template <int B>
static void launch_pupdate32(amr_model *m, AmrSolveWork *w) {
    using PT = typename DirVec<B>::T;
    k_pupdate32v<B><<<(unsigned)w->grid, kThreads, 0, m->stream>>>(m->nnodes, w->z32, reinterpret_cast<PT *>(w->p32[0]),
                                                                    w->ctl);
    AMR_COUNT(1);
}

template <int B>
static AmrSolveResult solve_mixed(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o) {
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    int64_t nn = m->nnodes;
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    double tol2 = o.rtol * o.rtol;
    AMR_CUDA(cudaMemsetAsync(w->x32, 0, w->n * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w->p32[0], 0, (size_t)nn * DirVec<B>::S * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w->q32, 0, w->n * sizeof(float), s));
    {
        Ctl c0{};
        c0.first = 1;
        AMR_CUDA(cudaMemcpyAsync(w->ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    }
    // free slots of x start at zero (the reduced system's initial guess)
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    unsigned g = (unsigned)w->grid;
    k_refine<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, x, reac, w->r32,
                                       w->z32, m->Minv32, w->ctl, w->partials, 1, tol2);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    int every = o.refine_every > 0 ? o.refine_every : 32;  // iterations between host checks
    double stop_rr_rel = 0.25 * 0.25 * tol2;  // refresh early once the FP32 residual looks converged
    const double delta2 = 1e-2;                // refresh after a 10x drop of the residual
    int since = 0;
    for (;;) {
        AMR_CUDA(cudaMemcpyAsync(w->h_ctl, w->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        Ctl c = *w->h_ctl;
        res.iterations = c.iters;
        if (c.bnorm2 == 0.0 || c.converged) break;
        if (c.breakdown) { res.status = AMR_ENOCONV; break; }
        if (c.iters >= o.max_iters) { res.status = AMR_ENOCONV; break; }
        if (c.stop || since >= 16 * every) {
            // fold the FP32 correction into the FP64 solution and refresh the true residual
            k_fold<B><<<nblk(w->n, 256), 256, 0, s>>>(nn, m->free_mask, w->x32, x);
            AMR_COUNT(1);
            AMR_CUDA(cudaMemsetAsync(&w->ctl->stop, 0, sizeof(int32_t), s));
            k_refine<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, x,
                                               reac, w->r32, w->z32, m->Minv32, w->ctl, w->partials, 0, tol2);
            AMR_COUNT(1);
            res.refinements++;
            since = 0;
            continue;
        }
        double stop_rr = stop_rr_rel * c.bnorm2;
        int nit = std::min(every, o.max_iters - c.iters);
        for (int it = 0; it < nit; it++) {
            launch_pupdate32<B>(m, w);
            launch_spmv32<B>(m, w, w->p32[0], w->q32);
            k_update32<B, DirVec<B>::S><<<g, kThreads, 0, s>>>(nn, m->Minv32, w->p32[0], w->q32, w->x32, w->r32,
                                                                w->z32, w->ctl, w->partials, stop_rr, delta2);
            AMR_COUNT(1);
        }
        AMR_CUDA(cudaGetLastError());
        since += nit;
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    res.seconds = ms * 1e-3;
    Ctl c = *w->h_ctl;
    res.rel_residual = c.bnorm2 > 0 ? std::sqrt(c.rr_true / c.bnorm2) : 0.0;
    // the iteration count is the number of launched iterations that did work; an early
    // stop inside a chunk makes the remainder no-ops
    return res;
}

// The V-cycle's kernels read the solve's stop flag while this scope lives: the iterations a replayed chunk
// holds after the flag is raised (a refresh or convergence is due) then cost launches only.
struct HaltScope {
    amr_model *m;
    HaltScope(amr_model *m_, const int32_t *flag) : m(m_) { amr_amg_set_halt(m, flag); }
    ~HaltScope() { amr_amg_set_halt(m, nullptr); }
};

// solve_system! with the multigrid preconditioner: the mixed solver's PCG (FP32 Krylov vectors,
// FP64 true-residual refreshes decide convergence) with z = V-cycle(r) in place of block-Jacobi.
template <int B>
static AmrSolveResult solve_amg(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o) {
    amr_amg_prepare(m);
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    int64_t nn = m->nnodes;
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    double tol2 = o.rtol * o.rtol;
    AMR_CUDA(cudaMemsetAsync(w->x32, 0, w->n * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w->p32[0], 0, (size_t)nn * DirVec<B>::S * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w->q32, 0, w->n * sizeof(float), s));
    {
        Ctl c0{};
        c0.first = 1;
        AMR_CUDA(cudaMemcpyAsync(w->ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    }
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    const unsigned g = (unsigned)w->grid;
    auto refresh = [&](int first) {
        k_refine<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, x, reac,
                                           w->r32, w->z32, m->Minv32, w->ctl, w->partials, first, tol2);
        amr_amg_vcycle(m, w->r32, w->z32);
        k_rz32<B><<<g, kThreads, 0, s>>>(nn, w->r32, w->z32, w->ctl, w->partials, 0.0, 0.0, 1);
        AMR_COUNT(2);
        AMR_CUDA(cudaGetLastError());
    };
    refresh(1);
    HaltScope halt_scope(m, &w->ctl->stop);
    // one iteration as a CUDA graph, captured once its arguments are fixed (after the first
    // refresh: stop_rr depends on |b|), then replayed; its kernels are counted per replay
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long per_iter = 0;
    struct GraphFree {
        cudaGraph_t &g;
        cudaGraphExec_t &x;
        ~GraphFree() {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
        }
    } graph_free{graph, gexec};
    const int every = 4;  // iterations between host checks (each iteration is a whole V-cycle)
    // refresh after a 100x drop of the residual norm: the few, fast-converging iterations between
    // refreshes keep the FP32 recursion accurate, and convergence is judged on the FP64 residual
    const double stop_rr_rel = 0.25 * 0.25 * tol2, delta2 = 1e-4;
    int since = 0;
    for (;;) {
        AMR_CUDA(cudaMemcpyAsync(w->h_ctl, w->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        Ctl c = *w->h_ctl;
        res.iterations = c.iters;
        if (c.bnorm2 == 0.0 || c.converged) break;
        if (c.breakdown) { res.status = AMR_ENOCONV; break; }
        if (c.iters >= o.max_iters) { res.status = AMR_ENOCONV; break; }
        if (c.stop || since >= 64) {
            k_fold<B><<<nblk(w->n, 256), 256, 0, s>>>(nn, m->free_mask, w->x32, x);
            AMR_COUNT(1);
            AMR_CUDA(cudaMemsetAsync(&w->ctl->stop, 0, sizeof(int32_t), s));
            refresh(0);
            res.refinements++;
            since = 0;
            continue;
        }
        const double stop_rr = stop_rr_rel * c.bnorm2;
        const int nit = std::min(every, o.max_iters - c.iters);
        if (!gexec) {
            const long long before = amr_g_launches.load();
            AMR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            launch_pupdate32<B>(m, w);
            launch_spmv32<B>(m, w, w->p32[0], w->q32);
            k_update32a<B, DirVec<B>::S><<<g, kThreads, 0, s>>>(nn, w->p32[0], w->q32, w->x32, w->r32, w->ctl);
            amr_amg_vcycle(m, w->r32, w->z32);
            k_rz32<B><<<g, kThreads, 0, s>>>(nn, w->r32, w->z32, w->ctl, w->partials, stop_rr, delta2, 0);
            AMR_COUNT(2);
            const cudaError_t ce = cudaStreamEndCapture(s, &graph);
            per_iter = amr_g_launches.load() - before;
            AMR_COUNT(-per_iter);
            AMR_CUDA(ce);
            AMR_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
        }
        for (int it = 0; it < nit; it++) {
            AMR_CUDA(cudaGraphLaunch(gexec, s));
            AMR_COUNT(per_iter);
        }
        since += nit;
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    res.seconds = ms * 1e-3;
    Ctl c = *w->h_ctl;
    res.rel_residual = c.bnorm2 > 0 ? std::sqrt(c.rr_true / c.bnorm2) : 0.0;
    return res;
}

// The all-FP64 comparator of solve_mixed: the same block-Jacobi PCG, with the FP64 matrix, FP64
// block inverses and FP64 vectors, so that the two differ in precision only.  The solution is updated in
// place (x at free slots); convergence is decided, as in the mixed path, on the true residual
// ||mask(b - K64 x)|| / ||mask(b - K64 x0)||, recomputed whenever the recursive residual looks converged.
template <int B>
static AmrSolveResult solve_fp64(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o) {
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    const int64_t nn = m->nnodes;
    if (!w->r64) {
        amr_alloc(&w->r64, w->n); amr_alloc(&w->z64, w->n); amr_alloc(&w->p64, w->n); amr_alloc(&w->q64, w->n);
    }
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    const double tol2 = o.rtol * o.rtol;
    AMR_CUDA(cudaMemsetAsync(w->p64, 0, w->n * sizeof(double), s));
    {
        Ctl c0{};
        c0.first = 1;
        AMR_CUDA(cudaMemcpyAsync(w->ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    }
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    const unsigned g = (unsigned)w->grid;
    k_refine<B, double><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, x,
                                               reac, w->r64, w->z64, m->Minv64, w->ctl, w->partials, 1, tol2);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    const int every = o.refine_every > 0 ? o.refine_every : 32;  // iterations between host checks
    for (;;) {
        AMR_CUDA(cudaMemcpyAsync(w->h_ctl, w->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        const Ctl c = *w->h_ctl;
        res.iterations = c.iters;
        if (c.bnorm2 == 0.0 || c.converged) break;
        if (c.breakdown) { res.status = AMR_ENOCONV; break; }
        if (c.iters >= o.max_iters) { res.status = AMR_ENOCONV; break; }
        if (c.stop) {  // the recursive residual looks converged: check the true one
            AMR_CUDA(cudaMemsetAsync(&w->ctl->stop, 0, sizeof(int32_t), s));
            k_refine<B, double><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b,
                                                       x, reac, w->r64, w->z64, m->Minv64, w->ctl, w->partials, 0,
                                                       tol2);
            AMR_COUNT(1);
            res.refinements++;
            continue;
        }
        const double stop_rr = 0.25 * 0.25 * tol2 * c.bnorm2;
        const int nit = std::min(every, o.max_iters - c.iters);
        for (int it = 0; it < nit; it++) {
            k_pupdate64<B><<<g, kThreads, 0, s>>>(nn, w->z64, w->p64, w->ctl);
            k_spmv64<B><<<grid_of(k_spmv64<B>), kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, w->p64,
                                               w->q64, w->ctl, w->partials);
            k_update64<B><<<g, kThreads, 0, s>>>(nn, m->Minv64, w->p64, w->q64, x, w->r64, w->z64, w->ctl,
                                                 w->partials, stop_rr);
            AMR_COUNT(3);
        }
        AMR_CUDA(cudaGetLastError());
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    res.seconds = ms * 1e-3;
    const Ctl c = *w->h_ctl;
    res.rel_residual = c.bnorm2 > 0 ? std::sqrt(c.rr_true / c.bnorm2) : 0.0;
    return res;
}

// The all-FP64 comparator of solve_amg: the same PCG with the same multigrid hierarchy (aggregates,
// prolongators, Chebyshev smoothing, dense coarsest level) built and applied in FP64 on K64.  The
// iteration is one CUDA graph, as in solve_amg; convergence is decided on the true residual.
template <int B>
static AmrSolveResult solve_amg_fp64(amr_model *m, double *x, const double *b, double *reac,
                                     const amr_solve_opts &o) {
    amr_amg_prepare64(m);
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    const int64_t nn = m->nnodes;
    if (!w->r64) {
        amr_alloc(&w->r64, w->n); amr_alloc(&w->z64, w->n); amr_alloc(&w->p64, w->n); amr_alloc(&w->q64, w->n);
    }
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    const double tol2 = o.rtol * o.rtol;
    AMR_CUDA(cudaMemsetAsync(w->p64, 0, w->n * sizeof(double), s));
    {
        Ctl c0{};
        c0.first = 1;
        AMR_CUDA(cudaMemcpyAsync(w->ctl, &c0, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    }
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    const unsigned g = (unsigned)w->grid;
    auto refresh = [&](int first) {
        k_refine<B, double><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, x,
                                                   reac, w->r64, w->z64, m->Minv64, w->ctl, w->partials, first, tol2);
        amr_amg_vcycle64(m, w->r64, w->z64);
        k_rz64<B><<<g, kThreads, 0, s>>>(nn, w->r64, w->z64, w->ctl, w->partials, 0.0, 1);
        AMR_COUNT(2);
        AMR_CUDA(cudaGetLastError());
    };
    refresh(1);
    HaltScope halt_scope(m, &w->ctl->stop);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    long long per_iter = 0;
    struct GraphFree {
        cudaGraph_t &g;
        cudaGraphExec_t &x;
        ~GraphFree() {
            if (x) cudaGraphExecDestroy(x);
            if (g) cudaGraphDestroy(g);
        }
    } graph_free{graph, gexec};
    const int every = 4;  // iterations between host checks (each iteration is a whole V-cycle)
    for (;;) {
        AMR_CUDA(cudaMemcpyAsync(w->h_ctl, w->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        const Ctl c = *w->h_ctl;
        res.iterations = c.iters;
        if (c.bnorm2 == 0.0 || c.converged) break;
        if (c.breakdown) { res.status = AMR_ENOCONV; break; }
        if (c.iters >= o.max_iters) { res.status = AMR_ENOCONV; break; }
        if (c.stop) {
            AMR_CUDA(cudaMemsetAsync(&w->ctl->stop, 0, sizeof(int32_t), s));
            refresh(0);
            res.refinements++;
            continue;
        }
        const int nit = std::min(every, o.max_iters - c.iters);
        if (!gexec) {
            const double stop_rr = 0.25 * 0.25 * tol2 * c.bnorm2;
            const long long before = amr_g_launches.load();
            AMR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            k_pupdate64<B><<<g, kThreads, 0, s>>>(nn, w->z64, w->p64, w->ctl);
            k_spmv64<B><<<grid_of(k_spmv64<B>), kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, w->p64,
                                               w->q64, w->ctl, w->partials);
            k_update64a<B><<<g, kThreads, 0, s>>>(nn, w->p64, w->q64, x, w->r64, w->ctl);
            amr_amg_vcycle64(m, w->r64, w->z64);
            k_rz64<B><<<g, kThreads, 0, s>>>(nn, w->r64, w->z64, w->ctl, w->partials, stop_rr, 0);
            AMR_COUNT(4);
            const cudaError_t ce = cudaStreamEndCapture(s, &graph);
            per_iter = amr_g_launches.load() - before;
            AMR_COUNT(-per_iter);
            AMR_CUDA(ce);
            AMR_CUDA(cudaGraphInstantiate(&gexec, graph, 0));
        }
        for (int it = 0; it < nit; it++) {
            AMR_CUDA(cudaGraphLaunch(gexec, s));
            AMR_COUNT(per_iter);
        }
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    res.seconds = ms * 1e-3;
    const Ctl c = *w->h_ctl;
    res.rel_residual = c.bnorm2 > 0 ? std::sqrt(c.rr_true / c.bnorm2) : 0.0;
    return res;
}

// ---- small vector helpers ----
namespace {
__global__ void k_absmax(int64_t n, const double *v, const uint8_t *fm, double *partials, unsigned int *ticket,
                         double *out) {
    double mx = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (fm && !fm[i]) continue;
        double a = fabs(v[i]);
        if (isnan(a)) a = INFINITY;  // NaN propagates as +inf; caller checks isnan separately
        mx = fmax(mx, a);
    }
    // max-reduction: reuse the sum tree on a max via shared memory
    __shared__ double sh[kThreads];
    __shared__ bool last;
    sh[threadIdx.x] = mx;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = sh[0];
        __threadfence();
        last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0;
    for (unsigned j = threadIdx.x; j < gridDim.x; j += blockDim.x) a = fmax(a, ((volatile double *)partials)[j]);
    sh[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) { *out = sh[0]; *ticket = 0; }
}
}  // namespace

double amr_norm_inf(amr_model *m, const double *v, const uint8_t *mask) {
    AmrSolveWork *w = work(m);
    double *out = (double *)(w->partials + 3 * (size_t)w->grid);
    k_absmax<<<w->grid, kThreads, 0, m->stream>>>(w->n, v, mask, w->partials, &w->ctl->ticket[3], out);
    AMR_COUNT(1);
    double h = 0.0;
    AMR_CUDA(cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    AMR_CUDA(cudaStreamSynchronize(m->stream));
    return h;
}

void amr_eq_to_nm(amr_model *m, const double *d_eq, double *d_nm) {
    int64_t nt = m->nnodes * m->B;
    AMR_CUDA(cudaMemsetAsync(d_nm, 0, nt * sizeof(double), m->stream));
    k_scatter_eq<<<nblk(nt, 256), 256, 0, m->stream>>>(m->nnodes, m->B, m->eq_id, m->ndofs, d_nm, (double *)d_eq, 0);
    AMR_COUNT(1);
}

void amr_nm_to_eq(amr_model *m, const double *d_nm, double *d_eq) {
    int64_t nt = m->nnodes * m->B;
    k_scatter_eq<<<nblk(nt, 256), 256, 0, m->stream>>>(m->nnodes, m->B, m->eq_id, m->ndofs, (double *)d_nm, d_eq, 1);
    AMR_COUNT(1);
}

AmrSolveResult amr_solve_device(amr_model *m, double *x, const double *b, double *reac, const amr_solve_opts &o) {
    if (m->batch && (o.method == AMR_SOLVER_MIXED || o.method == AMR_SOLVER_AMG))
        return amr_batch_solve(m, x, b, reac, o);  // per part: one CTA each, or the joined multigrid
    if (o.method == AMR_SOLVER_AMG) return m->B == 3 ? solve_amg<3>(m, x, b, reac, o) : solve_amg<2>(m, x, b, reac, o);
    if (o.method == AMR_SOLVER_FP64) return m->B == 3 ? solve_fp64<3>(m, x, b, reac, o) : solve_fp64<2>(m, x, b, reac, o);
    if (o.method == AMR_SOLVER_AMG_FP64)
        return m->B == 3 ? solve_amg_fp64<3>(m, x, b, reac, o) : solve_amg_fp64<2>(m, x, b, reac, o);
    return m->B == 3 ? solve_mixed<3>(m, x, b, reac, o) : solve_mixed<2>(m, x, b, reac, o);
}

// ---- kernel timing for the roofline report (CUDA events on the handle's stream) ----
template <int B>
static double time_spmv32(amr_model *m, int reps) {
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    Ctl c{};
    c.rz = 1.0;
    c.first = 1;
    AMR_CUDA(cudaMemcpyAsync(w->ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int i = 0; i < reps; i++) {
        launch_spmv32<B>(m, w, w->p32[0], w->s32);
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    return ms * 1e-3 / reps;
}

template <int B>
static double time_spmv64(amr_model *m, int reps) {
    AmrSolveWork *w = work(m);
    if (!w->p64) throw AmrError(AMR_EINVAL, "run an all-FP64 solve on the current K first");
    cudaStream_t s = m->stream;
    Ctl c{};
    c.rz = 1.0;
    c.first = 1;
    AMR_CUDA(cudaMemcpyAsync(w->ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    const unsigned g = (unsigned)w->grid;
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int i = 0; i < reps; i++) {
        k_spmv64<B><<<grid_of(k_spmv64<B>), kThreads, 0, s>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, w->z64,
                                           w->q64, w->ctl, w->partials);
        AMR_COUNT(1);
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    return ms * 1e-3 / reps;
}

template <int B>
static double time_residual64(amr_model *m, int reps) {
    AmrSolveWork *w = work(m);
    cudaStream_t s = m->stream;
    unsigned g = (unsigned)w->grid;
    double *u = m->vtmp[5], *b = m->vtmp[6];
    AMR_CUDA(cudaMemsetAsync(u, 0, w->n * sizeof(double), s));
    AMR_CUDA(cudaMemsetAsync(b, 0, w->n * sizeof(double), s));
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int i = 0; i < reps; i++) {
        k_refine<B><<<g, kThreads, 0, s>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b, u,
                                           nullptr, w->r32, w->z32, m->Minv32, w->ctl, w->partials, 1, 1e-16);
        AMR_COUNT(1);
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    return ms * 1e-3 / reps;
}

double amr_time_solver_kernel(amr_model *m, int which, int reps) {
    if (which == AMR_KERNEL_SPMV32) return m->B == 3 ? time_spmv32<3>(m, reps) : time_spmv32<2>(m, reps);
    if (which == AMR_KERNEL_SPMV64) return m->B == 3 ? time_spmv64<3>(m, reps) : time_spmv64<2>(m, reps);
    return m->B == 3 ? time_residual64<3>(m, reps) : time_residual64<2>(m, reps);
}

// ===========================================================================
// solve_system! with caller-owned device buffers and no device allocation.
//
// For callers that cannot allocate GPU memory while they solve: an embedding
// that hands the library a fixed memory budget up front, a real-time loop
// that must not enter the CUDA allocator, or code whose memory pool forbids
// growth.  All scratch of the mixed-precision solve -- the node-major FP64
// work vectors, the FP32 Krylov vectors, the per-CTA reduction partials and
// the control block -- lives in one file-scope device array of fixed size.
// The model itself (pattern, K, masks) is created and assembled beforehand by
// the ordinary entry points, which do allocate.
// ===========================================================================
namespace {

// node-major slots (nnodes x ndim) the scratch array serves
constexpr int64_t kNoAllocMaxSlots = int64_t(1) << 18;  // 262 144 (e.g. 87 381 nodes in 3-D)
constexpr int64_t kNoAllocPartials = 8192;              // doubles of CTA partials
constexpr size_t kNoAllocAlign = 256;
constexpr size_t align_up(size_t v) { return (v + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
constexpr size_t kNoAllocBytes = 3 * align_up(sizeof(double) * kNoAllocMaxSlots) +  // x, b, reactions (FP64)
                                 5 * align_up(sizeof(float) * kNoAllocMaxSlots) +   // x32 r32 z32 p32 q32
                                 align_up(sizeof(double) * kNoAllocPartials) + align_up(sizeof(Ctl));

// The scratch.  Every GPU that loads the library holds these ~11.5 MB until the process exits.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
void *g_noalloc_addr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mutex;

// Device address of g_noalloc_scratch for the current device, looked up once per device.
// (In host code the symbol name is only a host-side stand-in, not a device address.)  A thread
// that finds the lookup under way sleeps on the mutex while the first one may be loading the module.
void *noalloc_base() {
    int dev = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw AmrError(AMR_EINVAL, "device ordinal out of range");
    void *p = nullptr;
    cudaError_t e = cudaSuccess;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        p = g_noalloc_addr[dev];
        if (!p) {
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e == cudaSuccess) g_noalloc_addr[dev] = p;
        }
    }
    if (e != cudaSuccess)
        throw AmrError(AMR_ECUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    return p;
}

struct NoAllocView {
    double *x, *b, *reac, *partials;
    float *x32, *r32, *z32, *p32, *q32;
    Ctl *ctl;
};

NoAllocView noalloc_view(void *base) {
    unsigned char *c = (unsigned char *)base;
    NoAllocView v;
    size_t d = align_up(sizeof(double) * kNoAllocMaxSlots), f = align_up(sizeof(float) * kNoAllocMaxSlots);
    v.x = (double *)c; c += d;
    v.b = (double *)c; c += d;
    v.reac = (double *)c; c += d;
    v.x32 = (float *)c; c += f;
    v.r32 = (float *)c; c += f;
    v.z32 = (float *)c; c += f;
    v.p32 = (float *)c; c += f;
    v.q32 = (float *)c; c += f;
    v.partials = (double *)c; c += align_up(sizeof(double) * kNoAllocPartials);
    v.ctl = (Ctl *)c;
    return v;
}

// node-major <- eq_id entries in [nu, ndofs) (prescribed values), 0 elsewhere
__global__ void k_gather_prescribed(int64_t nnodes, int B, const int64_t *eq_id, int64_t nu, int64_t ndofs,
                                    const double *eq, double *nm) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * B) return;
    int64_t e = eq_id[(t / B) * 3 + t % B];
    nm[t] = (e >= nu && e < ndofs) ? eq[e] : 0.0;
}

// eq_id entries in [nu, ndofs) <- node-major values (the reactions of solve_system!)
__global__ void k_scatter_prescribed(int64_t nnodes, int B, const int64_t *eq_id, int64_t nu, int64_t ndofs,
                                     const double *nm, double *eq) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * B) return;
    int64_t e = eq_id[(t / B) * 3 + t % B];
    if (e >= nu && e < ndofs) eq[e] = nm[t];
}

template <int B>
AmrSolveResult solve_mixed_noalloc(amr_model *m, const NoAllocView &w, int grid, const amr_solve_opts &o) {
    cudaStream_t s = m->stream;
    const int64_t nn = m->nnodes, n = nn * B;
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    const double tol2 = o.rtol * o.rtol;
    // everything that must start at zero is cleared here: the array keeps the previous call's contents
    AMR_CUDA(cudaMemsetAsync(w.x32, 0, n * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w.p32, 0, n * sizeof(float), s));
    AMR_CUDA(cudaMemsetAsync(w.q32, 0, n * sizeof(float), s));
    Ctl hc{};
    hc.first = 1;
    AMR_CUDA(cudaMemcpyAsync(w.ctl, &hc, sizeof(Ctl), cudaMemcpyHostToDevice, s));
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    const unsigned g = (unsigned)grid;
    k_refine<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, w.b, w.x, w.reac,
                                       w.r32, w.z32, m->Minv32, w.ctl, w.partials, 1, tol2);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    const int every = o.refine_every > 0 ? o.refine_every : 32;
    const double stop_rr_rel = 0.25 * 0.25 * tol2;
    const double delta2 = 1e-2;
    int since = 0;
    for (;;) {
        AMR_CUDA(cudaMemcpyAsync(&hc, w.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s));  // pageable: no pinned buffer
        AMR_CUDA(cudaStreamSynchronize(s));
        res.iterations = hc.iters;
        if (hc.bnorm2 == 0.0 || hc.converged) break;
        if (hc.breakdown) { res.status = AMR_ENOCONV; break; }
        if (hc.iters >= o.max_iters) { res.status = AMR_ENOCONV; break; }
        if (hc.stop || since >= 16 * every) {
            k_fold<B><<<nblk(n, 256), 256, 0, s>>>(nn, m->free_mask, w.x32, w.x);
            AMR_COUNT(1);
            AMR_CUDA(cudaMemsetAsync(&w.ctl->stop, 0, sizeof(int32_t), s));
            k_refine<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, w.b, w.x,
                                               w.reac, w.r32, w.z32, m->Minv32, w.ctl, w.partials, 0, tol2);
            AMR_COUNT(1);
            res.refinements++;
            since = 0;
            continue;
        }
        const double stop_rr = stop_rr_rel * hc.bnorm2;
        const int nit = std::min(every, o.max_iters - hc.iters);
        for (int it = 0; it < nit; it++) {
            k_pupdate32<B><<<g, kThreads, 0, s>>>(nn, w.z32, w.p32, w.ctl);
            k_spmv32<B><<<g, kThreads, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K32, w.p32, w.q32, w.ctl,
                                               w.partials);
            k_update32<B><<<g, kThreads, 0, s>>>(nn, m->Minv32, w.p32, w.q32, w.x32, w.r32, w.z32, w.ctl, w.partials,
                                                 stop_rr, delta2);
            AMR_COUNT(3);
        }
        AMR_CUDA(cudaGetLastError());
        since += nit;
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, m->ev0, m->ev1);
    res.seconds = ms * 1e-3;
    res.rel_residual = hc.bnorm2 > 0 ? std::sqrt(hc.rr_true / hc.bnorm2) : 0.0;
    return res;
}

}  // namespace

extern "C" int amr_solve_noalloc(amr_model *m, double *d_U, double *d_F, const amr_solve_opts *opts,
                                 amr_solve_stats *stats) {
    if (!m) return AMR_EINVAL;
    try {
        m->err.clear();
        if (!m->dofs_set) throw AmrError(AMR_EINVAL, "amr_set_dofs must be called first");
        if (!m->K_valid) throw AmrError(AMR_EINVAL, "K has not been assembled");
        if (m->batch) throw AmrError(AMR_EUNSUPPORTED, "no-allocation solves of batched parts are not supported");
        if (!d_U || !d_F) throw AmrError(AMR_EINVAL, "null device buffer");
        const int64_t n = m->nnodes * m->B;
        if (n > kNoAllocMaxSlots)
            throw AmrError(AMR_EINVAL, "amr_solve_noalloc serves models of at most " + std::to_string(kNoAllocMaxSlots) +
                                           " node-DOF slots (nnodes x ndim); this model has " + std::to_string(n) +
                                           ": use amr_solve");
        int dev = 0, sms = 0;
        AMR_CUDA(cudaGetDevice(&dev));
        AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int grid = sms * 8;
        if (2 * grid + 8 > kNoAllocPartials) throw AmrError(AMR_EUNSUPPORTED, "too many SMs for the reduction scratch");
        amr_solve_opts o;
        amr_default_solve_opts(&o);
        if (opts) o = *opts;
        if (o.method != AMR_SOLVER_MIXED) throw AmrError(AMR_EINVAL, "amr_solve_noalloc runs the mixed-precision solver");
        const NoAllocView w = noalloc_view(noalloc_base());
        cudaStream_t s = m->stream;
        const int64_t nt = n;
        // x: prescribed values at prescribed slots, 0 at free slots; b: natural values at free slots
        AMR_CUDA(cudaMemsetAsync(w.x, 0, nt * sizeof(double), s));
        AMR_CUDA(cudaMemsetAsync(w.b, 0, nt * sizeof(double), s));
        AMR_CUDA(cudaMemsetAsync(w.reac, 0, nt * sizeof(double), s));
        k_gather_prescribed<<<nblk(nt, 256), 256, 0, s>>>(m->nnodes, m->B, m->eq_id, m->nu, m->ndofs, d_U, w.x);
        k_scatter_eq<<<nblk(nt, 256), 256, 0, s>>>(m->nnodes, m->B, m->eq_id, m->ndofs, w.b, d_F, 0);
        AMR_COUNT(2);
        AMR_CUDA(cudaGetLastError());
        AmrSolveResult r = m->B == 3 ? solve_mixed_noalloc<3>(m, w, grid, o) : solve_mixed_noalloc<2>(m, w, grid, o);
        if (stats) {
            stats->iterations = r.iterations;
            stats->refinements = r.refinements;
            stats->rel_residual = r.rel_residual;
            stats->seconds = r.seconds;
        }
        if (r.status) throw AmrError(r.status, "solve_system!: Krylov solver did not converge");
        // |U1|max > 1e8 check of solve_system! (src/solver.jl:68-71), partials as scratch
        double *out = w.partials + (kNoAllocPartials - 1);
        k_absmax<<<grid, kThreads, 0, s>>>(nt, w.x, m->free_mask, w.partials, &w.ctl->ticket[3], out);
        AMR_COUNT(1);
        double umax = 0.0;
        AMR_CUDA(cudaMemcpyAsync(&umax, out, sizeof(double), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        if (std::isnan(umax) || std::isinf(umax)) throw AmrError(AMR_ENAN, "solve_system!: NaN values in the solution");
        if (umax > 1e8) throw AmrError(AMR_ESINGULAR, "solve_system!: Possible syngular matrix");
        // U[:nu] <- solution, F[nu:] <- reactions
        k_scatter_eq<<<nblk(nt, 256), 256, 0, s>>>(m->nnodes, m->B, m->eq_id, m->nu, w.x, d_U, 1);
        k_scatter_prescribed<<<nblk(nt, 256), 256, 0, s>>>(m->nnodes, m->B, m->eq_id, m->nu, m->ndofs, w.reac, d_F);
        AMR_COUNT(2);
        AMR_CUDA(cudaGetLastError());
        AMR_CUDA(cudaStreamSynchronize(s));
        return AMR_OK;
    } catch (const AmrError &e) {
        m->err = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        m->err = e.what();
        return AMR_EINVAL;
    }
}
