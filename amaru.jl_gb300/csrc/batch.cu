// Batches of independent models: many FE models of uneven size joined into one
// handle, each a contiguous range of nodes ("part") with no element joining two.
//
// * Solve (solve_system!, src/solver.jl:5-79, once per part): one persistent
//   kernel.  CTAs take parts from an integer work counter, largest first, and
//   run the part's whole mixed-precision solve -- FP32 block-Jacobi PCG on the
//   part's rows of K32 with FP64 true-residual refreshes from K64 -- with
//   CTA barriers and fixed-order CTA reductions only.  No CTA waits on another.
//   The CTA size is fixed, so a part's arithmetic, and its result, is the same
//   whichever CTA takes it and whatever else is in the batch.
// * Stage (mech_stage_solver!, src/mech/mech-solver.jl:186-492, once per part):
//   each part keeps its own increment and Newton state (T, dT, iteration,
//   residue, status) on the device.  One Newton iteration of every part that is
//   still running is a fixed sequence of kernels -- per-part control, the
//   vector updates, the batched solve, the element update of the active parts,
//   the per-part residue, the commit or restore -- captured once as a CUDA graph
//   and replayed until every part has finished its stage.
// * Autotuner: elements per CTA of the element kernels and resident CTAs per SM
//   of the batched solve, timed on the model itself.
// * Multigrid solve (AMR_SOLVER_AMG): no element joins two parts, so neither do the
//   aggregates, prolongators and Galerkin products of the joined model's aggregation
//   multigrid: one V-cycle of the joined model preconditions every part at once.  The
//   PCG around it keeps its scalars per part (dot products per part, in a fixed order)
//   and its state per part (iterating, refreshing the FP64 residual, done); one
//   iteration of all parts is one CUDA graph, replayed until no part runs.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <functional>
#include <numeric>

#include <cooperative_groups.h>

#include "amr_internal.h"

namespace cg = cooperative_groups;

namespace {

constexpr int kPartThreads = 512;  // fixed: the reduction order of a part depends on it
constexpr int kWarps = kPartThreads / 32;
constexpr int kCluster = 8;                 // CTAs that solve one large part together
constexpr int64_t kClusterMinNodes = 2048;  // parts with this many nodes or more are large (fixed: results depend on it)

struct PartStat {
    int32_t iters, refreshes, status, pad;
    double rel_residual, umax;
};

enum { PH_START = 0, PH_ITER = 1, PH_DONE = 2 };
enum { ACT_NONE = 0, ACT_COMMIT = 1, ACT_RESTORE = 2 };

// per-part Newton / increment state of a batched stage
struct PartCtl {
    double T, dT, dTbk, Tcheck, acr, cR, res, res1, lastres, err;
    int32_t phase, it, increments, iterations, krylov, status, start, syserr, action, pad;
};

struct StageP {
    double tol, rtol, rspan, dTmin, dTmax, dTcheck;
    int32_t maxits, autoinc;
};

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// what the host reads after each Newton iteration of a batched stage
struct StepInfo {
    unsigned long long t0, t1;  // %globaltimer span of the batched solve (ns): first CTA start, last CTA end
    int32_t remaining, pad;     // parts still running their stage
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// CTA-wide sums: FP32 partials per thread, FP32 warp trees, the warps' sums
// added in FP64 in warp order.  Every thread receives the totals.
// ---------------------------------------------------------------------------
template <int NV>
__device__ void cta_sum(const float (&v)[NV], double (&out)[NV], float *sh, double *shd) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; i++) {
        float x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[i * kWarps + w] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int q = 0; q < kWarps; q++) s += (double)sh[threadIdx.x * kWarps + q];
        shd[threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; i++) out[i] = shd[i];
    __syncthreads();
}

__device__ double cta_max(double v, double *shd) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) shd[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0.0;
        for (int q = 0; q < kWarps; q++) m = fmax(m, shd[q]);
        shd[kWarps] = m;
    }
    __syncthreads();
    double r = shd[kWarps];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double absnan(double x) {  // |x|, NaN as +inf (as the whole-model norm)
    double a = fabs(x);
    return isnan(a) ? INFINITY : a;
}

// q = K32 p on rows [n0, n1), a half-warp per row, kRows rows per half-warp in flight
// (two measured faster than four: register pressure).  Returns this thread's part of
// p.q (its rows in increasing order).
constexpr int kRows = 2;
template <int B>
__device__ float part_spmv32(int64_t n0, int64_t n1, int64_t nb, const int64_t *__restrict__ rp,
                             const int32_t *__restrict__ cj, const float *__restrict__ A, const float *__restrict__ p,
                             float *__restrict__ q) {
    constexpr int G = 16;
    const int lane = threadIdx.x & (G - 1);
    const int hw = threadIdx.x / G, nhw = kPartThreads / G;
    const unsigned hmask = 0xffffu << (16 * (hw & 1));
    float dot = 0.0f;
    for (int64_t base = n0 + hw; base < n1; base += kRows * nhw) {
        float acc[kRows][B];
        int64_t a0[kRows], e0[kRows];
        int64_t len = 0;
#pragma unroll
        for (int r = 0; r < kRows; r++) {
            const int64_t row = base + r * nhw;
            a0[r] = row < n1 ? __ldg(rp + row) : 0;
            e0[r] = row < n1 ? __ldg(rp + row + 1) : 0;
            len = max(len, e0[r] - a0[r]);
#pragma unroll
            for (int c = 0; c < B; c++) acc[r][c] = 0.0f;
        }
        for (int64_t k = lane; k < len; k += G) {
#pragma unroll
            for (int r = 0; r < kRows; r++) {
                if (a0[r] + k < e0[r]) {
                    const int64_t kk = a0[r] + k, j = __ldg(cj + kk);
                    float av[B * B], xv[B];
#pragma unroll
                    for (int t = 0; t < B * B; t++) av[t] = __ldcs(A + (int64_t)t * nb + kk);
#pragma unroll
                    for (int d = 0; d < B; d++) xv[d] = p[j * B + d];
#pragma unroll
                    for (int c = 0; c < B; c++)
#pragma unroll
                        for (int d = 0; d < B; d++) acc[r][c] = fmaf(av[c * B + d], xv[d], acc[r][c]);
                }
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int r = 0; r < kRows; r++)
#pragma unroll
                for (int c = 0; c < B; c++) acc[r][c] += __shfl_down_sync(hmask, acc[r][c], o, G);
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < kRows; r++) {
                const int64_t row = base + r * nhw;
                if (row < n1) {
#pragma unroll
                    for (int c = 0; c < B; c++) {
                        q[row * B + c] = acc[r][c];
                        dot = fmaf(p[row * B + c], acc[r][c], dot);
                    }
                }
            }
        }
    }
    return dot;
}

// FP64 true residual on rows [n0, n1): r = b - K64 u at free slots (0 at prescribed ones),
// reactions K64 u at prescribed slots, r32 = r, z = Minv r32; adds r.z and |r|^2 (FP32) to rz, rr.
template <int B>
__device__ void part_residual64(int64_t n0, int64_t n1, int64_t nb, const int64_t *__restrict__ rp,
                                const int32_t *__restrict__ cj, const double *__restrict__ A,
                                const uint8_t *__restrict__ fm, const double *__restrict__ b,
                                const double *__restrict__ u, double *__restrict__ reac, float *__restrict__ r32,
                                float *__restrict__ z, const float *__restrict__ Minv, float &rz, float &rr) {
    constexpr int G = 16;
    const int lane = threadIdx.x & (G - 1);
    const int hw = threadIdx.x / G, nhw = kPartThreads / G;
    const unsigned hmask = 0xffffu << (16 * (hw & 1));
    for (int64_t n = n0 + hw; n < n1; n += nhw) {
        double acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0;
        for (int64_t k = rp[n] + lane; k < rp[n + 1]; k += G) {
            const int64_t j = cj[k];
#pragma unroll
            for (int c = 0; c < B; c++)
#pragma unroll
                for (int d = 0; d < B; d++) acc[c] = fma(A[(int64_t)(c * B + d) * nb + k], u[j * B + d], acc[c]);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < B; c++) acc[c] += __shfl_down_sync(hmask, acc[c], o, G);
        if (lane == 0) {
            float rv[B];
#pragma unroll
            for (int c = 0; c < B; c++) {
                double res = 0.0;
                if (fm[n * B + c]) res = b[n * B + c] - acc[c];
                else reac[n * B + c] = acc[c];
                rv[c] = (float)res;
                r32[n * B + c] = rv[c];
                rr = fmaf(rv[c], rv[c], rr);
            }
#pragma unroll
            for (int c = 0; c < B; c++) {
                float s = 0.0f;
#pragma unroll
                for (int d = 0; d < B; d++) s = fmaf(Minv[n * B * B + c * B + d], rv[d], s);
                z[n * B + c] = s;
                rz = fmaf(rv[c], s, rz);
            }
        }
    }
}

struct PcgArgs {
    int64_t nlarge, nsmall;   // parts solved by a CTA cluster / by one CTA
    const int64_t *part_ptr;  // node ranges
    const int64_t *order;     // parts, most nodes first: the nlarge large ones, then the small ones
    const uint8_t *active;    // null: every part
    int64_t nb;
    const int64_t *rp;
    const int32_t *cj;
    const float *K32;
    const double *K64;
    const float *Minv;
    const uint8_t *fm;
    const double *b;
    double *x;  // in: prescribed values at prescribed slots, 0 at free ones; out: solution
    double *reac;
    float *x32, *r32, *z32, *p32, *q32;
    PartStat *stat;
    unsigned long long *counter;  // [0]: next large part (per cluster), [1]: next small part (per CTA)
    StepInfo *step;               // null: no timing
    double tol2;
    int max_iters, force_every;
};

struct PartSmem {
    float sh[2 * kWarps];
    double shd[kWarps + 1];
    double slot[2][4];  // this CTA's partials for the cluster sums, two sets used alternately
    long long part;
};

// Sums over the CTAs of the part: per CTA as cta_sum, then, in a cluster, the CTAs'
// totals read from each CTA's shared memory and added in rank order (a fixed shuffle
// tree).  Every thread of every CTA receives the same totals.
template <int NV, bool CL>
__device__ void part_sum(const float (&v)[NV], double (&out)[NV], PartSmem &S, int &phase) {
    double cta[NV];
    cta_sum<NV>(v, cta, S.sh, S.shd);
    if (!CL) {
#pragma unroll
        for (int i = 0; i < NV; i++) out[i] = cta[i];
        return;
    }
    cg::cluster_group cl = cg::this_cluster();
    double *slot = S.slot[phase & 1];
    phase++;
    if (threadIdx.x == 0)
        for (int i = 0; i < NV; i++) slot[i] = cta[i];
    cl.sync();
    if (threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
        const double *rs = lane < kCluster ? cl.map_shared_rank(slot, lane) : nullptr;
#pragma unroll
        for (int i = 0; i < NV; i++) {
            double t = rs ? rs[i] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (lane == 0) S.shd[i] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; i++) out[i] = S.shd[i];
    __syncthreads();
}

template <bool CL>
__device__ double part_max(double v, PartSmem &S, int &phase) {
    double m = cta_max(v, S.shd);
    if (!CL) return m;
    cg::cluster_group cl = cg::this_cluster();
    double *slot = S.slot[phase & 1];
    phase++;
    if (threadIdx.x == 0) slot[0] = m;
    cl.sync();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (unsigned r = 0; r < kCluster; r++) t = fmax(t, cl.map_shared_rank(slot, r)[0]);
        S.shd[0] = t;
    }
    __syncthreads();
    m = S.shd[0];
    __syncthreads();
    return m;
}

// One part's solve: PCG with reliable updates, as the whole-model mixed solver
// (restart-free; refresh when the recursive residual has dropped 100x since the last
// refresh or looks converged; convergence judged on the FP64 residual).  In a cluster
// (CL) CTA `rank` owns a contiguous slice of the part's rows; p and the FP64 solution,
// the only vectors read across slices, are published by cluster barriers.
template <int B, bool CL>
__device__ void solve_part(const PcgArgs &a, long long part, int rank, PartSmem &S, int &phase) {
    constexpr int nranks = CL ? kCluster : 1;
    const int64_t P0 = a.part_ptr[part], P1 = a.part_ptr[part + 1], len = P1 - P0;
    const int64_t n0 = P0 + len * rank / nranks, n1 = P0 + len * (rank + 1) / nranks;
    const int64_t i0 = n0 * B, i1 = n1 * B;
    auto publish = [&]() {
        if (CL) cg::this_cluster().sync();
        else __syncthreads();
    };
    for (int64_t i = i0 + threadIdx.x; i < i1; i += kPartThreads) {
        a.x32[i] = 0.0f;
        a.p32[i] = 0.0f;
    }
    float rz = 0.0f, rr = 0.0f;
    part_residual64<B>(n0, n1, a.nb, a.rp, a.cj, a.K64, a.fm, a.b, a.x, a.reac, a.r32, a.z32, a.Minv, rz, rr);
    double t2[2];
    part_sum<2, CL>({rz, rr}, t2, S, phase);
    double gam = t2[0], rr_true = t2[1];
    const double bnorm2 = rr_true;
    const double stop_rr = 0.0625 * a.tol2 * bnorm2;
    int iters = 0, refreshes = 0, status = 0, since = 0;
    bool first = true, done = !(bnorm2 > 0.0) || rr_true <= a.tol2 * bnorm2;
    double beta = 0.0;
    if (isnan(rr_true)) { status = AMR_ENOCONV; done = true; }
    while (!done) {
        if (iters >= a.max_iters) { status = AMR_ENOCONV; break; }
        const float bf = first ? 0.0f : (float)beta;
        for (int64_t i = i0 + threadIdx.x; i < i1; i += kPartThreads) a.p32[i] = fmaf(bf, a.p32[i], a.z32[i]);
        publish();
        const float pq = part_spmv32<B>(n0, n1, a.nb, a.rp, a.cj, a.K32, a.p32, a.q32);
        double t1[1];
        part_sum<1, CL>({pq}, t1, S, phase);
        if (!(t1[0] > 0.0)) { status = AMR_ENOCONV; break; }
        const float af = (float)(gam / t1[0]);
        first = false;
        float rzl = 0.0f, rrl = 0.0f;
        for (int64_t n = n0 + threadIdx.x; n < n1; n += kPartThreads) {
            float rv[B];
#pragma unroll
            for (int c = 0; c < B; c++) {
                const int64_t i = n * B + c;
                a.x32[i] = fmaf(af, a.p32[i], a.x32[i]);
                rv[c] = fmaf(-af, a.q32[i], a.r32[i]);
                a.r32[i] = rv[c];
            }
#pragma unroll
            for (int c = 0; c < B; c++) {
                float s = 0.0f;
#pragma unroll
                for (int d = 0; d < B; d++) s = fmaf(a.Minv[n * B * B + c * B + d], rv[d], s);
                a.z32[n * B + c] = s;
                rzl = fmaf(rv[c], s, rzl);
                rrl = fmaf(rv[c], rv[c], rrl);
            }
        }
        part_sum<2, CL>({rzl, rrl}, t2, S, phase);
        beta = t2[0] / gam;
        gam = t2[0];
        iters++;
        since++;
        if (!(t2[1] > stop_rr) || t2[1] <= 1e-2 * rr_true || since >= a.force_every) {
            for (int64_t i = i0 + threadIdx.x; i < i1; i += kPartThreads) {
                if (a.fm[i]) a.x[i] += (double)a.x32[i];
                a.x32[i] = 0.0f;
            }
            publish();
            rz = 0.0f;
            rr = 0.0f;
            part_residual64<B>(n0, n1, a.nb, a.rp, a.cj, a.K64, a.fm, a.b, a.x, a.reac, a.r32, a.z32, a.Minv, rz,
                               rr);
            part_sum<2, CL>({rz, rr}, t2, S, phase);
            gam = t2[0];
            rr_true = t2[1];
            refreshes++;
            since = 0;
            if (isnan(rr_true)) { status = AMR_ENOCONV; break; }
            if (rr_true <= a.tol2 * bnorm2) done = true;
        }
    }
    double um = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += kPartThreads)
        if (a.fm[i]) um = fmax(um, absnan(a.x[i]));
    um = part_max<CL>(um, S, phase);
    if (rank == 0 && threadIdx.x == 0) {
        a.stat[part].iters = iters;
        a.stat[part].refreshes = refreshes;
        a.stat[part].status = status;
        a.stat[part].rel_residual = bnorm2 > 0.0 ? sqrt(rr_true / bnorm2) : 0.0;
        a.stat[part].umax = um;
    }
}

// Persistent batched solve.  Clusters of kCluster CTAs first take the large parts
// (at least kClusterMinNodes nodes) from counter[0], one part per cluster; then every
// CTA takes small parts from counter[1] alone.  No CTA waits on a CTA outside its
// cluster, and a cluster's CTAs are resident together by construction.
// Occupancy: latency-bound, so in 2-D four resident CTAs per SM (32 registers, some spills) measured
// faster than two (64 registers, none): 512 QUAD8 models 0.48 s against 0.65 s.
template <int B>
constexpr int part_min_blocks() { return B == 2 ? 4 : 2; }

template <int B>
__global__ void __cluster_dims__(kCluster, 1, 1) __launch_bounds__(kPartThreads, part_min_blocks<B>())
    k_part_pcg(PcgArgs a) {
    __shared__ PartSmem S;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    int phase = 0;
    if (a.step && threadIdx.x == 0) atomicMin(&a.step->t0, global_ns());
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            const unsigned long long t = atomicAdd(&a.counter[0], 1ULL);
            S.part = (t < (unsigned long long)a.nlarge) ? (long long)a.order[t] : -1;
        }
        cl.sync();
        const long long part = *cl.map_shared_rank(&S.part, 0);
        cl.sync();
        if (part < 0) break;
        if (a.active && !a.active[part]) continue;
        solve_part<B, true>(a, part, rank, S, phase);
    }
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long t = atomicAdd(&a.counter[1], 1ULL);
            S.part = (t < (unsigned long long)a.nsmall) ? (long long)a.order[a.nlarge + t] : -1;
        }
        __syncthreads();
        const long long part = S.part;
        __syncthreads();
        if (part < 0) break;
        if (a.active && !a.active[part]) continue;
        solve_part<B, false>(a, part, 0, S, phase);
    }
    if (a.step && threadIdx.x == 0) atomicMax(&a.step->t1, global_ns());
}

// ---------------------------------------------------------------------------
// Batched stage: per-part control and per-slot vector kernels.  The vector
// arithmetic is that of the whole-model stage driver, slot by slot.
// ---------------------------------------------------------------------------
__device__ double round_sig3_d(double x) {  // round(x, sigdigits=3)
    if (x == 0.0 || !isfinite(x)) return x;
    const double e = floor(log10(fabs(x)));
    const double sc = pow(10.0, 2.0 - e);
    return round(x * sc) / sc;
}

__global__ void k_ctl_begin(int64_t np, PartCtl *c, uint8_t *active, int32_t *perr, StageP p) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    PartCtl q = c[i];
    perr[i] = 0;
    q.action = ACT_NONE;
    if (q.phase == PH_DONE) {
        active[i] = 0;
        c[i] = q;
        return;
    }
    if (q.phase == PH_START) {
        const double dTcr = fmin(p.rspan, 1.0 - q.T);
        q.acr = fmin(q.dT / dTcr, 1.0);
        q.cR = (q.T < 1.0 - p.rspan) ? q.acr : 0.0;
        q.start = 1;
        q.it = 0;
        q.res = q.res1 = q.err = 0.0;
        q.phase = PH_ITER;
    } else {
        q.start = 0;
    }
    q.syserr = 0;
    q.it += 1;
    q.lastres = q.res;
    active[i] = 1;
    c[i] = q;
}

struct SlotArgs {
    int64_t n;
    int B;
    double p1, q11;  // the predictor's factors of the scheme (mech-solver.jl:280-288)
    int corrector;   // ME / BE / Ralston: dUi comes from the corrector solve
    const int32_t *node_part;
    const PartCtl *c;
    const uint8_t *active;
    const uint8_t *fm;
    const double *Uex, *Fex;
    double *U, *F, *R, *Rc, *dUa, *dUi, *dUitr, *Rtr, *dUt, *dFin, *dFex;
};

__global__ void k_slot_begin(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    const int32_t p = a.node_part[t / a.B];
    if (!a.active[p]) return;
    const PartCtl &q = a.c[p];
    if (q.start) {
        const double f = q.dT * a.Fex[t] + q.cR * a.Rc[t];
        a.dFex[t] = f;
        a.R[t] = f;
        a.dUa[t] = 0.0;
        a.dUi[t] = q.dT * a.Uex[t] + 0.0;
    } else {
        a.dUi[t] = 0.0;
    }
    a.dUitr[t] = a.fm[t] ? 0.0 : a.p1 * a.dUi[t];
    a.Rtr[t] = a.q11 * a.R[t] + 0.0;
}

// corrector of ME / BE / Ralston (mech-solver.jl:341-348): parts whose predictor update failed leave the
// iteration; the others solve the weighted tangent for dUi (prescribed values kept) with the residual R
__global__ void k_ctl_corr(int64_t np, const int32_t *perr, uint8_t *active) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np && active[i] && perr[i]) active[i] = 0;
}

__global__ void k_slot_corr(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    if (!a.active[a.node_part[t / a.B]]) return;
    if (a.fm[t]) a.dUi[t] = 0.0;
    a.Rtr[t] = 1.0 * a.R[t] + 0.0;
}

__global__ void k_slot_mid2(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    if (!a.active[a.node_part[t / a.B]]) return;
    a.dUt[t] = 1.0 * a.dUa[t] + 1.0 * a.dUi[t];
}

__global__ void k_ctl_mid(int64_t np, PartCtl *c, const PartStat *st, uint8_t *active) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np || !active[i]) return;
    c[i].krylov += st[i].iters;
    if (st[i].status) {
        c[i].syserr = 1;  // Krylov solver did not converge
        active[i] = 0;
    } else if (!(st[i].umax <= 1e8)) {
        c[i].syserr = 2;  // possible singular matrix
        active[i] = 0;
    }
}

__global__ void k_slot_mid(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    if (!a.active[a.node_part[t / a.B]]) return;
    a.dUt[t] = 1.0 * a.dUa[t] + 1.0 * a.dUitr[t];
}

__global__ void k_slot_post(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    if (!a.active[a.node_part[t / a.B]]) return;
    const double di = a.corrector ? a.dUi[t] : a.dUitr[t];
    a.dUi[t] = di;
    a.dUa[t] = 1.0 * a.dUa[t] + 1.0 * di;
    const double r = 1.0 * a.dFex[t] + -1.0 * a.dFin[t];
    a.R[t] = a.fm[t] ? r : 0.0;
}

// residue max|R|, and |dUi|, |dUa| of each active part (CTA per part)
__global__ void __launch_bounds__(kPartThreads) k_part_norms(int64_t np, int B, const int64_t *part_ptr,
                                                             const uint8_t *active, const double *R,
                                                             const double *dUi, const double *dUa, PartCtl *c) {
    __shared__ double shd[kWarps + 1];
    for (int64_t p = blockIdx.x; p < np; p += gridDim.x) {
        if (!active[p]) continue;
        const int64_t i0 = part_ptr[p] * B, i1 = part_ptr[p + 1] * B;
        double r = 0.0, ui = 0.0, ua = 0.0;
        for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
            r = fmax(r, absnan(R[i]));
            ui = fmax(ui, absnan(dUi[i]));
            ua = fmax(ua, absnan(dUa[i]));
        }
        r = cta_max(r, shd);
        ui = cta_max(ui, shd);
        ua = cta_max(ua, shd);
        if (threadIdx.x == 0) {
            c[p].res = r;
            c[p].err = ui / ua;
        }
    }
}

__global__ void k_ctl_end(int64_t np, PartCtl *c, const int32_t *perr, StageP p, StepInfo *step) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    PartCtl q = c[i];
    if (q.phase != PH_ITER) return;
    const double eps = DBL_EPSILON;
    bool conv = false, fail = false;
    if (q.syserr) {
        fail = true;
    } else if (perr[i]) {
        q.syserr = 3;  // return mapping failed / NaN internal forces
        fail = true;
    } else {
        q.iterations++;
        if (q.it == 1) q.res1 = q.res;
        if (q.res < p.tol) conv = true;
        else if (q.err < p.rtol) conv = true;
        else if (isnan(q.res)) fail = true;
        else if (q.it > 1 && q.res > q.lastres) fail = true;
        else if (q.it >= p.maxits) fail = true;
    }
    if (conv) {
        q.action = ACT_COMMIT;
        q.T += q.dT;
        q.increments++;
        if (q.T > q.Tcheck - p.dTmin) q.Tcheck += p.dTcheck;
        if (p.autoinc) {
            if (q.dTbk > 0.0) {
                q.dT = fmin(q.dTbk, q.Tcheck - q.T);
                q.dTbk = 0.0;
            } else {
                double f = 1.0 + tanh(log10(p.tol / (q.res1 + eps)));
                f = fmax(f, 1.1);
                const double dTtr = fmin(fmin(f * q.dT, p.dTmax), 1.0 - q.T);
                if (q.T + dTtr > q.Tcheck - p.dTmin) {
                    q.dTbk = q.dT;
                    q.dT = q.Tcheck - q.T;
                } else {
                    q.dT = dTtr;
                    q.dTbk = 0.0;
                }
            }
        }
        q.phase = (q.T < 1.0 - p.dTmin) ? PH_START : PH_DONE;
    } else if (fail) {
        q.action = ACT_RESTORE;
        if (p.autoinc) {
            double f = 1.0 + tanh(log10(p.tol / (q.res1 + eps)));
            f = fmin(fmax(f, 0.2), 0.9);
            if (q.syserr) f = 0.7;
            q.dT = round_sig3_d(f * q.dT);
            if (q.dT < p.dTmin) {
                q.status = AMR_ESTAGE;
                q.phase = PH_DONE;
            } else {
                q.phase = PH_START;
            }
        } else {
            q.status = AMR_ESTAGE;
            q.phase = PH_DONE;
        }
    }
    if (q.phase != PH_DONE) atomicAdd(&step->remaining, 1);
    c[i] = q;
}

__global__ void k_slot_commit(SlotArgs a) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.n) return;
    const PartCtl &q = a.c[a.node_part[t / a.B]];
    if (q.action != ACT_COMMIT) return;
    a.U[t] = 1.0 * a.U[t] + 1.0 * a.dUa[t];
    a.F[t] = 1.0 * a.F[t] + 1.0 * a.dFin[t];
    a.Rc[t] = (1.0 - q.acr) * a.Rc[t] + 1.0 * a.R[t];
}

// StateBk <- State for committing parts, State <- StateBk for failing ones
__global__ void k_ip_commit(int64_t nip, const int32_t *ip_part, const PartCtl *c, double *st, double *stbk) {
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nip) return;
    const int32_t act = c[ip_part[g]].action;
    if (act == ACT_COMMIT) {
        for (int f = 0; f < AMR_NST; f++) stbk[f * nip + g] = st[f * nip + g];
    } else if (act == ACT_RESTORE) {
        for (int f = 0; f < AMR_NST; f++) st[f * nip + g] = stbk[f * nip + g];
    }
}

// ---------------------------------------------------------------------------
// Multigrid-preconditioned batched PCG: per-part state and kernels.  A part is BA_REFRESH for one
// iteration whenever its FP64 true residual is due (at the start, after a 100x drop of the recursive
// residual norm, when it looks converged, or every kBaSince iterations): its FP32 correction is folded
// into the FP64 solution and r = b - K64 x recomputed, instead of a CG step.  Every other running part
// takes a CG step; the V-cycle serves both.  Convergence is judged on the true residual, as in the
// whole-model multigrid solver.
// ---------------------------------------------------------------------------
enum { BA_DONE = 0, BA_ITER = 1, BA_REFRESH = 2 };
constexpr int kBaSince = 64;

struct PartAmg {
    double rz, pq, alpha, beta, rr, rr_true, bnorm2;
    int32_t state, iters, refreshes, since, first, status, initial, pad;
};

__global__ void k_ba_init(int64_t np, const uint8_t *active, PartAmg *pa) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    PartAmg a{};
    a.state = (!active || active[p]) ? BA_REFRESH : BA_DONE;
    a.first = 1;
    a.initial = 1;
    pa[p] = a;
}

// the fine-level rows the V-cycle works on: the nodes of running parts
__global__ void k_ba_gate(int64_t nn, const int32_t *__restrict__ node_part, const PartAmg *__restrict__ pa,
                          uint8_t *__restrict__ gate) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n < nn) gate[n] = pa[node_part[n]].state != BA_DONE;
}

__global__ void k_ba_stamp(StepInfo *step, int end) {
    if (end) atomicMax(&step->t1, global_ns());
    else atomicMin(&step->t0, global_ns());
}

template <int B>
__global__ void k_ba_pupdate(int64_t nn, const int32_t *__restrict__ node_part, const PartAmg *__restrict__ pa,
                             const float *__restrict__ z, float *__restrict__ p) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn * B) return;
    const PartAmg &a = pa[node_part[i / B]];
    if (a.state != BA_ITER) return;
    p[i] = a.first ? z[i] : fmaf((float)a.beta, p[i], z[i]);
}

// q = K32 p on the rows of the iterating parts: a half-warp per row
template <int B>
__global__ void __launch_bounds__(256) k_ba_spmv(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                 const int32_t *__restrict__ cj, const float *__restrict__ K,
                                                 const int32_t *__restrict__ node_part, const PartAmg *__restrict__ pa,
                                                 const float *__restrict__ p, float *__restrict__ q) {
    constexpr int G = 16;
    const int lane = threadIdx.x % G;
    const unsigned hmask = 0xffffu << (16 * ((threadIdx.x >> 4) & 1));
    const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t row = grp; row < nn; row += ng) {
        if (pa[node_part[row]].state != BA_ITER) continue;  // uniform over the half-warp
        float acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0f;
        for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += G) {
            const int64_t j = cj[k];
            float xv[B];
#pragma unroll
            for (int d = 0; d < B; d++) xv[d] = __ldg(p + j * B + d);
#pragma unroll
            for (int c = 0; c < B; c++)
#pragma unroll
                for (int d = 0; d < B; d++) acc[c] = fmaf(__ldcs(K + (int64_t)(c * B + d) * nb + k), xv[d], acc[c]);
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < B; c++) acc[c] += __shfl_down_sync(hmask, acc[c], o, G);
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < B; c++) q[row * B + c] = acc[c];
    }
}

// sums of two per-slot products over a part's slots [i0, i1): FP64 per thread in slot order, then a
// fixed tree over the CTA; every thread receives the totals
__device__ void ba_part_sums(int64_t i0, int64_t i1, const float *a, const float *b, const float *c,
                             const float *d, double &s0, double &s1, double *sh) {
    double v0 = 0.0, v1 = 0.0;
    for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        v0 += (double)a[i] * (double)b[i];
        if (c) v1 += (double)c[i] * (double)d[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, o);
        v1 += __shfl_down_sync(0xffffffffu, v1, o);
    }
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if ((threadIdx.x & 31) == 0) { sh[w] = v0; sh[32 + w] = v1; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t0 = 0.0, t1 = 0.0;
        for (int k = 0; k < nw; k++) { t0 += sh[k]; t1 += sh[32 + k]; }
        sh[64] = t0;
        sh[65] = t1;
    }
    __syncthreads();
    s0 = sh[64];
    s1 = sh[65];
    __syncthreads();
}

// alpha = rz / p.q of every iterating part (CTA per part)
__global__ void __launch_bounds__(256) k_ba_pq(int64_t np, int B, const int64_t *__restrict__ part_ptr,
                                               const float *__restrict__ p, const float *__restrict__ q, PartAmg *pa) {
    __shared__ double sh[66];
    for (int64_t part = blockIdx.x; part < np; part += gridDim.x) {
        if (pa[part].state != BA_ITER) continue;  // uniform over the CTA
        double pq, unused;
        ba_part_sums(part_ptr[part] * B, part_ptr[part + 1] * B, p, q, nullptr, nullptr, pq, unused, sh);
        if (threadIdx.x == 0) {
            PartAmg &a = pa[part];
            if (!(pq > 0.0)) {  // breakdown (or NaN)
                a.status = AMR_ENOCONV;
                a.state = BA_DONE;
            } else {
                a.pq = pq;
                a.alpha = a.rz / pq;
                a.first = 0;
            }
        }
        __syncthreads();
    }
}

template <int B>
__global__ void k_ba_update(int64_t nn, const int32_t *__restrict__ node_part, const PartAmg *__restrict__ pa,
                            const float *__restrict__ p, const float *__restrict__ q, float *__restrict__ x32,
                            float *__restrict__ r32) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn * B) return;
    const PartAmg &a = pa[node_part[i / B]];
    if (a.state != BA_ITER) return;
    const float al = (float)a.alpha;
    x32[i] = fmaf(al, p[i], x32[i]);
    r32[i] = fmaf(-al, q[i], r32[i]);
}

// refreshing parts: x += x32 at free slots, x32 = 0
template <int B>
__global__ void k_ba_fold(int64_t nn, const int32_t *__restrict__ node_part, const PartAmg *__restrict__ pa,
                          const uint8_t *__restrict__ fm, float *__restrict__ x32, double *__restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn * B) return;
    if (pa[node_part[i / B]].state != BA_REFRESH) return;
    if (fm[i]) x[i] += (double)x32[i];
    x32[i] = 0.0f;
}

// refreshing parts' rows: r = b - K64 x at free slots (0 at prescribed ones), reac = (K64 x) at prescribed
// slots, r32 = r; four lanes per row
template <int B>
__global__ void __launch_bounds__(256) k_ba_refine(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                   const int32_t *__restrict__ cj, const double *__restrict__ A,
                                                   const uint8_t *__restrict__ fm, const int32_t *__restrict__ node_part,
                                                   const PartAmg *__restrict__ pa, const double *__restrict__ b,
                                                   const double *__restrict__ x, double *__restrict__ reac,
                                                   float *__restrict__ r32) {
    constexpr int L = 4, RPW = 32 / L;
    const int lane = threadIdx.x & 31, sub = lane & (L - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t n0 = warp * RPW; n0 < nn; n0 += nw * RPW) {  // whole warps: every lane reaches the shuffles
        const int64_t n = n0 + lane / L;
        const bool valid = n < nn && pa[node_part[n < nn ? n : 0]].state == BA_REFRESH;
        double acc[B];
#pragma unroll
        for (int c = 0; c < B; c++) acc[c] = 0.0;
        if (valid)
            for (int64_t k = rp[n] + sub; k < rp[n + 1]; k += L) {
                const int64_t j = __ldg(cj + k);
                double xv[B];
#pragma unroll
                for (int d = 0; d < B; d++) xv[d] = __ldg(x + j * B + d);
#pragma unroll
                for (int c = 0; c < B; c++)
#pragma unroll
                    for (int d = 0; d < B; d++) acc[c] = fma(__ldg(A + (int64_t)(c * B + d) * nb + k), xv[d], acc[c]);
            }
#pragma unroll
        for (int c = 0; c < B; c++)
#pragma unroll
            for (int o = L / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (valid && sub == 0)
#pragma unroll
            for (int c = 0; c < B; c++) {
                const int64_t i = n * B + c;
                double res = 0.0;
                if (fm[i]) res = b[i] - acc[c];
                else if (reac) reac[i] = acc[c];
                r32[i] = (float)res;
            }
    }
}

// after the V-cycle: r.z and |r|^2 per running part (CTA per part), and its next state
__global__ void __launch_bounds__(256) k_ba_rz(int64_t np, int B, const int64_t *__restrict__ part_ptr,
                                               const float *__restrict__ r, const float *__restrict__ z, PartAmg *pa,
                                               double stop_rel, double delta2, double tol2, int max_iters) {
    __shared__ double sh[66];
    for (int64_t part = blockIdx.x; part < np; part += gridDim.x) {
        const int state = pa[part].state;
        if (state == BA_DONE) continue;  // uniform over the CTA
        double rz, rr;
        ba_part_sums(part_ptr[part] * B, part_ptr[part + 1] * B, r, z, r, r, rz, rr, sh);
        if (threadIdx.x == 0) {
            PartAmg &a = pa[part];
            if (state == BA_ITER) {
                a.beta = rz / a.rz;
                a.rz = rz;
                a.rr = rr;
                a.iters++;
                a.since++;
                if (isnan(rr)) { a.status = AMR_ENOCONV; a.state = BA_DONE; }
                else if (!(rr > stop_rel * a.bnorm2) || rr <= delta2 * a.rr_true || a.since >= kBaSince) a.state = BA_REFRESH;
                else if (a.iters >= max_iters) { a.status = AMR_ENOCONV; a.state = BA_DONE; }
            } else {  // the true residual of a refresh
                a.rz = rz;
                a.rr = rr;
                a.rr_true = rr;
                if (a.initial) { a.bnorm2 = rr; a.initial = 0; }
                else a.refreshes++;
                a.since = 0;
                if (isnan(rr)) { a.status = AMR_ENOCONV; a.state = BA_DONE; }
                else if (!(a.bnorm2 > 0.0) || rr <= tol2 * a.bnorm2) a.state = BA_DONE;
                else if (a.iters >= max_iters) { a.status = AMR_ENOCONV; a.state = BA_DONE; }
                else a.state = BA_ITER;
            }
        }
        __syncthreads();
    }
}

// parts still running and the largest iteration count
__global__ void k_ba_summary(int64_t np, const PartAmg *pa, int32_t *out) {
    __shared__ int run, its;
    if (threadIdx.x == 0) { run = 0; its = 0; }
    __syncthreads();
    int r = 0, m = 0;
    for (int64_t p = threadIdx.x; p < np; p += blockDim.x) {
        if (pa[p].state != BA_DONE) r++;
        m = max(m, pa[p].iters);
    }
    atomicAdd(&run, r);
    atomicMax(&its, m);
    __syncthreads();
    if (threadIdx.x == 0) { out[0] = run; out[1] = its; }
}

// the parts' results into the part statistics (CTA per part of the solve)
__global__ void __launch_bounds__(256) k_ba_finish(int64_t np, int B, const int64_t *__restrict__ part_ptr,
                                                   const uint8_t *__restrict__ active, const uint8_t *__restrict__ fm,
                                                   const double *__restrict__ x, PartAmg *pa, PartStat *stat,
                                                   int abort) {
    __shared__ double sh[32];
    for (int64_t part = blockIdx.x; part < np; part += gridDim.x) {
        if (active && !active[part]) continue;
        double um = 0.0;
        for (int64_t i = part_ptr[part] * B + threadIdx.x; i < part_ptr[part + 1] * B; i += blockDim.x)
            if (fm[i]) um = fmax(um, absnan(x[i]));
        for (int o = 16; o > 0; o >>= 1) um = fmax(um, __shfl_down_sync(0xffffffffu, um, o));
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = um;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int k = 1; k < (int)(blockDim.x >> 5); k++) um = fmax(um, sh[k]);
            PartAmg &a = pa[part];
            if (abort && a.state != BA_DONE) { a.status = AMR_ENOCONV; a.state = BA_DONE; }
            PartStat s;
            s.iters = a.iters;
            s.refreshes = a.refreshes;
            s.status = a.status;
            s.pad = 0;
            s.rel_residual = a.bnorm2 > 0.0 ? sqrt(a.rr_true / a.bnorm2) : 0.0;
            s.umax = fmax(um, sh[0]);
            stat[part] = s;
        }
        __syncthreads();
    }
}

}  // namespace

struct AmrBatch {
    int64_t nparts = 0, nlarge = 0;
    std::vector<int64_t> h_ptr;
    int64_t *part_ptr = nullptr, *order = nullptr;
    int32_t *node_part = nullptr, *elem_part = nullptr, *ip_part = nullptr;
    PartStat *stat = nullptr;
    PartCtl *ctl = nullptr;
    uint8_t *active = nullptr;
    int32_t *perr = nullptr;
    StepInfo *step = nullptr, *h_step = nullptr;
    unsigned long long *counter = nullptr;
    float *x32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr;
    PartAmg *pamg = nullptr;         // per-part state of the multigrid solve
    uint8_t *gate = nullptr;         // its fine-level row gate (nodes of running parts)
    int32_t *bsum = nullptr, *h_bsum = nullptr;  // its summary: parts running, largest iteration count
    int ctas_per_sm = 2;  // until tuned: the residency the kernel is compiled for
    std::vector<PartCtl> h_ctl;
    std::vector<PartStat> h_stat;
    double stage_seconds = 0.0, stage_solve_seconds = 0.0;
    bool have_stage = false;
};

void amr_batch_free(amr_model *m) {
    AmrBatch *b = m->batch;
    if (!b) return;
    amr_free(b->part_ptr); amr_free(b->order); amr_free(b->node_part); amr_free(b->elem_part);
    amr_free(b->ip_part); amr_free(b->stat); amr_free(b->ctl); amr_free(b->active); amr_free(b->perr);
    amr_free(b->step); amr_free(b->counter);
    amr_free(b->x32); amr_free(b->r32); amr_free(b->z32); amr_free(b->p32); amr_free(b->q32);
    amr_free(b->pamg); amr_free(b->bsum); amr_free(b->gate);
    amr_pinned_free(b->h_step);
    amr_pinned_free(b->h_bsum);
    delete b;
    m->batch = nullptr;
}

void amr_batch_set(amr_model *m, int64_t nparts, const int64_t *ptr) {
    if (nparts < 1) throw AmrError(AMR_EINVAL, "nparts must be >= 1");
    if (!ptr) throw AmrError(AMR_EINVAL, "null node_ptr");
    if (nparts > INT32_MAX) throw AmrError(AMR_EINVAL, "too many parts");
    if (ptr[0] != 0 || ptr[nparts] != m->nnodes) throw AmrError(AMR_EINVAL, "parts must cover nodes 0..nnodes-1");
    for (int64_t i = 0; i < nparts; i++)
        if (ptr[i + 1] <= ptr[i]) throw AmrError(AMR_EINVAL, "parts must be non-empty node ranges in increasing order");
    std::vector<int32_t> npart(m->nnodes);
    for (int64_t i = 0; i < nparts; i++)
        for (int64_t n = ptr[i]; n < ptr[i + 1]; n++) npart[n] = (int32_t)i;
    std::vector<int32_t> epart(m->nelems);
    for (int64_t s = 0; s < m->nelems; s++) {  // sorted element order
        const int32_t q = npart[m->h_conn[m->h_conn_ptr[s]]];
        for (int64_t k = m->h_conn_ptr[s]; k < m->h_conn_ptr[s + 1]; k++)
            if (npart[m->h_conn[k]] != q)
                throw AmrError(AMR_EINVAL, "element " + std::to_string(m->perm[s] + 1) + " joins two parts");
        epart[s] = q;
    }
    std::vector<int32_t> ipart(m->nip_total);
    for (int64_t s = 0; s < m->nelems; s++)
        for (int64_t g = m->h_ip_ptr[s]; g < m->h_ip_ptr[s + 1]; g++) ipart[g] = epart[s];
    std::vector<int64_t> order(nparts);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int64_t x, int64_t y) { return ptr[x + 1] - ptr[x] > ptr[y + 1] - ptr[y]; });
    int64_t nlarge = 0;
    while (nlarge < nparts && ptr[order[nlarge] + 1] - ptr[order[nlarge]] >= kClusterMinNodes) nlarge++;
    amr_batch_free(m);
    AmrBatch *b = new AmrBatch();
    m->batch = b;
    try {
        b->nparts = nparts;
        b->nlarge = nlarge;
        b->ctas_per_sm = m->B == 2 ? part_min_blocks<2>() : part_min_blocks<3>();
        b->h_ptr.assign(ptr, ptr + nparts + 1);
        const int64_t n = m->nnodes * m->B;
        amr_alloc(&b->part_ptr, nparts + 1);
        amr_alloc(&b->order, nparts);
        amr_alloc(&b->node_part, m->nnodes);
        amr_alloc(&b->elem_part, m->nelems);
        amr_alloc(&b->ip_part, m->nip_total);
        amr_alloc(&b->stat, nparts);
        amr_alloc(&b->ctl, nparts);
        amr_alloc(&b->active, nparts);
        amr_alloc(&b->perr, nparts);
        amr_alloc(&b->step, 1);
        amr_alloc(&b->counter, 2);
        amr_alloc(&b->x32, n); amr_alloc(&b->r32, n); amr_alloc(&b->z32, n); amr_alloc(&b->p32, n);
        amr_alloc(&b->q32, n);
        b->h_step = (StepInfo *)amr_pinned_alloc(sizeof(StepInfo));
        amr_h2d(m, b->part_ptr, ptr, (nparts + 1) * sizeof(int64_t));
        amr_h2d(m, b->order, order.data(), nparts * sizeof(int64_t));
        amr_h2d(m, b->node_part, npart.data(), npart.size() * sizeof(int32_t));
        amr_h2d(m, b->elem_part, epart.data(), epart.size() * sizeof(int32_t));
        amr_h2d(m, b->ip_part, ipart.data(), ipart.size() * sizeof(int32_t));
        b->h_ctl.resize(nparts);
        b->h_stat.resize(nparts);
    } catch (...) {
        amr_batch_free(m);
        throw;
    }
}

namespace {

int device_sms() {
    int dev = 0, sms = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    return sms;
}

PcgArgs pcg_args(amr_model *m, double *x, const double *b_, double *reac, const amr_solve_opts &o,
                 const uint8_t *active) {
    AmrBatch *b = m->batch;
    PcgArgs a;
    a.nlarge = b->nlarge; a.nsmall = b->nparts - b->nlarge; a.part_ptr = b->part_ptr; a.order = b->order;
    a.active = active;
    a.nb = m->bstride; a.rp = m->brow_ptr; a.cj = m->bcol; a.K32 = m->K32; a.K64 = m->K64; a.Minv = m->Minv32;
    a.fm = m->free_mask; a.b = b_; a.x = x; a.reac = reac;
    a.x32 = b->x32; a.r32 = b->r32; a.z32 = b->z32; a.p32 = b->p32; a.q32 = b->q32;
    a.stat = b->stat; a.counter = b->counter; a.step = nullptr; a.tol2 = o.rtol * o.rtol; a.max_iters = o.max_iters;
    a.force_every = 16 * (o.refine_every > 0 ? o.refine_every : 32);
    return a;
}

void launch_pcg(amr_model *m, const PcgArgs &a, int ctas_per_sm) {
    AmrBatch *b = m->batch;
    AMR_CUDA(cudaMemsetAsync(b->counter, 0, 2 * sizeof(unsigned long long), m->stream));
    // whole clusters: as many CTAs as the parts can use (a cluster per large part, a CTA per small
    // one), at most ctas_per_sm per SM
    const int64_t need = b->nlarge * kCluster + (b->nparts - b->nlarge);
    const int64_t ctas = std::min<int64_t>(std::max<int64_t>(need, kCluster), (int64_t)device_sms() * ctas_per_sm);
    const unsigned grid = (unsigned)(std::max<int64_t>(1, ctas / kCluster) * kCluster);
    if (m->B == 3) k_part_pcg<3><<<grid, kPartThreads, 0, m->stream>>>(a);
    else k_part_pcg<2><<<grid, kPartThreads, 0, m->stream>>>(a);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

struct GraphScope {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    ~GraphScope() {
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
    }
};

constexpr int kBaEvery = 4;  // iterations of the multigrid solve between host checks

// The multigrid-preconditioned solve of every part (the active ones when active is given): x (free slots)
// updated in place from b, reactions at the prescribed slots; the parts' results into the part statistics.
// The iteration is captured as a CUDA graph once per call and replayed kBaEvery times between host checks.
void batch_solve_amg(amr_model *m, double *x, const double *b_, double *reac, const amr_solve_opts &o,
                     const uint8_t *active, StepInfo *step) {
    AmrBatch *b = m->batch;
    cudaStream_t s = m->stream;
    const int64_t np = b->nparts, nn = m->nnodes, n = nn * m->B;
    const int B = m->B;
    amr_amg_prepare(m);
    if (!b->pamg) {
        amr_alloc(&b->pamg, np);
        amr_alloc(&b->gate, nn);
        amr_alloc(&b->bsum, 2);
        b->h_bsum = (int32_t *)amr_pinned_alloc(2 * sizeof(int32_t));
    }
    if (step) {
        k_ba_stamp<<<1, 1, 0, s>>>(step, 0);
        AMR_COUNT(1);
    }
    k_ba_init<<<nblk(np, 128), 128, 0, s>>>(np, active, b->pamg);
    AMR_COUNT(1);
    // every vector starts finite: the V-cycle runs over all parts, running or not
    for (float *v : {b->x32, b->p32, b->r32, b->z32, b->q32}) AMR_CUDA(cudaMemsetAsync(v, 0, n * sizeof(float), s));
    const double tol2 = o.rtol * o.rtol, stop_rel = 0.0625 * tol2, delta2 = 1e-4;
    const int max_iters = o.max_iters > 0 ? o.max_iters : 20000;
    const unsigned gs = nblk(n, 256), gsp = (unsigned)std::min<int64_t>(nblk(nn * 16, 256), (int64_t)device_sms() * 8);
    const unsigned gr = (unsigned)std::min<int64_t>(nblk(nn * 8, 256), (int64_t)device_sms() * 8);
    const unsigned gparts = (unsigned)std::min<int64_t>(np, (int64_t)device_sms() * 8);
    auto one = [&]() {
        if (B == 3) {
            k_ba_pupdate<3><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, b->z32, b->p32);
            k_ba_spmv<3><<<gsp, 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K32, b->node_part, b->pamg, b->p32, b->q32);
        } else {
            k_ba_pupdate<2><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, b->z32, b->p32);
            k_ba_spmv<2><<<gsp, 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K32, b->node_part, b->pamg, b->p32, b->q32);
        }
        k_ba_pq<<<gparts, 256, 0, s>>>(np, B, b->part_ptr, b->p32, b->q32, b->pamg);
        if (B == 3) {
            k_ba_update<3><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, b->p32, b->q32, b->x32, b->r32);
            k_ba_fold<3><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, m->free_mask, b->x32, x);
            k_ba_refine<3><<<gr, 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b->node_part,
                                               b->pamg, b_, x, reac, b->r32);
        } else {
            k_ba_update<2><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, b->p32, b->q32, b->x32, b->r32);
            k_ba_fold<2><<<gs, 256, 0, s>>>(nn, b->node_part, b->pamg, m->free_mask, b->x32, x);
            k_ba_refine<2><<<gr, 256, 0, s>>>(nn, m->bstride, m->brow_ptr, m->bcol, m->K64, m->free_mask, b->node_part,
                                               b->pamg, b_, x, reac, b->r32);
        }
        k_ba_gate<<<nblk(nn, 256), 256, 0, s>>>(nn, b->node_part, b->pamg, b->gate);
        AMR_COUNT(7);
        amr_amg_vcycle(m, b->r32, b->z32);
        k_ba_rz<<<gparts, 256, 0, s>>>(np, B, b->part_ptr, b->r32, b->z32, b->pamg, stop_rel, delta2, tol2, max_iters);
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
    };
    GraphScope gr_;
    struct GateScope {  // the cycle skips the rows of finished parts while this solve runs
        amr_model *m;
        GateScope(amr_model *m_, const uint8_t *g) : m(m_) { amr_amg_set_gate(m, g); }
        ~GateScope() { amr_amg_set_gate(m, nullptr); }
    } gate_scope(m, b->gate);
    const long long before = amr_g_launches.load();
    AMR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    try {
        one();
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        throw;
    }
    AMR_CUDA(cudaStreamEndCapture(s, &gr_.g));
    const long long per_iter = amr_g_launches.load() - before;
    AMR_COUNT(-per_iter);
    AMR_CUDA(cudaGraphInstantiate(&gr_.x, gr_.g, 0));
    // every part alternates CG steps and refreshes, so it is done within 2 max_iters + 2 iterations
    const long long cap = 2LL * max_iters + 2;
    long long done_iters = 0;
    bool abort = false;
    for (;;) {
        for (int i = 0; i < kBaEvery; i++) {
            AMR_CUDA(cudaGraphLaunch(gr_.x, s));
            AMR_COUNT(per_iter);
        }
        done_iters += kBaEvery;
        k_ba_summary<<<1, 256, 0, s>>>(np, b->pamg, b->bsum);
        AMR_COUNT(1);
        AMR_CUDA(cudaMemcpyAsync(b->h_bsum, b->bsum, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        if (b->h_bsum[0] == 0) break;
        if (done_iters >= cap) { abort = true; break; }
    }
    k_ba_finish<<<gparts, 256, 0, s>>>(np, B, b->part_ptr, active, m->free_mask, x, b->pamg, b->stat, abort ? 1 : 0);
    AMR_COUNT(1);
    if (step) {
        k_ba_stamp<<<1, 1, 0, s>>>(step, 1);
        AMR_COUNT(1);
    }
    AMR_CUDA(cudaGetLastError());
}

}  // namespace

AmrSolveResult amr_batch_solve(amr_model *m, double *x, const double *b_, double *reac, const amr_solve_opts &o) {
    AmrBatch *b = m->batch;
    AmrSolveResult res{AMR_OK, 0, 0, 0.0, 0.0};
    if (o.method != AMR_SOLVER_MIXED && o.method != AMR_SOLVER_AMG)
        throw AmrError(AMR_EUNSUPPORTED, "batched solves use the mixed-precision solver, block-Jacobi or multigrid");
    AMR_CUDA(cudaEventRecord(m->ev0, m->stream));
    if (o.method == AMR_SOLVER_AMG) batch_solve_amg(m, x, b_, reac, o, nullptr, nullptr);
    else launch_pcg(m, pcg_args(m, x, b_, reac, o, nullptr), b->ctas_per_sm);
    AMR_CUDA(cudaEventRecord(m->ev1, m->stream));
    AMR_CUDA(cudaMemcpyAsync(b->h_stat.data(), b->stat, b->nparts * sizeof(PartStat), cudaMemcpyDeviceToHost,
                             m->stream));
    AMR_CUDA(cudaStreamSynchronize(m->stream));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    res.seconds = ms * 1e-3;
    for (const PartStat &s : b->h_stat) {
        res.iterations = std::max(res.iterations, s.iters);
        res.refinements = std::max(res.refinements, s.refreshes);
        res.rel_residual = std::max(res.rel_residual, s.rel_residual);
        if (s.status && !res.status) res.status = s.status;
    }
    return res;
}

// ---------------------------------------------------------------------------
// Batched mech_stage_solver!
// ---------------------------------------------------------------------------
namespace {

// sets the element kernels' per-part masks for the duration of a batched stage
struct MaskScope {
    amr_model *m;
    MaskScope(amr_model *m_, AmrBatch *b) : m(m_) {
        m->bp_elem_part = b->elem_part;
        m->bp_node_part = b->node_part;
        m->bp_active = b->active;
        m->bp_err = b->perr;
    }
    ~MaskScope() {
        m->bp_elem_part = nullptr;
        m->bp_node_part = nullptr;
        m->bp_active = nullptr;
        m->bp_err = nullptr;
    }
};

}  // namespace

int amr_batch_stage(amr_model *m, const double *Uex, const double *Fex, const amr_stage_params &prm, double *U,
                    double *F, amr_stage_stats *stats) {
    AmrBatch *b = m->batch;
    cudaStream_t s = m->stream;
    // predictor-corrector schemes (mech-solver.jl:280-288), as the whole-model driver runs them
    double p1 = 1.0, q11 = 1.0, a1 = 0.0, a2 = 0.0;
    switch (prm.scheme) {
    case AMR_SCHEME_FE: break;
    case AMR_SCHEME_ME: a1 = 0.5; a2 = 0.5; break;
    case AMR_SCHEME_BE: a1 = 0.0; a2 = 1.0; break;
    case AMR_SCHEME_RALSTON: p1 = 2.0 / 3.0; q11 = 2.0 / 3.0; a1 = 0.25; a2 = 0.75; break;
    default: throw AmrError(AMR_EINVAL, "unknown scheme");
    }
    const bool corrector = prm.scheme != AMR_SCHEME_FE;
    if (prm.maxits < 1 || prm.nincs < 1) throw AmrError(AMR_EINVAL, "bad stage parameters");
    if (prm.linear.method != AMR_SOLVER_MIXED && prm.linear.method != AMR_SOLVER_AMG)
        throw AmrError(AMR_EUNSUPPORTED, "batched stages use the mixed-precision solver, block-Jacobi or multigrid");
    // the multigrid solve runs its own graph with host checks: its Newton iterations run uncaptured
    const bool amg = prm.linear.method == AMR_SOLVER_AMG;
    const int64_t n = m->nnodes * m->B, np = b->nparts;
    std::vector<double *> v(10, nullptr);
    double *Ks = nullptr;  // the predictor's tangent, kept for the weighted corrector tangent
    struct Release {
        std::vector<double *> &v;
        double *&Ks;
        ~Release() {
            for (auto &x : v) amr_free(x);
            amr_free(Ks);
        }
    } release{v, Ks};
    for (auto &x : v) amr_alloc(&x, n);
    const size_t nK = (size_t)m->bstride * m->BB;
    if (corrector) amr_alloc(&Ks, nK);
    double *R = v[0], *dUa = v[1], *dUi = v[2], *Rc = v[3], *dFin = v[4], *dFex = v[5], *dUitr = v[6], *Rtr = v[7],
           *reac = v[8], *dUt = v[9];
    b->have_stage = false;
    cudaEvent_t t0 = m->ev0, t1 = m->ev1;
    AMR_CUDA(cudaEventRecord(t0, s));
    for (double *x : {U, F, R, dUa, dUi, Rc, dFin, dFex, dUitr, Rtr, reac, dUt})
        AMR_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
    // stage parameters (src/solver.jl:128-140 for nouts)
    int nincs = prm.nincs;
    const bool saveouts = prm.nouts > 0, autoinc = prm.autoinc != 0;
    if (saveouts && !autoinc) {
        if (prm.nouts > nincs) nincs = prm.nouts;
        if (nincs % prm.nouts != 0) nincs = nincs - (nincs % prm.nouts) + prm.nouts;
    }
    StageP sp;
    sp.tol = prm.tol; sp.rtol = prm.rtol; sp.rspan = prm.rspan; sp.dTmin = prm.dTmin; sp.dTmax = prm.dTmax;
    sp.dTcheck = saveouts ? 1.0 / prm.nouts : 1.0;
    sp.maxits = prm.maxits; sp.autoinc = autoinc ? 1 : 0;
    PartCtl c0{};
    c0.T = 0.0;
    c0.dT = 1.0 / nincs;
    if (autoinc) c0.dT = std::min({c0.dT, prm.dTmax, sp.dTcheck, prm.dT0});
    c0.Tcheck = sp.dTcheck;
    c0.phase = PH_START;
    std::fill(b->h_ctl.begin(), b->h_ctl.end(), c0);
    AMR_CUDA(cudaMemcpyAsync(b->ctl, b->h_ctl.data(), np * sizeof(PartCtl), cudaMemcpyHostToDevice, s));
    AMR_CUDA(cudaMemcpyAsync(m->stbk, m->st, (size_t)AMR_NST * m->nip_total * sizeof(double),
                             cudaMemcpyDeviceToDevice, s));
    // the element-force staging is read for every node: start it at zero
    {
        int64_t nfel = 0;
        AMR_CUDA(cudaMemcpyAsync(&nfel, m->fel_ptr + m->nelems, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        AMR_CUDA(cudaMemsetAsync(m->Fel, 0, nfel * sizeof(double), s));
    }
    // every stage mounts K once; a state-dependent K is mounted in every Newton iteration (inside the graph)
    m->K_valid = false;
    amr_stiffness(m);
    {
        int rc = amr_check_status(m);
        if (rc == AMR_ENEGJAC)
            throw AmrError(rc, "Negative Jacobian determinant in cell " + std::to_string(m->perm[m->h_status[1]] + 1));
        if (rc) throw AmrError(rc, "assembly failed");
    }
    m->K_valid = true;

    SlotArgs sa;
    sa.n = n; sa.B = m->B; sa.node_part = b->node_part; sa.c = b->ctl; sa.active = b->active; sa.fm = m->free_mask;
    sa.Uex = Uex; sa.Fex = Fex; sa.U = U; sa.F = F; sa.R = R; sa.Rc = Rc; sa.dUa = dUa; sa.dUi = dUi;
    sa.dUitr = dUitr; sa.Rtr = Rtr; sa.dUt = dUt; sa.dFin = dFin; sa.dFex = dFex;
    sa.p1 = p1; sa.q11 = q11; sa.corrector = corrector ? 1 : 0;
    PcgArgs pa = pcg_args(m, dUitr, Rtr, reac, prm.linear, b->active);
    pa.step = b->step;
    PcgArgs pc = pcg_args(m, dUi, Rtr, reac, prm.linear, b->active);  // the corrector's solve
    pc.step = b->step;
    const unsigned gs = nblk(n, 256), gp = nblk(np, 128), gi = nblk(m->nip_total, 256);
    const unsigned gn = (unsigned)std::min<int64_t>(np, (int64_t)device_sms() * 4);

    MaskScope mask(m, b);
    GraphScope gr;
    auto solve = [&](const PcgArgs &a) {
        if (amg) batch_solve_amg(m, a.x, a.b, a.reac, prm.linear, b->active, b->step);
        else launch_pcg(m, a, b->ctas_per_sm);
    };
    // one Newton iteration of every running part
    auto iteration = [&]() {
        AMR_CUDA(cudaMemsetAsync(&b->step->t0, 0xff, sizeof(unsigned long long), s));
        AMR_CUDA(cudaMemsetAsync(&b->step->t1, 0, sizeof(StepInfo) - sizeof(unsigned long long), s));
        k_ctl_begin<<<gp, 128, 0, s>>>(np, b->ctl, b->active, b->perr, sp);
        k_slot_begin<<<gs, 256, 0, s>>>(sa);
        AMR_COUNT(2);
        // the tangent at the current states (a corrector left the weighted one in K: mount it again)
        if (m->any_plastic || corrector) amr_stiffness(m);
        solve(pa);
        k_ctl_mid<<<gp, 128, 0, s>>>(np, b->ctl, b->stat, b->active);
        k_slot_mid<<<gs, 256, 0, s>>>(sa);
        AMR_COUNT(2);
        amr_update_elements(m, dUt, dFin);
        if (corrector) {
            // K = a1 K + a2 K2, K2 the tangent at the predictor's trial states (mech-solver.jl:341-348)
            k_ctl_corr<<<gp, 128, 0, s>>>(np, b->perr, b->active);
            AMR_COUNT(1);
            AMR_CUDA(cudaMemcpyAsync(Ks, m->K64, nK * sizeof(double), cudaMemcpyDeviceToDevice, s));
            if (m->any_plastic) amr_stiffness(m);  // a state-independent K2 equals K
            amr_combine_K(m, a1, Ks, a2);
            k_slot_corr<<<gs, 256, 0, s>>>(sa);
            AMR_COUNT(1);
            if (amg) amr_amg_invalidate(m);  // K is the weighted tangent now
            solve(pc);
            k_ctl_mid<<<gp, 128, 0, s>>>(np, b->ctl, b->stat, b->active);
            k_slot_mid2<<<gs, 256, 0, s>>>(sa);
            AMR_COUNT(2);
            amr_update_elements(m, dUt, dFin);
        }
        k_slot_post<<<gs, 256, 0, s>>>(sa);
        k_part_norms<<<gn, kPartThreads, 0, s>>>(np, m->B, b->part_ptr, b->active, R, dUi, dUa, b->ctl);
        k_ctl_end<<<gp, 128, 0, s>>>(np, b->ctl, b->perr, sp, b->step);
        k_slot_commit<<<gs, 256, 0, s>>>(sa);
        k_ip_commit<<<gi, 256, 0, s>>>(m->nip_total, b->ip_part, b->ctl, m->st, m->stbk);
        AMR_COUNT(5);
        AMR_CUDA(cudaGetLastError());
    };
    // capture it once; count its kernels per replay instead of at capture
    long long per_iter = 0;
    if (!amg) {
        const long long before = amr_g_launches.load();
        AMR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        try {
            iteration();
        } catch (...) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            throw;
        }
        AMR_CUDA(cudaStreamEndCapture(s, &gr.g));
        per_iter = amr_g_launches.load() - before;
        AMR_COUNT(-per_iter);
        AMR_CUDA(cudaGraphInstantiate(&gr.x, gr.g, 0));
    }

    double solve_s = 0.0;
    int steps = 0;
    const int max_steps = 1000000;
    for (;;) {
        if (amg) {
            iteration();
        } else {
            AMR_CUDA(cudaGraphLaunch(gr.x, s));
            AMR_COUNT(per_iter);
        }
        AMR_CUDA(cudaMemcpyAsync(b->h_step, b->step, sizeof(StepInfo), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        if (b->h_step->t1 > b->h_step->t0) solve_s += (double)(b->h_step->t1 - b->h_step->t0) * 1e-9;
        steps++;
        if (b->h_step->remaining == 0) break;
        if (steps >= max_steps) throw AmrError(AMR_ESTAGE, "batched stage did not finish");
    }
    AMR_CUDA(cudaEventRecord(t1, s));
    AMR_CUDA(cudaMemcpyAsync(b->h_ctl.data(), b->ctl, np * sizeof(PartCtl), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaEventSynchronize(t1));
    AMR_CUDA(cudaStreamSynchronize(s));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, t0, t1));
    // element kernels wrote their errors per part; leave the handle's own status clear
    {
        int32_t reset[2] = {0, INT32_MAX};
        amr_h2d(m, m->d_status, reset, sizeof reset);
    }
    // K holds the tangent of some part's last trial state, or a corrector's weighted tangent
    if (m->any_plastic || corrector) m->K_valid = false;
    b->stage_seconds = ms * 1e-3;
    b->stage_solve_seconds = solve_s;
    b->have_stage = true;
    amr_stage_stats st{};
    st.status = AMR_OK;
    st.T = 1.0;
    int64_t failed = -1;
    for (int64_t i = 0; i < np; i++) {
        const PartCtl &q = b->h_ctl[i];
        if (q.status && failed < 0) failed = i;
        st.increments = std::max(st.increments, q.increments);
        st.krylov_iterations += q.krylov;
        st.residue = std::max(st.residue, q.res);
        st.T = std::min(st.T, q.T);
    }
    st.iterations = steps;
    st.seconds = b->stage_seconds;
    st.solve_seconds = solve_s;
    int status = AMR_OK;
    if (failed >= 0) {
        status = AMR_ESTAGE;
        st.status = status;
        m->err = "part " + std::to_string(failed) + ": Solver did not converge.";
    }
    if (stats) *stats = st;
    return status;
}

void amr_batch_part_stats(const amr_model *m, int64_t nparts, amr_stage_stats *out) {
    const AmrBatch *b = m->batch;
    if (!b) throw AmrError(AMR_EINVAL, "no parts set");
    if (!b->have_stage) throw AmrError(AMR_EINVAL, "no batched stage has run");
    if (nparts != b->nparts) throw AmrError(AMR_EINVAL, "nparts does not match the parts set");
    for (int64_t i = 0; i < nparts; i++) {
        const PartCtl &q = b->h_ctl[i];
        amr_stage_stats &s = out[i];
        s.status = q.status;
        s.increments = q.increments;
        s.iterations = q.iterations;
        s.krylov_iterations = q.krylov;
        s.residue = q.res;
        s.T = q.T;
        s.seconds = b->stage_seconds;
        s.solve_seconds = b->stage_solve_seconds;
    }
}

// ---------------------------------------------------------------------------
// Autotuner
// ---------------------------------------------------------------------------
namespace {

double time_ms(amr_model *m, const std::function<void()> &f, int reps) {
    f();  // warm-up (and attribute set-up)
    AMR_CUDA(cudaEventRecord(m->ev0, m->stream));
    for (int r = 0; r < reps; r++) f();
    AMR_CUDA(cudaEventRecord(m->ev1, m->stream));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    return ms / reps;
}

int pairs_of(int nen) { return nen * (nen + 1) / 2; }

}  // namespace

void amr_autotune_model(amr_model *m, amr_tuning *out) {
    if (!m->dofs_set) throw AmrError(AMR_EINVAL, "amr_set_dofs must be called first");
    cudaStream_t s = m->stream;
    const size_t nst = (size_t)AMR_NST * m->nip_total;
    const int64_t n = m->nnodes * m->B;
    double *st_save = nullptr, *dU = nullptr, *dF = nullptr;
    struct Free {
        double *&a, *&b, *&c;
        ~Free() { amr_free(a); amr_free(b); amr_free(c); }
    } fr{st_save, dU, dF};
    amr_alloc(&st_save, nst);
    amr_alloc(&dU, n);
    amr_alloc(&dF, n);
    AMR_CUDA(cudaMemcpyAsync(st_save, m->st, nst * sizeof(double), cudaMemcpyDeviceToDevice, s));
    AMR_CUDA(cudaMemsetAsync(dU, 0, n * sizeof(double), s));
    const int saved_mode = m->assembly_mode;
    m->assembly_mode = AMR_ASSEMBLY_FAST;
    amr_tuning t{};
    t.ngroups = (int32_t)std::min<size_t>(m->groups.size(), AMR_MAX_TUNED_GROUPS);
    t.stiffness_seconds = 0.0;
    t.internal_seconds = 0.0;
    std::vector<AmrGroup> all = m->groups;
    try {
        for (size_t gi = 0; gi < m->groups.size(); gi++) {
            // time this group's kernels alone: the other groups are taken out of the list meanwhile
            AmrGroup g = all[gi];
            const int np = pairs_of(g.nen), ndim = amr::shape_ndim(g.shape);
            double best = 1e300;
            int best_epb = g.epb;
            for (int e : {1, 2, 3, 4, 6, 8}) {
                if (e > 1 && e * np > 512) continue;
                const size_t smem = sizeof(double) * (size_t)e * (g.nen * ndim + 3 * g.nip * g.nen * ndim + 2 * g.nip);
                if (smem > 200 * 1024) continue;  // the stiffness kernel's shared memory (launch_stiff)
                g.epb = e;
                m->groups.assign(1, g);
                const double ms = time_ms(m, [&] { amr_stiffness_elements(m); }, 3);
                if (ms < best) { best = ms; best_epb = e; }
            }
            g.epb = best_epb;
            t.stiffness_seconds += best * 1e-3;
            double besti = 1e300;
            int best_int = g.epb_int;
            for (int e : {1, 2, 4, 8, 16}) {
                const size_t smem = sizeof(double) * (size_t)e * (2 * g.nen * ndim + g.nip * g.nen * ndim);
                if (smem > 200 * 1024) continue;
                g.epb_int = e;
                m->groups.assign(1, g);
                const double ms = time_ms(m, [&] { amr_update_elements(m, dU, dF); }, 3);
                if (ms < besti) { besti = ms; best_int = e; }
            }
            g.epb_int = best_int;
            t.internal_seconds += besti * 1e-3;
            all[gi] = g;
            if (gi < AMR_MAX_TUNED_GROUPS) {
                t.shape[gi] = g.shape;
                t.stiffness_epb[gi] = g.epb;
                t.internal_epb[gi] = g.epb_int;
            }
        }
    } catch (...) {
        m->groups = all;
        m->assembly_mode = saved_mode;
        throw;
    }
    m->groups = all;
    m->assembly_mode = saved_mode;
    amr_check_status(m);  // a trial update with dU = 0 reports nothing the caller asked for
    AMR_CUDA(cudaMemcpyAsync(m->st, st_save, nst * sizeof(double), cudaMemcpyDeviceToDevice, s));
    // batched solve: resident CTAs per SM, on a capped run of the assembled K with a unit load
    if (m->batch && m->K_valid) {
        AmrBatch *b = m->batch;
        double *x = dU, *rhs = dF, *reac = nullptr;
        amr_alloc(&reac, n);
        struct FreeOne {
            double *&p;
            ~FreeOne() { amr_free(p); }
        } fo{reac};
        std::vector<double> ones(n, 1.0);
        AMR_CUDA(cudaMemcpyAsync(rhs, ones.data(), n * sizeof(double), cudaMemcpyHostToDevice, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        amr_solve_opts o;
        amr_default_solve_opts(&o);
        o.max_iters = 50;
        double best = 1e300;
        int best_k = b->ctas_per_sm;
        for (int k : {1, 2, 3, 4}) {
            const double ms = time_ms(m, [&] {
                AMR_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), s));
                launch_pcg(m, pcg_args(m, x, rhs, reac, o, nullptr), k);
            }, 2);
            if (ms < best) { best = ms; best_k = k; }
        }
        b->ctas_per_sm = best_k;
        AMR_CUDA(cudaStreamSynchronize(s));
    }
    t.batch_threads = kPartThreads;
    t.batch_ctas_per_sm = m->batch ? m->batch->ctas_per_sm : 0;
    if (out) *out = t;
}
