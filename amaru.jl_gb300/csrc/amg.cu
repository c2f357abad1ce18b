// Aggregation multigrid preconditioner for the FP32 PCG of solve_system!
// (src/solver.jl:5-79): an optional, stronger replacement for block-Jacobi.
//
// Levels.  Level 0 is the Dirichlet-masked node-block matrix K32 (B x B blocks).
// Each coarser level groups the nodes of the level below into aggregates
// (greedy, on the node graph, deterministic) and keeps, per aggregate, an
// orthonormal basis of the rigid-body modes restricted to it (3 translations +
// 3 rotations in 3-D, 2 + 1 in 2-D; zero at prescribed DOFs): the tentative
// prolongator T.  A coarse node is an aggregate with NM DOFs, and the coarse
// operator is the Galerkin product T' A T, gathered per coarse block from a
// contribution list fixed at set-up, in a fixed order (no atomics).  The last
// level (at most kDenseMax DOFs) is inverted densely.
//
// Smoothed aggregation (the default).  Each prolongator but the coarsest is
// P = (I - w D^-1 A) T, w = 4 / (3 lambda), and the coarse operator P' A P is
// formed on the device as P' (A P): A P per block of its pattern as a sum over
// the row's blocks in order, then each coarse block as a sum over the fine rows
// P reaches it from, in order.  The patterns of P, A P and P' A P and their
// position maps are built on the host with the aggregation.
//
// Cycle.  V-cycle with a degree-2 Chebyshev smoother on the block-Jacobi
// preconditioned operator (interval [lambda/30, 1.1 lambda], lambda estimated
// by power iteration after each assembly) before and after the coarse
// correction; all in FP32.  It is a fixed linear operator, so the outer CG
// stays a plain PCG, and the FP64 true-residual refreshes of the mixed solver
// still decide convergence.
//
// Set-up is split: the aggregation, the prolongator blocks and the coarse
// patterns depend only on the pattern, the coordinates and the DOF numbering
// (host, once); the coarse values, block inverses, lambdas and the dense
// inverse depend on K (device, after each assembly).
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>

#include "amr_internal.h"

namespace {

constexpr int kDenseMax = 2048;  // DOFs of the coarsest (dense) level at most
constexpr int kMaxLevels = 8;
constexpr int kNormCtas = 512;  // CTAs of the power-iteration norm

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// host set-up
// ---------------------------------------------------------------------------
struct HostLevel {
    int b = 0;                   // DOFs per node of this level
    int64_t n = 0;               // nodes
    std::vector<int64_t> rp;     // node-block pattern
    std::vector<int32_t> cj;
    std::vector<int64_t> diag;   // position of each node's diagonal block
    std::vector<double> nns;     // near-null space per node: n x b x NM (row-major per node)
};

// greedy aggregation: roots whose whole neighbourhood is free, then stragglers join a neighbour's
// aggregate, then the rest form aggregates with their free neighbours
int64_t aggregate(const HostLevel &h, std::vector<int32_t> &agg) {
    agg.assign(h.n, -1);
    int32_t na = 0;
    for (int64_t i = 0; i < h.n; i++) {
        bool free = true;
        for (int64_t k = h.rp[i]; k < h.rp[i + 1] && free; k++) free = agg[h.cj[k]] < 0;
        if (!free || agg[i] >= 0) continue;
        for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++) agg[h.cj[k]] = na;
        agg[i] = na++;
    }
    const std::vector<int32_t> roots = agg;  // phase 2 joins phase-1 aggregates only
    for (int64_t i = 0; i < h.n; i++) {
        if (agg[i] >= 0) continue;
        for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++)
            if (roots[h.cj[k]] >= 0) { agg[i] = roots[h.cj[k]]; break; }
    }
    for (int64_t i = 0; i < h.n; i++) {
        if (agg[i] >= 0) continue;
        agg[i] = na;
        for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++)
            if (agg[h.cj[k]] < 0) agg[h.cj[k]] = na;
        na++;
    }
    return na;
}

// symmetric eigen-decomposition of a small matrix by cyclic Jacobi rotations
void sym_eig(int n, double *A, double *V, double *w) {
    for (int i = 0; i < n * n; i++) V[i] = (i % (n + 1) == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; sweep++) {
        double off = 0.0;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) off += A[p * n + q] * A[p * n + q];
        if (off < 1e-30) break;
        for (int p = 0; p < n; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = A[p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double th = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; i++) w[i] = A[i * n + i];
}

// f(a, e) on contiguous ranges of [0, n), one per thread (per-thread work arrays live in f)
template <class F>
void parallel_ranges(int64_t n, F f) {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 4096) nt = 1;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++) th.emplace_back([&, t] { f(n * t / nt, n * (t + 1) / nt); });
    for (auto &x : th) x.join();
}

template <class F>
void parallel_for(int64_t n, F f) {
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < 4096) nt = 1;
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            const int64_t a = n * t / nt, e = n * (t + 1) / nt;
            for (int64_t i = a; i < e; i++) f(i);
        });
    for (auto &x : th) x.join();
}

// Patterns of the smoothed prolongator P = (I - w D^-1 A) T of one level (T: node i -> aggregate agg[i]),
// of A P and of the coarse operator P' A P, with the maps their device builds read.
struct SaPattern {
    std::vector<int64_t> prp, pkp, qrp, ptp, crp;
    std::vector<int32_t> pcj, prow, pkk, qcj, qrow, pti, pts, ccj, crow;
};

// rows [0, n): out[r] = sorted distinct values that cand(r, push) pushes; two passes (count, fill)
template <class C>
void distinct_rows(int64_t n, int64_t nvals, C cand, std::vector<int64_t> &ptr, std::vector<int32_t> &col) {
    ptr.assign(n + 1, 0);
    parallel_ranges(n, [&](int64_t a, int64_t e) {
        std::vector<int64_t> mark(nvals, -1);
        for (int64_t r = a; r < e; r++) {
            int64_t cnt = 0;
            cand(r, [&](int32_t v) {
                if (mark[v] != r) { mark[v] = r; cnt++; }
            });
            ptr[r + 1] = cnt;
        }
    });
    for (int64_t r = 0; r < n; r++) ptr[r + 1] += ptr[r];
    col.resize(ptr[n]);
    parallel_ranges(n, [&](int64_t a, int64_t e) {
        std::vector<int64_t> mark(nvals, -1);
        for (int64_t r = a; r < e; r++) {
            int32_t *o = col.data() + ptr[r];
            int64_t cnt = 0;
            cand(r, [&](int32_t v) {
                if (mark[v] != r) { mark[v] = r; o[cnt++] = v; }
            });
            std::sort(o, o + cnt);
        }
    });
}

void sa_pattern(const HostLevel &h, const std::vector<int32_t> &agg, int64_t na, SaPattern &S) {
    const int64_t n = h.n;
    // P: row i reaches the aggregates of its neighbours
    distinct_rows(n, na, [&](int64_t i, auto push) {
        for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++) push(agg[h.cj[k]]);
    }, S.prp, S.pcj);
    const int64_t np = S.prp[n];
    S.prow.resize(np);
    parallel_for(n, [&](int64_t i) {
        for (int64_t t = S.prp[i]; t < S.prp[i + 1]; t++) S.prow[t] = (int32_t)i;
    });
    // each P block's blocks of A: the row's blocks whose column lies in that aggregate, in order
    S.pkp.assign(np + 1, 0);
    S.pkk.resize(h.rp[n]);
    parallel_ranges(n, [&](int64_t a, int64_t e) {
        for (int64_t i = a; i < e; i++) {
            int64_t o = h.rp[i];
            for (int64_t s = S.prp[i]; s < S.prp[i + 1]; s++) {
                S.pkp[s] = o;
                for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++)
                    if (agg[h.cj[k]] == S.pcj[s]) S.pkk[o++] = (int32_t)k;
            }
        }
    });
    S.pkp[np] = h.rp[n];
    // A P: row i reaches the aggregates of its neighbours' P rows
    distinct_rows(n, na, [&](int64_t i, auto push) {
        for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++) {
            const int32_t j = h.cj[k];
            for (int64_t t = S.prp[j]; t < S.prp[j + 1]; t++) push(S.pcj[t]);
        }
    }, S.qrp, S.qcj);
    S.qrow.resize(S.qrp[n]);
    parallel_for(n, [&](int64_t i) {
        for (int64_t q = S.qrp[i]; q < S.qrp[i + 1]; q++) S.qrow[q] = (int32_t)i;
    });
    // P by columns, rows ascending
    S.ptp.assign(na + 1, 0);
    for (int64_t s = 0; s < np; s++) S.ptp[S.pcj[s] + 1]++;
    for (int64_t c = 0; c < na; c++) S.ptp[c + 1] += S.ptp[c];
    S.pti.resize(np);
    S.pts.resize(np);
    {
        std::vector<int64_t> fill(S.ptp.begin(), S.ptp.end() - 1);
        for (int64_t i = 0; i < n; i++)
            for (int64_t s = S.prp[i]; s < S.prp[i + 1]; s++) {
                const int64_t o = fill[S.pcj[s]]++;
                S.pti[o] = (int32_t)i;
                S.pts[o] = (int32_t)s;
            }
    }
    // P' A P: coarse row I reaches the columns of the A P rows of the fine rows P reaches I from
    distinct_rows(na, na, [&](int64_t I, auto push) {
        push((int32_t)I);  // every coarse row has its diagonal block, even an aggregate of nodes without blocks
        for (int64_t e = S.ptp[I]; e < S.ptp[I + 1]; e++) {
            const int32_t i = S.pti[e];
            for (int64_t q = S.qrp[i]; q < S.qrp[i + 1]; q++) push(S.qcj[q]);
        }
    }, S.crp, S.ccj);
    S.crow.resize(S.crp[na]);
    for (int64_t I = 0; I < na; I++)
        for (int64_t c = S.crp[I]; c < S.crp[I + 1]; c++) S.crow[c] = (int32_t)I;
    if (S.crp[na] >= ((int64_t)1 << 31) || S.qrp[n] >= ((int64_t)1 << 31) || np >= ((int64_t)1 << 31) ||
        h.rp[n] >= ((int64_t)1 << 31))
        throw AmrError(AMR_EUNSUPPORTED, "the smoothed multigrid's patterns exceed 32-bit indices");
}

}  // namespace

// Values of one level in one precision: the FP32 cycle preconditions the mixed solver; the FP64 cycle,
// built on the same structure, preconditions the all-FP64 comparator.
template <class V>
struct AmgVals {
    V *A = nullptr;     // this level's matrix (levels >= 1): BSR, b x b blocks, SoA values [b*b][nbs]
    V *Dinv = nullptr;  // n x b*b block-Jacobi inverses (level 0: the solver's own)
    V *T = nullptr;     // n x b x NM prolongator blocks to the next level
    V *P = nullptr;     // smoothed prolongator: np blocks of b x NM (row-major), AoS
    V *Q = nullptr;     // A P: nq blocks of b x NM, AoS (work of the coarse operator's build)
    // the FP32 cycle's smoothed prolongator in FP16 (P holds the same rounded values, so the coarse operator
    // is the Galerkin product of the prolongator the cycle applies): by rows (prolongation) and by columns
    // in the order of ptp/pti (restriction), np blocks of b x NM each
    __half *P16 = nullptr, *P16T = nullptr;
    V *x = nullptr, *bv = nullptr, *r = nullptr, *d = nullptr;  // vectors of this level (n*b)
    double lam = 1.0;
};

struct AmgLevel {
    int b = 0;
    int64_t n = 0;
    int64_t nblocks = 0, nbs = 0;
    int64_t *rp = nullptr;
    int32_t *cj = nullptr;
    int64_t *diag = nullptr;
    // to the next coarser level
    int64_t naggs = 0;
    int32_t *agg = nullptr;   // node -> aggregate
    int64_t *aptr = nullptr;  // aggregate -> its nodes
    int32_t *anodes = nullptr;
    int64_t *cptr = nullptr;  // coarse block -> contributions (fine block k, fine row i)
    int32_t *ck = nullptr, *ci = nullptr;
    uint8_t *null_dof = nullptr;  // coarse DOFs with no mode (aggregate of prescribed DOFs): identity
    std::vector<double> hT;       // the prolongator blocks on the host (uploaded in FP64 on first use)
    // smoothed prolongator P (block rows = this level's nodes, block columns = aggregates): its pattern,
    // each P block's contributing blocks of A (pkk[pkp[s]..pkp[s+1]], ascending, a permutation of the
    // row's blocks), P by columns (aggregate -> (row, P block), rows ascending), the pattern of A P (with
    // each block's row) and the row of each coarse block
    bool smooth = false;
    int64_t np = 0, nq = 0;
    int p_steps = 0;  // halvings of a lower-bound search in the longest row of P
    int64_t *prp = nullptr, *pkp = nullptr, *qrp = nullptr, *ptp = nullptr;
    int32_t *pcj = nullptr, *prow = nullptr, *pkk = nullptr, *qcj = nullptr, *qrow = nullptr, *pti = nullptr,
            *pts = nullptr, *crow = nullptr;
    AmgVals<float> f32;
    AmgVals<double> f64;
};

struct AmrAmg {
    int NM = 6;
    std::vector<AmgLevel> L;
    int64_t nc = 0;             // DOFs of the dense coarsest level
    double *Cd = nullptr;       // nc x 2nc FP64 work (Gauss-Jordan)
    cudaGraphExec_t gj_exec = nullptr;  // the Gauss-Jordan steps, captured once
    float *Cinv = nullptr;      // nc x nc inverse, FP32 cycle
    double *Cinv64 = nullptr;   // nc x nc inverse, FP64 cycle
    double *scratch = nullptr;  // norms: [0] result, [1] the power iteration's estimate, [8..] per-CTA partials
    unsigned int *ticket = nullptr;
    int32_t *pstop = nullptr;   // the power iteration met a zero or non-finite norm: its remaining steps return
    int64_t dofs_version = -1;
    bool numeric_valid = false, numeric64_valid = false;
    // The FP32 cycle's fine-level residual reads an FP16 copy of the symmetrically scaled matrix
    // A16 = S K32 S, S = diag(s_n) per node with s_n = 1/rs_n a power of two and rs_n^2 >= the node's
    // largest diagonal entry, so |A16| <= 1 for an SPD K and the copy is exactly symmetric.  The residual
    // r = b - K x is then rs_i sum_j A16_ij xt_j with xt = x rs kept, one 16-byte gather per block, by the
    // smoother and the prolongation of that level.
    // fine-level row gate of the FP32 cycle (nnodes bytes, null: every row): rows with 0 are skipped by the
    // fine level's smoothing, residual, restriction and prolongation (their values go stale); set by the
    // batched solve to the rows of its running parts, whose V-cycle is block diagonal over the parts
    const uint8_t *gate = nullptr;
    // the solve's stop flag (null: none): set while a PCG iteration graph is replayed, so the V-cycles of the
    // iterations left in a chunk after the recursive residual has triggered a refresh return at once
    const int32_t *halt = nullptr;
    __half *A16 = nullptr;      // SoA [B*B][bstride]
    float *rs = nullptr;        // nnodes: 1 / s_n
    float *xt = nullptr;        // nnodes x 4 (3-D) or x 2 (2-D): x rs
};

namespace {
template <class V>
AmgVals<V> &vals(AmgLevel &L);
template <>
AmgVals<float> &vals<float>(AmgLevel &L) { return L.f32; }
template <>
AmgVals<double> &vals<double>(AmgLevel &L) { return L.f64; }

template <class V>
void free_vals(AmgVals<V> &v, bool owns_matrix) {
    if (owns_matrix) {
        amr_free(v.A);
        amr_free(v.Dinv);
    }
    amr_free(v.T); amr_free(v.P); amr_free(v.Q); amr_free(v.P16); amr_free(v.P16T);
    amr_free(v.x); amr_free(v.bv); amr_free(v.r); amr_free(v.d);
}
}  // namespace

void amr_amg_free(amr_model *m) {
    AmrAmg *g = m->amg;
    if (!g) return;
    for (size_t l = 0; l < g->L.size(); l++) {
        AmgLevel &v = g->L[l];
        if (l > 0) {
            amr_free(v.rp); amr_free(v.cj);
        }
        free_vals(v.f32, l > 0);
        free_vals(v.f64, l > 0);
        amr_free(v.diag); amr_free(v.agg); amr_free(v.aptr); amr_free(v.anodes);
        amr_free(v.cptr); amr_free(v.ck); amr_free(v.ci); amr_free(v.null_dof);
        amr_free(v.prp); amr_free(v.pkp); amr_free(v.qrp); amr_free(v.ptp); amr_free(v.pcj); amr_free(v.prow);
        amr_free(v.pkk);
        amr_free(v.qcj); amr_free(v.qrow); amr_free(v.pti); amr_free(v.pts); amr_free(v.crow);
    }
    if (g->gj_exec) cudaGraphExecDestroy(g->gj_exec);
    amr_free(g->Cd); amr_free(g->Cinv); amr_free(g->Cinv64); amr_free(g->scratch); amr_free(g->ticket); amr_free(g->pstop);
    amr_free(g->A16); amr_free(g->rs); amr_free(g->xt);
    delete g;
    m->amg = nullptr;
}

// Host part of the set-up: levels, aggregates, prolongator blocks, coarse patterns.
static void amg_build_structure(amr_model *m) {
    amr_amg_free(m);
    AmrAmg *g = new AmrAmg();
    m->amg = g;
    const int B = m->B, NM = B == 3 ? 6 : 3;
    g->NM = NM;
    // level 0 on the host: the pattern, the masked rigid-body modes at each node
    std::vector<HostLevel> H(1);
    H[0].b = B;
    H[0].n = m->nnodes;
    H[0].rp = m->h_brow_ptr;
    H[0].cj = m->h_bcol;
    H[0].nns.assign((size_t)m->nnodes * B * NM, 0.0);
    for (int64_t i = 0; i < m->nnodes; i++) {
        const double x = m->h_coords[3 * i], y = m->h_coords[3 * i + 1], z = m->h_coords[3 * i + 2];
        double *N = &H[0].nns[(size_t)i * B * NM];
        for (int c = 0; c < B; c++) {
            const int64_t e = m->h_eq_id[3 * i + c];
            if (!(e >= 0 && e < m->nu)) continue;  // prescribed or absent: the masked system has no mode there
            N[c * NM + c] = 1.0;
            if (B == 3) {  // rotations about x, y, z: (0,-z,y), (z,0,-x), (-y,x,0)
                if (c == 0) { N[c * NM + 4] = z; N[c * NM + 5] = -y; }
                if (c == 1) { N[c * NM + 3] = -z; N[c * NM + 5] = x; }
                if (c == 2) { N[c * NM + 3] = y; N[c * NM + 4] = -x; }
            } else {
                if (c == 0) N[c * NM + 2] = -y;
                if (c == 1) N[c * NM + 2] = x;
            }
        }
    }
    for (int l = 0;; l++) {
        HostLevel &h = H[l];
        h.diag.assign(h.n, -1);
        for (int64_t i = 0; i < h.n; i++)
            for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++)
                if (h.cj[k] == i) h.diag[i] = k;
        AmgLevel lv;
        lv.b = h.b;
        lv.n = h.n;
        lv.nblocks = h.rp[h.n];
        lv.nbs = (lv.nblocks + 3) / 4 * 4 + 4;
        // the fine level is always aggregated; a coarse level small enough is the dense one
        const bool last = l > 0 && ((int64_t)h.n * h.b <= kDenseMax || l + 1 >= kMaxLevels);
        if (l > 0) {
            amr_alloc(&lv.rp, h.n + 1);
            amr_alloc(&lv.cj, std::max<int64_t>(lv.nblocks, 1));
            amr_h2d(m, lv.rp, h.rp.data(), (h.n + 1) * sizeof(int64_t));
            amr_h2d(m, lv.cj, h.cj.data(), lv.nblocks * sizeof(int32_t));
            amr_alloc(&lv.f32.A, (size_t)lv.nbs * h.b * h.b);
            amr_alloc(&lv.f32.Dinv, (size_t)h.n * h.b * h.b);
        } else {
            lv.rp = m->brow_ptr;
            lv.cj = m->bcol;
            lv.nbs = m->bstride;
        }
        amr_alloc(&lv.diag, h.n);
        amr_h2d(m, lv.diag, h.diag.data(), h.n * sizeof(int64_t));
        const int64_t nv = h.n * h.b;
        amr_alloc(&lv.f32.x, nv); amr_alloc(&lv.f32.bv, nv); amr_alloc(&lv.f32.r, nv); amr_alloc(&lv.f32.d, nv);
        if (last) {
            g->nc = nv;
            g->L.push_back(lv);
            break;
        }
        // aggregates and their node lists
        std::vector<int32_t> agg;
        const int64_t na = aggregate(h, agg);
        std::vector<int64_t> aptr(na + 1, 0);
        for (int64_t i = 0; i < h.n; i++) aptr[agg[i] + 1]++;
        for (int64_t a = 0; a < na; a++) aptr[a + 1] += aptr[a];
        std::vector<int32_t> anodes(h.n);
        {
            std::vector<int64_t> fill(aptr.begin(), aptr.end() - 1);
            for (int64_t i = 0; i < h.n; i++) anodes[fill[agg[i]]++] = (int32_t)i;
        }
        // per aggregate: orthonormal basis of the near-null space (T) and its coordinates (next level's modes)
        std::vector<double> T((size_t)h.n * h.b * NM, 0.0);
        HostLevel hc;
        hc.b = NM;
        hc.n = na;
        hc.nns.assign((size_t)na * NM * NM, 0.0);
        std::vector<uint8_t> nulld((size_t)na * NM, 0);
        parallel_for(na, [&](int64_t a) {
            const int64_t cnt = aptr[a + 1] - aptr[a];
            const int rows = (int)(cnt * h.b);
            std::vector<double> Bm((size_t)rows * NM);
            for (int64_t q = 0; q < cnt; q++) {
                const int64_t i = anodes[aptr[a] + q];
                for (int c = 0; c < h.b; c++)
                    for (int k = 0; k < NM; k++) Bm[(q * h.b + c) * NM + k] = h.nns[((size_t)i * h.b + c) * NM + k];
            }
            double G[36], V[36], w[6];
            for (int p = 0; p < NM; p++)
                for (int q = 0; q < NM; q++) {
                    double s = 0.0;
                    for (int r = 0; r < rows; r++) s += Bm[(size_t)r * NM + p] * Bm[(size_t)r * NM + q];
                    G[p * NM + q] = s;
                }
            sym_eig(NM, G, V, w);
            double wmax = 0.0;
            for (int k = 0; k < NM; k++) wmax = std::max(wmax, w[k]);
            double sc[6];
            for (int k = 0; k < NM; k++) {
                const bool keep = wmax > 0.0 && w[k] > 1e-8 * wmax;
                sc[k] = keep ? 1.0 / std::sqrt(w[k]) : 0.0;
                if (!keep) nulld[a * NM + k] = 1;
            }
            // T = Bm V diag(sc); next-level modes R = diag(sqrt(w)) V' (rows of kept directions)
            for (int64_t q = 0; q < cnt; q++) {
                const int64_t i = anodes[aptr[a] + q];
                for (int c = 0; c < h.b; c++)
                    for (int k = 0; k < NM; k++) {
                        double s = 0.0;
                        for (int p = 0; p < NM; p++) s += Bm[(q * h.b + c) * NM + p] * V[p * NM + k];
                        T[((size_t)i * h.b + c) * NM + k] = s * sc[k];
                    }
            }
            for (int k = 0; k < NM; k++)
                for (int p = 0; p < NM; p++)
                    hc.nns[((size_t)a * NM + k) * NM + p] = sc[k] > 0.0 ? std::sqrt(w[k]) * V[p * NM + k] : 0.0;
        });
        if (m->amg_smooth) {
            SaPattern S;
            sa_pattern(h, agg, na, S);
            lv.smooth = true;
            lv.np = S.prp[h.n];
            lv.nq = S.qrp[h.n];
            {
                int64_t mp = 0;
                for (int64_t i = 0; i < h.n; i++) mp = std::max(mp, S.prp[i + 1] - S.prp[i]);
                int b = 0;
                for (int64_t v = mp; v > 0; v >>= 1) b++;
                lv.p_steps = b;
            }
            auto up64 = [&](int64_t *&d, const std::vector<int64_t> &v) {
                amr_alloc(&d, std::max<size_t>(v.size(), 1));
                amr_h2d(m, d, v.data(), v.size() * sizeof(int64_t));
            };
            auto up32 = [&](int32_t *&d, const std::vector<int32_t> &v) {
                amr_alloc(&d, std::max<size_t>(v.size(), 1));
                amr_h2d(m, d, v.data(), v.size() * sizeof(int32_t));
            };
            up64(lv.prp, S.prp); up64(lv.pkp, S.pkp); up64(lv.qrp, S.qrp); up64(lv.ptp, S.ptp);
            up32(lv.pcj, S.pcj); up32(lv.prow, S.prow); up32(lv.pkk, S.pkk); up32(lv.qcj, S.qcj); up32(lv.qrow, S.qrow);
            up32(lv.pti, S.pti); up32(lv.pts, S.pts); up32(lv.crow, S.crow);
            amr_alloc(&lv.f32.P, (size_t)std::max<int64_t>(lv.np, 1) * h.b * NM);
            amr_alloc(&lv.f32.P16, (size_t)std::max<int64_t>(lv.np, 1) * h.b * NM);
            amr_alloc(&lv.f32.P16T, (size_t)std::max<int64_t>(lv.np, 1) * h.b * NM);
            amr_alloc(&lv.f32.Q, (size_t)std::max<int64_t>(lv.nq, 1) * h.b * NM);
            hc.rp = std::move(S.crp);
            hc.cj = std::move(S.ccj);
        } else {
            // coarse pattern and contribution lists, coarse row by coarse row
            std::vector<std::vector<int32_t>> ccols(na);
            std::vector<std::vector<int64_t>> ccnt(na);
            std::vector<std::vector<int32_t>> ck(na), ci(na);
            parallel_for(na, [&](int64_t a) {
                std::vector<std::tuple<int32_t, int32_t, int32_t>> e;  // (coarse column, fine block, fine row)
                // every coarse row has its diagonal block, even an aggregate of nodes without blocks
                e.emplace_back((int32_t)a, -1, -1);
                for (int64_t q = aptr[a]; q < aptr[a + 1]; q++) {
                    const int32_t i = anodes[q];
                    for (int64_t k = h.rp[i]; k < h.rp[i + 1]; k++) e.emplace_back(agg[h.cj[k]], (int32_t)k, i);
                }
                std::stable_sort(e.begin(), e.end(),
                                 [](const auto &u, const auto &v) { return std::get<0>(u) < std::get<0>(v); });
                for (size_t s = 0; s < e.size(); s++) {
                    if (s == 0 || std::get<0>(e[s]) != std::get<0>(e[s - 1])) {
                        ccols[a].push_back(std::get<0>(e[s]));
                        ccnt[a].push_back(0);
                    }
                    if (std::get<1>(e[s]) < 0) continue;  // the diagonal sentinel contributes nothing
                    ccnt[a].back()++;
                    ck[a].push_back(std::get<1>(e[s]));
                    ci[a].push_back(std::get<2>(e[s]));
                }
            });
            hc.rp.assign(na + 1, 0);
            for (int64_t a = 0; a < na; a++) hc.rp[a + 1] = hc.rp[a] + (int64_t)ccols[a].size();
            hc.cj.resize(hc.rp[na]);
            std::vector<int64_t> cptr(hc.rp[na] + 1, 0);
            std::vector<int32_t> cks, cis;
            cks.reserve(lv.nblocks);
            cis.reserve(lv.nblocks);
            for (int64_t a = 0; a < na; a++) {
                for (size_t s = 0; s < ccols[a].size(); s++) {
                    const int64_t cb = hc.rp[a] + (int64_t)s;
                    hc.cj[cb] = ccols[a][s];
                    cptr[cb + 1] = cptr[cb] + ccnt[a][s];
                }
                cks.insert(cks.end(), ck[a].begin(), ck[a].end());
                cis.insert(cis.end(), ci[a].begin(), ci[a].end());
            }
            amr_alloc(&lv.cptr, cptr.size());
            amr_alloc(&lv.ck, std::max<size_t>(cks.size(), 1));
            amr_alloc(&lv.ci, std::max<size_t>(cis.size(), 1));
            amr_h2d(m, lv.cptr, cptr.data(), cptr.size() * sizeof(int64_t));
            amr_h2d(m, lv.ck, cks.data(), cks.size() * sizeof(int32_t));
            amr_h2d(m, lv.ci, cis.data(), cis.size() * sizeof(int32_t));
        }
        lv.naggs = na;
        amr_alloc(&lv.agg, h.n);
        amr_alloc(&lv.f32.T, T.size());
        amr_alloc(&lv.aptr, na + 1);
        amr_alloc(&lv.anodes, h.n);
        amr_alloc(&lv.null_dof, nulld.size());
        amr_h2d(m, lv.agg, agg.data(), h.n * sizeof(int32_t));
        {
            const std::vector<float> T32(T.begin(), T.end());
            amr_h2d(m, lv.f32.T, T32.data(), T32.size() * sizeof(float));
        }
        lv.hT = std::move(T);
        amr_h2d(m, lv.aptr, aptr.data(), aptr.size() * sizeof(int64_t));
        amr_h2d(m, lv.anodes, anodes.data(), h.n * sizeof(int32_t));
        amr_h2d(m, lv.null_dof, nulld.data(), nulld.size());
        g->L.push_back(lv);
        H.push_back(std::move(hc));
    }
    if (g->nc > 32768) throw AmrError(AMR_EUNSUPPORTED, "the multigrid's coarsest level is too large to invert densely");
    amr_alloc(&g->Cd, (size_t)g->nc * 2 * g->nc);  // [A | I] for Gauss-Jordan
    amr_alloc(&g->Cinv, (size_t)g->nc * g->nc);
    amr_alloc(&g->scratch, 8 + kNormCtas);
    amr_alloc(&g->ticket, 1);
    amr_alloc(&g->pstop, 1);
    amr_alloc(&g->A16, (size_t)m->bstride * B * B);
    amr_alloc(&g->rs, m->nnodes);
    amr_alloc(&g->xt, (size_t)m->nnodes * (B == 3 ? 4 : 2));
    AMR_CUDA(cudaMemsetAsync(g->xt, 0, (size_t)m->nnodes * (B == 3 ? 4 : 2) * sizeof(float), m->stream));
    AMR_CUDA(cudaMemsetAsync(g->ticket, 0, sizeof(unsigned int), m->stream));
    g->numeric_valid = false;
}

// ---------------------------------------------------------------------------
// device kernels, templated on the value type V of the level's matrix and vectors (float for the
// mixed solver's cycle, double for the all-FP64 comparator's)
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }

// coarse block (warp) = sum over its contributions (fine block k of row i, column j) of T_i' A_k T_j
template <int BF, int NM, class V>
__global__ void k_galerkin(int64_t ncb, const int64_t *cptr, const int32_t *ck, const int32_t *ci,
                           const int32_t *cjf, const V *Af, int64_t nbsf, const V *T, V *Ac, int64_t nbsc) {
    const int lane = threadIdx.x & 31;
    const int64_t cb = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (cb >= ncb) return;
    V acc[NM * NM];
#pragma unroll
    for (int q = 0; q < NM * NM; q++) acc[q] = V(0);
    for (int64_t e = cptr[cb] + lane; e < cptr[cb + 1]; e += 32) {
        const int64_t k = ck[e];
        const int32_t i = ci[e], j = cjf[k];
        V M[BF * NM];  // A_k T_j
#pragma unroll
        for (int c = 0; c < BF; c++)
#pragma unroll
            for (int m = 0; m < NM; m++) {
                V s = V(0);
#pragma unroll
                for (int d = 0; d < BF; d++) s = vfma(Af[(int64_t)(c * BF + d) * nbsf + k], T[((int64_t)j * BF + d) * NM + m], s);
                M[c * NM + m] = s;
            }
#pragma unroll
        for (int p = 0; p < NM; p++)
#pragma unroll
            for (int m = 0; m < NM; m++) {
                V s = acc[p * NM + m];
#pragma unroll
                for (int c = 0; c < BF; c++) s = vfma(T[((int64_t)i * BF + c) * NM + p], M[c * NM + m], s);
                acc[p * NM + m] = s;
            }
    }
#pragma unroll
    for (int q = 0; q < NM * NM; q++) {
        V v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) Ac[(int64_t)q * nbsc + cb] = v;
    }
}

// coarse DOFs without a mode get an identity equation
// smoothed prolongator, thread per block s of P (row i = prow[s]): P_s = [pcj[s] == agg(i)] T_i - w Dinv_i
// sum_k A_k T_cj[k] over the P block's blocks k of A in order; rows of prescribed DOFs (mask 0) are zero
template <int BF, int NM, class V>
__global__ void k_sa_prolongator(int64_t np, const int32_t *prow, const int32_t *pcj, const int64_t *pkp,
                                 const int32_t *pkk, const int32_t *cjf, const V *Af, int64_t nbsf, const V *T,
                                 const V *Dinv, const int32_t *agg, V w, const uint8_t *mask, V *P) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= np) return;
    const int64_t i = prow[s];
    const int32_t ai = agg[i];
    V Di[BF * BF];
#pragma unroll
    for (int q = 0; q < BF * BF; q++) Di[q] = Dinv[i * BF * BF + q];
    bool fr[BF];
#pragma unroll
    for (int c = 0; c < BF; c++) fr[c] = mask ? mask[i * BF + c] != 0 : true;
    {
        V M[BF * NM];  // sum of A_k T_j
#pragma unroll
        for (int q = 0; q < BF * NM; q++) M[q] = V(0);
        for (int64_t e = pkp[s]; e < pkp[s + 1]; e++) {
            const int64_t k = pkk[e];
            const int64_t j = cjf[k];
            V a[BF * BF];
#pragma unroll
            for (int q = 0; q < BF * BF; q++) a[q] = Af[(int64_t)q * nbsf + k];
#pragma unroll
            for (int d = 0; d < BF; d++)
#pragma unroll
                for (int mm = 0; mm < NM; mm++) {
                    const V t = T[(j * BF + d) * NM + mm];
#pragma unroll
                    for (int c = 0; c < BF; c++) M[c * NM + mm] = vfma(a[c * BF + d], t, M[c * NM + mm]);
                }
        }
        const bool own = pcj[s] == ai;
#pragma unroll
        for (int c = 0; c < BF; c++)
#pragma unroll
            for (int mm = 0; mm < NM; mm++) {
                V v = V(0);
#pragma unroll
                for (int d = 0; d < BF; d++) v = vfma(Di[c * BF + d], M[d * NM + mm], v);
                const V p = (own ? T[(i * BF + c) * NM + mm] : V(0)) - w * v;
                P[s * BF * NM + c * NM + mm] = fr[c] ? p : V(0);
            }
    }
}

// Lower bound of J in the sorted columns c[base, base + len) in `steps` halvings (steps >= the bit length of
// the longest row), for U independent rows at once so that their dependent loads overlap: on return
// base[u] is the first position whose column is >= J[u].
template <int U>
__device__ __forceinline__ void lower_bounds(const int32_t *c, int64_t *base, int64_t *len, const int32_t *J,
                                             int steps) {
    for (int st = 0; st < steps; st++)
#pragma unroll
        for (int u = 0; u < U; u++)
            if (len[u] > 0) {
                const int64_t half = len[u] >> 1;
                if (c[base[u] + half] < J[u]) {
                    base[u] += half + 1;
                    len[u] -= half + 1;
                } else {
                    len[u] = half;
                }
            }
}

// A P, thread per block q of its pattern (row i, aggregate J): sum over the row's blocks k of A in order of
// A_k P_t, t the block of P row cj[k] in column J (if any).  Four blocks k at a time: their P rows are searched
// together, then the products are added in order of k.
template <int BF, int NM, class V>
__global__ void __launch_bounds__(128) k_sa_ap(int64_t nq, const int32_t *qrow, const int32_t *qcj,
                                                const int64_t *rpf, const int32_t *cjf, const V *Af, int64_t nbsf,
                                                const int64_t *prp, const int32_t *pcj, const V *P, V *Q,
                                                int steps) {
    constexpr int U = 4;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int64_t i = qrow[q];
    const int32_t J = qcj[q];
    const int32_t Ju[U] = {J, J, J, J};
    V acc[BF * NM];
#pragma unroll
    for (int u = 0; u < BF * NM; u++) acc[u] = V(0);
    const int64_t k1 = rpf[i + 1];
    for (int64_t kb = rpf[i]; kb < k1; kb += U) {
        int64_t base[U], len[U], end[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (kb + u < k1) {
                const int64_t j = cjf[kb + u];
                base[u] = prp[j];
                end[u] = prp[j + 1];
            } else {
                base[u] = end[u] = 0;
            }
            len[u] = end[u] - base[u];
        }
        lower_bounds<U>(pcj, base, len, Ju, steps);
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (base[u] >= end[u] || pcj[base[u]] != J) continue;
            const int64_t k = kb + u;
            const V *pt = P + base[u] * BF * NM;
#pragma unroll
            for (int d = 0; d < BF; d++) {
                V a[BF];
#pragma unroll
                for (int c = 0; c < BF; c++) a[c] = Af[(int64_t)(c * BF + d) * nbsf + k];
#pragma unroll
                for (int mm = 0; mm < NM; mm++) {
                    const V pv = pt[d * NM + mm];
#pragma unroll
                    for (int c = 0; c < BF; c++) acc[c * NM + mm] = vfma(a[c], pv, acc[c * NM + mm]);
                }
            }
        }
    }
    V *o = Q + q * BF * NM;
#pragma unroll
    for (int u = 0; u < BF * NM; u++) o[u] = acc[u];
}

// coarse operator P' (A P), thread per coarse block (I, J): sum over the fine rows i that P reaches I from
// (block s), in order, of P_s' Q_iJ (if row i of A P has column J)
template <int BF, int NM, class V>
__global__ void k_sa_galerkin(int64_t ncb, const int32_t *crow, const int32_t *ccj, const int64_t *ptp,
                              const int32_t *pti, const int32_t *pts, const V *P, const int64_t *qrp,
                              const int32_t *qcj, const V *Q, V *Ac, int64_t nbsc) {
    const int64_t cb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (cb >= ncb) return;
    const int32_t I = crow[cb], J = ccj[cb];
    V acc[NM * NM];
#pragma unroll
    for (int u = 0; u < NM * NM; u++) acc[u] = V(0);
    for (int64_t e = ptp[I]; e < ptp[I + 1]; e++) {
        const int64_t i = pti[e];
        int64_t lo = qrp[i], hi = qrp[i + 1];  // J in the sorted columns of row i of A P
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (qcj[mid] < J) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= qrp[i + 1] || qcj[lo] != J) continue;
        const V *ps = P + (int64_t)pts[e] * BF * NM, *qv = Q + lo * BF * NM;
#pragma unroll
        for (int c = 0; c < BF; c++) {
            V pr[NM], qr[NM];
#pragma unroll
            for (int u = 0; u < NM; u++) { pr[u] = ps[c * NM + u]; qr[u] = qv[c * NM + u]; }
#pragma unroll
            for (int a = 0; a < NM; a++)
#pragma unroll
                for (int b = 0; b < NM; b++) acc[a * NM + b] = vfma(pr[a], qr[b], acc[a * NM + b]);
        }
    }
#pragma unroll
    for (int u = 0; u < NM * NM; u++) Ac[(int64_t)u * nbsc + cb] = acc[u];
}

// The FP32 cycle's prolongator rounded to FP16 (saturated at the FP16 range): P16 by rows, P16T by columns
// (block e = block pts[e]), and P replaced by the rounded values.  Thread per entry (np blocks of S).
__global__ void k_sa_half(int64_t n, float *P, __half *P16) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const __half h = __float2half_rn(fminf(fmaxf(P[t], -65504.0f), 65504.0f));
    P16[t] = h;
    P[t] = __half2float(h);
}
template <int S>
__global__ void k_sa_half_t(int64_t np, const int32_t *pts, const __half *P16, __half *P16T) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= np * S) return;
    const int64_t e = t / S;
    P16T[t] = P16[(int64_t)pts[e] * S + (t - e * S)];
}

template <int NM, class V>
__global__ void k_null_identity(int64_t n, const uint8_t *nulld, const int64_t *diag, V *A, int64_t nbs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * NM) return;
    if (nulld[t]) A[(int64_t)((t % NM) * NM + t % NM) * nbs + diag[t / NM]] = V(1);
}

// block-Jacobi inverses of the diagonal blocks (Gauss-Jordan with partial pivoting in FP64)
template <int NB, class V>
__global__ void k_block_inverse(int64_t n, const int64_t *diag, const V *A, int64_t nbs, V *Dinv) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double M[NB][2 * NB];
    for (int r = 0; r < NB; r++)
        for (int c = 0; c < NB; c++) {
            M[r][c] = A[(int64_t)(r * NB + c) * nbs + diag[i]];
            M[r][NB + c] = (r == c) ? 1.0 : 0.0;
        }
    for (int c = 0; c < NB; c++) {
        int piv = c;
        for (int r = c + 1; r < NB; r++)
            if (fabs(M[r][c]) > fabs(M[piv][c])) piv = r;
        if (piv != c)
            for (int q = 0; q < 2 * NB; q++) { const double t = M[c][q]; M[c][q] = M[piv][q]; M[piv][q] = t; }
        const double d = M[c][c];
        const double inv = d != 0.0 ? 1.0 / d : 0.0;
        for (int q = 0; q < 2 * NB; q++) M[c][q] *= inv;
        for (int r = 0; r < NB; r++) {
            if (r == c) continue;
            const double f = M[r][c];
            for (int q = 0; q < 2 * NB; q++) M[r][q] -= f * M[c][q];
        }
    }
    for (int r = 0; r < NB; r++)
        for (int c = 0; c < NB; c++) Dinv[i * NB * NB + r * NB + c] = (V)M[r][NB + c];
}

// r = b - A x  (or y = A x with b == nullptr): a half-warp per node row, two blocks per lane in
// flight, x through the read-only path (it is constant here).  A fine-level matrix (3x3 or 2x2 blocks) is
// streamed (evict-first); a coarse level's (NB x NB, the modes' count) is read with the default policy, so
// that it stays in L2 between the cycle's passes while the fine level streams past it.
template <int NB>
__global__ void __launch_bounds__(256) k_bsr_res(int64_t n, const int64_t *__restrict__ rp,
                                                 const int32_t *__restrict__ cj, const float *__restrict__ A,
                                                 int64_t nbs, const float *__restrict__ x,
                                                 const float *__restrict__ b, float *__restrict__ out,
                                                 const int32_t *__restrict__ halt = nullptr) {
    if (halt && *halt) return;
    constexpr int G = 16, U = 2;
    const int lane = threadIdx.x % G;
    const unsigned hmask = 0xffffu << (16 * ((threadIdx.x >> 4) & 1));
    const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t row = grp; row < n; row += ng) {
        float acc[NB];
#pragma unroll
        for (int c = 0; c < NB; c++) acc[c] = 0.0f;
        const int64_t k0 = rp[row], k1 = rp[row + 1];
        for (int64_t kb = k0 + lane; kb < k1; kb += G * U) {
            int32_t j[U];
            float a[U][NB * NB];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int64_t k = kb + u * G;
                const bool ok = k < k1;
                if constexpr (NB <= 3) {
                    j[u] = ok ? __ldcs(cj + k) : 0;
#pragma unroll
                    for (int q = 0; q < NB * NB; q++) a[u][q] = ok ? __ldcs(A + (int64_t)q * nbs + k) : 0.0f;
                } else {
                    j[u] = ok ? __ldg(cj + k) : 0;
#pragma unroll
                    for (int q = 0; q < NB * NB; q++) a[u][q] = ok ? __ldg(A + (int64_t)q * nbs + k) : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                float xv[NB];
#pragma unroll
                for (int d = 0; d < NB; d++) xv[d] = __ldg(x + (int64_t)NB * j[u] + d);
#pragma unroll
                for (int c = 0; c < NB; c++)
#pragma unroll
                    for (int d = 0; d < NB; d++) acc[c] = fmaf(a[u][c * NB + d], xv[d], acc[c]);
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < NB; c++) acc[c] += __shfl_down_sync(hmask, acc[c], o, G);
        if (lane == 0)
#pragma unroll
            for (int c = 0; c < NB; c++) out[row * NB + c] = b ? b[row * NB + c] - acc[c] : acc[c];
    }
}

// The FP64 residual of the comparator's cycle: 4 lanes per block row (the FP64 pipe, not HBM, bounds it
// on GB300; two shuffle steps per row).  With a row mask (the fine level, whose matrix is K64 itself and
// not a masked copy) a masked row is that of the identity: out = b - x (or x).
template <int NB>
__global__ void __launch_bounds__(256) k_bsr_res64(int64_t n, const int64_t *__restrict__ rp,
                                                   const int32_t *__restrict__ cj, const double *__restrict__ A,
                                                   int64_t nbs, const uint8_t *__restrict__ mask,
                                                   const double *__restrict__ x, const double *__restrict__ b,
                                                   double *__restrict__ out, const int32_t *__restrict__ halt = nullptr) {
    if (halt && *halt) return;
    constexpr int RL = 4, RPW = 32 / RL;
    const int lane = threadIdx.x & 31, sub = lane & (RL - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r0 = warp * RPW; r0 < n; r0 += nw * RPW) {
        const int64_t row = r0 + lane / RL;
        const bool valid = row < n;
        double acc[NB];
#pragma unroll
        for (int c = 0; c < NB; c++) acc[c] = 0.0;
        if (valid)
            for (int64_t k = rp[row] + sub; k < rp[row + 1]; k += RL) {
                const int64_t j = __ldg(cj + k);
                double xv[NB];
#pragma unroll
                for (int d = 0; d < NB; d++) xv[d] = __ldg(x + (int64_t)NB * j + d);
#pragma unroll
                for (int c = 0; c < NB; c++)
#pragma unroll
                    for (int d = 0; d < NB; d++) acc[c] = fma(__ldg(A + (int64_t)(c * NB + d) * nbs + k), xv[d], acc[c]);
            }
#pragma unroll
        for (int c = 0; c < NB; c++)
#pragma unroll
            for (int o = RL / 2; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
        if (valid && sub == 0)
#pragma unroll
            for (int c = 0; c < NB; c++) {
                const int64_t i = row * NB + c;
                const double ax = (!mask || mask[i]) ? acc[c] : x[i];
                out[i] = b ? b[i] - ax : ax;
            }
    }
}

// The fine-level FP16 copy: rs_n = the smallest power of two >= sqrt(the node's largest diagonal entry)
template <int NB>
__global__ void k_fine_scale(int64_t n, const int64_t *diag, const float *A, int64_t nbs, float *rs) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float dmax = 0.0f;
    if (diag[i] >= 0)
#pragma unroll
        for (int c = 0; c < NB; c++) dmax = fmaxf(dmax, A[(int64_t)(c * NB + c) * nbs + diag[i]]);
    float r = 1.0f;
    if (dmax > 0.0f && isfinite(dmax)) {
        int e = 0;
        frexpf(sqrtf(dmax), &e);  // sqrt(dmax) < 2^e
        r = ldexpf(1.0f, e);
    }
    rs[i] = r;
}

// A16 = (A_ij / (rs_i rs_j)) in FP16 (power-of-two scaling: exact before the rounding), saturated; warp per row
template <int NB>
__global__ void k_fine_half(int64_t n, const int64_t *rp, const int32_t *cj, const float *A, int64_t nbs,
                            const float *rs, __half *A16) {
    const int lane = threadIdx.x & 31;
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= n) return;
    const float si = 1.0f / rs[row];
    for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += 32) {
        const float sij = si / rs[cj[k]];
#pragma unroll
        for (int q = 0; q < NB * NB; q++) {
            const float v = fminf(fmaxf(A[(int64_t)q * nbs + k] * sij, -65504.0f), 65504.0f);
            A16[(int64_t)q * nbs + k] = __float2half_rn(v);
        }
    }
}

// the scaled iterate xt of the fine level: one 16-byte (3-D) or 8-byte (2-D) gather per block; coarse
// block sizes have none (their kernels get a null xt)
template <int NB>
struct FineX {
    using T = float4;
    __device__ static T make(const float *) { return make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    __device__ static void get(const T &, float *) {}
};
template <>
struct FineX<3> {
    using T = float4;
    __device__ static T make(const float *v) { return make_float4(v[0], v[1], v[2], 0.0f); }
    __device__ static void get(const T &t, float *v) { v[0] = t.x; v[1] = t.y; v[2] = t.z; }
};
template <>
struct FineX<2> {
    using T = float2;
    __device__ static T make(const float *v) { return make_float2(v[0], v[1]); }
    __device__ static void get(const T &t, float *v) { v[0] = t.x; v[1] = t.y; }
};

// r = b - K x (b null: K x) from A16 and xt: G lanes per row, each lane 8 consecutive blocks per step (one
// 16-byte load per component and two of column indices, from the row's start rounded down to 8), the
// matrix streamed (evict-first), xt through the read-only path
template <int NB>
__global__ void __launch_bounds__(256) k_bsr_res16(int64_t n, const int64_t *__restrict__ rp,
                                                   const int32_t *__restrict__ cj, const __half *__restrict__ A,
                                                   int64_t nbs, const float *__restrict__ rs,
                                                   const typename FineX<NB>::T *__restrict__ xt,
                                                   const float *__restrict__ b, float *__restrict__ out,
                                                   const uint8_t *__restrict__ gate, const int32_t *__restrict__ halt) {
    if (halt && *halt) return;
    constexpr int G = 4;
    const int lane = threadIdx.x % G;
    const unsigned gmask = 0xfu << (G * ((threadIdx.x & 31) / G));
    const int64_t grp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const int64_t ng = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t row = grp; row < n; row += ng) {
        if (gate && !gate[row]) continue;  // uniform over the row's lanes
        float acc[NB];
#pragma unroll
        for (int c = 0; c < NB; c++) acc[c] = 0.0f;
        const int64_t k0 = rp[row], k1 = rp[row + 1];
        for (int64_t kc = (k0 & ~int64_t(7)) + 8 * lane; kc < k1; kc += 8 * G) {
            const int4 j0 = __ldcs(reinterpret_cast<const int4 *>(cj + kc));
            const int4 j1 = __ldcs(reinterpret_cast<const int4 *>(cj + kc + 4));
            uint4 a[NB * NB];
#pragma unroll
            for (int q = 0; q < NB * NB; q++) a[q] = __ldcs(reinterpret_cast<const uint4 *>(A + (int64_t)q * nbs + kc));
            const int js[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
#pragma unroll
            for (int u2 = 0; u2 < 4; u2++) {
                float2 av[NB * NB];
#pragma unroll
                for (int q = 0; q < NB * NB; q++) {
                    const unsigned w = u2 == 0 ? a[q].x : u2 == 1 ? a[q].y : u2 == 2 ? a[q].z : a[q].w;
                    av[q] = __half22float2(*reinterpret_cast<const __half2 *>(&w));
                }
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int u = 2 * u2 + h;
                    const int64_t k = kc + u;
                    if (k < k0 || k >= k1) continue;
                    float xv[NB];
                    FineX<NB>::get(__ldg(xt + js[u]), xv);
#pragma unroll
                    for (int c = 0; c < NB; c++)
#pragma unroll
                        for (int d = 0; d < NB; d++) acc[c] = fmaf(h ? av[c * NB + d].y : av[c * NB + d].x, xv[d], acc[c]);
                }
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
            for (int c = 0; c < NB; c++) acc[c] += __shfl_down_sync(gmask, acc[c], o, G);
        if (lane == 0) {
            const float r = rs[row];
#pragma unroll
            for (int c = 0; c < NB; c++) out[row * NB + c] = b ? b[row * NB + c] - r * acc[c] : r * acc[c];
        }
    }
}

// Chebyshev steps on D^-1 A (node-block D^-1):
//   mode 0: d = s2 Dinv r; x = d           (first step from x = 0; r is the right-hand side)
//   mode 1: d = s2 Dinv r; x += d          (first step from a given x; r = b - A x)
//   mode 2: d = s1 d + s2 Dinv r; x += d   (second step)
//   xt (fine level of the FP32 cycle, may be null): xt_i = rs_i x_i as well
template <int NB, class V>
__global__ void k_cheb(int64_t n, int mode, V s1, V s2, const V *__restrict__ Dinv, const V *__restrict__ r,
                       V *__restrict__ d, V *__restrict__ x, const float *__restrict__ rs = nullptr,
                       typename FineX<NB>::T *__restrict__ xt = nullptr, const uint8_t *__restrict__ gate = nullptr,
                       const int32_t *__restrict__ halt = nullptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (gate && !gate[i]) || (halt && *halt)) return;
    V rv[NB], xn[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) rv[c] = r[i * NB + c];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        V s = V(0);
#pragma unroll
        for (int e = 0; e < NB; e++) s = vfma(Dinv[i * NB * NB + c * NB + e], rv[e], s);
        const V dv = mode == 2 ? vfma(s1, d[i * NB + c], s2 * s) : s2 * s;
        d[i * NB + c] = dv;
        xn[c] = mode == 0 ? dv : x[i * NB + c] + dv;
        x[i * NB + c] = xn[c];
    }
    if (xt) {
        float v[NB];
#pragma unroll
        for (int c = 0; c < NB; c++) v[c] = (float)xn[c] * rs[i];
        xt[i] = FineX<NB>::make(v);
    }
}

// bc[a] = sum over the aggregate's nodes (in order) of T_i' r_i; warp per aggregate
template <int NB, int NM, class V>
__global__ void k_restrict(int64_t na, const int64_t *aptr, const int32_t *anodes, const V *T, const V *r, V *bc,
                           const uint8_t *gate = nullptr, const int32_t *halt = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= na || (halt && *halt)) return;
    if (gate && !gate[anodes[aptr[a]]]) return;  // an aggregate lies in one part (uniform over the warp)
    V acc[NM];
#pragma unroll
    for (int m = 0; m < NM; m++) acc[m] = V(0);
    for (int64_t q = aptr[a] + lane; q < aptr[a + 1]; q += 32) {
        const int64_t i = anodes[q];
#pragma unroll
        for (int c = 0; c < NB; c++) {
            const V rv = r[i * NB + c];
#pragma unroll
            for (int m = 0; m < NM; m++) acc[m] = vfma(T[(i * NB + c) * NM + m], rv, acc[m]);
        }
    }
#pragma unroll
    for (int m = 0; m < NM; m++) {
        V v = acc[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) bc[a * NM + m] = v;
    }
}

// x_i += T_i xc[agg(i)]
// x_i += T_i xc[agg(i)]  (and xt_i = rs_i x_i on the fine level of the FP32 cycle)
template <int NB, int NM, class V>
__global__ void k_prolong(int64_t n, const int32_t *agg, const V *T, const V *xc, V *x, const float *rs = nullptr,
                          typename FineX<NB>::T *xt = nullptr, const uint8_t *gate = nullptr,
                          const int32_t *halt = nullptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (gate && !gate[i]) || (halt && *halt)) return;
    const int64_t a = agg[i];
    float v[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        V s = x[i * NB + c];
#pragma unroll
        for (int m = 0; m < NM; m++) s = vfma(T[(i * NB + c) * NM + m], xc[a * NM + m], s);
        x[i * NB + c] = s;
        v[c] = (float)s;
    }
    if (xt) {
#pragma unroll
        for (int c = 0; c < NB; c++) v[c] *= rs[i];
        xt[i] = FineX<NB>::make(v);
    }
}

// bc[I] = sum over the fine rows i that P reaches I from (block s), in order, of P_s' r_i; warp per aggregate
template <int NB, int NM, class V>
__global__ void k_restrict_sa(int64_t na, const int64_t *ptp, const int32_t *pti, const int32_t *pts, const V *P,
                              const V *r, V *bc, const uint8_t *gate = nullptr, const int32_t *halt = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= na || (halt && *halt)) return;
    // the rows P reaches an aggregate from lie in the aggregate's part (uniform over the warp)
    if (gate && ptp[a] < ptp[a + 1] && !gate[pti[ptp[a]]]) return;
    V acc[NM];
#pragma unroll
    for (int mm = 0; mm < NM; mm++) acc[mm] = V(0);
    for (int64_t e = ptp[a] + lane; e < ptp[a + 1]; e += 32) {
        const int64_t i = pti[e];
        const V *ps = P + (int64_t)pts[e] * NB * NM;
#pragma unroll
        for (int c = 0; c < NB; c++) {
            const V rv = r[i * NB + c];
#pragma unroll
            for (int mm = 0; mm < NM; mm++) acc[mm] = vfma(ps[c * NM + mm], rv, acc[mm]);
        }
    }
#pragma unroll
    for (int mm = 0; mm < NM; mm++) {
        V v = acc[mm];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) bc[a * NM + mm] = v;
    }
}

// x_i += sum over row i's P blocks s of P_s xc[pcj[s]]  (and xt_i = rs_i x_i on the fine level of the FP32
// cycle)
template <int NB, int NM, class V>
__global__ void k_prolong_sa(int64_t n, const int64_t *prp, const int32_t *pcj, const V *P, const V *xc, V *x,
                             const float *rs = nullptr, typename FineX<NB>::T *xt = nullptr,
                             const uint8_t *gate = nullptr, const int32_t *halt = nullptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (gate && !gate[i]) || (halt && *halt)) return;
    V s[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) s[c] = x[i * NB + c];
    for (int64_t t = prp[i]; t < prp[i + 1]; t++) {
        const V *pt = P + t * NB * NM;
        const V *xa = xc + (int64_t)pcj[t] * NM;
        V xv[NM];
#pragma unroll
        for (int mm = 0; mm < NM; mm++) xv[mm] = xa[mm];
#pragma unroll
        for (int c = 0; c < NB; c++)
#pragma unroll
            for (int mm = 0; mm < NM; mm++) s[c] = vfma(pt[c * NM + mm], xv[mm], s[c]);
    }
    float v[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        x[i * NB + c] = s[c];
        v[c] = (float)s[c];
    }
    if (xt) {
#pragma unroll
        for (int c = 0; c < NB; c++) v[c] *= rs[i];
        xt[i] = FineX<NB>::make(v);
    }
}

// row c of an FP16 prolongator block (NM entries) as floats: paired loads when NM is even (the block then
// starts on a 4-byte boundary)
template <int NM>
__device__ __forceinline__ void half_row(const __half *blk, int c, float *v) {
    if constexpr (NM % 2 == 0) {
        const __half2 *p2 = reinterpret_cast<const __half2 *>(blk + c * NM);
#pragma unroll
        for (int h = 0; h < NM / 2; h++) {
            const float2 f = __half22float2(p2[h]);
            v[2 * h] = f.x;
            v[2 * h + 1] = f.y;
        }
    } else {
#pragma unroll
        for (int mm = 0; mm < NM; mm++) v[mm] = __half2float(blk[c * NM + mm]);
    }
}

// the FP32 cycle's restriction with the FP16 prolongator by columns: bc[I] = sum over e of P16T_e' r_pti[e];
// TPA threads per aggregate (a warp, or a whole CTA of TPA threads where the aggregates are few and long),
// threads over consecutive blocks, the partial sums reduced in a fixed order
template <int NB, int NM, int TPA>
__global__ void k_restrict_sa16(int64_t na, const int64_t *ptp, const int32_t *pti, const __half *PT,
                                const float *r, float *bc, const uint8_t *gate = nullptr,
                                const int32_t *halt = nullptr) {
    static_assert(TPA == 32 || TPA == 256, "a warp or a CTA of 256 per aggregate");
    const int lane = threadIdx.x & 31, tid = threadIdx.x % TPA;
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TPA;
    if (a >= na || (halt && *halt)) return;  // (uniform over a CTA when TPA is the CTA)
    if (gate && ptp[a] < ptp[a + 1] && !gate[pti[ptp[a]]]) return;
    float acc[NM];
#pragma unroll
    for (int mm = 0; mm < NM; mm++) acc[mm] = 0.0f;
    for (int64_t e = ptp[a] + tid; e < ptp[a + 1]; e += TPA) {
        const int64_t i = pti[e];
        const __half *ps = PT + e * NB * NM;
#pragma unroll
        for (int c = 0; c < NB; c++) {
            const float rv = r[i * NB + c];
            float pv[NM];
            half_row<NM>(ps, c, pv);
#pragma unroll
            for (int mm = 0; mm < NM; mm++) acc[mm] = fmaf(pv[mm], rv, acc[mm]);
        }
    }
#pragma unroll
    for (int mm = 0; mm < NM; mm++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[mm] += __shfl_down_sync(0xffffffffu, acc[mm], o);
    if constexpr (TPA == 32) {
        if (lane == 0)
#pragma unroll
            for (int mm = 0; mm < NM; mm++) bc[a * NM + mm] = acc[mm];
    } else {
        __shared__ float part[TPA / 32][NM];
        if (lane == 0)
#pragma unroll
            for (int mm = 0; mm < NM; mm++) part[tid >> 5][mm] = acc[mm];
        __syncthreads();
        if (tid < NM) {
            float v = 0.0f;
            for (int w = 0; w < TPA / 32; w++) v += part[w][tid];
            bc[a * NM + tid] = v;
        }
    }
}

// the FP32 cycle's prolongation with the FP16 prolongator by rows: x_i += sum over row i's blocks t of
// P16_t xc[pcj[t]] (and xt_i = rs_i x_i on the fine level)
template <int NB, int NM>
__global__ void k_prolong_sa16(int64_t n, const int64_t *prp, const int32_t *pcj, const __half *P, const float *xc,
                               float *x, const float *rs = nullptr, typename FineX<NB>::T *xt = nullptr,
                               const uint8_t *gate = nullptr, const int32_t *halt = nullptr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (gate && !gate[i]) || (halt && *halt)) return;
    float s[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) s[c] = x[i * NB + c];
    for (int64_t t = prp[i]; t < prp[i + 1]; t++) {
        const __half *pt = P + t * NB * NM;
        const float *xa = xc + (int64_t)pcj[t] * NM;
        float xv[NM];
#pragma unroll
        for (int mm = 0; mm < NM; mm++) xv[mm] = xa[mm];
#pragma unroll
        for (int c = 0; c < NB; c++) {
            float pv[NM];
            half_row<NM>(pt, c, pv);
#pragma unroll
            for (int mm = 0; mm < NM; mm++) s[c] = fmaf(pv[mm], xv[mm], s[c]);
        }
    }
    float v[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        x[i * NB + c] = s[c];
        v[c] = s[c];
    }
    if (xt) {
#pragma unroll
        for (int c = 0; c < NB; c++) v[c] *= rs[i];
        xt[i] = FineX<NB>::make(v);
    }
}

// dense coarsest level: expand the BSR matrix, invert it (Gauss-Jordan, FP64), multiply
template <int NM, class V>
__global__ void k_dense_expand(int64_t n, const int64_t *rp, const int32_t *cj, const V *A, int64_t nbs, double *C,
                               int64_t nc) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t k = rp[i]; k < rp[i + 1]; k++)
        for (int c = 0; c < NM; c++)
            for (int d = 0; d < NM; d++)
                C[(i * NM + c) * 2 * nc + (int64_t)cj[k] * NM + d] = A[(int64_t)(c * NM + d) * nbs + k];
}
__global__ void k_dense_init(int64_t nc, double *C) {  // C is nc x 2nc: [A | I]
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * 2 * nc) return;
    const int64_t r = t / (2 * nc), c = t % (2 * nc);
    C[t] = (c >= nc && c - nc == r) ? 1.0 : 0.0;
}
// One Gauss-Jordan step on pivot p of an SPD matrix (no pivoting needed), one launch: a grid row per matrix
// row r != p, with the factor f_r = C[r][p] / C[p][p] (rows with f_r = 0, every row outside the pivot's block
// when the level is block diagonal as for the parts of a batch, are left as they are), then
// C[r][c] -= f_r C[p][c] for the columns c > p.  Columns c <= p of the left half are not updated: the pivot
// row is zero there once eliminated, and of them only the diagonal, which no later step changes, is read
// afterwards.  Nothing a step writes (rows r != p, columns > p) is read by another CTA of the same step.
__global__ void k_gj_step(int64_t nc, int64_t p, double *C) {
    const int64_t r = blockIdx.y;
    if (r == p) return;
    const int64_t w = 2 * nc;
    __shared__ double sf;  // the FP64 division once per CTA, not per thread: the FP64 pipe is narrow
    if (threadIdx.x == 0) sf = C[r * w + p] / C[p * w + p];
    __syncthreads();
    const double fr = sf;
    if (fr == 0.0) return;
    const int64_t c = p + 1 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= w) return;
    C[r * w + c] -= fr * C[p * w + c];
}
template <class V>
__global__ void k_dense_extract(int64_t nc, const double *C, V *Cinv) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * nc) return;
    const int64_t r = t / nc, c = t % nc;
    Cinv[t] = (V)(C[r * 2 * nc + nc + c] / C[r * 2 * nc + r]);
}
// x = Cinv b, warp per row
template <class V>
__global__ void k_dense_mv(int64_t nc, const V *Cinv, const V *b, V *x, const int32_t *halt = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= nc || (halt && *halt)) return;
    V s = V(0);
    // zero entries skipped: the inverse of a block-diagonal level (the parts of a batch) is block
    // diagonal, and a part's non-finite values must not reach the others through 0 * inf
    for (int64_t c = lane; c < nc; c += 32) {
        const V a = Cinv[r * nc + c];
        if (a != V(0)) s = vfma(a, b[c], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[r] = s;
}

// sum of squares for the power iteration: per-CTA partials (fixed element assignment), the last CTA
// adds them in CTA order
template <class V>
__global__ void k_norm2(int64_t n, const V *v, double *partials, unsigned int *ticket, double *out,
                        const int32_t *halt = nullptr) {
    if (halt && *halt) return;  // (uniform: no CTA takes a ticket)
    __shared__ double sh[256];
    __shared__ bool last;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double x = v[i];
        s += x * x;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = sh[0];
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t = 0.0;
    for (unsigned b = 0; b < gridDim.x; b++) t += ((volatile double *)partials)[b];
    *out = t;
    *ticket = 0;
}
// deterministic pseudo-random start vector in [-1, 1) (integer hash of the index), scaled by s; zero
// where a mask is given and clear
template <class V>
__global__ void k_fill_random(int64_t n, double s, const uint8_t *mask, V *x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = (uint32_t)i * 2654435761u + 0x9E3779B9u;
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    const V v = (V)s * ((V)(h >> 8) * (V)(1.0f / 8388608.0f) - V(1));
    x[i] = (mask && !mask[i]) ? V(0) : v;
}
template <class V>
__global__ void k_scale(int64_t n, V s, V *x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= s;
}

// xt_i = rs_i x_i (the fine level's scaled iterate), thread per node
template <int NB>
__global__ void k_make_xt(int64_t n, const float *x, const float *rs, typename FineX<NB>::T *xt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) v[c] = x[i * NB + c] * rs[i];
    xt[i] = FineX<NB>::make(v);
}

// Power iteration on the device, with one host read at the end.  Start: the estimate 1 and no stop.
__global__ void k_power_init(double *scratch, int32_t *stop) {
    scratch[1] = 1.0;
    *stop = 0;
}
// Next iterate from bv = Dinv A x and n2 = |bv|^2 (scratch[0]): x = bv / sqrt(n2), the estimate sqrt(n2) kept
// in scratch[1]; a zero or non-finite n2 raises the stop flag and keeps the previous estimate and iterate.
// Thread per node; xt_i = rs_i x_i as well where the fine level of the FP32 cycle reads it.
template <int NB, class V>
__global__ void k_power_next(int64_t n, const V *bv, V *x, double *scratch, int32_t *stop, const float *rs,
                             typename FineX<NB>::T *xt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || *stop) return;
    const double n2 = scratch[0];
    if (!(n2 > 0.0)) {
        if (i == 0) *stop = 1;  // (every thread sees the same n2 and leaves x as it is)
        return;
    }
    const double lam = sqrt(n2);
    if (i == 0) scratch[1] = lam;
    const V sc = (V)(1.0 / lam);
    float v[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        const V xv = bv[i * NB + c] * sc;
        x[i * NB + c] = xv;
        v[c] = (float)xv;
    }
    if (xt) {
#pragma unroll
        for (int c = 0; c < NB; c++) v[c] *= rs[i];
        xt[i] = FineX<NB>::make(v);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
namespace {

int sm_count() {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

// the FP32 cycle's fine residual r = b - K x from the FP16 copy.  Its registers allow 3 CTAs per SM; a grid of
// 8 per SM (2.67 waves) measured faster than one resident wave.
template <int NB>
void launch_res16(amr_model *m, const AmrAmg *g, const AmgLevel &L, const typename FineX<NB>::T *xt, const float *b,
                  float *r, const uint8_t *gate, const int32_t *halt) {
    const unsigned grid = (unsigned)std::min<int64_t>(nblk(L.n * 4, 256), (int64_t)sm_count() * 8);
    k_bsr_res16<NB><<<grid, 256, 0, m->stream>>>(L.n, L.rp, L.cj, g->A16, m->bstride, g->rs, xt, b, r, gate, halt);
    AMR_COUNT(1);
}

// r = b - A x on a level (mask: rows of the identity, FP64 fine level only)
template <int NB, class V>
void bsr_res(cudaStream_t s, const AmgLevel &L, const V *A, int64_t nbs, const uint8_t *mask, const V *x, const V *b,
             V *out, const int32_t *halt = nullptr) {
    if constexpr (std::is_same<V, float>::value) {
        const unsigned grid = (unsigned)std::min<int64_t>(nblk(L.n * 16, 256), (int64_t)sm_count() * 8);
        k_bsr_res<NB><<<grid, 256, 0, s>>>(L.n, L.rp, L.cj, A, nbs, x, b, out, halt);
    } else {
        const unsigned grid = (unsigned)std::min<int64_t>(nblk(L.n * 4, 256), (int64_t)sm_count() * 8);
        k_bsr_res64<NB><<<grid, 256, 0, s>>>(L.n, L.rp, L.cj, A, nbs, mask, x, b, out, halt);
    }
    AMR_COUNT(1);
}

struct Cheb {
    double s1, s2a, s2b;  // d = s2a Dinv r (first), d = s1 d + s2b Dinv r (second)
};
Cheb cheb_coef(double lam) {
    // a power-iteration estimate approaches lambda_max from below: the interval's top has a margin,
    // as a smoother that sees eigenvalues above it amplifies them
    const double lo = lam / 30.0, hi = 1.25 * lam, th = 0.5 * (hi + lo), de = 0.5 * (hi - lo);
    const double sig = th / de, rho0 = 1.0 / sig, rho1 = 1.0 / (2.0 * sig - rho0);
    return Cheb{rho1 * rho0, 1.0 / th, 2.0 * rho1 / de};
}

// The V-cycle on value type V.  The fine level's matrix is the solver's: K32 (masked) for float, K64 with
// a row mask for double; its block inverses are the solver's Minv32 / Minv64.
template <int B, int NM, class V>
struct Cycle {
    static const V *fine_A(amr_model *m) {
        if constexpr (std::is_same<V, float>::value) return m->K32;
        else return m->K64;
    }
    static V *fine_Dinv(amr_model *m) {
        if constexpr (std::is_same<V, float>::value) return m->Minv32;
        else return m->Minv64;
    }
    static const uint8_t *fine_mask(amr_model *m) {
        if constexpr (std::is_same<V, float>::value) return nullptr;
        else return m->free_mask;
    }
    static V *coarse_inverse(AmrAmg *g) {
        if constexpr (std::is_same<V, float>::value) return g->Cinv;
        else return g->Cinv64;
    }
    static void level(amr_model *m, AmrAmg *g, size_t l, const V *b, V *x) {
        cudaStream_t s = m->stream;
        AmgLevel &L = g->L[l];
        if (l + 1 == g->L.size()) {
            k_dense_mv<V><<<nblk(g->nc * 32, 256), 256, 0, s>>>(g->nc, coarse_inverse(g), b, x, g->halt);
            AMR_COUNT(1);
            return;
        }
        if (l == 0) run<B>(m, g, l, L, fine_A(m), m->bstride, fine_mask(m), b, x);
        else run<NM>(m, g, l, L, vals<V>(L).A, L.nbs, nullptr, b, x);
    }
    template <int NB>
    static void run(amr_model *m, AmrAmg *g, size_t l, AmgLevel &L, const V *A, int64_t nbs, const uint8_t *mask,
                    const V *b, V *x) {
        cudaStream_t s = m->stream;
        AmgVals<V> &v = vals<V>(L);
        const Cheb c = cheb_coef(v.lam);
        const V s1 = (V)c.s1, s2a = (V)c.s2a, s2b = (V)c.s2b;
        const unsigned gn = nblk(L.n, 256);
        // the FP32 cycle's fine level: residuals from the FP16 copy and the scaled iterate xt
        using XT = typename FineX<NB>::T;
        constexpr bool kHalf = std::is_same<V, float>::value && NB == B && (NB == 2 || NB == 3);
        const bool half = kHalf && l == 0;
        XT *xt = half ? reinterpret_cast<XT *>(g->xt) : nullptr;
        const float *rs = half ? g->rs : nullptr;
        const uint8_t *gate = half ? g->gate : nullptr;
        const int32_t *halt = g->halt;
        auto residual = [&]() {
            if constexpr (kHalf) {
                if (half) {
                    launch_res16<NB>(m, g, L, xt, b, v.r, g->gate, g->halt);
                    return;
                }
            }
            bsr_res<NB, V>(s, L, A, nbs, mask, x, b, v.r, halt);
        };
        // pre-smoothing from x = 0
        k_cheb<NB, V><<<gn, 256, 0, s>>>(L.n, 0, V(0), s2a, v.Dinv, b, v.d, x, rs, xt, gate, halt);
        residual();
        k_cheb<NB, V><<<gn, 256, 0, s>>>(L.n, 2, s1, s2b, v.Dinv, v.r, v.d, x, rs, xt, gate, halt);
        // coarse correction
        residual();
        AmgLevel &C = g->L[l + 1];
        AmgVals<V> &cv = vals<V>(C);
        if (L.smooth) {
            if constexpr (std::is_same<V, float>::value)
            {
                // a warp per aggregate, or a CTA per aggregate where there are too few for a wave of warps
                if (L.naggs >= 8 * (int64_t)sm_count())
                    k_restrict_sa16<NB, NM, 32><<<nblk(L.naggs * 32, 256), 256, 0, s>>>(L.naggs, L.ptp, L.pti,
                                                                                       v.P16T, v.r, cv.bv, gate, halt);
                else
                    k_restrict_sa16<NB, NM, 256><<<(unsigned)L.naggs, 256, 0, s>>>(L.naggs, L.ptp, L.pti, v.P16T, v.r,
                                                                                   cv.bv, gate, halt);
            }
            else
                k_restrict_sa<NB, NM, V><<<nblk(L.naggs * 32, 256), 256, 0, s>>>(L.naggs, L.ptp, L.pti, L.pts, v.P,
                                                                                 v.r, cv.bv, gate, halt);
        } else
            k_restrict<NB, NM, V><<<nblk(L.naggs * 32, 256), 256, 0, s>>>(L.naggs, L.aptr, L.anodes, v.T, v.r,
                                                                          cv.bv, gate, halt);
        level(m, g, l + 1, cv.bv, cv.x);
        if (L.smooth) {
            if constexpr (std::is_same<V, float>::value)
                k_prolong_sa16<NB, NM><<<gn, 256, 0, s>>>(L.n, L.prp, L.pcj, v.P16, cv.x, x, rs, xt, gate, halt);
            else
                k_prolong_sa<NB, NM, V><<<gn, 256, 0, s>>>(L.n, L.prp, L.pcj, v.P, cv.x, x, rs, xt, gate, halt);
        } else
            k_prolong<NB, NM, V><<<gn, 256, 0, s>>>(L.n, L.agg, v.T, cv.x, x, rs, xt, gate, halt);
        // post-smoothing
        residual();
        k_cheb<NB, V><<<gn, 256, 0, s>>>(L.n, 1, V(0), s2a, v.Dinv, v.r, v.d, x, rs, xt, gate, halt);
        residual();
        k_cheb<NB, V><<<gn, 256, 0, s>>>(L.n, 2, s1, s2b, v.Dinv, v.r, v.d, x, nullptr, nullptr, gate, halt);
        AMR_COUNT(7);
        AMR_CUDA(cudaGetLastError());
    }
    // largest eigenvalue of Dinv A by power iteration (15 steps from a pseudo-random start, which excites
    // the localized high-frequency modes of distorted elements; |x| = 1 after each step)
    template <int NB>
    // (the fine level of the FP32 cycle iterates on the FP16 copy the cycle's residuals read; the steps run
    // without host reads, a device flag ending them early at a zero or non-finite norm)
    static double lambda(amr_model *m, AmrAmg *g, AmgLevel &L, const V *A, int64_t nbs, const uint8_t *mask) {
        cudaStream_t s = m->stream;
        AmgVals<V> &v = vals<V>(L);
        const int64_t nv = L.n * NB;
        const unsigned gnorm = (unsigned)std::min<int64_t>(kNormCtas, std::max<int64_t>(1, nblk(nv, 256)));
        using XT = typename FineX<NB>::T;
        constexpr bool kHalf = std::is_same<V, float>::value && NB == B && (NB == 2 || NB == 3);
        const bool half = kHalf && &L == &g->L[0];
        XT *xt = half ? reinterpret_cast<XT *>(g->xt) : nullptr;
        const float *rs = half ? g->rs : nullptr;
        const int32_t *stop = g->pstop;
        k_power_init<<<1, 1, 0, s>>>(g->scratch, g->pstop);
        k_fill_random<V><<<nblk(nv, 256), 256, 0, s>>>(nv, std::sqrt(3.0 / (double)nv), mask, v.x);
        AMR_COUNT(2);
        if (half) {  // xt of the start vector
            k_make_xt<NB><<<nblk(L.n, 256), 256, 0, s>>>(L.n, reinterpret_cast<const float *>(v.x), rs, xt);
            AMR_COUNT(1);
        }
        for (int it = 0; it < 15; it++) {
            if constexpr (kHalf) {
                if (half) launch_res16<NB>(m, g, L, xt, nullptr, v.r, nullptr, stop);
                else bsr_res<NB, V>(s, L, A, nbs, mask, v.x, nullptr, v.r, stop);
            } else {
                bsr_res<NB, V>(s, L, A, nbs, mask, v.x, nullptr, v.r, stop);
            }
            k_cheb<NB, V><<<nblk(L.n, 256), 256, 0, s>>>(L.n, 0, V(0), V(1), v.Dinv, v.r, v.d, v.bv, nullptr,
                                                         nullptr, nullptr, stop);  // bv = Dinv A x
            k_norm2<V><<<gnorm, 256, 0, s>>>(nv, v.bv, g->scratch + 8, g->ticket, g->scratch, stop);
            k_power_next<NB, V><<<nblk(L.n, 256), 256, 0, s>>>(L.n, v.bv, v.x, g->scratch, g->pstop, rs, xt);
            AMR_COUNT(3);
        }
        double lam = 1.0;
        AMR_CUDA(cudaMemcpyAsync(&lam, g->scratch + 1, sizeof(double), cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        return lam;
    }
    // the coarse operator of level l + 1 from level l: T' A T, or P' (A P) with P smoothed from T
    template <int BF>
    static void coarse(amr_model *m, AmrAmg *g, size_t l, const V *A, int64_t nbs, const uint8_t *mask) {
        cudaStream_t s = m->stream;
        AmgLevel &F = g->L[l], &C = g->L[l + 1];
        AmgVals<V> &fv = vals<V>(F), &cv = vals<V>(C);
        if (!F.smooth) {
            k_galerkin<BF, NM, V><<<nblk(C.nblocks * 32, 256), 256, 0, s>>>(C.nblocks, F.cptr, F.ck, F.ci, F.cj, A,
                                                                             nbs, fv.T, cv.A, C.nbs);
            AMR_COUNT(1);
            return;
        }
        fv.lam = lambda<BF>(m, g, F, A, nbs, mask);
        const V w = (V)(4.0 / (3.0 * fv.lam));
        auto grid = [](int64_t n) { return std::max(1u, nblk(n, 128)); };
        k_sa_prolongator<BF, NM, V><<<grid(F.np), 128, 0, s>>>(F.np, F.prow, F.pcj, F.pkp, F.pkk, F.cj, A, nbs,
                                                                    fv.T, fv.Dinv, F.agg, w, mask, fv.P);
        if constexpr (std::is_same<V, float>::value) {  // the FP32 cycle applies P in FP16
            k_sa_half<<<grid(F.np * BF * NM), 128, 0, s>>>(F.np * BF * NM, fv.P, fv.P16);
            k_sa_half_t<BF * NM><<<grid(F.np * BF * NM), 128, 0, s>>>(F.np, F.pts, fv.P16, fv.P16T);
            AMR_COUNT(2);
        }
        k_sa_ap<BF, NM, V><<<grid(F.nq), 128, 0, s>>>(F.nq, F.qrow, F.qcj, F.rp, F.cj, A, nbs, F.prp, F.pcj,
                                                            fv.P, fv.Q, F.p_steps);
        k_sa_galerkin<BF, NM, V><<<grid(C.nblocks), 128, 0, s>>>(C.nblocks, F.crow, C.cj, F.ptp, F.pti, F.pts,
                                                                       fv.P, F.qrp, F.qcj, fv.Q, cv.A, C.nbs);
        AMR_COUNT(3);
    }
    static void numeric(amr_model *m, AmrAmg *g) {
        cudaStream_t s = m->stream;
        const size_t nl = g->L.size();
        vals<V>(g->L[0]).Dinv = fine_Dinv(m);
        // (first: the fine level's power iteration reads it)
        if constexpr (std::is_same<V, float>::value) {  // the fine level's FP16 copy
            AmgLevel &F = g->L[0];
            k_fine_scale<B><<<nblk(F.n, 256), 256, 0, s>>>(F.n, F.diag, m->K32, m->bstride, g->rs);
            k_fine_half<B><<<nblk(F.n * 32, 256), 256, 0, s>>>(F.n, F.rp, F.cj, m->K32, m->bstride, g->rs, g->A16);
            AMR_COUNT(2);
            AMR_CUDA(cudaGetLastError());
        }
        for (size_t l = 0; l + 1 < nl; l++) {
            AmgLevel &F = g->L[l], &C = g->L[l + 1];
            AmgVals<V> &fv = vals<V>(F), &cv = vals<V>(C);
            if (l == 0) coarse<B>(m, g, l, fine_A(m), m->bstride, fine_mask(m));
            else coarse<NM>(m, g, l, fv.A, F.nbs, nullptr);
            k_null_identity<NM, V><<<nblk(C.n * NM, 256), 256, 0, s>>>(C.n, F.null_dof, C.diag, cv.A, C.nbs);
            AMR_COUNT(1);
            if (l + 2 < nl) {
                k_block_inverse<NM, V><<<nblk(C.n, 128), 128, 0, s>>>(C.n, C.diag, cv.A, C.nbs, cv.Dinv);
                AMR_COUNT(1);
            }
            AMR_CUDA(cudaGetLastError());
        }
        for (size_t l = 0; l + 1 < nl; l++) {  // (a smoothed level's lambda came with its prolongator)
            AmgLevel &L = g->L[l];
            if (L.smooth) continue;
            vals<V>(L).lam = l == 0 ? lambda<B>(m, g, L, fine_A(m), m->bstride, fine_mask(m))
                                    : lambda<NM>(m, g, L, vals<V>(L).A, L.nbs, nullptr);
        }
        // dense coarsest level
        AmgLevel &D = g->L[nl - 1];
        const int64_t nc = g->nc, w = 2 * nc;
        k_dense_init<<<nblk(nc * w, 256), 256, 0, s>>>(nc, g->Cd);
        k_dense_expand<NM, V><<<nblk(D.n, 128), 128, 0, s>>>(D.n, D.rp, D.cj, vals<V>(D).A, D.nbs, g->Cd, nc);
        AMR_COUNT(2);
        // the nc pivot steps as one CUDA graph, captured once per hierarchy (its buffers are fixed)
        if (!g->gj_exec) {
            cudaGraph_t gr = nullptr;
            AMR_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
            for (int64_t p = 0; p < nc; p++)
                k_gj_step<<<dim3(nblk(w - p - 1, 256), (unsigned)nc), 256, 0, s>>>(nc, p, g->Cd);
            const cudaError_t ce = cudaStreamEndCapture(s, &gr);
            if (ce == cudaSuccess) {
                const cudaError_t ie = cudaGraphInstantiate(&g->gj_exec, gr, 0);
                cudaGraphDestroy(gr);
                AMR_CUDA(ie);
            } else {
                if (gr) cudaGraphDestroy(gr);
                AMR_CUDA(ce);
            }
        }
        AMR_CUDA(cudaGraphLaunch(g->gj_exec, s));
        AMR_COUNT(nc);
        k_dense_extract<V><<<nblk(nc * nc, 256), 256, 0, s>>>(nc, g->Cd, coarse_inverse(g));
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
    }
};

// The FP64 values of every level, allocated (and the prolongator uploaded) on first use.
void ensure_fp64(amr_model *m, AmrAmg *g) {
    if (g->Cinv64) return;
    for (size_t l = 0; l < g->L.size(); l++) {
        AmgLevel &L = g->L[l];
        AmgVals<double> &v = L.f64;
        const int64_t nv = L.n * L.b;
        if (l > 0) {
            amr_alloc(&v.A, (size_t)L.nbs * L.b * L.b);
            amr_alloc(&v.Dinv, (size_t)L.n * L.b * L.b);
        }
        amr_alloc(&v.x, nv); amr_alloc(&v.bv, nv); amr_alloc(&v.r, nv); amr_alloc(&v.d, nv);
        if (!L.hT.empty()) {
            amr_alloc(&v.T, L.hT.size());
            amr_h2d(m, v.T, L.hT.data(), L.hT.size() * sizeof(double));
        }
        if (L.smooth) {
            amr_alloc(&v.P, (size_t)std::max<int64_t>(L.np, 1) * L.b * g->NM);
            amr_alloc(&v.Q, (size_t)std::max<int64_t>(L.nq, 1) * L.b * g->NM);
        }
    }
    amr_alloc(&g->Cinv64, (size_t)g->nc * g->nc);
}

void prepare_structure(amr_model *m) {
    if (!m->amg || m->amg->dofs_version != m->dofs_version) {
        amg_build_structure(m);
        m->amg->dofs_version = m->dofs_version;
    }
}

}  // namespace

// Structure once per DOF numbering, values after each assembly of K.
void amr_amg_prepare(amr_model *m) {
    prepare_structure(m);
    if (!m->amg->numeric_valid) {
        if (m->B == 3) Cycle<3, 6, float>::numeric(m, m->amg);
        else Cycle<2, 3, float>::numeric(m, m->amg);
        m->amg->numeric_valid = true;
    }
}

// The same hierarchy in FP64 (the all-FP64 comparator's preconditioner).
void amr_amg_prepare64(amr_model *m) {
    prepare_structure(m);
    ensure_fp64(m, m->amg);
    if (!m->amg->numeric64_valid) {
        if (m->B == 3) Cycle<3, 6, double>::numeric(m, m->amg);
        else Cycle<2, 3, double>::numeric(m, m->amg);
        m->amg->numeric64_valid = true;
    }
}

// z = V-cycle(r), fine-level node-major FP32 vectors, on the handle's stream
void amr_amg_set_gate(amr_model *m, const uint8_t *gate) {
    if (m->amg) m->amg->gate = gate;
}

// a device flag read by every kernel of the cycle: while it is nonzero they return at once
void amr_amg_set_halt(amr_model *m, const int32_t *halt) {
    if (m->amg) m->amg->halt = halt;
}

void amr_amg_vcycle(amr_model *m, const float *r, float *z) {
    if (m->B == 3) Cycle<3, 6, float>::level(m, m->amg, 0, r, z);
    else Cycle<2, 3, float>::level(m, m->amg, 0, r, z);
}

// z = V-cycle(r) in FP64 (zero at prescribed slots when r is)
void amr_amg_vcycle64(amr_model *m, const double *r, double *z) {
    if (m->B == 3) Cycle<3, 6, double>::level(m, m->amg, 0, r, z);
    else Cycle<2, 3, double>::level(m, m->amg, 0, r, z);
}

// average device time of the cycle's fine-level residual r = b - K x (CUDA events on the handle's stream) and
// its algorithmic bytes per launch: the FP32 cycle's kernel on the FP16 copy, or with fp64 the comparator's on
// K64
double amr_amg_time_residual(amr_model *m, int reps, bool fp64, double *bytes) {
    AmrAmg *g = m->amg;
    if (!g || !(fp64 ? g->numeric64_valid : g->numeric_valid))
        throw AmrError(AMR_EINVAL, "run a multigrid solve of this precision on the current K first");
    AmgLevel &L = g->L[0];
    cudaStream_t s = m->stream;
    const int B = m->B;
    const double nb = (double)m->nblocks, nn = (double)m->nnodes;
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int i = 0; i < reps; i++) {
        if (fp64) {
            if (B == 3) bsr_res<3, double>(s, L, m->K64, m->bstride, m->free_mask, L.f64.x, L.f64.bv, L.f64.r);
            else bsr_res<2, double>(s, L, m->K64, m->bstride, m->free_mask, L.f64.x, L.f64.bv, L.f64.r);
        } else if (B == 3) {
            launch_res16<3>(m, g, L, reinterpret_cast<const float4 *>(g->xt), L.f32.bv, L.f32.r, nullptr, nullptr);
        } else {
            launch_res16<2>(m, g, L, reinterpret_cast<const float2 *>(g->xt), L.f32.bv, L.f32.r, nullptr, nullptr);
        }
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    if (bytes) {
        // blocks (values + column) + row pointers + per node: b read, r written, and x (FP64: read once, plus
        // the row mask) or the FP16 path's scale and scaled iterate (one 16- or 8-byte vector per node)
        if (fp64) *bytes = nb * (8.0 * B * B + 4.0) + (nn + 1) * 8.0 + nn * B * (8.0 * 3.0 + 1.0);
        else *bytes = nb * (2.0 * B * B + 4.0) + (nn + 1) * 8.0 + nn * (4.0 * B * 2.0 + 4.0 + (B == 3 ? 16.0 : 8.0));
    }
    return ms * 1e-3 / reps;
}

void amr_amg_invalidate(amr_model *m) {
    if (m->amg) m->amg->numeric_valid = m->amg->numeric64_valid = false;
}
