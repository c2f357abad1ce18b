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
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

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

}  // namespace

struct AmgLevel {
    int b = 0;
    int64_t n = 0;
    // matrix of this level (levels >= 1): BSR, b x b blocks, SoA values [b*b][nbs]
    int64_t nblocks = 0, nbs = 0;
    int64_t *rp = nullptr;
    int32_t *cj = nullptr;
    int64_t *diag = nullptr;
    float *A = nullptr;
    float *Dinv = nullptr;  // n x b*b block-Jacobi inverses (level 0: the solver's Minv32)
    double lam = 1.0;
    // to the next coarser level
    int64_t naggs = 0;
    int32_t *agg = nullptr;   // node -> aggregate
    float *T = nullptr;       // n x b x NM prolongator blocks
    int64_t *aptr = nullptr;  // aggregate -> its nodes
    int32_t *anodes = nullptr;
    int64_t *cptr = nullptr;  // coarse block -> contributions (fine block k, fine row i)
    int32_t *ck = nullptr, *ci = nullptr;
    uint8_t *null_dof = nullptr;  // coarse DOFs with no mode (aggregate of prescribed DOFs): identity
    // vectors of this level: x, b, r, d (n*b)
    float *x = nullptr, *bv = nullptr, *r = nullptr, *d = nullptr;
};

struct AmrAmg {
    int NM = 6;
    std::vector<AmgLevel> L;
    int64_t nc = 0;             // DOFs of the dense coarsest level
    double *Cd = nullptr;       // nc x nc FP64 work (Gauss-Jordan)
    float *Cinv = nullptr;      // nc x nc FP32 inverse
    double *scratch = nullptr;  // norms: [0] result, [8..] per-CTA partials
    unsigned int *ticket = nullptr;
    int64_t dofs_version = -1;
    bool numeric_valid = false;
};

void amr_amg_free(amr_model *m) {
    AmrAmg *g = m->amg;
    if (!g) return;
    for (size_t l = 0; l < g->L.size(); l++) {
        AmgLevel &v = g->L[l];
        if (l > 0) {
            amr_free(v.rp); amr_free(v.cj); amr_free(v.A); amr_free(v.Dinv);
        }
        amr_free(v.diag); amr_free(v.agg); amr_free(v.T); amr_free(v.aptr); amr_free(v.anodes);
        amr_free(v.cptr); amr_free(v.ck); amr_free(v.ci); amr_free(v.null_dof);
        amr_free(v.x); amr_free(v.bv); amr_free(v.r); amr_free(v.d);
    }
    amr_free(g->Cd); amr_free(g->Cinv); amr_free(g->scratch); amr_free(g->ticket);
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
            AMR_CUDA(cudaMemcpy(lv.rp, h.rp.data(), (h.n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
            AMR_CUDA(cudaMemcpy(lv.cj, h.cj.data(), lv.nblocks * sizeof(int32_t), cudaMemcpyHostToDevice));
            amr_alloc(&lv.A, (size_t)lv.nbs * h.b * h.b);
            amr_alloc(&lv.Dinv, (size_t)h.n * h.b * h.b);
        } else {
            lv.rp = m->brow_ptr;
            lv.cj = m->bcol;
            lv.nbs = m->bstride;
        }
        amr_alloc(&lv.diag, h.n);
        AMR_CUDA(cudaMemcpy(lv.diag, h.diag.data(), h.n * sizeof(int64_t), cudaMemcpyHostToDevice));
        const int64_t nv = h.n * h.b;
        amr_alloc(&lv.x, nv); amr_alloc(&lv.bv, nv); amr_alloc(&lv.r, nv); amr_alloc(&lv.d, nv);
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
        std::vector<float> T((size_t)h.n * h.b * NM, 0.0f);
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
                        T[((size_t)i * h.b + c) * NM + k] = (float)(s * sc[k]);
                    }
            }
            for (int k = 0; k < NM; k++)
                for (int p = 0; p < NM; p++)
                    hc.nns[((size_t)a * NM + k) * NM + p] = sc[k] > 0.0 ? std::sqrt(w[k]) * V[p * NM + k] : 0.0;
        });
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
        lv.naggs = na;
        amr_alloc(&lv.agg, h.n);
        amr_alloc(&lv.T, T.size());
        amr_alloc(&lv.aptr, na + 1);
        amr_alloc(&lv.anodes, h.n);
        amr_alloc(&lv.cptr, cptr.size());
        amr_alloc(&lv.ck, cks.size());
        amr_alloc(&lv.ci, cis.size());
        amr_alloc(&lv.null_dof, nulld.size());
        AMR_CUDA(cudaMemcpy(lv.agg, agg.data(), h.n * sizeof(int32_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.T, T.data(), T.size() * sizeof(float), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.aptr, aptr.data(), aptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.anodes, anodes.data(), h.n * sizeof(int32_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.cptr, cptr.data(), cptr.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.ck, cks.data(), cks.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.ci, cis.data(), cis.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
        AMR_CUDA(cudaMemcpy(lv.null_dof, nulld.data(), nulld.size(), cudaMemcpyHostToDevice));
        g->L.push_back(lv);
        H.push_back(std::move(hc));
    }
    amr_alloc(&g->Cd, (size_t)g->nc * 2 * g->nc);  // [A | I] for Gauss-Jordan
    amr_alloc(&g->Cinv, (size_t)g->nc * g->nc);
    amr_alloc(&g->scratch, 8 + kNormCtas);
    amr_alloc(&g->ticket, 1);
    AMR_CUDA(cudaMemset(g->ticket, 0, sizeof(unsigned int)));
    g->numeric_valid = false;
}

// ---------------------------------------------------------------------------
// device kernels
// ---------------------------------------------------------------------------
namespace {

// coarse block (warp) = sum over its contributions (fine block k of row i, column j) of T_i' A_k T_j
template <int BF, int NM>
__global__ void k_galerkin(int64_t ncb, const int64_t *cptr, const int32_t *ck, const int32_t *ci,
                           const int32_t *cjf, const float *Af, int64_t nbsf, const float *T, float *Ac,
                           int64_t nbsc) {
    const int lane = threadIdx.x & 31;
    const int64_t cb = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (cb >= ncb) return;
    float acc[NM * NM];
#pragma unroll
    for (int q = 0; q < NM * NM; q++) acc[q] = 0.0f;
    for (int64_t e = cptr[cb] + lane; e < cptr[cb + 1]; e += 32) {
        const int64_t k = ck[e];
        const int32_t i = ci[e], j = cjf[k];
        float M[BF * NM];  // A_k T_j
#pragma unroll
        for (int c = 0; c < BF; c++)
#pragma unroll
            for (int m = 0; m < NM; m++) {
                float s = 0.0f;
#pragma unroll
                for (int d = 0; d < BF; d++) s = fmaf(Af[(int64_t)(c * BF + d) * nbsf + k], T[((int64_t)j * BF + d) * NM + m], s);
                M[c * NM + m] = s;
            }
#pragma unroll
        for (int p = 0; p < NM; p++)
#pragma unroll
            for (int m = 0; m < NM; m++) {
                float s = acc[p * NM + m];
#pragma unroll
                for (int c = 0; c < BF; c++) s = fmaf(T[((int64_t)i * BF + c) * NM + p], M[c * NM + m], s);
                acc[p * NM + m] = s;
            }
    }
#pragma unroll
    for (int q = 0; q < NM * NM; q++) {
        float v = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) Ac[(int64_t)q * nbsc + cb] = v;
    }
}

// coarse DOFs without a mode get an identity equation
template <int NM>
__global__ void k_null_identity(int64_t n, const uint8_t *nulld, const int64_t *diag, float *A, int64_t nbs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * NM) return;
    if (nulld[t]) A[(int64_t)((t % NM) * NM + t % NM) * nbs + diag[t / NM]] = 1.0f;
}

// block-Jacobi inverses of the diagonal blocks (Gauss-Jordan with partial pivoting in FP64)
template <int NB>
__global__ void k_block_inverse(int64_t n, const int64_t *diag, const float *A, int64_t nbs, float *Dinv) {
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
        for (int c = 0; c < NB; c++) Dinv[i * NB * NB + r * NB + c] = (float)M[r][NB + c];
}

// r = b - A x  (or y = A x with b == nullptr): a half-warp per node row, two blocks per lane in
// flight, the matrix streamed (evict-first), x through the read-only path (it is constant here)
template <int NB>
__global__ void __launch_bounds__(256) k_bsr_res(int64_t n, const int64_t *__restrict__ rp,
                                                 const int32_t *__restrict__ cj, const float *__restrict__ A,
                                                 int64_t nbs, const float *__restrict__ x,
                                                 const float *__restrict__ b, float *__restrict__ out) {
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
                j[u] = ok ? __ldcs(cj + k) : 0;
#pragma unroll
                for (int q = 0; q < NB * NB; q++) a[u][q] = ok ? __ldcs(A + (int64_t)q * nbs + k) : 0.0f;
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

// Chebyshev steps on D^-1 A (node-block D^-1):
//   mode 0: d = s2 Dinv r; x = d           (first step from x = 0; r is the right-hand side)
//   mode 1: d = s2 Dinv r; x += d          (first step from a given x; r = b - A x)
//   mode 2: d = s1 d + s2 Dinv r; x += d   (second step)
template <int NB>
__global__ void k_cheb(int64_t n, int mode, float s1, float s2, const float *__restrict__ Dinv,
                       const float *__restrict__ r, float *__restrict__ d, float *__restrict__ x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float rv[NB];
#pragma unroll
    for (int c = 0; c < NB; c++) rv[c] = r[i * NB + c];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        float s = 0.0f;
#pragma unroll
        for (int e = 0; e < NB; e++) s = fmaf(Dinv[i * NB * NB + c * NB + e], rv[e], s);
        const float dv = mode == 2 ? fmaf(s1, d[i * NB + c], s2 * s) : s2 * s;
        d[i * NB + c] = dv;
        x[i * NB + c] = mode == 0 ? dv : x[i * NB + c] + dv;
    }
}

// bc[a] = sum over the aggregate's nodes (in order) of T_i' r_i; warp per aggregate
template <int NB, int NM>
__global__ void k_restrict(int64_t na, const int64_t *aptr, const int32_t *anodes, const float *T,
                           const float *r, float *bc) {
    const int lane = threadIdx.x & 31;
    const int64_t a = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= na) return;
    float acc[NM];
#pragma unroll
    for (int m = 0; m < NM; m++) acc[m] = 0.0f;
    for (int64_t q = aptr[a] + lane; q < aptr[a + 1]; q += 32) {
        const int64_t i = anodes[q];
#pragma unroll
        for (int c = 0; c < NB; c++) {
            const float rv = r[i * NB + c];
#pragma unroll
            for (int m = 0; m < NM; m++) acc[m] = fmaf(T[(i * NB + c) * NM + m], rv, acc[m]);
        }
    }
#pragma unroll
    for (int m = 0; m < NM; m++) {
        float v = acc[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) bc[a * NM + m] = v;
    }
}

// x_i += T_i xc[agg(i)]
template <int NB, int NM>
__global__ void k_prolong(int64_t n, const int32_t *agg, const float *T, const float *xc, float *x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t a = agg[i];
#pragma unroll
    for (int c = 0; c < NB; c++) {
        float s = x[i * NB + c];
#pragma unroll
        for (int m = 0; m < NM; m++) s = fmaf(T[(i * NB + c) * NM + m], xc[a * NM + m], s);
        x[i * NB + c] = s;
    }
}

// dense coarsest level: expand the BSR matrix, invert it (Gauss-Jordan, FP64), multiply
template <int NM>
__global__ void k_dense_expand(int64_t n, const int64_t *rp, const int32_t *cj, const float *A, int64_t nbs,
                               double *C, int64_t nc) {
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
// one Gauss-Jordan step on pivot p of an SPD matrix (no pivoting needed): rows r != p
__global__ void k_gj_eliminate(int64_t nc, int64_t p, double *C) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t w = 2 * nc;
    if (t >= nc * w) return;
    const int64_t r = t / w, c = t % w;
    if (r == p || c == p) return;
    const double f = C[r * w + p] / C[p * w + p];
    C[r * w + c] -= f * C[p * w + c];
}
__global__ void k_gj_column(int64_t nc, int64_t p, double *C) {  // clear column p below/above the pivot
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nc || r == p) return;
    C[r * 2 * nc + p] = 0.0;
}
__global__ void k_dense_extract(int64_t nc, const double *C, float *Cinv) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc * nc) return;
    const int64_t r = t / nc, c = t % nc;
    Cinv[t] = (float)(C[r * 2 * nc + nc + c] / C[r * 2 * nc + r]);
}
// x = Cinv b, warp per row
__global__ void k_dense_mv(int64_t nc, const float *Cinv, const float *b, float *x) {
    const int lane = threadIdx.x & 31;
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= nc) return;
    float s = 0.0f;
    for (int64_t c = lane; c < nc; c += 32) s = fmaf(Cinv[r * nc + c], b[c], s);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[r] = s;
}

// sum of squares for the power iteration: per-CTA partials (fixed element assignment), the last CTA
// adds them in CTA order
__global__ void k_norm2(int64_t n, const float *v, double *partials, unsigned int *ticket, double *out) {
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
// deterministic pseudo-random start vector in [-1, 1) (integer hash of the index), scaled by s
__global__ void k_fill_random(int64_t n, float s, float *x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = (uint32_t)i * 2654435761u + 0x9E3779B9u;
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    x[i] = s * ((float)(h >> 8) * (1.0f / 8388608.0f) - 1.0f);
}
__global__ void k_scale(int64_t n, float s, float *x) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] *= s;
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

template <int NB>
void bsr_res(cudaStream_t s, const AmgLevel &L, const float *A, int64_t nbs, const float *x, const float *b,
             float *out) {
    const unsigned grid = (unsigned)std::min<int64_t>(nblk(L.n * 16, 256), (int64_t)sm_count() * 8);
    k_bsr_res<NB><<<grid, 256, 0, s>>>(L.n, L.rp, L.cj, A, nbs, x, b, out);
    AMR_COUNT(1);
}

struct Cheb {
    float s1, s2a, s2b;  // d = s2a Dinv r (first), d = s1 d + s2b Dinv r (second)
};
Cheb cheb_coef(double lam) {
    // a power-iteration estimate approaches lambda_max from below: the interval's top has a margin,
    // as a smoother that sees eigenvalues above it amplifies them
    const double lo = lam / 30.0, hi = 1.25 * lam, th = 0.5 * (hi + lo), de = 0.5 * (hi - lo);
    const double sig = th / de, rho0 = 1.0 / sig, rho1 = 1.0 / (2.0 * sig - rho0);
    return Cheb{(float)(rho1 * rho0), (float)(1.0 / th), (float)(2.0 * rho1 / de)};
}

template <int B, int NM>
struct Cycle {
    static void level(amr_model *m, AmrAmg *g, size_t l, const float *b, float *x) {
        cudaStream_t s = m->stream;
        AmgLevel &L = g->L[l];
        if (l + 1 == g->L.size()) {
            k_dense_mv<<<nblk(g->nc * 32, 256), 256, 0, s>>>(g->nc, g->Cinv, b, x);
            AMR_COUNT(1);
            return;
        }
        if (l == 0) run<B>(m, g, l, L, m->K32, m->bstride, b, x);
        else run<NM>(m, g, l, L, L.A, L.nbs, b, x);
    }
    template <int NB>
    static void run(amr_model *m, AmrAmg *g, size_t l, AmgLevel &L, const float *A, int64_t nbs, const float *b,
                    float *x) {
        cudaStream_t s = m->stream;
        const Cheb c = cheb_coef(L.lam);
        const unsigned gn = nblk(L.n, 256);
        // pre-smoothing from x = 0
        k_cheb<NB><<<gn, 256, 0, s>>>(L.n, 0, 0.0f, c.s2a, L.Dinv, b, L.d, x);
        bsr_res<NB>(s, L, A, nbs, x, b, L.r);
        k_cheb<NB><<<gn, 256, 0, s>>>(L.n, 2, c.s1, c.s2b, L.Dinv, L.r, L.d, x);
        // coarse correction
        bsr_res<NB>(s, L, A, nbs, x, b, L.r);
        AmgLevel &C = g->L[l + 1];
        k_restrict<NB, NM><<<nblk(L.naggs * 32, 256), 256, 0, s>>>(L.naggs, L.aptr, L.anodes, L.T, L.r, C.bv);
        level(m, g, l + 1, C.bv, C.x);
        k_prolong<NB, NM><<<gn, 256, 0, s>>>(L.n, L.agg, L.T, C.x, x);
        // post-smoothing
        bsr_res<NB>(s, L, A, nbs, x, b, L.r);
        k_cheb<NB><<<gn, 256, 0, s>>>(L.n, 1, 0.0f, c.s2a, L.Dinv, L.r, L.d, x);
        bsr_res<NB>(s, L, A, nbs, x, b, L.r);
        k_cheb<NB><<<gn, 256, 0, s>>>(L.n, 2, c.s1, c.s2b, L.Dinv, L.r, L.d, x);
        AMR_COUNT(7);
        AMR_CUDA(cudaGetLastError());
    }
    // largest eigenvalue of Dinv A by power iteration (15 steps from a pseudo-random start, which excites
    // the localized high-frequency modes of distorted elements; |x| = 1 after each step)
    template <int NB>
    static double lambda(amr_model *m, AmrAmg *g, AmgLevel &L, const float *A, int64_t nbs) {
        cudaStream_t s = m->stream;
        const int64_t nv = L.n * NB;
        const unsigned gnorm = (unsigned)std::min<int64_t>(kNormCtas, std::max<int64_t>(1, nblk(nv, 256)));
        k_fill_random<<<nblk(nv, 256), 256, 0, s>>>(nv, (float)(std::sqrt(3.0 / (double)nv)), L.x);
        AMR_COUNT(1);
        double lam = 1.0;
        for (int it = 0; it < 15; it++) {
            bsr_res<NB>(s, L, A, nbs, L.x, nullptr, L.r);
            k_cheb<NB><<<nblk(L.n, 256), 256, 0, s>>>(L.n, 0, 0.0f, 1.0f, L.Dinv, L.r, L.d, L.bv);  // bv = Dinv A x
            k_norm2<<<gnorm, 256, 0, s>>>(nv, L.bv, g->scratch + 8, g->ticket, g->scratch);
            AMR_COUNT(2);
            double n2 = 0.0;
            AMR_CUDA(cudaMemcpyAsync(&n2, g->scratch, sizeof(double), cudaMemcpyDeviceToHost, s));
            AMR_CUDA(cudaStreamSynchronize(s));
            if (!(n2 > 0.0)) break;
            lam = std::sqrt(n2);
            AMR_CUDA(cudaMemcpyAsync(L.x, L.bv, nv * sizeof(float), cudaMemcpyDeviceToDevice, s));
            k_scale<<<nblk(nv, 256), 256, 0, s>>>(nv, (float)(1.0 / lam), L.x);
            AMR_COUNT(1);
        }
        return lam;
    }
    static void numeric(amr_model *m, AmrAmg *g) {
        cudaStream_t s = m->stream;
        const size_t nl = g->L.size();
        g->L[0].Dinv = m->Minv32;
        for (size_t l = 0; l + 1 < nl; l++) {
            AmgLevel &F = g->L[l], &C = g->L[l + 1];
            const unsigned gc = nblk(C.nblocks * 32, 256);
            if (l == 0)
                k_galerkin<B, NM><<<gc, 256, 0, s>>>(C.nblocks, F.cptr, F.ck, F.ci, F.cj, m->K32, m->bstride, F.T,
                                                     C.A, C.nbs);
            else
                k_galerkin<NM, NM><<<gc, 256, 0, s>>>(C.nblocks, F.cptr, F.ck, F.ci, F.cj, F.A, F.nbs, F.T, C.A,
                                                      C.nbs);
            k_null_identity<NM><<<nblk(C.n * NM, 256), 256, 0, s>>>(C.n, F.null_dof, C.diag, C.A, C.nbs);
            AMR_COUNT(2);
            if (l + 2 < nl) {
                k_block_inverse<NM><<<nblk(C.n, 128), 128, 0, s>>>(C.n, C.diag, C.A, C.nbs, C.Dinv);
                AMR_COUNT(1);
            }
            AMR_CUDA(cudaGetLastError());
        }
        for (size_t l = 0; l + 1 < nl; l++) {
            AmgLevel &L = g->L[l];
            L.lam = l == 0 ? lambda<B>(m, g, L, m->K32, m->bstride) : lambda<NM>(m, g, L, L.A, L.nbs);
        }
        // dense coarsest level
        AmgLevel &D = g->L[nl - 1];
        const int64_t nc = g->nc, w = 2 * nc;
        k_dense_init<<<nblk(nc * w, 256), 256, 0, s>>>(nc, g->Cd);
        k_dense_expand<NM><<<nblk(D.n, 128), 128, 0, s>>>(D.n, D.rp, D.cj, D.A, D.nbs, g->Cd, nc);
        AMR_COUNT(2);
        for (int64_t p = 0; p < nc; p++) {
            k_gj_eliminate<<<nblk(nc * w, 256), 256, 0, s>>>(nc, p, g->Cd);
            k_gj_column<<<nblk(nc, 256), 256, 0, s>>>(nc, p, g->Cd);
        }
        AMR_COUNT(2 * nc);
        k_dense_extract<<<nblk(nc * nc, 256), 256, 0, s>>>(nc, g->Cd, g->Cinv);
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
        g->numeric_valid = true;
    }
};

}  // namespace

// Structure once per DOF numbering, values after each assembly of K.
void amr_amg_prepare(amr_model *m) {
    if (!m->amg || m->amg->dofs_version != m->dofs_version) {
        amg_build_structure(m);
        m->amg->dofs_version = m->dofs_version;
    }
    if (!m->amg->numeric_valid) {
        if (m->B == 3) Cycle<3, 6>::numeric(m, m->amg);
        else Cycle<2, 3>::numeric(m, m->amg);
    }
}

// z = V-cycle(r), fine-level node-major FP32 vectors, on the handle's stream
void amr_amg_vcycle(amr_model *m, const float *r, float *z) {
    if (m->B == 3) Cycle<3, 6>::level(m, m->amg, 0, r, z);
    else Cycle<2, 3>::level(m, m->amg, 0, r, z);
}

// average device time of the cycle's fine-level residual r = b - K32 x (CUDA events on the handle's stream)
double amr_amg_time_residual(amr_model *m, int reps) {
    AmrAmg *g = m->amg;
    if (!g || !g->numeric_valid) throw AmrError(AMR_EINVAL, "run a multigrid solve on the current K first");
    AmgLevel &L = g->L[0];
    cudaStream_t s = m->stream;
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int i = 0; i < reps; i++) {
        if (m->B == 3) bsr_res<3>(s, L, m->K32, m->bstride, L.x, L.bv, L.r);
        else bsr_res<2>(s, L, m->K32, m->bstride, L.x, L.bv, L.r);
    }
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    return ms * 1e-3 / reps;
}

void amr_amg_invalidate(amr_model *m) {
    if (m->amg) m->amg->numeric_valid = false;
}
