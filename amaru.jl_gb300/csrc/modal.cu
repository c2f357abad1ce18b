// Modal analysis on the device: mech_modal_solver! (src/mech/mech-modal-solver.jl:72-235).
//
// The reference takes the nmodes eigenpairs of smallest magnitude of P = K11 ./ L, with L the column
// sums of M11 (row-sum lumped masses), keeps the real positive ones and returns omega = sqrt(lambda)
// and P's unit eigenvectors.  P's eigenpairs are those of the pencil K11 phi = lambda D phi,
// D = diag(L), with v = D phi.  Serendipity cells have negative corner masses, so D can be
// indefinite; K11 is SPD, so the pencil D phi = mu K11 phi (mu = 1/lambda) is symmetric-definite
// whatever D's signs, and the wanted modes are its largest positive mu.
//
// LOBPCG (Knyazev's locally optimal block preconditioned CG) on that pencil: block X of nmodes + guard
// vectors, B-orthonormal in K11; residuals R = D X - K X diag(theta); preconditioned W = T R with T one
// aggregation-multigrid V-cycle of K (FP32, the solver's); Rayleigh-Ritz on [X, W, P] from the Gram
// matrices S'DS and S'(KS), solved on the host after scaling to unit diagonal and dropping the
// directions whose K-Gram eigenvalue is below 1e-12 of the largest.  Device vectors are node-major
// (nnodes x B) columns, zero outside the unknown DOFs.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "amr_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxCols = 16;   // columns per launch of the multi-vector SpMV and of the combination kernel
constexpr int kMaxBlock = 64;  // LOBPCG block width limit (nmodes + guard vectors)
constexpr int kRowLanes = 4;   // lanes per block row in the SpMV
constexpr int kGramTile = 32;  // rows per shared-memory tile of the Gram kernel (fewer for wide blocks)
constexpr int kGramCtas = 304;
constexpr int kGramItems = 10; // Gram items per thread and launch (wider Grams take several launches)
constexpr size_t kGramSmem = 48 * 1024;

unsigned blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kThreads - 1) / kThreads); }

// D: row sums of M11 (sum over the unknown columns of each unknown row; M's blocks are m I)
template <int B>
__global__ void k_lumped(int64_t nn, int64_t nb, const int64_t *rp, const int32_t *cj, const double *M,
                         const uint8_t *fm, double *D) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nn * B) return;
    const int64_t n = t / B;
    const int c = (int)(t % B);
    double s = 0.0;
    if (fm[t])
        for (int64_t k = rp[n]; k < rp[n + 1]; k++)
            if (fm[(int64_t)cj[k] * B + c]) s += M[k];
    D[t] = s;
}

// out_c = mask(K x_c) for the block's ncol columns (column stride n); K read once for all columns
template <int B>
__global__ void __launch_bounds__(kThreads) k_spmv_multi(int64_t nn, int64_t nb, const int64_t *__restrict__ rp,
                                                         const int32_t *__restrict__ cj, const double *__restrict__ K,
                                                         const uint8_t *__restrict__ fm, int ncol,
                                                         const double *__restrict__ x, double *__restrict__ out) {
    constexpr int RPW = 32 / kRowLanes;
    const int64_t n = nn * B;
    const int lane = threadIdx.x & 31, sub = lane & (kRowLanes - 1);
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r0 = warp * RPW; r0 < nn; r0 += nw * RPW) {  // whole warps: every lane reaches the shuffles
        const int64_t row = r0 + lane / kRowLanes;
        const bool valid = row < nn;
        double acc[kMaxCols][B];
#pragma unroll
        for (int q = 0; q < kMaxCols; q++)
#pragma unroll
            for (int c = 0; c < B; c++) acc[q][c] = 0.0;
        if (valid)
            for (int64_t k = rp[row] + sub; k < rp[row + 1]; k += kRowLanes) {
                const int64_t j = cj[k];
                double a[B * B];
#pragma unroll
                for (int e = 0; e < B * B; e++) a[e] = K[(int64_t)e * nb + k];
#pragma unroll
                for (int q = 0; q < kMaxCols; q++) {
                    if (q >= ncol) break;
                    const double *xq = x + (int64_t)q * n + j * B;
                    double xj[B];
#pragma unroll
                    for (int d = 0; d < B; d++) xj[d] = xq[d];
#pragma unroll
                    for (int c = 0; c < B; c++)
#pragma unroll
                        for (int d = 0; d < B; d++) acc[q][c] = fma(a[c * B + d], xj[d], acc[q][c]);
                }
            }
#pragma unroll
        for (int q = 0; q < kMaxCols; q++) {
            if (q >= ncol) break;
#pragma unroll
            for (int c = 0; c < B; c++)
#pragma unroll
                for (int o = kRowLanes / 2; o > 0; o >>= 1) acc[q][c] += __shfl_xor_sync(0xffffffffu, acc[q][c], o);
        }
        if (valid && sub == 0)
#pragma unroll
            for (int q = 0; q < kMaxCols; q++) {
                if (q >= ncol) break;
#pragma unroll
                for (int c = 0; c < B; c++) out[(int64_t)q * n + row * B + c] = fm[row * B + c] ? acc[q][c] : 0.0;
            }
    }
}

// Up to three column blocks seen as one matrix of ncol columns (column stride n).
struct Cols {
    const double *p[3];
    int w[3];  // columns per block
    int ncol;
    __host__ __device__ const double *col(int j, int64_t n) const {
        int b = 0;
        while (b < 2 && j >= w[b]) { j -= w[b]; b++; }
        return p[b] + (int64_t)j * n;
    }
};

// Per-CTA partial Gram sums over a contiguous row range: items [0, npairs) are S_a' diag(D) S_b (D null:
// weight 1), items [npairs, 2 npairs) are S_a' T_b (when T is given), (a <= b), upper triangle by rows.
// This launch computes items [item0, item0 + kGramItems * blockDim.x) of the nitems; tile rows per
// shared-memory stage.
__global__ void __launch_bounds__(kThreads) k_gram(int64_t n, Cols S, Cols T, const double *D, int nitems,
                                                   int item0, int tile, double *partials) {
    extern __shared__ double sm[];
    const int m = S.ncol;
    const int npairs = m * (m + 1) / 2;
    double *sS = sm;                       // tile x m
    double *sT = sS + tile * m;            // tile x m
    double *sD = sT + tile * m;            // tile
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * per, r1 = min(n, r0 + per);
    // this thread's items and their (a, b, kind); fixed-size loops keep them in registers
    int ia[kGramItems], ib[kGramItems], kind[kGramItems];
    double acc[kGramItems];
#pragma unroll
    for (int q = 0; q < kGramItems; q++) {
        int v = item0 + threadIdx.x + q * blockDim.x, k = 0, a = 0;
        if (v >= npairs) { v -= npairs; k = 1; }
        if (v < npairs)
            while (v >= m - a) { v -= m - a; a++; }
        ia[q] = a; ib[q] = a + v; kind[q] = k; acc[q] = 0.0;
    }
    for (int64_t t0 = r0; t0 < r1; t0 += tile) {
        const int rows = (int)min((int64_t)tile, r1 - t0);
        for (int e = threadIdx.x; e < rows * m; e += blockDim.x) {
            const int r = e / m, j = e % m;
            sS[r * m + j] = S.col(j, n)[t0 + r];
            if (T.ncol) sT[r * m + j] = T.col(j, n)[t0 + r];
        }
        for (int r = threadIdx.x; r < rows; r += blockDim.x) sD[r] = D ? D[t0 + r] : 1.0;
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kGramItems; q++) {
            if (item0 + threadIdx.x + q * blockDim.x >= nitems) break;
            double s = acc[q];
            const double *pa = sS + ia[q];
            const double *pb = (kind[q] ? sT : sS) + ib[q];
            if (kind[q] == 0)
                for (int r = 0; r < rows; r++) s = fma(pa[r * m] * sD[r], pb[r * m], s);
            else
                for (int r = 0; r < rows; r++) s = fma(pa[r * m], pb[r * m], s);
            acc[q] = s;
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < kGramItems; q++) {
        const int w = item0 + threadIdx.x + q * blockDim.x;
        if (w < nitems) partials[(int64_t)blockIdx.x * nitems + w] = acc[q];
    }
}

// sum of the per-CTA partials, CTA order
__global__ void k_gram_reduce(int nctas, int nitems, const double *partials, double *out) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nitems) return;
    double s = 0.0;
    for (int c = 0; c < nctas; c++) s += partials[(int64_t)c * nitems + w];
    out[w] = s;
}

// out (nout columns, nout <= kMaxCols) = S C with C's nout columns read at row stride ldc (C row-major,
// S.ncol rows) into shared memory; thread per row
__global__ void __launch_bounds__(kThreads) k_combo(int64_t n, Cols S, const double *C, int ldc, int nout,
                                                    double *out) {
    extern __shared__ double sC[];
    const int m = S.ncol;
    for (int e = threadIdx.x; e < m * nout; e += blockDim.x) sC[e] = C[(int64_t)(e / nout) * ldc + e % nout];
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double acc[kMaxCols];
#pragma unroll
    for (int c = 0; c < kMaxCols; c++) acc[c] = 0.0;
    for (int j = 0; j < m; j++) {
        const double s = S.col(j, n)[i];
#pragma unroll
        for (int c = 0; c < kMaxCols; c++)
            if (c < nout) acc[c] = fma(s, sC[j * nout + c], acc[c]);
    }
#pragma unroll
    for (int c = 0; c < kMaxCols; c++)
        if (c < nout) out[(int64_t)c * n + i] = acc[c];
}

// R_c = D X_c - theta_c (K X)_c
__global__ void k_resid(int64_t n, int ncol, const double *D, const double *X, const double *KX, const double *theta,
                        double *R) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * ncol) return;
    const int c = (int)(t / n);
    const int64_t i = t % n;
    R[t] = D[i] * X[t] - theta[c] * KX[t];
}

// FP64 column -> FP32 at unknown slots (0 elsewhere), and back
__global__ void k_to_f32(int64_t n, const uint8_t *fm, const double *x, float *y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fm[i] ? (float)x[i] : 0.0f;
}
__global__ void k_from_f32(int64_t n, const uint8_t *fm, const float *x, double *y) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = fm[i] ? (double)x[i] : 0.0;
}

// deterministic start block: a hash of (slot, column) in [-0.5, 0.5) at unknown slots
__global__ void k_init(int64_t n, int ncol, const uint8_t *fm, double *X) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * ncol) return;
    const int64_t i = t % n;
    uint64_t h = (uint64_t)t * 0x9E3779B97F4A7C15ull + 0xD1B54A32D192ED03ull;
    h ^= h >> 31; h *= 0xBF58476D1CE4E5B9ull; h ^= h >> 29; h *= 0x94D049BB133111EBull; h ^= h >> 32;
    X[t] = fm[i] ? ((double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5) : 0.0;
}

// v_c = D phi_c (P's eigenvectors)
__global__ void k_dscale(int64_t n, int ncol, const double *D, const double *X, double *V) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n * ncol) V[t] = D[t % n] * X[t];
}

}  // namespace

namespace {

// eigenvalues w (ascending) and eigenvectors V (row-major, V[i*n + k] = component i of vector k) of
// the symmetric n x n matrix A (row-major), by cyclic Jacobi rotations
void sym_eig(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &V) {
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < n; i++) {
            dg += A[(size_t)i * n + i] * A[(size_t)i * n + i];
            for (int j = i + 1; j < n; j++) off += A[(size_t)i * n + j] * A[(size_t)i * n + j];
        }
        if (!(off > 1e-32 * dg)) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                const double apq = A[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double d = A[(size_t)q * n + q] - A[(size_t)p * n + p], e = 2.0 * apq;
                const double t = std::copysign(1.0, d) * e / (std::fabs(d) + std::sqrt(d * d + e * e));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {  // A <- A J (columns p, q)
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - s * akq;
                    A[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {  // A <- J' A (rows p, q)
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - s * aqk;
                    A[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> o(n);
    std::iota(o.begin(), o.end(), 0);
    std::sort(o.begin(), o.end(), [&](int a, int b) { return A[(size_t)a * n + a] < A[(size_t)b * n + b]; });
    w.resize(n);
    std::vector<double> V2((size_t)n * n);
    for (int k = 0; k < n; k++) {
        w[k] = A[(size_t)o[k] * n + o[k]];
        for (int i = 0; i < n; i++) V2[(size_t)i * n + k] = V[(size_t)i * n + o[k]];
    }
    V.swap(V2);
}

// Rayleigh-Ritz for the k largest eigenpairs of (GA, GB) (packed upper triangles of m x m): C (m x k,
// row-major) and theta (descending).  GB is scaled to unit diagonal and its eigen-directions below
// 1e-12 of the largest are dropped.  False when fewer than k directions remain.
bool rayleigh_ritz(int m, const double *GAp, const double *GBp, int k, std::vector<double> &C,
                   std::vector<double> &theta) {
    std::vector<double> GA((size_t)m * m), GB((size_t)m * m);
    int t = 0;
    for (int a = 0; a < m; a++)
        for (int b = a; b < m; b++, t++) {
            GA[(size_t)a * m + b] = GA[(size_t)b * m + a] = GAp[t];
            GB[(size_t)a * m + b] = GB[(size_t)b * m + a] = GBp[t];
        }
    std::vector<double> s(m);
    for (int a = 0; a < m; a++) s[a] = GB[(size_t)a * m + a] > 0.0 ? 1.0 / std::sqrt(GB[(size_t)a * m + a]) : 0.0;
    std::vector<double> Bs((size_t)m * m);
    for (int a = 0; a < m; a++)
        for (int b = 0; b < m; b++) Bs[(size_t)a * m + b] = s[a] * GB[(size_t)a * m + b] * s[b];
    std::vector<double> lb, Q;
    sym_eig(m, Bs, lb, Q);
    const double lmax = lb.empty() ? 0.0 : lb.back();
    std::vector<int> keep;
    for (int j = 0; j < m; j++)
        if (lb[j] > 1e-12 * lmax) keep.push_back(j);
    const int r = (int)keep.size();
    if (r < k) return false;
    std::vector<double> Z((size_t)m * r);  // diag(s) Q_keep diag(lb^-1/2)
    for (int a = 0; a < m; a++)
        for (int j = 0; j < r; j++) Z[(size_t)a * r + j] = s[a] * Q[(size_t)a * m + keep[j]] / std::sqrt(lb[keep[j]]);
    std::vector<double> AZ((size_t)m * r, 0.0), H((size_t)r * r, 0.0);
    for (int a = 0; a < m; a++)
        for (int j = 0; j < r; j++) {
            double v = 0.0;
            for (int b = 0; b < m; b++) v += GA[(size_t)a * m + b] * Z[(size_t)b * r + j];
            AZ[(size_t)a * r + j] = v;
        }
    for (int i = 0; i < r; i++)
        for (int j = 0; j < r; j++) {
            double v = 0.0;
            for (int a = 0; a < m; a++) v += Z[(size_t)a * r + i] * AZ[(size_t)a * r + j];
            H[(size_t)i * r + j] = v;
        }
    for (int i = 0; i < r; i++)
        for (int j = i + 1; j < r; j++) H[(size_t)i * r + j] = H[(size_t)j * r + i] = 0.5 * (H[(size_t)i * r + j] + H[(size_t)j * r + i]);
    std::vector<double> th, Y;
    sym_eig(r, H, th, Y);
    C.assign((size_t)m * k, 0.0);
    theta.resize(k);
    for (int c = 0; c < k; c++) {
        const int col = r - 1 - c;  // largest first
        theta[c] = th[col];
        for (int a = 0; a < m; a++) {
            double v = 0.0;
            for (int j = 0; j < r; j++) v += Z[(size_t)a * r + j] * Y[(size_t)j * r + col];
            C[(size_t)a * k + c] = v;
        }
    }
    return true;
}

struct ModalWork {
    amr_model *m;
    int64_t n;
    double *partials = nullptr, *gout = nullptr;
    int max_items = 0;
    std::vector<double> host;

    Cols cols(std::initializer_list<std::pair<const double *, int>> blocks) const {
        Cols c{};
        int i = 0;
        for (auto &b : blocks) {
            c.p[i] = b.first;
            c.w[i] = b.second;
            c.ncol += b.second;
            i++;
        }
        for (; i < 3; i++) { c.p[i] = nullptr; c.w[i] = 0; }
        return c;
    }
    // Gram items of S (weights D, or 1 when null) and S'T into host[0 .. nitems): launches of
    // kGramItems * kThreads items each, all into the same per-CTA partials
    void gram(const Cols &S, const Cols &T, const double *D) {
        const int npairs = S.ncol * (S.ncol + 1) / 2;
        const int nitems = T.ncol ? 2 * npairs : npairs;
        if (nitems > max_items) throw AmrError(AMR_EINVAL, "modal block too large");
        const int tile = (int)std::min<size_t>(kGramTile, kGramSmem / (sizeof(double) * (2 * (size_t)S.ncol + 1)));
        const size_t smem = sizeof(double) * (2 * (size_t)tile * S.ncol + tile);
        for (int i0 = 0; i0 < nitems; i0 += kGramItems * kThreads) {
            k_gram<<<kGramCtas, kThreads, smem, m->stream>>>(n, S, T, D, nitems, i0, tile, partials);
            AMR_COUNT(1);
        }
        k_gram_reduce<<<(nitems + kThreads - 1) / kThreads, kThreads, 0, m->stream>>>(kGramCtas, nitems, partials, gout);
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
        host.resize(nitems);
        AMR_CUDA(cudaMemcpyAsync(host.data(), gout, nitems * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
        AMR_CUDA(cudaStreamSynchronize(m->stream));
    }
    // out_c = mask(K x_c), c < ncol, in launches of kMaxCols columns
    void spmv(int ncol, const double *x, double *out) {
        int dev = 0, sms = 0;
        AMR_CUDA(cudaGetDevice(&dev));
        AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const unsigned g = (unsigned)std::max<int64_t>(
            1, std::min<int64_t>((m->nnodes * kRowLanes + kThreads - 1) / kThreads, (int64_t)sms * 8));
        for (int c0 = 0; c0 < ncol; c0 += kMaxCols) {
            const int nc = std::min(kMaxCols, ncol - c0);
            const double *xc = x + (size_t)c0 * n;
            double *oc = out + (size_t)c0 * n;
            if (m->B == 3)
                k_spmv_multi<3><<<g, kThreads, 0, m->stream>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->K64,
                                                               m->free_mask, nc, xc, oc);
            else
                k_spmv_multi<2><<<g, kThreads, 0, m->stream>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->K64,
                                                               m->free_mask, nc, xc, oc);
            AMR_COUNT(1);
        }
        AMR_CUDA(cudaGetLastError());
    }
    // out (nout columns) = S C, C row-major S.ncol x nout, in launches of kMaxCols columns
    void combo(const Cols &S, const double *d_C, int nout, double *out) {
        for (int c0 = 0; c0 < nout; c0 += kMaxCols) {
            const int nc = std::min(kMaxCols, nout - c0);
            const size_t smem = sizeof(double) * (size_t)S.ncol * nc;
            k_combo<<<blocks(n), kThreads, smem, m->stream>>>(n, S, d_C + c0, nout, nc, out + (size_t)c0 * n);
            AMR_COUNT(1);
        }
        AMR_CUDA(cudaGetLastError());
    }
};

}  // namespace

int amr_modal_device(amr_model *m, const amr_modal_params &p, double *omega, double *d_modes_nm,
                     amr_modal_stats *stats) {
    if (m->batch) throw AmrError(AMR_EUNSUPPORTED, "modal analyses of batched parts are not supported");
    if (!m->rho) throw AmrError(AMR_EINVAL, "no density set (amr_set_density)");
    const int nm = p.nmodes;
    auto block_of = [](int q) { return q + std::max(2, (q + 1) / 2); };
    int nmax = 1;
    while (block_of(nmax + 1) <= kMaxBlock) nmax++;
    if (nm < 1 || nm > nmax) throw AmrError(AMR_EINVAL, "nmodes must be in 1.." + std::to_string(nmax));
    const int k = block_of(nm);
    if (m->nu < 3 * k) throw AmrError(AMR_EINVAL, "too few unknown DOFs for " + std::to_string(nm) + " modes");
    {
        std::vector<double> r(m->nelems);
        amr_d2h(m, r.data(), m->rho, m->nelems * sizeof(double));
        for (double v : r)
            if (!(v > 0.0)) throw AmrError(AMR_EINVAL, "mech_modal_solver: density should not be zero");
    }
    cudaStream_t s = m->stream;
    const int64_t n = m->nnodes * m->B;
    AmrEventPair ev;  // destroyed on every exit
    cudaEvent_t t0 = ev.t0, t1 = ev.t1;
    AMR_CUDA(cudaEventRecord(t0, s));
    // K11 (masked K64, its FP32 copy and the multigrid hierarchy) and D
    amr_stiffness(m);
    if (int rc = amr_check_status(m)) throw AmrError(rc, "assembly failed");
    m->K_valid = true;
    amr_mass(m);
    if (int rc = amr_check_status(m)) throw AmrError(rc, "mass assembly failed");
    amr_amg_prepare(m);
    std::vector<double *> buf(12, nullptr);
    float *r32 = nullptr, *z32 = nullptr;
    ModalWork W{m, n};
    auto release = [&]() {
        for (auto &x : buf) amr_free(x);
        amr_free(r32);
        amr_free(z32);
        amr_free(W.partials);
        amr_free(W.gout);
    };
    amr_modal_stats st{};
    try {
        const size_t nk = (size_t)n * k;
        for (int i = 0; i < 11; i++) amr_alloc(&buf[i], nk);
        amr_alloc(&buf[11], n + 2 * k);
        amr_alloc(&r32, n);
        amr_alloc(&z32, n);
        W.max_items = 2 * (3 * k) * (3 * k + 1) / 2;
        amr_alloc(&W.partials, (size_t)kGramCtas * W.max_items);
        amr_alloc(&W.gout, W.max_items);
        double *X = buf[0], *KX = buf[1], *Wv = buf[2], *KW = buf[3], *P = buf[4], *KP = buf[5], *R = buf[6],
               *Xn = buf[7], *KXn = buf[8], *Pn = buf[9], *KPn = buf[10];
        double *D = buf[11], *d_theta = buf[11] + n, *d_C = nullptr;
        amr_alloc(&d_C, (size_t)3 * k * k);
        buf.push_back(d_C);
        if (m->B == 3)
            k_lumped<3><<<blocks(n), kThreads, 0, s>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->M64, m->free_mask, D);
        else
            k_lumped<2><<<blocks(n), kThreads, 0, s>>>(m->nnodes, m->bstride, m->brow_ptr, m->bcol, m->M64, m->free_mask, D);
        AMR_COUNT(1);
        k_init<<<blocks((int64_t)nk), kThreads, 0, s>>>(n, k, m->free_mask, X);
        AMR_COUNT(1);
        W.spmv(k, X, KX);
        std::vector<double> C, theta;
        auto ritz = [&](const Cols &S, const Cols &T) {
            W.gram(S, T, D);
            const int np = S.ncol * (S.ncol + 1) / 2;
            if (!rayleigh_ritz(S.ncol, W.host.data(), W.host.data() + np, k, C, theta))
                throw AmrError(AMR_ENOCONV, "modal: the search space lost rank");
            AMR_CUDA(cudaMemcpyAsync(d_C, C.data(), C.size() * sizeof(double), cudaMemcpyHostToDevice, s));
            AMR_CUDA(cudaMemcpyAsync(d_theta, theta.data(), k * sizeof(double), cudaMemcpyHostToDevice, s));
        };
        ritz(W.cols({{X, k}}), W.cols({{KX, k}}));
        W.combo(W.cols({{X, k}}), d_C, k, Xn);
        W.combo(W.cols({{KX, k}}), d_C, k, KXn);
        std::swap(X, Xn);
        std::swap(KX, KXn);
        bool haveP = false, converged = false;
        double maxres = 0.0;
        int it = 0;
        for (; it < p.max_iters; it++) {
            k_resid<<<blocks((int64_t)nk), kThreads, 0, s>>>(n, k, D, X, KX, d_theta, R);
            AMR_COUNT(1);
            W.gram(W.cols({{R, k}, {KX, k}}), Cols{}, nullptr);
            maxres = 0.0;
            const int m2 = 2 * k;
            auto diag = [&](int a) { return W.host[(size_t)a * m2 - (size_t)a * (a - 1) / 2]; };
            for (int c = 0; c < nm; c++) {
                const double rr = diag(c), kk = diag(k + c);
                const double res = std::sqrt(std::max(rr, 0.0)) / (std::fabs(theta[c]) * std::sqrt(std::max(kk, 1e-300)));
                maxres = std::max(maxres, std::isfinite(res) ? res : 1e300);
            }
            if (maxres <= p.tol) { converged = true; break; }
            // W = T R, one V-cycle per column
            for (int c = 0; c < k; c++) {
                k_to_f32<<<blocks(n), kThreads, 0, s>>>(n, m->free_mask, R + (size_t)c * n, r32);
                amr_amg_vcycle(m, r32, z32);
                k_from_f32<<<blocks(n), kThreads, 0, s>>>(n, m->free_mask, z32, Wv + (size_t)c * n);
                AMR_COUNT(2);
            }
            AMR_CUDA(cudaGetLastError());
            W.spmv(k, Wv, KW);
            // W and P made K-orthogonal to X (X'KX = I): the Rayleigh-Ritz basis stays well conditioned
            {
                Cols S0 = haveP ? W.cols({{X, k}, {Wv, k}, {P, k}}) : W.cols({{X, k}, {Wv, k}});
                Cols T0 = haveP ? W.cols({{KX, k}, {KW, k}, {KP, k}}) : W.cols({{KX, k}, {KW, k}});
                W.gram(S0, T0, D);
                const int m0 = S0.ncol, np0 = m0 * (m0 + 1) / 2;
                auto kx = [&](int a, int b) {  // X_a' K S_b, a < k <= b
                    return W.host[np0 + (size_t)a * m0 - (size_t)a * (a - 1) / 2 + (b - a)];
                };
                for (int blk = 1; blk < (haveP ? 3 : 2); blk++) {
                    std::vector<double> Cp((size_t)2 * k * k, 0.0);  // [-X'KV; I]
                    for (int a = 0; a < k; a++)
                        for (int c = 0; c < k; c++) Cp[(size_t)a * k + c] = -kx(a, blk * k + c);
                    for (int c = 0; c < k; c++) Cp[(size_t)(k + c) * k + c] = 1.0;
                    AMR_CUDA(cudaMemcpyAsync(d_C, Cp.data(), Cp.size() * sizeof(double), cudaMemcpyHostToDevice, s));
                    double *V = blk == 1 ? Wv : P, *KV = blk == 1 ? KW : KP;
                    W.combo(W.cols({{X, k}, {V, k}}), d_C, k, Xn);
                    W.combo(W.cols({{KX, k}, {KV, k}}), d_C, k, KXn);
                    AMR_CUDA(cudaMemcpyAsync(V, Xn, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
                    AMR_CUDA(cudaMemcpyAsync(KV, KXn, (size_t)n * k * sizeof(double), cudaMemcpyDeviceToDevice, s));
                }
            }
            Cols S = haveP ? W.cols({{X, k}, {Wv, k}, {P, k}}) : W.cols({{X, k}, {Wv, k}});
            Cols T = haveP ? W.cols({{KX, k}, {KW, k}, {KP, k}}) : W.cols({{KX, k}, {KW, k}});
            ritz(S, T);
            W.combo(S, d_C, k, Xn);
            Cols St = haveP ? W.cols({{Wv, k}, {P, k}}) : W.cols({{Wv, k}});
            W.combo(St, d_C + (size_t)k * k, k, Pn);
            // K X and K P from the new vectors themselves (no drift of the combined products)
            W.spmv(k, Xn, KXn);
            W.spmv(k, Pn, KPn);
            std::swap(X, Xn);
            std::swap(KX, KXn);
            std::swap(P, Pn);
            std::swap(KP, KPn);
            haveP = true;
        }
        st.iterations = it;
        st.block = k;
        st.max_residual = maxres;
        if (!converged) {
            if (stats) *stats = st;  // the caller sees how far it got
            throw AmrError(AMR_ENOCONV, "modal: LOBPCG did not converge in " + std::to_string(p.max_iters) +
                                            " iterations (largest relative residual " + std::to_string(maxres) + ")");
        }
        for (int c = 0; c < nm; c++) {
            if (!(theta[c] > 0.0)) throw AmrError(AMR_ENOCONV, "modal: fewer than nmodes positive eigenvalues");
            omega[c] = std::sqrt(1.0 / theta[c]);
        }
        // P's eigenvectors D phi (the caller normalises them in the DOF order)
        k_dscale<<<blocks((int64_t)n * nm), kThreads, 0, s>>>(n, nm, D, X, d_modes_nm);
        AMR_COUNT(1);
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
    return AMR_OK;
}
