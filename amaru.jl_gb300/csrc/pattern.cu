// Device construction of the node-block sparsity pattern and of the
// element-entry -> nonzero contribution lists.
//
// Replaces the COO push + SparseArrays.sparse step of mount_K
// (src/mech/mech-solver.jl:78-110) with a pattern built once per model:
//   1. node -> (element, local node) incidence, ordered by element id;
//   2. per node row the sorted unique neighbour nodes (warp-level bitonic sort);
//   3. per nonzero block the list of element-block slots that contribute to it,
//      in element order (the order in which sparse() sums duplicates).
// Everything is integer work and deterministic: atomics only count, and every
// list they fill is sorted afterwards.
#include <algorithm>
#include <climits>

#include "amr_internal.h"

namespace {

constexpr int kScanBlock = 1024;
constexpr int kScanItems = 4;

__global__ void scan_blocks(const int64_t *in, int64_t *out, int64_t *sums, int64_t n) {
    __shared__ int64_t sh[kScanBlock];
    int64_t base = (int64_t)blockIdx.x * kScanBlock * kScanItems + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t t = 0;
    for (int i = 0; i < kScanItems; i++) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        t += v[i];
    }
    sh[threadIdx.x] = t;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        int64_t x = (threadIdx.x >= off) ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += x;
        __syncthreads();
    }
    int64_t run = sh[threadIdx.x] - t;  // exclusive prefix of this thread
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void scan_add(int64_t *out, const int64_t *offs, int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t per = (int64_t)kScanBlock * kScanItems;
    if (i < n) out[i] += offs[i / per];
}

__global__ void set_total(int64_t *out, const int64_t *in, int64_t n) {
    // out[n] = out[n-1] + in[n-1]
    if (n > 0) out[n] = out[n - 1] + in[n - 1];
    else out[0] = 0;
}

// ---- incidence ----
__global__ void inc_count(const int32_t *conn, int64_t nconn, int64_t *cnt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nconn) atomicAdd((unsigned long long *)&cnt[conn[i]], 1ULL);
}

__global__ void inc_fill(const int32_t *conn, const int64_t *conn_ptr, int64_t nelems, const int64_t *perm,
                         const int64_t *inc_ptr, int64_t *fill, int64_t *inc) {
    int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelems) return;
    int64_t p0 = conn_ptr[e], p1 = conn_ptr[e + 1];
    for (int64_t p = p0; p < p1; p++) {
        int32_t n = conn[p];
        unsigned long long slot = atomicAdd((unsigned long long *)&fill[n], 1ULL);
        inc[inc_ptr[n] + (int64_t)slot] = (perm[e] << 8) | (int64_t)(p - p0);  // caller id for ordering
    }
}

__global__ void inc_sort(const int64_t *inc_ptr, int64_t *inc, int64_t nnodes, const int64_t *inv_perm) {
    int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nnodes) return;
    int64_t a = inc_ptr[n], b = inc_ptr[n + 1];
    for (int64_t i = a + 1; i < b; i++) {  // insertion sort: lists are short
        int64_t x = inc[i];
        int64_t j = i - 1;
        while (j >= a && inc[j] > x) { inc[j + 1] = inc[j]; j--; }
        inc[j + 1] = x;
    }
    for (int64_t i = a; i < b; i++) {  // caller id -> sorted element index
        int64_t x = inc[i];
        inc[i] = (inv_perm[x >> 8] << 8) | (x & 0xff);
    }
}

// ---- pattern: warp per node row ----
constexpr int kPatWarps = 4;
constexpr int kPatCap = 1024;  // candidate neighbours per node (power of two)

__device__ int warp_unique_sorted(int32_t *buf, int cnt, int lane) {
    // bitonic sort buf[0..P) with P = next pow2 >= cnt, padded with INT_MAX
    int P = 1;
    while (P < cnt) P <<= 1;
    for (int i = cnt + lane; i < P; i += 32) buf[i] = INT_MAX;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < P; i += 32) {
                int ixj = i ^ j;
                if (ixj > i) {
                    int32_t x = buf[i], y = buf[ixj];
                    bool up = ((i & k) == 0);
                    if ((x > y) == up) { buf[i] = y; buf[ixj] = x; }
                }
            }
            __syncwarp();
        }
    }
    // compact unique values in place (order preserving), return the count
    int total = 0;
    for (int base = 0; base < cnt; base += 32) {
        int i = base + lane;
        bool keep = (i < cnt) && (i == 0 || buf[i] != buf[i - 1]);
        unsigned mask = __ballot_sync(0xffffffffu, keep);
        int pos = total + __popc(mask & ((1u << lane) - 1u));
        int32_t v = (i < cnt) ? buf[i] : 0;
        __syncwarp();
        if (keep) buf[pos] = v;  // pos <= i: never overwrites an unread later entry of this pass
        total += __popc(mask);
        __syncwarp();
    }
    return total;
}

__global__ void pattern_rows(const int32_t *conn, const int64_t *conn_ptr, const int64_t *inc_ptr, const int64_t *inc,
                             int64_t nnodes, const int64_t *brow_ptr, int64_t *row_cnt, int32_t *bcol,
                             int32_t *overflow) {
    __shared__ int32_t sbuf[kPatWarps][kPatCap];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t n = (int64_t)blockIdx.x * kPatWarps + w;
    if (n >= nnodes) return;
    int32_t *buf = sbuf[w];
    int cnt = 0;
    for (int64_t q = inc_ptr[n]; q < inc_ptr[n + 1]; q++) {
        int64_t e = inc[q] >> 8;
        int64_t p0 = conn_ptr[e], ne = conn_ptr[e + 1] - p0;
        if (cnt + ne > kPatCap) { if (lane == 0) atomicExch(overflow, 1); return; }
        for (int b = lane; b < ne; b += 32) buf[cnt + b] = conn[p0 + b];
        cnt += (int)ne;
    }
    __syncwarp();
    int u = warp_unique_sorted(buf, cnt, lane);
    if (row_cnt) {
        if (lane == 0) row_cnt[n] = u;
    } else {
        int64_t o = brow_ptr[n];
        for (int i = lane; i < u; i += 32) bcol[o + i] = buf[i];
    }
}

// ---- contributions: warp per node row, element order ----
__device__ __forceinline__ int64_t find_col(const int32_t *cols, int64_t len, int32_t m) {
    int64_t lo = 0, hi = len;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (cols[mid] < m) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void contrib_rows(const int32_t *conn, const int64_t *conn_ptr, const int64_t *kel_ptr,
                             const int64_t *inc_ptr, const int64_t *inc, int64_t nnodes, const int64_t *brow_ptr,
                             const int32_t *bcol, int64_t *cnt, const int64_t *contrib_ptr, int64_t *contrib) {
    int lane = threadIdx.x & 31;
    int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (n >= nnodes) return;
    int64_t r0 = brow_ptr[n], rl = brow_ptr[n + 1] - r0;
    for (int64_t q = inc_ptr[n]; q < inc_ptr[n + 1]; q++) {
        int64_t e = inc[q] >> 8;
        int a = (int)(inc[q] & 0xff);
        int64_t p0 = conn_ptr[e];
        int ne = (int)(conn_ptr[e + 1] - p0);
        for (int b = lane; b < ne; b += 32) {
            int64_t k = r0 + find_col(bcol + r0, rl, conn[p0 + b]);
            if (contrib == nullptr) {
                cnt[k] += 1;
            } else {
                int64_t slot = kel_ptr[e] + (int64_t)a * ne + b;
                contrib[contrib_ptr[k] + cnt[k]] = slot;
                cnt[k] += 1;
            }
        }
        __syncwarp();  // the next element of this row may hit the same blocks
    }
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---- the gather's block order ----
constexpr int kCountCap = 32;  // contribution counts above it share the last group
__device__ __forceinline__ int count_group(const int64_t *cptr, int64_t k) {
    const int64_t c = cptr[k + 1] - cptr[k];
    return c < kCountCap ? (int)c : kCountCap;
}
__global__ void block_rows(int64_t nnodes, const int64_t *brow_ptr, int32_t *grow) {  // warp per row
    const int lane = threadIdx.x & 31;
    const int64_t n = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (n >= nnodes) return;
    for (int64_t k = brow_ptr[n] + lane; k < brow_ptr[n + 1]; k += 32) grow[k] = (int32_t)n;
}
__global__ void group_hist(int64_t nb, const int64_t *cptr, unsigned long long *hist) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nb) atomicAdd(hist + count_group(cptr, k), 1ull);  // integer counts: the totals are exact
}
__global__ void group_flags(int64_t nb, const int64_t *cptr, int v, int64_t *flags) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nb) flags[k] = count_group(cptr, k) == v;
}
__global__ void group_scatter(int64_t nb, const int64_t *cptr, int v, const int64_t *pos, int64_t off,
                              int32_t *order) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nb && count_group(cptr, k) == v) order[off + pos[k]] = (int32_t)k;
}

}  // namespace

void amr_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s) {
    int64_t per = (int64_t)kScanBlock * kScanItems;
    int64_t nb = (n + per - 1) / per;
    if (nb == 0) nb = 1;
    int64_t *sums = nullptr, *soff = nullptr;
    amr_alloc(&sums, nb);
    amr_alloc(&soff, nb + 1);
    scan_blocks<<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, sums, n);
    AMR_COUNT(1);
    if (nb > 1) {
        amr_scan_i64(sums, soff, nb, s);
        scan_add<<<nblk(n, 256), 256, 0, s>>>(out, soff, n);
        AMR_COUNT(1);
    }
    set_total<<<1, 1, 0, s>>>(out, in, n);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    AMR_CUDA(cudaStreamSynchronize(s));
    amr_free(sums);
    amr_free(soff);
}

void amr_build_pattern(amr_model *m) {
    cudaStream_t s = m->stream;
    int64_t nconn = m->h_conn_ptr.back();
    // 1. incidence
    int64_t *cnt = nullptr, *perm = nullptr, *inv = nullptr;
    amr_alloc(&cnt, m->nnodes);
    amr_alloc(&perm, m->nelems);
    amr_alloc(&inv, m->nelems);
    AMR_CUDA(cudaMemcpyAsync(perm, m->perm.data(), m->nelems * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    AMR_CUDA(cudaMemcpyAsync(inv, m->inv_perm.data(), m->nelems * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    AMR_CUDA(cudaMemsetAsync(cnt, 0, m->nnodes * sizeof(int64_t), s));
    inc_count<<<nblk(nconn, 256), 256, 0, s>>>(m->conn, nconn, cnt);
    AMR_COUNT(1);
    amr_alloc(&m->inc_ptr, m->nnodes + 1);
    amr_scan_i64(cnt, m->inc_ptr, m->nnodes, s);
    m->ninc = nconn;
    amr_alloc(&m->inc, nconn);
    AMR_CUDA(cudaMemsetAsync(cnt, 0, m->nnodes * sizeof(int64_t), s));
    inc_fill<<<nblk(m->nelems, 128), 128, 0, s>>>(m->conn, m->conn_ptr, m->nelems, perm, m->inc_ptr, cnt, m->inc);
    AMR_COUNT(1);
    inc_sort<<<nblk(m->nnodes, 128), 128, 0, s>>>(m->inc_ptr, m->inc, m->nnodes, inv);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());

    // 2. node-block pattern
    int32_t *overflow = nullptr;
    amr_alloc(&overflow, 1);
    AMR_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int32_t), s));
    unsigned gp = nblk(m->nnodes, kPatWarps);
    pattern_rows<<<gp, kPatWarps * 32, 0, s>>>(m->conn, m->conn_ptr, m->inc_ptr, m->inc, m->nnodes, nullptr, cnt,
                                               nullptr, overflow);
    AMR_COUNT(1);
    int32_t hov = 0;
    AMR_CUDA(cudaMemcpyAsync(&hov, overflow, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (hov) throw AmrError(AMR_EUNSUPPORTED, "a node has more than 1024 element-node incidences");
    amr_alloc(&m->brow_ptr, m->nnodes + 1);
    amr_scan_i64(cnt, m->brow_ptr, m->nnodes, s);
    AMR_CUDA(cudaMemcpyAsync(&m->nblocks, m->brow_ptr + m->nnodes, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    if (m->nblocks >= INT32_MAX) throw AmrError(AMR_EUNSUPPORTED, "more than 2^31 nonzero blocks");
    m->bstride = (m->nblocks + 7) / 8 * 8 + 8;
    amr_alloc(&m->bcol, m->bstride);
    pattern_rows<<<gp, kPatWarps * 32, 0, s>>>(m->conn, m->conn_ptr, m->inc_ptr, m->inc, m->nnodes, m->brow_ptr,
                                               nullptr, m->bcol, overflow);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());

    // 3. contributions, element order per block
    int64_t *bcnt = nullptr;
    amr_alloc(&bcnt, m->nblocks);
    AMR_CUDA(cudaMemsetAsync(bcnt, 0, m->nblocks * sizeof(int64_t), s));
    unsigned gc = nblk(m->nnodes * 32, 256);
    contrib_rows<<<gc, 256, 0, s>>>(m->conn, m->conn_ptr, m->kel_ptr, m->inc_ptr, m->inc, m->nnodes, m->brow_ptr,
                                    m->bcol, bcnt, nullptr, nullptr);
    AMR_COUNT(1);
    amr_alloc(&m->contrib_ptr, m->nblocks + 1);
    amr_scan_i64(bcnt, m->contrib_ptr, m->nblocks, s);
    AMR_CUDA(cudaMemcpyAsync(&m->ncontrib, m->contrib_ptr + m->nblocks, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    amr_alloc(&m->contrib, m->ncontrib);
    AMR_CUDA(cudaMemsetAsync(bcnt, 0, m->nblocks * sizeof(int64_t), s));
    contrib_rows<<<gc, 256, 0, s>>>(m->conn, m->conn_ptr, m->kel_ptr, m->inc_ptr, m->inc, m->nnodes, m->brow_ptr,
                                    m->bcol, bcnt, m->contrib_ptr, m->contrib);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    // 4. the gather's order: blocks grouped by contribution count, block order kept within a group (a
    // deterministic scan per non-empty group), and each block's row
    amr_alloc(&m->grow, std::max<int64_t>(m->nblocks, 1));
    amr_alloc(&m->gorder, std::max<int64_t>(m->nblocks, 1));
    block_rows<<<gc, 256, 0, s>>>(m->nnodes, m->brow_ptr, m->grow);
    AMR_COUNT(1);
    {
        unsigned long long *hist = nullptr;
        amr_alloc(&hist, kCountCap + 1);
        AMR_CUDA(cudaMemsetAsync(hist, 0, (kCountCap + 1) * sizeof(unsigned long long), s));
        group_hist<<<nblk(m->nblocks, 256), 256, 0, s>>>(m->nblocks, m->contrib_ptr, hist);
        AMR_COUNT(1);
        unsigned long long hh[kCountCap + 1];
        AMR_CUDA(cudaMemcpyAsync(hh, hist, sizeof hh, cudaMemcpyDeviceToHost, s));
        AMR_CUDA(cudaStreamSynchronize(s));
        amr_free(hist);
        int64_t *flags = nullptr, *pos = nullptr;
        amr_alloc(&flags, std::max<int64_t>(m->nblocks, 1));
        amr_alloc(&pos, m->nblocks + 1);
        int64_t off = 0;
        for (int v = 0; v <= kCountCap; v++) {
            if (hh[v] == 0) continue;
            group_flags<<<nblk(m->nblocks, 256), 256, 0, s>>>(m->nblocks, m->contrib_ptr, v, flags);
            AMR_COUNT(1);
            amr_scan_i64(flags, pos, m->nblocks, s);
            group_scatter<<<nblk(m->nblocks, 256), 256, 0, s>>>(m->nblocks, m->contrib_ptr, v, pos, off, m->gorder);
            AMR_COUNT(1);
            off += (int64_t)hh[v];
        }
        AMR_CUDA(cudaGetLastError());
        AMR_CUDA(cudaStreamSynchronize(s));
        amr_free(flags);
        amr_free(pos);
    }
    // host copy of the pattern (export in the reference layout)
    m->h_brow_ptr.resize(m->nnodes + 1);
    m->h_bcol.resize(m->nblocks);
    AMR_CUDA(cudaMemcpyAsync(m->h_brow_ptr.data(), m->brow_ptr, (m->nnodes + 1) * sizeof(int64_t),
                             cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaMemcpyAsync(m->h_bcol.data(), m->bcol, m->nblocks * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    amr_free(bcnt);
    amr_free(cnt);
    amr_free(perm);
    amr_free(inv);
    amr_free(overflow);
}
