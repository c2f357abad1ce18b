// Nodal output recovery of the IP fields on the device: nodal_patch_recovery
// (src/fe-model.jl:504-702) as called by update_output_data! (:341-427) and
// get_node_and_elem_vals (:430-485).
//
// Structure (once per model, host): outer facets -> boundary nodes; one patch per
// corner node with the elements that have it as a corner (interior nodes), and the
// reference's fallback to boundary patches of >= 3, 2, 1 elements for boundary
// nodes that no interior patch reaches; per patch and per set of materials sharing
// a field ("mask"), one fit task: its elements, IPs and nodes (unique, in order of
// appearance).  Contribution lists give every node its task slots in patch order,
// the order of the reference's V_vals[node] += V[i].
//
// Values (per call, device):
//   k_ip_fields   thread per IP: ip_state_vals of the IP's material
//                 (linear-elastic.jl:140-164, von-mises.jl:159-168,330-341,
//                 drucker-prager.jl:152-163 over tensors.jl:162-215)
//   k_patch_fit   warp per task: the least-squares polynomial of reg_terms
//                 (fe-model.jl:488-501) through the task's IP values, evaluated at
//                 its nodes.  The regression runs in patch-centred coordinates
//                 scaled per axis, which span the same polynomial space as the
//                 global x, y, z the reference uses, so the fitted values are the
//                 same; the normal equations are solved by Cholesky when they are
//                 well conditioned.
//   k_patch_svd   warp per task the Cholesky path left (rank-deficient or badly
//                 conditioned patches): one-sided Jacobi SVD of the regression
//                 matrix in the reference's own global coordinates and the
//                 pseudo-inverse with LinearAlgebra.pinv's cut-off (singular values
//                 above eps * min(m, n) * max).  A minimum-norm solution depends on
//                 the basis, so this path keeps the reference's.
//   k_node_avg    thread per (node, field): the sum over the node's slots in patch
//                 order divided by their count; nodes no patch reaches (0/0) and NaN
//                 results give 0, as V_vals[isnan.(V_vals)] .= 0.0.
// nodal_local_recovery (fe-model.jl:705-747) only recovers joint elements, none of
// which are on this path, so it adds no field.
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <numeric>
#include <vector>

#include "amr_internal.h"

namespace {

constexpr double SR2 = 1.4142135623730951;  // src/tools/constants.jl:3
constexpr int kFitWarps = 4;                 // warps per CTA of the fit kernels
constexpr int kTermPad = 8;                  // doubles per regression row (<= 7 terms)
constexpr int kRedStride = 29;               // Gram partials per lane in shared memory (28 + pad)
constexpr int kInvDiag = 72;                 // offset of the reciprocal Cholesky pivots in the factor area

// ---------------------------------------------------------------------------
// host tables
// ---------------------------------------------------------------------------
struct FacetTab {
    int nf, np;
    int idx[6][8];
};

// local node lists of each cell's facets (src/shape/solids3d.jl, solids2d.jl facet_idxs)
const FacetTab *facet_table(int shape) {
    static const FacetTab hex8 = {6, 4, {{0, 4, 7, 3}, {1, 2, 6, 5}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 3, 2, 1}, {4, 5, 6, 7}}};
    static const FacetTab hex20 = {6, 8, {{0, 4, 7, 3, 16, 15, 19, 11}, {1, 2, 6, 5, 9, 18, 13, 17},
                                          {0, 1, 5, 4, 8, 17, 12, 16}, {2, 3, 7, 6, 10, 19, 14, 18},
                                          {0, 3, 2, 1, 11, 10, 9, 8}, {4, 5, 6, 7, 12, 13, 14, 15}}};
    static const FacetTab tet4 = {4, 3, {{0, 3, 2}, {0, 1, 3}, {0, 2, 1}, {1, 2, 3}}};
    static const FacetTab tet10 = {4, 6, {{0, 3, 2, 7, 9, 6}, {0, 1, 3, 4, 8, 7}, {0, 2, 1, 6, 5, 4}, {1, 2, 3, 5, 9, 8}}};
    static const FacetTab quad4 = {4, 2, {{0, 1}, {1, 2}, {2, 3}, {3, 0}}};
    static const FacetTab quad8 = {4, 3, {{0, 1, 4}, {1, 2, 5}, {2, 3, 6}, {3, 0, 7}}};
    static const FacetTab tri3 = {3, 2, {{0, 1}, {1, 2}, {2, 0}}};
    static const FacetTab tri6 = {3, 3, {{0, 1, 3}, {1, 2, 4}, {2, 0, 5}}};
    switch (shape) {
    case AMR_HEX8: return &hex8;
    case AMR_HEX20: return &hex20;
    case AMR_TET4: return &tet4;
    case AMR_TET10: return &tet10;
    case AMR_QUAD4: return &quad4;
    case AMR_QUAD8: case AMR_QUAD9: return &quad8;
    case AMR_TRI3: return &tri3;
    case AMR_TRI6: return &tri6;
    }
    return nullptr;
}

// corner points of the cell's basic shape (elem.shape.basic_shape.npoints)
int corners(int shape) {
    switch (shape) {
    case AMR_HEX8: case AMR_HEX20: return 8;
    case AMR_TET4: case AMR_TET10: case AMR_QUAD4: case AMR_QUAD8: case AMR_QUAD9: return 4;
    case AMR_TRI3: case AMR_TRI6: return 3;
    }
    return 0;
}

// keys of ip_state_vals for one material under the model's stress model, in the reference's order
int field_codes(int stressmodel, int mat, int32_t *out) {
    int n = 0;
    const bool d3 = stressmodel == AMR_D3;
    if (stressmodel == AMR_AXISYMMETRIC) {  // σrr σyy σtt σry σvm εrr εyy εtt εry (tensors.jl:182-193)
        const int32_t ax[9] = {AMR_FIELD_SXX, AMR_FIELD_SYY, AMR_FIELD_SZZ, AMR_FIELD_SXY, AMR_FIELD_SVM,
                               AMR_FIELD_EXX, AMR_FIELD_EYY, AMR_FIELD_EZZ, AMR_FIELD_EXY};
        for (int k = 0; k < 9; k++) out[n++] = ax[k];
        if (mat == AMR_VON_MISES) out[n++] = AMR_FIELD_EP;
        else if (mat == AMR_DRUCKER_PRAGER) { out[n++] = AMR_FIELD_EPA; out[n++] = AMR_FIELD_J1; out[n++] = AMR_FIELD_SRJ2D; }
        return n;
    }
    for (int c = AMR_FIELD_SXX; c <= AMR_FIELD_S1; c++) out[n++] = c;
    if (d3) out[n++] = AMR_FIELD_S2;
    out[n++] = AMR_FIELD_S3;
    out[n++] = AMR_FIELD_EXX; out[n++] = AMR_FIELD_EYY; out[n++] = AMR_FIELD_EZZ;
    if (d3) { out[n++] = AMR_FIELD_EYZ; out[n++] = AMR_FIELD_EXZ; }
    out[n++] = AMR_FIELD_EXY;
    if (mat == AMR_VON_MISES) {
        out[n++] = AMR_FIELD_EP;
        if (stressmodel == AMR_PLANESTRESS) { out[n++] = AMR_FIELD_J1; out[n++] = AMR_FIELD_SRJ2D; }
    } else if (mat == AMR_DRUCKER_PRAGER) {
        out[n++] = AMR_FIELD_EPA; out[n++] = AMR_FIELD_J1; out[n++] = AMR_FIELD_SRJ2D;
    }
    return n;
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double j2(const double *s) {  // src/tools/tensors.jl:24-27, operations as written
    const double t11 = s[0], t22 = s[1], t33 = s[2];
    const double t23 = __ddiv_rn(s[3], SR2), t13 = __ddiv_rn(s[4], SR2), t12 = __ddiv_rn(s[5], SR2);
    const double a = __dsub_rn(t11, t22), b = __dsub_rn(t22, t33), c = __dsub_rn(t33, t11);
    double q = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
    q = __dmul_rn(1.0 / 6.0, q);
    q = __dadd_rn(q, __dmul_rn(t23, t23));
    q = __dadd_rn(q, __dmul_rn(t13, t13));
    return __dadd_rn(q, __dmul_rn(t12, t12));
}

// eigenvalues of the symmetric 3x3 tensor (eigvals, src/tools/tensors.jl:80-91), largest first:
// cyclic Jacobi rotations until the off-diagonal part is below rounding
__device__ void eig3(const double *s, double *L) {
    double a[3][3];
    a[0][0] = s[0]; a[1][1] = s[1]; a[2][2] = s[2];
    a[1][2] = a[2][1] = s[3] / SR2;
    a[0][2] = a[2][0] = s[4] / SR2;
    a[0][1] = a[1][0] = s[5] / SR2;
    for (int sweep = 0; sweep < 16; sweep++) {
        const double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        const double dg = a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (!(off > 1e-36 * dg)) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                const double apq = a[p][q];
                if (apq == 0.0) continue;
                // tangent of the rotation angle, the smaller root of t^2 + 2 theta t - 1 = 0 with
                // theta = d / e: t = sign(d) e / (|d| + sqrt(d^2 + e^2))
                const double d = a[q][q] - a[p][p], e = 2.0 * apq;
                const double t = copysign(1.0, d) * e / (fabs(d) + sqrt(d * d + e * e));
                const double c = rsqrt(t * t + 1.0), sn = t * c;
                a[p][p] -= t * apq;
                a[q][q] += t * apq;
                a[p][q] = a[q][p] = 0.0;
                const int r = 3 - p - q;
                const double arp = a[r][p], arq = a[r][q];
                a[r][p] = a[p][r] = c * arp - sn * arq;
                a[r][q] = a[q][r] = sn * arp + c * arq;
            }
    }
    double x = a[0][0], y = a[1][1], z = a[2][2], u;
    if (x < y) { u = x; x = y; y = u; }
    if (y < z) { u = y; y = z; z = u; }
    if (x < y) { u = x; x = y; y = u; }
    L[0] = x; L[1] = y; L[2] = z;
}

// IP global coordinates C' N (setquadrature!, src/element.jl:160-164), one group
__global__ void k_ip_coords(int64_t first, int64_t count, int nen, int nip, int ndim, const double *Ntab,
                            const int64_t *conn_ptr, const int32_t *conn, const int64_t *ip_ptr,
                            const double *coords, double *ipx) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count * nip) return;
    const int64_t e = first + t / nip;
    const int q = (int)(t % nip);
    const int32_t *cn = conn + conn_ptr[e];
    const double *N = Ntab + (int64_t)q * nen;
    double x[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < nen; a++) {
        const double *c = coords + 3 * (int64_t)cn[a];
        for (int d = 0; d < ndim; d++) x[d] += c[d] * N[a];
    }
    double *o = ipx + 3 * (ip_ptr[e] + q);
    o[0] = x[0]; o[1] = x[1]; o[2] = x[2];
}

// ip_state_vals of every IP into ipv[gi][field]
__global__ void k_ip_fields(int64_t nip_total, int stressmodel, const int32_t *ip_elem, const int32_t *mat_type,
                            const double *st, const int32_t *fmap, int nf, double *ipv) {
    int64_t gi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gi >= nip_total) return;
    const int mat = mat_type[ip_elem[gi]];
    double s[6], e[6];
    for (int k = 0; k < 6; k++) {
        s[k] = st[(int64_t)(AMR_ST_SIG + k) * nip_total + gi];
        e[k] = st[(int64_t)(AMR_ST_EPS + k) * nip_total + gi];
    }
    const double epa = st[(int64_t)AMR_ST_EPA * nip_total + gi];
    double v[AMR_NFIELD_CODES];
    const double J2 = j2(s);
    double L[3];
    eig3(s, L);
    v[AMR_FIELD_SXX] = s[0]; v[AMR_FIELD_SYY] = s[1]; v[AMR_FIELD_SZZ] = s[2];
    v[AMR_FIELD_SYZ] = __ddiv_rn(s[3], SR2); v[AMR_FIELD_SXZ] = __ddiv_rn(s[4], SR2);
    v[AMR_FIELD_SXY] = __ddiv_rn(s[5], SR2);
    v[AMR_FIELD_SVM] = __dsqrt_rn(__dmul_rn(3.0, J2));
    v[AMR_FIELD_S1] = L[0]; v[AMR_FIELD_S2] = L[1]; v[AMR_FIELD_S3] = L[2];
    v[AMR_FIELD_EXX] = e[0]; v[AMR_FIELD_EYY] = e[1]; v[AMR_FIELD_EZZ] = e[2];
    v[AMR_FIELD_EYZ] = __ddiv_rn(e[3], SR2); v[AMR_FIELD_EXZ] = __ddiv_rn(e[4], SR2);
    v[AMR_FIELD_EXY] = __ddiv_rn(e[5], SR2);
    v[AMR_FIELD_EP] = epa; v[AMR_FIELD_EPA] = epa;
    v[AMR_FIELD_J1] = __dadd_rn(__dadd_rn(s[0], s[1]), s[2]);
    v[AMR_FIELD_SRJ2D] = __dsqrt_rn(J2);
    (void)stressmodel;
    const int32_t *fm = fmap + mat * AMR_NFIELD_CODES;
    double *o = ipv + gi * nf;
#pragma unroll
    for (int c = 0; c < AMR_NFIELD_CODES; c++)
        if (fm[c] >= 0) o[fm[c]] = v[c];
}

// number of regression terms for m IPs (fe-model.jl:633-639)
template <int DIM>
__device__ __forceinline__ int nterms(int m) {
    if (DIM == 3) return m >= 7 ? 7 : (m >= 4 ? 4 : 1);
    return m >= 6 ? 6 : (m >= 4 ? 4 : (m >= 3 ? 3 : 1));
}

// reg_terms (fe-model.jl:488-501) of scaled coordinates
template <int DIM>
__device__ __forceinline__ void terms(const double *x, int nt, double *p) {
    p[0] = 1.0;
    if (DIM == 3) {
        if (nt >= 4) { p[1] = x[0]; p[2] = x[1]; p[3] = x[2]; }
        if (nt >= 7) { p[4] = x[0] * x[1]; p[5] = x[1] * x[2]; p[6] = x[0] * x[2]; }
    } else {
        if (nt >= 3) { p[1] = x[0]; p[2] = x[1]; }
        if (nt >= 4) p[3] = x[0] * x[1];
        if (nt >= 6) { p[4] = x[0] * x[0]; p[5] = x[1] * x[1]; }
    }
}

// index of entry (a, b), a <= b, of the packed upper triangle of a 7 x 7 matrix stored row by row
__device__ __forceinline__ int packed(int a, int b) { return a * 7 - a * (a - 1) / 2 + (b - a); }

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

struct FitArgs {
    int64_t ntasks;
    const int64_t *t_elem_ptr, *t_node_ptr;
    const int32_t *t_elem, *t_node, *t_mask, *t_center, *t_m;
    const int32_t *mask_nf, *mask_fields;  // mask_fields: nmask x AMR_NFIELD_CODES
    const int64_t *ip_ptr;
    const double *ipx, *coords, *ipv;
    int nf, m_max, e_max;
    double *vst;
    int32_t *t_flag;
};

// per-warp shared memory, in doubles
__host__ __device__ inline int64_t fit_warp_doubles(int m_max, int e_max) {
    return (int64_t)m_max * kTermPad     // scaled regression rows
           + m_max                       // IP global indices
           + 32 * kRedStride             // Gram partials
           + AMR_NFIELD_CODES * kTermPad // right-hand sides / coefficients
           + 2 * kTermPad * kTermPad     // Cholesky factor / right singular vectors
           + (e_max + 2) / 2 + 1;        // element IP offsets (int32)
}

struct WarpMem {
    double *phi, *red, *bA, *R;
    int64_t *gidx;
    int32_t *eoff;
};

__device__ __forceinline__ WarpMem warp_mem(double *smem, int warp, int m_max, int e_max) {
    WarpMem w;
    double *b = smem + warp * fit_warp_doubles(m_max, e_max);
    w.phi = b; b += (int64_t)m_max * kTermPad;
    w.gidx = (int64_t *)b; b += m_max;
    w.red = b; b += 32 * kRedStride;
    w.bA = b; b += AMR_NFIELD_CODES * kTermPad;
    w.R = b; b += 2 * kTermPad * kTermPad;
    w.eoff = (int32_t *)b;
    return w;
}

// Loads the task's IPs: global indices, scaled regression rows; returns the number of terms, the centre c
// of the coordinates and their reciprocal scales h (x_scaled = (x - c) * h).
// raw: the reference's own basis (global coordinates, no centring or scaling)
template <int DIM>
__device__ int load_task(const FitArgs &A, int64_t t, const WarpMem &w, int lane, double *c, double *h, bool raw) {
    const int m = A.t_m[t];
    const int nt = nterms<DIM>(m);
    const int64_t e0 = A.t_elem_ptr[t], ne = A.t_elem_ptr[t + 1] - e0;
    if (lane == 0) {
        int32_t o = 0;
        for (int64_t j = 0; j < ne; j++) {
            w.eoff[j] = o;
            const int32_t e = A.t_elem[e0 + j];
            o += (int32_t)(A.ip_ptr[e + 1] - A.ip_ptr[e]);
        }
        w.eoff[ne] = o;
    }
    __syncwarp();
    const int32_t cn = A.t_center[t];
    for (int d = 0; d < 3; d++) c[d] = A.coords[3 * (int64_t)cn + d];
    double hm[3] = {0.0, 0.0, 0.0};
    for (int i = lane; i < m; i += 32) {
        int lo = 0, hi = (int)ne - 1;  // element j with eoff[j] <= i < eoff[j+1]
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (w.eoff[mid] <= i) lo = mid; else hi = mid - 1;
        }
        const int64_t gi = A.ip_ptr[A.t_elem[e0 + lo]] + (i - w.eoff[lo]);
        w.gidx[i] = gi;
        for (int d = 0; d < DIM; d++) hm[d] = fmax(hm[d], fabs(A.ipx[3 * gi + d] - c[d]));
    }
    for (int d = 0; d < DIM; d++) {  // h holds the reciprocal scale from here on
        const double hd = warp_max_d(hm[d]);
        h[d] = (!(hd > 0.0) || raw) ? 1.0 : 1.0 / hd;
    }
    if (raw) c[0] = c[1] = c[2] = 0.0;
    __syncwarp();
    for (int i = lane; i < m; i += 32) {
        double x[3], p[kTermPad];
        const int64_t gi = w.gidx[i];
        for (int d = 0; d < DIM; d++) x[d] = (A.ipx[3 * gi + d] - c[d]) * h[d];
        terms<DIM>(x, nt, p);
        for (int k = 0; k < nt; k++) w.phi[i * kTermPad + k] = p[k];
    }
    __syncwarp();
    return nt;
}

// values at the task's nodes from the coefficients in w.bA (field k of the mask at bA[k*kTermPad])
template <int DIM>
__device__ void write_nodes(const FitArgs &A, int64_t t, const WarpMem &w, int lane, int nt, int nfm,
                            const int32_t *flds, const double *c, const double *h) {
    const int64_t s0 = A.t_node_ptr[t], n = A.t_node_ptr[t + 1] - s0;
    for (int64_t j = lane; j < n; j += 32) {
        const int32_t node = A.t_node[s0 + j];
        double x[3], p[kTermPad];
        for (int d = 0; d < DIM; d++) x[d] = (A.coords[3 * (int64_t)node + d] - c[d]) * h[d];
        terms<DIM>(x, nt, p);
        double *o = A.vst + (s0 + j) * A.nf;
        for (int k = 0; k < nfm; k++) {
            double v = 0.0;
            for (int q = 0; q < nt; q++) v = fma(p[q], w.bA[k * kTermPad + q], v);
            o[flds[k]] = v;
        }
    }
}

// b[k][q] = sum_i phi[i][q] * W_k(i) for the mask's fields, lanes over (field, term) pairs
__device__ void field_moments(const FitArgs &A, const WarpMem &w, int lane, int m, int nt, int nfm,
                              const int32_t *flds) {
    const int P = nfm * nt;
    for (int p0 = 0; p0 < P; p0 += 32) {
        const int p = p0 + lane;
        double acc = 0.0;
        if (p < P) {
            const int k = p / nt, q = p % nt;
            const int f = flds[k];
            for (int i = 0; i < m; i++) acc = fma(w.phi[i * kTermPad + q], A.ipv[w.gidx[i] * A.nf + f], acc);
            w.bA[k * kTermPad + q] = acc;
        }
    }
    __syncwarp();
}

template <int DIM>
__global__ void __launch_bounds__(32 * kFitWarps) k_patch_fit(FitArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const WarpMem w = warp_mem(smem, warp, A.m_max, A.e_max);
    for (int64_t t = (int64_t)blockIdx.x * kFitWarps + warp; t < A.ntasks; t += (int64_t)gridDim.x * kFitWarps) {
        double c[3], h[3];
        const int m = A.t_m[t];
        const int nt = load_task<DIM>(A, t, w, lane, c, h, false);
        // Gram matrix of the scaled rows: lane partials, then lane k sums entry k over the lanes
        double g[28];
#pragma unroll
        for (int k = 0; k < 28; k++) g[k] = 0.0;
        for (int i = lane; i < m; i += 32) {
            const double *p = w.phi + i * kTermPad;
            int k = 0;
#pragma unroll
            for (int a = 0; a < 7; a++)
#pragma unroll
                for (int b = a; b < 7; b++, k++)
                    if (b < nt) g[k] = fma(p[a], p[b], g[k]);
        }
#pragma unroll
        for (int k = 0; k < 28; k++) w.red[lane * kRedStride + k] = g[k];
        __syncwarp();
        if (lane < 28) {
            double s = 0.0;
            for (int l = 0; l < 32; l++) s += w.red[l * kRedStride + lane];
            w.bA[lane] = s;  // packed upper triangle, row by row (bA is free until the moments)
        }
        __syncwarp();
        // Cholesky G = R'R: the pivots on every lane, row j's off-diagonal entries on lanes i > j.
        // R[j][i] at R[j*kTermPad+i], the reciprocal pivots at R[kInvDiag+j]
        const double *G = w.bA;
        double *R = w.R;
        bool ok = true;
        double dmin = DBL_MAX, dmax = 0.0;
#pragma unroll
        for (int j = 0; j < 7; j++) {
            if (j >= nt) break;
            double d = G[packed(j, j)];
#pragma unroll
            for (int q = 0; q < 7; q++)
                if (q < j) d -= R[q * kTermPad + j] * R[q * kTermPad + j];
            if (!(d > 0.0)) { ok = false; break; }
            const double r = sqrt(d), ir = 1.0 / r;
            dmin = fmin(dmin, r);
            dmax = fmax(dmax, r);
            if (lane > j && lane < nt) {
                double v = G[packed(j, lane)];
#pragma unroll
                for (int q = 0; q < 7; q++)
                    if (q < j) v -= R[q * kTermPad + j] * R[q * kTermPad + lane];
                R[j * kTermPad + lane] = v * ir;
            } else if (lane == j) {
                R[j * kTermPad + j] = r;
                R[kInvDiag + j] = ir;
            }
            __syncwarp();
        }
        // the normal equations square the condition number: patches conditioned worse than 1e4 go to
        // the SVD path
        if (ok && !(dmin > 1e-4 * dmax)) ok = false;
        if (lane == 0) A.t_flag[t] = ok ? 0 : 1;
        if (!ok) {
            __syncwarp();
            continue;
        }
        const int mk = A.t_mask[t];
        const int nfm = A.mask_nf[mk];
        const int32_t *flds = A.mask_fields + mk * AMR_NFIELD_CODES;
        field_moments(A, w, lane, m, nt, nfm, flds);
        // coefficients: R'y = b, R a = y (lane per field)
        if (lane < nfm) {
            double y[7];
            double *b = w.bA + lane * kTermPad;
#pragma unroll
            for (int j = 0; j < 7; j++) {
                if (j < nt) {
                    double v = b[j];
#pragma unroll
                    for (int q = 0; q < 7; q++)
                        if (q < j) v -= R[q * kTermPad + j] * y[q];
                    y[j] = v * R[kInvDiag + j];
                }
            }
#pragma unroll
            for (int j = 6; j >= 0; j--) {
                if (j < nt) {
                    double v = y[j];
#pragma unroll
                    for (int q = 0; q < 7; q++)
                        if (q > j && q < nt) v -= R[j * kTermPad + q] * y[q];
                    y[j] = v * R[kInvDiag + j];
                }
            }
#pragma unroll
            for (int j = 0; j < 7; j++)
                if (j < nt) b[j] = y[j];
        }
        __syncwarp();
        write_nodes<DIM>(A, t, w, lane, nt, nfm, flds, c, h);
        __syncwarp();
    }
}

// Rank-deficient or ill-conditioned tasks: pinv through a one-sided Jacobi SVD of the rows in global coordinates.
template <int DIM>
__global__ void __launch_bounds__(32 * kFitWarps) k_patch_svd(FitArgs A) {
    extern __shared__ double smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const WarpMem w = warp_mem(smem, warp, A.m_max, A.e_max);
    for (int64_t t = (int64_t)blockIdx.x * kFitWarps + warp; t < A.ntasks; t += (int64_t)gridDim.x * kFitWarps) {
        if (!A.t_flag[t]) continue;
        double c[3], h[3];
        const int m = A.t_m[t];
        const int nt = load_task<DIM>(A, t, w, lane, c, h, true);
        double *V = w.R;  // nt x nt right singular vectors, row-major
        if (lane < kTermPad * kTermPad) {
            V[lane] = (lane / kTermPad == lane % kTermPad) ? 1.0 : 0.0;
            V[lane + 32] = ((lane + 32) / kTermPad == (lane + 32) % kTermPad) ? 1.0 : 0.0;
        }
        __syncwarp();
        for (int sweep = 0; sweep < 60; sweep++) {
            bool rotated = false;
            for (int p = 0; p < nt - 1; p++)
                for (int q = p + 1; q < nt; q++) {
                    double al = 0.0, be = 0.0, ga = 0.0;
                    for (int i = lane; i < m; i += 32) {
                        const double ap = w.phi[i * kTermPad + p], aq = w.phi[i * kTermPad + q];
                        al = fma(ap, ap, al);
                        be = fma(aq, aq, be);
                        ga = fma(ap, aq, ga);
                    }
                    al = warp_sum_d(al);
                    be = warp_sum_d(be);
                    ga = warp_sum_d(ga);
                    if (!(fabs(ga) > DBL_EPSILON * sqrt(al * be))) continue;
                    rotated = true;
                    const double z = (be - al) / (2.0 * ga);
                    const double tn = fabs(z) > 1e150 ? 0.5 / z : copysign(1.0, z) / (fabs(z) + sqrt(1.0 + z * z));
                    const double cs = 1.0 / sqrt(1.0 + tn * tn), sn = cs * tn;
                    for (int i = lane; i < m; i += 32) {
                        const double ap = w.phi[i * kTermPad + p], aq = w.phi[i * kTermPad + q];
                        w.phi[i * kTermPad + p] = cs * ap - sn * aq;
                        w.phi[i * kTermPad + q] = sn * ap + cs * aq;
                    }
                    if (lane < nt) {
                        const double vp = V[lane * kTermPad + p], vq = V[lane * kTermPad + q];
                        V[lane * kTermPad + p] = cs * vp - sn * vq;
                        V[lane * kTermPad + q] = sn * vp + cs * vq;
                    }
                    __syncwarp();
                }
            if (!rotated) break;
        }
        // singular values (column norms) and LinearAlgebra.pinv's cut-off
        double sig2[7], smax = 0.0;
        for (int k = 0; k < nt; k++) {
            double s = 0.0;
            for (int i = lane; i < m; i += 32) s = fma(w.phi[i * kTermPad + k], w.phi[i * kTermPad + k], s);
            sig2[k] = warp_sum_d(s);
            smax = fmax(smax, sqrt(sig2[k]));
        }
        const double tol = DBL_EPSILON * (double)min(m, nt) * smax;
        const int mk = A.t_mask[t];
        const int nfm = A.mask_nf[mk];
        const int32_t *flds = A.mask_fields + mk * AMR_NFIELD_CODES;
        field_moments(A, w, lane, m, nt, nfm, flds);  // b[k][q] = a_q . W_k (a_q = sigma_q u_q)
        if (lane < nfm) {
            double y[7];
            double *b = w.bA + lane * kTermPad;
            for (int q = 0; q < nt; q++) y[q] = (sqrt(sig2[q]) > tol) ? b[q] / sig2[q] : 0.0;
            for (int r = 0; r < nt; r++) {
                double v = 0.0;
                for (int q = 0; q < nt; q++) v = fma(V[r * kTermPad + q], y[q], v);
                b[r] = v;
            }
        }
        __syncwarp();
        write_nodes<DIM>(A, t, w, lane, nt, nfm, flds, c, h);
        __syncwarp();
    }
}

// V[f][node] = (sum over the node's slots, in patch order) / count; 0 where that is NaN
__global__ void k_node_avg(int64_t nnodes, int nf, const int32_t *field_mask, const int64_t *c_ptr,
                           const int64_t *c_slot, const double *vst, double *V) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nnodes * nf) return;
    const int f = (int)(t % nf);
    const int64_t n = t / nf;
    const int64_t *cp = c_ptr + (int64_t)field_mask[f] * (nnodes + 1);
    double s = 0.0;
    const int64_t a = cp[n], b = cp[n + 1];
    for (int64_t k = a; k < b; k++) s += vst[c_slot[k] * nf + f];
    double v = s / (double)(b - a);
    if (isnan(v)) v = 0.0;
    V[(int64_t)f * nnodes + n] = v;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct AmrRecovery {
    int nf = 0, nmask = 0, m_max = 1, e_max = 1;
    std::vector<int32_t> codes;      // output field codes, reference order
    int64_t ntasks = 0, nslots = 0, ncontrib = 0;
    double fit_flops = 0.0;          // algorithmic FP64 operations of one k_patch_fit launch
    int64_t n_svd = 0;               // tasks on the SVD path (known after a launch)
    // device
    double *ipx = nullptr, *ipv = nullptr, *vst = nullptr;
    int32_t *ip_elem = nullptr, *fmap = nullptr, *mask_nf = nullptr, *mask_fields = nullptr, *field_mask = nullptr;
    int64_t *t_elem_ptr = nullptr, *t_node_ptr = nullptr, *c_ptr = nullptr, *c_slot = nullptr;
    int32_t *t_elem = nullptr, *t_node = nullptr, *t_mask = nullptr, *t_center = nullptr, *t_m = nullptr,
            *t_flag = nullptr;
};

namespace {

template <class T>
void put(T **d, const std::vector<T> &h, cudaStream_t s) {
    amr_alloc(d, h.size());
    if (!h.empty()) AMR_CUDA(cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

void build(amr_model *m) {
    auto *R = new AmrRecovery();
    m->rec = R;
    cudaStream_t s = m->stream;
    const int64_t nn = m->nnodes, ne = m->nelems;
    // outer facets: node sets that occur an odd number of times (get_outer_facets, src/mesh/mesh.jl:69-85)
    std::vector<std::array<int32_t, 8>> keys;
    for (int64_t e = 0; e < ne; e++) {
        const FacetTab *ft = facet_table(m->h_shape[e]);
        const int32_t *cn = m->h_conn.data() + m->h_conn_ptr[e];
        for (int f = 0; f < ft->nf; f++) {
            std::array<int32_t, 8> k;
            k.fill(INT32_MAX);
            for (int j = 0; j < ft->np; j++) k[j] = cn[ft->idx[f][j]];
            std::sort(k.begin(), k.begin() + ft->np);
            keys.push_back(k);
        }
    }
    std::sort(keys.begin(), keys.end());
    std::vector<uint8_t> at_bound(nn, 0);
    for (size_t i = 0; i < keys.size();) {
        size_t j = i;
        while (j < keys.size() && keys[j] == keys[i]) j++;
        if ((j - i) & 1)
            for (int32_t v : keys[i])
                if (v != INT32_MAX) at_bound[v] = 1;
        i = j;
    }
    // interior and boundary patches, caller element order
    std::vector<int64_t> ip_cnt(nn + 1, 0), bp_cnt(nn + 1, 0);
    for (int64_t ec = 0; ec < ne; ec++) {
        const int64_t e = m->inv_perm[ec];
        const int32_t *cn = m->h_conn.data() + m->h_conn_ptr[e];
        for (int j = 0; j < corners(m->h_shape[e]); j++) (at_bound[cn[j]] ? bp_cnt : ip_cnt)[cn[j] + 1]++;
    }
    for (int64_t n = 0; n < nn; n++) { ip_cnt[n + 1] += ip_cnt[n]; bp_cnt[n + 1] += bp_cnt[n]; }
    std::vector<int32_t> ip_list(ip_cnt[nn]), bp_list(bp_cnt[nn]);
    {
        std::vector<int64_t> fi(ip_cnt.begin(), ip_cnt.end() - 1), fb(bp_cnt.begin(), bp_cnt.end() - 1);
        for (int64_t ec = 0; ec < ne; ec++) {
            const int64_t e = m->inv_perm[ec];
            const int32_t *cn = m->h_conn.data() + m->h_conn_ptr[e];
            for (int j = 0; j < corners(m->h_shape[e]); j++) {
                if (at_bound[cn[j]]) bp_list[fb[cn[j]]++] = (int32_t)e;
                else ip_list[fi[cn[j]]++] = (int32_t)e;
            }
        }
    }
    // which list serves as each node's patch: 0 none, 1 interior, 2 boundary
    std::vector<uint8_t> src(nn, 0), haspatch(nn, 0);
    auto mark = [&](const int32_t *b, const int32_t *en) {
        for (const int32_t *p = b; p < en; p++) {
            const int32_t *cn = m->h_conn.data() + m->h_conn_ptr[*p];
            for (int64_t j = 0; j < m->h_conn_ptr[*p + 1] - m->h_conn_ptr[*p]; j++) haspatch[cn[j]] = 1;
        }
    };
    for (int64_t n = 0; n < nn; n++)
        if (ip_cnt[n + 1] > ip_cnt[n]) { src[n] = 1; mark(&ip_list[ip_cnt[n]], &ip_list[0] + ip_cnt[n + 1]); }
    std::vector<int64_t> orphans;
    for (int64_t n = 0; n < nn; n++)
        if (!haspatch[n] && at_bound[n]) orphans.push_back(n);
    for (int k = 3; k >= 1 && !orphans.empty(); k--) {
        for (int64_t n : orphans)
            if (bp_cnt[n + 1] - bp_cnt[n] >= k) src[n] = 2;
        for (int64_t n : orphans)
            if (src[n] == 2) mark(&bp_list[bp_cnt[n]], &bp_list[0] + bp_cnt[n + 1]);
        std::vector<int64_t> left;
        for (int64_t n : orphans)
            if (!haspatch[n]) left.push_back(n);
        orphans.swap(left);
    }
    // fields: first appearance over the elements in caller order
    std::vector<int32_t> h_mat(ne);
    AMR_CUDA(cudaMemcpyAsync(h_mat.data(), m->mat_type, ne * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    AMR_CUDA(cudaStreamSynchronize(s));
    int32_t lists[3][AMR_NFIELD_CODES];
    int nlist[3];
    for (int mt = 0; mt < 3; mt++) nlist[mt] = field_codes(m->stressmodel, mt, lists[mt]);
    std::vector<int32_t> fmap(3 * AMR_NFIELD_CODES, -1);
    bool seen[3] = {false, false, false};
    for (int64_t ec = 0; ec < ne; ec++) {
        const int mt = h_mat[m->inv_perm[ec]];
        if (seen[mt]) continue;
        seen[mt] = true;
        for (int j = 0; j < nlist[mt]; j++)
            if (std::find(R->codes.begin(), R->codes.end(), lists[mt][j]) == R->codes.end())
                R->codes.push_back(lists[mt][j]);
    }
    R->nf = (int)R->codes.size();
    for (int mt = 0; mt < 3; mt++)
        for (int j = 0; j < nlist[mt]; j++) {
            const int f = (int)(std::find(R->codes.begin(), R->codes.end(), lists[mt][j]) - R->codes.begin());
            if (f < R->nf) fmap[mt * AMR_NFIELD_CODES + lists[mt][j]] = f;
        }
    // masks: the set of materials that carry each field
    std::vector<int> fmaskbits(R->nf, 0), masks;
    std::vector<int32_t> field_mask(R->nf);
    for (int f = 0; f < R->nf; f++) {
        for (int mt = 0; mt < 3; mt++)
            if (seen[mt] && fmap[mt * AMR_NFIELD_CODES + R->codes[f]] >= 0) fmaskbits[f] |= 1 << mt;
        auto it = std::find(masks.begin(), masks.end(), fmaskbits[f]);
        field_mask[f] = (int32_t)(it - masks.begin());
        if (it == masks.end()) masks.push_back(fmaskbits[f]);
    }
    R->nmask = (int)masks.size();
    std::vector<int32_t> mask_nf(R->nmask, 0), mask_fields((size_t)R->nmask * AMR_NFIELD_CODES, 0);
    for (int f = 0; f < R->nf; f++) mask_fields[field_mask[f] * AMR_NFIELD_CODES + mask_nf[field_mask[f]]++] = f;
    // fit tasks, patch (node) order; per mask the elements of the patch that carry its fields
    std::vector<int64_t> t_elem_ptr{0}, t_node_ptr{0};
    std::vector<int32_t> t_elem, t_node, t_mask, t_center, t_m;
    std::vector<int64_t> stamp(nn, -1);
    const int nt_max = m->ndim == 3 ? 7 : 6;
    double flops = 0.0;
    for (int64_t n = 0; n < nn; n++) {
        if (!src[n]) continue;
        const int32_t *pb = src[n] == 1 ? &ip_list[ip_cnt[n]] : &bp_list[bp_cnt[n]];
        const int64_t pc = src[n] == 1 ? ip_cnt[n + 1] - ip_cnt[n] : bp_cnt[n + 1] - bp_cnt[n];
        for (int mk = 0; mk < R->nmask; mk++) {
            const int64_t tid = (int64_t)t_mask.size();
            int32_t mcount = 0;
            int64_t ecount = 0;
            for (int64_t j = 0; j < pc; j++) {
                const int32_t e = pb[j];
                if (!((masks[mk] >> h_mat[e]) & 1)) continue;
                t_elem.push_back(e);
                ecount++;
                mcount += (int32_t)(m->h_ip_ptr[e + 1] - m->h_ip_ptr[e]);
                const int32_t *cn = m->h_conn.data() + m->h_conn_ptr[e];
                for (int64_t a = 0; a < m->h_conn_ptr[e + 1] - m->h_conn_ptr[e]; a++)
                    if (stamp[cn[a]] != tid) { stamp[cn[a]] = tid; t_node.push_back(cn[a]); }
            }
            if (!ecount) continue;
            t_elem_ptr.push_back((int64_t)t_elem.size());
            t_node_ptr.push_back((int64_t)t_node.size());
            t_mask.push_back(mk);
            t_center.push_back((int32_t)n);
            t_m.push_back(mcount);
            R->m_max = std::max(R->m_max, (int)mcount);
            R->e_max = std::max(R->e_max, (int)ecount);
            const int nt = m->ndim == 3 ? (mcount >= 7 ? 7 : mcount >= 4 ? 4 : 1)
                                        : (mcount >= 6 ? 6 : mcount >= 4 ? 4 : mcount >= 3 ? 3 : 1);
            const double nnod = (double)(t_node_ptr.back() - t_node_ptr[t_node_ptr.size() - 2]);
            // Gram (nt(nt+1)/2 FMA per IP), moments (nt per IP and field), node values (nt per node and field)
            flops += 2.0 * mcount * (nt * (nt + 1) / 2) + 2.0 * mcount * nt * mask_nf[mk] + 2.0 * nnod * nt * mask_nf[mk];
            (void)nt_max;
        }
    }
    R->fit_flops = flops;
    R->ntasks = (int64_t)t_mask.size();
    R->nslots = (int64_t)t_node.size();
    if (R->nslots >= INT32_MAX) throw AmrError(AMR_EUNSUPPORTED, "recovery: too many patch slots");
    const int64_t per_warp = fit_warp_doubles(R->m_max, R->e_max) * (int64_t)sizeof(double);
    if (per_warp * kFitWarps > 227 * 1024)
        throw AmrError(AMR_EUNSUPPORTED, "recovery: a patch has too many integration points (" +
                                             std::to_string(R->m_max) + ")");
    // contribution lists per (mask, node) in task order
    std::vector<int64_t> c_ptr((size_t)R->nmask * (nn + 1), 0);
    for (int64_t t = 0; t < R->ntasks; t++)
        for (int64_t j = t_node_ptr[t]; j < t_node_ptr[t + 1]; j++) c_ptr[(size_t)t_mask[t] * (nn + 1) + t_node[j] + 1]++;
    for (int mk = 0; mk < R->nmask; mk++) {
        int64_t *cp = c_ptr.data() + (size_t)mk * (nn + 1);
        for (int64_t n = 0; n < nn; n++) cp[n + 1] += cp[n];
    }
    std::vector<int64_t> fill(c_ptr);
    std::vector<int64_t> c_slot(R->nslots);
    // slots of every mask share one numbering: offset each mask's lists by the slots before it
    std::vector<int64_t> moff(R->nmask + 1, 0);
    for (int mk = 0; mk < R->nmask; mk++) moff[mk + 1] = moff[mk] + c_ptr[(size_t)mk * (nn + 1) + nn];
    for (int mk = 0; mk < R->nmask; mk++)
        for (int64_t n = 0; n <= nn; n++) c_ptr[(size_t)mk * (nn + 1) + n] += moff[mk];
    for (int64_t t = 0; t < R->ntasks; t++)
        for (int64_t j = t_node_ptr[t]; j < t_node_ptr[t + 1]; j++) {
            const size_t at = (size_t)t_mask[t] * (nn + 1) + t_node[j];
            c_slot[moff[t_mask[t]] + fill[at]++] = j;
        }
    R->ncontrib = R->nslots;
    // IP -> element
    std::vector<int32_t> ip_elem(m->nip_total);
    for (int64_t e = 0; e < ne; e++)
        for (int64_t g = m->h_ip_ptr[e]; g < m->h_ip_ptr[e + 1]; g++) ip_elem[g] = (int32_t)e;
    put(&R->t_elem_ptr, t_elem_ptr, s); put(&R->t_node_ptr, t_node_ptr, s);
    put(&R->t_elem, t_elem, s); put(&R->t_node, t_node, s); put(&R->t_mask, t_mask, s);
    put(&R->t_center, t_center, s); put(&R->t_m, t_m, s);
    put(&R->c_ptr, c_ptr, s); put(&R->c_slot, c_slot, s);
    put(&R->ip_elem, ip_elem, s); put(&R->fmap, fmap, s); put(&R->mask_nf, mask_nf, s);
    put(&R->mask_fields, mask_fields, s); put(&R->field_mask, field_mask, s);
    amr_alloc(&R->t_flag, std::max<int64_t>(1, R->ntasks));
    amr_alloc(&R->ipx, 3 * m->nip_total);
    amr_alloc(&R->ipv, std::max<int64_t>(1, m->nip_total * R->nf));
    amr_alloc(&R->vst, std::max<int64_t>(1, R->nslots * R->nf));
    AMR_CUDA(cudaMemsetAsync(R->ipx, 0, 3 * m->nip_total * sizeof(double), s));
    for (const AmrGroup &g : m->groups) {
        const double *Ntab = g.tab + (size_t)g.nip * g.nen * m->ndim + g.nip;
        const int64_t nt = g.count * g.nip;
        k_ip_coords<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(g.first, g.count, g.nen, g.nip, m->ndim, Ntab,
                                                                 m->conn_ptr, m->conn, m->ip_ptr, m->coords, R->ipx);
        AMR_COUNT(1);
        AMR_CUDA(cudaGetLastError());
    }
    AMR_CUDA(cudaStreamSynchronize(s));
}

FitArgs fit_args(amr_model *m) {
    AmrRecovery *R = m->rec;
    FitArgs A;
    A.ntasks = R->ntasks;
    A.t_elem_ptr = R->t_elem_ptr; A.t_node_ptr = R->t_node_ptr; A.t_elem = R->t_elem; A.t_node = R->t_node;
    A.t_mask = R->t_mask; A.t_center = R->t_center; A.t_m = R->t_m; A.mask_nf = R->mask_nf;
    A.mask_fields = R->mask_fields; A.ip_ptr = m->ip_ptr; A.ipx = R->ipx; A.coords = m->coords; A.ipv = R->ipv;
    A.nf = R->nf; A.m_max = R->m_max; A.e_max = R->e_max; A.vst = R->vst; A.t_flag = R->t_flag;
    return A;
}

unsigned fit_grid(amr_model *m, size_t smem) {
    int dev = 0, sms = 0, per_sm = 0;
    AMR_CUDA(cudaGetDevice(&dev));
    AMR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (m->ndim == 3)
        AMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_fit<3>, 32 * kFitWarps, smem));
    else
        AMR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_patch_fit<2>, 32 * kFitWarps, smem));
    const int64_t need = (m->rec->ntasks + kFitWarps - 1) / kFitWarps;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * std::max(1, per_sm)));
}

template <class K>
void set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) AMR_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
}

// the fit and SVD launches over all tasks
void launch_fit(amr_model *m, bool svd) {
    AmrRecovery *R = m->rec;
    if (!R->ntasks) return;
    const size_t smem = (size_t)fit_warp_doubles(R->m_max, R->e_max) * sizeof(double) * kFitWarps;
    FitArgs A = fit_args(m);
    if (m->ndim == 3) {
        set_smem(k_patch_fit<3>, smem);
        set_smem(k_patch_svd<3>, smem);
    } else {
        set_smem(k_patch_fit<2>, smem);
        set_smem(k_patch_svd<2>, smem);
    }
    const unsigned grid = fit_grid(m, smem);
    if (!svd) {
        if (m->ndim == 3) k_patch_fit<3><<<grid, 32 * kFitWarps, smem, m->stream>>>(A);
        else k_patch_fit<2><<<grid, 32 * kFitWarps, smem, m->stream>>>(A);
    } else {
        if (m->ndim == 3) k_patch_svd<3><<<grid, 32 * kFitWarps, smem, m->stream>>>(A);
        else k_patch_svd<2><<<grid, 32 * kFitWarps, smem, m->stream>>>(A);
    }
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

}  // namespace

void amr_recovery_prepare(amr_model *m) {
    if (!m->rec) {
        try {
            build(m);
        } catch (...) {
            amr_recovery_free(m);
            throw;
        }
    }
}

const std::vector<int32_t> &amr_recovery_codes(amr_model *m) {
    amr_recovery_prepare(m);
    return m->rec->codes;
}

void amr_recover(amr_model *m, double *d_V) {
    amr_recovery_prepare(m);
    AmrRecovery *R = m->rec;
    cudaStream_t s = m->stream;
    if (!R->nf) return;
    const int64_t nip = m->nip_total;
    k_ip_fields<<<(unsigned)((nip + 255) / 256), 256, 0, s>>>(nip, m->stressmodel, R->ip_elem, m->mat_type, m->st,
                                                              R->fmap, R->nf, R->ipv);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
    launch_fit(m, false);
    launch_fit(m, true);
    const int64_t nt = m->nnodes * R->nf;
    k_node_avg<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(m->nnodes, R->nf, R->field_mask, R->c_ptr, R->c_slot,
                                                            R->vst, d_V);
    AMR_COUNT(1);
    AMR_CUDA(cudaGetLastError());
}

double amr_recovery_time_fit(amr_model *m, int reps, double *flops, int64_t *n_svd) {
    amr_recovery_prepare(m);
    AmrRecovery *R = m->rec;
    cudaStream_t s = m->stream;
    const int64_t nip = m->nip_total;
    k_ip_fields<<<(unsigned)((nip + 255) / 256), 256, 0, s>>>(nip, m->stressmodel, R->ip_elem, m->mat_type, m->st,
                                                              R->fmap, R->nf, R->ipv);
    AMR_COUNT(1);
    launch_fit(m, false);
    AMR_CUDA(cudaStreamSynchronize(s));
    AMR_CUDA(cudaEventRecord(m->ev0, s));
    for (int r = 0; r < reps; r++) launch_fit(m, false);
    AMR_CUDA(cudaEventRecord(m->ev1, s));
    AMR_CUDA(cudaEventSynchronize(m->ev1));
    float ms = 0.0f;
    AMR_CUDA(cudaEventElapsedTime(&ms, m->ev0, m->ev1));
    if (flops) *flops = R->fit_flops;
    if (n_svd) {
        std::vector<int32_t> fl(R->ntasks);
        if (R->ntasks)
            amr_d2h(m, fl.data(), R->t_flag, R->ntasks * sizeof(int32_t));
        *n_svd = std::count(fl.begin(), fl.end(), 1);
    }
    return ms * 1e-3 / std::max(1, reps);
}

void amr_recovery_free(amr_model *m) {
    AmrRecovery *R = m->rec;
    if (!R) return;
    amr_free(R->ipx); amr_free(R->ipv); amr_free(R->vst); amr_free(R->ip_elem); amr_free(R->fmap);
    amr_free(R->mask_nf); amr_free(R->mask_fields); amr_free(R->field_mask); amr_free(R->t_elem_ptr);
    amr_free(R->t_node_ptr); amr_free(R->c_ptr); amr_free(R->c_slot); amr_free(R->t_elem); amr_free(R->t_node);
    amr_free(R->t_mask); amr_free(R->t_center); amr_free(R->t_m); amr_free(R->t_flag);
    delete R;
    m->rec = nullptr;
}
