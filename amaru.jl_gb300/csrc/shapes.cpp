// Shape functions and quadrature rules of the isoparametric cells on the GPU path.
//
// The functions are written in generic form -- tensor products of 1-D
// Lagrange polynomials, the serendipity corner/mid-side rules and barycentric
// coordinates for simplices -- over the node tables of Amaru's cells
// (src/shape/solids2d.jl, src/shape/solids3d.jl, src/shape/lines.jl), so the
// local node order matches Amaru's.  They only feed host-built per-shape
// tables (dN/dR at the integration points); no shape function is evaluated
// on the device.
#include <cmath>
#include <cstring>

#include "amr_internal.h"

namespace amr {
namespace {

// natural coordinates of the nodes, Amaru's local order
const double kHex[20][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, 1, 1},
                            {-1, 1, 1},   {0, -1, -1}, {1, 0, -1}, {0, 1, -1}, {-1, 0, -1}, {0, -1, 1}, {1, 0, 1},
                            {0, 1, 1},    {-1, 0, 1},  {-1, -1, 0}, {1, -1, 0}, {1, 1, 0},  {-1, 1, 0}};
const double kQuad[9][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}, {0, -1}, {1, 0}, {0, 1}, {-1, 0}, {0, 0}};
// mid-edge nodes of the simplices as pairs of vertices
const int kTet10Edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
const int kTri6Edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};

// 1-D quadratic Lagrange basis on nodes {-1, 0, 1}: value and derivative at x for node c
inline void lag2(double c, double x, double &v, double &d) {
    if (c < -0.5) { v = 0.5 * x * (x - 1.0); d = x - 0.5; }
    else if (c > 0.5) { v = 0.5 * x * (x + 1.0); d = x + 0.5; }
    else { v = 1.0 - x * x; d = -2.0 * x; }
}

// barycentric coordinates and their derivatives w.r.t. (r,s[,t])
void bary(int dim, const double *R, double *L, double *dL) {
    double sum = 0.0;
    for (int k = 0; k < dim; k++) sum += R[k];
    L[0] = 1.0 - sum;
    for (int k = 0; k < dim; k++) dL[0 * dim + k] = -1.0;
    for (int i = 1; i <= dim; i++) {
        L[i] = R[i - 1];
        for (int k = 0; k < dim; k++) dL[i * dim + k] = (k == i - 1) ? 1.0 : 0.0;
    }
}

// quadratic simplex (TRI6 / TET10): corners L(2L-1), edges 4 La Lb
void simplex2(int dim, const int (*edges)[2], int nedges, const double *R, double *N, double *D) {
    double L[4], dL[12];
    bary(dim, R, L, dL);
    for (int i = 0; i <= dim; i++) {
        if (N) N[i] = L[i] * (2.0 * L[i] - 1.0);
        if (D)
            for (int k = 0; k < dim; k++) D[i * dim + k] = (4.0 * L[i] - 1.0) * dL[i * dim + k];
    }
    for (int e = 0; e < nedges; e++) {
        int a = edges[e][0], b = edges[e][1], i = dim + 1 + e;
        if (N) N[i] = 4.0 * L[a] * L[b];
        if (D)
            for (int k = 0; k < dim; k++) D[i * dim + k] = 4.0 * (dL[a * dim + k] * L[b] + L[a] * dL[b * dim + k]);
    }
}

// serendipity quadratic brick / quad in `dim` dimensions over the node table
void serendipity(int dim, int nn, const double *X, int stride, const double *R, double *N, double *D) {
    for (int i = 0; i < nn; i++) {
        const double *c = X + i * stride;
        bool corner = true;
        for (int k = 0; k < dim; k++) corner = corner && (c[k] != 0.0);
        double f[3], df[3];
        if (corner) {
            // prod (1 + x_k c_k) * (sum x_k c_k - (dim-1)) / 2^dim
            double lin = 0.0;
            for (int k = 0; k < dim; k++) { f[k] = 1.0 + R[k] * c[k]; lin += R[k] * c[k]; }
            double scale = (dim == 3) ? 0.125 : 0.25;
            double g = lin - (dim - 1);
            double p = 1.0;
            for (int k = 0; k < dim; k++) p *= f[k];
            if (N) N[i] = scale * p * g;
            if (D)
                for (int k = 0; k < dim; k++) {
                    double pk = 1.0;
                    for (int l = 0; l < dim; l++)
                        if (l != k) pk *= f[l];
                    D[i * dim + k] = scale * (c[k] * pk * g + p * c[k]);
                }
        } else {
            // mid-side: (1 - x_m^2) along the zero coordinate m, linear in the others
            double scale = (dim == 3) ? 0.25 : 0.5;
            for (int k = 0; k < dim; k++) {
                if (c[k] == 0.0) { f[k] = 1.0 - R[k] * R[k]; df[k] = -2.0 * R[k]; }
                else { f[k] = 1.0 + R[k] * c[k]; df[k] = c[k]; }
            }
            double p = 1.0;
            for (int k = 0; k < dim; k++) p *= f[k];
            if (N) N[i] = scale * p;
            if (D)
                for (int k = 0; k < dim; k++) {
                    double pk = df[k];
                    for (int l = 0; l < dim; l++)
                        if (l != k) pk *= f[l];
                    D[i * dim + k] = scale * pk;
                }
        }
    }
}

// multilinear cells (QUAD4 / HEX8): prod (1 + x_k c_k) / 2
void multilinear(int dim, int nn, const double *X, int stride, const double *R, double *N, double *D) {
    for (int i = 0; i < nn; i++) {
        const double *c = X + i * stride;
        double f[3];
        for (int k = 0; k < dim; k++) f[k] = 0.5 * (1.0 + R[k] * c[k]);
        if (N) {
            double p = 1.0;
            for (int k = 0; k < dim; k++) p *= f[k];
            N[i] = p;
        }
        if (D)
            for (int k = 0; k < dim; k++) {
                double pk = 0.5 * c[k];
                for (int l = 0; l < dim; l++)
                    if (l != k) pk *= f[l];
                D[i * dim + k] = pk;
            }
    }
}

void eval(int shape, const double *R, double *N, double *D) {
    switch (shape) {
    case AMR_LIN2: {
        if (N) { N[0] = 0.5 * (1.0 - R[0]); N[1] = 0.5 * (1.0 + R[0]); }
        if (D) { D[0] = -0.5; D[1] = 0.5; }
        return;
    }
    case AMR_LIN3: {  // nodes at -1, 1, 0
        const double c[3] = {-1.0, 1.0, 0.0};
        for (int i = 0; i < 3; i++) {
            double v, d;
            lag2(c[i], R[0], v, d);
            if (N) N[i] = v;
            if (D) D[i] = d;
        }
        return;
    }
    case AMR_TRI3: case AMR_TET4: {
        int dim = (shape == AMR_TRI3) ? 2 : 3;
        double L[4], dL[12];
        bary(dim, R, L, dL);
        for (int i = 0; i <= dim; i++) {
            if (N) N[i] = L[i];
            if (D)
                for (int k = 0; k < dim; k++) D[i * dim + k] = dL[i * dim + k];
        }
        return;
    }
    case AMR_TRI6: simplex2(2, kTri6Edges, 3, R, N, D); return;
    case AMR_TET10: simplex2(3, kTet10Edges, 6, R, N, D); return;
    case AMR_QUAD4: multilinear(2, 4, &kQuad[0][0], 2, R, N, D); return;
    case AMR_HEX8: multilinear(3, 8, &kHex[0][0], 3, R, N, D); return;
    case AMR_QUAD8: serendipity(2, 8, &kQuad[0][0], 2, R, N, D); return;
    case AMR_HEX20: serendipity(3, 20, &kHex[0][0], 3, R, N, D); return;
    case AMR_QUAD9: {
        for (int i = 0; i < 9; i++) {
            double v0, d0, v1, d1;
            lag2(kQuad[i][0], R[0], v0, d0);
            lag2(kQuad[i][1], R[1], v1, d1);
            if (N) N[i] = v0 * v1;
            if (D) { D[2 * i] = d0 * v1; D[2 * i + 1] = v0 * d1; }
        }
        return;
    }
    }
}

// Gauss rules: src/shape/quadrature.jl (the same literal point/weight values)
const double kG2 = 0.577350269189625764509149;
const double kG3 = 0.774596669241483377035835, kG3w0 = 0.555555555555555555555556, kG3w1 = 0.888888888888888888888889;
const double kG4a = 0.861136311594052575223946, kG4b = 0.339981043584856264802666;
const double kG4wa = 0.34785484513745385737306, kG4wb = 0.65214515486254614262694;
const double kQ4 = 0.577350269189626;  // QUAD_IP4 / HEX_IP8 literal
const double kH27 = 0.774596669241483;
const double kH27w[4] = {0.171467764060357, 0.274348422496571, 0.438957475994513, 0.702331961591221};

int put(double *R, double *w, int i, double r, double s, double t, double wt) {
    R[3 * i] = r; R[3 * i + 1] = s; R[3 * i + 2] = t; w[i] = wt;
    return i + 1;
}

int rule_line(int n, double *R, double *w) {
    int i = 0;
    switch (n) {
    case 1: i = put(R, w, i, 0, 0, 0, 2.0); break;
    case 2: i = put(R, w, i, -kG2, 0, 0, 1.0); i = put(R, w, i, kG2, 0, 0, 1.0); break;
    case 3: i = put(R, w, i, -kG3, 0, 0, kG3w0); i = put(R, w, i, 0, 0, 0, kG3w1); i = put(R, w, i, kG3, 0, 0, kG3w0); break;
    case 4:
        i = put(R, w, i, -kG4a, 0, 0, kG4wa); i = put(R, w, i, -kG4b, 0, 0, kG4wb);
        i = put(R, w, i, kG4b, 0, 0, kG4wb); i = put(R, w, i, kG4a, 0, 0, kG4wa);
        break;
    default: return -1;
    }
    return i;
}

int rule_tri(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) return put(R, w, 0, 1.0 / 3.0, 1.0 / 3.0, 0, 0.5);
    if (n == 3) {
        const double a = 1.0 / 6.0, b = 2.0 / 3.0;
        i = put(R, w, i, a, a, 0, a); i = put(R, w, i, b, a, 0, a); i = put(R, w, i, a, b, 0, a);
        return i;
    }
    if (n == 6) {
        const double a = 0.091576213509771, b = 0.816847572980459, c = 0.445948490915965, d = 0.108103018168070;
        const double wa = 0.109951743655322 / 2.0, wc = 0.223381589678011 / 2.0;
        i = put(R, w, i, a, a, 0, wa); i = put(R, w, i, b, a, 0, wa); i = put(R, w, i, a, b, 0, wa);
        i = put(R, w, i, c, c, 0, wc); i = put(R, w, i, d, c, 0, wc); i = put(R, w, i, c, d, 0, wc);
        return i;
    }
    return -1;
}

int rule_quad(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) return put(R, w, 0, 0, 0, 0, 4.0);
    if (n == 4) {
        for (int j = 0; j < 2; j++)
            for (int k = 0; k < 2; k++) i = put(R, w, i, k ? kQ4 : -kQ4, j ? kQ4 : -kQ4, 0, 1.0);
        return i;
    }
    if (n == 9) {
        const double a = 0.2 * std::sqrt(15.0);
        const double p[3] = {-a, 0.0, a}, q[3] = {25.0 / 81.0, 40.0 / 81.0, 64.0 / 81.0};
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) {
                int m = (j == 1) + (k == 1);
                i = put(R, w, i, p[k], p[j], 0, q[m]);
            }
        return i;
    }
    if (n == 16) {
        const double p[4] = {-0.861136311594053, -0.339981043584856, 0.339981043584856, 0.861136311594053};
        const double q[3] = {0.121002993285602, 0.226851851851852, 0.425293303010694};
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++) {
                int m = (j == 1 || j == 2) + (k == 1 || k == 2);
                i = put(R, w, i, p[k], p[j], 0, q[m]);
            }
        return i;
    }
    return -1;
}

int rule_tet(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) return put(R, w, 0, 0.25, 0.25, 0.25, 1.0 / 6.0);
    if (n == 4) {
        const double a = 0.5854101966249685, b = 0.1381966011250105, q = 0.04166666666666667;
        i = put(R, w, i, a, b, b, q); i = put(R, w, i, b, a, b, q); i = put(R, w, i, b, b, a, q);
        i = put(R, w, i, b, b, b, q);
        return i;
    }
    if (n == 5) {
        const double s = 1.0 / 6.0;
        i = put(R, w, i, 0.25, 0.25, 0.25, -2.0 / 15.0);
        i = put(R, w, i, s, s, s, 3.0 / 40.0); i = put(R, w, i, s, s, 0.5, 3.0 / 40.0);
        i = put(R, w, i, s, 0.5, s, 3.0 / 40.0); i = put(R, w, i, 0.5, s, s, 3.0 / 40.0);
        return i;
    }
    return -1;
}

int rule_hex(int n, double *R, double *w) {
    int i = 0;
    if (n == 8) {
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                for (int l = 0; l < 2; l++) i = put(R, w, i, l ? kQ4 : -kQ4, j ? kQ4 : -kQ4, k ? kQ4 : -kQ4, 1.0);
        return i;
    }
    if (n == 27) {
        const double p[3] = {-kH27, 0.0, kH27};
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                for (int l = 0; l < 3; l++) i = put(R, w, i, p[l], p[j], p[k], kH27w[(l == 1) + (j == 1) + (k == 1)]);
        return i;
    }
    return -1;
}

}  // namespace

int shape_npoints(int shape) {
    static const int n[12] = {0, 2, 3, 3, 6, 4, 8, 9, 4, 10, 8, 20};
    return (shape >= 1 && shape <= 11) ? n[shape] : -1;
}

int shape_ndim(int shape) {
    static const int d[12] = {0, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3};
    return (shape >= 1 && shape <= 11) ? d[shape] : -1;
}

int shape_facet_shape(int shape) {
    switch (shape) {
    case AMR_HEX8: return AMR_QUAD4;
    case AMR_HEX20: return AMR_QUAD8;
    case AMR_TET4: return AMR_TRI3;
    case AMR_TET10: return AMR_TRI6;
    case AMR_QUAD4: case AMR_TRI3: return AMR_LIN2;
    case AMR_QUAD8: case AMR_QUAD9: case AMR_TRI6: return AMR_LIN3;
    }
    return -1;
}

void shape_func(int shape, const double *R, double *N) { eval(shape, R, N, nullptr); }
void shape_deriv(int shape, const double *R, double *D) { eval(shape, R, nullptr, D); }

// Default keys follow each shape's quadrature dictionary (src/shape/*.jl).
int quadrature(int shape, int nips, double *R, double *w) {
    switch (shape) {
    case AMR_LIN2: case AMR_LIN3: return rule_line(nips ? nips : 2, R, w);
    case AMR_TRI3: return rule_tri(nips ? nips : 3, R, w);
    case AMR_TRI6: return nips == 1 ? -1 : rule_tri(nips ? nips : 3, R, w);
    case AMR_QUAD4: case AMR_QUAD8: return rule_quad(nips ? nips : 4, R, w);
    case AMR_QUAD9: return nips == 1 ? -1 : rule_quad(nips ? nips : 9, R, w);
    case AMR_TET4: case AMR_TET10: return rule_tet(nips ? nips : 4, R, w);
    case AMR_HEX8: case AMR_HEX20: return rule_hex(nips ? nips : 8, R, w);
    }
    return -1;
}

}  // namespace amr
