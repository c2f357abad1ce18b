// Shape functions and quadrature rules of the isoparametric cells on the GPU path.
//
// They only feed host-built per-shape tables (N and dN/dR at the integration
// points); no shape function is evaluated on the device.
#include <cmath>
#include <cstring>

#include "amr_internal.h"

namespace amr {
namespace {

// Shape functions and derivatives at a point.  The derivative tables of the
// element kernels must carry bitwise the values Amaru computes at each
// integration point: where a derivative is mathematically zero only by
// cancellation (e.g. 4 - 8r - 4s - 4t of TET10 at a Gauss point), the exact
// zero or residue it evaluates to decides which entries of K_e survive the
// |K_ij| >= eps() drop rule of mount_K.  So the polynomials are evaluated in
// the expanded forms of src/shape/solids2d.jl, solids3d.jl and lines.jl.
void eval(int shape, const double *R, double *N, double *D) {
    const double r = R[0], s = R[1], t = R[2];
    switch (shape) {
    case AMR_LIN2:
        if (N) { N[0] = 0.5 * (1 - r); N[1] = 0.5 * (1 + r); }
        if (D) { D[0] = -0.5; D[1] = 0.5; }
        return;
    case AMR_LIN3:
        if (N) { N[0] = 0.5 * (r * r - r); N[1] = 0.5 * (r * r + r); N[2] = 1.0 - r * r; }
        if (D) { D[0] = r - 0.5; D[1] = r + 0.5; D[2] = -2.0 * r; }
        return;
    case AMR_TRI3:
        if (N) { N[0] = 1.0 - r - s; N[1] = r; N[2] = s; }
        if (D) { const double d[6] = {-1.0, -1.0, 1.0, 0.0, 0.0, 1.0}; std::memcpy(D, d, sizeof d); }
        return;
    case AMR_TRI6: {
        const double rs = r + s;
        if (N) {
            N[0] = 1.0 - rs * (3.0 - 2.0 * rs); N[1] = r * (2.0 * r - 1.0); N[2] = s * (2.0 * s - 1.0);
            N[3] = 4.0 * r * (1.0 - rs); N[4] = 4.0 * r * s; N[5] = 4.0 * s * (1.0 - rs);
        }
        if (D) {
            const double d[12] = {-3.0 + 4.0 * rs, -3.0 + 4.0 * rs, 4.0 * r - 1.0, 0.0, 0.0, 4.0 * s - 1.0,
                                  4.0 - 8.0 * r - 4.0 * s, -4.0 * r, 4.0 * s, 4.0 * r, -4.0 * s, 4.0 - 4.0 * r - 8.0 * s};
            std::memcpy(D, d, sizeof d);
        }
        return;
    }
    case AMR_QUAD4:
        if (N) {
            N[0] = 0.25 * (1.0 - r - s + r * s); N[1] = 0.25 * (1.0 + r - s - r * s);
            N[2] = 0.25 * (1.0 + r + s + r * s); N[3] = 0.25 * (1.0 - r + s - r * s);
        }
        if (D) {
            const double d[8] = {0.25 * (-1.0 + s), 0.25 * (-1.0 + r), 0.25 * (+1.0 - s), 0.25 * (-1.0 - r),
                                 0.25 * (+1.0 + s), 0.25 * (+1.0 + r), 0.25 * (-1.0 - s), 0.25 * (+1.0 - r)};
            std::memcpy(D, d, sizeof d);
        }
        return;
    case AMR_QUAD8: {
        const double rp = 1.0 + r, rm = 1.0 - r, sp = 1.0 + s, sm = 1.0 - s;
        if (N) {
            N[0] = 0.25 * rm * sm * (rm + sm - 3.0); N[1] = 0.25 * rp * sm * (rp + sm - 3.0);
            N[2] = 0.25 * rp * sp * (rp + sp - 3.0); N[3] = 0.25 * rm * sp * (rm + sp - 3.0);
            N[4] = 0.50 * sm * (1.0 - r * r); N[5] = 0.50 * rp * (1.0 - s * s);
            N[6] = 0.50 * sp * (1.0 - r * r); N[7] = 0.50 * rm * (1.0 - s * s);
        }
        if (D) {
            const double d[16] = {-0.25 * sm * (rm + rm + sm - 3.0), -0.25 * rm * (sm + rm + sm - 3.0),
                                  0.25 * sm * (rp + rp + sm - 3.0),  -0.25 * rp * (sm + rp + sm - 3.0),
                                  0.25 * sp * (rp + rp + sp - 3.0),  0.25 * rp * (sp + rp + sp - 3.0),
                                  -0.25 * sp * (rm + rm + sp - 3.0), 0.25 * rm * (sp + rm + sp - 3.0),
                                  -r * sm,                           -0.50 * (1.0 - r * r),
                                  0.50 * (1.0 - s * s),              -s * rp,
                                  -r * sp,                           0.50 * (1.0 - r * r),
                                  -0.5 * (1.0 - s * s),              -s * rm};
            std::memcpy(D, d, sizeof d);
        }
        return;
    }
    case AMR_QUAD9: {
        const double rp = r + 1.0, rm = r - 1.0, sp = s + 1.0, sm = s - 1.0;
        if (N) {
            N[0] = 0.25 * r * s * sm * rm; N[1] = 0.25 * r * s * sm * rp; N[2] = 0.25 * r * s * sp * rp;
            N[3] = 0.25 * r * s * sp * rm; N[4] = -0.50 * s * sm * rp * rm; N[5] = -0.50 * r * sp * sm * rp;
            N[6] = -0.50 * s * sp * rp * rm; N[7] = -0.50 * r * sp * sm * rm; N[8] = sp * sm * rp * rm;
        }
        if (D) {
            const double d[18] = {(r + rm) * s * sm / 4.0,         r * rm * (s + sm) / 4.0,
                                  (r + rp) * s * sm / 4.0,         r * rp * (s + sm) / 4.0,
                                  (r + rp) * s * sp / 4.0,         r * rp * (s + sp) / 4.0,
                                  (r + rm) * s * sp / 4.0,         r * rm * (s + sp) / 4.0,
                                  -(r + r) * s * (sm) / 2.0,       -(r * r - 1.0) * (s + sm) / 2.0,
                                  -(r + rp) * (s * s - 1.0) / 2.0, -r * rp * (s + s) / 2.0,
                                  -(r + r) * s * (sp) / 2.0,       -(r * r - 1.0) * (s + sp) / 2.0,
                                  -(r + rm) * (s * s - 1.0) / 2.0, -r * rm * (s + s) / 2.0,
                                  2.0 * r * (s * s - 1.0),         2.0 * s * (r * r - 1.0)};
            std::memcpy(D, d, sizeof d);
        }
        return;
    }
    case AMR_TET4:
        if (N) { N[0] = 1.0 - r - s - t; N[1] = r; N[2] = s; N[3] = t; }
        if (D) {
            const double d[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0};
            std::memcpy(D, d, sizeof d);
        }
        return;
    case AMR_TET10: {
        const double u = 1.0 - r - s - t;
        if (N) {
            N[0] = u * (2.0 * u - 1.0); N[1] = r * (2.0 * r - 1.0); N[2] = s * (2.0 * s - 1.0);
            N[3] = t * (2.0 * t - 1.0); N[4] = 4.0 * u * r; N[5] = 4.0 * r * s; N[6] = 4.0 * s * u;
            N[7] = 4.0 * u * t; N[8] = 4.0 * r * t; N[9] = 4.0 * s * t;
        }
        if (D) {
            const double c = 4.0 * (r + s + t) - 3.0;
            const double d[30] = {c, c, c,
                                  4.0 * r - 1.0, 0.0, 0.0,
                                  0.0, 4.0 * s - 1.0, 0.0,
                                  0.0, 0.0, 4.0 * t - 1.0,
                                  4.0 - 8.0 * r - 4.0 * s - 4.0 * t, -4.0 * r, -4.0 * r,
                                  4.0 * s, 4.0 * r, 0.0,
                                  -4.0 * s, 4.0 - 4.0 * r - 8.0 * s - 4.0 * t, -4.0 * s,
                                  -4.0 * t, -4.0 * t, 4.0 - 4.0 * r - 4.0 * s - 8.0 * t,
                                  4.0 * t, 0.0, 4.0 * r,
                                  0.0, 4.0 * t, 4.0 * s};
            std::memcpy(D, d, sizeof d);
        }
        return;
    }
    case AMR_HEX8: {
        if (N) {
            N[0] = 0.125 * (1.0 - r - s + r * s - t + s * t + r * t - r * s * t);
            N[1] = 0.125 * (1.0 + r - s - r * s - t + s * t - r * t + r * s * t);
            N[2] = 0.125 * (1.0 + r + s + r * s - t - s * t - r * t - r * s * t);
            N[3] = 0.125 * (1.0 - r + s - r * s - t - s * t + r * t + r * s * t);
            N[4] = 0.125 * (1.0 - r - s + r * s + t - s * t - r * t + r * s * t);
            N[5] = 0.125 * (1.0 + r - s - r * s + t - s * t + r * t - r * s * t);
            N[6] = 0.125 * (1.0 + r + s + r * s + t + s * t + r * t + r * s * t);
            N[7] = 0.125 * (1.0 - r + s - r * s + t + s * t - r * t - r * s * t);
        }
        if (D) {
            const double st = s * t, rt = r * t, rs = r * s;
            const double d[24] = {-1.0 + s + t - st, -1.0 + r + t - rt, -1.0 + r + s - rs,
                                  +1.0 - s - t + st, -1.0 - r + t + rt, -1.0 - r + s + rs,
                                  +1.0 + s - t - st, +1.0 + r - t - rt, -1.0 - r - s - rs,
                                  -1.0 - s + t + st, +1.0 - r - t + rt, -1.0 + r - s + rs,
                                  -1.0 + s - t + st, -1.0 + r - t + rt, +1.0 - r - s + rs,
                                  +1.0 - s + t - st, -1.0 - r - t - rt, +1.0 + r - s - rs,
                                  +1.0 + s + t + st, +1.0 + r + t + rt, +1.0 + r + s + rs,
                                  -1.0 - s - t - st, +1.0 - r + t - rt, +1.0 - r + s - rs};
            for (int i = 0; i < 24; i++) D[i] = 0.125 * d[i];
        }
        return;
    }
    case AMR_HEX20: {
        const double rp = 1.0 + r, rm = 1.0 - r, sp = 1.0 + s, sm = 1.0 - s, tp = 1.0 + t, tm = 1.0 - t;
        if (N) {
            N[0] = 0.125 * rm * sm * tm * (-r - s - t - 2.0); N[1] = 0.125 * rp * sm * tm * (r - s - t - 2.0);
            N[2] = 0.125 * rp * sp * tm * (r + s - t - 2.0);  N[3] = 0.125 * rm * sp * tm * (-r + s - t - 2.0);
            N[4] = 0.125 * rm * sm * tp * (-r - s + t - 2.0); N[5] = 0.125 * rp * sm * tp * (r - s + t - 2.0);
            N[6] = 0.125 * rp * sp * tp * (r + s + t - 2.0);  N[7] = 0.125 * rm * sp * tp * (-r + s + t - 2.0);
            N[8] = 0.25 * (1.0 - r * r) * sm * tm;  N[9] = 0.25 * rp * (1.0 - s * s) * tm;
            N[10] = 0.25 * (1.0 - r * r) * sp * tm; N[11] = 0.25 * rm * (1.0 - s * s) * tm;
            N[12] = 0.25 * (1.0 - r * r) * sm * tp; N[13] = 0.25 * rp * (1.0 - s * s) * tp;
            N[14] = 0.25 * (1.0 - r * r) * sp * tp; N[15] = 0.25 * rm * (1.0 - s * s) * tp;
            N[16] = 0.25 * rm * sm * (1.0 - t * t); N[17] = 0.25 * rp * sm * (1.0 - t * t);
            N[18] = 0.25 * rp * sp * (1.0 - t * t); N[19] = 0.25 * rm * sp * (1.0 - t * t);
        }
        if (D) {
            double *d = D;
            // d/dr
            d[0] = -0.125 * sm * tm * (-r - s - t - 2) - 0.125 * rm * sm * tm;
            d[3] = 0.125 * sm * tm * (r - s - t - 2) + 0.125 * rp * sm * tm;
            d[6] = 0.125 * sp * tm * (r + s - t - 2) + 0.125 * rp * sp * tm;
            d[9] = -0.125 * sp * tm * (-r + s - t - 2) - 0.125 * rm * sp * tm;
            d[12] = -0.125 * sm * tp * (-r - s + t - 2) - 0.125 * rm * sm * tp;
            d[15] = 0.125 * sm * tp * (r - s + t - 2) + 0.125 * rp * sm * tp;
            d[18] = 0.125 * sp * tp * (r + s + t - 2) + 0.125 * rp * sp * tp;
            d[21] = -0.125 * sp * tp * (-r + s + t - 2) - 0.125 * rm * sp * tp;
            d[24] = -0.5 * r * sm * tm;  d[27] = 0.25 * (1 - s * s) * tm; d[30] = -0.5 * r * sp * tm;
            d[33] = -0.25 * (1 - s * s) * tm; d[36] = -0.5 * r * sm * tp; d[39] = 0.25 * (1 - s * s) * tp;
            d[42] = -0.5 * r * sp * tp; d[45] = -0.25 * (1 - s * s) * tp; d[48] = -0.25 * sm * (1 - t * t);
            d[51] = 0.25 * sm * (1 - t * t); d[54] = 0.25 * sp * (1 - t * t); d[57] = -0.25 * sp * (1 - t * t);
            // d/ds
            d[1] = -0.125 * rm * tm * (-r - s - t - 2) - 0.125 * rm * sm * tm;
            d[4] = -0.125 * rp * tm * (r - s - t - 2) - 0.125 * rp * sm * tm;
            d[7] = 0.125 * rp * tm * (r + s - t - 2) + 0.125 * rp * sp * tm;
            d[10] = 0.125 * rm * tm * (-r + s - t - 2) + 0.125 * rm * sp * tm;
            d[13] = -0.125 * rm * tp * (-r - s + t - 2) - 0.125 * rm * sm * tp;
            d[16] = -0.125 * rp * tp * (r - s + t - 2) - 0.125 * rp * sm * tp;
            d[19] = 0.125 * rp * tp * (r + s + t - 2) + 0.125 * rp * sp * tp;
            d[22] = 0.125 * rm * tp * (-r + s + t - 2) + 0.125 * rm * sp * tp;
            d[25] = -0.25 * (1 - r * r) * tm; d[28] = -0.5 * s * rp * tm; d[31] = 0.25 * (1 - r * r) * tm;
            d[34] = -0.5 * s * rm * tm; d[37] = -0.25 * (1 - r * r) * tp; d[40] = -0.5 * s * rp * tp;
            d[43] = 0.25 * (1 - r * r) * tp; d[46] = -0.5 * s * rm * tp; d[49] = -0.25 * rm * (1 - t * t);
            d[52] = -0.25 * rp * (1 - t * t); d[55] = 0.25 * rp * (1 - t * t); d[58] = 0.25 * rm * (1 - t * t);
            // d/dt
            d[2] = -0.125 * rm * sm * (-r - s - t - 2) - 0.125 * rm * sm * tm;
            d[5] = -0.125 * rp * sm * (r - s - t - 2) - 0.125 * rp * sm * tm;
            d[8] = -0.125 * rp * sp * (r + s - t - 2) - 0.125 * rp * sp * tm;
            d[11] = -0.125 * rm * sp * (-r + s - t - 2) - 0.125 * rm * sp * tm;
            d[14] = 0.125 * rm * sm * (-r - s + t - 2) + 0.125 * rm * sm * tp;
            d[17] = 0.125 * rp * sm * (r - s + t - 2) + 0.125 * rp * sm * tp;
            d[20] = 0.125 * rp * sp * (r + s + t - 2) + 0.125 * rp * sp * tp;
            d[23] = 0.125 * rm * sp * (-r + s + t - 2) + 0.125 * rm * sp * tp;
            d[26] = -0.25 * (1 - r * r) * sm; d[29] = -0.25 * rp * (1 - s * s); d[32] = -0.25 * (1 - r * r) * sp;
            d[35] = -0.25 * rm * (1 - s * s); d[38] = 0.25 * (1 - r * r) * sm; d[41] = 0.25 * rp * (1 - s * s);
            d[44] = 0.25 * (1 - r * r) * sp; d[47] = 0.25 * rm * (1 - s * s); d[50] = -0.5 * t * rm * sm;
            d[53] = -0.5 * t * rp * sm; d[56] = -0.5 * t * rp * sp; d[59] = -0.5 * t * rm * sp;
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
