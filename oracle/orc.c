/*
 * CPU oracle for the Amaru mechanical hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the Float64 algorithms of NumSoftware/Amaru.jl
 * (v0.7.1) for solid elements: shape functions and quadrature tables, the
 * Mandel-notation B matrix, the element stiffness, the constitutive updates of
 * LinearElastic / VonMises / DruckerPrager, the threaded element loops of
 * mount_K and update_state!, and the duplicate-summing COO->CSC conversion of
 * SparseArrays.sparse.  It is the checker for the CUDA library: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  It is
 * never part of the product path.
 *
 * Citations are paths inside the Amaru.jl source tree.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SR2 1.4142135623730951 /* src/tools/constants.jl:3  SR2 = sqrt(2.0) */

/* Shape codes (shared numbering with the library's public header). */
enum {
    ORC_LIN2 = 1, ORC_LIN3 = 2, ORC_TRI3 = 3, ORC_TRI6 = 4, ORC_QUAD4 = 5,
    ORC_QUAD8 = 6, ORC_QUAD9 = 7, ORC_TET4 = 8, ORC_TET10 = 9, ORC_HEX8 = 10,
    ORC_HEX20 = 11
};

/* Stress models: src/mech/mech-solver.jl:9 */
enum { ORC_D3 = 0, ORC_PLANESTRAIN = 1, ORC_PLANESTRESS = 2, ORC_AXISYM = 3 };

/* Materials */
enum { ORC_LINEAR_ELASTIC = 0, ORC_VON_MISES = 1, ORC_DRUCKER_PRAGER = 2 };

/* Per-IP state record (doubles): sigma[6], eps[6], epa, dlambda (or dgamma). */
#define ORC_ST_SIG 0
#define ORC_ST_EPS 6
#define ORC_ST_EPA 12
#define ORC_ST_DL 13
#define ORC_ST_LEN 16

typedef struct {
    int32_t ndim;
    int32_t stressmodel;
    double thickness;
    int64_t nnodes;
    const double *coords;    /* nnodes x 3 */
    int64_t nelem;
    const int32_t *shape;    /* nelem */
    const int64_t *conn_ptr; /* nelem+1 */
    const int64_t *conn;     /* 0-based node indices, Amaru local order */
    const int32_t *nips;     /* nelem: quadrature key (0 = shape default) */
    const int32_t *mat_type; /* nelem */
    const double *mat_par;   /* nelem x 8: E nu fy|alpha H kappa ... */
    const int64_t *eq_id;    /* nnodes x 3, 0-based, -1 when absent */
    const int64_t *ip_ptr;   /* nelem+1 offsets into state */
    double *state;           /* nip_total x ORC_ST_LEN */
    const int64_t *active;   /* the active elements in id order (mech-solver.jl:216-220), or null: all */
    int64_t nactive;
} orc_model;

/* the element loops of mount_K and update_state! run over active_elems */
static int64_t n_active(const orc_model *m) { return m->active ? m->nactive : m->nelem; }
static int64_t active_elem(const orc_model *m, int64_t i) { return m->active ? m->active[i] : i; }

/* ------------------------------------------------------------------------ */
/* Shapes: src/shape/lines.jl, solids2d.jl, solids3d.jl                      */
/* ------------------------------------------------------------------------ */

int orc_shape_npoints(int shape) {
    switch (shape) {
    case ORC_LIN2: return 2;  case ORC_LIN3: return 3;  case ORC_TRI3: return 3;
    case ORC_TRI6: return 6;  case ORC_QUAD4: return 4; case ORC_QUAD8: return 8;
    case ORC_QUAD9: return 9; case ORC_TET4: return 4;  case ORC_TET10: return 10;
    case ORC_HEX8: return 8;  case ORC_HEX20: return 20;
    }
    return -1;
}

int orc_shape_ndim(int shape) {
    switch (shape) {
    case ORC_LIN2: case ORC_LIN3: return 1;
    case ORC_TRI3: case ORC_TRI6: case ORC_QUAD4: case ORC_QUAD8: case ORC_QUAD9: return 2;
    case ORC_TET4: case ORC_TET10: case ORC_HEX8: case ORC_HEX20: return 3;
    }
    return -1;
}

/* N(R): shape_func_* */
void orc_shape_func(int shape, const double *R, double *N) {
    double r = R[0], s = R[1], t = R[2];
    switch (shape) {
    case ORC_LIN2: /* lines.jl:10-16 */
        N[0] = 0.5 * (1 - r); N[1] = 0.5 * (1 + r); break;
    case ORC_LIN3: /* lines.jl:67-73 */
        N[0] = 0.5 * (r * r - r); N[1] = 0.5 * (r * r + r); N[2] = 1.0 - r * r; break;
    case ORC_TRI3: /* solids2d.jl:32-39 */
        N[0] = 1.0 - r - s; N[1] = r; N[2] = s; break;
    case ORC_TRI6: /* solids2d.jl:109-121 */
        N[0] = 1.0 - (r + s) * (3.0 - 2.0 * (r + s));
        N[1] = r * (2.0 * r - 1.0);
        N[2] = s * (2.0 * s - 1.0);
        N[3] = 4.0 * r * (1.0 - (r + s));
        N[4] = 4.0 * r * s;
        N[5] = 4.0 * s * (1.0 - (r + s));
        break;
    case ORC_QUAD4: /* solids2d.jl:295-302 */
        N[0] = 0.25 * (1.0 - r - s + r * s);
        N[1] = 0.25 * (1.0 + r - s - r * s);
        N[2] = 0.25 * (1.0 + r + s + r * s);
        N[3] = 0.25 * (1.0 - r + s - r * s);
        break;
    case ORC_QUAD8: { /* solids2d.jl:367-381 */
        double rp1 = 1.0 + r, rm1 = 1.0 - r, sp1 = 1.0 + s, sm1 = 1.0 - s;
        N[0] = 0.25 * rm1 * sm1 * (rm1 + sm1 - 3.0);
        N[1] = 0.25 * rp1 * sm1 * (rp1 + sm1 - 3.0);
        N[2] = 0.25 * rp1 * sp1 * (rp1 + sp1 - 3.0);
        N[3] = 0.25 * rm1 * sp1 * (rm1 + sp1 - 3.0);
        N[4] = 0.50 * sm1 * (1.0 - r * r);
        N[5] = 0.50 * rp1 * (1.0 - s * s);
        N[6] = 0.50 * sp1 * (1.0 - r * r);
        N[7] = 0.50 * rm1 * (1.0 - s * s);
        break;
    }
    case ORC_QUAD9: { /* solids2d.jl QUAD9 shape_func */
        double rp1 = r + 1.0, rm1 = r - 1.0, sp1 = s + 1.0, sm1 = s - 1.0;
        N[0] = 0.25 * r * s * sm1 * rm1;
        N[1] = 0.25 * r * s * sm1 * rp1;
        N[2] = 0.25 * r * s * sp1 * rp1;
        N[3] = 0.25 * r * s * sp1 * rm1;
        N[4] = -0.50 * s * sm1 * rp1 * rm1;
        N[5] = -0.50 * r * sp1 * sm1 * rp1;
        N[6] = -0.50 * s * sp1 * rp1 * rm1;
        N[7] = -0.50 * r * sp1 * sm1 * rm1;
        N[8] = sp1 * sm1 * rp1 * rm1;
        break;
    }
    case ORC_TET4: /* solids3d.jl TET4 shape_func */
        N[0] = 1.0 - r - s - t; N[1] = r; N[2] = s; N[3] = t; break;
    case ORC_TET10: { /* solids3d.jl:124-146 */
        double u = 1.0 - r - s - t;
        N[0] = u * (2.0 * u - 1.0); N[1] = r * (2.0 * r - 1.0);
        N[2] = s * (2.0 * s - 1.0); N[3] = t * (2.0 * t - 1.0);
        N[4] = 4.0 * u * r; N[5] = 4.0 * r * s; N[6] = 4.0 * s * u;
        N[7] = 4.0 * u * t; N[8] = 4.0 * r * t; N[9] = 4.0 * s * t;
        break;
    }
    case ORC_HEX8: /* solids3d.jl:473-485 */
        N[0] = 0.125 * (1.0 - r - s + r * s - t + s * t + r * t - r * s * t);
        N[1] = 0.125 * (1.0 + r - s - r * s - t + s * t - r * t + r * s * t);
        N[2] = 0.125 * (1.0 + r + s + r * s - t - s * t - r * t - r * s * t);
        N[3] = 0.125 * (1.0 - r + s - r * s - t - s * t + r * t + r * s * t);
        N[4] = 0.125 * (1.0 - r - s + r * s + t - s * t - r * t + r * s * t);
        N[5] = 0.125 * (1.0 + r - s - r * s + t - s * t + r * t - r * s * t);
        N[6] = 0.125 * (1.0 + r + s + r * s + t + s * t + r * t + r * s * t);
        N[7] = 0.125 * (1.0 - r + s - r * s + t + s * t - r * t - r * s * t);
        break;
    case ORC_HEX20: { /* solids3d.jl:584-613 */
        double rp1 = 1.0 + r, rm1 = 1.0 - r, sp1 = 1.0 + s, sm1 = 1.0 - s, tp1 = 1.0 + t, tm1 = 1.0 - t;
        N[0] = 0.125 * rm1 * sm1 * tm1 * (-r - s - t - 2.0);
        N[1] = 0.125 * rp1 * sm1 * tm1 * (r - s - t - 2.0);
        N[2] = 0.125 * rp1 * sp1 * tm1 * (r + s - t - 2.0);
        N[3] = 0.125 * rm1 * sp1 * tm1 * (-r + s - t - 2.0);
        N[4] = 0.125 * rm1 * sm1 * tp1 * (-r - s + t - 2.0);
        N[5] = 0.125 * rp1 * sm1 * tp1 * (r - s + t - 2.0);
        N[6] = 0.125 * rp1 * sp1 * tp1 * (r + s + t - 2.0);
        N[7] = 0.125 * rm1 * sp1 * tp1 * (-r + s + t - 2.0);
        N[8] = 0.25 * (1.0 - r * r) * sm1 * tm1;
        N[9] = 0.25 * rp1 * (1.0 - s * s) * tm1;
        N[10] = 0.25 * (1.0 - r * r) * sp1 * tm1;
        N[11] = 0.25 * rm1 * (1.0 - s * s) * tm1;
        N[12] = 0.25 * (1.0 - r * r) * sm1 * tp1;
        N[13] = 0.25 * rp1 * (1.0 - s * s) * tp1;
        N[14] = 0.25 * (1.0 - r * r) * sp1 * tp1;
        N[15] = 0.25 * rm1 * (1.0 - s * s) * tp1;
        N[16] = 0.25 * rm1 * sm1 * (1.0 - t * t);
        N[17] = 0.25 * rp1 * sm1 * (1.0 - t * t);
        N[18] = 0.25 * rp1 * sp1 * (1.0 - t * t);
        N[19] = 0.25 * rm1 * sp1 * (1.0 - t * t);
        break;
    }
    }
}

/* dN/dR(R), stored D[i*ndim + k]: shape_deriv_* */
void orc_shape_deriv(int shape, const double *R, double *D) {
    double r = R[0], s = R[1], t = R[2];
#define D2(i, a, b) (D[2 * (i)] = (a), D[2 * (i) + 1] = (b))
#define D3(i, a, b, c) (D[3 * (i)] = (a), D[3 * (i) + 1] = (b), D[3 * (i) + 2] = (c))
    switch (shape) {
    case ORC_LIN2: D[0] = -0.5; D[1] = 0.5; break;
    case ORC_LIN3: D[0] = r - 0.5; D[1] = r + 0.5; D[2] = -2.0 * r; break;
    case ORC_TRI3: D2(0, -1.0, -1.0); D2(1, 1.0, 0.0); D2(2, 0.0, 1.0); break;
    case ORC_TRI6:
        D2(0, -3.0 + 4.0 * (r + s), -3.0 + 4.0 * (r + s));
        D2(1, 4.0 * r - 1.0, 0.0);
        D2(2, 0.0, 4.0 * s - 1.0);
        D2(3, 4.0 - 8.0 * r - 4.0 * s, -4.0 * r);
        D2(4, 4.0 * s, 4.0 * r);
        D2(5, -4.0 * s, 4.0 - 4.0 * r - 8.0 * s);
        break;
    case ORC_QUAD4:
        D2(0, 0.25 * (-1.0 + s), 0.25 * (-1.0 + r));
        D2(1, 0.25 * (+1.0 - s), 0.25 * (-1.0 - r));
        D2(2, 0.25 * (+1.0 + s), 0.25 * (+1.0 + r));
        D2(3, 0.25 * (-1.0 - s), 0.25 * (+1.0 - r));
        break;
    case ORC_QUAD8: {
        double rp1 = 1.0 + r, rm1 = 1.0 - r, sp1 = 1.0 + s, sm1 = 1.0 - s;
        D2(0, -0.25 * sm1 * (rm1 + rm1 + sm1 - 3.0), -0.25 * rm1 * (sm1 + rm1 + sm1 - 3.0));
        D2(1, 0.25 * sm1 * (rp1 + rp1 + sm1 - 3.0), -0.25 * rp1 * (sm1 + rp1 + sm1 - 3.0));
        D2(2, 0.25 * sp1 * (rp1 + rp1 + sp1 - 3.0), 0.25 * rp1 * (sp1 + rp1 + sp1 - 3.0));
        D2(3, -0.25 * sp1 * (rm1 + rm1 + sp1 - 3.0), 0.25 * rm1 * (sp1 + rm1 + sp1 - 3.0));
        D2(4, -r * sm1, -0.50 * (1.0 - r * r));
        D2(5, 0.50 * (1.0 - s * s), -s * rp1);
        D2(6, -r * sp1, 0.50 * (1.0 - r * r));
        D2(7, -0.5 * (1.0 - s * s), -s * rm1);
        break;
    }
    case ORC_QUAD9: {
        double rp1 = r + 1.0, rm1 = r - 1.0, sp1 = s + 1.0, sm1 = s - 1.0;
        D2(0, (r + rm1) * s * sm1 / 4.0, r * rm1 * (s + sm1) / 4.0);
        D2(1, (r + rp1) * s * sm1 / 4.0, r * rp1 * (s + sm1) / 4.0);
        D2(2, (r + rp1) * s * sp1 / 4.0, r * rp1 * (s + sp1) / 4.0);
        D2(3, (r + rm1) * s * sp1 / 4.0, r * rm1 * (s + sp1) / 4.0);
        D2(4, -(r + r) * s * (sm1) / 2.0, -(r * r - 1.0) * (s + sm1) / 2.0);
        D2(5, -(r + rp1) * (s * s - 1.0) / 2.0, -r * rp1 * (s + s) / 2.0);
        D2(6, -(r + r) * s * (sp1) / 2.0, -(r * r - 1.0) * (s + sp1) / 2.0);
        D2(7, -(r + rm1) * (s * s - 1.0) / 2.0, -r * rm1 * (s + s) / 2.0);
        D2(8, 2.0 * r * (s * s - 1.0), 2.0 * s * (r * r - 1.0));
        break;
    }
    case ORC_TET4:
        D3(0, -1.0, -1.0, -1.0); D3(1, 1.0, 0.0, 0.0); D3(2, 0.0, 1.0, 0.0); D3(3, 0.0, 0.0, 1.0);
        break;
    case ORC_TET10:
        D3(0, 4.0 * (r + s + t) - 3.0, 4.0 * (r + s + t) - 3.0, 4.0 * (r + s + t) - 3.0);
        D3(1, 4.0 * r - 1.0, 0.0, 0.0);
        D3(2, 0.0, 4.0 * s - 1.0, 0.0);
        D3(3, 0.0, 0.0, 4.0 * t - 1.0);
        D3(4, 4.0 - 8.0 * r - 4.0 * s - 4.0 * t, -4.0 * r, -4.0 * r);
        D3(5, 4.0 * s, 4.0 * r, 0.0);
        D3(6, -4.0 * s, 4.0 - 4.0 * r - 8.0 * s - 4.0 * t, -4.0 * s);
        D3(7, -4.0 * t, -4.0 * t, 4.0 - 4.0 * r - 4.0 * s - 8.0 * t);
        D3(8, 4.0 * t, 0.0, 4.0 * r);
        D3(9, 0.0, 4.0 * t, 4.0 * s);
        break;
    case ORC_HEX8: {
        double st = s * t, rt = r * t, rs = r * s;
        D3(0, -1.0 + s + t - st, -1.0 + r + t - rt, -1.0 + r + s - rs);
        D3(1, +1.0 - s - t + st, -1.0 - r + t + rt, -1.0 - r + s + rs);
        D3(2, +1.0 + s - t - st, +1.0 + r - t - rt, -1.0 - r - s - rs);
        D3(3, -1.0 - s + t + st, +1.0 - r - t + rt, -1.0 + r - s + rs);
        D3(4, -1.0 + s - t + st, -1.0 + r - t + rt, +1.0 - r - s + rs);
        D3(5, +1.0 - s + t - st, -1.0 - r - t - rt, +1.0 + r - s - rs);
        D3(6, +1.0 + s + t + st, +1.0 + r + t + rt, +1.0 + r + s + rs);
        D3(7, -1.0 - s - t - st, +1.0 - r + t - rt, +1.0 - r + s - rs);
        for (int i = 0; i < 24; i++) D[i] = 0.125 * D[i];
        break;
    }
    case ORC_HEX20: {
        double rp1 = 1.0 + r, rm1 = 1.0 - r, sp1 = 1.0 + s, sm1 = 1.0 - s, tp1 = 1.0 + t, tm1 = 1.0 - t;
        D3(0, -0.125 * sm1 * tm1 * (-r - s - t - 2) - 0.125 * rm1 * sm1 * tm1,
              -0.125 * rm1 * tm1 * (-r - s - t - 2) - 0.125 * rm1 * sm1 * tm1,
              -0.125 * rm1 * sm1 * (-r - s - t - 2) - 0.125 * rm1 * sm1 * tm1);
        D3(1, 0.125 * sm1 * tm1 * (r - s - t - 2) + 0.125 * rp1 * sm1 * tm1,
              -0.125 * rp1 * tm1 * (r - s - t - 2) - 0.125 * rp1 * sm1 * tm1,
              -0.125 * rp1 * sm1 * (r - s - t - 2) - 0.125 * rp1 * sm1 * tm1);
        D3(2, 0.125 * sp1 * tm1 * (r + s - t - 2) + 0.125 * rp1 * sp1 * tm1,
              0.125 * rp1 * tm1 * (r + s - t - 2) + 0.125 * rp1 * sp1 * tm1,
              -0.125 * rp1 * sp1 * (r + s - t - 2) - 0.125 * rp1 * sp1 * tm1);
        D3(3, -0.125 * sp1 * tm1 * (-r + s - t - 2) - 0.125 * rm1 * sp1 * tm1,
              0.125 * rm1 * tm1 * (-r + s - t - 2) + 0.125 * rm1 * sp1 * tm1,
              -0.125 * rm1 * sp1 * (-r + s - t - 2) - 0.125 * rm1 * sp1 * tm1);
        D3(4, -0.125 * sm1 * tp1 * (-r - s + t - 2) - 0.125 * rm1 * sm1 * tp1,
              -0.125 * rm1 * tp1 * (-r - s + t - 2) - 0.125 * rm1 * sm1 * tp1,
              0.125 * rm1 * sm1 * (-r - s + t - 2) + 0.125 * rm1 * sm1 * tp1);
        D3(5, 0.125 * sm1 * tp1 * (r - s + t - 2) + 0.125 * rp1 * sm1 * tp1,
              -0.125 * rp1 * tp1 * (r - s + t - 2) - 0.125 * rp1 * sm1 * tp1,
              0.125 * rp1 * sm1 * (r - s + t - 2) + 0.125 * rp1 * sm1 * tp1);
        D3(6, 0.125 * sp1 * tp1 * (r + s + t - 2) + 0.125 * rp1 * sp1 * tp1,
              0.125 * rp1 * tp1 * (r + s + t - 2) + 0.125 * rp1 * sp1 * tp1,
              0.125 * rp1 * sp1 * (r + s + t - 2) + 0.125 * rp1 * sp1 * tp1);
        D3(7, -0.125 * sp1 * tp1 * (-r + s + t - 2) - 0.125 * rm1 * sp1 * tp1,
              0.125 * rm1 * tp1 * (-r + s + t - 2) + 0.125 * rm1 * sp1 * tp1,
              0.125 * rm1 * sp1 * (-r + s + t - 2) + 0.125 * rm1 * sp1 * tp1);
        D3(8, -0.5 * r * sm1 * tm1, -0.25 * (1 - r * r) * tm1, -0.25 * (1 - r * r) * sm1);
        D3(9, 0.25 * (1 - s * s) * tm1, -0.5 * s * rp1 * tm1, -0.25 * rp1 * (1 - s * s));
        D3(10, -0.5 * r * sp1 * tm1, 0.25 * (1 - r * r) * tm1, -0.25 * (1 - r * r) * sp1);
        D3(11, -0.25 * (1 - s * s) * tm1, -0.5 * s * rm1 * tm1, -0.25 * rm1 * (1 - s * s));
        D3(12, -0.5 * r * sm1 * tp1, -0.25 * (1 - r * r) * tp1, 0.25 * (1 - r * r) * sm1);
        D3(13, 0.25 * (1 - s * s) * tp1, -0.5 * s * rp1 * tp1, 0.25 * rp1 * (1 - s * s));
        D3(14, -0.5 * r * sp1 * tp1, 0.25 * (1 - r * r) * tp1, 0.25 * (1 - r * r) * sp1);
        D3(15, -0.25 * (1 - s * s) * tp1, -0.5 * s * rm1 * tp1, 0.25 * rm1 * (1 - s * s));
        D3(16, -0.25 * sm1 * (1 - t * t), -0.25 * rm1 * (1 - t * t), -0.5 * t * rm1 * sm1);
        D3(17, 0.25 * sm1 * (1 - t * t), -0.25 * rp1 * (1 - t * t), -0.5 * t * rp1 * sm1);
        D3(18, 0.25 * sp1 * (1 - t * t), 0.25 * rp1 * (1 - t * t), -0.5 * t * rp1 * sp1);
        D3(19, -0.25 * sp1 * (1 - t * t), 0.25 * rm1 * (1 - t * t), -0.5 * t * rm1 * sp1);
        break;
    }
    }
#undef D2
#undef D3
}

/* ------------------------------------------------------------------------ */
/* Quadrature: src/shape/quadrature.jl (same literal values as the tables)   */
/* ------------------------------------------------------------------------ */

static const double G2A = 0.577350269189625764509149;  /* LIN_IP2 */
static const double G3A = 0.774596669241483377035835;  /* LIN_IP3 */
static const double G3W0 = 0.555555555555555555555556, G3W1 = 0.888888888888888888888889;
static const double G4A = 0.861136311594052575223946, G4B = 0.339981043584856264802666;
static const double G4WA = 0.34785484513745385737306, G4WB = 0.65214515486254614262694;
static const double Q4A = 0.577350269189626;           /* QUAD_IP4 / HEX_IP8 */
static const double H27A = 0.774596669241483;          /* HEX_IP27 */
static const double H27W[4] = {0.171467764060357, 0.274348422496571, 0.438957475994513, 0.702331961591221};

static int set_pt(double *R, double *w, int i, double r, double s, double t, double wt) {
    R[3 * i] = r; R[3 * i + 1] = s; R[3 * i + 2] = t; w[i] = wt;
    return i + 1;
}

static int quad_lin(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) i = set_pt(R, w, i, 0.0, 0, 0, 2.0);
    else if (n == 2) { i = set_pt(R, w, i, -G2A, 0, 0, 1.0); i = set_pt(R, w, i, G2A, 0, 0, 1.0); }
    else if (n == 3) {
        i = set_pt(R, w, i, -G3A, 0, 0, G3W0); i = set_pt(R, w, i, 0.0, 0, 0, G3W1);
        i = set_pt(R, w, i, G3A, 0, 0, G3W0);
    } else if (n == 4) {
        i = set_pt(R, w, i, -G4A, 0, 0, G4WA); i = set_pt(R, w, i, -G4B, 0, 0, G4WB);
        i = set_pt(R, w, i, G4B, 0, 0, G4WB); i = set_pt(R, w, i, G4A, 0, 0, G4WA);
    } else return -1;
    return i;
}

static int quad_tri(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) i = set_pt(R, w, i, 1.0 / 3.0, 1.0 / 3.0, 0, 1.0 / 2.0);
    else if (n == 3) {
        i = set_pt(R, w, i, 1.0 / 6.0, 1.0 / 6.0, 0, 1.0 / 6.0);
        i = set_pt(R, w, i, 2.0 / 3.0, 1.0 / 6.0, 0, 1.0 / 6.0);
        i = set_pt(R, w, i, 1.0 / 6.0, 2.0 / 3.0, 0, 1.0 / 6.0);
    } else if (n == 6) {
        i = set_pt(R, w, i, 0.091576213509771, 0.091576213509771, 0, 0.109951743655322 / 2.0);
        i = set_pt(R, w, i, 0.816847572980459, 0.091576213509771, 0, 0.109951743655322 / 2.0);
        i = set_pt(R, w, i, 0.091576213509771, 0.816847572980459, 0, 0.109951743655322 / 2.0);
        i = set_pt(R, w, i, 0.445948490915965, 0.445948490915965, 0, 0.223381589678011 / 2.0);
        i = set_pt(R, w, i, 0.108103018168070, 0.445948490915965, 0, 0.223381589678011 / 2.0);
        i = set_pt(R, w, i, 0.445948490915965, 0.108103018168070, 0, 0.223381589678011 / 2.0);
    } else return -1;
    return i;
}

static int quad_quad(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) i = set_pt(R, w, i, 0.0, 0.0, 0, 4.0);
    else if (n == 4) {
        i = set_pt(R, w, i, -Q4A, -Q4A, 0, 1.0); i = set_pt(R, w, i, Q4A, -Q4A, 0, 1.0);
        i = set_pt(R, w, i, -Q4A, Q4A, 0, 1.0);  i = set_pt(R, w, i, Q4A, Q4A, 0, 1.0);
    } else if (n == 9) {
        double a = 0.2 * sqrt(15.0), w25 = 25.0 / 81.0, w40 = 40.0 / 81.0, w64 = 64.0 / 81.0;
        const double p[3] = {-a, 0.0, a};
        const double ww[3][3] = {{w25, w40, w25}, {w40, w64, w40}, {w25, w40, w25}};
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++) i = set_pt(R, w, i, p[k], p[j], 0, ww[j][k]);
    } else if (n == 16) {
        const double p[4] = {-0.861136311594053, -0.339981043584856, 0.339981043584856, 0.861136311594053};
        const double wa = 0.121002993285602, wb = 0.226851851851852, wc = 0.425293303010694;
        const double ww[4][4] = {{wa, wb, wb, wa}, {wb, wc, wc, wb}, {wb, wc, wc, wb}, {wa, wb, wb, wa}};
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++) i = set_pt(R, w, i, p[k], p[j], 0, ww[j][k]);
    } else return -1;
    return i;
}

static int quad_tet(int n, double *R, double *w) {
    int i = 0;
    if (n == 1) i = set_pt(R, w, i, 0.25, 0.25, 0.25, 1.0 / 6.0);
    else if (n == 4) {
        const double a = 0.5854101966249685, b = 0.1381966011250105, wt = 0.04166666666666667;
        i = set_pt(R, w, i, a, b, b, wt); i = set_pt(R, w, i, b, a, b, wt);
        i = set_pt(R, w, i, b, b, a, wt); i = set_pt(R, w, i, b, b, b, wt);
    } else if (n == 5) {
        i = set_pt(R, w, i, 0.25, 0.25, 0.25, -2.0 / 15.0);
        i = set_pt(R, w, i, 1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0, 3.0 / 40.0);
        i = set_pt(R, w, i, 1.0 / 6.0, 1.0 / 6.0, 0.5, 3.0 / 40.0);
        i = set_pt(R, w, i, 1.0 / 6.0, 0.5, 1.0 / 6.0, 3.0 / 40.0);
        i = set_pt(R, w, i, 0.5, 1.0 / 6.0, 1.0 / 6.0, 3.0 / 40.0);
    } else return -1;
    return i;
}

static int quad_hex(int n, double *R, double *w) {
    int i = 0;
    if (n == 8) {
        for (int k = 0; k < 2; k++)
            for (int j = 0; j < 2; j++)
                for (int l = 0; l < 2; l++)
                    i = set_pt(R, w, i, l ? Q4A : -Q4A, j ? Q4A : -Q4A, k ? Q4A : -Q4A, 1.0);
    } else if (n == 27) {
        const double p[3] = {-H27A, 0.0, H27A};
        for (int k = 0; k < 3; k++)
            for (int j = 0; j < 3; j++)
                for (int l = 0; l < 3; l++) {
                    int nz = (l == 1) + (j == 1) + (k == 1);
                    i = set_pt(R, w, i, p[l], p[j], p[k], H27W[nz]);
                }
    } else return -1;
    return i;
}

/* get_ip_coords(shape, nips) with the default key 0 (src/shape/shape.jl:61) */
int orc_quadrature(int shape, int nips, double *R, double *w) {
    switch (shape) {
    case ORC_LIN2: case ORC_LIN3: return quad_lin(nips == 0 ? 2 : nips, R, w);
    case ORC_TRI3: return quad_tri(nips == 0 ? 3 : nips, R, w);
    case ORC_TRI6: return (nips == 1) ? -1 : quad_tri(nips == 0 ? 3 : nips, R, w);
    case ORC_QUAD4: case ORC_QUAD8: return quad_quad(nips == 0 ? 4 : nips, R, w);
    case ORC_QUAD9: return (nips == 1) ? -1 : quad_quad(nips == 0 ? 9 : nips, R, w);
    case ORC_TET4: case ORC_TET10: return quad_tet(nips == 0 ? 4 : nips, R, w);
    case ORC_HEX8: case ORC_HEX20: return quad_hex(nips == 0 ? 8 : nips, R, w);
    }
    return -1;
}

/* ------------------------------------------------------------------------ */
/* Tensors and materials (Mandel notation)                                   */
/* ------------------------------------------------------------------------ */

/* src/tools/tensors.jl:18-27 */
static double J2(const double *s) {
    double t11 = s[0], t22 = s[1], t33 = s[2], t23 = s[3] / SR2, t13 = s[4] / SR2, t12 = s[5] / SR2;
    return 1.0 / 6.0 * ((t11 - t22) * (t11 - t22) + (t22 - t33) * (t22 - t33) + (t33 - t11) * (t33 - t11)) +
           t23 * t23 + t13 * t13 + t12 * t12;
}

/* dev(T) = Psd*T  (src/tools/tensors.jl:4-12) */
static void dev(const double *T, double *S) {
    S[0] = 2.0 / 3.0 * T[0] - 1.0 / 3.0 * T[1] - 1.0 / 3.0 * T[2];
    S[1] = -1.0 / 3.0 * T[0] + 2.0 / 3.0 * T[1] - 1.0 / 3.0 * T[2];
    S[2] = -1.0 / 3.0 * T[0] - 1.0 / 3.0 * T[1] + 2.0 / 3.0 * T[2];
    S[3] = T[3]; S[4] = T[4]; S[5] = T[5];
}

static double norm6(const double *v) {
    double a = 0.0;
    for (int i = 0; i < 6; i++) a += v[i] * v[i];
    return sqrt(a);
}

static void matvec6(const double *A, const double *x, double *y) {
    for (int i = 0; i < 6; i++) {
        double a = 0.0;
        for (int j = 0; j < 6; j++) a += A[6 * i + j] * x[j];
        y[i] = a;
    }
}

/* calcDe: src/mech/mat/linear-elastic.jl:98-119 (row-major 6x6) */
static void calcDe(double E, double nu, int planestress, double *De) {
    memset(De, 0, 36 * sizeof(double));
    if (planestress) {
        double c = E / (1 - nu * nu);
        De[0] = c; De[1] = c * nu; De[6] = c * nu; De[7] = c;
        De[21] = c * (1.0 - nu); De[28] = c * (1.0 - nu); De[35] = c * (1.0 - nu);
    } else {
        double c = E / ((1 + nu) * (1 - 2 * nu));
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) De[6 * i + j] = (i == j) ? c * (1 - nu) : c * nu;
        De[21] = c * (1 - 2 * nu); De[28] = c * (1 - 2 * nu); De[35] = c * (1 - 2 * nu);
    }
}

/* D - (D a)(D b)^T / den  with a, b vectors (generic rank-one correction) */
static void rank1_correct(double *D, const double *De, const double *a, const double *b, double den) {
    double Da[6], Db[6];
    matvec6(De, a, Da);
    /* b' * De  (De symmetric) */
    matvec6(De, b, Db);
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++) D[6 * i + j] = De[6 * i + j] - Da[i] * Db[j] / den;
}

static void calcD(int mtype, const double *par, int stressmodel, const double *st, double *D) {
    double E = par[0], nu = par[1];
    int ps = (stressmodel == ORC_PLANESTRESS);
    double De[36];
    if (mtype == ORC_LINEAR_ELASTIC) { /* linear-elastic.jl:125-127,148-150 */
        calcDe(E, nu, ps, D);
        return;
    }
    if (mtype == ORC_VON_MISES) {
        double H = par[3], fy = par[2];
        calcDe(E, nu, ps, De);
        if (st[ORC_ST_DL] == 0.0) { memcpy(D, De, sizeof De); return; }
        const double *s0 = st + ORC_ST_SIG;
        if (!ps) { /* von-mises.jl:112-126 */
            double s[6], a[6], Da[6];
            dev(s0, s);
            double ns = norm6(s);
            for (int i = 0; i < 6; i++) a[i] = sqrt(1.5) * s[i] / ns;
            matvec6(De, a, Da);
            double aDa = 0.0;
            for (int i = 0; i < 6; i++) aDa += a[i] * Da[i];
            rank1_correct(D, De, a, a, aDa - sqrt(1.5) * (-H));
        } else { /* von-mises.jl:187-198 */
            const double *sg = s0;
            double s[6] = {2.0 / 3.0 * sg[0] - 1.0 / 3.0 * sg[1], 2.0 / 3.0 * sg[1] - 1.0 / 3.0 * sg[0],
                           -1.0 / 3.0 * sg[0] - 1.0 / 3.0 * sg[1], sg[3], sg[4], sg[5]};
            double dfdep = -2.0 / 3.0 * H * (fy + H * st[ORC_ST_EPA]);
            double Ds[6], sDs = 0.0;
            matvec6(De, s, Ds);
            for (int i = 0; i < 6; i++) sDs += s[i] * Ds[i];
            rank1_correct(D, De, s, s, sDs - norm6(s) * dfdep);
        }
        return;
    }
    /* DruckerPrager: drucker-prager.jl:86-109 */
    {
        double alpha = par[2], H = par[4];
        calcDe(E, nu, ps, De);
        if (st[ORC_ST_DL] == 0.0) { memcpy(D, De, sizeof De); return; }
        const double *sg = st + ORC_ST_SIG;
        double V[6], Nu[6];
        double j2d = J2(sg);
        if (j2d != 0.0) {
            double s[6];
            dev(sg, s);
            double ns = norm6(s);
            for (int i = 0; i < 6; i++) V[i] = alpha * (i < 3 ? 1.0 : 0.0) + (s[i] / ns) / SR2;
            double nv = norm6(V);
            for (int i = 0; i < 6; i++) Nu[i] = V[i] / nv;
        } else {
            for (int i = 0; i < 6; i++) { Nu[i] = (i < 3) ? 1.0 / sqrt(3.0) : 0.0; V[i] = Nu[i]; }
        }
        double DNu[6], VDNu = 0.0;
        matvec6(De, Nu, DNu);
        for (int i = 0; i < 6; i++) VDNu += V[i] * DNu[i];
        rank1_correct(D, De, Nu, V, VDNu + H);
    }
}

/* Plane-stress von Mises helpers: von-mises.jl:306-333 */
static void vm_ps_sigma(double E, double nu, double epa0, const double *str, double dl, double *sig, double *epa) {
    double G = E / (2 * (1 + nu));
    double den = E * E * dl * dl - 2 * E * nu * dl + 4 * E * dl - 3 * nu * nu + 3;
    double m11 = (2 * E * dl - E * nu * dl - 3 * nu * nu + 3) / den;
    double m12 = (E * dl - 2 * E * nu * dl) / den;
    double m66 = 1 / (2 * G * dl + 1);
    sig[0] = m11 * str[0] + m12 * str[1];
    sig[1] = m12 * str[0] + m11 * str[1];
    sig[2] = 0.0;
    sig[3] = m66 * str[3]; sig[4] = m66 * str[4]; sig[5] = m66 * str[5];
    double d[6] = {2.0 / 3.0 * sig[0] - 1.0 / 3.0 * sig[1], 2.0 / 3.0 * sig[1] - 1.0 / 3.0 * sig[0],
                   -1.0 / 3.0 * sig[0] - 1.0 / 3.0 * sig[1], sig[3], sig[4], sig[5]};
    *epa = epa0 + dl * norm6(d);
}

static double vm_ps_yield(double fy, double H, const double *sig, double epa) {
    double j2d = J2(sig);
    return j2d - 1.0 / 3.0 * (fy + H * epa) * (fy + H * epa);
}

/* update_state!(mat, state, dε) -> dσ; returns 0 on success */
static int update_mat(int mtype, const double *par, int stressmodel, double *st, const double *de, double *dsig,
                      char *msg, int msglen) {
    double E = par[0], nu = par[1];
    int ps = (stressmodel == ORC_PLANESTRESS);
    double De[36], sini[6], str[6], tmp[6];
    double *sig = st + ORC_ST_SIG, *eps = st + ORC_ST_EPS;
    calcDe(E, nu, ps, De);
    memcpy(sini, sig, sizeof sini);
    matvec6(De, de, tmp);
    for (int i = 0; i < 6; i++) str[i] = sig[i] + tmp[i];

    if (mtype == ORC_LINEAR_ELASTIC) { /* linear-elastic.jl:130-137,153-159 */
        for (int i = 0; i < 6; i++) { dsig[i] = tmp[i]; eps[i] += de[i]; sig[i] += tmp[i]; }
        return 0;
    }
    if (mtype == ORC_VON_MISES && !ps) { /* von-mises.jl:128-157 */
        double fy = par[2], H = par[3];
        double ftr = sqrt(3 * J2(str)) - fy - H * st[ORC_ST_EPA];
        if (ftr < 1e-8) {
            st[ORC_ST_DL] = 0.0;
            memcpy(sig, str, sizeof str);
        } else {
            double G = E / (2 * (1 + nu));
            double j2dtr = J2(str);
            st[ORC_ST_DL] = ftr / (3 * G + sqrt(1.5) * H);
            if (!(sqrt(j2dtr) - st[ORC_ST_DL] * sqrt(3.0) * G >= 0.0)) {
                snprintf(msg, msglen, "VonMisses: Negative value for \xe2\x88\x9aJ2D");
                return -4;
            }
            double s[6], d[6];
            dev(str, d);
            double f = 1 - sqrt(3.0) * G * st[ORC_ST_DL] / sqrt(j2dtr);
            for (int i = 0; i < 6; i++) s[i] = f * d[i];
            double ns = norm6(s);
            for (int i = 0; i < 6; i++) sig[i] = str[i] - sqrt(6.0) * G * st[ORC_ST_DL] * s[i] / ns;
            st[ORC_ST_EPA] += st[ORC_ST_DL];
        }
        for (int i = 0; i < 6; i++) { eps[i] += de[i]; dsig[i] = sig[i] - sini[i]; }
        return 0;
    }
    if (mtype == ORC_VON_MISES && ps) { /* von-mises.jl:200-303 */
        double fy = par[2], H = par[3];
        double ftr = vm_ps_yield(fy, H, str, st[ORC_ST_EPA]);
        if (ftr < 1e-8) {
            st[ORC_ST_DL] = 0.0;
            memcpy(sig, str, sizeof str);
        } else {
            double dfds[6] = {2.0 / 3.0 * str[0] - 1.0 / 3.0 * str[1], 2.0 / 3.0 * str[1] - 1.0 / 3.0 * str[0],
                              -1.0 / 3.0 * str[0] - 1.0 / 3.0 * str[1], str[3], str[4], str[5]};
            double Dd[6], dd[6];
            matvec6(De, dfds, Dd);
            for (int i = 0; i < 6; i++) dd[i] = str[i] - sig[i];
            double dl0 = norm6(dd) / norm6(Dd);
            double a = 0.0, b = dl0, sg[6], epa, fa, fb, f = 0.0, dl = 0.0;
            double epa0 = st[ORC_ST_EPA];
            vm_ps_sigma(E, nu, epa0, str, a, sg, &epa);
            fa = vm_ps_yield(fy, H, sg, epa);
            vm_ps_sigma(E, nu, epa0, str, b, sg, &epa);
            fb = vm_ps_yield(fy, H, sg, epa);
            if (fa * fb > 0) {
                int maxits = 50;
                for (int i = 1; i <= maxits; i++) {
                    b += dl0 * pow(1.6, i);
                    vm_ps_sigma(E, nu, epa0, str, b, sg, &epa);
                    fb = vm_ps_yield(fy, H, sg, epa);
                    if (fa * fb < 0.0) break;
                    if (i == maxits) {
                        snprintf(msg, msglen, "VonMises: Could not find interval for \xce\x94\xce\xbb");
                        return -4;
                    }
                }
            }
            double s0[6] = {0, 0, 0, 0, 0, 0};
            double tol = pow(10.0, -(10 - log10(fy)));
            int maxits = 50;
            for (int i = 1; i <= maxits; i++) {
                dl = (a + b) / 2;
                vm_ps_sigma(E, nu, epa0, str, dl, sg, &epa);
                f = vm_ps_yield(fy, H, sg, epa);
                if (fa * f < 0) b = dl;
                else { a = dl; fa = f; }
                double mx = 0.0;
                for (int k = 0; k < 6; k++) mx = fmax(mx, fabs(sg[k] - s0[k]));
                if (mx <= tol) break;
                memcpy(s0, sg, sizeof s0);
                if (i == maxits) {
                    snprintf(msg, msglen, "VonMises: could not find \xce\x94\xce\xbb with NR/bissection (maxits reached, f=%g)", f);
                    return -4;
                }
            }
            memcpy(sig, sg, sizeof sg);
            st[ORC_ST_EPA] = epa;
            st[ORC_ST_DL] = dl;
        }
        for (int i = 0; i < 6; i++) { eps[i] += de[i]; dsig[i] = sig[i] - sini[i]; }
        return 0;
    }
    /* DruckerPrager: drucker-prager.jl:112-149 */
    {
        double alpha = par[2], kappa = par[3], H = par[4];
        double j1 = str[0] + str[1] + str[2];
        double ftr = alpha * j1 + sqrt(J2(str)) - kappa - H * st[ORC_ST_EPA];
        if (ftr < 1.e-8) {
            st[ORC_ST_DL] = 0.0;
            memcpy(sig, str, sizeof str);
        } else {
            double K = E / (3.0 * (1.0 - 2.0 * nu)), G = E / (2.0 * (1.0 + nu));
            double n = 1.0 / sqrt(3.0 * alpha * alpha + 0.5);
            double j1tr = j1, j2dtr = J2(str);
            if (sqrt(j2dtr) - st[ORC_ST_DL] * n * G > 0.0) {
                st[ORC_ST_DL] = ftr / (9 * alpha * alpha * n * K + n * G + H);
                double jj1 = j1tr - 9 * st[ORC_ST_DL] * alpha * n * K;
                double m = 1.0 - st[ORC_ST_DL] * n * G / sqrt(j2dtr);
                double d[6];
                dev(str, d);
                for (int i = 0; i < 6; i++) sig[i] = m * d[i] + (i < 3 ? jj1 / 3.0 : 0.0);
            } else {
                st[ORC_ST_DL] = (alpha * j1tr - kappa - H * st[ORC_ST_EPA]) / (3 * sqrt(3.0) * alpha * K + H);
                double jj1 = j1tr - 3 * sqrt(3.0) * st[ORC_ST_DL] * K;
                for (int i = 0; i < 6; i++) sig[i] = (i < 3 ? jj1 / 3.0 : 0.0);
            }
            st[ORC_ST_EPA] += st[ORC_ST_DL];
        }
        for (int i = 0; i < 6; i++) { eps[i] += de[i]; dsig[i] = sig[i] - sini[i]; }
        return 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Element level: src/mech/elem/mech-solid.jl                                */
/* ------------------------------------------------------------------------ */

#define MAXN 27
#define MAXND (3 * MAXN)
#define MAXIP 27

typedef struct {
    int nn, nd, ndim, nip;
    double C[MAXN * 3];
    double R[MAXIP * 3], w[MAXIP];
    int64_t map[MAXND];
} elem_ctx;

static int load_elem(const orc_model *m, int64_t e, elem_ctx *E) {
    int shape = m->shape[e];
    int64_t p0 = m->conn_ptr[e];
    E->nn = (int)(m->conn_ptr[e + 1] - p0);
    E->ndim = m->ndim;
    E->nd = E->nn * m->ndim;
    if (E->nn != orc_shape_npoints(shape)) return -1;
    for (int i = 0; i < E->nn; i++) {
        int64_t n = m->conn[p0 + i];
        for (int k = 0; k < m->ndim; k++) {
            E->C[i * m->ndim + k] = m->coords[3 * n + k];
            E->map[i * m->ndim + k] = m->eq_id[3 * n + k];
        }
    }
    E->nip = orc_quadrature(shape, m->nips[e], E->R, E->w);
    if (E->nip <= 0) return -1;
    if (m->ip_ptr[e + 1] - m->ip_ptr[e] != E->nip) return -1;
    return 0;
}

/* J = C'*dNdR ; dNdX = dNdR*inv(J) ; detJ = det(J)   (mech-solid.jl:146-149) */
static double jacobian(const elem_ctx *E, const double *dNdR, double *dNdX) {
    int nn = E->nn, nd = E->ndim;
    double J[9] = {0}, iJ[9], det;
    for (int a = 0; a < nd; a++)
        for (int b = 0; b < nd; b++) {
            double s = 0.0;
            for (int i = 0; i < nn; i++) s += E->C[i * nd + a] * dNdR[i * nd + b];
            J[a * nd + b] = s;
        }
    if (nd == 2) {
        det = J[0] * J[3] - J[1] * J[2];
        iJ[0] = J[3] / det; iJ[1] = -J[1] / det; iJ[2] = -J[2] / det; iJ[3] = J[0] / det;
    } else {
        det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
        iJ[0] = (J[4] * J[8] - J[5] * J[7]) / det;
        iJ[1] = (J[2] * J[7] - J[1] * J[8]) / det;
        iJ[2] = (J[1] * J[5] - J[2] * J[4]) / det;
        iJ[3] = (J[5] * J[6] - J[3] * J[8]) / det;
        iJ[4] = (J[0] * J[8] - J[2] * J[6]) / det;
        iJ[5] = (J[2] * J[3] - J[0] * J[5]) / det;
        iJ[6] = (J[3] * J[7] - J[4] * J[6]) / det;
        iJ[7] = (J[1] * J[6] - J[0] * J[7]) / det;
        iJ[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    }
    for (int i = 0; i < nn; i++)
        for (int b = 0; b < nd; b++) {
            double s = 0.0;
            for (int a = 0; a < nd; a++) s += dNdR[i * nd + a] * iJ[a * nd + b];
            dNdX[i * nd + b] = s;
        }
    return det;
}

/* setB: mech-solid.jl:82-121 ; B is 6 x nd row-major */
static void setB(const elem_ctx *E, int stressmodel, const double *dNdX, const double *N, double r, double *B) {
    int nn = E->nn, nd = E->nd;
    memset(B, 0, 6 * nd * sizeof(double));
    if (E->ndim == 2) {
        for (int i = 0; i < nn; i++) {
            B[0 * nd + 2 * i] = dNdX[2 * i];
            B[1 * nd + 2 * i + 1] = dNdX[2 * i + 1];
            B[5 * nd + 2 * i] = dNdX[2 * i + 1] / SR2;
            B[5 * nd + 2 * i + 1] = dNdX[2 * i] / SR2;
        }
        if (stressmodel == ORC_AXISYM)
            for (int i = 0; i < nn; i++) B[2 * nd + 2 * i] = N[i] / r;
    } else {
        for (int i = 0; i < nn; i++) {
            double dx = dNdX[3 * i], dy = dNdX[3 * i + 1], dz = dNdX[3 * i + 2];
            B[0 * nd + 3 * i] = dx;
            B[1 * nd + 3 * i + 1] = dy;
            B[2 * nd + 3 * i + 2] = dz;
            B[3 * nd + 3 * i + 1] = dz / SR2; B[3 * nd + 3 * i + 2] = dy / SR2;
            B[4 * nd + 3 * i] = dz / SR2;     B[4 * nd + 3 * i + 2] = dx / SR2;
            B[5 * nd + 3 * i] = dy / SR2;     B[5 * nd + 3 * i + 1] = dx / SR2;
        }
    }
}

/* IP geometry: returns detJ, fills B and coef-thickness */
static double ip_geometry(const orc_model *m, const elem_ctx *E, int shape, int ip, double *B, double *th) {
    double dNdR[MAXN * 3], dNdX[MAXN * 3], N[MAXN];
    const double *R = E->R + 3 * ip;
    orc_shape_deriv(shape, R, dNdR);
    orc_shape_func(shape, R, N);
    double detJ = jacobian(E, dNdR, dNdX);
    double r = 0.0;
    for (int i = 0; i < E->nn; i++) r += E->C[i * E->ndim] * N[i];
    *th = (m->stressmodel == ORC_AXISYM) ? 2 * M_PI * r : m->thickness;
    setB(E, m->stressmodel, dNdX, N, r, B);
    return detJ;
}

/* elem_stiffness: mech-solid.jl:124-166 ; Ke row-major nd x nd */
int orc_elem_stiffness(const orc_model *m, int64_t e, double *Ke, int64_t *map) {
    elem_ctx E;
    if (load_elem(m, e, &E)) return -1;
    int nd = E.nd, shape = m->shape[e];
    double B[6 * MAXND], DB[6 * MAXND], D[36];
    memset(Ke, 0, (size_t)nd * nd * sizeof(double));
    for (int ip = 0; ip < E.nip; ip++) {
        double th;
        double detJ = ip_geometry(m, &E, shape, ip, B, &th);
        if (!(detJ > 0.0)) return -3;
        double coef = detJ * E.w[ip] * th;
        const double *st = m->state + ORC_ST_LEN * (m->ip_ptr[e] + ip);
        calcD(m->mat_type[e], m->mat_par + 8 * e, m->stressmodel, st, D);
        for (int i = 0; i < 6; i++)
            for (int j = 0; j < nd; j++) {
                double s = 0.0;
                for (int k = 0; k < 6; k++) s += D[6 * i + k] * B[k * nd + j];
                DB[i * nd + j] = s;
            }
        for (int i = 0; i < nd; i++)
            for (int j = 0; j < nd; j++) {
                double s = 0.0;
                for (int k = 0; k < 6; k++) s += B[k * nd + i] * DB[k * nd + j];
                Ke[i * nd + j] += coef * s;
            }
    }
    for (int i = 0; i < nd; i++) map[i] = E.map[i];
    return nd;
}

/*
 * mount_K COO part (mech-solver.jl:78-98): every element entry with
 * |Ke_ij| >= eps() is pushed in element order, rows outer, cols inner.
 * R/C/V must hold sum(nd^2) entries.  Returns the number of triples, or a
 * negative status (-3 negative Jacobian, -1 bad element).
 */
int64_t orc_mount_K_coo(const orc_model *m, int nthreads, int64_t *R, int64_t *C, double *V, int64_t *bad_elem) {
    int64_t ne = n_active(m);
    int64_t *off = (int64_t *)malloc((ne + 1) * sizeof(int64_t));
    int64_t *cnt = (int64_t *)calloc(ne, sizeof(int64_t));
    int status = 0;
    off[0] = 0;
    for (int64_t i = 0; i < ne; i++) {
        int64_t e = active_elem(m, i);
        int64_t nn = m->conn_ptr[e + 1] - m->conn_ptr[e];
        off[i + 1] = off[i] + nn * m->ndim * nn * m->ndim;
    }
    *bad_elem = -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        double *Ke = (double *)malloc(MAXND * MAXND * sizeof(double));
        int64_t map[MAXND];
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int64_t i = 0; i < ne; i++) {
            int64_t e = active_elem(m, i);
            int nd = orc_elem_stiffness(m, e, Ke, map);
            if (nd < 0) {
#ifdef _OPENMP
#pragma omp critical
#endif
                {
                    if (*bad_elem < 0 || e < *bad_elem) { *bad_elem = e; status = nd; }
                }
                continue;
            }
            int64_t k = off[i];
            for (int i = 0; i < nd; i++)
                for (int j = 0; j < nd; j++) {
                    double val = Ke[i * nd + j];
                    if (fabs(val) < 2.220446049250313e-16) continue; /* eps() */
                    R[k] = map[i]; C[k] = map[j]; V[k] = val; k++;
                }
            cnt[i] = k - off[i];
        }
        free(Ke);
    }
    if (status) { free(off); free(cnt); return status; }
    /* compact in element order */
    int64_t w = 0;
    for (int64_t i = 0; i < ne; i++) {
        int64_t s = off[i];
        if (w != s) {
            memmove(R + w, R + s, cnt[i] * sizeof(int64_t));
            memmove(C + w, C + s, cnt[i] * sizeof(int64_t));
            memmove(V + w, V + s, cnt[i] * sizeof(double));
        }
        w += cnt[i];
    }
    free(off); free(cnt);
    return w;
}

/*
 * SparseArrays.sparse(I, J, V, n, n) with combine=+ : duplicates are summed in
 * input order, summed zeros are kept, row indices sorted within columns.
 * colptr has n+1 entries; rowval/nzval hold at most cnt entries.  0-based.
 */
int64_t orc_sparse_csc(int64_t n, int64_t cnt, const int64_t *R, const int64_t *C, const double *V,
                       int64_t *colptr, int64_t *rowval, double *nzval) {
    int64_t *cc = (int64_t *)calloc(n + 1, sizeof(int64_t));
    int64_t *ord = (int64_t *)malloc((cnt > 0 ? cnt : 1) * sizeof(int64_t));
    int64_t *last = (int64_t *)malloc((n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t k = 0; k < cnt; k++) cc[C[k] + 1]++;
    for (int64_t j = 0; j < n; j++) cc[j + 1] += cc[j];
    {
        int64_t *pos = (int64_t *)malloc((n + 1) * sizeof(int64_t));
        memcpy(pos, cc, (n + 1) * sizeof(int64_t));
        for (int64_t k = 0; k < cnt; k++) ord[pos[C[k]]++] = k; /* stable by column */
        free(pos);
    }
    for (int64_t i = 0; i < n; i++) last[i] = -1;
    int64_t nnz = 0;
    colptr[0] = 0;
    for (int64_t j = 0; j < n; j++) {
        int64_t start = nnz;
        for (int64_t q = cc[j]; q < cc[j + 1]; q++) {
            int64_t k = ord[q], r = R[k];
            if (last[r] >= start) nzval[last[r]] += V[k];
            else { last[r] = nnz; rowval[nnz] = r; nzval[nnz] = V[k]; nnz++; }
        }
        /* insertion sort rows of this column */
        for (int64_t a = start + 1; a < nnz; a++) {
            int64_t rr = rowval[a];
            double vv = nzval[a];
            int64_t b = a - 1;
            while (b >= start && rowval[b] > rr) { rowval[b + 1] = rowval[b]; nzval[b + 1] = nzval[b]; b--; }
            rowval[b + 1] = rr; nzval[b + 1] = vv;
        }
        colptr[j + 1] = nnz;
    }
    free(cc); free(ord); free(last);
    return nnz;
}

/* update_elem!: mech-solid.jl:243-279.  dF has nd entries. */
static int update_elem(orc_model *m, int64_t e, const double *U, double *dF, int64_t *map, char *msg, int msglen) {
    elem_ctx E;
    if (load_elem(m, e, &E)) { snprintf(msg, msglen, "bad element %lld", (long long)e); return -1; }
    int nd = E.nd, shape = m->shape[e];
    double B[6 * MAXND], dU[MAXND];
    for (int i = 0; i < nd; i++) { map[i] = E.map[i]; dU[i] = U[E.map[i]]; dF[i] = 0.0; }
    for (int ip = 0; ip < E.nip; ip++) {
        double th;
        double detJ = ip_geometry(m, &E, shape, ip, B, &th);
        double de[6], ds[6];
        for (int i = 0; i < 6; i++) {
            double s = 0.0;
            for (int j = 0; j < nd; j++) s += B[i * nd + j] * dU[j];
            de[i] = s;
        }
        double *st = m->state + ORC_ST_LEN * (m->ip_ptr[e] + ip);
        int rc = update_mat(m->mat_type[e], m->mat_par + 8 * e, m->stressmodel, st, de, ds, msg, msglen);
        if (rc) return rc;
        double coef = detJ * E.w[ip] * th;
        for (int j = 0; j < nd; j++) {
            double s = 0.0;
            for (int i = 0; i < 6; i++) s += B[i * nd + j] * ds[i];
            dF[j] += coef * s;
        }
    }
    return nd;
}

/*
 * update_state!(active_elems, dU, t): mech-solver.jl:124-144 with the
 * @withthreads contiguous chunking (src/tools/threads.jl:86-126).  States are
 * updated in place; dFin (ndofs) receives the sum of element forces, thread
 * partials reduced in thread order.  Returns 0, or the first failure status
 * in thread order (its message in msg).
 */
int orc_update_state(orc_model *m, int nthreads, int64_t ndofs, const double *U, double *dFin, char *msg, int msglen) {
    int64_t ne = n_active(m);
    int nt = nthreads > 0 ? nthreads : 1;
    if (ne < nt) nt = (int)(ne > 0 ? ne : 1);
    double *part = (double *)calloc((size_t)nt * ndofs, sizeof(double));
    int *st = (int *)calloc(nt, sizeof(int));
    char *msgs = (char *)calloc((size_t)nt * 256, 1);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static, 1)
#endif
    for (int tid = 0; tid < nt; tid++) {
        int64_t nmin = (int64_t)tid * (ne / nt);
        int64_t nmax = (tid == nt - 1) ? ne : (int64_t)(tid + 1) * (ne / nt);
        double dF[MAXND];
        int64_t map[MAXND];
        for (int64_t i = nmin; i < nmax; i++) {
            int nd = update_elem(m, active_elem(m, i), U, dF, map, msgs + 256 * tid, 256);
            if (nd < 0) { st[tid] = nd; break; }
            for (int i = 0; i < nd; i++) part[(size_t)tid * ndofs + map[i]] += dF[i];
        }
    }
    for (int64_t i = 0; i < ndofs; i++) dFin[i] = 0.0;
    for (int tid = 0; tid < nt; tid++)
        for (int64_t i = 0; i < ndofs; i++) dFin[i] += part[(size_t)tid * ndofs + i];
    int rc = 0;
    for (int tid = 0; tid < nt; tid++)
        if (st[tid]) { rc = st[tid]; snprintf(msg, msglen, "%s", msgs + 256 * tid); break; }
    free(part); free(st); free(msgs);
    return rc;
}

/* Standalone single-IP material update (unit harness in the spirit of
 * src/mech/mat/integrator.jl). */
int orc_material_update(int mtype, const double *par, int stressmodel, double *st, const double *de, double *dsig,
                        char *msg, int msglen) {
    return update_mat(mtype, par, stressmodel, st, de, dsig, msg, msglen);
}

void orc_material_tangent(int mtype, const double *par, int stressmodel, const double *st, double *D) {
    calcD(mtype, par, stressmodel, st, D);
}
