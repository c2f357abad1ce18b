"""Oracle restatement of Amaru.jl's mechanical path (test infrastructure only).

Numerical kernels live in ``orc.c`` (compiled on first use into
``oracle/_build/liborc.so``); this module restates the host-side logic that
surrounds them.  Every function cites the Amaru.jl file it follows.
"""
import ast
import ctypes as C
import math
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liborc.so")

# shape codes, identical to the library header's numbering
LIN2, LIN3, TRI3, TRI6, QUAD4, QUAD8, QUAD9, TET4, TET10, HEX8, HEX20 = range(1, 12)
SHAPE_NAMES = {LIN2: "LIN2", LIN3: "LIN3", TRI3: "TRI3", TRI6: "TRI6", QUAD4: "QUAD4", QUAD8: "QUAD8",
               QUAD9: "QUAD9", TET4: "TET4", TET10: "TET10", HEX8: "HEX8", HEX20: "HEX20"}
NPOINTS = {LIN2: 2, LIN3: 3, TRI3: 3, TRI6: 6, QUAD4: 4, QUAD8: 8, QUAD9: 9, TET4: 4, TET10: 10, HEX8: 8, HEX20: 20}
SHAPE_NDIM = {LIN2: 1, LIN3: 1, TRI3: 2, TRI6: 2, QUAD4: 2, QUAD8: 2, QUAD9: 2, TET4: 3, TET10: 3, HEX8: 3, HEX20: 3}

# facet tables (1-based in the reference; 0-based here): shape/solids2d.jl, solids3d.jl
FACETS = {
    HEX8: (QUAD4, [[1, 5, 8, 4], [2, 3, 7, 6], [1, 2, 6, 5], [3, 4, 8, 7], [1, 4, 3, 2], [5, 6, 7, 8]]),
    HEX20: (QUAD8, [[1, 5, 8, 4, 17, 16, 20, 12], [2, 3, 7, 6, 10, 19, 14, 18], [1, 2, 6, 5, 9, 18, 13, 17],
                    [3, 4, 8, 7, 11, 20, 15, 19], [1, 4, 3, 2, 12, 11, 10, 9], [5, 6, 7, 8, 13, 14, 15, 16]]),
    TET4: (TRI3, [[1, 4, 3], [1, 2, 4], [1, 3, 2], [2, 3, 4]]),
    TET10: (TRI6, [[1, 4, 3, 8, 10, 7], [1, 2, 4, 5, 9, 8], [1, 3, 2, 7, 6, 5], [2, 3, 4, 6, 10, 9]]),
    QUAD4: (LIN2, [[1, 2], [2, 3], [3, 4], [4, 1]]),
    QUAD8: (LIN3, [[1, 2, 5], [2, 3, 6], [3, 4, 7], [4, 1, 8]]),
    QUAD9: (LIN3, [[1, 2, 5], [2, 3, 6], [3, 4, 7], [4, 1, 8]]),
    TRI3: (LIN2, [[1, 2], [2, 3], [3, 1]]),
    TRI6: (LIN3, [[1, 2, 4], [2, 3, 5], [3, 1, 6]]),
}
FACETS = {k: (fs, [[i - 1 for i in f] for f in fl]) for k, (fs, fl) in FACETS.items()}

D3, PLANESTRAIN, PLANESTRESS, AXISYM = 0, 1, 2, 3
STRESSMODELS = {"d3": D3, "planestrain": PLANESTRAIN, "planestress": PLANESTRESS, "axisymmetric": AXISYM}
LINEAR_ELASTIC, VON_MISES, DRUCKER_PRAGER = 0, 1, 2
ST_LEN = 16

_lock = threading.Lock()
_lib = None


def build(force=False):
    """Compile orc.c into oracle/_build/liborc.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "orc.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src,
                           "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class OrcModel(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("stressmodel", C.c_int32), ("thickness", C.c_double),
                ("nnodes", C.c_int64), ("coords", C.c_void_p), ("nelem", C.c_int64), ("shape", C.c_void_p),
                ("conn_ptr", C.c_void_p), ("conn", C.c_void_p), ("nips", C.c_void_p), ("mat_type", C.c_void_p),
                ("mat_par", C.c_void_p), ("eq_id", C.c_void_p), ("ip_ptr", C.c_void_p), ("state", C.c_void_p),
                ("active", C.c_void_p), ("nactive", C.c_int64)]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build())
            L.orc_quadrature.restype = C.c_int
            L.orc_quadrature.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
            L.orc_shape_func.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
            L.orc_shape_deriv.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
            L.orc_elem_stiffness.restype = C.c_int
            L.orc_elem_stiffness.argtypes = [C.POINTER(OrcModel), C.c_int64, C.c_void_p, C.c_void_p]
            L.orc_mount_K_coo.restype = C.c_int64
            L.orc_mount_K_coo.argtypes = [C.POINTER(OrcModel), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.POINTER(C.c_int64)]
            L.orc_sparse_csc.restype = C.c_int64
            L.orc_sparse_csc.argtypes = [C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p]
            L.orc_update_state.restype = C.c_int
            L.orc_update_state.argtypes = [C.POINTER(OrcModel), C.c_int, C.c_int64, C.c_void_p, C.c_void_p,
                                           C.c_char_p, C.c_int]
            L.orc_material_update.restype = C.c_int
            L.orc_material_update.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_char_p, C.c_int]
            L.orc_material_tangent.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
            _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def quadrature(shape, nips=0):
    """get_ip_coords(shape, nips): src/shape/shape.jl:61 + src/shape/quadrature.jl"""
    R = np.zeros((64, 3)); w = np.zeros(64)
    n = lib().orc_quadrature(shape, nips, _p(R), _p(w))
    if n <= 0:
        raise ValueError("shape %s cannot use %d integration points" % (SHAPE_NAMES[shape], nips))
    return R[:n].copy(), w[:n].copy()


def shape_func(shape, R):
    N = np.zeros(NPOINTS[shape]); RR = np.zeros(3); RR[:len(R)] = R
    lib().orc_shape_func(shape, _p(RR), _p(N))
    return N


def shape_deriv(shape, R):
    nd = SHAPE_NDIM[shape]
    D = np.zeros((NPOINTS[shape], nd)); RR = np.zeros(3); RR[:len(R)] = R
    lib().orc_shape_deriv(shape, _p(RR), _p(D))
    return D


# --------------------------------------------------------------------------
# Expressions: src/tools/expr.jl (comparisons with arith_tol = 1e-6)
# --------------------------------------------------------------------------
ARITH_TOL = 1e-6


def _jl_to_py(s):
    return s.replace("&&", " and ").replace("||", " or ").replace("^", "**")


def evaluate(expr, **vars):
    """evaluate(expr; vars...) for numbers, strings in Julia syntax, or callables."""
    if isinstance(expr, (int, float)):
        return float(expr)
    if callable(expr):
        return expr(**vars)
    tree = ast.parse(_jl_to_py(expr), mode="eval")
    return _ev(tree.body, vars)


def _ev(n, v):
    if isinstance(n, ast.Constant):
        return n.value
    if isinstance(n, ast.Name):
        if n.id == "pi":
            return math.pi
        return v[n.id]
    if isinstance(n, ast.BoolOp):
        if isinstance(n.op, ast.And):
            return all(_ev(x, v) for x in n.values)
        return any(_ev(x, v) for x in n.values)
    if isinstance(n, ast.UnaryOp):
        a = _ev(n.operand, v)
        return -a if isinstance(n.op, ast.USub) else (not a if isinstance(n.op, ast.Not) else a)
    if isinstance(n, ast.BinOp):
        a, b = _ev(n.left, v), _ev(n.right, v)
        op = type(n.op)
        return {ast.Add: lambda: a + b, ast.Sub: lambda: a - b, ast.Mult: lambda: a * b,
                ast.Div: lambda: a / b, ast.Pow: lambda: a ** b}[op]()
    if isinstance(n, ast.Compare):
        a = _ev(n.left, v)
        for op, rhs in zip(n.ops, n.comparators):
            b = _ev(rhs, v)
            t = type(op)
            ok = {ast.Gt: a > b + ARITH_TOL, ast.Lt: a < b - ARITH_TOL, ast.GtE: a > b - ARITH_TOL,
                  ast.LtE: a < b + ARITH_TOL, ast.Eq: abs(a - b) < ARITH_TOL,
                  ast.NotEq: abs(a - b) >= ARITH_TOL}[t]
            if not ok:
                return False
            a = b
        return True
    if isinstance(n, ast.Call):
        f = {"abs": abs, "sin": math.sin, "cos": math.cos, "tan": math.tan, "exp": math.exp,
             "log": math.log, "log10": math.log10, "sqrt": math.sqrt, "max": max, "min": min}[n.func.id]
        return f(*[_ev(a, v) for a in n.args])
    if isinstance(n, ast.IfExp):
        return _ev(n.body, v) if _ev(n.test, v) else _ev(n.orelse, v)
    raise ValueError("expression not supported: %s" % ast.dump(n))


# --------------------------------------------------------------------------
# Structured mesher: src/mesh/block.jl, src/mesh/structured.jl, src/mesh/mesh.jl
# --------------------------------------------------------------------------
class Block:
    """Block(coords; nx, ny, nz, cellshape, tag): src/mesh/block.jl:42-182 (box blocks)."""

    def __init__(self, coords, nx=0, ny=0, nz=0, cellshape=None, tag="", rx=1.0, ry=1.0, rz=1.0):
        coords = np.array(coords, dtype=float)
        if coords.shape[1] == 2:
            coords = np.hstack([coords, np.zeros((coords.shape[0], 1))])
        sumy, sumz = np.abs(coords[:, 1]).sum(), np.abs(coords[:, 2]).sum()
        ndim = 3
        if sumz == 0:
            ndim = 2
        if sumy + sumz == 0:
            ndim = 1
        if coords.shape[0] == 2 and ndim in (2, 3):
            x1, y1, z1 = coords[0]
            lx, ly, lz = coords[1] - coords[0]
            if ndim == 2:
                coords = np.array([[x1, y1, 0], [x1 + lx, y1, 0], [x1 + lx, y1 + ly, 0], [x1, y1 + ly, 0]])
            else:
                coords = np.array([[x1, y1, z1], [x1 + lx, y1, z1], [x1 + lx, y1 + ly, z1], [x1, y1 + ly, z1],
                                   [x1, y1, z1 + lz], [x1 + lx, y1, z1 + lz], [x1 + lx, y1 + ly, z1 + lz],
                                   [x1, y1 + ly, z1 + lz]])
        if nz == 0 and ndim == 3:
            nz = 1
        if ny == 0 and ndim >= 2:
            ny = 1
        self.ndim, self.nx, self.ny, self.nz = ndim, nx, ny, nz
        self.rx, self.ry, self.rz = rx, ry, rz
        self.points = coords
        self.shape = HEX8 if ndim == 3 else QUAD4
        if cellshape is None:
            cellshape = HEX8 if ndim == 3 else QUAD4
        self.cellshape = cellshape
        self.tag = tag


class Cell:
    __slots__ = ("shape", "nodes", "tag", "owner", "id")

    def __init__(self, shape, nodes, tag="", owner=None):
        self.shape, self.nodes, self.tag, self.owner, self.id = shape, list(nodes), tag, owner, -1


class Mesh:
    """Mesh(blocks...): src/mesh/genmesh.jl:69-108 -> split_block! + synchronize!."""

    def __init__(self, *blocks):
        self.coords = []
        self.elems = []
        self._pointdict = {}
        self.ndim = 0
        for b in blocks:
            self.ndim = max(self.ndim, b.ndim)
            self._split_block(b)
        self.coords = np.array(self.coords, dtype=float).reshape(-1, 3)
        for i, c in enumerate(self.elems):
            c.id = i
        self._compute_facets()

    def _new_node(self, C, dedup):
        if dedup:
            C = tuple(round(float(c), 8) for c in C)
            key = (C[0] + 1.0, C[1] + 2.0, C[2] + 3.0)
            if key in self._pointdict:
                return self._pointdict[key]
            idx = len(self.coords)
            self.coords.append(C)
            self._pointdict[key] = idx
            return idx
        idx = len(self.coords)
        self.coords.append(tuple(float(c) for c in C))
        return idx

    def _pt(self, b, n2, r):
        # r = -1 + 2*(i-1)/n for uniform spacing (structured.jl:132,190,475)
        return -1.0 + 2.0 * ((1.0 / n2) * r)

    def _split_block(self, bl):
        sh = bl.cellshape
        nx, ny, nz = bl.nx, bl.ny, bl.nz
        P = bl.points
        if sh in (QUAD4, TRI3):
            parr = {}
            for j in range(ny + 1):
                for i in range(nx + 1):
                    N = shape_func(bl.shape, [self._pt(bl, nx, i), self._pt(bl, ny, j)])
                    C = N @ P
                    parr[i, j] = self._new_node(C, i in (0, nx) or j in (0, ny))
            for j in range(ny):
                for i in range(nx):
                    p1, p2, p3, p4 = parr[i, j], parr[i + 1, j], parr[i + 1, j + 1], parr[i, j + 1]
                    if sh == QUAD4:
                        self.elems.append(Cell(sh, [p1, p2, p3, p4], bl.tag))
                    else:
                        C = (np.array(self.coords[p1]) + self.coords[p2] + np.array(self.coords[p3]) +
                             self.coords[p4]) / 4
                        p5 = self._new_node(C, False)
                        key = tuple(C + np.array([1.0, 2.0, 3.0]))
                        self._pointdict[key] = p5
                        for cn in ([p1, p2, p5], [p2, p3, p5], [p3, p4, p5], [p4, p1, p5]):
                            self.elems.append(Cell(sh, cn, bl.tag))
            return
        if sh in (QUAD8, QUAD9):
            parr = {}
            for j in range(2 * ny + 1):
                for i in range(2 * nx + 1):
                    if sh == QUAD8 and i % 2 == 1 and j % 2 == 1:
                        continue
                    N = shape_func(bl.shape, [self._pt(bl, 2 * nx, i), self._pt(bl, 2 * ny, j)])
                    parr[i, j] = self._new_node(N @ P, i in (0, 2 * nx) or j in (0, 2 * ny))
            for j in range(0, 2 * ny, 2):
                for i in range(0, 2 * nx, 2):
                    cn = [parr[i, j], parr[i + 2, j], parr[i + 2, j + 2], parr[i, j + 2],
                          parr[i + 1, j], parr[i + 2, j + 1], parr[i + 1, j + 2], parr[i, j + 1]]
                    if sh == QUAD9:
                        cn.append(parr[i + 1, j + 1])
                    self.elems.append(Cell(sh, cn, bl.tag))
            return
        if sh == TRI6:
            parr = {}
            for j in range(2 * ny + 1):
                for i in range(2 * nx + 1):
                    r = (1.0 / nx) * i - 1.0
                    s = (1.0 / ny) * j - 1.0
                    N = shape_func(bl.shape, [r, s])
                    parr[i, j] = self._new_node(N @ P, i in (0, 2 * nx) or j in (0, 2 * ny))
            for j in range(0, 2 * ny, 2):
                for i in range(0, 2 * nx, 2):
                    p1, p2, p3, p4 = parr[i, j], parr[i + 2, j], parr[i + 2, j + 2], parr[i, j + 2]
                    p5, p6, p7, p8 = parr[i + 1, j], parr[i + 2, j + 1], parr[i + 1, j + 2], parr[i, j + 1]
                    p9 = parr[i + 1, j + 1]
                    self.elems.append(Cell(sh, [p1, p2, p3, p5, p6, p9], bl.tag))
                    self.elems.append(Cell(sh, [p4, p1, p3, p8, p9, p7], bl.tag))
            return
        if sh in (HEX8, TET4):
            parr = {}
            for k in range(nz + 1):
                for j in range(ny + 1):
                    for i in range(nx + 1):
                        N = shape_func(bl.shape, [self._pt(bl, nx, i), self._pt(bl, ny, j), self._pt(bl, nz, k)])
                        b = i in (0, nx) or j in (0, ny) or k in (0, nz)
                        parr[i, j, k] = self._new_node(N @ P, b)
            for k in range(nz):
                for j in range(ny):
                    for i in range(nx):
                        p = [parr[i, j, k], parr[i + 1, j, k], parr[i + 1, j + 1, k], parr[i, j + 1, k],
                             parr[i, j, k + 1], parr[i + 1, j, k + 1], parr[i + 1, j + 1, k + 1], parr[i, j + 1, k + 1]]
                        if sh == HEX8:
                            self.elems.append(Cell(sh, p, bl.tag))
                        else:
                            p1, p2, p3, p4, p5, p6, p7, p8 = p
                            for cn in ([p2, p4, p1, p8], [p2, p1, p5, p8], [p2, p5, p6, p8], [p2, p6, p7, p8],
                                       [p2, p3, p4, p8], [p2, p7, p3, p8]):
                                self.elems.append(Cell(sh, cn, bl.tag))
            return
        if sh in (HEX20, TET10):
            parr = {}
            for k in range(2 * nz + 1):
                for j in range(2 * ny + 1):
                    for i in range(2 * nx + 1):
                        if sh == HEX20:
                            if i % 2 == 1 and j % 2 == 1:
                                continue
                            if j % 2 == 1 and k % 2 == 1:
                                continue
                            if k % 2 == 1 and i % 2 == 1:
                                continue
                        N = shape_func(bl.shape, [self._pt(bl, 2 * nx, i), self._pt(bl, 2 * ny, j),
                                                  self._pt(bl, 2 * nz, k)])
                        b = i in (0, 2 * nx) or j in (0, 2 * ny) or k in (0, 2 * nz)
                        parr[i, j, k] = self._new_node(N @ P, b)
            for k in range(0, 2 * nz, 2):
                for j in range(0, 2 * ny, 2):
                    for i in range(0, 2 * nx, 2):
                        g = lambda a, b, c: parr[i + a, j + b, k + c]  # noqa: E731
                        p1, p2, p3, p4 = g(0, 0, 0), g(2, 0, 0), g(2, 2, 0), g(0, 2, 0)
                        p5, p6, p7, p8 = g(0, 0, 2), g(2, 0, 2), g(2, 2, 2), g(0, 2, 2)
                        p9, p10, p11, p12 = g(1, 0, 0), g(2, 1, 0), g(1, 2, 0), g(0, 1, 0)
                        p13, p14, p15, p16 = g(1, 0, 2), g(2, 1, 2), g(1, 2, 2), g(0, 1, 2)
                        p17, p18, p19, p20 = g(0, 0, 1), g(2, 0, 1), g(2, 2, 1), g(0, 2, 1)
                        if sh == HEX20:
                            self.elems.append(Cell(sh, [p1, p2, p3, p4, p5, p6, p7, p8, p9, p10, p11, p12, p13, p14,
                                                        p15, p16, p17, p18, p19, p20], bl.tag))
                        else:
                            p21, p22, p23, p24 = g(0, 1, 1), g(2, 1, 1), g(1, 0, 1), g(1, 2, 1)
                            p25, p26, p27 = g(1, 1, 0), g(1, 1, 2), g(1, 1, 1)
                            for cn in ([p2, p4, p1, p8, p25, p12, p9, p27, p20, p21],
                                       [p2, p1, p5, p8, p9, p17, p23, p27, p21, p16],
                                       [p2, p5, p6, p8, p23, p13, p18, p27, p16, p26],
                                       [p2, p6, p7, p8, p18, p14, p22, p27, p26, p15],
                                       [p2, p3, p4, p8, p10, p11, p25, p27, p24, p20],
                                       [p2, p7, p3, p8, p22, p19, p10, p27, p15, p24]):
                                self.elems.append(Cell(sh, cn, bl.tag))
            return
        raise ValueError("block: cannot discretize using shape %s" % SHAPE_NAMES[sh])

    def _compute_facets(self):
        """compute_facets!: src/mesh/mesh.jl:318-331 with get_outer_facets (:69-85)."""
        d = {}
        for c in self.elems:
            fsh, fl = FACETS[c.shape]
            for f in fl:
                nodes = [c.nodes[i] for i in f]
                key = frozenset(nodes)
                if key in d:
                    del d[key]
                else:
                    d[key] = Cell(fsh, nodes, owner=c)
        self.faces = list(d.values())
        if self.ndim == 2:
            self.edges = self.faces
        else:
            ed = {}
            for f in self.faces:
                esh, el = FACETS[f.shape]
                for e in el:
                    nodes = [f.nodes[i] for i in e]
                    ed[frozenset(nodes)] = Cell(esh, nodes, owner=f.owner)
            self.edges = list(ed.values())

    def select_nodes(self, expr):
        """nodes[expr]: src/node.jl:191-215"""
        return [i for i in range(len(self.coords))
                if evaluate(expr, x=self.coords[i, 0], y=self.coords[i, 1], z=self.coords[i, 2])]

    def select_cells(self, cells, expr):
        """cells[expr]: all nodes of the cell satisfy expr (src/mesh/cell.jl:251-271)."""
        if isinstance(expr, str) and expr in ("all", ":all"):
            return list(cells)
        T = {}
        out = []
        for c in cells:
            ok = True
            for n in c.nodes:
                if n not in T:
                    x, y, z = self.coords[n]
                    T[n] = bool(evaluate(expr, x=x, y=y, z=z))
                if not T[n]:
                    ok = False
                    break
            if ok:
                out.append(c)
        return out


# --------------------------------------------------------------------------
# Model and materials
# --------------------------------------------------------------------------
class Material:
    def __init__(self, kind, **p):
        self.kind = kind
        self.p = p

    def params(self):
        p = self.p
        if self.kind == LINEAR_ELASTIC:
            return [p["E"], p.get("nu", 0.0), 0, 0, 0, 0, 0, 0]
        if self.kind == VON_MISES:
            return [p["E"], p.get("nu", 0.0), p["fy"], p.get("H", 0.0), 0, 0, 0, 0]
        return [p["E"], p.get("nu", 0.0), p.get("alpha", 0.0), p["kappa"], p.get("H", 0.0), 0, 0, 0]


def LinearElastic(**p):
    return Material(LINEAR_ELASTIC, **p)


def VonMises(**p):
    return Material(VON_MISES, **p)


def DruckerPrager(**p):
    return Material(DRUCKER_PRAGER, **p)


class FEModel:
    """FEModel(mesh, matbinds, ctx): src/fe-model.jl:66-255 for MechSolid elements.

    matbinds: list of (filter, Material) pairs; filter is a tag string, an expression, or "all".
    """

    def __init__(self, mesh, matbinds, stressmodel="d3", thickness=1.0, nips=0, elem_E=None):
        self.mesh = mesh
        self.ndim = mesh.ndim
        if stressmodel in (None, "none"):
            stressmodel = "planestrain" if self.ndim == 2 else "d3"
        self.stressmodel = STRESSMODELS[stressmodel]
        self.thickness = thickness
        ne = len(mesh.elems)
        self.mat_type = np.full(ne, -1, dtype=np.int32)
        self.mat_par = np.zeros((ne, 8))
        self.rho = np.zeros(ne)  # element density (MechSolid props rho, src/mech/elem/mech-solid.jl:6-29)
        for filt, mat in matbinds:
            if isinstance(filt, str) and not any(ch in filt for ch in "=<>"):
                sel = [c for c in mesh.elems if filt in ("all", c.tag)]
            else:
                sel = mesh.select_cells(mesh.elems, filt)
            for c in sel:
                self.mat_type[c.id] = mat.kind
                self.mat_par[c.id] = mat.params()
                self.rho[c.id] = mat.p.get("rho", 0.0)
        if (self.mat_type < 0).any():
            raise ValueError("elements without material")
        if elem_E is not None:
            self.mat_par[:, 0] = elem_E
        self.shape = np.array([c.shape for c in mesh.elems], dtype=np.int32)
        self.conn_ptr = np.zeros(ne + 1, dtype=np.int64)
        self.conn_ptr[1:] = np.cumsum([len(c.nodes) for c in mesh.elems])
        self.conn = np.array([n for c in mesh.elems for n in c.nodes], dtype=np.int64)
        self.nips = np.full(ne, nips, dtype=np.int32)
        self.active = np.ones(ne, dtype=bool)  # elem.active (src/element.jl:40, fe-model.jl:156)
        self.coords = np.ascontiguousarray(mesh.coords)
        self.nnodes = len(self.coords)
        self._setup_ips()
        # node dofs (elem_config_dofs, src/mech/elem/mech.jl:12-18): names per node
        self.dof_names = ["ux", "uy", "uz"][: self.ndim]
        self.eq_id = np.full((self.nnodes, 3), -1, dtype=np.int64)
        # dof values (dof.vals): displacements and natural values per node-dof
        self.U = np.zeros((self.nnodes, self.ndim))
        self.F = np.zeros((self.nnodes, self.ndim))

    def _setup_ips(self):
        ne = len(self.shape)
        cnt = np.array([quadrature(int(s), int(n))[0].shape[0] for s, n in zip(self.shape, self.nips)])
        self.ip_ptr = np.zeros(ne + 1, dtype=np.int64)
        self.ip_ptr[1:] = np.cumsum(cnt)
        self.state = np.zeros((int(self.ip_ptr[-1]), ST_LEN))

    def changequadrature(self, n):
        """changequadrature!(elems, n): src/element.jl:185-188"""
        self.nips[:] = n
        self._setup_ips()

    def active_elems(self):
        """filter(elem -> elem.active, model.elems) (src/mech/mech-solver.jl:220): element ids."""
        return np.nonzero(self.active)[0].astype(np.int64)

    def active_nodes(self):
        """The nodes of the active elements, by id (configure_dofs!, src/bc.jl:200-203)."""
        act = self.active_elems()
        if len(act) == len(self.shape):
            return np.unique(self.conn)
        return np.unique(np.concatenate([self.conn[self.conn_ptr[e]:self.conn_ptr[e + 1]] for e in act]))

    def cstruct(self):
        m = OrcModel()
        act = None if self.active.all() else self.active_elems()
        self._keep = [self.coords, self.shape, self.conn_ptr, self.conn, self.nips, self.mat_type, self.mat_par,
                      self.eq_id, self.ip_ptr, self.state, act]
        m.ndim, m.stressmodel, m.thickness = self.ndim, self.stressmodel, self.thickness
        m.nnodes, m.coords = self.nnodes, _p(self.coords)
        m.nelem, m.shape = len(self.shape), _p(self.shape)
        m.conn_ptr, m.conn, m.nips = _p(self.conn_ptr), _p(self.conn), _p(self.nips)
        m.mat_type, m.mat_par = _p(self.mat_type), _p(self.mat_par)
        m.eq_id, m.ip_ptr, m.state = _p(self.eq_id), _p(self.ip_ptr), _p(self.state)
        m.active, m.nactive = (None, 0) if act is None else (_p(act), len(act))
        return m

    def elem_stiffness(self, e):
        nd = (self.conn_ptr[e + 1] - self.conn_ptr[e]) * self.ndim
        K = np.zeros((nd, nd)); mp = np.zeros(nd, dtype=np.int64)
        m = self.cstruct()
        rc = lib().orc_elem_stiffness(C.byref(m), e, _p(K), _p(mp))
        if rc < 0:
            raise RuntimeError("elem_stiffness failed (%d)" % rc)
        return K, mp


def mount_K(model, ndofs, nthreads=1, return_coo=False):
    """mount_K(elems, ndofs): src/mech/mech-solver.jl:78-110 -> scipy CSC (0-based)."""
    import scipy.sparse as sp
    nd = np.diff(model.conn_ptr) * model.ndim
    cap = int((nd * nd).sum())
    R = np.empty(cap, dtype=np.int64); Cc = np.empty(cap, dtype=np.int64); V = np.empty(cap)
    bad = C.c_int64(-1)
    m = model.cstruct()
    cnt = lib().orc_mount_K_coo(C.byref(m), nthreads, _p(R), _p(Cc), _p(V), C.byref(bad))
    if cnt < 0:
        raise RuntimeError("Negative Jacobian determinant in cell %d" % (bad.value + 1))
    colptr = np.zeros(ndofs + 1, dtype=np.int64)
    rowval = np.empty(max(cnt, 1), dtype=np.int64); nzval = np.empty(max(cnt, 1))
    nnz = lib().orc_sparse_csc(ndofs, cnt, _p(R), _p(Cc), _p(V), _p(colptr), _p(rowval), _p(nzval))
    K = sp.csc_matrix((nzval[:nnz], rowval[:nnz], colptr), shape=(ndofs, ndofs))
    if return_coo:
        return K, (R[:cnt], Cc[:cnt], V[:cnt])
    return K


def update_state(model, dU, nthreads=1):
    """update_state!(active_elems, ΔUt, t): src/mech/mech-solver.jl:124-144 -> (ΔFin, status msg or None)."""
    ndofs = len(dU)
    dU = np.ascontiguousarray(dU, dtype=float)
    dF = np.zeros(ndofs)
    msg = C.create_string_buffer(256)
    m = model.cstruct()
    rc = lib().orc_update_state(C.byref(m), nthreads, ndofs, _p(dU), _p(dF), msg, 256)
    if rc:
        return dF, msg.value.decode("utf-8", "replace") or "update_state failed"
    if np.isnan(dF).any():
        return dF, "solve_system!: NaN values in internal forces vector"
    return dF, None


def solve_system(K, U, F, nu):
    """solve_system!(K, U, F, nu): src/solver.jl:5-79 with SuperLU in place of UMFPACK.

    Fills U[:nu] and F[nu:]; returns None or a failure message."""
    import scipy.sparse.linalg as sla
    K = K.tocsc()
    K11 = K[:nu, :nu]; K12 = K[:nu, nu:]; K21 = K[nu:, :nu]; K22 = K[nu:, nu:]
    F1 = F[:nu]; U2 = U[nu:]
    F2 = K22 @ U2
    U1 = np.zeros(nu)
    if nu > 0:
        RHS = F1 - K12 @ U2
        try:
            lu = sla.splu(K11.tocsc(), permc_spec="COLAMD")
            U1 = lu.solve(RHS)
            F2 = F2 + K21 @ U1
        except Exception as err:  # singular etc.
            msg = ""
            if np.isnan(K11.data).any():
                msg = "\nsolve_system!: NaN values in coefficients matrix"
            return "%s\nsolve_system!: %s" % (msg, err)
    if nu > 0 and np.abs(U1).max() > 1e8:
        return "\nsolve_system!: Possible syngular matrix"
    U[:nu] = U1
    F[nu:] = F2
    return None


# --------------------------------------------------------------------------
# Boundary conditions: src/bc.jl
# --------------------------------------------------------------------------
class NodeBC:
    def __init__(self, **conds):
        self.conds = conds


class SurfaceBC:
    def __init__(self, **conds):
        self.conds = conds


class EdgeBC:
    def __init__(self, **conds):
        self.conds = conds


class BodyC:
    def __init__(self, **conds):
        self.conds = conds


FaceBC = SurfaceBC
NAT = {"fx": "ux", "fy": "uy", "fz": "uz"}


def _setup_bcs(model, bcs):
    """setup_bc! for each bc (src/bc.jl:22-40,86-113,155-172): filtered objects + prescribed flags."""
    mesh = model.mesh
    presc = np.zeros((model.nnodes, 3), dtype=bool)
    out = []
    for filt, bc in bcs:
        if isinstance(bc, NodeBC):
            if isinstance(filt, (int, np.integer)):
                objs = [int(filt)]
            elif isinstance(filt, (list, tuple)):
                objs = list(filt)
            else:
                objs = mesh.select_nodes(filt)
            nodes = objs
        elif isinstance(bc, (SurfaceBC, EdgeBC)):
            if isinstance(bc, SurfaceBC):
                src = mesh.edges if model.ndim == 2 else mesh.faces
            else:
                src = mesh.edges
            objs = _select_tagged(mesh, src, filt)
            nodes = sorted({n for f in objs for n in f.nodes})
        else:  # over the active elements only (bc.jl:159)
            objs = [c for c in _select_tagged(mesh, mesh.elems, filt) if model.active[c.id]]
            nodes = sorted({n for c in objs for n in c.nodes})
        for key in bc.conds:
            if key in model.dof_names:
                k = model.dof_names.index(key)
                for n in nodes:
                    presc[n, k] = True
        out.append((bc, objs))
    return presc, out


def _select_tagged(mesh, cells, filt):
    if isinstance(filt, str) and not any(ch in filt for ch in "=<>") and filt != "all":
        return [c for c in cells if c.tag == filt]
    return mesh.select_cells(cells, filt)


def configure_dofs(model, bcs):
    """configure_dofs!(model, bcs): src/bc.jl:198-233.  Returns (dof list, nu, bc setup)."""
    active = model.active_nodes().tolist()
    presc, setup = _setup_bcs(model, bcs)
    dofs = [(n, k) for n in active for k in range(model.ndim)]
    udofs = [d for d in dofs if not presc[d]]
    pdofs = [d for d in dofs if presc[d]]
    dofs = udofs + pdofs
    model.eq_id[:] = -1
    for i, (n, k) in enumerate(dofs):
        model.eq_id[n, k] = i
    return dofs, len(udofs), setup


def _facet_forces(model, facet, key, val, t=0.0):
    """mech_boundary_forces: src/mech/elem/distributed.jl:76-152"""
    ndim = model.ndim
    isedge = key in ("qx", "qy", "qz", "qn")
    if isedge and model.stressmodel == AXISYM:  # distributed.jl:89
        raise ValueError("mech_boundary_forces: boundary condition %s is not applicable in a axisymmetric analysis" % key)
    th = 1.0 if isedge else model.thickness
    Cc = model.coords[facet.nodes, :ndim]
    R, W = quadrature(facet.shape, 0)
    F = np.zeros((len(facet.nodes), ndim))
    for ip in range(len(W)):
        N = shape_func(facet.shape, R[ip])
        D = shape_deriv(facet.shape, R[ip])
        J = Cc.T @ D
        X = Cc.T @ N
        if ndim == 2:
            vip = evaluate(val, t=t, x=X[0], y=X[1], z=0.0)
            if model.stressmodel == AXISYM:
                th = 2 * math.pi * X[0]
        else:
            vip = evaluate(val, t=t, x=X[0], y=X[1], z=X[2])
        Q = np.zeros(ndim)
        if key in ("tx", "qx"):
            Q[0] = vip
        elif key in ("ty", "qy"):
            Q[1] = vip
        elif key in ("tz", "qz"):
            Q[2] = vip
        elif key in ("tn", "qn"):
            n = np.array([J[1, 0], -J[0, 0]]) if ndim == 2 else np.cross(J[:, 0], J[:, 1])
            Q = vip * n / np.linalg.norm(n)
        else:
            raise ValueError("boundary condition %s not applicable as distributed bc" % key)
        coef = _norm2(J) * W[ip] * th
        F += coef * np.outer(N, Q)
    return F.reshape(-1)


def _norm2(J):
    """norm2: src/tools/linalg.jl:50-72"""
    r, c = J.shape
    if r == c:
        return np.linalg.det(J)
    if r == 1 or c == 1:
        return np.linalg.norm(J)
    if r == 3 and c == 2:
        j1 = J[0, 0] * J[1, 1] - J[0, 1] * J[1, 0]
        j2 = J[0, 0] * J[2, 1] - J[0, 1] * J[2, 0]
        j3 = J[1, 0] * J[2, 1] - J[1, 1] * J[2, 0]
        return (j1 * j1 + j2 * j2 + j3 * j3) ** 0.5
    raise ValueError("norm2 of %dx%d" % (r, c))


def _body_forces(model, cell, key, val):
    """mech_solid_body_forces: src/mech/elem/distributed.jl:157-217 (default quadrature)."""
    ndim = model.ndim
    th = model.thickness
    Cc = model.coords[cell.nodes, :ndim]
    R, W = quadrature(cell.shape, 0)
    F = np.zeros((len(cell.nodes), ndim))
    for ip in range(len(W)):
        N = shape_func(cell.shape, R[ip])
        D = shape_deriv(cell.shape, R[ip])
        J = Cc.T @ D
        X = Cc.T @ N
        if ndim == 2:
            vip = evaluate(val, x=X[0], y=X[1], z=0.0)
            if model.stressmodel == AXISYM:
                th = 2 * math.pi * X[0]
        else:
            vip = evaluate(val, x=X[0], y=X[1], z=X[2])
        Q = np.zeros(ndim)
        idx = {"wx": 0, "wy": 1, "wz": 2}[key]
        Q[idx] = vip
        F += np.linalg.det(J) * W[ip] * th * np.outer(N, Q)
    return F.reshape(-1)


def _no_dof(model, nodes):
    """A node of no active element keeps eq_id 0 (Dof(), src/dof.jl:15-17), so the reference's U[dof.eq_id] and
    F[map] raise a BoundsError there: the oracle raises too."""
    bad = [n for n in np.atleast_1d(nodes) if model.eq_id[n, 0] < 0]
    if bad:
        raise ValueError("boundary condition on node %d, which belongs to no active element" % (bad[0] + 1))


def get_bc_vals(model, setup, ndofs, t=0.0):
    """get_bc_vals(model, bcs): src/bc.jl:237-249 (compute_bc_vals! :43-58,116-136,175-194)."""
    for bc, objs in setup:
        if isinstance(bc, NodeBC):
            _no_dof(model, objs)
        else:
            for f in objs:
                _no_dof(model, f.nodes)
    U = np.zeros(ndofs)
    F = np.zeros(ndofs)
    names = model.dof_names
    for bc, objs in setup:
        if isinstance(bc, NodeBC):
            for n in objs:
                x, y, z = model.coords[n]
                for key, cond in bc.conds.items():
                    if key in names:
                        U[model.eq_id[n, names.index(key)]] = evaluate(cond, x=x, y=y, z=z, t=t)
                    elif key in NAT and NAT[key] in names:
                        F[model.eq_id[n, names.index(NAT[key])]] += evaluate(cond, x=x, y=y, z=z, t=t)
        elif isinstance(bc, (SurfaceBC, EdgeBC)):
            for f in objs:
                for key, val in bc.conds.items():
                    if key in names:
                        for n in f.nodes:
                            x, y, z = model.coords[n]
                            U[model.eq_id[n, names.index(key)]] = evaluate(val, x=x, y=y, z=z, t=t)
                    else:
                        Fd = _facet_forces(model, f, key, val, t)
                        mp = model.eq_id[f.nodes, :model.ndim].reshape(-1)
                        F[mp] += Fd
        else:
            for c in objs:
                for key, val in bc.conds.items():
                    if key in names:
                        for n in c.nodes:
                            x, y, z = model.coords[n]
                            U[model.eq_id[n, names.index(key)]] = evaluate(val, x=x, y=y, z=z, t=t)
                    else:
                        Fd = _body_forces(model, c, key, val)
                        mp = model.eq_id[c.nodes, :model.ndim].reshape(-1)
                        F[mp] += Fd
    return U, F


# --------------------------------------------------------------------------
# Staged Newton driver: src/mech/mech-solver.jl:155-492, src/solver.jl:82-198
# --------------------------------------------------------------------------
class Stage:
    def __init__(self, bcs, nincs=1, nouts=0, toactivate=()):
        self.bcs, self.nincs, self.nouts, self.status = bcs, nincs, nouts, "pending"
        self.toactivate = list(toactivate)  # element ids (src/stage.jl:8,16)


class MechAnalysis:
    def __init__(self, model):
        self.model = model
        self.stages = []
        self.log = []

    def addstage(self, bcs, nincs=1, nouts=0, toactivate=()):
        """addstage!: src/analysis.jl:27-32"""
        self.stages.append(Stage(list(bcs), nincs, nouts, toactivate))

    def solve(self, tol=0.01, rtol=0.01, rspan=0.01, dT0=0.01, dTmin=1e-7, dTmax=0.1, scheme="FE", maxits=5,
              autoinc=False, quiet=True, nthreads=1, record=None):
        """solve!(ana; args...): stage_iterator! over pending stages; returns (success, message)."""
        for st in self.stages:
            if st.status == "done":
                continue
            nincs = st.nincs
            if st.nouts > 0 and not autoinc:  # solver.jl:128-140
                if st.nouts > nincs:
                    nincs = st.nouts
                if nincs % st.nouts != 0:
                    nincs = nincs - (nincs % st.nouts) + st.nouts
            st.nincs = nincs
            ok, msg = self._stage(st, tol, rtol, rspan, dT0, dTmin, dTmax, scheme, maxits, autoinc, nthreads,
                                  record)
            st.status = "done" if ok else "error"
            if not ok:
                return False, msg
        return True, ""

    def _stage(self, stage, tol, rtol, rspan, dT0, dTmin, dTmax, scheme, maxits, autoinc, nthreads, record):
        model = self.model
        model.active[np.asarray(stage.toactivate, dtype=np.int64)] = True  # mech-solver.jl:216-219
        dofs, nu, setup = configure_dofs(model, stage.bcs)
        ndofs = len(dofs)
        dof_n = np.array([d[0] for d in dofs], dtype=np.int64)
        dof_k = np.array([d[1] for d in dofs], dtype=np.int64)
        pmap = slice(nu, ndofs)
        StateBk = model.state.copy()
        ftol = tol
        saveouts = stage.nouts > 0
        dTcheck = 1.0 / stage.nouts if saveouts else 1.0
        Tcheck = dTcheck
        T = 0.0
        dT = 1.0 / stage.nincs
        if autoinc:
            dT = min(dT, dTmax, dTcheck, dT0)
        dTbk = 0.0
        inc = 0
        F = np.zeros(ndofs); U = np.zeros(ndofs); R = np.zeros(ndofs)
        dUa = np.zeros(ndofs); dUi = np.zeros(ndofs); Rc = np.zeros(ndofs)
        dFin = np.zeros(ndofs)
        still_linear = True
        Uex, Fex = get_bc_vals(model, setup, ndofs)
        if scheme == "FE":
            p1, q11 = 1.0, 1.0
        elif scheme == "ME":
            p1, q11, a1, a2 = 1.0, 1.0, 0.5, 0.5
        elif scheme == "BE":
            p1, q11, a1, a2 = 1.0, 1.0, 0.0, 1.0
        else:  # Ralston
            p1, q11, a1, a2 = 2 / 3, 2 / 3, 1 / 4, 3 / 4
        solstatus = (True, "")
        eps = np.finfo(float).eps
        while T < 1.0 - dTmin:
            inc += 1
            dUex, dFex = dT * Uex, dT * Fex
            dTcr = min(rspan, 1 - T)
            acr = min(dT / dTcr, 1.0)
            if T < 1 - rspan:
                dFex = dFex + acr * Rc
            R[:] = dFex
            dUa[:] = 0.0
            dUi = dUex.copy()
            nits = 0; err = 0.0; res = 0.0; res1 = 0.0
            converged = False; syserror = False; sysmsg = None
            for it in range(1, maxits + 1):
                nits += 1
                if it > 1:
                    dUi[:] = 0.0
                lastres = res
                K = mount_K(model, ndofs, nthreads)
                dUitr = p1 * dUi
                Rtr = q11 * R
                sysmsg = solve_system(K, dUitr, Rtr, nu)
                if sysmsg:
                    syserror = True
                    break
                model.state[:] = StateBk
                dUt = dUa + dUitr
                dFin, sysmsg = update_state(model, dUt, nthreads)
                if sysmsg:
                    syserror = True
                    break
                if scheme == "FE":
                    dUi = dUitr
                else:
                    K2 = mount_K(model, ndofs, nthreads)
                    K = a1 * K + a2 * K2
                    sysmsg = solve_system(K, dUi, R, nu)
                    if sysmsg:
                        syserror = True
                        break
                    model.state[:] = StateBk
                    dUt = dUa + dUi
                    dFin, sysmsg = update_state(model, dUt, nthreads)
                    if sysmsg:
                        syserror = True
                        break
                dUa += dUi
                R[:] = dFex - dFin
                R[pmap] = 0.0
                res = np.abs(R).max() if ndofs else 0.0
                with np.errstate(divide="ignore", invalid="ignore"):
                    err = float(np.float64(np.abs(dUi).max()) / np.float64(np.abs(dUa).max())) if ndofs else np.nan
                self.log.append((stage, inc, it, res))
                if it == 1:
                    res1 = res
                if it > 1:
                    still_linear = False
                if res < ftol:
                    converged = True
                    break
                if err < rtol:
                    converged = True
                    break
                if np.isnan(res):
                    break
                if it > 1 and res > lastres:
                    break
            if syserror:
                converged = False
            if converged:
                U += dUa
                F += dFin
                Rc = (1.0 - acr) * Rc + R
                StateBk = model.state.copy()
                model.U[dof_n, dof_k] += dUa
                model.F[dof_n, dof_k] += dFin
                T += dT
                checkpoint = T > Tcheck - dTmin
                if checkpoint:
                    Tcheck += dTcheck
                if record is not None:
                    record(self, T, checkpoint)
                if autoinc:
                    if dTbk > 0.0:
                        dT = min(dTbk, Tcheck - T)
                        dTbk = 0.0
                    else:
                        q = 1 + math.tanh(math.log10(ftol / (res1 + eps)))
                        q = max(q, 1.1)
                        dTtr = min(q * dT, dTmax, 1 - T)
                        if T + dTtr > Tcheck - dTmin:
                            dTbk = dT
                            dT = Tcheck - T
                        else:
                            dT = dTtr
                            dTbk = 0.0
            else:
                inc -= 1
                model.state[:] = StateBk
                if autoinc:
                    q = 1 + math.tanh(math.log10(ftol / (res1 + eps)))
                    q = min(max(q, 0.2), 0.9)
                    if syserror:
                        q = 0.7
                    dT = q * dT
                    dT = float("%.3g" % dT)
                    if dT < dTmin:
                        solstatus = (False, "Solver did not converge.")
                        break
                else:
                    solstatus = (False, "Solver did not converge. Try `autoinc=true`. ")
                    break
        self.ndofs, self.nu, self.dofs = ndofs, nu, dofs
        return solstatus
