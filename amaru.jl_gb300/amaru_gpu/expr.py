"""Vectorised evaluation of Amaru filter / value expressions.

Expressions use Amaru's syntax (src/tools/expr.jl): `x==0 && y>=1`, `3*z`,
with comparisons taken with the absolute tolerance arith_tol = 1e-6
(src/tools/expr.jl:98-115).  Python callables f(x=, y=, z=, t=) are accepted
too.  Evaluation is over numpy arrays of coordinates.
"""
import ast
import math

import numpy as np

ARITH_TOL = 1e-6
_FUNCS = {"abs": np.abs, "sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log,
          "log10": np.log10, "sqrt": np.sqrt, "max": np.maximum, "min": np.minimum}


def _to_py(s):
    return s.replace("&&", " and ").replace("||", " or ").replace("^", "**")


def evaluate(expr, x=0.0, y=0.0, z=0.0, t=0.0):
    """Value of expr at the given (broadcastable) coordinates."""
    env = {"x": np.asarray(x, dtype=float), "y": np.asarray(y, dtype=float), "z": np.asarray(z, dtype=float),
           "t": np.asarray(t, dtype=float)}
    if isinstance(expr, (bool, np.bool_)):
        return np.broadcast_to(np.asarray(expr), np.broadcast(env["x"], env["y"], env["z"]).shape)
    if isinstance(expr, (int, float, np.integer, np.floating)):
        return np.broadcast_to(np.float64(expr), np.broadcast(env["x"], env["y"], env["z"]).shape)
    if callable(expr):
        return np.asarray(expr(x=env["x"], y=env["y"], z=env["z"], t=env["t"]))
    tree = ast.parse(_to_py(str(expr)), mode="eval")
    return _ev(tree.body, env)


def _ev(n, env):
    if isinstance(n, ast.Constant):
        return n.value
    if isinstance(n, ast.Name):
        if n.id == "pi":
            return math.pi
        if n.id in env:
            return env[n.id]
        raise ValueError("variable %s not defined for this context" % n.id)
    if isinstance(n, ast.BoolOp):
        vals = [np.asarray(_ev(v, env), dtype=bool) for v in n.values]
        out = vals[0]
        for v in vals[1:]:
            out = (out & v) if isinstance(n.op, ast.And) else (out | v)
        return out
    if isinstance(n, ast.UnaryOp):
        a = _ev(n.operand, env)
        if isinstance(n.op, ast.USub):
            return -a
        if isinstance(n.op, ast.Not):
            return ~np.asarray(a, dtype=bool)
        return a
    if isinstance(n, ast.BinOp):
        a, b = _ev(n.left, env), _ev(n.right, env)
        if isinstance(n.op, ast.Add):
            return a + b
        if isinstance(n.op, ast.Sub):
            return a - b
        if isinstance(n.op, ast.Mult):
            return a * b
        if isinstance(n.op, ast.Div):
            return a / b
        if isinstance(n.op, ast.Pow):
            return a ** b
        raise ValueError("operator not allowed")
    if isinstance(n, ast.Compare):
        a = _ev(n.left, env)
        out = None
        for op, rhs in zip(n.ops, n.comparators):
            b = _ev(rhs, env)
            if isinstance(op, ast.Gt):
                r = a > b + ARITH_TOL
            elif isinstance(op, ast.Lt):
                r = a < b - ARITH_TOL
            elif isinstance(op, ast.GtE):
                r = a > b - ARITH_TOL
            elif isinstance(op, ast.LtE):
                r = a < b + ARITH_TOL
            elif isinstance(op, ast.Eq):
                r = np.abs(a - b) < ARITH_TOL
            elif isinstance(op, ast.NotEq):
                r = np.abs(a - b) >= ARITH_TOL
            else:
                raise ValueError("comparison not allowed")
            out = r if out is None else (out & r)
            a = b
        return out
    if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _FUNCS:
        return _FUNCS[n.func.id](*[_ev(a, env) for a in n.args])
    if isinstance(n, ast.IfExp):
        return np.where(_ev(n.test, env), _ev(n.body, env), _ev(n.orelse, env))
    raise ValueError("expression not supported: %s" % ast.dump(n))


def affine_coefficients(expr, ndim):
    """(c0, cx, cy, cz, ct) with expr == c0 + cx x + cy y + cz z + ct t, or raise.

    The device load kernels integrate affine values; anything else is rejected
    rather than evaluated on the host."""
    def f(x, y, z, t):
        return float(np.asarray(evaluate(expr, x=x, y=y, z=z, t=t)))
    c0 = f(0.0, 0.0, 0.0, 0.0)
    c = [c0, f(1.0, 0, 0, 0) - c0, f(0, 1.0, 0, 0) - c0, f(0, 0, 1.0, 0) - c0, f(0, 0, 0, 1.0) - c0]
    rng = np.random.default_rng(12345)
    for _ in range(4):
        x, y, z, t = rng.uniform(-3, 3, 4)
        want = f(x, y, z, t)
        got = c[0] + c[1] * x + c[2] * y + c[3] * z + c[4] * t
        if abs(want - got) > 1e-9 * (1.0 + abs(want)):
            raise NotImplementedError("load value %r is not affine in (x, y, z, t); the GPU load kernels "
                                      "integrate affine values only" % (expr,))
    return c
