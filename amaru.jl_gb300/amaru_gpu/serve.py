"""Serving: staged analyses submitted as they arrive, run with continuous batching.

Server wraps the library's request loop (amr_server_*): a request is one stage of
mech_stage_solver! (src/mech/mech-solver.jl:186-492) on its own model.  Up to
max_active requests are on the device at once, each on its own CUDA stream; a
request is admitted in arrival order once a slot is free and its device
footprint (amr_estimate_bytes) fits the HBM budget beside the running ones.  A
request keeps its pattern, K, IP states and solution on the device across all
increments of its stage, and its result is the one it gets when run alone.
"""
import ctypes as C

import numpy as np

from . import _lib as L
from .args import MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, checkargs
from .model import number_dofs

_SCHEMES = {"FE": 0, "ME": 1, "BE": 2, "Ralston": 3}


def stage_params(nincs=1, nouts=0, tol=0.01, rtol=0.01, rspan=0.01, dT0=0.01, dTmin=1e-7, dTmax=0.1, scheme="FE",
                 maxits=5, autoinc=False, linear_rtol=1e-8, solver="mixed", refine_every=32, max_iters=20000):
    """amr_stage_params with the keyword defaults of solve!(ana; ...) (src/mech/mech-solver.jl:155-168),
    checked against the conditions of that table."""
    checkargs("solve!", MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, tol=tol, rspan=rspan, rtol=rtol, dT0=dT0,
              dTmin=dTmin, dTmax=dTmax, maxits=maxits, scheme=scheme)
    method = {"mixed": L.SOLVER_MIXED, "fp64": L.SOLVER_FP64, "amg": L.SOLVER_AMG, "amg_fp64": L.SOLVER_AMG_FP64}[solver]
    lin = L.default_solve_opts(method=method, rtol=linear_rtol, refine_every=refine_every, max_iters=max_iters)
    return L.default_stage_params(tol=tol, rtol=rtol, rspan=rspan, dT0=dT0, dTmin=dTmin, dTmax=dTmax,
                                  scheme=_SCHEMES[scheme], maxits=maxits, autoinc=int(autoinc), nincs=nincs,
                                  nouts=nouts, linear=lin)


def estimate_bytes(model):
    """Upper bound of the device bytes the model and one stage of it take (amr_estimate_bytes)."""
    d, keep = L.model_desc(model.ndim, model.stressmodel, model.thickness, model.mesh.coords, model.mesh.shape,
                           model.nips, model.mesh.conn_ptr, model.mesh.conn, model.mat_type, model.mat_params)
    b = C.c_int64()
    L.check(None, L.lib().amr_estimate_bytes(C.byref(d), C.byref(b)))
    return b.value


class Ticket:
    """A submitted request: its id and what is needed to map its results to nodes."""

    def __init__(self, rid, nnodes, ndim, ndofs, nu, dof_node, dof_comp):
        self.id, self.nnodes, self.ndim, self.ndofs, self.nu = rid, nnodes, ndim, ndofs, nu
        self.dof_node, self.dof_comp = dof_node, dof_comp


class Server:
    def __init__(self, hbm_budget_bytes, max_active=4):
        cfg = L.ServerConfig()
        cfg.hbm_budget_bytes = float(hbm_budget_bytes)
        cfg.max_active = int(max_active)
        h = C.c_void_p()
        L.check(None, L.lib().amr_server_create(C.byref(cfg), C.byref(h)))
        self.h = h

    def submit(self, model, bcs, **kw):
        """Queues one stage of `model` (an FEModel; device=False suffices) with boundary conditions
        `bcs` as for addstage; keywords as stage_params.  Returns a Ticket."""
        presc, setup = model._prescribed(bcs)
        (model.eq_id, model.ndofs, model.nu, model.dof_node,
         model.dof_comp) = number_dofs(model.active_nodes, presc, model.nnodes)
        U, F, loads = model.bc_vals(setup)
        d, keep = L.model_desc(model.ndim, model.stressmodel, model.thickness, model.mesh.coords, model.mesh.shape,
                               model.nips, model.mesh.conn_ptr, model.mesh.conn, model.mat_type, model.mat_params)
        arr, keep_loads = L.load_array(loads)
        eq = np.ascontiguousarray(model.eq_id, dtype=np.int64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.float64)
        req = L.Request()
        req.model = d
        req.eq_id, req.ndofs, req.nu = eq.ctypes.data, model.ndofs, model.nu
        req.Uex, req.Fex = U.ctypes.data, F.ctypes.data
        req.loads, req.nloads = C.cast(arr, C.c_void_p), len(loads)
        req.stage = stage_params(**kw)
        rid = C.c_int64()
        rc = L.lib().amr_server_submit(self.h, C.byref(req), C.byref(rid))
        if rc:
            raise L.AmrError(rc, "amr_server_submit: " + ("the request can never fit the HBM budget"
                                                         if rc == -9 else "bad request"))
        return Ticket(rid.value, model.nnodes, model.ndim, model.ndofs, model.nu, model.dof_node.copy(),
                      model.dof_comp.copy())

    def wait(self, t):
        """Blocks until the request is done: returns (status, U, F, result, message) with U and F the
        stage's node-major (nnodes, ndim) displacement and force increments."""
        U = np.zeros(t.ndofs)
        F = np.zeros(t.ndofs)
        res = L.RequestResult()
        msg = C.create_string_buffer(512)
        rc = L.lib().amr_server_wait(self.h, t.id, U.ctypes.data_as(C.c_void_p), F.ctypes.data_as(C.c_void_p),
                                     C.byref(res), msg, 512)
        Un = np.zeros((t.nnodes, t.ndim))
        Fn = np.zeros((t.nnodes, t.ndim))
        Un[t.dof_node, t.dof_comp] = U
        Fn[t.dof_node, t.dof_comp] = F
        return rc, Un, Fn, res, msg.value.decode("utf-8", "replace")

    def info(self):
        s = L.ServerInfo()
        L.check(None, L.lib().amr_server_stats(self.h, C.byref(s)))
        return s

    def close(self):
        if getattr(self, "h", None):
            L.lib().amr_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
