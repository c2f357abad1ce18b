"""ctypes binding of libamaru_gpu.so (include/amaru_gpu.h).

The shared library is built in-tree (amaru.jl_gb300/build.py).  Loading fails
loudly when it is missing: there is no CPU fallback for any operation.
"""
import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libamaru_gpu.so")

AMR_OK = 0
ERRORS = {-1: "EINVAL", -2: "ECUDA", -3: "ENEGJAC", -4: "ERETMAP", -5: "ENAN", -6: "ESINGULAR", -7: "ENOCONV",
          -8: "ETIMEOUT", -9: "ENOMEM", -10: "EUNSUPPORTED", -11: "ESTAGE"}

LIN2, LIN3, TRI3, TRI6, QUAD4, QUAD8, QUAD9, TET4, TET10, HEX8, HEX20 = range(1, 12)
D3, PLANESTRAIN, PLANESTRESS, AXISYMMETRIC = 0, 1, 2, 3
LINEAR_ELASTIC, VON_MISES, DRUCKER_PRAGER = 0, 1, 2
LOAD_FACET, LOAD_BODY = 0, 1
SOLVER_MIXED, SOLVER_FP64, SOLVER_AMG, SOLVER_AMG_FP64 = 0, 1, 2, 3
ASSEMBLY_FAST, ASSEMBLY_REFERENCE = 0, 1
KERNEL_SPMV32, KERNEL_RESIDUAL64, KERNEL_STIFFNESS, KERNEL_AMG_RESIDUAL, KERNEL_DYN_RHS = 0, 1, 2, 5, 6
KERNEL_SPMV64, KERNEL_AMG_RESIDUAL64 = 7, 8
PEAK_FP64_FMA, PEAK_FP32_FMA = 0, 1
COUPLED_HYDRO, COUPLED_THERMO = 0, 1


class AmrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%s)" % (msg, ERRORS.get(code, code)))
        self.code = code
        self.msg = msg


class ModelDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("stressmodel", C.c_int32), ("thickness", C.c_double), ("nnodes", C.c_int64),
                ("coords", C.c_void_p), ("nelems", C.c_int64), ("shape", C.c_void_p), ("nips", C.c_void_p),
                ("conn_ptr", C.c_void_p), ("conn", C.c_void_p), ("mat_type", C.c_void_p), ("mat_params", C.c_void_p)]


class Load(C.Structure):
    _fields_ = [("kind", C.c_int32), ("dir", C.c_int32), ("edge_key", C.c_int32), ("facet_shape", C.c_int32),
                ("nitems", C.c_int64), ("items", C.c_void_p), ("coef", C.c_double * 5)]


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int32), ("rtol", C.c_double), ("max_iters", C.c_int32), ("refine_every", C.c_int32)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("rel_residual", C.c_double),
                ("seconds", C.c_double)]


class StageParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("rtol", C.c_double), ("rspan", C.c_double), ("dT0", C.c_double),
                ("dTmin", C.c_double), ("dTmax", C.c_double), ("scheme", C.c_int32), ("maxits", C.c_int32),
                ("autoinc", C.c_int32), ("nincs", C.c_int32), ("nouts", C.c_int32), ("linear", SolveOpts)]


class StageStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("increments", C.c_int32), ("iterations", C.c_int32),
                ("krylov_iterations", C.c_int32), ("residue", C.c_double), ("T", C.c_double),
                ("seconds", C.c_double), ("solve_seconds", C.c_double)]


class IterationRecord(C.Structure):
    _fields_ = [("increment", C.c_int32), ("iteration", C.c_int32), ("krylov_iterations", C.c_int32),
                ("converged", C.c_int32), ("T", C.c_double), ("dT", C.c_double), ("residue", C.c_double)]


class IncrementInfo(C.Structure):
    _fields_ = [("T", C.c_double), ("increment", C.c_int32), ("checkpoint", C.c_int32), ("ndofs", C.c_int64),
                ("U", C.POINTER(C.c_double)), ("F", C.POINTER(C.c_double))]


INCREMENT_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(IncrementInfo))


MAX_TUNED_GROUPS = 8


class Tuning(C.Structure):
    _fields_ = [("ngroups", C.c_int32), ("shape", C.c_int32 * MAX_TUNED_GROUPS),
                ("stiffness_epb", C.c_int32 * MAX_TUNED_GROUPS), ("internal_epb", C.c_int32 * MAX_TUNED_GROUPS),
                ("batch_threads", C.c_int32), ("batch_ctas_per_sm", C.c_int32),
                ("stiffness_seconds", C.c_double), ("internal_seconds", C.c_double)]


class DynParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("dTmin", C.c_double), ("dTmax", C.c_double), ("rspan", C.c_double),
                ("alpha", C.c_double), ("beta", C.c_double), ("tspan", C.c_double), ("maxits", C.c_int32),
                ("autoinc", C.c_int32), ("nincs", C.c_int32), ("nouts", C.c_int32), ("linear", SolveOpts),
                ("sism", C.c_int32), ("sism_dir", C.c_int32), ("tss", C.c_double), ("tds", C.c_double),
                ("sism_acc", C.c_void_p), ("sism_n", C.c_int64)]


class CoupledDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("pad", C.c_int32), ("gammaw", C.c_double), ("T0", C.c_double),
                ("params", C.c_void_p)]


class ModalParams(C.Structure):
    _fields_ = [("nmodes", C.c_int32), ("max_iters", C.c_int32), ("tol", C.c_double)]


class ModalStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("block", C.c_int32), ("max_residual", C.c_double),
                ("seconds", C.c_double)]


class VtuArray(C.Structure):
    _fields_ = [("name", C.c_char_p), ("type", C.c_int32), ("ncomp", C.c_int32), ("on_device", C.c_int32),
                ("pad", C.c_int32), ("data", C.c_void_p)]


VTU_TYPES = {np.dtype(np.float64): 0, np.dtype(np.int32): 1, np.dtype(np.int64): 2, np.dtype(np.uint64): 3}


def vtu_arrays(items):
    """(name, numpy array) pairs -> (ctypes array of VtuArray, kept buffers); arrays are nrows x ncomp."""
    keep = []
    arr = (VtuArray * max(1, len(items)))()
    for i, (name, a) in enumerate(items):
        a = np.asarray(a)
        if a.dtype not in VTU_TYPES:
            a = a.astype(np.float64)
        a = np.asfortranarray(a)
        nm = name.encode("utf-8")
        keep += [a, nm]
        arr[i].name, arr[i].type = nm, VTU_TYPES[a.dtype]
        arr[i].ncomp = 1 if a.ndim == 1 else a.shape[1]
        arr[i].on_device, arr[i].data = 0, a.ctypes.data
    return arr, keep


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("max_active", C.c_int32), ("pad", C.c_int32)]


class Request(C.Structure):
    _fields_ = [("model", ModelDesc), ("eq_id", C.c_void_p), ("ndofs", C.c_int64), ("nu", C.c_int64),
                ("Uex", C.c_void_p), ("Fex", C.c_void_p), ("loads", C.c_void_p), ("nloads", C.c_int32),
                ("pad", C.c_int32), ("stage", StageParams)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("active_at_admit", C.c_int32), ("bytes", C.c_int64),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double), ("stage", StageStats),
                ("t_stage", C.c_double), ("dev_start", C.c_double), ("dev_end", C.c_double)]


class ServerInfo(C.Structure):
    _fields_ = [("queued", C.c_int64), ("active", C.c_int64), ("peak_active", C.c_int64), ("completed", C.c_int64),
                ("active_bytes", C.c_int64), ("peak_bytes", C.c_int64), ("seconds", C.c_double)]


# recovered field codes (AMR_FIELD_*) and the reference's ip_state_vals keys
FIELD_NAMES = ["σxx", "σyy", "σzz", "σyz", "σxz", "σxy", "σvm", "σ1", "σ2", "σ3", "εxx", "εyy", "εzz", "εyz", "εxz",
               "εxy", "ep", "epa", "j1", "srj2d"]
NFIELD_CODES = len(FIELD_NAMES)
# the keys the codes carry in an axisymmetric analysis (src/tools/tensors.jl:182-193)
AXI_FIELD_NAMES = {0: "σrr", 2: "σtt", 5: "σry", 10: "εrr", 12: "εtt", 15: "εry"}

# Every exported entry point of include/amaru_gpu.h with its ctypes signature.
P = C.c_void_p
SIGNATURES = {
    "amr_model_create": (C.c_int, [C.POINTER(ModelDesc), C.POINTER(C.c_void_p)]),
    "amr_model_destroy": (C.c_int, [P]),
    "amr_last_error": (C.c_int, [P, C.c_char_p, C.c_size_t]),
    "amr_create_error": (C.c_char_p, []),
    "amr_set_dofs": (C.c_int, [P, P, C.c_int64, C.c_int64]),
    "amr_set_youngs": (C.c_int, [P, P]),
    "amr_set_assembly": (C.c_int, [P, C.c_int32]),
    "amr_set_amg_smoothing": (C.c_int, [P, C.c_int32]),
    "amr_assemble_K": (C.c_int, [P]),
    "amr_get_K_nnz": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "amr_get_K_csc": (C.c_int, [P, P, P, P]),
    "amr_update_state": (C.c_int, [P, P, P]),
    "amr_state_commit": (C.c_int, [P]),
    "amr_state_restore": (C.c_int, [P]),
    "amr_get_state": (C.c_int, [P, P]),
    "amr_set_state": (C.c_int, [P, P]),
    "amr_get_elem_nips": (C.c_int, [P, P]),
    "amr_get_sizes": (C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                C.POINTER(C.c_int64)]),
    "amr_assemble_loads": (C.c_int, [P, C.POINTER(Load), C.c_int32, C.c_double, P]),
    "amr_solve": (C.c_int, [P, P, P, C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    "amr_stage_run": (C.c_int, [P, P, P, C.POINTER(StageParams), P, P, C.POINTER(StageStats)]),
    "amr_stage_run_dev": (C.c_int, [P, P, P, C.POINTER(StageParams), P, P, C.POINTER(StageStats)]),
    "amr_solve_noalloc": (C.c_int, [P, P, P, C.POINTER(SolveOpts), C.POINTER(SolveStats)]),
    "amr_set_parts": (C.c_int, [P, C.c_int64, P]),
    "amr_get_part_stats": (C.c_int, [P, C.c_int64, P]),
    "amr_autotune": (C.c_int, [P, C.POINTER(Tuning)]),
    "amr_estimate_bytes": (C.c_int, [C.POINTER(ModelDesc), C.POINTER(C.c_int64)]),
    "amr_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "amr_server_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(C.c_int64)]),
    "amr_server_wait": (C.c_int, [P, C.c_int64, P, P, C.POINTER(RequestResult), C.c_char_p, C.c_size_t]),
    "amr_server_stats": (C.c_int, [P, C.POINTER(ServerInfo)]),
    "amr_server_destroy": (C.c_int, [P]),
    "amr_time_kernel": (C.c_int, [P, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "amr_launch_count": (C.c_int, [P, C.POINTER(C.c_int64)]),
    "amr_alloc_count": (C.c_int, [C.POINTER(C.c_int64)]),
    "amr_coupled_mount": (C.c_int, [P, C.POINTER(CoupledDesc), P, C.c_int64, C.c_double, P, C.POINTER(C.c_int64),
                                    P, P, P, P]),
    "amr_get_stage_log": (C.c_int, [P, P, C.c_int32, C.POINTER(C.c_int32)]),
    "amr_set_increment_callback": (C.c_int, [P, INCREMENT_FN, C.c_void_p]),
    "amr_measure_peak": (C.c_int, [C.c_int32, C.POINTER(C.c_double)]),
    "amr_set_density": (C.c_int, [P, P]),
    "amr_assemble_M": (C.c_int, [P]),
    "amr_get_M_csc": (C.c_int, [P, C.POINTER(C.c_int64), P, P, P]),
    "amr_dyn_stage_run": (C.c_int, [P, P, P, P, P, C.POINTER(DynParams), P, P, P, P, C.POINTER(StageStats)]),
    "amr_default_dyn_params": (None, [C.POINTER(DynParams)]),
    "amr_modal_run": (C.c_int, [P, C.POINTER(ModalParams), P, P, C.POINTER(ModalStats)]),
    "amr_default_modal_params": (None, [C.POINTER(ModalParams)]),
    "amr_write_vtu": (C.c_int, [P, C.c_char_p, P, C.c_int32, P, C.c_int32, C.c_int32]),
    "amr_write_vtu_compressed": (C.c_int, [P, C.c_char_p, P, C.c_int32, P, C.c_int32, C.c_int32]),
    "amr_recovery_fields": (C.c_int, [P, P, C.c_int32, C.POINTER(C.c_int32)]),
    "amr_recover_nodal": (C.c_int, [P, P]),
    "amr_recover_nodal_dev": (C.c_int, [P, P]),
    "amr_time_recovery": (C.c_int, [P, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int64)]),
    "amr_default_solve_opts": (None, [C.POINTER(SolveOpts)]),
    "amr_default_stage_params": (None, [C.POINTER(StageParams)]),
}

_lock = threading.Lock()
_lib = None


def lib():
    """Load the CUDA library (raises if it was not built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("libamaru_gpu.so is not built (run amaru.jl_gb300/build.py); "
                                   "the GPU path has no CPU fallback")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def check(h, rc):
    if rc != AMR_OK:
        buf = C.create_string_buffer(1024)
        if h:
            lib().amr_last_error(h, buf, 1024)
            msg = buf.value.decode("utf-8", "replace")
        else:
            msg = (lib().amr_create_error() or b"").decode("utf-8", "replace")
        raise AmrError(rc, msg)
    return rc


def measure_peak(which):
    """TFLOP/s of fused multiply-adds on the current GPU (amr_measure_peak): PEAK_FP64_FMA or PEAK_FP32_FMA."""
    t = C.c_double()
    check(None, lib().amr_measure_peak(which, C.byref(t)))
    return t.value


def default_solve_opts(**kw):
    o = SolveOpts()
    lib().amr_default_solve_opts(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def default_stage_params(**kw):
    p = StageParams()
    lib().amr_default_stage_params(C.byref(p))
    for k, v in kw.items():
        if k == "linear":
            p.linear = v
        else:
            setattr(p, k, v)
    return p


def default_dyn_params(**kw):
    p = DynParams()
    lib().amr_default_dyn_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def model_desc(ndim, stressmodel, thickness, coords, shape, nips, conn_ptr, conn, mat_type, mat_params):
    """(ModelDesc, arrays it points into): keep the arrays alive while the desc is used."""
    keep = [np.ascontiguousarray(coords, dtype=np.float64), np.ascontiguousarray(shape, dtype=np.int32),
            np.ascontiguousarray(nips, dtype=np.int32), np.ascontiguousarray(conn_ptr, dtype=np.int64),
            np.ascontiguousarray(conn, dtype=np.int64), np.ascontiguousarray(mat_type, dtype=np.int32),
            np.ascontiguousarray(mat_params, dtype=np.float64)]
    c, s, n, cp, cn, mt, mp = keep
    d = ModelDesc()
    d.ndim, d.stressmodel, d.thickness = ndim, stressmodel, thickness
    d.nnodes, d.coords = c.shape[0], ptr(c)
    d.nelems, d.shape, d.nips = s.shape[0], ptr(s), ptr(n)
    d.conn_ptr, d.conn, d.mat_type, d.mat_params = ptr(cp), ptr(cn), ptr(mt), ptr(mp)
    return d, keep


def load_array(loads):
    """(Load array, arrays it points into) from (kind, dir, edge_key, facet_shape, items, coef) tuples."""
    arr = (Load * max(len(loads), 1))()
    keep = []
    for i, (kind, dr, edge, fshape, items, coef) in enumerate(loads):
        it = np.ascontiguousarray(items, dtype=np.int64)
        keep.append(it)
        arr[i].kind, arr[i].dir, arr[i].edge_key, arr[i].facet_shape = kind, dr, edge, fshape
        arr[i].nitems = it.shape[0] if it.ndim > 0 else 0
        arr[i].items = ptr(it)
        for k in range(5):
            arr[i].coef[k] = coef[k]
    return arr, keep


class DeviceModel:
    """Owning wrapper of an amr_model handle."""

    def __init__(self, ndim, stressmodel, thickness, coords, shape, nips, conn_ptr, conn, mat_type, mat_params):
        d, self._keep = model_desc(ndim, stressmodel, thickness, coords, shape, nips, conn_ptr, conn, mat_type,
                                   mat_params)
        h = C.c_void_p()
        check(None, lib().amr_model_create(C.byref(d), C.byref(h)))
        self.h = h
        self._keep = None
        self.ndim = ndim
        self.stressmodel = stressmodel
        self.ndofs = 0
        self.nu = 0

    def close(self):
        if getattr(self, "h", None):
            lib().amr_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sizes(self):
        a, b, c, d = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(self.h, lib().amr_get_sizes(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return dict(nnodes=a.value, nelems=b.value, nip_total=c.value, nblocks=d.value)

    def set_dofs(self, eq_id, ndofs, nu):
        eq = np.ascontiguousarray(eq_id, dtype=np.int64)
        check(self.h, lib().amr_set_dofs(self.h, ptr(eq), ndofs, nu))
        self.ndofs, self.nu = ndofs, nu

    def set_youngs(self, E):
        E = np.ascontiguousarray(E, dtype=np.float64)
        check(self.h, lib().amr_set_youngs(self.h, ptr(E)))

    def assemble_K(self):
        check(self.h, lib().amr_assemble_K(self.h))

    def set_assembly(self, mode):
        check(self.h, lib().amr_set_assembly(self.h, mode))

    def set_amg_smoothing(self, on):
        """Smoothed-aggregation prolongators (True, the default) or the tentative ones (False) for the
        multigrid solvers (amr_set_amg_smoothing)."""
        check(self.h, lib().amr_set_amg_smoothing(self.h, 1 if on else 0))

    def K_csc(self):
        """K as a scipy CSC matrix in eq_id order with the reference's stored-entry pattern."""
        import scipy.sparse as sp
        nnz = C.c_int64()
        check(self.h, lib().amr_get_K_nnz(self.h, C.byref(nnz)))
        cp = np.zeros(self.ndofs + 1, dtype=np.int64)
        rv = np.zeros(max(nnz.value, 1), dtype=np.int64)
        nz = np.zeros(max(nnz.value, 1))
        check(self.h, lib().amr_get_K_csc(self.h, ptr(cp), ptr(rv), ptr(nz)))
        return sp.csc_matrix((nz[:nnz.value], rv[:nnz.value], cp), shape=(self.ndofs, self.ndofs))

    def update_state(self, dU):
        dU = np.ascontiguousarray(dU, dtype=np.float64)
        dF = np.zeros(self.ndofs)
        check(self.h, lib().amr_update_state(self.h, ptr(dU), ptr(dF)))
        return dF

    def commit(self):
        check(self.h, lib().amr_state_commit(self.h))

    def restore(self):
        check(self.h, lib().amr_state_restore(self.h))

    def state(self):
        n = self.sizes()["nip_total"]
        s = np.zeros((n, 16))
        check(self.h, lib().amr_get_state(self.h, ptr(s)))
        return s

    def elem_nips(self):
        """The IP count of each element (its rows of state()), element order."""
        out = np.zeros(self.sizes()["nelems"], dtype=np.int32)
        check(self.h, lib().amr_get_elem_nips(self.h, ptr(out)))
        return out

    def set_state(self, state):
        s = np.ascontiguousarray(state, dtype=np.float64)
        if s.shape != (self.sizes()["nip_total"], 16):
            raise ValueError("state must be nip_total x 16")
        check(self.h, lib().amr_set_state(self.h, ptr(s)))

    def assemble_loads(self, loads, F, t=0.0):
        arr, keep = load_array(loads)
        F = np.ascontiguousarray(F, dtype=np.float64)
        check(self.h, lib().amr_assemble_loads(self.h, arr, len(loads), t, ptr(F)))
        return F

    def solve(self, U, F, opts=None):
        U = np.ascontiguousarray(U, dtype=np.float64).copy()
        F = np.ascontiguousarray(F, dtype=np.float64).copy()
        st = SolveStats()
        o = opts if opts is not None else default_solve_opts()
        check(self.h, lib().amr_solve(self.h, ptr(U), ptr(F), C.byref(o), C.byref(st)))
        return U, F, st

    def stage_run(self, Uex, Fex, params, out=None):
        """out: (U, F) host arrays (ndofs float64, C-contiguous, e.g. views of pinned memory) to write into."""
        Uex = np.ascontiguousarray(Uex, dtype=np.float64)
        Fex = np.ascontiguousarray(Fex, dtype=np.float64)
        if out is None:
            U = np.zeros(self.ndofs)
            F = np.zeros(self.ndofs)
        else:
            U, F = out
            for a in (U, F):
                if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.ndofs:
                    raise ValueError("out arrays must be C-contiguous float64 of ndofs entries")
        st = StageStats()
        rc = lib().amr_stage_run(self.h, ptr(Uex), ptr(Fex), C.byref(params), ptr(U), ptr(F), C.byref(st))
        return rc, U, F, st

    def stage_log(self):
        """The last whole-model stage's Newton iterations (amr_get_stage_log)."""
        n = C.c_int32()
        check(self.h, lib().amr_get_stage_log(self.h, None, 0, C.byref(n)))
        rec = (IterationRecord * max(n.value, 1))()
        check(self.h, lib().amr_get_stage_log(self.h, rec, n.value, C.byref(n)))
        return list(rec[:n.value])

    def set_increment_callback(self, fn):
        """fn(T, increment, checkpoint, U, F) -> truthy to stop, after every converged increment of a stage
        (amr_set_increment_callback); U and F are copies.  None clears it."""
        if fn is None:
            self._inc_cb = None
            check(self.h, lib().amr_set_increment_callback(self.h, INCREMENT_FN(), None))
            return

        def tramp(_user, info):
            i = info.contents
            U = np.ctypeslib.as_array(i.U, shape=(i.ndofs,)).copy() if i.ndofs else np.zeros(0)
            F = np.ctypeslib.as_array(i.F, shape=(i.ndofs,)).copy() if i.ndofs else np.zeros(0)
            try:
                return 1 if fn(i.T, i.increment, bool(i.checkpoint), U, F) else 0
            except Exception:  # noqa: BLE001 -- an exception must not cross the C ABI: stop the stage
                return 1
        self._inc_cb = INCREMENT_FN(tramp)  # kept alive while the library holds it
        check(self.h, lib().amr_set_increment_callback(self.h, self._inc_cb, None))

    def stage_run_dev(self, d_Uex, d_Fex, params, d_U, d_F):
        """Device-pointer variant: arguments are raw CUDA device addresses (ints) of ndofs doubles."""
        st = StageStats()
        rc = lib().amr_stage_run_dev(self.h, C.c_void_p(d_Uex), C.c_void_p(d_Fex), C.byref(params), C.c_void_p(d_U),
                                     C.c_void_p(d_F), C.byref(st))
        return rc, st

    def set_parts(self, node_ptr):
        """Declares the handle a batch of independent parts (node ranges node_ptr[i]..node_ptr[i+1]-1)."""
        a = np.ascontiguousarray(node_ptr, dtype=np.int64)
        self.nparts = len(a) - 1 if len(a) else 0
        check(self.h, lib().amr_set_parts(self.h, self.nparts, ptr(a) if len(a) else None))

    def part_stats(self):
        out = (StageStats * self.nparts)()
        check(self.h, lib().amr_get_part_stats(self.h, self.nparts, C.cast(out, C.c_void_p)))
        return list(out)

    def autotune(self):
        t = Tuning()
        check(self.h, lib().amr_autotune(self.h, C.byref(t)))
        return t

    def time_kernel(self, which, reps):
        t, b = C.c_double(), C.c_double()
        check(self.h, lib().amr_time_kernel(self.h, which, reps, C.byref(t), C.byref(b)))
        return t.value, b.value

    def set_density(self, rho):
        r = np.ascontiguousarray(rho, dtype=np.float64)
        check(self.h, lib().amr_set_density(self.h, ptr(r)))

    def assemble_M(self):
        check(self.h, lib().amr_assemble_M(self.h))

    def M_csc(self):
        import scipy.sparse as sp
        nnz = C.c_int64()
        check(self.h, lib().amr_get_M_csc(self.h, C.byref(nnz), None, None, None))
        colptr = np.zeros(self.ndofs + 1, dtype=np.int64)
        rowval = np.zeros(max(nnz.value, 1), dtype=np.int64)
        nzval = np.zeros(max(nnz.value, 1))
        check(self.h, lib().amr_get_M_csc(self.h, C.byref(nnz), ptr(colptr), ptr(rowval), ptr(nzval)))
        return sp.csc_matrix((nzval[:nnz.value], rowval[:nnz.value], colptr), shape=(self.ndofs, self.ndofs))

    def dyn_stage_run(self, U0, U1, F0, F1, params):
        """dyn_stage_solver!: boundary values U0 + t U1, F0 + t F1; returns (rc, U, V, A, F, stats)."""
        ins = [np.ascontiguousarray(a, dtype=np.float64) for a in (U0, U1, F0, F1)]
        outs = [np.zeros(self.ndofs) for _ in range(4)]
        st = StageStats()
        rc = lib().amr_dyn_stage_run(self.h, *[ptr(a) for a in ins], C.byref(params), *[ptr(a) for a in outs],
                                     C.byref(st))
        return (rc, *outs, st)

    def modal(self, nmodes=5, tol=1e-7, max_iters=1000):
        """mech_modal_solver!: (omega (nmodes), modes (nu x nmodes), stats)."""
        p = ModalParams()
        lib().amr_default_modal_params(C.byref(p))
        p.nmodes, p.tol, p.max_iters = nmodes, tol, max_iters
        w = np.zeros(nmodes)
        V = np.zeros((nmodes, self.nu))
        st = ModalStats()
        check(self.h, lib().amr_modal_run(self.h, C.byref(p), ptr(w), ptr(V), C.byref(st)))
        return w, V.T.copy(), st

    def write_vtu(self, path, point_items, cell_items, nthreads=0, compress=False):
        pa, k1 = vtu_arrays(point_items)
        ca, k2 = vtu_arrays(cell_items)
        fn = lib().amr_write_vtu_compressed if compress else lib().amr_write_vtu
        check(self.h, fn(self.h, str(path).encode("utf-8"), C.cast(pa, C.c_void_p), len(point_items),
                         C.cast(ca, C.c_void_p), len(cell_items), nthreads))

    def recovery_fields(self):
        """Field names of the nodal recovery, in the reference's column order."""
        codes = np.zeros(NFIELD_CODES, dtype=np.int32)
        n = C.c_int32()
        check(self.h, lib().amr_recovery_fields(self.h, ptr(codes), NFIELD_CODES, C.byref(n)))
        names = AXI_FIELD_NAMES if self.stressmodel == AXISYMMETRIC else {}
        return [names.get(int(c), FIELD_NAMES[c]) for c in codes[:n.value]]

    def recover_nodal(self):
        """nodal_patch_recovery: (V (nnodes x nfields), field names) from the current IP states."""
        names = self.recovery_fields()
        V = np.zeros((len(names), self.sizes()["nnodes"]))
        if names:
            check(self.h, lib().amr_recover_nodal(self.h, ptr(V)))
        return V.T, names

    def recover_nodal_dev(self, d_V):
        """Device-pointer variant: d_V is the raw CUDA address of nnodes x nfields doubles (column-major)."""
        check(self.h, lib().amr_recover_nodal_dev(self.h, C.c_void_p(d_V)))

    def time_recovery(self, reps):
        t, f, n = C.c_double(), C.c_double(), C.c_int64()
        check(self.h, lib().amr_time_recovery(self.h, reps, C.byref(t), C.byref(f), C.byref(n)))
        return t.value, f.value, n.value

    def launch_count(self):
        n = C.c_int64()
        check(self.h, lib().amr_launch_count(self.h, C.byref(n)))
        return n.value

    @staticmethod
    def alloc_count():
        """Device allocations and frees the library has made in this process (all handles)."""
        n = C.c_int64()
        check(None, lib().amr_alloc_count(C.byref(n)))
        return n.value

    def last_error(self):
        buf = C.create_string_buffer(1024)
        lib().amr_last_error(self.h, buf, 1024)
        return buf.value.decode("utf-8", "replace")
