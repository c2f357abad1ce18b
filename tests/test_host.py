"""Host-side logic (no GPU).

  * the C-ABI library's exports, and the Julia binding's entry points and struct layouts against them;
  * the structured mesher, expression evaluation and DOF numbering, each checked against the oracle;
  * the boundary's refusals of bad model descriptions and solver keywords, before any device call;
  * no CPU fallback: the GPU path raises without its library.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle as O
import amaru_gpu as A
from amaru_gpu import _lib
from amaru_gpu.expr import affine_coefficients, evaluate
from amaru_gpu.model import number_dofs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    src = open(os.path.join(ROOT, "include", "amaru_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(amr_[A-Za-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    assert os.path.exists(_lib.LIB_PATH), "build() must have produced libamaru_gpu.so"
    so = ctypes.CDLL(_lib.LIB_PATH)
    names = _header_functions()
    assert len(names) >= 19
    for n in names:
        assert hasattr(so, n), n
    assert sorted(_lib.SIGNATURES) == names


def test_julia_binding_calls_only_declared_symbols():
    """Julia is not installed, so the ccall binding cannot run here: every entry point it names must at
    least be one the header declares and the library exports."""
    src = open(os.path.join(ROOT, "amaru.jl_gb300", "julia", "AmaruGPU.jl")).read()
    called = set(re.findall(r"ccall\(\(:(amr_[A-Za-z0-9_]+)\s*,", src))
    assert len(called) >= 30
    assert called <= set(_header_functions()), sorted(called - set(_header_functions()))


def _julia_structs():
    """A builder of ctypes layouts for the Julia binding's structs, from their field declarations."""
    src = open(os.path.join(ROOT, "amaru.jl_gb300", "julia", "AmaruGPU.jl")).read()
    blocks = re.findall(r"^(?:mutable )?struct (\w+)\n(.*?)^end", src, flags=re.S | re.M)
    decls = {name: re.findall(r"(\w+)::([\w{}, ]+?)\s*(?=;|\n|$)", body) for name, body in blocks}
    prim = {"Int32": ctypes.c_int32, "Int64": ctypes.c_int64, "Float64": ctypes.c_double, "Cstring": ctypes.c_char_p,
            "Int": ctypes.c_int64}
    built = {}

    def ctype(t):
        t = t.strip()
        if t in prim:
            return prim[t]
        if t.startswith("Ptr{"):
            return ctypes.c_void_p
        m = re.match(r"NTuple\{(\d+),\s*(\w+)\}", t)
        if m:
            return ctype(m.group(2)) * int(m.group(1))
        return build(t)

    def build(name):
        if name not in built:
            built[name] = type(name, (ctypes.Structure,), {"_fields_": [(f, ctype(t)) for f, t in decls[name]]})
        return built[name]

    return build


def _layout(cls):
    return ctypes.sizeof(cls), [(getattr(cls, f).offset, getattr(cls, f).size) for f, _ in cls._fields_]


@pytest.mark.parametrize("name", ["ModelDesc", "SolveOpts", "SolveStats", "StageParams", "StageStats", "DynParams",
                                  "VtuArray", "ModalParams", "ModalStats", "Request", "RequestResult",
                                  "ServerConfig", "ServerInfo", "Tuning", "IncrementInfo",
                                  "CoupledDesc"])
def test_julia_struct_layouts_match_the_c_abi(name):
    """Each struct the Julia binding passes by reference has the byte layout of the ctypes mirror of the
    same C struct (offsets and sizes field by field)."""
    jl = _julia_structs()(name)
    py = getattr(_lib, name)
    assert _layout(jl) == _layout(py)


@pytest.mark.parametrize("shape,n", [(A.HEX8, (3, 2, 2)), (A.HEX20, (3, 2, 2)), (A.TET10, (2, 2, 2)),
                                     (A.TET4, (2, 2, 1)), (A.QUAD8, (3, 2)), (A.QUAD4, (3, 2)), (A.QUAD9, (2, 2)),
                                     (A.TRI3, (2, 2)), (A.TRI6, (2, 2))])
def test_mesher_matches_oracle(shape, n):
    """Node numbering, connectivity and outer facets equal the restated split_block!/synchronize!."""
    if len(n) == 3:
        bm = A.Block([[0, 0, 0], [1, 0.5, 0.7]], nx=n[0], ny=n[1], nz=n[2], cellshape=shape)
        bo = O.Block([[0, 0, 0], [1, 0.5, 0.7]], nx=n[0], ny=n[1], nz=n[2], cellshape=shape)
    else:
        bm = A.Block([[0, 0], [1, 0.5]], nx=n[0], ny=n[1], cellshape=shape)
        bo = O.Block([[0, 0], [1, 0.5]], nx=n[0], ny=n[1], cellshape=shape)
    mm, mo = A.Mesh(bm), O.Mesh(bo)
    np.testing.assert_allclose(mm.coords, mo.coords, rtol=0, atol=1e-15)
    assert (mm.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    assert [list(r[r >= 0]) for r in mm.face_nodes] == [f.nodes for f in mo.faces]
    assert sorted(map(lambda r: tuple(sorted(r)), mm.edge_nodes.tolist())) == \
        sorted(tuple(sorted(e.nodes)) for e in mo.edges)


@pytest.mark.parametrize("shape,n,nodes", [(A.HEX8, (10, 10, 10), 1331), (A.HEX20, (10, 10, 10), 4961),
                                           (A.TET10, (10, 10, 10), 9261), (A.QUAD8, (10, 10), 341),
                                           (A.TRI6, (10, 10), 441), (A.TRI3, (10, 10), 221)])
def test_mesher_node_counts(shape, n, nodes):
    """test/mesh/structured.jl node counts."""
    if len(n) == 3:
        b = A.Block([[0, 0, 0], [1, 1, 1]], nx=n[0], ny=n[1], nz=n[2], cellshape=shape)
    else:
        b = A.Block([[0, 0], [1, 1]], nx=n[0], ny=n[1], cellshape=shape)
    assert len(A.Mesh(b).coords) == nodes


def test_config_mesh_counts():
    """Mesh sizes of the benchmark workloads (HEX8 20x4x4, HEX20 100x40x40 is checked by formula)."""
    m = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.2, 0.2]], nx=20, ny=4, nz=4, cellshape=A.HEX8))
    assert len(m.coords) == 525 and len(m.shape) == 320
    m = A.Mesh(A.Block([[0, 0, 0], [10, 4, 4]], nx=10, ny=4, nz=4, cellshape=A.HEX20))
    nx, ny, nz = 10, 4, 4
    full = (2 * nx + 1) * (2 * ny + 1) * (2 * nz + 1)
    assert len(m.coords) == full - (nx * ny * (nz + 1) + nx * nz * (ny + 1) + ny * nz * (nx + 1)) - nx * ny * nz


@pytest.mark.parametrize("expr,pt,want", [("x==0 && y==0", (0, 0, 0), True), ("x==0 && y==0", (0, 1e-7, 0), True),
                                          ("x==0 || y==1", (2, 1, 0), True), ("x>=0.5", (0.4999999, 0, 0), True),
                                          ("x>0.5", (0.5000005, 0, 0), False), ("3*z", (0, 0, 2.0), 6.0),
                                          ("x^2+1", (2.0, 0, 0), 5.0)])
def test_expressions_match_oracle(expr, pt, want):
    x, y, z = pt
    assert evaluate(expr, x=np.array([x]), y=np.array([y]), z=np.array([z]))[0] == want
    assert O.evaluate(expr, x=x, y=y, z=z, t=0.0) == want


def test_affine_loads():
    assert affine_coefficients("3*z", 3) == [0.0, 0.0, 0.0, 3.0, 0.0]
    assert affine_coefficients(-10.0, 3)[0] == -10.0
    with pytest.raises(NotImplementedError):
        affine_coefficients("x*x", 3)


def test_dof_numbering_matches_oracle():
    """configure_dofs!: unknowns first, prescribed last, node order then component order."""
    mesh = O.Mesh(O.Block([[0, 0, 0], [1, 1, 1]], nx=2, ny=2, nz=1, cellshape=O.HEX8))
    model = O.FEModel(mesh, [("all", O.LinearElastic(E=1.0, nu=0.3))])
    bcs = [("z==0", O.NodeBC(ux=0, uz=0)), ("x==1", O.NodeBC(uy=0))]
    dofs, nu, _ = O.configure_dofs(model, bcs)
    presc = np.zeros((len(mesh.coords), 3), dtype=bool)
    for e, k in dofs[nu:]:
        presc[e, k] = True
    eq, ndofs, nu2, dn, dk = number_dofs(np.arange(len(mesh.coords)), presc, len(mesh.coords))
    assert nu2 == nu and ndofs == len(dofs)
    assert (eq == model.eq_id).all()


def test_slope_mesh_keeps_boundary_planes_and_orientation():
    """Slope mapping + interior jitter: boundary nodes stay on their planes, edge nodes at edge
    midpoints, and every TET10 keeps the orientation it had in the block."""
    from amaru_gpu import workloads as W
    g = W.SLOPE
    n = (10, 2, 4)
    mesh = A.Mesh(A.Block([[0, 0, 0], [g["L"], g["W"], g["H"]]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    en = mesh.elem_nodes()
    c0 = mesh.coords
    c = W.slope_coords(c0, en, W.boundary_nodes(mesh), 4, *n, seed=7)
    for k, v in ((0, 0.0), (0, g["L"]), (1, 0.0), (1, g["W"]), (2, 0.0)):
        on = c0[:, k] == v
        assert on.any() and (c[on, k] == v).all()
    crest = (c0[:, 2] == g["H"]) & (c0[:, 0] <= g["x1"])
    assert crest.any() and (c[crest, 2] == g["H"]).all()
    for j, a, b in W.edge_pairs(c0, en, 4):
        assert np.allclose(c[en[:, j]], 0.5 * (c[en[:, a]] + c[en[:, b]]))

    def vol(x):
        v = x[en[:, 1:4]] - x[en[:, [0]]]
        return np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2]))
    v0, v1 = vol(c0), vol(c)
    assert (np.sign(v0) == np.sign(v1)).all() and (np.abs(v1) > 0.2 * np.abs(v0)).all()
    assert not np.allclose(c, c0 * [1, 1, 1])  # jittered


def test_dynamic_and_modal_defaults_mirror_the_reference():
    """dyn_solver_params (src/mech/dyn-solver.jl:166-180) and mech_modal_solver_params
    (src/mech/mech-modal-solver.jl:49-56) defaults, as the C ABI fills them."""
    from amaru_gpu import _lib as L
    p = L.default_dyn_params()
    assert (p.tol, p.dTmin, p.dTmax, p.rspan, p.maxits, p.autoinc) == (0.01, 1e-7, 0.1, 0.01, 5, 0)
    assert (p.alpha, p.beta, p.nincs, p.nouts) == (0.0, 0.0, 1, 0)
    q = L.ModalParams()
    L.lib().amr_default_modal_params(L.C.byref(q))
    assert q.nmodes == 5 and q.max_iters > 0 and 0 < q.tol < 1e-4


def test_vtu_arrays_are_column_major_with_their_types():
    import numpy as np
    from amaru_gpu import _lib as L
    U = np.arange(12, dtype=np.float64).reshape(4, 3)  # C order in, column-major out
    ids = np.arange(1, 5, dtype=np.int64)
    arr, keep = L.vtu_arrays([("U", U), ("node-id", ids), ("f", np.arange(4, dtype=np.int16))])
    assert arr[0].name == b"U" and arr[0].type == 0 and arr[0].ncomp == 3
    buf = np.ctypeslib.as_array((L.C.c_double * 12).from_address(arr[0].data))
    assert np.array_equal(buf, U.T.reshape(-1))
    assert arr[1].type == 2 and arr[1].ncomp == 1
    assert arr[2].type == 0  # other dtypes are converted to Float64: the writer takes four element types


def _desc(ndim=3, stressmodel=_lib.D3, thickness=1.0, **over):
    """A one-element model description (HEX8 or QUAD4) with fields replaced by `over`."""
    shape = A.HEX8 if ndim == 3 else A.QUAD4
    box = [[0, 0, 0], [1, 1, 1]] if ndim == 3 else [[0, 0], [1, 1]]
    mesh = A.Mesh(A.Block(box, nx=1, ny=1, nz=1 if ndim == 3 else 0, cellshape=shape))
    arrays = dict(coords=mesh.coords, shape=np.array([over.pop("shape", shape)]), nips=np.zeros(1),
                  conn_ptr=np.array([0, len(mesh.conn)]), conn=mesh.conn, mat_type=np.zeros(1),
                  mat_params=np.array([200e3, 0.3, 0, 0, 0, 0, 0, 0]))
    arrays.update(over)
    return _lib.model_desc(ndim, stressmodel, thickness, **arrays)


@pytest.mark.parametrize("kw,code,words", [
    (dict(ndim=4), -1, "ndim must be 2 or 3"),
    (dict(stressmodel=_lib.PLANESTRAIN), -1, "d3 stress model"),
    (dict(ndim=2, stressmodel=_lib.PLANESTRESS, thickness=0.0), -1, "thickness must be > 0"),
    (dict(ndim=2, stressmodel=_lib.PLANESTRAIN, thickness=float("nan")), -1, "thickness must be > 0"),
    (dict(shape=A.QUAD4), -10, "shape not a bulk cell"),
    (dict(conn_ptr=np.array([0, 7])), -1, "wrong node count"),
    (dict(conn=np.array([0, 1, 2, 3, 4, 5, 6, 99])), -1, "node index out of range"),
    (dict(nips=np.array([5])), -1, "integration points"),
    (dict(mat_type=np.array([7])), -10, "unsupported material"),
    (dict(mat_params=np.array([0.0, 0.3, 0, 0, 0, 0, 0, 0])), -1, "E > 0"),
    (dict(mat_params=np.array([1.0, 0.5, 0, 0, 0, 0, 0, 0])), -1, "nu < 0.5"),
])
def test_model_description_refusals(kw, code, words):
    """amr_model_create refuses a bad description with its status code and message before any device
    call (so on a host without a GPU as well), and hands out no handle."""
    d, keep = _desc(**kw)
    h = ctypes.c_void_p(0)
    rc = _lib.lib().amr_model_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == code and not h.value
    assert words in _lib.lib().amr_create_error().decode()


def test_model_description_refuses_null_and_empty():
    L = _lib.lib()
    h = ctypes.c_void_p(0)
    assert L.amr_model_create(None, ctypes.byref(h)) == -1 and "null argument" in L.amr_create_error().decode()
    d, keep = _desc()
    d.coords = None
    assert L.amr_model_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert "null array" in L.amr_create_error().decode()
    d, keep = _desc()
    d.nelems = 0
    assert L.amr_model_create(ctypes.byref(d), ctypes.byref(h)) == -1 and "empty model" in L.amr_create_error().decode()


@pytest.mark.parametrize("kw,words", [
    (dict(tol=0.0), "tol which must satisfy tol > 0"),
    (dict(rspan=1.0), "rspan which must satisfy 0 < rspan < 1"),
    (dict(rtol=-1e-3), "rtol which must satisfy rtol > 0"),
    (dict(dT0=1.5), "dT0 which must satisfy 0 < dT0 <= 1"),
    (dict(dTmin=0.0), "dTmin which must satisfy 0 < dTmin < 1"),
    (dict(dTmax=1.0), "dTmax which must satisfy 0 < dTmax < 1"),
    (dict(maxits=11), "maxits which must satisfy 1 <= maxits <= 10"),
    (dict(scheme="RK4"), "scheme which must be one of"),
])
def test_solver_keywords_are_checked_as_the_reference_does(kw, words):
    """solve!'s keyword conditions (mech_solver_params, src/mech/mech-solver.jl:155-167), checked on the host
    before anything reaches the device: no model is needed to see the refusal."""
    from amaru_gpu import serve
    with pytest.raises(A.ArgumentError, match=words.replace("(", r"\(")):
        A.MechAnalysis(None).solve(**kw)
    with pytest.raises(A.ArgumentError):
        serve.stage_params(**kw)


@pytest.mark.parametrize("kw", [dict(tol=-1.0), dict(dTmin=2.0), dict(dTmax=0.0), dict(rspan=0.0), dict(maxits=0),
                                dict(scheme="RK4")])
def test_dynamic_solver_keywords_are_checked(kw):
    """dyn_solver_params (src/mech/dyn-solver.jl:166-186)."""
    with pytest.raises(A.ArgumentError, match="solve!: Invalid value for argument"):
        A.DynAnalysis(None).solve(**kw)


def test_solver_keyword_defaults_pass_the_checks():
    from amaru_gpu.args import MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, checkargs
    checkargs("solve!", MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, tol=0.01, rspan=0.01, rtol=0.01, dT0=0.01,
              dTmin=1e-7, dTmax=0.1, maxits=5, scheme="FE")
    checkargs("solve!", MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, dT0=1.0, maxits=10, scheme="Ralston")


def test_the_gpu_path_fails_loudly_without_its_library(monkeypatch, tmp_path):
    """No CPU fallback: with the CUDA library absent, loading it and building a model raise."""
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libamaru_gpu.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()
    mesh = A.Mesh(A.Block([[0, 0, 0], [1, 1, 1]], nx=1, ny=1, nz=1, cellshape=A.HEX8))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        A.FEModel(mesh, [("all", A.LinearElastic(E=1.0, nu=0.2))])
