"""Edge cases of the drop-in path: inputs the reference handles specially, bad inputs the
C ABI must refuse with a status (never a crash), and failures it must report.

* every DOF prescribed (nu = 0): solve_system! (src/solver.jl:5-79) only computes the
  reactions F2 = K22 U2;
* no load at all: the stage converges with U = 0;
* nodes that no element uses: no DOFs (configure_dofs!, src/bc.jl:198-233) and empty
  rows in the pattern;
* an inverted element: mount_K's "Negative Jacobian determinant in cell i"
  (src/mech/elem/mech-solid.jl:150), with the reference's 1-based cell number;
* NaN loads: the stage fails, as the reference's does;
* bad descriptions and call orders: AMR_EINVAL / AMR_EUNSUPPORTED with a message.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from amaru_gpu import _lib as L

pytestmark = pytest.mark.gpu

BOX = [[0, 0, 0], [1.0, 0.2, 0.2]]


def _pair(n=(4, 2, 2)):
    mo = O.Mesh(O.Block(BOX, nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX8))
    mg = A.Mesh(A.Block(BOX, nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX8))
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, [("all", O.LinearElastic(E=200e3, nu=0.3))])
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=200e3, nu=0.3))])
    return om, gm


def _run(om, gm, bcs_of):
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(bcs_of(O))
    ag.addstage(bcs_of(A))
    return ao.solve(), ag.solve()


def test_every_dof_prescribed():
    om, gm = _pair()
    ro, rg = _run(om, gm, lambda M: [("x>=0", M.NodeBC(ux=0, uy=0, uz=0)), ("x==1", M.NodeBC(uz=-1e-3))])
    assert ro[0] and rg[0]
    assert gm.nu == 0
    assert np.array_equal(gm.U, om.U)
    assert np.abs(gm.F - om.F).max() <= 1e-10 * np.abs(om.F).max()
    assert np.abs(om.F).max() > 0


def test_no_load():
    om, gm = _pair()
    ro, rg = _run(om, gm, lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0, uz=0))])
    assert ro[0] and rg[0]
    assert not gm.U.any() and not gm.F.any()


def test_nodes_without_elements():
    om, gm = _pair()
    _, base = _pair()
    mesh = gm.mesh
    mesh.coords = np.vstack([mesh.coords, [[5.0, 5.0, 5.0], [6.0, 5.0, 5.0]]])  # two unused nodes
    gx = A.FEModel(mesh, [("all", A.LinearElastic(E=200e3, nu=0.3))])
    bcs = [("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", A.SurfaceBC(tz=-1.0))]
    ax, ab = A.MechAnalysis(gx), A.MechAnalysis(base)
    ax.addstage(bcs)
    ab.addstage(bcs)
    assert ax.solve()[0] and ab.solve()[0]
    assert (gx.eq_id[-2:] == -1).all() and gx.ndofs == base.ndofs
    n = base.nnodes
    assert np.abs(gx.U[:n] - base.U).max() <= 1e-12 * np.abs(base.U).max()
    assert not gx.U[n:].any() and not gx.F[n:].any()


def test_inverted_element_reports_its_cell():
    mo = O.Mesh(O.Block(BOX, nx=3, ny=1, nz=1, cellshape=A.HEX8))
    mg = A.Mesh(A.Block(BOX, nx=3, ny=1, nz=1, cellshape=A.HEX8))
    mg.coords = np.ascontiguousarray(mo.coords)
    # turn the second element inside out: swap its bottom and top faces
    e = 1
    c = mg.conn[mg.conn_ptr[e]:mg.conn_ptr[e + 1]].copy()
    mg.conn[mg.conn_ptr[e]:mg.conn_ptr[e + 1]] = np.concatenate([c[4:], c[:4]])
    mo.elems[e].nodes = list(np.concatenate([c[4:], c[:4]]))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=200e3, nu=0.3))])
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=200e3, nu=0.3))])
    gm.configure_dofs([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0))])
    O.configure_dofs(om, [("x==0", O.SurfaceBC(ux=0, uy=0, uz=0))])
    with pytest.raises(RuntimeError) as eo:
        O.mount_K(om, int(gm.ndofs))
    with pytest.raises(A.AmrError) as eg:
        gm.dev.assemble_K()
    assert eg.value.code == -3
    assert "Negative Jacobian determinant in cell 2" in str(eo.value)
    assert "Negative Jacobian determinant in cell 2" in eg.value.msg


def test_nan_load_fails_the_stage():
    om, gm = _pair()
    nan = float("nan")
    ro, rg = _run(om, gm, lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", M.NodeBC(fz=nan))])
    assert not ro[0] and not rg[0]


def _desc(**over):
    mesh = A.Mesh(A.Block(BOX, nx=2, ny=1, nz=1, cellshape=A.HEX8))
    ne = len(mesh.shape)
    args = dict(ndim=3, stressmodel=0, thickness=1.0, coords=mesh.coords, shape=mesh.shape.copy(),
                nips=np.zeros(ne, dtype=np.int32), conn_ptr=mesh.conn_ptr.copy(), conn=mesh.conn.copy(),
                mat_type=np.zeros(ne, dtype=np.int32), mat_params=np.tile([200e3, 0.3, 0, 0, 0, 0, 0, 0], (ne, 1)))
    args.update(over)
    return args


@pytest.mark.parametrize("case, code, words", [
    ("node out of range", -1, "node index out of range"),
    ("wrong node count", -1, "wrong node count"),
    ("bad quadrature", -1, "integration points"),
    ("E not positive", -1, "E > 0"),
    ("nu at 0.5", -1, "nu < 0.5"),
    ("plane strain in 3-D", -1, "d3 stress model"),
    ("unknown material", -10, "material"),
    ("no elements", -1, "empty model"),
])
def test_bad_descriptions_are_refused(case, code, words):
    d = _desc()
    if case == "node out of range":
        d["conn"][3] = len(d["coords"])
    elif case == "wrong node count":
        d["conn_ptr"] = d["conn_ptr"].copy()
        d["conn_ptr"][1] -= 1
    elif case == "bad quadrature":
        d["nips"][0] = 5
    elif case == "E not positive":
        d["mat_params"][1, 0] = 0.0
    elif case == "nu at 0.5":
        d["mat_params"][0, 1] = 0.5
    elif case == "plane strain in 3-D":
        d["stressmodel"] = 1
    elif case == "unknown material":
        d["mat_type"][0] = 7
    elif case == "no elements":
        d = _desc(shape=d["shape"][:0], nips=d["nips"][:0], conn_ptr=d["conn_ptr"][:1], conn=d["conn"][:0],
                  mat_type=d["mat_type"][:0], mat_params=d["mat_params"][:0])
    with pytest.raises(A.AmrError) as e:
        L.DeviceModel(d["ndim"], d["stressmodel"], d["thickness"], d["coords"], d["shape"], d["nips"], d["conn_ptr"],
                      d["conn"], d["mat_type"], d["mat_params"])
    assert e.value.code == code
    assert words in e.value.msg


def test_call_order_and_dof_errors():
    d = _desc()
    dev = L.DeviceModel(d["ndim"], d["stressmodel"], d["thickness"], d["coords"], d["shape"], d["nips"],
                        d["conn_ptr"], d["conn"], d["mat_type"], d["mat_params"])
    with pytest.raises(A.AmrError) as e:
        dev.assemble_K()  # no DOFs yet
    assert e.value.code == -1 and "amr_set_dofs" in e.value.msg
    nn = len(d["coords"])
    eq = np.arange(3 * nn, dtype=np.int64).reshape(nn, 3)
    with pytest.raises(A.AmrError) as e:
        dev.set_dofs(eq, 3 * nn, 3 * nn + 1)  # nu > ndofs
    assert e.value.code == -1
    dev.set_dofs(eq, 3 * nn, 3 * nn - 12)
    with pytest.raises(A.AmrError) as e:
        dev.solve(np.zeros(3 * nn), np.zeros(3 * nn))  # K not assembled
    assert e.value.code == -1 and "assembled" in e.value.msg
    p = L.default_stage_params(maxits=0)
    rc, U, F, st = dev.stage_run(np.zeros(3 * nn), np.zeros(3 * nn), p)
    assert rc == -1
