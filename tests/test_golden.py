"""Stored golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py from the oracle).

The CPU tests check that the oracle still reproduces every fixture:
  * K (colptr, rowval, nzval) bit for bit;
  * the other arrays to 1e-12 of their scale;
  * the frequencies to 1e-11, as the ARPACK iteration's last bits follow the host's BLAS;
  * the modes to 1e-9, up to sign and the span of equal frequencies.
The oracle's K is computed in C without FMA contraction, so the stored arrays hold on any IEEE host.

The GPU tests compare the CUDA path, through the C ABI, with the stored values.
Tolerances (stated per quantity):
  * K's pattern: bit-exact, in the reference CSC layout;
  * K's values: 1e-12 of max|K|;
  * U, F of a linear stage (mixed-precision solver to a 1e-8 relative residual): 1e-6 of their scale;
  * U, F of the plane-stress von Mises stage: 1e-5 of their scale. Each increment converges in the
    oracle's number of iterations, which is checked;
  * recovered nodal fields: 1e-8 of each field's scale;
  * natural frequencies: 1e-8 of the largest;
  * mode shapes: 1e-5, up to sign;
  * Newmark U, V, A, F: 1e-7 of their scale.
"""
import importlib.util
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def _close(a, b, tol):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(np.asarray(a) - b).max() <= tol * s


def _same_span(Va, Vb, w, tol):
    """Columns of Vb lie in the span of the columns of Va for each group of equal frequencies."""
    i = 0
    while i < len(w):
        j = i + 1
        while j < len(w) and abs(w[j] - w[i]) <= 1e-6 * w[i]:
            j += 1
        Q, _ = np.linalg.qr(Va[:, i:j])
        if np.abs(Vb[:, i:j] - Q @ (Q.T @ Vb[:, i:j])).max() > tol:
            return False
        i = j
    return True


# ---------------------------------------------------------------------------------------------- CPU


def _generator():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["c1_hex8", "tet10_k", "vm_planestress", "recovery", "modal_quad4", "dyn_solid"])
def test_oracle_reproduces_the_fixture(name):
    stored, now = _load(name), getattr(_generator(), name)()
    assert sorted(stored) == sorted(now)
    for k, v in stored.items():
        if k in ("colptr", "rowval", "nzval", "coords", "state", "names", "iterations"):
            assert np.array_equal(np.asarray(now[k]), v), k
        elif k == "modes":
            assert _same_span(v, now[k], stored["omega"], 1e-9)
        elif k == "omega":  # the ARPACK iteration's last bits follow the host's BLAS
            assert _close(now[k], v, 1e-11), k
        else:
            assert _close(now[k], v, 1e-12), k


def test_fixtures_are_what_they_claim():
    c1 = _load("c1_hex8")
    assert c1["coords"].shape == (21 * 5 * 5, 3) and len(c1["colptr"]) == 3 * 21 * 5 * 5 + 1
    # the tip load tz = -1 over the 0.2 x 0.2 face comes back as the reactions at x = 0
    fixed = np.abs(c1["coords"][:, 0]) < 1e-12
    assert abs(c1["F"][fixed, 2].sum() - 0.04) < 1e-9
    t10 = _load("tet10_k")
    ncol = np.diff(t10["colptr"])
    assert (ncol > 0).all() and np.all(np.diff(t10["rowval"][t10["colptr"][0]:t10["colptr"][1]]) > 0)
    md = _load("modal_quad4")
    assert (np.diff(md["omega"]) >= 0).all() and md["omega"][0] > 0
    rc = _load("recovery")
    assert rc["state"].shape == (12 * 27, 16) and list(rc["names"][:2]) == ["σxx", "σyy"]


# ---------------------------------------------------------------------------------------------- GPU


def _gpu_model(A, shape, n, box, mats, coords, ctx="d3", **kw):
    if len(n) == 3:
        mesh = A.Mesh(A.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
    else:
        mesh = A.Mesh(A.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    assert mesh.coords.shape == coords.shape
    mesh.coords = np.ascontiguousarray(coords)
    return mesh, A.FEModel(mesh, mats, A.MechContext(stressmodel=ctx), **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["c1_hex8", "tet10_k"])
def test_gpu_K_against_the_fixture(name):
    import amaru_gpu as A
    g = _load(name)
    if name == "c1_hex8":
        _, gm = _gpu_model(A, A.HEX8, (20, 4, 4), [[0, 0, 0], [1.0, 0.2, 0.2]],
                           [("all", A.LinearElastic(E=200e3, nu=0.3))], g["coords"])
        bcs = [("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", A.SurfaceBC(tz=-1.0))]
    else:
        _, gm = _gpu_model(A, A.TET10, (2, 2, 2), [[0, 0, 0], [1.0, 1.0, 1.0]],
                           [("all", A.LinearElastic(E=100.0, nu=0.25))], g["coords"])
        bcs = [("z==0", A.SurfaceBC(ux=0, uy=0, uz=0))]
    gm.configure_dofs(bcs)
    K = gm.mount_K(reference_order=True)
    assert np.array_equal(K.indptr, g["colptr"]), "colptr differs"
    assert np.array_equal(K.indices, g["rowval"]), "rowval differs"
    assert np.abs(K.data - g["nzval"]).max() <= 1e-12 * np.abs(g["nzval"]).max()
    if name == "c1_hex8":
        ana = A.MechAnalysis(gm)
        ana.addstage(bcs)
        assert ana.solve()[0]
        assert _close(gm.U, g["U"], 1e-6) and _close(gm.F, g["F"], 1e-6)


@pytest.mark.gpu
def test_gpu_plane_stress_von_mises_stage_against_the_fixture():
    import amaru_gpu as A
    g = _load("vm_planestress")
    _, gm = _gpu_model(A, A.QUAD8, (12, 4), [[0, 0], [2.0, 0.5]],
                       [("all", A.VonMises(E=200e3, nu=0.3, fy=240.0, H=2e3))], g["coords"], ctx="planestress")
    ana = A.MechAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(ty=-16.0))], nincs=8)
    assert ana.solve()[0]
    assert gm.state()[:, 12].max() > 0
    assert ana.stats[0].iterations == int(g["iterations"][0])
    assert _close(gm.U, g["U"], 1e-5) and _close(gm.F, g["F"], 1e-5)


@pytest.mark.gpu
def test_gpu_recovery_against_the_fixture():
    import amaru_gpu as A
    g = _load("recovery")
    _, gm = _gpu_model(A, A.HEX20, (3, 2, 2), [[0, 0, 0], [1.5, 1.0, 1.0]],
                       [("all", A.LinearElastic(E=30e3, nu=0.2))], g["coords"], nips=27)
    gm.set_state(g["state"])
    V, names = gm.nodal_patch_recovery()
    assert names == [str(s) for s in g["names"]]
    for j, k in enumerate(names):
        assert _close(V[:, j], g["V"][:, j], 1e-8), k


@pytest.mark.gpu
def test_gpu_modal_against_the_fixture():
    import amaru_gpu as A
    g = _load("modal_quad4")
    _, gm = _gpu_model(A, A.QUAD4, (4, 40), [[0, 0], [1.0, 10.0]],
                       [("all", A.LinearElastic(E=2e6, nu=0.2, rho=15.0))], g["coords"], ctx="planestrain")
    ana = A.ModalAnalysis(gm)
    ana.addstage([("y==0", A.NodeBC(ux=0, uy=0))])
    assert ana.solve(nmodes=6, tol=1e-8)[0]
    assert np.abs(ana.freqs - g["omega"]).max() <= 1e-8 * g["omega"].max()
    assert _same_span(g["modes"], ana.modes, g["omega"], 1e-5)


@pytest.mark.gpu
def test_gpu_newmark_stage_against_the_fixture():
    import amaru_gpu as A
    g = _load("dyn_solid")
    _, gm = _gpu_model(A, A.HEX8, (1, 10, 1), [[0, 0, 0], [0.2, 2.0, 0.2]],
                       [("all", A.LinearElastic(E=30e6, nu=0.2, rho=24.0))], g["coords"])
    ana = A.DynAnalysis(gm)
    ana.addstage([("y==0 && z==0", A.NodeBC(ux=0, uy=0, uz=0)), ("y==2 && z==0", A.NodeBC(uz=0)),
                  ("y==1 && z==0.2", A.NodeBC(fz=-10))], tspan=0.1, nincs=6, nouts=1)
    ok, msg = ana.solve(alpha=4.2038, beta=174.2803e-6, linear_rtol=1e-10)
    assert ok, msg
    for k in ("U", "V", "A", "F"):
        assert _close(getattr(gm, k), g[k], 1e-7), k
