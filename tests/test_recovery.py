"""Nodal output recovery: nodal_patch_recovery (src/fe-model.jl:504-702) as
update_output_data! (:341-427) calls it.

The reference's tests hold no recovered values, so the oracle's restatement is
pinned by what a least-squares patch fit must reproduce exactly: IP fields that
are polynomials of the regression space (linear and bilinear in 3-D, quadratic in
2-D), in interior patches and in the boundary patches of one-element-thick
strips.  The CUDA path (amr_recover_nodal) is then compared with the oracle on the
same IP states: after elastic and elastoplastic solves, in 3-D, plane strain and
plane stress, with mixed materials (fields that only some elements carry), on a
jittered TET10 slope, with rank-deficient boundary patches and with unused nodes;
and at the HEX20 100x40x40 size through the polynomial property.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from oracle.recovery import SR2


def _plant(state, ipx, ndim):
    """Writes polynomial fields into the IP states: sigma_xx linear, eps_xy bilinear (3-D) or quadratic (2-D)."""
    x, y, z = ipx[:, 0], ipx[:, 1], ipx[:, 2]
    state[:, 0] = 3.0 + 2.0 * x - y + (0.5 * z if ndim == 3 else 0.0)
    if ndim == 3:
        state[:, 11] = (x * y - 0.25 * y * z + 1.5) * SR2
    else:
        state[:, 11] = (x * x - 0.5 * x * y + 2.0 * y * y - y) * SR2
    state[:, 12] = 0.0


def _expected(coords, ndim):
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    sxx = 3.0 + 2.0 * x - y + (0.5 * z if ndim == 3 else 0.0)
    exy = (x * y - 0.25 * y * z + 1.5) if ndim == 3 else (x * x - 0.5 * x * y + 2.0 * y * y - y)
    return sxx, exy


def _oracle_model(box, n, shape, **kw):
    if len(n) == 3:
        mesh = O.Mesh(O.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
    else:
        mesh = O.Mesh(O.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    return O.FEModel(mesh, [("all", O.LinearElastic(E=200e3, nu=0.3))], **kw)


@pytest.mark.parametrize("shape, n, nips", [(A.HEX8, (4, 3, 3), 0), (A.HEX20, (3, 2, 2), 27), (A.TET10, (2, 2, 2), 0),
                                            (A.QUAD8, (5, 4), 0), (A.QUAD4, (5, 4), 0), (A.QUAD8, (6, 1), 9)])
def test_oracle_reproduces_polynomial_fields(shape, n, nips):
    """(A one-element strip needs three rows of IPs: with two, its boundary patches cannot determine the
    quadratic terms, and the pseudo-inverse's minimum-norm fit is not the field.)"""
    box = [[0, 0, 0], [1.5, 1.0, 0.8]] if len(n) == 3 else [[0, 0], [1.5, 1.0]]
    om = _oracle_model(box, n, shape, stressmodel="d3" if len(n) == 3 else "planestrain", nips=nips)
    ipx = O.ip_coords(om)
    _plant(om.state, ipx, om.ndim)
    V, names = O.nodal_patch_recovery(om, ipx)
    sxx, exy = _expected(om.coords, om.ndim)
    assert np.abs(V[:, names.index("σxx")] - sxx).max() < 1e-11
    assert np.abs(V[:, names.index("εxy")] - exy).max() < 1e-11


def test_oracle_field_order_follows_the_first_element():
    mesh = O.Mesh(O.Block([[0, 0, 0], [1.0, 1.0, 1.0]], nx=2, ny=2, nz=2, cellshape=O.HEX8))
    om = O.FEModel(mesh, [("all", O.DruckerPrager(E=1e4, nu=0.25, alpha=0.1, kappa=1.0, H=0.0)),
                          ("x<=0.5", O.VonMises(E=1e4, nu=0.25, fy=1.0, H=0.0))])
    _, names = O.nodal_patch_recovery(om)
    assert names == O.recovery.BASE_3D + ["ep", "epa", "j1", "srj2d"]


# ---------------------------------------------------------------------------------------------- GPU


def _pair(box, n, shape, mats_o, mats_g, ctx="d3", **kw):
    if len(n) == 3:
        mo = O.Mesh(O.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
        mg = A.Mesh(A.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
    else:
        mo = O.Mesh(O.Block(box, nx=n[0], ny=n[1], cellshape=shape))
        mg = A.Mesh(A.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, mats_o, stressmodel=ctx, **kw)
    gm = A.FEModel(mg, mats_g, A.MechContext(stressmodel=ctx), **kw)
    return om, gm


def _compare(om, gm, tol=1e-9):
    """GPU recovery against the oracle's on the GPU's IP states."""
    om.state[:] = gm.state()
    Vo, no = O.nodal_patch_recovery(om)
    Vg, ng = gm.nodal_patch_recovery()
    assert ng == no
    for j, k in enumerate(no):
        scale = max(np.abs(Vo[:, j]).max(), 1e-300)
        err = np.abs(Vg[:, j] - Vo[:, j]).max() / scale
        assert err <= tol, (k, err)
    return Vg, ng


@pytest.mark.gpu
def test_gpu_recovery_after_an_elastic_hex20_solve():
    box = [[0, 0, 0], [3.0, 1.0, 1.0]]
    E = np.exp(np.random.default_rng(7).normal(np.log(30e3), 0.3, 6 * 2 * 2))
    om, gm = _pair(box, (6, 2, 2), A.HEX20, [("all", O.LinearElastic(E=30e3, nu=0.2))],
                   [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27)
    gm.mat_params[:, 0] = E
    gm.dev.set_youngs(E)
    ag = A.MechAnalysis(gm)
    ag.addstage([("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("z==1", A.SurfaceBC(tz=-1.0))])
    assert ag.solve()[0]
    V, names = _compare(om, gm)
    assert names == O.recovery.BASE_3D
    # the model's output data carries the same columns
    node, elem = gm.update_output_data()
    assert np.array_equal(node["σvm"], V[:, names.index("σvm")])
    assert np.array_equal(node["U"][:, 2], gm.U[:, 2]) and (elem["cell-type"] == 25).all()


@pytest.mark.gpu
@pytest.mark.parametrize("ctx", ["planestrain", "planestress"])
def test_gpu_recovery_after_a_plastic_quad8_stage(ctx):
    box = [[0, 0], [2.0, 0.5]]
    mat = dict(E=200e3, nu=0.3, fy=240.0, H=2e3)
    om, gm = _pair(box, (12, 4), A.QUAD8, [("all", O.VonMises(**mat))], [("all", A.VonMises(**mat))], ctx=ctx)
    ag = A.MechAnalysis(gm)
    ag.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(ty=-20.0))], nincs=4)
    assert ag.solve(autoinc=True)[0]
    assert gm.state()[:, 12].max() > 0
    _, names = _compare(om, gm)
    assert names == O.recovery.field_names(O.PLANESTRESS if ctx == "planestress" else O.PLANESTRAIN, O.VON_MISES)


@pytest.mark.gpu
def test_gpu_recovery_with_mixed_materials():
    """Fields only some elements carry (ep on VonMises, epa/j1/srj2d on DruckerPrager) are fitted on the
    elements of the patch that carry them."""
    box = [[0, 0, 0], [2.0, 1.0, 1.0]]
    dp = dict(E=1e4, nu=0.25, alpha=0.05, kappa=5.0, H=50.0)
    vm = dict(E=1e4, nu=0.25, fy=8.0, H=100.0)
    om, gm = _pair(box, (6, 3, 3), A.HEX8, [("all", O.DruckerPrager(**dp)), ("x<=1", O.VonMises(**vm))],
                   [("all", A.DruckerPrager(**dp)), ("x<=1", A.VonMises(**vm))])
    ag = A.MechAnalysis(gm)
    ag.addstage([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==2", A.SurfaceBC(tz=-0.8))], nincs=4)
    assert ag.solve(autoinc=True)[0]
    _, names = _compare(om, gm)
    assert names[-4:] == ["ep", "epa", "j1", "srj2d"]


@pytest.mark.gpu
def test_gpu_recovery_on_the_jittered_tet10_slope():
    from amaru_gpu import workloads as W
    g = W.SLOPE
    n = (10, 2, 4)
    mo = O.Mesh(O.Block([[0, 0, 0], [g["L"], g["W"], g["H"]]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    mg = A.Mesh(A.Block([[0, 0, 0], [g["L"], g["W"], g["H"]]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    mg.coords = W.slope_coords(mo.coords, mg.elem_nodes(), W.boundary_nodes(mg), 4, *n, seed=0xC3)
    mo.coords = mg.coords.copy()
    mat = dict(E=50e3, nu=0.3, fy=100.0, H=1e3)
    om = O.FEModel(mo, [("all", O.VonMises(**mat))])
    gm = A.FEModel(mg, [("all", A.VonMises(**mat))])
    ag = A.MechAnalysis(gm)
    ag.addstage(W.slope_bcs(A, 200.0), nincs=3)
    assert ag.solve(tol=1e-6)[0]
    _compare(om, gm)


@pytest.mark.gpu
def test_gpu_recovery_on_strips_with_boundary_patches_and_an_unused_node():
    """One element thick: every node is on the boundary, so the patches are the reference's fallback
    boundary patches; QUAD4 strips give rank-deficient patches (two rows of IPs under a quadratic basis),
    solved by the pseudo-inverse path."""
    for shape, nips in ((A.QUAD8, 9), (A.QUAD4, 0)):
        mo = O.Mesh(O.Block([[0, 0], [3.0, 0.5]], nx=6, ny=1, cellshape=shape))
        mg = A.Mesh(A.Block([[0, 0], [3.0, 0.5]], nx=6, ny=1, cellshape=shape))
        mg.coords = np.vstack([mo.coords, [[9.0, 9.0, 0.0]]])
        om = O.FEModel(mo, [("all", O.LinearElastic(E=200e3, nu=0.3))], stressmodel="planestrain", nips=nips)
        gm = A.FEModel(mg, [("all", A.LinearElastic(E=200e3, nu=0.3))], A.MechContext(stressmodel="planestrain"),
                       nips=nips)
        ag = A.MechAnalysis(gm)
        ag.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==3", A.SurfaceBC(ty=-1.0))])
        assert ag.solve()[0]
        n = len(mo.coords)
        om.state[:] = gm.state()
        Vo, no = O.nodal_patch_recovery(om)
        Vg, ng = gm.nodal_patch_recovery()
        assert ng == no and not Vg[n:].any()
        for j in range(len(no)):
            scale = np.abs(Vo[:, j]).max()
            assert np.abs(Vg[:n, j] - Vo[:, j]).max() <= 1e-8 * scale, no[j]
        t, flops, nsvd = gm.dev.time_recovery(1)
        assert (nsvd > 0) == (shape == A.QUAD4)


@pytest.mark.gpu
def test_gpu_recovery_reproduces_polynomial_fields_at_full_size():
    """HEX20 100x40x40 (669 161 nodes, 160 000 elements, 27 IPs): the recovered nodal values of planted
    linear / bilinear IP fields equal the fields at the nodes."""
    n = (100, 40, 40)
    mg = A.Mesh(A.Block([[0, 0, 0], [10.0, 4.0, 4.0]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX20))
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27)
    st = np.zeros((gm.dev.sizes()["nip_total"], 16))
    ipx = _ip_coords(gm)
    _plant(st, ipx, 3)
    gm.set_state(st)
    V, names = gm.nodal_patch_recovery()
    sxx, exy = _expected(mg.coords, 3)
    assert np.abs(V[:, names.index("σxx")] - sxx).max() < 1e-9
    assert np.abs(V[:, names.index("εxy")] - exy).max() < 1e-9
    assert np.abs(V[:, names.index("σyy")]).max() == 0.0


def _ip_coords(gm):
    """IP coordinates in the caller's element and IP order, vectorised over elements of one shape."""
    mesh = gm.mesh
    sh = int(mesh.shape[0])
    R, _ = O.quadrature(sh, int(gm.nips[0]))
    N = np.array([O.shape_func(sh, r) for r in R])  # nip x nen
    C = mesh.coords[mesh.elem_nodes()]              # ne x nen x 3
    return np.einsum("qa,ead->eqd", N, C).reshape(-1, 3)
