"""Axisymmetric analyses: stressmodel=:axisymmetric (src/mech/elem/mech-solid.jl:94-102 for the hoop row of B,
:143,180,223,260 for the thickness 2 pi r at the IP; src/mech/elem/distributed.jl:89,121,193 for the loads;
src/tools/tensors.jl:182-193 for the output keys).

The oracle's restatement is pinned on the reference's own axisymmetric test (test/mech/elem/axisymmetric.jl,
tests/test_oracle_golden.py) and here by two exact properties: a uniform radial expansion u_r = c r, u_z = 0 is
a rigid-free homogeneous strain (eps_rr = eps_tt = c) whose internal forces are those of the stress
(lambda 2c + 2 mu c) integrated over the ring, and the mass of a ring section sums to rho 2 pi r_c A.  The CUDA
path is compared with the oracle: the reference-order K bit for bit, the fast K to 1e-12, internal forces and
states to 1e-10, the mass matrix to 1e-12, von Mises stages and the recovered fields under their
axisymmetric keys.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

SHAPES = [O.QUAD4, O.QUAD8, O.TRI3, O.TRI6, O.QUAD9]
BOX = [[0.5, 0.0], [1.5, 1.0]]  # a ring section off the axis


def _oracle(shape, mat=None, n=(4, 4), box=BOX):
    mesh = O.Mesh(O.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    return O.FEModel(mesh, [("all", mat or O.LinearElastic(E=100.0, nu=0.2))], stressmodel="axisymmetric")


def test_oracle_radial_expansion_is_exact():
    """u_r = c r: eps = (c, 0, c, 0, 0, 0), sigma = (lambda 2c + 2 mu c, lambda 2c, lambda 2c + 2 mu c, ...); on
    the free faces of the ring the nodal forces balance, so the internal forces vanish at interior nodes and
    sum to zero in the axial direction."""
    E, nu, c = 100.0, 0.2, 1e-3
    for shape in SHAPES:
        om = _oracle(shape)
        dofs, nu_, _ = O.configure_dofs(om, [])
        dU = np.zeros(len(dofs))
        for i, (n, k) in enumerate(dofs):
            if k == 0:
                dU[i] = c * om.coords[n, 0]
        F, msg = O.update_state(om, dU)
        assert msg is None
        lam, mu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
        s = om.state
        np.testing.assert_allclose(s[:, 0], lam * 2 * c + 2 * mu * c, rtol=1e-12)
        np.testing.assert_allclose(s[:, 2], lam * 2 * c + 2 * mu * c, rtol=1e-12)
        np.testing.assert_allclose(s[:, 1], lam * 2 * c, rtol=1e-12)
        inner = [i for i, (n, k) in enumerate(dofs)
                 if 0.5 + 1e-9 < om.coords[n, 0] < 1.5 - 1e-9 and 1e-9 < om.coords[n, 1] < 1 - 1e-9]
        assert np.abs(F[inner]).max() <= 1e-12 * np.abs(F).max()
        assert abs(sum(F[i] for i, (n, k) in enumerate(dofs) if k == 1)) <= 1e-12 * np.abs(F).max()


def test_oracle_ring_mass():
    from oracle import dynamic as OD
    for shape in SHAPES:
        om = _oracle(shape)
        om.rho[:] = 3.0
        dofs, nu, _ = O.configure_dofs(om, [])
        M = OD.mount_M(om, len(dofs))
        # a ring of section 1 x 1 centred at r = 1: volume 2 pi
        assert abs(M.sum() / 2 - 3.0 * 2 * np.pi) <= 1e-12 * 3.0 * 2 * np.pi


def test_oracle_axisymmetric_output_keys():
    assert O.recovery.field_names(O.AXISYM, O.VON_MISES) == ["σrr", "σyy", "σtt", "σry", "σvm", "εrr", "εyy",
                                                             "εtt", "εry", "ep"]


def test_oracle_refuses_edge_loads():
    om = _oracle(O.QUAD4)
    dofs, nu, setup = O.configure_dofs(om, [("y==1", O.EdgeBC(qy=-1.0))])
    with pytest.raises(ValueError, match="axisymmetric"):
        O.get_bc_vals(om, setup, len(dofs))


# ---------------------------------------------------------------------------------------------- GPU


def _pair(shape, mat=("LinearElastic", dict(E=100.0, nu=0.2)), n=(4, 4), box=BOX):
    mo = O.Mesh(O.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    mg = A.Mesh(A.Block(box, nx=n[0], ny=n[1], cellshape=shape))
    assert (mg.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, [("all", getattr(O, mat[0])(**mat[1]))], stressmodel="axisymmetric")
    gm = A.FEModel(mg, [("all", getattr(A, mat[0])(**mat[1]))], A.MechContext(stressmodel="axisymmetric"))
    return om, gm


BCS = [("y==0", "uy"), ("x==0.5", "ux")]


def _bcs(api):
    return [("y==0", api.SurfaceBC(uy=0)), ("x==0.5", api.SurfaceBC(ux=0)), ("y==1", api.SurfaceBC(ty=-10.0))]


@pytest.mark.gpu
@pytest.mark.parametrize("shape", SHAPES)
def test_gpu_K_matches_the_oracle(shape):
    om, gm = _pair(shape)
    dofs, nu, _ = O.configure_dofs(om, _bcs(O))
    gm.configure_dofs(_bcs(A))
    assert (gm.eq_id == om.eq_id).all()
    Ko = O.mount_K(om, len(dofs))
    Kr = gm.mount_K(reference_order=True)
    assert (Kr.indptr == Ko.indptr).all() and (Kr.indices == Ko.indices).all()
    assert np.array_equal(Kr.data, Ko.data)
    Kf = gm.mount_K(reference_order=False)
    assert np.abs((Kf - Ko).toarray()).max() <= 1e-12 * np.abs(Ko.data).max()


@pytest.mark.gpu
@pytest.mark.parametrize("mat", [("LinearElastic", dict(E=100.0, nu=0.2)),
                                 ("VonMises", dict(E=100.0, nu=0.3, fy=0.05, H=5.0)),
                                 ("DruckerPrager", dict(E=100.0, nu=0.25, alpha=0.05, kappa=0.02, H=1.0))])
@pytest.mark.parametrize("shape", [O.QUAD8, O.TRI6])
def test_gpu_update_state_and_tangent(mat, shape):
    om, gm = _pair(shape, mat)
    dofs, nu, _ = O.configure_dofs(om, _bcs(O))
    gm.configure_dofs(_bcs(A))
    dU = np.random.default_rng(5).uniform(-2e-3, 2e-3, len(dofs))
    Fo, msg = O.update_state(om, dU)
    assert msg is None
    Fg = gm.update_state(dU)
    assert np.abs(Fg - Fo).max() <= 1e-10 * np.abs(Fo).max()
    sg = gm.state()
    for f in range(14):
        assert np.abs(sg[:, f] - om.state[:, f]).max() <= 1e-9 * max(np.abs(om.state[:, f]).max(), 1e-30) + 1e-15
    if mat[0] != "LinearElastic":
        assert (om.state[:, 13] > 0).any()
    Ko = O.mount_K(om, len(dofs))
    Kg = gm.mount_K(reference_order=False)
    assert np.abs((Kg - Ko).toarray()).max() <= 1e-10 * np.abs(Ko.data).max()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [O.TRI3, O.TRI6, O.QUAD4, O.QUAD8])
def test_gpu_reference_axisymmetric_block(shape):
    """test/mech/elem/axisymmetric.jl through the GPU stage solver: node (1, 1) at (0.02, -0.1) to 1e-3."""
    mesh = A.Mesh(A.Block([[0, 0], [1, 1]], nx=4, ny=4, cellshape=shape))
    gm = A.FEModel(mesh, [("all", A.LinearElastic(E=100.0, nu=0.2))], A.MechContext(stressmodel="axisymmetric"))
    ana = A.MechAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0)), ("y==0", A.SurfaceBC(uy=0)), ("y==1", A.SurfaceBC(ty=-10))])
    assert ana.solve()[0]
    n = mesh.select_nodes("x==1 && y==1")[0]
    np.testing.assert_allclose(gm.U[n, :2], [0.02, -0.1], atol=1e-3)


@pytest.mark.gpu
def test_gpu_von_mises_stage_and_output_match_the_oracle():
    mat = ("VonMises", dict(E=100.0, nu=0.3, fy=6.0, H=20.0))
    om, gm = _pair(O.QUAD8, mat, n=(6, 4))
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    for api, ana in ((O, ao), (A, ag)):
        ana.addstage([("y==0", api.SurfaceBC(uy=0)), ("x==0.5", api.SurfaceBC(ux=0)),
                      ("y==1 && x<=1", api.SurfaceBC(ty=-12.0)), ("all", api.BodyC(wy=-1.0))], nincs=4)
    assert ao.solve(tol=1e-6, autoinc=True)[0]
    assert ag.solve(tol=1e-6, autoinc=True, solver="fp64", linear_rtol=1e-12)[0]
    assert sum(1 for _ in ao.log) == sum(1 for _ in ag.log)
    assert np.abs(gm.U - om.U).max() <= 1e-7 * np.abs(om.U).max()
    assert np.abs(gm.F - om.F).max() <= 1e-7 * np.abs(om.F).max()
    assert gm.state()[:, 12].max() > 0
    om.state[:] = gm.state()
    Vo, no = O.nodal_patch_recovery(om)
    Vg, ng = gm.nodal_patch_recovery()
    assert ng == no and ng[:5] == ["σrr", "σyy", "σtt", "σry", "σvm"]
    for j in range(len(no)):
        assert np.abs(Vg[:, j] - Vo[:, j]).max() <= 1e-9 * max(np.abs(Vo[:, j]).max(), 1e-300)
    # (the oracle's recovery ran on the GPU's states: the recovery itself is compared to 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [O.QUAD8, O.TRI6])
def test_gpu_mass_matches_the_oracle(shape):
    from oracle import dynamic as OD
    om, gm = _pair(shape)
    om.rho[:] = 2.5
    gm.rho[:] = 2.5
    dofs, nu, _ = O.configure_dofs(om, [])
    gm.configure_dofs([])
    Mo = OD.mount_M(om, len(dofs))
    gm.dev.set_density(gm.rho)
    gm.dev.assemble_M()
    Mg = gm.dev.M_csc()
    assert np.abs((Mg - Mo).toarray()).max() <= 1e-12 * np.abs(Mo.data).max()


@pytest.mark.gpu
def test_gpu_refuses_edge_loads():
    mesh = A.Mesh(A.Block(BOX, nx=2, ny=2, cellshape=A.QUAD4))
    gm = A.FEModel(mesh, [("all", A.LinearElastic(E=100.0, nu=0.2))], A.MechContext(stressmodel="axisymmetric"))
    ana = A.MechAnalysis(gm)
    ana.addstage([("y==0", A.SurfaceBC(uy=0)), ("y==1", A.EdgeBC(qy=-1.0))])
    with pytest.raises(A.AmrError, match="axisymmetric"):
        ana.solve()
