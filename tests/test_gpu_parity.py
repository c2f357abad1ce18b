"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances (stated per quantity):
  * sparsity pattern of K (colptr/rowval in the reference CSC layout): bit-exact;
  * K values: |K_gpu - K_oracle| <= 1e-12 * max|K| (FP64 element integration in a
    different operation order);
  * internal forces / IP states: relative 1e-10 of their scale;
  * displacements and reactions of a solve with the 1e-8 relative-residual
    mixed-precision solver: relative 1e-6 of max|U| (cond(K) amplifies the residual);
  * staged Newton results: the reference test tolerances.
"""
import numpy as np
import pytest

import oracle as O
import amaru_gpu as A

pytestmark = pytest.mark.gpu

SHAPES_3D = [A.HEX8, A.HEX20, A.TET10, A.TET4]
SHAPES_2D = [A.QUAD8, A.QUAD4, A.QUAD9, A.TRI6, A.TRI3]


def _bc(api, kind, conds):
    return {"node": api.NodeBC, "surface": api.SurfaceBC, "edge": api.EdgeBC, "body": api.BodyC}[kind](**conds)


def _models(shape, n, box, mat, bcs, stressmodel="d3", thickness=1.0, nips=0, E=None):
    """The same problem for the oracle and the GPU library."""
    bo = O.Block(box, nx=n[0], ny=n[1], nz=n[2] if len(n) > 2 else 0, cellshape=shape)
    bg = A.Block(box, nx=n[0], ny=n[1], nz=n[2] if len(n) > 2 else 0, cellshape=shape)
    mo, mg = O.Mesh(bo), A.Mesh(bg)
    # identical inputs: the two meshers agree on numbering and to 1 ulp on coordinates (tested in
    # test_host.py); the bitwise comparisons below need the very same coordinates
    assert (mg.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    mg.coords = np.ascontiguousarray(mo.coords)
    kind, params = mat
    om = O.FEModel(mo, [("all", getattr(O, kind)(**params))], stressmodel=stressmodel, thickness=thickness,
                   nips=nips, elem_E=E)
    gm = A.FEModel(mg, [("all", getattr(A, kind)(**params))], A.MechContext(stressmodel=stressmodel),
                   thickness=thickness, nips=nips, E=E)
    ob = [(f, _bc(O, k, c)) for f, k, c in bcs]
    gb = [(f, _bc(A, k, c)) for f, k, c in bcs]
    return om, gm, ob, gb


CASES = [
    (A.HEX8, (4, 2, 2), [[0, 0, 0], [1.0, 0.2, 0.2]]),
    (A.HEX20, (3, 2, 2), [[0, 0, 0], [1.0, 0.4, 0.4]]),
    (A.TET10, (2, 2, 2), [[0, 0, 0], [1.0, 0.5, 0.5]]),
    (A.TET4, (3, 2, 2), [[0, 0, 0], [1.0, 0.5, 0.5]]),
    (A.QUAD8, (4, 3), [[0, 0], [1.0, 0.5]]),
    (A.QUAD4, (4, 3), [[0, 0], [1.0, 0.5]]),
    (A.QUAD9, (3, 3), [[0, 0], [1.0, 0.5]]),
    (A.TRI6, (3, 2), [[0, 0], [1.0, 0.5]]),
    (A.TRI3, (3, 2), [[0, 0], [1.0, 0.5]]),
]
BCS_3D = [("x==0", "surface", dict(ux=0, uy=0, uz=0)), ("x==1", "surface", dict(tz=-1.0))]
BCS_2D = [("x==0", "surface", dict(ux=0, uy=0)), ("x==1", "surface", dict(ty=-1.0))]


@pytest.mark.parametrize("shape,n,box", CASES)
def test_K_pattern_bit_exact_and_values(shape, n, box):
    """Reference-order assembly: colptr/rowval and every value bitwise equal to the oracle's mount_K."""
    bcs = BCS_3D if len(n) == 3 else BCS_2D
    om, gm, ob, gb = _models(shape, n, box, ("LinearElastic", dict(E=200e3, nu=0.3)), bcs)
    dofs, nu, _ = O.configure_dofs(om, ob)
    gm.configure_dofs(gb)
    assert (gm.eq_id == om.eq_id).all() and gm.nu == nu
    Ko = O.mount_K(om, len(dofs))
    Kg = gm.mount_K(reference_order=True)
    assert (Kg.indptr == Ko.indptr).all(), "colptr differs"
    assert (Kg.indices == Ko.indices).all(), "rowval differs"
    assert np.array_equal(Kg.data, Ko.data), "values differ (max %g)" % np.abs(Kg.data - Ko.data).max()


def _fragile_positions(om, ndofs, rel=1e-9):
    """Positions of K whose element contributions are all below rel * max|Ke|: whether they are
    stored depends only on rounding residues of mathematically-zero entries."""
    robust, seen = set(), set()
    for e in range(len(om.shape)):
        K, mp = om.elem_stiffness(e)
        big = np.abs(K) >= rel * np.abs(K).max()
        ii, jj = np.nonzero(np.ones_like(big))
        for i, j, b in zip(ii, jj, big[ii, jj]):
            p = (int(mp[i]), int(mp[j]))
            seen.add(p)
            if b:
                robust.add(p)
    return seen - robust


@pytest.mark.parametrize("shape,n,box", CASES)
def test_K_fast_assembly(shape, n, box):
    """Fast (pair-tensor, FMA) assembly of the Newton loop: values within 1e-12 max|K|; stored pattern equal
    to the reference's on every position that has a non-negligible contribution."""
    bcs = BCS_3D if len(n) == 3 else BCS_2D
    om, gm, ob, gb = _models(shape, n, box, ("LinearElastic", dict(E=200e3, nu=0.3)), bcs)
    dofs, nu, _ = O.configure_dofs(om, ob)
    gm.configure_dofs(gb)
    Ko = O.mount_K(om, len(dofs)).tocoo()
    Kg = gm.mount_K(reference_order=False).tocoo()
    fragile = _fragile_positions(om, len(dofs))
    po = set(zip(Ko.row.tolist(), Ko.col.tolist())) - fragile
    pg = set(zip(Kg.row.tolist(), Kg.col.tolist())) - fragile
    assert po == pg
    d = (Kg.tocsr() - Ko.tocsr()).tocoo()
    assert np.abs(d.data).max(initial=0.0) <= 1e-12 * np.abs(Ko.data).max()


def test_K_assembly_is_deterministic():
    om, gm, ob, gb = _models(A.HEX20, (3, 2, 2), [[0, 0, 0], [1, 0.4, 0.4]], ("LinearElastic", dict(E=1.0, nu=0.2)),
                             BCS_3D)
    gm.configure_dofs(gb)
    K1 = gm.mount_K().data.copy()
    K2 = gm.mount_K().data.copy()
    assert np.array_equal(K1, K2)


@pytest.mark.parametrize("mat", [("LinearElastic", dict(E=200e3, nu=0.3)),
                                 ("VonMises", dict(E=200e3, nu=0.3, fy=50.0, H=1e3)),
                                 ("DruckerPrager", dict(E=100.0, nu=0.25, alpha=0.05, kappa=0.1, H=1.0))])
@pytest.mark.parametrize("shape,n,box", [CASES[0], CASES[1], CASES[2], CASES[4]])
def test_update_state_and_tangent(mat, shape, n, box):
    """update_state! (internal forces, IP states) and the plastic tangent in K after it."""
    bcs = BCS_3D if len(n) == 3 else BCS_2D
    om, gm, ob, gb = _models(shape, n, box, mat, bcs)
    dofs, nu, _ = O.configure_dofs(om, ob)
    gm.configure_dofs(gb)
    rng = np.random.default_rng(7)
    amp = 2e-3 if mat[0] != "DruckerPrager" else 2e-2
    dU = rng.uniform(-amp, amp, len(dofs))
    Fo, msg = O.update_state(om, dU)
    assert msg is None
    Fg = gm.update_state(dU)
    assert np.abs(Fg - Fo).max() <= 1e-10 * max(np.abs(Fo).max(), 1e-300)
    so = om.state
    sg = gm.state()
    for f in range(14):
        sc = max(np.abs(so[:, f]).max(), 1e-30)
        assert np.abs(sg[:, f] - so[:, f]).max() <= 1e-9 * sc + 1e-15, "state field %d" % f
    if mat[0] != "LinearElastic":
        assert (so[:, 13] > 0).any(), "case must yield"
    # tangent stiffness at the trial state (IP states agree to rounding, so the pattern is compared on the
    # positions with a non-negligible contribution)
    Ko = O.mount_K(om, len(dofs)).tocoo()
    Kg = gm.mount_K().tocoo()
    fragile = _fragile_positions(om, len(dofs))
    assert set(zip(Ko.row.tolist(), Ko.col.tolist())) - fragile == set(zip(Kg.row.tolist(), Kg.col.tolist())) - fragile
    d = (Kg.tocsr() - Ko.tocsr()).tocoo()
    assert np.abs(d.data).max(initial=0.0) <= 1e-10 * np.abs(Ko.data).max()


SOLVERS = {"mixed": A.SOLVER_MIXED, "fp64": A.SOLVER_FP64, "amg": A.SOLVER_AMG, "amg_fp64": A.SOLVER_AMG_FP64}


@pytest.mark.parametrize("solver", ["mixed", "fp64", "amg", "amg_fp64"])
@pytest.mark.parametrize("shape,n,box", [CASES[0], CASES[1], CASES[2], CASES[4], CASES[5]])
def test_solve_system(solver, shape, n, box):
    """solve_system! with prescribed nonzero values: U1 and reactions F2 vs the direct solve, for the
    mixed-precision solvers and their all-FP64 comparators (the same method in FP64)."""
    bcs = BCS_3D if len(n) == 3 else BCS_2D
    om, gm, ob, gb = _models(shape, n, box, ("LinearElastic", dict(E=200e3, nu=0.3)), bcs)
    dofs, nu, setup = O.configure_dofs(om, ob)
    gm.configure_dofs(gb)
    Uo, Fo = O.get_bc_vals(om, setup, len(dofs))
    Ug, Fg = gm.get_bc_vals(gm.configure_dofs(gb))
    np.testing.assert_allclose(Fg, Fo, rtol=0, atol=1e-12 * np.abs(Fo).max())
    rng = np.random.default_rng(3)
    Uo[nu:] = rng.uniform(-1e-4, 1e-4, len(dofs) - nu)  # prescribed displacements
    Ug = Uo.copy()
    Fg = Fo.copy()
    K = O.mount_K(om, len(dofs))
    assert O.solve_system(K, Uo, Fo, nu) is None
    gm.mount_K()
    st = gm.solve_system(Ug, Fg, method=SOLVERS[solver], rtol=1e-10)
    assert st.rel_residual <= 1e-10
    sc = np.abs(Uo[:nu]).max()
    assert np.abs(Ug[:nu] - Uo[:nu]).max() <= 1e-6 * sc
    fs = np.abs(Fo[nu:]).max()
    assert np.abs(Fg[nu:] - Fo[nu:]).max() <= 1e-6 * fs


@pytest.mark.parametrize("solver", ["fp64", "amg_fp64"])
def test_fp64_comparator_matches_its_mixed_method(solver):
    """The all-FP64 comparators solve the system the mixed solvers solve: the same solution to the
    tolerance, a bitwise repeatable result, no more iterations than the mixed method, and timed
    kernels (the FP64 SpMV / cycle residual) that run on the current K."""
    om, gm, ob, gb = _models(A.HEX20, (8, 3, 3), [[0, 0, 0], [4, 1, 1]], ("LinearElastic", dict(E=30e3, nu=0.2)),
                             [("z==0", "surface", dict(ux=0, uy=0, uz=0)), ("z==1", "surface", dict(tz=-1.0))])
    U, F = gm.get_bc_vals(gm.configure_dofs(gb))
    gm.mount_K()
    mixed = "mixed" if solver == "fp64" else "amg"
    Um, Fm = U.copy(), F.copy()
    sm = gm.solve_system(Um, Fm, method=SOLVERS[mixed], rtol=1e-10)
    U1, F1 = U.copy(), F.copy()
    s1 = gm.solve_system(U1, F1, method=SOLVERS[solver], rtol=1e-10)
    U2, F2 = U.copy(), F.copy()
    gm.solve_system(U2, F2, method=SOLVERS[solver], rtol=1e-10)
    nu = gm.nu
    assert s1.rel_residual <= 1e-10 and sm.rel_residual <= 1e-10
    assert np.array_equal(U1, U2) and np.array_equal(F1, F2)
    assert np.abs(U1[:nu] - Um[:nu]).max() <= 1e-7 * np.abs(Um[:nu]).max()
    assert np.abs(F1[nu:] - Fm[nu:]).max() <= 1e-7 * np.abs(Fm[nu:]).max()
    assert s1.iterations <= 1.1 * sm.iterations + 3  # FP64 vectors never need more iterations
    kernel = A._lib.KERNEL_SPMV64 if solver == "fp64" else A._lib.KERNEL_AMG_RESIDUAL64
    t, nbytes = gm.dev.time_kernel(kernel, 3)
    assert t > 0 and nbytes > 0


def test_fp64_fma_peak_is_measured():
    t64 = A._lib.measure_peak(A._lib.PEAK_FP64_FMA)
    t32 = A._lib.measure_peak(A._lib.PEAK_FP32_FMA)
    assert 0.1 < t64 < t32 < 1000.0


def test_solver_reaches_1e8_and_is_reproducible():
    om, gm, ob, gb = _models(A.HEX20, (6, 3, 3), [[0, 0, 0], [3, 1, 1]], ("LinearElastic", dict(E=30e3, nu=0.2)),
                             [("z==0", "surface", dict(ux=0, uy=0, uz=0)), ("z==1", "surface", dict(tz=-1.0))])
    setup = gm.configure_dofs(gb)
    U, F = gm.get_bc_vals(setup)
    gm.mount_K()
    U1, F1 = U.copy(), F.copy()
    s1 = gm.solve_system(U1, F1, rtol=1e-8)
    U2, F2 = U.copy(), F.copy()
    gm.solve_system(U2, F2, rtol=1e-8)
    assert s1.rel_residual <= 1e-8
    assert np.array_equal(U1, U2) and np.array_equal(F1, F2)


# ---- known-answer tests of the reference, through the GPU staged solver
def _solve_both(om, gm, ob, gb, **kw):
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(ob, **kw.pop("stage", {}))
    ag.addstage(gb, **kw.pop("stage_g", {}))
    return ao, ag


@pytest.mark.parametrize("case,expected", [
    (("z==1", "node", dict(fz=1)), [0, 0, 0, 0, 4.0, 4.0, 4.0, 4.0]),
    (("y==1 && z==1", "edge", dict(qy=2)), [0, 0, 0, 0, 3.32088, 3.1998, -4.6002, -4.32047]),
    (("x==1", "surface", dict(tx="3*z")), [0, 0, 0, 0, 1.51044, -2.4501, 1.4499, -2.31023]),
    (("x>=0", "body", dict(wz=-1)), [0, 0, 0, 0, -0.5, -0.5, -0.5, -0.5]),
])
def test_gpu_elastic_hex8(case, expected):
    """test/mech/elem/elastic-hex8.jl through the GPU (atol 1e-5)."""
    base = [("x==0 && y==0 && z==0", "node", dict(ux=0, uy=0)), ("x==1 && y==0 && z==0", "node", dict(uy=0)),
            ("x==0 && y==1 && z==0", "node", dict(ux=0)), ("z==0", "node", dict(uz=0))]
    mesh = A.Mesh(A.Block([[0, 0, 0], [1, 1, 1]], nx=1, ny=1, nz=1, cellshape=A.HEX8))
    model = A.FEModel(mesh, [("all", A.MechSolid, A.LinearElastic, dict(E=1.0, nu=0.3))])
    ana = A.MechAnalysis(model)
    ana.addstage([(f, _bc(A, k, c)) for f, k, c in base + [case]], nouts=1)
    assert ana.solve()[0]
    np.testing.assert_allclose(model.U[:, 2], expected, atol=1e-5)


def test_gpu_elastic_quad4():
    """test/mech/elem/elastic-quad4.jl through the GPU (atol 1e-5)."""
    mesh = A.Mesh(A.Block([[0, 0], [1, 1]], nx=1, ny=1, cellshape=A.QUAD4))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=1.0, nu=0.25))], A.MechContext(stressmodel="planestrain"))
    ana = A.MechAnalysis(model)
    ana.addstage([("x==0.", A.SurfaceBC(ux=0.)), ("y==0.", A.SurfaceBC(uy=0)), ("y==1.", A.SurfaceBC(ty=-1.))])
    assert ana.solve()[0]
    dis = np.array([[0.0, 0.0], [0.3125, 0.0], [0.0, -9.3750e-01], [0.3125, -9.3750e-01]])
    np.testing.assert_allclose(model.U, dis, atol=1e-5)


@pytest.mark.parametrize("shape", SHAPES_3D)
def test_gpu_elastic_elems_3d(shape):
    """test/mech/elem/elastic-elems.jl 3-D part (atol 1e-2), and equal to the oracle to 1e-7."""
    mesh = A.Mesh(A.Block([[0, 0, 0], [1, 1, 1]], nx=2, ny=2, nz=2, cellshape=shape))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=100.0, nu=0.2))])
    ana = A.MechAnalysis(model)
    ana.addstage([("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==0 || x==1", A.SurfaceBC(ux=0)),
                  ("z==1", A.SurfaceBC(tz=-10.))])
    assert ana.solve()[0]
    top = mesh.select_nodes("z==1")[0]
    np.testing.assert_allclose(model.U[top, 1:], [-0.012, -0.095], atol=1e-2)
    mo = O.Mesh(O.Block([[0, 0, 0], [1, 1, 1]], nx=2, ny=2, nz=2, cellshape=shape))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=100.0, nu=0.2))])
    ao = O.MechAnalysis(om)
    ao.addstage([("z==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("x==0 || x==1", O.SurfaceBC(ux=0)),
                 ("z==1", O.SurfaceBC(tz=-10.))])
    assert ao.solve()[0]
    assert np.abs(model.U - om.U).max() <= 1e-7 * np.abs(om.U).max()
    assert np.abs(model.F - om.F).max() <= 1e-6 * np.abs(om.F).max()


@pytest.mark.parametrize("shape", SHAPES_2D)
def test_gpu_elastic_elems_2d(shape):
    """test/mech/elem/elastic-elems.jl 2-D part (atol 4e-2)."""
    mesh = A.Mesh(A.Block([[0, 0], [1, 1]], nx=2, ny=2, cellshape=shape))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=100.0, nu=0.2))])
    ana = A.MechAnalysis(model)
    ana.addstage([("y==0", A.SurfaceBC(ux=0, uy=0)), ("y==1", A.SurfaceBC(ty=-10.))])
    assert ana.solve()[0]
    top = mesh.select_nodes("y==1")[0]
    np.testing.assert_allclose(model.U[top], [-0.012, -0.095], atol=4e-2)


def test_gpu_vm_3d():
    """test/mech/mat/vm-3d.jl: HEX20 von Mises cantilever, autoinc; tip fz = -30 +- 0.7; and equal to the
    oracle's staged result within 2e-3 relative."""
    th, E, fy, H, nu = 0.05, 210e6, 240e3, 0.0, 0.3
    tip = "x==%r && y==1 && z==0" % (th / 2)
    bcs = [("y==0", "node", dict(uy=0)), ("y==0 && z==0", "node", dict(uz=0)),
           ("x==%r && y==0 && z==0" % (th / 2), "node", dict(ux=0)), (tip, "node", dict(uz=-0.08))]
    om, gm, ob, gb = _models(A.HEX20, (1, 50, 2), [[0, 0, -0.05], [0.05, 1.0, 0.05]],
                             ("VonMises", dict(E=E, nu=nu, fy=fy, H=H)), bcs)
    ag = A.MechAnalysis(gm)
    ag.addstage(gb, nincs=20, nouts=1)
    assert ag.solve(autoinc=True)[0]
    n = gm.mesh.select_nodes(tip)[0]
    assert abs(gm.F[n, 2] - (-30)) <= 0.7
    ao = O.MechAnalysis(om)
    ao.addstage(ob, nincs=20, nouts=1)
    assert ao.solve(autoinc=True)[0]
    assert abs(gm.F[n, 2] - om.F[n, 2]) <= 2e-3 * abs(om.F[n, 2])


def test_gpu_vm_2d_plane_stress():
    """test/mech/mat/vm-2d.jl: QUAD8 plane-stress von Mises; fy = -30 +- 0.4."""
    h, th, E, fy, H, nu = 0.1, 0.05, 210e6, 240e3, 0.0, 0.3
    mesh = A.Mesh(A.Block([[0, 0], [1.0, h]], nx=50, ny=2, cellshape=A.QUAD8))
    model = A.FEModel(mesh, [("all", A.VonMises(E=E, nu=nu, fy=fy, H=H))], A.MechContext(stressmodel="planestress"),
                      thickness=th)
    ana = A.MechAnalysis(model)
    ana.addstage([("x==0", A.NodeBC(ux=0)), ("x==0 && y==%r" % (h / 2), A.NodeBC(uy=0)),
                  ("x==1.0 && y==%r" % (h / 2), A.NodeBC(uy=-0.08))], nincs=30, nouts=1)
    assert ana.solve(autoinc=True)[0]
    n = mesh.select_nodes("y==%r && x==1" % (h / 2))[0]
    assert abs(model.F[n, 1] - (-30)) <= 0.4


def test_gpu_dp_two_stages():
    """test/mech/mat/dp.jl: HEX8 Drucker-Prager, load / unload stages -> success."""
    mesh = A.Mesh(A.Block([[0, 0, 0], [1, 1, 0.5]], nx=2, ny=2, nz=2))
    model = A.FEModel(mesh, [("all", A.DruckerPrager(E=100., nu=0.25, alpha=0.05, kappa=0.1))])
    ana = A.MechAnalysis(model)
    bcs = [("z==0.0", A.NodeBC(ux=0, uy=0, uz=0)), ("z==0.5", A.NodeBC(uz=-0.033)),
           ("x==0 || x==1.0", A.NodeBC(ux=0, uy=0)), ("y==0 || y==1.0", A.NodeBC(ux=0, uy=0))]
    ana.addstage(bcs, nincs=10)
    bcs2 = list(bcs)
    bcs2[1] = ("z==0.5", A.NodeBC(uz=+0.008))
    ana.addstage(bcs2, nincs=10)
    assert ana.solve(tol=1e-2, autoinc=True)[0]
    assert model.state()[:, 12].max() > 0


@pytest.mark.parametrize("n", [(20, 4, 4), (80, 4, 4)])
def test_config1_cantilever(n):
    """Linear HEX8 cantilever 1.0 x 0.2 x 0.2, E=200e3, nu=0.3, x=0 fixed, tz=-1 on x=1, one increment:
    displacements, reactions and the K pattern against the oracle."""
    bcs = [("x==0", "surface", dict(ux=0, uy=0, uz=0)), ("x==1", "surface", dict(tz=-1.0))]
    om, gm, ob, gb = _models(A.HEX8, n, [[0, 0, 0], [1.0, 0.2, 0.2]], ("LinearElastic", dict(E=200e3, nu=0.3)), bcs)
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(ob)
    ag.addstage(gb)
    assert ao.solve()[0] and ag.solve()[0]
    su = np.abs(om.U).max()
    assert np.abs(gm.U - om.U).max() <= 1e-6 * su
    sf = np.abs(om.F).max()
    assert np.abs(gm.F - om.F).max() <= 1e-6 * sf
    Ko = O.mount_K(om, ao.ndofs)
    Kg = gm.mount_K()
    assert (Kg.indptr == Ko.indptr).all() and (Kg.indices == Ko.indices).all()


@pytest.mark.parametrize("scheme", ["ME", "BE", "Ralston"])
def test_predictor_corrector_schemes(scheme):
    """mech_stage_solver! with the ME / BE / Ralston schemes (src/mech/mech-solver.jl:280-288, corrector
    with K = a1*K + a2*K2 at :338-349) on an elastoplastic HEX8 cantilever with autoinc: the same Newton
    iterations as the oracle and U, F within 1e-4 of max."""
    bcs = [("x==0", "surface", dict(ux=0, uy=0, uz=0)), ("x==1", "surface", dict(tz=-30.0))]
    om, gm, ob, gb = _models(A.HEX8, (6, 2, 2), [[0, 0, 0], [1.0, 0.2, 0.2]],
                             ("VonMises", dict(E=200e3, nu=0.3, fy=240.0, H=2e3)), bcs)
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(ob, nincs=6)
    ag.addstage(gb, nincs=6)
    assert ao.solve(scheme=scheme, autoinc=True)[0]
    assert ag.solve(scheme=scheme, autoinc=True)[0]
    assert gm.state()[:, 12].max() > 0
    assert ag.stats[0].iterations == len(ao.log)  # the same Newton path, iteration for iteration
    assert np.abs(gm.U - om.U).max() <= 1e-4 * np.abs(om.U).max()
    assert np.abs(gm.F - om.F).max() <= 1e-4 * np.abs(om.F).max()
