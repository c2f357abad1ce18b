"""The aggregation-multigrid preconditioner (AMR_SOLVER_AMG): solve_system!
(src/solver.jl:5-79) to the same FP64 relative residual as the block-Jacobi path,
equal to the oracle's direct solve, in far fewer Krylov iterations; inside the
staged Newton loop with K reassembled every iteration; with unused nodes; bitwise
repeatable."""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from amaru_gpu import _lib as L

pytestmark = pytest.mark.gpu


def _hex20_block(n, seed=0xA11A):
    g = dict(box=[[0, 0, 0], [10.0, 4.0, 4.0]])
    mo = O.Mesh(O.Block(g["box"], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX20))
    mg = A.Mesh(A.Block(g["box"], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX20))
    mg.coords = np.ascontiguousarray(mo.coords)
    E = np.exp(np.random.default_rng(seed).normal(np.log(30e3), 0.3, len(mg.shape)))
    om = O.FEModel(mo, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27, elem_E=E)
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27, E=E)
    bcs = lambda M: [("z==0", M.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", M.SurfaceBC(tz=-1.0))]
    return om, gm, bcs


def _solve_both(gm, U, F, method, rtol=1e-10):
    U1, F1, st = gm.dev.solve(U, F, L.default_solve_opts(method=method, rtol=rtol))
    return U1, F1, st


def test_amg_solve_matches_the_oracle_in_few_iterations():
    om, gm, bcs = _hex20_block((12, 5, 5))
    dofs, nu, setup = O.configure_dofs(om, bcs(O))
    Uo, Fo = O.get_bc_vals(om, setup, len(dofs))
    K = O.mount_K(om, len(dofs))
    assert O.solve_system(K, Uo, Fo, nu) is None
    gs = gm.configure_dofs(bcs(A))
    U, F = gm.get_bc_vals(gs)
    gm.dev.assemble_K()
    Ua, Fa, sa = _solve_both(gm, U, F, L.SOLVER_AMG)
    Ub, Fb, sb = _solve_both(gm, U, F, L.SOLVER_MIXED)
    assert sa.rel_residual <= 1e-10 and sb.rel_residual <= 1e-10
    assert sa.iterations * 8 <= sb.iterations
    su, sf = np.abs(Uo).max(), np.abs(Fo[nu:]).max()
    assert np.abs(Ua[:nu] - Uo[:nu]).max() <= 1e-6 * su
    assert np.abs(Fa[nu:] - Fo[nu:]).max() <= 1e-6 * sf
    # bitwise repeatable
    Uc, Fc, _ = _solve_both(gm, U, F, L.SOLVER_AMG)
    assert np.array_equal(Ua, Uc) and np.array_equal(Fa, Fc)


def test_amg_in_2d_and_with_unused_nodes():
    mo = O.Mesh(O.Block([[0, 0], [4.0, 1.0]], nx=24, ny=8, cellshape=A.QUAD8))
    mg = A.Mesh(A.Block([[0, 0], [4.0, 1.0]], nx=24, ny=8, cellshape=A.QUAD8))
    mg.coords = np.vstack([mo.coords, [[9.0, 9.0, 0.0]]])  # one node no element uses
    om = O.FEModel(mo, [("all", O.LinearElastic(E=200e3, nu=0.3))], stressmodel="planestrain")
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=200e3, nu=0.3))], A.MechContext(stressmodel="planestrain"))
    bcs = lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0)), ("x==4", M.SurfaceBC(ty=-1.0))]
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(bcs(O))
    ag.addstage(bcs(A))
    assert ao.solve()[0] and ag.solve(solver="amg")[0]
    n = len(mo.coords)
    assert np.abs(gm.U[:n] - om.U).max() <= 1e-6 * np.abs(om.U).max()
    assert np.abs(gm.F[:n] - om.F).max() <= 1e-6 * np.abs(om.F).max()
    assert not gm.U[n:].any()


def test_amg_in_the_elastoplastic_newton_loop():
    bcs = [("x==0", "surface", dict(ux=0, uy=0, uz=0)), ("x==1", "surface", dict(tz=-30.0))]
    mo = O.Mesh(O.Block([[0, 0, 0], [1.0, 0.2, 0.2]], nx=16, ny=3, nz=3, cellshape=A.HEX8))
    mg = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.2, 0.2]], nx=16, ny=3, nz=3, cellshape=A.HEX8))
    mg.coords = np.ascontiguousarray(mo.coords)
    mat = dict(E=200e3, nu=0.3, fy=240.0, H=2e3)
    om = O.FEModel(mo, [("all", O.VonMises(**mat))])
    gm = A.FEModel(mg, [("all", A.VonMises(**mat))])
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage([("x==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", O.SurfaceBC(tz=-30.0))], nincs=6)
    ag.addstage([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", A.SurfaceBC(tz=-30.0))], nincs=6)
    assert ao.solve(autoinc=True)[0] and ag.solve(autoinc=True, solver="amg")[0]
    assert gm.state()[:, 12].max() > 0
    assert ag.stats[0].iterations == len(ao.log)
    assert np.abs(gm.U - om.U).max() <= 1e-6 * np.abs(om.U).max()


def test_amg_on_the_jittered_tet10_slope():
    """The slope workload (distorted TET10, rollers, gravity + surcharge): the multigrid stage equals the
    block-Jacobi stage to the solver tolerance."""
    from amaru_gpu import workloads as W
    g = W.SLOPE
    n = (20, 3, 8)
    out = []
    for solver in ("mixed", "amg"):
        mesh = A.Mesh(A.Block([[0, 0, 0], [g["L"], g["W"], g["H"]]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
        mesh.coords = W.slope_coords(mesh.coords, mesh.elem_nodes(), W.boundary_nodes(mesh), 4, *n, seed=0xC3)
        model = A.FEModel(mesh, [("all", A.VonMises(E=50e3, nu=0.3, fy=100.0, H=1e3))])
        ana = A.MechAnalysis(model)
        ana.addstage(W.slope_bcs(A, 200.0), nincs=5)
        assert ana.solve(tol=1e-6, solver=solver)[0]
        out.append((model.U.copy(), ana.stats[0]))
    (Um, sm), (Ua, sa) = out
    assert sa.iterations == sm.iterations and sa.krylov_iterations * 5 < sm.krylov_iterations
    assert np.abs(Ua - Um).max() <= 1e-6 * np.abs(Um).max()


@pytest.mark.parametrize("method", [L.SOLVER_AMG, L.SOLVER_AMG_FP64])
def test_smoothed_prolongators_cut_the_iterations(method):
    """Smoothed aggregation (the default) against the tentative prolongators on the lognormal-E HEX20 block:
    the same solution to the solve's tolerance in fewer Krylov iterations, bitwise repeatable, and equal to
    the oracle's direct solve."""
    om, gm, bcs = _hex20_block((16, 6, 6))
    dofs, nu, setup = O.configure_dofs(om, bcs(O))
    Uo, Fo = O.get_bc_vals(om, setup, len(dofs))
    assert O.solve_system(O.mount_K(om, len(dofs)), Uo, Fo, nu) is None
    gs = gm.configure_dofs(bcs(A))
    U, F = gm.get_bc_vals(gs)
    gm.dev.assemble_K()
    out = {}
    for smooth in (False, True):
        gm.dev.set_amg_smoothing(smooth)
        out[smooth] = _solve_both(gm, U, F, method)
    (Uu, Fu, su), (Us, Fs, ss) = out[False], out[True]
    assert su.rel_residual <= 1e-10 and ss.rel_residual <= 1e-10
    assert ss.iterations < su.iterations, (ss.iterations, su.iterations)
    scale = np.abs(Uo).max()
    assert np.abs(Us[:nu] - Uu[:nu]).max() <= 1e-7 * scale
    assert np.abs(Us[:nu] - Uo[:nu]).max() <= 1e-6 * scale
    assert np.abs(Fs[nu:] - Fo[nu:]).max() <= 1e-6 * np.abs(Fo[nu:]).max()
    Ur, Fr, _ = _solve_both(gm, U, F, method)
    assert np.array_equal(Us, Ur) and np.array_equal(Fs, Fr)


def test_smoothed_prolongators_in_2d_with_unused_nodes():
    mo = O.Mesh(O.Block([[0, 0], [4.0, 1.0]], nx=40, ny=10, cellshape=A.QUAD8))
    mg = A.Mesh(A.Block([[0, 0], [4.0, 1.0]], nx=40, ny=10, cellshape=A.QUAD8))
    mg.coords = np.vstack([mo.coords, [[9.0, 9.0, 0.0]]])  # one node no element uses
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=200e3, nu=0.3))], A.MechContext(stressmodel="planestrain"))
    gs = gm.configure_dofs([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==4", A.SurfaceBC(ty=-1.0))])
    U, F = gm.get_bc_vals(gs)
    gm.dev.assemble_K()
    its = {}
    for smooth in (False, True):
        gm.dev.set_amg_smoothing(smooth)
        Ux, Fx, st = _solve_both(gm, U, F, L.SOLVER_AMG)
        assert st.rel_residual <= 1e-10
        its[smooth] = (st.iterations, Ux)
    assert its[True][0] < its[False][0]
    assert np.abs(its[True][1] - its[False][1]).max() <= 1e-7 * np.abs(its[False][1]).max()
