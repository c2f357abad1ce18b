"""Nonlinear geomechanics: the plane-strain slope extruded along y on a jittered TET10
mesh, von Mises with linear hardening (E=50e3, nu=0.3, fy=100, H=1e3), gravity and a
crest surcharge ramped over 20 increments with Newton tolerance 1e-6; the staged
result of the GPU path against the oracle's (mech_stage_solver!,
src/mech/mech-solver.jl:186-492, with update_state! of von-mises.jl:128-157): on a
small block, and on a mid-size block (1 296 elements, 6 825 DOFs) with U, F, the
accumulated plastic strain and every Newton iteration's increment, number and
residue.  Also the update_records! hook at the checkpoints of nouts."""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from amaru_gpu import workloads as W

pytestmark = pytest.mark.gpu


def _slope_models(n, seed):
    g = W.SLOPE
    box = [[0, 0, 0], [g["L"], g["W"], g["H"]]]
    mg = A.Mesh(A.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    mo = O.Mesh(O.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    assert (mg.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    c = W.slope_coords(mo.coords, mg.elem_nodes(), W.boundary_nodes(mg), 4, *n, seed=seed)
    mo.coords = c
    mg.coords = c.copy()
    mat = dict(E=50e3, nu=0.3, fy=100.0, H=1e3)
    om = O.FEModel(mo, [("all", O.VonMises(**mat))])
    gm = A.FEModel(mg, [("all", A.VonMises(**mat))])
    return om, gm


def test_slope_tet10_von_mises_matches_the_oracle():
    om, gm = _slope_models((10, 2, 4), seed=7)
    ag, ao = A.MechAnalysis(gm), O.MechAnalysis(om)
    ag.addstage(W.slope_bcs(A, 200.0), nincs=20)
    ao.addstage(W.slope_bcs(O, 200.0), nincs=20)
    assert ag.solve(tol=1e-6)[0] and ao.solve(tol=1e-6)[0]
    assert ag.stats[0].increments == 20
    assert gm.state()[:, 12].max() > 0  # the surcharge yields the crest
    su, sf = np.abs(om.U).max(), np.abs(om.F).max()
    assert np.abs(gm.U - om.U).max() <= 1e-6 * su
    assert np.abs(gm.F - om.F).max() <= 1e-6 * sf


def test_slope_mid_size_matches_the_oracle_iteration_by_iteration():
    om, gm = _slope_models((12, 3, 6), seed=11)
    ag, ao = A.MechAnalysis(gm), O.MechAnalysis(om)
    ag.addstage(W.slope_bcs(A, 200.0), nincs=20)
    ao.addstage(W.slope_bcs(O, 200.0), nincs=20)
    okg, msg = ag.solve(tol=1e-6, solver="amg")
    assert okg, msg
    assert ao.solve(tol=1e-6, nthreads=4)[0]
    assert ag.stats[0].increments == 20
    # the Newton log: the same increments and iterations, residues to the solve's tolerance
    lg = [(inc, it) for _, inc, it, _ in ag.log]
    lo = [(inc, it) for _, inc, it, _ in ao.log]
    assert lg == lo
    sf = np.abs(om.F).max()
    for (_, _, _, rg), (_, _, _, ro) in zip(ag.log, ao.log):
        assert abs(rg - ro) <= 1e-6 * sf + 1e-3 * ro
    su = np.abs(om.U).max()
    assert np.abs(gm.U - om.U).max() <= 1e-6 * su
    assert np.abs(gm.F - om.F).max() <= 1e-6 * sf
    epa_g, epa_o = gm.state()[:, 12], om.state[:, 12]
    assert (epa_o > 0).sum() > 100  # a plastic zone under the crest
    assert np.abs(epa_g - epa_o).max() <= 1e-6 * epa_o.max()


def test_checkpoint_records_match_the_oracle():
    """nouts = 4 over 8 increments: the hook runs after every converged increment with the dof values so far;
    the checkpoints fall at T = 0.25, 0.5, 0.75, 1 as in the reference's Tcheck rule."""
    box = [[0, 0, 0], [1.0, 0.2, 0.2]]
    mg = A.Mesh(A.Block(box, nx=10, ny=2, nz=2, cellshape=A.HEX8))
    mo = O.Mesh(O.Block(box, nx=10, ny=2, nz=2, cellshape=A.HEX8))
    mat = dict(E=200e3, nu=0.3, fy=250.0, H=1e4)
    gm, om = A.FEModel(mg, [("all", A.VonMises(**mat))]), O.FEModel(mo, [("all", O.VonMises(**mat))])
    bcs = lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", M.SurfaceBC(tz=-30.0))]  # noqa: E731
    ag, ao = A.MechAnalysis(gm), O.MechAnalysis(om)
    ag.addstage(bcs(A), nincs=8, nouts=4)
    ao.addstage(bcs(O), nincs=8, nouts=4)
    rg, ro = [], []
    assert ag.solve(record=lambda ana, T, cp: rg.append((T, cp, ana.model.U.copy())))[0]
    assert ao.solve(record=lambda ana, T, cp: ro.append((T, cp, ana.model.U.copy())))[0]
    assert len(rg) == len(ro) == 8
    assert [cp for _, cp, _ in rg] == [cp for _, cp, _ in ro] == [False, True] * 4
    for (tg, _, ug), (to, _, uo) in zip(rg, ro):
        assert abs(tg - to) <= 1e-12
        assert np.abs(ug - uo).max() <= 1e-6 * np.abs(ro[-1][2]).max()
    assert np.array_equal(rg[-1][2], gm.U)
