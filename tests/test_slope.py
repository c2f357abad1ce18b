"""Nonlinear geomechanics: the plane-strain slope extruded along y on a jittered TET10
mesh, von Mises with linear hardening (E=50e3, nu=0.3, fy=100, H=1e3), gravity and a
crest surcharge ramped over 20 increments with Newton tolerance 1e-6; the staged
result of the GPU path against the oracle's (mech_stage_solver!,
src/mech/mech-solver.jl:186-492, with update_state! of von-mises.jl)."""
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
