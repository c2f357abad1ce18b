"""The staged solver at the benchmark's full size, through properties that hold at any size.

The file runs after the small-case parity files (it holds two full-size models on the device).

Workload: HEX20 100x40x40 block 10x4x4 (669 161 nodes, 2 007 483 DOFs, 27 IPs), lognormal E per element,
base z=0 fixed, pressure 1.0 on the top z=4; one linear increment with the multigrid-preconditioned mixed
solver, as the benchmark runs it.

  * global equilibrium: the base reactions balance the applied load, 40 = 1.0 x 10 x 4. At a relative
    residual of 1e-8 the imbalance is bounded by sqrt(nu) * 1e-8 * |F1| (about 2e-7 of the load here), so
    the test allows 1e-5;
  * the horizontal reactions sum to zero, to the same bound (no horizontal load);
  * the top moves down and every displacement is finite;
  * the stage is bitwise repeatable.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

SEED = 0xA11A


def _stage():
    mesh = A.Mesh(A.Block([[0, 0, 0], [10.0, 4.0, 4.0]], nx=100, ny=40, nz=40, cellshape=A.HEX20))
    E = np.exp(np.random.default_rng(SEED).normal(np.log(30e3), 0.3, len(mesh.shape)))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27, E=E)
    ana = A.MechAnalysis(model)
    ana.addstage([("z==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", A.SurfaceBC(tz=-1.0))])
    ok, msg = ana.solve(solver="amg")
    assert ok, msg
    return mesh, model, ana


def test_oracle_stage_equilibrium_on_the_same_workload_family():
    """The property itself, on the oracle's direct solve at HEX20 5x2x2: reactions (40, 0, 0 up to round-off)."""
    mesh = O.Mesh(O.Block([[0, 0, 0], [10.0, 4.0, 4.0]], nx=5, ny=2, nz=2, cellshape=O.HEX20))
    E = np.exp(np.random.default_rng(SEED).normal(np.log(30e3), 0.3, len(mesh.elems)))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27, elem_E=E)
    ana = O.MechAnalysis(om)
    ana.addstage([("z==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", O.SurfaceBC(tz=-1.0))])
    assert ana.solve()[0]
    R = om.F[mesh.select_nodes("z==0")].sum(axis=0)
    assert abs(R[2] - 40.0) <= 1e-12 * 40.0 and np.abs(R[:2]).max() <= 1e-12 * 40.0
    assert om.U[mesh.select_nodes("z==4"), 2].max() < 0.0


@pytest.mark.gpu
def test_full_size_stage_equilibrium_and_repeatability():
    mesh, model, ana = _stage()
    assert model.ndofs == 2007483
    base = mesh.select_nodes("z==0")
    R = model.F[base].sum(axis=0)
    assert abs(R[2] - 40.0) <= 1e-5 * 40.0, R
    assert np.abs(R[:2]).max() <= 1e-5 * 40.0, R
    assert np.isfinite(model.U).all()
    top = mesh.select_nodes("z==4")
    assert model.U[top, 2].max() < 0.0
    U1 = model.U.copy()
    _, model2, _ = _stage()
    assert np.array_equal(model2.U, U1)
