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

pytestmark = pytest.mark.gpu

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
