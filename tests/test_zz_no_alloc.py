"""amr_solve_noalloc: the solve for callers that cannot allocate GPU memory.

Some callers must not enter the CUDA allocator while they solve: a host
application that hands the library a fixed memory budget up front, a real-time
loop, or a memory pool that may not grow.  amr_solve_noalloc runs the
mixed-precision solve_system! on caller-owned device buffers with all of its
scratch in one static device array.  Here it is checked against the ordinary
amr_solve (same model, same K, same inputs) on two calls in a row, within the
tolerance of the solve parity tests (1e-6 of max|U| and of max|F|); the
library's device-allocation counter stays unchanged across those calls; a
model beyond the array's limit is refused with a clear error, and so is a
batch of parts, whose solve judges convergence per part.

This file is collected last so that a run stopping at its first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import amaru_gpu as A
from amaru_gpu import _lib as L

pytestmark = pytest.mark.gpu


def _model(n):
    mesh = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.3, 0.3]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX8))
    model = A.FEModel(mesh, [("all", A.LinearElastic(E=200e3, nu=0.3))])
    setup = model.configure_dofs([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", A.SurfaceBC(tz=-1.0)),
                                  ("x==1 && z==0.3", A.NodeBC(uz=-1e-4))])
    U, F = model.get_bc_vals(setup)
    return model, U, F


def _noalloc(model, U, F, opts):
    torch = pytest.importorskip("torch")
    dU = torch.from_numpy(U.copy()).cuda()
    dF = torch.from_numpy(F.copy()).cuda()
    st = L.SolveStats()
    rc = L.lib().amr_solve_noalloc(model.dev.h, C.c_void_p(dU.data_ptr()), C.c_void_p(dF.data_ptr()),
                                   C.byref(opts), C.byref(st))
    torch.cuda.synchronize()
    return rc, dU.cpu().numpy(), dF.cpu().numpy(), st


def test_noalloc_solve_matches_amr_solve_twice():
    model, U, F = _model((12, 4, 4))
    model.dev.assemble_K()
    opts = L.default_solve_opts(method=L.SOLVER_MIXED, rtol=1e-10)
    Ur, Fr, sr = model.dev.solve(U, F, opts)  # the ordinary entry point
    nu = model.nu
    assert sr.rel_residual <= 1e-10
    torch = pytest.importorskip("torch")
    dU = torch.from_numpy(U.copy()).cuda()
    dF = torch.from_numpy(F.copy()).cuda()
    for _ in range(2):  # the second call starts from the scratch contents the first one left
        dU.copy_(torch.from_numpy(U))
        dF.copy_(torch.from_numpy(F))
        torch.cuda.synchronize()
        before = model.dev.alloc_count()
        st = L.SolveStats()
        rc = L.lib().amr_solve_noalloc(model.dev.h, C.c_void_p(dU.data_ptr()), C.c_void_p(dF.data_ptr()),
                                       C.byref(opts), C.byref(st))
        assert model.dev.alloc_count() == before  # no cudaMalloc / cudaFree inside the call
        torch.cuda.synchronize()
        Un, Fn, sn = dU.cpu().numpy(), dF.cpu().numpy(), st
        assert rc == 0, model.dev.last_error()
        assert sn.rel_residual <= 1e-10
        assert np.abs(Un[:nu] - Ur[:nu]).max() <= 1e-6 * np.abs(Ur[:nu]).max()
        assert np.abs(Fn[nu:] - Fr[nu:]).max() <= 1e-6 * np.abs(Fr[nu:]).max()
        # the entries the solve does not write are passed through unchanged
        assert np.array_equal(Un[nu:], U[nu:]) and np.array_equal(Fn[:nu], F[:nu])


def test_noalloc_solve_refuses_batched_parts():
    parts = []
    for n in (3, 4):
        mesh = A.Mesh(A.Block([[0, 0], [2.0, 1.0]], nx=n, ny=n, cellshape=A.QUAD8))
        parts.append(A.FEModel(mesh, [("all", A.LinearElastic(E=200e3, nu=0.3))],
                               A.MechContext(stressmodel="planestrain"), device=False))
    ba = A.BatchAnalysis(parts)
    ba.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(tx=1.0))])
    U, F = ba.configure(ba.stages[0].bcs)
    J = ba.joined
    J.dev.assemble_K()
    rc, _, _, _ = _noalloc(J, U, F, L.default_solve_opts())
    assert rc == -10  # AMR_EUNSUPPORTED
    assert "batched" in J.dev.last_error()


def test_noalloc_solve_rejects_models_beyond_its_scratch():
    model, U, F = _model((45, 45, 44))  # 46 * 46 * 45 nodes x 3 > 262 144 slots
    model.dev.assemble_K()
    rc, _, _, _ = _noalloc(model, U, F, L.default_solve_opts())
    assert rc == -1  # AMR_EINVAL
    assert "262144" in model.dev.last_error()
