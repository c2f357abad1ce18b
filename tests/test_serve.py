"""Serving: staged analyses submitted to the request loop (amr_server_*) and run with
continuous batching.

Checked here:
* a mix of linear HEX8 and elastoplastic TET10 requests, several on the device at
  once, gives for every request bitwise the result of the same stage run alone
  (MechAnalysis on its own handle), and that equals the oracle within 1e-6;
* admission never lets the admitted footprints exceed the HBM budget, and a
  request waits for memory that running requests free;
* a request that can never fit is refused at submit;
* two admitted requests run on the GPU at the same time: their stages' spans on the
  device clock (CUDA events on each request's stream) intersect, and each result is
  bitwise the one it gets alone.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from amaru_gpu import serve

pytestmark = pytest.mark.gpu


def _hex8(n, E):
    mesh = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.2, 0.2]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX8))
    return A.FEModel(mesh, [("all", A.LinearElastic(E=E, nu=0.3))], device=False)


def _hex8_bcs(mod):
    return [("x==0", mod.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", mod.SurfaceBC(tz=-1.0))]


def _tet10(n):
    mesh = A.Mesh(A.Block([[0, 0, 0], [1.0, 0.5, 0.5]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.TET10))
    return A.FEModel(mesh, [("all", A.VonMises(E=50e3, nu=0.3, fy=100.0, H=1e3))], device=False)


def _tet10_bcs(mod):
    return [("z==0", mod.SurfaceBC(ux=0, uy=0, uz=0)), ("z==0.5", mod.SurfaceBC(tz=-120.0)),
            ("all", mod.BodyC(wz=-20.0))]


REQUESTS = [  # (kind, size, Young's modulus, increments)
    ("hex8", (30, 6, 6), 150e3, 3),
    ("tet10", (3, 2, 2), None, 4),
    ("hex8", (12, 3, 3), 200e3, 1),
    ("hex8", (6, 2, 2), 210e3, 2),
    ("tet10", (4, 2, 2), None, 3),
    ("hex8", (20, 4, 4), 180e3, 1),
]


def _model(kind, n, E, device=False):
    m = _hex8(n, E) if kind == "hex8" else _tet10(n)
    if device:
        m.dev = A._lib.DeviceModel(m.ndim, m.stressmodel, m.thickness, m.mesh.coords, m.mesh.shape, m.nips,
                                   m.mesh.conn_ptr, m.mesh.conn, m.mat_type, m.mat_params)
    return m


def _bcs(kind, mod=A):
    return _hex8_bcs(mod) if kind == "hex8" else _tet10_bcs(mod)


def _kw(kind):
    # past the yield load the continuum tangent (as the reference's) needs smaller steps than nincs gives
    return dict(autoinc=True) if kind == "tet10" else {}


def test_requests_in_the_mix_match_each_run_alone():
    models = [_model(k, n, E) for k, n, E, _ in REQUESTS]  # built first: the requests arrive back to back
    with serve.Server(hbm_budget_bytes=64e9, max_active=4) as srv:
        tickets = [srv.submit(m, _bcs(k), nincs=inc, **_kw(k)) for m, (k, n, E, inc) in zip(models, REQUESTS)]
        out = [srv.wait(t) for t in tickets]
        info = srv.info()
    assert info.completed == len(REQUESTS) and info.peak_active >= 2
    for (k, n, E, inc), (rc, U, F, res, msg) in zip(REQUESTS, out):
        assert rc == 0, msg
        assert res.stage.increments >= inc and res.t_submit <= res.t_admit <= res.t_done
        alone = _model(k, n, E, device=True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(k), nincs=inc)
        assert ana.solve(**_kw(k))[0]
        assert np.array_equal(U, alone.U) and np.array_equal(F, alone.F)
        if k == "tet10":
            assert alone.state()[:, 12].max() > 0  # the surcharge yields the material
    # one of each kind against the oracle
    for i in (2, 1):
        k, n, E, inc = REQUESTS[i]
        cell = A.HEX8 if k == "hex8" else A.TET10
        box = [[0, 0, 0], [1.0, 0.2, 0.2]] if k == "hex8" else [[0, 0, 0], [1.0, 0.5, 0.5]]
        mat = O.LinearElastic(E=E, nu=0.3) if k == "hex8" else O.VonMises(E=50e3, nu=0.3, fy=100.0, H=1e3)
        om = O.FEModel(O.Mesh(O.Block(box, nx=n[0], ny=n[1], nz=n[2], cellshape=cell)), [("all", mat)])
        ao = O.MechAnalysis(om)
        ao.addstage(_bcs(k, O), nincs=inc)
        assert ao.solve(**_kw(k))[0]
        U, F = out[i][1], out[i][2]
        assert np.abs(U - om.U).max() <= 1e-6 * np.abs(om.U).max()
        assert np.abs(F - om.F).max() <= 1e-6 * np.abs(om.F).max()


def test_admission_keeps_within_the_hbm_budget():
    models = [_model("hex8", (24, 4, 4), 200e3) for _ in range(6)]
    est = serve.estimate_bytes(models[0])
    budget = 2.5 * est  # two at a time
    with serve.Server(hbm_budget_bytes=budget, max_active=4) as srv:
        tickets = [srv.submit(m, _bcs("hex8"), nincs=2) for m in models]
        out = [srv.wait(t) for t in tickets]
        info = srv.info()
    assert all(rc == 0 for rc, *_ in out)
    assert info.peak_bytes <= budget and info.peak_active <= 2
    res = [o[3] for o in out]
    assert all(r.bytes == est for r in res)
    # admitted in arrival order, the third only after one of the first two finished
    assert res[2].t_admit >= min(res[0].t_done, res[1].t_done)
    assert all(res[i].t_admit <= res[i + 1].t_admit for i in range(len(res) - 1))
    for (rc, U, F, r, msg) in out[1:]:
        assert np.array_equal(U, out[0][1])


def test_request_beyond_the_budget_is_refused():
    m = _model("hex8", (8, 2, 2), 200e3)
    with serve.Server(hbm_budget_bytes=serve.estimate_bytes(m) / 2, max_active=1) as srv:
        with pytest.raises(A.AmrError) as e:
            srv.submit(m, _bcs("hex8"))
        assert e.value.code == -9


def test_admitted_requests_overlap_on_the_device():
    reqs = [("hex8", (40, 8, 8), 190e3, 6), ("hex8", (40, 8, 8), 210e3, 6)]
    models = [_model(k, n, E) for k, n, E, _ in reqs]
    with serve.Server(hbm_budget_bytes=64e9, max_active=2) as srv:
        tickets = [srv.submit(m, _bcs(k), nincs=inc, solver="amg") for m, (k, n, E, inc) in zip(models, reqs)]
        out = [srv.wait(t) for t in tickets]
    (rc0, U0, F0, r0, m0), (rc1, U1, F1, r1, m1) = out
    assert rc0 == 0 and rc1 == 0, (m0, m1)
    assert r0.dev_end > r0.dev_start > 0 and r1.dev_end > r1.dev_start > 0
    assert r0.dev_start < r1.dev_end and r1.dev_start < r0.dev_end  # both stages on the GPU at once
    assert r0.stage.seconds <= (r0.dev_end - r0.dev_start) * 1.01 + 1e-4
    for (k, n, E, inc), (rc, U, F, res, msg) in zip(reqs, out):
        alone = _model(k, n, E, device=True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(k), nincs=inc)
        assert ana.solve(solver="amg")[0]
        assert np.array_equal(U, alone.U) and np.array_equal(F, alone.F)
