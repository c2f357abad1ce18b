"""Batches of independent models: many plane-strain QUAD8 rectangles of uneven size,
each its own mech_stage_solver! (src/mech/mech-solver.jl:186-492), joined into one
device handle (amr_set_parts) and run together.

Checked here:
* every part against the same model run alone through the whole-model path and
  against the oracle (1e-6 of max|U| and of max|F|);
* a part's result is bitwise the same alone (a batch of one) and in the mix;
* elastoplastic parts over several increments, with Newton iteration counts equal
  to the model run alone;
* the ME / BE / Ralston schemes per part, against each model alone with the scheme;
* the batched solve_system! per part;
* the multigrid-preconditioned batched solve (the joined model's V-cycle, scalars per part): each part
  against the model alone to the solver tolerance, linear and elastoplastic stages, far fewer Krylov
  iterations than block-Jacobi;
* a part that fails its stage leaves the others untouched;
* the autotuner changes launch shapes only, not results.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

pytestmark = pytest.mark.gpu

BOX = [[0, 0], [2.0, 1.0]]


def _instances(seed, count, nmin, nmax):
    """(n, E, nu) per model: n uniform in [nmin, nmax], E lognormal(ln 200e3, 0.2), nu uniform [0.2, 0.35]."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(nmin, nmax + 1)), float(np.exp(rng.normal(np.log(200e3), 0.2))),
             float(rng.uniform(0.2, 0.35))) for _ in range(count)]


def _gpu_model(n, mat, device):
    mesh = A.Mesh(A.Block(BOX, nx=n, ny=n, cellshape=A.QUAD8))
    return A.FEModel(mesh, [("all", mat)], A.MechContext(stressmodel="planestrain"), nips=9, device=device)


def _bcs(mod, load):
    return [("x==0", mod.SurfaceBC(ux=0, uy=0)), ("x==2", mod.SurfaceBC(tx=load))]


def _linear(inst, device=False):
    return [_gpu_model(n, A.LinearElastic(E=E, nu=nu), device) for n, E, nu in inst]


def _close(a, b, tol=1e-6):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * s


def test_batch_matches_each_model_alone_and_the_oracle():
    # the last two have >= 2048 nodes: each is solved by a cluster of CTAs
    inst = _instances(7, 6, 2, 12) + [(28, 190e3, 0.25), (34, 210e3, 0.3)]
    ba = A.BatchAnalysis(_linear(inst))
    ba.addstage(_bcs(A, 1.0))
    res = ba.solve()
    assert all(ok for ok, _ in res)
    for (n, E, nu), m in zip(inst, ba.models):
        alone = _gpu_model(n, A.LinearElastic(E=E, nu=nu), True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(A, 1.0))
        assert ana.solve()[0]
        assert _close(m.U, alone.U) and _close(m.F, alone.F)
        mo = O.Mesh(O.Block(BOX, nx=n, ny=n, cellshape=A.QUAD8))
        om = O.FEModel(mo, [("all", O.LinearElastic(E=E, nu=nu))], stressmodel="planestrain", nips=9)
        ao = O.MechAnalysis(om)
        ao.addstage(_bcs(O, 1.0))
        assert ao.solve()[0]
        assert _close(m.U, om.U) and _close(m.F, om.F)
    st = ba.part_stats[0]
    assert all(s.status == 0 and s.increments == 1 for s in st)


def test_part_result_is_the_same_alone_and_in_the_mix():
    inst = _instances(11, 9, 2, 14) + [(30, 200e3, 0.3), (40, 180e3, 0.22)]
    mix = A.BatchAnalysis(_linear(inst))
    mix.addstage(_bcs(A, 1.0))
    assert all(ok for ok, _ in mix.solve())
    for k in (int(np.argmin([i[0] for i in inst])), 9, 10, 3):
        one = A.BatchAnalysis(_linear([inst[k]]))
        one.addstage(_bcs(A, 1.0))
        assert one.solve()[0][0]
        assert np.array_equal(one.models[0].U, mix.models[k].U)
        assert np.array_equal(one.models[0].F, mix.models[k].F)


def test_elastoplastic_parts_over_increments():
    inst = _instances(3, 4, 2, 6)
    mats = [A.VonMises(E=E, nu=nu, fy=0.9, H=1e3) for _, E, nu in inst]
    ba = A.BatchAnalysis([_gpu_model(n, mat, False) for (n, _, _), mat in zip(inst, mats)])
    ba.addstage(_bcs(A, 1.0), nincs=5)
    assert all(ok for ok, _ in ba.solve(tol=1e-6))
    for k, ((n, E, nu), m) in enumerate(zip(inst, ba.models)):
        alone = _gpu_model(n, A.VonMises(E=E, nu=nu, fy=0.9, H=1e3), True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(A, 1.0), nincs=5)
        assert ana.solve(tol=1e-6)[0]
        assert ba.part_stats[0][k].iterations == ana.stats[0].iterations
        assert _close(m.U, alone.U) and _close(m.F, alone.F)
        assert alone.state()[:, 12].max() > 0  # the load yields the material
    one = A.BatchAnalysis([_gpu_model(inst[2][0], A.VonMises(E=inst[2][1], nu=inst[2][2], fy=0.9, H=1e3), False)])
    one.addstage(_bcs(A, 1.0), nincs=5)
    assert one.solve(tol=1e-6)[0][0]
    assert np.array_equal(one.models[0].U, ba.models[2].U)


@pytest.mark.parametrize("scheme", ["ME", "BE", "Ralston"])
def test_predictor_corrector_schemes_per_part(scheme):
    """The ME / BE / Ralston schemes (src/mech/mech-solver.jl:280-288,341-350) run per part in the batched
    stage: each part takes the Newton iterations of the same model run alone with the scheme, and its U and F
    agree with it; a part's result is bitwise the same alone and in the mix."""
    inst = _instances(13, 4, 2, 6)
    kw = dict(tol=1e-6, scheme=scheme, autoinc=True)
    mats = [A.VonMises(E=E, nu=nu, fy=0.9, H=1e3) for _, E, nu in inst]
    ba = A.BatchAnalysis([_gpu_model(n, mat, False) for (n, _, _), mat in zip(inst, mats)])
    ba.addstage(_bcs(A, 1.0), nincs=4)
    res = ba.solve(**kw)
    assert any(ok for ok, _ in res)
    for k, ((n, E, nu), m) in enumerate(zip(inst, ba.models)):
        alone = _gpu_model(n, A.VonMises(E=E, nu=nu, fy=0.9, H=1e3), True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(A, 1.0), nincs=4)
        ok = ana.solve(**kw)[0]
        assert ok == res[k][0]  # the same outcome as the model alone
        assert ba.part_stats[0][k].increments == ana.stats[0].increments
        assert ba.part_stats[0][k].iterations == ana.stats[0].iterations
        if ok:
            assert _close(m.U, alone.U) and _close(m.F, alone.F)
    one = A.BatchAnalysis([_gpu_model(inst[1][0], A.VonMises(E=inst[1][1], nu=inst[1][2], fy=0.9, H=1e3), False)])
    one.addstage(_bcs(A, 1.0), nincs=4)
    assert one.solve(**kw)[0][0] == res[1][0]
    assert np.array_equal(one.models[0].U, ba.models[1].U)


def test_batched_solve_system_per_part():
    inst = _instances(5, 5, 2, 10)
    ba = A.BatchAnalysis(_linear(inst))
    Uex, Fex = ba.configure([_bcs(A, 1.0)] * len(inst))
    J = ba.joined
    J.dev.assemble_K()
    U, F = Uex.copy(), Fex.copy()
    st = J.solve_system(U, F, rtol=1e-10)
    assert st.rel_residual <= 1e-10
    Us, Fs = ba.split(U), ba.split(F)
    for (n, E, nu), Ui, Fi in zip(inst, Us, Fs):
        alone = _gpu_model(n, A.LinearElastic(E=E, nu=nu), True)
        setup = alone.configure_dofs(_bcs(A, 1.0))
        Ua, Fa = alone.get_bc_vals(setup)
        alone.dev.assemble_K()
        alone.solve_system(Ua, Fa, rtol=1e-10)
        Un = np.zeros((alone.nnodes, 2))
        Fn = np.zeros((alone.nnodes, 2))
        Un[alone.dof_node, alone.dof_comp] = Ua
        Fn[alone.dof_node, alone.dof_comp] = Fa
        assert _close(Ui, Un) and _close(Fi, Fn)


def test_failing_part_leaves_the_others_untouched():
    inst = _instances(13, 4, 2, 6)
    mats = [A.VonMises(E=E, nu=nu, fy=0.9, H=0.0) for _, E, nu in inst]
    loads = [0.5, 50.0, 0.5, 0.5]  # part 1: far beyond the limit load of a perfectly plastic strip
    ba = A.BatchAnalysis([_gpu_model(n, mat, False) for (n, _, _), mat in zip(inst, mats)])
    ba.addstage([_bcs(A, q) for q in loads], nincs=2)
    res = ba.solve(tol=1e-6, maxits=3)
    assert not res[1][0] and all(res[k][0] for k in (0, 2, 3))
    assert ba.part_stats[0][1].status == -11
    rest = A.BatchAnalysis([_gpu_model(inst[k][0], mats[k], False) for k in (0, 2, 3)])
    rest.addstage([_bcs(A, loads[k]) for k in (0, 2, 3)], nincs=2)
    assert all(ok for ok, _ in rest.solve(tol=1e-6, maxits=3))
    for j, k in enumerate((0, 2, 3)):
        assert np.array_equal(rest.models[j].U, ba.models[k].U)


def test_autotune_changes_launch_shapes_not_results():
    inst = _instances(17, 12, 2, 16)
    a = A.BatchAnalysis(_linear(inst))
    a.addstage(_bcs(A, 1.0))
    assert all(ok for ok, _ in a.solve())
    b = A.BatchAnalysis(_linear(inst))
    b.addstage(_bcs(A, 1.0))
    t = b.autotune()
    assert t.ngroups == 1 and t.shape[0] == A.QUAD8
    assert t.stiffness_epb[0] >= 1 and t.internal_epb[0] >= 1 and 1 <= t.batch_ctas_per_sm <= 4
    assert t.batch_threads == 512 and t.stiffness_seconds > 0 and t.internal_seconds > 0
    assert all(ok for ok, _ in b.solve())
    for ma, mb in zip(a.models, b.models):
        assert np.array_equal(ma.U, mb.U) and np.array_equal(ma.F, mb.F)


def test_batched_multigrid_solve_system_per_part():
    """solve_system! per part with the joined model's multigrid: every part reaches 1e-10 of its own right-hand
    side and agrees with the model alone, in far fewer iterations than block-Jacobi needs."""
    inst = _instances(5, 7, 2, 16) + [(30, 200e3, 0.3)]
    ba = A.BatchAnalysis(_linear(inst))
    Uex, Fex = ba.configure([_bcs(A, 1.0)] * len(inst))
    J = ba.joined
    J.dev.assemble_K()
    U, F = Uex.copy(), Fex.copy()
    st = J.solve_system(U, F, rtol=1e-10, method=A.SOLVER_AMG)
    assert st.rel_residual <= 1e-10 and st.iterations < 200
    Us, Fs = ba.split(U), ba.split(F)
    for (n, E, nu), Ui, Fi in zip(inst, Us, Fs):
        alone = _gpu_model(n, A.LinearElastic(E=E, nu=nu), True)
        setup = alone.configure_dofs(_bcs(A, 1.0))
        Ua, Fa = alone.get_bc_vals(setup)
        alone.dev.assemble_K()
        alone.solve_system(Ua, Fa, rtol=1e-12, method=A.SOLVER_FP64, max_iters=100000)
        Un = np.zeros((alone.nnodes, 2))
        Fn = np.zeros((alone.nnodes, 2))
        Un[alone.dof_node, alone.dof_comp] = Ua
        Fn[alone.dof_node, alone.dof_comp] = Fa
        assert _close(Ui, Un, 1e-7) and _close(Fi, Fn, 1e-7)
    U2, F2 = Uex.copy(), Fex.copy()
    bj = J.solve_system(U2, F2, rtol=1e-10)
    assert bj.iterations > 5 * st.iterations


@pytest.mark.parametrize("plastic", [False, True])
def test_batched_multigrid_stage_matches_each_model_alone(plastic):
    inst = _instances(21, 6, 3, 14) + [(36, 200e3, 0.3)]
    mat = (lambda E, nu: A.VonMises(E=E, nu=nu, fy=0.9, H=1e3)) if plastic else (lambda E, nu: A.LinearElastic(E=E, nu=nu))
    ba = A.BatchAnalysis([_gpu_model(n, mat(E, nu), False) for n, E, nu in inst])
    ba.addstage(_bcs(A, 1.0), nincs=3 if plastic else 1)
    kw = dict(tol=1e-6, solver="amg", linear_rtol=1e-10)
    res = ba.solve(**kw)
    assert all(ok for ok, _ in res)
    for k, ((n, E, nu), m) in enumerate(zip(inst, ba.models)):
        alone = _gpu_model(n, mat(E, nu), True)
        ana = A.MechAnalysis(alone)
        ana.addstage(_bcs(A, 1.0), nincs=3 if plastic else 1)
        assert ana.solve(**kw)[0]
        assert ba.part_stats[0][k].iterations == ana.stats[0].iterations
        assert _close(m.U, alone.U, 1e-7) and _close(m.F, alone.F, 1e-7)
    # the same batch with block-Jacobi needs many times the Krylov iterations
    bj = A.BatchAnalysis([_gpu_model(n, mat(E, nu), False) for n, E, nu in inst])
    bj.addstage(_bcs(A, 1.0), nincs=3 if plastic else 1)
    assert all(ok for ok, _ in bj.solve(tol=1e-6, linear_rtol=1e-10))
    kry_amg = sum(p.krylov_iterations for p in ba.part_stats[0])
    kry_bj = sum(p.krylov_iterations for p in bj.part_stats[0])
    assert kry_amg * 5 < kry_bj
