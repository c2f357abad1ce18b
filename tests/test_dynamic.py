"""Dynamic analyses: mount_M (src/mech/dyn-solver.jl:71-104, elem_mass src/mech/elem/mech-solid.jl:169-205)
and dyn_stage_solver! (src/mech/dyn-solver.jl:203-534), Newmark's average-acceleration rule with
Rayleigh damping inside the reference's Newton loop.

The reference's dynamic test (test/dynamic/dyn-solid.jl) runs without assertions, so the oracle's
restatement is pinned by properties of the method: the consistent mass matrix carries rho times the
volume per component; undamped, under a constant load, the trapezoidal rule conserves the discrete
energy 1/2 V'MV + 1/2 U'KU - F'U; with damping, the Newton loop of a linear model reproduces the
closed recursion U_{n+1} = Keff^-1 (F + M(4/dt^2 U + 4/dt V + A) + C(2/dt U + V)).  The CUDA path
(amr_assemble_M, amr_dyn_stage_run) is then compared with the oracle: M entry by entry, and U, V, A,
F and the increment counts of elastic and elastoplastic stages, 2-D and 3-D, with time-dependent
loads; at larger size through the energy property.

Seismic input (sism, sismic_force, src/mech/dyn-solver.jl:106-157,271-287,348-352): the acceleration
record is interpolated as the reference does (a leading 0, samples spread over tds, linear between
them); the oracle's stage equals the closed recursion with the load M (a(t) e_dir) at every step while
the record runs; the CUDA path equals the oracle, with the record starting at t = 0 and later.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O


def _beam(M, shape=A.HEX8, n=(1, 10, 1), box=((0, 0, 0), (0.2, 2.0, 0.2)), mat=None, **kw):
    mat = mat or M.LinearElastic(E=30e6, nu=0.2, rho=24.0)
    mesh = M.Mesh(M.Block([list(box[0]), list(box[1])], nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
    return mesh, M.FEModel(mesh, [("all", mat)], **kw)


DYN_SOLID_BCS = lambda M: [("y==0 && z==0", M.NodeBC(ux=0, uy=0, uz=0)), ("y==2 && z==0", M.NodeBC(uz=0)),
                           ("y==1 && z==0.2", M.NodeBC(fz=-10))]


def _partition(ana, model):
    K = O.mount_K(model, ana.ndofs).tocsc()
    Mm = O.mount_M(model, ana.ndofs).tocsc()
    nu = ana.nu
    return K[:nu, :nu], Mm[:nu, :nu]


def test_oracle_mass_matrix_carries_rho_times_volume():
    _, om = _beam(O, shape=O.HEX20, n=(2, 3, 2), box=((0, 0, 0), (0.4, 1.5, 0.3)),
                  mat=O.LinearElastic(E=1e4, nu=0.3, rho=7.5), nips=27)
    dofs, nu, _ = O.configure_dofs(om, [])
    Mm = O.mount_M(om, len(dofs)).toarray()
    ux = om.eq_id[:, 0][om.eq_id[:, 0] >= 0]
    assert abs(Mm[np.ix_(ux, ux)].sum() - 7.5 * 0.4 * 1.5 * 0.3) < 1e-12
    assert np.allclose(Mm, Mm.T, rtol=0, atol=1e-15)


def test_oracle_undamped_newmark_conserves_energy():
    _, om = _beam(O, n=(1, 6, 1))
    ana = O.DynAnalysis(om)
    ana.addstage(DYN_SOLID_BCS(O), tspan=0.02, nincs=8)
    assert ana.solve()[0] and ana.increments == 8
    K, Mm = _partition(ana, om)
    nu = ana.nu
    F = np.zeros(ana.ndofs)
    F[om.eq_id[om.mesh.select_nodes("y==1 && z==0.2"), 2]] = -10.0
    F = F[:nu]
    # energy of the initial state (U = V = 0) is 0; after 8 steps it must still be 0
    U, V = ana.U[:nu], ana.V[:nu]
    E = 0.5 * V @ (Mm @ V) + 0.5 * U @ (K @ U) - F @ U
    scale = 0.5 * U @ (K @ U)
    assert scale > 0 and abs(E) <= 1e-9 * scale


def test_oracle_matches_the_closed_newmark_recursion():
    alpha, beta, tspan, nincs = 4.2038, 174.2803e-6, 0.05, 5
    _, om = _beam(O, n=(1, 6, 1))
    ana = O.DynAnalysis(om)
    ana.addstage(DYN_SOLID_BCS(O), tspan=tspan, nincs=nincs)
    assert ana.solve(alpha=alpha, beta=beta)[0]
    K, Mm = _partition(ana, om)
    nu = ana.nu
    K, Mm = K.toarray(), Mm.toarray()
    Cm = alpha * Mm + beta * K
    F = np.zeros(ana.ndofs)
    F[om.eq_id[om.mesh.select_nodes("y==1 && z==0.2"), 2]] = -10.0
    F = F[:nu]
    dt = tspan / nincs
    U, V = np.zeros(nu), np.zeros(nu)
    Ac = np.linalg.solve(Mm, F)
    Keff = K + 4 / dt ** 2 * Mm + 2 / dt * Cm
    for _ in range(nincs):
        Un = np.linalg.solve(Keff, F + Mm @ (4 / dt ** 2 * U + 4 / dt * V + Ac) + Cm @ (2 / dt * U + V))
        Vn = 2 / dt * (Un - U) - V
        Ac = 4 / dt ** 2 * (Un - U) - 4 / dt * V - Ac
        U, V = Un, Vn
    sc = np.abs(U).max()
    assert np.abs(ana.U[:nu] - U).max() <= 1e-9 * sc
    assert np.abs(ana.V[:nu] - V).max() <= 1e-9 * np.abs(V).max()
    assert np.abs(ana.A[:nu] - Ac).max() <= 1e-8 * np.abs(Ac).max()


SEIS_BCS = lambda M: [("y==0", M.SurfaceBC(ux=0, uy=0, uz=0))]  # noqa: E731
SEIS_RECORD = "0.10 0.35 -0.20\n-0.45 0.05 0.30\n"            # readdlm's 2 x 3 matrix, read row by row


def test_oracle_seismic_acceleration_interpolates_the_record():
    from oracle.dynamic import sismic_acceleration
    acc = np.array([1.0, 3.0, 2.0])
    for t, a in ((0.0, 0.0), (0.05, 0.5), (0.1, 1.0), (0.15, 2.0), (0.25, 2.5), (0.3, 2.0)):
        assert abs(sismic_acceleration(acc, 0.3, t) - a) < 1e-12
    with pytest.raises(ValueError):
        sismic_acceleration(acc, 0.3, 0.31)


def test_oracle_seismic_stage_matches_the_closed_recursion(tmp_path):
    f = tmp_path / "record.dat"
    f.write_text(SEIS_RECORD)
    alpha, beta, tspan, nincs = 2.0, 1e-4, 0.06, 6
    _, om = _beam(O, n=(1, 6, 1))
    ana = O.DynAnalysis(om)
    ana.addstage(SEIS_BCS(O), tspan=tspan, nincs=nincs)
    assert ana.solve(alpha=alpha, beta=beta, sism=True, tss=0.0, tds=tspan, sism_file=str(f), sism_dir="fx")[0]
    from oracle.dynamic import sismic_acceleration
    nu, nd = ana.nu, ana.ndofs
    Kf = O.mount_K(om, nd).toarray()
    Mf = O.mount_M(om, nd).toarray()
    e = np.zeros(nd)
    e[om.eq_id[:, 0][om.eq_id[:, 0] >= 0]] = 1.0  # the x component of every node, prescribed ones too
    acc = 9.81 * np.loadtxt(str(f), ndmin=2).reshape(-1)
    K, Mm = Kf[:nu, :nu], Mf[:nu, :nu]
    Cm = alpha * Mm + beta * K
    dt = tspan / nincs
    F = lambda t: (Mf @ (sismic_acceleration(acc, tspan, t) * e))[:nu]  # noqa: E731
    U, V = np.zeros(nu), np.zeros(nu)
    Ac = np.linalg.solve(Mm, F(0.0))
    Keff = K + 4 / dt ** 2 * Mm + 2 / dt * Cm
    for i in range(1, nincs + 1):
        Un = np.linalg.solve(Keff, F(i * dt) + Mm @ (4 / dt ** 2 * U + 4 / dt * V + Ac) + Cm @ (2 / dt * U + V))
        Vn = 2 / dt * (Un - U) - V
        Ac = 4 / dt ** 2 * (Un - U) - 4 / dt * V - Ac
        U, V = Un, Vn
    assert np.abs(U).max() > 0
    assert np.abs(ana.U[:nu] - U).max() <= 1e-9 * np.abs(U).max()
    assert np.abs(ana.V[:nu] - V).max() <= 1e-9 * np.abs(V).max()
    assert np.abs(ana.A[:nu] - Ac).max() <= 1e-8 * np.abs(Ac).max()


# ---------------------------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("tss,tds", [(0.0, 0.04), (0.02, 0.06)])
def test_gpu_seismic_stage_matches_the_oracle(tmp_path, tss, tds):
    """The record ends inside the stage (0, 0.04), or starts late (0.02); sismic_force reads the record at
    the absolute time t + dt, so a late start needs a record that still covers it."""
    f = tmp_path / "record.dat"
    f.write_text(SEIS_RECORD)
    mat = dict(E=30e6, nu=0.2, rho=24.0)
    om, gm = _pair(A.HEX8, (2, 8, 2), ((0, 0, 0), (0.2, 2.0, 0.2)), O.LinearElastic(**mat), A.LinearElastic(**mat))
    ao, ag = O.DynAnalysis(om), A.DynAnalysis(gm)
    ao.addstage(SEIS_BCS(O), tspan=0.06, nincs=6)
    ag.addstage(SEIS_BCS(A), tspan=0.06, nincs=6)
    kw = dict(alpha=2.0, beta=1e-4, sism=True, tss=tss, tds=tds, sism_file=str(f), sism_dir="ux")
    assert ao.solve(**kw)[0]
    ok, msg = ag.solve(linear_rtol=1e-10, **kw)
    assert ok, msg
    assert ag.stats.increments == ao.increments == 6
    for k in ("U", "V", "A", "F"):
        assert _close(getattr(gm, k), getattr(om, k), 1e-7), k
    assert np.abs(gm.U[:, 0]).max() > 0


def _pair(shape, n, box, mat_o, mat_g, ctx="d3", **kw):
    mo, om = _beam(O, shape=shape, n=n, box=box, mat=mat_o, stressmodel=ctx, **kw) if len(n) == 3 else (None, None)
    if len(n) == 2:
        mo = O.Mesh(O.Block([list(box[0]), list(box[1])], nx=n[0], ny=n[1], cellshape=shape))
        om = O.FEModel(mo, [("all", mat_o)], stressmodel=ctx, **kw)
        mg = A.Mesh(A.Block([list(box[0]), list(box[1])], nx=n[0], ny=n[1], cellshape=shape))
    else:
        mg = A.Mesh(A.Block([list(box[0]), list(box[1])], nx=n[0], ny=n[1], nz=n[2], cellshape=shape))
    mg.coords = np.ascontiguousarray(mo.coords)
    gm = A.FEModel(mg, [("all", mat_g)], A.MechContext(stressmodel=ctx), **kw)
    return om, gm


def _close(a, b, tol):
    s = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= tol * s


@pytest.mark.gpu
def test_gpu_mass_matrix_matches_the_oracle():
    om, gm = _pair(A.HEX20, (2, 3, 2), ((0, 0, 0), (0.4, 1.5, 0.3)), O.LinearElastic(E=1e4, nu=0.3, rho=7.5),
                   A.LinearElastic(E=1e4, nu=0.3, rho=7.5), nips=27)
    bcs = lambda M: [("y==0", M.SurfaceBC(ux=0, uy=0, uz=0))]
    dofs, nu, _ = O.configure_dofs(om, bcs(O))
    Mo = O.mount_M(om, len(dofs)).tocsc()
    Mo.sort_indices()
    gm.configure_dofs(bcs(A))
    gm.dev.set_density(gm.rho)
    gm.dev.assemble_M()
    Mg = gm.dev.M_csc()
    assert (Mg.indptr == Mo.indptr).all() and (Mg.indices == Mo.indices).all()
    assert np.abs(Mg.data - Mo.data).max() <= 1e-13 * np.abs(Mo.data).max()


@pytest.mark.gpu
@pytest.mark.parametrize("solver", ["mixed", "amg"])
def test_gpu_dyn_stage_matches_the_oracle(solver):
    """The reference's dyn-solid.jl model, Rayleigh-damped, over several increments."""
    mat = dict(E=30e6, nu=0.2, rho=24.0)
    om, gm = _pair(A.HEX8, (1, 10, 1), ((0, 0, 0), (0.2, 2.0, 0.2)), O.LinearElastic(**mat), A.LinearElastic(**mat))
    ao, ag = O.DynAnalysis(om), A.DynAnalysis(gm)
    ao.addstage(DYN_SOLID_BCS(O), tspan=0.1, nincs=6, nouts=1)
    ag.addstage(DYN_SOLID_BCS(A), tspan=0.1, nincs=6, nouts=1)
    kw = dict(alpha=4.2038, beta=174.2803e-6)
    assert ao.solve(**kw)[0]
    ok, msg = ag.solve(solver=solver, linear_rtol=1e-10, **kw)
    assert ok, msg
    assert ag.stats.increments == ao.increments and ag.stats.iterations == ao.iterations
    for k in ("U", "V", "A", "F"):
        assert _close(getattr(gm, k), getattr(om, k), 1e-7), k


@pytest.mark.gpu
def test_gpu_dyn_stage_2d_with_a_time_dependent_load():
    mat = dict(E=200e3, nu=0.3, rho=7.8e-3)
    om, gm = _pair(A.QUAD8, (12, 3), ((0, 0), (3.0, 0.5)), O.LinearElastic(**mat), A.LinearElastic(**mat),
                   ctx="planestrain")
    bcs = lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0)), ("x==3", M.SurfaceBC(ty="-2.0*t"))]
    ao, ag = O.DynAnalysis(om), A.DynAnalysis(gm)
    ao.addstage(bcs(O), tspan=0.05, nincs=10)
    ag.addstage(bcs(A), tspan=0.05, nincs=10)
    assert ao.solve(alpha=0.5, beta=1e-4)[0]
    ok, msg = ag.solve(alpha=0.5, beta=1e-4, linear_rtol=1e-10)
    assert ok, msg
    assert ag.stats.increments == ao.increments == 10
    for k in ("U", "V", "A", "F"):
        assert _close(getattr(gm, k), getattr(om, k), 1e-7), k
    # the stage leaves the pseudo-stiffness in K's storage: K must be mounted again before it is read
    from amaru_gpu import _lib as L
    with pytest.raises(L.AmrError):
        gm.dev.K_csc()
    gm.dev.assemble_K()
    assert gm.dev.K_csc().nnz > 0
    # boundary values that are not affine in time are refused on the host
    ag2 = A.DynAnalysis(gm)
    ag2.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==3", A.SurfaceBC(ty="-2.0*t*t"))], tspan=0.05)
    with pytest.raises(NotImplementedError):
        ag2.solve()


@pytest.mark.gpu
def test_gpu_dyn_stage_with_plasticity():
    """VonMises under a sudden tip load: the tangent changes with the IP states, K is mounted at every
    iteration, and the Newton loop takes the reference's number of iterations."""
    mat = dict(E=200e3, nu=0.3, fy=240.0, H=2e3, rho=7.8e-3)
    om, gm = _pair(A.HEX8, (12, 2, 2), ((0, 0, 0), (1.0, 0.1, 0.1)), O.VonMises(**mat), A.VonMises(**mat))
    bcs = lambda M: [("x==0", M.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", M.SurfaceBC(tz=-40.0))]
    ao, ag = O.DynAnalysis(om), A.DynAnalysis(gm)
    ao.addstage(bcs(O), tspan=2e-3, nincs=8)
    ag.addstage(bcs(A), tspan=2e-3, nincs=8)
    assert ao.solve(tol=1e-4, maxits=10, alpha=20.0)[0]
    ok, msg = ag.solve(tol=1e-4, maxits=10, alpha=20.0, linear_rtol=1e-11)
    assert ok, msg
    assert gm.state()[:, 12].max() > 0
    assert ag.stats.increments == ao.increments and ag.stats.iterations == ao.iterations
    for k in ("U", "V", "A"):
        assert _close(getattr(gm, k), getattr(om, k), 1e-6), k


@pytest.mark.gpu
def test_gpu_undamped_newmark_conserves_energy_at_size():
    """HEX20 40x8x8 cantilever (about 24 k nodes), sudden constant tip load, undamped: the discrete energy
    after 10 steps stays zero to the solver's tolerance."""
    mat = A.LinearElastic(E=30e3, nu=0.2, rho=2.4e-3)
    mesh = A.Mesh(A.Block([[0, 0, 0], [4.0, 0.8, 0.8]], nx=40, ny=8, nz=8, cellshape=A.HEX20))
    gm = A.FEModel(mesh, [("all", mat)], nips=27)
    ag = A.DynAnalysis(gm)
    ag.addstage([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==4", A.SurfaceBC(tz=-1.0))], tspan=0.02, nincs=10)
    ok, msg = ag.solve(solver="amg", linear_rtol=1e-10)  # 1e-12 is beyond the FP32 PCG's refinement here
    assert ok, msg
    K = gm.mount_K()
    gm.dev.assemble_M()
    Mm = gm.dev.M_csc()
    nu = gm.nu
    U = np.zeros(gm.ndofs); V = np.zeros(gm.ndofs)
    U[:] = gm.U[gm.dof_node, gm.dof_comp]
    V[:] = gm.V[gm.dof_node, gm.dof_comp]
    Uex, Fex = gm.get_bc_vals(gm.configure_dofs([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)),
                                                 ("x==4", A.SurfaceBC(tz=-1.0))]))
    K11, M11 = K[:nu, :nu], Mm[:nu, :nu]
    u, v, f = U[:nu], V[:nu], Fex[:nu]
    E = 0.5 * v @ (M11 @ v) + 0.5 * u @ (K11 @ u) - f @ u
    assert abs(E) <= 1e-6 * (0.5 * u @ (K11 @ u))
