"""Modal analysis: mech_modal_solver! (src/mech/mech-modal-solver.jl:72-235).

The reference takes the nmodes eigenpairs of smallest magnitude of P = K11 ./ L (L the row-sum lumped
masses of M11) with Arpack and keeps the real positive ones; its modal test (test/dynamic/modal.jl)
has no assertion.  The oracle solves the equivalent symmetric-definite pencil diag(L) phi = mu K11 phi
and is pinned against the reference's own formulation, the dense non-symmetric P and numpy's eig, on
linear and serendipity cells (whose corner masses are negative).  The CUDA path (amr_modal_run,
LOBPCG with the multigrid preconditioner) is compared with the oracle: frequencies, and modes up to the
span of degenerate groups; at larger size through the eigen-residual of P.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

CASES = [(A.QUAD4, (4, 40), 0), (A.QUAD8, (3, 20), 0), (A.HEX8, (2, 12, 2), 0), (A.HEX20, (2, 8, 2), 27),
         (A.TET10, (1, 5, 1), 0)]


def _mesh(M, shape, n):
    if len(n) == 2:
        return M.Mesh(M.Block([[0, 0], [1.0, 10.0]], nx=n[0], ny=n[1], cellshape=shape))
    return M.Mesh(M.Block([[0, 0, 0], [1.0, 10.0, 1.0]], nx=n[0], ny=n[1], nz=n[2], cellshape=shape))


def _bcs(M, ndim):
    return [("y==0", M.NodeBC(ux=0, uy=0) if ndim == 2 else M.NodeBC(ux=0, uy=0, uz=0))]


MAT = dict(E=2e6, nu=0.2, rho=15.0)  # test/dynamic/modal.jl


def _same_modes(Va, Vb, w, tol):
    """Modes agree up to the span of each group of equal frequencies."""
    i = 0
    while i < len(w):
        j = i + 1
        while j < len(w) and abs(w[j] - w[i]) <= 1e-6 * w[i]:
            j += 1
        Q, _ = np.linalg.qr(Va[:, i:j])
        res = Vb[:, i:j] - Q @ (Q.T @ Vb[:, i:j])
        if np.abs(res).max() > tol:
            return False
        i = j
    return True


@pytest.mark.parametrize("shape, n, nips", CASES)
def test_oracle_pencil_matches_the_dense_P_formulation(shape, n, nips):
    om = O.FEModel(_mesh(O, shape, n), [("all", O.LinearElastic(**MAT))],
                   stressmodel="planestrain" if len(n) == 2 else "d3", nips=nips)
    w, V, _ = O.modal(om, _bcs(O, len(n)), 6)
    wd, Vd, _ = O.modal_dense(om, _bcs(O, len(n)), 6)
    assert np.abs(w - wd).max() <= 1e-9 * w.max()
    assert _same_modes(V, Vd, w, 1e-7)


def test_oracle_refuses_zero_density():
    om = O.FEModel(_mesh(O, O.QUAD4, (2, 4)), [("all", O.LinearElastic(E=1.0, nu=0.2))], stressmodel="planestrain")
    with pytest.raises(ValueError):
        O.modal(om, _bcs(O, 2), 2)


# ---------------------------------------------------------------------------------------------- GPU


@pytest.mark.gpu
@pytest.mark.parametrize("shape, n, nips", CASES)
def test_gpu_modes_match_the_oracle(shape, n, nips):
    sm = "planestrain" if len(n) == 2 else "d3"
    mo, mg = _mesh(O, shape, n), _mesh(A, shape, n)
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, [("all", O.LinearElastic(**MAT))], stressmodel=sm, nips=nips)
    gm = A.FEModel(mg, [("all", A.LinearElastic(**MAT))], A.MechContext(stressmodel=sm), nips=nips)
    w, V, nu = O.modal(om, _bcs(O, len(n)), 6)
    ana = A.ModalAnalysis(gm)
    ana.addstage(_bcs(A, len(n)))
    assert ana.solve(nmodes=6, tol=1e-8)[0]
    assert gm.nu == nu and ana.modes.shape == (nu, 6)
    assert np.abs(ana.freqs - w).max() <= 1e-8 * w.max(), (ana.freqs, w)
    assert _same_modes(V, ana.modes, w, 1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("shape, n, nmodes, tol, mode_tol", [(A.HEX8, (3, 16, 3), 24, 1e-8, 1e-5),
                                                             (A.QUAD4, (8, 40), 42, 1e-6, 1e-3),
                                                             (A.QUAD8, (4, 30), 24, 1e-6, 1e-3)])
def test_gpu_many_modes_match_the_oracle(shape, n, nmodes, tol, mode_tol):
    """Blocks wider than one launch of the multi-vector kernels (24 modes: block 36; 42 modes, the largest: block
    63) against the oracle: frequencies to 1e-8, modes up to degenerate groups (a group the nmodes cut splits is
    left out: any basis of its span is right).  In 2-D, with many modes, the LOBPCG residual levels off between
    1e-7 and 1e-6 (serendipity cells, with their negative corner masses, lowest): those cases are asked for
    the reference's Arpack tolerance, 1e-6."""
    sm = "planestrain" if len(n) == 2 else "d3"
    mo, mg = _mesh(O, shape, n), _mesh(A, shape, n)
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, [("all", O.LinearElastic(**MAT))], stressmodel=sm)
    gm = A.FEModel(mg, [("all", A.LinearElastic(**MAT))], A.MechContext(stressmodel=sm))
    w1, V1, nu = O.modal(om, _bcs(O, len(n)), nmodes + 1)
    w, V = w1[:nmodes], V1[:, :nmodes]
    ana = A.ModalAnalysis(gm)
    ana.addstage(_bcs(A, len(n)))
    assert ana.solve(nmodes=nmodes, tol=tol, max_iters=800)[0]
    assert ana.modes.shape == (nu, nmodes)
    assert np.abs(ana.freqs - w).max() <= 1e-8 * w.max(), (ana.freqs, w)
    keep = nmodes
    while keep > 0 and abs(w1[nmodes] - w1[keep - 1]) <= 1e-6 * w1[nmodes]:
        keep -= 1  # the last group continues past the cut
    assert keep >= nmodes - 3
    assert _same_modes(V[:, :keep], ana.modes[:, :keep], w[:keep], mode_tol)


@pytest.mark.gpu
def test_gpu_modal_block_limit_is_refused():
    gm = A.FEModel(_mesh(A, A.QUAD4, (4, 40)), [("all", A.LinearElastic(**MAT))],
                   A.MechContext(stressmodel="planestrain"))
    ana = A.ModalAnalysis(gm)
    ana.addstage(_bcs(A, 2))
    with pytest.raises(Exception, match="nmodes must be in 1..42"):
        ana.solve(nmodes=43)


@pytest.mark.gpu
def test_gpu_modal_residual_at_size():
    """HEX20 40x8x8 cantilever (about 73 k DOFs, 27 IPs): P v = lambda v for the returned pairs."""
    mesh = A.Mesh(A.Block([[0, 0, 0], [4.0, 0.8, 0.8]], nx=40, ny=8, nz=8, cellshape=A.HEX20))
    gm = A.FEModel(mesh, [("all", A.LinearElastic(E=30e3, nu=0.2, rho=2.4e-3))], nips=27)
    ana = A.ModalAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0))])
    assert ana.solve(nmodes=8, tol=1e-8)[0]
    w, V = ana.freqs, ana.modes
    assert (np.diff(w) >= 0).all() and w[0] > 0
    nu = gm.nu
    K11 = gm.mount_K()[:nu, :nu]
    gm.dev.assemble_M()
    L = np.asarray(gm.dev.M_csc()[:nu, :nu].sum(axis=0)).ravel()
    for i in range(len(w)):
        Pv = K11 @ (V[:, i] / L)
        assert np.linalg.norm(Pv - w[i] ** 2 * V[:, i]) <= 1e-6 * np.linalg.norm(Pv)


def test_rayleigh_coefficients_give_the_requested_damping_ratios():
    """mech_modal_solver!'s rayleigh option (src/mech/mech-modal-solver.jl:204-226): alpha/(2w) + beta w/2
    equals xi1 at w1 and xi2 at w2."""
    from amaru_gpu.model import rayleigh_coefficients
    for w1, w2, xi1, xi2 in [(3.81, 22.9, 0.02, 0.05), (598.2, 709.0, 0.05, 0.05), (10.0, 1.0, 0.1, 0.01)]:
        a, b = rayleigh_coefficients(w1, w2, xi1, xi2)
        for w, xi in ((w1, xi1), (w2, xi2)):
            assert abs(a / (2 * w) + b * w / 2 - xi) <= 1e-14 * max(1.0, xi)
    ana = A.ModalAnalysis(None)
    ana.freqs = np.array([3.81, 22.9, 58.6])
    a, b = ana.set_rayleigh(0.02, 0.05, 1, 3)
    assert (a, b) == (ana.alpha, ana.beta) == rayleigh_coefficients(3.81, 58.6, 0.02, 0.05)
    with pytest.raises(ValueError):
        ana.set_rayleigh(0.02, 0.05, 2, 2)
    with pytest.raises(ValueError):
        ana.set_rayleigh(0.02, 0.05, 1, 4)
