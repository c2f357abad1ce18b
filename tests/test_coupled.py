"""Coupled mounts: hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) and
tm_mount_global_matrices (src/thermomech/thermomech-solver.jl:80-170) for linear elastic solids carrying a
scalar field on their basic nodes (HMSolid / TMSolid).

The reference's hydromechanical and thermomechanical tests run whole transient analyses and assert on no
mount, so the oracle's restatement (oracle/coupled.py) is pinned by properties of the formulation:
  * the u-u block is the element stiffnesses assembled as mount_K's element loop adds them (no eps() drop);
  * H annihilates a constant field (rows sum to zero), so with a storativity the w-w block sums to -S V;
  * the coupling sees no volume change in a rigid translation: G[w, u_x] 1 = 0;
  * the hydraulic mount is symmetric; the thermal one's w-u block is (T0 + 273.15) times the transposed u-w one;
  * the right-hand side of a linear pressure field p = z is (1 + 1/gammaw) times that of p = 0 (H p = -Q / gammaw),
    and the fluxes Q sum to zero.
The CUDA path (amr_coupled_mount) is then compared with the oracle: the CSC pattern bit for bit, every
DOF-type block (u-u, u-w, w-u, w-w) to 1e-12 of its largest entry, and the right-hand side to 1e-12.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O
from oracle import coupled as OC

PRM = {OC.HYDRO: (0.9, 2.5e-3, 1e-4), OC.THERMO: (1.2e-5, 1.7, 2.4e3)}


def _oracle_model(shape, n, box, stressmodel="d3", E=1e4, nu=0.25):
    kw = dict(nx=n[0], ny=n[1], nz=n[2]) if len(n) == 3 else dict(nx=n[0], ny=n[1])
    mesh = O.Mesh(O.Block(box, cellshape=shape, **kw))
    return O.FEModel(mesh, [("all", O.LinearElastic(E=E, nu=nu))], stressmodel=stressmodel)


def _setup(om, kind, seed=1, with_presc=True):
    nn = om.nnodes
    pres = np.zeros((nn, 4), dtype=bool)
    if with_presc:
        z = om.coords[:, om.ndim - 1]
        pres[np.isclose(z, z.min()), :om.ndim] = True      # base fixed
        pres[np.isclose(z, z.max()), 3] = True             # drained top
    eq4, nd, nu = OC.coupled_dofs(om, pres)
    prm = np.tile(PRM[kind], (len(om.shape), 1))
    prm[:, 1] *= np.exp(np.random.default_rng(seed).normal(0.0, 0.3, len(om.shape)))
    phi = np.random.default_rng(seed + 1).normal(size=nd)
    return eq4, nd, nu, prm, phi


def _blocks(G, eq4, ndim):
    u = np.sort(eq4[:, :ndim][eq4[:, :ndim] >= 0])
    w = np.sort(eq4[:, 3][eq4[:, 3] >= 0])
    Gd = G.toarray()
    return {"uu": Gd[np.ix_(u, u)], "uw": Gd[np.ix_(u, w)], "wu": Gd[np.ix_(w, u)], "ww": Gd[np.ix_(w, w)]}, u, w


CASES_3D = [(O.HEX20, (2, 2, 1), [[0, 0, 0], [1.0, 0.8, 0.5]]), (O.TET10, (2, 1, 1), [[0, 0, 0], [1.0, 0.5, 0.5]])]
CASES_2D = [(O.QUAD8, (3, 2), [[0, 0], [1.5, 1.0]])]


@pytest.mark.parametrize("shape,n,box", CASES_3D + CASES_2D)
def test_oracle_hydro_mount_properties(shape, n, box):
    om = _oracle_model(shape, n, box, "d3" if len(n) == 3 else "planestrain")
    eq4, nd, nu, prm, phi = _setup(om, OC.HYDRO, with_presc=False)
    gw, dt = 10.0, 0.05
    G, R0 = OC.mount_coupled(om, OC.HYDRO, prm, eq4, nd, dt, np.zeros(nd), gammaw=gw)
    b, u, w = _blocks(G, eq4, om.ndim)
    # u-u: the element stiffnesses added element by element
    Kd = np.zeros((nd, nd))
    for e in range(len(om.shape)):
        Ke, _ = om.elem_stiffness(e)
        nodes = om.conn[om.conn_ptr[e]:om.conn_ptr[e + 1]]
        mu = eq4[nodes][:, :om.ndim].reshape(-1)
        Kd[np.ix_(mu, mu)] += Ke
    assert np.array_equal(b["uu"], Kd[np.ix_(u, u)])
    # symmetric (s = 1); a rigid translation changes no volume
    Gd = G.toarray()
    assert np.abs(Gd - Gd.T).max() <= 1e-12 * np.abs(Gd).max()
    ux = np.zeros(nd)
    ux[eq4[:, 0][eq4[:, 0] >= 0]] = 1.0
    assert np.abs(Gd[w] @ ux).max() <= 1e-12 * np.abs(b["wu"]).max()
    # with the storativity the w-w block sums to dt * 0 - S V
    V = np.prod(np.diff(np.array(box), axis=0))
    S = prm[0, 2]
    assert abs(b["ww"].sum() + S * V) <= 1e-12 * S * V * 1e3
    # without it, H annihilates a constant field
    prm0 = prm.copy()
    prm0[:, 2] = 0.0
    G0, _ = OC.mount_coupled(om, OC.HYDRO, prm0, eq4, nd, dt, np.zeros(nd), gammaw=gw)
    b0, _, _ = _blocks(G0, eq4, om.ndim)
    assert np.abs(b0["ww"].sum(axis=1)).max() <= 1e-12 * np.abs(b0["ww"]).max()
    # fluxes sum to zero; a linear pressure p = z gives (1 + 1/gammaw) times the RHS of p = 0
    assert abs(R0[w].sum()) <= 1e-12 * np.abs(R0).max()
    pz = np.zeros(nd)
    for node in range(om.nnodes):
        if eq4[node, 3] >= 0:
            pz[eq4[node, 3]] = om.coords[node, om.ndim - 1]
    _, Rz = OC.mount_coupled(om, OC.HYDRO, prm, eq4, nd, dt, pz, gammaw=gw)
    assert np.abs(Rz - (1.0 + 1.0 / gw) * R0).max() <= 1e-12 * np.abs(R0).max()


@pytest.mark.parametrize("shape,n,box", CASES_3D + CASES_2D)
def test_oracle_thermo_mount_properties(shape, n, box):
    om = _oracle_model(shape, n, box, "d3" if len(n) == 3 else "planestress")
    eq4, nd, nu, prm, phi = _setup(om, OC.THERMO, with_presc=False)
    T0 = 20.0
    G, R = OC.mount_coupled(om, OC.THERMO, prm, eq4, nd, 0.5, phi, T0=T0)
    b, u, w = _blocks(G, eq4, om.ndim)
    assert np.abs(b["wu"] - (T0 + 273.15) * b["uw"].T).max() <= 1e-12 * np.abs(b["wu"]).max()
    # a uniform temperature loads the skeleton with forces that sum to zero (sum of gradients)
    f = b["uw"] @ np.ones(len(w))
    ax = [np.where(np.isin(u, eq4[:, c][eq4[:, c] >= 0]))[0] for c in range(om.ndim)]
    for idx in ax:
        assert abs(f[idx].sum()) <= 1e-12 * np.abs(f).max() * len(f)
    # the RHS is -dt H phi only: with phi constant it vanishes
    _, R1 = OC.mount_coupled(om, OC.THERMO, prm, eq4, nd, 0.5, np.ones(nd), T0=T0)
    assert np.abs(R1).max() <= 1e-12 * np.abs(R).max()


# ---------------------------------------------------------------------------------------------- GPU


def _pair(shape, n, box, stressmodel):
    om = _oracle_model(shape, n, box, stressmodel)
    kw = dict(nx=n[0], ny=n[1], nz=n[2]) if len(n) == 3 else dict(nx=n[0], ny=n[1])
    mg = A.Mesh(A.Block(box, cellshape=shape, **kw))
    assert (mg.conn == om.conn).all()
    mg.coords = np.ascontiguousarray(om.mesh.coords)
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=1e4, nu=0.25))], A.MechContext(stressmodel=stressmodel))
    return om, gm


@pytest.mark.gpu
@pytest.mark.parametrize("kind,shape,n,box,sm", [
    (OC.HYDRO, O.HEX20, (2, 2, 2), [[0, 0, 0], [1.0, 0.8, 0.6]], "d3"),
    (OC.HYDRO, O.TET10, (2, 2, 1), [[0, 0, 0], [1.0, 0.5, 0.5]], "d3"),
    (OC.HYDRO, O.QUAD4, (4, 3), [[0, 0], [2.0, 1.0]], "planestrain"),
    (OC.THERMO, O.HEX8, (3, 2, 2), [[0, 0, 0], [1.5, 1.0, 1.0]], "d3"),
    (OC.THERMO, O.QUAD8, (4, 3), [[0, 0], [2.0, 1.0]], "planestress"),
])
def test_gpu_coupled_mount_matches_the_oracle(kind, shape, n, box, sm):
    om, gm = _pair(shape, n, box, sm)
    eq4, nd, nu, prm, phi = _setup(om, kind)
    dt, gw, T0 = 0.05, 10.0, 15.0
    Go, Ro = OC.mount_coupled(om, kind, prm, eq4, nd, dt, phi, gammaw=gw, T0=T0)
    Gg, Rg = A.coupled.mount_coupled(gm, kind, prm, eq4, nd, dt, phi, gammaw=gw, T0=T0)
    assert np.array_equal(Gg.indptr, Go.indptr) and np.array_equal(Gg.indices, Go.indices)
    bo, _, _ = _blocks(Go, eq4, om.ndim)
    bg, _, _ = _blocks(Gg, eq4, om.ndim)
    for k in ("uu", "uw", "wu", "ww"):
        assert np.abs(bg[k] - bo[k]).max() <= 1e-12 * np.abs(bo[k]).max(), k
    assert np.abs(Rg - Ro).max() <= 1e-12 * np.abs(Ro).max()
