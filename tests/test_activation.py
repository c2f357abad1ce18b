"""Element activation: elem.active and a stage's toactivate (src/mech/mech-solver.jl:216-220).

mech_stage_solver! activates the stage's toactivate elements, assembles and updates only the active ones
(mount_K(active_elems), update_state!(active_elems)), and configure_dofs! numbers only the nodes of active
elements (src/bc.jl:200-203); element conditions select among the active elements (bc.jl:159).  A node of
no active element keeps eq_id 0 (src/dof.jl:15-17), so a boundary condition that reaches it fails in the
reference (a BoundsError); the oracle and the library raise.  The reference's tests hold no activation case,
so the oracle is pinned by the element-by-element definition of the active assembly and by the loads; the
CUDA path (a device model over the active elements, rebuilt when the set changes, the IP states carried
with their elements) is compared with the oracle over a three-stage construction sequence, and its output
(recovery) covers every element, as update_output_data! does.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

BOX = [[0, 0], [4.0, 2.0]]
N = (8, 4)
VM = dict(E=2e4, nu=0.3, fy=12.0, H=200.0)


def _oracle(shape=O.QUAD8, mat=None):
    mesh = O.Mesh(O.Block(BOX, nx=N[0], ny=N[1], cellshape=shape))
    return O.FEModel(mesh, [("all", (mat or O.LinearElastic)(**(VM if mat else dict(E=2e4, nu=0.3))))],
                     stressmodel="planestrain")


def _upper(model):
    """The elements whose centroid lies above y = 1 (the second lift of an embankment)."""
    c = np.array([model.coords[model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]], 1].mean()
                  for e in range(len(model.shape))])
    return np.nonzero(c > 1.0)[0]


def test_oracle_active_assembly_is_the_active_elements_only():
    om = _oracle()
    up = _upper(om)
    om.active[up] = False
    dofs, nu, _ = O.configure_dofs(om, [("y==0", O.NodeBC(ux=0, uy=0))])
    nodes = om.active_nodes()
    assert np.all(om.coords[nodes, 1] <= 1.0 + 1e-12) and len(dofs) == 2 * len(nodes)
    assert (om.eq_id[np.setdiff1d(np.arange(om.nnodes), nodes), :2] == -1).all()
    assert [d[0] for d in dofs[:nu]] == sorted([d[0] for d in dofs[:nu]])  # node order within the unknowns
    nd = len(dofs)
    K = O.mount_K(om, nd).toarray()
    Kd = np.zeros((nd, nd))
    for e in np.nonzero(om.active)[0]:
        Ke, mp = om.elem_stiffness(e)
        Ke = np.where(np.abs(Ke) >= np.finfo(float).eps, Ke, 0.0)
        Kd[np.ix_(mp, mp)] += Ke
    assert np.abs(K - Kd).max() <= 1e-12 * np.abs(Kd).max()


def test_oracle_body_load_and_bc_rules():
    om = _oracle()
    up = _upper(om)
    om.active[up] = False
    # gravity over "all" acts on the active elements only: total = -(active area)
    dofs, nu, setup = O.configure_dofs(om, [("y==0", O.NodeBC(ux=0, uy=0)), ("all", O.BodyC(wy=-1.0))])
    _, F = O.get_bc_vals(om, setup, len(dofs))
    ydofs = [i for i, d in enumerate(dofs) if d[1] == 1]
    assert abs(F[ydofs].sum() + 4.0 * 1.0) <= 1e-12
    # a condition on a node of no active element fails, as the reference's U[dof.eq_id] does
    dofs, nu, setup = O.configure_dofs(om, [("y==0", O.NodeBC(ux=0, uy=0)), ("y==2", O.NodeBC(uy=-0.1))])
    with pytest.raises(ValueError, match="no active element"):
        O.get_bc_vals(om, setup, len(dofs))


def test_oracle_stage_activation():
    """toactivate takes effect before the stage's numbering; the newly active elements start from their
    initial (zero) IP states while the others carry theirs."""
    om = _oracle(mat=O.VonMises)
    up = _upper(om)
    om.active[up] = False
    ana = O.MechAnalysis(om)
    ana.addstage([("y==0", O.NodeBC(ux=0, uy=0)), ("all", O.BodyC(wy=-10.0))], nincs=2)
    ana.addstage([("y==0", O.NodeBC(ux=0, uy=0)), ("y>=1", O.BodyC(wy=-10.0))], nincs=2, toactivate=up)
    S1 = None

    def rec(a, T, checkpoint):
        nonlocal S1
        if S1 is None and T == 1.0:
            S1 = om.state.copy()

    assert ana.solve(tol=1e-6, record=rec)[0]
    assert om.active.all()
    rows = np.concatenate([np.arange(om.ip_ptr[e], om.ip_ptr[e + 1]) for e in up])
    assert (S1[rows] == 0).all() and np.abs(om.state[rows]).max() > 0
    assert np.abs(om.U[om.coords[:, 1] > 1.0 + 1e-12]).max() > 0


# ---------------------------------------------------------------------------------------------- GPU


def _pair(shape, mat):
    mo = O.Mesh(O.Block(BOX, nx=N[0], ny=N[1], cellshape=shape))
    mg = A.Mesh(A.Block(BOX, nx=N[0], ny=N[1], cellshape=shape))
    assert (mg.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    mg.coords = np.ascontiguousarray(mo.coords)
    om = O.FEModel(mo, [("all", getattr(O, mat)(**VM))], stressmodel="planestrain")
    gm = A.FEModel(mg, [("all", getattr(A, mat)(**VM))], A.MechContext(stressmodel="planestrain"))
    return om, gm


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [A.QUAD8, A.QUAD4])
def test_gpu_construction_sequence_matches_the_oracle(shape):
    """Lift 1 under its own weight, lift 2 activated under the weight of both, then a crest surcharge: the
    stage iterations, U, F and every element's IP states (inactive ones included) against the oracle."""
    om, gm = _pair(shape, "VonMises")
    up = _upper(om)
    om.active[up] = False
    gm.set_active(up, False)
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    for api, ana in ((O, ao), (A, ag)):
        base = [("y==0", api.NodeBC(ux=0, uy=0))]
        sides = [("x==0 || x==4", api.NodeBC(ux=0))]
        ana.addstage(base + [("all", api.BodyC(wy=-10.0))], nincs=2)
        ana.addstage(base + sides + [("y>=1", api.BodyC(wy=-10.0))], nincs=2, toactivate=up)
        ana.addstage(base + sides + [("y==2 && x<=1", api.SurfaceBC(ty=-25.0))], nincs=4)
    assert ao.solve(tol=1e-6, autoinc=True)[0]
    assert ag.solve(tol=1e-6, autoinc=True, solver="fp64", linear_rtol=1e-12)[0]
    assert gm.active.all() and om.active.all()
    its_o = [sum(1 for r in ao.log if r[0] is st) for st in ao.stages]
    its_g = [sum(1 for r in ag.log if r[0] is st) for st in ag.stages]
    assert its_o == its_g
    scale = np.abs(om.U).max()
    assert np.abs(gm.U - om.U).max() <= 1e-8 * scale
    assert np.abs(gm.F - om.F).max() <= 1e-8 * np.abs(om.F).max()
    S = gm.state()
    assert np.abs(S[:, :12] - om.state[:, :12]).max() <= 1e-8 * np.abs(om.state[:, :12]).max()
    assert S[:, 12].max() > 0  # the surcharge yields the crest


@pytest.mark.gpu
def test_gpu_inactive_elements_keep_their_states_and_output_covers_them():
    om, gm = _pair(A.QUAD8, "VonMises")
    up = _upper(om)
    om.active[up] = False
    gm.set_active(up, False)
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    for api, ana in ((O, ao), (A, ag)):
        ana.addstage([("y==0", api.NodeBC(ux=0, uy=0)), ("all", api.BodyC(wy=-10.0))], nincs=2)
    assert ao.solve(tol=1e-6)[0] and ag.solve(tol=1e-6, solver="fp64", linear_rtol=1e-12)[0]
    S = gm.state()
    rows_up = np.concatenate([np.arange(om.ip_ptr[e], om.ip_ptr[e + 1]) for e in up])
    assert (S[rows_up] == 0).all() and np.abs(S).max() > 0
    assert (gm.eq_id[gm.mesh.coords[:, 1] > 1.0 + 1e-12] == -1).all()
    # the device model holds the active elements; recovery and the output data cover every element
    assert gm.dev.sizes()["nelems"] == len(om.shape) - len(up)
    om.state[:] = S
    Vo, no = O.nodal_patch_recovery(om)
    Vg, ng = gm.nodal_patch_recovery()
    assert ng == no
    for j in range(len(no)):
        assert np.abs(Vg[:, j] - Vo[:, j]).max() <= 1e-9 * max(np.abs(Vo[:, j]).max(), 1e-300)
    node, elem = gm.update_output_data()
    assert len(elem["elem-id"]) == len(om.shape)
    # a condition on a node of no active element is refused, as in the reference
    ag.addstage([("y==2", A.NodeBC(uy=-0.1))])
    with pytest.raises(ValueError, match="no active element"):
        ag.solve()
