"""Pin the CPU oracle against the reference's own known-answer tests.

Each case restates a test script of Amaru.jl (path cited per test) with its
expected values and tolerance.  These run without a GPU.
"""
import numpy as np
import pytest

import oracle as O

BASE_HEX8 = [("x==0 && y==0 && z==0", O.NodeBC(ux=0, uy=0)), ("x==1 && y==0 && z==0", O.NodeBC(uy=0)),
             ("x==0 && y==1 && z==0", O.NodeBC(ux=0)), ("z==0", O.NodeBC(uz=0))]


@pytest.mark.parametrize("case,expected", [
    (("z==1", O.NodeBC(fz=1)), [0, 0, 0, 0, 4.0, 4.0, 4.0, 4.0]),
    (("y==1 && z==1", O.EdgeBC(qy=2)), [0, 0, 0, 0, 3.32088, 3.1998, -4.6002, -4.32047]),
    (("x==1", O.SurfaceBC(tx="3*z")), [0, 0, 0, 0, 1.51044, -2.4501, 1.4499, -2.31023]),
    (("x>=0", O.BodyC(wz=-1)), [0, 0, 0, 0, -0.5, -0.5, -0.5, -0.5]),
])
def test_elastic_hex8(case, expected):
    """test/mech/elem/elastic-hex8.jl:1-86 (Weaver & Johnston), atol 1e-5."""
    mesh = O.Mesh(O.Block([[0, 0, 0], [1, 1, 1]], nx=1, ny=1, nz=1, cellshape=O.HEX8, tag="solid"))
    model = O.FEModel(mesh, [("solid", O.LinearElastic(E=1.0, nu=0.3))])
    ana = O.MechAnalysis(model)
    ana.addstage(BASE_HEX8 + [case], nouts=1)
    assert ana.solve()[0]
    np.testing.assert_allclose(model.U[:, 2], expected, atol=1e-5)


def test_elastic_quad4():
    """test/mech/elem/elastic-quad4.jl:1-53, atol 1e-5."""
    mesh = O.Mesh(O.Block([[0, 0], [1, 1]], nx=1, ny=1, cellshape=O.QUAD4, tag="solid"))
    model = O.FEModel(mesh, [("solid", O.LinearElastic(E=1.0, nu=0.25))], stressmodel="planestrain")
    ana = O.MechAnalysis(model)
    ana.addstage([("x==0.", O.SurfaceBC(ux=0.)), ("y==0.", O.SurfaceBC(uy=0)), ("y==1.", O.SurfaceBC(ty=-1.))])
    assert ana.solve()[0]
    dis = np.array([[0.0, 0.0], [0.3125, 0.0], [0.0, -9.3750e-01], [0.3125, -9.3750e-01]])
    np.testing.assert_allclose(model.U, dis, atol=1e-5)


@pytest.mark.parametrize("shape", [O.TRI3, O.TRI6, O.QUAD4, O.QUAD8, O.QUAD9])
def test_elastic_elems_2d(shape):
    """test/mech/elem/elastic-elems.jl:6-32: top node (ux,uy) ≈ (-0.012,-0.095), atol 4e-2."""
    mesh = O.Mesh(O.Block([[0, 0], [1, 1]], nx=2, ny=2, cellshape=shape, tag="solids"))
    model = O.FEModel(mesh, [("solids", O.LinearElastic(E=100.0, nu=0.2))])
    ana = O.MechAnalysis(model)
    ana.addstage([("y==0", O.SurfaceBC(ux=0, uy=0)), ("y==1", O.SurfaceBC(ty=-10.))])
    assert ana.solve()[0]
    top = mesh.select_nodes("y==1")[0]
    np.testing.assert_allclose(model.U[top], [-0.012, -0.095], atol=4e-2)


@pytest.mark.parametrize("shape", [O.TET4, O.TET10, O.HEX8, O.HEX20])
def test_elastic_elems_3d(shape):
    """test/mech/elem/elastic-elems.jl:35-68: top node (uy,uz) ≈ (-0.012,-0.095), atol 1e-2."""
    mesh = O.Mesh(O.Block([[0, 0, 0], [1, 1, 1]], nx=2, ny=2, nz=2, cellshape=shape, tag="solids"))
    model = O.FEModel(mesh, [("solids", O.LinearElastic(E=100.0, nu=0.2))])
    ana = O.MechAnalysis(model)
    ana.addstage([("z==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("x==0 || x==1", O.SurfaceBC(ux=0)),
                  ("z==1", O.SurfaceBC(tz=-10.))])
    assert ana.solve()[0]
    top = mesh.select_nodes("z==1")[0]
    np.testing.assert_allclose(model.U[top, 1:], [-0.012, -0.095], atol=1e-2)


def test_vm_3d():
    """test/mech/mat/vm-3d.jl:1-44: HEX20 cantilever, von Mises, autoinc; tip fz ≈ -30, atol 0.7."""
    th, E, fy, H, nu = 0.05, 210e6, 240e3, 0.0, 0.3
    mesh = O.Mesh(O.Block([[0, 0, -0.05], [0.05, 1.0, 0.05]], nx=1, ny=50, nz=2, cellshape=O.HEX20))
    model = O.FEModel(mesh, [("all", O.VonMises(E=E, nu=nu, fy=fy, H=H))])
    ana = O.MechAnalysis(model)
    tip = "x==%r && y==1 && z==0" % (th / 2)
    ana.addstage([("y==0", O.NodeBC(uy=0)), ("y==0 && z==0", O.NodeBC(uz=0)),
                  ("x==%r && y==0 && z==0" % (th / 2), O.NodeBC(ux=0)), (tip, O.NodeBC(uz=-0.08))],
                 nincs=20, nouts=1)
    assert ana.solve(autoinc=True)[0]
    n = mesh.select_nodes(tip)
    assert len(n) == 1
    assert abs(model.F[n[0], 2] - (-30)) <= 0.7


def test_vm_2d():
    """test/mech/mat/vm-2d.jl:1-45: QUAD8 plane-stress von Mises cantilever; fy ≈ -30, atol 0.4."""
    h, th, E, fy, H, nu = 0.1, 0.05, 210e6, 240e3, 0.0, 0.3
    mesh = O.Mesh(O.Block([[0, 0], [1.0, h]], nx=50, ny=2, cellshape=O.QUAD8))
    model = O.FEModel(mesh, [("all", O.VonMises(E=E, nu=nu, fy=fy, H=H))], stressmodel="planestress",
                      thickness=th)
    ana = O.MechAnalysis(model)
    ana.addstage([("x==0", O.NodeBC(ux=0)), ("x==0 && y==%r" % (h / 2), O.NodeBC(uy=0)),
                  ("x==1.0 && y==%r" % (h / 2), O.NodeBC(uy=-0.08))], nincs=30, nouts=1)
    assert ana.solve(autoinc=True)[0]
    n = mesh.select_nodes("y==%r && x==1" % (h / 2))
    assert abs(model.F[n[0], 1] - (-30)) <= 0.4


def test_dp_two_stages():
    """test/mech/mat/dp.jl:1-43: HEX8 Drucker-Prager, load/unload stages, tol=1e-2, autoinc -> success."""
    mesh = O.Mesh(O.Block([[0, 0, 0], [1, 1, 0.5]], nx=2, ny=2, nz=2, tag="solids"))
    model = O.FEModel(mesh, [("solids", O.DruckerPrager(E=100., nu=0.25, alpha=0.05, kappa=0.1))])
    ana = O.MechAnalysis(model)
    bcs = [("z==0.0", O.NodeBC(ux=0, uy=0, uz=0)), ("z==0.5", O.NodeBC(uz=-0.033)),
           ("x==0 || x==1.0", O.NodeBC(ux=0, uy=0)), ("y==0 || y==1.0", O.NodeBC(ux=0, uy=0))]
    ana.addstage(bcs, nincs=10)
    bcs2 = list(bcs)
    bcs2[1] = ("z==0.5", O.NodeBC(uz=+0.008))
    ana.addstage(bcs2, nincs=10)
    assert ana.solve(tol=1e-2, autoinc=True)[0]
    assert model.state[:, O.ST_LEN - 4].max() > 0  # plastic flow happened (εpa > 0)


@pytest.mark.parametrize("shape,n,nodes", [
    (O.TRI3, (10, 10), 221), (O.TRI6, (10, 10), 441), (O.QUAD4, (10, 10), 121), (O.QUAD8, (10, 10), 341),
    (O.QUAD9, (10, 10), 441), (O.HEX8, (10, 10, 10), 1331), (O.HEX20, (10, 10, 10), 4961),
    (O.TET4, (10, 10, 10), 1331), (O.TET10, (10, 10, 10), 9261),
])
def test_structured_node_counts(shape, n, nodes):
    """test/mesh/structured.jl:7-63 node counts."""
    if len(n) == 2:
        bl = O.Block([[0, 0], [1, 1]], nx=n[0], ny=n[1], cellshape=shape)
    else:
        bl = O.Block([[0, 0, 0], [1, 1, 1]], nx=n[0], ny=n[1], nz=n[2], cellshape=shape)
    assert len(O.Mesh(bl).coords) == nodes


@pytest.mark.parametrize("shape", [O.TRI3, O.TRI6, O.QUAD4, O.QUAD8, O.QUAD9, O.TET4, O.TET10, O.HEX8, O.HEX20])
def test_shape_functions(shape):
    """test/mesh/shape/shape_deriv.jl: N(node_i)=e_i, sum N = 1 at the IPs, dN/dR matches a
    central finite difference (1e-6)."""
    R, W = O.quadrature(shape, 0)
    nd = O.SHAPE_NDIM[shape]
    for r in R:
        assert abs(O.shape_func(shape, r[:nd]).sum() - 1.0) < 1e-10
        D = O.shape_deriv(shape, r[:nd])
        h = 1e-6
        for k in range(nd):
            rp = r[:nd].copy(); rm = r[:nd].copy()
            rp[k] += h; rm[k] -= h
            fd = (O.shape_func(shape, rp) - O.shape_func(shape, rm)) / (2 * h)
            np.testing.assert_allclose(D[:, k], fd, atol=1e-6)


@pytest.mark.parametrize("shape", [O.TRI3, O.TRI6, O.QUAD4, O.QUAD8])
def test_axisymmetric(shape):
    """test/mech/elem/axisymmetric.jl: the axisymmetric block [0,1]^2 (4x4 cells, E=100, nu=0.2, axis x=0 with
    ux=0, base uy=0, ty=-10 on top) equals its 3-D revolution at node (1, 1) to 1e-3.  Uniaxial compression is
    homogeneous, so both equal the exact u_r = nu*10/E = 0.02, u_y = -10/E = -0.1, which the restatement must
    give."""
    mesh = O.Mesh(O.Block([[0, 0], [1, 1]], nx=4, ny=4, cellshape=shape))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=100.0, nu=0.2))], stressmodel="axisymmetric")
    ana = O.MechAnalysis(om)
    ana.addstage([("x==0", O.SurfaceBC(ux=0)), ("y==0", O.SurfaceBC(uy=0)), ("y==1", O.SurfaceBC(ty=-10))])
    assert ana.solve()[0]
    n = mesh.select_nodes("x==1 && y==1")[0]
    np.testing.assert_allclose(om.U[n, :2], [0.02, -0.1], atol=1e-3)


@pytest.mark.parametrize("shape,n,box", [(O.HEX8, (4, 2, 2), [[0, 0, 0], [1, 0.2, 0.2]]),
                                         (O.HEX20, (3, 2, 2), [[0, 0, 0], [1, 0.4, 0.4]]),
                                         (O.TET10, (2, 2, 2), [[0, 0, 0], [1, 0.5, 0.5]]),
                                         (O.TET4, (3, 2, 2), [[0, 0, 0], [1, 0.5, 0.5]]),
                                         (O.QUAD8, (4, 3), [[0, 0], [1, 0.5]])])
def test_K_symmetry_and_its_one_sided_residues(shape, n, box):
    """mount_K (src/mech/mech-solver.jl:78-110) drops element entries below eps() before summing, and Ke_ij and
    Ke_ji are separate floating-point sums, so the stored pattern is not always structurally symmetric: a
    cancellation residue can survive on one side only.  Pinned: the values are symmetric to round-off, every
    position stored on one side only holds a residue (below 1e-14 of max|K|), and the shapes without such
    cancellations (HEX8, TET4) have a symmetric pattern.  CSR(K) is therefore not CSC(K) reinterpreted;
    the library exports the reference's own CSC layout."""
    import scipy.sparse as sp
    m = O.Mesh(O.Block(box, nx=n[0], ny=n[1], nz=n[2] if len(n) > 2 else 0, cellshape=shape))
    om = O.FEModel(m, [("all", O.LinearElastic(E=200e3, nu=0.3))], stressmodel="d3" if len(n) == 3 else "planestrain")
    dofs, nu, _ = O.configure_dofs(om, [])
    K = O.mount_K(om, len(dofs)).tocsc()
    kmax = np.abs(K.data).max()
    assert abs(K - K.T).max() <= 1e-15 * kmax
    S = sp.csc_matrix((np.ones(K.nnz), K.indices, K.indptr), shape=K.shape)
    A = (S - S.T).tocoo()
    one_sided = [(i, j) for i, j, v in zip(A.row, A.col, A.data) if v > 0]
    assert all(abs(K[i, j]) <= 1e-14 * kmax for i, j in one_sided)
    if shape in (O.HEX8, O.TET4):
        assert not one_sided
    else:
        assert one_sided
