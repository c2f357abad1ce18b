"""Writes the golden fixtures of tests/test_golden.py from the oracle.

The oracle is pinned against the reference's known-answer tests (tests/test_oracle_golden.py);
these fixtures freeze its outputs for cases the reference's tests do not cover, so that the CUDA
path is compared with stored values and any drift of the oracle itself shows:

  c1_hex8.npz        benchmark config 1, HEX8 20x4x4 cantilever: K (CSC, reference-order assembly)
                     and the stage's U, F
  tet10_k.npz        TET10 2x2x2 block: K's pattern, where cancellation residues decide the entries
  vm_planestress.npz von Mises plane-stress QUAD8 beam, 4 increments with autoinc: U, F
  recovery.npz       nodal_patch_recovery of seeded IP states on a HEX20 3x2x2 block
  modal_quad4.npz    the 6 lowest frequencies and modes of the QUAD4 plate of test/dynamic/modal.jl
  dyn_solid.npz      test/dynamic/dyn-solid.jl with Rayleigh damping over 6 increments: U, V, A, F

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def c1_hex8():
    mesh = O.Mesh(O.Block([[0, 0, 0], [1.0, 0.2, 0.2]], nx=20, ny=4, nz=4, cellshape=O.HEX8))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=200e3, nu=0.3))])
    bcs = [("x==0", O.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1", O.SurfaceBC(tz=-1.0))]
    dofs, nu, _ = O.configure_dofs(om, bcs)
    K = O.mount_K(om, len(dofs)).tocsc()
    K.sort_indices()
    ana = O.MechAnalysis(om)
    ana.addstage(bcs)
    assert ana.solve()[0]
    return dict(coords=om.coords, colptr=K.indptr, rowval=K.indices, nzval=K.data, U=om.U, F=om.F)


def tet10_k():
    mesh = O.Mesh(O.Block([[0, 0, 0], [1.0, 1.0, 1.0]], nx=2, ny=2, nz=2, cellshape=O.TET10))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=100.0, nu=0.25))])
    dofs, nu, _ = O.configure_dofs(om, [("z==0", O.SurfaceBC(ux=0, uy=0, uz=0))])
    K = O.mount_K(om, len(dofs)).tocsc()
    K.sort_indices()
    return dict(coords=om.coords, colptr=K.indptr, rowval=K.indices, nzval=K.data)


def vm_planestress():
    mesh = O.Mesh(O.Block([[0, 0], [2.0, 0.5]], nx=12, ny=4, cellshape=O.QUAD8))
    om = O.FEModel(mesh, [("all", O.VonMises(E=200e3, nu=0.3, fy=240.0, H=2e3))], stressmodel="planestress")
    ana = O.MechAnalysis(om)
    ana.addstage([("x==0", O.SurfaceBC(ux=0, uy=0)), ("x==2", O.SurfaceBC(ty=-16.0))], nincs=8)
    assert ana.solve()[0]
    assert om.state[:, 12].max() > 0
    return dict(coords=om.coords, U=om.U, F=om.F, iterations=np.array([len(ana.log)]))


def recovery():
    mesh = O.Mesh(O.Block([[0, 0, 0], [1.5, 1.0, 1.0]], nx=3, ny=2, nz=2, cellshape=O.HEX20))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27)
    rng = np.random.default_rng(0x5EED)
    om.state[:, :12] = rng.normal(size=(len(om.state), 12))
    V, names = O.nodal_patch_recovery(om)
    return dict(coords=om.coords, state=om.state, V=V, names=np.array(names))


def modal_quad4():
    mesh = O.Mesh(O.Block([[0, 0], [1.0, 10.0]], nx=4, ny=40, cellshape=O.QUAD4))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=2e6, nu=0.2, rho=15.0))], stressmodel="planestrain")
    w, V, nu = O.modal(om, [("y==0", O.NodeBC(ux=0, uy=0))], 6)
    return dict(coords=om.coords, omega=w, modes=V)


def dyn_solid():
    mesh = O.Mesh(O.Block([[0, 0, 0], [0.2, 2.0, 0.2]], nx=1, ny=10, nz=1, cellshape=O.HEX8))
    om = O.FEModel(mesh, [("all", O.LinearElastic(E=30e6, nu=0.2, rho=24.0))])
    ana = O.DynAnalysis(om)
    ana.addstage([("y==0 && z==0", O.NodeBC(ux=0, uy=0, uz=0)), ("y==2 && z==0", O.NodeBC(uz=0)),
                  ("y==1 && z==0.2", O.NodeBC(fz=-10))], tspan=0.1, nincs=6, nouts=1)
    assert ana.solve(alpha=4.2038, beta=174.2803e-6)[0]
    return dict(coords=om.coords, U=om.U, V=om.V, A=om.A, F=om.F)


CASES = dict(c1_hex8=c1_hex8, tet10_k=tet10_k, vm_planestress=vm_planestress, recovery=recovery,
             modal_quad4=modal_quad4, dyn_solid=dyn_solid)


def main():
    for name, fn in CASES.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **fn())
        print("wrote", name)


if __name__ == "__main__":
    main()
