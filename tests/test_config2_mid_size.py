"""The mixed-precision solve workload (HEX20 block 10 x 4 x 4, 27 IPs, lognormal E per element from seed
0xA11A, nu = 0.2, base z = 0 fixed, pressure 1.0 on the top) at HEX20 20 x 8 x 8 (19 035 DOFs), the size the
CPU baseline times, against the oracle: mount_K in the reference's operation order (src/mech/elem/
mech-solid.jl:124-166, mech-solver.jl:78-110) exported in the reference's CSC layout, pattern and values bit
for bit; the staged solver's U and F, with the multigrid solver and with block-Jacobi, to 1e-6 of their
maxima against the oracle's direct solve.
"""
import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

pytestmark = pytest.mark.gpu

SEED = 0xA11A
N = (20, 8, 8)


def _models():
    box = [[0, 0, 0], [10.0, 4.0, 4.0]]
    mg = A.Mesh(A.Block(box, nx=N[0], ny=N[1], nz=N[2], cellshape=A.HEX20))
    mo = O.Mesh(O.Block(box, nx=N[0], ny=N[1], nz=N[2], cellshape=O.HEX20))
    # the two meshers agree to 1 ulp on coordinates: the bitwise comparison needs the very same ones
    assert (mg.conn == np.array([v for c in mo.elems for v in c.nodes])).all()
    mg.coords = np.ascontiguousarray(mo.coords)
    E = np.exp(np.random.default_rng(SEED).normal(np.log(30e3), 0.3, len(mg.shape)))
    gm = A.FEModel(mg, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27, E=E)
    om = O.FEModel(mo, [("all", O.LinearElastic(E=30e3, nu=0.2))], nips=27, elem_E=E)
    return om, gm


def _bcs(M):
    return [("z==0", M.SurfaceBC(ux=0, uy=0, uz=0)), ("z==4", M.SurfaceBC(tz=-1.0))]


def test_config2_pattern_and_K_match_the_oracle_bit_for_bit():
    om, gm = _models()
    dofs, nu, _ = O.configure_dofs(om, _bcs(O))
    gm.configure_dofs(_bcs(A))
    assert gm.ndofs == len(dofs) == 19035 and gm.nu == nu
    Ko = O.mount_K(om, len(dofs), 8).tocsc()
    Ko.sort_indices()
    Kg = gm.mount_K(reference_order=True)
    assert np.array_equal(Kg.indptr, Ko.indptr) and np.array_equal(Kg.indices, Ko.indices)
    assert np.array_equal(Kg.data, Ko.data)


@pytest.mark.parametrize("solver", ["amg", "mixed"])
def test_config2_stage_matches_the_oracle(solver):
    om, gm = _models()
    ao, ag = O.MechAnalysis(om), A.MechAnalysis(gm)
    ao.addstage(_bcs(O))
    ag.addstage(_bcs(A))
    assert ao.solve(nthreads=8)[0]
    ok, msg = ag.solve(solver=solver)
    assert ok, msg
    assert np.abs(gm.U - om.U).max() <= 1e-6 * np.abs(om.U).max()
    assert np.abs(gm.F - om.F).max() <= 1e-6 * np.abs(om.F).max()
    # the base reactions balance the 40 units of applied load
    base = gm.mesh.select_nodes("z==0")
    assert abs(gm.F[base, 2].sum() - 40.0) <= 1e-6 * 40.0
