"""VTU output: save(model, "file.vtu") -> save_vtu (src/mesh/io.jl:167-274, ascii) with get_array_node!
(:117-158) and the XML writer (src/tools/xml.jl:250-318).

The oracle's restatement is pinned by a golden snippet written out from the reference's formatting
rules (Float32 values as "%20.10e", integers followed by two blanks, each row's leading blanks replaced
by the element's indentation, DataArray elements of the ascii format).  The library's writer
(amr_write_vtu) must produce the oracle's bytes: for arrays of every type with NaN, infinities, signed
zeros, subnormal and extreme values, and for a model's whole output data after a solve.
"""
import os

import numpy as np
import pytest

import amaru_gpu as A
import oracle as O

GOLDEN_QUAD4 = """<?xml version="1.0" encoding="UTF-8"?>
<!-- File generated by Amaru Finite Element Code -->
<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64" compressor="vtkZLibDataCompressor">
   <UnstructuredGrid>
      <Piece NumberOfPoints="4" NumberOfCells="1">
         <Points>
            <DataArray type="Float64" Name="Points" NumberOfComponents="3" format="ascii">
               0.0000000000e+00    0.0000000000e+00    0.0000000000e+00
               1.0000000000e+00    0.0000000000e+00    0.0000000000e+00
               1.0000000000e+00    5.0000000000e-01    0.0000000000e+00
               0.0000000000e+00    5.0000000000e-01    0.0000000000e+00
            </DataArray>
         </Points>
         <Cells>
            <DataArray type="Int32" Name="connectivity" NumberOfComponents="1" format="ascii">
               0{sp}
               1{sp}
               2{sp}
               3{sp}
            </DataArray>
            <DataArray type="Int32" Name="offsets" NumberOfComponents="1" format="ascii">
               4{sp}
            </DataArray>
            <DataArray type="Int32" Name="types" NumberOfComponents="1" format="ascii">
               9{sp}
            </DataArray>
         </Cells>
         <PointData>
            <DataArray type="Float64" Name="ux" NumberOfComponents="1" format="ascii">
               1.0000000475e-03
               -2.5000000000e+00
               NaN
               -0.0000000000e+00
            </DataArray>
         </PointData>
         <CellData>
            <DataArray type="Int64" Name="elem-id" NumberOfComponents="1" format="ascii">
               1{sp}
            </DataArray>
         </CellData>
      </Piece>
   </UnstructuredGrid>
</VTKFile>
""".format(sp="  ")  # integer entries end with two blanks


def test_oracle_writer_matches_the_golden_snippet():
    coords = np.array([[0, 0, 0], [1, 0, 0], [1, 0.5, 0], [0, 0.5, 0]], dtype=float)
    txt = O.vtu.save_vtu(coords, np.array([0, 4]), np.array([0, 1, 2, 3]), np.array([A.QUAD4]),
                         [("ux", np.array([1e-3, -2.5, np.nan, -0.0]))], [("elem-id", np.array([1], dtype=np.int64))])
    assert txt == GOLDEN_QUAD4


def test_oracle_float_format():
    f = O.vtu._float
    assert f(0.1) == "    1.0000000149e-01"  # Float32(0.1) = 0.100000001490116..., to 11 digits
    assert f(np.inf) == "                 Inf" and f(-np.inf) == "                -Inf"
    assert f(1e-45) == "    1.4012984643e-45" and f(3.4e38) == "    3.3999999521e+38"


# ---------------------------------------------------------------------------------------------- GPU


def _hex_model(n=(3, 2, 2)):
    mesh = A.Mesh(A.Block([[0, 0, 0], [1.5, 1.0, 1.0]], nx=n[0], ny=n[1], nz=n[2], cellshape=A.HEX20))
    return A.FEModel(mesh, [("all", A.LinearElastic(E=30e3, nu=0.2))], nips=27)


@pytest.mark.gpu
def test_gpu_writer_matches_the_oracle_on_every_type(tmp_path):
    gm = _hex_model()
    nn, ne = gm.nnodes, len(gm.mesh.shape)
    rng = np.random.default_rng(11)
    f = rng.normal(size=(nn, 3)) * 10.0 ** rng.integers(-40, 38, size=(nn, 3))
    f[:6, 0] = [np.nan, np.inf, -np.inf, -0.0, 1e-45, 3.4e38]
    pts = [("vec", f), ("s", rng.normal(size=nn)), ("id", np.arange(nn, dtype=np.int64) - 5),
           ("i32", rng.integers(-2 ** 31, 2 ** 31 - 1, size=nn).astype(np.int32)),
           ("u64", rng.integers(0, 2 ** 63, size=nn).astype(np.uint64)), ("empty", np.zeros((0,)))]
    cells = [("elem-id", np.arange(1, ne + 1, dtype=np.int64)), ("val", rng.normal(size=(ne, 2)))]
    path = tmp_path / "out.vtu"
    gm.dev.write_vtu(path, [p for p in pts if p[1].size], cells, nthreads=3)
    want = O.vtu.save_vtu(gm.mesh.coords, gm.mesh.conn_ptr, gm.mesh.conn, gm.mesh.shape,
                          [p for p in pts if p[1].size], cells)
    assert path.read_bytes() == want.encode("utf-8")


@pytest.mark.gpu
def test_gpu_model_save_matches_the_oracle(tmp_path):
    """A solved model's output (dof values, recovered fields, U) written by FEModel.save equals the oracle's
    writer on the same arrays."""
    gm = _hex_model((6, 2, 2))
    ana = A.MechAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0, uy=0, uz=0)), ("x==1.5", A.SurfaceBC(tz=-1.0))])
    assert ana.solve()[0]
    path = tmp_path / "model.vtu"
    gm.save(path)
    V, names = gm.nodal_patch_recovery()
    node, elem = O.vtu.output_data(gm.ndim, gm.nnodes, gm.mesh.shape, gm.eq_id, gm.U, gm.F, V, names)
    want = O.vtu.save_vtu(gm.mesh.coords, gm.mesh.conn_ptr, gm.mesh.conn, gm.mesh.shape, node, elem)
    got = path.read_bytes()
    assert got == want.encode("utf-8")
    assert b'Name="\xcf\x83vm"' in got and os.path.getsize(path) > 10000


@pytest.mark.gpu
def test_gpu_model_save_2d_matches_the_oracle(tmp_path):
    """A plane-strain QUAD8 model: points with z = 0, two dof components, the 2-D field list."""
    mesh = A.Mesh(A.Block([[0, 0], [2.0, 0.5]], nx=8, ny=2, cellshape=A.QUAD8))
    gm = A.FEModel(mesh, [("all", A.VonMises(E=200e3, nu=0.3, fy=240.0, H=2e3))],
                   A.MechContext(stressmodel="planestrain"))
    ana = A.MechAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(ty=-20.0))], nincs=3)
    assert ana.solve(autoinc=True)[0]
    path = tmp_path / "model2d.vtu"
    gm.save(path)
    V, names = gm.nodal_patch_recovery()
    assert "ep" in names and "σ2" not in names
    node, elem = O.vtu.output_data(gm.ndim, gm.nnodes, gm.mesh.shape, gm.eq_id, gm.U, gm.F, V, names)
    want = O.vtu.save_vtu(gm.mesh.coords, gm.mesh.conn_ptr, gm.mesh.conn, gm.mesh.shape, node, elem)
    assert path.read_bytes() == want.encode("utf-8")
