"""VTU output: save(model, "file.vtu"; compress) -> save_vtu (src/mesh/io.jl:167-274, ascii or compressed)
with get_array_node! (:117-158) and the XML writer (src/tools/xml.jl:250-318).

The oracle's restatement is pinned by a golden snippet written out from the reference's formatting
rules (Float32 values as "%20.10e", integers followed by two blanks, each row's leading blanks replaced
by the element's indentation, DataArray elements of the ascii format).  The library's writer
(amr_write_vtu) must produce the oracle's bytes: for arrays of every type with NaN, infinities, signed
zeros, subnormal and extreme values, and for a model's whole output data after a solve.  The compressed
form is pinned by its own structure (self-closing appended DataArrays whose offsets walk the blocks, each
block's UInt64 header and a zlib stream that inflates to the array's row-major bytes) and compared byte for
byte with the library's; the tag columns by the reference's encoders applied by hand.
"""
import re
import struct
import zlib
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


def _blocks(doc):
    """(DataArray headers, their decoded arrays' bytes) of a compressed document."""
    head, _, tail = doc.partition(b'<AppendedData encoding="raw">\n_')
    data = tail[:tail.rindex(b"\n   </AppendedData>\n</VTKFile>\n")]
    out = []
    for m in re.finditer(rb'<DataArray type="(\w+)" Name="([^"]*)" NumberOfComponents="(\d+)" format="appended" '
                         rb'offset="(\d+)"/>', head):
        o = int(m.group(4))
        nb, n1, n2, nz = struct.unpack("<4Q", data[o:o + 32])
        raw = zlib.decompress(data[o + 32:o + 32 + nz])
        assert nb == 1 and n1 == n2 == len(raw)
        out.append((m.group(1).decode(), m.group(2).decode(), int(m.group(3)), raw, o + 32 + nz))
    return out, len(data)


def test_oracle_compressed_form_round_trips():
    coords = np.array([[0, 0, 0], [1, 0, 0], [1, 0.5, 0], [0, 0.5, 0]], dtype=float)
    ux = np.array([1e-3, -2.5, np.nan, -0.0])
    vec = np.arange(12.0).reshape(4, 3)
    doc = O.vtu.save_vtu(coords, np.array([0, 4]), np.array([0, 1, 2, 3]), np.array([A.QUAD4]),
                         [("ux", ux), ("v", vec)], [("elem-id", np.array([1], dtype=np.int64))], compress=True)
    blocks, size = _blocks(doc)
    assert [b[1] for b in blocks] == ["Points", "connectivity", "offsets", "types", "ux", "v", "elem-id"]
    assert blocks[-1][4] == size  # the blocks tile the appended data
    assert blocks[0][3] == coords.tobytes() and blocks[5][3] == vec.tobytes()  # row-major, full precision
    assert blocks[4][3] == ux.tobytes() and blocks[3][3] == np.array([9], dtype=np.int32).tobytes()
    assert doc.startswith(GOLDEN_QUAD4[:GOLDEN_QUAD4.index("<Points>")].encode())


def test_tag_columns_use_the_reference_encoders():
    """save_vtu's tag fields: encode_string_to_uint64 of safe_string_cut(tag, 8) (src/tools/encode.jl)."""
    from amaru_gpu.model import vtu_tag_columns
    assert vtu_tag_columns(np.array(["", ""], dtype=object)) == []
    cols = dict(vtu_tag_columns(np.array(["soil", "rock-layer-1", "soil", "abcdefgh"], dtype=object)))
    le = lambda b: int.from_bytes(b, "little")  # noqa: E731
    assert list(cols["tag-s1"]) == [le(b"soil"), le(b"rock-lay"), le(b"soil"), le(b"abcdefgh")]
    assert list(cols["tag-s2"]) == [0, le(b"er-1"), 0, 0]
    assert list(cols["tag"]) == [0, 1, 0, 2] and cols["tag"].dtype == np.int64 and cols["tag-s1"].dtype == np.uint64
    with pytest.raises(ValueError, match="too long"):
        vtu_tag_columns(np.array(["a" * 17], dtype=object))
    with pytest.raises(ValueError):
        vtu_tag_columns(np.array(["abcdefg\u00e9"], dtype=object))  # byte 8 inside a two-byte character


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


@pytest.mark.gpu
def test_gpu_compressed_writer_matches_the_oracle(tmp_path):
    gm = _hex_model()
    nn, ne = gm.nnodes, len(gm.mesh.shape)
    rng = np.random.default_rng(12)
    pts = [("vec", rng.normal(size=(nn, 3))), ("id", np.arange(nn, dtype=np.int64)),
           ("i32", rng.integers(-9, 9, size=nn).astype(np.int32)), ("u64", rng.integers(0, 2 ** 63, size=nn).astype(np.uint64))]
    cells = [("elem-id", np.arange(1, ne + 1, dtype=np.int64)), ("val", rng.normal(size=(ne, 2)))]
    path = tmp_path / "out_z.vtu"
    gm.dev.write_vtu(path, pts, cells, nthreads=3, compress=True)
    want = O.vtu.save_vtu(gm.mesh.coords, gm.mesh.conn_ptr, gm.mesh.conn, gm.mesh.shape, pts, cells, compress=True)
    got = path.read_bytes()
    assert got == want
    blocks, _ = _blocks(got)
    assert blocks[4][3] == np.ascontiguousarray(pts[0][1]).tobytes()


@pytest.mark.gpu
def test_gpu_model_save_compressed_with_tags(tmp_path):
    """A tagged, solved model saved compressed: the oracle's writer on the same output data plus the tag
    columns; the ascii form of the same model carries the same tag columns."""
    mesh = A.Mesh(A.Block([[0, 0], [2.0, 0.5]], nx=8, ny=2, cellshape=A.QUAD8))
    c = mesh.coords[mesh.conn[mesh.conn_ptr[:-1]], 0]
    mesh.tags = np.array(["left" if x < 1.0 else "right-abutment" for x in c], dtype=object)
    gm = A.FEModel(mesh, [("all", A.LinearElastic(E=200e3, nu=0.3))], A.MechContext(stressmodel="planestrain"))
    ana = A.MechAnalysis(gm)
    ana.addstage([("x==0", A.SurfaceBC(ux=0, uy=0)), ("x==2", A.SurfaceBC(ty=-20.0))])
    assert ana.solve()[0]
    V, names = gm.nodal_patch_recovery()
    node, elem = O.vtu.output_data(gm.ndim, gm.nnodes, gm.mesh.shape, gm.eq_id, gm.U, gm.F, V, names)
    elem = elem + A.model.vtu_tag_columns(mesh.tags)
    for compress in (True, False):
        path = tmp_path / ("t%d.vtu" % compress)
        gm.save(path, compress=compress)
        want = O.vtu.save_vtu(gm.mesh.coords, gm.mesh.conn_ptr, gm.mesh.conn, gm.mesh.shape, node, elem,
                              compress=compress)
        assert path.read_bytes() == (want if compress else want.encode("utf-8"))
