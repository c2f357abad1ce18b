"""Oracle restatement of Amaru.jl's VTU writer (test infrastructure only).

save_vtu (src/mesh/io.jl:167-274) in ascii format and with compress=true, get_array_node! (:117-158) and
the XML writer (src/tools/xml.jl:250-318), and the node_data / elem_data that update_output_data!
(src/fe-model.jl:341-427) gives a model on this path.  Plain Python string building: meant for small
models.  The compressed form deflates with Python's zlib at level 4 and the zlib stream defaults
(window 15, memory level 8, default strategy), the settings of the reference's ZlibCompressorStream
(CodecZlib).
"""
import struct
import zlib

import numpy as np

TAB = "   "
TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.int32): "Int32", np.dtype(np.int64): "Int64",
         np.dtype(np.uint64): "UInt64"}
VTK = {3: 5, 4: 22, 5: 9, 6: 23, 7: 28, 8: 10, 9: 24, 10: 12, 11: 25, 1: 3, 2: 21}  # shape code -> vtk type


def _float(x):
    """@printf "%20.10e" Float32(x)"""
    f = float(np.float32(x))
    if f != f:
        return "%20s" % "NaN"
    if f in (float("inf"), float("-inf")):
        return "%20s" % ("Inf" if f > 0 else "-Inf")
    return "%20.10e" % f


def array_content(a):
    """get_array_node!'s ascii content: rows joined by newlines, no trailing newline."""
    a = np.asarray(a)
    if a.ndim == 1:
        a = a[:, None]
    isfloat = a.dtype.kind == "f"
    rows = []
    for i in range(a.shape[0]):
        if isfloat:
            rows.append("".join(_float(v) for v in a[i]))
        else:
            rows.append("".join("%d  " % v for v in a[i]))
    return "\n".join(rows)


def data_array(name, a, level):
    """writenode of a DataArray element: header, content lines with their leading blanks replaced by the
    next level's indentation, closing tag."""
    a = np.asarray(a)
    ncomp = 1 if a.ndim == 1 else a.shape[1]
    out = TAB * level + '<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="ascii">\n' % (
        TYPES[a.dtype], name, ncomp)
    content = array_content(a)
    out += "\n".join(TAB * (level + 1) + line.lstrip(" ") for line in content.split("\n")) + "\n"
    out += TAB * level + "</DataArray>\n"
    return out


def appended_array(name, a, level, buf):
    """get_array_node! with compressed=true: a self-closing DataArray with format "appended" and the offset
    of its block in buf, to which it appends the UInt64 header (1, size, size, compressed size) and the
    zlib stream of the array's row-major bytes."""
    a = np.asarray(a)
    ncomp = 1 if a.ndim == 1 else a.shape[1]
    node = TAB * level + '<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="appended" offset="%d"/>\n' % (
        TYPES[a.dtype], name, ncomp, len(buf))
    raw = np.ascontiguousarray(a).tobytes()
    z = zlib.compress(raw, 4)
    buf += struct.pack("<4Q", 1, len(raw), len(raw), len(z)) + z
    return node


def save_vtu(coords, conn_ptr, conn, shapes, node_data, elem_data, compress=False):
    """-> the file's text (bytes when compress).  node_data / elem_data: lists of (name, array) in order."""
    nn, ne = len(coords), len(shapes)
    buf = bytearray()
    if compress:
        def data_array(name, a, level):  # noqa: F811  (the appended form)
            return appended_array(name, a, level, buf)
    else:
        data_array = globals()["data_array"]
    s = '<?xml version="1.0" encoding="UTF-8"?>\n'
    s += "<!-- File generated by Amaru Finite Element Code -->\n"
    s += ('<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64" '
          'compressor="vtkZLibDataCompressor">\n')
    s += TAB + "<UnstructuredGrid>\n"
    s += TAB * 2 + '<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (nn, ne)
    s += TAB * 3 + "<Points>\n" + data_array("Points", np.asarray(coords, dtype=np.float64)[:, :3], 4)
    s += TAB * 3 + "</Points>\n"
    s += TAB * 3 + "<Cells>\n"
    s += data_array("connectivity", np.asarray(conn, dtype=np.int32), 4)
    s += data_array("offsets", np.asarray(conn_ptr[1:], dtype=np.int32), 4)
    s += data_array("types", np.array([VTK[int(t)] for t in shapes], dtype=np.int32), 4)
    s += TAB * 3 + "</Cells>\n"
    for tag, data in (("PointData", node_data), ("CellData", elem_data)):
        if not data:
            continue
        arrs = [(k, np.asarray(v)) for k, v in data if np.asarray(v).size > 0]
        if not arrs:
            s += TAB * 3 + "<%s/>\n" % tag
            continue
        s += TAB * 3 + "<%s>\n" % tag
        for k, v in arrs:
            s += data_array(k, v, 4)
        s += TAB * 3 + "</%s>\n" % tag
    s += TAB * 2 + "</Piece>\n" + TAB + "</UnstructuredGrid>\n"
    if not compress:
        return s + "</VTKFile>\n"
    s += TAB + '<AppendedData encoding="raw">\n'
    return s.encode("utf-8") + b"_" + bytes(buf) + b"\n" + (TAB + "</AppendedData>\n</VTKFile>\n").encode("utf-8")


def output_data(ndim, nnodes, shapes, eq_id, U, F, V_rec, fields):
    """update_output_data!'s node_data and elem_data: node-id, per node the dof values (ux, fx, uy, fy[, uz,
    fz], 0 where a node has no dofs), the recovered fields, U (nnodes x 3); elem-id, cell-type."""
    node = [("node-id", np.arange(1, nnodes + 1, dtype=np.int64))]
    has = eq_id[:, 0] >= 0
    for i, (u, f) in enumerate((("ux", "fx"), ("uy", "fy"), ("uz", "fz"))[:ndim]):
        node.append((u, np.where(has, U[:, i], 0.0)))
        node.append((f, np.where(has, F[:, i], 0.0)))
    for j, k in enumerate(fields):
        node.append((k, np.asarray(V_rec[:, j], dtype=np.float64)))
    Um = np.zeros((nnodes, 3))
    Um[:, :ndim] = np.stack([dict(node)[k] for k in ("ux", "uy", "uz")[:ndim]], 1)
    node.append(("U", Um))
    elem = [("elem-id", np.arange(1, len(shapes) + 1, dtype=np.int64)),
            ("cell-type", np.array([VTK[int(t)] for t in shapes], dtype=np.int64))]
    return node, elem
