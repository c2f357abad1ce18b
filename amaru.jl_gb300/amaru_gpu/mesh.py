"""Structured block meshes with Amaru's node and element numbering, vectorised.

Block / Mesh follow src/mesh/block.jl:42-182 and split_block!
(src/mesh/structured.jl:37-554) + synchronize! (src/mesh/mesh.jl:335-394):
nodes are numbered in generation order (i fastest, then j, then k; points on
block boundaries are de-duplicated by rounded coordinates), elements in
generation order, and the outer facets in first-occurrence order
(get_outer_facets, src/mesh/mesh.jl:69-85).  The numbering fixes the DOF
order and therefore the sparsity pattern of K.
"""
import numpy as np

from . import _lib as L
from .expr import evaluate

NPOINTS = {L.LIN2: 2, L.LIN3: 3, L.TRI3: 3, L.TRI6: 6, L.QUAD4: 4, L.QUAD8: 8, L.QUAD9: 9, L.TET4: 4,
           L.TET10: 10, L.HEX8: 8, L.HEX20: 20}
SHAPE_NDIM = {L.LIN2: 1, L.LIN3: 1, L.TRI3: 2, L.TRI6: 2, L.QUAD4: 2, L.QUAD8: 2, L.QUAD9: 2, L.TET4: 3, L.TET10: 3,
              L.HEX8: 3, L.HEX20: 3}
# facet tables, 0-based local indices (src/shape/solids2d.jl, solids3d.jl)
_F = {
    L.HEX8: (L.QUAD4, [[0, 4, 7, 3], [1, 2, 6, 5], [0, 1, 5, 4], [2, 3, 7, 6], [0, 3, 2, 1], [4, 5, 6, 7]]),
    L.HEX20: (L.QUAD8, [[0, 4, 7, 3, 16, 15, 19, 11], [1, 2, 6, 5, 9, 18, 13, 17], [0, 1, 5, 4, 8, 17, 12, 16],
                        [2, 3, 7, 6, 10, 19, 14, 18], [0, 3, 2, 1, 11, 10, 9, 8], [4, 5, 6, 7, 12, 13, 14, 15]]),
    L.TET4: (L.TRI3, [[0, 3, 2], [0, 1, 3], [0, 2, 1], [1, 2, 3]]),
    L.TET10: (L.TRI6, [[0, 3, 2, 7, 9, 6], [0, 1, 3, 4, 8, 7], [0, 2, 1, 6, 5, 4], [1, 2, 3, 5, 9, 8]]),
    L.QUAD4: (L.LIN2, [[0, 1], [1, 2], [2, 3], [3, 0]]),
    L.QUAD8: (L.LIN3, [[0, 1, 4], [1, 2, 5], [2, 3, 6], [3, 0, 7]]),
    L.QUAD9: (L.LIN3, [[0, 1, 4], [1, 2, 5], [2, 3, 6], [3, 0, 7]]),
    L.TRI3: (L.LIN2, [[0, 1], [1, 2], [2, 0]]),
    L.TRI6: (L.LIN3, [[0, 1, 3], [1, 2, 4], [2, 0, 5]]),
}
FACETS = {k: (fs, np.array(fl)) for k, (fs, fl) in _F.items()}


def _box_shape(ndim, r, s, t=None):
    """Multilinear block map N(r,s[,t]) over the corner points (QUAD4 / HEX8 node order)."""
    if ndim == 2:
        c = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=float)
        return np.stack([0.25 * (1 + r * a) * (1 + s * b) for a, b in c], axis=-1)
    c = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1],
                  [-1, 1, 1]], dtype=float)
    return np.stack([0.125 * (1 + r * a) * (1 + s * b) * (1 + t * d) for a, b, d in c], axis=-1)


class Block:
    """Block(coords; nx, ny, nz, cellshape, tag): a box split into a structured mesh."""

    def __init__(self, coords, nx=0, ny=0, nz=0, cellshape=None, tag=""):
        coords = np.array(coords, dtype=float)
        if coords.shape[1] == 2:
            coords = np.hstack([coords, np.zeros((coords.shape[0], 1))])
        sumy, sumz = np.abs(coords[:, 1]).sum(), np.abs(coords[:, 2]).sum()
        ndim = 3 if sumz != 0 else (2 if sumy != 0 else 1)
        if ndim == 1:
            raise NotImplementedError("1-D blocks are not part of the solid-element path")
        if coords.shape[0] == 2:
            (x1, y1, z1), (x2, y2, z2) = coords
            if ndim == 2:
                coords = np.array([[x1, y1, 0], [x2, y1, 0], [x2, y2, 0], [x1, y2, 0]], dtype=float)
            else:
                coords = np.array([[x1, y1, z1], [x2, y1, z1], [x2, y2, z1], [x1, y2, z1], [x1, y1, z2], [x2, y1, z2],
                                   [x2, y2, z2], [x1, y2, z2]], dtype=float)
        if ndim == 3 and nz == 0:
            nz = 1
        if ny == 0:
            ny = 1
        self.ndim, self.nx, self.ny, self.nz = ndim, int(nx), int(ny), int(nz)
        self.points = coords
        if cellshape is None:
            cellshape = L.HEX8 if ndim == 3 else L.QUAD4
        if SHAPE_NDIM[cellshape] != ndim:
            raise ValueError("cell shape does not match the block dimension")
        self.cellshape, self.tag = cellshape, tag


_ROW_MULT = np.array([0x9E3779B97F4A7C15, 0xC2B2AE3D27D4EB4F, 0x165667B19E3779F9, 0xD6E8FEB86659FD93,
                      0xFF51AFD7ED558CCD, 0xC4CEB9FE1A85EC53, 0x94D049BB133111EB, 0xBF58476D1CE4E5B9,
                      0x2545F4914F6CDD1D], dtype=np.uint64)


def _distinct_rows(rows):
    """For each distinct row of an int64 table: the index of its first occurrence and its count
    (np.unique(rows, axis=0, return_index=True, return_counts=True) up to the order of the distinct
    rows).  Rows are grouped by a 64-bit hash, and the grouping is verified row by row; a hash
    collision falls back to the exact row sort."""
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    if len(rows) == 0 or rows.shape[1] > len(_ROW_MULT):
        _, first, cnt = np.unique(rows, axis=0, return_index=True, return_counts=True)
        return first, cnt
    with np.errstate(over="ignore"):
        h = (rows.view(np.uint64) * _ROW_MULT[:rows.shape[1]]).sum(axis=1, dtype=np.uint64)
        h ^= h >> np.uint64(31)
    order = np.argsort(h)
    hs = h[order]
    start = np.empty(len(hs), dtype=bool)
    start[0] = True
    start[1:] = hs[1:] != hs[:-1]
    starts = np.nonzero(start)[0]
    grp = np.cumsum(start) - 1
    first = np.minimum.reduceat(order, starts)
    if not np.array_equal(rows[order], rows[first[grp]]):
        _, first, cnt = np.unique(rows, axis=0, return_index=True, return_counts=True)
        return first, cnt
    cnt = np.diff(np.append(starts, len(hs)))
    return first, cnt


class Mesh:
    """Mesh(blocks...): nodes (coords), elements (shape, conn), outer facets and edges."""

    def __init__(self, *blocks):
        self.ndim = max(b.ndim for b in blocks)
        self._coords = []
        self._dict = {}
        self._n = 0
        shapes, conns, tags = [], [], []
        for b in blocks:
            sh, cn = self._split(b)
            shapes.append(np.full(len(cn), sh, dtype=np.int32))
            conns.append(cn)
            tags += [b.tag] * len(cn)
        self.coords = np.concatenate(self._coords, axis=0) if self._coords else np.zeros((0, 3))
        self.shape = np.concatenate(shapes)
        self.conn_list = conns
        self.conn_ptr = np.zeros(len(self.shape) + 1, dtype=np.int64)
        self.conn_ptr[1:] = np.cumsum(np.concatenate([np.full(len(c), c.shape[1]) for c in conns]))
        self.conn = np.concatenate([c.reshape(-1) for c in conns]).astype(np.int64)
        self.tags = np.array(tags, dtype=object)
        self._facets()

    @classmethod
    def join(cls, meshes):
        """Meshes side by side as one mesh, without merging any nodes: mesh i's nodes and
        elements follow those of meshes 0..i-1.  Returns (mesh, node offsets, element offsets);
        the offsets have len(meshes)+1 entries."""
        meshes = list(meshes)
        if not meshes:
            raise ValueError("Mesh.join needs at least one mesh")
        noff = np.zeros(len(meshes) + 1, dtype=np.int64)
        eoff = np.zeros(len(meshes) + 1, dtype=np.int64)
        noff[1:] = np.cumsum([len(m.coords) for m in meshes])
        eoff[1:] = np.cumsum([len(m.shape) for m in meshes])

        def shift(a, o):
            return np.where(a >= 0, a + o, a)

        out = cls.__new__(cls)
        out.ndim = max(m.ndim for m in meshes)
        out.coords = np.concatenate([m.coords for m in meshes], axis=0)
        out.shape = np.concatenate([m.shape for m in meshes])
        out.conn_list = [c + noff[i] for i, m in enumerate(meshes) for c in m.conn_list]
        out.conn_ptr = np.zeros(len(out.shape) + 1, dtype=np.int64)
        out.conn_ptr[1:] = np.cumsum(np.concatenate([np.diff(m.conn_ptr) for m in meshes]))
        out.conn = np.concatenate([m.conn + noff[i] for i, m in enumerate(meshes)])
        out.tags = np.concatenate([m.tags for m in meshes])
        out.faces = []
        w = max(m.face_nodes.shape[1] for m in meshes)
        out.face_nodes = np.concatenate([np.pad(shift(m.face_nodes, noff[i]), ((0, 0), (0, w - m.face_nodes.shape[1])),
                                                constant_values=-1) for i, m in enumerate(meshes)])
        out.face_shape = np.concatenate([m.face_shape for m in meshes])
        out.face_owner = np.concatenate([m.face_owner + eoff[i] for i, m in enumerate(meshes)])
        w = max(m.edge_nodes.shape[1] for m in meshes)
        out.edge_nodes = np.concatenate([np.pad(shift(m.edge_nodes, noff[i]), ((0, 0), (0, w - m.edge_nodes.shape[1])),
                                                constant_values=-1) for i, m in enumerate(meshes)])
        out.edge_shape = np.concatenate([m.edge_shape for m in meshes])
        return out, noff, eoff

    # -- node creation with de-duplication on block boundaries
    def _add_nodes(self, C, boundary):
        ids = np.empty(len(C), dtype=np.int64)
        C = np.array(C, dtype=float)
        if boundary.any():
            C[boundary] = np.round(C[boundary], 8)
        bidx = np.nonzero(boundary)[0]
        existing = np.full(len(C), -1, dtype=np.int64)
        keys = [(C[q, 0] + 1.0, C[q, 1] + 2.0, C[q, 2] + 3.0) for q in bidx]
        if self._dict:
            for q, key in zip(bidx, keys):
                hit = self._dict.get(key)
                if hit is not None:
                    existing[q] = hit
        new = existing < 0
        nnew = int(new.sum())
        ids[new] = self._n + np.arange(nnew)
        ids[~new] = existing[~new]
        for q, key in zip(bidx, keys):
            if new[q]:
                self._dict[key] = int(ids[q])
        self._n += nnew
        if nnew:
            self._coords.append(C[new])
        return ids

    def _split(self, b):
        sh = b.cellshape
        P = b.points
        nx, ny, nz = b.nx, b.ny, b.nz
        if b.ndim == 2:
            q = 2 if sh in (L.QUAD8, L.QUAD9, L.TRI6) else 1
            mx, my = q * nx, q * ny
            j, i = np.meshgrid(np.arange(my + 1), np.arange(mx + 1), indexing="ij")
            i, j = i.ravel(), j.ravel()
            keep = np.ones(i.shape, dtype=bool)
            if sh == L.QUAD8:
                keep = ~((i % 2 == 1) & (j % 2 == 1))
            i, j = i[keep], j[keep]
            if sh == L.TRI6:  # structured.jl:342-343
                r = (1.0 / nx) * i - 1.0
                s = (1.0 / ny) * j - 1.0
            else:
                r = -1.0 + 2.0 * ((1.0 / mx) * i)
                s = -1.0 + 2.0 * ((1.0 / my) * j)
            C = _box_shape(2, r, s) @ P
            bnd = (i == 0) | (i == mx) | (j == 0) | (j == my)
            ids = self._add_nodes(C, bnd)
            g = -np.ones((mx + 1, my + 1), dtype=np.int64)
            g[i, j] = ids
            if sh in (L.QUAD4, L.TRI3):
                jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
                ii, jj = ii.ravel(), jj.ravel()
                p1, p2, p3, p4 = g[ii, jj], g[ii + 1, jj], g[ii + 1, jj + 1], g[ii, jj + 1]
                if sh == L.QUAD4:
                    return sh, np.stack([p1, p2, p3, p4], axis=1)
                cc = self.coords_of([p1, p2, p3, p4])
                center = (cc[0] + cc[1] + cc[2] + cc[3]) / 4
                p5 = self._add_nodes(center, np.zeros(len(center), dtype=bool))
                for q5, c5 in zip(p5, center):
                    self._dict[(c5[0] + 1.0, c5[1] + 2.0, c5[2] + 3.0)] = q5
                tris = np.stack([np.stack([p1, p2, p5], 1), np.stack([p2, p3, p5], 1), np.stack([p3, p4, p5], 1),
                                 np.stack([p4, p1, p5], 1)], axis=1)
                return sh, tris.reshape(-1, 3)
            jj, ii = np.meshgrid(np.arange(0, my, 2), np.arange(0, mx, 2), indexing="ij")
            ii, jj = ii.ravel(), jj.ravel()
            p = [g[ii, jj], g[ii + 2, jj], g[ii + 2, jj + 2], g[ii, jj + 2], g[ii + 1, jj], g[ii + 2, jj + 1],
                 g[ii + 1, jj + 2], g[ii, jj + 1], g[ii + 1, jj + 1]]
            if sh == L.QUAD8:
                return sh, np.stack(p[:8], axis=1)
            if sh == L.QUAD9:
                return sh, np.stack(p, axis=1)
            p1, p2, p3, p4, p5, p6, p7, p8, p9 = p
            tris = np.stack([np.stack([p1, p2, p3, p5, p6, p9], 1), np.stack([p4, p1, p3, p8, p9, p7], 1)], axis=1)
            return sh, tris.reshape(-1, 6)
        # 3-D
        q = 2 if sh in (L.HEX20, L.TET10) else 1
        mx, my, mz = q * nx, q * ny, q * nz
        k, j, i = np.meshgrid(np.arange(mz + 1), np.arange(my + 1), np.arange(mx + 1), indexing="ij")
        i, j, k = i.ravel(), j.ravel(), k.ravel()
        if sh == L.HEX20:
            odd = (i % 2) + (j % 2) + (k % 2)
            keep = odd <= 1
            i, j, k = i[keep], j[keep], k[keep]
        r = -1.0 + 2.0 * ((1.0 / mx) * i)
        s = -1.0 + 2.0 * ((1.0 / my) * j)
        t = -1.0 + 2.0 * ((1.0 / mz) * k)
        C = _box_shape(3, r, s, t) @ P
        bnd = (i == 0) | (i == mx) | (j == 0) | (j == my) | (k == 0) | (k == mz)
        ids = self._add_nodes(C, bnd)
        g = -np.ones((mx + 1, my + 1, mz + 1), dtype=np.int64)
        g[i, j, k] = ids
        step = q
        kk, jj, ii = np.meshgrid(np.arange(0, mz, step), np.arange(0, my, step), np.arange(0, mx, step),
                                 indexing="ij")
        ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
        d = step
        p1, p2, p3, p4 = g[ii, jj, kk], g[ii + d, jj, kk], g[ii + d, jj + d, kk], g[ii, jj + d, kk]
        p5, p6, p7, p8 = g[ii, jj, kk + d], g[ii + d, jj, kk + d], g[ii + d, jj + d, kk + d], g[ii, jj + d, kk + d]
        if sh == L.HEX8:
            return sh, np.stack([p1, p2, p3, p4, p5, p6, p7, p8], axis=1)
        if sh == L.TET4:
            tets = [[p2, p4, p1, p8], [p2, p1, p5, p8], [p2, p5, p6, p8], [p2, p6, p7, p8], [p2, p3, p4, p8],
                    [p2, p7, p3, p8]]
            return sh, np.stack([np.stack(t, 1) for t in tets], axis=1).reshape(-1, 4)
        G = lambda a, b, c: g[ii + a, jj + b, kk + c]  # noqa: E731
        p9, p10, p11, p12 = G(1, 0, 0), G(2, 1, 0), G(1, 2, 0), G(0, 1, 0)
        p13, p14, p15, p16 = G(1, 0, 2), G(2, 1, 2), G(1, 2, 2), G(0, 1, 2)
        p17, p18, p19, p20 = G(0, 0, 1), G(2, 0, 1), G(2, 2, 1), G(0, 2, 1)
        if sh == L.HEX20:
            return sh, np.stack([p1, p2, p3, p4, p5, p6, p7, p8, p9, p10, p11, p12, p13, p14, p15, p16, p17, p18, p19,
                                 p20], axis=1)
        p21, p22, p23, p24 = G(0, 1, 1), G(2, 1, 1), G(1, 0, 1), G(1, 2, 1)
        p25, p26, p27 = G(1, 1, 0), G(1, 1, 2), G(1, 1, 1)
        tets = [[p2, p4, p1, p8, p25, p12, p9, p27, p20, p21], [p2, p1, p5, p8, p9, p17, p23, p27, p21, p16],
                [p2, p5, p6, p8, p23, p13, p18, p27, p16, p26], [p2, p6, p7, p8, p18, p14, p22, p27, p26, p15],
                [p2, p3, p4, p8, p10, p11, p25, p27, p24, p20], [p2, p7, p3, p8, p22, p19, p10, p27, p15, p24]]
        return sh, np.stack([np.stack(t, 1) for t in tets], axis=1).reshape(-1, 10)

    def coords_of(self, ids_list):
        allc = np.concatenate(self._coords, axis=0)
        return [allc[np.asarray(ids)] for ids in ids_list]

    # -- outer facets (faces in 3-D, edges in 2-D) and 3-D edges
    def _facets(self):
        fac_nodes, fac_shape, owner = [], [], []
        start = 0
        for cn in self.conn_list:
            sh = int(self.shape[start]) if len(cn) else None
            if sh is None:
                continue
            fs, idx = FACETS[sh]
            f = cn[:, idx]  # (ne, nf, nfn)
            fac_nodes.append(f.reshape(-1, f.shape[2]))
            fac_shape.append(np.full(f.shape[0] * f.shape[1], fs))
            owner.append(np.repeat(np.arange(start, start + len(cn)), f.shape[1]))
            start += len(cn)
        self.faces = []
        self.face_shape = np.zeros(0, dtype=np.int32)
        self.face_owner = np.zeros(0, dtype=np.int64)
        if not fac_nodes:
            return
        # one facet shape per mesh is enough for block meshes of one cell shape
        width = max(f.shape[1] for f in fac_nodes)
        allf = np.full((sum(len(f) for f in fac_nodes), width), -1, dtype=np.int64)
        o = 0
        for f in fac_nodes:
            allf[o:o + len(f), :f.shape[1]] = f
            o += len(f)
        fshape = np.concatenate(fac_shape)
        fowner = np.concatenate(owner)
        first, cnt = _distinct_rows(np.sort(allf, axis=1))
        sel = np.sort(first[cnt == 1])
        self.face_nodes = allf[sel]
        self.face_shape = fshape[sel]
        self.face_owner = fowner[sel]
        if self.ndim == 2:
            self.edge_nodes, self.edge_shape = self.face_nodes, self.face_shape
        else:
            en, es = [], []
            for fs in np.unique(self.face_shape):
                es_shape, eidx = FACETS[int(fs)]
                f = self.face_nodes[self.face_shape == fs][:, :NPOINTS[int(fs)]]
                e = f[:, eidx].reshape(-1, eidx.shape[1])
                en.append(e)
                es.append(np.full(len(e), es_shape))
            e = np.concatenate(en)
            es = np.concatenate(es)
            first, _ = _distinct_rows(np.sort(e, axis=1))
            first = np.sort(first)
            self.edge_nodes, self.edge_shape = e[first], es[first]

    # -- selections
    def select_nodes(self, expr):
        """Node ids satisfying expr (nodes[expr], src/node.jl:191-215)."""
        x, y, z = self.coords[:, 0], self.coords[:, 1], self.coords[:, 2]
        return np.nonzero(np.asarray(evaluate(expr, x=x, y=y, z=z), dtype=bool).reshape(-1))[0]

    def node_mask(self, expr):
        x, y, z = self.coords[:, 0], self.coords[:, 1], self.coords[:, 2]
        return np.asarray(evaluate(expr, x=x, y=y, z=z), dtype=bool).reshape(-1)

    def select_cells(self, nodes2d, expr):
        """Rows of an (n, k) node table whose nodes all satisfy expr (src/mesh/cell.jl:251-271)."""
        if isinstance(expr, str) and expr == "all":
            return np.arange(len(nodes2d))
        ok = self.node_mask(expr)
        valid = nodes2d >= 0
        return np.nonzero(np.all(ok[np.where(valid, nodes2d, 0)] | ~valid, axis=1))[0]

    def elem_nodes(self):
        """(nelems, max nen) node table, -1 padded."""
        w = int(np.diff(self.conn_ptr).max())
        out = -np.ones((len(self.shape), w), dtype=np.int64)
        o = 0
        for cn in self.conn_list:
            out[o:o + len(cn), :cn.shape[1]] = cn
            o += len(cn)
        return out
