"""Synthetic workloads of the benchmark configurations, built on the Block mesher.

slope_coords: a plane-strain slope extruded along y.  The block [0, L] x [0, W] x
[0, H] is mapped so that its top follows a crest (height H up to x1), a straight
slope down to the toe height Ht at x2, and the toe plateau beyond; every node keeps
x and y and has z scaled by ztop(x) / H.  Interior vertex nodes (on no outer
facet) are then jittered uniformly by up to +-jitter*h per coordinate from a
seed, and every edge node is put back at the midpoint of its two vertices, so the
mesh is no longer structured, its edges stay straight and every boundary node
stays on its plane.
"""
import numpy as np

SLOPE = dict(L=10.0, W=1.7, H=4.0, x1=3.0, x2=6.0, Ht=2.0)


def slope_top(x, L, H, x1, x2, Ht, **_):
    return np.where(x <= x1, H, np.where(x >= x2, Ht, H + (Ht - H) * (x - x1) / (x2 - x1)))


def edge_pairs(coords, elem_nodes, nvert):
    """For a mesh of one quadratic cell type: (local edge node, local vertex a, local vertex b), found from
    the first element, where the edge node sits at the midpoint of the two vertices."""
    e = elem_nodes[0]
    out = []
    for j in range(nvert, len(e)):
        # the closest vertex pair, within a millionth of the edge's length (the mesher rounds coordinates)
        dist, a, b = min((np.abs(coords[e[j]] - 0.5 * (coords[e[a]] + coords[e[b]])).max(), a, b)
                         for a in range(nvert) for b in range(a + 1, nvert))
        if dist > 1e-6 * np.abs(coords[e[a]] - coords[e[b]]).max():
            raise ValueError("edge nodes not at edge midpoints")
        out.append((j, a, b))
    return out


def slope_coords(coords, elem_nodes, boundary_nodes, nvert, nx, ny, nz, seed, jitter=0.1, geom=SLOPE):
    """Slope mapping and interior jitter of a block mesh (nnodes x 3 coords, nelems x nen node table).
    h is the smallest cell size of the mapped block; returns a new coordinate array."""
    c = np.array(coords, dtype=np.float64, copy=True)
    pairs = edge_pairs(c, elem_nodes, nvert)
    c[:, 2] = c[:, 2] * (slope_top(c[:, 0], **geom) / geom["H"])
    h = min(geom["L"] / nx, geom["W"] / ny, geom["Ht"] / nz)
    verts = np.unique(elem_nodes[:, :nvert])
    move = np.zeros(len(c), dtype=bool)
    move[verts] = True
    move[np.asarray(boundary_nodes, dtype=np.int64)] = False
    rng = np.random.default_rng(seed)
    d = rng.uniform(-jitter * h, jitter * h, size=(len(c), 3))
    c[move] += d[move]
    for j, a, b in pairs:
        c[elem_nodes[:, j]] = 0.5 * (c[elem_nodes[:, a]] + c[elem_nodes[:, b]])
    return c


def slope_bcs(mod, q):
    """Base fixed, rollers on the four sides, gravity 20 kN/m3, surcharge q on the crest."""
    g = SLOPE
    return [("z==0", mod.SurfaceBC(ux=0, uy=0, uz=0)),
            ("x==0 || x==%r" % g["L"], mod.SurfaceBC(ux=0)),
            ("y==0 || y==%r" % g["W"], mod.SurfaceBC(uy=0)),
            ("all", mod.BodyC(wz=-20.0)),
            ("z==%r" % g["H"], mod.SurfaceBC(tz=-q))]


def boundary_nodes(mesh):
    """Nodes on outer facets of a mesh (face_nodes table, -1 padded)."""
    f = np.asarray(mesh.face_nodes)
    return np.unique(f[f >= 0])
