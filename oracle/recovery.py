"""Oracle restatement of Amaru.jl's nodal output recovery (test infrastructure only).

nodal_patch_recovery (src/fe-model.jl:504-702): per corner node, a least-squares
polynomial fitted through the IP values of the elements around it (pinv of the
regression matrix, Julia's default cut-off), evaluated at the patch's nodes and
averaged over all patches that reach a node.  The IP values are ip_state_vals of
the three materials on the GPU path (src/mech/mat/linear-elastic.jl:140-164,
von-mises.jl:159-168,330-341, drucker-prager.jl:152-163) over stress_strain_dict
(src/tools/tensors.jl:162-215).  nodal_local_recovery (src/fe-model.jl:705-747)
only has joint elements to work on, none of which are on this path, so it
contributes no field.

Plain Python loops: meant for meshes of a few thousand nodes.
"""
import numpy as np

from .core import AXISYM, D3, PLANESTRESS, DRUCKER_PRAGER, VON_MISES, HEX8, HEX20, QUAD4, QUAD8, QUAD9, TET4, TET10, TRI3, \
    TRI6, quadrature, shape_func

SR2 = 1.4142135623730951  # src/tools/constants.jl:3

# corner points of each cell's basic shape (elem.shape.basic_shape.npoints)
CORNERS = {HEX8: 8, HEX20: 8, TET4: 4, TET10: 4, QUAD4: 4, QUAD8: 4, QUAD9: 4, TRI3: 3, TRI6: 3}

BASE_3D = ["σxx", "σyy", "σzz", "σyz", "σxz", "σxy", "σvm", "σ1", "σ2", "σ3",
           "εxx", "εyy", "εzz", "εyz", "εxz", "εxy"]
BASE_2D = ["σxx", "σyy", "σzz", "σyz", "σxz", "σxy", "σvm", "σ1", "σ3", "εxx", "εyy", "εzz", "εxy"]
BASE_AXI = ["σrr", "σyy", "σtt", "σry", "σvm", "εrr", "εyy", "εtt", "εry"]  # tensors.jl:182-193


def J2(s):
    """src/tools/tensors.jl:24-27"""
    t11, t22, t33, t23, t13, t12 = s[0], s[1], s[2], s[3] / SR2, s[4] / SR2, s[5] / SR2
    return 1 / 6 * ((t11 - t22) ** 2 + (t22 - t33) ** 2 + (t33 - t11) ** 2) + t23 ** 2 + t13 ** 2 + t12 ** 2


def eigvals(s):
    """eigvals(T::Vec6) (src/tools/tensors.jl:80-91): eigenvalues of the full 3x3 tensor, largest first."""
    t11, t22, t33, t23, t13, t12 = s[0], s[1], s[2], s[3] / SR2, s[4] / SR2, s[5] / SR2
    F = np.array([[t11, t12, t13], [t12, t22, t23], [t13, t23, t33]])
    return np.sort(np.linalg.eigvalsh(F))[::-1]


def field_names(stressmodel, mat):
    """Keys of ip_state_vals for one material under one stress model, in the reference's order."""
    base = BASE_3D if stressmodel == D3 else (BASE_AXI if stressmodel == AXISYM else BASE_2D)
    if mat == VON_MISES:
        return base + (["ep", "j1", "srj2d"] if stressmodel == PLANESTRESS else ["ep"])
    if mat == DRUCKER_PRAGER:
        return base + ["epa", "j1", "srj2d"]
    return list(base)


def ip_state_vals(stressmodel, mat, st):
    """ip_state_vals(mat, state) as an ordered dict (src/tools/tensors.jl:162-215 and the material files)."""
    s, e = st[0:6], st[6:12]
    svm = np.sqrt(3 * J2(s))
    L = eigvals(s)
    d = {"σxx": s[0], "σyy": s[1], "σzz": s[2], "σyz": s[3] / SR2, "σxz": s[4] / SR2, "σxy": s[5] / SR2,
         "σvm": svm}
    if stressmodel == AXISYM:
        d.update({"σrr": s[0], "σtt": s[2], "σry": s[5] / SR2, "εrr": e[0], "εyy": e[1], "εtt": e[2],
                  "εry": e[5] / SR2})
    elif stressmodel == D3:
        d.update({"σ1": L[0], "σ2": L[1], "σ3": L[2], "εxx": e[0], "εyy": e[1], "εzz": e[2],
                  "εyz": e[3] / SR2, "εxz": e[4] / SR2, "εxy": e[5] / SR2})
    else:
        d.update({"σ1": L[0], "σ3": L[2], "εxx": e[0], "εyy": e[1], "εzz": e[2], "εxy": e[5] / SR2})
    if mat == VON_MISES:
        d["ep"] = st[12]
        if stressmodel == PLANESTRESS:
            d["j1"] = s[0] + s[1] + s[2]
            d["srj2d"] = np.sqrt(J2(s))
    elif mat == DRUCKER_PRAGER:
        d["epa"] = st[12]
        d["j1"] = s[0] + s[1] + s[2]
        d["srj2d"] = np.sqrt(J2(s))
    return {k: d[k] for k in field_names(stressmodel, mat)}


def ip_coords(model):
    """ip.coord = C' * N at every IP (setquadrature!, src/element.jl:160-164), extended to 3 components."""
    out = np.zeros((int(model.ip_ptr[-1]), 3))
    for e in range(len(model.shape)):
        sh = int(model.shape[e])
        nodes = model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]]
        C = model.coords[nodes, :model.ndim]
        R, _ = quadrature(sh, int(model.nips[e]))
        for q in range(len(R)):
            out[model.ip_ptr[e] + q, :model.ndim] = C.T @ shape_func(sh, R[q])
    return out


def reg_terms(x, y, z, ndim, nterms):
    """reg_terms (src/fe-model.jl:488-501)"""
    if ndim == 3:
        return {10: (1.0, x, y, z, x * y, y * z, x * z, x ** 2, y ** 2, z ** 2), 7: (1.0, x, y, z, x * y, y * z, x * z),
                4: (1.0, x, y, z)}.get(nterms, (1.0,))
    return {6: (1.0, x, y, x * y, x ** 2, y ** 2), 4: (1.0, x, y, x * y), 3: (1.0, x, y)}.get(nterms, (1.0,))


def pinv(M):
    """LinearAlgebra.pinv with its default tolerances: singular values above eps * min(m, n) * max(S) kept."""
    U, S, Vt = np.linalg.svd(M, full_matrices=False)
    tol = np.finfo(float).eps * min(M.shape) * (S.max() if S.size else 0.0)
    Sinv = np.where(S > tol, 1.0 / np.where(S > tol, S, 1.0), 0.0)
    return Vt.T @ (Sinv[:, None] * U.T)


def nodal_patch_recovery(model, ipx=None):
    """nodal_patch_recovery(model) (src/fe-model.jl:504-702) -> (V (nnodes x nfields), field names)."""
    mesh = model.mesh
    ndim, nnodes, ne = model.ndim, model.nnodes, len(model.shape)
    if not mesh.faces:
        return np.zeros((nnodes, 0)), []
    if ipx is None:
        ipx = ip_coords(model)
    conn = [model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]] for e in range(ne)]
    at_bound = np.zeros(nnodes, dtype=bool)
    for f in mesh.faces:
        at_bound[list(f.nodes)] = True
    patches = [[] for _ in range(nnodes)]
    bry_patches = [[] for _ in range(nnodes)]
    for e in range(ne):
        for n in conn[e][:CORNERS[int(model.shape[e])]]:
            (bry_patches if at_bound[n] else patches)[n].append(e)
    haspatch = np.zeros(nnodes, dtype=bool)
    for p in patches:
        for e in p:
            haspatch[conn[e]] = True
    orphans = [n for n in range(nnodes) if not haspatch[n] and at_bound[n]]
    if orphans:
        for k in (3, 2, 1):
            for n in orphans:
                if len(bry_patches[n]) >= k:
                    patches[n] = bry_patches[n]
            for n in orphans:
                for e in patches[n]:
                    haspatch[conn[e]] = True
            orphans = [n for n in orphans if not haspatch[n]]
            if not orphans:
                break
    # IP values and the field order (first appearance over the elements)
    vals, fields = [], []
    for e in range(ne):
        mt = int(model.mat_type[e])
        vals.append([ip_state_vals(model.stressmodel, mt, model.state[i]) for i in range(model.ip_ptr[e],
                                                                                          model.ip_ptr[e + 1])])
        for k in vals[e][0]:
            if k not in fields:
                fields.append(k)
    fidx = {k: i for i, k in enumerate(fields)}
    if not fields:
        return np.zeros((nnodes, 0)), []
    Vv = np.zeros((nnodes, len(fields)))
    Vr = np.zeros((nnodes, len(fields)), dtype=np.int64)
    for patch in patches:
        if not patch:
            continue
        pf = []
        for e in patch:
            for k in vals[e][0]:
                if k not in pf:
                    pf.append(k)
        for field in pf:
            sub = [e for e in patch if field in vals[e][0]]
            ips = [i for e in sub for i in range(model.ip_ptr[e], model.ip_ptr[e + 1])]
            nodes = []
            for e in sub:
                for n in conn[e]:
                    if n not in nodes:
                        nodes.append(n)
            m = len(ips)
            if ndim == 3:
                nt = 7 if m >= 7 else 4 if m >= 4 else 1
            else:
                nt = 6 if m >= 6 else 4 if m >= 4 else 3 if m >= 3 else 1
            M = np.array([reg_terms(*ipx[i], ndim, nt) for i in ips])
            N = np.array([reg_terms(*model.coords[n], ndim, nt) for n in nodes])
            W = np.array([d[field] for e in sub for d in vals[e]])
            V = N @ (pinv(M) @ W)
            j = fidx[field]
            for i, n in enumerate(nodes):
                Vv[n, j] += V[i]
                Vr[n, j] += 1
    with np.errstate(invalid="ignore", divide="ignore"):
        Vv = Vv / Vr
    Vv[np.isnan(Vv)] = 0.0
    return Vv, fields
