"""Oracle restatement of Amaru.jl's coupled mounts (test infrastructure only).

hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) for HMSolid elements
(src/hydromech/elem/hydromech-solid.jl: elem_stiffness :176-212, elem_coupling_matrix :215-252,
elem_conductivity_matrix :255-290, elem_compressibility_matrix :293-322, elem_RHS_vector :325-362) with a
linear elastic skeleton and a constant isotropic permeability (LinearElasticSeep,
src/hydromech/mat/elastic-solid-lin-seep.jl), and tm_mount_global_matrices
(src/thermomech/thermomech-solver.jl:80-170) for TMSolid elements (src/thermomech/elem/thermomech-solid.jl:
elem_stiffness :93-126, elem_coupling_matrix :129-174, elem_conductivity_matrix :177-209, elem_mass_matrix
:212-240) with a constant conductivity.

The mounts push every entry of every element matrix, without the eps() drop of mount_K: K (u-u), the
coupling C (u-w) and its transpose (w-u, times T0 + 273.15 in the thermal case), dt H (w-w) and the
capacity (w-w), in that order per element and element by element; sparse() sums duplicates in that order.
The scalar field w (pore pressure uw, or temperature ut) lives on the basic (corner) nodes.  Plain Python
loops: meant for meshes of a few hundred elements.
"""
import numpy as np

from .core import (D3, HEX8, HEX20, PLANESTRESS, QUAD4, QUAD8, QUAD9, TET4, TET10, TRI3, TRI6, quadrature,
                   shape_deriv, shape_func)

HYDRO, THERMO = 0, 1
BASIC = {HEX8: HEX8, HEX20: HEX8, TET4: TET4, TET10: TET4, QUAD4: QUAD4, QUAD8: QUAD4, QUAD9: QUAD4, TRI3: TRI3,
         TRI6: TRI3}


def coupled_dofs(model, prescribed):
    """configure_dofs! (src/bc.jl:198-233) for coupled elements: per node ux, uy[, uz] and, on basic nodes, the
    scalar w (elem_config_dofs, hydromech-solid.jl:51-61), numbered node by node with the unknowns first and the
    prescribed last.  prescribed: boolean (nnodes, 4) (slot 3 the scalar).  Returns (eq4, ndofs, nu)."""
    nn, ndim = model.nnodes, model.ndim
    basic = np.zeros(nn, dtype=bool)
    used = np.zeros(nn, dtype=bool)
    for e in range(len(model.shape)):
        nodes = model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]]
        used[nodes] = True
        basic[nodes[:len(shape_func(BASIC[int(model.shape[e])], np.zeros(3)))]] = True
    slots = []
    for n in range(nn):
        if not used[n]:
            continue
        for c in list(range(ndim)) + ([3] if basic[n] else []):
            slots.append((n, c))
    free = [s for s in slots if not prescribed[s[0], s[1]]]
    pres = [s for s in slots if prescribed[s[0], s[1]]]
    eq4 = np.full((nn, 4), -1, dtype=np.int64)
    for i, (n, c) in enumerate(free + pres):
        eq4[n, c] = i
    return eq4, len(slots), len(free)


def _elem(model, e, kind, prm, gammaw):
    """The coupled element matrices of element e: K (nn*ndim square), C (nn*ndim x nb), H (nb x nb),
    capacity (nb x nb) and, hydro only, Q (nb): the reference's forms with its signs."""
    ndim, th = model.ndim, model.thickness
    sh = int(model.shape[e])
    bsh = BASIC[sh]
    nodes = model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]]
    nn = len(nodes)
    X = model.coords[nodes, :ndim]
    R, w = quadrature(sh, int(model.nips[e]))
    nb = len(shape_func(bsh, R[0]))
    K, _ = model.elem_stiffness(e)
    Cm = np.zeros((nn * ndim, nb))
    H = np.zeros((nb, nb))
    Cap = np.zeros((nb, nb))
    Q = np.zeros(nb)
    E, nu = model.mat_par[e, 0], model.mat_par[e, 1]
    alpha, k, cap = prm[e, 0], prm[e, 1], prm[e, 2]
    if kind == HYDRO:
        cc = alpha  # Biot's coefficient (hydromech-solid.jl:240)
    elif model.stressmodel == PLANESTRESS:
        cc = E * alpha / (1 - nu)  # thermal stress modulus (thermomech-solid.jl:143-147)
    else:
        cc = E * alpha / (1 - 2 * nu)
    for q in range(len(R)):
        D = shape_deriv(sh, R[q][:ndim])
        J = X.T @ D
        detJ = np.linalg.det(J)
        if not detJ > 0.0:
            raise RuntimeError("Negative Jacobian determinant in cell %d" % (e + 1))
        Ji = np.linalg.inv(J)
        dNdX = D @ Ji
        Nw = shape_func(bsh, R[q])
        dNwdX = shape_deriv(bsh, R[q][:ndim]) @ Ji
        dv = detJ * w[q] * th
        # C -= coef Bu' m Nw' : Bu' m is the nodal gradient (the normal-strain rows of B; in 2-D the zz row
        # of B is zero, so m's plane-stress zz entry does not matter)
        for a in range(nn):
            for c in range(ndim):
                Cm[a * ndim + c, :] -= cc * dv * dNdX[a, c] * Nw
        if kind == HYDRO:
            H -= (k / gammaw) * dv * (dNwdX @ dNwdX.T)   # conductivity, K = k I (hydromech-solid.jl:276-280)
            Cap -= cap * dv * np.outer(Nw, Nw)           # compressibility, S (:311-314)
            Q += dv * k * dNwdX[:, ndim - 1]             # Bw' K Z, Z the last axis (:349-352)
        else:
            H -= k * dv * (dNwdX @ dNwdX.T)              # thermomech-solid.jl:197-202
            Cap -= cap * dv * np.outer(Nw, Nw)           # rho cv (:232-235)
    return K, Cm, H, Cap, Q, nodes, nb


def mount_coupled(model, kind, prm, eq4, ndofs, dt, phi, gammaw=1.0, T0=0.0):
    """hm_mount_global_matrices / tm_mount_global_matrices -> (G as scipy CSC, RHS).  prm: nelems x 3 (hydro:
    Biot alpha, permeability k, storativity S; thermo: expansion alpha, conductivity k, rho cv); phi: the
    current dof values (eq order) of which the scalar DOFs are read (dof.vals[:uw] / [:ut])."""
    import scipy.sparse as sp
    ndim = model.ndim
    s = 1.0 if kind == HYDRO else T0 + 273.15
    R, Cc, V = [], [], []
    RHS = np.zeros(ndofs)
    for e in range(len(model.shape)):
        K, Cm, H, Cap, Q, nodes, nb = _elem(model, e, kind, prm, gammaw)
        mu = eq4[nodes][:, :ndim].reshape(-1)
        mw = eq4[nodes[:nb], 3]
        nr = len(mu)
        R.append(np.repeat(mu, nr)); Cc.append(np.tile(mu, nr)); V.append(K.reshape(-1))
        # Cup and Cup' interleaved entry by entry (hydromech-solver.jl:65-79)
        for i in range(nr):
            for j in range(nb):
                R.append([mu[i], mw[j]]); Cc.append([mw[j], mu[i]]); V.append([Cm[i, j], s * Cm[i, j]])
        R.append(np.repeat(mw, nb)); Cc.append(np.tile(mw, nb)); V.append((1.0 * dt * H).reshape(-1))
        RHS[mw] -= dt * (H @ phi[mw])
        R.append(np.repeat(mw, nb)); Cc.append(np.tile(mw, nb)); V.append(Cap.reshape(-1))
        if kind == HYDRO:
            RHS[mw] += dt * Q
    R = np.concatenate([np.asarray(r, dtype=np.int64).reshape(-1) for r in R])
    Cc = np.concatenate([np.asarray(c, dtype=np.int64).reshape(-1) for c in Cc])
    V = np.concatenate([np.asarray(v, dtype=np.float64).reshape(-1) for v in V])
    # sparse(): duplicates summed in input order (a stable sort by column, then row)
    order = np.lexsort((R, Cc))
    R, Cc, V = R[order], Cc[order], V[order]
    key = Cc * ndofs + R
    first = np.concatenate([[True], key[1:] != key[:-1]])
    idx = np.cumsum(first) - 1
    vals = np.zeros(first.sum())
    for i in range(len(V)):  # each entry's values summed in input order, from its first one
        vals[idx[i]] = V[i] if first[i] else vals[idx[i]] + V[i]
    rows, cols = R[first], Cc[first]
    G = sp.csc_matrix((vals, (rows, cols)), shape=(ndofs, ndofs))
    G.sort_indices()
    return G, RHS
