"""Coupled mounts on the device: hm_mount_global_matrices (src/hydromech/hydromech-solver.jl:31-130) and
tm_mount_global_matrices (src/thermomech/thermomech-solver.jl:80-170).

A coupled model is an FEModel of linear elastic solids whose basic (corner) nodes also carry a scalar
field: the pore pressure uw of HMSolid elements (src/hydromech/elem/hydromech-solid.jl) or the temperature
ut of TMSolid elements (src/thermomech/elem/thermomech-solid.jl).  The per-element coupled parameters are
passed beside the model: for the hydraulic mount Biot's alpha, the permeability k and the storativity S
(LinearElasticSeep, src/hydromech/mat/elastic-solid-lin-seep.jl) with the analysis' water unit weight
gammaw; for the thermal mount the thermal expansion alpha, the conductivity k and rho cv with the reference
temperature T0.
"""
import ctypes as C

import numpy as np

from . import _lib as L

HYDRO, THERMO = L.COUPLED_HYDRO, L.COUPLED_THERMO
_BASIC_NPOINTS = {L.HEX8: 8, L.HEX20: 8, L.TET4: 4, L.TET10: 4, L.QUAD4: 4, L.QUAD8: 4, L.QUAD9: 4, L.TRI3: 3,
                  L.TRI6: 3}


def coupled_dofs(model, prescribed):
    """configure_dofs! (src/bc.jl:198-233) for coupled elements (elem_config_dofs, hydromech-solid.jl:51-61):
    per node of an active element ux, uy[, uz], and on basic nodes the scalar, numbered node by node, unknowns
    first and prescribed last.  prescribed: boolean (nnodes, 4), column 3 the scalar.  Returns (eq4, ndofs, nu)."""
    mesh = model.mesh
    nn, ndim = model.nnodes, model.ndim
    used = np.zeros(nn, dtype=bool)
    basic = np.zeros(nn, dtype=bool)
    for e in np.nonzero(model.active)[0]:
        nodes = mesh.conn[mesh.conn_ptr[e]:mesh.conn_ptr[e + 1]]
        used[nodes] = True
        basic[nodes[:_BASIC_NPOINTS[int(mesh.shape[e])]]] = True
    has = np.zeros((nn, 4), dtype=bool)
    has[used, :ndim] = True
    has[:, 3] = basic
    pres = np.asarray(prescribed, dtype=bool) & has
    free = has & ~pres
    eq4 = np.full((nn, 4), -1, dtype=np.int64)
    nf = int(free.sum())
    eq4[free] = np.arange(nf)      # row-major: node by node, slot by slot
    eq4[pres] = nf + np.arange(int(pres.sum()))
    return eq4, int(has.sum()), nf


def mount_coupled(model, kind, params, eq4, ndofs, dt, phi, gammaw=1.0, T0=0.0):
    """(G, RHS): G as a scipy CSC matrix in the reference's layout (every element entry, duplicates summed in
    the reference's order), RHS = -dt H phi (+ dt Q for HYDRO).  params: nelems x 3 (HYDRO: Biot alpha, k, S;
    THERMO: expansion alpha, k, rho cv); phi: the current DOF values (eq order).  The mounts loop over the
    active elements (hydromech-solver.jl:211-213); the device model holds them after configure_dofs!."""
    import scipy.sparse as sp
    model._sync_active()
    prm = np.asarray(params, dtype=np.float64).reshape(-1, 3)
    eq = np.asarray(eq4, dtype=np.int64)
    if model._dev_elems is not None:
        prm, eq = prm[model._dev_elems], eq[model._dev_nodes]
    prm = np.ascontiguousarray(prm)
    eq = np.ascontiguousarray(eq)
    ph = np.ascontiguousarray(phi, dtype=np.float64)
    d = L.CoupledDesc()
    d.kind, d.gammaw, d.T0, d.params = int(kind), float(gammaw), float(T0), prm.ctypes.data
    nnz = C.c_int64()
    h = model.dev.h
    L.check(h, L.lib().amr_coupled_mount(h, C.byref(d), L.ptr(eq), ndofs, float(dt), L.ptr(ph), C.byref(nnz),
                                         None, None, None, None))
    cp = np.zeros(ndofs + 1, dtype=np.int64)
    rv = np.zeros(max(nnz.value, 1), dtype=np.int64)
    nz = np.zeros(max(nnz.value, 1))
    rhs = np.zeros(ndofs)
    L.check(h, L.lib().amr_coupled_mount(h, C.byref(d), L.ptr(eq), ndofs, float(dt), L.ptr(ph), C.byref(nnz),
                                         L.ptr(cp), L.ptr(rv), L.ptr(nz), L.ptr(rhs)))
    n = nnz.value
    return sp.csc_matrix((nz[:n], rv[:n], cp), shape=(ndofs, ndofs)), rhs
