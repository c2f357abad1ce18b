"""Amaru's element/material/stage API on top of the GB300 library.

Mirrors FEModel (src/fe-model.jl:66-255), MechContext / MechAnalysis / solve!
(src/mech/mech-solver.jl:6-181), addstage! (src/analysis.jl:27-32), the
boundary-condition types (src/bc.jl) and the solver-level plugin functions
mount_K / update_state! / solve_system! that the GPU library replaces.
All numerical work runs in libamaru_gpu.so; this module numbers DOFs,
evaluates essential values and nodal loads, and moves arrays across the ABI.
"""
import numpy as np

from . import _lib as L
from .args import DYN_SOLVER_PARAMS, MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, checkargs
from .expr import affine_coefficients, evaluate
from .mesh import NPOINTS, Mesh

# VTK cell type of each shape (vtk_type in src/shape/*.jl, codes of src/shape/vtk.jl)
VTK_TYPES = {L.TRI3: 5, L.TRI6: 22, L.QUAD4: 9, L.QUAD8: 23, L.QUAD9: 28, L.TET4: 10, L.TET10: 24, L.HEX8: 12,
             L.HEX20: 25}
STRESSMODELS = {"d3": L.D3, "planestrain": L.PLANESTRAIN, "planestress": L.PLANESTRESS,
                "axisymmetric": L.AXISYMMETRIC}


# ---- materials (src/mech/mat/*.jl) and the element type
class MechSolid:
    """Isoparametric bulk element (src/mech/elem/mech-solid.jl)."""


class _Mat:
    kind = None

    def __init__(self, **p):
        self.p = p

    def params(self):
        raise NotImplementedError


class LinearElastic(_Mat):
    """LinearElastic(E, nu): src/mech/mat/linear-elastic.jl:5-20"""
    kind = L.LINEAR_ELASTIC

    def params(self):
        return [self.p["E"], self.p.get("nu", 0.0), 0, 0, 0, 0, 0, 0]


class VonMises(_Mat):
    """VonMises(E, nu, fy, H): src/mech/mat/von-mises.jl:3-27"""
    kind = L.VON_MISES

    def params(self):
        return [self.p["E"], self.p.get("nu", 0.0), self.p["fy"], self.p.get("H", 0.0), 0, 0, 0, 0]


class DruckerPrager(_Mat):
    """DruckerPrager(E, nu, alpha, kappa, H): src/mech/mat/drucker-prager.jl:5-33"""
    kind = L.DRUCKER_PRAGER

    def params(self):
        return [self.p["E"], self.p.get("nu", 0.0), self.p.get("alpha", 0.0), self.p["kappa"], self.p.get("H", 0.0),
                0, 0, 0]


# ---- boundary conditions (src/bc.jl)
class _BC:
    def __init__(self, **conds):
        if not conds:
            raise ValueError("a boundary condition needs at least one condition")
        self.conds = conds


class NodeBC(_BC):
    pass


class SurfaceBC(_BC):
    pass


class EdgeBC(_BC):
    pass


class BodyC(_BC):
    pass


FaceBC = SurfaceBC
ElemBC = BodyC
_NAT = {"fx": 0, "fy": 1, "fz": 2}
_DIR = {"x": 0, "y": 1, "z": 2, "n": 3}


def number_dofs(active_nodes, presc, nnodes):
    """DOF numbering of configure_dofs! (src/bc.jl:198-233): active nodes by id, (ux, uy[, uz]) per node,
    unknown DOFs first and prescribed ones last, both in that order.  Returns (eq_id, ndofs, nu, node, comp)."""
    ndim = presc.shape[1]
    act = np.asarray(active_nodes, dtype=np.int64)
    flags = presc[act].reshape(-1)
    dn = np.repeat(act, ndim)
    dk = np.tile(np.arange(ndim), len(act))
    order = np.concatenate([np.nonzero(~flags)[0], np.nonzero(flags)[0]])
    eq_id = -np.ones((nnodes, 3), dtype=np.int64)
    eq_id[dn[order], dk[order]] = np.arange(len(order))
    return eq_id, len(order), int((~flags).sum()), dn[order], dk[order]


class MechContext:
    """MechContext(ndim, stressmodel): src/mech/mech-solver.jl:6-33"""

    def __init__(self, ndim=0, stressmodel="d3"):
        self.ndim, self.stressmodel = ndim, stressmodel


class FEModel:
    """FEModel(mesh, matbinds, ctx; thickness): model on the device.

    matbinds: list of (filter, MechSolid, MaterialType, params-dict) or (filter, material instance);
    filter is a tag, an expression over the element's nodes, or "all"."""

    def __init__(self, mesh, matbinds, ctx=None, thickness=1.0, nips=0, E=None, device=True):
        """device=False keeps the model on the host only, to be joined with others (FEModel.join)."""
        ctx = ctx or MechContext()
        self.mesh = mesh
        self.ndim = mesh.ndim
        sm = ctx.stressmodel
        if self.ndim == 2 and sm == "d3":
            sm = "planestrain"
        self.stressmodel = STRESSMODELS[sm]
        self.thickness = float(thickness)
        ne = len(mesh.shape)
        self.mat_type = np.full(ne, -1, dtype=np.int32)
        self.mat_params = np.zeros((ne, 8))
        self.rho = np.zeros(ne)  # element density (MechSolid props rho, src/mech/elem/mech-solid.jl:6-29)
        enodes = mesh.elem_nodes()
        for bind in matbinds:
            if len(bind) == 4:
                filt, _elem, mtype, params = bind
                mat = mtype(**params)
            else:
                filt, mat = bind
            if isinstance(filt, str) and (filt == "all" or not any(ch in filt for ch in "=<>")):
                sel = np.arange(ne) if filt == "all" else np.nonzero(mesh.tags == filt)[0]
            else:
                sel = mesh.select_cells(enodes, filt)
            self.mat_type[sel] = mat.kind
            self.mat_params[sel] = mat.params()
            self.rho[sel] = mat.p.get("rho", 0.0)
        if (self.mat_type < 0).any():
            raise ValueError("FEModel: some elements have no material")
        if E is not None:
            self.mat_params[:, 0] = E
        self.nips = np.full(ne, nips, dtype=np.int32)
        self.active = np.ones(ne, dtype=bool)  # elem.active (src/fe-model.jl:156)
        self.dev = None
        if device:
            self.dev = L.DeviceModel(self.ndim, self.stressmodel, self.thickness, mesh.coords, mesh.shape, self.nips,
                                     mesh.conn_ptr, mesh.conn, self.mat_type, self.mat_params)
        self._host_fields()

    def _host_fields(self):
        mesh = self.mesh
        self.nnodes = len(mesh.coords)
        self.U = np.zeros((self.nnodes, self.ndim))  # dof.vals of the displacement keys
        self.F = np.zeros((self.nnodes, self.ndim))  # dof.vals of the natural keys
        self.eq_id = -np.ones((self.nnodes, 3), dtype=np.int64)
        self.ndofs = self.nu = 0
        self.used_nodes = np.nonzero(np.bincount(mesh.conn, minlength=self.nnodes))[0]  # the nodes with dofs
        self.active_nodes = self.used_nodes
        self._dof_names = ["ux", "uy", "uz"][: self.ndim]
        # the device model holds the active elements (_dev_elems, None: all) and their nodes (_dev_nodes)
        self._dev_elems = self._dev_nodes = None
        self._g2l = self._e2l = None
        self._state_rest = None  # IP states of every element while the device holds a subset
        self._ip_ptr = None

    @classmethod
    def join(cls, models):
        """One device model holding independent models side by side, each a part (amr_set_parts):
        the batched solver and stage driver then run every part as if it were alone."""
        models = list(models)
        m0 = models[0]
        if any(not m.active.all() for m in models):
            raise ValueError("joined models must have every element active")
        for m in models:
            if (m.ndim, m.stressmodel, m.thickness) != (m0.ndim, m0.stressmodel, m0.thickness):
                raise ValueError("joined models must share ndim, stress model and thickness")
        mesh, noff, eoff = Mesh.join([m.mesh for m in models])
        out = cls.__new__(cls)
        out.mesh, out.ndim, out.stressmodel, out.thickness = mesh, m0.ndim, m0.stressmodel, m0.thickness
        out.mat_type = np.concatenate([m.mat_type for m in models])
        out.mat_params = np.concatenate([m.mat_params for m in models])
        out.nips = np.concatenate([m.nips for m in models])
        out.rho = np.concatenate([m.rho for m in models])
        out.active = np.ones(len(out.mat_type), dtype=bool)
        out.dev = L.DeviceModel(out.ndim, out.stressmodel, out.thickness, mesh.coords, mesh.shape, out.nips,
                                mesh.conn_ptr, mesh.conn, out.mat_type, out.mat_params)
        out._host_fields()
        out.node_offsets, out.elem_offsets = noff, eoff
        out.dev.set_parts(noff)
        return out

    def changequadrature(self, n):
        """changequadrature!(elems, n) (src/element.jl:185-188): rebuilds the device model."""
        self.nips[:] = n
        self.dev.close()
        self.dev = self._device_over(None)  # fresh IP states; the next configure_dofs! takes the active set
        self._dev_elems = self._state_rest = self._ip_ptr = None
        self.active_nodes = self.used_nodes

    # ---- element activation: elem.active and a stage's toactivate (src/mech/mech-solver.jl:216-220)
    def set_active(self, sel, active=True):
        """elem.active = active for the selected elements: ids, a boolean mask, a tag or a filter expression."""
        self.active[self._elem_sel(sel)] = bool(active)

    def _elem_sel(self, sel):
        if isinstance(sel, str):
            if sel == "all":
                return np.arange(len(self.active))
            if not any(ch in sel for ch in "=<>"):
                return np.nonzero(self.mesh.tags == sel)[0]
            return self.mesh.select_cells(self.mesh.elem_nodes(), sel)
        a = np.asarray(sel)
        return np.nonzero(a)[0] if a.dtype == bool else a.astype(np.int64).reshape(-1)

    def _device_over(self, elems):
        """A device model over the elements elems (None: all) and the nodes they use, renumbered in id order."""
        mesh = self.mesh
        if elems is None:
            self._dev_nodes = self._g2l = self._e2l = None
            return L.DeviceModel(self.ndim, self.stressmodel, self.thickness, mesh.coords, mesh.shape, self.nips,
                                 mesh.conn_ptr, mesh.conn, self.mat_type, self.mat_params)
        cp = mesh.conn_ptr
        cnt = cp[elems + 1] - cp[elems]
        conn = np.concatenate([mesh.conn[cp[e]:cp[e + 1]] for e in elems]) if len(elems) else np.zeros(0, np.int64)
        nodes = np.unique(conn)
        g2l = np.full(self.nnodes, -1, dtype=np.int64)
        g2l[nodes] = np.arange(len(nodes))
        e2l = np.full(len(self.active), -1, dtype=np.int64)
        e2l[elems] = np.arange(len(elems))
        ptr = np.zeros(len(elems) + 1, dtype=np.int64)
        ptr[1:] = np.cumsum(cnt)
        self._dev_nodes, self._g2l, self._e2l = nodes, g2l, e2l
        return L.DeviceModel(self.ndim, self.stressmodel, self.thickness, mesh.coords[nodes], mesh.shape[elems],
                             self.nips[elems], ptr, g2l[conn], self.mat_type[elems], self.mat_params[elems])

    def _ip_rows(self, elems):
        """The rows of the given elements in the all-element state layout."""
        if self._ip_ptr is None:
            nips = self.dev.elem_nips()
            if self._dev_elems is not None:
                raise RuntimeError("IP layout unknown")
            self._ip_ptr = np.concatenate([[0], np.cumsum(nips)]).astype(np.int64)
        p = self._ip_ptr
        return np.concatenate([np.arange(p[e], p[e + 1]) for e in elems]) if len(elems) else np.zeros(0, np.int64)

    def _sync_active(self):
        """Rebuilds the device model over the active elements when the set changed since the last stage; the IP
        states move with their elements (inactive ones keep theirs on the host)."""
        if self.dev is None:
            return
        want = None if self.active.all() else np.nonzero(self.active)[0].astype(np.int64)
        have = self._dev_elems
        if (want is None and have is None) or (want is not None and have is not None and np.array_equal(want, have)):
            return
        if getattr(self, "node_offsets", None) is not None:
            raise ValueError("joined models must have every element active")
        if self._ip_ptr is None and have is None:
            self._ip_rows(np.zeros(0, np.int64))
        full = self.state()
        self.dev.close()
        self.dev = self._device_over(want)
        self._dev_elems = want
        self._state_rest = None if want is None else full
        self.dev.set_state(full if want is None else full[self._ip_rows(want)])
        self.active_nodes = self.used_nodes if want is None else self._dev_nodes

    def dev_rho(self):
        """The densities of the elements on the device."""
        return self.rho if self._dev_elems is None else self.rho[self._dev_elems]

    # ---- configure_dofs! (src/bc.jl:198-233)
    def _select(self, bc, filt):
        mesh = self.mesh
        if isinstance(bc, NodeBC):
            if isinstance(filt, (int, np.integer)):
                return np.array([filt]), np.array([[filt]])
            if isinstance(filt, (list, tuple, np.ndarray)):
                a = np.asarray(filt, dtype=np.int64)
                return a, a[:, None]
            ids = mesh.select_nodes(filt)
            return ids, ids[:, None]
        if isinstance(bc, SurfaceBC) or isinstance(bc, EdgeBC):
            if isinstance(bc, EdgeBC) or self.ndim == 2:
                table, shapes = mesh.edge_nodes, mesh.edge_shape
            else:
                table, shapes = mesh.face_nodes, mesh.face_shape
            sel = mesh.select_cells(table, filt)
            return sel, (table[sel], shapes[sel])
        enodes = mesh.elem_nodes()
        if isinstance(filt, str) and not any(ch in filt for ch in "=<>") and filt != "all":
            sel = np.nonzero(mesh.tags == filt)[0]
        else:
            sel = mesh.select_cells(enodes, filt)
        sel = sel[self.active[sel]]  # model.elems.active[bc.filter] (src/bc.jl:159)
        return sel, enodes[sel]

    def _prescribed(self, bcs):
        presc = np.zeros((self.nnodes, self.ndim), dtype=bool)
        setup = []
        for filt, bc in bcs:
            sel, objs = self._select(bc, filt)
            nodes = objs if isinstance(bc, NodeBC) else (objs[0] if isinstance(objs, tuple) else objs)
            nodes = np.unique(nodes[nodes >= 0]) if len(nodes) else np.zeros(0, dtype=np.int64)
            for key in bc.conds:
                if key in self._dof_names:
                    presc[nodes, self._dof_names.index(key)] = True
            setup.append((bc, sel, objs, nodes))
        return presc, setup

    def configure_dofs(self, bcs):
        """configure_dofs! (src/bc.jl:198-233) over the nodes of the active elements."""
        self._sync_active()
        presc, setup = self._prescribed(bcs)
        self.eq_id, self.ndofs, self.nu, self.dof_node, self.dof_comp = number_dofs(self.active_nodes, presc,
                                                                                   self.nnodes)
        if self.dev is not None:
            self.dev.set_dofs(self.eq_id if self._dev_nodes is None else self.eq_id[self._dev_nodes], self.ndofs,
                              self.nu)
        return setup

    # ---- get_bc_vals (src/bc.jl:237-249)
    def get_bc_vals(self, setup, t=0.0):
        U, F, loads = self.bc_vals(setup, t)
        if loads:
            F = self.dev.assemble_loads(loads, F, t)
        return U, F

    def bc_vals(self, setup, t=0.0):
        """Essential values U, concentrated natural values F, and the distributed loads as
        amr_load tuples still to be integrated into F (on the device)."""
        U = np.zeros(self.ndofs)
        F = np.zeros(self.ndofs)
        loads = []
        c = self.mesh.coords
        for bc, sel, objs, nodes in setup:
            if len(nodes) and (self.eq_id[nodes, 0] < 0).any():
                # such a node keeps eq_id 0 (Dof(), src/dof.jl:15-17): the reference's U[dof.eq_id] fails there
                bad = int(nodes[self.eq_id[nodes, 0] < 0][0])
                raise ValueError("boundary condition on node %d, which belongs to no active element" % (bad + 1))
            for key, val in bc.conds.items():
                if key in self._dof_names:
                    k = self._dof_names.index(key)
                    v = np.broadcast_to(evaluate(val, x=c[nodes, 0], y=c[nodes, 1], z=c[nodes, 2], t=t), nodes.shape)
                    U[self.eq_id[nodes, k]] = v
                elif isinstance(bc, NodeBC):
                    if key not in _NAT or _NAT[key] >= self.ndim:
                        raise ValueError("NodeBC key %s not applicable" % key)
                    k = _NAT[key]
                    v = np.broadcast_to(evaluate(val, x=c[nodes, 0], y=c[nodes, 1], z=c[nodes, 2], t=t), nodes.shape)
                    np.add.at(F, self.eq_id[nodes, k], v)
                elif isinstance(bc, (SurfaceBC, EdgeBC)):
                    table, shapes = objs
                    if len(table) == 0:
                        continue
                    if key[0] not in "tq" or key[1:] not in _DIR:
                        raise ValueError("boundary condition %s is not applicable as distributed bc" % key)
                    cf = affine_coefficients(val, self.ndim)
                    for fs in np.unique(shapes):
                        rows = table[shapes == fs][:, :NPOINTS[int(fs)]]
                        if self._g2l is not None:
                            rows = self._g2l[rows]
                        loads.append((L.LOAD_FACET, _DIR[key[1:]], 1 if key[0] == "q" else 0, int(fs), rows, cf))
                else:
                    if key not in ("wx", "wy", "wz"):
                        raise ValueError("body condition %s is not applicable" % key)
                    cf = affine_coefficients(val, self.ndim)
                    items = np.asarray(sel, dtype=np.int64)
                    loads.append((L.LOAD_BODY, _DIR[key[1]], 0, 0, items if self._e2l is None else self._e2l[items], cf))
        return U, F, loads

    # ---- the solver-level plugin functions the library replaces
    def mount_K(self, reference_order=True):
        """mount_K(elems, ndofs) (src/mech/mech-solver.jl:78-110): device assembly, exported in the
        reference's CSC layout.  reference_order=True evaluates K_e in the reference's operation order,
        so the stored-entry pattern follows the reference's |Ke_ij| >= eps() decisions; False uses the
        fast pair-tensor kernel of the Newton loop."""
        self.dev.set_assembly(L.ASSEMBLY_REFERENCE if reference_order else L.ASSEMBLY_FAST)
        try:
            self.dev.assemble_K()
            return self.dev.K_csc()
        finally:
            self.dev.set_assembly(L.ASSEMBLY_FAST)

    def update_state(self, dU):
        """update_state!(elems, dU, t) (src/mech/mech-solver.jl:124-144): returns dFin."""
        return self.dev.update_state(dU)

    def solve_system(self, U, F, **opts):
        """solve_system!(K, U, F, nu) (src/solver.jl:5-79) on the last assembled K."""
        o = L.default_solve_opts(**opts)
        U2, F2, st = self.dev.solve(U, F, o)
        U[:self.nu] = U2[:self.nu]
        F[self.nu:] = F2[self.nu:]
        return st

    def state(self):
        """IP states of every element (nip_total x 16, element order); inactive elements keep theirs."""
        if self._dev_elems is None:
            return self.dev.state()
        full = self._state_rest.copy()
        full[self._ip_rows(self._dev_elems)] = self.dev.state()
        return full

    def set_state(self, state):
        if self._dev_elems is None:
            self.dev.set_state(state)
            return
        state = np.asarray(state, dtype=np.float64)
        if state.shape != self._state_rest.shape:
            raise ValueError("state must be nip_total x 16")
        self._state_rest = state.copy()
        self.dev.set_state(state[self._ip_rows(self._dev_elems)])

    def _with_all_elements(self, fn):
        """fn(device model over every element, with the current IP states): output covers every element, as
        update_output_data! does (src/fe-model.jl:341-427)."""
        if self._dev_elems is None:
            return fn(self.dev)
        full = self.state()
        dev = L.DeviceModel(self.ndim, self.stressmodel, self.thickness, self.mesh.coords, self.mesh.shape, self.nips,
                            self.mesh.conn_ptr, self.mesh.conn, self.mat_type, self.mat_params)
        try:
            dev.set_state(full)
            return fn(dev)
        finally:
            dev.close()

    # ---- output data
    def nodal_patch_recovery(self):
        """nodal_patch_recovery(model) (src/fe-model.jl:504-702) on the device: (V (nnodes x nfields), names)."""
        return self._with_all_elements(lambda d: d.recover_nodal())

    def update_output_data(self):
        """node_data / elem_data of update_output_data! (src/fe-model.jl:341-427): ids, cell types, the dof values
        (displacements and natural values), the recovered IP fields and the vector U."""
        nn, ne = self.nnodes, len(self.mesh.shape)
        node = {"node-id": np.arange(1, nn + 1)}
        nat = ["fx", "fy", "fz"]
        has = np.zeros(nn, dtype=bool)
        has[self.used_nodes] = True
        for i in range(self.ndim):
            node[self._dof_names[i]] = np.where(has, self.U[:, i], 0.0)
            node[nat[i]] = np.where(has, self.F[:, i], 0.0)
        V, names = self.nodal_patch_recovery()
        for j, k in enumerate(names):
            node[k] = V[:, j]
        U = np.zeros((nn, 3))
        U[:, : self.ndim] = np.stack([node[k] for k in self._dof_names], 1)
        node["U"] = U
        elem = {"elem-id": np.arange(1, ne + 1), "cell-type": np.array([VTK_TYPES[int(s)] for s in self.mesh.shape])}
        self.node_data, self.elem_data = node, elem
        return node, elem

    def save(self, path, nthreads=0, compress=False):
        """save(model, "file.vtu"; compress) (src/mesh/io.jl:167-274, 323-342): update_output_data! and the VTU
        file written by the library, byte for byte as the reference writes it: ascii, or the arrays appended as
        zlib blocks with compress=True.  Tagged elements add the tag columns save_vtu adds."""
        node, elem = self.update_output_data()
        items = list(elem.items()) + vtu_tag_columns(self.mesh.tags)
        self._with_all_elements(lambda d: d.write_vtu(path, list(node.items()), items, nthreads, compress))


def vtu_tag_columns(tags):
    """The tag fields save_vtu adds to elem_data (src/mesh/io.jl:168-192) when the elements carry tags: tag-s1
    and tag-s2, the tag's UTF-8 bytes cut at 8 (safe_string_cut, src/tools/encode.jl:25-36) and packed
    little-endian (encode_string_to_uint64, :3-11), and tag, the tag's index.  The reference numbers the
    tags in the iteration order of a Julia Set, which follows Julia's string hash; here they are numbered
    in order of first appearance, so the tag column is a permutation of the reference's while tag-s1 and
    tag-s2 are the same."""
    tags = ["" if t is None else str(t) for t in tags]
    uniq = list(dict.fromkeys(tags))
    if len(uniq) == 0 or (len(uniq) == 1 and uniq[0] == ""):
        return []
    idx = {t: i for i, t in enumerate(uniq)}

    def cut(t):
        # safe_string_cut(t, 8): whole when shorter than 8 bytes; else cut after byte 8, which the
        # reference manages only when byte 8 is a one-byte character (else its s[1:8] / s[p+1:end]
        # raise): the same cases are refused here
        b = t.encode("utf-8")
        if len(b) > 16:
            raise ValueError("Mesh: tag '%s' too long. Max length is 16 UTF units." % t)
        if 8 > len(b):
            return b, b""
        if b[7] >= 0x80:
            raise ValueError("Mesh: tag '%s' cannot be cut after its 8th byte" % t)
        return b[:8], b[8:]

    def pack(b):
        return sum(int(c) << (8 * i) for i, c in enumerate(b))

    parts = {t: cut(t) for t in uniq}
    s1 = np.array([pack(parts[t][0]) for t in tags], dtype=np.uint64)
    s2 = np.array([pack(parts[t][1]) for t in tags], dtype=np.uint64)
    return [("tag-s1", s1), ("tag-s2", s2), ("tag", np.array([idx[t] for t in tags], dtype=np.int64))]


class Stage:
    def __init__(self, bcs, nincs=1, nouts=0, toactivate=()):
        self.bcs, self.nincs, self.nouts, self.status = list(bcs), nincs, nouts, "pending"
        self.toactivate = toactivate  # element ids, a mask, a tag or a filter (src/stage.jl:8,16)

    def activate(self, model):
        """elem.active = true for the stage's toactivate (src/mech/mech-solver.jl:216-219)."""
        if self.toactivate is not None and not (isinstance(self.toactivate, (list, tuple)) and not self.toactivate):
            model.set_active(self.toactivate, True)


class MechAnalysis:
    """MechAnalysis(model): staged Newton solver on the device."""

    def __init__(self, model):
        self.model = model
        self.stages = []
        self.stats = []
        self.log = []  # (stage, inc, it, residue) per Newton iteration, as the reference's log lines

    def addstage(self, bcs, nincs=1, nouts=0, toactivate=()):
        """addstage!(ana, bcs; nincs, nouts, toactivate): src/analysis.jl:27-32"""
        self.stages.append(Stage(bcs, nincs, nouts, toactivate))

    def solve(self, tol=0.01, rtol=0.01, rspan=0.01, dT0=0.01, dTmin=1e-7, dTmax=0.1, scheme="FE", maxits=5,
              autoinc=False, quiet=True, linear_rtol=1e-8, solver="mixed", refine_every=32, max_iters=20000,
              record=None):
        """solve!(ana; args...) (src/mech/mech-solver.jl:155-181): returns (success, message).
        record(ana, T, checkpoint), if given, runs after every converged increment, where the reference calls
        update_records! (:410-424), with model.U and model.F holding the dof values so far."""
        checkargs("solve!", MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, tol=tol, rspan=rspan, rtol=rtol, dT0=dT0,
                  dTmin=dTmin, dTmax=dTmax, maxits=maxits, scheme=scheme)
        model = self.model
        method = {"mixed": L.SOLVER_MIXED, "fp64": L.SOLVER_FP64, "amg": L.SOLVER_AMG, "amg_fp64": L.SOLVER_AMG_FP64}[solver]
        lin = L.default_solve_opts(method=method, rtol=linear_rtol, refine_every=refine_every, max_iters=max_iters)
        for st in self.stages:
            if st.status == "done":
                continue
            st.activate(model)
            setup = model.configure_dofs(st.bcs)
            Uex, Fex = model.get_bc_vals(setup)
            p = L.default_stage_params(tol=tol, rtol=rtol, rspan=rspan, dT0=dT0, dTmin=dTmin, dTmax=dTmax,
                                       scheme={"FE": 0, "ME": 1, "BE": 2, "Ralston": 3}[scheme], maxits=maxits,
                                       autoinc=int(autoinc), nincs=st.nincs, nouts=st.nouts, linear=lin)
            if record is not None:
                U0, F0 = model.U.copy(), model.F.copy()

                def hook(T, inc, checkpoint, Us, Fs):
                    model.U[:], model.F[:] = U0, F0
                    model.U[model.dof_node, model.dof_comp] += Us
                    model.F[model.dof_node, model.dof_comp] += Fs
                    return record(self, T, checkpoint)
                model.dev.set_increment_callback(hook)
            try:
                rc, U, F, stats = model.dev.stage_run(Uex, Fex, p)
            finally:
                if record is not None:
                    model.dev.set_increment_callback(None)
                    model.U[:], model.F[:] = U0, F0
            self.stats.append(stats)
            self.log += [(st, r.increment, r.iteration, r.residue) for r in model.dev.stage_log()]
            if rc not in (0, -11):
                raise L.AmrError(rc, model.dev.last_error())
            model.U[model.dof_node, model.dof_comp] += U
            model.F[model.dof_node, model.dof_comp] += F
            if rc != 0:
                st.status = "error"
                return False, model.dev.last_error()
            st.status = "done"
        return True, ""


class DynAnalysis:
    """DynamicAnalysis(model) (src/mech/dyn-solver.jl:34-66) with addstage! and solve! (:166-186): the
    Newmark stage solver dyn_stage_solver! (:203-534) on the device.  Boundary values must be affine in
    time (get_bc_vals at t = Uex(0) + t (Uex(1) - Uex(0))).  The reference defines velocities and
    accelerations only in the first stage, so an analysis has one stage."""

    def __init__(self, model):
        self.model = model
        self.stages = []
        self.stats = None

    def addstage(self, bcs, nincs=1, nouts=0, tspan=0.0, toactivate=()):
        st = Stage(bcs, nincs, nouts, toactivate)
        st.tspan = float(tspan)
        self.stages.append(st)

    def solve(self, tol=0.01, dTmin=1e-7, dTmax=0.1, rspan=0.01, maxits=5, autoinc=False, alpha=0.0, beta=0.0,
              solver="mixed", linear_rtol=1e-8, quiet=True, scheme="FE", sism=False, tss=0.0, tds=0.0,
              sism_file="", sism_dir="fx"):
        """Returns (ok, message); dof values land in model.U, model.V, model.A, model.F (node-major).  `scheme`
        is checked as dyn_solver_params checks it and, as in dyn_stage_solver!, not used.  sism: seismic input,
        the record of sism_file (read as readdlm reads it, times 9.81) spread over tds from t = 0, applied as
        M (a(t) e_dir) while tss <= t <= tss + tds (sismic_force, src/mech/dyn-solver.jl:106-157)."""
        checkargs("solve!", DYN_SOLVER_PARAMS, MECH_SOLVER_VALUES, tol=tol, dTmin=dTmin, dTmax=dTmax, rspan=rspan,
                  maxits=maxits, scheme=scheme)
        if len(self.stages) != 1:
            raise ValueError("a dynamic analysis has one stage (the reference defines V and A in the first only)")
        stage = self.stages[0]
        model = self.model
        stage.activate(model)
        setup = model.configure_dofs(stage.bcs)
        U0, F0 = model.get_bc_vals(setup, 0.0)
        U1, F1 = model.get_bc_vals(setup, 1.0)
        Uh, Fh = model.get_bc_vals(setup, 0.5)
        dU, dF = U1 - U0, F1 - F0
        for a, b, c in ((U0, dU, Uh), (F0, dF, Fh)):
            if np.abs(a + 0.5 * b - c).max(initial=0.0) > 1e-12 * max(np.abs(c).max(initial=0.0), 1.0):
                raise NotImplementedError("boundary values must be affine in time on the GPU path")
        model.dev.set_density(model.dev_rho())
        method = {"mixed": L.SOLVER_MIXED, "fp64": L.SOLVER_FP64, "amg": L.SOLVER_AMG, "amg_fp64": L.SOLVER_AMG_FP64}[solver]
        p = L.default_dyn_params(tol=tol, dTmin=dTmin, dTmax=dTmax, rspan=rspan, alpha=alpha, beta=beta,
                                 tspan=stage.tspan, maxits=maxits, autoinc=int(autoinc), nincs=stage.nincs,
                                 nouts=stage.nouts, linear=L.default_solve_opts(method=method, rtol=linear_rtol))
        acc = None
        if sism:
            dirs = {"ux": 0, "fx": 0, "uy": 1, "fy": 1, "uz": 2, "fz": 2}
            if sism_dir not in dirs:
                raise KeyError(sism_dir)  # node.dofdict[keysis] fails for a key no node has
            acc = np.ascontiguousarray(9.81 * np.loadtxt(sism_file, ndmin=2).reshape(-1), dtype=np.float64)
            p.sism, p.sism_dir, p.tss, p.tds = 1, dirs[sism_dir], float(tss), float(tds)
            p.sism_acc, p.sism_n = acc.ctypes.data, len(acc)
        rc, U, V, A, F, st = model.dev.dyn_stage_run(U0, dU, F0, dF, p)
        del acc
        self.stats = st
        if rc not in (0, -11):
            return False, model.dev.last_error()
        for name, vec in (("U", U), ("V", V), ("A", A), ("F", F)):
            out = np.zeros((model.nnodes, model.ndim))
            out[model.dof_node, model.dof_comp] = vec
            setattr(model, name, out)
        stage.status = "done" if rc == 0 else "failed"
        return rc == 0, ("" if rc == 0 else model.dev.last_error())


class ModalAnalysis:
    """MechModalAnalysis(model) (src/mech/mech-modal-solver.jl:12-55) with addstage! and solve!(; nmodes):
    the frequencies (freqs, rad/s) and modes (nu x nmodes) of mech_modal_solver! on the device."""

    def __init__(self, model):
        self.model = model
        self.stages = []
        self.freqs = np.zeros(0)
        self.modes = np.zeros((0, 0))
        self.stats = None
        self.alpha = self.beta = None

    def addstage(self, bcs, nincs=1, nouts=0, toactivate=()):
        self.stages.append(Stage(bcs, nincs, nouts, toactivate))

    def solve(self, nmodes=5, tol=1e-7, max_iters=1000, quiet=True, rayleigh=None):
        """rayleigh=(xi1, xi2, i1, i2) also sets self.alpha, self.beta (see set_rayleigh)."""
        model = self.model
        for stage in self.stages:
            stage.activate(model)
            model.configure_dofs(stage.bcs)
            model.dev.set_density(model.dev_rho())
            self.freqs, self.modes, self.stats = model.dev.modal(nmodes, tol, max_iters)
            stage.status = "done"
        if rayleigh is not None:
            self.set_rayleigh(*rayleigh)
        return True, ""

    def set_rayleigh(self, xi1, xi2, i1=1, i2=2):
        """The rayleigh option of mech_modal_solver! (src/mech/mech-modal-solver.jl:204-226): Rayleigh damping
        C = alpha M + beta K whose damping ratio alpha/(2w) + beta w/2 is xi1 at mode i1 and xi2 at mode i2
        (1-based, as the reference reads them).  The reference asks for the four values on standard input;
        here they are arguments.  Returns and keeps (alpha, beta)."""
        if not (1 <= i1 <= len(self.freqs) and 1 <= i2 <= len(self.freqs)) or i1 == i2:
            raise ValueError("two different modes among the %d computed are needed" % len(self.freqs))
        self.alpha, self.beta = rayleigh_coefficients(self.freqs[i1 - 1], self.freqs[i2 - 1], xi1, xi2)
        return self.alpha, self.beta



def rayleigh_coefficients(w1, w2, xi1, xi2):
    """(alpha, beta) of Rayleigh damping with damping ratio xi1 at circular frequency w1 and xi2 at w2: the
    solution of alpha/(2 w) + beta w/2 = xi at both (src/mech/mech-modal-solver.jl:221-222)."""
    d = w1 * w1 - w2 * w2
    if d == 0.0:
        raise ValueError("the two frequencies must differ")
    return 2.0 * (w1 * w1 * w2 * xi2 - w1 * w2 * w2 * xi1) / d, 2.0 * (w1 * xi1 - w2 * xi2) / d


def _shift_setup(setup, noff, eoff):
    """A part's BC selections in the joined model's node and element numbering."""
    def sh(a):
        a = np.asarray(a)
        return np.where(a >= 0, a + noff, a)
    out = []
    for bc, sel, objs, nodes in setup:
        if isinstance(bc, NodeBC):
            out.append((bc, sh(sel), sh(objs), sh(nodes)))
        elif isinstance(bc, (SurfaceBC, EdgeBC)):
            out.append((bc, sel, (sh(objs[0]), objs[1]), sh(nodes)))
        else:
            out.append((bc, np.asarray(sel) + eoff, sh(objs), sh(nodes)))
    return out


class BatchAnalysis:
    """Independent staged analyses run together on one device handle.

    models: FEModel instances built with device=False, one per part; they are joined
    (FEModel.join) into one device model.  Each part runs its own mech_stage_solver!
    (src/mech/mech-solver.jl:186-492): its own increments, Newton iterations, residue
    checks and failure handling, with its DOFs numbered as if it were alone.  Every
    kernel launch serves all parts at once."""

    def __init__(self, models):
        self.models = list(models)
        self.joined = FEModel.join(self.models)
        self.stages = []
        self.stats = []
        self.part_stats = []

    def addstage(self, bcs, nincs=1, nouts=0):
        """bcs: one BC list for every part, or a list with one BC list per part."""
        if bcs and isinstance(bcs[0], list):
            if len(bcs) != len(self.models):
                raise ValueError("one BC list per part")
            per = [list(b) for b in bcs]
        else:
            per = [list(bcs)] * len(self.models)
        self.stages.append(Stage(per, nincs, nouts))

    def configure(self, bcs_per_part):
        """configure_dofs! and get_bc_vals for every part: each part's DOFs numbered as if it were
        alone, the joined model's numbering (all unknowns first) on the device; returns (Uex, Fex)."""
        J = self.joined
        pres, setup = [], []
        for i, (m, bcs) in enumerate(zip(self.models, bcs_per_part)):
            p, su = m._prescribed(bcs)
            m.eq_id, m.ndofs, m.nu, m.dof_node, m.dof_comp = number_dofs(m.active_nodes, p, m.nnodes)
            pres.append(p)
            setup += _shift_setup(su, J.node_offsets[i], J.elem_offsets[i])
        J.eq_id, J.ndofs, J.nu, J.dof_node, J.dof_comp = number_dofs(J.active_nodes, np.concatenate(pres), J.nnodes)
        J.dev.set_dofs(J.eq_id, J.ndofs, J.nu)
        U, F, loads = J.bc_vals(setup)
        # the parts' nodes are disjoint: loads that differ only in their items are one load (same sums)
        merged = {}
        for kind, dr, edge, fshape, items, cf in loads:
            key = (kind, dr, edge, fshape, tuple(np.asarray(cf, dtype=np.float64).tolist()))
            merged.setdefault(key, []).append(np.asarray(items, dtype=np.int64))
        loads = [(k[0], k[1], k[2], k[3], np.concatenate(v), list(k[4])) for k, v in merged.items()]
        if loads:
            F = J.dev.assemble_loads(loads, F, 0.0)
        return U, F

    def split(self, V):
        """A joined eq_id-ordered vector as one node-major (nnodes, ndim) array per part."""
        J = self.joined
        Vn = np.zeros((J.nnodes, J.ndim))
        Vn[J.dof_node, J.dof_comp] = V
        return [Vn[J.node_offsets[i]:J.node_offsets[i + 1]] for i in range(len(self.models))]

    def autotune(self):
        """Picks the element kernels' and the batched solver's launch shapes on this batch (amr_autotune);
        results do not depend on them."""
        pending = [st for st in self.stages if st.status != "done"]
        if pending:
            self.configure(pending[0].bcs)
        self.joined.dev.assemble_K()
        return self.joined.dev.autotune()

    def solve(self, tol=0.01, rtol=0.01, rspan=0.01, dT0=0.01, dTmin=1e-7, dTmax=0.1, scheme="FE", maxits=5,
              autoinc=False, quiet=True, linear_rtol=1e-8, refine_every=32, max_iters=20000, solver="mixed"):
        """solve!(ana; args...) for every part; returns a list of (success, message), one per part.  solver:
        "mixed" (per-part block-Jacobi PCG, one persistent launch) or "amg" (per-part PCG preconditioned by
        the joined model's multigrid V-cycle)."""
        checkargs("solve!", MECH_SOLVER_PARAMS, MECH_SOLVER_VALUES, tol=tol, rspan=rspan, rtol=rtol, dT0=dT0,
                  dTmin=dTmin, dTmax=dTmax, maxits=maxits, scheme=scheme)
        J = self.joined
        method = {"mixed": L.SOLVER_MIXED, "amg": L.SOLVER_AMG}[solver]
        lin = L.default_solve_opts(method=method, rtol=linear_rtol, refine_every=refine_every,
                                   max_iters=max_iters)
        result = [(True, "")] * len(self.models)
        failed = np.zeros(len(self.models), dtype=bool)
        for st in self.stages:
            if st.status == "done":
                continue
            Uex, Fex = self.configure(st.bcs)
            p = L.default_stage_params(tol=tol, rtol=rtol, rspan=rspan, dT0=dT0, dTmin=dTmin, dTmax=dTmax,
                                       scheme={"FE": 0, "ME": 1, "BE": 2, "Ralston": 3}[scheme], maxits=maxits,
                                       autoinc=int(autoinc), nincs=st.nincs, nouts=st.nouts, linear=lin)
            rc, U, F, stats = J.dev.stage_run(Uex, Fex, p)
            if rc not in (0, -11):
                raise L.AmrError(rc, J.dev.last_error())
            self.stats.append(stats)
            ps = J.dev.part_stats()
            self.part_stats.append(ps)
            Us, Fs = self.split(U), self.split(F)
            for i, m in enumerate(self.models):
                if failed[i]:
                    continue
                m.U += Us[i]
                m.F += Fs[i]
                if ps[i].status != 0:
                    failed[i] = True
                    result[i] = (False, "Solver did not converge.")
            st.status = "done"
        return result
