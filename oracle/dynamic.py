"""Oracle restatement of Amaru.jl's dynamic mechanical solver (test infrastructure only).

mount_M (src/mech/dyn-solver.jl:71-104) over elem_mass (src/mech/elem/mech-solid.jl:169-205),
and dyn_stage_solver! (src/mech/dyn-solver.jl:203-534): Newmark's average-acceleration rule with
Rayleigh damping C = alpha M + beta K, a Newton loop on the pseudo-stiffness
Kp = K + 4/dt^2 M + 2/dt C, and the reference's increment control.  The reference defines the
velocities and accelerations only in the first stage (:270-296), so an analysis is one stage.
Plain Python loops over elements: meant for meshes of a few thousand nodes.
"""
import math

import numpy as np

from .core import AXISYM, configure_dofs, get_bc_vals, mount_K, quadrature, shape_deriv, shape_func, solve_system, \
    update_state

EPS = 2.220446049250313e-16


def elem_mass(model, e):
    """elem_mass(elem::MechSolid) -> (Me, map): sum over the IPs of rho detJ w th N'N."""
    ndim = model.ndim
    sh = int(model.shape[e])
    nodes = model.conn[model.conn_ptr[e]:model.conn_ptr[e + 1]]
    nn = len(nodes)
    C = model.coords[nodes, :ndim]
    R, w = quadrature(sh, int(model.nips[e]))
    M = np.zeros((nn * ndim, nn * ndim))
    Nm = np.zeros((ndim, nn * ndim))
    rho = model.rho[e]
    for q in range(len(R)):
        N = shape_func(sh, R[q])
        D = shape_deriv(sh, R[q][:ndim])
        for i in range(nn):
            for j in range(ndim):
                Nm[j, i * ndim + j] = N[i]
        J = C.T @ D
        detJ = np.linalg.det(J)
        if not detJ > 0.0:
            raise RuntimeError("Negative Jacobian determinant in cell %d" % (e + 1))
        th = model.thickness
        if model.stressmodel == AXISYM:  # th = 2 pi r at the IP (mech-solid.jl:180)
            th = 2 * math.pi * float(C[:, 0] @ N)
        coef = rho * detJ * w[q] * th
        M += coef * (Nm.T @ Nm)
    mp = model.eq_id[nodes, :ndim].reshape(-1)
    return M, mp


def mount_M(model, ndofs):
    """mount_M(elems, ndofs): entries with |M_ij| >= eps, duplicates summed -> scipy CSC."""
    import scipy.sparse as sp
    R, Cc, V = [], [], []
    for e in range(len(model.shape)):
        Me, mp = elem_mass(model, e)
        r, c = np.nonzero(np.abs(Me) >= EPS)
        R.append(mp[r]); Cc.append(mp[c]); V.append(Me[r, c])
    R, Cc, V = np.concatenate(R), np.concatenate(Cc), np.concatenate(V)
    return sp.coo_matrix((V, (R, Cc)), shape=(ndofs, ndofs)).tocsc()


SISM_DIRS = {"ux": 0, "fx": 0, "uy": 1, "fy": 1, "uz": 2, "fz": 2}


def sismic_acceleration(acc, tds, tf):
    """The acceleration of sismic_force (dyn-solver.jl:110-146): samples acc (the record, row by row)
    preceded by 0 at times i tds / n, linear between them, from the last interval holding tf (its loop
    never breaks early); no interval holds tf beyond tds, where the reference fails."""
    n = len(acc)
    AS2 = np.concatenate([[0.0], acc])
    vts = np.array([i * tds / n for i in range(n + 1)])
    ini = -1
    for i in range(n):
        if vts[i] <= tf <= vts[i + 1]:
            ini = i
    if ini < 0:
        raise ValueError("the seismic record does not cover t = %g" % tf)
    m = (AS2[ini + 1] - AS2[ini]) / (vts[ini + 1] - vts[ini])
    return AS2[ini] + m * (tf - vts[ini])


class DynStage:
    def __init__(self, bcs, nincs=1, nouts=0, tspan=0.0):
        self.bcs, self.nincs, self.nouts, self.tspan = list(bcs), nincs, nouts, float(tspan)


class DynAnalysis:
    """DynamicAnalysis(model) with addstage! and solve! (dyn_solver_params, dyn-solver.jl:166-186)."""

    def __init__(self, model):
        self.model = model
        self.stages = []
        self.t = 0.0
        self.log = []  # (increment, iteration, residue)

    def addstage(self, bcs, nincs=1, nouts=0, tspan=0.0):
        self.stages.append(DynStage(bcs, nincs, nouts, tspan))

    def solve(self, tol=0.01, dTmin=1e-7, dTmax=0.1, rspan=0.01, scheme="FE", maxits=5, autoinc=False,
              alpha=0.0, beta=0.0, sism=False, tss=0.0, tds=0.0, sism_file="", sism_dir="fx"):
        """sism: seismic input as dyn_stage_solver! intends it (dyn-solver.jl:106-157,271-287,348-352): the
        record of sism_file (readdlm, times 9.81) spread uniformly over tds, the force M (a(t) e_dir)
        added to Fex while tss <= t <= tss + tds."""
        if len(self.stages) != 1:
            raise ValueError("the dynamic solver runs one stage (velocities and accelerations exist in the first)")
        seis = None
        if sism:
            AS = 9.81 * np.loadtxt(sism_file, ndmin=2)
            seis = (AS.reshape(-1), float(tss), float(tds), SISM_DIRS[sism_dir])
        return self._stage(self.stages[0], tol, dTmin, dTmax, maxits, autoinc, alpha, beta, seis)

    def _seismic(self, M, ndofs, seis, tf):
        """sismic_force (dyn-solver.jl:106-157): a(tf) interpolated in the record, M (a e_dir)."""
        acc, _, tds, comp = seis
        a = sismic_acceleration(acc, tds, tf)
        VAS = np.zeros(ndofs)
        q = self.model.eq_id[:, comp]
        VAS[q[q >= 0]] += a
        return M @ VAS

    def _stage(self, stage, tol, dTmin, dTmax, maxits, autoinc, alpha, beta, seis=None):
        model = self.model
        dofs, nu, setup = configure_dofs(model, stage.bcs)
        ndofs = len(dofs)
        self.ndofs, self.nu = ndofs, nu
        umap = slice(0, nu)
        pmap = slice(nu, ndofs)
        nincs, nouts, tspan = stage.nincs, stage.nouts, stage.tspan
        saveouts = nouts > 0
        # initial accelerations (stage 1): M A = Fex
        K = mount_K(model, ndofs)
        M = mount_M(model, ndofs)
        A = np.zeros(ndofs)
        V = np.zeros(ndofs)
        Uex, Fex = get_bc_vals(model, setup, ndofs, 0.0)
        if seis is not None and seis[1] <= 0.0:
            Fex = Fex + self._seismic(M, ndofs, seis, 0.0)
        msg = solve_system(M, A, Fex, nu)
        self.A0, self.F0 = A.copy(), Fex.copy()
        StateBk = model.state.copy()
        dTbk = 0.0
        dTcheck = 1.0 / nouts if saveouts else 1.0
        Tcheck = dTcheck
        T = 0.0
        dT = 1.0 / nincs
        if autoinc:
            dT = min(dT, dTmax, dTcheck)
        t = self.t
        inc = 0
        U = np.zeros(ndofs)
        Fin = np.zeros(ndofs)
        Fina = np.zeros(ndofs)
        TFin = np.zeros(ndofs)
        dUa = np.zeros(ndofs)
        dUi = np.zeros(ndofs)
        Aa = np.zeros(ndofs)
        Va = np.zeros(ndofs)
        self.increments = 0
        self.iterations = 0
        while T < 1.0 - dTmin:
            dt = tspan * dT
            inc += 1
            Uex, Fex = get_bc_vals(model, setup, ndofs, t + dt)
            if seis is not None and seis[1] <= t + dt <= seis[2] + seis[1]:
                Fex = Fex + self._seismic(M, ndofs, seis, t + dt)
            Fex_Fin = Fex - Fina
            dUa[:] = 0.0
            dUi[:] = Uex
            residue = 0.0
            maxfails = 3
            nfails = 0
            nits = 0
            residue1 = 0.0
            converged = False
            for it in range(1, maxits + 1):
                if it > 1:
                    dUi[:] = 0.0
                lastres = residue
                K = mount_K(model, ndofs)
                # M depends on geometry and density only: the reference mounts it again here, with the
                # same values
                Cm = alpha * M + beta * K
                Kp = K + (4 / (dt ** 2)) * M + (2 / dt) * Cm
                dFp = Fex_Fin + M @ (A + 4 * V / dt - 4 * dUa / dt ** 2) + Cm @ (V - 2 * dUa / dt)
                solve_system(Kp, dUi, dFp, nu)
                model.state[:] = StateBk
                dUt = dUa + dUi
                dFin, status = update_state(model, dUt)
                Fina = Fin + dFin
                Va = -V + 2 * dUt / dt
                Aa = -A + 4 * (dUt - V * dt) / dt ** 2
                TFin = Fina + Cm @ Va + M @ Aa
                residue = np.abs((Fex - TFin)[umap]).max() if nu else 0.0
                dUa += dUi
                Fex_Fin = Fex - Fina
                Fex_Fin[pmap] = 0.0
                self.log.append((inc, it, residue))
                self.iterations += 1
                if it == 1:
                    residue1 = residue
                if residue > tol:
                    Fina = Fina - dFin
                if residue < tol:
                    converged = True
                    break
                if math.isnan(residue):
                    break
                if it > 1 and residue > lastres:
                    break
                if residue > 0.9 * lastres:
                    nfails += 1
                if nfails == maxfails:
                    break
            if converged:
                Fin = Fina
                U += dUa
                StateBk = model.state.copy()
                A = Aa
                V = Va
                T += dT
                t += dt
                self.increments += 1
                if T > Tcheck - dTmin:
                    Tcheck += dTcheck
                if autoinc:
                    if dTbk > 0.0:
                        dT = min(dTbk, Tcheck - T)
                        dTbk = 0.0
                    else:
                        q = (1 + math.tanh(math.log10(tol / residue1))) if nits == 1 else 1.0
                        dTtr = min(q * dT, 1 / nincs, 1 - T)
                        if T + dTtr > Tcheck - dTmin:
                            dTbk = dT
                            dT = Tcheck - T
                        else:
                            dT = dTtr
                            dTbk = 0.0
            else:
                inc -= 1
                model.state[:] = StateBk
                if autoinc:
                    q = 1 + math.tanh(math.log10(tol / residue1))
                    q = min(max(q, 0.2), 0.9)
                    dT = float("%.3g" % (q * dT))
                    if dT < dTmin:
                        return False, "solver did not converge"
                else:
                    return False, "solver did not converge"
        self.t = t
        self.T = T
        self.U, self.V, self.A, self.F = U, V, A, TFin
        self._to_nodes(dofs, U, V, A, TFin)
        return True, msg

    def _to_nodes(self, dofs, U, V, A, F):
        """dof.vals[us, vs, as, fs] per node (dyn-solver.jl:420-425), node-major arrays."""
        m = self.model
        for name, vec in (("U", U), ("V", V), ("A", A), ("F", F)):
            out = np.zeros((m.nnodes, m.ndim))
            for n in range(m.nnodes):
                for k in range(m.ndim):
                    q = m.eq_id[n, k]
                    if q >= 0:
                        out[n, k] = vec[q]
            setattr(m, name, out)
