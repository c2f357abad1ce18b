"""Oracle restatement of Amaru.jl's modal solver (test infrastructure only).

mech_modal_solver! (src/mech/mech-modal-solver.jl:72-235): K11 and M11 mounted on the unknown DOFs,
L = sum(M11, dims=1) (the row-sum lumped masses), P = K11 ./ L (column j divided by L[j]), and the
nmodes eigenpairs of P of smallest magnitude (Arpack's eigs(P, nev=nmodes, which=:SM)), kept when
real and positive, sorted ascending; omega = sqrt(lambda), the modes are P's eigenvectors (unit
2-norm).  P = K11 diag(L)^-1 has the eigenpairs of the pencil K11 phi = lambda diag(L) phi with
v = diag(L) phi.  The row-sum lumped masses of serendipity cells (QUAD8, HEX20, TET10) are negative at
the corners, so diag(L) is indefinite; the restatement solves the reciprocal pencil
diag(L) phi = mu K11 phi, symmetric-definite with K11, for its largest positive mu = 1/lambda (scipy's
eigsh).  When the reference's filter succeeds, its nmodes eigenvalues of smallest magnitude are
positive, and they are these.
"""
import numpy as np

from .core import configure_dofs, mount_K
from .dynamic import mount_M


def lumped(M11):
    """L = sum(M11, dims=1) as a vector."""
    return np.asarray(M11.sum(axis=0)).ravel()


def modal(model, bcs, nmodes=5):
    """-> (omega (nmodes), modes (nu x nmodes, unit 2-norm columns, sign: largest entry positive), nu)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    if (model.rho <= 0).any():
        raise ValueError("mech_modal_solver: density should not be zero")
    dofs, nu, _ = configure_dofs(model, bcs)
    nd = len(dofs)
    K11 = mount_K(model, nd).tocsc()[:nu, :nu]
    M11 = mount_M(model, nd).tocsc()[:nu, :nu]
    L = lumped(M11)
    k = min(nu - 1, 2 * nmodes + 4)
    # a fixed start vector (ARPACK draws a random one otherwise), so that repeated runs agree bit for bit
    v0 = np.random.default_rng(0x5EED).uniform(-1.0, 1.0, nu)
    mu, phi = sla.eigsh(sp.diags(L).tocsc(), k=k, M=K11, which="LA", v0=v0)
    keep = np.nonzero(mu > 0)[0]
    keep = keep[np.argsort(-mu[keep])][:nmodes]
    lam, phi = 1.0 / mu[keep], phi[:, keep]
    V = L[:, None] * phi
    V /= np.linalg.norm(V, axis=0)
    V *= np.sign(V[np.abs(V).argmax(axis=0), np.arange(V.shape[1])])
    return np.sqrt(lam), V, nu


def modal_dense(model, bcs, nmodes=5):
    """The same from the dense, non-symmetric P = K11 ./ L with numpy's eig (small models only): the
    reference's formulation, used to pin the symmetric restatement."""
    dofs, nu, _ = configure_dofs(model, bcs)
    nd = len(dofs)
    K11 = mount_K(model, nd).toarray()[:nu, :nu]
    M11 = mount_M(model, nd).toarray()[:nu, :nu]
    L = M11.sum(axis=0)
    P = K11 / L[None, :]
    lam, V = np.linalg.eig(P)
    # P is similar to a symmetric matrix: its eigenvalues are real, and an imaginary part of the
    # non-symmetric solver's size is round-off (isreal in the reference's filter, for Arpack's output)
    keep = [i for i in range(len(lam)) if abs(lam[i].imag) <= 1e-9 * abs(lam[i]) and lam[i].real > 0]
    keep = sorted(keep, key=lambda i: lam[i].real)[:nmodes]
    lam = lam[keep].real
    V = V[:, keep].real
    V /= np.linalg.norm(V, axis=0)
    V *= np.sign(V[np.abs(V).argmax(axis=0), np.arange(V.shape[1])])
    return np.sqrt(lam), V, nu
