"""CPU oracle for the Amaru mechanical hot path.

TEST INFRASTRUCTURE ONLY: a restatement of NumSoftware/Amaru.jl's Float64
algorithms (element stiffness, constitutive updates, mount_K, update_state!,
solve_system!, get_bc_vals, the staged Newton driver, the structured mesher
and the nodal patch recovery of the output data, mount_M, the dynamic
Newmark solver, the modal solver and the VTU writer).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import it, and
only as the checker.  The CUDA library never calls it.

Parity pin: tests/test_oracle_golden.py checks this oracle against every
known-answer test of the reference's test suite for this path
(test/mech/elem/elastic-hex8.jl, elastic-quad4.jl, elastic-elems.jl,
test/mech/mat/vm-3d.jl, vm-2d.jl, dp.jl, test/mesh/structured.jl, test/mech/elem/axisymmetric.jl).  The
reference's tests hold no nodal recovery values; the recovery restatement is
pinned by the fields it must reproduce exactly (polynomials of the regression
space) in tests/test_recovery.py.  The dynamic and modal restatements are pinned
by properties of their methods (tests/test_dynamic.py: the consistent mass, the
conserved discrete energy, the closed Newmark recursion; tests/test_modal.py: the
dense eigenproblem), and the VTU writer by a snippet written from the
reference's writer (tests/test_vtu.py).  tests/golden/ stores outputs of this
oracle, and tests/test_golden.py checks that it still reproduces them.
"""
from .core import *  # noqa: F401,F403
from .recovery import nodal_patch_recovery, ip_coords, ip_state_vals, field_names  # noqa: F401
from .dynamic import DynAnalysis, mount_M, elem_mass  # noqa: F401
from .modal import modal, modal_dense  # noqa: F401
from . import vtu  # noqa: F401
