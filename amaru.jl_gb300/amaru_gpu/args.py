"""Keyword-argument checks of the analysis solvers, as checkargs applies them (src/tools/arguments.jl:228-245).

Each table restates the conditions of the reference's parameter table for that solver:
  MECH_SOLVER_PARAMS   mech_solver_params, src/mech/mech-solver.jl:155-167
  DYN_SOLVER_PARAMS    dyn_solver_params, src/mech/dyn-solver.jl:166-186

A value that breaks a condition raises ArgumentError with the reference's message. The checks run on the
host before anything reaches the device.
"""


class ArgumentError(ValueError):
    """AmaruException raised by checkargs for an argument outside its condition or set of values."""


# (key, condition as the reference writes it, predicate)
MECH_SOLVER_PARAMS = [
    ("tol", "tol > 0", lambda v: v > 0),
    ("rspan", "0 < rspan < 1", lambda v: 0 < v < 1),
    ("rtol", "rtol > 0", lambda v: v > 0),
    ("dT0", "0 < dT0 <= 1", lambda v: 0 < v <= 1),
    ("dTmin", "0 < dTmin < 1", lambda v: 0 < v < 1),
    ("dTmax", "0 < dTmax < 1", lambda v: 0 < v < 1),
    ("maxits", "1 <= maxits <= 10", lambda v: 1 <= v <= 10),
]
MECH_SOLVER_VALUES = {"scheme": ("FE", "ME", "BE", "Ralston")}

DYN_SOLVER_PARAMS = [
    ("tol", "tol > 0", lambda v: v > 0),
    ("dTmin", "0 < dTmin < 1", lambda v: 0 < v < 1),
    ("dTmax", "0 < dTmax < 1", lambda v: 0 < v < 1),
    ("rspan", "0 < rspan < 1", lambda v: 0 < v < 1),
    ("maxits", "1 <= maxits <= 10", lambda v: 1 <= v <= 10),
]


def checkargs(fname, table, values=None, **kw):
    """Raises ArgumentError for the first argument (in table order) that breaks its condition, then for
    the first one outside its set of values."""
    for key, cond, ok in table:
        if key in kw and kw[key] is not None:
            v = kw[key]
            try:
                good = bool(ok(v))
            except TypeError:
                good = False
            if not good:
                raise ArgumentError("%s: Invalid value for argument %s which must satisfy %s.\nGot %s = %r"
                                    % (fname, key, cond, key, v))
    for key, allowed in (values or {}).items():
        if key in kw and kw[key] not in allowed:
            raise ArgumentError("%s: Invalid value for argument %s which must be one of %s.\nGot %s = %r"
                                % (fname, key, allowed, key, kw[key]))
