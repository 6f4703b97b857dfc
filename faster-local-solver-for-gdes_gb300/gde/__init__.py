"""GB300-native local push solvers for graph diffusion equations.

``gde.api`` is the host API over ``libgde.so`` (C ABI in ``include/gde.h``);
``gde.graphs`` generates the seeded synthetic graphs.  The drop-in modules
``ppr_solver``, ``katz_solver``, ``hk_solver`` and ``InstantGNN`` sit next to
this package and keep the reference's function names and signatures.
"""
from . import _lib  # noqa: F401
