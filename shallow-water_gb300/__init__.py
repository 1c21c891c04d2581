"""GB300-native (sm_103a) backend for the shallow-water hot path of
LukasBlanck/shallow-water: MUSCL + hydrostatic reconstruction + HLL + SSP-RK3 +
wall boundary conditions + the CFL max-wave-speed reduction.

The compute lives in ``libswe_gb300.so`` (CUDA, built in-tree by ``build.py``) behind
the C ABI in ``include/swe_gb300.h``; this package is the Python host side of that
ABI.  Import it with ``importlib.import_module("shallow-water_gb300")``.
"""
from . import problems  # noqa: F401
from ._lib import lib  # noqa: F401
from .solver import Solver, SweError  # noqa: F401
from .ensemble import Ensemble  # noqa: F401
from . import adjoint  # noqa: F401
from . import slabs  # noqa: F401
from . import output  # noqa: F401

__all__ = ["Solver", "SweError", "Ensemble", "adjoint", "slabs", "output", "problems", "lib"]
