"""GB300-native exact-diagonalization hot path of lattice-symmetries.

Import with ``importlib.import_module("lattice-symmetries_gb300")`` (the directory name is not a
Python identifier).  The public names mirror the reference's ``lattice_symmetries`` module:

    Symmetry, Symmetries, SpinBasis, SpinfulFermionBasis, SpinlessFermionBasis, Expr, Operator

plus the batched GPU additions SectorBatch (many symmetry sectors in one launch) and the
block-Lanczos driver in ``lanczos``.

All numeric work (orbit scan, basis enumeration, state index, H*x) runs in libls_gb300.so on the
GPU; importing this package fails if that library has not been built.
"""

from ._group import Symmetry, Symmetries  # noqa: F401
from ._expr import Expr  # noqa: F401
from . import _native  # noqa: F401
from ._api import (Basis, Operator, SectorBatch, SpinBasis, SpinfulFermionBasis,  # noqa: F401
                   SpinlessFermionBasis, basis_from_json, load_basis, load_library, set_tracing,
                   stage_times)

__version__ = "2.2.0+gb300"

_native.load()
