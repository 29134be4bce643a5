"""GB300-native (sm_103a) tensor-product spectral path of jaxfun.

Transforms (forward / backward / scalar_product), fast-diagonalisation solves
and the variable-coefficient PCG run as hand-written CUDA kernels behind the C
ABI in ``include/jaxfun_gb300.h``; this package is the host-side mirror of the
jaxfun.galerkin / jaxfun.la call surface for that path.
"""

from . import _lib  # noqa: F401

__version__ = "0.1.0"


def load_library():
    """Load (building if needed) the CUDA library; raises if it is unavailable."""
    return _lib.load()
