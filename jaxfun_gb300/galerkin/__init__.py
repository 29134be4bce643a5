"""Spaces and tensor-product transforms (mirrors jaxfun.galerkin)."""

from .spaces import (  # noqa: F401
    DIRICHLET,
    Chebyshev,
    Composite,
    FunctionSpace,
    Legendre,
    OrthogonalSpace,
    chebyshev_gauss,
    legendre_gauss,
)
from .tensorproductspace import TensorProduct, TensorProductSpace, tp_apply  # noqa: F401
