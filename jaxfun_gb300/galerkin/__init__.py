"""Spaces and tensor-product transforms (mirrors jaxfun.galerkin)."""

from .spaces import (  # noqa: F401
    DIRICHLET,
    BCGeneric,
    BCValue,
    DirectSum,
    Chebyshev,
    Composite,
    FunctionSpace,
    Legendre,
    OrthogonalSpace,
    chebyshev_gauss,
    legendre_gauss,
)
from .tensorproductspace import (  # noqa: F401
    DirectSumTPS,
    TensorProduct,
    TensorProductSpace,
    tp_apply,
    tp_apply_affine,
)
