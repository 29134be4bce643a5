"""CPU FP64 oracle for the tensor-product spectral path (TEST INFRASTRUCTURE ONLY).

This package restates, in NumPy/SciPy FP64, the algorithms jaxfun uses on the
transform / fast-diagonalisation / variable-coefficient path.  It is the
checker: only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
legs of ``bench.py`` may import it.  The product (``jaxfun_gb300``) never
imports it and has no CPU fallback.

Parity pin: jaxfun (JAX/XLA) cannot be imported in this environment, so the
restatement is pinned against the reference's own known-answer tests
(tests/galerkin/test_inner.py:580-650 quadrature values,
tests/la/test_tpmatrices_solvers.py:91-104 manufactured Poisson solution,
tests/galerkin/test_forward_backward.py:20-104 round trips,
src/jaxfun/galerkin/arguments.py:728-737 Chebyshev scalar product) and the
committed fixtures in ``tests/golden`` generated by
``tests/golden/make_golden.py``.
"""

from . import spectral  # noqa: F401
