"""Generate the known-answer fixtures in tests/golden/kat.json.

The values are the known answers the jaxfun test-suite checks its own
quadrature against, computed the same way the reference tests compute them:
  * tests/galerkin/test_inner.py:580-609 — sympy exact integral of
    (x^2+y^2) P5(x)^2 P5(y)^2 over [-1,1]^2 (TensorMatrix corner entry,
    Legendre N=6, exact with 7x7 quadrature points);
  * tests/galerkin/test_inner.py:611-650 — scipy dblquad of
    sqrt(x^2+y^2) P5(x)^2 P5(y)^2 (exact to sqrt(ulp(100)) with 32x32 points);
  * src/jaxfun/galerkin/arguments.py:728-737 — Chebyshev N=4 scalar product of
    w = 1: [pi, pi/2, pi/2, pi/2];
  * tests/la/test_tpmatrices_solvers.py:91-104 — manufactured Poisson solution
    u = (1-x^2)(1-y^2), N=16, L2 error on the 40x40 grid below ulp(100);
    stored here as the bound.
Run: python tests/golden/make_golden.py
"""

import json
import os

import numpy as np
import sympy as sp
from scipy.integrate import dblquad

x, y = sp.symbols("x y", real=True)
N = 6
t_exact = sp.integrate(
    (x**2 + y**2) * sp.legendre(N - 1, x) ** 2 * sp.legendre(N - 1, y) ** 2,
    (x, -1, 1), (y, -1, 1),
)
f = sp.lambdify((x, y), sp.sqrt(x**2 + y**2) * sp.legendre(N - 1, x) ** 2 * sp.legendre(N - 1, y) ** 2)
ulp100 = float(np.spacing(100.0))
t_sqrt, _ = dblquad(f, -1, 1, -1, 1, epsabs=ulp100)
out = {
    "tensormatrix_x2y2_legendre6": float(t_exact),
    "tensormatrix_sqrt_legendre6": float(t_sqrt),
    "atol_sqrt_ulp100": float(np.sqrt(ulp100)),
    "chebyshev4_scalar_product_of_one": [float(np.pi), float(np.pi / 2), float(np.pi / 2), float(np.pi / 2)],
    "poisson_manufactured_l2_bound": ulp100,
}
path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
with open(path, "w") as fh:
    json.dump(out, fh, indent=1)
print(json.dumps(out, indent=1))
