"""Linear algebra on the GPU path (mirrors jaxfun.la)."""

from .tpmatrix import (  # noqa: F401
    SolverNotApplicable,
    TPMatrices,
    TPMatricesLUFactors,
    TPMatrix,
    fd_eig,
    tpmats_lu_factor,
)
from .mixed import MixedVarCoefSolver, split_tf32  # noqa: F401
from .varcoef import (  # noqa: F401
    VarCoefMatrix,
    fd_preconditioner,
    helmholtz_system,
    pack_varcoef_ops,
    pcg,
    poisson_tpmatrices,
)
from .wavenumber import DiaMatrix, TPMatricesWavenumberSolver  # noqa: F401
