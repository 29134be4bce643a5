"""Edge cases of the public GPU path: empty batches return empty results
without launching, shapes the tensor cores cannot take fail loudly, and the
C ABI accepts a zero batch as a no-op."""

import numpy as np
import pytest
import torch

from jaxfun_gb300 import _lib
from jaxfun_gb300.galerkin import DIRICHLET, FunctionSpace, Legendre, TensorProduct
from jaxfun_gb300.galerkin.tensorproductspace import tp_apply_tc
from jaxfun_gb300.la import poisson_tpmatrices

pytestmark = pytest.mark.gpu


def _T(N, nd=2):
    D = FunctionSpace(N, Legendre, bcs=DIRICHLET)
    return TensorProduct(*([D] * nd))


def test_empty_batches():
    T = _T(16)
    c = torch.zeros((0, 14, 14), dtype=torch.float64, device="cuda")
    u = T.backward(c)
    assert tuple(u.shape) == (0, 16, 16)
    assert tuple(T.forward(u).shape) == (0, 14, 14)
    assert tuple(T.scalar_product(u).shape) == (0, 14, 14)
    assert tuple(poisson_tpmatrices(T).solve(c).shape) == (0, 14, 14)
    Tl = TensorProduct(FunctionSpace(16, Legendre, bcs={"left": {"D": 1.0}, "right": {"D": 2.0}}),
                       FunctionSpace(16, Legendre, bcs=DIRICHLET))
    assert tuple(Tl.backward(c).shape) == (0, 16, 16)


def test_zero_batch_contraction_is_a_no_op():
    L = _lib.lib()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    d = _lib.ContractDesc(batch=0, nseg=1, M=4, P=4, K=4, op_ld=4, in_ld=4, in_batch=16,
                          out_ld=4, out_batch=16, alpha=1.0, beta=0.0)
    for fn in (L.jfg_contract_f64, L.jfg_contract_df64):
        assert fn(d, x.data_ptr(), x.data_ptr(), x.data_ptr(), _lib.stream_handle()) == 0
    torch.cuda.synchronize()
    assert int(L.jfg_device_status()) == 0


def test_tensor_core_shape_limits_fail_loudly():
    """Split-TF32 passes need operator rows / columns that are multiples of 4
    (16-byte TMA rows); other sizes raise instead of falling back."""
    mats = [np.random.default_rng(0).standard_normal((17, 17))] * 2
    with pytest.raises(_lib.JfgError):
        tp_apply_tc(mats, torch.zeros((1, 17, 17), dtype=torch.float32, device="cuda"))
    torch.cuda.synchronize()
    assert int(_lib.lib().jfg_device_status()) == 0


def test_shape_mismatch_is_a_value_error():
    T = _T(16)
    with pytest.raises(ValueError):
        T.backward(torch.zeros((2, 13, 14), dtype=torch.float64, device="cuda"))
