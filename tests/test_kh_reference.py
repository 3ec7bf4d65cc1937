"""The PyTorch FP64 restatement of the frozen-mesh KH step (tests/kh_reference.py),
which supplies the reference gradient of the adjoint tests, against the
oracle: same problem, same steps, interior state equal to rounding."""
import numpy as np
import torch

import amr2d_mhd_gb300 as amr
import kh_reference as K
from oracle import pyoracle as P
from parity_util import oracle_kw


def test_torch_kh_step_matches_oracle():
    c = amr.kh_config(5)
    a = torch.tensor(list(c.ic_param[:16]), dtype=torch.float64)
    U, Bx, By = K.kh_ic(a)
    o = P.Oracle(**oracle_kw(c, 16)).init()
    ic = o.get("icoord")
    U0 = K.from_blocks(o.get("U"), ic)
    assert np.allclose(U.numpy(), U0, rtol=1e-14, atol=1e-15)
    for _ in range(6):
        U, Bx, By = K.step(U, Bx, By, 2e-4, 5.0 / 3.0, 1.0 / 256)
    o.run(6)
    Uo = K.from_blocks(o.get("U"), ic)
    Bo = K.from_blocks(o.get("Bi"), ic)
    scale = np.abs(Uo).max(axis=(1, 2), keepdims=True) + 1e-30
    assert np.abs(U.numpy() - Uo).max() / scale.max() < 1e-12
    for k in range(8):
        assert np.abs(U.numpy()[k] - Uo[k]).max() <= 1e-11 * scale[k, 0, 0] + 1e-16, k
    assert np.abs(Bx.numpy() - Bo[0]).max() < 1e-13
    assert np.abs(By.numpy() - Bo[1]).max() < 1e-13
