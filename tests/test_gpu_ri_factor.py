"""The RI factor b_mnl = (mn|k) metric^(-1/2) (compute_integrals,
integrals.py:35-49) on the device against the oracle: the metric power with
its eigenvalue cutoff on the host, the contraction in FP64 DMMA (1e-12) and
in the split-product form (S = 6: 1e-10)."""
import numpy as np
import pytest

from conftest import nrel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _inputs(N, Q, seed):
    rng = np.random.default_rng(seed)
    mnk = rng.standard_normal((N, N, Q)) * np.exp(-0.05 * np.add.outer(np.arange(N), np.arange(N)))[:, :, None]
    mnk = 0.5 * (mnk + mnk.transpose(1, 0, 2))
    # SPD metric with a spread of eigenvalues, a few below the 1e-14 cutoff
    V, _ = np.linalg.qr(rng.standard_normal((Q, Q)))
    ev = np.logspace(0, -12, Q)
    ev[-3:] = 1e-16
    return mnk, (V * ev) @ V.T


@pytest.mark.parametrize("N,Q", [(24, 116), (40, 160)])
def test_ri_factor_vs_oracle(torch_cuda, N, Q):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import integrals

    mnk, metric = _inputs(N, Q, N + Q)
    ref = orc.b_mnl(mnk, metric)
    M = integrals.metric_power(metric)
    assert nrel(M, orc.metric_power(metric)) < 1e-12
    b64 = integrals.compute_b_mnl(mnk, metric).cpu().numpy()
    assert nrel(b64, ref) < 1e-12
    b6 = integrals.compute_b_mnl(mnk, M, nslices=6, metric_is_power=True).cpu().numpy()
    assert nrel(b6, ref) < 1e-10
    # the result keeps the (m, n) symmetry the JK kernels rely on
    assert np.array_equal(b64, b64.transpose(1, 0, 2))
