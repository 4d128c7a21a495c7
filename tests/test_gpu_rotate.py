"""Device orbital rotation (rotate_orbital, utils.py:550-565) against the
oracle's scipy expm: C' to 1e-12 normwise, U orthogonal to 1e-13."""
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


def _p(nbf, nbf5):
    class P:
        pass

    p = P()
    p.nbf, p.nbf5 = nbf, nbf5
    return p


def _nvar(N, P):
    return N * (N - 1) // 2 - (N - P) * (N - P - 1) // 2


@pytest.mark.parametrize("N,P,scale", [(24, 24, 0.02), (37, 20, 0.05), (64, 32, 1.0), (150, 75, 0.3),
                                       (300, 150, 0.01), (128, 64, 5.0)])
def test_rotate_matches_scipy(torch_cuda, N, P, scale):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops

    rng = np.random.default_rng(N + P)
    y = rng.standard_normal(_nvar(N, P)) * scale
    C, _ = np.linalg.qr(rng.standard_normal((N, N)))
    ref = orc.rotate_orbital(y, C, _p(N, P))
    out = ops.rotate_orbital(ops.to_device(y), ops.to_device(C), P).cpu().numpy()
    err = nrel(out, ref)
    print(f"N={N} P={P} |y|~{scale}: {err:.2e}")
    assert err < 1e-12


def test_rotate_identity_and_orthogonality(torch_cuda):
    from pynof_gb300 import ops

    N, P = 96, 48
    rng = np.random.default_rng(3)
    eye = ops.to_device(np.eye(N))
    U0 = ops.rotate_orbital(ops.to_device(np.zeros(_nvar(N, P))), eye, P).cpu().numpy()
    assert np.array_equal(U0, np.eye(N))
    U = ops.rotate_orbital(ops.to_device(rng.standard_normal(_nvar(N, P)) * 0.7), eye, P).cpu().numpy()
    assert np.abs(U.T @ U - np.eye(N)).max() < 1e-13


def test_dropin_rotate_orbital(torch_cuda):
    """utils.rotate_orbital keeps the reference's host-in / host-out signature."""
    from oracle import pynof_oracle as orc
    from pynof_gb300 import utils

    N, P = 40, 20
    rng = np.random.default_rng(9)
    y = rng.standard_normal(_nvar(N, P)) * 0.1
    C, _ = np.linalg.qr(rng.standard_normal((N, N)))
    out = utils.rotate_orbital(y, C, _p(N, P))
    assert isinstance(out, np.ndarray) and out.shape == (N, N)
    assert nrel(out, orc.rotate_orbital(y, C, _p(N, P))) < 1e-12


def test_rotate_rejects_bad_input(torch_cuda):
    from pynof_gb300 import _lib, ops

    N, P = 16, 8
    C = ops.to_device(np.eye(N))
    y = ops.to_device(np.full(_nvar(N, P), np.nan))
    with pytest.raises(_lib.GBError):
        ops.rotate_orbital(y, C, P)
    with pytest.raises(ValueError):
        ops.rotate_orbital(ops.to_device(np.zeros(3)), C, P)


def test_host_norm_bound_matches_device_norm(torch_cuda):
    """A caller-supplied ||Y||_1 (no synchronisation) picks the same number of
    squarings as the device measurement: bitwise-identical results."""
    from pynof_gb300 import ops

    N, P = 80, 40
    rng = np.random.default_rng(5)
    y = rng.standard_normal(_nvar(N, P)) * 0.4
    C, _ = np.linalg.qr(rng.standard_normal((N, N)))
    dy, dC = ops.to_device(y), ops.to_device(C)
    a = ops.rotate_orbital(dy, dC, P).cpu().numpy()
    b = ops.rotate_orbital(dy, dC, P, norm1=ops.AntisymNorm(N, P)(y)).cpu().numpy()
    assert np.array_equal(a, b)
