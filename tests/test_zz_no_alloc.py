"""The allocation-free JK build entry point agrees with the regular one.

gb_jkj_ri_noalloc_f64 serves callers that may not allocate device memory
(their HBM belongs to another allocator or a fixed arena, or cudaMalloc would
synchronise a latency-critical loop): it takes its scratch from a built-in
device array instead of a caller workspace.  This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

from conftest import load_golden, nrel, param_for

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _noalloc(torch, dC, db, P):
    from pynof_gb300 import _lib

    N, _, Q = db.shape
    J = torch.full((P, N, N), float("nan"), dtype=torch.float64, device=db.device)
    K = torch.full((P, N, N), float("nan"), dtype=torch.float64, device=db.device)
    stream = torch.cuda.current_stream().cuda_stream
    _lib.call("gb_jkj_ri_noalloc_f64", dC.data_ptr(), db.data_ptr(), N, P, Q, J.data_ptr(), K.data_ptr(), stream)
    torch.cuda.synchronize()
    return J.cpu().numpy(), K.cpu().numpy()


def test_noalloc_matches_regular_entry_point_twice(torch_cuda):
    from pynof_gb300 import ops

    # two different problems back to back: the second call finds the first
    # call's data in the shared scratch and must not depend on it
    for name in ("ragged", "c1", "ragged"):
        g = load_golden(name)
        p = param_for(name)
        dC, db = ops.to_device(g["C"]), ops.to_device(g["b"])
        J0, K0 = (t.cpu().numpy() for t in ops.jkj_ri(dC, db, p.nbf5))
        for _ in range(2):
            J, K = _noalloc(torch_cuda, dC, db, p.nbf5)
            assert np.isfinite(J).all() and np.isfinite(K).all()
            assert nrel(J, J0) < TOL and nrel(K, K0) < TOL
            assert nrel(J, g["J_ri"]) < TOL and nrel(K, g["K_ri"]) < TOL


def test_noalloc_rejects_oversized_problem(torch_cuda):
    from pynof_gb300 import _lib, ops

    N, P, Q = 64, 64, 2100  # P*N*Q doubles = 68.8 MB > 64 MiB of built-in scratch
    assert _lib.query("gb_jkj_ri_workspace_f64", N, P, Q) > 64 * 1024 * 1024
    C = torch_cuda.zeros((N, N), dtype=torch_cuda.float64, device="cuda")
    b = torch_cuda.zeros((N, N, Q), dtype=torch_cuda.float64, device="cuda")
    J = torch_cuda.zeros((P, N, N), dtype=torch_cuda.float64, device="cuda")
    K = torch_cuda.zeros((P, N, N), dtype=torch_cuda.float64, device="cuda")
    with pytest.raises(_lib.GBError) as ei:
        _lib.call("gb_jkj_ri_noalloc_f64", C.data_ptr(), b.data_ptr(), N, P, Q, J.data_ptr(), K.data_ptr(),
                  torch_cuda.cuda.current_stream().cuda_stream)
    assert ei.value.status == 3 and "built-in scratch" in str(ei.value)
