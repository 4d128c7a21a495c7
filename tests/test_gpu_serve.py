"""Served solves on the GPU: continuous batching with overlap, and every
result is the same alone and in the mix (the kernels and the host math are
deterministic, so the energies must agree to the last bit)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("occupations", ["host", "device", "device_sync"])
def test_alone_equals_in_mix(torch_cuda, occupations):
    """With the occupation CG on the host, or on the device per request (its
    own workspace and graphs, fixed-order reductions), from a conditional
    node or driven from the host."""
    from pynof_gb300 import serve

    reqs = serve.poisson_stream(6, rate=200.0, nbf_lo=24, nbf_hi=48, seed=5)
    mixed = serve.Server(slots=4, tol=1e-4, maxit=60, occupations=occupations)
    rep = mixed.run(reqs)
    assert rep["completed"] == 6 and rep["failed"] == 0, mixed.errors
    assert rep["peak_active"] > 1  # requests were on the GPU together
    in_mix = {r.rid: r.E_elec for r in mixed.results}
    for req in reqs[:3]:
        alone = serve.Server(slots=1, tol=1e-4, maxit=60, occupations=occupations)
        rep1 = alone.run([serve.Request(req.rid, req.nbf, req.seed, 0.0)])
        assert rep1["completed"] == 1
        assert alone.results[0].E_elec == in_mix[req.rid]


def test_fp64_plain_path_serves(torch_cuda):
    from pynof_gb300 import serve

    reqs = serve.poisson_stream(3, rate=100.0, nbf_lo=24, nbf_hi=32, seed=9)
    srv = serve.Server(slots=3, precision="fp64", tol=1e-4, maxit=60)
    rep = srv.run(reqs)
    assert rep["completed"] == 3 and rep["p99_latency_s"] >= rep["p50_latency_s"] > 0
