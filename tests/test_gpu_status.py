"""The tensor-core kernels' failure reporting, made to fail on purpose without
faulting the GPU.

* Timeout: a test hook makes the first CTA's producer withhold one pipeline
  stage, with every bounded wait limited to 1 ms.  The MMA issuer's wait for
  that stage runs out, the CTA gives up cleanly (its copies and MMAs drained,
  TMEM freed), GB_ERR_TIMEOUT is recorded, and the callers raise.  The same
  GEMM then runs correctly: the context stays usable.
* Non-finite operand: a NaN in C cannot be cut into digit slices; the slicer
  records GB_ERR_NONFINITE and the split-product kernels refuse to start.

Every test leaves the hook off, the wait limit at its default and the status
word clear.
"""
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


@pytest.fixture
def clean_status(torch_cuda):
    from pynof_gb300 import _lib, ops

    ops.reset_device_status()
    yield
    _lib.call("gb_test_withhold_stage", -1)
    _lib.call("gb_set_wait_limit_ns", 0)
    torch_cuda.cuda.synchronize()
    ops.reset_device_status()


def _withheld(stage, limit_ns=1_000_000):
    from pynof_gb300 import _lib

    _lib.call("gb_set_wait_limit_ns", limit_ns)
    _lib.call("gb_test_withhold_stage", stage)


def _restore():
    from pynof_gb300 import _lib

    _lib.call("gb_test_withhold_stage", -1)
    _lib.call("gb_set_wait_limit_ns", 0)


def test_timeout_one_cta_per_tile(torch_cuda, clean_status):
    """C = A B^T with a row-major C takes the one-CTA-per-tile kernel."""
    from pynof_gb300 import _lib, ops

    rng = np.random.default_rng(5)
    A = rng.standard_normal((256, 96))
    B = rng.standard_normal((160, 96))
    dA, dB = ops.to_device(A), ops.to_device(B)
    _withheld(2)
    try:
        ops.dgemm_mixed(dA, dB, 6)
        torch_cuda.cuda.synchronize()
    finally:
        _restore()
    assert _lib.device_status(reset=False) == 5
    with pytest.raises(_lib.GBError) as ei:
        ops.check_device_status()
    assert ei.value.status == 5
    # while the word is set, later split-product launches refuse work and
    # report it again
    ops.dgemm_mixed(dA, dB, 6)
    with pytest.raises(_lib.GBError):
        ops.check_device_status()
    assert ops.reset_device_status() == 5
    C = ops.dgemm_mixed(dA, dB, 6)
    ops.check_device_status()
    assert nrel(C.cpu().numpy(), A @ B.T) < 1e-10


def test_timeout_persistent_build_and_drop_in_raises(torch_cuda, clean_status):
    """The JK build's GEMMs run on the persistent kernel; the drop-in
    JKj_RI_GPU raises instead of returning the unwritten J, K."""
    from oracle import pynof_oracle as orc
    from pynof_gb300 import _lib, integrals, ops, synthetic

    st = synthetic.Structure(nbf=96, nbfaux=180, ndoc=8, ncwo=4)
    b, C, H, n = synthetic.make_inputs(st, 4)
    db = ops.to_device(b)
    integrals.set_precision("mixed", 6)
    _withheld(1)
    try:
        with pytest.raises(_lib.GBError) as ei:
            integrals.JKj_RI_GPU(C, db, st)
    finally:
        _restore()
    assert ei.value.status == 5
    ops.reset_device_status()
    J, K = integrals.JKj_RI_GPU(C, db, st)
    Jr, Kr = orc.jkj_ri(C, b, st.nbf5)
    assert nrel(J, Jr) < 1e-10 and nrel(K, Kr) < 1e-10


def test_timeout_reaches_the_solver_step(torch_cuda, clean_status):
    """An orbital step of the device-resident solve loop raises too."""
    from pynof_gb300 import _lib, nof, solver, synthetic

    st = synthetic.Structure(nbf=48, nbfaux=120, ndoc=4, ncwo=4)
    b, C, H, n = synthetic.make_inputs(st, 6)
    be = solver.Backend(st, b, H, precision="mixed", use_graphs=False)
    cj, ck = nof.cjckd8(n, st)
    np.fill_diagonal(cj, 0.0)
    np.fill_diagonal(ck, 0.0)
    be.orbital_begin(C, n, cj, ck)
    _withheld(0)
    try:
        with pytest.raises(_lib.GBError):
            be.orbital_step(np.zeros(st.nvar))
    finally:
        _restore()


def test_nonfinite_operand_reported(torch_cuda, clean_status):
    from pynof_gb300 import _lib, integrals, ops, synthetic

    st = synthetic.Structure(nbf=64, nbfaux=128, ndoc=6, ncwo=4)
    b, C, H, n = synthetic.make_inputs(st, 9)
    db = ops.to_device(b)
    prep = ops.PreparedRI(db, 6)
    ops.check_device_status()
    Cbad = C.copy()
    Cbad[3, 5] = np.nan
    ops.jkj_ri_mixed(ops.to_device(Cbad), prep, st.nbf5)
    with pytest.raises(_lib.GBError) as ei:
        ops.check_device_status()
    assert ei.value.status == 6
    ops.reset_device_status()
    Cinf = C.copy()
    Cinf[7, 2] = np.inf
    integrals.set_precision("mixed", 6)
    with pytest.raises(_lib.GBError) as ei:
        integrals.JKj_RI_GPU(Cinf, db, st)
    assert ei.value.status == 6
    ops.reset_device_status()
    # finite inputs go through again
    ops.jkj_ri_mixed(ops.to_device(C), prep, st.nbf5)
    ops.check_device_status()
