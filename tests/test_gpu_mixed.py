"""Split-product tensor-core path (tcgen05) against FP64.

Tolerances (normwise max|d| / max|ref|): nslices=6 must meet the FP64 bar of
1e-10 (it lands near 1e-12); nslices=2 (bf16x3, 14-bit digits) is held to 1e-3.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, nrel, param_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_dgemm_small_integers_exact(torch_cuda):
    """Integers below 128 are one exact digit: nslices=1 must be exact."""
    from pynof_gb300 import ops

    rng = np.random.default_rng(1)
    A = rng.integers(-100, 100, (128, 32)).astype(np.float64)
    B = rng.integers(-100, 100, (128, 32)).astype(np.float64)
    C = ops.dgemm_mixed(ops.to_device(A), ops.to_device(B), nslices=1).cpu().numpy()
    ops.check_device_status()
    assert np.array_equal(C, A @ B.T)


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (200, 300, 500), (77, 130, 1000), (256, 384, 2400),
                                   (130, 70, 30000)])
def test_dgemm_random(torch_cuda, M, N, K):
    from pynof_gb300 import ops

    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((M, K)) * np.exp(-0.05 * np.arange(M))[:, None]
    B = rng.standard_normal((N, K))
    ref = A @ B.T
    # tf32x3 accumulates in the tensor core's FP32 accumulator over all of K,
    # whose rounding error grows with K (2e-4 at K = 30000 on GB300)
    for S, tol in ((6, 1e-10), (2, 1e-3), (ops.SPLIT_TF32X3, 1e-4 if K <= 4096 else 1e-3)):
        C = ops.dgemm_mixed(ops.to_device(A), ops.to_device(B), nslices=S).cpu().numpy()
        ops.check_device_status()
        err = nrel(C, ref)
        print(f"dgemm M={M} N={N} K={K} nslices={S}: {err:.2e}")
        assert err < tol, (S, err)


@pytest.fixture(params=sorted(GOLDEN_CASES))
def case(request, torch_cuda):
    from pynof_gb300 import ops

    name = request.param
    g = load_golden(name)
    return g, param_for(GOLDEN_CASES[name]), {k: ops.to_device(g[k]) for k in ("b", "C")}


def test_jkj_ri_mixed_golden(case):
    from pynof_gb300 import ops

    g, p, d = case
    prep = ops.PreparedRI(d["b"], nslices=6)
    J, K = ops.jkj_ri_mixed(d["C"], prep, p.nbf5)
    ops.check_device_status()
    assert nrel(J.cpu().numpy(), g["J_ri"]) < 1e-10
    assert nrel(K.cpu().numpy(), g["K_ri"]) < 1e-10


@pytest.mark.parametrize("code,tol", [(2, 1e-3), (32, 1e-4)])
def test_jkj_ri_split3_golden(case, code, tol):
    """The three-product forms: bf16x3 (nslices=2) and tf32x3 (GB_SPLIT_TF32X3)."""
    from pynof_gb300 import ops

    g, p, d = case
    prep = ops.PreparedRI(d["b"], nslices=code)
    J, K = ops.jkj_ri_mixed(d["C"], prep, p.nbf5)
    ops.check_device_status()
    ej, ek = nrel(J.cpu().numpy(), g["J_ri"]), nrel(K.cpu().numpy(), g["K_ri"])
    print(f"split code {code}: J {ej:.2e} K {ek:.2e}")
    assert ej < tol and ek < tol


@pytest.mark.parametrize("N,Q,ndoc,ncwo,seed", [(67, 131, 6, 4, 12), (150, 600, 15, 4, 5), (300, 600, 30, 4, 3)])
def test_jkj_ri_mixed_vs_oracle(torch_cuda, N, Q, ndoc, ncwo, seed):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    st = synthetic.Structure(nbf=N, nbfaux=Q, ndoc=ndoc, ncwo=ncwo)
    b, C, H, n = synthetic.make_inputs(st, seed)
    Jr, Kr = orc.jkj_ri(C, b, st.nbf5)
    db, dC = ops.to_device(b), ops.to_device(C)
    for S, tol in ((6, 1e-10), (2, 1e-3)):
        prep = ops.PreparedRI(db, nslices=S)
        J, K = ops.jkj_ri_mixed(dC, prep, st.nbf5)
        ops.check_device_status()
        print(f"jkj N={N} Q={Q} nslices={S}: J {nrel(J.cpu().numpy(), Jr):.2e} K {nrel(K.cpu().numpy(), Kr):.2e}")
        assert nrel(J.cpu().numpy(), Jr) < tol, (S, nrel(J.cpu().numpy(), Jr))
        assert nrel(K.cpu().numpy(), Kr) < tol, (S, nrel(K.cpu().numpy(), Kr))


def test_jkh_mo_and_lagrange2_mixed_golden(case):
    from pynof_gb300 import ops

    g, p, d = case
    prep = ops.PreparedRI(d["b"], nslices=6)
    dH = ops.to_device(g["H"])
    a, b, c = ops.jkh_mo_ri_mixed(d["C"], dH, prep, p.nbf5)
    ops.check_device_status()
    assert nrel(a.cpu().numpy(), g["J_MO_ri"]) < 1e-10
    assert nrel(b.cpu().numpy(), g["K_MO_ri"]) < 1e-10
    assert nrel(c.cpu().numpy(), g["H_core"]) < 1e-10
    el, Hm = ops.lagrange2_ri_mixed(d["C"], dH, prep, ops.to_device(g["n_soft"]), ops.to_device(g["cj12"]),
                                    ops.to_device(g["ck12"]), p.nbf5, p.nbeta, p.nalpha)
    ops.check_device_status()
    assert nrel(el.cpu().numpy(), g["elag2_ri"]) < 1e-10
    assert nrel(Hm.cpu().numpy(), g["Hmat"]) < 1e-10


def test_jkh_mo_and_lagrange2_mixed_vs_oracle(torch_cuda):
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    st = synthetic.Structure(nbf=150, nbfaux=600, ndoc=15, ncwo=4)
    b, C, H, n = synthetic.make_inputs(st, 8)
    P = st.nbf5
    db, dC, dH = ops.to_device(b), ops.to_device(C), ops.to_device(H)
    cj = 2 * np.outer(n, n)
    ck = np.outer(n, n) + 0.1
    ar, br, cr = orc.jkh_mo_ri(C, H, b, P)
    elr, Hr = orc.lagrange2(n, cj.copy(), ck.copy(), C, H, None, b, st)
    for S, tol in ((6, 1e-10), (2, 1e-3)):
        prep = ops.PreparedRI(db, nslices=S)
        a, bb, c = ops.jkh_mo_ri_mixed(dC, dH, prep, P)
        el, Hm = ops.lagrange2_ri_mixed(dC, dH, prep, ops.to_device(n), ops.to_device(cj), ops.to_device(ck), P,
                                        st.nbeta, st.nalpha)
        ops.check_device_status()
        errs = [nrel(a.cpu().numpy(), ar), nrel(bb.cpu().numpy(), br), nrel(el.cpu().numpy(), elr)]
        print(f"nslices={S}: J_MO {errs[0]:.2e} K_MO {errs[1]:.2e} elag {errs[2]:.2e}")
        assert max(errs) < tol, (S, errs)
        assert nrel(c.cpu().numpy(), cr) < 1e-12 and nrel(Hm.cpu().numpy(), Hr) < 1e-12


def test_jkh_lagrange2_fused_mixed(torch_cuda):
    """computeJKH_MO and computeLagrange2 in one call (one half transform and
    one MO transform for both) against the oracle, and against the two
    separate calls on the same inputs."""
    from oracle import pynof_oracle as orc
    from pynof_gb300 import ops, synthetic

    st = synthetic.Structure(nbf=130, nbfaux=520, ndoc=13, ncwo=4)
    b, C, H, n = synthetic.make_inputs(st, 11)
    P = st.nbf5
    db, dC, dH = ops.to_device(b), ops.to_device(C), ops.to_device(H)
    cj = 2 * np.outer(n, n)
    ck = np.outer(n, n) + 0.1
    ar, br, cr = orc.jkh_mo_ri(C, H, b, P)
    elr, Hr = orc.lagrange2(n, cj.copy(), ck.copy(), C, H, None, b, st)
    dn, dcj, dck = ops.to_device(n), ops.to_device(cj), ops.to_device(ck)
    for S, tol in ((6, 1e-10), (2, 1e-3)):
        prep = ops.PreparedRI(db, nslices=S)
        a, bb, c, el, Hm = ops.jkh_lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta, st.nalpha)
        ops.check_device_status()
        errs = [nrel(a.cpu().numpy(), ar), nrel(bb.cpu().numpy(), br), nrel(el.cpu().numpy(), elr)]
        print(f"fused nslices={S}: J_MO {errs[0]:.2e} K_MO {errs[1]:.2e} elag {errs[2]:.2e}")
        assert max(errs) < tol, (S, errs)
        assert nrel(c.cpu().numpy(), cr) < 1e-12 and nrel(Hm.cpu().numpy(), Hr) < 1e-12
        a2, b2, c2 = ops.jkh_mo_ri_mixed(dC, dH, prep, P)
        el2, Hm2 = ops.lagrange2_ri_mixed(dC, dH, prep, dn, dcj, dck, P, st.nbeta, st.nalpha)
        ops.check_device_status()
        # the same FP64 assembly (H_core, Hmat) and the same Lagrangian code path
        assert torch_cuda.equal(c, c2) and torch_cuda.equal(Hm, Hm2) and torch_cuda.equal(el, el2)
        # J_MO, K_MO from a differently shaped transform: equal to the split precision
        assert nrel(a.cpu().numpy(), a2.cpu().numpy()) < tol and nrel(bb.cpu().numpy(), b2.cpu().numpy()) < tol


def test_jkh_lagrange2_fused_mixed_golden(case):
    from pynof_gb300 import ops

    g, p, d = case
    prep = ops.PreparedRI(d["b"], nslices=6)
    dH = ops.to_device(g["H"])
    a, b, c, el, Hm = ops.jkh_lagrange2_ri_mixed(d["C"], dH, prep, ops.to_device(g["n_soft"]),
                                                  ops.to_device(g["cj12"]), ops.to_device(g["ck12"]), p.nbf5,
                                                  p.nbeta, p.nalpha)
    ops.check_device_status()
    for got, want in ((a, "J_MO_ri"), (b, "K_MO_ri"), (c, "H_core"), (el, "elag2_ri"), (Hm, "Hmat")):
        assert nrel(got.cpu().numpy(), g[want]) < 1e-10, want


@pytest.mark.parametrize("N,P,Q,block", [(96, 40, 180, 128), (170, 150, 340, 128), (300, 290, 120, 256)])
def test_split_build_matches_one_call(torch_cuda, N, P, Q, block):
    """J and K formed in parts (the prelude, then J and K over alternating
    ranges of orbitals), copied to the host on a second stream, equal the
    one-call build bitwise."""
    from pynof_gb300 import ops

    rng = np.random.default_rng(N)
    b = rng.standard_normal((N, N, Q)) * 0.1
    b = 0.5 * (b + b.transpose(1, 0, 2))
    C, _ = np.linalg.qr(rng.standard_normal((N, N)))
    db, dC = ops.to_device(b), ops.to_device(C)
    prep = ops.PreparedRI(db, 6)
    J, K = ops.jkj_ri_mixed(dC, prep, P)
    Jh, Kh = ops.jkj_ri_mixed_host(dC, prep, P, block=block)
    assert np.array_equal(Jh, J.cpu().numpy())
    assert np.array_equal(Kh, K.cpu().numpy())


def test_split_build_rejects_bad_range(torch_cuda):
    from pynof_gb300 import _lib, ops

    N, P, Q = 32, 10, 40
    wp, wn = ops._ws("gb_jkj_ri_workspace_mixed", N, P, Q, 6, device=torch_cuda.device("cuda", 0))
    K = torch_cuda.empty((P, N, N), dtype=torch_cuda.float64, device="cuda")
    with pytest.raises(_lib.GBError):
        _lib.call("gb_jkj_ri_mixed_k", N, P, Q, 6, 3, P + 1, K.data_ptr(), wp, wn, ops._stream())
    with pytest.raises(_lib.GBError):
        _lib.call("gb_jkj_ri_mixed_k", N, P, Q, 6, 5, 4, K.data_ptr(), wp, wn, ops._stream())
    prep = ops.PreparedRI(ops.to_device(np.zeros((N, N, Q))), 6)
    with pytest.raises(_lib.GBError):  # a J range must start on a 128-orbital block
        _lib.call("gb_jkj_ri_mixed_jr", prep.buf.data_ptr(), N, P, Q, 6, 3, P, K.data_ptr(), wp, wn, ops._stream())
