"""The installer rebinds PyNOF's GPU entry points (no GPU needed).

A stand-in ``pynof`` package with the reference's module layout and function
names is built here; the installer must rebind every p.gpu entry point, keep
the CPU branches behind p.gpu=False, and be reversible.
"""
import types

from pynof_gb300 import install as inst
from pynof_gb300 import integrals, integrals_full, integrals_hf, utils


def fake_pynof():
    pynof = types.ModuleType("pynof")
    pynof.integrals = types.ModuleType("pynof.integrals")
    pynof.utils = types.ModuleType("pynof.utils")
    for dotted in inst.GPU_FUNCTIONS:
        mod, attr = dotted.split(".")
        fn = lambda *a, _n=attr: ("reference", _n)
        setattr(getattr(pynof, mod), attr, fn)
        setattr(pynof, attr, fn)
    pynof.utils.computeLagrange2 = lambda *a: ("reference-cpu", "computeLagrange2")
    pynof.utils.ENERGY1r = lambda *a: ("reference-cpu", "ENERGY1r")
    pynof.utils.rotate_orbital = lambda *a: ("reference-cpu", "rotate_orbital")
    pynof.integrals.computeD_HF = lambda *a: ("reference-cpu", "computeD_HF")
    pynof.integrals.computeDalpha_HF = lambda *a: ("reference-cpu", "computeDalpha_HF")
    pynof.computeLagrange2 = pynof.utils.computeLagrange2
    pynof.ENERGY1r = pynof.utils.ENERGY1r
    pynof.rotate_orbital = pynof.utils.rotate_orbital
    pynof.integrals.compute_integrals = lambda wfn, mol, p: (1, 2, 3, 4, [], [], 7)
    pynof.compute_integrals = pynof.integrals.compute_integrals
    pynof.pnof = types.ModuleType("pynof.pnof")
    pynof.pnof.calcocce = lambda *a: ("reference", "calcocce")
    pynof.pnof.calcoccg = lambda *a: ("reference", "calcoccg")
    pynof.calcocce = pynof.pnof.calcocce
    pynof.calcoccg = pynof.pnof.calcoccg
    pynof.minimization = types.ModuleType("pynof.minimization")
    pynof.minimization.occoptr = lambda *a: ("reference", "occoptr")
    pynof.occoptr = pynof.minimization.occoptr
    return pynof


def test_install_occoptr_dispatch():
    """occoptr becomes the device optimiser's dispatcher; structures it does
    not cover (and p.gpu = False) reach the reference's own occoptr."""
    from pynof_gb300 import minimization, synthetic

    pynof = fake_pynof()
    orig = pynof.occoptr
    saved = inst.install(pynof)
    assert pynof.occoptr is pynof.minimization.occoptr and pynof.occoptr is not orig
    st = synthetic.structure("water")
    assert minimization.device_ok(st)
    for other in (dict(gpu=False), dict(ipnof=7), dict(occ_method="Trigonometric"),
                  dict(occupation_optimizer="L-BFGS-B"), dict(freeze_occ=True), dict(MSpin=1)):
        q = types.SimpleNamespace(**{**vars(st), **other})
        assert not minimization.device_ok(q)
        assert pynof.occoptr(None, None, None, None, None, q) == ("reference", "occoptr")
    inst.uninstall(pynof, saved)
    assert pynof.occoptr is orig and pynof.minimization.occoptr is orig


def test_install_occupation_function():
    """pynof.calcocce / calcoccg: the compiled loop for GNOF + softmax closed
    shell on the device path, the reference's functions otherwise."""
    import numpy as np

    from pynof_gb300 import build, nof
    from pynof_gb300.synthetic import Structure

    build.build()
    pynof = fake_pynof()
    saved = inst.install(pynof)
    st = Structure(nbf=24, nbfaux=96, ndoc=4, ncwo=3)
    rng = np.random.default_rng(3)
    A = rng.standard_normal((st.nbf5, st.nbf5))
    J = A @ A.T
    K = 0.5 * J
    H = rng.standard_normal(st.nbf5)
    gamma = rng.standard_normal(st.nv)
    p = types.SimpleNamespace(**{**vars(st), "gpu": True, "ipnof": 8, "occ_method": "Softmax"})
    assert abs(pynof.calcocce(gamma, J, K, H, p) - nof.calcocce(gamma, J, K, H, st)) < 1e-12 * abs(J).max()
    assert np.abs(pynof.calcoccg(gamma, J, K, H, p) - nof.calcoccg(gamma, J, K, H, st)).max() < 1e-11 * abs(J).max()
    for other in (dict(gpu=False), dict(ipnof=7), dict(occ_method="Trigonometric")):
        q = types.SimpleNamespace(**{**vars(p), **other})
        assert pynof.calcocce(gamma, J, K, H, q) == ("reference", "calcocce")
        assert pynof.pnof.calcoccg(gamma, J, K, H, q) == ("reference", "calcoccg")
    inst.uninstall(pynof, saved)
    assert pynof.calcocce(gamma, J, K, H, p) == ("reference", "calcocce")


def test_install_rebinds_and_restores():
    pynof = fake_pynof()
    before = {d: getattr(getattr(pynof, d.split(".")[0]), d.split(".")[1]) for d in inst.GPU_FUNCTIONS}
    saved = inst.install(pynof)
    assert pynof.integrals.JKj_RI_GPU is integrals.JKj_RI_GPU
    assert pynof.JKj_RI_GPU is integrals.JKj_RI_GPU
    assert pynof.integrals.JKj_Full_GPU is integrals_full.JKj_Full_GPU
    assert pynof.integrals.JKH_MO_RI_GPU is integrals.JKH_MO_RI_GPU
    assert pynof.integrals.Integrals_MO_RI_GPU is integrals.Integrals_MO_RI_GPU
    assert pynof.utils.computeF_RC_GPU is utils.computeF_RC_GPU
    # whole-function replacements dispatch on p.gpu
    p = types.SimpleNamespace(gpu=False)
    assert pynof.computeLagrange2(1, 2, 3, 4, 5, 6, 7, p) == ("reference-cpu", "computeLagrange2")
    assert pynof.utils.ENERGY1r(1, 2, 3, 4, 5, 6, 7, p) == ("reference-cpu", "ENERGY1r")
    assert pynof.integrals.computeD_HF(1, p) == ("reference-cpu", "computeD_HF")
    assert pynof.integrals.JK_HF_Full_GPU is integrals_hf.JK_HF_Full_GPU
    assert pynof.rotate_orbital(1, 2, p) == ("reference-cpu", "rotate_orbital")
    assert "p.gpu" in (pynof.rotate_orbital.__doc__ or "")  # the installed dispatcher
    # compute_integrals with p.gpu=False is the reference's
    assert pynof.compute_integrals(None, None, p) == (1, 2, 3, 4, [], [], 7)
    inst.uninstall(pynof, saved)
    for d, fn in before.items():
        mod, attr = d.split(".")
        assert getattr(getattr(pynof, mod), attr) is fn
    assert pynof.computeLagrange2(1, 2, 3, 4, 5, 6, 7, p) == ("reference-cpu", "computeLagrange2")
    assert pynof.rotate_orbital(1, 2, p) == ("reference-cpu", "rotate_orbital")


def test_precision_switch():
    old = dict(integrals.PRECISION)
    try:
        integrals.set_precision("fp64")
        assert integrals.PRECISION["mode"] == "fp64"
        integrals.set_precision("mixed", 2)
        assert integrals.PRECISION == {"mode": "mixed", "nslices": 2}
        import pytest

        with pytest.raises(ValueError):
            integrals.set_precision("fp16")
        with pytest.raises(ValueError):
            integrals.set_precision("mixed", 7)
    finally:
        integrals.PRECISION.update(old)
