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
    return pynof


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
