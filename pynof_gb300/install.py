"""Install the GB300 path into an imported ``pynof`` package.

PyNOF resolves its contraction functions through module attributes at call
time (``pynof.computeJKj``, ``pynof.integrals.JKj_RI_GPU``, ...), so
rebinding those attributes makes every caller -- ``compute_energy``,
``occoptr``, ``orbopt_adam``, ``calcorbe`` / ``calcorbg``, ``hfidr`` -- use the
CUDA kernels when ``p.gpu`` is set, with ``param`` and every signature
unchanged; ``occoptr`` itself becomes the device occupation optimiser for the
structures it covers.  The dispatchers keep the reference's CPU branches for
``p.gpu = False``.
"""
from __future__ import annotations

from . import integrals, integrals_full, integrals_hf, minimization, nof, utils

#: (module attribute path in pynof, replacement) for the p.gpu branches
GPU_FUNCTIONS = {
    "integrals.JKj_RI_GPU": integrals.JKj_RI_GPU,
    "integrals.JKj_Full_GPU": integrals_full.JKj_Full_GPU,
    "integrals.JKH_MO_RI_GPU": integrals.JKH_MO_RI_GPU,
    "integrals.JKH_MO_Full_GPU": integrals_full.JKH_MO_Full_GPU,
    "integrals.Integrals_MO_RI_GPU": integrals.Integrals_MO_RI_GPU,
    "integrals.Integrals_MO_Full_GPU": integrals_full.Integrals_MO_Full_GPU,
    "utils.computeF_RC_GPU": utils.computeF_RC_GPU,
    "utils.computeF_RO_GPU": utils.computeF_RO_GPU,
    "integrals.JK_HF_Full_GPU": integrals_hf.JK_HF_Full_GPU,
    "integrals.JKalpha_HF_Full_GPU": integrals_hf.JKalpha_HF_Full_GPU,
    "integrals.iajb_Full_GPU": integrals_full.iajb_Full_GPU,
    "integrals.pqrt_Full_GPU": integrals_full.pqrt_Full_GPU,
}


def _gpu_or_cpu(gpu_fn, cpu_fn):
    def dispatch(*args):
        p = args[-1]
        return gpu_fn(*args) if getattr(p, "gpu", False) else cpu_fn(*args)

    dispatch.__name__ = getattr(cpu_fn, "__name__", "dispatch")
    dispatch.__doc__ = f"p.gpu -> pynof_gb300, else the reference's {dispatch.__name__}"
    return dispatch


def _occ_native(p) -> bool:
    """GNOF (ipnof 8) with softmax occupations, closed shell: the structures
    the compiled occupation function covers."""
    return (getattr(p, "gpu", False) and getattr(p, "ipnof", None) == 8
            and getattr(p, "occ_method", None) == "Softmax" and nof.native_occ_ok(p))


def _occ_dispatch(cpu_fn, grad: bool):
    """calcocce / calcoccg (pnof.py:994-1033), which occoptr hands to scipy's
    minimize (minimization.py:84-86): the library's compiled host loop where
    it applies, else the reference's own function."""

    def fn(gamma, J_MO, K_MO, H_core, p):
        if _occ_native(p):
            f = nof.OccFunction(J_MO, K_MO, H_core, p)
            return f(gamma)[1] if grad else f.energy(gamma)
        return cpu_fn(gamma, J_MO, K_MO, H_core, p)

    fn.__name__ = getattr(cpu_fn, "__name__", "calcoccg" if grad else "calcocce")
    fn.__doc__ = (f"p.gpu, GNOF, softmax, closed shell -> the compiled occupation function, "
                  f"else the reference's {fn.__name__}")
    return fn


def _occoptr_dispatch(cpu_fn):
    """occoptr (minimization.py:77-97): the device optimiser where it
    applies (GNOF, softmax, closed shell, CG, p.gpu), else the reference's."""

    def occoptr(gamma, C, H, I, b_mnl, p):
        if minimization.device_ok(p):
            return minimization.occoptr(gamma, C, H, I, b_mnl, p)
        return cpu_fn(gamma, C, H, I, b_mnl, p)

    occoptr.__doc__ = "p.gpu, GNOF, softmax, closed shell, CG -> the device occupation optimiser, else the reference's occoptr"
    return occoptr


def install(pynof) -> dict:
    """Rebind the GPU entry points of an imported ``pynof`` package.

    Returns the previous bindings ({dotted name: object}) so that
    :func:`uninstall` can restore them.
    """
    saved = {}
    for dotted, fn in GPU_FUNCTIONS.items():
        modname, attr = dotted.split(".")
        mod = getattr(pynof, modname)
        saved[dotted] = getattr(mod, attr)
        setattr(mod, attr, fn)
        if hasattr(pynof, attr):
            saved["pynof." + attr] = getattr(pynof, attr)
            setattr(pynof, attr, fn)
    # compute_integrals uploads b_mnl / I with cupy (integrals.py:51-53): run it
    # host-side and keep the tensors resident as CUDA tensors instead
    orig_ci = pynof.integrals.compute_integrals

    def compute_integrals(wfn, mol, p):
        gpu = p.gpu
        p.gpu = False
        try:
            S, T, V, H, I, b_mnl, Dipole = orig_ci(wfn, mol, p)
        finally:
            p.gpu = gpu
        if gpu:
            I, b_mnl = integrals.upload_integrals(I, b_mnl)
        return S, T, V, H, I, b_mnl, Dipole

    saved["integrals.compute_integrals"] = orig_ci
    saved["pynof.compute_integrals"] = getattr(pynof, "compute_integrals", orig_ci)
    pynof.integrals.compute_integrals = compute_integrals
    pynof.compute_integrals = compute_integrals
    # computeLagrange2 and ENERGY1r hold cupy code inline (utils.py:272-327),
    # so they are replaced whole; the reference CPU branch stays behind p.gpu=False
    # rotate_orbital (utils.py:550-565) runs scipy expm on the host: on the
    # device path it becomes the FP64 device rotation
    for modname, name, gpu_fn in (("utils", "computeLagrange2", utils.computeLagrange2),
                                  ("utils", "ENERGY1r", utils.ENERGY1r),
                                  ("utils", "rotate_orbital", utils.rotate_orbital),
                                  # cupy inline (integrals.py:493-510)
                                  ("integrals", "computeD_HF", integrals_hf.computeD_HF),
                                  ("integrals", "computeDalpha_HF", integrals_hf.computeDalpha_HF)):
        mod = getattr(pynof, modname)
        cpu_fn = getattr(mod, name)
        saved[modname + "." + name] = cpu_fn
        saved["pynof." + name] = getattr(pynof, name, cpu_fn)
        disp = _gpu_or_cpu(gpu_fn, cpu_fn)
        setattr(mod, name, disp)
        setattr(pynof, name, disp)
    # the occupation optimiser's function and gradient (pnof.py:994-1033)
    if hasattr(pynof, "pnof"):
        for name, grad in (("calcocce", False), ("calcoccg", True)):
            cpu_fn = getattr(pynof.pnof, name)
            saved["pnof." + name] = cpu_fn
            saved["pynof." + name] = getattr(pynof, name, cpu_fn)
            disp = _occ_dispatch(cpu_fn, grad)
            setattr(pynof.pnof, name, disp)
            setattr(pynof, name, disp)
    # the occupation optimiser itself (compute_energy calls pynof.occoptr,
    # energy.py:94, 126)
    if hasattr(pynof, "minimization") and hasattr(pynof.minimization, "occoptr"):
        cpu_fn = pynof.minimization.occoptr
        saved["minimization.occoptr"] = cpu_fn
        saved["pynof.occoptr"] = getattr(pynof, "occoptr", cpu_fn)
        disp = _occoptr_dispatch(cpu_fn)
        pynof.minimization.occoptr = disp
        pynof.occoptr = disp
    return saved


def uninstall(pynof, saved: dict) -> None:
    for dotted, obj in saved.items():
        modname, attr = dotted.split(".")
        setattr(pynof if modname == "pynof" else getattr(pynof, modname), attr, obj)
