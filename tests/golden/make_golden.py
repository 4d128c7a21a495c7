"""Generate the golden fixtures by running PyNOF's own functions.

This script is the only place that executes the reference.  It imports PyNOF
from a source checkout (``--ref``, default ``/root/reference/src``) with two
stub modules standing in for packages that are not installed and that the hot
path does not need:

* ``psi4``: an empty module (only referenced at import time and by functions
  off the path -- integral generation, basis sets, HF guesses);
* ``numba``: ``njit``/``jit`` as identity decorators and ``prange = range``, so
  the ``*_jit`` variants run as plain Python with the same arithmetic.

``sys.pycache_prefix`` points at a scratch directory so that only the ``.py``
sources are executed.

For each case it draws the seeded synthetic inputs
(``pynof_gb300.synthetic.make_inputs``), calls the reference functions on
copies of them, cross-checks the numpy and ``*_jit`` variants against each
other, and writes inputs plus outputs to ``tests/golden/<case>.npz``.

Run:  python tests/golden/make_golden.py [--ref PATH]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from pynof_gb300 import synthetic  # noqa: E402

CASES = {
    # name: (workload, seed, run_full_eri, run_jit_variants)
    "c1": ("c1", 0, True, True),
    "water": ("water", 0, True, False),
    "ragged": ("ragged", 3, False, False),
}

#: outer iterations of the reference's solve loop recorded for the loop parity test
LOOP_CASE = ("water", 0, 3)

#: restricted open shell (two singly occupied orbitals, two inactive ones):
#: the computeF_RO route of ENERGY1r (utils.py:423-425)
OPEN_SHELL = dict(nbf=30, nbfaux=120, no1=2, ndoc=3, ncwo=3, nsoc=2, MSpin=1)


def run_loop(pynof, workload, seed, n_outer):
    """The body of compute_energy's loop (energy.py:94-153) with the
    reference's own functions, psi4-free: occoptr, then per outer iteration
    orbopt_adam, occoptr, order_occupations_softmax and the two gradients."""
    st = synthetic.structure(workload)
    b, C, H, n = synthetic.make_inputs(st, seed)
    p = make_param(st)
    g0 = np.log(max(0.001 / st.ncwo, 1e-16)) - np.log(0.999)
    gamma = np.full(st.nv, g0)
    out = dict(b=b, C0=C, H=H, gamma0=gamma.copy())
    E_occ, nit_occ, ok_occ, gamma, n, cj12, ck12 = pynof.occoptr(gamma, C, H, [], b, p)
    rec = {"E_orb": [], "E_occ": [E_occ], "g_orb": [], "g_occ": [], "nit_orb": [], "nit_occ": [nit_occ]}
    for it in range(n_outer):
        E_orb, C, nit_orb, ok_orb = pynof.orbopt_adam(gamma, C, H, [], b, p)
        E_occ, nit_occ, ok_occ, gamma, n, cj12, ck12 = pynof.occoptr(gamma, C, H, [], b, p)
        C, gamma = pynof.order_occupations_softmax(C, gamma, H, [], b, p)
        y = np.zeros(p.nvar)
        g_orb = pynof.calcorbg(y, n, cj12, ck12, C, H, [], b, p)
        J_MO, K_MO, H_core = pynof.computeJKH_MO(C, H, [], b, p)
        g_occ = pynof.calcoccg(gamma, J_MO, K_MO, H_core, p)
        rec["E_orb"].append(E_orb)
        rec["E_occ"].append(E_occ)
        rec["g_orb"].append(np.linalg.norm(g_orb))
        rec["g_occ"].append(np.linalg.norm(g_occ))
        rec["nit_orb"].append(nit_orb)
        rec["nit_occ"].append(nit_occ)
        out[f"C_{it}"] = C.copy()
        out[f"gamma_{it}"] = gamma.copy()
    out.update({k: np.array(v) for k, v in rec.items()})
    out["alpha_final"] = np.array(p.alpha)
    out["maxloop_final"] = np.array(p.maxloop)
    return out


def import_reference(ref_src):
    sys.pycache_prefix = tempfile.mkdtemp(prefix="pycache_ref_")
    psi4 = types.ModuleType("psi4")
    psi4.core = types.ModuleType("psi4.core")
    sys.modules["psi4"] = psi4
    sys.modules["psi4.core"] = psi4.core
    numba = types.ModuleType("numba")

    def njit(*args, **kwargs):
        if len(args) == 1 and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    numba.njit = njit
    numba.jit = njit
    numba.prange = range
    sys.modules["numba"] = numba
    sys.path.insert(0, ref_src)
    import pynof  # noqa: F401

    return pynof


def make_param(st: synthetic.Structure, **over):
    keys = ["nbf", "nbfaux", "ndoc", "ncwo", "no1", "nsoc", "MSpin", "HighSpin", "RI", "ipnof",
            "occ_method", "nbeta", "nalpha", "ndns", "nac", "nbf5", "no0", "noptorb", "nv", "nvar",
            "maxloop", "alpha"]
    d = {k: getattr(st, k) for k in keys}
    d.update(gpu=False, jit=False, ista=0, lamb=0.0, freeze_occ=False, occupation_optimizer="CG")
    d.update(over)
    return types.SimpleNamespace(**d)


def nrel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def run_case(pynof, name, workload, seed, full, jit):
    st = synthetic.structure(workload)
    b, C, H, n = synthetic.make_inputs(st, seed)
    p = make_param(st)
    P = st.nbf5
    out = dict(b=b, C=C, H=H, n=n)
    checks = {}

    # occupation parameters (softmax encoding) and GNOF coefficients
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    # compute_gammas_softmax (utils.py:680-689) indexes with stride ncwo and
    # overruns its array when ndoc < ncwo; every entry it writes has the same
    # value, so the guess is built directly here.
    g0 = np.log(max(0.001 / st.ncwo, 1e-16)) - np.log(0.999)
    gamma = np.full(st.nv, g0) + 0.3 * rng.standard_normal(st.nv)
    n_soft, dn = pynof.ocupacion_softmax(gamma, st.no1, st.ndoc, st.nalpha, st.nv, P, st.ndns, st.ncwo,
                                         st.HighSpin)
    cj12, ck12 = pynof.PNOFi_selector(n_soft, p)
    Dcj, Dck = pynof.der_PNOFi_selector(n_soft, dn, p)
    out.update(gamma=gamma, n_soft=n_soft, dn_soft=dn, cj12=cj12.copy(), ck12=ck12.copy(),
               Dcj12=Dcj, Dck12=Dck)

    # A1 computeJKj (RI)
    J, K = pynof.computeJKj(C, [], b, p)
    out.update(J_ri=J, K_ri=K)
    if jit:
        Jj, Kj = pynof.JKj_RI_jit(C, b, st.nbf, P, st.nbfaux)
        checks["JKj_RI_jit_vs_numpy"] = max(nrel(Jj, J), nrel(Kj, K))

    # A3 computeJKH_MO (RI)
    J_MO, K_MO, H_core = pynof.computeJKH_MO(C, H, [], b, p)
    out.update(J_MO_ri=J_MO, K_MO_ri=K_MO, H_core=H_core)
    if jit:
        a, bb, c = pynof.JKH_MO_RI_jit(C, H, b, st.nbf, P, st.nbfaux)
        checks["JKH_MO_RI_jit_vs_numpy"] = max(nrel(a, J_MO), nrel(bb, K_MO), nrel(c, H_core))

    # A5 Integrals_MO_RI + computeLagrange2 (RI)
    Hmat, bmo = pynof.Integrals_MO_RI_CPU(C, H, b, p)
    out.update(Hmat=Hmat, b_MO=bmo)
    elag2, Hmat2 = pynof.computeLagrange2(n_soft, cj12.copy(), ck12.copy(), C, H, [], b, p)
    out.update(elag2_ri=elag2)

    # A7 ENERGY1r (no1 == 0 route)
    E, elag, sd, md = pynof.ENERGY1r(C, n_soft, H, [], b, cj12.copy(), ck12.copy(), p)
    out.update(E1r=np.array(E), elag1r=elag, sumdiff1r=np.array(sd), maxdiff1r=np.array(md))

    # A8 generalized Fock route on the recipe occupations
    F = pynof.computeF_RC_CPU(J, K, n_soft, H, cj12.copy(), ck12.copy(), p)
    elagF = pynof.computeLagrange(F, C, p)
    EF = pynof.computeE_elec(H, C, n_soft, elagF, p)
    out.update(F_rc=F, elag_F=elagF, E_F=np.array(EF))
    checks["E_fock_route_vs_lagrange2_route"] = abs(EF - E)

    # ENERGY1r with no1 = nbeta (the HF-like route hfidr takes, minimization.py:9-19)
    ph = make_param(st, no1=st.nbeta)
    nh = np.zeros(P)
    nh[: st.nbeta] = 1.0
    cjh = 2 * np.outer(nh, nh)
    ckh = np.outer(nh, nh)
    Eh, elagh, sdh, mdh = pynof.ENERGY1r(C, nh, H, [], b, cjh, ckh, ph)
    out.update(E1r_hf=np.array(Eh), elag1r_hf=elagh)

    # A9 occupation energy and gradient
    Ec = pynof.calce(n_soft, cj12.copy(), ck12.copy(), J_MO, K_MO, H_core, p)
    Eo = pynof.calcocce(gamma, J_MO, K_MO, H_core, p)
    go = pynof.calcoccg(gamma, J_MO, K_MO, H_core, p)
    out.update(E_calce=np.array(Ec), E_calcocce=np.array(Eo), g_occ=go)

    # A10 / A11 orbital gradient, orbital energy, rotation
    y0 = np.zeros(st.nvar)
    g_orb = pynof.calcorbg(y0, n_soft, cj12.copy(), ck12.copy(), C, H, [], b, p)
    y = 0.01 * rng.standard_normal(st.nvar)
    Cr = pynof.rotate_orbital(y, C, p)
    Eorb = pynof.calcorbe(y, n_soft, cj12.copy(), ck12.copy(), C, H, [], b, p)
    out.update(g_orb=g_orb, y=y, C_rot=Cr, E_orb=np.array(Eorb))

    # order_occupations_softmax (guess.py:77-106)
    Cs, gs = pynof.order_occupations_softmax(C, gamma, H, [], b, p)
    out.update(C_sorted=Cs, gamma_sorted=gs)

    if full:
        I = np.einsum("mnQ,slQ->mnsl", b, b, optimize=True)
        pf = make_param(st, RI=False)
        Jf, Kf = pynof.computeJKj(C, I, [], pf)
        out.update(J_full=Jf, K_full=Kf)
        checks["JKj_full_vs_ri"] = max(nrel(Jf, J), nrel(Kf, K))
        a, bb, c = pynof.computeJKH_MO(C, H, I, [], pf)
        out.update(J_MO_full=a, K_MO_full=bb)
        checks["JKH_MO_full_vs_ri"] = max(nrel(a, J_MO), nrel(bb, K_MO))
        ef, _ = pynof.computeLagrange2(n_soft, cj12.copy(), ck12.copy(), C, H, I, [], pf)
        out.update(elag2_full=ef)
        checks["lagrange2_full_vs_ri"] = nrel(ef, elag2)
        if jit:
            Jj, Kj = pynof.JKj_Full_jit(C, I, st.nbf, P)
            checks["JKj_Full_jit_vs_numpy"] = max(nrel(Jj, Jf), nrel(Kj, Kf))
            a2, b2, c2 = pynof.JKH_MO_Full_jit(C, H, I, st.nbf, P)
            checks["JKH_MO_Full_jit_vs_numpy"] = max(nrel(a2, a), nrel(b2, bb))
        # HF-JK helpers (integrals.py:490-560): closed-shell density and its
        # J, K; the singly-occupied density and its J, K with two open shells
        D_hf = pynof.computeD_HF(C, pf)
        J_hf, K_hf = pynof.computeJK_HF(D_hf, I, [], pf)
        pa = make_param(st, RI=False, nsoc=2, nalpha=st.nbeta + 2)
        # JKalpha_HF_Full_GPU (integrals.py:557-562) = computeDalpha_HF's einsum
        # then JK_HF_Full's einsums; the CPU route (JKalpha_HF_Full_jit) loops
        # over nu < mu only and leaves the diagonals of D, J and K at zero
        Da_hf = pynof.computeDalpha_HF(C, pa)
        Ja_hf, Ka_hf = pynof.JK_HF_Full_jit(Da_hf, I, pa.nbeta, pa.nbf, pa.nbf5)
        Dj, Jj, Kj = pynof.computeJKalpha_HF(C, I, [], pa)
        off = ~np.eye(st.nbf, dtype=bool)
        checks["JKalpha_HF_jit_D_offdiag_vs_einsum"] = nrel(Dj[off], Da_hf[off])
        checks["JKalpha_HF_jit_D_J_diagonal_max"] = float(max(np.abs(np.diag(Dj)).max(), np.abs(np.diag(Jj)).max()))
        checks["JKalpha_HF_jit_J_vs_gpu_route"] = nrel(Jj, Ja_hf)  # differs: D's diagonal is missing
        out.update(D_hf=D_hf, J_hf=J_hf, K_hf=K_hf, Da_hf=Da_hf, Ja_hf=Ja_hf, Ka_hf=Ka_hf)
        # post-NOF four-index transforms (integrals.py:601-662)
        out.update(iajb=pynof.compute_iajb(C, I, [], pf), pqrt=pynof.compute_pqrt(C, I, [], pf))

    meta = dict(case=name, workload=workload, seed=seed, sizes=synthetic.WORKLOADS[workload],
                numpy=np.__version__, checks=checks)
    return out, meta


def run_open_shell(pynof, seed=5):
    """computeF_RO_CPU, computeLagrange, computeE_elec (both HighSpin
    settings) and ENERGY1r with no1 > 0 and MSpin != 0, on seeded inputs with
    GNOF coefficients from the reference's PNOFi_selector."""
    st = synthetic.Structure(**OPEN_SHELL)
    b, C, H, _ = synthetic.make_inputs(st, seed)
    p = make_param(st)
    P, nb, na = st.nbf5, st.nbeta, st.nalpha
    rng = np.random.Generator(np.random.PCG64(seed + 200))
    n = np.zeros(P)
    n[: st.no1] = 1.0
    n[st.no1:nb] = np.sort(rng.uniform(0.6, 0.99, st.ndoc))[::-1]
    n[nb:na] = 0.5
    n[na:] = np.sort(rng.uniform(0.001, 0.2, P - na))[::-1]
    cj12, ck12 = pynof.PNOFi_selector(n, p)
    out = dict(b=b, C=C, H=H, n=n, cj12=cj12.copy(), ck12=ck12.copy())
    J, K = pynof.computeJKj(C, [], b, p)
    out.update(J_ri=J, K_ri=K)
    cj, ck = cj12.copy(), ck12.copy()
    F = pynof.computeF_RO_CPU(J, K, n, H, cj, ck, p)
    out.update(F_ro=F, cj12_zeroed=cj, ck12_zeroed=ck)
    elag = pynof.computeLagrange(F, C, p)
    out.update(elag_F=elag, E_F=np.array(pynof.computeE_elec(H, C, n, elag, p)))
    ph = make_param(st, HighSpin=True)
    out.update(E_F_highspin=np.array(pynof.computeE_elec(H, C, n, elag, ph)))
    E, el1, sd, md = pynof.ENERGY1r(C, n, H, [], b, cj12.copy(), ck12.copy(), p)
    out.update(E1r=np.array(E), elag1r=el1, sumdiff1r=np.array(sd), maxdiff1r=np.array(md))
    meta = dict(case="open_shell", seed=seed, sizes=OPEN_SHELL, numpy=np.__version__,
                checks={"E1r_vs_fock_route": abs(float(E) - float(out["E_F"]))})
    return out, meta


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference/src")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", default=None, help="write just this fixture (a case name, 'loop' or 'open_shell')")
    args = ap.parse_args()
    pynof = import_reference(args.ref)
    meta_path = os.path.join(args.out, "golden_meta.json")
    if args.only:
        with open(meta_path) as f:
            allmeta = json.load(f)
        if args.only == "open_shell":
            out, meta = run_open_shell(pynof)
        elif args.only in CASES:
            out, meta = run_case(pynof, args.only, *CASES[args.only])
        else:
            raise SystemExit(f"unknown fixture {args.only!r}")
        np.savez_compressed(os.path.join(args.out, f"{args.only}.npz"), **out)
        allmeta[args.only] = meta
        print(args.only, json.dumps(meta["checks"]))
        with open(meta_path, "w") as f:
            json.dump(allmeta, f, indent=1, sort_keys=True)
        return
    allmeta = {}
    out, meta = run_open_shell(pynof)
    np.savez_compressed(os.path.join(args.out, "open_shell.npz"), **out)
    allmeta["open_shell"] = meta
    for name, (workload, seed, full, jit) in CASES.items():
        out, meta = run_case(pynof, name, workload, seed, full, jit)
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **out)
        allmeta[name] = meta
        print(name, json.dumps(meta["checks"]))
    wl, seed, n_outer = LOOP_CASE
    loop = run_loop(pynof, wl, seed, n_outer)
    np.savez_compressed(os.path.join(args.out, "loop_water.npz"), **loop)
    allmeta["loop_water"] = dict(workload=wl, seed=seed, n_outer=n_outer, E_orb=loop["E_orb"].tolist(),
                                 g_orb=loop["g_orb"].tolist(), g_occ=loop["g_occ"].tolist())
    print("loop", allmeta["loop_water"])
    with open(meta_path, "w") as f:
        json.dump(allmeta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
