"""The installer against the reference package itself (not a stand-in).

PyNOF is imported from its source checkout with the stub ``psi4`` / ``numba``
modules of ``tests/golden/make_golden.py`` (in a child process, so the stubs
and the import path stay out of this test session).  After
``install.install(pynof)``:

* every replaced entry point is bound in its module, and the reference's own
  dispatchers (``computeJKj``, ``computeJKH_MO``, ``JKH_MO_tmp``,
  ``computeF_RC_driver``, ``compute_energy``'s callees) resolve it through
  their module globals -- the lookup PyNOF makes at call time;
* the names re-exported at the package top level point at the same objects;
* ``occoptr``, which ``compute_energy`` calls as ``pynof.occoptr``, becomes
  the device occupation optimiser's dispatcher;
* the p.gpu=False branches of the replaced-whole functions
  (``computeLagrange2``, ``calcocce``) still return the reference's CPU
  results on the golden inputs;

and ``uninstall`` restores every original binding.  Skipped where the
reference checkout is absent.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _reference_src():
    """PYNOF_REFERENCE_SRC, else the golden generator's default ``--ref``."""
    src = os.environ.get("PYNOF_REFERENCE_SRC")
    if src:
        return src
    import ast

    tree = ast.parse(open(os.path.join(GOLDEN, "make_golden.py")).read())
    for node in ast.walk(tree):
        if (isinstance(node, ast.Call) and getattr(node.func, "attr", "") == "add_argument" and node.args
                and isinstance(node.args[0], ast.Constant) and node.args[0].value == "--ref"):
            for kw in node.keywords:
                if kw.arg == "default":
                    return kw.value.value
    return None


CHILD = r"""
import json, sys, types
ROOT, GOLDEN, SRC = sys.argv[1:4]
sys.path.insert(0, ROOT)
sys.path.insert(0, GOLDEN)
import numpy as np
import make_golden
pynof = make_golden.import_reference(SRC)
from pynof_gb300 import install, integrals, integrals_full, utils
out = {"bound": {}, "resolved": {}, "toplevel": {}, "cpu": {}, "restored": None}
before = {}
for dotted in install.GPU_FUNCTIONS:
    m, a = dotted.split(".")
    before[dotted] = getattr(getattr(pynof, m), a)
saved = install.install(pynof)
for dotted, fn in install.GPU_FUNCTIONS.items():
    m, a = dotted.split(".")
    out["bound"][dotted] = getattr(getattr(pynof, m), a) is fn
    if hasattr(pynof, a):
        out["toplevel"][a] = getattr(pynof, a) is fn
# the reference's dispatchers look the replaced names up in their module globals
for disp, name, fn in (("computeJKj", "JKj_RI_GPU", integrals.JKj_RI_GPU),
                       ("computeJKj", "JKj_Full_GPU", integrals_full.JKj_Full_GPU),
                       ("computeJKH_MO", "JKH_MO_RI_GPU", integrals.JKH_MO_RI_GPU),
                       ("computeJKH_MO", "JKH_MO_Full_GPU", integrals_full.JKH_MO_Full_GPU),
                       ("JKH_MO_tmp", "Integrals_MO_RI_GPU", integrals.Integrals_MO_RI_GPU)):
    g = getattr(pynof.integrals, disp).__globals__
    out["resolved"][disp + "->" + name] = g.get(name) is fn
g = pynof.utils.computeF_RC_driver.__globals__
out["resolved"]["computeF_RC_driver->computeF_RC_GPU"] = g.get("computeF_RC_GPU") is utils.computeF_RC_GPU
for name in ("computeLagrange2", "ENERGY1r", "rotate_orbital"):
    out["resolved"]["utils." + name] = getattr(pynof.utils, name).__doc__.startswith("p.gpu -> pynof_gb300")
    out["toplevel"][name] = getattr(pynof, name, getattr(pynof.utils, name)) is getattr(pynof.utils, name)
for name in ("calcocce", "calcoccg"):
    out["resolved"]["pnof." + name] = "compiled occupation function" in getattr(pynof.pnof, name).__doc__
# compute_energy calls pynof.occoptr (energy.py:94, 126)
out["resolved"]["occoptr"] = (pynof.occoptr is pynof.minimization.occoptr
                              and "device occupation optimiser" in pynof.occoptr.__doc__)
# p.gpu = False: the reference's CPU branches behind the dispatchers
z = np.load(GOLDEN + "/c1.npz")
from pynof_gb300 import synthetic
st = synthetic.structure("c1")
p = make_golden.make_param(st)
cj, ck = z["cj12"].copy(), z["ck12"].copy()
elag, Hmat = pynof.utils.computeLagrange2(z["n_soft"], cj, ck, z["C"], z["H"], None, z["b"], p)
out["cpu"]["computeLagrange2"] = make_golden.nrel(elag, z["elag2_ri"])
E = pynof.pnof.calcocce(z["gamma"], z["J_MO_ri"], z["K_MO_ri"], z["H_core"], p)
out["cpu"]["calcocce"] = abs(float(E) - float(z["E_calcocce"])) / abs(float(z["E_calcocce"]))
install.uninstall(pynof, saved)
out["restored"] = all(getattr(getattr(pynof, d.split(".")[0]), d.split(".")[1]) is f for d, f in before.items())
out["restored_lagrange2"] = not (pynof.utils.computeLagrange2.__doc__ or "").startswith("p.gpu -> pynof_gb300")
out["restored_occoptr"] = "device occupation optimiser" not in (pynof.occoptr.__doc__ or "")
print("RESULT " + json.dumps(out))
"""


def test_install_on_reference_package(tmp_path):
    src = _reference_src()
    if not src or not os.path.isdir(os.path.join(src, "pynof")):
        pytest.skip("reference checkout not present")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, GOLDEN, src], capture_output=True, text=True, timeout=600,
                       cwd=tmp_path)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")]
    assert r.returncode == 0 and line, r.stdout[-2000:] + r.stderr[-2000:]
    out = json.loads(line[-1][7:])
    assert out["bound"] and all(out["bound"].values()), out["bound"]
    assert all(out["resolved"].values()), out["resolved"]
    assert all(out["toplevel"].values()), out["toplevel"]
    assert out["cpu"]["computeLagrange2"] < 1e-12 and out["cpu"]["calcocce"] < 1e-12, out["cpu"]
    assert out["restored"] and out["restored_lagrange2"] and out["restored_occoptr"]
