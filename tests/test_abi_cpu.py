"""The C-ABI library builds, loads and exports every symbol the header declares.

No GPU needed: only size queries (pure host arithmetic) are called.
"""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pynof_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from pynof_gb300 import _lib, build

    build.build()
    return _lib.load()


def test_header_symbols_exported(lib):
    from pynof_gb300 import _lib

    names = declared_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} missing from the ctypes signature table"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (gb_\w+)", out))
    assert set(names) <= exported
    assert set(_lib.SIGNATURES) <= exported


def test_workspace_queries(lib):
    from pynof_gb300 import _lib

    N, P, Q = 600, 300, 2400
    ws = _lib.query("gb_jkj_ri_workspace_f64", N, P, Q)
    assert ws >= P * N * Q * 8 + P * Q * 8
    assert ws % 256 == 0
    assert _lib.query("gb_lagrange2_ri_workspace_f64", N, P, Q) >= 2 * N * P * Q * 8


def test_split_codes(lib):
    """GB_SPLIT_TF32X3 in the header is ops.SPLIT_TF32X3, and its prepared
    factor (two 32-bit planes of b's half-transform copy, N Q rows x N, and of
    its pair copy, the N (N + 1) / 2 pairs m <= n x Q) is smaller than six
    bf16 digit planes."""
    from pynof_gb300 import _lib, ops

    hdr = open(HEADER).read()
    m = re.search(r"#define\s+GB_SPLIT_TF32X3\s+(\d+)", hdr)
    assert m and int(m.group(1)) == ops.SPLIT_TF32X3
    N, Q = 600, 2400
    tf = _lib.query("gb_ri_prepare_bytes_mixed", N, Q, ops.SPLIT_TF32X3)
    s6 = _lib.query("gb_ri_prepare_bytes_mixed", N, Q, 6)
    assert 8 * (N * Q * N + N * (N + 1) // 2 * Q) <= tf < s6


def test_version_and_error(lib):
    assert lib.gb_version() >= 100
    assert isinstance(lib.gb_last_error(), bytes)


def declared_arity():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(gb_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_header(lib):
    from pynof_gb300 import _lib

    arity = declared_arity()
    for name, (_, args) in _lib.SIGNATURES.items():
        assert name in arity, name
        assert len(args) == arity[name], f"{name}: ctypes has {len(args)} arguments, header {arity[name]}"
