"""CPU checks of the C ABI: the library builds, loads and exports every symbol the
public header declares (no compute call is made without a GPU)."""
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "stokes_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(stg_[A-Za-z0-9_]+)\s*\(", txt)))


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_library_exports_every_declared_symbol(stg):
    L = stg.lib()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(stg.EXPORTS)


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_default_opts_and_version(stg):
    o = stg.default_opts()
    assert o.method == stg.STG_METHOD_PLAIN and o.tol == 1e-8 and o.inner_max == 30
    assert b"sm_103a" in stg.lib().stg_version()
