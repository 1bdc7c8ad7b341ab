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


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_opts_and_stats_layout_match_the_header(stg, tmp_path):
    """The ctypes mirrors of stg_opts and stg_stats (capi.Opts, capi.Stats) have the C
    structs' size and field offsets: a field added to the header must be added to the
    binding in the same place."""
    import ctypes
    import subprocess

    fields = {"stg_opts": [f for f, _ in stg.Opts._fields_], "stg_stats": [f for f, _ in stg.Stats._fields_]}
    src = ['#include <cstddef>', '#include <cstdio>', '#include "stokes_gb300.h"', "int main() {"]
    for st, fs in fields.items():
        src.append(f'    std::printf("{st} size %zu\\n", sizeof({st}));')
        for f in fs:
            src.append(f'    std::printf("{st} {f} %zu\\n", offsetof({st}, {f}));')
    src.append("    return 0;\n}")
    cpp = tmp_path / "layout.cpp"
    cpp.write_text("\n".join(src) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(cpp), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, stdout=subprocess.PIPE, text=True).stdout.split("\n")
    c = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for st, cls in (("stg_opts", stg.Opts), ("stg_stats", stg.Stats)):
        assert c[(st, "size")] == ctypes.sizeof(cls), st
        for f in fields[st]:
            assert c[(st, f)] == getattr(cls, f).offset, (st, f)
