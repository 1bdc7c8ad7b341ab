"""Builds oracle/_ref/libref_emu.so: the reference's own CUDA solver path (operators,
transfers, Vanka smoothers, coarsest solves, V-cycle, GMRES, energy operator; 3D and 2D)
compiled from the reference sources where they lie, for the host, on the CUDA stand-in of
oracle/ref_emu/emu.h. TEST INFRASTRUCTURE ONLY: the library makes the golden vectors
(tests/golden/make_ref_golden.py) that pin the oracle; nothing else loads it.

Kernel launches (`k<<<grid, block>>>(args)`) are not C++, so each reference translation
unit is read, its reference-local headers are inlined (once each, as #pragma once would),
every launch is rewritten into a call of emu::launch with the same configuration and
arguments, and the result is compiled from standard input: no rewritten copy of a
reference source is written to disk. One further edit, made explicit here:

* BlockMatrixReorderKernel (common_cpx/BatchInverse.cuh:13-47) runs as a single 32-thread
  warp and reads its shared `start`/`end` counters while thread 0 advances them, relying
  on the warp executing in lockstep. The stand-in runs threads one after another, so a
  barrier is inserted before thread 0 advances `start`: exactly the ordering lockstep
  execution gives.

usage: python oracle/ref_emu/build.py REFERENCE_ROOT
"""
import concurrent.futures as cf
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libref_emu.so")

CC = "simplex/src/common_cpx"
ST = "complex/proj/PainlessSolver/proj/stoke"
FT = "complex/proj/PainlessSolver/proj/fluid_topo"

SOURCES = [
    (CC, "grid3D.cu"), (CC, "form01mapping.cu"), (CC, "DescentSmoother.cu"), (CC, "MultigridSolve.cpp"),
    (CC, "GMRES.cpp"),
    (ST, "StokeFlowDescriptor3D.cu"), (ST, "StokeFlowMapping3D.cu"), (ST, "StokeFlowSubSystem3D.cu"),
    (ST, "StokeLike.cu"), (ST, "StokeFlowDescriptor.cpp"), (ST, "StokeFlowMapping.cu"), (ST, "StokeFlowSmoothing.cu"),
    (ST, "StokeFlowSubSystem.cu"), (ST, "StokeFlowDirectSolve.cpp"),
    (FT, "FluidEnergyGrad3D.cu"), (FT, "FluidEnergyGrad.cu"),
]

REORDER_OLD = "\t\tif (idx == 0) start = end;"
REORDER_NEW = "\t\t__syncthreads();\n\t\tif (idx == 0) start = end;"

INCLUDE = re.compile(r'^[ \t]*#[ \t]*include[ \t]*"([^"]+)"[^\n]*$', re.M)
PRAGMA_ONCE = re.compile(r'^[ \t]*#[ \t]*pragma[ \t]+once[^\n]*$', re.M)
LAUNCH = re.compile(r'([A-Za-z_]\w*(?:[ \t]*<[^<>;(){}]*>)?)[ \t]*<<[ \t]*<')


def _resolve(name, cur_dir, dirs):
    """Quote-include search: the including file's directory, then the reference
    directories; a case-insensitive match is accepted (the reference was built on a
    case-insensitive file system)."""
    for d in [cur_dir] + dirs:
        p = os.path.join(d, name)
        if os.path.isfile(p):
            return os.path.realpath(p)
    for d in [cur_dir] + dirs:
        sub, base = os.path.split(os.path.join(d, name))
        if os.path.isdir(sub):
            for f in os.listdir(sub):
                if f.lower() == base.lower():
                    return os.path.realpath(os.path.join(sub, f))
    return None


def _rewrite_launches(text, where):
    out, pos = [], 0
    while True:
        m = LAUNCH.search(text, pos)
        if not m:
            break
        name = m.group(1)
        i, depth = m.end(), 0
        while True:  # the configuration ends at the first '>>' '>' outside parentheses
            c = text[i]
            if c in "([":
                depth += 1
            elif c in ")]":
                depth -= 1
            elif depth == 0 and text.startswith(">>", i):
                j = i + 2
                while text[j] in " \t":
                    j += 1
                if text[j] == ">":
                    cfg_end, after = i, j + 1
                    break
            i += 1
        cfg = text[m.end():cfg_end]
        k = after
        while text[k] in " \t\r\n\\":
            k += 1
        if text[k] != "(":
            raise RuntimeError(f"{where}: launch of {name} without an argument list")
        e, depth = k, 0
        while True:
            if text[e] == "(":
                depth += 1
            elif text[e] == ")":
                depth -= 1
                if depth == 0:
                    break
            e += 1
        args = text[k + 1:e]
        span = text[m.start():e + 1]
        out.append(text[pos:m.start()])
        call = f"::emu::launch(::emu::Cfg({cfg}), [&]() {{ {name}({args}); }})"
        out.append(call.replace("\\\n", " ").replace("\n", " ") + "\n" * span.count("\n"))
        pos = e + 1
    out.append(text[pos:])
    return "".join(out)


def translation_unit(path, dirs, ref_root):
    """The text of one translation unit with its reference-local headers inlined and its
    launches rewritten."""
    seen = set()

    def expand(p):
        rp = os.path.realpath(p)
        if rp in seen:
            return ""
        seen.add(rp)
        with open(rp, encoding="utf-8", errors="replace") as f:
            text = f.read().replace("\r\n", "\n")
        if os.path.basename(rp) == "BatchInverse.cuh":
            if text.count(REORDER_OLD) != 1:
                raise RuntimeError("BatchInverse.cuh: the reorder kernel's counter update was not found once")
            text = text.replace(REORDER_OLD, REORDER_NEW)
        text = PRAGMA_ONCE.sub("", text)
        text = _rewrite_launches(text, rp)
        parts, pos = [], 0
        for m in INCLUDE.finditer(text):
            tgt = _resolve(m.group(1), os.path.dirname(rp), dirs)
            if tgt is None or not tgt.startswith(ref_root):
                continue  # stand-in headers, Eigen and the system are left to the compiler
            line = text.count("\n", 0, m.start()) + 1
            parts.append(text[pos:m.start()])
            parts.append(f'#line 1 "{tgt}"\n' + expand(tgt) + f'\n#line {line + 1} "{rp}"\n')
            pos = m.end()
        parts.append(text[pos:])
        return f'#line 1 "{rp}"\n' + "".join(parts)

    return expand(path)


def build(ref_root):
    ref_root = os.path.realpath(ref_root)
    dirs = [os.path.join(ref_root, d) for d in (CC, ST, FT)]
    eigen = os.path.join(ref_root, "simplex", "ext", "eigen")
    os.makedirs(OUT, exist_ok=True)
    objdir = os.path.join(OUT, "emu_obj")
    os.makedirs(objdir, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    flags = ["-std=c++17", "-O2", "-fPIC", "-DNDEBUG", "-w", "-include", os.path.join(HERE, "emu.h"),
             "-I", os.path.join(HERE, "shim"), "-I", HERE] + sum([["-I", d] for d in dirs], []) + ["-I", eigen]

    def compile_tu(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        text = translation_unit(src, dirs, ref_root)
        r = subprocess.run([cxx] + flags + ["-x", "c++", "-", "-c", "-o", obj], input=text, text=True,
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stdout[-6000:]}")
        return obj

    srcs = [os.path.join(ref_root, d, f) for d, f in SOURCES] + [os.path.join(HERE, "ref_api.cpp")]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_tu, srcs))
    emu_obj = os.path.join(objdir, "emu.o")
    subprocess.run([cxx, "-std=c++17", "-O2", "-fPIC", "-c", os.path.join(HERE, "emu.cpp"), "-o", emu_obj], check=True)
    subprocess.run([cxx, "-shared", "-o", LIB] + objs + [emu_obj], check=True)
    return LIB


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    print("built", build(sys.argv[1]))
