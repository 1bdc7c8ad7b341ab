"""Build libstokes_gb300.so (sm_103a) and the fluid_topo driver in-tree.

Every translation unit is compiled by nvcc in parallel with one -gencode for sm_103a,
then linked into stokes_to_gb300/libstokes_gb300.so. The C++ driver links against it.
Host code is portable C++17 (no x86 intrinsics), so the same recipe builds on the
aarch64 GPU hosts.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libstokes_gb300.so")
DRIVER = os.path.join(HERE, "fluid_topo")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "--expt-relaxed-constexpr",
            "-I", os.path.join(ROOT, "include")]
SOURCES = ["kernels.cu", "sweep.cu", "blas.cu", "dense.cu", "topo.cu", "solver.cu", "solver2d.cu", "mma.cu", "noalloc.cu", "general.cu",
           "unet_kernels.cu", "unet.cu"]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose=False, ptxas_v=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "stokes_gb300.h"))
    objs, jobs = [], []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if not _newer(obj, [src] + headers) or ptxas_v:
            extra = ["-Xptxas", "-v"] if ptxas_v else []
            jobs.append([NVCC] + ARCH + CU_FLAGS + extra + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose or ptxas_v:
        for o in outs:
            sys.stdout.write(o)
    if jobs or not os.path.exists(LIB):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    drv_src = os.path.join(HERE, "host", "fluid_topo.cpp")
    drv_hdr = [os.path.join(HERE, "host", f) for f in os.listdir(os.path.join(HERE, "host")) if f.endswith(".h")]
    if os.path.exists(drv_src) and not _newer(DRIVER, [drv_src, LIB] + drv_hdr):
        _run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "host"),
              drv_src, "-o", DRIVER, "-L", HERE, "-lstokes_gb300", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_v="--ptxas" in sys.argv)
    print("built", LIB)
