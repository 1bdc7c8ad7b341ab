"""Generates tests/golden/ref_*.npz: golden vectors from the reference's OWN solver code.

The reference ships no tests or golden vectors for this path, and its solver is CUDA
code (operators, transfers, Vanka smoothers, coarsest solves, V-cycle) driven by host
classes and a host GMRES. oracle/ref_emu/build.py compiles those sources, where they lie
in the reference checkout, against a host stand-in for the CUDA runtime, cuBLAS and
cuSOLVER (oracle/ref_emu/emu.h), so the reference's kernels and classes run unchanged on
the CPU. This script drives them on seeded problems and stores every result; the CPU
tests pin the oracle to these fixtures and the GPU tests compare the product with them.

Vectors fed to the operators come from tests.helpers.stable_vec(seed, n) (SplitMix64;
the seeds are stored, not the vectors). The problem data (finest-level vol, fixed and
penalty arrays, right-hand side) are stored in the reference's blocked layout.

usage: python tests/golden/make_ref_golden.py [REFERENCE_ROOT] [OUT_DIR]   (needs the
       reference checkout; writes OUT_DIR/ref_*.npz, by default into tests/golden)

Running it with EMU_REVERSE=1 (every kernel's blocks and threads in reverse order) or
EMU_FILL_NAN=1 (device memory starts as NaN) into another directory must reproduce the
same vectors: no result depends on the stand-in's scheduling or on unwritten memory.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as po  # noqa: E402
from tests.helpers import problem, problem2, stable_vec  # noqa: E402

P, I = ctypes.c_void_p, ctypes.c_int
DP, U8 = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint8)


def load_lib(ref_root):
    lib = os.path.join(ROOT, "oracle", "_ref", "libref_emu.so")
    subprocess.run([sys.executable, os.path.join(ROOT, "oracle", "ref_emu", "build.py"), ref_root], check=True)
    L = ctypes.CDLL(lib)
    for d in ("3", "2"):
        getattr(L, f"ref{d}_create").restype = P
        getattr(L, f"ref{d}_create").argtypes = [I, I]
        getattr(L, f"ref{d}_levels").restype = I
        getattr(L, f"ref{d}_levels").argtypes = [P]
        getattr(L, f"ref{d}_level_dof").restype = I
        getattr(L, f"ref{d}_level_dof").argtypes = [P, I]
        getattr(L, f"ref{d}_set_descr").argtypes = [P, DP, U8, DP]
        getattr(L, f"ref{d}_apply_A").argtypes = [P, I, DP, DP]
        getattr(L, f"ref{d}_apply_E").argtypes = [P, DP, DP]
        getattr(L, f"ref{d}_restrict").argtypes = [P, I, DP, DP]
        getattr(L, f"ref{d}_prolong").argtypes = [P, I, DP, DP]
        getattr(L, f"ref{d}_smooth").argtypes = [P, I, I, DP, DP]
        getattr(L, f"ref{d}_coarse").argtypes = [P, DP, DP]
        getattr(L, f"ref{d}_vcycle").argtypes = [P, DP, DP]
        getattr(L, f"ref{d}_solve").argtypes = [P, DP, DP, I, ctypes.c_double, ctypes.c_double, ctypes.c_double]
    L.ref3_update.argtypes = [P]
    L.ref3_level_descr.argtypes = [P, I, DP, DP, U8]
    L.ref3_vanka.argtypes = [P, I, I, DP, DP]
    L.ref2_level_descr.argtypes = [P, I, DP, DP, U8, DP]
    L.ref2_smooth_colour.argtypes = [P, I, I, DP, DP]
    return L


def dp(a):
    return a.ctypes.data_as(DP)


def blocked_problem3(n, kind):
    """Finest-level vol, fixed, penalty and rhs in the blocked layout.
    noise: the parabolic-inlet problem on a seeded smoothed-noise density (BP alpha law);
    general: non-uniform vol on cells and faces in [0.5, 2], about 3 % of the interior faces
    fixed besides the walls, random face penalties, random rhs;
    fixedcells: as general, with about 3 % of the cells fixed and random cell penalties.
    The reference's coarsest matrix (DirectSolve3D::update, stoke/StokeLike.cu:427-641)
    never reads the cell-cell entries off its probes (only the closed-domain block of ones
    is added), so a fixed coarse cell leaves that matrix singular and the reference's
    V-cycle returns NaN: that case pins the operators and smoothers only."""
    if kind == "noise":
        b, rho, phys, fp = problem(po, n, seed=11, sigma=2.0)
        cell_vol, face_vol, cell_fixed, face_fixed = b.cell_vol, b.face_vol, b.cell_fixed, b.face_fixed
        cell_pen, face_pen = np.zeros((n, n, n)), fp
        rhs = po.field_to_blocked(n, b.cell_b, b.face_b)
    else:
        b = po.bc_parabolic(n)
        u = lambda s, shape: 0.5 * (stable_vec(s, int(np.prod(shape))).reshape(shape) + 1.0)
        cell_vol = 0.5 + 1.5 * u(21, (n, n, n))
        face_vol = [0.5 + 1.5 * u(22 + d, po.face_shape(n, d)) for d in range(3)]
        cells = kind == "fixedcells"
        cell_fixed = (u(25, (n, n, n)) < (0.03 if cells else 0.0)).astype(np.int32)
        face_fixed = [((b.face_fixed[d] != 0) | (u(26 + d, po.face_shape(n, d)) < 0.03)).astype(np.int32)
                      for d in range(3)]
        cell_pen = np.where(u(29, (n, n, n)) < (0.5 if cells else 0.0), 10.0 * u(30, (n, n, n)), 0.0)
        face_pen = [100.0 * u(31 + d, po.face_shape(n, d)) ** 4 for d in range(3)]
        rhs = None
    vol = po.field_to_blocked(n, cell_vol, face_vol)
    fixed = po.field_to_blocked(n, cell_fixed.astype(float), [f.astype(float) for f in face_fixed]).astype(np.uint8)
    pen = po.field_to_blocked(n, cell_pen, face_pen)
    if rhs is None:
        # random, with the continuity (cell) part summing to zero: every wall face is
        # fixed, so a closed domain's divergence constraint needs a compatible right side
        rhs = stable_vec(40, vol.size)
        rhs[:n ** 3] -= rhs[:n ** 3].mean()
    return vol, fixed, pen, rhs


def blocked_problem2(n, kind):
    law, bc = ("ref", "test0") if kind == "test0" else ("bp", "parabolic")
    b, rho, phys, fp = problem2(po, n, seed=3, law=law, bc=bc)
    vol = po.field_to_blocked2(n, b.cell_vol, b.face_vol)
    fixed = po.field_to_blocked2(n, b.cell_fixed.astype(float), [f.astype(float) for f in b.face_fixed]).astype(np.uint8)
    pen = po.field_to_blocked2(n, np.zeros((n, n)), fp)
    rhs = po.field_to_blocked2(n, b.cell_b, b.face_b)
    return vol, fixed, pen, rhs


def run3(L, n, kind, full, solve_iters=50, solve=True):
    vol, fixed, pen, rhs = blocked_problem3(n, kind)
    h = L.ref3_create(n, 1)
    L.ref3_set_descr(h, dp(vol), fixed.ctypes.data_as(U8), dp(pen))
    L.ref3_update(h)
    lv = L.ref3_levels(h)
    dof = [L.ref3_level_dof(h, i) for i in range(lv)]
    out = dict(n=n, dim=3, levels=lv, closed=1, vol=vol, fixed=fixed, pen=pen, rhs=rhs)
    for i in range(lv):
        v, p_, f = np.zeros(dof[i]), np.zeros(dof[i]), np.zeros(dof[i], dtype=np.uint8)
        L.ref3_level_descr(h, i, dp(v), dp(p_), f.ctypes.data_as(U8))
        out[f"descr_vol_{i}"], out[f"descr_pen_{i}"], out[f"descr_fixed_{i}"] = v, p_, f
        y = np.zeros(dof[i])
        L.ref3_apply_A(h, i, dp(stable_vec(100 + i, dof[i])), dp(y))
        out[f"A_{i}"] = y
    y = np.zeros(dof[-1])
    L.ref3_apply_E(h, dp(stable_vec(150, dof[-1])), dp(y))
    out["E"] = y
    for i in range(lv - 1):
        if full or i < lv - 2:
            y = np.zeros(dof[i])
            L.ref3_restrict(h, i, dp(stable_vec(200 + i, dof[i + 1])), dp(y))
            out[f"R_{i}"] = y
            y = np.zeros(dof[i + 1])
            L.ref3_prolong(h, i, dp(stable_vec(300 + i, dof[i])), dp(y))
            out[f"P_{i}"] = y
    for i in range(1, lv):
        if not full and i == lv - 1:
            continue
        r = stable_vec(400 + i, dof[i])
        for flag in (0, 1):
            y = np.zeros(dof[i])
            L.ref3_vanka(h, i, flag, dp(r), dp(y))
            out[f"vanka_{i}_{flag}"] = y
        for post in (0, 1):
            y = np.zeros(dof[i])
            L.ref3_smooth(h, i, post, dp(r), dp(y))
            out[f"smooth_{i}_{post}"] = y
    if not solve:
        return out
    y = np.zeros(dof[0])
    L.ref3_coarse(h, dp(stable_vec(500, dof[0])), dp(y))
    out["coarse"] = y
    y = np.zeros(dof[-1])
    L.ref3_vcycle(h, dp(stable_vec(600, dof[-1])), dp(y))
    out["vcycle"] = y
    # the reference's multigrid never corrects fixed unknowns (their rows are the
    # identity): a right side it can solve is zero there, as the drivers' right sides are
    rhs = np.where(out[f"descr_fixed_{lv - 1}"] != 0, 0.0, rhs)
    out["rhs"] = rhs
    x = np.zeros(dof[-1])
    L.ref3_solve(h, dp(rhs), dp(x), solve_iters, 0.0, 1e-15, 0.0)
    Ax = np.zeros(dof[-1])
    L.ref3_apply_A(h, lv - 1, dp(x), dp(Ax))
    out["solve_x"], out["solve_iters"] = x, solve_iters
    out["solve_rel"] = np.linalg.norm(rhs - Ax) / np.linalg.norm(rhs)
    return out


def run2(L, n, kind, full, solve_iters=40):
    vol, fixed, pen, rhs = blocked_problem2(n, kind)
    h = L.ref2_create(n, 1)
    L.ref2_set_descr(h, dp(vol), fixed.ctypes.data_as(U8), dp(pen))
    lv = L.ref2_levels(h)
    dof = [L.ref2_level_dof(h, i) for i in range(lv)]
    out = dict(n=n, dim=2, levels=lv, closed=1, vol=vol, fixed=fixed, pen=pen, rhs=rhs)
    for i in range(lv):
        v, p_, f, lap = np.zeros(dof[i]), np.zeros(dof[i]), np.zeros(dof[i], dtype=np.uint8), np.zeros(1)
        L.ref2_level_descr(h, i, dp(v), dp(p_), f.ctypes.data_as(U8), dp(lap))
        out[f"descr_vol_{i}"], out[f"descr_pen_{i}"], out[f"descr_fixed_{i}"] = v, p_, f
        out[f"descr_lap_{i}"] = lap[0]
        y = np.zeros(dof[i])
        L.ref2_apply_A(h, i, dp(stable_vec(100 + i, dof[i])), dp(y))
        out[f"A_{i}"] = y
    y = np.zeros(dof[-1])
    L.ref2_apply_E(h, dp(stable_vec(150, dof[-1])), dp(y))
    out["E"] = y
    for i in range(lv - 1):
        if not full and i == lv - 2:
            continue
        y = np.zeros(dof[i])
        L.ref2_restrict(h, i, dp(stable_vec(200 + i, dof[i + 1])), dp(y))
        out[f"R_{i}"] = y
        y = np.zeros(dof[i + 1])
        L.ref2_prolong(h, i, dp(stable_vec(300 + i, dof[i])), dp(y))
        out[f"P_{i}"] = y
    for i in range(1, lv):
        if not full and i == lv - 1:
            continue
        r = stable_vec(400 + i, dof[i])
        for flag in (0, 1):
            y = np.zeros(dof[i])
            L.ref2_smooth_colour(h, i, flag, dp(r), dp(y))
            out[f"colour_{i}_{flag}"] = y
        for post in (0, 1):
            y = np.zeros(dof[i])
            L.ref2_smooth(h, i, post, dp(r), dp(y))
            out[f"smooth_{i}_{post}"] = y
    y = np.zeros(dof[0])
    L.ref2_coarse(h, dp(stable_vec(500, dof[0])), dp(y))
    out["coarse"] = y
    y = np.zeros(dof[-1])
    L.ref2_vcycle(h, dp(stable_vec(600, dof[-1])), dp(y))
    out["vcycle"] = y
    x = np.zeros(dof[-1])
    L.ref2_solve(h, dp(rhs), dp(x), solve_iters, 0.0, 1e-15, 0.0)
    Ax = np.zeros(dof[-1])
    L.ref2_apply_A(h, lv - 1, dp(x), dp(Ax))
    out["solve_x"], out["solve_iters"] = x, solve_iters
    out["solve_rel"] = np.linalg.norm(rhs - Ax) / np.linalg.norm(rhs)
    return out


CASES = {
    "ref3d_n8_noise": lambda L: run3(L, 8, "noise", True),
    "ref3d_n8_general": lambda L: run3(L, 8, "general", True),
    "ref3d_n8_fixedcells": lambda L: run3(L, 8, "fixedcells", True, solve=False),
    "ref3d_n16_noise": lambda L: run3(L, 16, "noise", False),
    "ref2d_n16_noise": lambda L: run2(L, 16, "noise", True),
    "ref2d_n64_test0": lambda L: run2(L, 64, "test0", False),
}


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STOKES_TO_REFERENCE", "/root/reference")
    out_dir = sys.argv[2] if len(sys.argv) > 2 else HERE
    L = load_lib(ref_root)
    for name, fn in CASES.items():
        out = fn(L)
        path = os.path.join(out_dir, name + ".npz")
        np.savez_compressed(path, **out)
        rel = f"{out['solve_rel']:.2e}" if "solve_rel" in out else "(no solve)"
        print(f"{name}: {os.path.getsize(path) / 1024:.0f} KB, reference GMRES rel. residual {rel}")


if __name__ == "__main__":
    main()
