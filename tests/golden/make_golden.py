"""Generates the committed golden fixtures under tests/golden/.

ref_grid3d_index.npz   blocked-layout index tables produced by the reference's OWN
                       grid3D host code (oracle/_ref/libref_grid3d.so, built from the
                       reference sources by oracle/ref_build.sh). Pins the layout.
oracle_n8.npz          oracle outputs on a seeded 8^3 problem (A x, E x, a V-cycle, the
                       solution to 1e-12) as a regression fixture for the oracle and
                       the GPU path.
ref_grid2d_index.npz   the 2D blocked-layout tables produced by the reference's own grid2D
                       host code (oracle/_ref/libref_grid2d.so).
oracle2d_n16.npz       2D oracle outputs on a seeded 16^2 problem (same contents as the
                       3D fixture).
oracle_loop2d_n64.npz  the oracle's 20-iteration design loop of the 2D 64^2 benchmark case
                       (parabolic inlet on a centred 16-cell segment, uniform 0.3 start,
                       volume fraction 0.3, BP law, filter radius 1.5, OC with move limit 0.2,
                       every solve to FP64 relative residual 1e-11): objective per iteration
                       and the design of the last iteration (before its update).
oracle_loop3d_n32.npz  the same for the 3D loop at 32^3 (parabolic inlet on a centred 8x8
                       patch, uniform 0.15 start, volume fraction 0.15), 8 iterations; from
                       iteration 5 the designs are high-contrast.
ref_mma.npz            six updates of the reference's own MMA solver (oracle/_ref/libref_mma.so,
                       built from simplex/ext/mma by oracle/ref_build.sh) on a seeded problem
                       with the reference optimizer's settings (one volume constraint with
                       coefficient 1e4, move limit 0.2, bounds [0.01, 1]).

usage: python tests/golden/make_golden.py [3d] [2d] [mma] [loop2d] [loop3d]
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def ref_index_tables():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_grid3d.so"))
    out = {}
    for n in (4, 8, 16):
        cells = np.array([[x, y, z, lib.ref_cell_ind(n, x, y, z)] for x in range(n) for y in range(n) for z in range(n)],
                         dtype=np.int32)
        out[f"cell_ind_{n}"] = cells
        for d in range(3):
            rows = []
            for x in range(n + 4 * (d == 0)):
                for y in range(n + 4 * (d == 1)):
                    for z in range(n + 4 * (d == 2)):
                        rows.append([x, y, z, lib.ref_face_ind(n, x, y, z, d), lib.ref_face_valid(n, x, y, z, d)])
            out[f"face_ind_{n}_{d}"] = np.array(rows, dtype=np.int32)
            xyz = (ctypes.c_int * 3)()
            inv = []
            for i in range(lib.ref_face_size(n, d)):
                lib.ref_ind_face(n, i, d, xyz)
                inv.append([i, xyz[0], xyz[1], xyz[2]])
            out[f"ind_face_{n}_{d}"] = np.array(inv, dtype=np.int32)
            erows = []
            for x in range(n + (d != 0)):
                for y in range(n + (d != 1)):
                    for z in range(n + (d != 2)):
                        erows.append([x, y, z, lib.ref_edge_ind(n, x, y, z, d)])
            out[f"edge_ind_{n}_{d}"] = np.array(erows, dtype=np.int32)
        xyz = (ctypes.c_int * 3)()
        inv = []
        for i in range(lib.ref_cell_size(n)):
            lib.ref_ind_cell(n, i, xyz)
            inv.append([i, xyz[0], xyz[1], xyz[2]])
        out[f"ind_cell_{n}"] = np.array(inv, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_grid3d_index.npz"), **out)


def oracle_regression():
    from oracle import pyoracle as po
    from tests.helpers import problem

    n = 8
    b, rho, phys, fp = problem(po, n, seed=11, sigma=2.0)
    o = po.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    o.setup()
    x = np.random.default_rng(12).standard_normal(o.level_dof(o.levels - 1))
    bb = po.field_to_blocked(n, b.cell_b, b.face_b)
    sol, st = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-14, norm_thr=0.0, restarts=4, true_tol=1e-12)
    np.savez_compressed(os.path.join(HERE, "oracle_n8.npz"), rho=rho, x=x, Ax=o.apply_A(x), Ex=o.apply_E(x),
                        b=bb, vcycle_b=o.vcycle(bb), solution=sol, rel_true=st["rel_true"])


def ref_index_tables_2d():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_grid2d.so"))
    out = {}
    for n in (8, 16, 32):
        out[f"cell_ind_{n}"] = np.array([[x, y, lib.ref2_cell_ind(n, x, y)] for x in range(n) for y in range(n)],
                                        dtype=np.int32)
        for d in range(2):
            out[f"face_ind_{n}_{d}"] = np.array([[x, y, lib.ref2_face_ind(n, x, y, d)] for x in range(n + 8 * (d == 0))
                                                 for y in range(n + 8 * (d == 1))], dtype=np.int32)
            out[f"face_size_{n}_{d}"] = np.array([lib.ref2_face_size(n, d)], dtype=np.int32)
        out[f"node_ind_{n}"] = np.array([[x, y, lib.ref2_node_ind(n, x, y)] for x in range(n + 8) for y in range(n + 8)],
                                        dtype=np.int32)
        xy = (ctypes.c_int * 2)()
        inv = []
        for i in range(lib.ref2_cell_size(n)):
            lib.ref2_ind_cell(n, i, xy)
            inv.append([i, xy[0], xy[1]])
        out[f"ind_cell_{n}"] = np.array(inv, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "ref_grid2d_index.npz"), **out)


def oracle_regression_2d():
    from oracle import pyoracle as po
    from tests.helpers import problem2

    n = 16
    b, rho, phys, fp = problem2(po, n, seed=11, sigma=2.0)
    o = po.Steady2D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    x = np.random.default_rng(12).standard_normal(o.level_dof(o.levels - 1))
    bb = po.field_to_blocked2(n, b.cell_b, b.face_b)
    sol, st = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-14, norm_thr=0.0, restarts=4, true_tol=1e-12)
    np.savez_compressed(os.path.join(HERE, "oracle2d_n16.npz"), rho=rho, x=x, Ax=o.apply_A(x), Ex=o.apply_E(x), b=bb,
                        vcycle_b=o.vcycle(bb), solution=sol, rel_true=st["rel_true"])


def mma_problem(n=4096, iters=6, seed=0):
    """Seeded inputs of the MMA fixture: per update a negative sensitivity, the volume
    constraint g = 1e4 (mean x - 0.3) with gradient 1e4 / n, and bounds
    [max(0.01, x - 0.2), min(1, x + 0.2)] (simplex/src/optimization/OptimizerMma.h:96-128)."""
    rng = np.random.default_rng(seed)
    return [-np.abs(rng.standard_normal(n)) * (1 + 3 * rng.random(n)) for _ in range(iters)]


def mma_run(solver, n, dfs, frac=0.3):
    x = np.full(n, frac)
    xs = []
    for df in dfs:
        g = 1e4 * (x.mean() - frac)
        dg = np.full(n, 1e4 / n)
        solver.update(x, df, g, dg, np.maximum(0.01, x - 0.2), np.minimum(1.0, x + 0.2))
        xs.append(x.copy())
    return np.array(xs)


def ref_mma():
    from oracle import pyoracle as po

    n = 4096  # the cells of a 64^2 (or 16^3) design
    dfs = mma_problem(n)
    xs = mma_run(po.RefMma(n), n, dfs)
    np.savez_compressed(os.path.join(HERE, "ref_mma.npz"), dfdx=np.array(dfs), x=xs)


def oracle_loop2d(n=64, iters=20, frac=0.3, rmin=1.5, save=True):
    from oracle import pyoracle as po

    po.build()
    b = po.bc_parabolic(n, 2, width=n // 4)
    vw = po.filt(np.ones((n, n)), rmin, transpose=True)
    x = np.full((n, n), frac)
    Js = []
    for it in range(iters):
        x_last = x.copy()
        phys = po.filt(x, rmin)
        fp = po.face_penalty(phys, 1, [1e4], dim=2)
        o = po.Steady2D(n)
        o.init_boundary(b)
        o.update_penalty(np.zeros((n, n)), fp)
        o.update_b(b.cell_b, b.face_b)
        u, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=8, true_tol=1e-11)
        Js.append(o.energy(u))
        o.set_b_blocked(o.apply_E(u))
        lam, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=8, true_tol=1e-11)
        _, uf = po.blocked_to_field2(n, u)
        _, lf = po.blocked_to_field2(n, lam)
        sens = po.sensitivity(phys, 1, [1e4], uf, lf, dim=2)
        dc = po.filt(sens, rmin, transpose=True)
        x = po.oc_update(x, dc, vw / n ** 2, vw, frac)[0].reshape(n, n)
        print("loop2d", it, Js[-1], flush=True)
    if save:
        np.savez_compressed(os.path.join(HERE, "oracle_loop2d_n64.npz"), objective=np.array(Js), x_last=x_last)
    return np.array(Js), x_last


def oracle_loop3d(n=32, iters=8, frac=0.15, rmin=1.5, save=True):
    """The 3D design loop (parabolic inlet on a centred n/4 square, OC, filter 1.5, BP alpha
    1e4) for `iters` iterations; from iteration 5 the designs are high-contrast (density
    down to 1e-6 .. 1e-8) and each solve takes over a hundred GMRES steps."""
    from oracle import pyoracle as po

    po.build()
    b = po.bc_parabolic(n)
    vw = po.filt(np.ones((n, n, n)), rmin, transpose=True)
    x = np.full((n, n, n), frac)
    Js = []
    for it in range(iters):
        x_last = x.copy()
        phys = po.filt(x, rmin)
        fp = po.face_penalty(phys, 1, [1e4])
        o = po.Steady3D(n)
        o.init_boundary(b)
        o.update_penalty(np.zeros((n, n, n)), fp)
        o.update_b(b.cell_b, b.face_b)
        o.setup()
        u, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=10, true_tol=1e-11)
        Js.append(o.energy(u))
        o.set_b_blocked(o.apply_E(u))
        lam, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=10, true_tol=1e-11)
        _, uf = po.blocked_to_field(n, u)
        _, lf = po.blocked_to_field(n, lam)
        sens = po.sensitivity(phys, 1, [1e4], uf, lf)
        dc = po.filt(sens, rmin, transpose=True)
        x = po.oc_update(x, dc, vw / n ** 3, vw, frac)[0].reshape(n, n, n)
        print("loop3d", it, Js[-1], flush=True)
    if save:
        np.savez_compressed(os.path.join(HERE, "oracle_loop3d_n32.npz"), objective=np.array(Js), x_last=x_last)
    return np.array(Js), x_last


if __name__ == "__main__":
    what = sys.argv[1:] or ["3d", "2d", "mma", "loop2d", "loop3d"]
    if "3d" in what:
        ref_index_tables()
        oracle_regression()
    if "2d" in what:
        ref_index_tables_2d()
        oracle_regression_2d()
    if "mma" in what:
        ref_mma()
    if "loop2d" in what:
        oracle_loop2d()
    if "loop3d" in what:
        oracle_loop3d()
    print("wrote", os.listdir(HERE))
