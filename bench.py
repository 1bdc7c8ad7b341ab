"""Benchmark: seconds per 256^3 Brinkman-Stokes solve to FP64 relative residual 1e-8.

One step = one full solve (coarse re-discretisation, coarsest inverse, FP32 V-cycle
FGMRES inside FP64 refinement) of the 256^3 parabolic-inlet problem with a seeded,
Gaussian-smoothed density (sigma 4 cells), density filter r = 1.5 and the
Borrvall-Petersson alpha law (amax 1e4). Working set is ~27 GB, far above the 129 MB L2.

  value  device-resident inputs, CUDA events on the solve stream (method: plain, the
         library default: FP32 V-cycle with one smoother sweep per colour, FGMRES in FP64
         refinement)
  e2e    host buffers through the C ABI: set_penalty + set_rhs + solve + read back
  methods  the same solve with the reference's two sweeps per colour, the mixed form (BF16
         coarse corrections) and the learned form (U-Net trained on the GPU at 64^3 on the
         same problem family, applied at 256^3); training time reported, not in the timed region
  design_loop_2d / design_loop_3d  the fluid_topo driver's design loops (2D 64^2, 20
         iterations; 3D 128^3 at fraction 0.15, 40 iterations), every solve to its FP64
         tolerance, with the largest final residual of any solve
  roofline / vcycle_hbm  the dominant kernel class and the whole V-cycle: algorithmic bytes
         over CUDA-event time against the measured copy bandwidth; traffic from the
         committed ncu summary
  solve_batches  the configurations' batches of independent solves: 100 at 128^3 (plain)
         and 50 at 256^3 (mixed), each on its own seeded density
  cpu_baseline  a bounded sample of the 256^3 oracle solve on the host cores (its set-up
         and a two-iteration GMRES(V-cycle) run), scaled to the V-cycle count of the full
         256^3 oracle solve recorded in profiles/oracle_solve_256cube.md
  --impl reference: the same 256^3 oracle (the reference's FP64 GMRES(V-cycle) path
         restated, pinned to the reference's own code) on all the host cores: set-up once,
         a two-iteration GMRES run per step, scaled the same way.
  --oracle-check: the GPU solutions against the FP64 oracle per field, J and dJ/drho.
  --learned-config: the learned configuration (training on noise and OC trajectories,
         then learned against plain on solves and the 40-iteration design loop, and the
         learned warm start against the plain one on that loop).
  --learned-warm: the learned warm start (warm_start 2, network trained at 64^3 on noise
         as in the bench's learned leg) against the plain warm start on the n^3
         40-iteration design loop.

N>1 (torchrun): independent replicas, one per GPU, barrier + max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 256
TOL = 1e-8
FALLBACK_HBM_GBS = 6800.0
METRIC = "s per 256^3 Stokes solve to FP64 resid 1e-8"
NET_TRAIN_N = 64
NET_TRAIN_STEPS = 3000
NET_LR = 3e-4


PROFILED_SOLVES = 2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-methods", action="store_true", help="skip the reference-smoother, mixed and learned legs")
    ap.add_argument("--oracle-check", action="store_true",
                    help="per-field error of the GPU solve against the full FP64 oracle solve (minutes on the host)")
    ap.add_argument("--learned-config", action="store_true",
                    help="train the network per the learned configuration and compare it with plain (minutes)")
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--learned-warm", action="store_true",
                    help="the learned warm start against the plain one on the 40-iteration design loop")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def face_shape(n, d):
    s = [n, n, n]
    s[d] += 1
    return tuple(s)


def parabolic_bc(n):
    """Parabolic inlet on a centred N/4 x N/4 patch of x = 0, mirrored outlet at x = 1,
    every boundary face fixed, in the reference's source-term encoding."""
    W = n // 4
    lo = n // 2 - W // 2
    cell_vol = np.ones((n, n, n))
    cell_fixed = np.zeros((n, n, n), dtype=np.int32)
    cell_b = np.zeros((n, n, n))
    face_vol = [np.ones(face_shape(n, d)) for d in range(3)]
    face_fixed = [np.zeros(face_shape(n, d), dtype=np.int32) for d in range(3)]
    face_b = [np.zeros(face_shape(n, d)) for d in range(3)]
    face_fixed[0][0], face_fixed[0][n] = 1, 1
    face_fixed[1][:, 0], face_fixed[1][:, n] = 1, 1
    face_fixed[2][:, :, 0], face_fixed[2][:, :, n] = 1, 1
    t = np.arange(lo, lo + W)
    s = (t + 0.5) - n / 2.0
    g1 = 1.0 - (2.0 * s / W) ** 2
    g = np.outer(g1, g1)
    cell_b[0, lo:lo + W, lo:lo + W] = g
    face_b[0][1, lo:lo + W, lo:lo + W] = g
    cell_b[n - 1, lo:lo + W, lo:lo + W] = -g
    face_b[0][n - 1, lo:lo + W, lo:lo + W] = g
    return cell_vol, cell_fixed, cell_b, face_vol, face_fixed, face_b


def face_penalty_host(rho_f, amax=1e4):
    """Face penalty = sum over the two adjacent cells of 1/2 alpha(rho~) (host arrays for e2e)."""
    a = 0.5 * amax * 0.1 * (1.0 - rho_f) / (0.1 + rho_f)
    out = []
    for d in range(3):
        f = np.zeros(face_shape(rho_f.shape[0], d))
        sl_lo = [slice(None)] * 3
        sl_hi = [slice(None)] * 3
        sl_lo[d] = slice(0, -1)
        sl_hi[d] = slice(1, None)
        f[tuple(sl_hi)] += a
        f[tuple(sl_lo)] += a
        out.append(f)
    return out


class Clocks:
    """Samples nvidia-smi every 200 ms while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            for k in ("hbm_gbs", "hbm_GBps", "hbm"):
                if k in d:
                    v = d[k]
                    return float(v["burst"] if isinstance(v, dict) and "burst" in v else v), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    """DRAM bytes per launch of each kernel class from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic_256.txt")
    out = {}
    if os.path.exists(p):
        for ln in open(p):
            ln = ln.strip()
            if ln.startswith("traffic "):
                _, cls, val = ln.split()[:3]
                out[cls] = float(val)
    return out


def design_loop(driver, dim, n, frac, iters):
    """Runs the fluid_topo driver's design loop (test 1: parabolic inlet, uniform start at
    the volume fraction, filter 1.5, OC with move 0.2, no frames written) and returns the
    time per design iteration (two solves, sensitivity, filter, OC update) from the
    driver's own log."""
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        cmd = [driver, "-driver", "0" if dim == 2 else "1", "-test", "1", "-s", str(n), "-frac", str(frac), "-lf", str(iters),
               "-frames", "0", "-o", d]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
        if r.returncode != 0:
            return {"error": r.stderr.strip()[-300:]}
        log = np.genfromtxt(os.path.join(d, "log.csv"), delimiter=",", names=True)
    it_ms = np.atleast_1d(log["iteration_ms"])
    vf, va = np.atleast_1d(log["v_cycles_forward"]), np.atleast_1d(log["v_cycles_adjoint"])
    tol = "1e-10" if dim == 2 else "1e-8"
    return {"workload": f"{dim}D {n}^{dim} design loop (fluid_topo -driver {0 if dim == 2 else 1} -test 1 -s {n} -frac {frac}), "
                        f"OC, filter 1.5, every solve to FP64 rel. residual {tol}",
            "iterations": int(iters), "total_s": round(float(np.sum(it_ms)) / 1e3, 3),
            "ms_per_iteration_median": round(float(np.median(it_ms[1:])), 3),
            "v_cycles_per_iteration_median": float(np.median((vf + va)[1:])),
            "v_cycles_per_solve_max": int(max(vf.max(), va.max())),
            "rel_residual_max": float(max(np.max(np.atleast_1d(log["rel_residual_forward"])),
                                          np.max(np.atleast_1d(log["rel_residual_adjoint"])))),
            "final_objective": float(np.atleast_1d(log["objective"])[-1])}


# ------------------------------------------------------------------ reference (CPU) arm
ORACLE_RECORD = os.path.join(ROOT, "profiles", "oracle_solve_256cube.md")


def oracle_problem(n):
    """The bench problem on the oracle: the same seeded density (seed 1, sigma 4), filter and
    BP law as make_solver on rank 0."""
    from oracle import pyoracle as po

    po.build()
    b = po.bc_parabolic(n)
    rho = po.density_noise(n, 1, 4.0)
    phys = po.filt(rho, 1.5)
    fp = po.face_penalty(phys, 1, [1e4])
    o = po.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    return po, o, b, phys


def oracle_record():
    """GMRES iterations and time of the full 256^3 oracle solve measured on this machine
    (written by `bench.py --oracle-check`)."""
    out = {}
    if os.path.exists(ORACLE_RECORD):
        for ln in open(ORACLE_RECORD):
            p = ln.strip().split()
            if len(p) == 3 and p[0] == "record":
                out[p[1]] = float(p[2])
    return out


def oracle_full_solve(n, tol=TOL, max_iter=60, restarts=6):
    """The reference algorithm on the host cores (the oracle: the reference's FP64 V-cycle -
    Vanka smoother, re-discretised coarse levels, dense coarsest solve - as GMRES
    preconditioner), solved to FP64 true relative residual `tol`. Returns the solution and
    the timings of the set-up and of the Krylov solve."""
    po, o, b, phys = oracle_problem(n)
    t0 = time.perf_counter()
    o.setup()
    t1 = time.perf_counter()
    x, st = o.solve(max_iter=max_iter, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=restarts, true_tol=tol)
    t2 = time.perf_counter()
    return po, o, b, phys, x, st, t1 - t0, t2 - t1


def oracle_sample(n):
    """The oracle's 256^3 set-up and a bounded piece of its GMRES: returns (set-up s, the
    oracle handle, a function that times one GMRES run of two iterations - three V-cycles
    and two operator applications - and returns seconds per V-cycle)."""
    po, o, b, phys = oracle_problem(n)
    t0 = time.perf_counter()
    o.setup()
    setup_s = time.perf_counter() - t0

    def step():
        t1 = time.perf_counter()
        o.solve(max_iter=3, abs_thr=0.0, rel_thr=0.0, norm_thr=0.0)
        return (time.perf_counter() - t1) / 3.0

    return setup_s, o, step


def scale_to_solve(setup_s, per_vcycle, n):
    """s per solve from a sample: the set-up plus the V-cycles of the full 256^3 oracle solve
    to 1e-8 recorded in profiles/oracle_solve_256cube.md (measured there in full)."""
    rec = oracle_record() if n == 256 else {}
    vc = rec.get("vcycles")
    if vc:
        return setup_s + per_vcycle * vc, (f"scaled to the {int(vc)} V-cycles of the full {n}^3 oracle solve to {TOL:g} "
                                           f"(profiles/oracle_solve_256cube.md, measured there at {rec.get('total_s', 0):.0f} s)")
    return setup_s + per_vcycle * 3, "not scaled (no full-solve record for this size)"


def cpu_reference_sample(n=N_DEFAULT):
    """cpu_baseline: the oracle's full 256^3 set-up and one GMRES run of two iterations,
    measured on the host cores, scaled to a whole solve (scale_to_solve)."""
    setup_s, o, step = oracle_sample(n)
    per_vc = step()
    o.close()
    value, how = scale_to_solve(setup_s, per_vc, n)
    sample = (f"oracle at {n}^3 (the reference's FP64 GMRES(V-cycle) path restated): set-up {setup_s:.1f} s and a "
              f"GMRES run of 2 iterations ({per_vc:.2f} s per V-cycle), measured; {how}")
    return value, sample, setup_s + 3 * per_vc


def run_reference(args):
    """--impl reference: the oracle (the reference's FP64 GMRES(V-cycle) path restated, pinned
    to its own code) at 256^3 on all the host cores. Its set-up is measured once; every step
    (warm-up or timed) is one GMRES run of two iterations at 256^3, so a step takes a few
    seconds; the line's value is s per whole solve: set-up plus the mean V-cycle time times
    the V-cycles of the full 256^3 oracle solve (recorded, measured in full, in
    profiles/oracle_solve_256cube.md)."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    n = args.n
    setup_s, o, step = oracle_sample(n)
    for _ in range(args.warmup):
        step()
    per = [step() for _ in range(args.steps)]
    o.close()
    per_vc = statistics.mean(per)
    value, how = scale_to_solve(setup_s, per_vc, n)
    sample = (f"oracle at {n}^3 on {cores} host threads: set-up {setup_s:.1f} s (once), then per step a GMRES run of "
              f"2 iterations (3 V-cycles, {per_vc:.2f} s each); value = set-up + V-cycle time x V-cycles, {how}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s/solve", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 3e3 * per_vc, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"3D {n}^3 Brinkman-Stokes solve to FP64 rel. residual {TOL:g}", "n": n, "tol": TOL},
        "cpu_baseline": {"value": value, "unit": "s/solve", "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "s/solve", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def oracle_check(args):
    """--oracle-check: the GPU solves of the bench problem (plain and mixed) against the FP64
    oracle at n^3, per field (velocity components, pressure modulo a constant), the energy J
    and the adjoint sensitivity dJ/drho; and the oracle's own timings, including its solve to
    the bench tolerance. Writes one JSON line."""
    import torch

    from stokes_to_gb300 import build, capi

    build.build()
    n = args.n
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cell_vol, cell_fixed, cell_b, face_vol, face_fixed, face_b = parabolic_bc(n)
    law = capi.alpha_bp(1e4)
    out = {}
    for method, name in ((capi.STG_METHOD_PLAIN, "plain"), (capi.STG_METHOD_MIXED, "mixed")):
        s = capi.Solver(n, method=method, tol=1e-9)
        s.set_boundary(cell_vol, cell_fixed, face_vol, face_fixed, True)
        s.density_noise(1, 4.0, want=False)
        s.filter(1.5, None, want=False)
        s.set_density(None, law)
        s.set_rhs(cell_b, face_b)
        p, vel, st = s.solve()
        J = s.energy()
        g, ast = s.adjoint_sensitivity(law)
        out[name] = {"p": p, "vel": vel, "J": J, "sens": g, "rel_residual": st["rel_residual"],
                     "adjoint_rel_residual": ast["rel_residual"]}
        s.close()
    torch.cuda.empty_cache()
    # the oracle's solve to the bench tolerance first (its timing is the CPU record), then
    # a tighter one for the comparison
    po8, o8, b8, phys8, x8, st8, setup8, solve8 = oracle_full_solve(n, TOL)
    o8.close()
    po, o, b, phys, x, st, setup_s, solve_s = oracle_full_solve(n, 1e-10)
    t0 = time.perf_counter()
    o.set_b_blocked(o.apply_E(x))
    lam, ast = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=6, true_tol=1e-10)
    adj_s = time.perf_counter() - t0
    p_ref, vel_ref = po.blocked_to_field(n, x)
    _, lam_f = po.blocked_to_field(n, lam)
    g_ref = po.sensitivity(phys, 1, [1e4], vel_ref, lam_f)
    J_ref = o.energy(x)

    def rel(a, b_):
        return float(np.linalg.norm(np.asarray(a) - np.asarray(b_)) / np.linalg.norm(np.asarray(b_)))

    res = {"workload": f"3D {n}^3 bench problem, GPU solves to 1e-9 against the FP64 oracle solves to 1e-10",
           "oracle_to_bench_tol": {"setup_s": round(setup8, 2), "solve_s": round(solve8, 2), "iterations": st8["iters"],
                                   "restarts": st8["restarts"], "rel_true": st8["rel_true"],
                                   "total_s": round(setup8 + solve8, 2), "cores": int(os.environ["OMP_NUM_THREADS"])},
           "oracle_to_1e-10": {"setup_s": round(setup_s, 2), "solve_s": round(solve_s, 2), "iterations": st["iters"],
                               "restarts": st["restarts"], "rel_true": st["rel_true"], "adjoint_s": round(adj_s, 2),
                               "adjoint_rel_true": ast["rel_true"]}}
    for name in ("plain", "mixed"):
        r = out[name]
        res[name] = {"u": rel(r["vel"][0], vel_ref[0]), "v": rel(r["vel"][1], vel_ref[1]), "w": rel(r["vel"][2], vel_ref[2]),
                     "p_mod_const": rel(r["p"] - r["p"].mean(), p_ref - p_ref.mean()),
                     "J": abs(r["J"] - J_ref) / abs(J_ref), "sensitivity": rel(r["sens"], g_ref),
                     "gpu_rel_residual": r["rel_residual"], "gpu_adjoint_rel_residual": r["adjoint_rel_residual"]}
    print(json.dumps(res), flush=True)


# ------------------------------------------------------------------ learned-preconditioner configuration
def oc_loop(capi, s, n, frac, iters, law, on_iteration=None):
    """The OC design loop of the fluid_topo driver (test 1: filter 1.5, move 0.2, uniform start
    at the volume fraction) through the C ABI; on_iteration(it) runs after each iteration.
    Returns per iteration (ms, V-cycles of both solves, objective, largest final residual)."""
    import torch

    x = np.full((n, n, n), frac)
    out = []
    for it in range(iters):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        phys = s.filter(1.5, x)
        s.set_density(phys, law)
        _, _, st = s.solve(want=False)
        J = s.energy()
        dc, ast = s.adjoint_sensitivity(law)
        dc = s.filter(1.5, dc, transpose=True)
        x, _ = s.oc_update(1.5, x, dc, frac)
        torch.cuda.synchronize()
        out.append(((time.perf_counter() - t0) * 1e3, st["inner_iters"] + ast["inner_iters"], J,
                    max(st["rel_residual"], ast["rel_residual"])))
        if on_iteration:
            on_iteration(it)
    return out


def learned_config(args):
    """--learned-config: the learned-preconditioner configuration as specified - the network
    trained on the GPU by its own kernels at n^3 on residual/error pairs from the plain
    solver's operators on seeded smoothed-noise densities (sigma 2..8) and on snapshots of
    40-iteration OC runs at volume fractions 0.1..0.4 (Adam, lr 1e-3, --pairs in all) - then
    applied inside FGMRES against the plain method: independent solves and the 40-iteration
    design loop at fraction 0.15, every solve to FP64 rel. residual 1e-8. One JSON line."""
    import torch

    from stokes_to_gb300 import build, capi

    build.build()
    n = args.n
    cell_vol, cell_fixed, cell_b, face_vol, face_fixed, face_b = parabolic_bc(n)
    law = capi.alpha_bp(1e4)

    def solver(method, **kw):
        s = capi.Solver(n, method=method, tol=TOL, **kw)
        s.set_boundary(cell_vol, cell_fixed, face_vol, face_fixed, True)
        s.set_rhs(cell_b, face_b)
        return s

    tr = solver(capi.STG_METHOD_PLAIN, warm_start=1)
    tr.net_init(7)
    pairs, losses = 0, []
    per_noise = max(1, args.pairs // 5 // 7)
    t0 = time.perf_counter()
    for q, sig in enumerate(range(2, 9)):
        tr.density_noise(200 + q, float(sig), want=False)
        tr.filter(1.5, None, want=False)
        tr.set_density(None, law)
        losses.extend(tr.net_train(per_noise, lr=1e-3, seed=11 + q).tolist())
        pairs += per_noise
    fracs = (0.1, 0.2, 0.3, 0.4)
    per_snap = max(1, (args.pairs - pairs) // (len(fracs) * 20))

    def snap(it):
        nonlocal pairs
        if it % 2 == 1:
            losses.extend(tr.net_train(per_snap, lr=1e-3, seed=1000 + pairs).tolist())
            pairs += per_snap

    for f in fracs:
        oc_loop(capi, tr, n, f, 40, law, snap)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    params = tr.net_params()
    tr.close()

    res = {"workload": f"3D {n}^3 learned-preconditioner configuration, every solve to FP64 rel. residual {TOL:g}",
           "train": {"pairs": pairs, "s": round(train_s, 1), "noise_sigmas": "2..8",
                     "trajectories": "OC runs of 40 iterations at fractions 0.1, 0.2, 0.3, 0.4; a training burst on "
                                     "every second iteration's operator", "loss_first_100": round(float(np.mean(losses[:100])), 4),
                     "loss_last_500": round(float(np.mean(losses[-500:])), 4)}}
    for method, name in ((capi.STG_METHOD_PLAIN, "plain"), (capi.STG_METHOD_LEARNED, "learned")):
        s = solver(method, warm_start=1)
        if method == capi.STG_METHOD_LEARNED:
            s.net_init(7)
            s.net_set_params(params)
        times, its, falls = [], [], []
        for seed in range(11):
            s.density_noise(3000 + seed, 4.0, want=False)
            s.filter(1.5, None, want=False)
            s.set_density(None, law)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            _, _, st = s.solve(want=False)
            torch.cuda.synchronize()
            if seed > 0:  # the first solve warms the CUDA graphs
                times.append(time.perf_counter() - t1)
                its.append(st["inner_iters"])
                falls.append(st["fallbacks"])
        res[f"solves_{name}"] = {"s_per_solve": round(float(np.mean(times)), 5), "v_cycles_mean": float(np.mean(its)),
                                 "fallbacks": int(sum(falls))}
        res[f"loop_{name}"] = loop_summary(oc_loop(capi, s, n, 0.15, 40, law))
        s.close()
    # the learned warm start: plain solves, each warm start corrected by one learned step
    s = solver(capi.STG_METHOD_PLAIN, warm_start=2)
    s.net_init(7)
    s.net_set_params(params)
    res["loop_plain_learned_warm_start"] = loop_summary(oc_loop(capi, s, n, 0.15, 40, law))
    s.close()
    print(json.dumps(res), flush=True)


def loop_summary(loop):
    ms = np.array([q[0] for q in loop])
    vc = np.array([q[1] for q in loop])
    return {"total_s": round(float(ms.sum()) / 1e3, 3), "ms_per_iteration_median": round(float(np.median(ms)), 2),
            "v_cycles_per_iteration_median": float(np.median(vc)), "v_cycles_total": int(vc.sum()),
            "final_objective": float(loop[-1][2]), "rel_residual_max": float(max(q[3] for q in loop))}


def learned_warm(args):
    """--learned-warm: the learned warm start (warm_start 2: the previous solution plus one
    FGMRES step whose preconditioner is the network-corrected V-cycle) against the plain warm
    start on the n^3 40-iteration OC loop at fraction 0.15, every solve to FP64 rel. residual
    1e-8; the network trained at 64^3 on seeded noise densities as in the bench's learned
    leg. One JSON line."""
    import torch

    from stokes_to_gb300 import build, capi

    build.build()
    n = args.n
    law = capi.alpha_bp(1e4)

    def solver(nn, **kw):
        bc = parabolic_bc(nn)
        s = capi.Solver(nn, method=capi.STG_METHOD_PLAIN, tol=TOL, **kw)
        s.set_boundary(bc[0], bc[1], bc[3], bc[4], True)
        s.set_rhs(bc[2], bc[5])
        return s

    tr = solver(NET_TRAIN_N)
    tr.density_noise(1, 4.0, want=False)
    tr.filter(1.5, None, want=False)
    tr.set_density(None, law)
    tr.net_init(7)
    t0 = time.perf_counter()
    losses = tr.net_train(NET_TRAIN_STEPS, lr=NET_LR, seed=3)
    torch.cuda.synchronize()
    res = {"workload": f"3D {n}^3 40-iteration OC loop at fraction 0.15, plain solves to FP64 rel. residual {TOL:g}: "
                       "plain warm start against the learned warm start",
           "train": {"s": round(time.perf_counter() - t0, 1), "steps": NET_TRAIN_STEPS, "n": NET_TRAIN_N,
                     "final_loss": round(float(np.mean(losses[-100:])), 4)}}
    params = tr.net_params()
    tr.close()
    for ws, name in ((1, "plain_warm_start"), (2, "learned_warm_start")):
        s = solver(n, warm_start=ws)
        if ws == 2:
            s.net_init(7)
            s.net_set_params(params)
        res[name] = loop_summary(oc_loop(capi, s, n, 0.15, 40, law))
        s.close()
    print(json.dumps(res), flush=True)


# ------------------------------------------------------------------ replicas
class Ranks:
    """Bookkeeping of N independent replicas (one process per GPU, no data-path
    collective): barriers around the timed region and the max / sum of per-rank scalars.
    The timing reductions run on `device` ("cuda" with NCCL on the GPU boxes, "cpu" with
    gloo in the tests)."""

    def __init__(self, world, rank, device="cuda"):
        self.world, self.rank, self.device = world, rank, device

    def barrier(self):
        import torch

        if self.world > 1:
            torch.distributed.barrier()
        if self.device == "cuda":
            torch.cuda.synchronize()

    def _reduce(self, v, op):
        import torch

        if self.world == 1:
            return v
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        torch.distributed.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        import torch

        return self._reduce(v, torch.distributed.ReduceOp.MAX if self.world > 1 else None)

    def sum(self, v):
        import torch

        return self._reduce(v, torch.distributed.ReduceOp.SUM if self.world > 1 else None)


def whole_job_seconds_per_solve(t_max_s, steps, world):
    """Weak scaling: every rank solves `steps` problems of its own; the job's time per solve
    is the slowest rank's time over all ranks' solves."""
    return t_max_s / (steps * world)


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from stokes_to_gb300 import build, capi

    build.build()
    n = args.n
    cell_vol, cell_fixed, cell_b, face_vol, face_fixed, face_b = parabolic_bc(n)

    ranks = Ranks(world, rank, "cuda")
    barrier, max_over_ranks, sum_over_ranks = ranks.barrier, ranks.max, ranks.sum

    stream = torch.cuda.current_stream()

    def make_solver(method, nn=n, **kw):
        bc = parabolic_bc(nn) if nn != n else (cell_vol, cell_fixed, cell_b, face_vol, face_fixed, face_b)
        s = capi.Solver(nn, method=method, tol=TOL, **kw)
        s.set_stream(stream.cuda_stream)
        s.set_boundary(bc[0], bc[1], bc[3], bc[4], True)
        s.density_noise(1 + rank, 4.0, want=False)
        s.filter(1.5, None, want=False)
        s.set_density(None, capi.alpha_bp(1e4))
        s.set_rhs(bc[2], bc[5])
        return s

    def timed_device(s, steps, warmup, profile=False):
        for _ in range(warmup):
            s.solve(want=False)
        barrier()
        if profile:
            s.profile(True)
        l0 = capi.kernel_launches()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stats = []
        with Clocks(local) as clk:
            barrier()
            e0.record(stream)
            for _ in range(steps):
                _, _, st = s.solve(want=False)
                stats.append(st)
            e1.record(stream)
            barrier()
        ms = e0.elapsed_time(e1)
        launches = capi.kernel_launches() - l0
        prof = None
        if profile:
            prof = s.profile_read()
            s.profile(False)  # the later measurements run with the CUDA graphs, unprofiled
        return ms, stats, launches, clk.summary(), prof

    # ---- headline: plain method, inputs resident (no per-kernel events in this region)
    s = make_solver(capi.STG_METHOD_PLAIN)
    ms, stats, launches, clocks, _ = timed_device(s, args.steps, args.warmup, profile=False)
    t_max = max_over_ranks(ms / 1e3)
    value = whole_job_seconds_per_solve(t_max, args.steps, world)
    launches = int(sum_over_ranks(launches))
    # per-kernel-class CUDA-event timing of separate solves, for the roofline and the table
    _, _, _, _, prof = timed_device(s, PROFILED_SOLVES, 0, profile=True)

    # ---- e2e: host (pinned) buffers through the C ABI, copies inside the timed region
    rho = s.density_noise(1 + rank, 4.0, want=True)
    rho_f = s.filter(1.5, rho, want=True)
    fpen = face_penalty_host(rho_f)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    fpen_p = [pin(f) for f in fpen]
    cb_p, fb_p = pin(cell_b), [pin(f) for f in face_b]
    p_out = pin(np.zeros((n, n, n)))
    v_out = [pin(np.zeros(face_shape(n, d))) for d in range(3)]
    tabs = (capi.DP * 3)(*[capi.dp(v) for v in v_out])
    ftab = (capi.DP * 3)(*[capi.dp(f) for f in fpen_p])
    btab = (capi.DP * 3)(*[capi.dp(f) for f in fb_p])
    L = capi.lib()

    def e2e_step():
        capi.check(L.stg_set_penalty(s.h, None, ftab))
        capi.check(L.stg_set_rhs(s.h, capi.dp(cb_p), btab))
        st = capi.Stats()
        capi.check(L.stg_solve(s.h, capi.dp(p_out), tabs, capi.ctypes.byref(st)))
        return st

    for _ in range(args.warmup):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    barrier()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    e2e_value = whole_job_seconds_per_solve(max_over_ranks(e2e_ms / 1e3), args.steps, world)
    h2d = sum(f.nbytes for f in fpen_p) + cb_p.nbytes + sum(f.nbytes for f in fb_p)
    d2h = p_out.nbytes + sum(v.nbytes for v in v_out)

    # ---- the other methods on the same problem, for the comparison the metric names
    methods = {"plain": {"s_per_solve": value, "v_cycles": statistics.mean(st["inner_iters"] for st in stats)}}
    if not args.no_methods:
        k = max(2, args.steps // 2)

        def leg(sv):
            ms_, st_, _, _, _ = timed_device(sv, k, 1)
            return {"s_per_solve": whole_job_seconds_per_solve(max_over_ranks(ms_ / 1e3), k, world),
                    "v_cycles": statistics.mean(x["inner_iters"] for x in st_),
                    "max_rel_residual": max(x["rel_residual"] for x in st_)}

        sv = make_solver(capi.STG_METHOD_PLAIN, smooth_sweeps=2)
        methods["plain_reference_smoother"] = leg(sv)
        sv.close()
        sv = make_solver(capi.STG_METHOD_MIXED)
        methods["mixed"] = leg(sv)
        sv.close()
        # learned: train at NET_TRAIN_N^3 on the same problem family, apply at n^3
        tr = make_solver(capi.STG_METHOD_PLAIN, nn=NET_TRAIN_N)
        tr.net_init(7)
        barrier()
        t0 = time.perf_counter()
        losses = tr.net_train(NET_TRAIN_STEPS, lr=NET_LR, seed=3)
        barrier()
        train_s = time.perf_counter() - t0
        params = tr.net_params()
        tr.close()
        sv = make_solver(capi.STG_METHOD_LEARNED)
        sv.net_init(7)
        sv.net_set_params(params)
        r = leg(sv)
        _, _, st1 = sv.solve(want=False)
        r.update({"learned_iters": st1["learned_iters"], "fallbacks": st1["fallbacks"], "train_s": round(train_s, 2),
                  "train": f"{NET_TRAIN_STEPS} Adam steps (lr {NET_LR:g}) at {NET_TRAIN_N}^3, one fresh pair per step",
                  "final_loss": round(float(np.mean(losses[-100:])), 4)})
        methods["learned"] = r
        sv.close()

    # ---- the batches of independent solves the benchmark configurations name: 100 solves at
    # 128^3 (plain) and 50 at 256^3 (mixed), each on its own seeded density (sigma 4), every
    # solve to FP64 rel. residual 1e-8; per solve: the density, filter and penalty set-up on
    # the GPU and the solve, CUDA events around the whole batch
    batches = None
    if rank == 0 and world == 1 and not args.no_methods:
        batches = {}
        for nn, count, meth, name in ((128, 100, capi.STG_METHOD_PLAIN, "solves_128_plain"),
                                      (n, 50, capi.STG_METHOD_MIXED, f"solves_{n}_mixed")):
            sv = make_solver(meth, nn=nn)
            sv.solve(want=False)
            its, rels = [], []
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for seed in range(count):
                sv.density_noise(1000 + seed, 4.0, want=False)
                sv.filter(1.5, None, want=False)
                sv.set_density(None, capi.alpha_bp(1e4))
                _, _, st_ = sv.solve(want=False)
                its.append(st_["inner_iters"])
                rels.append(st_["rel_residual"])
            e1.record(stream)
            torch.cuda.synchronize()
            ms_ = e0.elapsed_time(e1)
            batches[name] = {"workload": f"{count} independent {nn}^3 solves ({'mixed' if meth else 'plain'}), seeded "
                                         f"densities {1000}..{1000 + count - 1} (sigma 4), to FP64 rel. residual {TOL:g}",
                             "s_total": round(ms_ / 1e3, 3), "s_per_solve": round(ms_ / 1e3 / count, 5),
                             "v_cycles_mean": round(float(np.mean(its)), 2), "v_cycles_max": int(max(its)),
                             "rel_residual_max": float(max(rels))}
            sv.close()

    # ---- design loops through the fluid_topo driver: the 2D 64^2 one (uniform 0.3 start, solves
    # to 1e-10; latency-bound) and the 3D 128^3 one at fraction 0.15, 40 iterations (from
    # iteration 5 on high-contrast designs)
    loop2d = loop3d = None
    if rank == 0 and world == 1 and not args.no_methods:
        loop2d = design_loop(build.DRIVER, 2, 64, 0.3, 20)
        loop3d = design_loop(build.DRIVER, 3, 128, 0.15, 40)

    # ---- roofline of the dominant kernel class, measured over the timed region
    peak, peak_kind = measured_peak()
    dom = max((k for k in prof if prof[k]["launches"]), key=lambda k: prof[k]["ms"])
    d = prof[dom]
    achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9
    traffic = ncu_traffic().get(dom)
    # the V-cycle as a whole (every level's sweeps, the transfers and the coarsest GEMV):
    # algorithmic bytes over CUDA-event time, against the same measured peak
    vc_cls = [k for k in ("sweep32", "sweep32_coarse", "restrict32", "prolong32", "coarse") if k in prof]
    vc_ms = sum(prof[k]["ms"] for k in vc_cls)
    vc_bytes = sum(prof[k]["bytes"] for k in vc_cls)
    vcycle = {"classes": vc_cls, "ms_per_solve": round(vc_ms / PROFILED_SOLVES, 3),
              "achieved_GBps": round(vc_bytes / (vc_ms * 1e-3) / 1e9, 1) if vc_ms > 0 else None,
              "frac": round(vc_bytes / (vc_ms * 1e-3) / 1e9 / peak, 4) if vc_ms > 0 else None}
    kernel_table = {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                        "GBps": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1) if v["ms"] > 0 and v["bytes"] > 0 else None}
                    for k, v in prof.items() if v["launches"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
        cv, csample, csec = cpu_reference_sample(n)
        cpu = {"value": cv, "unit": "s/solve", "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": "port",
               "sample": csample, "sample_s": round(csec, 2)}

    vc = statistics.mean(st["inner_iters"] for st in stats)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "s/solve", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value * 1e3 * world, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 V-cycle and Krylov / f64 refinement", "data": "synthetic",
            "config": {"workload": f"3D {n}^3 Brinkman-Stokes solve to FP64 rel. residual {TOL:g}",
                       "n": n, "method": "plain (FP32 V-cycle, 1 smoother sweep per colour, FGMRES in FP64 refinement)",
                       "tol": TOL, "bc": "parabolic inlet N/4 patch, mirrored outlet",
                       "density": "seeded U[0,1], Gaussian sigma 4, filter r 1.5, BP alpha amax 1e4",
                       "l2": "inputs larger than L2 (~27 GB working set)", "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e_value, "unit": "s/solve", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes_per_launch": d["bytes"] / d["launches"]},
            "vcycle_hbm": vcycle,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "solver": {"v_cycles_per_solve": vc, "outer_per_solve": statistics.mean(st["outer_iters"] for st in stats),
                       "final_rel_residual_max": max(st["rel_residual"] for st in stats)},
            "methods": methods,
            "solve_batches": batches,
            "design_loop_2d": loop2d,
            "design_loop_3d": loop3d,
            "kernels": kernel_table,
        }
        print(json.dumps(line), flush=True)
    s.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.oracle_check:
        oracle_check(args)
    elif args.learned_config:
        learned_config(args)
    elif args.learned_warm:
        learned_warm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
