"""The fluid_topo command-line driver (stokes_to_gb300/host): its boundary builders
against the oracle's restatement of the reference drivers (CPU), its refusal to run
without a GPU (CPU), and a short 2D optimization against the oracle's design loop (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from tests.helpers import relerr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "stokes_to_gb300", "fluid_topo")


@pytest.fixture(scope="module")
def driver(stg):
    assert os.path.exists(DRIVER), "fluid_topo was not built"
    return DRIVER


def read_field(path, n, dim):
    """A scalar Field<double,3> file of the reference frame format: int32 counts[3] + values."""
    raw = open(path, "rb").read()
    counts = np.frombuffer(raw[:12], dtype=np.int32)
    assert tuple(counts) == (n, n, n if dim == 3 else 1)
    return np.frombuffer(raw[12:], dtype=np.float64).reshape((n,) * dim)


def _dump(driver, tmp_path, dim, test, n):
    out = tmp_path / f"b{dim}_{test}_{n}"
    subprocess.run([driver, "-driver", "0" if dim == 2 else "1", "-test", str(test), "-s", str(n), "-frac", "0.3",
                    "-dump_boundary", str(out)], check=True)
    f64 = np.fromfile(out / "boundary_f64.bin", dtype=np.float64)
    i32 = np.fromfile(out / "boundary_i32.bin", dtype=np.int32)
    nc = n ** dim
    nf = n ** (dim - 1) * (n + 1)
    cv, cb = f64[:nc], f64[nc:2 * nc]
    fv = [f64[2 * nc + q * nf: 2 * nc + (q + 1) * nf] for q in range(dim)]
    fb = [f64[2 * nc + (dim + q) * nf: 2 * nc + (dim + q + 1) * nf] for q in range(dim)]
    cf = i32[:nc]
    ff = [i32[nc + q * nf: nc + (q + 1) * nf] for q in range(dim)]
    return cv, cb, cf, fv, fb, ff


@pytest.mark.parametrize("dim,test,n", [(2, 0, 64), (2, 1, 64), (3, 0, 64), (3, 1, 32)])
def test_driver_boundaries_match_oracle(oracle, driver, tmp_path, dim, test, n):
    cv, cb, cf, fv, fb, ff = _dump(driver, tmp_path, dim, test, n)
    if test == 0:
        b = oracle.bc_test0_2d(n) if dim == 2 else oracle.bc_test0_3d(n)
    else:
        b = oracle.bc_parabolic(n, dim, width=n // 4)
    assert np.array_equal(cv, b.cell_vol.ravel()) and np.array_equal(cb, b.cell_b.ravel())
    assert np.array_equal(cf, b.cell_fixed.ravel())
    for q in range(dim):
        assert np.array_equal(fv[q], b.face_vol[q].ravel())
        assert np.array_equal(fb[q], b.face_b[q].ravel())
        assert np.array_equal(ff[q], b.face_fixed[q].ravel())


def test_driver_rejects_bad_flags(driver, tmp_path):
    r = subprocess.run([driver, "-driver", "0", "-s", "64", "-lf", "1", "-o", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 2 and "-frac" in r.stderr
    r = subprocess.run([driver, "-bogus", "1"], capture_output=True, text=True)
    assert r.returncode == 2 and "unknown flag" in r.stderr
    # the solver flags are known (parsed before the boundary dump, which needs no GPU)
    out = tmp_path / "dump"
    r = subprocess.run([driver, "-driver", "1", "-test", "1", "-s", "16", "-frac", "0.15", "-inner", "24", "-maxouter", "40",
                        "-warm", "0", "-dump_boundary", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_driver_fails_loudly_without_gpu(driver, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([driver, "-driver", "0", "-test", "1", "-s", "64", "-frac", "0.3", "-lf", "1", "-o", str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "stokes_gb300" in r.stderr


def _oracle_loop(oracle, b, n, iters, frac, update, law, prm, rmin):
    """The design loop on the oracle: per iteration the objective at design k, the
    adjoint sensitivity, then the design update; returns objectives and designs."""
    x = np.full((n, n), frac)
    Js, xs = [], []
    for it in range(iters):
        xs.append(x.copy())
        phys = oracle.filt(x, rmin) if rmin > 1 else x
        fp = oracle.face_penalty(phys, law, prm, dim=2)
        o = oracle.Steady2D(n)
        o.init_boundary(b)
        o.update_penalty(np.zeros((n, n)), fp)
        o.update_b(b.cell_b, b.face_b)
        u_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        Js.append(o.energy(u_ref))
        o.set_b_blocked(o.apply_E(u_ref))
        lam_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        _, u = oracle.blocked_to_field2(n, u_ref)
        _, lam = oracle.blocked_to_field2(n, lam_ref)
        sens = oracle.sensitivity(phys, law, prm, u, lam, dim=2)
        dc = oracle.filt(sens, rmin, transpose=True) if rmin > 1 else sens
        x = update(x, dc)
    return np.array(Js), xs


@pytest.mark.gpu
def test_driver_2d_optimization_matches_oracle(oracle, driver, tmp_path):
    """fluid_topo -driver 0 -test 1 -s 64 -frac 0.3 (OC): uniform 0.3 start, BP law,
    filter 1.5, move 0.2, solves to 1e-10; objective history and designs against the
    oracle's loop, plus the reference frame layout."""
    n, iters, frac, rmin = 64, 4, 0.3, 1.5
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "0", "-test", "1", "-s", str(n), "-frac", str(frac), "-lf", str(iters), "-o",
                    str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    b = oracle.bc_parabolic(n, 2, width=n // 4)
    vw = oracle.filt(np.ones((n, n)), rmin, transpose=True)

    def oc(x, dc):
        return oracle.oc_update(x, dc, vw / n ** 2, vw, frac)[0].reshape(n, n)

    J, xs = _oracle_loop(oracle, b, n, iters, frac, oc, 1, [1e4], rmin)
    assert np.allclose(log["objective"], J, rtol=1e-6, atol=0)
    for k in range(iters):
        assert relerr(read_field(out / str(k) / "x", n, 2), xs[k]) < 1e-5, k
    # reference frame layout: grid at frame 0, last_frame.txt, velocity as cell vectors,
    # psi_N holding the 4N fixed boundary faces
    assert (out / "0" / "grid").stat().st_size == 3 * 4 + 8 + 3 * 8
    assert (out / "0" / "last_frame.txt").read_text().strip() == str(iters - 1)
    assert (out / "1" / "velocity").stat().st_size == 3 * 4 + n * n * 3 * 8
    assert int(np.fromfile(out / "1" / "psi_N", dtype=np.int32, count=1)[0]) == 4 * n


@pytest.mark.gpu
def test_driver_2d_reference_test0_mma_matches_oracle(oracle, driver, tmp_path):
    """fluid_topo -driver 0 -test 0 -s 64 -frac 0.3: the reference's own configuration
    (test 0 boundary, reference alpha law on rho^3, unfiltered design, MMA with the
    reference settings) against the oracle's loop with the oracle MMA (which is pinned to
    the reference MMA solver)."""
    n, iters, frac = 64, 3, 0.3
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "0", "-test", "0", "-s", str(n), "-frac", str(frac), "-lf", str(iters), "-o",
                    str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    b = oracle.bc_test0_2d(n)
    prm = [5e2 / (n / 32.0), 1e-3, 0.014]
    mma = oracle.Mma(n * n)

    def mma_step(x, dc):
        x = np.ascontiguousarray(x, dtype=np.float64).ravel().copy()
        g = 1e4 * (x.mean() - frac)
        mma.update(x, dc, g, np.full(x.size, 1e4 / x.size), np.maximum(0.01, x - 0.2), np.minimum(1.0, x + 0.2))
        return x.reshape(n, n)

    J, xs = _oracle_loop(oracle, b, n, iters, frac, mma_step, 0, prm, 0.0)
    assert np.allclose(log["objective"], J, rtol=1e-6, atol=0)
    for k in range(iters):
        assert relerr(read_field(out / str(k) / "x", n, 2), xs[k]) < 1e-6, k


@pytest.mark.gpu
def test_driver_2d_benchmark_loop_matches_oracle_fixture(driver, tmp_path):
    """The 2D 64^2 benchmark case end to end: fluid_topo -driver 0 -test 1 -s 64 -frac 0.3
    -lf 20 (parabolic inlet, OC, filter 1.5, every solve to 1e-10) against the oracle's
    20-iteration loop (tests/golden/oracle_loop2d_n64.npz): objective at every iteration
    within 1e-6, the last iteration's design within 1e-4. From iteration 4 on the designs
    are high-contrast (density down to 1e-8): the V-cycle is a weak preconditioner there
    and solves take hundreds of V-cycles over several refinement steps."""
    n, iters = 64, 20
    g = np.load(os.path.join(ROOT, "tests", "golden", "oracle_loop2d_n64.npz"))
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "0", "-test", "1", "-s", str(n), "-frac", "0.3", "-lf", str(iters), "-frames",
                    str(iters - 1), "-o", str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    assert np.allclose(log["objective"], g["objective"], rtol=1e-6, atol=0)
    assert relerr(read_field(out / str(iters - 1) / "x", n, 2), g["x_last"]) < 1e-4


@pytest.mark.gpu
def test_driver_3d_loop_matches_oracle_fixture(driver, tmp_path):
    """The 3D design loop end to end at 32^3: fluid_topo -driver 1 -test 1 -s 32 -frac 0.15
    -lf 8 (parabolic inlet, OC, filter 1.5, every solve to 1e-10) against the oracle's
    8-iteration loop (tests/golden/oracle_loop3d_n32.npz): objective at every iteration
    within 1e-6, the last iteration's design within 1e-4. Iterations 5-7 run on
    high-contrast designs (density down to 1e-8)."""
    n, iters = 32, 8
    g = np.load(os.path.join(ROOT, "tests", "golden", "oracle_loop3d_n32.npz"))
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "1", "-test", "1", "-s", str(n), "-frac", "0.15", "-lf", str(iters), "-tol", "1e-10",
                    "-frames", str(iters - 1), "-o", str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    assert np.all(log["rel_residual_forward"] <= 1e-10) and np.all(log["rel_residual_adjoint"] <= 1e-10)
    assert np.allclose(log["objective"], g["objective"], rtol=1e-6, atol=0)
    assert relerr(read_field(out / str(iters - 1) / "x", n, 3), g["x_last"]) < 1e-4


@pytest.mark.gpu
def test_driver_3d_high_contrast_solves_converge(driver, tmp_path):
    """64^3 loop at fraction 0.15 through iteration 11: from iteration 5 the designs are
    channels with density 1 in solid 1e-8 .. 1e-30 (penalty contrast 1e4). With the
    reference's coarse penalties (sums over the children) the restarted solve stagnated
    there (relative residual 0.21 after 20 x 30 V-cycles at iteration 5); the solver's flow
    rule keeps every solve converged to 1e-8 in well under the cap."""
    n, iters = 64, 12
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "1", "-test", "1", "-s", str(n), "-frac", "0.15", "-lf", str(iters), "-frames", "0",
                    "-o", str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    assert len(log) == iters
    assert np.all(np.diff(log["objective"]) < 0), log["objective"]
    assert np.all(log["rel_residual_forward"] <= 1e-8) and np.all(log["rel_residual_adjoint"] <= 1e-8)
    # the refinement cap is 20 x 30 = 600 V-cycles
    assert np.max(log["v_cycles_forward"]) <= 150, log["v_cycles_forward"]
    assert np.max(log["v_cycles_adjoint"]) <= 150, log["v_cycles_adjoint"]
