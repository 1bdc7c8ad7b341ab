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


def test_driver_fails_loudly_without_gpu(driver, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([driver, "-driver", "0", "-test", "1", "-s", "64", "-frac", "0.3", "-lf", "1", "-o", str(tmp_path)],
                       capture_output=True, text=True)
    assert r.returncode == 2 and "stokes_gb300" in r.stderr


@pytest.mark.gpu
def test_driver_2d_optimization_matches_oracle(oracle, driver, tmp_path):
    """fluid_topo -driver 0 -test 1 -s 64 -frac 0.3: uniform 0.3 start, BP law, filter
    1.5, OC move 0.2, solves to 1e-10; objective history and final design against the
    oracle's loop."""
    n, iters, frac, rmin = 64, 4, 0.3, 1.5
    out = tmp_path / "run"
    subprocess.run([driver, "-driver", "0", "-test", "1", "-s", str(n), "-frac", str(frac), "-lf", str(iters), "-o",
                    str(out)], check=True)
    log = np.genfromtxt(out / "log.csv", delimiter=",", names=True)
    x_gpu = read_field(out / str(iters) / "x", n, 2)
    # reference frame layout: grid at frame 0, last_frame.txt, velocity as cell vectors,
    # psi_N holding the 4N fixed boundary faces
    assert np.array_equal(read_field(out / "0" / "x", n, 2), np.full((n, n), frac))
    assert (out / "0" / "grid").stat().st_size == 3 * 4 + 8 + 3 * 8
    assert (out / "0" / "last_frame.txt").read_text().strip() == str(iters)
    assert (out / str(iters) / "velocity").stat().st_size == 3 * 4 + n * n * 3 * 8
    assert int(np.fromfile(out / str(iters) / "psi_N", dtype=np.int32, count=1)[0]) == 4 * n

    b = oracle.bc_parabolic(n, 2, width=n // 4)
    x = np.full((n, n), frac)
    vw = oracle.filt(np.ones((n, n)), rmin, transpose=True)
    J = []
    for it in range(iters):
        phys = oracle.filt(x, rmin)
        fp = oracle.face_penalty(phys, 1, [1e4], dim=2)
        o = oracle.Steady2D(n)
        o.init_boundary(b)
        o.update_penalty(np.zeros((n, n)), fp)
        o.update_b(b.cell_b, b.face_b)
        u_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        J.append(o.energy(u_ref))
        o.set_b_blocked(o.apply_E(u_ref))
        lam_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        _, u = oracle.blocked_to_field2(n, u_ref)
        _, lam = oracle.blocked_to_field2(n, lam_ref)
        dc = oracle.filt(oracle.sensitivity(phys, 1, [1e4], u, lam, dim=2), rmin, transpose=True)
        x, _, _ = oracle.oc_update(x, dc, vw / n ** 2, vw, frac)
        x = x.reshape(n, n)
    assert np.allclose(log["objective"], J, rtol=1e-6, atol=0)
    assert relerr(x_gpu, x) < 1e-5
