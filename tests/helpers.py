"""Shared problem builders for the parity tests (seeded, small)."""
import numpy as np


def problem(po, n, seed=1, sigma=2.0, law="bp", bc="parabolic"):
    """Boundary + penalty + rhs of a seeded Brinkman-Stokes problem in Field order."""
    b = po.bc_parabolic(n) if bc == "parabolic" else po.bc_test0_3d(n)
    rho = po.density_noise(n, seed, sigma)
    if law == "bp":
        rf = po.filt(rho, 1.5)
        fp = po.face_penalty(rf, 1, [1e4])
        phys = rf
    else:
        prm = [5e2 / (n / 32.0), 1e-3, 0.01]
        fp = po.face_penalty(rho, 0, prm)
        phys = rho
    return b, rho, phys, fp


def problem2(po, n, seed=1, sigma=2.0, law="bp", bc="parabolic"):
    """2D counterpart of problem(): parabolic inlet on a centred n/4 segment (16 cells at
    64^2) or the reference's 2D test 0, seeded density, BP or reference alpha law."""
    b = po.bc_parabolic(n, 2, width=n // 4) if bc == "parabolic" else po.bc_test0_2d(n)
    rho = po.density_noise(n, seed, sigma, dim=2)
    if law == "bp":
        rf = po.filt(rho, 1.5)
        fp = po.face_penalty(rf, 1, [1e4], dim=2)
        phys = rf
    else:
        prm = [5e2 / (n / 32.0), 1e-3, 0.014]
        fp = po.face_penalty(rho, 0, prm, dim=2)
        phys = rho
    return b, rho, phys, fp


def relerr(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    d = np.linalg.norm(a - b)
    s = np.linalg.norm(b)
    return d / s if s > 0 else d


def pressure_free(p):
    """Pressure modulo a constant (the closed-domain null space)."""
    return p - p.mean()


def stable_vec(seed, n):
    """n values in [-1, 1) from SplitMix64 over (seed, index): a generator whose stream
    never changes, so fixtures can store the seed instead of the vector."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + np.arange(n, dtype=np.uint64) + np.uint64(
            0x632BE59BD9B4E019)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0
