"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
import this module; the product library never does.  Arrays use the simplex Field
order (cell (i,j,k) -> (i*N + j)*N + k, face axis d with N+1 entries along d).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

D = ctypes.c_double
I = ctypes.c_int
P = ctypes.c_void_p
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int)
U8P = ctypes.POINTER(ctypes.c_uint8)


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc3_create.restype = P
        L.orc3_create.argtypes = [I]
        L.orc3_destroy.argtypes = [P]
        L.orc3_dof.restype = I
        L.orc3_levels.restype = I
        L.orc3_level_n.restype = I
        L.orc3_index.restype = I
        L.orc3_index.argtypes = [I, I, I, I, I, I, IP]
        L.orc3_level_dof.restype = I
        L.orc3_level_dof.argtypes = [P, I]
        L.orc3_solve.restype = I
        L.orc3_solve.argtypes = [P, I, D, D, D, I, D, DP, DP]
        L.orc3_energy.restype = D
        L.orc3_energy.argtypes = [P, DP]
        L.orc3_coarse_info.restype = I
        L.orc3_coarse_info.argtypes = [P]
        for name in ["orc3_init_boundary", "orc3_update_penalty", "orc3_update_b", "orc3_set_b_blocked", "orc3_setup",
                     "orc3_setup_flow", "orc3_setup_as_run",
                     "orc3_apply_A", "orc3_apply_E", "orc3_level_descr", "orc3_update_subsystems", "orc3_restrict",
                     "orc3_prolong", "orc3_vanka_apply", "orc3_smooth", "orc3_coarse_apply", "orc3_vcycle"]:
            getattr(L, name).restype = None
        L.orc3_init_boundary.argtypes = [P, DP, IP, DP, DP, DP, IP, IP, IP, I]
        L.orc3_update_penalty.argtypes = [P, DP, DP, DP, DP]
        L.orc3_update_b.argtypes = [P, DP, DP, DP, DP]
        L.orc3_set_b_blocked.argtypes = [P, DP]
        L.orc3_setup.argtypes = [P]
        L.orc3_setup_flow.argtypes = [P]
        L.orc3_setup_as_run.argtypes = [P]
        L.orc3_apply_A.argtypes = [P, I, DP, DP]
        L.orc3_apply_E.argtypes = [P, DP, DP]
        L.orc3_level_descr.argtypes = [P, I, DP, DP, U8P]
        L.orc3_update_subsystems.argtypes = [P]
        L.orc3_restrict.argtypes = [P, I, DP, DP]
        L.orc3_prolong.argtypes = [P, I, DP, DP]
        L.orc3_vanka_apply.argtypes = [P, I, I, DP, DP]
        L.orc3_smooth.argtypes = [P, I, I, DP, DP]
        L.orc3_coarse_apply.argtypes = [P, DP, DP]
        L.orc3_vcycle.argtypes = [P, DP, DP]
        L.orc3_field_to_blocked.argtypes = [I, DP, DP, DP, DP, DP]
        L.orc3_blocked_to_field.argtypes = [I, DP, DP, DP, DP, DP]
        L.orc_uniform.restype = D
        L.orc_uniform.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_face_penalty.argtypes = [I, I, DP, I, DP, DP, DP, DP]
        L.orc_sensitivity.argtypes = [I, I, DP, I, DP, ctypes.POINTER(DP), ctypes.POINTER(DP), DP]
        L.orc_filter.argtypes = [I, I, D, DP, DP, I]
        L.orc_oc_update.restype = I
        L.orc_oc_update.argtypes = [I, DP, DP, DP, DP, D, D, D, D, D, I, DP, DP]
        L.orc_density_noise.argtypes = [I, I, ctypes.c_uint64, D, DP]
        L.orc_bc_parabolic.argtypes = [I, I, I, DP, IP, DP, DP, DP, DP, IP, IP, IP, DP, DP, DP]
        L.orc_bc_test0_3d.argtypes = [I, DP, IP, DP, DP, DP, DP, IP, IP, IP, DP, DP, DP]
        L.orc_mma_create.restype = P
        L.orc_mma_create.argtypes = [I]
        L.orc_mma_destroy.argtypes = [P]
        L.orc_mma_update.restype = D
        L.orc_mma_update.argtypes = [P, DP, DP, D, DP, DP, DP]
        _LIB = L
    return _LIB


def dp(a):
    return None if a is None else a.ctypes.data_as(DP)


def ip(a):
    return None if a is None else a.ctypes.data_as(IP)


def face_shape(n, d, dim=3):
    s = [n] * dim
    s[d] += 1
    return tuple(s)


# ------------------------------------------------------------------ layout helpers
def dof(n):
    return lib().orc3_dof(n)


def levels(n):
    return lib().orc3_levels(n)


def field_to_blocked(n, cell, faces):
    out = np.zeros(dof(n))
    f = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None for x in faces]
    c = np.ascontiguousarray(cell, dtype=np.float64) if cell is not None else None
    lib().orc3_field_to_blocked(n, dp(c), dp(f[0]), dp(f[1]), dp(f[2]), dp(out))
    return out


def blocked_to_field(n, v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    cell = np.zeros((n, n, n))
    faces = [np.zeros(face_shape(n, d)) for d in range(3)]
    lib().orc3_blocked_to_field(n, dp(v), dp(cell), dp(faces[0]), dp(faces[1]), dp(faces[2]))
    return cell, faces


# ------------------------------------------------------------------ boundary and design helpers
class Boundary:
    """Boundary description in Field order (FluidTopoOptDriver3D::init_boundary outputs)."""

    def __init__(self, n, dim=3):
        self.n, self.dim = n, dim
        cs = (n,) * dim
        self.cell_vol = np.zeros(cs)
        self.cell_fixed = np.zeros(cs, dtype=np.int32)
        self.cell_b = np.zeros(cs)
        self.face_vol = [np.zeros(face_shape(n, d, dim)) for d in range(dim)]
        self.face_fixed = [np.zeros(face_shape(n, d, dim), dtype=np.int32) for d in range(dim)]
        self.face_b = [np.zeros(face_shape(n, d, dim)) for d in range(dim)]
        self.closed = True


def _pad3(lst):
    return list(lst) + [None] * (3 - len(lst))


def bc_parabolic(n, dim=3, width=None):
    b = Boundary(n, dim)
    w = width if width is not None else n // 4
    fv, ff, fb = _pad3(b.face_vol), _pad3(b.face_fixed), _pad3(b.face_b)
    lib().orc_bc_parabolic(dim, n, w, dp(b.cell_vol), ip(b.cell_fixed), dp(b.cell_b), dp(fv[0]), dp(fv[1]), dp(fv[2]),
                           ip(ff[0]), ip(ff[1]), ip(ff[2]), dp(fb[0]), dp(fb[1]), dp(fb[2]))
    return b


def bc_test0_3d(n):
    b = Boundary(n, 3)
    lib().orc_bc_test0_3d(n, dp(b.cell_vol), ip(b.cell_fixed), dp(b.cell_b), dp(b.face_vol[0]), dp(b.face_vol[1]),
                          dp(b.face_vol[2]), ip(b.face_fixed[0]), ip(b.face_fixed[1]), ip(b.face_fixed[2]),
                          dp(b.face_b[0]), dp(b.face_b[1]), dp(b.face_b[2]))
    return b


def face_penalty(rho, law, params, dim=3):
    n = rho.shape[0]
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    f = [np.zeros(face_shape(n, d, dim)) for d in range(dim)]
    f3 = _pad3(f)
    prm = np.ascontiguousarray(params, dtype=np.float64)
    lib().orc_face_penalty(dim, n, dp(rho), law, dp(prm), dp(f3[0]), dp(f3[1]), dp(f3[2]))
    return f


def sensitivity(rho, law, params, u, lam, dim=3):
    n = rho.shape[0]
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    prm = np.ascontiguousarray(params, dtype=np.float64)
    uu = [np.ascontiguousarray(x, dtype=np.float64) for x in u] + [np.zeros(1)] * (3 - dim)
    ll = [np.ascontiguousarray(x, dtype=np.float64) for x in lam] + [np.zeros(1)] * (3 - dim)
    ua = (DP * 3)(*[dp(x) for x in uu])
    la = (DP * 3)(*[dp(x) for x in ll])
    g = np.zeros_like(rho)
    lib().orc_sensitivity(dim, n, dp(rho), law, dp(prm), ua, la, dp(g))
    return g


def filt(rho, rmin, transpose=False):
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    out = np.zeros_like(rho)
    lib().orc_filter(rho.ndim, rho.shape[0], rmin, dp(rho), dp(out), 1 if transpose else 0)
    return out


def oc_update(x, dc, dv, vw, frac, move=0.2, lo=0.0, hi=1.0, tol=1e-9, max_steps=200):
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    xn = np.zeros_like(x)
    lam = np.zeros(1)
    steps = lib().orc_oc_update(x.size, dp(x), dp(np.ascontiguousarray(dc, dtype=np.float64).ravel()),
                                dp(np.ascontiguousarray(dv, dtype=np.float64).ravel()),
                                dp(np.ascontiguousarray(vw, dtype=np.float64).ravel()), frac, move, lo, hi, tol,
                                max_steps, dp(xn), dp(lam))
    return xn, float(lam[0]), steps


def density_noise(n, seed, sigma, dim=3):
    out = np.zeros((n,) * dim)
    lib().orc_density_noise(dim, n, seed, sigma, dp(out))
    return out


# ------------------------------------------------------------------ 3D solver handle
class Steady3D:
    """Mirror of FluidSteadyState3D (+ FluidEnergy3D) on the CPU oracle."""

    def __init__(self, n):
        self.n = n
        self.L = lib()
        self.h = self.L.orc3_create(n)
        self.levels = levels(n)

    def close(self):
        if self.h:
            self.L.orc3_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def level_dof(self, level):
        return self.L.orc3_level_dof(self.h, level)

    def init_boundary(self, b):
        ff = [np.ascontiguousarray(x, dtype=np.int32) for x in b.face_fixed]
        fv = [np.ascontiguousarray(x, dtype=np.float64) for x in b.face_vol]
        self.L.orc3_init_boundary(self.h, dp(np.ascontiguousarray(b.cell_vol, dtype=np.float64)),
                                  ip(np.ascontiguousarray(b.cell_fixed, dtype=np.int32)), dp(fv[0]), dp(fv[1]),
                                  dp(fv[2]), ip(ff[0]), ip(ff[1]), ip(ff[2]), 1 if b.closed else 0)

    def update_penalty(self, cell_pen, face_pen):
        fp = [np.ascontiguousarray(x, dtype=np.float64) for x in face_pen]
        self.L.orc3_update_penalty(self.h, dp(np.ascontiguousarray(cell_pen, dtype=np.float64)), dp(fp[0]),
                                   dp(fp[1]), dp(fp[2]))

    def update_b(self, cell_b, face_b):
        fb = [np.ascontiguousarray(x, dtype=np.float64) for x in face_b]
        self.L.orc3_update_b(self.h, dp(np.ascontiguousarray(cell_b, dtype=np.float64)), dp(fb[0]), dp(fb[1]),
                             dp(fb[2]))

    def set_b_blocked(self, b):
        self.L.orc3_set_b_blocked(self.h, dp(np.ascontiguousarray(b, dtype=np.float64)))

    def setup(self, flow=False, as_run=False):
        """The hierarchy set-up; flow=True builds the GPU solver's coarse penalties (8 x the
        smallest free child) instead of the reference's sums; as_run=True builds the Vanka
        blocks as the reference's block packing leaves them (oracle3d.cpp vanka_setup)."""
        if as_run:
            self.L.orc3_setup_as_run(self.h)
        else:
            (self.L.orc3_setup_flow if flow else self.L.orc3_setup)(self.h)

    def solve(self, max_iter=50, abs_thr=1e-3, rel_thr=1e-4, norm_thr=1e-3, restarts=0, true_tol=0.0):
        x = np.zeros(self.level_dof(self.levels - 1))
        st = np.zeros(6)
        self.L.orc3_solve(self.h, max_iter, abs_thr, rel_thr, norm_thr, restarts, true_tol, dp(x), dp(st))
        return x, dict(iters=int(st[0]), restarts=int(st[1]), rel_true=st[2], abs_true=st[3], precond_res=st[4],
                       seconds=st[5])

    def _vec_op(self, fn, level_in, level_out, x, *extra):
        y = np.zeros(self.level_dof(level_out))
        x = np.ascontiguousarray(x, dtype=np.float64)
        fn(self.h, *extra, dp(x), dp(y))
        return y

    def apply_A(self, x, level=None):
        level = self.levels - 1 if level is None else level
        return self._vec_op(self.L.orc3_apply_A, level, level, x, level)

    def apply_E(self, x):
        return self._vec_op(self.L.orc3_apply_E, self.levels - 1, self.levels - 1, x)

    def energy(self, x):
        return self.L.orc3_energy(self.h, dp(np.ascontiguousarray(x, dtype=np.float64)))

    def descr(self, level):
        s = self.level_dof(level)
        vol, pen, fx = np.zeros(s), np.zeros(s), np.zeros(s, dtype=np.uint8)
        self.L.orc3_level_descr(self.h, level, dp(vol), dp(pen), fx.ctypes.data_as(U8P))
        return vol, pen, fx

    def update_subsystems(self):
        self.L.orc3_update_subsystems(self.h)

    def restrict(self, coarse_level, rf):
        return self._vec_op(self.L.orc3_restrict, coarse_level + 1, coarse_level, rf, coarse_level)

    def prolong(self, coarse_level, xc):
        return self._vec_op(self.L.orc3_prolong, coarse_level, coarse_level + 1, xc, coarse_level)

    def vanka_apply(self, level, flag, r):
        return self._vec_op(self.L.orc3_vanka_apply, level, level, r, level, flag)

    def smooth(self, level, post, r):
        return self._vec_op(self.L.orc3_smooth, level, level, r, level, post)

    def coarse_apply(self, r):
        return self._vec_op(self.L.orc3_coarse_apply, 0, 0, r)

    def coarse_info(self):
        return self.L.orc3_coarse_info(self.h)

    def vcycle(self, r):
        return self._vec_op(self.L.orc3_vcycle, self.levels - 1, self.levels - 1, r)


# ------------------------------------------------------------------ 2D solver handle
_L2 = {}


def _lib2():
    L = lib()
    if "init" not in _L2:
        L.orc2_create.restype = P
        L.orc2_create.argtypes = [I]
        L.orc2_destroy.argtypes = [P]
        L.orc2_dof.restype = I
        L.orc2_levels.restype = I
        L.orc2_index.restype = I
        L.orc2_index.argtypes = [I, I, I, I, I]
        L.orc2_level_dof.restype = I
        L.orc2_level_dof.argtypes = [P, I]
        L.orc2_solve.restype = I
        L.orc2_solve.argtypes = [P, I, D, D, D, I, D, DP, DP]
        L.orc2_energy.restype = D
        L.orc2_energy.argtypes = [P, DP]
        L.orc2_coarse_info.restype = I
        L.orc2_coarse_info.argtypes = [P]
        for name in ["orc2_init_boundary", "orc2_update_penalty", "orc2_set_flow", "orc2_update_b", "orc2_set_b_blocked",
                     "orc2_apply_A",
                     "orc2_apply_E", "orc2_level_descr", "orc2_restrict", "orc2_prolong", "orc2_smooth_colour",
                     "orc2_smooth", "orc2_coarse_apply", "orc2_vcycle", "orc2_field_to_blocked", "orc2_blocked_to_field",
                     "orc_bc_test0_2d"]:
            getattr(L, name).restype = None
        L.orc2_init_boundary.argtypes = [P, DP, IP, DP, DP, IP, IP, I]
        L.orc2_update_penalty.argtypes = [P, DP, DP, DP]
        L.orc2_set_flow.argtypes = [P, I]
        L.orc2_update_b.argtypes = [P, DP, DP, DP]
        L.orc2_set_b_blocked.argtypes = [P, DP]
        L.orc2_apply_A.argtypes = [P, I, DP, DP]
        L.orc2_apply_E.argtypes = [P, DP, DP]
        L.orc2_level_descr.argtypes = [P, I, DP, DP, U8P, DP]
        L.orc2_restrict.argtypes = [P, I, DP, DP]
        L.orc2_prolong.argtypes = [P, I, DP, DP]
        L.orc2_smooth_colour.argtypes = [P, I, I, DP, DP]
        L.orc2_smooth.argtypes = [P, I, I, DP, DP]
        L.orc2_coarse_apply.argtypes = [P, DP, DP]
        L.orc2_vcycle.argtypes = [P, DP, DP]
        L.orc2_field_to_blocked.argtypes = [I, DP, DP, DP, DP]
        L.orc2_blocked_to_field.argtypes = [I, DP, DP, DP, DP]
        L.orc_bc_test0_2d.argtypes = [I, DP, IP, DP, DP, DP, IP, IP, DP, DP]
        _L2["init"] = True
    return L


def dof2(n):
    return _lib2().orc2_dof(n)


def field_to_blocked2(n, cell, faces):
    out = np.zeros(dof2(n))
    f = [np.ascontiguousarray(x, dtype=np.float64) for x in faces]
    c = np.ascontiguousarray(cell, dtype=np.float64) if cell is not None else None
    _lib2().orc2_field_to_blocked(n, dp(c), dp(f[0]), dp(f[1]), dp(out))
    return out


def blocked_to_field2(n, v):
    v = np.ascontiguousarray(v, dtype=np.float64)
    cell = np.zeros((n, n))
    faces = [np.zeros(face_shape(n, d, 2)) for d in range(2)]
    _lib2().orc2_blocked_to_field(n, dp(v), dp(cell), dp(faces[0]), dp(faces[1]))
    return cell, faces


def bc_test0_2d(n):
    b = Boundary(n, 2)
    _lib2().orc_bc_test0_2d(n, dp(b.cell_vol), ip(b.cell_fixed), dp(b.cell_b), dp(b.face_vol[0]), dp(b.face_vol[1]),
                            ip(b.face_fixed[0]), ip(b.face_fixed[1]), dp(b.face_b[0]), dp(b.face_b[1]))
    return b


class Steady2D:
    """Mirror of FluidSteadyState (2D) + FluidEnergy on the CPU oracle."""

    def __init__(self, n):
        self.n = n
        self.L = _lib2()
        self.h = self.L.orc2_create(n)
        self.levels = self.L.orc2_levels(n)

    def close(self):
        if self.h:
            self.L.orc2_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def level_dof(self, level):
        return self.L.orc2_level_dof(self.h, level)

    def init_boundary(self, b):
        ff = [np.ascontiguousarray(x, dtype=np.int32) for x in b.face_fixed]
        fv = [np.ascontiguousarray(x, dtype=np.float64) for x in b.face_vol]
        self.L.orc2_init_boundary(self.h, dp(np.ascontiguousarray(b.cell_vol, dtype=np.float64)),
                                  ip(np.ascontiguousarray(b.cell_fixed, dtype=np.int32)), dp(fv[0]), dp(fv[1]), ip(ff[0]),
                                  ip(ff[1]), 1 if b.closed else 0)

    def update_penalty(self, cell_pen, face_pen, flow=False):
        """The penalty with the coarse levels and coarsest matrix; flow=True builds the GPU
        solver's coarse penalties (4 x the smallest child) instead of the reference's sums."""
        fp = [np.ascontiguousarray(x, dtype=np.float64) for x in face_pen]
        self.L.orc2_set_flow(self.h, 1 if flow else 0)
        self.L.orc2_update_penalty(self.h, dp(np.ascontiguousarray(cell_pen, dtype=np.float64)), dp(fp[0]), dp(fp[1]))

    def update_b(self, cell_b, face_b):
        fb = [np.ascontiguousarray(x, dtype=np.float64) for x in face_b]
        self.L.orc2_update_b(self.h, dp(np.ascontiguousarray(cell_b, dtype=np.float64)), dp(fb[0]), dp(fb[1]))

    def set_b_blocked(self, b):
        self.L.orc2_set_b_blocked(self.h, dp(np.ascontiguousarray(b, dtype=np.float64)))

    def solve(self, max_iter=40, abs_thr=1e-3, rel_thr=1e-4, norm_thr=1e-3, restarts=0, true_tol=0.0):
        x = np.zeros(self.level_dof(self.levels - 1))
        st = np.zeros(6)
        self.L.orc2_solve(self.h, max_iter, abs_thr, rel_thr, norm_thr, restarts, true_tol, dp(x), dp(st))
        return x, dict(iters=int(st[0]), restarts=int(st[1]), rel_true=st[2], abs_true=st[3], precond_res=st[4])

    def _op(self, fn, nout, x, *extra):
        y = np.zeros(nout)
        fn(self.h, *extra, dp(np.ascontiguousarray(x, dtype=np.float64)), dp(y))
        return y

    def apply_A(self, x, level=None):
        level = self.levels - 1 if level is None else level
        return self._op(self.L.orc2_apply_A, self.level_dof(level), x, level)

    def apply_E(self, x):
        return self._op(self.L.orc2_apply_E, self.level_dof(self.levels - 1), x)

    def energy(self, x):
        return self.L.orc2_energy(self.h, dp(np.ascontiguousarray(x, dtype=np.float64)))

    def descr(self, level):
        s = self.level_dof(level)
        vol, pen, fx, lap = np.zeros(s), np.zeros(s), np.zeros(s, dtype=np.uint8), np.zeros(1)
        self.L.orc2_level_descr(self.h, level, dp(vol), dp(pen), fx.ctypes.data_as(U8P), dp(lap))
        return vol, pen, fx, float(lap[0])

    def restrict(self, coarse_level, rf):
        return self._op(self.L.orc2_restrict, self.level_dof(coarse_level), rf, coarse_level)

    def prolong(self, coarse_level, xc):
        return self._op(self.L.orc2_prolong, self.level_dof(coarse_level + 1), xc, coarse_level)

    def smooth_colour(self, level, flag, r):
        return self._op(self.L.orc2_smooth_colour, self.level_dof(level), r, level, flag)

    def smooth(self, level, post, r):
        return self._op(self.L.orc2_smooth, self.level_dof(level), r, level, post)

    def coarse_apply(self, r):
        return self._op(self.L.orc2_coarse_apply, self.level_dof(0), r)

    def coarse_info(self):
        return self.L.orc2_coarse_info(self.h)

    def vcycle(self, r):
        return self._op(self.L.orc2_vcycle, self.level_dof(self.levels - 1), r)


# ------------------------------------------------------------------ MMA (one constraint)
class Mma:
    """The oracle's MMA restatement (oracle/mma_oracle.cpp): update(x, dfdx, g, dgdx,
    xmin, xmax) replaces x in place by the next design and returns the dual variable."""

    def __init__(self, n):
        self.n = n
        self.L = lib()
        self.h = self.L.orc_mma_create(n)

    def close(self):
        if self.h:
            self.L.orc_mma_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def update(self, x, dfdx, g, dgdx, xmin, xmax):
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()
        assert x.dtype == np.float64 and x.flags["C_CONTIGUOUS"]
        d, dg, lo, hi = c(dfdx), c(dgdx), c(xmin), c(xmax)
        return self.L.orc_mma_update(self.h, dp(x), dp(d), float(g), dp(dg), dp(lo), dp(hi))


class RefMma:
    """The reference's own MMASolver (simplex/ext/mma), built from the reference sources by
    oracle/ref_build.sh into oracle/_ref (only where those sources are present)."""

    def __init__(self, n, m=1):
        path = os.path.join(_HERE, "_ref", "libref_mma.so")
        self.L = ctypes.CDLL(path)
        self.L.ref_mma_create.restype = P
        self.L.ref_mma_create.argtypes = [I, I]
        self.L.ref_mma_destroy.argtypes = [P]
        self.L.ref_mma_update.argtypes = [P, DP, DP, DP, DP, DP, DP]
        self.h = self.L.ref_mma_create(n, m)

    def close(self):
        if self.h:
            self.L.ref_mma_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def update(self, x, dfdx, g, dgdx, xmin, xmax):
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64).ravel()
        assert x.dtype == np.float64 and x.flags["C_CONTIGUOUS"]
        d, gg, dg, lo, hi = c(dfdx), np.array([g], dtype=np.float64), c(dgdx), c(xmin), c(xmax)
        self.L.ref_mma_update(self.h, dp(x), dp(d), dp(gg), dp(dg), dp(lo), dp(hi))
