"""ctypes binding of libstokes_gb300.so (include/stokes_gb300.h).

This is the Python-side stub of the C ABI, used by the tests and by bench.py. It loads
the in-tree library and fails loudly when it is missing: there is no fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstokes_gb300.so")

STG_OK = 0
STG_E_INVALID = -1
STG_E_CUDA = -2
STG_E_NOMEM = -3
STG_E_UNSUPPORTED = -4
STG_E_NOT_CONVERGED = -5
STG_E_NONFINITE = -6

STG_METHOD_PLAIN = 0
STG_METHOD_MIXED = 1
STG_METHOD_LEARNED = 2
STG_ALPHA_REF = 0
STG_ALPHA_BP = 1

STG_OP_RESTRICT = 1
STG_OP_PROLONG = 2
STG_OP_SMOOTH_PRE = 3
STG_OP_SMOOTH_POST = 4
STG_OP_VANKA_RED = 5
STG_OP_VANKA_BLACK = 6
STG_OP_COARSE = 7

# every symbol include/stokes_gb300.h declares
EXPORTS = [
    "stg_default_opts", "stg_last_error", "stg_version", "stg_create", "stg_destroy", "stg_levels", "stg_level_n",
    "stg_level_dof", "stg_set_boundary", "stg_set_penalty", "stg_set_rhs", "stg_solve", "stg_get_solution", "stg_energy",
    "stg_energy_grad_x", "stg_energy_grad_q", "stg_set_density", "stg_adjoint_sensitivity", "stg_filter", "stg_oc_update",
    "stg_apply_A_device", "stg_apply_E_device", "stg_update", "stg_vcycle_device", "stg_apply_op_device",
    "stg_level_descr_device", "stg_density_noise", "stg_set_stream", "stg_kernel_launches", "stg_profile",
    "stg_profile_read", "stg_profile_name", "stg_oc_update_noalloc", "stg_mma_update", "stg_mma_reset",
    "stg_set_method", "stg_net_init", "stg_net_num_params", "stg_net_get_params", "stg_net_set_params",
    "stg_net_forward_backward", "stg_net_adam_step", "stg_net_train",
]
STG_PROF_NCLASS = 12


class Opts(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("tol", ctypes.c_double), ("max_outer", ctypes.c_int),
                ("inner_max", ctypes.c_int), ("inner_tol", ctypes.c_double), ("verbose", ctypes.c_int),
                ("smooth_sweeps", ctypes.c_int), ("warm_start", ctypes.c_int), ("prolong", ctypes.c_int),
                ("basis16", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("outer_iters", ctypes.c_int), ("inner_iters", ctypes.c_int), ("rel_residual", ctypes.c_double),
                ("abs_residual", ctypes.c_double), ("setup_ms", ctypes.c_double), ("solve_ms", ctypes.c_double),
                ("status", ctypes.c_int), ("learned_iters", ctypes.c_int), ("fallbacks", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Alpha(ctypes.Structure):
    _fields_ = [("law", ctypes.c_int), ("alpha_os", ctypes.c_double), ("alpha_us", ctypes.c_double),
                ("q", ctypes.c_double), ("amax", ctypes.c_double)]


class StgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"stokes_gb300 error {code}: {msg}")
        self.code = code


_LIB = None
D = ctypes.c_double
I = ctypes.c_int
P = ctypes.c_void_p
DP = ctypes.POINTER(ctypes.c_double)
IP = ctypes.POINTER(ctypes.c_int32)
DPP = ctypes.POINTER(DP)
IPP = ctypes.POINTER(IP)


def lib():
    """Load the in-tree library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with python -m stokes_to_gb300.build")
        L = ctypes.CDLL(LIB_PATH)
        L.stg_last_error.restype = ctypes.c_char_p
        L.stg_version.restype = ctypes.c_char_p
        L.stg_default_opts.argtypes = [ctypes.POINTER(Opts)]
        L.stg_default_opts.restype = None
        L.stg_create.argtypes = [I, I, ctypes.POINTER(Opts), ctypes.POINTER(P)]
        L.stg_destroy.argtypes = [P]
        L.stg_levels.argtypes = [P]
        L.stg_level_n.argtypes = [P, I]
        L.stg_level_dof.argtypes = [P, I]
        L.stg_level_dof.restype = ctypes.c_int64
        L.stg_set_boundary.argtypes = [P, DP, IP, DPP, IPP, I]
        L.stg_set_penalty.argtypes = [P, DP, DPP]
        L.stg_set_rhs.argtypes = [P, DP, DPP]
        L.stg_solve.argtypes = [P, DP, DPP, ctypes.POINTER(Stats)]
        L.stg_get_solution.argtypes = [P, DP, DPP]
        L.stg_energy.argtypes = [P, DP, DPP, DP]
        L.stg_energy_grad_x.argtypes = [P, DP, DPP, DP, DPP]
        L.stg_energy_grad_q.argtypes = [P, DP, DPP, DP, DPP]
        L.stg_set_density.argtypes = [P, DP, ctypes.POINTER(Alpha)]
        L.stg_adjoint_sensitivity.argtypes = [P, ctypes.POINTER(Alpha), DP, ctypes.POINTER(Stats)]
        L.stg_filter.argtypes = [P, D, DP, DP, I]
        L.stg_oc_update.argtypes = [P, D, DP, DP, D, D, D, D, DP, DP]
        L.stg_mma_update.argtypes = [P, DP, DP, D, D, D, D, D, DP, DP]
        L.stg_mma_reset.argtypes = [P]
        L.stg_apply_A_device.argtypes = [P, I, P, P]
        L.stg_apply_E_device.argtypes = [P, P, P]
        L.stg_update.argtypes = [P]
        L.stg_vcycle_device.argtypes = [P, P, P]
        L.stg_apply_op_device.argtypes = [P, I, I, P, P]
        L.stg_level_descr_device.argtypes = [P, I, P, P, P]
        L.stg_density_noise.argtypes = [P, ctypes.c_uint64, D, DP]
        L.stg_set_stream.argtypes = [P, P]
        L.stg_kernel_launches.restype = ctypes.c_int64
        L.stg_kernel_launches.argtypes = []
        L.stg_profile.argtypes = [P, I]
        L.stg_profile_read.argtypes = [P, I, ctypes.POINTER(ctypes.c_int64), DP, DP]
        L.stg_profile_name.restype = ctypes.c_char_p
        L.stg_profile_name.argtypes = [I]
        L.stg_oc_update_noalloc.argtypes = [I, D, P, P, D, D, D, D, P, DP, P]
        FP = ctypes.POINTER(ctypes.c_float)
        L.stg_set_method.argtypes = [P, I]
        L.stg_net_init.argtypes = [P, ctypes.c_uint64]
        L.stg_net_num_params.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        L.stg_net_get_params.argtypes = [P, FP, ctypes.c_int64]
        L.stg_net_set_params.argtypes = [P, FP, ctypes.c_int64]
        L.stg_net_forward_backward.argtypes = [P, I, FP, FP, FP, FP, DP]
        L.stg_net_adam_step.argtypes = [P, D]
        L.stg_net_train.argtypes = [P, I, D, ctypes.c_uint64, FP]
        _LIB = L
    return _LIB


def check(rc, allow=()):
    if rc != STG_OK and rc not in allow:
        raise StgError(rc, lib().stg_last_error().decode())
    return rc


def dp(a):
    return None if a is None else a.ctypes.data_as(DP)


def fp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _c64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _faces(arrs, ctype=DP, dtype=np.float64):
    if arrs is None:
        return None, []
    keep = [np.ascontiguousarray(a, dtype=dtype) for a in arrs]
    tab = (ctype * len(keep))(*[k.ctypes.data_as(ctype) for k in keep])
    return tab, keep


def default_opts(**kw):
    o = Opts()
    lib().stg_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def alpha_bp(amax=1e4):
    return Alpha(STG_ALPHA_BP, 0.0, 0.0, 0.0, amax)


def alpha_ref(n, dim=3):
    # FluidTopoOpt3D.h:42-46 / Init (alpha_os /= N/32); FluidTopoOpt.h:43-46 for 2D
    return Alpha(STG_ALPHA_REF, 5e2 / (n / 32.0), 1e-3, 0.01 if dim == 3 else 0.014, 0.0)


def face_shape(n, d, dim=3):
    s = [n] * dim
    s[d] += 1
    return tuple(s)


class Solver:
    """Thin Python handle over the C ABI (mirrors FluidSteadyState3D + FluidEnergy3D for
    dim = 3, FluidSteadyState + FluidEnergy for dim = 2). Field-order arrays: cells
    (n,)*dim, faces of axis d one longer along d."""

    def __init__(self, n, dim=3, **opts):
        self.n, self.dim = n, dim
        self.L = lib()
        self.opts = default_opts(**opts)
        h = P()
        check(self.L.stg_create(dim, n, ctypes.byref(self.opts), ctypes.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.stg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    @property
    def levels(self):
        return self.L.stg_levels(self.h)

    def level_dof(self, level):
        return int(self.L.stg_level_dof(self.h, level))

    def set_boundary(self, cell_vol, cell_fixed, face_vol, face_fixed, closed=True):
        fv, k1 = _faces(face_vol)
        ff, k2 = _faces(face_fixed, IP, np.int32)
        cv = _c64(cell_vol)
        cf = np.ascontiguousarray(cell_fixed, dtype=np.int32) if cell_fixed is not None else None
        return check(self.L.stg_set_boundary(self.h, dp(cv), cf.ctypes.data_as(IP) if cf is not None else None, fv, ff,
                                             1 if closed else 0))

    def set_boundary_from(self, b):
        return self.set_boundary(b.cell_vol, b.cell_fixed, b.face_vol, b.face_fixed, b.closed)

    def set_penalty(self, cell_pen, face_pen):
        fp, keep = _faces(face_pen)
        return check(self.L.stg_set_penalty(self.h, dp(_c64(cell_pen)), fp))

    def set_rhs(self, cell_b, face_b):
        fb, keep = _faces(face_b)
        return check(self.L.stg_set_rhs(self.h, dp(_c64(cell_b)), fb))

    def _out_fields(self):
        n, dim = self.n, self.dim
        p = np.zeros((n,) * dim)
        vel = [np.zeros(face_shape(n, d, dim)) for d in range(dim)]
        tab = (DP * dim)(*[dp(v) for v in vel])
        return p, vel, tab

    def solve(self, want=True, allow_not_converged=False):
        st = Stats()
        if want:
            p, vel, tab = self._out_fields()
            rc = self.L.stg_solve(self.h, dp(p), tab, ctypes.byref(st))
        else:
            p = vel = None
            rc = self.L.stg_solve(self.h, None, None, ctypes.byref(st))
        check(rc, allow=(STG_E_NOT_CONVERGED,) if allow_not_converged else ())
        return p, vel, st.as_dict()

    def energy(self, p=None, vel=None):
        J = np.zeros(1)
        if p is None:
            check(self.L.stg_energy(self.h, None, None, dp(J)))
        else:
            tab, keep = _faces(vel)
            check(self.L.stg_energy(self.h, dp(_c64(p)), tab, dp(J)))
        return float(J[0])

    def energy_grad_x(self, p=None, vel=None):
        gp, gv, gtab = self._out_fields()
        if p is None:
            check(self.L.stg_energy_grad_x(self.h, None, None, dp(gp), gtab))
        else:
            tab, keep = _faces(vel)
            check(self.L.stg_energy_grad_x(self.h, dp(_c64(p)), tab, dp(gp), gtab))
        return gp, gv

    def energy_grad_q(self, p=None, vel=None):
        gp, gv, gtab = self._out_fields()
        if p is None:
            check(self.L.stg_energy_grad_q(self.h, None, None, dp(gp), gtab))
        else:
            tab, keep = _faces(vel)
            check(self.L.stg_energy_grad_q(self.h, dp(_c64(p)), tab, dp(gp), gtab))
        return gp, gv

    def set_density(self, rho, law):
        return check(self.L.stg_set_density(self.h, dp(_c64(rho)), ctypes.byref(law)))

    def adjoint_sensitivity(self, law, want=True):
        st = Stats()
        g = np.zeros((self.n,) * self.dim) if want else None
        check(self.L.stg_adjoint_sensitivity(self.h, ctypes.byref(law), dp(g), ctypes.byref(st)))
        return g, st.as_dict()

    def filter(self, rmin, rho=None, transpose=False, want=True):
        out = np.zeros((self.n,) * self.dim) if want else None
        check(self.L.stg_filter(self.h, rmin, dp(_c64(rho)), dp(out), 1 if transpose else 0))
        return out

    def oc_update(self, rmin, x, dc, frac, move=0.2, lo=0.0, hi=1.0, want=True):
        out = np.zeros((self.n,) * self.dim) if want else None
        lam = np.zeros(1)
        check(self.L.stg_oc_update(self.h, rmin, dp(_c64(x)), dp(_c64(dc)), frac, move, lo, hi, dp(out), dp(lam)))
        return out, float(lam[0])

    def mma_update(self, x, dfdx, frac, coef=1e4, lo=0.01, hi=1.0, move=0.2, want=True):
        """One MMA design update (reference optimizer); returns (x_new, change)."""
        out = np.zeros((self.n,) * self.dim) if want else None
        ch = np.zeros(1)
        check(self.L.stg_mma_update(self.h, dp(_c64(x)), dp(_c64(dfdx)), frac, coef, lo, hi, move, dp(out), dp(ch)))
        return out, float(ch[0])

    def mma_reset(self):
        return check(self.L.stg_mma_reset(self.h))

    def density_noise(self, seed, sigma, want=True):
        out = np.zeros((self.n,) * self.dim) if want else None
        check(self.L.stg_density_noise(self.h, seed, sigma, dp(out)))
        return out

    def set_method(self, method):
        return check(self.L.stg_set_method(self.h, method))

    # ---- learned preconditioner
    def net_init(self, seed=0):
        return check(self.L.stg_net_init(self.h, seed))

    def net_num_params(self):
        c = ctypes.c_int64()
        check(self.L.stg_net_num_params(self.h, ctypes.byref(c)))
        return int(c.value)

    def net_params(self):
        out = np.zeros(self.net_num_params(), dtype=np.float32)
        check(self.L.stg_net_get_params(self.h, fp(out), out.size))
        return out

    def net_set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        return check(self.L.stg_net_set_params(self.h, fp(p), p.size))

    def net_forward_backward(self, n, inp, target=None):
        """inp [n^3][8], target [n^3][4] or None -> (out, loss, grad)."""
        inp = np.ascontiguousarray(inp, dtype=np.float32)
        tgt = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
        out = np.zeros((n ** 3, 4), dtype=np.float32)
        grad = np.zeros(self.net_num_params(), dtype=np.float32) if tgt is not None else None
        loss = np.zeros(1)
        check(self.L.stg_net_forward_backward(self.h, n, fp(inp), fp(tgt), fp(out), fp(grad), dp(loss)))
        return out, (float(loss[0]) if tgt is not None else None), grad

    def net_adam_step(self, lr):
        return check(self.L.stg_net_adam_step(self.h, lr))

    def net_train(self, steps, lr=1e-3, seed=0):
        losses = np.zeros(max(steps, 1), dtype=np.float32)
        check(self.L.stg_net_train(self.h, steps, lr, seed, fp(losses)))
        return losses[:steps]

    # ---- device-pointer LinearMapping adapters (pointers are ints from torch.Tensor.data_ptr())
    def apply_A_device(self, level, out_ptr, in_ptr):
        return check(self.L.stg_apply_A_device(self.h, level, out_ptr, in_ptr))

    def apply_E_device(self, out_ptr, in_ptr):
        return check(self.L.stg_apply_E_device(self.h, out_ptr, in_ptr))

    def update(self):
        return check(self.L.stg_update(self.h))

    def vcycle_device(self, out_ptr, in_ptr):
        return check(self.L.stg_vcycle_device(self.h, out_ptr, in_ptr))

    def apply_op_device(self, op, level, out_ptr, in_ptr):
        return check(self.L.stg_apply_op_device(self.h, op, level, out_ptr, in_ptr))

    def level_descr_device(self, level, vol_ptr, pen_ptr, fixed_ptr):
        return check(self.L.stg_level_descr_device(self.h, level, vol_ptr, pen_ptr, fixed_ptr))

    # ---- streams and kernel accounting
    def set_stream(self, stream_ptr):
        return check(self.L.stg_set_stream(self.h, stream_ptr))

    def profile(self, enable=True):
        return check(self.L.stg_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        out = {}
        for c in range(STG_PROF_NCLASS):
            nl = ctypes.c_int64()
            ms = ctypes.c_double()
            by = ctypes.c_double()
            check(self.L.stg_profile_read(self.h, c, ctypes.byref(nl), ctypes.byref(ms), ctypes.byref(by)))
            out[self.L.stg_profile_name(c).decode()] = dict(launches=nl.value, ms=ms.value, bytes=by.value)
        return out


def kernel_launches():
    return int(lib().stg_kernel_launches())
