"""The allocation-free optimality-criteria update against the handle-based one.

stg_oc_update_noalloc serves callers that cannot allocate device memory (applications
that pre-reserve the whole GPU for their own pool, plugins living under another
framework's allocator budget, loops that cannot afford cudaMalloc's device-wide
synchronisation): it works on the caller's device arrays and keeps its only scratch in
a fixed array inside the library. This file runs last so that a failure here never hides
the other tests; it passes alone in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(capi, n, rmin, dx, ddc, frac, dout, move=0.2, lo=0.0, hi=1.0):
    lam = ctypes.c_double()
    stream = torch.cuda.current_stream().cuda_stream
    rc = capi.lib().stg_oc_update_noalloc(n, rmin, dx.data_ptr(), ddc.data_ptr(), frac, move, lo, hi, dout.data_ptr(),
                                          ctypes.byref(lam), stream)
    capi.check(rc)
    torch.cuda.synchronize()
    return lam.value


@pytest.mark.parametrize("rmin", [1.5, 2.5])
def test_oc_update_noalloc_matches_handle_entry_point(stg, rmin):
    n = 16
    rng = np.random.default_rng(21)
    s = stg.Solver(n)
    # two calls in a row with different inputs: the shared scratch keeps the previous
    # call's partial sums and weight table, which must not leak into the next result
    for call, frac in enumerate((0.3, 0.45)):
        x = 0.2 + 0.6 * rng.random((n, n, n))
        dc = -np.abs(rng.standard_normal((n, n, n))) * (1.0 + call)
        ref, lam_ref = s.oc_update(rmin, x, dc, frac)
        dx = torch.from_numpy(x).cuda()
        ddc = torch.from_numpy(dc).cuda()
        dout = torch.full_like(dx, -1.0)
        lam = _noalloc(stg, n, rmin, dx, ddc, frac, dout)
        out = dout.cpu().numpy()
        assert np.max(np.abs(out - ref)) <= 1e-12, f"call {call}"
        assert abs(lam - lam_ref) <= 1e-12 * abs(lam_ref), f"call {call}"
        # the result written over the design itself (d_xnew == d_x)
        lam2 = _noalloc(stg, n, rmin, dx, ddc, frac, dx)
        assert np.max(np.abs(dx.cpu().numpy() - ref)) <= 1e-12, f"aliased call {call}"
        assert abs(lam2 - lam_ref) <= 1e-12 * abs(lam_ref), f"aliased call {call}"
    s.close()


def test_oc_update_noalloc_rejects_out_of_range_arguments(stg):
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    lam = ctypes.c_double()
    for n in (1025, 1 << 21):
        rc = stg.lib().stg_oc_update_noalloc(n, 1.5, d.data_ptr(), d.data_ptr(), 0.3, 0.2, 0.0, 1.0, d.data_ptr(),
                                             ctypes.byref(lam), None)
        assert rc == stg.STG_E_INVALID
        assert b"1024" in stg.lib().stg_last_error()
    for rmin in (0.0, 4.5, 50.0):
        rc = stg.lib().stg_oc_update_noalloc(2, rmin, d.data_ptr(), d.data_ptr(), 0.3, 0.2, 0.0, 1.0, d.data_ptr(),
                                             ctypes.byref(lam), None)
        assert rc == stg.STG_E_INVALID
        assert b"rmin" in stg.lib().stg_last_error()
