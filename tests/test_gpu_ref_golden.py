"""The GPU solver against the reference's OWN solver code (golden vectors made by
tests/golden/make_ref_golden.py from the reference's kernels and classes), through the C
ABI: per-level descriptors, A on every level and E (1e-12 relative), restriction and
prolongation (1e-13), the coarsest dense solve (1e-9: Gauss-Jordan against LU), and the
full solve to FP64 relative residual 1e-10 against the reference GMRES(V-cycle) solution
(1e-6 relative L2, pressure modulo a constant). The smoothers and V-cycle are compared
with the oracle's intended blocks in test_gpu_parity*.py; the oracle itself is pinned to
these fixtures by test_ref_golden_cpu.py.
"""
import os

import numpy as np
import pytest

from tests.helpers import pressure_free, relerr, stable_vec

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gpu_solver(po, capi, g, **opts):
    n, dim = int(g["n"]), int(g["dim"])
    to_field = po.blocked_to_field if dim == 3 else po.blocked_to_field2
    s = capi.Solver(n, dim=dim, **opts)
    cv, fv = to_field(n, g["vol"])
    cf, ff = to_field(n, g["fixed"].astype(float))
    s.set_boundary(cv, cf.astype(np.int32), fv, [f.astype(np.int32) for f in ff], bool(g["closed"]))
    s.set_penalty(*to_field(n, g["pen"]))
    s.set_rhs(*to_field(n, g["rhs"]))
    return s, to_field


@pytest.mark.parametrize("case", ["ref3d_n8_noise", "ref3d_n16_noise", "ref2d_n16_noise", "ref2d_n64_test0"])
def test_gpu_components_match_reference(oracle, stg, case):
    g = np.load(os.path.join(GOLD, case + ".npz"))
    s, _ = gpu_solver(oracle, stg, g)
    s.update()
    lv = int(g["levels"])
    assert s.levels == lv
    for i in range(lv):
        m = s.level_dof(i)
        vol = torch.zeros(m, dtype=torch.float64, device="cuda")
        pen = torch.zeros(m, dtype=torch.float64, device="cuda")
        fix = torch.zeros(m, dtype=torch.uint8, device="cuda")
        s.level_descr_device(i, vol.data_ptr(), pen.data_ptr(), fix.data_ptr())
        assert np.array_equal(host(fix), g[f"descr_fixed_{i}"]), f"fixed, level {i}"
        assert relerr(host(pen), g[f"descr_pen_{i}"]) < 1e-13, f"penalty, level {i}"
        nc = (int(g["n"]) >> (lv - 1 - i)) ** int(g["dim"])
        assert np.array_equal(host(vol)[nc:], g[f"descr_vol_{i}"][nc:]), f"face vol, level {i}"
        x = dev(stable_vec(100 + i, m))
        y = torch.zeros_like(x)
        s.apply_A_device(i, y.data_ptr(), x.data_ptr())
        assert relerr(host(y), g[f"A_{i}"]) < 1e-12, f"A, level {i}"
    x = dev(stable_vec(150, s.level_dof(lv - 1)))
    y = torch.zeros_like(x)
    s.apply_E_device(y.data_ptr(), x.data_ptr())
    assert relerr(host(y), g["E"]) < 1e-12
    for i in range(lv - 1):
        if f"R_{i}" not in g.files:
            continue
        rc = torch.zeros(s.level_dof(i), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_RESTRICT, i, rc.data_ptr(), dev(stable_vec(200 + i, s.level_dof(i + 1))).data_ptr())
        assert relerr(host(rc), g[f"R_{i}"]) < 1e-13, f"restriction to level {i}"
        xf = torch.zeros(s.level_dof(i + 1), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_PROLONG, i, xf.data_ptr(), dev(stable_vec(300 + i, s.level_dof(i))).data_ptr())
        assert relerr(host(xf), g[f"P_{i}"]) < 1e-13, f"prolongation from level {i}"
    r0 = dev(stable_vec(500, s.level_dof(0)))
    c0 = torch.zeros_like(r0)
    s.apply_op_device(stg.STG_OP_COARSE, 0, c0.data_ptr(), r0.data_ptr())
    assert relerr(host(c0), g["coarse"]) < 1e-9
    s.close()


@pytest.mark.parametrize("case", ["ref3d_n8_noise", "ref3d_n16_noise", "ref2d_n16_noise", "ref2d_n64_test0"])
@pytest.mark.parametrize("method", ["plain", "mixed"])
def test_gpu_solve_matches_reference_solve(oracle, stg, case, method):
    g = np.load(os.path.join(GOLD, case + ".npz"))
    meth = {"plain": stg.STG_METHOD_PLAIN, "mixed": stg.STG_METHOD_MIXED}[method]
    s, to_field = gpu_solver(oracle, stg, g, tol=1e-10, method=meth)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10, st
    assert float(g["solve_rel"]) <= 1e-11
    n = int(g["n"])
    p_ref, vel_ref = to_field(n, g["solve_x"])
    for d in range(int(g["dim"])):
        assert relerr(vel[d], vel_ref[d]) < 1e-6, f"velocity {d}"
    assert relerr(pressure_free(p), pressure_free(p_ref)) < 1e-6
    s.close()
