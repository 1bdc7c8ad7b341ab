"""The general-coefficient form of the 3D solver (non-uniform face vols, fixed cells)
against the reference's own solver code and the oracle, through the C ABI.

FluidSteadyState3D::init_boundary accepts any vol and fixed flags; with one vol value on
the free faces and no fixed cell the solver uses its uniform form (closed-form Vanka
blocks), otherwise the general form (general.cu: per-face vols, probed and LU-factored
Vanka blocks, an FP64 V-cycle). Tolerances: operators, transfers, descriptors 1e-12
relative; the FP64 Vanka block solves, smoothers and V-cycle 1e-10 against the oracle's
intended blocks; solves to FP64 relative residual 1e-10, within 1e-6 of the reference's
GMRES solution (pressure modulo a constant) where the reference solves.
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


def pair(po, capi, g, **opts):
    n = int(g["n"])
    b = po.Boundary(n)
    b.cell_vol, b.face_vol = po.blocked_to_field(n, g["vol"])
    cf, ff = po.blocked_to_field(n, g["fixed"].astype(float))
    b.cell_fixed, b.face_fixed = cf.astype(np.int32), [f.astype(np.int32) for f in ff]
    b.closed = bool(g["closed"])
    cp, fp = po.blocked_to_field(n, g["pen"])
    o = po.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(cp, fp)
    o.set_b_blocked(g["rhs"])
    o.setup()
    s = capi.Solver(n, **opts)
    s.set_boundary_from(b)
    s.set_penalty(cp, fp)
    s.set_rhs(*po.blocked_to_field(n, g["rhs"]))
    return o, s


@pytest.mark.parametrize("case", ["ref3d_n8_general", "ref3d_n8_fixedcells"])
def test_general_components_match_reference_and_oracle(oracle, stg, case):
    g = np.load(os.path.join(GOLD, case + ".npz"))
    o, s = pair(oracle, stg, g)
    s.update()
    lv = int(g["levels"])
    for i in range(lv):
        m = s.level_dof(i)
        vol = torch.zeros(m, dtype=torch.float64, device="cuda")
        pen = torch.zeros(m, dtype=torch.float64, device="cuda")
        fix = torch.zeros(m, dtype=torch.uint8, device="cuda")
        s.level_descr_device(i, vol.data_ptr(), pen.data_ptr(), fix.data_ptr())
        assert np.array_equal(host(fix), g[f"descr_fixed_{i}"]), f"fixed, level {i}"
        assert relerr(host(pen), g[f"descr_pen_{i}"]) < 1e-13, f"penalty, level {i}"
        assert relerr(host(vol), g[f"descr_vol_{i}"]) < 1e-13, f"vol, level {i}"
        x = dev(stable_vec(100 + i, m))
        y = torch.zeros_like(x)
        s.apply_A_device(i, y.data_ptr(), x.data_ptr())
        assert relerr(host(y), g[f"A_{i}"]) < 1e-12, f"A, level {i}"
    x = dev(stable_vec(150, s.level_dof(lv - 1)))
    y = torch.zeros_like(x)
    s.apply_E_device(y.data_ptr(), x.data_ptr())
    assert relerr(host(y), g["E"]) < 1e-12
    for i in range(lv - 1):
        rc = torch.zeros(s.level_dof(i), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_RESTRICT, i, rc.data_ptr(), dev(stable_vec(200 + i, s.level_dof(i + 1))).data_ptr())
        assert relerr(host(rc), g[f"R_{i}"]) < 1e-13
        xf = torch.zeros(s.level_dof(i + 1), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_PROLONG, i, xf.data_ptr(), dev(stable_vec(300 + i, s.level_dof(i))).data_ptr())
        assert relerr(host(xf), g[f"P_{i}"]) < 1e-13
    # the Vanka block solves and smoothers against the oracle's intended blocks (FP64)
    for i in range(1, lv):
        r = stable_vec(400 + i, s.level_dof(i))
        rd = dev(r)
        out = torch.zeros_like(rd)
        for op, flag in ((stg.STG_OP_VANKA_RED, 0), (stg.STG_OP_VANKA_BLACK, 1)):
            s.apply_op_device(op, i, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.vanka_apply(i, flag, r)) < 1e-10, f"Vanka colour {flag}, level {i}"
        for op, post in ((stg.STG_OP_SMOOTH_PRE, 0), (stg.STG_OP_SMOOTH_POST, 1)):
            s.apply_op_device(op, i, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.smooth(i, post, r)) < 1e-10, f"smoother post={post}, level {i}"
    if "vcycle" in g.files:
        r = stable_vec(600, s.level_dof(lv - 1))
        out = torch.zeros(r.size, dtype=torch.float64, device="cuda")
        s.vcycle_device(out.data_ptr(), dev(r).data_ptr())
        assert relerr(host(out), o.vcycle(r)) < 1e-10
    s.close()


def test_general_solve_matches_reference_solve(oracle, stg):
    g = np.load(os.path.join(GOLD, "ref3d_n8_general.npz"))
    o, s = pair(oracle, stg, g, tol=1e-10)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10, st
    n = int(g["n"])
    p_ref, vel_ref = oracle.blocked_to_field(n, g["solve_x"])
    for d in range(3):
        assert relerr(vel[d], vel_ref[d]) < 1e-6, f"velocity {d}"
    assert relerr(pressure_free(p), pressure_free(p_ref)) < 1e-6
    s.close()


@pytest.mark.parametrize("n,cells", [(16, False), (16, True), (32, False), (32, True)])
def test_general_solves_reach_the_fp64_tolerance(oracle, stg, n, cells):
    """Random vols in [0.5, 2] on cells and faces, the walls fixed, and an obstacle in the
    channel: without `cells` a baffle of fixed x-faces across the middle of the duct (a
    quarter of the cross-section), with `cells` a solid block of fixed cells whose faces are
    fixed too. A BP-law penalty; the solve reaches FP64 relative residual 1e-10 as measured
    by the oracle's operator. The reference cannot solve the fixed-cell problems (its
    coarsest matrix is singular); the GPU's coarsest matrix keeps the fixed cells' identity
    rows. (Scattered fixed faces are not a fair input: the coarse levels OR their
    children's flags, so they soon isolate cells there, for the reference as for this
    library.)"""
    b = oracle.bc_parabolic(n)
    u = lambda sd, shape: 0.5 * (stable_vec(sd, int(np.prod(shape))).reshape(shape) + 1.0)
    b.cell_vol = 0.5 + 1.5 * u(61, (n, n, n))
    b.face_vol = [0.5 + 1.5 * u(62 + d, oracle.face_shape(n, d)) for d in range(3)]
    q, h = n // 4, n // 2
    if cells:
        lo, hi = (h, h + q), (q, h)  # x range, y/z range of the solid block
        b.cell_fixed[lo[0]:lo[1], hi[0]:hi[1], hi[0]:hi[1]] = 1
        b.face_fixed[0][lo[0]:lo[1] + 1, hi[0]:hi[1], hi[0]:hi[1]] = 1
        b.face_fixed[1][lo[0]:lo[1], hi[0]:hi[1] + 1, hi[0]:hi[1]] = 1
        b.face_fixed[2][lo[0]:lo[1], hi[0]:hi[1], hi[0]:hi[1] + 1] = 1
    else:
        b.face_fixed[0][h, q:h, q:h + q] = 1
    rho = oracle.density_noise(n, 5, 2.0)
    fp = oracle.face_penalty(oracle.filt(rho, 1.5), 1, [1e4])
    rhs = stable_vec(69, oracle.dof(n))
    o = oracle.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n, n)), fp)
    fixed = o.descr(o.levels - 1)[2]
    rhs = np.where(fixed != 0, 0.0, rhs)
    free_cells = fixed[: n ** 3] == 0
    rhs[: n ** 3][free_cells] -= rhs[: n ** 3][free_cells].mean()
    s = stg.Solver(n, tol=1e-10)
    s.set_boundary_from(b)
    s.set_penalty(np.zeros((n, n, n)), fp)
    cb, fb = oracle.blocked_to_field(n, rhs)
    s.set_rhs(cb, fb)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10, st
    bb = oracle.field_to_blocked(n, cb, fb)
    assert relerr(o.apply_A(oracle.field_to_blocked(n, p, vel)), bb) <= 2e-10
    s.close()
