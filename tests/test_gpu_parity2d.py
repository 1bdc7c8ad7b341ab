"""GPU parity of the 2D path (dim = 2) against the 2D CPU oracle, through the C ABI.

Tolerances as in the 3D parity tests: FP64 operators, transfers and descriptors 1e-12
relative; the FP32 smoother 2e-5; the FP32 V-cycle 1e-4; the coarsest inverse (GPU
Gauss-Jordan against the oracle's LU) 1e-9; full solves reach the FP64 true relative
residual asked for and match the oracle's FP64 solution within 1e-6 relative L2
(pressure modulo a constant).
"""
import numpy as np
import pytest

from tests.helpers import pressure_free, problem2, relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def build_pair(po, capi, n, seed=1, law="bp", bc="parabolic", **opts):
    b, rho, phys, fp = problem2(po, n, seed=seed, law=law, bc=bc)
    o = po.Steady2D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    s = capi.Solver(n, dim=2, **opts)
    s.set_boundary_from(b)
    s.set_penalty(np.zeros((n, n)), fp)
    s.set_rhs(b.cell_b, b.face_b)
    s.update()
    return b, rho, phys, fp, o, s


@pytest.mark.parametrize("n,bc", [(16, "parabolic"), (64, "test0")])
def test_descriptors_all_levels_2d(oracle, stg, n, bc):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, bc=bc)
    assert s.levels == o.levels
    for lvl in range(s.levels):
        m = s.level_dof(lvl)
        assert m == o.level_dof(lvl)
        vol_o, pen_o, fix_o, _ = o.descr(lvl)
        vol = torch.zeros(m, dtype=torch.float64, device="cuda")
        pen = torch.zeros(m, dtype=torch.float64, device="cuda")
        fix = torch.zeros(m, dtype=torch.uint8, device="cuda")
        s.level_descr_device(lvl, vol.data_ptr(), pen.data_ptr(), fix.data_ptr())
        assert np.array_equal(host(fix), fix_o), f"fixed mask differs at level {lvl}"
        assert np.array_equal(host(vol), vol_o), f"vol differs at level {lvl}"
        assert relerr(host(pen), pen_o) < 1e-14


@pytest.mark.parametrize("n,bc", [(16, "parabolic"), (64, "test0")])
def test_operator_A_every_level_2d(oracle, stg, n, bc):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, bc=bc)
    rng = np.random.default_rng(3)
    for lvl in range(s.levels):
        x = rng.standard_normal(o.level_dof(lvl))
        xd = dev(x)
        yd = torch.zeros_like(xd)
        s.apply_A_device(lvl, yd.data_ptr(), xd.data_ptr())
        assert relerr(host(yd), o.apply_A(x, lvl)) < 1e-12, f"level {lvl}"


def test_operator_E_2d(oracle, stg):
    n = 32
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    x = np.random.default_rng(4).standard_normal(o.level_dof(o.levels - 1))
    xd = dev(x)
    yd = torch.zeros_like(xd)
    s.apply_E_device(yd.data_ptr(), xd.data_ptr())
    assert relerr(host(yd), o.apply_E(x)) < 1e-12


def test_transfers_2d(oracle, stg):
    n = 64
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(5)
    for lvl in range(s.levels - 1):
        rf = rng.standard_normal(o.level_dof(lvl + 1))
        out = torch.zeros(o.level_dof(lvl), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_RESTRICT, lvl, out.data_ptr(), dev(rf).data_ptr())
        assert relerr(host(out), o.restrict(lvl, rf)) < 1e-13
        xc = rng.standard_normal(o.level_dof(lvl))
        outf = torch.zeros(o.level_dof(lvl + 1), dtype=torch.float64, device="cuda")
        s.apply_op_device(stg.STG_OP_PROLONG, lvl, outf.data_ptr(), dev(xc).data_ptr())
        assert relerr(host(outf), o.prolong(lvl, xc)) < 1e-13


@pytest.mark.parametrize("n", [16, 64])
def test_smoother_2d(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(6)
    for lvl in range(1, s.levels):
        m = o.level_dof(lvl)
        fixed = o.descr(lvl)[2]
        r = rng.standard_normal(m) * (1 - fixed)
        rd = dev(r)
        out = torch.zeros_like(rd)
        for op, flag in ((stg.STG_OP_VANKA_RED, 0), (stg.STG_OP_VANKA_BLACK, 1)):
            s.apply_op_device(op, lvl, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.smooth_colour(lvl, flag, r)) < 2e-5, f"colour {flag} level {lvl}"
        for op, post in ((stg.STG_OP_SMOOTH_PRE, 0), (stg.STG_OP_SMOOTH_POST, 1)):
            s.apply_op_device(op, lvl, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.smooth(lvl, post, r)) < 2e-5, f"smoother post={post} level {lvl}"


@pytest.mark.parametrize("n", [8, 64])
def test_coarsest_dense_solve_2d(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    assert o.coarse_info() == 0
    fixed = o.descr(0)[2]
    r = np.random.default_rng(7).standard_normal(o.level_dof(0)) * (1 - fixed)
    out = torch.zeros(o.level_dof(0), dtype=torch.float64, device="cuda")
    s.apply_op_device(stg.STG_OP_COARSE, 0, out.data_ptr(), dev(r).data_ptr())
    assert relerr(host(out), o.coarse_apply(r)) < 1e-9


@pytest.mark.parametrize("n", [16, 64, 128])
def test_vcycle_2d(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    bb = oracle.field_to_blocked2(n, b.cell_b, b.face_b)
    out = torch.zeros(bb.size, dtype=torch.float64, device="cuda")
    s.vcycle_device(out.data_ptr(), dev(bb).data_ptr())
    assert relerr(host(out), o.vcycle(bb)) < 1e-4


@pytest.mark.parametrize("n,law,bc", [(16, "bp", "parabolic"), (64, "bp", "parabolic"), (64, "ref", "test0"),
                                      (128, "ref", "parabolic")])
def test_solve_2d_matches_oracle(oracle, stg, n, law, bc):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, law=law, bc=bc, tol=1e-10)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10
    x_ref, ost = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
    assert ost["rel_true"] <= 1e-10
    p_ref, vel_ref = oracle.blocked_to_field2(n, x_ref)
    for d in range(2):
        assert relerr(vel[d], vel_ref[d]) < 1e-6
    assert relerr(pressure_free(p), pressure_free(p_ref)) < 1e-6
    J = s.energy()
    assert abs(J - o.energy(x_ref)) <= 1e-6 * abs(o.energy(x_ref))


def test_energy_gradients_2d(oracle, stg):
    n = 32
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(8)
    p = rng.standard_normal((n, n))
    vel = [rng.standard_normal(oracle.face_shape(n, d, 2)) for d in range(2)]
    x = oracle.field_to_blocked2(n, p, vel)
    assert abs(s.energy(p, vel) - o.energy(x)) <= 1e-12 * abs(o.energy(x))
    gp, gv = s.energy_grad_x(p, vel)
    gp_ref, gv_ref = oracle.blocked_to_field2(n, o.apply_E(x))
    for d in range(2):
        assert relerr(gv[d], gv_ref[d]) < 1e-12
    qp, qv = s.energy_grad_q(p, vel)
    for d in range(2):
        assert relerr(qv[d], 0.5 * vel[d] ** 2) < 1e-15


@pytest.mark.parametrize("law", ["bp", "ref"])
def test_adjoint_sensitivity_2d(oracle, stg, law):
    n = 64
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, law=law, tol=1e-11)
    L = stg.alpha_bp() if law == "bp" else stg.alpha_ref(n, dim=2)
    s.set_density(phys, L)
    p, vel, st = s.solve()
    g, ast = s.adjoint_sensitivity(L)
    assert ast["rel_residual"] <= 1e-11
    x_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-12)
    o.set_b_blocked(o.apply_E(x_ref))
    lam_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-12)
    _, u = oracle.blocked_to_field2(n, x_ref)
    _, lam = oracle.blocked_to_field2(n, lam_ref)
    prm = [1e4] if law == "bp" else [5e2 / (n / 32.0), 1e-3, 0.014]
    g_ref = oracle.sensitivity(phys, 1 if law == "bp" else 0, prm, u, lam, dim=2)
    assert relerr(g, g_ref) < 1e-6


def test_filter_oc_and_noise_2d(oracle, stg):
    n = 64
    s = stg.Solver(n, dim=2)
    rho = s.density_noise(7, 2.0)
    assert rho.shape == (n, n)
    assert relerr(rho, oracle.density_noise(n, 7, 2.0, dim=2)) < 1e-14
    assert relerr(s.filter(1.5, rho), oracle.filt(rho, 1.5)) < 1e-14
    g = np.random.default_rng(9).standard_normal((n, n))
    assert relerr(s.filter(1.5, g, transpose=True), oracle.filt(g, 1.5, transpose=True)) < 1e-14
    dc = -np.abs(np.random.default_rng(10).standard_normal((n, n)))
    xn, lam = s.oc_update(1.5, rho, dc, 0.3)
    vw = oracle.filt(np.ones((n, n)), 1.5, transpose=True)
    xn_ref, lam_ref, _ = oracle.oc_update(rho, dc, vw / n ** 2, vw, 0.3)
    assert relerr(xn, xn_ref.reshape(n, n)) < 1e-9
    assert abs(np.sum(vw * xn) / n ** 2 - 0.3) < 1e-6


def test_design_loop_2d_64_matches_oracle(oracle, stg):
    """Five OC iterations of the 64x64 BP-law problem (parabolic inlet on a centred
    16-cell segment), every solve to 1e-10, on the device-resident design path."""
    n, rmin, frac, iters = 64, 1.5, 0.3, 5
    b = oracle.bc_parabolic(n, 2, width=16)
    L = stg.alpha_bp()
    s = stg.Solver(n, dim=2, tol=1e-10)
    s.set_boundary_from(b)
    s.set_rhs(b.cell_b, b.face_b)
    x = s.density_noise(5, 2.0)
    x_ref = x.copy()
    vw = oracle.filt(np.ones((n, n)), rmin, transpose=True)
    J_gpu, J_ref = [], []
    for it in range(iters):
        # GPU: design -> filter -> penalty -> solve -> adjoint -> chain rule -> OC
        s.filter(rmin, want=False)
        s.set_density(None, L)
        s.solve(want=False)
        J_gpu.append(s.energy())
        s.adjoint_sensitivity(L, want=False)
        s.filter(rmin, transpose=True, want=False)
        x, _ = s.oc_update(rmin, None, None, frac)
        # oracle
        phys = oracle.filt(x_ref, rmin)
        fp = oracle.face_penalty(phys, 1, [1e4], dim=2)
        o = oracle.Steady2D(n)
        o.init_boundary(b)
        o.update_penalty(np.zeros((n, n)), fp)
        o.update_b(b.cell_b, b.face_b)
        u_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        J_ref.append(o.energy(u_ref))
        o.set_b_blocked(o.apply_E(u_ref))
        lam_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
        _, u = oracle.blocked_to_field2(n, u_ref)
        _, lam = oracle.blocked_to_field2(n, lam_ref)
        dc = oracle.filt(oracle.sensitivity(phys, 1, [1e4], u, lam, dim=2), rmin, transpose=True)
        x_ref, _, _ = oracle.oc_update(x_ref, dc, vw / n ** 2, vw, frac)
        x_ref = x_ref.reshape(n, n)
    assert np.allclose(J_gpu, J_ref, rtol=1e-6, atol=0)
    assert relerr(x, x_ref) < 1e-5


def test_errors_are_reported_2d(stg):
    with pytest.raises(stg.StgError) as e:
        stg.Solver(12, dim=2)  # the 2D layout needs N % 8 == 0
    assert e.value.code == stg.STG_E_INVALID
    with pytest.raises(stg.StgError) as e:
        stg.Solver(8, dim=4)
    assert e.value.code == stg.STG_E_INVALID
    s = stg.Solver(16, dim=2)
    with pytest.raises(stg.StgError):
        s.solve()  # no rhs
