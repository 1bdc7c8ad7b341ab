"""GPU parity of every hot-path component against the CPU oracle, through the C ABI.

Tolerances: FP64 operators and transfers 1e-12 relative; FP32 smoothing components
2e-5 relative (single-precision arithmetic); full solves reach the FP64 true relative
residual asked for and match the oracle's FP64 solution within 1e-6 relative L2
(pressure compared modulo a constant: closed domains have a constant-pressure null space).
"""
import numpy as np
import pytest

from tests.helpers import pressure_free, problem, relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def build_pair(po, capi, n, seed=1, law="bp", bc="parabolic", **opts):
    b, rho, phys, fp = problem(po, n, seed=seed, law=law, bc=bc)
    o = po.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    o.setup()
    s = capi.Solver(n, **opts)
    s.set_boundary_from(b)
    s.set_penalty(np.zeros((n, n, n)), fp)
    s.set_rhs(b.cell_b, b.face_b)
    s.update()
    return b, rho, phys, fp, o, s


@pytest.mark.parametrize("n", [8, 16])
def test_descriptors_all_levels(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    assert s.levels == o.levels
    for lvl in range(s.levels):
        m = s.level_dof(lvl)
        assert m == o.level_dof(lvl)
        vol_o, pen_o, fix_o = o.descr(lvl)
        vol = torch.zeros(m, dtype=torch.float64, device="cuda")
        pen = torch.zeros(m, dtype=torch.float64, device="cuda")
        fix = torch.zeros(m, dtype=torch.uint8, device="cuda")
        s.level_descr_device(lvl, vol.data_ptr(), pen.data_ptr(), fix.data_ptr())
        assert np.array_equal(host(fix), fix_o), f"fixed mask differs at level {lvl}"
        assert relerr(host(pen), pen_o) < 1e-13
        nc = (n >> (s.levels - 1 - lvl)) ** 3
        # face vol (cell vol never enters A) must agree exactly
        assert np.array_equal(host(vol)[nc:], vol_o[nc:])


@pytest.mark.parametrize("n", [8, 16])
def test_operator_A_every_level(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(3)
    for lvl in range(s.levels):
        x = rng.standard_normal(o.level_dof(lvl))
        y_ref = o.apply_A(x, lvl)
        xd = dev(x)
        yd = torch.zeros_like(xd)
        s.apply_A_device(lvl, yd.data_ptr(), xd.data_ptr())
        assert relerr(host(yd), y_ref) < 1e-12, f"level {lvl}"


def test_operator_E(oracle, stg):
    n = 16
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    x = np.random.default_rng(4).standard_normal(o.level_dof(o.levels - 1))
    xd = dev(x)
    yd = torch.zeros_like(xd)
    s.apply_E_device(yd.data_ptr(), xd.data_ptr())
    assert relerr(host(yd), o.apply_E(x)) < 1e-12


@pytest.mark.parametrize("n", [8, 16])
def test_transfers(oracle, stg, n):
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


@pytest.mark.parametrize("n", [8, 16])
def test_vanka_blocks_and_smoothers(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(6)
    for lvl in range(1, s.levels):
        m = o.level_dof(lvl)
        _, _, fixed = o.descr(lvl)
        r = rng.standard_normal(m) * (1 - fixed)
        rd = dev(r)
        out = torch.zeros_like(rd)
        for op, flag in ((stg.STG_OP_VANKA_RED, 0), (stg.STG_OP_VANKA_BLACK, 1)):
            s.apply_op_device(op, lvl, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.vanka_apply(lvl, flag, r)) < 2e-5, f"vanka flag {flag} level {lvl}"
        for op, post in ((stg.STG_OP_SMOOTH_PRE, 0), (stg.STG_OP_SMOOTH_POST, 1)):
            s.apply_op_device(op, lvl, out.data_ptr(), rd.data_ptr())
            assert relerr(host(out), o.smooth(lvl, post, r)) < 2e-5, f"smoother post={post} level {lvl}"


@pytest.mark.parametrize("n", [4, 8])
def test_coarsest_dense_solve(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    assert o.coarse_info() == 0
    _, _, fixed = o.descr(0)
    r = np.random.default_rng(7).standard_normal(o.level_dof(0)) * (1 - fixed)
    out = torch.zeros(o.level_dof(0), dtype=torch.float64, device="cuda")
    s.apply_op_device(stg.STG_OP_COARSE, 0, out.data_ptr(), dev(r).data_ptr())
    assert relerr(host(out), o.coarse_apply(r)) < 1e-9


@pytest.mark.parametrize("n", [8, 16, 32])
def test_vcycle(oracle, stg, n):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    bb = oracle.field_to_blocked(n, b.cell_b, b.face_b)
    out = torch.zeros(bb.size, dtype=torch.float64, device="cuda")
    s.vcycle_device(out.data_ptr(), dev(bb).data_ptr())
    assert relerr(host(out), o.vcycle(bb)) < 1e-4


@pytest.mark.parametrize("n", [16, 32])
def test_vcycle_laplacian_and_general_paths(oracle, stg, n):
    """A right-hand side that is zero on fixed unknowns runs the Laplacian-form kernels
    (every boundary face is fixed here); one with nonzero fixed entries runs the general
    masked stencil. Both must reproduce the oracle's V-cycle."""
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    fixed = o.descr(o.levels - 1)[2]
    rng = np.random.default_rng(11)
    r = rng.standard_normal(o.level_dof(o.levels - 1))
    for rhs in (r * (1 - fixed), r):
        out = torch.zeros(rhs.size, dtype=torch.float64, device="cuda")
        s.vcycle_device(out.data_ptr(), dev(rhs).data_ptr())
        assert relerr(host(out), o.vcycle(rhs)) < 1e-4


@pytest.mark.parametrize("n,law,bc", [(8, "bp", "parabolic"), (16, "bp", "parabolic"), (32, "bp", "parabolic"),
                                      (64, "ref", "test0")])
@pytest.mark.parametrize("method", [0, 1])
def test_solve_matches_oracle(oracle, stg, n, law, bc, method):
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, law=law, bc=bc, tol=1e-10, method=method)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-10
    x_ref, ost = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-11)
    assert ost["rel_true"] <= 1e-10
    p_ref, vel_ref = oracle.blocked_to_field(n, x_ref)
    for d in range(3):
        assert relerr(vel[d], vel_ref[d]) < 1e-6
    assert relerr(pressure_free(p), pressure_free(p_ref)) < 1e-6
    # the oracle's operator confirms the residual the GPU reports
    bb = oracle.field_to_blocked(n, b.cell_b, b.face_b)
    x_gpu = oracle.field_to_blocked(n, p, vel)
    assert relerr(o.apply_A(x_gpu), bb) <= 2e-10
    # energy of the GPU solution against the oracle's energy of its own solution
    J = s.energy()
    assert abs(J - o.energy(x_ref)) <= 1e-6 * abs(o.energy(x_ref))


def test_solve_with_penalties_beyond_fp16_range(oracle, stg):
    """The solver's sweeps stage the penalty in FP16 divided by a per-level power-of-two
    scale taken from the largest finest-level penalty: with penalties up to 1.2e5 (FP16 ends
    at 65504; unscaled they would stage as infinities) the solve reaches the FP64
    tolerance of the design loop, which the oracle's operator confirms."""
    n = 16
    b, rho, phys, fp = problem(oracle, n, seed=4)
    fp = [f * 100.0 for f in fp]
    assert max(float(np.max(f)) for f in fp) > 65504.0
    o = oracle.Steady3D(n)
    o.init_boundary(b)
    o.update_penalty(np.zeros((n, n, n)), fp)
    o.update_b(b.cell_b, b.face_b)
    o.setup()
    s = stg.Solver(n, tol=1e-8)
    s.set_boundary_from(b)
    s.set_penalty(np.zeros((n, n, n)), fp)
    s.set_rhs(b.cell_b, b.face_b)
    p, vel, st = s.solve()
    assert st["status"] == 0 and st["rel_residual"] <= 1e-8 and st["inner_iters"] < 200, st
    bb = oracle.field_to_blocked(n, b.cell_b, b.face_b)
    assert relerr(o.apply_A(oracle.field_to_blocked(n, p, vel)), bb) <= 2e-8


def test_energy_gradients(oracle, stg):
    n = 16
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n)
    rng = np.random.default_rng(8)
    p = rng.standard_normal((n, n, n))
    vel = [rng.standard_normal(oracle.face_shape(n, d)) for d in range(3)]
    x = oracle.field_to_blocked(n, p, vel)
    assert abs(s.energy(p, vel) - o.energy(x)) <= 1e-12 * abs(o.energy(x))
    gp, gv = s.energy_grad_x(p, vel)
    gp_ref, gv_ref = oracle.blocked_to_field(n, o.apply_E(x))
    for d in range(3):
        assert relerr(gv[d], gv_ref[d]) < 1e-12
    qp, qv = s.energy_grad_q(p, vel)
    for d in range(3):
        assert relerr(qv[d], 0.5 * vel[d] ** 2) < 1e-15


@pytest.mark.parametrize("law", ["bp", "ref"])
def test_adjoint_sensitivity(oracle, stg, law):
    n = 16
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, law=law, tol=1e-11)
    L = stg.alpha_bp() if law == "bp" else stg.alpha_ref(n)
    s.set_density(phys, L)
    p, vel, st = s.solve()
    g, ast = s.adjoint_sensitivity(L)
    assert ast["rel_residual"] <= 1e-11
    # oracle: forward solve, adjoint rhs E x, adjoint solve, chain rule
    x_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-12)
    o.set_b_blocked(o.apply_E(x_ref))
    lam_ref, _ = o.solve(max_iter=60, abs_thr=0.0, rel_thr=1e-13, norm_thr=0.0, restarts=4, true_tol=1e-12)
    _, u = oracle.blocked_to_field(n, x_ref)
    _, lam = oracle.blocked_to_field(n, lam_ref)
    prm = [1e4] if law == "bp" else [5e2 / (n / 32.0), 1e-3, 0.01]
    g_ref = oracle.sensitivity(phys, 1 if law == "bp" else 0, prm, u, lam)
    assert relerr(g, g_ref) < 1e-6


def test_filter_oc_and_noise(oracle, stg):
    n = 16
    s = stg.Solver(n)
    rho = s.density_noise(7, 2.0)
    assert relerr(rho, oracle.density_noise(n, 7, 2.0)) < 1e-14
    rf = s.filter(1.5, rho)
    assert relerr(rf, oracle.filt(rho, 1.5)) < 1e-14
    g = np.random.default_rng(9).standard_normal((n, n, n))
    gt = s.filter(1.5, g, transpose=True)
    assert relerr(gt, oracle.filt(g, 1.5, transpose=True)) < 1e-14
    vw = oracle.filt(np.ones((n, n, n)), 1.5, transpose=True)
    # scale 1e8: the multiplier lies above the initial bracket [0, 1e9] (as at 512^3)
    for scale in (1.0, 1e8):
        dc = -np.abs(np.random.default_rng(10).standard_normal((n, n, n))) * scale
        xn, lam = s.oc_update(1.5, rho, dc, 0.3)
        xn_ref, lam_ref, _ = oracle.oc_update(rho, dc, vw / n ** 3, vw, 0.3)
        assert relerr(xn, xn_ref.reshape(n, n, n)) < 1e-9
        assert abs(lam - lam_ref) <= 1e-9 * lam_ref
        assert abs(np.sum(vw * xn) / n ** 3 - 0.3) < 1e-6


def test_errors_are_reported(stg):
    with pytest.raises(stg.StgError) as e:
        stg.Solver(6)
    assert e.value.code == stg.STG_E_INVALID
    s = stg.Solver(8)
    with pytest.raises(stg.StgError):
        s.solve()  # no rhs
    n = 8
    vol = [np.ones(stg.face_shape(n, d)) for d in range(3)]
    vol[0][3, 3, 3] = 2.0
    fixed = [np.zeros(stg.face_shape(n, d), dtype=np.int32) for d in range(3)]
    # non-uniform vols run the general-coefficient form, which the learned method lacks
    learned = stg.Solver(n, method=stg.STG_METHOD_LEARNED)
    with pytest.raises(stg.StgError) as e:
        learned.set_boundary(np.ones((n, n, n)), np.zeros((n, n, n), dtype=np.int32), vol, fixed)
    assert e.value.code == stg.STG_E_UNSUPPORTED
    s.set_boundary(np.ones((n, n, n)), np.zeros((n, n, n), dtype=np.int32), vol, fixed)
    with pytest.raises(stg.StgError) as e:
        s.set_method(stg.STG_METHOD_LEARNED)
    assert e.value.code == stg.STG_E_UNSUPPORTED


def test_warm_start_reaches_the_same_solution(oracle, stg):
    """A warm-started solve (previous solution as the initial guess) reaches the same
    tolerance and solution as a cold one, in fewer V-cycles when the design moved little."""
    n = 32
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, tol=1e-10, warm_start=1)
    s.solve()
    fp2 = [f * 1.001 for f in fp]
    s.set_penalty(np.zeros((n, n, n)), fp2)
    p_w, vel_w, st_w = s.solve()
    cold = stg.Solver(n, tol=1e-10)
    cold.set_boundary_from(b)
    cold.set_penalty(np.zeros((n, n, n)), fp2)
    cold.set_rhs(b.cell_b, b.face_b)
    p_c, vel_c, st_c = cold.solve()
    assert st_w["status"] == 0 and st_w["rel_residual"] <= 1e-10
    assert st_w["inner_iters"] < st_c["inner_iters"]
    for d in range(3):
        assert relerr(vel_w[d], vel_c[d]) < 1e-8


@pytest.mark.parametrize("method", [0, 1])
def test_graph_replay_matches_direct_launches(oracle, stg, method):
    """The V-cycle below the finest level and the coarsest set-up run as replayed CUDA
    graphs; the per-kernel profiler switches the graphs off. Repeated solves with and
    without the graphs give the same bits (same kernels, same inputs, fixed reductions),
    and the replay restores the host-side ping-pong state it leaves."""
    n = 32
    b, rho, phys, fp, o, s = build_pair(oracle, stg, n, tol=1e-10, method=method)
    runs = []
    for _ in range(3):  # first solve direct, graphs captured during it, replayed after
        runs.append(s.solve())
    s.profile(True)
    direct = s.solve()
    s.profile(False)
    for p, vel, st in runs + [direct]:
        assert st["status"] == 0 and st["inner_iters"] == direct[2]["inner_iters"]
        assert np.array_equal(p, direct[0])
        for d in range(3):
            assert np.array_equal(vel[d], direct[1][d])
