"""GPU checks of the solver's alternative paths, through the C ABI: the FP16 copies of the
FGMRES basis (stg_opts.basis16) and the set-up that stg_set_rhs overlaps with the copy of
b. Each must give the solution of the other path to the solve tolerance, or bit for bit
where the same kernels run."""
import numpy as np
import pytest

from tests.helpers import pressure_free, problem, relerr

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def solver(stg, b, fp, n, **opts):
    s = stg.Solver(n, **opts)
    s.set_boundary_from(b)
    s.set_penalty(np.zeros((n, n, n)), fp)
    s.set_rhs(b.cell_b, b.face_b)
    return s


def test_fp16_basis_copies_same_solution(oracle, stg):
    """The multi-dot reads FP16 copies of the basis; the projections keep FP32, so the
    Arnoldi relation is exact and the solve reaches the same FP64 tolerance and solution
    in the same number of V-cycles (give or take one)."""
    n = 32
    b, rho, phys, fp = problem(oracle, n, seed=3)
    runs = {}
    for b16 in (0, 1):
        s = solver(stg, b, fp, n, tol=1e-10, basis16=b16)
        runs[b16] = s.solve()
        s.close()
    (p0, v0, st0), (p1, v1, st1) = runs[0], runs[1]
    assert st0["status"] == 0 and st1["status"] == 0
    assert st1["rel_residual"] <= 1e-10 and abs(st1["inner_iters"] - st0["inner_iters"]) <= 1
    for d in range(3):
        assert relerr(v1[d], v0[d]) < 1e-8
    assert relerr(pressure_free(p1), pressure_free(p0)) < 1e-8


def test_setup_overlapped_with_rhs_copy(oracle, stg):
    """stg_set_rhs runs a pending set-up (the penalty changed) while b is copied, and the
    next stg_solve uses it: the same kernels as a set-up inside stg_solve, so the same
    bits. The other order (b first, then the penalty) takes the set-up inside the solve."""
    n = 32
    b, rho, phys, fp = problem(oracle, n, seed=5)
    a = stg.Solver(n, tol=1e-10)
    a.set_boundary_from(b)
    a.set_penalty(np.zeros((n, n, n)), fp)
    a.set_rhs(b.cell_b, b.face_b)  # set-up here, overlapping the copy of b
    pa, va, sa = a.solve()
    c = stg.Solver(n, tol=1e-10)
    c.set_boundary_from(b)
    c.set_rhs(b.cell_b, b.face_b)
    c.set_penalty(np.zeros((n, n, n)), fp)  # set-up inside the solve
    pc, vc, sc = c.solve()
    assert sa["status"] == 0 and sa["inner_iters"] == sc["inner_iters"]
    assert np.array_equal(pa, pc)
    for d in range(3):
        assert np.array_equal(va[d], vc[d])
    # a changed penalty after set_rhs is not hidden by the overlapped set-up
    fp2 = [f * 3.0 for f in fp]
    a.set_penalty(np.zeros((n, n, n)), fp2)
    pa2, va2, sa2 = a.solve()
    d = solver(stg, b, fp2, n, tol=1e-10)
    pd, vd, sd = d.solve()
    assert sa2["inner_iters"] == sd["inner_iters"]
    for k in range(3):
        assert np.array_equal(va2[k], vd[k])


def test_learned_warm_start(oracle, stg):
    """warm_start 2: a warm-started solve first takes one FGMRES step whose preconditioner
    is the learned correction of the V-cycle (the step length minimises the residual), then
    continues as the plain warm start. It needs a network, counts as a learned iteration
    and reaches the tolerance and solution of the plain warm start."""
    n = 32
    b, rho, phys, fp = problem(oracle, n, seed=2)
    law = stg.alpha_bp(1e4)
    runs = {}
    for ws in (1, 2):
        s = stg.Solver(n, tol=1e-10, warm_start=ws)
        s.set_boundary_from(b)
        s.set_density(phys, law)
        s.set_rhs(b.cell_b, b.face_b)
        if ws == 2:
            with pytest.raises(stg.StgError):
                s.solve()  # no network yet
            s.net_init(7)
            s.net_train(300, lr=3e-4, seed=3)
        _, _, st = s.solve()
        assert st["learned_iters"] == 0  # a cold start takes no prediction step
        # the next design, close enough that the previous solution is kept as the start
        # (the penalty terms of this problem exceed b by about three orders, so a change of
        # 1e-3 in the density already leaves a residual above ||b|| and a zero start)
        s.set_density(np.clip(phys * (1.0 + 1e-5), 0.0, 1.0), law)
        runs[ws] = s.solve()
        s.close()
    (p1, v1, st1), (p2, v2, st2) = runs[1], runs[2]
    assert st2["status"] == 0 and st2["rel_residual"] <= 1e-10 and st2["learned_iters"] == 1
    assert st1["learned_iters"] == 0
    for d in range(3):
        assert relerr(v2[d], v1[d]) < 1e-8
    assert relerr(pressure_free(p2), pressure_free(p1)) < 1e-8
