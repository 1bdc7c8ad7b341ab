"""GPU checks of the learned preconditioner through the C ABI.

* forward pass, loss and every parameter gradient of the network against the CPU oracle
  (oracle/unet_oracle.py, which mirrors the GPU's bfloat16 rounding points and accumulates
  in FP64): outputs and loss within 1e-2 relative L2, each parameter block's gradient
  within 5e-2 (bfloat16 activations and gradients carry 8 significant bits, so a rounding
  flip between the FP32 GPU sums and the FP64 oracle sums moves a value by 2^-8 relative;
  the flips compound through the backward pass, and the gradients of the coarsest level
  sum over only n^3/64 cells, 64 at n = 16);
* one Adam step against the oracle's restatement with the GPU's own gradient (1e-6);
* training on the solver's own operator lowers the loss below the loss of the zero
  correction, i.e. the trained network removes part of the error a V-cycle leaves;
* the LEARNED method reaches the same FP64 tolerance and solution as PLAIN in fewer
  V-cycles.
"""
import numpy as np
import pytest

from oracle import unet_oracle as U
from tests.helpers import problem, relerr

pytestmark = pytest.mark.gpu


def net_handle(capi, n=16, seed=5):
    s = capi.Solver(n)
    s.net_init(seed)
    return s


def rand_io(n, seed):
    rng = np.random.default_rng(seed)
    inp = rng.normal(size=(n ** 3, U.IN_USED)).astype(np.float32)
    inp[:, 0] = rng.uniform(0, 1, n ** 3)
    tgt = rng.normal(size=(n ** 3, 4)).astype(np.float32)
    return inp, tgt


@pytest.mark.parametrize("n", [8, 12, 16, 32])
def test_forward_backward_matches_oracle(stg, n):
    # n = 8 runs every convolution on the mma.sync kernel; larger grids run the tcgen05
    # kernel wherever its tile plan fits (n >= 12) and mma.sync on the coarser levels
    s = net_handle(stg)
    p = s.net_params()
    L = U.layout()
    # non-zero biases and head so every parameter block carries signal
    rng = np.random.default_rng(11)
    for l in range(U.NCONV):
        p[L["boff"][l]:L["boff"][l] + L["cout"][l]] = rng.uniform(-0.05, 0.05, L["cout"][l])
    p[L["hb"]:L["hb"] + 4] = rng.uniform(-0.1, 0.1, 4)
    p[L["kappa"]] = 1.0
    s.net_set_params(p)
    inp, tgt = rand_io(n, 3 + n)
    out, loss, grad = s.net_forward_backward(n, inp, tgt)
    ref = U.forward_backward(p.astype(np.float64), inp, tgt, bf=True)
    assert relerr(out, ref["out"]) < 1e-2
    assert abs(loss - ref["loss"]) <= 1e-2 * ref["loss"]
    blocks = [(L["woff"][l], L["boff"][l]) for l in range(U.NCONV)]
    blocks += [(L["boff"][l], L["boff"][l] + L["cout"][l]) for l in range(U.NCONV)]
    blocks += [(L["hw"], L["hb"]), (L["hb"], L["kappa"])]
    for a, b in blocks:
        g, r = grad[a:b], ref["grad"][a:b]
        assert np.linalg.norm(r) > 0, (a, b)
        assert relerr(g, r) < 5e-2, (a, b, relerr(g, r))
    assert grad[L["kappa"]] == 0
    # forward only gives the same output
    out2, _, _ = s.net_forward_backward(n, inp)
    assert np.array_equal(out, out2)


def test_adam_step_matches_oracle(stg):
    s = net_handle(stg)
    p0 = s.net_params().astype(np.float64)
    inp, tgt = rand_io(8, 1)
    m = np.zeros_like(p0)
    v = np.zeros_like(p0)
    p = p0
    for t in range(1, 4):
        _, _, g = s.net_forward_backward(8, inp, tgt)
        s.net_adam_step(1e-3)
        p, m, v = U.adam(p, g.astype(np.float64), m, v, t, 1e-3)
        got = s.net_params()
        assert np.max(np.abs(got - p)) < 1e-6 * max(1.0, np.max(np.abs(p)))
    assert np.max(np.abs(p - p0)) > 1e-4


def setup_problem(po, capi, n, method):
    b, rho, phys, fp = problem(po, n, seed=2)
    s = capi.Solver(n, method=method)
    s.set_boundary_from(b)
    s.set_density(phys, capi.alpha_bp(1e4))
    s.set_rhs(b.cell_b, b.face_b)
    return s


def test_training_removes_error_left_by_the_vcycle(oracle, stg):
    n = 32
    s = setup_problem(oracle, stg, n, stg.STG_METHOD_PLAIN)
    s.net_init(7)
    losses = s.net_train(1200, lr=3e-4, seed=3)
    assert np.all(np.isfinite(losses))
    # the target is (e - M A e) / (kappa rms(r1)) with kappa fixed from the first pair, so
    # the zero correction scores about 1: the trained network must do clearly better
    first, last = float(np.mean(losses[:20])), float(np.mean(losses[-50:]))
    assert last < 0.6 * first, (first, last)
    assert last < 0.7, last


def test_learned_solve_matches_plain(oracle, stg):
    n = 32
    s = setup_problem(oracle, stg, n, stg.STG_METHOD_LEARNED)
    with pytest.raises(stg.StgError):
        s.solve()  # no network yet
    s.net_init(7)
    s.net_train(1200, lr=3e-4, seed=3)
    p1, v1, st1 = s.solve()
    assert st1["rel_residual"] <= 1e-8 and st1["learned_iters"] > 0
    s.set_method(stg.STG_METHOD_PLAIN)
    p0, v0, st0 = s.solve()
    assert st0["learned_iters"] == 0
    for a, b in zip(v1, v0):
        assert relerr(a, b) < 1e-6
    # what the trained network gains: fewer V-cycles to the same tolerance (10-11 against
    # 16 on this problem)
    assert st1["inner_iters"] < st0["inner_iters"], (st1, st0)
