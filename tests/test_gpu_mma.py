"""The GPU MMA update (stg_mma_update) against the reference MMA solver's fixture
(tests/golden/ref_mma.npz: six updates made by the reference's own simplex/ext/mma code)
and against the oracle MMA on a fresh problem, in 2D and 3D handles. Tolerance 1e-9 on
the designs (the GPU sums the dual reductions in a different order)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("dim,n", [(2, 64), (3, 16)])
def test_mma_matches_reference_fixture(stg, dim, n):
    g = np.load(os.path.join(GOLD, "ref_mma.npz"))
    s = stg.Solver(n, dim=dim)
    x = np.full((n,) * dim, 0.3)
    for k, df in enumerate(g["dfdx"]):
        x, ch = s.mma_update(x, df.reshape(x.shape), 0.3)
        assert np.max(np.abs(x.ravel() - g["x"][k])) < 1e-9, k
        prev = g["x"][k - 1] if k else np.full(x.size, 0.3)
        assert abs(ch - np.max(np.abs(g["x"][k] - prev))) < 1e-9


def test_mma_matches_oracle_and_reset(oracle, stg):
    n = 32
    rng = np.random.default_rng(3)
    s = stg.Solver(n, dim=3)
    for run in range(2):
        if run:
            s.mma_reset()
        o = oracle.Mma(n ** 3)
        x = np.full((n, n, n), 0.2)
        xo = x.ravel().copy()
        for k in range(4):
            df = -np.abs(rng.standard_normal((n, n, n))) * (0.5 + rng.random((n, n, n)))
            x, _ = s.mma_update(x, df, 0.2)
            g = 1e4 * (xo.mean() - 0.2)
            o.update(xo, df, g, np.full(xo.size, 1e4 / xo.size), np.maximum(0.01, xo - 0.2), np.minimum(1.0, xo + 0.2))
            assert np.max(np.abs(x.ravel() - xo)) < 1e-9, (run, k)
