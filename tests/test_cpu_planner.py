"""Planner on the CPU: the network oracle against finite differences and torch's BF16 rounding,
and the operator-node features."""
import sys
from pathlib import Path

import numpy as np
import pytest

import rhydb_gpu as R

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import mlp_oracle as M  # noqa: E402


def random_case(seed, n):
    rng = np.random.default_rng(seed)
    w = np.zeros(M.NPARAM, np.float32)
    w[M.W1:M.B1] = rng.normal(0, np.sqrt(2 / 24), M.B1 - M.W1)
    w[M.B1:M.W2] = rng.normal(0, 0.1, M.W2 - M.B1)
    w[M.W2:M.B2] = rng.normal(0, np.sqrt(2 / 64), M.B2 - M.W2)
    w[M.B2:M.W3] = rng.normal(0, 0.1, M.W3 - M.B2)
    w[M.W3:M.B3] = rng.normal(0, np.sqrt(2 / 64), M.B3 - M.W3)
    w[M.B3:] = rng.normal(0, 0.1, M.NPARAM - M.B3)
    x = rng.normal(0, 1, (n, 24)).astype(np.float32)
    t = rng.normal(0, 1, (n, 2)).astype(np.float32)
    return w, x, t


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    w, _, _ = random_case(1, 1)
    w = np.concatenate([w, np.array([1.00390625, 1.01171875, -2.5e-30, 3.0e38], np.float32)])
    ref = torch.from_numpy(w).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(M.to_bf16(w), ref)


def test_oracle_gradient_matches_finite_differences():
    w, x, t = random_case(2, 16)
    loss, g, _ = M.loss_and_grad(w, x, t)
    wb = M.to_bf16(w).astype(np.float64)
    assert abs(M.loss_of_bf16_weights(wb, x, t) - loss) < 1e-12
    rng = np.random.default_rng(3)
    for p in rng.choice(M.NPARAM, 300, replace=False):
        e = np.zeros(M.NPARAM)
        e[p] = 1e-6
        fd = (M.loss_of_bf16_weights(wb + e, x, t) - M.loss_of_bf16_weights(wb - e, x, t)) / 2e-6
        assert fd == pytest.approx(g[p], rel=1e-5, abs=1e-8), p


@pytest.fixture(scope="module")
def table():
    return R.Table.generate(20000, seed=5, n_aa_genes=12)


def test_features_are_finite_and_one_hot(table):
    qs = table.queries(60, seed=6, use_aa=True, use_metadata=True)
    for q in qs:
        x = table.plan_features(q)
        assert x.shape[1] == R.PLANNER_FEATURES and x.shape[0] >= 1
        assert np.isfinite(x).all()
        assert np.array_equal(x[:, :8].sum(1), np.ones(x.shape[0])), q
        assert (np.abs(x) <= 2.0).all(), q
        assert np.array_equal(x, table.plan_features(q))  # deterministic
