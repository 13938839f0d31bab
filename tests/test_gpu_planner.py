"""Learned planner on the GPU: the network's own kernels against the CPU oracle, training on traces
of the single-query path, and what the trained network gains over the rule-based estimator."""
import sys
import time
from pathlib import Path

import numpy as np
import pytest

import rhydb_gpu as R

sys.path.insert(0, str(Path(__file__).resolve().parent.parent / "oracle"))
import mlp_oracle as M  # noqa: E402
from test_cpu_planner import random_case  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    """200,000 rows with amino-acid genes and metadata; 1,500 training and 400 held-out queries."""
    t = R.Table.generate(200000, seed=11, n_aa_genes=12, null_fraction=0.002)
    train_q = t.queries(1500, seed=12, use_aa=True, use_metadata=True)
    held_q = t.queries(400, seed=13, use_aa=True, use_metadata=True)
    dev = R.Device(t, 0)
    yield t, dev, train_q, held_q
    dev.close()


@pytest.mark.parametrize("n", [1, 64, 300])
def test_mlp_gradient_matches_oracle(setup, n):
    """Forward and backward kernels (BF16 weights, FP32 arithmetic) against the float64 oracle."""
    _, dev, _, _ = setup
    w, x, t = random_case(100 + n, n)
    g, loss, y = dev.mlp_gradient(w, x, t)
    oloss, og, oy = M.loss_and_grad(w, x, t)
    assert np.allclose(y, oy, rtol=1e-4, atol=1e-4)
    assert loss == pytest.approx(oloss, rel=1e-4)
    scale = np.abs(og).max()
    assert np.allclose(g, og, rtol=2e-3, atol=2e-5 * scale), np.abs(g - og).max() / scale


def test_planner_trains_and_gains(setup):
    t, dev, train_q, held_q = setup
    # held-out ground truth from a second device image, so none of it reaches the training pool
    probe = R.Device(t, 0)
    probe.planner_collect(held_q)
    hx, hy = probe.planner_samples()
    probe.close()
    added = dev.planner_collect(train_q)
    assert added > 5000
    st = dev.planner_train(epochs=80, batch=1024, lr=2e-3, seed=7)
    print("planner training:", st)
    assert st["accepted"] == 1
    assert st["qerr_learned_median"] <= st["qerr_rule_median"] * (1 + 1e-4)
    assert st["qerr_learned_p90"] < st["qerr_rule_p90"]
    # gain on held-out queries: selectivity q-error of the network vs the rule estimate over the
    # nodes the rule has to estimate (index scans are exact for both: their containers count them)
    sel, cost = dev.planner_predict(hx)
    truth = hy[:, 0].astype(np.float64)
    est = (hx[:, 0] < 0.5) & (hx[:, 1] < 0.5)
    q_learned = np.exp(np.abs(np.log(np.maximum(sel, 1e-7)) - truth))
    q_rule = np.exp(np.abs(hy[:, 2] - truth))
    assert np.allclose(q_learned[~est], q_rule[~est], rtol=1e-5)
    c_err = np.abs(np.log(cost) - hy[:, 1])
    print("held-out estimated nodes %d: q-error median learned %.3f rule %.3f; p90 learned %.3f rule %.3f; "
          "cost |ln err| median %.3f" % (est.sum(), np.median(q_learned[est]), np.median(q_rule[est]),
                                          np.percentile(q_learned[est], 90), np.percentile(q_rule[est], 90),
                                          np.median(c_err)))
    assert est.sum() > 200
    assert np.median(q_learned[est]) < np.median(q_rule[est])
    assert np.percentile(q_learned[est], 90) < np.percentile(q_rule[est], 90)
    # plans from both planners give identical results; the batch filter time is reported
    act = (np.arange(len(held_q)) % 4 == 3).astype(np.int32)
    res, times = {}, {}
    for mode in (0, 1):
        dev.planner_mode(mode)
        res[mode] = dev.batch(held_q, act)
        dev.batch_prepare(held_q, act)
        dev.batch_launch()
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            dev.batch_launch_parts(1)
        torch.cuda.synchronize()
        times[mode] = (time.perf_counter() - t0) / 5
    dev.planner_mode(0)
    assert np.array_equal(res[0][0], res[1][0])
    for i in res[0][1]:
        assert np.array_equal(res[0][1][i], res[1][1][i]), held_q[i]
    print("batch filter ms: rule-based %.3f learned %.3f" % (1000 * times[0], 1000 * times[1]))


def test_mode_requires_accepted_network():
    t = R.Table.generate(5000, seed=3)
    dev = R.Device(t, 0)
    with pytest.raises(R.RhyError):
        dev.planner_mode(1)
    dev.planner_mode(0)
    with pytest.raises(R.RhyError):
        dev.planner_train()  # no samples
    dev.close()


def test_model_trained_on_one_table_plans_another(setup):
    """Train on one table's traces, export, import into a device over a larger table with another
    seed, judge there on held-out queries, and plan: results are identical under both planners."""
    t, dev, train_q, _ = setup
    src = R.Device(t, 0)
    src.planner_collect(train_q)
    st = src.planner_train(epochs=80, batch=1024, lr=2e-3, seed=7)
    model = src.planner_export()
    src.close()
    assert model.accepted == st["accepted"] == 1
    big = R.Table.generate(400000, seed=21, n_aa_genes=12, null_fraction=0.002)
    dst = R.Device(big, 0)
    with pytest.raises(R.RhyError):
        dst.planner_mode(1)  # nothing trained here yet
    dst.planner_import(model)
    assert np.array_equal(dst.planner_weights(), np.ctypeslib.as_array(model.weights))
    held = big.queries(600, seed=22, use_aa=True, use_metadata=True)
    ev = dst.planner_evaluate(held)
    print("judged on the other table:", ev)
    assert ev["n_val"] > 3000
    assert np.isfinite(ev["qerr_learned_median"]) and np.isfinite(ev["qerr_rule_p90"])
    if ev["accepted"]:
        dst.planner_mode(1)
    else:
        with pytest.raises(R.RhyError):
            dst.planner_mode(1)
    act = (np.arange(len(held)) % 4 == 3).astype(np.int32)
    learned = dst.batch(held, act)
    dst.planner_mode(0)
    rule = dst.batch(held, act)
    assert np.array_equal(learned[0], rule[0])
    assert all(np.array_equal(learned[1][i], rule[1][i]) for i in rule[1])
    # a model whose verdict was negative cannot enable the learned mode
    model.accepted = 0
    dst.planner_import(model)
    with pytest.raises(R.RhyError):
        dst.planner_mode(1)
    bad = R.PlannerModel()
    with pytest.raises(R.RhyError):
        dst.planner_import(bad)  # zero deviations
    dst.close()
