"""Serving loop: continuous batching gives every request the result it gets alone, admission
respects the device-memory budget, and user errors surface at submission."""
import threading

import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    t = R.Table.generate(300000, seed=21, n_aa_genes=12, null_fraction=0.002)
    qs = t.queries(240, seed=22, use_aa=True, use_metadata=True)
    # every 20th request filters by a MutationProfile (row-index pass before the filter programs)
    muts = "241:T,3037:T,14408:T,23403:G,28881:A"
    for j in range(0, len(qs), 20):
        d = (0, 2, 5, 30)[(j // 20) % 4]
        qs[j] = f"MutProfileMutations(main,{d},{muts})" if j % 40 else f"And({qs[j]},MutProfileMutations(main,{d},{muts}))"
    dev = R.Device(t, 0)
    rng = np.random.default_rng(23)
    acts = rng.choice([0, 1, 2], len(qs), p=[0.6, 0.25, 0.15])
    cols = rng.integers(0, t.n_seq, len(qs))
    props = rng.choice([0.0, 0.05, 0.5], len(qs))
    ks = rng.choice([1, 10, 1000, 5000], len(qs))
    yield t, dev, qs, acts, cols, props, ks
    dev.close()


def canon(res):
    return res["count"], tuple(map(tuple, res["rows"].tolist())), tuple(res["ids"].tolist())


def submit(srv, setup, i):
    _, _, qs, acts, cols, props, ks = setup
    return srv.submit(qs[i], int(acts[i]), int(cols[i]), float(props[i]), int(ks[i]))


def test_each_result_same_alone_and_in_the_mix(setup):
    t, dev, qs, acts, cols, props, ks = setup
    srv = R.Server(dev, max_batch=64, streams=3)
    alone = [canon(srv.result(submit(srv, setup, i))) for i in range(len(qs))]
    # the mix: four clients submit at once while earlier micro-batches are still on the device
    rids = [None] * len(qs)

    def client(part):
        for i in part:
            rids[i] = submit(srv, setup, i)

    threads = [threading.Thread(target=client, args=(range(j, len(qs), 4),)) for j in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    mixed = [canon(srv.result(rids[i])) for i in range(len(qs))]
    st = srv.stats()
    srv.stop()
    assert alone == mixed
    assert st["completed"] == 2 * len(qs) and st["rejected"] == 0
    assert st["batches"] < 2 * len(qs)  # requests were batched together
    assert 0 < st["p50_ms"] <= st["p99_ms"]
    # the results equal the batch path's and, for Details, the first ids of the row set
    counts, rows, begin, cnt = dev.batch_rows(qs, acts, cols, props)
    for i in range(len(qs)):
        c, r, ids = alone[i]
        assert c == counts[i], qs[i]
        if acts[i] == 1:
            want = rows[int(begin[i]):int(begin[i]) + int(cnt[i])]
            assert r == tuple(map(tuple, want.tolist())), qs[i]
        if acts[i] == 2:
            bits, n = dev.compute_filter(qs[i])
            assert n == c
            assert ids == tuple(R.bits_to_rows(bits)[:int(ks[i])].tolist()), qs[i]


@pytest.fixture(scope="module")
def oracle_results(setup):
    """The oracle's answer to every request of the mix: its count, its Mutations rows and its first
    k row ids."""
    t, dev, qs, acts, cols, props, ks = setup
    orc = oracle_for(t)
    mut = [i for i in range(len(qs)) if acts[i] == 1]
    counts, tables = orc.check_batch(qs, cols, tables=mut)
    out = []
    for i in range(len(qs)):
        rows = tuple(orc.mutation_rows(int(cols[i]), tables[i], float(props[i]))) if acts[i] == 1 else ()
        ids = ()
        if acts[i] == 2:
            bits, _ = orc.compute_filter(qs[i])
            ids = tuple(R.bits_to_rows(bits)[:int(ks[i])].tolist())
        out.append((int(counts[i]), rows, ids))
    return out


def canon_rows(res):
    rows = tuple((int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
                  float(r["proportion"])) for r in res["rows"])
    return res["count"], rows, tuple(res["ids"].tolist())


def test_served_results_equal_the_oracle(setup, oracle_results):
    """Counts, Mutations rows and Details ids served by continuous batching and by the plain arm
    (one request at a time through the single-query path) equal the oracle's."""
    t, dev, qs, acts, cols, props, ks = setup
    for plain in (False, True):
        srv = R.Server(dev, max_batch=64, streams=3, plain=plain)
        rids = [submit(srv, setup, i) for i in range(len(qs))]
        got = [canon_rows(srv.result(r)) for r in rids]
        st = srv.stats()
        srv.stop()
        for i in range(len(qs)):
            assert got[i] == oracle_results[i], (plain, qs[i], acts[i])
        assert st["completed"] == len(qs)
        if plain:
            assert st["batches"] == len(qs)  # no batching


def test_cancel_and_timeout(setup):
    """Requests queued behind others report RHY_TIMEOUT for a wait that runs out; cancelled requests
    report RHY_CANCELLED and the others complete with their own results."""
    t, dev, qs, acts, cols, props, ks = setup
    srv = R.Server(dev, max_batch=4, streams=1)
    mut = [i for i in range(len(qs)) if acts[i] == 1]
    order = (mut * 4)[:200]
    rids = [srv.submit(qs[i], 1, int(cols[i]), 0.05) for i in order]
    with pytest.raises(R.RhyError) as e:
        srv.result(rids[-1], timeout_ms=0)
    assert e.value.code == 6
    cancelled = [srv.cancel(r) for r in rids[100:]]
    assert any(cancelled)
    for j, r in enumerate(rids):
        if j >= 100 and cancelled[j - 100]:
            with pytest.raises(R.RhyError) as e:
                srv.result(r)
            assert e.value.code == 7
        else:
            assert srv.result(r)["count"] == dev.count(qs[order[j]])
    st = srv.stats()
    srv.stop()
    assert st["cancelled"] == sum(cancelled)
    assert st["completed"] + st["cancelled"] == len(rids)


def test_admission_by_device_memory(setup):
    t, dev, qs, acts, cols, props, ks = setup
    budget = 12 << 20  # a few Mutations queries at a time
    srv = R.Server(dev, max_batch=256, streams=3, memory_budget=budget)
    mut = [i for i in range(len(qs)) if acts[i] == 1][:40]
    rids = [srv.submit(qs[i], 1, int(cols[i]), 0.05) for i in mut]
    res = [srv.result(r) for r in rids]
    st = srv.stats()
    assert st["completed"] == len(mut)
    assert st["budget_bytes"] == budget and 0 < st["peak_bytes"] <= budget
    assert st["batches"] > 1  # the budget split the requests
    counts, rows, begin, cnt = dev.batch_rows([qs[i] for i in mut], [1] * len(mut), [int(cols[i]) for i in mut])
    for j, i in enumerate(mut):
        assert res[j]["count"] == counts[j]
    # a request larger than the whole budget is refused at submission
    tiny = R.Server(dev, memory_budget=1 << 16)
    with pytest.raises(R.RhyError):
        tiny.submit(qs[mut[0]], 1, 0, 0.05)
    tiny.stop()
    srv.stop()


def test_user_errors_surface_at_submit(setup):
    _, dev, qs, _, _, _, _ = setup
    srv = R.Server(dev)
    with pytest.raises(R.IllegalQuery):
        srv.submit("SymEq(main,99999999,A)")
    with pytest.raises(R.RhyError):
        srv.submit(qs[0], action=7)
    with pytest.raises(R.RhyError):
        srv.submit(qs[0], action=1, min_proportion=2.0)
    r = srv.result(srv.submit(qs[0]))
    assert r["count"] == dev.count(qs[0])
    srv.stop()
