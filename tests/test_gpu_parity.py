"""Bit-exact parity of the CUDA path (through the C-ABI) with the CPU oracle."""
import numpy as np
import pytest

import rhydb_gpu as R
import semantic
import workloads
import oracle as oracle_mod
from rawtable import RawBuilder, oracle_for

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def config1():
    """100,000 sequences over a 29,903-nt genome, nucleotide leaves only, 1,000 trees of depth <= 4
    with NOf(n <= 8) (the small configuration of the plain method)."""
    t = R.Table.generate(100000, seed=42)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    yield t, orc, dev, t.queries(1000, seed=43, max_depth=4, max_nof_children=8)
    dev.close()


@pytest.fixture(scope="module")
def config2_small():
    """The at-scale generator (12 amino-acid genes, metadata, null rows) at 100,000 rows."""
    t = R.Table.generate(100000, seed=7, n_aa_genes=12, null_fraction=0.003)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    yield t, orc, dev, t.queries(300, seed=8, use_aa=True, use_metadata=True)
    dev.close()


def check_filter(dev, orc, q):
    bits, n = dev.compute_filter(q)
    obits, on = orc.compute_filter(q)
    assert n == on, q
    assert np.array_equal(bits, obits), q


def test_config1_filters_and_counts(config1):
    t, orc, dev, qs = config1
    for q in qs:
        check_filter(dev, orc, q)
        assert dev.count(q) == orc.count(q)


def test_config1_mutations(config1):
    t, orc, dev, qs = config1
    for q in qs[:200]:
        m, n = dev.mutations(q, 0)
        om, on = orc.mutations(q, 0)
        assert n == on and np.array_equal(m, om), q
        assert t.mutation_rows(0, m, 0.05) == orc.mutation_rows(0, om, 0.05)


def test_config1_batched(config1):
    t, orc, dev, qs = config1
    act = np.array([1 if i % 5 == 0 else 0 for i in range(len(qs))], np.int32)
    counts, muts = dev.batch(qs, act)
    for i, q in enumerate(qs):
        assert counts[i] == orc.count(q), q
    for i in np.flatnonzero(act)[:120]:
        om, _ = orc.mutations(qs[i], 0)
        assert np.array_equal(muts[int(i)], om), qs[i]


def test_config2_all_columns(config2_small):
    t, orc, dev, qs = config2_small
    for q in qs:
        check_filter(dev, orc, q)
    rng = np.random.default_rng(3)
    for q in qs[:60]:
        col = int(rng.integers(0, t.n_seq))
        m, n = dev.mutations(q, col)
        om, on = orc.mutations(q, col)
        assert n == on and np.array_equal(m, om), (q, col)


def test_config2_batched_mixed_columns(config2_small):
    t, orc, dev, qs = config2_small
    rng = np.random.default_rng(4)
    act = (rng.random(len(qs)) < 0.35).astype(np.int32)
    col = rng.integers(0, t.n_seq, len(qs)).astype(np.uint32)
    for tb in (4096, 16384, 65536):
        counts, muts = dev.batch(qs, act, col, tile_bits=tb)
        for i, q in enumerate(qs):
            assert counts[i] == orc.count(q), (tb, q)
        for i in np.flatnonzero(act)[:40]:
            om, _ = orc.mutations(qs[i], int(col[i]))
            assert np.array_equal(muts[int(i)], om), (tb, qs[i], col[i])


def test_batched_mutation_rows(config2_small):
    """The Mutations output computed on the device (rhy_batch_rows) equals the host conversion of
    the dense counts, which equals the oracle's, row for row and bit for bit in the proportions."""
    t, orc, dev, qs = config2_small
    rng = np.random.default_rng(5)
    act = (rng.random(len(qs)) < 0.5).astype(np.int32)
    col = rng.integers(0, t.n_seq, len(qs)).astype(np.uint32)
    props = rng.choice([0.0, 0.05, 0.3, 1.0], len(qs))
    # a small buffer exercises the refetch of rows that did not fit
    counts, rows, begin, cnt = dev.batch_rows(qs, act, col, props, rows_cap=1000)
    dcounts, muts = dev.batch(qs, act, col)
    assert np.array_equal(counts, dcounts)
    assert len(rows) > 1000
    for i in range(len(qs)):
        if act[i] == 0:
            assert cnt[i] == 0
            continue
        got = rows[int(begin[i]):int(begin[i]) + int(cnt[i])]
        want = t.mutation_rows(int(col[i]), muts[i], float(props[i]))
        assert [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
                 float(r["proportion"])) for r in got] == want, (qs[i], props[i])
    for i in np.flatnonzero(act)[:12]:
        om, _ = orc.mutations(qs[i], int(col[i]))
        assert orc.mutation_rows(int(col[i]), om, float(props[i])) == t.mutation_rows(int(col[i]), muts[int(i)],
                                                                                      float(props[i]))
    with pytest.raises(R.RhyError):
        dev.batch_rows(qs[:4], [1, 1, 0, 0], None, [0.05, 1.5, 0.05, 0.05])


@pytest.mark.parametrize("heavy", [0.12, 0.5])
def test_batch_rows_in_parts(config2_small, heavy):
    """A batch run in parts (Mutations and Details first, about 256 at a time, then the counts,
    each planned while the earlier parts run) gives every query the counts and rows of the
    single-part dense batch, and a refetch returns the rows of every part."""
    t, orc, dev, qs = config2_small
    big = (qs * 6)[:1700]
    rng = np.random.default_rng(11)
    act = np.where(rng.random(len(big)) < heavy, 1, np.where(rng.random(len(big)) < 0.05, 2, 0)).astype(np.int32)
    col = rng.integers(0, t.n_seq, len(big)).astype(np.uint32)
    counts, rows, begin, cnt = dev.batch_rows(big, act, col, None, rows_cap=10)
    dense_act = np.where(act == 2, 0, act).astype(np.int32)
    dcounts, muts = dev.batch(big, dense_act, col)
    assert np.array_equal(counts, dcounts)
    assert int(cnt.sum()) == len(rows)
    ranges = sorted((int(begin[i]), int(cnt[i])) for i in range(len(big)) if cnt[i])
    assert all(a + n <= b for (a, n), (b, _) in zip(ranges, ranges[1:]))  # disjoint
    for i in range(len(big)):
        if act[i] != 1:
            assert cnt[i] == 0
            continue
        got = rows[int(begin[i]):int(begin[i]) + int(cnt[i])]
        want = t.mutation_rows(int(col[i]), muts[i], 0.05)
        assert [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
                 float(r["proportion"])) for r in got] == want, big[i]
    times = dev.batch_times()
    assert all(v >= 0 for v in times.values())


def test_autotuned_schedule_keeps_results(config2_small):
    """The autotuner times all 36 candidate schedules, keeps the fastest in force, and every
    schedule gives the same counts and Mutations tables."""
    t, orc, dev, qs = config2_small
    act = np.array([i % 4 == 3 for i in range(len(qs))], np.int32)
    default = dev.batch_schedule()
    ref_c, ref_m = dev.batch(qs, act)
    tried = dev.batch_autotune(qs, act, reps=3)
    assert len(tried) == 36
    assert all(np.isfinite(ms) and ms > 0 for _, ms in tried)
    assert [ms for _, ms in tried] == sorted(ms for _, ms in tried)
    assert dev.batch_schedule() == tried[0][0]
    for sch in (tried[0][0], tried[-1][0], dict(max_tile_bits=16384, stack_kb=24, ctas_per_sm=2, query_major=1)):
        dev.batch_schedule(**sch)
        c, m = dev.batch(qs, act)
        assert np.array_equal(c, ref_c)
        assert all(np.array_equal(m[k], ref_m[k]) for k in ref_m)
    with pytest.raises(R.RhyError):
        dev.batch_schedule(max_tile_bits=3000)
    dev.batch_schedule(**default)


@pytest.mark.parametrize("limit", ["dense", "sparse", "default"])
def test_row_index_and_dense_passes_agree(config2_small, limit):
    """Mutations counts from the row index (every filtered row adds its entries), from the dense
    passes over every container, and from the default split by filter size are the oracle's, for
    single queries and batch slots over every column (empty and full filters included)."""
    t, orc, dev, qs = config2_small
    default = dev.sparse_rows()
    lim = {"dense": (0, 0), "sparse": (t.n_rows, t.n_rows), "default": default}[limit]
    dev.sparse_rows(*lim)
    try:
        extra = ["True", "False", "SymEq(main,1,N)", "Not(HasMut(main,5))"]
        sample = qs[:40] + extra
        rng = np.random.default_rng(9)
        col = rng.integers(0, t.n_seq, len(sample)).astype(np.uint32)
        for q, c in zip(sample, col):
            m, n = dev.mutations(q, int(c))
            om, on = orc.mutations(q, int(c))
            assert n == on and np.array_equal(m, om), (limit, q, c)
        act = np.ones(len(sample), np.int32)
        counts, muts = dev.batch(sample, act, col)
        for i, q in enumerate(sample):
            om, on = orc.mutations(q, int(col[i]))
            assert counts[i] == on and np.array_equal(muts[i], om), (limit, q, col[i])
    finally:
        dev.sparse_rows(*default)
    assert default == (t.n_rows // 32, t.n_rows // 64)


def test_tile_widths(config2_small):
    t, orc, dev, qs = config2_small
    for tb in (4096, 8192, 32768, 65536):
        dev.set_tile_bits(tb)
        for q in qs[:80]:
            check_filter(dev, orc, q)
    dev.set_tile_bits(16384)


def test_graph_replay_matches_direct(config2_small):
    t, orc, dev, qs = config2_small
    act = np.array([i % 3 == 0 for i in range(len(qs))], np.int32)
    direct_c, direct_m = dev.batch(qs, act)
    dev.batch_prepare(qs, act)
    dev.batch_capture()
    for _ in range(2):
        dev.batch_replay()
    c, m = dev.batch_results()
    assert np.array_equal(c, direct_c)
    assert all(np.array_equal(m[k], direct_m[k]) for k in direct_m)


@pytest.mark.parametrize("rows", [1, 31, 65536, 65537, 131072])
def test_chunk_boundaries(rows):
    t = R.Table.generate(rows, seed=rows, genome_len=2000, pool_sites=200, n_aa_genes=1, null_fraction=0.05)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    qs = t.queries(60, seed=1, use_aa=True, use_metadata=True) + ["True", "False", "Not(True)", "NOf(0,exactly)"]
    for q in qs:
        check_filter(dev, orc, q)
    for q in qs[:15]:
        for col in range(t.n_seq):
            m, n = dev.mutations(q, col)
            om, on = orc.mutations(q, col)
            assert n == on and np.array_equal(m, om), (q, col)
    assert dev.count("True") == rows
    dev.close()


def test_wide_and_deep_trees(config1):
    t, orc, dev, qs = config1
    leaves = [q for q in qs if q.startswith("SymEq") or q.startswith("HasMut")][:64]
    assert len(leaves) >= 40
    k = len(leaves)
    exprs = [
        "And(" + ",".join(leaves) + ")",
        "Or(" + ",".join(leaves) + ")",
        f"NOf({k // 2},atleast," + ",".join(leaves) + ")",
        f"NOf(3,exactly," + ",".join(leaves) + ")",
        f"NOf({k - 1},atleast," + ",".join("Not(" + x + ")" for x in leaves) + ")",
        f"Maybe(NOf(2,exactly," + ",".join(leaves[:10]) + "))",
    ]
    nested = leaves[0]
    for x in leaves[1:24]:
        nested = f"Or(Not(And({nested},{x})),NOf(1,exactly,{x},{nested}))" if len(nested) < 3000 else nested
    exprs.append(nested)
    for q in exprs:
        check_filter(dev, orc, q)
    counts, _ = dev.batch(exprs)
    assert counts.tolist() == [orc.count(q) for q in exprs]


def test_complement_identity_at_scale():
    """At 2,000,000 rows: Count(X) + Count(Not X) == rows, batched == plain, and a few queries
    against the oracle."""
    t = R.Table.generate(2000000, seed=42, n_aa_genes=12)
    dev = R.Device(t, 0)
    qs = t.queries(64, seed=43, use_aa=True, use_metadata=True)
    plain = [dev.count(q) for q in qs]
    neg = [dev.count(f"Not({q})") for q in qs]
    assert all(a + b == t.n_rows for a, b in zip(plain, neg))
    act = np.array([i % 4 == 3 for i in range(len(qs))], np.int32)
    counts, muts = dev.batch(qs, act)
    assert counts.tolist() == plain
    for i in np.flatnonzero(act)[:6]:
        m, _ = dev.mutations(qs[i], 0)
        assert np.array_equal(m, muts[int(i)])
        # every covered, filtered row holds exactly one symbol per position
        assert int(m.sum(axis=0).max()) <= plain[int(i)]
    # MutationProfile at scale: row sets grow with the distance, the source row of the profile is
    # within its 20 substitutions, every row is within the genome's length, batched == plain
    seq = workloads.profile_query_sequence(t, row=123457, substitutions=20, seed=17)
    prev, sets = None, []
    for d in (0, 20, 50, 100, 200, t.columns[0].L):
        bits, n = dev.compute_filter(f"MutProfile(main,{d},{seq})")
        if prev is not None:
            assert np.array_equal(prev & bits, prev), d
        prev = bits
        sets.append(n)
        if d == 20:
            assert (bits[123457 // 32] >> (123457 % 32)) & 1
    assert sets == sorted(sets) and sets[-1] == t.n_rows
    pq = [f"MutProfile(main,{d},{seq})" for d in (0, 20, 50, 100, 200)]
    counts, _ = dev.batch(pq, np.zeros(len(pq), np.int32))
    assert counts.tolist() == sets[:-1]
    orc = oracle_for(t)
    for q in qs[:3]:
        check_filter(dev, orc, q)
    check_filter(dev, orc, pq[0])
    m, _ = dev.mutations(qs[3], 0)
    om, _ = orc.mutations(qs[3], 0)
    assert np.array_equal(m, om)
    dev.close()


def test_batching_shapes_in_one_captured_launch():
    """The batching shape: 4,096 trees of 1-64 leaves (NOf up to 64 children) with selectivities
    log-uniform over [1e-5, 0.9], evaluated by the persistent kernels inside one captured CUDA graph,
    bit-exact with the oracle for every query (counts) and for a sample of Mutations tables."""
    import re

    import workloads

    t = R.Table.generate(100000, seed=42, n_aa_genes=12, null_fraction=0.002)
    dev = R.Device(t, 0)
    qs = workloads.batching_workload(t, dev, n=4096, seed=44, candidates=40000)
    leaves = np.array([len(re.findall(r"SymEq|HasMut|StrEq|DateBetween", q)) for q in qs])
    assert leaves.min() >= 1 and leaves.max() <= 64 and (leaves == 64).sum() > 100
    assert max(len(re.findall(r",", q)) for q in qs if q.startswith("NOf")) > 40
    act = np.array([i % 8 == 7 for i in range(len(qs))], np.int32)
    dev.batch_prepare(qs, act)
    dev.batch_capture()
    dev.batch_replay()
    counts, muts = dev.batch_results()
    sel = counts / t.n_rows
    decades = np.histogram(np.log10(sel), bins=[-5, -4, -3, -2, -1, np.log10(0.9)])[0]
    assert decades.min() >= 600, decades   # log-uniform: about 820 per decade
    orc = oracle_for(t)
    import os

    _, _, want = orc.run_batch(qs, [0] * len(qs), [0] * len(qs), os.cpu_count() or 4)
    assert np.array_equal(counts, want)
    for i in np.flatnonzero(act)[::64]:
        om, _ = orc.mutations(qs[i], 0)
        assert np.array_equal(muts[int(i)], om), qs[i]
    dev.close()


def _expected_aggregation(t, orc, expr, dims):
    """The reference's grouping restated on the oracle: a sequence dimension's group of a row is the
    symbol c for which And(filter, SymEq(col, pos, c)) holds it (compileSymbolInSet for {c}), null
    rows last; a dictionary dimension's group is the row's value, values in string order, null last;
    combinations in depth-first (lexicographic group) order."""
    import ctypes as C

    bits, n = orc.compute_filter(expr)
    rows = R.bits_to_rows(bits)
    raw = t.raw()
    gid = {int(g): i for i, g in enumerate(rows)}
    per_dim = []
    for d in dims:
        g = np.full(len(rows), -2, np.int64)
        if d[0] == "seq":
            col = t.columns[d[1]]
            for s, ch in enumerate(col.symbols):
                b, _ = orc.compute_filter(f"And({expr},SymEq({col.name},{d[2]},{ch}))")
                for r in R.bits_to_rows(b):
                    assert g[gid[int(r)]] == -2, "symbol groups overlap"
                    g[gid[int(r)]] = s
            nulls = np.ctypeslib.as_array(C.cast(raw.seq[d[1]].is_null, C.POINTER(C.c_uint8)), shape=(t.n_rows,))
            order = list(range(col.n_symbols)) + [-1]
            labels = {s: col.symbols[s] for s in range(col.n_symbols)}
        else:
            rc = raw.dict[d[1]]
            ids = np.ctypeslib.as_array(C.cast(rc.ids, C.POINTER(C.c_uint32)), shape=(t.n_rows,))
            values = [rc.values[i].decode() for i in range(rc.n_values)]
            order = sorted(range(len(values)), key=lambda i: values[i]) + [-1]
            labels = {i: values[i] for i in range(len(values))}
            nulls = (ids == 0xFFFFFFFF).astype(np.uint8)
        for k, r in enumerate(rows):
            i = (int(r) >> 16) * 65536 + (int(r) & 0xFFFF)  # raw row index = chunk * 2^16 + row
            if d[0] == "seq":
                if nulls[i]:
                    assert g[k] == -2
                    g[k] = -1
            else:
                g[k] = -1 if nulls[i] else int(ids[i])
        assert (g != -2).all(), "every filtered row falls in one group"
        per_dim.append((g, {v: j for j, v in enumerate(order)}, labels))
    combos = {}
    for k in range(len(rows)):
        key = tuple(pd[1][int(pd[0][k])] for pd in per_dim)
        combos[key] = combos.get(key, 0) + 1
    out = []
    for key in sorted(combos):
        lab = []
        for j, pd in enumerate(per_dim):
            inv = {v: kk for kk, v in pd[1].items()}
            gg = inv[key[j]]
            lab.append(None if gg == -1 else pd[2][gg])
        out.append((tuple(lab), combos[key]))
    return out, n


def test_aggregation_matches_the_oracle(config2_small):
    """BitmapAggregation over sequence positions (nucleotide and amino-acid, pool sites and N runs)
    and dictionary columns, one to three dimensions, against the oracle's row sets."""
    t, orc, dev, qs = config2_small
    names = [c.name for c in t.columns]
    aa = names.index("S") if "S" in names else 1
    cases = [
        ("True", [("seq", 0, 1)]),
        (qs[0], [("seq", 0, 21618)]),
        (qs[1], [("seq", 0, 3037), ("dict", 0)]),
        (qs[2], [("dict", 1), ("seq", aa, 5)]),
        (qs[3], [("seq", 0, 241), ("seq", 0, 14408), ("dict", 0)]),
        ("Not(HasMut(main,23403))", [("seq", 0, 23403)]),
        ("False", [("seq", 0, 100)]),
    ]
    for expr, dims in cases:
        got, n = dev.aggregate(expr, dims)
        want, on = _expected_aggregation(t, orc, expr, dims)
        assert n == on, expr
        assert got == want, (expr, dims)
        assert sum(c for _, c in got) == n
    with pytest.raises(R.RhyError):
        dev.aggregate("True", [("seq", 0, 0)])
    with pytest.raises(R.RhyError):
        dev.aggregate("True", [("seq", 0, t.columns[0].L + 1)])
    with pytest.raises(R.RhyError):
        dev.aggregate("True", [("dict", 99)])


@pytest.fixture(scope="module")
def profile_table():
    """70,000 rows over a 600-nt genome with null rows; the row-level semantics for the profiles."""
    t = R.Table.generate(70000, seed=3, genome_len=600, pool_sites=120, n_aa_genes=2, null_fraction=0.002)
    raw = t.raw()
    orc = oracle_for(t, raw)
    dev = R.Device(t, 0)
    yield t, orc, dev, semantic.from_raw(raw)
    dev.close()


def test_mutation_profile(profile_table):
    """MutationProfile row sets (one pass over the row index) against the oracle's rewrite into
    Not(NOf(distance + 1, SymbolInSet per position)), alone, nested and in a batch."""
    t, orc, dev, sem = profile_table
    qs = semantic.profile_queries(sem, np.random.default_rng(3))
    for q in qs:
        check_filter(dev, orc, q)
        assert dev.count(q) == orc.count(q), q[:80]
    for q in (qs[1], qs[-1]):
        m, n = dev.mutations(q, 0)
        om, on = orc.mutations(q, 0)
        assert n == on and np.array_equal(m, om), q[:80]
    two = f"Or({qs[0]},{qs[5]})"  # two profiles in one program
    check_filter(dev, orc, two)
    mixed = qs + [two] + t.queries(40, seed=9, use_aa=True, use_metadata=True)
    act = np.array([1 if i % 3 == 1 else 0 for i in range(len(mixed))], np.int32)
    counts, muts = dev.batch(mixed, act)
    for i, q in enumerate(mixed):
        assert counts[i] == orc.count(q), q[:80]
    for i in np.flatnonzero(act):
        om, _ = orc.mutations(mixed[i], 0)
        assert np.array_equal(muts[int(i)], om), mixed[i][:80]
    L = len(sem.cols["main"].reference)
    for bad in (f"MutProfile(main,1,{'A' * (L - 1)})", f"MutProfile(main,1,{'A' * (L - 1)}!)",
                f"MutProfileMutations(main,1,{L + 1}:A)", "MutProfileMutations(main,-1,3:A)",
                "MutProfileMutations(nosuch,1,3:A)", "MutProfileMutations(main,1,3:J)"):
        with pytest.raises(R.RhyError):
            dev.count(bad)


def test_mutation_profile_full_genome(config2_small):
    """Profiles over the 29,903-nt genome and an amino-acid gene, distances 0, 5, 50 and 200."""
    t, orc, dev, _ = config2_small
    raw = t.raw()
    rng = np.random.default_rng(11)
    ref = raw.seq[0].reference[: raw.seq[0].L].decode()
    L = len(ref)
    muts = ",".join(f"{p + 1}:{'ACGTN-'[p % 6]}" for p in sorted(rng.choice(L, 25, replace=False)))
    prof = list(ref)
    for p in rng.choice(L, 40, replace=False):
        prof[p] = "ACGTNRY-"[rng.integers(8)]
    aa = raw.seq[1].name.decode()
    qs = [f"MutProfileMutations(main,{d},{muts})" for d in (0, 5, 50, 200)]
    qs += [f"MutProfile(main,{d},{''.join(prof)})" for d in (0, 5, 50)]
    qs += [f"MutProfileMutations({aa},2,3:X,10:K,11:*)", f"And(HasMut(main,241),MutProfileMutations(main,5,{muts}))"]
    want = []
    for q in qs:  # the oracle's NOf over ~30,000 children takes seconds: one call per query
        bits, n = dev.compute_filter(q)
        obits, on = orc.compute_filter(q)
        assert n == on and np.array_equal(bits, obits), q[:80]
        want.append(on)
    act = np.array([1 if i in (1, 5) else 0 for i in range(len(qs))], np.int32)
    counts, muts_out = dev.batch(qs, act)
    assert list(counts) == want
    for i in np.flatnonzero(act):
        om, _ = orc.mutations(qs[i], 0)
        assert np.array_equal(muts_out[int(i)], om), qs[i][:80]


def test_mutation_profile_long_genome():
    """A 40,000-position genome: the profile terms do not fit shared memory, so the row-index pass
    reads them through the caches instead."""
    t = R.Table.generate(20000, seed=5, genome_len=40000, pool_sites=300, n_aa_genes=1, null_fraction=0.01)
    orc = oracle_for(t)
    dev = R.Device(t, 0)
    try:
        rng = np.random.default_rng(2)
        muts = ",".join(f"{p + 1}:{'ACGTN'[p % 5]}" for p in sorted(rng.choice(40000, 30, replace=False)))
        for d in (0, 20, 60):
            check_filter(dev, orc, f"MutProfileMutations(main,{d},{muts})")
        qs = [f"MutProfileMutations(main,{d},{muts})" for d in (10, 40)]
        counts, _ = dev.batch(qs, np.zeros(2, np.int32))
        assert list(counts) == [orc.count(q) for q in qs]
    finally:
        dev.close()


def test_mutation_profile_sequence_id():
    """MutProfileSequenceId: the profile is the sequence of the first row holding a primary key,
    rebuilt on the host from the row index; the same row sets as the oracle's reconstruction from
    its vertical and coverage indexes, alone and in a batch."""
    from rawtable import accession_table

    b, raw, acc = accession_table(n_rows=70000, L=300, seed=9)
    t = R.Table.from_raw(raw)
    orc = oracle_mod.Oracle(raw, t.n_chunks, [(c.name, c.n_symbols, c.L) for c in t.columns])
    t.set_primary_key("accession")
    orc.set_primary_key("accession")
    dev = R.Device(t, 0)
    try:
        qs = [f"MutProfileSequenceId(main,{d},{k})" for k in ("seq_0003", "shared_a", "null_row", "seq_69999")
              for d in (0, 2, 8)]
        for q in qs:
            check_filter(dev, orc, q)
        act = np.array([1 if i % 3 == 1 else 0 for i in range(len(qs))], np.int32)
        counts, muts = dev.batch(qs, act)
        assert list(counts) == [orc.count(q) for q in qs]
        for i in np.flatnonzero(act)[:3]:
            om, _ = orc.mutations(qs[i], 0)
            assert np.array_equal(muts[int(i)], om), qs[i]
        with pytest.raises(R.RhyError):
            dev.count("MutProfileSequenceId(main,1,nosuch)")
    finally:
        dev.close()
