"""The reference's own known-answer scenarios (tests/golden/reference_cases.py) through the CPU
oracle, the host planner and (with -m gpu) the CUDA path."""
import numpy as np
import pytest

import oracle as oracle_mod
import rhydb_gpu as R
from golden import reference_cases as G
from rawtable import RawBuilder, date_days, oracle_for


def build(ds):
    b = RawBuilder(ds["n_rows"])
    for name, kind, ref, rows in ds["seq"]:
        b.add_sequences(name, kind, ref, rows)
    for name, values in ds.get("dict", []):
        b.add_dict(name, values)
    for name, values in ds.get("date", []):
        b.add_dates(name, [date_days(v) if v else None for v in values])
    raw = b.raw()
    table = R.Table.from_raw(raw)
    orc = oracle_for(table, raw)
    if ds.get("primary_key"):
        table.set_primary_key(ds["primary_key"])
        orc.set_primary_key(ds["primary_key"])
    return b, raw, table, orc


@pytest.fixture(scope="module", params=G.DATASETS, ids=lambda d: d["name"])
def dataset(request):
    return (request.param,) + build(request.param)


def test_oracle_counts(dataset):
    ds, _, _, table, orc = dataset
    for expr, expected in ds["cases"]:
        assert orc.count(expr) == expected, expr
    for expr, rows in ds.get("row_cases", []):
        bits, n = orc.compute_filter(expr)
        assert R.bits_to_rows(bits).tolist() == rows, expr


def test_errors_are_user_errors(dataset):
    ds, _, _, table, orc = dataset
    for expr in ds["errors"]:
        with pytest.raises(oracle_mod.OracleError) as e:
            orc.count(expr)
        assert e.value.code == 1
        with pytest.raises(R.IllegalQuery):
            table.plan(expr)


def test_storage_matches_oracle(dataset):
    ds, _, _, table, orc = dataset
    for ci in range(table.n_seq):
        assert table.local_reference(ci) == orc.local_reference(ci)
        pos, ch, sym, card, _ = table.containers(ci)
        p2, v2, s2, c2 = orc.vertical(ci)
        assert sorted(zip(pos.tolist(), ch.tolist(), sym.tolist(), card.tolist())) == sorted(
            zip(p2.tolist(), v2.tolist(), s2.tolist(), c2.tolist()))


@pytest.mark.parametrize("pos,neg,n,exact,expected", G.THRESHOLD_CASES)
def test_threshold_known_answers(pos, neg, n, exact, expected):
    assert oracle_mod.operator(0, [4], pos, neg, n, exact) == expected


def _threshold_table(pos, neg):
    sets = list(pos) + list(neg)
    b = RawBuilder(4)
    b.add_sequences("main", 0, "ACGT", ["ACGT"] * 4)
    for i, s in enumerate(sets):
        b.add_dict(f"c{i}", ["in" if r in s else "out" for r in range(4)])
    raw = b.raw()
    return b, raw, R.Table.from_raw(raw)


def _threshold_expr(pos, neg, n, exact):
    kids = [f"StrEq(c{i},in)" for i in range(len(pos))]
    kids += [f"Not(StrEq(c{len(pos) + i},in))" for i in range(len(neg))]
    return f"NOf({n},{'exactly' if exact else 'atleast'}," + ",".join(kids) + ")"


@pytest.mark.parametrize("pos,neg,n,exact,expected", G.THRESHOLD_CASES)
def test_threshold_cases_as_queries_on_oracle(pos, neg, n, exact, expected):
    b, raw, t = _threshold_table(pos, neg)
    orc = oracle_for(t, raw)
    bits, _ = orc.compute_filter(_threshold_expr(pos, neg, n, exact))
    assert R.bits_to_rows(bits).tolist() == expected


@pytest.mark.gpu
def test_gpu_golden(dataset):
    ds, _, _, table, orc = dataset
    dev = R.Device(table, 0)
    for expr, expected in ds["cases"]:
        assert dev.count(expr) == expected, expr
    for expr, rows in ds.get("row_cases", []):
        bits, n = dev.compute_filter(expr)
        assert R.bits_to_rows(bits).tolist() == rows, expr
        assert n == len(rows)
    for expr in ds["errors"]:
        with pytest.raises(R.IllegalQuery):
            dev.count(expr)
    # mutations of every sequence column for every case, against the oracle
    for expr, _ in ds["cases"] + ds.get("row_cases", []):
        for ci in range(table.n_seq):
            m, fc = dev.mutations(expr, ci)
            om, ofc = orc.mutations(expr, ci)
            assert fc == ofc and np.array_equal(m, om), (expr, ci)
    dev.close()


@pytest.mark.gpu
@pytest.mark.parametrize("pos,neg,n,exact,expected", G.THRESHOLD_CASES)
def test_gpu_threshold_cases(pos, neg, n, exact, expected):
    b, raw, t = _threshold_table(pos, neg)
    dev = R.Device(t, 0)
    bits, _ = dev.compute_filter(_threshold_expr(pos, neg, n, exact))
    assert R.bits_to_rows(bits).tolist() == expected
    dev.close()
