"""A C++ client compiled with g++ against include/rhydb_gpu.h alone (tests/capi_client.cpp), the way
RhyDB would bind the library. On CPU it runs the table, planning and operator-tree calls; with
-m gpu it also opens a device and its counts, row sets, Mutations and batch rows are compared with
the oracle."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import rhydb_gpu as R
from rawtable import oracle_for

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "lapis-silo_gb300"


@pytest.fixture(scope="module")
def client(tmp_path_factory):
    exe = tmp_path_factory.mktemp("capi") / "capi_client"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "capi_client.cpp"),
           f"-L{LIBDIR}", "-lrhygpu", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(exe, mode):
    r = subprocess.run([str(exe), mode], capture_output=True, text=True, timeout=600, env=dict(os.environ))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    out = {}
    for line in r.stdout.splitlines():
        kind, _, rest = line.partition(" ")
        out.setdefault(kind, []).append(rest)
    assert out.get("done") is not None
    return out


def same_table():
    return R.Table.generate(70000, seed=7, genome_len=3000, pool_sites=300, null_fraction=0.01)


def test_client_on_the_host(client):
    out = run(client, "host")
    t = same_table()
    assert out["info"] == [f"{t.n_rows} {t.n_chunks} {t.n_seq}"]
    queries = [q.split(" ", 1)[1] for q in out["query"]]
    assert queries == t.queries(16, seed=11, max_depth=4, max_nof_children=8, use_metadata=True)
    for line, q in zip(out["plan"], queries):
        i, n_instr, depth, same = line.split()
        _, n2, d2 = t.plan(q)
        assert (int(n_instr), int(depth), int(same)) == (n2, d2, 1), q
    # an illegal query (1) and a malformed operator tree (2), each with a message
    assert out["error"] == ["1 1", "2 1"]


@pytest.mark.gpu
def test_client_on_the_gpu_against_the_oracle(client):
    out = run(client, "gpu")
    t = same_table()
    orc = oracle_for(t)
    queries = [q.split(" ", 1)[1] for q in out["query"]]
    for line in out["count"]:
        i, c, ec, pc, first = (int(x) for x in line.split())
        bits, n = orc.compute_filter(queries[i])
        rows = R.bits_to_rows(bits)
        assert c == ec == pc == n, queries[i]
        assert first == (int(rows[0]) if rows.size else -1), queries[i]
    for line in out["mutations"]:
        i, fc, s, w = (int(x) for x in line.split())
        om, on = orc.mutations(queries[i], 0)
        flat = om.reshape(-1).astype(np.uint64)
        weights = np.arange(flat.size, dtype=np.uint64) % 9973 + 1
        assert (fc, s, w) == (on, int(flat.sum()), int((flat * weights).sum())), queries[i]
    for line in out["batch"]:
        parts = line.split()
        i, c, nrows = int(parts[0]), int(parts[1]), int(parts[2])
        assert c == orc.count(queries[i]), queries[i]
        if i % 2 == 1:
            om, _ = orc.mutations(queries[i], 0)
            want = orc.mutation_rows(0, om, 0.05)
            assert nrows == len(want), queries[i]
            for got, w in zip(parts[3:], want):
                pos, frm, to, cnt, cov, prop = got.split(":")
                assert (int(pos), frm, to, int(cnt), int(cov), float(prop)) == w, queries[i]
