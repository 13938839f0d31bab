#!/usr/bin/env python
"""Standard workloads for profiling the path under a profiler (ncu), one per subcommand.

  plain-mutations  single-query path: filter, then the Mutations passes, for Mutations queries whose
                   filter is neither empty nor every row (the container pass reads the whole column)
  batch            the batched path: prepare once, then launch the whole batch `--steps` times
  profile          MutationProfile counts (one row's sequence + 20 substitutions) at distances
                   0, 5, 50 and 200

The table and queries are the benchmark's seeded synthetic workload (sizes on the command line).
"""
from __future__ import annotations

import argparse
import ctypes
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import rhydb_gpu as R  # noqa: E402
import workloads  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("workload", choices=["plain-mutations", "batch", "profile"])
    ap.add_argument("--rows", type=int, default=2_000_000)
    ap.add_argument("--batch", type=int, default=2048)
    ap.add_argument("--queries", type=int, default=8, help="plain-mutations: queries to run")
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--qseed", type=int, default=43)
    ap.add_argument("--query-major", action="store_true", help="batch: query-major work items")
    args = ap.parse_args()

    import torch

    table = R.Table.generate(args.rows, seed=args.seed, n_aa_genes=12)
    queries = table.queries(args.batch, seed=args.qseed, use_aa=True, use_metadata=True)
    actions = (np.arange(len(queries)) % 4 == 3).astype(np.int32)
    columns = np.zeros(len(queries), np.uint32)
    dev = R.Device(table, 0)
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    if args.workload == "plain-mutations":
        counts, _ = dev.batch(queries, actions, columns)
        idx = [i for i in range(len(queries)) if actions[i] == 1 and 0 < counts[i] < table.n_rows][:args.queries]
        dev.plain_prepare(queries, actions, columns)
        for i in idx:
            dev.plain_launch(i, sp)
        stream.synchronize()
        print(f"plain-mutations: {len(idx)} queries over {table.n_rows} rows")
    elif args.workload == "profile":
        seq = workloads.profile_query_sequence(table)
        for d in (0, 5, 50, 200):
            n = dev.count(f"MutProfile(main,{d},{seq})", sp)
            print(f"profile: distance {d}: {n} of {table.n_rows} rows")
    else:
        if args.query_major:
            dev.batch_schedule(query_major=1)
        dev.batch_prepare(queries, actions, columns)
        for _ in range(args.steps):
            dev.batch_launch(sp, True, True)
        stream.synchronize()
        print(f"batch: {args.steps} x {len(queries)} queries over {table.n_rows} rows")
    dev.close()


if __name__ == "__main__":
    main()
