#!/usr/bin/env python
"""Benchmark of the filter / count / mutations hot path on one GB300.

Workload: a seeded synthetic table of 2,000,000 sequences (29,903-nt genome, 12 amino-acid genes
totalling 9,700 aa, country / lineage / date metadata) and seeded random filter expressions over
nucleotide, amino-acid and metadata leaves. A step is one batch of 2,048 queries: 75% Aggregated
count, 25% Mutations of the nucleotide column.

value      queries/s of the batched path (persistent filter kernel + batched mutations kernels,
           replayed from a captured CUDA graph) with programs and table resident in HBM, planned by
           the learned planner (trained first on traces of 1,000 other queries through the plain
           path; the rule-based ordering's time is reported beside it under "planner").
e2e        the same through the C-ABI call rhy_batch_rows with host buffers: planning, host->device
           copies, kernels, the Mutations output rows built on the device (minimum proportion
           0.05) and the device->host copy of every count and row.
plain      the plain single-query path over the same queries, one query at a time.
roofline   the plain container pass of the Mutations action (mut_ring_kernel), the kernel that
           streams the whole vertical index: algorithmic bytes = container payloads + descriptors
           + the filter tiles it stages, divided by its CUDA-event duration.
roofline_batch  the batched filter and container kernels: the algorithmic bytes of one batch
           (rhy_batch_info's filter bytes; per dense pass every container and the query masks)
           divided by their CUDA-event durations.
cpu_baseline  the CPU oracle (a restatement of the reference's operators) on a bounded sample of
           the same queries, one query per host thread as the reference serves them.
parity_oracle  the same leg as checker, outside every timed region: the oracle's count of every
           query of the batch and its Mutations tables and rows for the sample's Mutations queries,
           against the batched path's counts and tables and the rows built on the device.
planner    rule-based vs learned ordering: device time of the captured batch and end to end.
serving    Poisson arrivals at 2,000 and 20,000 requests/s on an 8M-sequence table: continuous
           batching (learned planner) against the plain single-query path, p50 / p99 and the rate.
ingestion  the serving table's raw partition built on the host (all host threads) and on the GPU:
           seconds of each and whether the two images are identical.

`python bench.py --impl reference` times that CPU implementation alone on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "lapis-silo_gb300"))

METRIC = "queries/s and p99 ms, batched+learned planner vs plain GPU path, bit-exact"
PEAKS = ROOT / "MEASURED_PEAKS.json"
MIN_PROPORTION = 0.05


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=150)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rows", type=int, default=2_000_000)
    ap.add_argument("--batch", type=int, default=2048)
    ap.add_argument("--mut-every", type=int, default=4, help="every n-th query is a Mutations query")
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--qseed", type=int, default=43)
    ap.add_argument("--plain-queries", type=int, default=256)
    ap.add_argument("--cpu-sample", type=int, default=256,
                    help="queries of the batch the CPU oracle times (one Mutations query in four)")
    ap.add_argument("--tile-bits", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--planner-samples", type=int, default=200_000,
                    help="operator-node traces of the plain path to train the planner on (0: no planner)")
    ap.add_argument("--planner-trace-rows", type=int, default=500_000,
                    help="sequences of the table the traces come from (its own seeded table)")
    ap.add_argument("--planner-heldout", type=int, default=10_000,
                    help="held-out queries on the benchmark table that judge the trained network")
    ap.add_argument("--no-planner", action="store_true", help="rule-based ordering only")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default filter schedule")
    ap.add_argument("--schedule", default="",
                    help="max_tile_bits,stack_kb,ctas_per_sm,query_major: this filter schedule instead of the autotuner's")
    ap.add_argument("--shape-queries", type=int, default=4096,
                    help="batching-shape leg: trees of 1-64 leaves, log-uniform selectivities (0: none)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="length of each serving run (0: none)")
    ap.add_argument("--serve-rates", default="2000,20000", help="Poisson arrival rates (requests/s) of the serving runs")
    ap.add_argument("--no-ingest", action="store_true",
                    help="skip the ingestion leg (host vs GPU build of the serving table's raw partition)")
    ap.add_argument("--serve-rows", type=int, default=8_000_000,
                    help="sequences of the serving table (its own seeded table when it differs from --rows)")
    ap.add_argument("--profile-workload", default="", choices=["", "plain-mutations", "batch", "profile"],
                    help="run one workload for a profiler and exit: plain-mutations (the single-query path for "
                         "Mutations queries whose filter is neither empty nor every row; --plain-queries of them), "
                         "batch (the batched path, --steps launches), profile (MutationProfile counts at "
                         "distances 0, 5, 50, 200)")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload_config(args, n, n_mut, ws):
    """The workload both arms run, identical in their JSON lines."""
    return {"workload": f"{args.rows} sequences x {args.batch}-query batches "
                        f"({n - n_mut} Aggregated count + {n_mut} nucleotide Mutations)",
            "rows": args.rows, "batch": n, "mutations_per_batch": n_mut, "aa_genes": 12,
            "seeds": {"table": args.seed, "queries": args.qseed},
            "l2": "flushed before every timed step (256 MiB write, outside the events)",
            "parallelism": f"replicas x{ws}"}


def oracle_build_info():
    """Compiler flags of the oracle library and the host CPU, for the CPU baseline's record."""
    flags = ""
    for line in (ROOT / "oracle" / "Makefile").read_text().splitlines():
        if line.startswith("CXXFLAGS"):
            flags = line.split("=", 1)[1].strip()
    model = ""
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            key = line.split(":")[0].strip().lower()
            if key in ("model name", "cpu part", "hardware") and not model:
                model = line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return {"compile_flags": flags, "cpu_model": model or "unknown", "machine": os.uname().machine}


def build_workload(R, args):
    table = R.Table.generate(args.rows, seed=args.seed, n_aa_genes=12)
    queries = table.queries(args.batch, seed=args.qseed, use_aa=True, use_metadata=True)
    actions = np.array([1 if (i % args.mut_every) == args.mut_every - 1 else 0 for i in range(len(queries))], np.int32)
    columns = np.zeros(len(queries), np.uint32)
    return table, queries, actions, columns


def cpu_leg(table, queries, actions, columns, n_sample: int, threads: int):
    """Times the CPU oracle on a sample of the workload; returns (queries/s, sample description, p50,
    p99, seconds, the oracle)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as oracle_mod

    t0 = time.perf_counter()
    orc = oracle_mod.Oracle(table.raw(), table.n_chunks, [(c.name, c.n_symbols, c.L) for c in table.columns])
    build_s = time.perf_counter() - t0
    idx = list(range(min(n_sample, len(queries))))
    secs, ms, _ = orc.run_batch([queries[i] for i in idx], [int(actions[i]) for i in idx],
                                [int(columns[i]) for i in idx], threads)
    qps = len(idx) / secs
    desc = (f"first {len(idx)} queries of the batch ({int(sum(actions[i] for i in idx))} Mutations), "
            f"{threads} worker threads, one query per thread; oracle ingestion {build_s:.1f} s not timed")
    return qps, desc, float(np.percentile(ms, 50)), float(np.percentile(ms, 99)), secs, orc


def oracle_parity(orc, table, queries, actions, columns, n_sample, b_counts, b_muts, rows, r_begin, r_cnt):
    """The CPU leg as checker (outside every timed region): the oracle's count of every query of the
    batch, and its Mutations tables and rows for the Mutations queries of the timed sample, against
    the batched path's counts and tables and the rows rhy_batch_rows built on the device."""
    t0 = time.perf_counter()
    mut = [i for i in range(min(n_sample, len(queries))) if actions[i] == 1]
    o_counts, o_tables = orc.check_batch(queries, columns, tables=mut)
    count_bad = int(np.sum(np.asarray(b_counts, np.uint64) != o_counts))
    table_bad = sum(int(not np.array_equal(b_muts[i], o_tables[i])) for i in mut)
    rows_bad = 0
    for i in mut:
        got = [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
                float(r["proportion"])) for r in rows[int(r_begin[i]):int(r_begin[i]) + int(r_cnt[i])]]
        rows_bad += int(got != orc.mutation_rows(int(columns[i]), o_tables[i], MIN_PROPORTION))
    return {"counts_checked": len(queries), "tables_checked": len(mut), "rows_checked": len(mut),
            "mismatches": count_bad + table_bad + rows_bad, "seconds": round(time.perf_counter() - t0, 1)}


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "lapis-silo_gb300"))
    import rhydb_gpu as R

    table, queries, actions, columns = build_workload(R, args)
    threads = os.cpu_count() or 1
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as oracle_mod

    orc = oracle_mod.Oracle(table.raw(), table.n_chunks, [(c.name, c.n_symbols, c.L) for c in table.columns])
    n = min(args.cpu_sample, len(queries))
    step_s = []
    all_ms = []
    for step in range(args.warmup + args.steps):
        lo = (step * n) % len(queries)
        idx = [(lo + i) % len(queries) for i in range(n)]
        secs, ms, _ = orc.run_batch([queries[i] for i in idx], [int(actions[i]) for i in idx],
                                    [int(columns[i]) for i in idx], threads)
        if step >= args.warmup:
            step_s.append(secs)
            all_ms.extend(ms.tolist())
    total = sum(step_s)
    qps = n * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded generator: 2M sequences, Zipf(1.1) substitutions, N-runs, gaps, 12 aa genes)",
        "config": workload_config(args, len(queries), int(actions.sum()), ws),
        "p50_ms": float(np.percentile(all_ms, 50)), "p99_ms": float(np.percentile(all_ms, 99)),
        "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"{n} consecutive queries of the batch per step (a rotating window, "
                                   f"1 in {args.mut_every} Mutations), one query per worker thread",
                         **oracle_build_info()},
        "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ingestion_leg(R, table, dev_index):
    """Ingestion of one raw partition (the rows of `table`) on the host (rhy_table_from_raw, all host
    threads) and on the GPU (rhy_table_from_raw_gpu): wall seconds of each, and whether every
    sequence column's image is identical (checksum over all of its arrays)."""
    raw = table.raw()
    t0 = time.perf_counter()
    host = R.Table.from_raw(raw)
    host_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    gpu = R.Table.from_raw_gpu(raw, dev_index)
    gpu_s = time.perf_counter() - t0
    same = all(host.checksum(c) == gpu.checksum(c) and host.local_reference(c) == gpu.local_reference(c)
               for c in range(host.n_seq))
    out = {"rows": table.n_rows, "sequence_columns": host.n_seq, "host_build_s": round(host_s, 2),
           "host_threads": os.cpu_count() or 1, "gpu_build_s": round(gpu_s, 2), "speedup": host_s / gpu_s,
           "images_identical": bool(same)}
    del host, gpu
    return out


def profile_workload(args, R, workloads, table, dev, queries, actions, columns, sp, stream):
    """One workload for a profiler (no timing of its own): see --profile-workload."""
    if args.profile_workload == "plain-mutations":
        counts, _ = dev.batch(queries, actions, columns)
        idx = [i for i in range(len(queries)) if actions[i] == 1 and 0 < counts[i] < table.n_rows][:args.plain_queries]
        dev.plain_prepare(queries, actions, columns)
        for i in idx:
            dev.plain_launch(i, sp)
        stream.synchronize()
        print(f"plain-mutations: {len(idx)} queries over {table.n_rows} rows")
    elif args.profile_workload == "profile":
        seq = workloads.profile_query_sequence(table, row=123457, substitutions=20, seed=17)
        for d in (0, 5, 50, 200):
            print(f"profile: distance {d}: {dev.count(f'MutProfile(main,{d},{seq})', sp)} of {table.n_rows} rows")
    else:
        if args.schedule:
            w, kb, cps, qm = (int(x) for x in args.schedule.split(","))
            dev.batch_schedule(max_tile_bits=w, stack_kb=kb, ctas_per_sm=cps, query_major=qm)
        dev.batch_prepare(queries, actions, columns)
        for _ in range(args.steps):
            dev.batch_launch(sp, True, True)
        stream.synchronize()
        print(f"batch: {args.steps} x {len(queries)} queries over {table.n_rows} rows")


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
        return
    import torch

    import rhydb_gpu as R
    import workloads

    R.lib()
    torch.cuda.set_device(local)
    dev_index = local
    table, queries, actions, columns = build_workload(R, args)
    dev = R.Device(table, dev_index)
    n = len(queries)
    n_mut = int(actions.sum())
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    if args.profile_workload:
        profile_workload(args, R, workloads, table, dev, queries, actions, columns, sp, stream)
        dev.close()
        return
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev_index}")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def time_batch(steps, warmup):
        dev.batch_prepare(queries, actions, columns, tile_bits=args.tile_bits)
        dev.batch_launch(sp, True, False)
        dev.batch_capture_ex(sp, copy_in=False, copy_out=False)
        torch.cuda.synchronize()
        for _ in range(warmup):
            flush_l2()
            dev.batch_replay(sp)
        ms = []
        for _ in range(steps):
            flush_l2()
            e0, e1 = ev(), ev()
            e0.record(stream)
            dev.batch_replay(sp)
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return statistics.median(ms)

    # ---------------- learned planner: traces of the plain path, trained on the GPU ----------------
    # traces on their own table, the trained model imported here and judged on held-out queries
    planner = {"mode": "rule-based ordering"}
    if not args.no_planner and args.planner_samples > 0:
        t0 = time.perf_counter()
        own = args.planner_trace_rows != args.rows
        tr_table = R.Table.generate(args.planner_trace_rows, seed=args.seed + 1, n_aa_genes=12) if own else table
        tr_dev = R.Device(tr_table, dev_index) if own else dev
        n_samples, n_trace_q, k = 0, 0, 0
        while n_samples < args.planner_samples and k < 64:
            qk = tr_table.queries(2000, seed=args.qseed + 1000 + k, use_aa=True, use_metadata=True)
            n_samples += tr_dev.planner_collect(qk)
            n_trace_q += len(qk)
            k += 1
        collect_s = time.perf_counter() - t0
        st = tr_dev.planner_train(epochs=40, batch=1024, lr=2e-3, seed=7)
        model = tr_dev.planner_export()
        if own:
            tr_dev.close()
            del tr_table
        dev.planner_import(model)
        held = table.queries(args.planner_heldout, seed=args.qseed + 5000, use_aa=True, use_metadata=True)
        t1 = time.perf_counter()
        judged = dev.planner_evaluate(held)
        planner = {"mode": "learned" if judged["accepted"] else "rule-based ordering (network rejected by the judge)",
                   "trace_rows": args.planner_trace_rows, "trace_queries": n_trace_q, "samples": n_samples,
                   "collect_s": round(collect_s, 2), "train_ms": round(st["train_ms"], 1),
                   "train_split_qerr_median": [st["qerr_learned_median"], st["qerr_rule_median"]],
                   "train_split_qerr_p90": [st["qerr_learned_p90"], st["qerr_rule_p90"]],
                   "heldout_queries": len(held), "heldout_nodes": judged["n_val"],
                   "heldout_evaluate_s": round(time.perf_counter() - t1, 2),
                   "heldout_qerr_median": [judged["qerr_learned_median"], judged["qerr_rule_median"]],
                   "heldout_qerr_p90": [judged["qerr_learned_p90"], judged["qerr_rule_p90"]],
                   "heldout_cost_ln_err_median": judged["cost_err_median"]}

    # ---------------- autotuner: schedule of the filter launches of this batch (untimed) ----------------
    autotune = None
    if args.schedule:
        w, kb, cps, qm = (int(x) for x in args.schedule.split(","))
        dev.batch_schedule(max_tile_bits=w, stack_kb=kb, ctas_per_sm=cps, query_major=qm)
    elif not args.no_autotune and not args.tile_bits:
        default_sched = dev.batch_schedule()
        t0 = time.perf_counter()
        tried = dev.batch_autotune(queries, actions, columns, reps=3, stream=sp)
        autotune = {"candidates": len(tried), "tune_s": round(time.perf_counter() - t0, 2),
                    "best_filter_ms": round(tried[0][1], 3),
                    "default_filter_ms": next((round(ms, 3) for sc, ms in tried if sc == default_sched), None),
                    "worst_filter_ms": round(tried[-1][1], 3)}

    min_props = np.full(n, MIN_PROPORTION)

    def e2e_run(steps):
        """rhy_batch_rows end to end (planning, copies, kernels, rows): one untimed call, then `steps`
        timed calls; queries/s of the median call and that call's phases."""
        dev.batch_rows(queries, actions, columns, min_props, tile_bits=args.tile_bits, stream=sp)
        secs, phases, last = [], [], None
        for _ in range(steps):
            t0 = time.perf_counter()
            last = dev.batch_rows(queries, actions, columns, min_props, tile_bits=args.tile_bits, stream=sp)
            secs.append(time.perf_counter() - t0)
            phases.append(dev.batch_times())
        mid = sorted(range(len(secs)), key=lambda i: secs[i])[len(secs) // 2]
        ph = {k: round(v, 3) for k, v in phases[mid].items()}
        top = ("plan_ms", "prepare_ms", "device_ms", "output_ms")  # the rest split plan_ms
        ph["other_ms"] = round(1000 * secs[mid] - sum(phases[mid][k] for k in top), 3)
        return n * ws / max_over_ranks(statistics.median(secs), ws), ph, last

    if planner["mode"] == "learned":
        # the same batch and schedule under both orderings: device time of the captured batch, and
        # end to end through rhy_batch_rows (planning included)
        planner["rule_ms_per_step"] = time_batch(10, 3)
        planner["rule_e2e_qps"], planner["rule_e2e_phases_ms"], _ = e2e_run(15)
        dev.planner_mode(1)
        planner["learned_ms_per_step"] = time_batch(10, 3)
        planner["learned_e2e_qps"], planner["learned_e2e_phases_ms"], _ = e2e_run(15)
        planner["learned_e2e_note"] = ("rhy_batch_rows plans its first part (the Mutations queries) by the rule, "
                                       "since the device waits for it; the network plans the counts while that "
                                       "part runs")
        planner["device_speedup"] = planner["rule_ms_per_step"] / planner["learned_ms_per_step"]
        planner["e2e_speedup"] = planner["learned_e2e_qps"] / planner["rule_e2e_qps"]

    # ---------------- batched path: device-resident ----------------
    dev.batch_prepare(queries, actions, columns, tile_bits=args.tile_bits)
    info = dev.batch_info()
    dev.batch_launch(sp, True, False)
    dev.batch_capture_ex(sp, copy_in=False, copy_out=False)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        flush_l2()
        dev.batch_replay(sp)
    torch.cuda.synchronize()
    barrier(ws)
    clocks = ClockSampler(dev_index)
    clocks.start()
    t_wall0 = time.perf_counter()
    step_ms = []
    for _ in range(args.steps):
        flush_l2()
        e0, e1 = ev(), ev()
        e0.record(stream)
        dev.batch_replay(sp)
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    barrier(ws)
    total_s = max_over_ranks(sum(step_ms) / 1000.0, ws)
    value = n * args.steps * ws / total_s
    # one persistent filter launch for all classes of programs, then per column with Mutations
    # queries: the slot split, transpose, container, coverage, row-index (when on) and final kernels
    per_col = 5 + (1 if dev.sparse_rows()[1] > 0 else 0)
    launches_per_step = info.n_filter_launches + per_col * len({int(c) for c, a in zip(columns, actions) if a == 1})

    # results of the batched path for the parity self-check against the plain path
    dev.batch_launch(sp, True, True)
    torch.cuda.synchronize()
    b_counts, b_muts = dev.batch_results()
    # row x position cells the batch's Mutations queries count: |F| x L per query
    cells = sum(int(b_counts[i]) * table.columns[int(columns[i])].L for i in range(n) if actions[i] == 1)
    step_s = statistics.median(step_ms) / 1000.0

    # per-kernel times of the batched path
    kernels_ms = {}
    for name, parts in (("filter_batch", 1), ("transpose", 2), ("mut_ctr_batch", 4), ("mut_cov_batch", 8),
                        ("mut_final_batch", 16), ("mut_sparse_batch", 32)):
        ts = []
        for _ in range(2):
            dev.batch_launch_parts(1, sp) if parts != 1 else None
            flush_l2()
            e0, e1 = ev(), ev()
            e0.record(stream)
            dev.batch_launch_parts(parts, sp)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        kernels_ms[name] = min(ts)

    # ---------------- plain path: one query at a time ----------------
    dev.plain_prepare(queries, actions, columns)
    m = min(args.plain_queries, n)
    for i in range(min(8, m)):
        dev.plain_launch(i, sp)
    torch.cuda.synchronize()
    flush_l2()
    torch.cuda.synchronize()
    plain_ms = []
    for i in range(m):
        e0, e1 = ev(), ev()
        e0.record(stream)
        dev.plain_launch(i, sp)
        e1.record(stream)
        e1.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    plain_qps = m / (sum(plain_ms) / 1000.0)
    # parity self-check: plain vs batched on the same queries (bit-exact)
    mismatches = 0
    for i in range(min(64, m)):
        if actions[i] == 1:
            cnt, fc = dev.mutations(queries[i], 0)
            if fc != b_counts[i] or not np.array_equal(cnt, b_muts[i]):
                mismatches += 1
        else:
            if dev.count(queries[i]) != b_counts[i]:
                mismatches += 1

    # plain e2e (C-ABI calls with host buffers)
    t0 = time.perf_counter()
    e2e_plain_ms = []
    for i in range(m):
        q0 = time.perf_counter()
        if actions[i] == 1:
            dev.mutations(queries[i], 0)
        else:
            dev.count(queries[i])
        e2e_plain_ms.append(1000 * (time.perf_counter() - q0))
    plain_e2e_qps = m / (time.perf_counter() - t0)

    # ---------------- batched e2e through the C-ABI ----------------
    # rows of the Mutations action built on the device; the dense-count variant is kept for context.
    # Host wall time per phase of the median step; "other" is the binding's own time.
    e2e_qps, e2e_phase_ms, (r_counts, rows, r_begin, r_cnt) = e2e_run(max(3, min(args.steps, 10)))
    dense_s = []
    for step in range(2):
        t0 = time.perf_counter()
        dev.batch(queries, actions, columns, tile_bits=args.tile_bits, stream=sp)
        dense_s.append(time.perf_counter() - t0)
    dense_qps = n * ws / max_over_ranks(statistics.median(dense_s), ws)
    # the device rows equal the host conversion of the dense counts
    rows_mismatches = int(not np.array_equal(r_counts, b_counts))
    for i in [j for j in range(n) if actions[j] == 1][:64]:
        got = rows[int(r_begin[i]):int(r_begin[i]) + int(r_cnt[i])]
        want = table.mutation_rows(0, b_muts[i], 0.05)
        if [(int(r["position"]), r["from_"].decode(), r["to"].decode(), int(r["count"]), int(r["coverage"]),
             float(r["proportion"])) for r in got] != want:
            rows_mismatches += 1
    col0 = table.columns[0]
    prog_bytes = info.n_instr * 16 + n * 16 + info.n_items * 8 + n_mut * 12
    d2h = n * 8 + n * 12 + len(rows) * 24

    # ---------------- serving: Poisson arrivals, continuous batching vs the plain path ----------------
    serving, ingestion = None, None
    if args.serve_seconds > 0:
        t_setup = time.perf_counter()
        s_table, s_dev, s_queries = table, dev, queries
        if args.serve_rows != args.rows:
            s_table = R.Table.generate(args.serve_rows, seed=args.seed, n_aa_genes=12)
            s_dev = R.Device(s_table, dev_index)
            s_queries = s_table.queries(n, seed=args.qseed, use_aa=True, use_metadata=True)
            if planner["mode"] == "learned":  # the model trained on its own table plans here too
                s_dev.planner_import(dev.planner_export())  # with the verdict judged on this table
                s_dev.planner_mode(1)
        s_planner = "learned" if planner["mode"] == "learned" else "rule-based ordering"
        setup_s = time.perf_counter() - t_setup
        rng = np.random.default_rng(args.qseed + 7)
        rates = [float(x) for x in args.serve_rates.split(",") if x]
        traces = []
        for rate in rates:
            nreq = max(1, int(rate * args.serve_seconds))
            traces.append((rate, np.cumsum(rng.exponential(1.0 / rate, nreq)),
                           rng.choice(3, nreq, p=[0.70, 0.25, 0.05]).astype(np.int32), rng.integers(0, n, nreq)))
        arms = {}
        # continuous batching, then the plain arm (one request at a time through the single-query
        # path, the reference's one-query-per-request model). The plain arm saturates far below the
        # high rates, so its traces are cut to the first 4,000 requests (the same arrival times).
        for arm, kw in (("batched", {"max_batch": 512, "streams": 3}), ("plain", {"plain": True})):
            srv = R.Server(s_dev, **kw)
            runs = []
            for rate, arrivals, mix, pick in traces:
                m = len(arrivals) if arm == "batched" else min(len(arrivals), 4000)
                lat, wall = srv.replay([s_queries[i] for i in pick[:m]], mix[:m], np.zeros(m, np.uint32),
                                       np.full(m, MIN_PROPORTION), np.full(m, 1000, np.uint32), arrivals[:m])
                ok = lat[np.isfinite(lat)]
                runs.append({"arrival_qps": rate, "requests": m, "achieved_qps": m / wall,
                             "p50_ms": float(np.percentile(ok, 50)), "p99_ms": float(np.percentile(ok, 99)),
                             "failed": int(m - len(ok))})
            st = srv.stats()
            srv.stop()
            arms[arm] = {"runs": runs, "mean_batch": st["mean_batch"], "batches": st["batches"],
                         "peak_device_bytes": st["peak_bytes"]}
        serving = {"mix": "70% count / 25% mutations (nucleotide, min proportion 0.05) / 5% details (first 1000 ids)",
                   "arrivals": "Poisson, open loop (native submitter thread)", "rows": s_table.n_rows,
                   "table_setup_s": round(setup_s, 1), "planner": s_planner, **arms}
        if not args.no_ingest:
            ingestion = ingestion_leg(R, s_table, dev_index)
        if s_dev is not dev:
            s_dev.close()
            del s_table

    # ---------------- aggregation: grouped counts of one filter (BitmapAggregation) ----------------
    agg_q = next(queries[i] for i in range(n) if 0.01 * table.n_rows < int(b_counts[i]) < 0.5 * table.n_rows)
    agg_dims = [("seq", 0, 21618), ("dict", 0)]
    agg_ms = []
    for _ in range(6):
        t0 = time.perf_counter()
        agg_rows, agg_n = dev.aggregate(agg_q, agg_dims)
        agg_ms.append(1000 * (time.perf_counter() - t0))
    aggregate = {"dimensions": "nucleotide position 21618 x country", "filter_rows": agg_n,
                 "combinations": len(agg_rows), "ms_per_call": round(statistics.median(agg_ms[1:]), 3)}

    # ---------------- MutationProfile: rows within a distance of a profile (one row-index pass) ----------------
    # The profile is one row's own aligned sequence with 20 substitutions, given as a query
    # sequence (the reference's nof_sequence_filter case: a ~genome-length NOf after its rewrite).
    pseq = workloads.profile_query_sequence(table, row=123457, substitutions=20, seed=17)
    pstats = table.column_stats(0)
    p_bytes = 4 * (table.n_chunks * 65536 + pstats.n_row_index_entries) + table.n_chunks * 8192 * 2
    profile = {"profile": "row 123457's nucleotide sequence + 20 substitutions, as a query sequence",
               "row_index_entries": pstats.n_row_index_entries, "row_index_bytes": p_bytes, "distances": {}}
    for d in (0, 5, 50, 200):
        pq = f"MutProfile(main,{d},{pseq})"
        pn = dev.count(pq, sp)
        p_ms = []
        for _ in range(5):
            flush_l2()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            dev.count(pq, sp)
            p_ms.append(1000 * (time.perf_counter() - t0))
        profile["distances"][str(d)] = {"rows": int(pn), "ms_per_count": round(statistics.median(p_ms), 3)}

    # ---------------- batching shape: trees of 1-64 leaves, selectivities log-uniform in [1e-5, 0.9] ----------------
    shape = None
    if args.shape_queries:
        t0 = time.perf_counter()
        s_qs = workloads.batching_workload(table, dev, n=args.shape_queries, seed=44,
                                           candidates=10 * args.shape_queries)
        pick_s = time.perf_counter() - t0

        def shape_steps():
            dev.batch_prepare(s_qs)
            dev.batch_launch(sp, True, False)
            dev.batch_capture_ex(sp, copy_in=False, copy_out=False)
            for _ in range(3):
                flush_l2()
                dev.batch_replay(sp)
            torch.cuda.synchronize()
            out = []
            for _ in range(20):
                flush_l2()
                e0, e1 = ev(), ev()
                e0.record(stream)
                dev.batch_replay(sp)
                e1.record(stream)
                e1.synchronize()
                out.append(e0.elapsed_time(e1))
            return out

        shape_rule_ms = None
        if planner["mode"] == "learned":  # the same trees under the rule-based ordering
            dev.planner_mode(0)
            shape_rule_ms = statistics.median(shape_steps())
            dev.planner_mode(1)
        s_ms = shape_steps()
        dev.batch_launch(sp, True, True)
        torch.cuda.synchronize()
        s_counts, _ = dev.batch_results()
        sel = np.asarray(s_counts, np.float64) / table.n_rows
        shape = {"queries": len(s_qs), "leaves": "1-64, NOf up to 64 children", "action": "Aggregated count",
                 "selectivity_min": float(sel.min()), "selectivity_max": float(sel.max()),
                 "queries_per_s": len(s_qs) / (statistics.median(s_ms) / 1000.0),
                 "batch_ms_p50": float(np.percentile(s_ms, 50)), "batch_ms_p99": float(np.percentile(s_ms, 99)),
                 "steps": len(s_ms), "l2": "flushed before every step", "pick_s": round(pick_s, 2),
                 "planner": planner["mode"], "rule_batch_ms_p50": shape_rule_ms}

    # ---------------- roofline: plain container pass ----------------
    payload_b, desc_b = dev.mutation_bytes(0)
    # queries whose filter is neither empty nor every row: the pass reads the whole column
    mut_idx = [i for i in range(n) if actions[i] == 1 and 0 < int(b_counts[i]) < table.n_rows][:16]
    ctr_ms = []
    for i in mut_idx:
        dev.plain_launch(i, sp, parts=1)  # filter tile and count
        # two flushes keep the GPU busy while the host submits the timed launch, so the events
        # bracket the kernel and not the submission
        flush_l2()
        flush_l2()
        e0, e1 = ev(), ev()
        e0.record(stream)
        dev.plain_launch(i, sp, parts=2)  # container pass only
        e1.record(stream)
        e1.synchronize()
        ctr_ms.append(e0.elapsed_time(e1))
    ctr_avg_ms = statistics.mean(ctr_ms)
    alg_bytes = payload_b + desc_b + table.n_chunks * 8192
    peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    achieved = alg_bytes / (ctr_avg_ms / 1000.0) / 1e9
    traffic = None
    prof = ROOT / "profiles" / "mut_ring_kernel_2M.traffic.json"
    if prof.exists():
        traffic = json.loads(prof.read_text()).get("dram_bytes_per_launch")

    # ---------------- roofline of the batched kernels ----------------
    # filter_batch_kernel: the algorithmic bytes of the batch's programs (container payloads and
    # descriptors of their index-scan leaves, coverage and date data, outputs) per launch.
    # mut_ctr_batch_kernel: per dense pass (up to 256 slots) every container payload and descriptor
    # plus the 32-byte query-mask sector of every row, and the count tables of the dense slots.
    sparse_b = dev.sparse_rows()[1]
    dense_slots = sum(1 for i in range(n) if actions[i] == 1 and int(b_counts[i]) > max(sparse_b, 0)
                      and int(b_counts[i]) > 0)
    passes = -(-dense_slots // 256)
    col0 = table.columns[0]
    ctr_alg = passes * (payload_b + desc_b + table.n_chunks * 65536 * 32) + dense_slots * col0.n_symbols * col0.L * 4
    roofline_batch = {
        "filter_batch_kernel": {"algorithmic_bytes_per_launch": int(info.filter_bytes),
                                "launch_ms": kernels_ms["filter_batch"],
                                "achieved": info.filter_bytes / (kernels_ms["filter_batch"] / 1000.0) / 1e9,
                                "unit": "GB/s", "peak": peak},
        "mut_ctr_batch_kernel": {"algorithmic_bytes_per_launch": int(ctr_alg), "dense_slots": dense_slots,
                                 "passes": passes, "launch_ms": kernels_ms["mut_ctr_batch"],
                                 "achieved": ctr_alg / (kernels_ms["mut_ctr_batch"] / 1000.0) / 1e9,
                                 "unit": "GB/s", "peak": peak},
    }
    for v in roofline_batch.values():
        v["frac"] = v["achieved"] / peak

    # ---------------- CPU baseline, then the oracle as checker of the batch ----------------
    cpu, parity = None, None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cqps, cdesc, cp50, cp99, csecs, orc = cpu_leg(table, queries, actions, columns, args.cpu_sample, threads)
        cpu = {"value": cqps, "unit": "queries/s", "cores": threads, "kind": "port", "sample": cdesc,
               "p50_ms": cp50, "p99_ms": cp99, "seconds": csecs, **oracle_build_info()}
        parity = oracle_parity(orc, table, queries, actions, columns, args.cpu_sample, b_counts, b_muts, rows,
                               r_begin, r_cnt)
        del orc

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded generator: 2M sequences, Zipf(1.1) substitutions, N-runs, gaps, 12 aa genes)",
            "config": workload_config(args, n, n_mut, ws),
            "schedule": {"tile_bits": info.tile_bits, "grid": info.grid, "planner": planner["mode"],
                         **dev.batch_schedule()},
            "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
            "latency_note": "batched: every query of a batch completes with its batch",
            "plain": {"qps": plain_qps, "p50_ms": float(np.percentile(plain_ms, 50)),
                      "p99_ms": float(np.percentile(plain_ms, 99)), "queries": m, "e2e_qps": plain_e2e_qps,
                      "e2e_p99_ms": float(np.percentile(e2e_plain_ms, 99))},
            "speedup_vs_plain": value / plain_qps,
            "row_position_counts_per_s": cells * ws / max_over_ranks(step_s, ws),
            "planner": planner,
            "autotune": autotune,
            "aggregate": aggregate,
            "mutation_profile": profile,
            "batching_shape": shape,
            "serving": serving,
            "ingestion": ingestion,
            "parity_plain_vs_batched_mismatches": mismatches,
            "parity_oracle": parity,
            "parity_oracle_mismatches": parity["mismatches"] if parity else None,
            "e2e": {"value": e2e_qps, "unit": "queries/s", "h2d_bytes_per_step": int(prog_bytes),
                    "d2h_bytes_per_step": int(d2h), "output": "Mutations rows (min proportion 0.05) + counts",
                    "rows_per_step": int(len(rows)), "rows_mismatches": rows_mismatches,
                    "dense_counts_qps": dense_qps, "phases_ms": e2e_phase_ms},
            "gpu_launches": launches_per_step * args.steps,
            "kernels_ms": kernels_ms,
            "roofline": {"kernel": "mut_ring_kernel (plain Mutations container pass, nucleotide column)",
                         "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "algorithmic_bytes_per_launch": alg_bytes, "launch_ms": ctr_avg_ms,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s"},
            "roofline_batch": roofline_batch,
            "cpu_baseline": cpu,
            "clocks": clk,
            "wall_s_timed_region": wall,
        }
        print(json.dumps(line), flush=True)
    dev.close()


if __name__ == "__main__":
    main()
