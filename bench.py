"""Benchmark: batched windowed tree-sequence statistics on one GB300.

Workload "windowed_n10k": a seeded SMC tree sequence with n=10,000 samples,
L=1e8 and 100,000 breakpoints (~5 sites per breakpoint), four disjoint random
sample sets of 2,500 and 1,000 equal windows.  One step computes diversity
(4 sets), divergence (6 pairs), Fst (6 pairs), Tajima's D (4 sets) and Y3
(4 triples) in both branch and site modes with span normalisation, as ONE
fused sweep at FP64 (the FP32-compensated form of the same sweep is timed
beside it).

Metric: edge-updates/s, counted as the reference runs the same queries: each
low-level call is one traversal applying every edge insertion and removal
(diversity 1, divergence 1, Fst 2, Tajima's D 2, Y3 1 traversal per mode; 14
in all).  `value` is measured with the tree sequence and the prepared query
resident in HBM; `e2e` goes through the C ABI host-pointer entry point with
host inputs and a host result.  L2 is flushed (256 MiB write) before every
timed step.

--impl reference times the reference's CPU implementation of the same
queries on the host cores (the C oracle restatement when the reference
library cannot be built on this machine).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = "windowed_n10k"
NUM_SETS = 4
NUM_WINDOWS = 1000
# per mode: diversity 1, divergence 1, Fst 2, Tajima's D 2, Y3 1 traversals
REFERENCE_TRAVERSALS_PER_MODE = 7
MODES = ("branch", "site")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", choices=["f64", "f32"], default=None,
                    help="profiling mode: only warmup + steps launches of the headline fused "
                         "query in this arithmetic (default compact plan, no tuning, no other "
                         "legs), for ncu captures")
    ap.add_argument("--serve-queries", type=int, default=2000,
                    help="serve_mix: requests in the stream")
    ap.add_argument("--serve-rate", type=float, default=5000.0,
                    help="serve_mix: Poisson arrival rate (requests/s), above what the "
                         "server absorbs, so that queries/s measures the server")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "afs_n200k", "grm_n20k", "serve_mix"],
                    help="the headline workload (default) or one of the other "
                         "configurations, each printing its own JSON line")
    return ap.parse_args()


def make_workload():
    from tskit_gb300 import sim

    tables = sim.workload(WORKLOAD)
    rng = np.random.default_rng(sim.WORKLOADS[WORKLOAD]["seed"] + 1)
    perm = rng.permutation(tables.samples())
    size = tables.num_samples if hasattr(tables, "num_samples") else len(tables.samples())
    k = len(perm) // NUM_SETS
    sets = [np.sort(perm[j * k:(j + 1) * k]).astype(np.int32) for j in range(NUM_SETS)]
    del size
    windows = np.linspace(0, tables.sequence_length, NUM_WINDOWS + 1)
    return tables, sets, windows


def term_list():
    from tskit_gb300 import _native as nat

    pairs = [(i, j) for i in range(NUM_SETS) for j in range(i + 1, NUM_SETS)]
    triples = [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)]
    terms = [(nat.DIVERSITY, (k,)) for k in range(NUM_SETS)]
    terms += [(nat.SEGREGATING_SITES, (k,)) for k in range(NUM_SETS)]
    terms += [(nat.DIVERGENCE, p) for p in pairs]
    terms += [(nat.Y3, t) for t in triples]
    return terms, pairs, triples


def edge_events(tables):
    return int(tables.num_edges + np.count_nonzero(tables.edge_right < tables.sequence_length))


def algorithmic_bytes(tables, sets, num_terms):
    """Compulsory HBM bytes of one fused both-mode traversal."""
    E, N, S, M = tables.num_edges, tables.num_nodes, tables.num_sites, tables.num_mutations
    return (32 * E + 12 * N + 8 * S + 13 * M + 4 * sum(len(s) for s in sets)
            + 8 * NUM_WINDOWS * num_terms * 2)


def finish(raw, windows, sets, pairs):
    """Derived statistics from the fused raw (not span-normalised) terms."""
    span = np.diff(windows)[:, None]
    K = NUM_SETS
    out = {}
    for m, mode in enumerate(MODES):
        r = raw[m]
        div, seg = r[:, :K] / span, r[:, K:2 * K]
        dvg = r[:, 2 * K:2 * K + len(pairs)] / span
        y3 = r[:, 2 * K + len(pairs):] / span
        fst = np.ones_like(dvg)
        for i, (u, v) in enumerate(pairs):
            with np.errstate(divide="ignore", invalid="ignore"):
                fst[:, i] -= 2 * (div[:, u] + div[:, v]) / (div[:, u] + div[:, v] + 2 * dvg[:, i])
        n = np.array([len(s) for s in sets], dtype=np.float64)
        T = r[:, :K]
        h = np.array([np.sum(1 / np.arange(1, nn)) for nn in n])
        g = np.array([np.sum(1 / np.arange(1, nn) ** 2) for nn in n])
        with np.errstate(invalid="ignore", divide="ignore"):
            a = (n + 1) / (3 * (n - 1) * h) - 1 / h**2
            b = 2 * (n**2 + n + 3) / (9 * n * (n - 1)) - (n + 2) / (h * n) + g / h**2
            tajd = (T - seg / h) / np.sqrt(a * seg + (b / (h**2 + g)) * seg * (seg - 1))
        out[mode] = dict(diversity=div, divergence=dvg, Fst=fst, Tajimas_D=tajd, Y3=y3,
                         _T=T, _S=seg)
    return out


def rel_err(got, exp):
    """Normwise relative error per statistic column, worst column: the
    largest |got - exp| over the windows divided by the largest |exp| (values
    near zero, such as Fst between samples of one population, are measured
    against the statistic's scale)."""
    got, exp = np.asarray(got, dtype=np.float64), np.asarray(exp, dtype=np.float64)
    if got.size == 0:
        return 0.0
    if got.ndim == 1:
        got, exp = got[:, None], exp[:, None]
    with np.errstate(invalid="ignore", divide="ignore"):
        num = np.nanmax(np.abs(got - exp), axis=0)
        den = np.nanmax(np.abs(exp), axis=0)
        e = np.where(den > 0, num / den, num)
    return float(np.nanmax(e))


# --------------------------------------------------------------- CPU side
def _oracle_queries(ots, sets, windows, pairs, triples):
    """The reference's decomposition of the workload: one traversal per
    low-level call, unnormalised raw terms (Fst and Tajima's D reuse them)."""
    import oracle as O

    calls = []
    for mode in MODES:
        calls.append((mode, "diversity", [(O.DIVERSITY, (k,)) for k in range(NUM_SETS)]))
        calls.append((mode, "divergence", [(O.DIVERGENCE, p) for p in pairs]))
        calls.append((mode, "Fst.divergence", [(O.DIVERGENCE, p) for p in pairs]))
        calls.append((mode, "Fst.diversity", [(O.DIVERSITY, (k,)) for k in range(NUM_SETS)]))
        calls.append((mode, "TajD.diversity", [(O.DIVERSITY, (k,)) for k in range(NUM_SETS)]))
        calls.append((mode, "TajD.segsites", [(O.SEGSITES, (k,)) for k in range(NUM_SETS)]))
        calls.append((mode, "Y3", [(O.Y3, t) for t in triples]))
    return calls


_worker_state = {}


def _worker_init(npz_path):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from tskit_gb300.tables import Tables

    data = np.load(npz_path)
    tables = Tables.from_npz(data, prefix="tables/")
    _worker_state["ots"] = O.OracleTS(tables)
    _worker_state["sets"] = [data[f"set{k}"] for k in range(NUM_SETS)]
    _worker_state["windows"] = data["windows"]


def _worker_run(call):
    import oracle as O

    mode, _, terms = call
    t0 = time.perf_counter()
    r = O.sample_count_stat(_worker_state["ots"], _worker_state["sets"], terms,
                            windows=_worker_state["windows"], mode=mode, span_normalise=False)
    return time.perf_counter() - t0, r


def cpu_oracle_run(tables, sets, windows, pairs, triples):
    """Single-core oracle over the whole workload; returns (seconds, raw)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    ots = O.OracleTS(tables)
    calls = _oracle_queries(ots, sets, windows, pairs, triples)
    t0 = time.perf_counter()
    outs = {}
    for mode, name, terms in calls:
        outs[(mode, name)] = O.sample_count_stat(ots, sets, terms, windows=windows, mode=mode,
                                                 span_normalise=False)
    dt = time.perf_counter() - t0
    raw = np.zeros((2, NUM_WINDOWS, 2 * NUM_SETS + len(pairs) + len(triples)))
    for m, mode in enumerate(MODES):
        raw[m] = np.concatenate([outs[(mode, "diversity")], outs[(mode, "TajD.segsites")],
                                 outs[(mode, "divergence")], outs[(mode, "Y3")]], axis=1)
    return dt, raw, len(calls)


def max_over_ranks(value, world, device="cuda"):
    """The largest of a per-rank figure over the job (the slowest rank's
    time); the value itself on one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args):
    """--impl reference: the CPU path with all host threads, rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    import tempfile

    tables, sets, windows = make_workload()
    terms, pairs, triples = term_list()
    events = edge_events(tables)
    logical = events * REFERENCE_TRAVERSALS_PER_MODE * len(MODES)
    kind = "port"
    tmp = tempfile.NamedTemporaryFile(suffix=".npz", delete=False)
    arrays = tables.save_npz_dict("tables/")
    for k, s in enumerate(sets):
        arrays[f"set{k}"] = s
    arrays["windows"] = windows
    np.savez(tmp.name, **arrays)
    cores = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    calls = _oracle_queries(O.OracleTS(tables), sets, windows, pairs, triples)
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(min(cores, len(calls)), initializer=_worker_init, initargs=(tmp.name,)) as pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            pool.map(_worker_run, calls, chunksize=1)
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
    os.unlink(tmp.name)
    ms = 1e3 * float(np.mean(times))
    value = logical / (ms / 1e3)
    line = {
        "impl": "reference",
        "metric": "edge-updates/s",
        "value": value,
        "unit": "edge-updates/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded SMC generator)",
        "config": workload_config(tables),
        "cpu_baseline": {
            "value": value, "unit": "edge-updates/s", "cores": min(cores, len(calls)),
            "kind": kind,
            "sample": f"the full workload ({len(calls)} single-stat traversals, as the "
                      "reference runs them) spread over a process pool, one traversal per task",
        },
        "e2e": {"value": value, "unit": "edge-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def workload_config(tables):
    return {
        "workload": f"{WORKLOAD}: batched windowed stats, n=10000 samples, L=1e8, 100000 "
                    f"breakpoints -> {tables.num_edges} edges, {tables.num_sites} sites; "
                    f"{NUM_SETS} disjoint sets of 2500, {NUM_WINDOWS} windows; diversity, "
                    "divergence (6 pairs), Fst (6 pairs), Tajima's D, Y3 (4 triples); branch "
                    "and site modes",
        "num_edges": int(tables.num_edges),
        "num_nodes": int(tables.num_nodes),
        "num_sites": int(tables.num_sites),
        "num_samples": int(len(tables.samples())),
        "l2": "flushed between timed steps (256 MiB write)",
        "traversals_counted_per_step": REFERENCE_TRAVERSALS_PER_MODE * len(MODES),
    }


# --------------------------------------------------------------- GPU side
class ClockSampler:
    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(REPO, ".cache", f"clocks_{os.getpid()}.csv")

    def _lines(self):
        try:
            with open(self.path) as f:
                return sum(1 for _ in f)
        except OSError:
            return 0

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            # line-buffered (stdbuf) so that each sample reaches the file
            # as it is taken, not when the sampler is stopped
            import shutil

            prefix = ["stdbuf", "-oL"] if shutil.which("stdbuf") else []
            self.proc = subprocess.Popen(
                prefix + ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL, bufsize=0)
        except Exception:
            self.proc = None
        # the sampler is running (its first sample written) before the
        # region starts, so a region shorter than its start-up is covered
        self.start_lines = 0
        if self.proc is not None:
            t0 = time.time()
            while self._lines() < 1 and time.time() - t0 < 5 and self.proc.poll() is None:
                time.sleep(0.01)
            self.start_lines = self._lines()
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            # at least one sample taken after the region started
            t0 = time.time()
            while (self._lines() <= self.start_lines and time.time() - t0 < 2
                   and self.proc.poll() is None):
                time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.f.close()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 7:
                    continue
                try:
                    sm.append(float(parts[0]))
                    mx.append(float(parts[1]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[3:7]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except FileNotFoundError:
            pass
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def profile_traffic():
    """DRAM bytes (read + write) of one compact replay launch on this
    workload, from the committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", "replay_compact_windowed_n10k.json")
    try:
        with open(p) as f:
            return json.load(f).get("dram_bytes_per_launch")
    except Exception:
        return None


def replay_algorithmic_bytes(tables, plan, kq=1):
    """Compulsory bytes of one compact replay launch (k_replay_compact):
    per edge its insertion and removal encodings (16) and at most one leaf
    mask per event (8); per tree its event, mutation and item ranges (40); per
    mutation its encoding (4) and the counts written under it (8 per count
    word); per span its sample-range endpoints (8 each) with the set-member
    counts before them (8 per count word, written by k_compact_rows), and its
    nodes' start parents and times (2 + 8 per node); every item written (16
    per count word + 16) with its two FP64 branch lengths (16).  The
    depth-first sample orders and the sample masks are read by
    k_compact_rows, not by the replay."""
    E, M = tables.num_edges, tables.num_mutations
    return (24 * E + 40 * plan["num_trees"] + (4 + 8 * kq) * M
            + (8 + 8 * kq) * plan["compact_endpoints"] + 10 * plan["compact_nodes"]
            + (16 * kq + 32) * plan["num_items"])


def run_gpu(args):
    import torch

    import tskit_gb300
    from tskit_gb300 import _build, _native as nat, tune

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    _build.build_all()
    lib = nat.load()

    tables, sets, windows = make_workload()
    terms, pairs, triples = term_list()
    events = edge_events(tables)
    traversals = REFERENCE_TRAVERSALS_PER_MODE * len(MODES)
    logical = events * traversals

    stream = torch.cuda.current_stream()

    def prepare(ts, precision):
        q = ts.query(sets, terms, windows=windows, both_modes=True, span_normalise=False,
                     precision=precision)
        ws = tskit_gb300.Workspace(q.workspace_bytes)
        res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
        return q, ws, res

    def tuning_step(ts):
        q, ws, res = prepare(ts, "f64")
        return lambda: q.launch(ws, res, stream)

    # the compact replay's span count is autotuned for this tree sequence
    # and fused query
    ts = tskit_gb300.TreeSequence(tables)
    tuned = tune.tune_compact_spans(ts, tuning_step, key=WORKLOAD, steps=3, warmup=1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed_fused(precision, steps, with_clocks=False):
        """Warm-up, then `steps` launches each after an L2 flush; returns the
        mean step and sweep-kernel times (CUDA events on the launch stream),
        the launches per step, the (2, windows, terms) raw result and the
        clock sampler."""
        q, ws, res = prepare(ts, precision)
        ev_sweep0 = torch.cuda.Event(enable_timing=True)
        ev_sweep1 = torch.cuda.Event(enable_timing=True)
        ev_rep0 = torch.cuda.Event(enable_timing=True)
        ev_rep1 = torch.cuda.Event(enable_timing=True)
        # torch creates the CUDA events on first record; the library
        # re-records them around the sweep kernels and around the replay
        # kernel of every launch
        for ev in (ev_sweep0, ev_sweep1, ev_rep0, ev_rep1):
            ev.record(stream)
        torch.cuda.synchronize()
        lib.tsg_query_set_sweep_events(q.handle, ev_sweep0.cuda_event, ev_sweep1.cuda_event)
        lib.tsg_query_set_replay_events(q.handle, ev_rep0.cuda_event, ev_rep1.cuda_event)
        for _ in range(args.warmup):
            flush.zero_()
            q.launch(ws, res, stream)
        torch.cuda.synchronize()
        q.check(ws)
        step_ms, sweep_ms, rep_ms = [], [], []
        launches0 = lib.tsg_launch_count()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local) if with_clocks else None
        if sampler is not None:
            sampler.__enter__()
        try:
            for _ in range(steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                q.launch(ws, res, stream)
                e1.record(stream)
                torch.cuda.synchronize()
                step_ms.append(e0.elapsed_time(e1))
                sweep_ms.append(ev_sweep0.elapsed_time(ev_sweep1))
                rep_ms.append(ev_rep0.elapsed_time(ev_rep1))
            torch.cuda.synchronize()
        finally:
            if sampler is not None:
                sampler.__exit__(None, None, None)
        launches = (lib.tsg_launch_count() - launches0) / steps
        q.check(ws)
        raw = res.cpu().numpy().reshape(2, NUM_WINDOWS, len(terms))
        return (max_over_ranks(float(np.mean(step_ms)), world), float(np.mean(sweep_ms)),
                launches, raw, sampler, float(np.mean(rep_ms)))

    def timed_graph(precision, steps):
        """The same fused launch captured once in a CUDA graph (the side
        streams' forks and joins become graph edges) and replayed each step
        after an L2 flush; returns the mean step time (CUDA events on the
        launch stream, max over ranks), the clock sampler and the raw
        result."""
        q, ws, res = prepare(ts, precision)
        st = torch.cuda.Stream()
        st.wait_stream(stream)
        with torch.cuda.stream(st):
            for _ in range(2):
                q.launch(ws, res, st)
        st.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=st):
            q.launch(ws, res, st)
        torch.cuda.synchronize()
        for _ in range(args.warmup):
            flush.zero_()
            g.replay()
        torch.cuda.synchronize()
        q.check(ws)
        times = []
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        sampler.__enter__()
        try:
            for _ in range(steps):
                flush.zero_()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                g.replay()
                e1.record(stream)
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
        finally:
            sampler.__exit__(None, None, None)
        q.check(ws)
        raw = res.cpu().numpy().reshape(2, NUM_WINDOWS, len(terms))
        return max_over_ranks(float(np.mean(times)), world), sampler, raw

    # the headline: one fused sweep at the reference's precision (FP64 window
    # and running sums; summaries as exact integer numerators with about one
    # FP64 fused multiply-add per item), enqueued from the host each step ...
    ms, sweep, launches, raw_batched, clocks, rep = timed_fused("f64", args.steps,
                                                                 with_clocks=True)
    eager = {"ms_per_step": ms, "value": world * logical / (ms / 1e3),
             "note": "the fused launch enqueued from the host each step (14 kernels, "
                     "memsets and the side streams' event forks and joins)"}
    # ... and replayed from a captured CUDA graph: the same kernels and work
    # each step, without the host's enqueue between them
    try:
        gms, gclocks, graw = timed_graph("f64", args.steps)
        eager["graph_result_equals_eager"] = bool(np.array_equal(graw, raw_batched))
        if eager["graph_result_equals_eager"]:
            ms, clocks = gms, gclocks
            eager["headline"] = "graph replay"
    except Exception as exc:  # the eager figure stands
        eager["graph_error"] = str(exc).splitlines()[0][:200]
    value = world * logical / (ms / 1e3)
    # the FP32-compensated form of the same sweep
    ms32, sweep32, _, raw_f32, _, _ = timed_fused("f32", max(3, min(args.steps, 10)))

    # plain FP64 per-query form: one launch per low-level call, FP64 throughout
    plain = []
    for mode in MODES:
        for name, tl in (("diversity", terms[:NUM_SETS]),
                         ("divergence", terms[2 * NUM_SETS:2 * NUM_SETS + len(pairs)]),
                         ("Fst.divergence", terms[2 * NUM_SETS:2 * NUM_SETS + len(pairs)]),
                         ("Fst.diversity", terms[:NUM_SETS]),
                         ("TajD.diversity", terms[:NUM_SETS]),
                         ("TajD.segsites", terms[NUM_SETS:2 * NUM_SETS]),
                         ("Y3", terms[2 * NUM_SETS + len(pairs):])):
            pq = ts.query(sets, tl, windows=windows, mode=mode, span_normalise=False,
                          precision="f64")
            pres = torch.zeros(pq.result_size, dtype=torch.float64, device="cuda")
            plain.append((mode, name, pq, pres))
    pws = tskit_gb300.Workspace(max(p[2].workspace_bytes for p in plain))
    for _, _, pq, pres in plain:
        pq.launch(pws, pres, stream)
    torch.cuda.synchronize()
    plain_ms = []
    for _ in range(max(1, min(args.steps, 5))):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _, _, pq, pres in plain:
            pq.launch(pws, pres, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
    plain_step_ms = float(np.mean(plain_ms))
    pout = {(m, n): r.cpu().numpy().reshape(NUM_WINDOWS, -1) for m, n, _, r in plain}
    raw_plain = np.zeros_like(raw_batched)
    for m, mode in enumerate(MODES):
        raw_plain[m] = np.concatenate([pout[(mode, "diversity")], pout[(mode, "TajD.segsites")],
                                       pout[(mode, "divergence")], pout[(mode, "Y3")]], axis=1)

    # e2e through the host-pointer C ABI (the headline's FP64 fused form):
    # host sample sets/windows in, host result out
    sizes = np.array([len(s) for s in sets], dtype=np.uint64)
    flat = np.concatenate(sets).astype(np.int32)
    e2e_ms = []
    host = None
    for j in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host = ts._ll_terms(terms, sizes, flat, windows, None, False, False,
                            extra=nat.STAT_BOTH_MODES)
        dt = time.perf_counter() - t0
        if j >= args.warmup:
            e2e_ms.append(dt * 1e3)
    e2e_ms = max_over_ranks(float(np.mean(e2e_ms)), world)
    e2e_value = world * logical / (e2e_ms / 1e3)
    h2d = int(sizes.nbytes + flat.nbytes + windows.nbytes + ts.num_samples * 4)
    d2h = int(host.nbytes)

    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return

    peaks, peak_kind = measured_peaks()
    algo = algorithmic_bytes(tables, sets, len(terms))
    achieved = algo / (sweep / 1e3) / 1e9
    plan = ts.plan_sizes()
    rep_algo = replay_algorithmic_bytes(tables, plan)
    rep_achieved = rep_algo / (rep / 1e3) / 1e9
    line = {
        "metric": "edge-updates/s",
        "value": value,
        "unit": "edge-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (window and running sums FP64; summaries as exact integer numerators, "
                 "about one FP64 FMA per item); int32 counts",
        "data": "synthetic (seeded SMC generator, tskit_gb300.sim)",
        "config": dict(workload_config(tables), num_compact_spans=tuned["num_spans"],
                       span_tuning_ms={str(k): v for k, v in tuned["ms"].items()}),
        "eager_launch": eager,
        "queries_per_s": world * traversals / (ms / 1e3),
        "physical_edge_updates_per_s": world * events / (ms / 1e3),
        "batched_f32_kahan": {
            "ms_per_step": ms32,
            "value": world * logical / (ms32 / 1e3),
            "kernel_ms": sweep32,
            "dtype": "f32 summaries with exact products and compensated sums; f64 windows",
        },
        "plain_fp64": {
            "ms_per_step": plain_step_ms,
            "value": world * logical / (plain_step_ms / 1e3),
            "launches": len(plain),
            "speedup_batched_vs_plain": plain_step_ms / ms,
            "speedup_batched_f32_vs_plain": plain_step_ms / ms32,
        },
        "e2e": {"value": e2e_value, "unit": "edge-updates/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {
            "bound": "hbm",
            "achieved": rep_achieved,
            "peak": peaks["hbm_gbs"],
            "unit": "GB/s",
            "frac": rep_achieved / peaks["hbm_gbs"],
            "traffic": profile_traffic(),
            "kernel": "k_replay_compact (the dominant kernel), timed between events on the "
                      "launch stream around it",
            "algorithmic_bytes_per_launch": rep_algo,
            "kernel_ms": rep,
            "peak_source": peak_kind,
            "plan": plan,
        },
        "pipeline": {
            "kernel_ms": sweep,
            "algorithmic_bytes_per_launch": algo,
            "achieved_gbs": achieved,
            "frac": achieved / peaks["hbm_gbs"],
            "note": "every kernel of one fused launch from the node masks to the site sums, "
                    "against the traversal's compulsory bytes",
        },
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if rank == 0:
        # batching across resident tree sequences (outside the timed region):
        # one fused query each on six smaller sequences, one launch per
        # stage for all of them against their own launches
        from tskit_gb300 import sim

        small = {f"n{n}_{i}": tskit_gb300.TreeSequence(sim.simulate(n, 1e7, 5 * n, 5 * n, 3000 + i))
                 for i, n in enumerate([1000, 2000, 5000, 10000, 20000, 20000])}
        line["batch_across_tree_sequences"] = batch_vs_single(small)
    if not args.no_cpu_baseline:
        cpu_s, raw_oracle, ncalls = cpu_oracle_run(tables, sets, windows, pairs, triples)
        line["cpu_baseline"] = {
            "value": logical / cpu_s, "unit": "edge-updates/s", "cores": 1, "kind": "port",
            "sample": f"the full workload: {ncalls} single-stat traversals of the C oracle "
                      "(restated reference algorithm), one core",
        }
        raw_dd = compensated_branch(tables, sets, windows, terms)
        line["error"] = error_report(
            {"batched_f64": raw_batched, "batched_f32k": raw_f32, "plain_f64": raw_plain,
             "e2e_f64": host.reshape(raw_batched.shape), "oracle_f64": raw_oracle},
            raw_oracle, raw_dd, windows, sets, pairs)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


def compensated_branch(tables, sets, windows, terms):
    """Branch-mode raw terms (not span-normalised) from the oracle's
    double-double restatement of the sweep."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    ots = O.OracleTS(tables)
    return O.branch_count_stat_dd(ots, sets, terms, windows=windows, span_normalise=False)


# Stated error bounds of the two arithmetic forms (normwise, conditioning
# scaled, see error_report): the FP64 form against the compensated oracle
# (branch) or the FP64 oracle (site, whose GPU sums are exact integers rounded
# once); the FP32-compensated form against the same.
ERROR_BOUNDS = {"f64": 1e-12, "f32k": 1e-5}


def error_report(forms, raw_oracle, raw_dd, windows, sets, pairs):
    """Errors of each form's statistics (raw terms and derived) against the
    FP64 oracle and, in branch mode, against the compensated oracle, with the
    stated bounds and every bound exceeded."""
    fin_o = finish(raw_oracle, windows, sets, pairs)
    dd = raw_oracle.copy()
    dd[0] = raw_dd
    fin_dd = finish(dd, windows, sets, pairs)
    out = {"vs_fp64_oracle": {}, "vs_compensated_oracle": {}, "bounds": ERROR_BOUNDS,
           "measure": "normwise per statistic column: max over windows of |error| / max over "
                      "windows of the statistic's componentwise condition scale in its raw "
                      "terms (|value| for raw terms; sum |d stat / d term| |term| for Fst and "
                      "Tajima's D), worst column",
           "exceeded": []}
    for name, raw in forms.items():
        fin = finish(raw, windows, sets, pairs)
        bound = ERROR_BOUNDS.get(name.split("_")[-1])
        for mode in MODES:
            for stat in fin_o[mode]:
                if stat.startswith("_"):
                    continue
                e = None
                if name != "oracle_f64":
                    e = cond_err(fin[mode], fin_o[mode], stat, pairs, sets)
                    out["vs_fp64_oracle"][f"{mode}.{stat}.{name}"] = e
                if mode == "branch":
                    e = cond_err(fin[mode], fin_dd[mode], stat, pairs, sets)
                    out["vs_compensated_oracle"][f"{mode}.{stat}.{name}"] = e
                if name != "oracle_f64" and bound is not None and not (e <= bound):
                    out["exceeded"].append(f"{mode}.{stat}.{name}")
    return out


def cond_scale(fin, stat, pairs, sets):
    """Componentwise condition scale of each window value of a statistic in
    the raw (span-normalised) terms it is computed from."""
    if stat == "Fst":
        div, dvg = fin["diversity"], fin["divergence"]
        out = np.zeros_like(dvg)
        for i, (u, v) in enumerate(pairs):
            a = np.abs(div[:, u]) + np.abs(div[:, v])
            b = div[:, u] + div[:, v] + 2 * dvg[:, i]
            with np.errstate(divide="ignore", invalid="ignore"):
                out[:, i] = 8 * np.abs(dvg[:, i]) * a / b ** 2
        return out
    if stat == "Tajimas_D":
        T, S = fin["_T"], fin["_S"]
        n = np.array([len(s) for s in sets], dtype=np.float64)
        h = np.array([np.sum(1 / np.arange(1, nn)) for nn in n])
        g = np.array([np.sum(1 / np.arange(1, nn) ** 2) for nn in n])
        a = (n + 1) / (3 * (n - 1) * h) - 1 / h**2
        b = 2 * (n**2 + n + 3) / (9 * n * (n - 1)) - (n + 2) / (h * n) + g / h**2
        c = b / (h**2 + g)
        with np.errstate(divide="ignore", invalid="ignore"):
            V = a * S + c * S * (S - 1)
            dT = 1 / np.sqrt(V)
            dS = -1 / (h * np.sqrt(V)) - (T - S / h) * (a + c * (2 * S - 1)) / (2 * V ** 1.5)
            return np.abs(dT * T) + np.abs(dS * S)
    return np.abs(fin[stat])


def cond_err(fin, ref, stat, pairs, sets):
    """Normwise error of one statistic, scaled by its condition (see
    cond_scale); equal infinities and NaNs count as agreement."""
    got, exp = np.asarray(fin[stat], dtype=np.float64), np.asarray(ref[stat], dtype=np.float64)
    if got.size == 0:
        return 0.0
    scale = cond_scale(ref, stat, pairs, sets)
    with np.errstate(invalid="ignore", divide="ignore"):
        both_inf = np.isinf(got) & np.isinf(exp) & (np.sign(got) == np.sign(exp))
        diff = np.where(both_inf | (np.isnan(got) & np.isnan(exp)), 0.0, np.abs(got - exp))
        num = np.nanmax(np.where(np.isfinite(scale), diff, 0.0), axis=0)
        den = np.nanmax(np.where(np.isfinite(scale), scale, 0.0), axis=0)
        e = np.where(den > 0, num / den, num)
    return float(np.nanmax(e))


# ------------------------------------------------------- other configurations
def _timed_steps(fn, steps, warmup, flush, stream):
    import torch

    for _ in range(warmup):
        flush.zero_()
        fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1))
    return float(np.mean(out))


def run_afs_n200k(args):
    """AFS (site, branch; all samples and a joint 2 x 500) in 10 windows and
    the branch relatedness-vector product with 64 N(0,1) columns, centred, on
    n=200,000, L=1e8, 1,000,000 breakpoints."""
    import torch

    import tskit_gb300
    from tskit_gb300 import _build, _native as nat, sim, tune
    from tskit_gb300.trees import AfsQuery, RelatednessVectorQuery

    torch.cuda.set_device(0)
    _build.build_all()
    lib = nat.load()
    tables = sim.workload("afs_n200k")
    seed = sim.WORKLOADS["afs_n200k"]["seed"]
    rng = np.random.default_rng(seed + 1)
    perm = rng.permutation(tables.samples())
    joint = [np.sort(perm[:500]), np.sort(perm[500:1000])]
    allset = [tables.samples()]
    L = tables.sequence_length
    windows = np.linspace(0, L, 11)
    W = np.random.default_rng(seed + 2).normal(size=(len(tables.samples()), 64))
    stream = torch.cuda.current_stream()
    span = nat.STAT_SPAN_NORMALISE
    Wd = torch.from_numpy(W).cuda()

    def prepare(ts):
        qs = [AfsQuery(ts, s, windows, None, m | span)
              for s in (allset, joint) for m in (nat.STAT_SITE, nat.STAT_BRANCH)]
        mv = RelatednessVectorQuery(ts, 64, None, None, nat.STAT_BRANCH | span)
        mv.set_weights(Wd)
        qs.append(mv)
        ws = tskit_gb300.Workspace(max(q.workspace_bytes for q in qs))
        outs = [torch.zeros(q.result_size, dtype=torch.float64, device="cuda") for q in qs]

        def step():
            for q, o in zip(qs, outs):
                q.launch(ws, o, stream)
        return qs, ws, outs, step

    # the span count is autotuned for this tree sequence and step
    ts, tuned = tune.tune_num_spans(tables, lambda t: prepare(t)[3], key="afs_n200k",
                                    steps=2, warmup=1)
    qs, ws, outs, step = prepare(ts)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    launches0 = lib.tsg_launch_count()
    with ClockSampler(0) as clocks:
        ms = _timed_steps(step, args.steps, args.warmup, flush, stream)
    launches = (lib.tsg_launch_count() - launches0) / (args.steps + args.warmup)
    per_q = []
    for q, o in zip(qs, outs):
        per_q.append(_timed_steps(lambda q=q, o=o: q.launch(ws, o, stream), 2, 1, flush, stream))
    events = edge_events(tables)
    value = len(qs) * events / (ms / 1e3)
    # end to end through the host-pointer entry points
    t0 = time.perf_counter()
    host = [ts.allele_frequency_spectrum(s, windows=windows, mode=m)
            for s in (allset, joint) for m in ("site", "branch")]
    host.append(ts.genetic_relatedness_vector(W, mode="branch"))
    e2e_s = time.perf_counter() - t0
    peaks, peak_kind = measured_peaks()
    algo = len(qs) * (32 * tables.num_edges + 12 * tables.num_nodes + 8 * tables.num_sites
                      + 13 * tables.num_mutations)
    line = {
        "metric": "edge-updates/s", "value": value, "unit": "edge-updates/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int counts; f64 (AFS branch areas exact in 2^-128 fixed point)",
        "data": "synthetic (seeded SMC generator, tskit_gb300.sim)",
        "config": {"workload": "afs_n200k: n=200000, L=1e8, 1000000 breakpoints -> "
                               f"{tables.num_edges} edges, {tables.num_sites} sites; AFS "
                               "site+branch (all samples; joint 2 x 500), 10 windows; "
                               "relatedness x 64 vectors, branch, centred",
                   "queries_per_step": len(qs),
                   "ms_per_query": dict(zip(["afs_site_all", "afs_branch_all", "afs_site_joint",
                                             "afs_branch_joint", "relatedness_vector_w64"],
                                            per_q)),
                   "l2": "flushed between timed steps (256 MiB write)",
                   "num_spans": tuned["num_spans"],
                   "span_tuning_ms": {str(k): v for k, v in tuned["ms"].items()}},
        "queries_per_s": len(qs) / (ms / 1e3),
        "e2e": {"value": len(qs) * events / e2e_s, "unit": "edge-updates/s",
                "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(W.nbytes + sum(s.nbytes for s in joint)
                                          + 2 * allset[0].nbytes),
                "d2h_bytes_per_step": int(sum(h.nbytes for h in host))},
        "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9,
                     "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": algo / (ms / 1e3) / 1e9 / peaks["hbm_gbs"], "traffic": None,
                     "peak_source": peak_kind},
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle as O

        ots = O.OracleTS(tables)
        t0 = time.perf_counter()
        ref = [O.allele_frequency_spectrum(ots, s, windows=windows, mode=m)
               for s in (allset, joint) for m in ("site", "branch")]
        ref.append(O.genetic_relatedness_vector(ots, W))
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(qs) * events / cpu_s, "unit": "edge-updates/s",
                                "cores": 1, "kind": "port",
                                "sample": "the full step (4 AFS + 1 relatedness-vector call) "
                                          "through the C oracle, one core"}
        names = ["afs_site_all", "afs_branch_all", "afs_site_joint", "afs_branch_joint",
                 "relatedness_vector_w64"]
        errs = {name: rel_err(np.asarray(h).reshape(-1), np.asarray(r).reshape(-1))
                for name, h, r in zip(names, host, ref)}
        line["error_vs_fp64_oracle"] = errs
        # site AFS bins are exact counts scaled by the window span: identical
        # bit for bit; branch AFS and the relatedness product: normwise 1e-12
        site_identical = {name: bool(np.array_equal(np.asarray(h).reshape(-1),
                                                    np.asarray(r).reshape(-1)))
                          for name, h, r in zip(names, host, ref) if "site" in name}
        line["parity"] = {
            "site_afs_identical": site_identical,
            "bound": 1e-12,
            "pass": all(site_identical.values())
                    and all(v <= 1e-12 for k, v in errs.items() if "site" not in k)}
    print(json.dumps(line))


def run_grm_n20k(args):
    """Site-mode genetic relatedness matrix, n=20,000 samples, ~500,000
    sites: the exact E4M3 Gram on tcgen05 (timed alone on the resident
    operand) and the whole call (decode, operand, Gram, normalisation, 3.2 GB
    result to the host)."""
    import ctypes

    import torch

    import tskit_gb300
    from tskit_gb300 import _build, _native as nat, sim

    torch.cuda.set_device(0)
    _build.build_all()
    lib = nat.load()
    tables = sim.workload("grm_n20k")
    ts = tskit_gb300.TreeSequence(tables)
    n, S = len(tables.samples()), tables.num_sites
    kp = (S + 127) // 128 * 128
    G = torch.zeros((n, kp), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    st = ctypes.c_void_p(stream.cuda_stream)
    nat.check(lib.tsg_treeseq_genotype_operand(ts._handle, 0, S, ctypes.c_void_p(G.data_ptr()),
                                               kp, st))
    P = torch.zeros((n, n), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def gram():
        nat.check(lib.tsg_gram_e4m3(ctypes.c_void_p(G.data_ptr()), n, kp, kp,
                                    ctypes.c_void_p(P.data_ptr()), n, st))

    with ClockSampler(0) as clocks:
        ms = _timed_steps(gram, args.steps, args.warmup, flush, stream)
    nb = (n + 255) // 256
    tiles = nb * (nb + 1) // 2  # 256 x 256 tiles, row block <= column block
    executed = tiles * 256 * 256 * kp * 2
    t0 = time.perf_counter()
    K = ts.genetic_relatedness_matrix()
    e2e_s = time.perf_counter() - t0
    pairs = n * (n - 1) / 2 * S
    line = {
        "metric": "sample-pair site comparisons/s", "value": pairs / (ms / 1e3),
        "unit": "pair-sites/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "e4m3 0/1 operands, fp32 accumulation (exact integers), int32 result",
        "data": "synthetic (seeded SMC generator, tskit_gb300.sim)",
        "config": {"workload": f"grm_n20k: n={n} samples, {S} sites (L=1e8, 100000 "
                               "breakpoints); site-mode genetic_relatedness_matrix",
                   "gram_tiles": tiles, "operand_bytes": int(n * kp),
                   "l2": "flushed between timed steps (256 MiB write); operand 10 GB"},
        # genotypes are decoded on the device: the call uploads per-site
        # column indexes, the sample sets and the tile list
        "e2e": {"value": pairs / e2e_s, "unit": "pair-sites/s", "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(S * 8 + n * 16 + 4 + tiles * 8 + 16),
                "d2h_bytes_per_step": int(K.nbytes)},
        "roofline": {"bound": "tensor", "achieved": executed / (ms / 1e3) / 1e12,
                     "peak": 4500.0, "unit": "TFLOP/s",
                     "frac": executed / (ms / 1e3) / 1e12 / 4500.0, "traffic": None,
                     "peak_source": "nominal dense FP8 (no measured FP8 peak); "
                                    "measured bf16 burst " +
                                    str(measured_peaks()[0].get("bf16_tflops"))},
        "gpu_launches": 1, "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle as O

        ots = O.OracleTS(tables)
        line["parity"] = grm_parity(O, ots, G, P, K, n, S, kp)
        # the reference's site divergence-matrix loop (variant decode, then
        # every pair of samples carrying different alleles), one core, on a
        # run of sites from the middle of the genome
        sample, s0 = 64, S // 2
        t0 = time.perf_counter()
        O.divergence_counts_site_range(ots, s0, s0 + sample, symmetric=False)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n * (n - 1) / 2 * sample / cpu_s,
                                "unit": "pair-sites/s", "cores": 1, "kind": "port",
                                "sample": f"sites {s0}..{s0 + sample - 1} of {S}: the reference's "
                                          "site divergence-matrix loop (trees.c:8685-8826) "
                                          "through the C oracle, one core, scaled per "
                                          "pair-site"}
    print(json.dumps(line))


def grm_parity(O, ots, G, P, K, n, S, kp):
    """Full-size parity of the site-mode relatedness matrix.

    1. Operand: the device-decoded genotypes of 2,048 sites equal the
       oracle's decode for all samples.
    2. Gram: 64 blocks of 128 x 256 (8 random row blocks x 8 random column
       blocks) of the int32 product equal a CPU integer product of the same
       operand rows (float32 BLAS over 32,768-site slices, exact since each
       slice's sums stay below 2^24, summed in int64).  Entries below the
       diagonal, which the Gram does not compute, are read from the
       transposed entry.
    3. Rows: 8 random full rows of the product equal the oracle's exact
       shared-derived counts, and the same rows of the final matrix are
       within 1e-12 (normwise per row) of the oracle's exact rows."""
    import torch

    rng = np.random.default_rng(11)
    out = {}
    # 1. operand vs the oracle's genotypes
    s0 = int(rng.integers(0, S - 2048))
    geno = O.genotype_rows(ots, s0, s0 + 2048)
    dev = (G[:, s0:s0 + 2048] == 0x38).cpu().numpy().T
    # every operand byte is E4M3 0 or 1 (0x38), the padding columns 0
    bad = 0
    for i in range(0, n, 2048):
        g = G[i:i + 2048]
        bad += int(((g[:, :S] != 0) & (g[:, :S] != 0x38)).sum()) + int((g[:, S:] != 0).sum())
    out["operand_sites"] = [s0, s0 + 2048]
    out["operand_bad_bytes"] = bad
    out["operand_equal"] = bool(np.array_equal(dev, geno != 0)) and bad == 0

    def full(rows, cols):
        """Product entries (rows x cols), each read from a tile the Gram
        computes: 256 x 256 tiles with row block <= column block."""
        r = torch.as_tensor(rows, device=P.device)
        c = torch.as_tensor(cols, device=P.device)
        direct = P.index_select(0, r).index_select(1, c)
        transposed = P.index_select(1, r).index_select(0, c).T
        computed = (c // 256)[None, :] >= (r // 256)[:, None]
        return torch.where(computed, direct, transposed).cpu().numpy().astype(np.int64)

    # 2. tiles vs a CPU integer product of the operand
    rb = np.sort(rng.choice(n // 128, 8, replace=False)) * 128
    cb = np.sort(rng.choice(n // 256, 8, replace=False)) * 256
    rows = (rb[:, None] + np.arange(128)).reshape(-1)
    cols = (cb[:, None] + np.arange(256)).reshape(-1)
    Xr = G[torch.as_tensor(rows, device=G.device)].cpu().numpy()
    Xc = G[torch.as_tensor(cols, device=G.device)].cpu().numpy()
    cpu = np.zeros((len(rows), len(cols)), dtype=np.int64)
    t0 = time.perf_counter()
    for k0 in range(0, kp, 32768):
        a = (Xr[:, k0:k0 + 32768] == 0x38).astype(np.float32)
        b = (Xc[:, k0:k0 + 32768] == 0x38).astype(np.float32)
        cpu += (a @ b.T).astype(np.int64)
    gpu = full(rows, cols)
    out["tiles"] = {"count": 64, "row_blocks": rb.tolist(), "col_blocks": cb.tolist(),
                    "entries": int(cpu.size), "mismatches": int(np.sum(cpu != gpu)),
                    "cpu_s": time.perf_counter() - t0}
    # 3. full rows vs the oracle's exact rows
    pick = np.sort(rng.choice(n, 8, replace=False))
    Kexp, Gexp = O.relatedness_rows_site(ots, pick)
    Grow = full(pick, np.arange(n))
    Krow = K[pick]
    out["rows"] = {"samples": pick.tolist(), "product_mismatches": int(np.sum(Grow != Gexp)),
                   "relatedness_max_rel_err": float(np.max(np.abs(Krow - Kexp))
                                                    / np.max(np.abs(Kexp))),
                   "bound": 1e-12}
    out["pass"] = (out["operand_equal"] and out["tiles"]["mismatches"] == 0
                   and out["rows"]["product_mismatches"] == 0
                   and out["rows"]["relatedness_max_rel_err"] <= 1e-12)
    return out


def run_serve_mix(args):
    """Eight resident tree sequences (n = 1k..200k, L = 1e8, breakpoints =
    5n); a Poisson stream of diversity / divergence / Fst / AFS / relatedness
    x 8 requests (sets of 10-10,000 samples, 1-1,000 equal windows, branch or
    site) arriving faster than the server absorbs them, served batched
    (fused queries grouped across tree sequences, 8 stream slots) and one at
    a time with a synchronous FP64 launch each."""
    import torch

    import tskit_gb300
    from tskit_gb300 import _build, sim
    from tskit_gb300.serve import GpuBackend, Server, poisson_requests

    torch.cuda.set_device(0)
    _build.build_all()
    ns = [1000, 2000, 5000, 20000, 20000, 50000, 100000, 200000]
    resident = {f"n{n}_{i}": tskit_gb300.TreeSequence(sim.simulate(n, 1e8, 5 * n, 5 * n, 2000 + i))
                for i, n in enumerate(ns)}
    batch_cmp = batch_vs_single(resident)
    num, rate = args.serve_queries, args.serve_rate
    reqs = poisson_requests(resident, num, rate, 7)
    be = GpuBackend(resident, num_slots=8)
    Server(be, num_slots=8).run(poisson_requests(resident, 60, 1e4, 8))  # warm-up
    with ClockSampler(0) as clocks:
        launches0 = be_launches()
        b = Server(be, num_slots=8).run(reqs)
        launches = be_launches() - launches0
    p = Server(GpuBackend(resident, num_slots=1), num_slots=1).run(reqs, mode="plain")
    served = [r for r in reqs if r.rid in b.results]
    h2d = sum(sum(len(s) * 4 for s in r.sample_sets)
              + (r.weights.nbytes if r.weights is not None else 0) for r in served)
    d2h = sum(np.asarray(b.results[r.rid]).nbytes for r in served)
    line = {
        "metric": "queries/s", "value": b.queries_per_s, "unit": "queries/s", "n_gpus": 1,
        "steps": b.num, "warmup": 60, "ms_per_step": 1e3 / b.queries_per_s,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": f"synthetic (seeded SMC generator; Poisson arrivals at {rate:g} requests/s, "
                "above the server's rate)",
        "config": {"workload": "serve_mix: 8 resident tree sequences n=" + ",".join(map(str, ns))
                               + ", L=1e8, breakpoints=5n; requests diversity / divergence / Fst "
                                 "/ AFS / relatedness x 8, sets of 10-10000, 1/10/100/1000 "
                                 "windows, branch or site",
                   "stream": f"{num} requests (a subset of the 100,000-request stream: at the "
                             "measured rates the full stream takes tens of minutes per arm); "
                             "results over 256 MiB rejected and counted",
                   "batched": b.summary(), "plain_one_at_a_time": p.summary()},
        "p50_ms": b.percentile_ms(50), "p99_ms": b.percentile_ms(99),
        "rejected": len(b.rejected),
        "plain": {"queries_per_s": p.queries_per_s, "p50_ms": p.percentile_ms(50),
                  "p99_ms": p.percentile_ms(99)},
        "e2e": {"value": b.queries_per_s, "unit": "queries/s",
                "h2d_bytes_per_step": int(h2d / max(1, b.num)),
                "d2h_bytes_per_step": int(d2h / max(1, b.num))},
        "gpu_launches": launches / max(1, b.num), "clocks": clocks.summary(),
        "batch_across_tree_sequences": batch_cmp,
    }
    print(json.dumps(line))


def batch_vs_single(resident, reps=20):
    """One fused query per resident tree sequence the batched kernels take
    (diversity and divergence of two random sets of 200, 10 windows, both
    modes, FP64), launched one by one on one stream and as one QueryBatch;
    device time per round of all the queries (CUDA events, median of
    `reps`), and the results compared bit for bit."""
    import torch

    import tskit_gb300
    from tskit_gb300 import _native as nat

    qs = []
    for i, (key, ts) in enumerate(sorted(resident.items())):
        if ts.num_samples > 65535:
            continue
        rng = np.random.default_rng(50 + i)
        perm = rng.permutation(ts.samples())
        sets = [np.sort(perm[:200]), np.sort(perm[200:400])]
        L = ts.sequence_length
        qs.append(ts.query(sets, [(nat.DIVERSITY, (0,)), (nat.DIVERSITY, (1,)),
                                  (nat.DIVERGENCE, (0, 1))],
                           windows=np.linspace(0, L, 11), both_modes=True))
    ws1 = [tskit_gb300.Workspace(q.workspace_bytes) for q in qs]
    own = [torch.zeros(q.result_size, dtype=torch.float64, device="cuda") for q in qs]
    res = [torch.zeros(q.result_size, dtype=torch.float64, device="cuda") for q in qs]
    batch = tskit_gb300.QueryBatch(qs, res, tskit_gb300.Workspace())
    st = torch.cuda.current_stream()

    def time_it(fn):
        ts_ = []
        for r in range(reps + 3):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            fn()
            b.record(st)
            torch.cuda.synchronize()
            if r >= 3:
                ts_.append(a.elapsed_time(b))
        return float(np.median(ts_))

    lib = nat.load()
    l0 = lib.tsg_launch_count()
    single_ms = time_it(lambda: [q.launch(w, o, st) for q, w, o in zip(qs, ws1, own)])
    l1 = lib.tsg_launch_count()
    batch_ms = time_it(lambda: batch.launch(st))
    l2 = lib.tsg_launch_count()
    batch.check()
    equal = all(torch.equal(a.view(torch.int64), b.view(torch.int64)) for a, b in zip(own, res))
    return {"queries": len(qs), "fused": batch.num_fused,
            "tree_sequences": [int(q.ts.num_samples) for q in qs],
            "one_by_one_ms": single_ms, "batched_ms": batch_ms,
            "launches_one_by_one": (l1 - l0) / (reps + 3), "launches_batched": (l2 - l1) / (reps + 3),
            "bitwise_equal": bool(equal)}


def be_launches():
    from tskit_gb300 import _native as nat

    return nat.load().tsg_launch_count()


def run_profile(args):
    """--profile: the headline query alone, warmup + steps launches."""
    import torch

    import tskit_gb300
    from tskit_gb300 import _build

    torch.cuda.set_device(0)
    _build.build_all()
    tables, sets, windows = make_workload()
    terms, _, _ = term_list()
    ts = tskit_gb300.TreeSequence(tables)
    q = ts.query(sets, terms, windows=windows, both_modes=True, span_normalise=False,
                 precision=args.profile)
    ws = tskit_gb300.Workspace(q.workspace_bytes)
    res = torch.zeros(q.result_size, dtype=torch.float64, device="cuda")
    for _ in range(args.warmup + args.steps):
        q.launch(ws, res)
    torch.cuda.synchronize()
    q.check(ws)
    print(json.dumps({"profile": args.profile, "launches": args.warmup + args.steps,
                      "plan": ts.plan_sizes()}))


def main():
    args = parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.workload == "afs_n200k":
        run_afs_n200k(args)
    elif args.workload == "grm_n20k":
        run_grm_n20k(args)
    elif args.workload == "serve_mix":
        run_serve_mix(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
