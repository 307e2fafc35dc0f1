"""Serving loop: statistics queries against tree sequences resident in HBM.

Several tree sequences stay on the device with their span plans.  Requests
(diversity, divergence, Fst, allele frequency spectrum, relatedness x
vectors) arrive over time; the loop

* admits every request that has arrived,
* batches compatible waiting requests into one fused launch -- sample-count
  statistics on the same tree sequence, mode and windows share one sweep
  (up to 8 sample sets; 4 when sample counts need 32 bits), and
  relatedness-vector requests on the same tree sequence and windows share
  one product with their weight columns side by side,
* launches a batch as soon as a stream slot is free and the device memory
  its workspace needs fits the budget (continuous batching: new requests
  join while earlier launches are still running, and launches on different
  slots overlap on the device),
* completes requests as their launch's event fires and records latency
  (completion - arrival).

``Server(backend).run(requests)`` drives a request stream; ``GpuBackend``
executes on the CUDA device through the library's prepared queries, and the
same loop runs against a host-only backend in the tests.  ``mode="plain"``
serves one request at a time with one synchronous launch each, the baseline
the batched loop is compared with.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import _native as nat

KINDS = {"diversity": "counts", "divergence": "counts", "Fst": "counts",
         "afs": "afs", "relatedness_vector": "rv"}


@dataclass
class Request:
    rid: int
    arrival: float            # seconds after the start of the stream
    ts: str                   # key of a resident tree sequence
    stat: str                 # one of KINDS
    sample_sets: list         # arrays of sample node ids
    windows: np.ndarray | None
    mode: str                 # "branch" or "site"
    weights: np.ndarray | None = None  # relatedness_vector: num_samples x columns

    @property
    def kind(self):
        return KINDS[self.stat]

    def batch_key(self):
        nw = 0 if self.windows is None else len(self.windows)
        return (self.ts, self.kind, self.mode, nw)


def poisson_requests(resident, num, rate, seed, window_choices=(1, 10, 100, 1000),
                     set_range=(10, 10000), rv_columns=8, sequence_length=None):
    """A Poisson stream of `num` requests at `rate` per second over the
    resident tree sequences (dict key -> object with ``samples()`` and
    ``sequence_length``): statistics drawn uniformly, sample sets of
    set_range samples (uniform), windows equal over the genome with a count
    drawn from window_choices, mode branch or site (relatedness vectors are
    branch-only)."""
    rng = np.random.default_rng(seed)
    keys = sorted(resident)
    stats = list(KINDS)
    out = []
    t = 0.0
    for rid in range(num):
        t += rng.exponential(1.0 / rate)
        key = keys[rng.integers(len(keys))]
        ts = resident[key]
        samples = np.asarray(ts.samples())
        L = ts.sequence_length if sequence_length is None else sequence_length
        stat = stats[rng.integers(len(stats))]
        mode = "branch" if stat == "relatedness_vector" else ("branch", "site")[rng.integers(2)]
        nwin = int(window_choices[rng.integers(len(window_choices))])
        windows = None if nwin == 1 else np.linspace(0, L, nwin + 1)
        nsets = 2 if stat in ("divergence", "Fst") else 1
        hi = min(set_range[1], len(samples) // nsets)
        m = int(rng.integers(min(set_range[0], hi), hi + 1))
        perm = rng.permutation(samples)
        sets = [np.sort(perm[j * m:(j + 1) * m]) for j in range(nsets)]
        weights = None
        if stat == "relatedness_vector":
            # an output of windows x samples x columns: at most 64 MiB
            cap = max(1, (64 << 20) // (len(samples) * rv_columns * 8))
            if nwin > cap:
                nwin = 1
                windows = None
            sets = []
            weights = rng.normal(size=(len(samples), rv_columns))
        out.append(Request(rid, t, key, stat, sets, windows, mode, weights))
    return out


@dataclass
class Batch:
    requests: list
    work: object = None       # the backend's launch record
    slot: int = -1
    nbytes: int = 0
    finished: bool = False


@dataclass
class ServeStats:
    mode: str
    num: int
    wall_s: float
    latencies_s: np.ndarray
    launches: int
    results: dict = field(default_factory=dict)

    @property
    def queries_per_s(self):
        return self.num / self.wall_s if self.wall_s > 0 else float("inf")

    def percentile_ms(self, p):
        return float(np.percentile(self.latencies_s, p) * 1e3) if self.num else 0.0

    def summary(self):
        return {"mode": self.mode, "queries": self.num, "wall_s": round(self.wall_s, 4),
                "queries_per_s": round(self.queries_per_s, 2),
                "p50_ms": round(self.percentile_ms(50), 3),
                "p99_ms": round(self.percentile_ms(99), 3), "launches": self.launches}


class Server:
    """The request loop over a backend (see GpuBackend for the interface)."""

    def __init__(self, backend, num_slots=8, hbm_budget=64 << 30, max_batch=32,
                 max_output_bytes=256 << 20):
        self.backend = backend
        self.num_slots = num_slots
        self.hbm_budget = hbm_budget
        self.max_batch = max_batch
        self.max_output_bytes = max_output_bytes

    def _form_batch(self, pending):
        """The oldest waiting request and the compatible ones behind it."""
        head = pending[0]
        key = head.batch_key()
        taken = [head]
        if head.kind != "afs":
            sets_cap = self.backend.max_sets(head.ts)
            nsets = len(head.sample_sets)
            nwin = 1 if head.windows is None else len(head.windows) - 1
            cols = 0 if head.weights is None else head.weights.shape[1]
            for r in pending[1:]:
                if len(taken) >= self.max_batch:
                    break
                if r.batch_key() != key or (r.windows is not None and not np.array_equal(
                        r.windows, head.windows)):
                    continue
                if head.kind == "counts":
                    if nsets + len(r.sample_sets) > sets_cap:
                        continue
                    nsets += len(r.sample_sets)
                else:
                    c = cols + r.weights.shape[1]
                    if nwin * len(r.weights) * c * 8 > self.max_output_bytes:
                        continue
                    cols = c
                taken.append(r)
        return taken

    def run(self, requests, mode="batched", clock=time.perf_counter, idle=None):
        reqs = sorted(requests, key=lambda r: r.arrival)
        n = len(reqs)
        lat = np.zeros(n)
        pos = {r.rid: i for i, r in enumerate(reqs)}
        results = {}
        pending = []
        busy = {}  # slot -> Batch
        slot_bytes = [0] * self.num_slots
        nxt = 0
        done = 0
        launches = 0
        t0 = clock()
        while done < n:
            now = clock() - t0
            while nxt < n and reqs[nxt].arrival <= now:
                pending.append(reqs[nxt])
                nxt += 1
            progressed = False
            # completions
            for s, b in list(busy.items()):
                if self.backend.ready(b.work):
                    out = self.backend.results(b.work)
                    t = clock() - t0
                    for r in b.requests:
                        lat[pos[r.rid]] = t - r.arrival
                        results[r.rid] = out[r.rid]
                        done += 1
                    del busy[s]
                    progressed = True
            # admissions
            while pending and (mode == "batched" or not busy):
                free = [s for s in range(self.num_slots) if s not in busy]
                if not free:
                    break
                batch = Batch(self._form_batch(pending) if mode == "batched" else [pending[0]])
                b_bytes = self.backend.workspace_bytes(batch.requests)
                s = free[0]
                others = sum(slot_bytes[o] for o in busy)
                need = max(slot_bytes[s], b_bytes)
                if busy and others + need > self.hbm_budget:
                    self.backend.discard(batch.requests)
                    break  # wait for memory
                for r in batch.requests:
                    pending.remove(r)
                slot_bytes[s] = need
                batch.work = self.backend.launch(batch.requests, s)
                batch.slot = s
                busy[s] = batch
                launches += 1
                progressed = True
                if mode == "plain":
                    self.backend.wait(batch.work)
            if not progressed:
                if idle is not None:
                    idle(reqs[nxt].arrival if nxt < n else None, busy)
                elif not busy and nxt < n:
                    gap = reqs[nxt].arrival - (clock() - t0)
                    if gap > 2e-4:
                        time.sleep(gap - 1e-4)
        wall = clock() - t0
        return ServeStats(mode, n, wall, lat, launches, results)


# ---------------------------------------------------------------- GPU backend
class GpuBackend:
    """Launches on CUDA streams through the library's prepared queries.

    ``resident``: dict key -> tskit_gb300.TreeSequence.  Each slot owns a
    stream and a workspace that grows to the largest launch it ran."""

    def __init__(self, resident, num_slots=8):
        import torch

        from .trees import Workspace

        self.torch = torch
        self.resident = resident
        self.streams = [torch.cuda.Stream() for _ in range(num_slots)]
        self.workspaces = [Workspace() for _ in range(num_slots)]
        self._prepared = {}

    def max_sets(self, key):
        return 8 if self.resident[key].num_samples <= 65535 else 4

    # ---- preparation (host): one fused query per batch
    def _prepare(self, reqs):
        from .trees import AfsQuery, Query, RelatednessVectorQuery

        head = reqs[0]
        ts = self.resident[head.ts]
        flags = (nat.STAT_BRANCH if head.mode == "branch" else nat.STAT_SITE)
        flags |= nat.STAT_SPAN_NORMALISE
        if head.kind == "afs":
            q = AfsQuery(ts, head.sample_sets, head.windows, None, flags)
            return q, None
        if head.kind == "rv":
            cols = sum(r.weights.shape[1] for r in reqs)
            q = RelatednessVectorQuery(ts, cols, head.windows, None, flags)
            W = np.ascontiguousarray(np.concatenate([r.weights for r in reqs], axis=1))
            return q, W
        sets, terms, plan = [], [], []
        for r in reqs:
            base = len(sets)
            sets.extend(r.sample_sets)
            t0 = len(terms)
            if r.stat == "diversity":
                terms.append((nat.DIVERSITY, (base,)))
            elif r.stat == "divergence":
                terms.append((nat.DIVERGENCE, (base, base + 1)))
            else:  # Fst from diversities and the divergence (trees.py:10076-10126)
                terms += [(nat.DIVERSITY, (base,)), (nat.DIVERSITY, (base + 1,)),
                          (nat.DIVERGENCE, (base, base + 1))]
            plan.append((r, t0, len(terms)))
        q = Query(ts, sets, terms, head.windows, flags)
        return q, plan

    def workspace_bytes(self, reqs):
        key = tuple(r.rid for r in reqs)
        if key not in self._prepared:
            self._prepared[key] = self._prepare(reqs)
        return self._prepared[key][0].workspace_bytes

    def discard(self, reqs):
        self._prepared.pop(tuple(r.rid for r in reqs), None)

    def launch(self, reqs, slot):
        torch = self.torch
        key = tuple(r.rid for r in reqs)
        q, extra = self._prepared.pop(key) if key in self._prepared else self._prepare(reqs)
        st = self.streams[slot]
        with torch.cuda.stream(st):
            res = torch.empty(q.result_size, dtype=torch.float64, device="cuda")
            W = None
            if reqs[0].kind == "rv":
                W = torch.from_numpy(extra).to("cuda", non_blocking=False)
                q.set_weights(W)
            q.launch(self.workspaces[slot], res, stream=st)
            host = torch.empty(q.result_size, dtype=torch.float64, pin_memory=True)
            host.copy_(res, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(st)
        return {"q": q, "extra": extra, "reqs": reqs, "res": res, "host": host, "ev": ev,
                "W": W, "slot": slot}

    def ready(self, work):
        return work["ev"].query()

    def wait(self, work):
        work["ev"].synchronize()

    def results(self, work):
        q, reqs = work["q"], work["reqs"]
        q.check(self.workspaces[work["slot"]])
        y = work["host"].numpy()
        out = {}
        head = reqs[0]
        if head.kind == "afs":
            out[head.rid] = y.reshape(q.shape)
        elif head.kind == "rv":
            Y = y.reshape(q.shape)
            c = 0
            for r in reqs:
                k = r.weights.shape[1]
                out[r.rid] = Y[:, :, c:c + k]
                c += k
        else:
            Y = y.reshape(q.num_windows, q.num_terms)
            for r, a, b in work["extra"]:
                v = Y[:, a:b]
                if r.stat == "Fst":
                    du, dv, dx = v[:, 0], v[:, 1], v[:, 2]
                    with np.errstate(divide="ignore", invalid="ignore"):
                        v = (1 - 2 * (du + dv) / (du + dv + 2 * dx))[:, None]
                out[r.rid] = v
        return out
