"""Serving loop: statistics queries against tree sequences resident in HBM.

Several tree sequences stay on the device with their span plans.  Requests
(diversity, divergence, Fst, allele frequency spectrum, relatedness x
vectors) arrive over time; the loop

* admits every request that has arrived, rejecting (and counting) those whose
  result alone exceeds the output cap,
* fuses compatible waiting requests into one query -- sample-count statistics
  on the same tree sequence, mode and windows share one sweep (up to 8
  sample sets; 4 when sample counts need 32 bits), and relatedness-vector
  requests on the same tree sequence and windows share one product with
  their weight columns side by side,
* groups up to ``group_size`` such fused queries -- on any of the resident
  tree sequences -- into one batched launch (``QueryBatch``: one kernel per
  pipeline stage for all of them, the replay one persistent kernel over all
  their spans),
* launches a group as soon as a stream slot is free and the device memory
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
from collections import deque
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
    branch-only).  Requests are kept as drawn: the server rejects those
    whose result is too large."""
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
            sets = []
            weights = rng.normal(size=(len(samples), rv_columns))
        out.append(Request(rid, t, key, stat, sets, windows, mode, weights))
    return out


@dataclass
class Batch:
    requests: list            # every request of the launch
    groups: list = None       # its fused queries (lists of requests)
    work: object = None       # the backend's launch record
    slot: int = -1
    nbytes: int = 0
    finished: bool = False


@dataclass
class ServeStats:
    mode: str
    num: int                  # requests served
    wall_s: float
    latencies_s: np.ndarray
    launches: int
    results: dict = field(default_factory=dict)
    rejected: list = field(default_factory=list)  # request ids over the output cap
    fused_queries: int = 0    # fused queries launched (groups hold several)

    @property
    def queries_per_s(self):
        return self.num / self.wall_s if self.wall_s > 0 else float("inf")

    def percentile_ms(self, p):
        return float(np.percentile(self.latencies_s, p) * 1e3) if self.num else 0.0

    def summary(self):
        return {"mode": self.mode, "queries": self.num, "rejected": len(self.rejected),
                "wall_s": round(self.wall_s, 4),
                "queries_per_s": round(self.queries_per_s, 2),
                "p50_ms": round(self.percentile_ms(50), 3),
                "p99_ms": round(self.percentile_ms(99), 3), "launches": self.launches,
                "fused_queries": self.fused_queries}


class _Pending:
    """Waiting requests in arrival order, with a queue per batch key; taken
    requests are dropped lazily from both."""

    def __init__(self):
        self.order = deque()
        self.by_key = {}
        self.taken = set()
        self.count = 0

    def add(self, r):
        self.order.append(r)
        self.by_key.setdefault(r.batch_key(), deque()).append(r)
        self.count += 1

    def take(self, reqs):
        for r in reqs:
            self.taken.add(r.rid)
        self.count -= len(reqs)

    def _trim(self, q):
        while q and q[0].rid in self.taken:
            q.popleft()

    def untaken(self):
        """Waiting requests, oldest first."""
        self._trim(self.order)
        for r in self.order:
            if r.rid not in self.taken:
                yield r

    def key_queue(self, key):
        q = self.by_key.get(key)
        if q is not None:
            self._trim(q)
        return q or ()

    def __bool__(self):
        return self.count > 0


class Server:
    """The request loop over a backend (see GpuBackend for the interface)."""

    def __init__(self, backend, num_slots=8, hbm_budget=64 << 30, max_batch=32,
                 max_output_bytes=256 << 20, group_size=8, scan_limit=128):
        self.backend = backend
        self.num_slots = num_slots
        self.hbm_budget = hbm_budget
        self.max_batch = max_batch
        self.max_output_bytes = max_output_bytes
        self.group_size = group_size
        self.scan_limit = scan_limit

    def _fuse(self, pend, head, chosen):
        """The request `head` and the compatible waiting ones behind it."""
        taken = [head]
        if head.kind == "afs":
            return taken
        sets_cap = self.backend.max_sets(head.ts)
        nsets = len(head.sample_sets)
        nwin = 1 if head.windows is None else len(head.windows) - 1
        cols = 0 if head.weights is None else head.weights.shape[1]
        out_cap = self.max_output_bytes
        for i, r in enumerate(pend.key_queue(head.batch_key())):
            if len(taken) >= self.max_batch or i >= self.scan_limit:
                break
            if r is head or r.rid in chosen or r.rid in pend.taken:
                continue
            if r.windows is not None and not np.array_equal(r.windows, head.windows):
                continue
            if head.kind == "counts":
                if nsets + len(r.sample_sets) > sets_cap:
                    continue
                nsets += len(r.sample_sets)
            else:
                c = cols + r.weights.shape[1]
                if nwin * len(r.weights) * c * 8 > out_cap:
                    continue
                cols = c
            taken.append(r)
        return taken

    def _form_group(self, pend):
        """Up to group_size fused queries, oldest requests first."""
        chosen = set()
        groups = []
        for head in pend.untaken():
            if head.rid in chosen:
                continue
            g = self._fuse(pend, head, chosen)
            chosen.update(r.rid for r in g)
            groups.append(g)
            if len(groups) >= self.group_size:
                break
        return groups

    def run(self, requests, mode="batched", clock=time.perf_counter, idle=None):
        reqs = sorted(requests, key=lambda r: r.arrival)
        n = len(reqs)
        lat = np.full(n, np.nan)
        pos = {r.rid: i for i, r in enumerate(reqs)}
        results = {}
        rejected = []
        pend = _Pending()
        busy = {}  # slot -> Batch
        slot_bytes = [0] * self.num_slots
        nxt = 0
        done = 0
        launches = 0
        fused = 0
        t0 = clock()
        while done + len(rejected) < n:
            now = clock() - t0
            while nxt < n and reqs[nxt].arrival <= now:
                r = reqs[nxt]
                if self.backend.output_bytes(r) > self.max_output_bytes:
                    rejected.append(r.rid)
                else:
                    pend.add(r)
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
            while pend and (mode == "batched" or not busy):
                free = [s for s in range(self.num_slots) if s not in busy]
                if not free:
                    break
                if mode == "batched":
                    groups = self._form_group(pend)
                else:
                    groups = [[next(pend.untaken())]]
                b_bytes = self.backend.workspace_bytes(groups)
                s = free[0]
                others = sum(slot_bytes[o] for o in busy)
                need = max(slot_bytes[s], b_bytes)
                if busy and others + need > self.hbm_budget:
                    self.backend.discard(groups)
                    break  # wait for memory
                flat = [r for g in groups for r in g]
                pend.take(flat)
                slot_bytes[s] = need
                batch = Batch(flat, groups)
                batch.work = self.backend.launch(groups, s)
                batch.slot = s
                busy[s] = batch
                launches += 1
                fused += len(groups)
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
        served = lat[~np.isnan(lat)]
        return ServeStats(mode, done, wall, served, launches, results, rejected, fused)


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

    def output_bytes(self, r):
        """Bytes of one request's result."""
        ts = self.resident[r.ts]
        nwin = 1 if r.windows is None else len(r.windows) - 1
        if r.kind == "rv":
            return nwin * ts.num_samples * r.weights.shape[1] * 8
        if r.kind == "afs":
            return nwin * int(np.prod([len(s) + 1 for s in r.sample_sets])) * 8
        return nwin * 3 * 8

    # ---- preparation (host): one fused query per group
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

    @staticmethod
    def _key(reqs):
        return tuple(r.rid for r in reqs)

    def _get(self, reqs):
        key = self._key(reqs)
        if key not in self._prepared:
            self._prepared[key] = self._prepare(reqs)
        return self._prepared[key]

    def workspace_bytes(self, groups):
        """The launch's workspace: the fused queries' side by side (the
        batch's layout), or the one query's."""
        sizes = [self._get(g)[0].workspace_bytes for g in groups]
        if len(sizes) == 1:
            return sizes[0]
        return sum((b + 255) // 256 * 256 for b in sizes) + 8 * 256

    def discard(self, groups):
        for g in groups:
            self._prepared.pop(self._key(g), None)

    def launch(self, groups, slot):
        from .trees import QueryBatch

        torch = self.torch
        preps = []
        for g in groups:
            key = self._key(g)
            preps.append(self._prepared.pop(key) if key in self._prepared else self._prepare(g))
        st = self.streams[slot]
        ws = self.workspaces[slot]
        with torch.cuda.stream(st):
            res = [torch.empty(q.result_size, dtype=torch.float64, device="cuda")
                   for q, _ in preps]
            weights = []
            for (q, extra), g in zip(preps, groups):
                if g[0].kind == "rv":
                    W = torch.from_numpy(extra).to("cuda", non_blocking=False)
                    q.set_weights(W)
                    weights.append(W)
            batch = None
            if len(preps) == 1:
                q = preps[0][0]
                q.launch(ws, res[0], stream=st)
            else:
                batch = QueryBatch([q for q, _ in preps], res, ws)
                batch.launch(st)
            total = sum(q.result_size for q, _ in preps)
            host = torch.empty(total, dtype=torch.float64, pin_memory=True)
            o = 0
            for (q, _), r in zip(preps, res):
                host[o:o + q.result_size].copy_(r, non_blocking=True)
                o += q.result_size
            ev = torch.cuda.Event()
            ev.record(st)
        return {"preps": preps, "groups": groups, "res": res, "host": host, "ev": ev,
                "W": weights, "slot": slot, "batch": batch}

    def ready(self, work):
        return work["ev"].query()

    def wait(self, work):
        work["ev"].synchronize()

    def results(self, work):
        if work["batch"] is not None:
            work["batch"].check()
        else:
            work["preps"][0][0].check(self.workspaces[work["slot"]])
        y_all = work["host"].numpy()
        out = {}
        o = 0
        for (q, extra), reqs in zip(work["preps"], work["groups"]):
            y = y_all[o:o + q.result_size]
            o += q.result_size
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
                for r, a, b in extra:
                    v = Y[:, a:b]
                    if r.stat == "Fst":
                        du, dv, dx = v[:, 0], v[:, 1], v[:, 2]
                        with np.errstate(divide="ignore", invalid="ignore"):
                            v = (1 - 2 * (du + dv) / (du + dv + 2 * dx))[:, None]
                    out[r.rid] = v
        return out
