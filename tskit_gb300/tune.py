"""Span-count autotuner for the replay kernels.

A tree sequence's span plan (built by ``tsg_treeseq_init`` beside the derived
state of ``tsk_treeseq_init``, c/tskit/trees.c:128-545) cuts the trees into
spans of equal edge-event work; every replay kernel runs one CTA per span.
More spans give more replay warps running at once, but every span also pays
a seek (its first tree rebuilt from the edges alive there) and, for window
outputs and the relatedness vector, work proportional to the number of
samples.  Which count is fastest depends on the tree sequence and on the
statistics asked of it, so it is measured rather than guessed:

* one :class:`~tskit_gb300.trees.TreeSequence` per candidate count (the
  default plan first), sharing the caller's tables;
* the caller's step for that tree sequence timed on the device with CUDA
  events on the current stream, the median of ``steps`` timings after
  ``warmup`` untimed ones;
* the fastest count kept (ties go to the fewer spans), its tree sequence
  returned, the others released.

Tree sequences of up to 65,535 samples also carry a compact replay plan
(short spans holding only the nodes their edge events touch) that the
sample-count statistics use; ``tune_compact_spans`` picks its span count the
same way on one tree sequence, rebuilding only that plan per candidate.

The CTA shape is not tuned: every replay kernel is compiled for one block
size (its launch bounds) and fills the SMs by occupancy.  An optional
``cache`` dict, keyed by the caller's workload key (the statistic family),
the tree sequence's shape and the SM count, skips the measurement for a tree
sequence seen before; ``save_cache`` / ``load_cache`` keep it across
processes as JSON.
"""
import numpy as np


def span_candidates(default_spans, num_trees, num_sms):
    """Counts to try: the default plan's, half and one SM's worth, and two,
    three and four per SM, each at most one span per tree."""
    c = {int(default_spans), max(1, num_sms // 2), num_sms, 2 * num_sms, 3 * num_sms,
         4 * num_sms}
    top = max(1, int(num_trees))
    return sorted({min(x, top) for x in c if x >= 1})


def time_step(step, steps=3, warmup=1):
    """Median device time (ms) of ``step()``, bracketed by CUDA events on the
    current stream, after ``warmup`` untimed calls."""
    import torch

    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        step()
    times = []
    for _ in range(steps):
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        start.record(stream)
        step()
        stop.record(stream)
        stop.synchronize()
        times.append(start.elapsed_time(stop))
    return float(np.median(times))


def _sm_count():
    """SMs of the current CUDA device (0 without one)."""
    try:
        import torch

        if torch.cuda.is_available():
            return int(torch.cuda.get_device_properties(torch.cuda.current_device())
                       .multi_processor_count)
    except Exception:
        pass
    return 0


def _shape_key(ts, key):
    """Cache key: the caller's workload (statistic family) key, the tree
    sequence's shape and the device's SM count."""
    return (f"{key}|edges={ts.num_edges}|trees={ts.num_trees}|samples={ts.num_samples}"
            f"|sms={_sm_count()}")


def load_cache(path):
    """A tuning cache saved by :func:`save_cache` (empty if there is none)."""
    import json
    import os

    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return {str(k): int(v) for k, v in json.load(f).items()}


def save_cache(cache, path):
    """Write a tuning cache (keys: workload, tree-sequence shape and SM
    count; values: span counts) as JSON."""
    import json

    with open(path, "w") as f:
        json.dump(dict(sorted(cache.items())), f, indent=1)


def tune_num_spans(tables, make_step, key="", candidates=None, steps=3, warmup=1, cache=None,
                   build=None, timer=None, num_sms=None):
    """Pick the span count for ``tables`` and the workload ``make_step``.

    ``make_step(ts)`` returns a callable that runs one step of the workload
    on ``ts`` (enqueued on the current stream, or synchronous).  Returns
    ``(ts, report)``: the tree sequence with the chosen plan and
    ``{"num_spans": chosen, "ms": {count: median ms}, "cached": bool}``.
    ``build(num_spans)`` and ``timer(step, steps, warmup)`` replace the
    device tree sequence and the CUDA-event timer (tests use host fakes).
    """
    if build is None:
        from .trees import TreeSequence

        def build(n):
            return TreeSequence(tables, num_spans=n)
    if timer is None:
        timer = time_step
    ts = build(0)
    default = int(ts.num_spans)
    shape = _shape_key(ts, key)
    if cache is not None and shape in cache:
        n = int(cache[shape])
        if n != default:
            ts = build(n)
        return ts, {"num_spans": int(ts.num_spans), "ms": {}, "cached": True}
    if num_sms is None:
        import torch

        num_sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    if candidates is None:
        candidates = span_candidates(default, ts.num_trees, num_sms)
    times = {}
    best, best_ms = None, None
    for n in [default] + [c for c in candidates if c != default]:
        t = ts if n == default else build(n)
        actual = int(t.num_spans)
        if actual in times:
            continue
        times[actual] = timer(make_step(t), steps, warmup)
        if best is None or times[actual] < best_ms or (
                times[actual] == best_ms and actual < int(best.num_spans)):
            best, best_ms = t, times[actual]
        t = None
        ts = None
    if cache is not None:
        cache[shape] = int(best.num_spans)
    return best, {"num_spans": int(best.num_spans), "ms": times, "cached": False}


def compact_candidates(default_spans, num_trees):
    """Compact span counts to try: half to twice the default in quarter
    steps (the fastest is about the most spans whose blocks are all resident
    at once), each at most one span per tree."""
    c = {max(1, int(default_spans * f)) for f in (0.5, 0.75, 1, 1.25, 1.5, 2)}
    return sorted({min(x, max(1, int(num_trees))) for x in c})


def tune_compact_spans(ts, make_step, key="", candidates=None, steps=3, warmup=1, cache=None,
                       timer=None):
    """Pick the compact plan's span count for ``ts`` and the workload
    ``make_step(ts)`` (as :func:`tune_num_spans`); leaves ``ts`` with the
    fastest plan and returns ``{"num_spans": chosen, "ms": {count: ms},
    "cached": bool}`` (``num_spans`` 0 when ``ts`` has no compact plan)."""
    if timer is None:
        timer = time_step
    default = int(ts.num_compact_spans)
    if default == 0:
        return {"num_spans": 0, "ms": {}, "cached": False}
    shape = _shape_key(ts, key) + "|compact"
    if cache is not None and shape in cache:
        n = int(cache[shape])
        if n != default:
            ts.set_compact_spans(n)
        return {"num_spans": int(ts.num_compact_spans), "ms": {}, "cached": True}
    if candidates is None:
        candidates = compact_candidates(default, ts.num_trees)
    times = {}
    # the count asked for that built each plan (the plan's own count can be
    # lower: spans never split a tree)
    asked = {default: None}
    best, best_ms = default, None
    for n in [default] + [c for c in candidates if c != default]:
        actual = int(ts.set_compact_spans(n)) if n != default else default
        if actual in times or actual == 0:
            continue
        asked.setdefault(actual, n)
        times[actual] = timer(make_step(ts), steps, warmup)
        if best_ms is None or times[actual] < best_ms or (
                times[actual] == best_ms and actual < best):
            best, best_ms = actual, times[actual]
    if int(ts.num_compact_spans) != best:
        if asked.get(best) is None:
            ts.set_compact_spans(-1)  # the default plan
        else:
            ts.set_compact_spans(asked[best])
    if cache is not None:
        cache[shape] = int(best)
    return {"num_spans": int(ts.num_compact_spans), "ms": times, "cached": False}
