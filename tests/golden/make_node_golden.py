"""Golden values of node-mode statistics with real-valued weights and user
summary functions, computed by the reference on the tree sequences it wrote
for the weighted general_stat fixtures (``weighted_<name>.trees``), and on a
copy of ``weighted_a`` with internal sample nodes (``node_internal.trees``).

Run in a container where the reference builds (``make -C oracle ref``), after
tests/golden/make_weighted_golden.py:

    python tests/golden/make_node_golden.py

Writes ``node_<name>.npz`` with, per key:
  * ``general_<summary>_<polarised>``: general_stat(W, f, mode="node") for
    each summary in tests/weighted_summaries.py (windows of the fixture);
  * ``count_<summary>_<polarised>``: sample_count_stat(..., mode="node");
  * ``grw_<centre>_<polarised>``: genetic_relatedness_weighted(mode="node")
    without windows.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REPO = os.path.dirname(TESTS)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, TESTS)

from ref_import import import_tskit  # noqa: E402
from weighted_summaries import COUNT_SUMMARIES, SUMMARIES  # noqa: E402


def internal_samples(tskit, ts, seed):
    """The same tree sequence with a few internal nodes marked as samples."""
    tables = ts.dump_tables()
    rng = np.random.default_rng(seed)
    parents = np.unique(tables.edges.parent)
    flags = tables.nodes.flags.copy()
    flags[rng.choice(parents, size=4, replace=False)] |= tskit.NODE_IS_SAMPLE
    tables.nodes.flags = flags
    return tables.tree_sequence()


def main():
    tskit = import_tskit()
    a = tskit.load(os.path.join(HERE, "weighted_a.trees"))
    b = tskit.load(os.path.join(HERE, "weighted_b.trees"))
    internal = internal_samples(tskit, a, 83)
    internal.dump(os.path.join(HERE, "node_internal.trees"))
    internal = tskit.load(os.path.join(HERE, "node_internal.trees"))
    for name, ts, seed in (("a", a, 81), ("b", b, 82), ("internal", internal, 84)):
        rng = np.random.default_rng(seed)
        windows = np.linspace(0, ts.sequence_length, 4)
        out = {"windows": windows}
        samples = ts.samples()
        for K in (1, 2, 3):
            out[f"W{K}"] = rng.normal(size=(ts.num_samples, K))
        for fname, (K, M, f) in SUMMARIES.items():
            for pol in (False, True):
                out[f"general_{fname}_{int(pol)}"] = ts.general_stat(
                    out[f"W{K}"], f, M, windows=windows, mode="node", polarised=pol,
                    strict=False)
        for fname, (sizes, M, f) in COUNT_SUMMARIES.items():
            sets, at = [], 0
            for s in sizes:
                sets.append(samples[at:at + s])
                at += s
            for pol in (False, True):
                out[f"count_{fname}_{int(pol)}"] = ts.sample_count_stat(
                    sets, f, M, windows=windows, mode="node", polarised=pol, strict=False)
        Wr = rng.normal(size=(ts.num_samples, 3))
        out["Wr"] = Wr
        for centre in (True, False):
            for pol in (False, True):
                out[f"grw_{int(centre)}_{int(pol)}"] = ts.genetic_relatedness_weighted(
                    Wr, indexes=[(0, 1), (2, 2)], mode="node", polarised=pol, centre=centre)
        np.savez(os.path.join(HERE, f"node_{name}.npz"), **out)
        print(name, ts.num_trees, "trees", ts.num_nodes, "nodes", ts.num_samples, "samples")


if __name__ == "__main__":
    main()
