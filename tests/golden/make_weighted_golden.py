"""Golden values of general_stat with real-valued weights, computed by the
reference on tree sequences it writes itself.

Run in a container where the reference builds (``make -C oracle ref``):

    python tests/golden/make_weighted_golden.py

Writes ``weighted_<name>.trees`` (the reference's dump) and
``weighted_<name>.npz`` (weights, windows and the reference's
``general_stat`` results for each summary function in
tests/weighted_summaries.py, both modes, polarised and not).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REPO = os.path.dirname(TESTS)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)
sys.path.insert(0, TESTS)
sys.path.insert(0, HERE)

from make_trees_files import from_sim  # noqa: E402
from ref_import import import_tskit  # noqa: E402
from weighted_summaries import SUMMARIES  # noqa: E402


def main():
    tskit = import_tskit()
    for name, (n, L, bps, sites, seed) in {"a": (24, 1e4, 60, 80, 61),
                                           "b": (40, 5e4, 150, 200, 62)}.items():
        tc = from_sim(tskit, n, L, bps, sites, seed)
        tc.sort()
        tc.build_index()
        tc.compute_mutation_parents()
        ts = tc.tree_sequence()
        path = os.path.join(HERE, f"weighted_{name}.trees")
        ts.dump(path)
        ts = tskit.load(path)
        rng = np.random.default_rng(seed)
        out = {}
        W = {K: rng.normal(size=(ts.num_samples, K)) for K in (1, 2, 3)}
        windows = np.linspace(0, ts.sequence_length, 4)
        for fname, (K, M, f) in SUMMARIES.items():
            out[f"W{K}"] = W[K]
            for mode in ("site", "branch"):
                for pol in (False, True):
                    out[f"{fname}_{mode}_{int(pol)}"] = ts.general_stat(
                        W[K], f, M, windows=windows, mode=mode, polarised=pol, strict=False)
        np.savez(os.path.join(HERE, f"weighted_{name}.npz"), windows=windows, **out)
        print(name, ts.num_trees, "trees", ts.num_sites, "sites")


if __name__ == "__main__":
    main()
