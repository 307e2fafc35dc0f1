"""Golden values of genetic_relatedness_weighted, computed by the reference on
the tree sequences it wrote for the weighted general_stat fixtures
(``weighted_<name>.trees``).

Run in a container where the reference builds (``make -C oracle ref``), after
tests/golden/make_weighted_golden.py:

    python tests/golden/make_relatedness_weighted_golden.py

Writes ``relatedness_weighted_<name>.npz``: the weights, the windows and the
reference's results for each case key ``<case>_<mode>_<polarised>_<centre>``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from ref_import import import_tskit  # noqa: E402

# case name -> (weight columns, indexes, windows given, span_normalise)
CASES = {
    "two": (2, None, True, True),
    "pairs": (3, [(0, 1), (1, 2), (2, 2), (0, 0), (2, 0)], True, True),
    "single": (3, [0, 2], True, False),
    "nowin": (4, [(3, 1), (0, 3)], False, True),
}


def main():
    tskit = import_tskit()
    for name, seed in (("a", 71), ("b", 72)):
        ts = tskit.load(os.path.join(HERE, f"weighted_{name}.trees"))
        rng = np.random.default_rng(seed)
        windows = np.linspace(0, ts.sequence_length, 5)
        out = {"windows": windows}
        for case, (K, indexes, with_win, span_norm) in CASES.items():
            W = rng.normal(size=(ts.num_samples, K))
            out[f"W_{case}"] = W
            for mode in ("site", "branch"):
                for pol in (False, True):
                    for centre in (True, False):
                        out[f"{case}_{mode}_{int(pol)}_{int(centre)}"] = (
                            ts.genetic_relatedness_weighted(
                                W, indexes=indexes, windows=windows if with_win else None,
                                mode=mode, span_normalise=span_norm, polarised=pol,
                                centre=centre))
        np.savez(os.path.join(HERE, f"relatedness_weighted_{name}.npz"), **out)
        print(name, ts.num_trees, "trees", ts.num_sites, "sites")


if __name__ == "__main__":
    main()
