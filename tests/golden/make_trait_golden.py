"""Golden values of the trait statistics (trait_covariance,
trait_correlation, trait_linear_model), computed by the reference on the
tree sequences it wrote for the weighted general_stat fixtures.

Run in a container where the reference builds (``make -C oracle ref``), after
tests/golden/make_weighted_golden.py and make_node_golden.py:

    python tests/golden/make_trait_golden.py

Writes ``traits_<name>.npz``: the traits W, covariates Z, windows, and the
reference's results keyed ``<stat>_<mode>_<windowed>`` (``lm`` without
covariates, ``lmz`` with them) plus ``cov_site_unnorm`` (span_normalise off).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from ref_import import import_tskit  # noqa: E402

FILES = {"a": "weighted_a.trees", "b": "weighted_b.trees", "internal": "node_internal.trees"}


def main():
    tskit = import_tskit()
    for name, fname in FILES.items():
        ts = tskit.load(os.path.join(HERE, fname))
        rng = np.random.default_rng(91)
        W = rng.normal(size=(ts.num_samples, 3))
        Z = rng.normal(size=(ts.num_samples, 2))
        windows = np.linspace(0, ts.sequence_length, 4)
        out = {"W": W, "Z": Z, "windows": windows}
        for mode in ("site", "branch", "node"):
            for wn, win in (("w", windows), ("n", None)):
                out[f"cov_{mode}_{wn}"] = ts.trait_covariance(W, windows=win, mode=mode)
                out[f"cor_{mode}_{wn}"] = ts.trait_correlation(W, windows=win, mode=mode)
                out[f"lm_{mode}_{wn}"] = ts.trait_linear_model(W, windows=win, mode=mode)
                out[f"lmz_{mode}_{wn}"] = ts.trait_linear_model(W, Z, windows=win, mode=mode)
        out["cov_site_unnorm"] = ts.trait_covariance(W, windows=windows, mode="site",
                                                     span_normalise=False)
        np.savez(os.path.join(HERE, f"traits_{name}.npz"), **out)
        print(name, ts.num_trees, "trees")


if __name__ == "__main__":
    main()
