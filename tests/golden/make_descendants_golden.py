"""Golden values of mean_descendants and genealogical_nearest_neighbours,
computed by the reference on the tree sequences it wrote for the weighted
general_stat and node-mode fixtures, with reference sets of samples and of
internal nodes.

Run in a container where the reference builds (``make -C oracle ref``), after
tests/golden/make_weighted_golden.py and make_node_golden.py:

    python tests/golden/make_descendants_golden.py

Writes ``descendants_<name>.npz``: the flattened sets with their sizes and
the reference's mean_descendants result; the focal nodes, disjoint sets and
the reference's genealogical_nearest_neighbours result (``gnn_*``).
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
        rng = np.random.default_rng(97)
        s = ts.samples()
        internal = np.setdiff1d(np.unique(ts.tables.edges.parent), s)
        sets = [list(s[: len(s) // 3]), list(s[len(s) // 3:]),
                sorted(rng.choice(internal, size=5, replace=False).tolist()),
                sorted(rng.choice(np.arange(ts.num_nodes), size=8, replace=False).tolist())]
        out = ts.mean_descendants(sets)
        # disjoint reference sets for the nearest neighbours: samples in
        # three groups and some internal nodes; focal nodes of every kind
        gsets = [list(s[0::3]), list(s[1::3]), list(s[2::3])[:-2],
                 sorted(rng.choice(internal, size=4, replace=False).tolist())]
        focal = np.concatenate([s, rng.choice(internal, size=6, replace=False)]).astype(np.int32)
        gnn = ts.genealogical_nearest_neighbours(focal, gsets)
        np.savez(os.path.join(HERE, f"descendants_{name}.npz"),
                 sizes=np.array([len(x) for x in sets]), flat=np.concatenate(sets).astype(np.int32),
                 result=out, gnn_focal=focal, gnn_sizes=np.array([len(x) for x in gsets]),
                 gnn_flat=np.concatenate(gsets).astype(np.int32), gnn_result=gnn)
        print(name, out.shape)


if __name__ == "__main__":
    main()
