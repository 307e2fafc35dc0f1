"""Golden values of TreeSequence.pca, computed by the reference on the tree
sequence it wrote for the weighted general_stat fixtures
(``weighted_b.trees``) and on a copy of it with diploid individuals
(``pca_individuals.trees``).

Run in a container where the reference builds (``make -C oracle ref``), after
tests/golden/make_weighted_golden.py:

    python tests/golden/make_pca_golden.py

Writes ``pca.npz``: for each case, the range sketch it starts from
(``<case>_sketch``, drawn as the reference draws it from the seed) and the
reference's factors, eigenvalues, final range sketch and error bound.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from ref_import import import_tskit  # noqa: E402


def with_individuals(tskit, ts):
    """Consecutive pairs of samples as diploid individuals."""
    tables = ts.dump_tables()
    samples = ts.samples()
    individual = np.full(tables.nodes.num_rows, -1, dtype=np.int32)
    for k in range(len(samples) // 2):
        tables.individuals.add_row()
        individual[samples[2 * k]] = k
        individual[samples[2 * k + 1]] = k
    tables.nodes.individual = individual
    return tables.tree_sequence()


def main():
    tskit = import_tskit()
    ts = tskit.load(os.path.join(HERE, "weighted_b.trees"))
    ind = with_individuals(tskit, ts)
    ind.dump(os.path.join(HERE, "pca_individuals.trees"))
    ind = tskit.load(os.path.join(HERE, "pca_individuals.trees"))
    L = ts.sequence_length
    t_mid = float(np.median(ts.tables.nodes.time[ts.tables.nodes.time > 0]))
    t_max = float(np.max(ts.tables.nodes.time)) + 1.0
    samples = ts.samples()
    # case -> (tree sequence, kwargs, windows given, rows, components, oversamples)
    cases = {
        "default": (ts, dict(num_components=3), False, len(samples), 3, 10),
        "windows": (ts, dict(num_components=4, windows=[0, L / 2, L], centre=False), True,
                    len(samples), 4, 10),
        "subset": (ts, dict(num_components=3, samples=samples[:25], num_iterations=3), False,
                   25, 3, 10),
        "individuals": (ind, dict(num_components=2, individuals=np.arange(20)), False, 20, 2,
                        10),
        "time": (ts, dict(num_components=3, time_windows=[0.0, t_mid]), False, len(samples), 3,
                 10),
        "time_high": (ts, dict(num_components=2, time_windows=[t_mid, t_max],
                               windows=[0, L / 3, L]), True, len(samples), 2, 5),
    }
    out = {"t_mid": t_mid}
    for j, (name, (tsx, kw, with_win, dim, k, over)) in enumerate(cases.items()):
        nw = len(kw["windows"]) - 1 if with_win else 1
        sketch = np.random.default_rng(100 + j).normal(size=(nw, dim, k + over))
        if not with_win:
            sketch = sketch[0]
        res = tsx.pca(range_sketch=sketch, **kw)
        out[f"{name}_sketch"] = sketch
        out[f"{name}_factors"] = res.factors
        out[f"{name}_eigenvalues"] = res.eigenvalues
        out[f"{name}_range_sketch"] = res.range_sketch
        out[f"{name}_error_bound"] = np.asarray(res.error_bound)
        print(name, res.eigenvalues.ravel()[:3])
    # the topology decapitate leaves (edges as left, right, child, parent time)
    for label, t in (("mid", t_mid), ("zero", 0.0)):
        d = ts.decapitate(t).tables
        out[f"decap_{label}_edges"] = np.column_stack(
            [d.edges.left, d.edges.right, d.edges.child, d.nodes.time[d.edges.parent]])
        out[f"decap_{label}_num_nodes"] = d.nodes.num_rows
    np.savez(os.path.join(HERE, "pca.npz"), **out)


if __name__ == "__main__":
    main()
