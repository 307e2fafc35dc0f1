"""Tree sequences with parentless stretches, for tests.

Splitting an edge [l, r) into [l, a) and [b, r) leaves its child without a
parent on [a, b): a leaf becomes isolated (missing data), an internal node
becomes an extra root.  The reference's branch allele frequency spectrum
credits such a child, once it regains a parent, from its last update
(c/tskit/trees.c:3639-3800), which these inputs exercise.
"""
import numpy as np

from tskit_gb300.tables import Tables


def with_gaps(tables, seed, frac=0.15):
    rng = np.random.default_rng(seed)
    L, R = tables.edge_left, tables.edge_right
    P, C = tables.edge_parent, tables.edge_child
    left, right, parent, child = [], [], [], []
    for e in range(len(L)):
        l, r = float(L[e]), float(R[e])
        if r - l > 4 and rng.random() < frac:
            a, b = np.sort(rng.uniform(l + 1, r - 1, size=2)).round(3)
            if l < a < b < r:
                left += [l, b]
                right += [a, r]
                parent += [P[e], P[e]]
                child += [C[e], C[e]]
                continue
        left.append(l)
        right.append(r)
        parent.append(P[e])
        child.append(C[e])
    return Tables.from_columns(
        tables.sequence_length, tables.node_time, tables.node_flags, left, right, parent,
        child, site_position=tables.site_position,
        site_ancestral_state=(tables.site_ancestral_state, tables.site_ancestral_state_offset),
        mutation_site=tables.mutation_site, mutation_node=tables.mutation_node,
        mutation_parent=tables.mutation_parent,
        mutation_derived_state=(tables.mutation_derived_state,
                                tables.mutation_derived_state_offset),
    )
