"""Write the .trees fixtures with the reference's own writer, and the values
the reference computes on them.

Run in a container where the reference builds (``make -C oracle ref``):

    python tests/golden/make_trees_files.py

For each fixture it writes ``<name>.trees`` (``tskit.TreeSequence.dump`` of
the reference) and ``<name>_trees.npz`` with the reference's own table
columns as it loads them back and a few statistics the reference computes
(branch and site diversity and divergence over windows).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, REPO)

from ref_import import import_tskit  # noqa: E402


def from_sim(tskit, n, L, breakpoints, sites, seed, time_units=None):
    from tskit_gb300 import sim

    t = sim.simulate(n, L, breakpoints, sites, seed)
    tc = tskit.TableCollection(sequence_length=t.sequence_length)
    if time_units is not None:
        tc.time_units = time_units
    tc.nodes.set_columns(flags=t.node_flags.astype(np.uint32), time=t.node_time)
    tc.edges.set_columns(left=t.edge_left, right=t.edge_right, parent=t.edge_parent,
                         child=t.edge_child)
    for pos in t.site_position:
        tc.sites.add_row(position=pos, ancestral_state="0")
    for s, u in zip(t.mutation_site, t.mutation_node):
        tc.mutations.add_row(site=int(s), node=int(u), derived_state="1")
    return tc


def multiallelic(tskit, seed):
    """Stacked and nested mutations with several derived states."""
    tc = from_sim(tskit, 30, 1e4, 40, 60, seed)
    rng = np.random.default_rng(seed)
    nodes = tc.nodes.num_rows
    for _ in range(40):
        s = int(rng.integers(tc.sites.num_rows))
        tc.mutations.add_row(site=s, node=int(rng.integers(nodes)),
                             derived_state=["A", "CG", "TTT"][int(rng.integers(3))],
                             time=tskit.UNKNOWN_TIME)
    tc.mutations.set_columns(site=tc.mutations.site, node=tc.mutations.node,
                             derived_state=tc.mutations.derived_state,
                             derived_state_offset=tc.mutations.derived_state_offset,
                             time=np.full(tc.mutations.num_rows, tskit.UNKNOWN_TIME))
    return tc


def main():
    tskit = import_tskit()
    cases = {
        "sim_n40": from_sim(tskit, 40, 1e5, 200, 300, 41),
        "multiallelic_n30": multiallelic(tskit, 43),
        "uncalibrated_n20": from_sim(tskit, 20, 1e4, 30, 50, 47, time_units="uncalibrated"),
    }
    for name, tc in cases.items():
        tc.sort()
        tc.build_index()
        tc.compute_mutation_parents()
        ts = tc.tree_sequence()
        path = os.path.join(HERE, name + ".trees")
        ts.dump(path)
        back = tskit.load(path)
        t = back.tables
        samples = back.samples()
        sets = [samples[: len(samples) // 2], samples[len(samples) // 2:]]
        windows = np.linspace(0, back.sequence_length, 5)
        stats = {}
        for mode in ("site", "branch"):
            if mode == "branch" and back.time_units == "uncalibrated":
                continue
            stats[f"diversity_{mode}"] = back.diversity(sets, windows=windows, mode=mode)
            stats[f"divergence_{mode}"] = back.divergence(sets, windows=windows, mode=mode)
        np.savez(
            os.path.join(HERE, name + "_trees.npz"),
            sequence_length=back.sequence_length,
            time_units=np.frombuffer(back.time_units.encode(), dtype=np.uint8),
            node_time=t.nodes.time, node_flags=t.nodes.flags,
            edge_left=t.edges.left, edge_right=t.edges.right,
            edge_parent=t.edges.parent, edge_child=t.edges.child,
            site_position=t.sites.position,
            site_ancestral_state=t.sites.ancestral_state.view(np.uint8),
            site_ancestral_state_offset=t.sites.ancestral_state_offset.astype(np.uint64),
            mutation_site=t.mutations.site, mutation_node=t.mutations.node,
            mutation_parent=t.mutations.parent,
            mutation_derived_state=t.mutations.derived_state.view(np.uint8),
            mutation_derived_state_offset=t.mutations.derived_state_offset.astype(np.uint64),
            set0=sets[0], set1=sets[1], windows=windows, **stats)
        print(name, os.path.getsize(path), "bytes", back.num_trees, "trees",
              back.num_sites, "sites", back.num_mutations, "mutations")


if __name__ == "__main__":
    main()
