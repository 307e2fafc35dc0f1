"""Generate the golden fixtures in this directory from the reference tskit.

Run where the reference is available (it is read from ``TSKIT_REFERENCE``,
else from where ``make -C oracle ref`` built it) after that build:

    python tests/golden/make_golden.py

For every fixture tree sequence this writes ``<name>.npz`` with the tables (as
the reference sorted them) and the reference's outputs for a list of
statistics calls, and ``cases.json`` listing the calls.  The fixtures are the
text tree sequences of the reference's C test library (c/tests/testlib.c:
single_tree_ex, paper_ex, nonbinary_ex, unary_ex, internal_sample_ex,
multiroot_ex, ...) parsed from that file, plus small seeded SMC tree
sequences from tskit_gb300.sim.  The statistics are run through the
reference's own Python API (python/tskit/trees.py) on its C library.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

import ref_import  # noqa: E402

from tskit_gb300 import sim  # noqa: E402
from tskit_gb300.tables import Tables  # noqa: E402

tskit = ref_import.import_tskit()

# sequence lengths the reference's C tests use with each text fixture
TEXT_FIXTURES = {
    "single_tree_ex": 1.0,
    "paper_ex": 10.0,
    "nonbinary_ex": 100.0,
    "unary_ex": 10.0,
    "multiple_tree_ex": 2.0,
    "odd_tree1_ex": 1.0,
    "multi_root_tree_ex": 1.0,
    "multi_path_tree_ex": 1.0,
    "multi_path_tree_ex2": 1.0,
    "internal_sample_ex": 10.0,
    "multiroot_ex": 10.0,
    "empty_ex": 1.0,
    "missing_ex": 5.0,
}


def c_strings(path):
    """name -> concatenated C string literal of `const char *name = ...;`."""
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"const char \*(\w+)\s*=\s*(.*?);", src, flags=re.S):
        lits = re.findall(r'"((?:[^"\\]|\\.)*)"', m.group(2))
        out[m.group(1)] = "".join(lits).encode().decode("unicode_escape")
    return out


def parse_text_fixture(strings, name, L):
    nodes = strings.get(name + "_nodes", "")
    edges = strings.get(name + "_edges", "")
    sites = strings.get(name + "_sites", "")
    muts = strings.get(name + "_mutations", "")
    tc = tskit.TableCollection(sequence_length=L)
    for line in nodes.splitlines():
        tok = line.split()
        if tok:
            tc.nodes.add_row(flags=int(tok[0]), time=float(tok[1]))
    for line in edges.splitlines():
        tok = line.split()
        if tok:
            for c in tok[3].split(","):
                tc.edges.add_row(float(tok[0]), float(tok[1]), int(tok[2]), int(c))
    for line in sites.splitlines():
        tok = line.split()
        if tok:
            tc.sites.add_row(float(tok[0]), tok[1])
    for line in muts.splitlines():
        tok = line.split()
        if tok:
            parent = int(tok[3]) if len(tok) > 3 else -1
            tc.mutations.add_row(int(tok[0]), int(tok[1]), tok[2], parent=parent)
    tc.sort()
    tc.build_index()
    tc.compute_mutation_parents()
    return tc


def to_reference(t: Tables):
    tc = tskit.TableCollection(sequence_length=t.sequence_length)
    tc.nodes.set_columns(flags=t.node_flags, time=t.node_time)
    tc.edges.set_columns(left=t.edge_left, right=t.edge_right, parent=t.edge_parent,
                         child=t.edge_child)
    tc.sites.set_columns(position=t.site_position,
                         ancestral_state=t.site_ancestral_state.view(np.int8),
                         ancestral_state_offset=t.site_ancestral_state_offset)
    tc.mutations.set_columns(site=t.mutation_site, node=t.mutation_node,
                             parent=t.mutation_parent,
                             derived_state=t.mutation_derived_state.view(np.int8),
                             derived_state_offset=t.mutation_derived_state_offset)
    tc.build_index()
    return tc


def from_reference(tc):
    return Tables(
        sequence_length=tc.sequence_length,
        node_time=tc.nodes.time.copy(),
        node_flags=tc.nodes.flags.copy(),
        edge_left=tc.edges.left.copy(),
        edge_right=tc.edges.right.copy(),
        edge_parent=tc.edges.parent.copy(),
        edge_child=tc.edges.child.copy(),
        site_position=tc.sites.position.copy(),
        site_ancestral_state=tc.sites.ancestral_state.view(np.uint8).copy(),
        site_ancestral_state_offset=tc.sites.ancestral_state_offset.astype(np.uint64),
        mutation_site=tc.mutations.site.copy(),
        mutation_node=tc.mutations.node.copy(),
        mutation_parent=tc.mutations.parent.copy(),
        mutation_derived_state=tc.mutations.derived_state.view(np.uint8).copy(),
        mutation_derived_state_offset=tc.mutations.derived_state_offset.astype(np.uint64),
        edge_insertion_order=tc.indexes.edge_insertion_order.copy(),
        edge_removal_order=tc.indexes.edge_removal_order.copy(),
    )


def cases_for(ts, rng):
    """(method, kwargs) calls run on the fixture; all kwargs JSON-able."""
    samples = [int(u) for u in ts.samples()]
    n = len(samples)
    L = ts.sequence_length
    perm = [int(u) for u in rng.permutation(samples)]
    cases = []
    wins = [None, [0.0, L / 3, L]]
    if n >= 2:
        for mode in ("site", "branch"):
            for w in wins:
                cases.append(("diversity", dict(mode=mode, windows=w)))
                cases.append(("segregating_sites", dict(mode=mode, windows=w)))
            cases.append(("diversity", dict(mode=mode, span_normalise=False)))
            cases.append(("diversity", dict(sample_sets=[samples], mode=mode, windows=wins[1])))
            cases.append(("allele_frequency_spectrum", dict(mode=mode)))
            cases.append(("allele_frequency_spectrum", dict(mode=mode, polarised=True,
                                                            windows=wins[1])))
            cases.append(("allele_frequency_spectrum", dict(mode=mode, span_normalise=False)))
        W = rng.normal(size=(n, 2)).round(6).tolist()
        cases.append(("genetic_relatedness_vector", dict(W=W, mode="branch")))
        cases.append(("genetic_relatedness_vector", dict(W=W, mode="branch", windows=wins[1],
                                                         centre=False)))
        cases.append(("genetic_relatedness_matrix", dict(mode="site")))
        cases.append(("genotype_matrix", dict()))
    if n >= 4:
        h = n // 2
        A, B = sorted(perm[:h]), sorted(perm[h:])
        sets2 = [A, B]
        for mode in ("site", "branch"):
            for w in wins:
                cases.append(("diversity", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("divergence", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("divergence", dict(sample_sets=sets2, indexes=[[0, 1], [1, 1],
                                                                             [0, 0]],
                                                  mode=mode, windows=w)))
                cases.append(("Fst", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("Y2", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("f2", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("Y1", dict(sample_sets=sets2, mode=mode, windows=w)))
                cases.append(("genetic_relatedness", dict(sample_sets=sets2, indexes=[[0, 1]],
                                                          mode=mode, windows=w,
                                                          proportion=False)))
                cases.append(("genetic_relatedness", dict(sample_sets=sets2, indexes=[[0, 1]],
                                                          mode=mode, windows=w,
                                                          proportion=False, centre=False)))
            cases.append(("Tajimas_D", dict(sample_sets=sets2, mode=mode)))
            cases.append(("allele_frequency_spectrum", dict(sample_sets=sets2, mode=mode,
                                                            windows=wins[1])))
            cases.append(("allele_frequency_spectrum", dict(sample_sets=sets2, mode=mode,
                                                            polarised=True)))
        cases.append(("allele_frequency_spectrum", dict(sample_sets=sets2, mode="branch",
                                                        time_windows=[0, 0.3, float("inf")])))
    if n >= 6:
        k3 = n // 3
        sets3 = [sorted(perm[:k3]), sorted(perm[k3:2 * k3]), sorted(perm[2 * k3:])]
        for mode in ("site", "branch"):
            cases.append(("Y3", dict(sample_sets=sets3, mode=mode, windows=wins[1])))
            cases.append(("f3", dict(sample_sets=sets3, mode=mode)))
            cases.append(("divergence", dict(sample_sets=sets3, indexes=[[0, 1], [1, 2],
                                                                         [0, 2]], mode=mode)))
    if n >= 8:
        k4 = n // 4
        sets4 = [sorted(perm[j * k4:(j + 1) * k4]) for j in range(4)]
        for mode in ("site", "branch"):
            cases.append(("f4", dict(sample_sets=sets4, mode=mode, windows=wins[1])))
            cases.append(("Y3", dict(sample_sets=sets4, indexes=[[0, 1, 2], [1, 2, 3]],
                                     mode=mode)))
    # size-1 sample set: the reference returns NaN (c/tests/test_stats.c:1734-1739)
    if n >= 1:
        cases.append(("diversity", dict(sample_sets=[[samples[0]]], mode="site")))
        cases.append(("diversity", dict(sample_sets=[[samples[0]]], mode="branch")))
    # node mode (trees.c:1788-1918), on the sets drawn above (no new draws, so
    # the earlier cases keep their inputs)
    if n >= 2:
        for w in wins:
            cases.append(("diversity", dict(mode="node", windows=w)))
            cases.append(("segregating_sites", dict(mode="node", windows=w)))
        cases.append(("diversity", dict(mode="node", span_normalise=False)))
    if n >= 4:
        for w in wins:
            cases.append(("divergence", dict(sample_sets=sets2, mode="node", windows=w)))
            cases.append(("Fst", dict(sample_sets=sets2, mode="node", windows=w)))
            cases.append(("genetic_relatedness", dict(sample_sets=sets2, indexes=[[0, 1], [1, 1]],
                                                      mode="node", windows=w,
                                                      proportion=False)))
        cases.append(("genetic_relatedness", dict(sample_sets=sets2, indexes=[[0, 1]],
                                                  mode="node", proportion=False, centre=False,
                                                  polarised=False)))
        cases.append(("Y2", dict(sample_sets=sets2, mode="node", windows=wins[1])))
        cases.append(("f2", dict(sample_sets=sets2, mode="node")))
        cases.append(("Y1", dict(sample_sets=sets2, mode="node")))
        cases.append(("Tajimas_D", dict(sample_sets=sets2, mode="node")))
    if n >= 6:
        cases.append(("Y3", dict(sample_sets=sets3, mode="node", windows=wins[1])))
        cases.append(("f3", dict(sample_sets=sets3, mode="node")))
    if n >= 8:
        cases.append(("f4", dict(sample_sets=sets4, mode="node", windows=wins[1])))
    if n >= 1:
        cases.append(("diversity", dict(sample_sets=[[samples[0]]], mode="node")))
    # branch-mode divergence and relatedness matrices (trees.c:8578-8672)
    if n >= 2:
        for w in wins:
            cases.append(("divergence_matrix", dict(mode="branch", windows=w)))
        cases.append(("divergence_matrix", dict(mode="branch", span_normalise=False)))
        cases.append(("divergence_matrix", dict(mode="site", windows=wins[1])))
        cases.append(("genetic_relatedness_matrix", dict(mode="branch")))
        cases.append(("genetic_relatedness_matrix", dict(mode="branch", windows=wins[1])))
    return cases


def run_case(ts, method, kw, arrays):
    kw = dict(kw)
    for k, v in kw.items():
        if isinstance(v, str) and v.startswith("@"):
            kw[k] = arrays[v[1:]]
    if method == "genotype_matrix":
        # the decoding the divergence matrix uses (isolated samples not missing)
        return ts.genotype_matrix(isolated_as_missing=False).astype(np.int8)
    if "time_windows" in kw:
        kw["time_windows"] = np.array(kw["time_windows"])
    return np.asarray(getattr(ts, method)(**kw), dtype=np.float64)


def main():
    strings = c_strings(os.path.join(ref_import.reference_root(), "c", "tests", "testlib.c"))
    rng = np.random.default_rng(20241203)
    fixtures = {}
    for name, L in TEXT_FIXTURES.items():
        if name + "_nodes" not in strings:
            continue
        fixtures[name] = parse_text_fixture(strings, name, L)
    for seed in (1, 2, 3):
        t = sim.simulate(12 + 4 * seed, 1e4, 20 * seed, 60, seed)
        fixtures[f"smc_small_{seed}"] = to_reference(t)
    w = sim.WORKLOADS["diversity_n100"]
    fixtures["smc_diversity_n100"] = to_reference(sim.simulate(**w))
    manifest = {}
    for name, tc in fixtures.items():
        ts = tc.tree_sequence()
        cases = cases_for(ts, rng)
        arrays = from_reference(tc).save_npz_dict("tables/")
        kept = []
        for j, (method, kw) in enumerate(cases):
            if name == "smc_diversity_n100" and method in ("genetic_relatedness_matrix",
                                                           "genotype_matrix"):
                continue
            if "W" in kw:
                arrays[f"case{j}_W"] = np.array(kw["W"])
                kw = dict(kw, W=f"@case{j}_W")
            try:
                out = run_case(ts, method, kw, arrays)
            except Exception as e:  # record the reference's error
                kept.append(dict(method=method, kwargs=kw, error=type(e).__name__))
                continue
            arrays[f"case{j}"] = out
            kept.append(dict(method=method, kwargs=kw, key=f"case{j}"))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        manifest[name] = kept
        print(name, ts.num_trees, "trees", ts.num_edges, "edges", len(kept), "cases")
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(manifest, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
