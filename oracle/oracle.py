"""ctypes bindings for the C oracle (tsstat_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
as the checker and by ``bench.py`` for the CPU baseline.  The product never
imports this module.

The functions mirror the reference Python API for the statistics path
(python/tskit/trees.py) closely enough for parity tests: each takes a
``tskit_gb300.tables.Tables`` and returns float64 arrays shaped as the
low-level reference call returns them (always with window and output
dimensions; no dimension dropping).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

STAT_SITE = 1 << 0
STAT_BRANCH = 1 << 1
STAT_NODE = 1 << 2
STAT_POLARISED = 1 << 10
STAT_SPAN_NORMALISE = 1 << 11
STAT_NONCENTRED = 1 << 14

DIVERSITY, SEGSITES, Y1, DIVERGENCE, Y2, F2, Y3, F3, F4, RELATEDNESS, RELATEDNESS_NC = range(1, 12)


class _TS(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("num_edges", ctypes.c_int32),
        ("num_sites", ctypes.c_int32),
        ("num_mutations", ctypes.c_int32),
        ("num_samples", ctypes.c_int32),
        ("sequence_length", ctypes.c_double),
        ("node_time", ctypes.c_void_p),
        ("samples", ctypes.c_void_p),
        ("edge_left", ctypes.c_void_p),
        ("edge_right", ctypes.c_void_p),
        ("edge_parent", ctypes.c_void_p),
        ("edge_child", ctypes.c_void_p),
        ("ins", ctypes.c_void_p),
        ("rem", ctypes.c_void_p),
        ("site_position", ctypes.c_void_p),
        ("mutation_site", ctypes.c_void_p),
        ("mutation_node", ctypes.c_void_p),
        ("mutation_allele", ctypes.c_void_p),
        ("mutation_alt", ctypes.c_void_p),
    ]


class _Output(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("idx", ctypes.c_int32 * 4)]


_lib = None


def build():
    """Compile liboracle.so for this machine (gcc)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
            os.path.join(HERE, "tsstat_oracle.c")
        ):
            build()
        lib = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        lib.orc_sample_count_stat.argtypes = [
            ctypes.POINTER(_TS), ctypes.c_int32, P, P, ctypes.c_int32, P,
            ctypes.c_int32, P, ctypes.c_uint32, P,
        ]
        lib.orc_afs.argtypes = [
            ctypes.POINTER(_TS), ctypes.c_int32, P, P, ctypes.c_int32, P,
            ctypes.c_int32, P, ctypes.c_uint32, P,
        ]
        lib.orc_relatedness_vector.argtypes = [
            ctypes.POINTER(_TS), ctypes.c_int32, P, ctypes.c_int32, P,
            ctypes.c_int32, P, ctypes.c_uint32, P,
        ]
        lib.orc_genotype_matrix.argtypes = [ctypes.POINTER(_TS), P]
        lib.orc_genotype_rows.argtypes = [ctypes.POINTER(_TS), ctypes.c_int32, ctypes.c_int32, P]
        lib.orc_divergence_matrix_site_range.argtypes = [
            ctypes.POINTER(_TS), ctypes.c_int32, ctypes.c_int32, P]
        lib.orc_site_path_sums.argtypes = [ctypes.POINTER(_TS), ctypes.c_int32, P, P]
        lib.orc_branch_count_stat_dd.argtypes = [
            ctypes.POINTER(_TS), ctypes.c_int32, P, P, ctypes.c_int32, P,
            ctypes.c_int32, P, ctypes.c_uint32, P,
        ]
        lib.orc_divergence_matrix_branch.argtypes = [ctypes.POINTER(_TS), ctypes.c_int32, P, P]
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None and a.size else None


class OracleTS:
    """Holds the arrays a C call needs (kept alive for the call's duration)."""

    def __init__(self, tables):
        t = tables
        self.tables = t
        self.samples = t.samples().astype(np.int32)
        allele, alt, _ = t.allele_codes()
        self.arrays = dict(
            node_time=np.ascontiguousarray(t.node_time, np.float64),
            samples=self.samples,
            edge_left=np.ascontiguousarray(t.edge_left, np.float64),
            edge_right=np.ascontiguousarray(t.edge_right, np.float64),
            edge_parent=np.ascontiguousarray(t.edge_parent, np.int32),
            edge_child=np.ascontiguousarray(t.edge_child, np.int32),
            ins=np.ascontiguousarray(t.edge_insertion_order, np.int32),
            rem=np.ascontiguousarray(t.edge_removal_order, np.int32),
            site_position=np.ascontiguousarray(t.site_position, np.float64),
            mutation_site=np.ascontiguousarray(t.mutation_site, np.int32),
            mutation_node=np.ascontiguousarray(t.mutation_node, np.int32),
            mutation_allele=np.ascontiguousarray(allele, np.int32),
            mutation_alt=np.ascontiguousarray(alt, np.int32),
        )
        s = _TS()
        s.num_nodes = t.num_nodes
        s.num_edges = t.num_edges
        s.num_sites = t.num_sites
        s.num_mutations = t.num_mutations
        s.num_samples = len(self.samples)
        s.sequence_length = t.sequence_length
        for k, v in self.arrays.items():
            setattr(s, k, _ptr(v))
        self.struct = s
        self.sample_index = np.full(t.num_nodes, -1, dtype=np.int64)
        self.sample_index[self.samples] = np.arange(len(self.samples))

    @property
    def num_samples(self):
        return len(self.samples)

    @property
    def num_nodes(self):
        return self.tables.num_nodes


def _windows(ts, windows):
    if windows is None:
        return np.array([0.0, ts.tables.sequence_length])
    return np.asarray(windows, dtype=np.float64)


def _mode_flags(mode):
    return {"branch": STAT_BRANCH, "site": STAT_SITE, "node": STAT_NODE, None: STAT_SITE}[mode]


def sample_count_stat(ts, sample_sets, outputs, windows=None, mode="site",
                      span_normalise=True, polarised=False):
    """Run a sample-count statistic.

    ``outputs`` is a list of (type, (i, j, k, l)) summary terms over the K
    sample sets.  Returns float64 (num_windows, len(outputs)).
    """
    lib = _load()
    K = len(sample_sets)
    W = np.zeros((ts.num_samples, K))
    for k, s in enumerate(sample_sets):
        W[ts.sample_index[np.asarray(s, dtype=np.int64)], k] = 1
    n = np.array([len(s) for s in sample_sets], dtype=np.float64)
    outs = (_Output * len(outputs))()
    for r, (typ, idx) in enumerate(outputs):
        outs[r].type = typ
        idx = list(idx) + [0] * (4 - len(idx))
        for q in range(4):
            outs[r].idx[q] = idx[q]
    win = _windows(ts, windows)
    Wn = len(win) - 1
    opts = _mode_flags(mode)
    if opts & STAT_NODE:
        res = np.zeros((Wn, ts.num_nodes, len(outputs)))
    else:
        res = np.zeros((Wn, len(outputs)))
    if span_normalise:
        opts |= STAT_SPAN_NORMALISE
    if polarised:
        opts |= STAT_POLARISED
    err = lib.orc_sample_count_stat(
        ctypes.byref(ts.struct), K, _ptr(W), _ptr(n), len(outputs),
        ctypes.cast(outs, ctypes.c_void_p), Wn, _ptr(win), opts, _ptr(res),
    )
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return res


def branch_count_stat_dd(ts, sample_sets, outputs, windows=None, span_normalise=True,
                         polarised=False):
    """Branch-mode sample-count statistic from the compensated (double-double)
    restatement of the sweep: the reference values to about 1e-16 relative,
    for attributing FP64 disagreements.  Integer summaries only (no centred
    relatedness) and sets below 2^15 samples.  Returns (num_windows,
    len(outputs))."""
    lib = _load()
    K = len(sample_sets)
    member = np.zeros((ts.num_samples, K), dtype=np.uint8)
    for k, s in enumerate(sample_sets):
        member[ts.sample_index[np.asarray(s, dtype=np.int64)], k] = 1
    n = np.array([len(s) for s in sample_sets], dtype=np.int64)
    outs = (_Output * len(outputs))()
    for r, (typ, idx) in enumerate(outputs):
        outs[r].type = typ
        idx = list(idx) + [0] * (4 - len(idx))
        for q in range(4):
            outs[r].idx[q] = idx[q]
    win = _windows(ts, windows)
    res = np.zeros((len(win) - 1, len(outputs)))
    opts = STAT_BRANCH
    if span_normalise:
        opts |= STAT_SPAN_NORMALISE
    if polarised:
        opts |= STAT_POLARISED
    err = lib.orc_branch_count_stat_dd(
        ctypes.byref(ts.struct), K, _ptr(member), _ptr(n), len(outputs),
        ctypes.cast(outs, ctypes.c_void_p), len(win) - 1, _ptr(win), opts, _ptr(res))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return res


def one_way(ts, typ, sample_sets, **kw):
    return sample_count_stat(ts, sample_sets, [(typ, (k,)) for k in range(len(sample_sets))], **kw)


def k_way(ts, typ, sample_sets, indexes, **kw):
    return sample_count_stat(ts, sample_sets, [(typ, tuple(ix)) for ix in indexes], **kw)


def allele_frequency_spectrum(ts, sample_sets, windows=None, time_windows=None,
                              mode="site", span_normalise=True, polarised=False):
    lib = _load()
    K = len(sample_sets)
    sizes = np.array([len(s) for s in sample_sets], dtype=np.int64)
    flat = np.concatenate([np.asarray(s, dtype=np.int32) for s in sample_sets]).astype(np.int32)
    win = _windows(ts, windows)
    tw = np.array([0.0, np.inf]) if time_windows is None else np.asarray(time_windows, np.float64)
    Wn, TW = len(win) - 1, len(tw) - 1
    shape = (Wn, TW) + tuple(int(s) + 1 for s in sizes)
    res = np.zeros(shape)
    opts = _mode_flags(mode)
    if span_normalise:
        opts |= STAT_SPAN_NORMALISE
    if polarised:
        opts |= STAT_POLARISED
    err = lib.orc_afs(ctypes.byref(ts.struct), K, _ptr(sizes), _ptr(flat), Wn, _ptr(win),
                      TW, _ptr(tw), opts, _ptr(res))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return res


def genetic_relatedness_vector(ts, W, windows=None, span_normalise=True, centre=True,
                               nodes=None):
    lib = _load()
    W = np.ascontiguousarray(W, dtype=np.float64)
    if W.ndim == 1:
        W = W[:, None]
    nw = W.shape[1]
    focal = ts.samples if nodes is None else np.asarray(nodes, dtype=np.int32)
    win = _windows(ts, windows)
    Wn = len(win) - 1
    res = np.zeros((Wn, len(focal), nw))
    opts = STAT_BRANCH
    if span_normalise:
        opts |= STAT_SPAN_NORMALISE
    if not centre:
        opts |= STAT_NONCENTRED
    err = lib.orc_relatedness_vector(ctypes.byref(ts.struct), nw, _ptr(W), Wn, _ptr(win),
                                     len(focal), _ptr(focal), opts, _ptr(res))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return res


def genotype_matrix(ts):
    """int8 (num_sites, num_samples) allele indexes."""
    lib = _load()
    G = np.zeros((ts.tables.num_sites, ts.num_samples), dtype=np.int8)
    err = lib.orc_genotype_matrix(ctypes.byref(ts.struct), _ptr(G))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return G


def genotype_rows(ts, site_start, site_stop):
    """int8 (site_stop - site_start, num_samples) allele indexes."""
    lib = _load()
    G = np.zeros((site_stop - site_start, ts.num_samples), dtype=np.int8)
    err = lib.orc_genotype_rows(ctypes.byref(ts.struct), site_start, site_stop, _ptr(G))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return G


def divergence_counts_site_range(ts, site_start, site_stop, symmetric=True):
    """Unnormalised site divergence counts over sites [site_start, site_stop)
    with every sample its own set, by the reference's pairwise loop
    (trees.c:8685-8716); float64 num_samples x num_samples, symmetric (else
    the upper triangle the loop fills)."""
    lib = _load()
    n = ts.num_samples
    D = np.zeros((n, n))
    err = lib.orc_divergence_matrix_site_range(ctypes.byref(ts.struct), site_start, site_stop,
                                               _ptr(D))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return D + D.T if symmetric else D


def site_path_sums(ts, sample_sets):
    """int64 (num_samples, 1 + K): per sample index j, the number of
    mutations above j and, per set k, the sum over those mutations of the
    set-k samples below the mutation (orc_site_path_sums)."""
    lib = _load()
    member = np.zeros((ts.num_samples, len(sample_sets)), dtype=np.uint8)
    index = np.full(ts.tables.num_nodes, -1, dtype=np.int64)
    index[ts.samples] = np.arange(ts.num_samples)
    for k, s in enumerate(sample_sets):
        member[index[np.asarray(s, dtype=np.int64)], k] = 1
    out = np.zeros((ts.num_samples, 1 + len(sample_sets)), dtype=np.int64)
    err = lib.orc_site_path_sums(ctypes.byref(ts.struct), len(sample_sets), _ptr(member),
                                 _ptr(out))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    return out


def _infinite_sites_biallelic(ts):
    t = ts.tables
    site = np.asarray(t.mutation_site)
    allele = ts.arrays["mutation_allele"]
    return (len(site) == t.num_sites and np.array_equal(site, np.arange(t.num_sites))
            and np.all(allele == 1))


def relatedness_rows_site(ts, rows):
    """Rows ``rows`` (sample indexes) of the site-mode
    genetic_relatedness_matrix with every sample its own set, one window,
    span-normalised, for infinite-sites biallelic data, exactly: with a_j
    the derived count of sample j and G[i][j] the shared derived count, the
    per-pair differing-site count is a_i + a_j - 2 G[i][j]; the divergence
    row sums are R_j = n a_j + sum(a) - 2 sum_s g_js c_s; and the
    normalisation of trees.py:9086-9095 gives
    K[i][j] = -(n^2 d_ij + sum(R) - n R_i - n R_j) / (2 n^2 L),
    its numerator an exact integer, rounded once.  Returns (K rows float64,
    shared-derived rows G[rows] int64)."""
    if not _infinite_sites_biallelic(ts):
        raise ValueError("relatedness_rows_site needs one biallelic mutation per site")
    rows = np.asarray(rows, dtype=np.int64)
    samples = ts.samples
    sums = site_path_sums(ts, [samples] + [[samples[i]] for i in rows])
    a, b, G = sums[:, 0], sums[:, 1], sums[:, 2:].T
    n = np.int64(ts.num_samples)
    R = n * a + a.sum() - 2 * b
    d = a[rows][:, None] + a[None, :] - 2 * G
    num = n * n * d + R.sum() - n * R[rows][:, None] - n * R[None, :]
    K = -num.astype(np.float64) / (2.0 * float(n) ** 2 * ts.tables.sequence_length)
    return K, G


def divergence_matrix_site(ts, windows=None, span_normalise=True):
    """Site-mode divergence matrix with every sample its own set
    (trees.c:8753-8899), computed from the decoded genotype matrix."""
    G = genotype_matrix(ts)
    win = _windows(ts, windows)
    pos = ts.tables.site_position
    n = ts.num_samples
    out = np.zeros((len(win) - 1, n, n))
    for w in range(len(win) - 1):
        sel = (pos >= win[w]) & (pos < win[w + 1])
        Gw = G[sel].astype(np.int64)
        # pairs carrying different alleles = sites - pairs carrying the same
        same = np.zeros((n, n), dtype=np.int64)
        for a in np.unique(Gw):
            Xa = (Gw == a).astype(np.int64)
            same += Xa.T @ Xa
        D = (Gw.shape[0] - same).astype(np.float64)
        np.fill_diagonal(D, 0.0)
        if span_normalise:
            D /= win[w + 1] - win[w]
        out[w] = D
    return out


def divergence_matrix_branch(ts, windows=None, span_normalise=True):
    """Branch-mode divergence matrix with every sample its own set
    (trees.c:8578-8672)."""
    lib = _load()
    win = _windows(ts, windows)
    n = ts.num_samples
    out = np.zeros((len(win) - 1, n, n))
    err = lib.orc_divergence_matrix_branch(ctypes.byref(ts.struct), len(win) - 1, _ptr(win),
                                           _ptr(out))
    if err != 0:
        raise RuntimeError(f"oracle error {err}")
    if span_normalise:
        out /= np.diff(win)[:, None, None]
    return out


def relatedness_from_divergence(D):
    """genetic_relatedness_matrix's normalisation (python/tskit/trees.py:9086-9095)
    for singleton sample sets."""
    n = np.ones(D.shape[-1])
    B = D.copy()
    np.fill_diagonal(B, np.diag(B) * (n - 1) / n)
    K = B + np.mean(B)
    y = np.mean(B, axis=0)
    K -= y[:, None] + y[None, :]
    return K / -2


# ------------------------------------------------------------------------
# Adapter from the reference's high-level method names to the oracle.  The
# outputs keep the low-level shapes; callers reshape to the expected shape
# (the reference only drops length-1 dimensions).
# ------------------------------------------------------------------------
_ONE_WAY = {"diversity": DIVERSITY, "segregating_sites": SEGSITES, "Y1": Y1}
_K_WAY = {"divergence": (DIVERGENCE, 2), "Y2": (Y2, 2), "f2": (F2, 2), "Y3": (Y3, 3),
          "f3": (F3, 3), "f4": (F4, 4)}


def _sets(ots, sample_sets):
    if sample_sets is None:
        return [ots.samples]
    a = sample_sets
    try:
        arr = np.array(a, dtype=np.int64)
        if arr.ndim == 1:
            return [arr]
    except ValueError:
        pass
    return [np.asarray(s, dtype=np.int64) for s in a]


def _tuples(indexes, k, nsets):
    if indexes is None:
        return [tuple(range(k))]
    idx = np.asarray(indexes, dtype=np.int64).reshape(-1, k)
    return [tuple(int(v) for v in row) for row in idx]


def call(ots, method, kwargs):
    """Evaluate one reference API call with the oracle."""
    kw = dict(kwargs)
    mode = kw.pop("mode", "site")
    windows = kw.pop("windows", None)
    if isinstance(windows, str):
        raise ValueError("string windows are resolved by the caller")
    span_normalise = kw.pop("span_normalise", True)
    if method in _ONE_WAY:
        sets = _sets(ots, kw.pop("sample_sets", None))
        return one_way(ots, _ONE_WAY[method], sets, windows=windows, mode=mode,
                       span_normalise=span_normalise)
    if method in _K_WAY:
        typ, k = _K_WAY[method]
        sets = _sets(ots, kw.pop("sample_sets"))
        return k_way(ots, typ, sets, _tuples(kw.pop("indexes", None), k, len(sets)),
                     windows=windows, mode=mode, span_normalise=span_normalise)
    if method == "genetic_relatedness":
        sets = _sets(ots, kw.pop("sample_sets"))
        typ = RELATEDNESS if kw.pop("centre", True) else RELATEDNESS_NC
        polarised = kw.pop("polarised", True)
        num = k_way(ots, typ, sets, _tuples(kw.pop("indexes", None), 2, len(sets)),
                    windows=windows, mode=mode, span_normalise=span_normalise,
                    polarised=polarised)
        if kw.pop("proportion", True):
            union = np.array(sorted({int(u) for s in sets for u in s}))
            den = one_way(ots, SEGSITES, [union], windows=windows, mode=mode,
                          span_normalise=span_normalise)
            with np.errstate(divide="ignore", invalid="ignore"):
                num = num / den
        return num
    if method == "Fst":
        sets = _sets(ots, kw.pop("sample_sets"))
        tuples = _tuples(kw.pop("indexes", None), 2, len(sets))
        dvg = k_way(ots, DIVERGENCE, sets, tuples, windows=windows, mode=mode,
                    span_normalise=span_normalise)
        dvs = one_way(ots, DIVERSITY, sets, windows=windows, mode=mode,
                      span_normalise=span_normalise)
        out = np.ones_like(dvg)
        for i, (u, v) in enumerate(tuples):
            with np.errstate(divide="ignore", invalid="ignore"):
                out[..., i] -= 2 * (dvs[..., u] + dvs[..., v]) / (
                    dvs[..., u] + dvs[..., v] + 2 * dvg[..., i])
        return out
    if method == "Tajimas_D":
        sets = _sets(ots, kw.pop("sample_sets", None))
        T = one_way(ots, DIVERSITY, sets, windows=windows, mode=mode, span_normalise=False)
        S = one_way(ots, SEGSITES, sets, windows=windows, mode=mode, span_normalise=False)
        n = np.array([len(s) for s in sets], dtype=np.float64)
        h = np.array([np.sum(1 / np.arange(1, nn)) for nn in n])
        g = np.array([np.sum(1 / np.arange(1, nn) ** 2) for nn in n])
        with np.errstate(invalid="ignore", divide="ignore"):
            a = (n + 1) / (3 * (n - 1) * h) - 1 / h**2
            b = 2 * (n**2 + n + 3) / (9 * n * (n - 1)) - (n + 2) / (h * n) + g / h**2
            return (T - S / h) / np.sqrt(a * S + (b / (h**2 + g)) * S * (S - 1))
    if method == "allele_frequency_spectrum":
        sets = kw.pop("sample_sets", None)
        if sets is None:
            sets = [ots.samples]
        else:
            try:
                arr = np.array(sets, dtype=np.int64)
                sets = [arr] if arr.ndim == 1 else list(arr)
            except ValueError:
                pass
        return allele_frequency_spectrum(ots, [np.asarray(s) for s in sets], windows=windows,
                                         time_windows=kw.pop("time_windows", None), mode=mode,
                                         span_normalise=span_normalise,
                                         polarised=kw.pop("polarised", False))
    if method == "genetic_relatedness_vector":
        return genetic_relatedness_vector(ots, kw.pop("W"), windows=windows,
                                          span_normalise=span_normalise,
                                          centre=kw.pop("centre", True),
                                          nodes=kw.pop("nodes", None))
    if method in ("divergence_matrix", "genetic_relatedness_matrix"):
        if mode == "branch":
            D = divergence_matrix_branch(ots, windows=windows, span_normalise=span_normalise)
        else:
            D = divergence_matrix_site(ots, windows=windows, span_normalise=span_normalise)
        if method == "divergence_matrix":
            return D
        return np.stack([relatedness_from_divergence(d) for d in D])
    if method == "genotype_matrix":
        return genotype_matrix(ots)
    raise NotImplementedError(method)
