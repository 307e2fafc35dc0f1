"""Drop-in ``TreeSequence`` statistics on the GPU.

The methods keep the signatures, defaults, output shapes and dimension
dropping of the reference's ``tskit.TreeSequence`` statistics
(python/tskit/trees.py:7911-10430); the arithmetic runs in the CUDA kernels
behind the C ABI (include/tskit_gb300.h).  The tables live on the device as
PyTorch tensors; the derived per-tree-sequence state is built there once.

Statistics that the reference computes with several traversals (Fst,
Tajima's D, relatedness as a proportion) are computed here in one fused
sweep whose summary terms are the same functions.
"""
from __future__ import annotations

import ctypes
import math
import numbers

import numpy as np

from . import _native as nat
from .pca import PCAResult  # noqa: F401 (re-exported)
from .tables import Tables


def _require_torch_cuda():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError(
            "tskit_gb300 needs a CUDA device: the statistics have no CPU implementation"
        )
    return torch


def safe_np_int_cast(int_array, dtype, copy=False):
    """Cast to an integer dtype, refusing lossy conversions (same contract as
    python/tskit/util.py:98-132)."""
    if not isinstance(int_array, np.ndarray):
        int_array = np.array(int_array)
        copy = False
    if int_array.size == 0:
        return int_array.astype(dtype, copy=copy)
    try:
        return int_array.astype(dtype, casting="safe", copy=copy)
    except TypeError:
        if int_array.dtype == np.dtype("O"):
            raise TypeError("Cannot convert to a rectangular array.")
        bounds = np.iinfo(dtype)
        if np.any(int_array < bounds.min) or np.any(int_array > bounds.max):
            raise OverflowError(f"Cannot convert safely to {dtype} type")
        if int_array.dtype.kind == "i" and np.dtype(dtype).kind == "u":
            casting = "unsafe"
        else:
            casting = "same_kind"
        return int_array.astype(dtype, casting=casting, copy=copy)


def _parse_mode(mode):
    if mode is None or mode == "site":
        return nat.STAT_SITE
    if mode == "branch":
        return nat.STAT_BRANCH
    if mode == "node":
        return nat.STAT_NODE
    raise ValueError("Unrecognised stats mode")


def _ptr(a):
    """A numpy array's data address for a ``void *`` argument (every native
    function's signature is declared, so the integer is passed as a
    pointer); None for an empty or absent array."""
    return a.ctypes.data if a is not None and a.size > 0 else None


def _outputs(terms):
    """The summary terms as the C ABI's tsg_output_t array (type, four set
    indexes; int32 each), built as one numpy array."""
    rows = []
    for typ, idx in terms:
        ix = [int(i) for i in list(idx)[:4]]
        rows.append([int(typ)] + ix + [0] * (4 - len(ix)))
    return np.array(rows if rows else [(0, 0, 0, 0, 0)], dtype=np.int32).reshape(-1, 5)


class Workspace:
    """Device scratch for query launches (owned by the caller)."""

    def __init__(self, nbytes=0):
        self._lib = nat.load()
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_workspace_create(ctypes.byref(h)))
        self.handle = h
        if nbytes:
            self.reserve(nbytes)

    def reserve(self, nbytes):
        nat.check(self._lib.tsg_workspace_reserve(self.handle, int(nbytes)))

    @property
    def nbytes(self):
        return self._lib.tsg_workspace_bytes(self.handle)

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self._lib.tsg_workspace_free(h)
            self.handle = None


class Query:
    """A prepared fused sample-count query (device resident).

    ``terms`` is a list of (type, (i, j, k, l)) summary terms over the sample
    sets.  ``launch(result, stream)`` enqueues the kernels; ``result`` is a
    float64 CUDA tensor of ``result_size`` elements laid out
    (modes, windows, terms).
    """

    def __init__(self, ts, sample_sets, terms, windows, flags):
        self._lib = nat.load()
        self.ts = ts
        sizes = np.array([len(s) for s in sample_sets], dtype=np.uint64)
        flat = (np.concatenate([np.asarray(s) for s in sample_sets])
                if len(sample_sets) else np.zeros(0))
        flat = safe_np_int_cast(flat, np.int32)
        outs = _outputs(terms)
        win = None if windows is None else np.ascontiguousarray(windows, dtype=np.float64)
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_query_create(
            ctypes.byref(h), ts._handle, len(sizes), _ptr(sizes), _ptr(flat), len(terms),
            _ptr(outs), 0 if win is None else len(win) - 1, _ptr(win), flags,
        ))
        self.handle = h
        self.num_terms = len(terms)
        self.num_windows = 1 if win is None else len(win) - 1
        self.result_size = self._lib.tsg_query_result_size(h)
        self.workspace_bytes = self._lib.tsg_query_workspace_bytes(h)

    def launch(self, workspace, result, stream=None):
        torch = _require_torch_cuda()
        if stream is None:
            stream = torch.cuda.current_stream()
        if workspace.nbytes < self.workspace_bytes:
            workspace.reserve(self.workspace_bytes)
        nat.check(self._lib.tsg_query_launch(
            self.handle, workspace.handle, ctypes.c_void_p(result.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream),
        ))

    def check(self, workspace):
        nat.check(self._lib.tsg_workspace_check(workspace.handle, self.handle))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self._lib.tsg_query_free(h)
            self.handle = None


class AfsQuery(Query):
    """A prepared allele frequency spectrum (device resident); result layout
    (windows, time windows, *(1 + set sizes))."""

    def __init__(self, ts, sample_sets, windows, time_windows, flags):
        self._lib = nat.load()
        self.ts = ts
        sizes = np.array([len(s) for s in sample_sets], dtype=np.uint64)
        flat = safe_np_int_cast(np.concatenate([np.asarray(s) for s in sample_sets]), np.int32)
        win = None if windows is None else np.ascontiguousarray(windows, dtype=np.float64)
        tw = None if time_windows is None else np.ascontiguousarray(time_windows, np.float64)
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_query_create_afs(
            ctypes.byref(h), ts._handle, len(sizes), _ptr(sizes), _ptr(flat),
            0 if win is None else len(win) - 1, _ptr(win), 0 if tw is None else len(tw) - 1,
            _ptr(tw), flags))
        self.handle = h
        self.num_windows = 1 if win is None else len(win) - 1
        self.shape = ((self.num_windows, 1 if tw is None else len(tw) - 1)
                      + tuple(int(n) + 1 for n in sizes))
        self.result_size = self._lib.tsg_query_result_size(h)
        self.workspace_bytes = self._lib.tsg_query_workspace_bytes(h)


class RelatednessVectorQuery(Query):
    """A prepared branch relatedness matrix-vector product (device
    resident); ``set_weights`` binds a float64 CUDA tensor (num_samples x
    columns) read by later launches.  Result layout (windows, focal nodes,
    columns)."""

    def __init__(self, ts, num_weights, windows, nodes, flags):
        self._lib = nat.load()
        self.ts = ts
        win = None if windows is None else np.ascontiguousarray(windows, dtype=np.float64)
        focal = np.ascontiguousarray(ts.samples() if nodes is None else nodes, dtype=np.int32)
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_query_create_relatedness_vector(
            ctypes.byref(h), ts._handle, int(num_weights), 0 if win is None else len(win) - 1,
            _ptr(win), len(focal), _ptr(focal), flags))
        self.handle = h
        self.num_windows = 1 if win is None else len(win) - 1
        self.shape = (self.num_windows, len(focal), int(num_weights))
        self.result_size = self._lib.tsg_query_result_size(h)
        self.workspace_bytes = self._lib.tsg_query_workspace_bytes(h)
        self._weights = None

    def set_weights(self, weights):
        self._weights = weights  # keep the tensor alive while launches read it
        nat.check(self._lib.tsg_query_set_weights(self.handle,
                                                  ctypes.c_void_p(weights.data_ptr())))


class QueryBatch:
    """Prepared queries on any resident tree sequences fused into one launch
    per pipeline stage (``tsg_batch_*``): the sample-count queries on the
    compact replay share each stage's kernel -- the replay one persistent
    kernel over all their spans -- and the others launch on their own in the
    same stream.  ``results`` are float64 CUDA tensors, one per query, of the
    queries' ``result_size``; the batch binds them and ``workspace`` (grown
    here to what the batch needs), and holds references to all three."""

    def __init__(self, queries, results, workspace):
        self._lib = nat.load()
        self.queries = list(queries)
        self.results = list(results)
        self.workspace = workspace
        n = len(self.queries)
        if n == 0 or len(self.results) != n:
            raise ValueError("a batch needs one result per query")
        handles = (ctypes.c_void_p * n)(*[q.handle.value for q in self.queries])
        need = ctypes.c_int64()
        nat.check(self._lib.tsg_batch_workspace_bytes(n, ctypes.cast(handles, ctypes.c_void_p),
                                                      ctypes.byref(need)))
        if workspace.nbytes < need.value:
            workspace.reserve(need.value)
        for q, r in zip(self.queries, self.results):
            if r.numel() < q.result_size:
                raise ValueError("result tensor smaller than its query's result")
        ptrs = (ctypes.c_void_p * n)(*[r.data_ptr() for r in self.results])
        h = ctypes.c_void_p()
        nat.check(self._lib.tsg_batch_create(ctypes.byref(h), n,
                                             ctypes.cast(handles, ctypes.c_void_p),
                                             ctypes.cast(ptrs, ctypes.c_void_p), workspace.handle))
        self.handle = h
        self.workspace_bytes = need.value
        self.num_fused = self._lib.tsg_batch_num_fused(h)

    def launch(self, stream=None):
        torch = _require_torch_cuda()
        if stream is None:
            stream = torch.cuda.current_stream()
        nat.check(self._lib.tsg_batch_launch(self.handle, ctypes.c_void_p(stream.cuda_stream)))

    def check(self):
        failed = ctypes.c_uint64()
        nat.check(self._lib.tsg_batch_check(self.handle, ctypes.byref(failed)))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self._lib.tsg_batch_free(h)
            self.handle = None


class TreeSequence:
    """A tree sequence resident on the GPU with the reference's statistics API."""

    def __init__(self, tables: Tables, num_spans=0):
        torch = _require_torch_cuda()
        self._lib = nat.load()
        tables.check()
        self.tables = tables
        allele, alt, _ = tables.allele_codes()
        dev = torch.device("cuda")

        def up(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            if a.size == 0:
                a = np.zeros(1, dtype=dtype)
            return torch.from_numpy(a).to(dev)

        t = tables
        self._dev = dict(
            node_time=up(t.node_time, np.float64),
            node_flags=up(t.node_flags.astype(np.int32), np.int32),
            edge_left=up(t.edge_left, np.float64),
            edge_right=up(t.edge_right, np.float64),
            edge_parent=up(t.edge_parent, np.int32),
            edge_child=up(t.edge_child, np.int32),
            edge_insertion_order=torch.zeros(max(t.num_edges, 1), dtype=torch.int32, device=dev),
            edge_removal_order=torch.zeros(max(t.num_edges, 1), dtype=torch.int32, device=dev),
            site_position=up(t.site_position, np.float64),
            mutation_site=up(t.mutation_site, np.int32),
            mutation_node=up(t.mutation_node, np.int32),
            mutation_allele=up(allele, np.int32),
            mutation_alt_allele=up(alt, np.int32),
        )
        # the edge indexes, sorted on the device (tables.c:11393-11450)
        d = self._dev
        nat.check(self._lib.tsg_edge_orders(
            t.num_edges, d["edge_left"].data_ptr(), d["edge_right"].data_ptr(),
            d["edge_parent"].data_ptr(), d["edge_child"].data_ptr(), d["node_time"].data_ptr(),
            None, d["edge_insertion_order"].data_ptr(), d["edge_removal_order"].data_ptr(),
            torch.cuda.current_stream().cuda_stream))
        tt = nat.Tables_t()
        tt.sequence_length = t.sequence_length
        tt.num_nodes = t.num_nodes
        tt.num_edges = t.num_edges
        tt.num_sites = t.num_sites
        tt.num_mutations = t.num_mutations
        for k, v in self._dev.items():
            setattr(tt, k, v.data_ptr())
        torch.cuda.synchronize()
        h = ctypes.c_void_p()
        opts = nat.TABLES_ON_DEVICE | (nat.TIME_UNCALIBRATED if t.time_uncalibrated else 0)
        nat.check(self._lib.tsg_treeseq_init(ctypes.byref(h), ctypes.byref(tt), int(num_spans),
                                             opts))
        self._handle = h
        self._samples = t.samples()
        self._breakpoints = None

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            self._lib.tsg_treeseq_free(h)
            self._handle = None

    # ----------------------------------------------------------- properties
    @property
    def sequence_length(self):
        return self.tables.sequence_length

    @property
    def num_samples(self):
        return len(self._samples)

    @property
    def num_nodes(self):
        return self.tables.num_nodes

    @property
    def num_edges(self):
        return self.tables.num_edges

    @property
    def num_sites(self):
        return self.tables.num_sites

    @property
    def num_mutations(self):
        return self.tables.num_mutations

    @property
    def num_trees(self):
        return self._lib.tsg_treeseq_get_num_trees(self._handle)

    @property
    def num_spans(self):
        return self._lib.tsg_treeseq_get_num_spans(self._handle)

    @property
    def num_compact_spans(self):
        """Spans of the compact replay plan (0: the general replay serves the
        sample-count statistics)."""
        return self._lib.tsg_treeseq_get_num_compact_spans(self._handle)

    def plan_sizes(self):
        """Sizes of the replay plans (tsg_treeseq_get_plan_sizes)."""
        out = np.zeros(8, dtype=np.int64)
        nat.check(self._lib.tsg_treeseq_get_plan_sizes(self._handle, _ptr(out)))
        keys = ("num_trees", "num_spans", "num_compact_spans", "compact_nodes",
                "compact_endpoints", "num_items", "num_chunks", "num_anchors")
        return dict(zip(keys, (int(v) for v in out)))

    def set_compact_spans(self, num_spans):
        """Rebuild the compact replay plan with about ``num_spans`` spans (-1:
        the default count; 0: use the general replay); returns the span count
        built.  Results do not depend on it."""
        nat.check(self._lib.tsg_treeseq_set_compact_spans(self._handle, int(num_spans)))
        return self.num_compact_spans

    @property
    def sites_position(self):
        return self.tables.site_position

    def samples(self):
        return self._samples.copy()

    def breakpoints(self, as_array=False):
        if self._breakpoints is None:
            bp = np.zeros(self.num_trees + 1)
            nat.check(self._lib.tsg_treeseq_get_breakpoints(self._handle, _ptr(bp)))
            self._breakpoints = bp
        if as_array:
            return self._breakpoints.copy()
        return iter(self._breakpoints)

    # ------------------------------------------------------- window parsing
    def parse_windows(self, windows):
        """Same rules as python/tskit/trees.py:8108-8131."""
        if windows is None:
            windows = [0.0, self.sequence_length]
        elif isinstance(windows, str):
            if windows == "trees":
                windows = self.breakpoints(as_array=True)
            elif windows == "sites":
                windows = np.concatenate(
                    [[] if self.num_sites > 0 else [0.0], self.sites_position,
                     [self.sequence_length]]
                )
                windows[0] = 0.0
            else:
                raise ValueError(
                    f"Unrecognized window specification {windows}:",
                    "the only allowed strings are 'sites' or 'trees'",
                )
        return np.array(windows)

    def parse_time_windows(self, time_windows):
        """python/tskit/trees.py:8133-8136."""
        if time_windows is None:
            time_windows = [0.0, math.inf]
        return np.array(time_windows)

    # --------------------------------------------------- low-level layer
    def _ll_terms(self, terms, sample_set_sizes, sample_sets, windows, mode, span_normalise,
                  polarised, extra=0):
        """Low-level fused call: returns (num_windows, num_terms) float64 (or
        (2, num_windows, num_terms) with both modes, or (num_windows,
        num_nodes, num_terms) in node mode)."""
        flags = _parse_mode(mode) if not (extra & nat.STAT_BOTH_MODES) else 0
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        flags |= extra
        sizes = np.ascontiguousarray(sample_set_sizes, dtype=np.uint64)
        flat = np.ascontiguousarray(sample_sets, dtype=np.int32)
        if np.sum(sizes) != len(flat):
            raise ValueError("Sum of sample_set_sizes must equal length of sample_sets array")
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        Wn = len(win) - 1
        outs = _outputs(terms)
        nmodes = 2 if extra & nat.STAT_BOTH_MODES else 1
        if flags & nat.STAT_NODE:
            # node mode: one row of outputs per node (trees.c:1788-1918)
            res = np.zeros((nmodes, Wn, self.num_nodes, len(terms)))
        else:
            res = np.zeros((nmodes, Wn, len(terms)))
        nat.check(self._lib.tsg_treeseq_sample_count_stat(
            self._handle, len(sizes), _ptr(sizes), _ptr(flat), len(terms),
            _ptr(outs), Wn, _ptr(win), flags, _ptr(res),
        ))
        return res if nmodes == 2 else res[0]

    def _ll_allele_frequency_spectrum(self, sample_set_sizes, sample_sets, windows,
                                      time_windows, mode=None, span_normalise=True,
                                      polarised=False):
        """Low-level call (python/_tskitmodule.c:6977-7062): result shape
        (num_windows, num_time_windows, *(1 + sample_set_sizes))."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        sizes = np.ascontiguousarray(sample_set_sizes, dtype=np.uint64)
        flat = np.ascontiguousarray(sample_sets, dtype=np.int32)
        if np.sum(sizes) != len(flat):
            raise ValueError("Sum of sample_set_sizes must equal length of sample_sets array")
        win = np.ascontiguousarray(windows, dtype=np.float64)
        tw = np.ascontiguousarray(time_windows, dtype=np.float64)
        for a in (win, tw):
            if a.ndim != 1 or len(a) < 2:
                raise ValueError("Windows arrays must have at least 2 elements")
        shape = (len(win) - 1, len(tw) - 1) + tuple(int(n) + 1 for n in sizes)
        res = np.zeros(shape)
        nat.check(self._lib.tsg_treeseq_allele_frequency_spectrum(
            self._handle, len(sizes), _ptr(sizes), _ptr(flat), len(win) - 1, _ptr(win),
            len(tw) - 1, _ptr(tw), flags, _ptr(res)))
        return res

    def _ll_genetic_relatedness_vector(self, weights, windows, mode=None, span_normalise=True,
                                       centre=True, nodes=None):
        """Low-level call (python/_tskitmodule.c:7196-7282): result shape
        (num_windows, num_focal_nodes, num_weights)."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if not centre:
            flags |= nat.STAT_NONCENTRED
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.ndim != 2:
            raise ValueError("Weights must be a 2D array")
        if w.shape[0] != self.num_samples:
            raise ValueError("First dimension must be num_samples")
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        focal = np.ascontiguousarray(nodes, dtype=np.int32)
        res = np.zeros((len(win) - 1, len(focal), w.shape[1]))
        nat.check(self._lib.tsg_treeseq_genetic_relatedness_vector(
            self._handle, w.shape[1], _ptr(w), len(win) - 1, _ptr(win), len(focal),
            _ptr(focal), _ptr(res), flags))
        return res

    def _ll_genetic_relatedness_weighted(self, weights, indexes, windows, mode=None,
                                         span_normalise=True, polarised=False, centre=True):
        """Low-level call (python/_tskitmodule.c:7292-7370): result shape
        (num_windows, num_index_tuples)."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        if not centre:
            flags |= nat.STAT_NONCENTRED
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.ndim != 2:
            raise ValueError("Weights must be a 2D array")
        if w.shape[0] != self.num_samples:
            raise ValueError("First dimension must be num_samples")
        idx = np.ascontiguousarray(indexes, dtype=np.int32)
        if idx.ndim != 2 or idx.shape[0] < 1 or idx.shape[1] != 2:
            raise ValueError("indexes must be a k x 2 array.")
        if flags & nat.STAT_NODE:
            res = np.zeros((len(win) - 1, self.num_nodes, idx.shape[0]))
        else:
            res = np.zeros((len(win) - 1, idx.shape[0]))
        nat.check(self._lib.tsg_treeseq_genetic_relatedness_weighted(
            self._handle, w.shape[1], _ptr(w), idx.shape[0], _ptr(idx), len(win) - 1,
            _ptr(win), _ptr(res), flags))
        return res

    def _ll_one_way(self, typ):
        def method(sample_set_sizes, sample_sets, windows, mode=None, span_normalise=True,
                   polarised=False):
            K = len(sample_set_sizes)
            return self._ll_terms([(typ, (k,)) for k in range(K)], sample_set_sizes,
                                  sample_sets, windows, mode, span_normalise, polarised)
        return method

    def _ll_k_way(self, typ, k):
        def method(sample_set_sizes, sample_sets, indexes, windows, mode=None,
                   span_normalise=True, polarised=False, centre=True):
            indexes = np.asarray(indexes, dtype=np.int32).reshape(-1, k)
            if len(indexes) < 1:
                raise nat.LibraryError(nat.ERR_INSUFFICIENT_INDEX_TUPLES)
            t = typ
            if typ == nat.RELATEDNESS and not centre:
                t = nat.RELATEDNESS_NONCENTRED
            return self._ll_terms([(t, tuple(ix)) for ix in indexes], sample_set_sizes,
                                  sample_sets, windows, mode, span_normalise, polarised)
        return method

    # ------------------------------------------------ python-level framework
    def __run_windowed_stat(self, windows, method, *args, **kwargs):
        strip_win = windows is None
        windows = self.parse_windows(windows)
        stat = method(*args, **kwargs, windows=windows)
        if strip_win:
            stat = stat[0]
        return stat

    def __run_windowed_stat_tw(self, windows, time_windows, method, *args, **kwargs):
        strip_win = windows is None
        strip_timewin = time_windows is None
        windows = self.parse_windows(windows)
        time_windows = self.parse_time_windows(time_windows)
        stat = method(*args, **kwargs, windows=windows, time_windows=time_windows)
        if strip_win and strip_timewin:
            stat = stat[0, 0, :]
        elif strip_win:
            stat = stat[0, :, :]
        elif strip_timewin:
            stat = stat[:, 0, :]
        return stat

    def __one_way_sample_set_stat(self, ll_method, sample_sets, windows=None, mode=None,
                                  span_normalise=True, polarised=False, time_windows=None,
                                  use_tw=False):
        if sample_sets is None:
            sample_sets = self.samples()
        drop_dimension = False
        try:
            sample_sets = np.array(sample_sets, dtype=np.uint64)
        except ValueError:
            pass
        else:
            if len(sample_sets.shape) == 1:
                sample_sets = [sample_sets]
                drop_dimension = True
        sample_set_sizes = np.array([len(s) for s in sample_sets], dtype=np.uint32)
        if np.any(sample_set_sizes == 0):
            raise ValueError("Sample sets must contain at least one element")
        flattened = safe_np_int_cast(np.hstack(sample_sets), np.int32)
        if use_tw:
            stat = self.__run_windowed_stat_tw(windows, time_windows, ll_method,
                                               sample_set_sizes, flattened, mode=mode,
                                               span_normalise=span_normalise,
                                               polarised=polarised)
        else:
            stat = self.__run_windowed_stat(windows, ll_method, sample_set_sizes, flattened,
                                            mode=mode, span_normalise=span_normalise,
                                            polarised=polarised)
        if drop_dimension:
            stat = stat.reshape(stat.shape[:-1])
            if stat.shape == () and windows is None and time_windows is None:
                stat = stat[()]
        return stat

    def __k_way_sample_set_stat(self, ll_method, k, sample_sets, indexes=None, windows=None,
                                mode=None, span_normalise=True, polarised=False, centre=True):
        sample_set_sizes = np.array([len(s) for s in sample_sets], dtype=np.uint32)
        if np.any(sample_set_sizes == 0):
            raise ValueError("Sample sets must contain at least one element")
        flattened = safe_np_int_cast(np.hstack(sample_sets), np.int32)
        drop_based_on_index = False
        if indexes is None:
            drop_based_on_index = True
            if len(sample_sets) != k:
                raise ValueError(
                    "Must specify indexes if there are not exactly {} sample sets.".format(k)
                )
            indexes = np.arange(k, dtype=np.int32)
        drop_dimension = False
        indexes = safe_np_int_cast(indexes, np.int32)
        if len(indexes.shape) == 1:
            indexes = indexes.reshape((1, indexes.shape[0]))
            drop_dimension = True
        if len(indexes.shape) != 2 or indexes.shape[1] != k:
            raise ValueError(
                "Indexes must be convertable to a 2D numpy array with {} columns".format(k)
            )
        stat = self.__run_windowed_stat(windows, ll_method, sample_set_sizes, flattened,
                                        indexes, mode=mode, span_normalise=span_normalise,
                                        polarised=polarised, centre=centre)
        if drop_dimension:
            stat = stat.reshape(stat.shape[:-1])
            if stat.shape == () and windows is None and drop_based_on_index:
                stat = stat[()]
        return stat

    # ------------------------------------------------------------ one-way
    # ------------------------------------------- arbitrary summary functions
    def _ll_general_stat(self, sample_set_sizes, sample_sets, f, output_dim, windows,
                         mode=None, span_normalise=True, polarised=False):
        """The sweep for 0/1 weights given as sample sets, with the summary
        function evaluated on the host once per distinct count vector."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        sizes = np.ascontiguousarray(sample_set_sizes, dtype=np.uint64)
        flat = np.ascontiguousarray(sample_sets, dtype=np.int32)
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        R = int(output_dim)
        if R < 1:
            raise ValueError("output_dim must be at least 1")
        g = ctypes.c_void_p()
        U = ctypes.c_int64()
        nat.check(self._lib.tsg_general_stat_prepare(
            ctypes.byref(g), self._handle, len(sizes), _ptr(sizes), _ptr(flat), R, len(win) - 1,
            _ptr(win), flags, ctypes.byref(U)))
        try:
            K = len(sizes)
            states = np.zeros((U.value, K), dtype=np.int32)
            nat.check(self._lib.tsg_general_stat_states(g, _ptr(states)))
            total = sizes.astype(np.float64)
            branch = bool(flags & nat.STAT_BRANCH)
            F = np.zeros((U.value, R))
            for i in range(U.value):
                x = states[i].astype(np.float64)
                v = np.asarray(f(x), dtype=np.float64).reshape(-1)
                if v.shape[0] != R:
                    raise ValueError("summary function output has the wrong dimension")
                if branch and not polarised:
                    v = v + np.asarray(f(total - x), dtype=np.float64).reshape(-1)
                F[i] = v
            res = np.zeros((len(win) - 1, R))
            if res.size != self._lib.tsg_general_stat_result_size(g):
                raise RuntimeError("result buffer does not match the statistic's output size")
            nat.check(self._lib.tsg_general_stat_finish(g, _ptr(F), _ptr(res)))
        finally:
            self._lib.tsg_general_stat_free(g)
        return res

    def _ll_general_weighted(self, W, f, output_dim, windows, mode=None, span_normalise=True,
                             polarised=False):
        """The weighted sweep: f evaluated on the host at every state listed
        by tsg_general_weighted_prepare (trees.c:1944-1972 for the
        unpolarised branch sum f(x) + f(total - x))."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        W = np.ascontiguousarray(W, dtype=np.float64)
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        R = int(output_dim)
        if R < 1:
            raise ValueError("output_dim must be at least 1")
        K = W.shape[1]
        g = ctypes.c_void_p()
        U = ctypes.c_int64()
        nat.check(self._lib.tsg_general_weighted_prepare(
            ctypes.byref(g), self._handle, K, _ptr(W), R, len(win) - 1, _ptr(win), flags,
            ctypes.byref(U)))
        try:
            states = np.zeros((U.value, K), dtype=np.float64)
            nat.check(self._lib.tsg_general_weighted_states(g, _ptr(states)))
            total = np.sum(W, axis=0)
            node = bool(flags & nat.STAT_NODE)
            branch = bool(flags & nat.STAT_BRANCH) or node
            F = np.zeros((U.value, R))
            for i in range(U.value):
                v = np.asarray(f(states[i]), dtype=np.float64).reshape(-1)
                if v.shape[0] != R:
                    raise ValueError("summary function output has the wrong dimension")
                if branch and not polarised:
                    v = v + np.asarray(f(total - states[i]), dtype=np.float64).reshape(-1)
                F[i] = v
            if node:
                # node mode: one row of outputs per node (trees.c:1788-1918)
                res = np.zeros((len(win) - 1, self.num_nodes, R))
            else:
                res = np.zeros((len(win) - 1, R))
            if res.size != self._lib.tsg_general_stat_result_size(g):
                raise RuntimeError("result buffer does not match the statistic's output size")
            nat.check(self._lib.tsg_general_stat_finish(g, _ptr(F), _ptr(res)))
        finally:
            self._lib.tsg_general_stat_free(g)
        return res

    def _check_summary(self, total, f, output_dim):
        """python/tskit/trees.py:7983-7993."""
        for x in [total, total * 0.0]:
            with np.errstate(invalid="ignore", divide="ignore"):
                fx = np.array(f(x))
            fx[np.isnan(fx)] = 0.0
            if not np.allclose(fx, np.zeros((output_dim,))):
                raise ValueError("Summary function does not return zero for both "
                                 "zero weight and total weight.")

    def general_stat(self, W, f, output_dim, windows=None, polarised=False, mode=None,
                     span_normalise=True, strict=True):
        """python/tskit/trees.py:7917-8004.  Weights of 0 and 1 (each column a
        set of samples) take the counting sweep, which evaluates f once per
        distinct count vector; other real-valued weights (up to 32 columns),
        and node mode, take the weighted sweep, which evaluates f once per
        state it meets."""
        if mode is None:
            mode = "site"
        W = np.asarray(W, dtype=np.float64)
        if W.ndim != 2 or W.shape[0] != self.num_samples:
            raise ValueError("First dimension of W must be number of samples")
        if strict:
            self._check_summary(np.sum(W, axis=0), f, output_dim)
        if mode == "node" or not np.all((W == 0) | (W == 1)):
            return self.__run_windowed_stat(windows, self._ll_general_weighted, W, f, output_dim,
                                            polarised=polarised, span_normalise=span_normalise,
                                            mode=mode)
        samples = self.samples()
        sets = [samples[W[:, k] == 1] for k in range(W.shape[1])]
        if any(len(s) == 0 for s in sets):
            raise ValueError("Each weight column must select at least one sample")
        sizes = np.array([len(s) for s in sets], dtype=np.uint64)
        flat = safe_np_int_cast(np.hstack(sets), np.int32)
        return self.__run_windowed_stat(windows, self._ll_general_stat, sizes, flat, f,
                                        output_dim, polarised=polarised,
                                        span_normalise=span_normalise, mode=mode)

    def sample_count_stat(self, sample_sets, f, output_dim, windows=None, polarised=False,
                          mode=None, span_normalise=True, strict=True):
        """python/tskit/trees.py:8006-8105: a summary function of the sample
        counts below each node (sample sets as 0/1 weights)."""
        for U in sample_sets:
            if len(U) != len(set(U)):
                raise ValueError(
                    "Elements of sample_sets must be lists without repeated elements.")
            if len(U) == 0:
                raise ValueError("Elements of sample_sets cannot be empty.")
            for u in U:
                if not (0 <= int(u) < self.num_nodes) or not (self.tables.node_flags[u] & 1):
                    raise ValueError("Not all elements of sample_sets are samples.")
        if mode is None:
            mode = "site"
        sizes = np.array([len(s) for s in sample_sets], dtype=np.uint64)
        if strict:
            self._check_summary(sizes.astype(np.float64), f, output_dim)
        flat = safe_np_int_cast(np.hstack(sample_sets), np.int32)
        if mode == "node":
            index = np.full(self.num_nodes, -1, dtype=np.int64)
            index[self.samples()] = np.arange(self.num_samples)
            W = np.zeros((self.num_samples, len(sample_sets)))
            for k, A in enumerate(sample_sets):
                W[index[np.asarray(A, dtype=np.int64)], k] = 1.0
            return self.__run_windowed_stat(windows, self._ll_general_weighted, W, f, output_dim,
                                            polarised=polarised, span_normalise=span_normalise,
                                            mode=mode)
        return self.__run_windowed_stat(windows, self._ll_general_stat, sizes, flat, f,
                                        output_dim, polarised=polarised,
                                        span_normalise=span_normalise, mode=mode)

    # ------------------------------------------------ divergence matrices
    @staticmethod
    def _parse_stat_matrix_sample_sets(ids):
        """python/tskit/trees.py:8708-8737."""
        id_dtype = np.int32
        size_dtype = np.uint64
        if isinstance(ids, (str, bytes, dict, numbers.Number)):
            raise TypeError(f"ID specification cannot be a {type(ids)}")
        if len(ids) == 0:
            return np.array([], dtype=id_dtype), np.array([], dtype=size_dtype)
        if isinstance(ids[0], numbers.Number):
            flat = safe_np_int_cast(ids, id_dtype)
            sizes = np.ones(len(flat), dtype=size_dtype)
        else:
            set_lists, sizes = [], []
            for id_list in ids:
                a = safe_np_int_cast(id_list, id_dtype)
                if len(a.shape) != 1:
                    raise ValueError("ID sets must be 1D integer arrays")
                set_lists.append(a)
                sizes.append(len(a))
            flat = np.hstack(set_lists)
            sizes = np.array(sizes, dtype=size_dtype)
        return flat, sizes

    def _divmat(self, fn, sample_sets, windows, mode, span_normalise):
        windows_specified = windows is not None
        windows = np.ascontiguousarray(self.parse_windows(windows), dtype=np.float64)
        mode = "site" if mode is None else mode
        if sample_sets is None:
            flat = np.ascontiguousarray(self.samples(), dtype=np.int32)
            sizes = np.ones(len(flat), dtype=np.uint64)
        else:
            flat, sizes = self._parse_stat_matrix_sample_sets(sample_sets)
            flat = np.ascontiguousarray(flat, dtype=np.int32)
            sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        K = len(sizes)
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        D = np.zeros((len(windows) - 1, K, K))
        nat.check(fn(self._handle, K, _ptr(sizes), _ptr(flat), len(windows) - 1, _ptr(windows),
                     flags, _ptr(D)))
        if not windows_specified:
            D = D[0]
        return D

    def divergence_matrix(self, sample_sets=None, *, windows=None, num_threads=0, mode=None,
                          span_normalise=True):
        """python/tskit/trees.py:8739-8829: mean divergence between the
        samples of each pair of sets, shape (windows, sets, sets), the window
        dimension dropped when not given; site mode through the exact Gram on
        the tensor cores, branch mode through the relatedness matrix-vector
        sweep.  num_threads is accepted for compatibility (the work runs on
        the GPU)."""
        return self._divmat(self._lib.tsg_treeseq_divergence_matrix, sample_sets, windows, mode,
                            span_normalise)

    def genetic_relatedness_matrix(self, sample_sets=None, *, windows=None, num_threads=0,
                                   mode=None, span_normalise=True):
        """python/tskit/trees.py:8978-9102 (site or branch mode): the
        divergence matrix normalised to centred relatedness, on the GPU."""
        return self._divmat(self._lib.tsg_treeseq_genetic_relatedness_matrix, sample_sets,
                            windows, mode, span_normalise)

    def genetic_relatedness_vector(self, W, windows=None, mode="site", span_normalise=True,
                                   centre=True, nodes=None):
        """python/tskit/trees.py:9157-9218: the genetic relatedness matrix
        times the weight columns W (one row per sample); shape (windows,
        focal nodes, columns), the window dimension dropped when not given.
        Branch mode only, as in the reference's C library."""
        if (not hasattr(W, "__len__")) or (len(W) != self.num_samples):
            raise ValueError("First weight dimension must be equal to number of samples.")
        W = np.asarray(W)
        if len(W.shape) == 1:
            W = W.reshape(W.shape[0], 1)
        if nodes is None:
            nodes = list(self.samples())
        elif centre:
            raise ValueError("If `nodes` is provided, must have centre=False.")
        try:
            nodes = safe_np_int_cast(nodes, np.int32)
        except Exception:
            raise ValueError("Could not interpret `nodes` as a list of node IDs.")
        return self.__run_windowed_stat(windows, self._ll_genetic_relatedness_vector, W,
                                        mode=mode, span_normalise=span_normalise,
                                        centre=centre, nodes=nodes)

    def genealogical_nearest_neighbours(self, focal, sample_sets, num_threads=0):
        """python/tskit/trees.py:10452-10530: for every focal node, the
        reference sets' mean shares of its nearest neighbours (the smallest
        subtree above it holding another reference node) over the trees;
        shape (num_focal, num_sets).  num_threads is accepted for
        compatibility (the work runs on the GPU)."""
        focal = np.ascontiguousarray(safe_np_int_cast(focal, np.int32), dtype=np.int32)
        sizes = np.array([len(s) for s in sample_sets], dtype=np.uint64)
        flat = (safe_np_int_cast(np.hstack([np.asarray(s) for s in sample_sets]), np.int32)
                if len(sample_sets) else np.zeros(0, dtype=np.int32))
        flat = np.ascontiguousarray(flat, dtype=np.int32)
        res = np.zeros((len(focal), len(sample_sets)))
        nat.check(self._lib.tsg_treeseq_genealogical_nearest_neighbours(
            self._handle, _ptr(focal), len(focal), len(sizes), _ptr(sizes), _ptr(flat), 0,
            _ptr(res)))
        return res

    def mean_descendants(self, sample_sets):
        """python/tskit/trees.py:10430-10450: for every node and set, the
        mean number of the set's nodes descending from it, over the parts of
        the genome where it is an ancestor of any node of the sets; shape
        (num_nodes, num_sets)."""
        sizes = np.array([len(s) for s in sample_sets], dtype=np.uint64)
        flat = (safe_np_int_cast(np.hstack([np.asarray(s) for s in sample_sets]), np.int32)
                if len(sample_sets) else np.zeros(0, dtype=np.int32))
        flat = np.ascontiguousarray(flat, dtype=np.int32)
        res = np.zeros((self.num_nodes, len(sample_sets)))
        nat.check(self._lib.tsg_treeseq_mean_descendants(
            self._handle, len(sizes), _ptr(sizes), _ptr(flat), 0, _ptr(res)))
        return res

    # --------------------------------------------------------------- traits
    def _ll_trait(self, fn, weights, windows, covariates=None, mode=None, span_normalise=True):
        """Low-level trait statistic (python/_tskitmodule.c weighted-stat
        methods): result (num_windows, num_weights), or (num_windows,
        num_nodes, num_weights) in node mode."""
        flags = _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.ndim != 2:
            raise ValueError("Weights must be a 2D array")
        if w.shape[0] != self.num_samples:
            raise ValueError("First dimension must be num_samples")
        win = np.ascontiguousarray(windows, dtype=np.float64)
        if win.ndim != 1 or len(win) < 2:
            raise ValueError("Windows arrays must have at least 2 elements")
        if flags & nat.STAT_NODE:
            res = np.zeros((len(win) - 1, self.num_nodes, w.shape[1]))
        else:
            res = np.zeros((len(win) - 1, w.shape[1]))
        if covariates is None:
            nat.check(fn(self._handle, w.shape[1], _ptr(w), len(win) - 1, _ptr(win), flags,
                         _ptr(res)))
        else:
            z = np.ascontiguousarray(covariates, dtype=np.float64)
            if z.ndim != 2 or z.shape[0] != self.num_samples:
                raise ValueError("First dimension of Z must equal the number of samples.")
            nat.check(fn(self._handle, w.shape[1], _ptr(w), z.shape[1], _ptr(z), len(win) - 1,
                         _ptr(win), flags, _ptr(res)))
        return res

    def trait_covariance(self, W, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:9559-9619: mean squared covariance of each
        column of W with inheritance (alleles, branches or nodes)."""
        if W.shape[0] != self.num_samples:
            raise ValueError("First trait dimension must be equal to number of samples.")
        return self.__run_windowed_stat(
            windows, lambda *a, **k: self._ll_trait(self._lib.tsg_treeseq_trait_covariance,
                                                    *a, **k),
            W, mode=mode, span_normalise=span_normalise)

    def trait_correlation(self, W, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:9621-9688: the covariance divided by each
        column's sample variance and p (1 - p), p the inheriting fraction."""
        if W.shape[0] != self.num_samples:
            raise ValueError("First trait dimension must be equal to number of samples.")
        sds = np.std(W, axis=0)
        if np.any(sds == 0):
            raise ValueError(
                "Weight columns must have positive variance", "to compute correlation.")
        return self.__run_windowed_stat(
            windows, lambda *a, **k: self._ll_trait(self._lib.tsg_treeseq_trait_correlation,
                                                    *a, **k),
            W, mode=mode, span_normalise=span_normalise)

    def trait_regression(self, *args, **kwargs):
        """Deprecated synonym for trait_linear_model (python/tskit/trees.py:
        9690-9700)."""
        import warnings

        warnings.warn("This is deprecated: please use trait_linear_model( ) instead.",
                      FutureWarning, stacklevel=4)
        return self.trait_linear_model(*args, **kwargs)

    def trait_linear_model(self, W, Z=None, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:9702-9787: the squared coefficient of
        inheritance in the least-squares fit of each trait on inheritance
        and the covariates Z (with an intercept), the covariates
        orthonormalised as the reference does."""
        if W.shape[0] != self.num_samples:
            raise ValueError("First trait dimension must be equal to number of samples.")
        if Z is None:
            Z = np.ones((self.num_samples, 1))
        else:
            tZ = np.column_stack([Z, np.ones((Z.shape[0], 1))])
            if np.linalg.matrix_rank(tZ) == tZ.shape[1]:
                Z = tZ
        if Z.shape[0] != self.num_samples:
            raise ValueError("First dimension of Z must equal the number of samples.")
        if np.linalg.matrix_rank(Z) < Z.shape[1]:
            raise ValueError("Matrix of covariates is computationally singular.")
        K = np.linalg.cholesky(np.matmul(Z.T, Z)).T
        Z = np.matmul(Z, np.linalg.inv(K))
        return self.__run_windowed_stat(
            windows, lambda W_, Z_, **k: self._ll_trait(
                self._lib.tsg_treeseq_trait_linear_model, W_, covariates=Z_, **k),
            W, Z, mode=mode, span_normalise=span_normalise)

    # ------------------------------------------------------------------ pca
    def _individual_nodes(self, i):
        ni = self.tables.node_individual
        if ni is None or not (0 <= int(i) < self.tables.num_individuals):
            raise ValueError(f"Individual {i} out of bounds")
        return np.flatnonzero(ni == int(i))

    def _decapitated(self, time):
        """This tree sequence's topology younger than ``time`` on the device
        (the branch-statistics part of decapitate)."""
        if not np.isfinite(time):
            raise nat.LibraryError(nat.ERR_TIME_NONFINITE)
        return TreeSequence(self.tables.decapitated_topology(float(time)))

    def pca(self, num_components, windows=None, samples=None, individuals=None,
            time_windows=None, mode="branch", centre=True, num_iterations=5,
            num_oversamples=None, random_seed=None, range_sketch=None):
        """python/tskit/trees.py:9284-9537: principal components of the
        genetic relatedness matrix by randomized SVD (tskit_gb300.pca), every
        product with the matrix one relatedness matrix-vector sweep on the
        GPU."""
        from . import pca as _pca

        return _pca.pca(self, num_components, windows=windows, samples=samples,
                        individuals=individuals, time_windows=time_windows, mode=mode,
                        centre=centre, num_iterations=num_iterations,
                        num_oversamples=num_oversamples, random_seed=random_seed,
                        range_sketch=range_sketch)

    def genetic_relatedness_weighted(self, W, indexes=None, windows=None, mode="site",
                                     span_normalise=True, polarised=False, centre=True):
        """python/tskit/trees.py:9104-9155 with the argument handling of
        __k_way_weighted_stat (trees.py:8414-8457): column k of the result
        is sum_{a,b} W[a,i] W[b,j] C[a,b] for the k-th index pair (i, j), C
        the genetic relatedness between samples; indexes default to (0, 1)
        when W has exactly two columns, and a single pair drops the last
        dimension."""
        if len(W) != self.num_samples:
            raise ValueError("First trait dimension must be equal to number of samples.")
        W = np.asarray(W)
        k = 2
        if indexes is None:
            if W.shape[1] != k:
                raise ValueError(
                    "Must specify indexes if there are not exactly {} columns "
                    "in W.".format(k))
            indexes = np.arange(k, dtype=np.int32)
        drop_dimension = False
        indexes = safe_np_int_cast(indexes, np.int32)
        if len(indexes.shape) == 1:
            indexes = indexes.reshape((1, indexes.shape[0]))
            drop_dimension = True
        if len(indexes.shape) != 2 or indexes.shape[1] != k:
            raise ValueError(
                "Indexes must be convertable to a 2D numpy array with {} columns".format(k))
        stat = self.__run_windowed_stat(windows, self._ll_genetic_relatedness_weighted, W,
                                        indexes, mode=mode, span_normalise=span_normalise,
                                        polarised=polarised, centre=centre)
        if drop_dimension:
            stat = stat.reshape(stat.shape[:-1])
        return stat

    def allele_frequency_spectrum(self, sample_sets=None, windows=None, time_windows=None,
                                  mode="site", span_normalise=True, polarised=False):
        """python/tskit/trees.py:9844-9965: the joint allele frequency spectrum
        of the sample sets, shape (windows, time windows, *(1 + set sizes)),
        window dimensions dropped when not given."""
        if sample_sets is None:
            sample_sets = [self.samples()]
        try:
            sample_sets = np.array(sample_sets, dtype=np.uint64)
        except ValueError:
            pass
        else:
            if len(sample_sets.shape) == 1:
                sample_sets = [sample_sets]
        return self.__one_way_sample_set_stat(
            self._ll_allele_frequency_spectrum, sample_sets, windows=windows,
            time_windows=time_windows, mode=mode, span_normalise=span_normalise,
            polarised=polarised, use_tw=True)

    def diversity(self, sample_sets=None, windows=None, mode="site", span_normalise=True):
        """Mean pairwise diversity (python/tskit/trees.py:8496-8556)."""
        return self.__one_way_sample_set_stat(self._ll_one_way(nat.DIVERSITY), sample_sets,
                                              windows=windows, mode=mode,
                                              span_normalise=span_normalise)

    def segregating_sites(self, sample_sets=None, windows=None, mode="site",
                          span_normalise=True):
        """python/tskit/trees.py:9790-9842"""
        return self.__one_way_sample_set_stat(self._ll_one_way(nat.SEGREGATING_SITES),
                                              sample_sets, windows=windows, mode=mode,
                                              span_normalise=span_normalise)

    def Y1(self, sample_sets, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:10235-10270"""
        return self.__one_way_sample_set_stat(self._ll_one_way(nat.Y1), sample_sets,
                                              windows=windows, mode=mode,
                                              span_normalise=span_normalise)

    # ------------------------------------------------------------- k-way
    def divergence(self, sample_sets, indexes=None, windows=None, mode="site",
                   span_normalise=True):
        """python/tskit/trees.py:8558-8627"""
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.DIVERGENCE, 2), 2, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def Y2(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.Y2, 2), 2, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def f2(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.F2, 2), 2, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def Y3(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:10138-10189"""
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.Y3, 3), 3, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def f3(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.F3, 3), 3, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def f4(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        return self.__k_way_sample_set_stat(self._ll_k_way(nat.F4, 4), 4, sample_sets,
                                            indexes=indexes, windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    def genetic_relatedness(self, sample_sets, indexes=None, windows=None, mode="site",
                            span_normalise=True, polarised=True, proportion=True,
                            centre=True):
        """python/tskit/trees.py:8830-8976.  With proportion=True the
        denominator (segregating sites of the union of the sets) is a fused
        extra term of the same sweep."""
        if not proportion:
            return self.__k_way_sample_set_stat(
                self._ll_k_way(nat.RELATEDNESS, 2), 2, sample_sets, indexes=indexes,
                windows=windows, mode=mode, span_normalise=span_normalise,
                polarised=polarised, centre=centre)
        all_samples = np.array(list({u for s in sample_sets for u in s}))
        K = len(sample_sets)

        def ll(sample_set_sizes, flattened, indexes, windows, mode=None, span_normalise=True,
               polarised=False, centre=True):
            idx = np.asarray(indexes, dtype=np.int32).reshape(-1, 2)
            t = nat.RELATEDNESS if centre else nat.RELATEDNESS_NONCENTRED
            terms = [(t, tuple(ix)) for ix in idx]
            # centred relatedness averages over the K original sets only, so the
            # union set's term runs as a separate (polarised=False) query
            num = self._ll_terms(terms, sample_set_sizes, flattened, windows, mode,
                                 span_normalise, polarised)
            den = self._ll_terms([(nat.SEGREGATING_SITES, (0,))], [len(all_samples)],
                                 safe_np_int_cast(all_samples, np.int32), windows, mode,
                                 span_normalise, False)
            with np.errstate(divide="ignore", invalid="ignore"):
                return num / den
        del K
        return self.__k_way_sample_set_stat(ll, 2, sample_sets, indexes=indexes,
                                            windows=windows, mode=mode,
                                            span_normalise=span_normalise,
                                            polarised=polarised, centre=centre)

    # ------------------------------------------------------ derived stats
    def Tajimas_D(self, sample_sets=None, windows=None, mode="site"):
        """python/tskit/trees.py:9967-10022; diversity and segregating sites
        come from one fused sweep."""

        def tjd_func(sample_set_sizes, flattened, windows, mode=None, span_normalise=True,
                     polarised=False):
            n = np.asarray(sample_set_sizes)
            K = len(n)
            terms = [(nat.DIVERSITY, (k,)) for k in range(K)]
            terms += [(nat.SEGREGATING_SITES, (k,)) for k in range(K)]
            both = self._ll_terms(terms, sample_set_sizes, flattened, windows, mode,
                                  span_normalise, polarised)
            T, S = both[..., :K], both[..., K:]
            h = np.array([np.sum(1 / np.arange(1, nn)) for nn in n])
            g = np.array([np.sum(1 / np.arange(1, nn) ** 2) for nn in n])
            with np.errstate(invalid="ignore", divide="ignore"):
                a = (n + 1) / (3 * (n - 1) * h) - 1 / h**2
                b = 2 * (n**2 + n + 3) / (9 * n * (n - 1)) - (n + 2) / (h * n) + g / h**2
                D = (T - S / h) / np.sqrt(a * S + (b / (h**2 + g)) * S * (S - 1))
            return D

        return self.__one_way_sample_set_stat(tjd_func, sample_sets, windows=windows,
                                              mode=mode, span_normalise=False)

    def Fst(self, sample_sets, indexes=None, windows=None, mode="site", span_normalise=True):
        """python/tskit/trees.py:10024-10136; divergences and diversities come
        from one fused sweep."""

        def fst_func(sample_set_sizes, flattened, indexes, windows, mode, span_normalise,
                     polarised, centre):
            K = len(sample_set_sizes)
            idx = np.asarray(indexes, dtype=np.int32).reshape(-1, 2)
            terms = [(nat.DIVERGENCE, tuple(ix)) for ix in idx]
            terms += [(nat.DIVERSITY, (k,)) for k in range(K)]
            both = self._ll_terms(terms, sample_set_sizes, flattened, windows, mode,
                                  span_normalise, polarised)
            dvg, dvs = both[..., : len(idx)], both[..., len(idx):]
            fst = np.ones_like(dvg)
            for i, (u, v) in enumerate(idx):
                denom = dvs[..., u] + dvs[..., v] + 2 * dvg[..., i]
                with np.errstate(divide="ignore", invalid="ignore"):
                    fst[..., i] -= 2 * (dvs[..., u] + dvs[..., v]) / denom
            return fst

        return self.__k_way_sample_set_stat(fst_func, 2, sample_sets, indexes=indexes,
                                            windows=windows, mode=mode,
                                            span_normalise=span_normalise)

    # ------------------------------------------------------- fused batches
    def query(self, sample_sets, terms, windows=None, mode="branch", span_normalise=True,
              polarised=False, both_modes=False, precision="f64", sweep="auto"):
        """Prepare a device-resident fused query (see :class:`Query`).

        ``sweep`` picks the kernels for testing: ``"global"`` forces the
        general sweep, ``"global_state"`` the item pipeline with its span node
        state in global memory (32-bit counts), where "auto" would choose
        shared memory."""
        flags = 0
        if sweep == "global":
            flags |= nat.FORCE_GLOBAL_SWEEP
        elif sweep == "global_state":
            flags |= nat.FORCE_GLOBAL_STATE
        elif sweep != "auto":
            raise ValueError("sweep must be 'auto', 'global' or 'global_state'")
        if both_modes:
            flags |= nat.STAT_BOTH_MODES
        else:
            flags |= _parse_mode(mode)
        if span_normalise:
            flags |= nat.STAT_SPAN_NORMALISE
        if polarised:
            flags |= nat.STAT_POLARISED
        if precision == "f32":
            flags |= nat.PRECISION_F32_KAHAN
        elif precision != "f64":
            raise ValueError("precision must be 'f64' or 'f32'")
        if isinstance(windows, (str,)) or (windows is not None and not isinstance(
                windows, np.ndarray) and not isinstance(windows, numbers.Number)):
            windows = self.parse_windows(windows)
        return Query(self, sample_sets, terms, windows, flags)


def load(path):
    """tskit.load: the tree sequence stored in a ``.trees`` file, resident on
    the GPU (python/tskit/trees.py load; the statistics' columns only)."""
    return TreeSequence(Tables.load(path))
