"""Seeded synthetic tree sequences (SMC-style generator, csrc/smc_sim.c).

``simulate(n, L, breakpoints, sites, seed)`` returns :class:`Tables` with
samples 0..n-1, binary coalescent trees, and one biallelic mutation
(ancestral "0", derived "1") per site.  Workload presets name the
configurations used by the benchmarks.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _build
from .tables import Tables


class _SmcResult(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int64),
        ("num_edges", ctypes.c_int64),
        ("num_sites", ctypes.c_int64),
        ("num_samples", ctypes.c_int64),
        ("node_time", ctypes.POINTER(ctypes.c_double)),
        ("edge_left", ctypes.POINTER(ctypes.c_double)),
        ("edge_right", ctypes.POINTER(ctypes.c_double)),
        ("edge_parent", ctypes.POINTER(ctypes.c_int32)),
        ("edge_child", ctypes.POINTER(ctypes.c_int32)),
        ("site_position", ctypes.POINTER(ctypes.c_double)),
        ("mutation_node", ctypes.POINTER(ctypes.c_int32)),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(_build.PKG, _build.SIM_NAME)
        if not os.path.exists(path):
            _build.build_sim()
        lib = ctypes.CDLL(path)
        lib.smc_simulate.argtypes = [
            ctypes.c_int64, ctypes.c_double, ctypes.c_int64, ctypes.c_double,
            ctypes.c_uint64, ctypes.POINTER(_SmcResult),
        ]
        lib.smc_simulate.restype = ctypes.c_int
        lib.smc_free_result.argtypes = [ctypes.POINTER(_SmcResult)]
        _lib = lib
    return _lib


def _copy(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def simulate(n, sequence_length, num_breakpoints, sites, seed):
    """Generate a tree sequence; ``sites`` is the expected number of sites."""
    lib = _load()
    res = _SmcResult()
    err = lib.smc_simulate(int(n), float(sequence_length), int(num_breakpoints),
                           float(sites), int(seed), ctypes.byref(res))
    if err != 0:
        raise RuntimeError(f"smc_simulate failed ({err})")
    try:
        N, E, S = res.num_nodes, res.num_edges, res.num_sites
        node_time = _copy(res.node_time, N, np.float64)
        flags = np.zeros(N, dtype=np.uint32)
        flags[:n] = 1
        site_pos = _copy(res.site_position, S, np.float64)
        t = Tables.from_columns(
            sequence_length,
            node_time,
            flags,
            _copy(res.edge_left, E, np.float64),
            _copy(res.edge_right, E, np.float64),
            _copy(res.edge_parent, E, np.int32),
            _copy(res.edge_child, E, np.int32),
            site_position=site_pos,
            site_ancestral_state=(np.full(S, ord("0"), np.uint8), np.arange(S + 1, dtype=np.uint64)),
            mutation_site=np.arange(S, dtype=np.int32),
            mutation_node=_copy(res.mutation_node, S, np.int32),
            mutation_derived_state=(np.full(S, ord("1"), np.uint8), np.arange(S + 1, dtype=np.uint64)),
        )
    finally:
        lib.smc_free_result(ctypes.byref(res))
    return t


# Workloads: (n, L, breakpoints, expected sites, seed).  Seeds are 1000 + the
# configuration's index; site counts are five per breakpoint.
WORKLOADS = {
    "diversity_n100": dict(n=100, sequence_length=1e6, num_breakpoints=1000, sites=5000, seed=1000),
    "windowed_n10k": dict(n=10_000, sequence_length=1e8, num_breakpoints=100_000, sites=500_000, seed=1001),
    "afs_n200k": dict(n=200_000, sequence_length=1e8, num_breakpoints=1_000_000, sites=5_000_000, seed=1002),
    "grm_n20k": dict(n=20_000, sequence_length=1e8, num_breakpoints=100_000, sites=500_000, seed=1003),
}


def workload(name, **overrides):
    kw = dict(WORKLOADS[name])
    kw.update(overrides)
    return simulate(**kw)
