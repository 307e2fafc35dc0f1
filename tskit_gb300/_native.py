"""ctypes binding of the C ABI in ``libtskit_gb300.so`` (include/tskit_gb300.h).

The library is built in place by ``tskit_gb300._build``.  Loading fails loudly
when it is missing: there is no CPU fallback for any statistic.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

STAT_SITE = 1 << 0
STAT_BRANCH = 1 << 1
STAT_NODE = 1 << 2
STAT_POLARISED = 1 << 10
STAT_SPAN_NORMALISE = 1 << 11
STAT_ALLOW_TIME_UNCALIBRATED = 1 << 12
STAT_PAIR_NORMALISE = 1 << 13
STAT_NONCENTRED = 1 << 14
STAT_BOTH_MODES = 1 << 20
PRECISION_F32_KAHAN = 1 << 21
FORCE_GLOBAL_SWEEP = 1 << 22
FORCE_GLOBAL_STATE = 1 << 23
TEST_WAIT_EXPIRES = 1 << 24
TABLES_ON_DEVICE = 1 << 0
TIME_UNCALIBRATED = 1 << 1

(DIVERSITY, SEGREGATING_SITES, Y1, DIVERGENCE, Y2, F2, Y3, F3, F4, RELATEDNESS,
 RELATEDNESS_NONCENTRED) = range(1, 12)

MAX_SAMPLE_SETS = 32
MAX_OUTPUTS = 64

# error codes (same values as the reference where the condition is the same)
ERR_NO_MEMORY = -2
ERR_IO = -3
ERR_FILE_FORMAT = -100
ERR_FILE_VERSION_TOO_OLD = -101
ERR_FILE_VERSION_TOO_NEW = -102
ERR_REQUIRED_COL_NOT_FOUND = -103
ERR_BOTH_COLUMNS_REQUIRED = -104
ERR_BAD_COLUMN_TYPE = -105
ERR_BAD_OFFSET = -200
ERR_BAD_PARAM_VALUE = -4
ERR_NODE_OUT_OF_BOUNDS = -202
ERR_TIME_NONFINITE = -210
ERR_DUPLICATE_SAMPLE = -600
ERR_BAD_SAMPLES = -601
ERR_BAD_NUM_WINDOWS = -900
ERR_BAD_WINDOWS = -901
ERR_MULTIPLE_STAT_MODES = -902
ERR_INSUFFICIENT_SAMPLE_SETS = -905
ERR_INSUFFICIENT_INDEX_TUPLES = -906
ERR_BAD_SAMPLE_SET_INDEX = -907
ERR_EMPTY_SAMPLE_SET = -908
ERR_UNSUPPORTED_STAT_MODE = -909
ERR_TIME_UNCALIBRATED = -910
ERR_INSUFFICIENT_WEIGHTS = -913
ERR_CUDA = -20001
ERR_TOO_MANY_SAMPLE_SETS = -20003
ERR_DEVICE_CHECK = -20002
ERR_NOALLOC_TOO_LARGE = -20007
NOALLOC_SCRATCH_BYTES = 32 << 20


class Tables_t(ctypes.Structure):
    _fields_ = [
        ("sequence_length", ctypes.c_double),
        ("num_nodes", ctypes.c_int64),
        ("num_edges", ctypes.c_int64),
        ("num_sites", ctypes.c_int64),
        ("num_mutations", ctypes.c_int64),
        ("node_time", ctypes.c_void_p),
        ("node_flags", ctypes.c_void_p),
        ("edge_left", ctypes.c_void_p),
        ("edge_right", ctypes.c_void_p),
        ("edge_parent", ctypes.c_void_p),
        ("edge_child", ctypes.c_void_p),
        ("edge_insertion_order", ctypes.c_void_p),
        ("edge_removal_order", ctypes.c_void_p),
        ("site_position", ctypes.c_void_p),
        ("mutation_site", ctypes.c_void_p),
        ("mutation_node", ctypes.c_void_p),
        ("mutation_allele", ctypes.c_void_p),
        ("mutation_alt_allele", ctypes.c_void_p),
    ]


class Output_t(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("idx", ctypes.c_int32 * 4)]


# name -> (restype, argtypes)
_P = ctypes.c_void_p
_U64 = ctypes.c_uint64
_I64 = ctypes.c_int64
_U32 = ctypes.c_uint32
_ONE_WAY = [_P, _U64, _P, _P, _U64, _P, _U32, _P]
_K_WAY = [_P, _U64, _P, _P, _U64, _P, _U64, _P, _U32, _P]
# int f(uint64_t state_dim, const double *state, uint64_t result_dim,
#       double *result, void *params): tsg_general_stat_func_t
GENERAL_STAT_FUNC = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                     ctypes.c_uint64, ctypes.POINTER(ctypes.c_double),
                                     ctypes.c_void_p)

SIGNATURES = {
    "tsg_treeseq_init": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(Tables_t), _I64, _U32]),
    "tsg_treeseq_free": (ctypes.c_int, [_P]),
    "tsg_treeseq_get_num_trees": (_I64, [_P]),
    "tsg_treeseq_get_num_samples": (_I64, [_P]),
    "tsg_treeseq_get_num_spans": (_I64, [_P]),
    "tsg_treeseq_get_num_compact_spans": (_I64, [_P]),
    "tsg_treeseq_get_plan_sizes": (ctypes.c_int, [_P, _P]),
    "tsg_treeseq_set_compact_spans": (ctypes.c_int, [_P, _I64]),
    "tsg_treeseq_get_breakpoints": (ctypes.c_int, [_P, _P]),
    "tsg_strerror": (ctypes.c_char_p, [ctypes.c_int]),
    "tsg_treeseq_diversity": (ctypes.c_int, _ONE_WAY),
    "tsg_treeseq_segregating_sites": (ctypes.c_int, _ONE_WAY),
    "tsg_treeseq_Y1": (ctypes.c_int, _ONE_WAY),
    "tsg_treeseq_divergence": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_Y2": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_f2": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_Y3": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_f3": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_f4": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_genetic_relatedness": (ctypes.c_int, _K_WAY),
    "tsg_treeseq_sample_count_stat": (ctypes.c_int, [_P, _U64, _P, _P, _U64, _P, _U64, _P, _U32, _P]),
    "tsg_query_create": (ctypes.c_int, [ctypes.POINTER(_P), _P, _U64, _P, _P, _U64, _P, _U64, _P, _U32]),
    "tsg_treeseq_allele_frequency_spectrum": (
        ctypes.c_int, [_P, _U64, _P, _P, _U64, _P, _U64, _P, _U32, _P]),
    "tsg_treeseq_genetic_relatedness_vector": (
        ctypes.c_int, [_P, _U64, _P, _U64, _P, _U64, _P, _P, _U32]),
    "tsg_query_create_relatedness_vector": (
        ctypes.c_int, [ctypes.POINTER(_P), _P, _U64, _U64, _P, _U64, _P, _U32]),
    "tsg_query_set_weights": (ctypes.c_int, [_P, _P]),
    "tsg_treeseq_divergence_matrix": (
        ctypes.c_int, [_P, _U64, _P, _P, _U64, _P, _U32, _P]),
    "tsg_treeseq_genetic_relatedness_matrix": (
        ctypes.c_int, [_P, _U64, _P, _P, _U64, _P, _U32, _P]),
    "tsg_gram_e4m3": (ctypes.c_int, [_P, _I64, _I64, _I64, _P, _I64, _P]),
    "tsg_treeseq_genotype_operand": (ctypes.c_int, [_P, _I64, _I64, _P, _I64, _P]),
    "tsg_general_stat_prepare": (
        ctypes.c_int, [ctypes.POINTER(_P), _P, _U64, _P, _P, _U64, _U64, _P, _U32,
                       ctypes.POINTER(_I64)]),
    "tsg_general_stat_states": (ctypes.c_int, [_P, _P]),
    "tsg_general_stat_finish": (ctypes.c_int, [_P, _P, _P]),
    "tsg_general_stat_result_size": (ctypes.c_int64, [_P]),
    "tsg_general_stat_free": (ctypes.c_int, [_P]),
    "tsg_treeseq_general_stat": (
        ctypes.c_int, [_P, _U64, _P, _U64, _P, _P, _U64, _P, _U32, _P]),
    "tsg_general_weighted_prepare": (
        ctypes.c_int, [ctypes.POINTER(_P), _P, _U64, _P, _U64, _U64, _P, _U32,
                       ctypes.POINTER(_I64)]),
    "tsg_general_weighted_states": (ctypes.c_int, [_P, _P]),
    "tsg_treeseq_genealogical_nearest_neighbours": (
        ctypes.c_int, [_P, _P, _U64, _U64, _P, _P, _U32, _P]),
    "tsg_treeseq_mean_descendants": (ctypes.c_int, [_P, _U64, _P, _P, _U32, _P]),
    "tsg_treeseq_trait_covariance": (ctypes.c_int, [_P, _U64, _P, _U64, _P, _U32, _P]),
    "tsg_treeseq_trait_correlation": (ctypes.c_int, [_P, _U64, _P, _U64, _P, _U32, _P]),
    "tsg_treeseq_trait_linear_model": (
        ctypes.c_int, [_P, _U64, _P, _U64, _P, _U64, _P, _U32, _P]),
    "tsg_treeseq_genetic_relatedness_weighted": (
        ctypes.c_int, [_P, _U64, _P, _U64, _P, _U64, _P, _P, _U32]),
    "tsg_query_create_afs": (
        ctypes.c_int, [ctypes.POINTER(_P), _P, _U64, _P, _P, _U64, _P, _U64, _P, _U32]),
    "tsg_query_free": (ctypes.c_int, [_P]),
    "tsg_query_workspace_bytes": (_I64, [_P]),
    "tsg_query_result_size": (_I64, [_P]),
    "tsg_query_launch": (ctypes.c_int, [_P, _P, _P, _P]),
    "tsg_query_set_sweep_events": (ctypes.c_int, [_P, _P, _P]),
    "tsg_query_set_replay_events": (ctypes.c_int, [_P, _P, _P]),
    "tsg_workspace_create": (ctypes.c_int, [ctypes.POINTER(_P)]),
    "tsg_workspace_reserve": (ctypes.c_int, [_P, _I64]),
    "tsg_workspace_bytes": (_I64, [_P]),
    "tsg_workspace_free": (ctypes.c_int, [_P]),
    "tsg_workspace_check": (ctypes.c_int, [_P, _P]),
    "tsg_launch_count": (_I64, []),
    "tsg_query_launch_noalloc": (ctypes.c_int, [_P, _P, _P]),
    "tsg_noalloc_check": (ctypes.c_int, [_P]),
    "tsg_batch_workspace_bytes": (ctypes.c_int, [_U64, _P, ctypes.POINTER(_I64)]),
    "tsg_batch_create": (ctypes.c_int, [ctypes.POINTER(_P), _U64, _P, _P, _P]),
    "tsg_batch_launch": (ctypes.c_int, [_P, _P]),
    "tsg_batch_check": (ctypes.c_int, [_P, ctypes.POINTER(_U64)]),
    "tsg_batch_num_fused": (ctypes.c_int, [_P]),
    "tsg_batch_free": (None, [_P]),
    "tsg_kastore_open": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "tsg_kastore_get": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int32),
                                       ctypes.POINTER(_I64), ctypes.POINTER(_P)]),
    "tsg_kastore_free": (ctypes.c_int, [_P]),
    "tsg_edge_orders": (ctypes.c_int, [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
}

_lib = None


def lib_path():
    return os.path.join(_build.PKG, _build.LIB_NAME)


def load():
    """Load libtskit_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError(
                f"{path} is missing: build it with tskit_gb300._build.build_all() "
                "(there is no CPU implementation of the statistics)"
            )
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class LibraryError(Exception):
    """Raised for a negative return code of the C ABI (the reference raises
    _tskit.LibraryError with tsk_strerror's message for the same codes)."""

    def __init__(self, code):
        self.code = code
        msg = load().tsg_strerror(code).decode()
        super().__init__(msg)


def check(code):
    if code != 0:
        raise LibraryError(code)
