"""GB300-native tree-sequence statistics.

A drop-in for the statistics methods of ``tskit.TreeSequence`` (diversity,
divergence, Fst, Tajima's D, Y-statistics, f-statistics, genetic relatedness,
allele frequency spectra, relatedness matrix-vector products) computed by
sm_103a CUDA kernels behind a C ABI (include/tskit_gb300.h).
"""
from ._native import LibraryError  # noqa: F401
from .tables import Tables  # noqa: F401
from .trees import PCAResult, Query, QueryBatch, TreeSequence, Workspace, load  # noqa: F401

__version__ = "0.1.0"
