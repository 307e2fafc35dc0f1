"""Summary functions of the real-weighted general_stat tests (shared by the
golden-value generator and the GPU test): name -> (state dimension K,
output dimension, f)."""
import numpy as np


def _square(x):
    return np.array([x[0] * x[0]])


def _mixed(x):
    return np.array([x[0] * x[1], np.sin(x[0]) - 0.5 * x[1], 1.0 + x[1] * x[1]])


def _three(x):
    return np.array([np.abs(x[0] - x[2]) * x[1], np.exp(-x[1] * x[1])])


SUMMARIES = {
    "square": (1, 1, _square),
    "mixed": (2, 3, _mixed),
    "three": (3, 2, _three),
}


def _count_pair(x):
    # sample_count_stat summaries see the set sizes through closure defaults
    return np.array([x[0] * (6.0 - x[0]), x[0] * x[1] - 2.0 * x[1]])


# sample_count_stat summaries: name -> (set sizes, output dimension, f); the
# sets are the first sizes[k] samples after the previous sets
COUNT_SUMMARIES = {
    "pair": ((6, 5), 2, _count_pair),
}
