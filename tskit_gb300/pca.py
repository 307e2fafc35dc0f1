"""Principal components of the genetic relatedness matrix, by randomized SVD.

The drop-in for ``TreeSequence.pca`` (python/tskit/trees.py:9284-9537): the
same arguments, checks, error messages, random sketch and outputs (factors,
eigenvalues, the final range sketch, an error bound).  The relatedness matrix
is never formed: every product with it is one branch relatedness
matrix-vector sweep on the GPU (``genetic_relatedness_vector``), all sketch
columns at once.

The method is the randomized SVD with power iterations of Halko, Martinsson
and Tropp (SIAM Review 53, 2011, sections 4.5 and 5.1) as stated in
Martinsson and Tropp, "Randomized numerical linear algebra" (arXiv:2002.01387,
Algorithms 8 and 9):

1. range finder: from a Gaussian sketch Y, alternate an orthonormalisation
   (QR) and a product with the operator q times, and orthonormalise once
   more: Q spans approximately the dominant range of A;
2. factorisation: B = (A Q)^T is small (columns x rows); its SVD
   B = U_B S V^T gives A ~ (Q U_B) S V^T, and since A is symmetric the left
   factors Q U_B are the principal directions and S the eigenvalues;
3. the a-posteriori bound of the paper's Corollary 10.10 form,
   sigma_{k+1} (1 + [1 + 4 sqrt(2 d / (k - 1))]^{1 / (2q + 1)}), as the
   reference reports it.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class PCAResult:
    """The result of ``TreeSequence.pca`` (python/tskit/trees.py PCAResult)."""

    factors: np.ndarray
    eigenvalues: np.ndarray
    range_sketch: np.ndarray
    error_bound: np.ndarray


class RelatednessOperator:
    """x -> A x for the centred branch relatedness matrix A of a set of rows
    (sample nodes, or individuals averaging their nodes) in one window,
    optionally the difference of two time slices of the genealogy (the
    topology younger than the upper time minus the one younger than the
    lower time)."""

    def __init__(self, upper, lower, ts, rows, by_individual, mode, centre, window):
        self.upper, self.lower = upper, lower
        self.mode, self.centre, self.window = mode, centre, window
        sample_index = np.full(ts.num_nodes, -1, dtype=np.int64)
        sample_index[ts.samples()] = np.arange(ts.num_samples)
        if by_individual:
            nodes, owner = [], []
            for k, ind in enumerate(rows):
                members = ts._individual_nodes(ind)
                nodes.extend(members.tolist())
                owner.extend([k] * len(members))
            self.nodes = np.asarray(nodes, dtype=np.int64)
            self.owner = np.asarray(owner, dtype=np.int64)
            self.ploidy = np.bincount(self.owner, minlength=len(rows)).astype(np.float64)
        else:
            self.nodes = np.asarray(rows, dtype=np.int64)
            self.owner = None
        self.rows = len(rows)
        self.positions = sample_index[self.nodes]
        if np.any(self.positions < 0):
            raise ValueError("pca rows must be sample nodes (or individuals of sample nodes)")
        self.num_samples = ts.num_samples

    def _node_weights(self, X):
        """Each node's weight row: its row of X, or its individual's row
        divided by the individual's number of nodes."""
        if self.owner is None:
            return X
        return X[self.owner] / self.ploidy[self.owner, None]

    def _rows_from_nodes(self, Y):
        if self.owner is None:
            return Y
        out = np.zeros((self.rows, Y.shape[1]))
        np.add.at(out, self.owner, Y)
        return out / self.ploidy[:, None]

    def _sweep(self, ts, W):
        return ts.genetic_relatedness_vector(W=W, windows=self.window, mode=self.mode,
                                             centre=False, nodes=self.nodes,
                                             span_normalise=False)[0]

    def __call__(self, X):
        X = np.asarray(X, dtype=np.float64)
        if self.centre:
            X = X - X.mean(axis=0)
        W = np.zeros((self.num_samples, X.shape[1]))
        W[self.positions] = self._node_weights(X)
        Y = self._sweep(self.upper, W)
        if self.lower is not None:
            Y = Y - self._sweep(self.lower, W)
        Y = self._rows_from_nodes(Y)
        return Y - Y.mean(axis=0) if self.centre else Y


def range_finder(op, sketch, iterations):
    """Orthonormal basis of the dominant range of ``op`` (Martinsson and
    Tropp, Algorithm 9 with re-orthonormalisation before every product)."""
    basis = sketch
    for _ in range(iterations):
        basis = op(np.linalg.qr(basis)[0])
    return np.linalg.qr(basis)[0]


def randomized_svd(op, dim, rank, iterations, sketch):
    """Leading ``rank`` singular vectors and values of the symmetric ``op``
    from ``sketch``; also the basis found and the a-posteriori bound."""
    basis = range_finder(op, sketch, iterations)
    small = op(basis).T
    u_small, values, _ = np.linalg.svd(small, full_matrices=False)
    vectors = basis @ u_small
    factor = (1 + 4 * np.sqrt(2 * dim / max(1, rank - 1))) ** (1 / (2 * iterations + 1))
    bound = values[rank] * (1 + factor)
    return vectors[:, :rank], values[:rank], basis, bound


def _check_and_sketch(ts, num_components, windows, samples, individuals, num_iterations,
                      num_oversamples, random_seed, range_sketch):
    """The reference's argument checks, in its order and with its messages
    (python/tskit/trees.py:9420-9500), and the Gaussian sketch it draws."""
    if (not isinstance(num_iterations, int)) or num_iterations < 1:
        raise ValueError("num_iterations should be a positive integer.")
    if samples is None and individuals is None:
        samples = ts.samples()
    if samples is not None and individuals is not None:
        raise ValueError("Samples and individuals cannot be used at the same time")
    by_individual = samples is None
    rows = individuals if by_individual else samples
    dim = len(rows)
    drop_windows = windows is None
    windows = ts.parse_windows(windows)
    num_windows = len(windows) - 1
    if num_windows < 1:
        raise ValueError("Must have at least one window.")
    if num_components > dim:
        raise ValueError(
            "Number of components must be less than or equal to "
            "the number of samples (or individuals, if specified).")
    if num_oversamples is not None and range_sketch is not None:
        raise ValueError("Cannot specify both num_oversamples and range_sketch.")
    if range_sketch is None:
        if num_oversamples is None:
            num_oversamples = min(10, dim - num_components)
        rng = np.random.default_rng(random_seed)
        range_sketch = rng.normal(size=(num_windows, dim, num_components + num_oversamples))
    else:
        if drop_windows:
            range_sketch = np.expand_dims(range_sketch, 0)
        if range_sketch.shape[-1] < num_components:
            raise ValueError("range_sketch must have at least as many columns as num_components")
        num_oversamples = range_sketch.shape[-1] - num_components
    num_vectors = num_components + num_oversamples
    if num_vectors > dim:
        raise ValueError(
            "Number of columns in range_sketch "
            "(num_components + num_oversamples) must be less"
            " than or equal to the number of samples"
            " (or individuals, if specified).")
    expected = (num_windows, dim, num_vectors)
    if range_sketch.shape != expected:
        got = range_sketch.shape
        if drop_windows:
            got, expected = got[1:], expected[1:]
        raise ValueError(f"Incorrect shape of range_sketch: expected {expected}; got {got}.")
    return rows, by_individual, dim, windows, drop_windows, range_sketch


def pca(ts, num_components, windows=None, samples=None, individuals=None, time_windows=None,
        mode="branch", centre=True, num_iterations=5, num_oversamples=None, random_seed=None,
        range_sketch=None):
    """TreeSequence.pca: one randomized SVD per window; see the module
    docstring."""
    rows, by_individual, dim, windows, drop_windows, range_sketch = _check_and_sketch(
        ts, num_components, windows, samples, individuals, num_iterations, num_oversamples,
        random_seed, range_sketch)
    if time_windows is None:
        upper, lower = ts, None
    else:
        assert time_windows[0] < time_windows[1], "The second argument should be larger."
        upper, lower = ts._decapitated(time_windows[1]), ts._decapitated(time_windows[0])
    results = []
    for w in range(len(windows) - 1):
        op = RelatednessOperator(upper, lower, ts, rows, by_individual, mode, centre,
                                 windows[w:w + 2])
        results.append(randomized_svd(op, dim, num_components, num_iterations,
                                      range_sketch[w]))
    factors, values, bases, bounds = (np.stack(part) for part in zip(*results))
    if drop_windows:
        factors, values, bases, bounds = factors[0], values[0], bases[0], bounds[0]
    return PCAResult(factors=factors, eigenvalues=values, range_sketch=bases, error_bound=bounds)
