"""CPU restatement of CTLIB's ``laplacian`` (TEST INFRASTRUCTURE ONLY).

Follows src/laplacian_cuda_kernel.cu:46-128 in numpy, in fp64:

* squared distances dist[i][j] = |x_i|^2 + |x_j|^2 - 2 <x_i, x_j>
  (``compute_squared_norm`` :10-22, ``add_norm`` :25-43, the GEMM :88-106);
* the k smallest entries of every row, in increasing order (``torch::topk(dist,
  k, 1, false)`` :112); ties go to the smaller column, as in this package;
* the lower median of all n*k selected distances (``torch::median`` :115);
* weights exp(-d / median), normalised to sum 1 per row (:116-119);
* COO indices (row, column) in row-major order and float32 values (:120-126).
"""

from __future__ import annotations

import numpy as np


def squared_distances(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=np.float64)
    norm = np.einsum("ij,ij->i", x, x)
    return norm[:, None] + norm[None, :] - 2.0 * (x @ x.T)


def knn(x: np.ndarray, k: int):
    """(distances, columns) of the k nearest points of every point, n x k."""
    d = squared_distances(x)
    idx = np.argsort(d, axis=1, kind="stable")[:, :k]
    return np.take_along_axis(d, idx, 1), idx


def lower_median(v: np.ndarray) -> float:
    s = np.sort(np.asarray(v).ravel())
    return float(s[(s.size - 1) // 2])


def laplacian(x: np.ndarray, k: int):
    """(indices 2 x n*k int64, values n*k float32, selected distances n x k,
    median) of the reference's kNN adjacency."""
    n = x.shape[0]
    if not 1 <= k <= n:
        raise ValueError("k must be in [1, n]")
    coef, idx = knn(x, k)
    med = lower_median(coef)
    w = np.exp(-(coef / med))
    w = w / w.sum(1, keepdims=True)
    rows = np.repeat(np.arange(n, dtype=np.int64), k)
    ind = np.stack([rows, idx.ravel().astype(np.int64)])
    return ind, w.ravel().astype(np.float32), coef, med


def distance_tol(x: np.ndarray) -> np.ndarray:
    """Per-row bound on the rounding error of a squared distance evaluated in
    x's precision as |x_i|^2 + |x_j|^2 - 2 <x_i, x_j>: 8 sqrt(dim) eps
    (|x_i|^2 + max_j |x_j|^2), eps the unit roundoff (a generous multiple of the
    typical error of a length-dim dot product)."""
    eps = 2.0 ** -24 if np.asarray(x).dtype == np.float32 else 2.0 ** -53
    x64 = np.asarray(x, dtype=np.float64)
    norm = np.einsum("ij,ij->i", x64, x64)
    return 8.0 * np.sqrt(x64.shape[1]) * eps * (norm + norm.max())


def near_tie_rows(d_sorted: np.ndarray, k: int, tol: np.ndarray) -> np.ndarray:
    """Rows whose k-th and (k+1)-th smallest exact distances are within twice
    the rounding bound `tol` of each other: there two evaluations of the
    distances may legitimately select different k-th neighbours."""
    if d_sorted.shape[1] <= k:
        return np.zeros(d_sorted.shape[0], dtype=bool)
    return (d_sorted[:, k] - d_sorted[:, k - 1]) <= 2.0 * tol
