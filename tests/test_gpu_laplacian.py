"""kNN graph adjacency (ctgb_laplacian / ctlib_gb300.laplacian) against the
fp64 oracle (oracle/laplacian.py) and against the reference's own laplacian run
on this GPU (its kernels and cuBLAS call, oracle/ref_cuda.py).

Parity bar, with tol_i the rounding bound of a squared distance in row i
(oracle/laplacian.py:distance_tol, 8 sqrt(dim) eps (|x_i|^2 + max |x_j|^2)):
* every row selects k points whose exact distances equal the oracle's k
  smallest, sorted, within tol_i;
* in increasing order of distance, within 2 tol_i;
* rows whose k-th and (k+1)-th exact distances are more than 2 tol_i apart
  select exactly the oracle's neighbours (in the others two evaluations may
  legitimately pick different k-th neighbours);
* the float32 weights of those rows within rel-L2 1e-5 (fp32 points) or 1e-6
  (fp64 points, whose weights are rounded to float32 at the end).
"""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ct():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import ctlib_gb300
    from ctlib_gb300 import _native
    _native.build()
    return ctlib_gb300


def _points(n, dim, seed, dtype=np.float32):
    return np.random.default_rng(seed).standard_normal((n, dim)).astype(dtype)


def _check_neighbours(cols, x, k, want_cols=None):
    """cols: n x k selected columns, in the order given. Returns the rows with
    a near tie at the k-th place."""
    from oracle import laplacian as OL
    d = OL.squared_distances(x)
    tol = OL.distance_tol(x)[:, None]
    d_sorted = np.sort(d, axis=1)
    got_d = np.take_along_axis(d, cols, 1)
    # the k smallest, within rounding, in increasing order within rounding
    assert np.all(np.abs(np.sort(got_d, axis=1) - d_sorted[:, :k]) <= tol)
    assert np.all(np.diff(got_d, axis=1) >= -2 * tol)
    ties = OL.near_tie_rows(d_sorted, k, tol[:, 0])
    if want_cols is not None:
        same = (np.sort(cols, axis=1) == np.sort(want_cols, axis=1)).all(1)
        bad = np.nonzero(~same & ~ties)[0]
        assert bad.size == 0, f"rows {bad[:10]} select other neighbours"
    return ties


def _by_column(cols, vals):
    o = np.argsort(cols, axis=1, kind="stable")
    return np.take_along_axis(vals, o, 1)


def _check_vs_oracle(W, x, k):
    from oracle import laplacian as OL
    n = x.shape[0]
    ind_w, val_w, coef, med = OL.laplacian(x, k)
    assert W.layout == torch.sparse_coo and W.dtype == torch.float32 and tuple(W.shape) == (n, n)
    assert not W.is_coalesced()
    ind = W._indices().cpu().numpy()
    val = W._values().cpu().numpy()
    assert ind.shape == (2, n * k) and val.shape == (n * k,)
    assert np.array_equal(ind[0], ind_w[0])
    cols, want = ind[1].reshape(n, k), ind_w[1].reshape(n, k)
    ties = _check_neighbours(cols, x, k, want)
    ok = ~ties
    tol = 1e-5 if x.dtype == np.float32 else 1e-6
    v = _by_column(cols, val.reshape(n, k))[ok]
    vw = _by_column(want, val_w.reshape(n, k))[ok]
    assert np.linalg.norm(v - vw) <= tol * np.linalg.norm(vw)
    return ties.sum()


@pytest.mark.parametrize("n,dim,k", [(1000, 16, 9), (777, 3, 5), (2048, 64, 16), (300, 129, 32),
                                     (130, 7, 130), (64, 1, 1), (50, 2, 2), (4100, 40, 256)])
def test_laplacian_vs_oracle(ct, n, dim, k):
    x = _points(n, dim, 100 + n + dim + k)
    W = ct.laplacian(torch.from_numpy(x).cuda(), k)
    torch.cuda.synchronize()
    if k <= 2:
        # the lower median of the selected distances is then a self-distance,
        # which is exactly 0 here (the norm and the dot product of a point
        # with itself are the same FMA chain), so the reference's weights
        # exp(-d/m) are 0/0; only the neighbours are compared
        _check_neighbours(W._indices()[1].cpu().numpy().reshape(n, k), x, k)
        return
    _check_vs_oracle(W, x, k)


def test_laplacian_fp64(ct):
    x = _points(900, 24, 7, np.float64)
    W = ct.laplacian(torch.from_numpy(x).cuda(), 12)
    assert W.dtype == torch.float32
    _check_vs_oracle(W, x, 12)


def test_ties_go_to_smaller_index(ct):
    # duplicated points: every point has an exact twin, so the two smallest
    # distances of a row tie (both 0 up to rounding of the same expression)
    base = _points(200, 8, 3)
    x = np.concatenate([base, base])
    W = ct.laplacian(torch.from_numpy(x).cuda(), 3)
    cols = W._indices()[1].cpu().numpy().reshape(400, 3)
    n = 200
    for i in range(400):
        twin = i + n if i < n else i - n
        assert set(cols[i, :2]) == {i, twin}
        assert cols[i, 0] == min(i, twin)


def test_deterministic_and_split_independent(ct):
    x = torch.from_numpy(_points(5000, 20, 11)).cuda()
    a = ct.laplacian(x, 10)
    b = ct.laplacian(x, 10)
    assert torch.equal(a._indices(), b._indices()) and torch.equal(a._values(), b._values())
    # a prefix of the points gives the same neighbours among themselves when
    # their neighbourhoods lie inside the prefix: compare with the oracle
    small = x[:700].contiguous()
    _check_vs_oracle(ct.laplacian(small, 10), small.cpu().numpy(), 10)


def test_errors(ct):
    x = torch.randn(10, 3, device="cuda")
    with pytest.raises(ValueError):
        ct.laplacian(x, 0)
    with pytest.raises(ValueError):
        ct.laplacian(x, 11)
    with pytest.raises(ValueError):
        ct.laplacian(x[None], 2)
    with pytest.raises(RuntimeError):
        ct.laplacian(x.t(), 2)
    with pytest.raises(RuntimeError):
        ct.laplacian(x.cpu(), 2)
    with pytest.raises(ValueError):
        ct.laplacian(torch.randn(300, 3, device="cuda"), 257)


@pytest.fixture(scope="module")
def ref():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import ref_cuda
    if not ref_cuda.laplacian_available():
        pytest.skip("reference cubins not built")
    return ref_cuda.get()


@pytest.mark.parametrize("n,dim,k,dtype", [(1000, 16, 9, np.float32), (2048, 64, 16, np.float32),
                                           (777, 3, 5, np.float32), (600, 24, 12, np.float64)])
def test_laplacian_vs_reference_gpu(ct, ref, n, dim, k, dtype):
    x = _points(n, dim, 500 + n, dtype)
    xt = torch.from_numpy(x).cuda()
    Wr = ref.laplacian(xt, k)
    W = ct.laplacian(xt, k)
    torch.cuda.synchronize()
    assert Wr.dtype == W.dtype == torch.float32 and tuple(Wr.shape) == tuple(W.shape)
    ir, io = Wr._indices().cpu().numpy(), W._indices().cpu().numpy()
    assert np.array_equal(ir[0], io[0])
    # both select correctly within the rounding bound, and identically outside
    # near ties
    cr, co = ir[1].reshape(n, k), io[1].reshape(n, k)
    _check_neighbours(cr, x, k)
    ties = _check_neighbours(co, x, k, cr)
    vr = _by_column(cr, Wr._values().cpu().numpy().reshape(n, k))[~ties]
    v = _by_column(co, W._values().cpu().numpy().reshape(n, k))[~ties]
    assert np.linalg.norm(v - vr) <= 1e-5 * np.linalg.norm(vr)


def test_fp64_large_k_fits_or_is_refused(ct):
    """fp64 lists of many neighbours outgrow a CTA's shared memory: the call is
    refused with a clear error instead of launching; a k that fits runs."""
    x64 = torch.from_numpy(_points(400, 8, 13, np.float64)).cuda()
    with pytest.raises(ValueError, match="shared memory"):
        ct.laplacian(x64, 256)
    W = ct.laplacian(x64, 64)
    _check_vs_oracle(W, x64.cpu().numpy(), 64)
