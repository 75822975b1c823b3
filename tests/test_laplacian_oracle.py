"""The CPU restatement of ``laplacian`` (oracle/laplacian.py) on small cases
worked out independently: brute-force neighbour lists, the lower median and
the row normalisation."""

import numpy as np

from oracle import laplacian as OL


def test_line_of_points():
    # points 0, 1, 3, 6 on a line: squared distances are exact
    x = np.array([[0.0], [1.0], [3.0], [6.0]])
    ind, val, coef, med = OL.laplacian(x, 3)
    assert ind.shape == (2, 12)
    assert np.array_equal(ind[0], np.repeat(np.arange(4), 3))
    assert np.array_equal(ind[1].reshape(4, 3), [[0, 1, 2], [1, 0, 2], [2, 1, 0], [3, 2, 1]])
    assert np.array_equal(coef, [[0, 1, 9], [0, 1, 4], [0, 4, 9], [0, 9, 25]])
    # 12 values 0,0,0,0,1,1,4,4,9,9,9,25: the lower median is the 6th, 1
    assert med == 1.0
    w = np.exp(-np.array([[0, 1, 9], [0, 1, 4], [0, 4, 9], [0, 9, 25]]) / 1.0)
    w = w / w.sum(1, keepdims=True)
    assert np.allclose(val, w.ravel().astype(np.float32), rtol=0, atol=0)
    assert val.dtype == np.float32


def test_ties_to_smaller_index():
    x = np.array([[0.0, 0.0], [1.0, 0.0], [-1.0, 0.0], [0.0, 1.0]])
    ind, _, _, _ = OL.laplacian(x, 3)
    # row 0: itself, then points 1, 2, 3 all at distance 1 -> 1 and 2
    assert list(ind[1][:3]) == [0, 1, 2]


def test_random_matches_brute_force():
    rng = np.random.default_rng(5)
    x = rng.standard_normal((60, 5))
    ind, val, coef, med = OL.laplacian(x, 7)
    for i in range(60):
        d = [float(((x[i] - x[j]) ** 2).sum()) for j in range(60)]
        order = sorted(range(60), key=lambda j: (d[j], j))[:7]
        assert list(ind[1][i * 7:(i + 1) * 7]) == order
        assert np.allclose(coef[i], [d[j] for j in order], rtol=1e-12, atol=1e-12)
    assert np.allclose(val.reshape(60, 7).sum(1), 1.0, atol=1e-6)


def test_near_tie_rows():
    d = np.array([[0.0, 1.0, 2.0, 2.0 + 1e-9], [0.0, 1.0, 2.0, 3.0]])
    assert list(OL.near_tie_rows(d, 3, 1e-6)) == [True, False]
