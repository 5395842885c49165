"""Post-processing restatement (exec/exec_helper.c:63-271, wrappers/src/param.c:1229-1357)
on a sample whose answers follow by hand from the reference's loops: 64 points
0..63 with weight 1/64 each (every cumulative sum exact), plus samples with
flg = 0 that must not count."""
import numpy as np
import pytest

import oracle as O


def sample():
    x = np.arange(64, dtype=np.float64)
    X = np.concatenate([x, [1e3, -1e3, 7.5]])[:, None] * np.ones((1, 2))
    X[:, 1] *= -1.0                            # a second parameter, mirrored
    w = np.concatenate([np.full(64, 1.0 / 64), [0.3, 0.3, 0.3]])
    flg = np.concatenate([np.ones(64), np.zeros(3)]).astype(np.int16)
    return X, w, flg


def test_mean_and_limits():
    X, w, flg = sample()
    c, s, st = O.weighted_summary(X, w, flg)
    assert np.all(st == 0)
    assert c[0] == 31.5 and c[1] == -31.5
    # imean = 32; 68.27 %: 22 points (22/64 > 0.3413) on each side -> samples 54 and 9
    # 95.45 %: 31 points -> samples 63 and 0; 99.73 %: the sample ends first -> -1
    np.testing.assert_array_equal(s[0], [22.5, 31.5, -1.0, 22.5, 31.5, -1.0])
    np.testing.assert_array_equal(s[1], [22.5, 31.5, -1.0, 22.5, 31.5, -1.0])


def test_median_and_limits():
    X, w, flg = sample()
    c, s, st = O.weighted_summary(X, w, flg, median=True)
    assert np.all(st == 0)
    # the cumulative weight reaches 1/2 exactly at sample 31
    assert c[0] == 31.0
    # imean = 31; right: 22, 31, 32 points -> samples 53, 62, 63; left from 30: 22 points -> 8, then the end
    np.testing.assert_array_equal(s[0], [22.0, 31.0, 32.0, 23.0, -1.0, -1.0])
    assert c[1] == -32.0   # mirrored values: the 32nd smallest is -32, reached exactly


def test_histograms():
    X, w, flg = sample()
    h = O.hist1d(X, w, flg, 8, [0.0, -64.0], [64.0, 0.0], 64.0)
    np.testing.assert_array_equal(h[0], np.full(8, 8.0))       # 8 points of weight 1/64, times 64
    # parameter 1 runs over [-63, 0]: -63..-57 (7 points) in the first bin, 0 in the last bin (closed edge)
    np.testing.assert_array_equal(h[1], [7.0, 8.0, 8.0, 8.0, 8.0, 8.0, 8.0, 9.0])
    # bins of 16: x // 16 against (64 - x) // 16 (0 in the closed last bin): x = 16, 32, 48 fall
    # one bin off the anti-diagonal
    h2 = O.hist2d(X, w, flg, 4, 0, 1, [0.0, -64.0], [64.0, 0.0], 64.0)
    np.testing.assert_array_equal(np.diag(h2[:, ::-1]), [16.0, 15.0, 15.0, 15.0])
    assert h2[1, 3] == 1.0 and h2[2, 2] == 1.0 and h2[3, 1] == 1.0 and h2.sum() == 64.0
