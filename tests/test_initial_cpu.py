"""CPU checks of the initial-conditions restatement and table."""
import numpy as np

from conftest import module
from oracle import ic_oracle as IO


def test_spectrum_amplitudes_follow_the_table():
    n, L = 16, 50.0
    ini = module("initial")
    K, P = ini.pk_table(n, L)
    assert K.dtype == np.float32 and len(K) == ini.TABLE_N and np.all(np.diff(K) > 0)
    ones = np.ones((n, n, n // 2 + 1), np.float32)
    H = IO.spectrum(n, L, ones, np.zeros_like(ones), K, P)
    assert H[0, 0, 0] == 0
    dk = np.float32(2 * np.pi / np.float32(L))
    # mode (1, 0, 0) on the kz = 0 plane: sqrt(P(dk) V), interior mode (0, 0, 1): divided by sqrt 2
    p1 = np.interp(dk, K, P)
    assert abs(H[1, 0, 0].real / np.sqrt(p1 * L ** 3) - 1) < 1e-4
    assert abs(H[0, 0, 1].real / np.sqrt(p1 * L ** 3 / 2) - 1) < 1e-4


def test_subsample_picks_the_nearest_cell():
    big = np.arange(8 ** 3, dtype=np.float32).reshape(8, 8, 8)
    small = IO.subsample(big, 4, 2.0)
    assert np.array_equal(small, big[0::2, 0::2, 0::2])   # floor(2 a + 0.5) = 2 a
    odd = IO.subsample(np.arange(12 ** 3, dtype=np.float32).reshape(12, 12, 12), 8, 1.5)
    idx = np.floor(np.arange(8) * 1.5 + 0.5).astype(int)               # 0 2 3 5 6 8 9 11
    assert list(idx) == [0, 2, 3, 5, 6, 8, 9, 11]
    assert np.array_equal(odd, np.arange(12 ** 3, dtype=np.float32).reshape(12, 12, 12)[np.ix_(idx, idx, idx)])
