"""The oracle's restatement of the synthetic producer (CPU): the two-tone
block's spectrum holds exactly the reference generator's two bins, and the
stream samples have the stated statistics and continue across blocks."""
import numpy as np

from oracle import gspec_oracle as O


def test_two_tone_bins():
    n = 1 << 14
    x = O.dummy_two_tone_block(n).astype(np.float64)
    p = np.abs(np.fft.rfft(x - x.mean())) ** 2
    nf = n // 2 + 1
    top = set(np.argsort(p)[-2:].tolist())
    assert top == {nf // 3, nf // 2}
    # the minimum maps to 0; the maximum to (max - min) / level, 255 or just below it (truncated)
    assert x.min() == -128 and x.max() in (126, 127)


def test_stream_statistics_and_continuation():
    a = O.dummy_stream_samples(11, 0, 0, 1 << 16, 80.0, 0.0, 0, 12)
    b = O.dummy_stream_samples(11, 0, 1 << 15, 1 << 15, 80.0, 0.0, 0, 12)
    assert np.array_equal(a[1 << 15:], b)
    assert abs(a.mean()) < 2.0 and abs(a.std() - 80.0) < 2.0
    c = O.dummy_stream_samples(11, 1, 0, 1 << 16, 80.0, 0.0, 0, 12)
    assert abs(np.corrcoef(a, c)[0, 1]) < 0.02     # pols independent
