"""The device Gaussian sketch: Philox4x32-10 + Box-Muller.

Philox4x32-10 is the published counter-based generator of Salmon, Moraes,
Dror and Shaw ("Parallel random numbers: as easy as 1, 2, 3", SC'11; the
Random123 library).  A plain-Python restatement here is first pinned to the
known-answer vectors published with Random123 (kat_vectors, philox4x32 with
10 rounds); the device sketch is then compared element by element with that
restatement plus the Box-Muller transform (numpy's log/sqrt/sin/cos: the
device's differ by a few ulps), and its moments are checked.
"""
import numpy as np
import pytest

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF

# (counter words, key words) -> output words, from Random123's kat_vectors.
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((MASK,) * 4, (MASK, MASK), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def philox4x32_10(ctr, key):
    """Vectorised over numpy uint64 arrays of 32-bit words."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) for x in ctr)
    k0, k1 = (np.asarray(x, dtype=np.uint64) for x in key)
    for _ in range(10):
        p0 = np.uint64(M0) * c0
        p1 = np.uint64(M1) * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
        k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
    return c0, c1, c2, c3


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_restatement_matches_published_vectors(ctr, key, want):
    got = philox4x32_10(ctr, key)
    assert tuple(int(x) for x in got) == want


def sketch_reference(rows, cols, seed):
    """The sketch as the device defines it, from the restatement."""
    total = rows * cols
    pairs = (total + 1) // 2
    p = np.arange(pairs, dtype=np.uint64)
    x0, x1, x2, x3 = philox4x32_10((p & np.uint64(MASK), p >> np.uint64(32), 0, 0),
                                   (seed & MASK, seed >> 32))
    a = (x1 << np.uint64(32)) | x0
    b = (x3 << np.uint64(32)) | x2
    u1 = ((a >> np.uint64(11)).astype(np.float64) + 1.0) * 2.0 ** -53
    u2 = (b >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    rad = np.sqrt(-2.0 * np.log(u1))
    out = np.empty(2 * pairs)
    out[0::2] = rad * np.cos(2.0 * np.pi * u2)
    out[1::2] = rad * np.sin(2.0 * np.pi * u2)
    return out[:total].reshape(cols, rows).T  # element e = c * rows + r


@pytest.mark.gpu
@pytest.mark.parametrize("rows,cols,seed", [(74, 2000, 12), (138, 16384, 12), (7, 5, 2 ** 40 + 3)])
def test_device_sketch_matches_restatement(hq, rows, cols, seed):
    G = hq.sketch_device(rows, cols, seed).cpu().numpy().T
    R = sketch_reference(rows, cols, seed)
    assert np.max(np.abs(G - R) / np.maximum(1.0, np.abs(R))) <= 1e-13


@pytest.mark.gpu
def test_device_sketch_moments(hq):
    G = hq.sketch_device(138, 16384, 12).cpu().numpy().ravel()
    N = G.size
    assert abs(G.mean()) <= 5.0 / np.sqrt(N)
    assert abs(G.var() - 1.0) <= 5.0 * np.sqrt(2.0 / N)
    assert abs(np.mean(G ** 4) - 3.0) <= 5.0 * np.sqrt(96.0 / N)
    from scipy import stats
    assert stats.kstest(G[:200000], "norm").pvalue > 1e-4
