"""The FP64 timestep's integer-arithmetic division (lbmath::div_rn, used by
the GPU kernels for F/rho and the weighted velocity) against the hardware
IEEE division: the same bits for every pair of doubles, including the cases
it hands back to a / b (zeros, subnormals, infinities, NaNs, powers of two,
overflowing and underflowing quotients)."""
import numpy as np

from oracle import oracle as orc


def _same(a, b):
    got = orc.div(a, b)
    with np.errstate(all="ignore"):
        want = a / b
    nan = np.isnan(got) & np.isnan(want)
    bad = ~nan & (got.view(np.uint64) != want.view(np.uint64))
    return bad


def test_random_bit_patterns():
    rng = np.random.default_rng(11)
    a = rng.integers(0, 2**64, 2_000_000, dtype=np.uint64).view(np.float64)
    b = rng.integers(0, 2**64, 2_000_000, dtype=np.uint64).view(np.float64)
    bad = _same(a, b)
    assert not bad.any(), (a[bad][:5], b[bad][:5])


def test_lattice_ranges_and_significand_edges():
    rng = np.random.default_rng(12)
    n = 1_000_000
    # forces over densities, momenta over total densities
    a = (rng.random(n) - 0.5) * 1e-2
    b = 0.02 + 2.0 * rng.random(n)
    assert not _same(a, b).any()
    # significands 1 + 2^-52 k and 2 - 2^-52 k, equal significands, exact quotients
    k = rng.integers(1, 2**20, n, dtype=np.uint64)
    e = rng.integers(900, 1100, n, dtype=np.uint64) << np.uint64(52)
    lo = (e | k).view(np.float64)
    hi = (e | ((np.uint64(1) << np.uint64(52)) - k)).view(np.float64)
    x = (e | rng.integers(0, 2**52, n, dtype=np.uint64)).view(np.float64)
    for num, den in ((x, lo), (x, hi), (lo, hi), (hi, lo), (lo, lo), (x * 3.0, x), (np.floor(x), 3.0 + 0 * x)):
        assert not _same(num, den).any()


def test_special_operands():
    vals = np.array([0.0, -0.0, 1.0, -1.0, 2.0, 0.5, 3.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308,
                     1.7976931348623157e308, 1e-300, 1e300, 0.7, 0.05])
    a, b = np.meshgrid(vals, vals)
    assert not _same(a.ravel(), b.ravel()).any()
    # quotients crossing the bottom (2^-1022) and the top of the normal range
    rng = np.random.default_rng(13)
    a = (1.0 + rng.random(100000)) * 2.0 ** -1000
    b = (1.0 + rng.random(100000)) * 2.0 ** rng.integers(18, 26, 100000)
    assert not _same(a, b).any()
    big = (1.0 + rng.random(100000)) * 2.0 ** 1022
    assert not _same(big, 0.25 + 1.5 * rng.random(100000)).any()
