"""The strict FP64 forms divide every stencil term by the grid spacing with a
reciprocal, one correction and an exact check (the IEEE division when the
check fails).  Here that quotient must equal the IEEE one bit for bit over
dividends chosen to be hard: every exponent, ties and near-ties, powers of two
on either side, zeros, subnormals, extremes and non-finite values, for
ordinary and unusual divisors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIVISORS = [10.0, 12.0, 11.0, 12.5, 3.0, 7.0, 0.1, 1.0, 0.5, -5.0, 1e-300, 3e300, 2.0 ** -1000, 5e-324,
            np.nextafter(10.0, 11.0)]


def hard_dividends(d, rng):
    parts = []
    n = 1 << 18
    # every exponent, both signs
    e = rng.integers(-1074, 1024, n)
    parts.append(rng.choice([-1.0, 1.0], n) * rng.uniform(1.0, 2.0, n) * np.ldexp(1.0, e - 1).astype(np.float64))
    # raw bit patterns (subnormals, infinities, NaNs included)
    parts.append(rng.integers(0, 2 ** 64, n, dtype=np.uint64).view(np.float64))
    # near-ties: a / d within an ulp of a midpoint between two doubles
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        q = rng.uniform(-1.0, 1.0, n) * np.ldexp(1.0, rng.integers(-900, 900, n))
        mid = q + np.spacing(q) / 2
        a = mid * d
        parts.append(np.concatenate([a, np.nextafter(a, np.inf), np.nextafter(a, -np.inf)]))
        # quotients next to powers of two, from either side
        k = np.arange(-1000, 1000, dtype=np.float64)
        p2 = np.ldexp(1.0, k.astype(int)) * d
        parts.append(np.concatenate([p2, np.nextafter(p2, np.inf), np.nextafter(p2, -np.inf), -p2]))
        # exact multiples (zero remainders)
        parts.append(d * rng.integers(-10 ** 6, 10 ** 6, n).astype(np.float64))
    parts.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                           np.finfo(np.float64).max, -np.finfo(np.float64).max, 1.0, -1.0, d, -d]))
    return np.concatenate(parts)


@pytest.mark.parametrize("d", DIVISORS)
def test_division_equals_ieee(gpu, d):
    S = gpu
    rng = np.random.default_rng(abs(hash(float(d))) % (2 ** 32))
    a = hard_dividends(d, rng)
    fast, ieee = S.debug_divide(a, d)
    fb, ib = fast.view(np.uint64), ieee.view(np.uint64)
    nan = np.isnan(ieee)
    assert np.array_equal(np.isnan(fast), nan)
    bad = np.flatnonzero((fb != ib) & ~nan)
    assert bad.size == 0, [(a[k], fast[k], ieee[k]) for k in bad[:5]]
    # and the IEEE quotient is the host's
    with np.errstate(all="ignore"):
        host = a / d
    assert np.array_equal(host.view(np.uint64)[~nan], ib[~nan])
