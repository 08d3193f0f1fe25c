"""CPU restatement of the random-number stream used by the reference's sweep sampler.

TEST INFRASTRUCTURE ONLY: this module is the oracle's RNG, used by tests/, __graft_entry__.smoke()
and bench.py's CPU baseline as a checker. The product path draws its numbers on the GPU.

The reference keeps one global ``std::mt19937_64`` (PyTAT/PyTAT.hpp:87) that ``TAT.random.seed``
re-seeds (PyTAT/PyTAT.hpp:89-94).  Each Metropolis proposal of ``SweepSampling._single_term``
(tetragono/tetragono/sampling_lattice/sampling.py:117-143) draws

* ``TAT.random.uniform_int(0, n-1)()`` - a fresh ``std::uniform_int_distribution<int>`` per call
  (PyTAT/PyTAT.hpp:95-103).  With a 64-bit engine libstdc++ 13 downscales with Lemire's
  nearly-divisionless method on a 128-bit product (bits/uniform_int_dist.h, ``_S_nd``);
* ``TAT.random.uniform_real(0, 1)()`` - ``std::uniform_real_distribution<double>``
  (PyTAT/PyTAT.hpp:104-113), i.e. ``generate_canonical<double, 53>``: one engine word
  converted to double (round to nearest) and divided by 2**64, clamped below 1.

The Mersenne-Twister itself is the published MT19937-64 algorithm (Matsumoto & Nishimura 2000):
n=312, m=156, twist matrix 0xB5026F5AA96619E9, the standard tempering shifts and masks, and the
standard single-word seeding recurrence with multiplier 6364136223846793005.
"""

MASK64 = (1 << 64) - 1

_NN = 312
_MM = 156
_MATRIX_A = 0xB5026F5AA96619E9
_UM = 0xFFFFFFFF80000000
_LM = 0x7FFFFFFF


class MT19937_64:
    """Published MT19937-64 generator; ``seed(s)`` matches ``std::mt19937_64::seed(s)``."""

    __slots__ = ["mt", "mti"]

    def __init__(self, seed=5489):
        self.seed(seed)

    def seed(self, seed):
        mt = [0] * _NN
        mt[0] = seed & MASK64
        for i in range(1, _NN):
            mt[i] = (6364136223846793005 * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i) & MASK64
        self.mt = mt
        self.mti = _NN

    def _twist(self):
        mt = self.mt
        for i in range(_NN):
            x = (mt[i] & _UM) | (mt[(i + 1) % _NN] & _LM)
            xa = x >> 1
            if x & 1:
                xa ^= _MATRIX_A
            mt[i] = mt[(i + _MM) % _NN] ^ xa
        self.mti = 0

    def __call__(self):
        if self.mti >= _NN:
            self._twist()
        y = self.mt[self.mti]
        self.mti += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & MASK64


def uniform_int(engine, a, b):
    """``std::uniform_int_distribution<int>(a, b)(engine)`` for a 64-bit engine (libstdc++ 13)."""
    n = b - a + 1  # "uerange"; urange = b - a can be zero
    product = engine() * n
    low = product & MASK64
    if low < n:
        threshold = ((1 << 64) - n) % n
        while low < threshold:
            product = engine() * n
            low = product & MASK64
    return (product >> 64) + a


def uniform_real01(engine):
    """``std::uniform_real_distribution<double>(0, 1)(engine)`` for a 64-bit engine (libstdc++ 13)."""
    x = engine()
    r = float(x) / 18446744073709551616.0
    if r >= 1.0:
        r = 0.99999999999999989  # nextafter(1.0, 0.0)
    return r * (1.0 - 0.0) + 0.0
