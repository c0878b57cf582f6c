"""The division of list entries by T used by the list, preparation and sweep kernels.

`div_t_magic` / `div_t` in `ksvd_gb300/csrc/update.cu` compute floor(e / T) for an entry
e = signal * T + slot (0 <= e < 2^31) as mulhi(2 e, m) >> l with l = ceil(log2 T) and
m = ceil(2^(31 + l) / T), a 32-bit constant (Granlund & Montgomery, PLDI 1994, Thm 4.2 with
31-bit dividends).  This restates the same arithmetic on Python integers and checks it at the
boundaries and on random entries for every support size the library accepts; the GPU parity
tests run the device code itself.
"""
import random

import pytest


def magic(T):
    l = 0
    while (1 << l) < T:
        l += 1
    m = ((1 << (31 + l)) + T - 1) // T
    return m, l


def div(e, m, l):
    return ((((e << 1) & 0xFFFFFFFF) * m) >> 32) >> l


@pytest.mark.parametrize("T", list(range(1, 65)) + [100, 1000, 65537])
def test_multiply_high_division_is_exact(T):
    m, l = magic(T)
    assert 0 < m < 2**32
    top = 2**31 - 1
    cases = [0, 1, T - 1, T, T + 1, top, top - 1, top - top % T, top - top % T - 1]
    rng = random.Random(T)
    cases += [rng.randrange(2**31) for _ in range(4000)]
    for e in cases:
        assert div(e, m, l) == e // T, (T, e)
