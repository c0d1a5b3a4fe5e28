"""Philox4x32-10 known-answer vectors (Salmon et al., SC'11 / Random123
kat_vectors) for both implementations: the oracle's C++ and the engine's
host-compiled copy are checked against the same published outputs."""
import pytest

from oracle import oracle as O

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_oracle_philox_kat(ctr, key, expect):
    assert tuple(O.philox(ctr, key)) == expect


def test_stream_layout():
    # counter = {slot, move lo, move hi, stream}, key = seed
    seed = 0x0123456789ABCDEF
    got = O.draw(seed, 7, (5 << 32) | 9, 2048)
    ref = O.philox((2048, 9, 5, 7), (seed & 0xFFFFFFFF, seed >> 32))
    assert got == ref


def test_select_trial_semantics():
    lw = [-3.0, -1.0, -2.0]
    import math
    w = [math.exp(x + 1.0) for x in lw]
    s = sum(w)
    assert O.select_trial(lw, 0.0) == 0
    assert O.select_trial(lw, (w[0] + 0.5 * w[1]) / s) == 1
    assert O.select_trial(lw, (w[0] + w[1] + 0.5 * w[2]) / s) == 2
    assert O.select_trial(lw, 0.99999999999) == 2
