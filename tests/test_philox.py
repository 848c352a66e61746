"""Philox4x32-10 known-answer vectors (Random123's published KATs) and the
statistics of the MCMC draws built on it."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import oracle

KAT = [  # counter (4 words), key (2 words), expected output (4 words)
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr, key, want", KAT)
def test_philox_kat(built, ctr, key, want):
    lib = oracle("Ball_1_Stick").lib
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    lib.orc_philox(c, k, out)
    assert list(out) == want


def test_mcmc_draw_statistics(built):
    lib = oracle("Ball_1_Stick").lib
    n = 200_000
    z = np.zeros(n, dtype=np.float32)
    u = np.zeros(n, dtype=np.float32)
    lib.orc_mcmc_draws(C.c_uint64(8219), C.c_uint32(7), C.c_uint32(n),
                       z.ctypes.data_as(C.c_void_p), u.ctypes.data_as(C.c_void_p))
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01
    assert abs(np.mean(z ** 4) - 3) < 0.05
    assert u.min() > 0 and u.max() <= 1 and abs(u.mean() - 0.5) < 0.005
