"""Philox4x32-10 known-answer vectors (Salmon et al., SC'11; Random123
kat_vectors) for the oracle's and the engine's host implementation, and the
uniform mapping."""
import ctypes

import numpy as np

KAT = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
       ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
       ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]


def _run(fn, ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    fn(c, k, o)
    return tuple(o)


def test_oracle_kat(oracle):
    lib = oracle._load(oracle.ORACLE_SO, "orc")
    for ctr, key, want in KAT:
        assert _run(lib.orc_philox4x32_10, ctr, key) == want


def test_engine_kat_and_stream_agree_with_oracle(oracle):
    import gpvmc_gb300
    from gpvmc_gb300 import build as b
    import os
    if not os.path.exists(b.LIB):
        b.build()
    L = gpvmc_gb300.lib()
    for ctr, key, want in KAT:
        assert _run(L.gv_philox4x32_10, ctr, key) == want
    for seed, w, s in [(1234, 0, 0), (2 ** 40 + 7, 513, 1), (99, 3, 2)]:
        for k in (0, 1, 2, 3, 1001, 2 ** 33 + 5):
            u = L.gv_uniform_at(seed, w, s, k)
            assert u == oracle.uniform_at(seed, w, s, k)
            assert 0.0 < u < 1.0


def test_uniform_extremes(oracle):
    lib = oracle._load(oracle.ORACLE_SO, "orc")
    lib.orc_u01.restype = ctypes.c_double
    lib.orc_u01.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    assert lib.orc_u01(0, 0) == 2.0 ** -53
    assert lib.orc_u01(0xffffffff, 0xffffffff) == 1.0 - 2.0 ** -53
    # int(Ns * u) < Ns for the largest uniform at every lattice size on the path
    umax = 1.0 - 2.0 ** -53
    for L in range(4, 40, 2):
        assert int(np.float64(L * L) * umax) == L * L - 1
