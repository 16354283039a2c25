"""The C-ABI library loads and exports every symbol include/*.h declares;
host-side entry points work without a GPU.  CPU only."""
import ctypes
import glob
import math
import os
import platform
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import gpvmc_gb300
    from gpvmc_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    return gpvmc_gb300.lib()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(gv_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_version_and_status(lib):
    assert b"sm_103a" in lib.gv_version()
    for s in range(10):
        assert lib.gv_status_string(s)


def test_invalid_arguments_are_rejected(lib):
    from gpvmc_gb300 import _lib
    cfg = _lib.JobConfig()
    cfg.L, cfg.n_walkers, cfg.precision = 7, 1, 0
    h = ctypes.c_void_p()
    assert lib.gv_job_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.GV_OK + 1
    assert lib.gv_job_create(None, ctypes.byref(h)) == 1
    # an unknown channel, and the longitudinal exciton beyond L = 24: rejected before any device call
    cfg.L, cfg.channel = 8, 3
    assert lib.gv_job_create(ctypes.byref(cfg), ctypes.byref(h)) == 1 and not h.value
    cfg.L, cfg.channel = 26, 2
    assert lib.gv_job_create(ctypes.byref(cfg), ctypes.byref(h)) == 1 and not h.value
    cfg.L = 16
    assert lib.gv_job_footprint(ctypes.byref(cfg), ctypes.byref(out := ctypes.c_uint64())) == 0
    assert out.value > 2 * 128 * 256 * 16                      # the overlap tables R per walker
    cfg.channel = 0
    out = ctypes.c_uint64()
    cfg.L = 16
    cfg.n_walkers = 2048
    assert lib.gv_job_footprint(ctypes.byref(cfg), ctypes.byref(out)) == 0
    assert out.value > 2048 * 2 * 128 * 128 * 16
    # checkpoint entry points reject a missing job or buffer before touching the device
    assert lib.gv_job_checkpoint_size(None, 0, ctypes.byref(out)) == 1
    assert lib.gv_job_checkpoint(None, 0, None, 0, None) == 1
    buf = (ctypes.c_char * 64)()
    assert lib.gv_job_restore(None, buf, 64) == 1


@pytest.mark.parametrize("name,L", [("phi_L4.npz", 4), ("phi_L6.npz", 6), ("phi_L8.npz", 8)])
def test_host_phi_table_matches_reference(lib, name, L):
    g = np.load(os.path.join(ROOT, "tests", "golden", name))
    bc = (ctypes.c_double * 2)(*g["bc"])
    for fl in (0, 1):
        out = np.zeros(2 * L ** 4)
        st = lib.gv_phi_table(L, float(g["phi"]), float(g["neel"]), float(g["neel_exp"]), bc, fl,
                              out.ctypes.data_as(ctypes.c_void_p))
        assert st == 0
        t = (out[0::2] + 1j * out[1::2]).reshape(L * L, L * L)[: g["phi%d" % fl].shape[0]]
        if platform.machine() in ("x86_64", "AMD64"):   # the fixtures' architecture: bit-exact
            np.testing.assert_array_equal(t, g["phi%d" % fl])
        else:                                            # other libm: last-bit differences
            np.testing.assert_allclose(t, g["phi%d" % fl], rtol=0, atol=1e-14)
    nbr = np.zeros(4 * L * L, dtype=np.int32)
    assert lib.gv_lattice_neighbours(L, nbr.ctypes.data_as(ctypes.c_void_p)) == 0
    np.testing.assert_array_equal(nbr.reshape(-1, 4), g["nbr"])
    orb = np.zeros(L * L // 2, dtype=np.int32)
    q = (ctypes.c_int32 * 2)(0, 0)
    N, Nexc = ctypes.c_int32(), ctypes.c_int32()
    assert lib.gv_channel_orbitals(L, bc, 0, q, 0, orb.ctypes.data_as(ctypes.c_void_p), ctypes.byref(N),
                                   ctypes.byref(Nexc)) == 0
    np.testing.assert_array_equal(orb, g["orb0"])


def test_python_api_lattice():
    import gpvmc_gb300 as g
    lat = g.SquareLattice(8)
    gold = np.load(os.path.join(ROOT, "tests", "golden", "phi_L8.npz"))
    np.testing.assert_array_equal(lat.neighbours, gold["nbr"])
    assert len(lat.edges) == 2 * 64
    assert g.pi_phi(0.25) == 0.25 * math.pi


def test_noalloc_rejects_bad_pointers_before_any_launch(lib):
    """gv_slater_invert_noalloc checks sizes and alignment on the host, before
    it touches the device (these calls run without a GPU)."""
    P = ctypes.c_void_p
    assert lib.gv_slater_invert_noalloc(P(0x10000), P(0x20000), 4, P(0x30004), None) == 1   # d_info: 4-byte aligned
    assert lib.gv_slater_invert_noalloc(P(0x10008), P(0x20000), 4, P(0x30000), None) == 1   # d_A: 8-byte aligned
    assert lib.gv_slater_invert_noalloc(P(0x10000), P(0x20008), 4, P(0x30000), None) == 1   # d_Ai: 8-byte aligned
    assert lib.gv_slater_invert_noalloc(None, P(0x20000), 4, P(0x30000), None) == 1
    assert lib.gv_slater_invert_noalloc(P(0x10000), P(0x20000), 129, P(0x30000), None) == 10
    assert lib.gv_slater_invert_noalloc(P(0x10000), P(0x20000), 0, P(0x30000), None) == 10


@pytest.mark.parametrize("L,q", [(4, (2, 0)), (4, (0, 0)), (8, (4, 4)), (8, (2, 2)), (16, (8, 8))])
def test_long_exciton_state_table(lib, L, q):
    """StagFluxLongExciton.cpp:6-66: states 2fe / 2fe + 1 put the pair (2fe + 1,
    hole at k - q) into flavour 0 / 1, the ground state is added at q = 0 and
    (pi, pi); every hole is a lower-band orbital, each once per flavour, and the
    pair carries momentum q up to the (pi, pi) fold."""
    bc = (ctypes.c_double * 2)(1.0, 1.0)
    qq = (ctypes.c_int32 * 2)(*q)
    Ns = L * L
    N, K = ctypes.c_int32(), ctypes.c_int32()
    orb = np.zeros(Ns, dtype=np.int32)
    assert lib.gv_channel_orbitals(L, bc, 2, qq, 0, orb.ctypes.data_as(ctypes.c_void_p), ctypes.byref(N),
                                   ctypes.byref(K)) == 0
    extra = q in ((0, 0), (L // 2, L // 2))
    assert N.value == Ns // 2 and K.value == Ns + (1 if extra else 0)
    up = np.zeros(K.value, dtype=np.int32)
    dn = np.zeros(K.value, dtype=np.int32)
    assert lib.gv_channel_states(L, bc, 2, qq, up.ctypes.data_as(ctypes.c_void_p),
                                 dn.ctypes.data_as(ctypes.c_void_p)) == 0
    fe = np.arange(Ns // 2)
    assert (up[0:Ns:2] == 2 * fe + 1).all() and (up[1:Ns:2] == 2 * fe + 1).all()
    assert (dn[0:Ns:2] == dn[1:Ns:2]).all() and (dn[:Ns] % 2 == 0).all()
    assert sorted(dn[0:Ns:2].tolist()) == list(range(0, Ns, 2))
    if extra:
        assert up[Ns] == -1 and dn[Ns] == -1
    qn = np.zeros(3 * Ns, dtype=np.int32)
    assert lib.gv_fock_quantum_numbers(L, bc, qn.ctypes.data_as(ctypes.c_void_p)) == 0
    qn = qn.reshape(Ns, 3)
    for k in range(0, Ns, 2):
        d = (qn[up[k], :2] - qn[dn[k], :2] - np.array(q)) % L
        assert tuple(d) in ((0, 0), (L // 2, L // 2))
