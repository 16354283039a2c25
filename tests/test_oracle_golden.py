"""The oracle restatement against golden fixtures produced by the reference
itself (tests/golden/make_golden.py).  CPU only."""
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PHI = 0.25 * math.pi


def load(name):
    return np.load(os.path.join(GOLD, name))


def same_trace(t, g):
    assert (t["v1"] == g["v1"]).all() and (t["v2"] == g["v2"]).all()
    assert (t["kind"] == g["kind"]).all() and (t["accepted"] == g["accepted"]).all()
    assert (t["u"][:, 3] == g["u4"]).all()
    real = t["kind"] == 1
    err = np.abs(t["ratio"][real] - g["ratio"][real])
    assert (err <= 1e-12 * np.abs(g["ratio"][real]) + 1e-15).all()


@pytest.mark.parametrize("L", [4, 6, 8])
def test_phi_tables(oracle, L):
    g = load("phi_L%d.npz" % L)
    o = oracle.OracleChain(L, float(g["phi"]), float(g["neel"]), neel_exp=float(g["neel_exp"]), bc=tuple(g["bc"]))
    for fl in (0, 1):
        t = o.phi_table(fl)[: g["phi%d" % fl].shape[0]]
        np.testing.assert_array_equal(t, g["phi%d" % fl])
    np.testing.assert_array_equal(o.neighbours(), g["nbr"])
    np.testing.assert_array_equal(o.orbitals(0), g["orb0"])


def test_groundstate_trace(oracle):
    g = load("gs_L8_trace.npz")
    o = oracle.OracleChain(8, PHI, 0.1, seed=1234, walker=0)
    assert o.random_start() == 0
    np.testing.assert_array_equal(o.config(), g["start"])
    m, e = o.amp()
    assert e == int(g["amp0"][2]) and abs(m - complex(g["amp0"][0], g["amp0"][1])) < 1e-12 * abs(m)
    np.testing.assert_allclose(o.inverse(0), g["inv0_up"], rtol=0, atol=1e-12 * np.abs(g["inv0_up"]).max())
    same_trace(o.walk(4000, trace=True), g)
    np.testing.assert_array_equal(o.config(), g["final"])
    m, e = o.amp()
    assert e == int(g["amp"][2]) and abs(m - complex(g["amp"][0], g["amp"][1])) < 1e-11 * abs(m)
    np.testing.assert_allclose(o.inverse(0), g["inv_up"], rtol=0, atol=1e-11 * np.abs(g["inv_up"]).max())


def test_groundstate_measurements(oracle):
    g = load("gs_meas.npz")
    o = oracle.OracleChain(8, PHI, 0.1, seed=5, walker=0)
    o.random_start()
    o.walk(200 * 64)
    o.walk(64 * 30, meas=64, mask=oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN)
    pj, n = o.projheis()
    assert n == int(g["n8"]) == 30
    np.testing.assert_allclose(pj, g["pj8"], rtol=1e-12, atol=1e-13)
    assert abs(o.stagmagn()[0] - g["sm8"]) < 1e-12
    np.testing.assert_array_equal(o.config(), g["final8"])
    o4 = oracle.OracleChain(4, PHI, 0.1, seed=int(g["seed4"]), walker=2)
    o4.random_start()
    o4.walk(200 * 16)
    o4.walk(16 * 40, meas=16, mask=7)
    np.testing.assert_allclose(o4.projheis()[0], g["pj4"], rtol=1e-12, atol=1e-13)
    ss, n4 = o4.statspin()
    assert n4 == int(g["n4"])
    np.testing.assert_allclose(ss, g["ss4"], rtol=1e-12, atol=1e-12)


def test_reinversion_trace(oracle):
    g = load("gs_L8_reinv.npz")
    o = oracle.OracleChain(8, PHI, 0.1, seed=11, walker=0)
    o.random_start()
    same_trace(o.walk(3000, reinv_every=64, trace=True), g)
    np.testing.assert_array_equal(o.config(), g["final"])
    assert o.counts()[3] == int(g["reinv"]) > 0


@pytest.mark.parametrize("L,steps", [(4, 2000), (8, 1500)])
def test_trans_exciton(oracle, L, steps):
    g = load("trans_L%d.npz" % L)
    o = oracle.OracleChain(L, PHI, 0.1, channel=oracle.TRANS, q=tuple(g["q"]), seed=7, walker=3)
    assert o.random_start() == 0
    assert o.current_state() == int(g["state0"])
    same_trace(o.walk(steps, trace=True), g)
    o.walk(L * L * 6, meas=L * L, mask=oracle.MEAS_PROJHEIS)
    pj, n = o.projheis()
    assert n == int(g["n"]) and o.current_state() == int(g["state"])
    np.testing.assert_allclose(pj, g["pj"], rtol=1e-11, atol=1e-11 * np.abs(g["pj"]).max())
    np.testing.assert_array_equal(o.config(), g["final"])


def test_virt_update(oracle):
    g = load("gs_L8_virt.npz")
    o = oracle.OracleChain(8, PHI, 0.1, seed=3, walker=0)
    o.random_start()
    np.testing.assert_array_equal(o.config(), g["config"])
    qm, qe = o.virt_update(g["hops"])
    np.testing.assert_array_equal(qe, g["qe"])
    np.testing.assert_allclose(qm, g["qm"], rtol=1e-12, atol=1e-12)
