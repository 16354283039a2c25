"""GPU engine vs the oracle on the same seeded inputs (through the C ABI).

Bar: bit-exact configurations, proposals and accept decisions (except
near-ties |u4 - ratio| < 1e-9, flagged), Metropolis ratios and amplitudes to
1e-10 relative, quantity sums to 1e-10 relative, in the plain FP64 form.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi
RTOL = 1e-10


def _pair(engine, oracle, L, neel, seed=1234, walkers=1, reinv=0, precision="fp64", walker=0):
    job = engine.Job(engine.StagFluxGroundState(L, PHI, neel), walkers=walkers, seed=seed,
                     precision=precision, reinv_every=reinv)
    orc = oracle.OracleChain(L, PHI, neel, seed=seed, walker=walker)
    return job, orc


def exact_ratio(fresh_chain, i, v1, v2):
    """The Metropolis ratio of step i from a freshly inverted FP64 state: a new
    oracle chain replayed to step i and re-inverted from its configuration
    (SlaterDeterminant::Init), then VirtUpdate of the exchange v1 <-> v2 and of
    no move: sum_k |q_k(moved)|^2 / sum_k |q_k(current)|^2 over the channel
    states (one state for the ground state)."""
    o = fresh_chain()
    if i:
        o.walk(i)
    assert o.reinit() == 0
    up = o.config().astype(bool)
    u, d = (v1, v2) if up[v1] else (v2, v1)
    qm, qe = o.virt_update(np.array([(u, d, d, u), (-1, -1, -1, -1)], dtype=np.int32))
    top = int(qe.max())
    w = (np.abs(qm) ** 2 * 100.0 ** (qe - top).astype(float)).sum(axis=0)
    return float(w[0] / w[1])


def check_ratios(tg, to, fresh_chain=None):
    """Ratios to 1e-10 relative (absolute floor 1e-13: ratios that vanish by
    symmetry are rounding noise in both codes).  Where the engine and the
    oracle differ by more, both running inverses carry the FP64
    Sherman-Morrison drift of their own rounding (at L = 16 the oracle's
    running inverse sits up to ~5e-11 relative from a fresh inversion after a
    few hundred accepted moves); the engine's ratio must then be no further
    from the exact one -- the same step from a freshly inverted state -- than
    the oracle's, up to 1e-10 relative."""
    real = np.flatnonzero(to["kind"] == 1)
    err = np.abs(tg["ratio"][real] - to["ratio"][real])
    bad = real[err > RTOL * np.abs(to["ratio"][real]) + 1e-13]
    if len(bad) and fresh_chain is not None:
        keep = []
        for i in bad[:20]:
            ex = exact_ratio(fresh_chain, int(i), int(to["v1"][i]), int(to["v2"][i]))
            if abs(tg["ratio"][i] - ex) > abs(to["ratio"][i] - ex) + RTOL * abs(ex) + 1e-13:
                keep.append(i)
        bad = np.array(keep + list(bad[20:]), dtype=np.int64)
    assert not len(bad), (bad[:5], to["ratio"][bad][:5], tg["ratio"][bad][:5])


def _compare_traces(tg, to, fresh_chain=None):
    assert (tg["v1"] == to["v1"]).all()
    assert (tg["v2"] == to["v2"]).all()
    assert (tg["kind"] == to["kind"]).all()
    tie = np.abs(to["u"][:, 3] - to["ratio"]) < 1e-9
    assert ((tg["accepted"] == to["accepted"]) | tie).all()
    check_ratios(tg, to, fresh_chain)
    assert (tg["u4"] == to["u"][:, 3]).all()
    return int(tie.sum())


@pytest.mark.parametrize("L,neel", [(4, 0.1), (8, 0.1), (12, 0.05), (16, 0.1)])
def test_start_and_inverse(engine, oracle, L, neel):
    job, orc = _pair(engine, oracle, L, neel)
    job.init_walkers()
    assert orc.random_start() == 0
    assert (job.config()[0] == orc.config()).all()
    m, e = job.amplitude()
    om, oe = orc.amp()
    a, b = m[0] * 10.0 ** (e[0] - oe), om
    assert abs(a - b) < RTOL * abs(b)
    for fl in (0, 1):
        gi, oi = job.inverse(0, fl), orc.inverse(fl)
        assert np.abs(gi - oi).max() < RTOL * np.abs(oi).max()


@pytest.mark.parametrize("L,neel,steps", [(4, 0.1, 3000), (8, 0.1, 6000), (12, 0.05, 4000), (16, 0.1, 3000)])
def test_trace_parity(engine, oracle, L, neel, steps):
    job, orc = _pair(engine, oracle, L, neel, seed=77)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(steps, 0)
    to = orc.walk(steps, trace=True)

    def fresh():
        o = oracle.OracleChain(L, PHI, neel, seed=77, walker=0)
        o.random_start()
        return o
    _compare_traces(tg, to, fresh)
    assert (job.config()[0] == orc.config()).all()
    m, e = job.amplitude()
    om, oe = orc.amp()
    assert abs(m[0] * 10.0 ** (e[0] - oe) - om) < 1e-9 * abs(om)
    for fl in (0, 1):
        gi, oi = job.inverse(0, fl), orc.inverse(fl)
        assert np.abs(gi - oi).max() < 1e-9 * np.abs(oi).max()
    c = job.counts()[0]
    assert c[0] == steps and c[1] == int((to["accepted"] & (to["kind"] == 1)).sum())


@pytest.mark.parametrize("L,therm,nmeas", [(8, 200, 30), (16, 20, 6)])
def test_measurements_parity(engine, oracle, L, therm, nmeas):
    """ProjHeis, StagMagnZ and StatSpinStruct sums over `nmeas` measured sweeps
    after `therm` sweeps of thermalisation; L = 16 is the headline lattice
    (N = 128 per flavour)."""
    neel = 0.1
    job, orc = _pair(engine, oracle, L, neel, seed=5)
    job.set_measurements(7)
    job.init_walkers()
    orc.random_start()
    job.walk(therm * L * L, 0)
    orc.walk(therm * L * L)
    tg = job.walk_traced(L * L * nmeas, L * L)
    to = orc.walk(L * L * nmeas, meas=L * L, mask=7, trace=True)

    def fresh():
        o = oracle.OracleChain(L, PHI, neel, seed=5, walker=0)
        o.random_start()
        o.walk(therm * L * L)
        return o
    _compare_traces(tg, to, fresh)
    assert (job.config()[0] == orc.config()).all()
    pj, n = job.projheis()
    opj, on = orc.projheis()
    assert n[0] == on == nmeas
    assert abs(pj[0, 0] - opj[0, 0]) < RTOL * abs(opj[0, 0])
    assert pj[0, 1].real == opj[1, 0].real
    sm, sn = job.stagmagn()
    osm, osn = orc.stagmagn()
    assert sn[0] == osn and abs(sm[0] - osm) < 1e-12 * max(1.0, abs(osm))
    ss, ssn = job.statspin()
    oss, ossn = orc.statspin()
    assert ssn == ossn == nmeas
    assert np.abs(ss - oss).max() < RTOL * np.abs(oss).max()


def test_reinversion_cadence(engine, oracle):
    """Config-1 form: FP64 re-inversion after every L^2 accepted exchanges."""
    L, neel = 8, 0.1
    job, orc = _pair(engine, oracle, L, neel, seed=11, reinv=L * L)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(8000, 0)
    to = orc.walk(8000, reinv_every=L * L, trace=True)
    _compare_traces(tg, to)
    assert job.counts()[0][4] == orc.counts()[3] > 0


def test_batched_walkers_match_single_chains(engine, oracle):
    L, neel, W, steps = 8, 0.1, 16, 1500
    job = engine.Job(engine.StagFluxGroundState(L, PHI, neel), walkers=W, seed=99)
    job.init_walkers()
    job.walk(steps, 0)
    cfg = job.config()
    for w in (0, 5, 15):
        orc = oracle.OracleChain(L, PHI, neel, seed=99, walker=w)
        orc.random_start()
        orc.walk(steps)
        assert (cfg[w] == orc.config()).all()


def test_virt_update_bond_ratios(engine, oracle):
    L, neel = 8, 0.1
    job, orc = _pair(engine, oracle, L, neel, seed=3)
    job.init_walkers()
    orc.random_start()
    up = job.config()[0].astype(bool)
    lat = engine.SquareLattice(L)
    hops = []
    for a, b in lat.edges:
        if up[a] != up[b]:
            u, d = (a, b) if up[a] else (b, a)
            hops.append((u, d, d, u))
    hops.append((5 if up[5] else 6, 9, -1, -1) if False else (-1, -1, -1, -1))
    hops = np.array(hops, dtype=np.int32)
    g = job.virt_update(0, hops)[0]
    qm, qe = orc.virt_update(hops)
    am, ae = orc.amp()
    ref = (qm[0] / am) * 10.0 ** (qe[0] - ae)
    assert np.abs(g - ref).max() < RTOL * np.abs(ref).max()


def test_mixed_precision_tracks_fp64(engine, oracle):
    L, neel, steps = 8, 0.1, 3000
    j64 = engine.Job(engine.StagFluxGroundState(L, PHI, neel), walkers=4, seed=21, precision="fp64")
    j32 = engine.Job(engine.StagFluxGroundState(L, PHI, neel), walkers=4, seed=21, precision="mixed")
    for j in (j64, j32):
        j.init_walkers()
    t64 = j64.walk_traced(steps, 0, walker=1)
    t32 = j32.walk_traced(steps, 0, walker=1)
    # until the chains part at a near-tie, the FP32 ratios follow the FP64 ones
    diff = np.nonzero((t64["accepted"] != t32["accepted"]) | (t64["v1"] != t32["v1"]))[0]
    upto = diff[0] if len(diff) else steps
    real = t64["kind"][:upto] == 1
    a, b = t32["ratio"][:upto][real], t64["ratio"][:upto][real]
    # FP32 dot products of length N: ~1e-6 relative typically, larger where
    # the ratio is small by cancellation (such ratios are rarely accepted)
    rel = np.abs(a - b) / (b + 1e-3)
    assert upto > 200 and np.median(rel) < 1e-5 and rel.max() < 1e-2
    if upto < steps:   # the chains may only part where u4 sits within FP32 error of the ratio
        assert abs(t64["u4"][upto] - t64["ratio"][upto]) < 1e-2 * max(1.0, t64["ratio"][upto])
    d = j32.drift()
    assert d.max() < 1e-3


def test_singular_start_retry_gives_clean_state(engine, oracle):
    """vmc.cpp:230-241 retries singular random starts; the reference's retry
    keeps stale occupancies (State::InitFock never clears m_fock), the engine
    restarts from a clean state and keeps drawing the same Philox stream."""
    L = 4
    seed = next(s for s in range(6, 200)
                if int(_start_config(oracle, L, s).sum()) != L * L // 2)
    job = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=1, seed=seed, walker_base=2)
    job.init_walkers()
    assert int(job.config()[0].sum()) == L * L // 2
    job.walk(500, 0)
    assert int(job.config()[0].sum()) == L * L // 2


def _start_config(oracle, L, seed):
    o = oracle.OracleChain(L, PHI, 0.1, seed=seed, walker=2)
    o.random_start()
    return o.config()


def test_deferred_reinversion_resets_drift(engine):
    """GV_FLAG_REINV_DEFERRED: walkers past reinv_every accepted exchanges are
    re-inverted in one batched launch at the end of the walk call."""
    L = 8
    job = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=8, seed=4, precision="mixed",
                     reinv_every=16, deferred_reinversion=True)
    job.init_walkers()
    job.walk(L * L * 4, 0)
    c = job.counts()
    assert (c[:, 4] >= 1).all() and (c[:, 1] >= 16).all()
    assert job.drift().max() < 1e-4


def test_measure_without_step_matches_oracle(engine, oracle):
    """gv_job_measure (Quantity::measure on the current configuration) equals
    the oracle's ProjHeis/StagMagnZ/StatSpinStruct measure on the same state."""
    L = 8
    job, orc = _pair(engine, oracle, L, 0.1, seed=31)
    job.set_measurements(7)
    job.init_walkers()
    orc.random_start()
    job.walk(500, 0)
    orc.walk(500)
    assert (job.config()[0] == orc.config()).all()
    job.reset_quantities()
    job.measure()
    orc.reset_quantities()
    orc.measure(7)
    pj, n = job.projheis()
    opj, on = orc.projheis()
    assert n[0] == on == 1 and abs(pj[0, 0] - opj[0, 0]) < RTOL * abs(opj[0, 0])
    assert abs(job.stagmagn()[0][0] - orc.stagmagn()[0]) < 1e-12
    ss, _ = job.statspin()
    oss, _ = orc.statspin()
    assert np.abs(ss - oss).max() < RTOL * np.abs(oss).max()


def test_drift_checked_reinversion(engine):
    L = 8
    job = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=16, seed=8, precision="mixed",
                     reinv_every=16, drift_threshold=1e-6)
    job.init_walkers()
    for _ in range(6):
        job.walk(L * L, 0)
    drift, checks = job.drift_checks()
    c = job.counts()
    assert (c[:, 4] + checks).min() >= 1          # every walker was checked at least once
    assert job.drift().max() < 1e-3


@pytest.mark.parametrize("L,steps", [(8, 6000), (16, 3000)])
def test_delayed_updates_fp64_parity(engine, oracle, L, steps):
    """Delayed rank-8 updates (GV_FLAG_DELAYED_UPDATES) walk the same chain as
    the immediate Sherman-Morrison: in FP64 the oracle's decisions and ratios
    to 1e-10 hold across many write-backs of the pending pairs."""
    job = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=2, seed=123, delayed_updates=True)
    orc = oracle.OracleChain(L, PHI, 0.1, seed=123, walker=1)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(steps, 0, walker=1)
    to = orc.walk(steps, trace=True)
    _compare_traces(tg, to)
    assert job.counts()[1][1] > 16
    for fl in (0, 1):
        gi, oi = job.inverse(1, fl), orc.inverse(fl)
        assert np.abs(gi - oi).max() < 1e-9 * np.abs(oi).max()


def test_delayed_updates_mixed_with_measurements(engine):
    """Mixed engine with delayed updates: ProjHeis on its own inverses equals
    the FP64 engine's on fresh inverses of the same configurations."""
    L = 16
    kw = dict(walkers=32, seed=5)
    a = engine.Job(engine.StagFluxGroundState(L, PHI, 0.05), precision="mixed", delayed_updates=True, **kw)
    a.set_measurements(3)
    a.init_walkers()
    a.walk(L * L * 6, L * L)
    assert a.drift().max() < 1e-3
    pj, n = a.projheis()
    assert (n == 6).all() and np.isfinite(pj).all()
    a.reset_quantities()
    a.measure()
    b = engine.Job(engine.StagFluxGroundState(L, PHI, 0.05), precision="fp64", **kw)
    b.set_measurements(1)
    b.init_walkers(a.config())
    b.measure()
    ea = a.projheis()[0][:, 0].real
    eb = b.projheis()[0][:, 0].real
    assert np.abs(ea - eb).max() < 1e-4
