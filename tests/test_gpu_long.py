"""GPU engine vs the oracle in the longitudinal-exciton channel
(StagFluxLongExciton, StagFluxLongExciton.cpp:6-66): states two orbital hops
apart in one flavour, the rank-2 row branches of linalg::DetUpdate / InvUpdate.

Bar, plain FP64 form (as the transverse channel's, test_gpu_trans): identical
start configuration, proposals and accept decisions (except flagged
near-ties), Metropolis ratios to 1e-10 (or no further than the oracle from a
freshly inverted state, test_gpu_parity.check_ratios), VirtUpdate amplitudes
of every state to 1e-9, H / O sums to 1e-9 of their largest entry; the
channel state is compared up to states of equal weight.  The engine's trace
is also compared with the reference build's own trace in the golden fixtures.
The mixed form is compared with the FP64 form.
"""
import math
import os

import numpy as np
import pytest
from test_gpu_parity import check_ratios
from test_gpu_trans import _compare_traces, _log10_weights, _state_amps

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = [(4, (2, 0), 7, 3), (4, (0, 0), 5, 3), (6, (2, 2), 2, 3), (8, (4, 4), 3, 3), (8, (2, 0), 1, 3)]


def _pair(engine, oracle, L, q, seed, walker, precision="fp64", reinv=0, walkers=1):
    wav = engine.StagFluxLongExciton(L, PHI, 0.1, q=q)
    job = engine.Job(wav, walkers=walkers, seed=seed, precision=precision, reinv_every=reinv, walker_base=walker)
    orc = oracle.OracleChain(L, PHI, 0.1, channel=oracle.LONG, q=q, seed=seed, walker=walker)
    return job, orc


def _check_state(job, orc, walker=0, rtol=1e-9):
    """The engine's current state ties the oracle's in weight, Amp() of the
    engine's state equals the oracle's amplitude of that state, and the
    stepper weight sum_k |q_k|^2 equals the oracle's."""
    kg, ko = int(job.state_index()[walker]), orc.current_state()
    qm, qe = _state_amps(orc)
    lw = _log10_weights(qm, qe)
    assert abs(lw[kg] - lw[ko]) < rtol, (kg, ko, lw[kg], lw[ko])
    m, e = job.amplitude()
    a = m[walker] * 10.0 ** float(e[walker] - qe[kg])
    assert abs(abs(a) - abs(qm[kg])) < rtol * abs(qm[kg])
    wm, we = orc.weight()
    wg = job.weight()[walker] * abs(m[walker]) ** 2 * 10.0 ** float(2 * e[walker] - we)
    assert abs(wg - wm) < rtol * wm, (wg, wm)
    return kg == ko


@pytest.mark.parametrize("L,q,seed,walker", CASES)
def test_long_start(engine, oracle, L, q, seed, walker):
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    assert job.Nexc == L * L + (1 if q in ((0, 0), (L // 2, L // 2)) else 0)
    assert job.N == (L * L // 2, L * L // 2)
    job.init_walkers()
    assert orc.random_start() == 0
    assert (job.config()[0] == orc.config()).all()
    if _check_state(job, orc):
        m, e = job.amplitude()
        om, oe = orc.amp()
        assert abs(m[0] * 10.0 ** float(e[0] - oe) - om) < 1e-10 * abs(om)
        for fl in (0, 1):
            gi, oi = job.inverse(0, fl), orc.inverse(fl)
            assert np.abs(gi - oi).max() < 1e-10 * np.abs(oi).max()
    assert job.drift().max() < 1e-12


@pytest.mark.parametrize("L,q,seed,walker", CASES)
def test_long_virt_update(engine, oracle, L, q, seed, walker):
    """Every state's amplitude after each antiparallel bond exchange and after
    no move, relative to Amp(): magnitudes always, values (hop signs
    included) where both codes hold the same state."""
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.init_walkers()
    orc.random_start()
    job.walk(L * L * 2, 0)
    orc.walk(L * L * 2)
    assert (job.config()[0] == orc.config()).all()
    up = orc.config().astype(bool)
    hops = [(-1, -1, -1, -1)]
    for x in range(L):
        for y in range(L):
            a = y * L + x
            for b in (((y + 1) % L) * L + x, y * L + (x + 1) % L):
                if up[a] != up[b]:
                    u, d = (a, b) if up[a] else (b, a)
                    hops.append((u, d, d, u))
    hops = np.array(hops, dtype=np.int32)
    qg = job.virt_update(0, hops)                  # (Nexc, nset), relative to the engine's Amp()
    qm, qe = orc.virt_update(hops)
    am, ae = orc.amp()
    qo = qm * 10.0 ** (qe - ae).astype(float) / am  # relative to the oracle's Amp()
    m, e = job.amplitude()
    scale = np.abs(qo).max()
    same = job.state_index()[0] == orc.current_state()
    if same:
        qg = qg * (m[0] * 10.0 ** float(e[0] - ae) / am)
        assert np.abs(qg - qo).max() < 1e-9 * scale
    else:   # tied states: |Amp| equal, so magnitudes relative to Amp() agree
        assert np.abs(np.abs(qg) - np.abs(qo)).max() < 1e-9 * scale


@pytest.mark.parametrize("L,q,seed,walker,steps", [(4, (2, 0), 7, 3, 1500), (4, (0, 0), 5, 3, 1500),
                                                   (6, (2, 2), 2, 3, 1000), (8, (4, 4), 3, 3, 800),
                                                   (8, (2, 0), 1, 3, 800)])
def test_long_trace_parity(engine, oracle, L, q, seed, walker, steps):
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(steps, 0)
    to = orc.walk(steps, trace=True)
    orc2 = oracle.OracleChain(L, PHI, 0.1, channel=oracle.LONG, q=q, seed=seed, walker=walker)
    orc2.random_start()

    def fresh():
        o = oracle.OracleChain(L, PHI, 0.1, channel=oracle.LONG, q=q, seed=seed, walker=walker)
        o.random_start()
        return o
    ties = _compare_traces(orc2, tg, to, fresh)
    assert (job.config()[0] == orc.config()).all()
    if _check_state(job, orc) and ties == 0:
        for fl in (0, 1):
            gi, oi = job.inverse(0, fl), orc.inverse(fl)
            assert np.abs(gi - oi).max() < 1e-9 * np.abs(oi).max()
    assert job.drift().max() < 1e-10
    c = job.counts()[0]
    assert c[0] == steps and c[1] == int((to["accepted"] & (to["kind"] == 1)).sum())


@pytest.mark.parametrize("name,steps", [("long_L4_q20.npz", 1500), ("long_L4_q00.npz", 1500)])
def test_long_matches_reference_fixture(engine, name, steps):
    """The engine against the reference build's own run (tests/golden,
    generated by tests/golden/make_golden.py from the reference compiled with
    its shims): proposals, decisions and ratios over 1500 steps, then the
    ProjHeis H / O sums of six measured sweeps and the final configuration
    (1e-9: the fixtures are x86_64 libm tables, the engine's host tables use
    this machine's libm)."""
    g = np.load(os.path.join(GOLD, name))
    L = 4
    job = engine.Job(engine.StagFluxLongExciton(L, PHI, 0.1, q=tuple(g["q"])), walkers=1, seed=7, walker_base=3)
    job.init_walkers()
    tg = job.walk_traced(steps, 0)
    n = len(g["v1"])
    assert (tg["v1"] == g["v1"]).all() and (tg["v2"] == g["v2"]).all()
    assert (tg["kind"] == g["kind"]).all()
    tie = np.abs(g["u4"] - g["ratio"]) < 1e-9
    assert ((tg["accepted"] == g["accepted"]) | tie).all()
    assert steps == n
    if not tie.any():
        real = g["kind"] == 1
        err = np.abs(tg["ratio"][real] - g["ratio"][real])
        assert (err <= 1e-9 * np.abs(g["ratio"][real]) + 1e-13).all()
        # then six measured sweeps: the reference's ProjHeis H / O sums and final configuration
        job.set_measurements(1)
        job.walk(L * L * 6, L * L)
        pj, nm = job.projheis()
        assert nm[0] == int(g["n"])
        assert (job.config()[0] == g["final"]).all()
        assert np.abs(pj[0] - g["pj"]).max() < 1e-9 * np.abs(g["pj"]).max()


@pytest.mark.parametrize("L,q,seed,walker", [(4, (2, 0), 7, 3), (6, (2, 2), 2, 3), (8, (4, 4), 3, 3)])
def test_long_measurements(engine, oracle, L, q, seed, walker):
    """ProjHeis H and O (ProjHeis.cpp:40-158) and StagMagnZ over measured
    sweeps; StatSpinStruct (swaps within the current state,
    StatSpinStruct.cpp:74) where both codes hold the same state."""
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN | oracle.MEAS_STATSPIN
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.set_measurements(mask)
    job.init_walkers()
    orc.random_start()
    job.walk(L * L * 4, 0)
    orc.walk(L * L * 4)
    job.walk(L * L * 5, L * L)
    orc.walk(L * L * 5, meas=L * L, mask=mask)
    assert (job.config()[0] == orc.config()).all()
    pg, ng = job.projheis()
    po, no = orc.projheis()
    assert ng[0] == no == 5
    assert np.abs(pg[0] - po).max() < 1e-9 * np.abs(po).max()
    sg, nsg = job.stagmagn()
    so, nso = orc.stagmagn()
    assert nsg[0] == nso and abs(sg[0] - so) < 1e-12
    if job.state_index()[0] == orc.current_state():
        job.reset_quantities()
        job.set_measurements(oracle.MEAS_STATSPIN)
        job.measure()
        orc.reset_quantities()
        orc.measure(oracle.MEAS_STATSPIN)
        ssg, _ = job.statspin()
        sso, _ = orc.statspin()
        assert np.abs(ssg - sso).max() < 1e-9 * max(1.0, np.abs(sso).max())


def test_long_reinversion_cadence(engine, oracle):
    L, q, seed, walker = 6, (2, 2), 4, 3
    job, orc = _pair(engine, oracle, L, q, seed, walker, reinv=L * L)
    job.init_walkers()
    assert orc.random_start() == 0
    tg = job.walk_traced(2000, 0)
    to = orc.walk(2000, reinv_every=L * L, trace=True)
    orc2 = oracle.OracleChain(L, PHI, 0.1, channel=oracle.LONG, q=q, seed=seed, walker=walker)
    orc2.random_start()
    _compare_traces(orc2, tg, to)
    assert (job.config()[0] == orc.config()).all()
    assert job.counts()[0][4] == orc.counts()[3] > 0
    _check_state(job, orc)


@pytest.mark.parametrize("L,q", [(8, (4, 4)), (16, (8, 8))])
def test_long_mixed_vs_fp64(engine, L, q):
    """Mixed-precision walk (FP32 inverses and overlap tables, drift-checked
    FP64 re-inversion) against FP64 on the same configurations: H and O
    depend on the configuration only."""
    W = 32 if L == 8 else 16
    wav = engine.StagFluxLongExciton(L, PHI, 0.1, q=q)
    mixed = engine.Job(wav, walkers=W, seed=21, precision="mixed", reinv_every=L * L, drift_threshold=1e-5)
    mixed.set_measurements(1)
    mixed.init_walkers()
    mixed.walk(L * L * 6, 0)
    assert (mixed.status() == 0).all()
    cfg = mixed.config()
    mixed.reset_quantities()
    mixed.measure()
    pm, _ = mixed.projheis()
    ref = engine.Job(wav, walkers=W, seed=21, precision="fp64")
    ref.set_measurements(1)
    ref.init_walkers(cfg)
    ref.reset_quantities()
    ref.measure()
    pr, _ = ref.projheis()
    err = np.abs(pm - pr).max(axis=(1, 2)) / np.abs(pr).max(axis=(1, 2))
    print("long exciton H/O error vs FP64: median %.2e max %.2e" % (np.median(err), err.max()))
    assert np.median(err) < 1e-4 and err.max() < 1e-2
    assert mixed.drift().max() < 1e-3


@pytest.mark.parametrize("L,q", [(4, (2, 2)), (8, (4, 4)), (12, (6, 6)), (12, (0, 0)), (16, (8, 8)), (16, (0, 0))])
def test_long_overlap_sums_on_tensor_cores(engine, L, q):
    """Longitudinal ProjHeis with the bonds' overlap sums Z_b = R^T C_b from
    split-TF32 tensor-core products (k_long_z_tc) against the FP32 CUDA-core
    sums (scalar_pairs) on the same FP32 state, and against the FP64 engine on
    the same configurations (H and O depend on the configuration only)."""
    W = 12
    wav = engine.StagFluxLongExciton(L, PHI, 0.1, q=q)
    mk = lambda prec, **kw: engine.Job(wav, walkers=W, seed=23, precision=prec, reinv_every=L * L,
                                       deferred_reinversion=True, **kw)
    j0 = mk("mixed")
    j0.set_measurements(1)
    j0.init_walkers()
    j0.walk(L * L * 3, 0)
    assert (j0.status() == 0).all()
    cfg = j0.config()
    j0.close()
    out = []
    for j in (mk("mixed"), mk("mixed", scalar_pairs=True), mk("fp64")):
        j.set_measurements(1)
        j.init_walkers(cfg)
        j.reset_quantities()
        j.measure()
        pj, n = j.projheis()
        assert (n == 1).all() and (j.status() == 0).all()
        out.append(pj)
        j.close()
    pt, ps, p64 = out
    scale = np.abs(p64).max(axis=(1, 2))
    e_ts = np.abs(pt - ps).max(axis=(1, 2)) / scale
    e_t64 = np.abs(pt - p64).max(axis=(1, 2)) / scale
    e_s64 = np.abs(ps - p64).max(axis=(1, 2)) / scale
    print("long H/O: tensor vs CUDA cores median %.2e max %.2e; vs FP64 median %.2e max %.2e (CUDA cores %.2e)"
          % (np.median(e_ts), e_ts.max(), np.median(e_t64), e_t64.max(), np.median(e_s64)))
    assert np.median(e_ts) < 2e-5 and e_ts.max() < 1e-3
    assert np.median(e_t64) < 1e-4 and e_t64.max() < 1e-2


def test_long_overlap_sums_bounded_wait(engine):
    """The tensor-core bond sums' mbarrier waits are bounded: with a poll
    budget of zero every wait gives up at once; the walker each CTA was on,
    and those it did not reach, report GV_ERR_TIMEOUT (a host-visible status;
    the MMAs issued finish before the kernel frees its tensor memory) and are
    skipped by the measurement, so no unwritten sums are read; the same job
    measures normally again with the default budget, as a fresh job on the
    same configurations does."""
    L, W = 8, 12
    wav = engine.StagFluxLongExciton(L, PHI, 0.1, q=(4, 4))
    mk = lambda: engine.Job(wav, walkers=W, seed=29, precision="mixed", reinv_every=L * L,
                            deferred_reinversion=True)
    job = mk()
    job.set_measurements(1)
    job.init_walkers()
    job.walk(L * L * 2, 0)
    cfg = job.config()
    job.reset_quantities()
    job.set_wait_limit(0)
    with pytest.raises(engine.GvError) as err:
        job.measure()
    assert err.value.status == 6
    st = job.status()
    assert (st == 6).any() and set(st.tolist()) <= {0, 6}
    job.set_wait_limit(-1)
    job.init_walkers(cfg)                 # clears the statuses, fresh FP64 inverses
    job.reset_quantities()
    job.measure()
    got, n = job.projheis()
    assert (n == 1).all() and (job.status() == 0).all()
    ref = mk()
    ref.set_measurements(1)
    ref.init_walkers(cfg)
    ref.reset_quantities()
    ref.measure()
    want, _ = ref.projheis()
    assert np.array_equal(got, want)
    job.close()
    ref.close()
