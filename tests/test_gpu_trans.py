"""GPU engine vs the oracle in the transverse-exciton channel (StagFluxTransExciton).

Bar, plain FP64 form: identical start configuration, proposals and accept
decisions (except flagged near-ties |u4 - ratio| < 1e-9), Metropolis ratios
to 1e-10 relative, amplitudes, weights and VirtUpdate ratios to 1e-9, ProjHeis
H / O sums to 1e-9 relative.  The mixed form is compared with the FP64 form.

Channel-state ties.  The stepper hops the wavefunction to the state of
largest |q_k|^2 (LatticeStepper.cpp:86-93), and in this channel states come in
groups of equal |q_k|^2 for every configuration (at L = 4 all eight states of
the start below tie).  Among tied states the reference's pick is decided by
the rounding of its own arithmetic, so the arg-max state is compared up to
ties: where the two picks differ, the oracle's VirtUpdate on the same
configuration must give both the same weight to 1e-9.  Everything the Markov
chain and the measurements depend on is independent of that pick -- the
weight sum_k |q_k|^2, the accept decisions, and H and O (the current state's
amplitude cancels in conj(a_k1) a_k2 / w) -- and is compared exactly; the
amplitude Amp() of the picked state is compared with the oracle's amplitude
of that same state.
"""
import math

import numpy as np
import pytest
from test_gpu_parity import check_ratios

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi
RTOL = 1e-10
CASES = [(4, (2, 2), 7, 3), (8, (4, 4), 7, 3), (8, (2, 0), 11, 0), (12, (6, 6), 5, 1), (16, (4, 4), 7, 3)]
EMPTY = (-1, -1, -1, -1)


def _pair(engine, oracle, L, q, seed, walker, neel=0.1, precision="fp64", reinv=0, walkers=1):
    wav = engine.StagFluxTransExciton(L, PHI, neel, q=q)
    job = engine.Job(wav, walkers=walkers, seed=seed, precision=precision, reinv_every=reinv, walker_base=walker)
    orc = oracle.OracleChain(L, PHI, neel, channel=oracle.TRANS, q=q, seed=seed, walker=walker)
    return job, orc


def _state_amps(orc, hop=EMPTY):
    """Amplitudes q_k of every channel state after the real hop set `hop`, as
    (complex mantissa, base-10 exponent) arrays (the reference's BigComplex)."""
    qm, qe = orc.virt_update(np.array([hop], dtype=np.int32))
    return qm[:, 0], qe[:, 0].astype(np.int64)


def _log10_weights(qm, qe):
    return 2.0 * np.log10(np.abs(qm)) + 2.0 * qe


def _check_state(job, orc, walker=0, rtol=1e-9):
    """The engine's current state ties the oracle's, and Amp() of the engine's
    state equals the oracle's amplitude of that state."""
    kg, ko = int(job.state_index()[walker]), orc.current_state()
    qm, qe = _state_amps(orc)
    lw = _log10_weights(qm, qe)
    assert abs(lw[kg] - lw[ko]) < rtol, (kg, ko, lw[kg], lw[ko])
    m, e = job.amplitude()
    a = m[walker] * 10.0 ** float(e[walker] - qe[kg])
    assert abs(a - qm[kg]) < rtol * abs(qm[kg]), (a, qm[kg])
    # weight sum_k |q_k|^2 against the oracle's (its stepper weight)
    wm, we = orc.weight()
    wg = job.weight()[walker] * abs(m[walker]) ** 2 * 10.0 ** float(2 * e[walker] - we)
    assert abs(wg - wm) < rtol * wm, (wg, wm)
    return kg == ko


def _compare_traces(orc2, tg, to, fresh_chain=None):
    """Trace comparison with the arg-max state compared up to ties (orc2 is a
    fresh oracle chain replayed in lockstep to read every state's weight).
    Ratios as in test_gpu_parity.check_ratios (1e-10, or no further than the
    oracle from the ratio of a freshly inverted state)."""
    assert (tg["v1"] == to["v1"]).all() and (tg["v2"] == to["v2"]).all()
    assert (tg["kind"] == to["kind"]).all()
    tie = np.abs(to["u"][:, 3] - to["ratio"]) < 1e-9
    assert ((tg["accepted"] == to["accepted"]) | tie).all()
    real = to["kind"] == 1
    check_ratios(tg, to, fresh_chain)
    ties = 0
    for i in range(len(to)):
        # a proposal whose weight vanishes (ratio < 1e-8, rejected) splits
        # rounding noise over the states: its arg-max carries no information
        if real[i] and tg["khop"][i] != to["khop"][i] and to["ratio"][i] > 1e-8:
            up = orc2.config().astype(bool)
            v1, v2 = int(to["v1"][i]), int(to["v2"][i])
            u, d = (v1, v2) if up[v1] else (v2, v1)
            lw = _log10_weights(*_state_amps(orc2, (u, d, d, u)))
            assert abs(lw[tg["khop"][i]] - lw[to["khop"][i]]) < 1e-9, (i, tg["khop"][i], to["khop"][i])
            ties += 1
        orc2.step()
    return ties


@pytest.mark.parametrize("L,q,seed,walker", CASES)
def test_trans_start(engine, oracle, L, q, seed, walker):
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    assert job.Nexc == L * L // 2 and job.N == (L * L // 2 + 1, L * L // 2 - 1)
    job.init_walkers()
    assert orc.random_start() == 0
    assert (job.config()[0] == orc.config()).all()
    if _check_state(job, orc, rtol=RTOL):
        for fl in (0, 1):
            gi, oi = job.inverse(0, fl), orc.inverse(fl)
            assert np.abs(gi - oi).max() < RTOL * np.abs(oi).max()
    assert job.drift().max() < 1e-12


@pytest.mark.parametrize("L,q,seed,walker", CASES[:3])
def test_trans_virt_update(engine, oracle, L, q, seed, walker):
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.init_walkers()
    orc.random_start()
    up = orc.config().astype(bool)
    hops = [EMPTY]
    for x in range(L):
        for y in range(L):
            a = y * L + x
            for b in (((y + 1) % L) * L + x, y * L + (x + 1) % L):
                if up[a] != up[b]:
                    u, d = (a, b) if up[a] else (b, a)
                    hops.append((u, d, d, u))
    hops.append((int(np.flatnonzero(up)[0]), int(np.flatnonzero(~up)[0]), -1, -1))
    hops.append((-1, -1, int(np.flatnonzero(~up)[1]), int(np.flatnonzero(up)[1])))
    hops = np.array(hops, dtype=np.int32)
    qg = job.virt_update(0, hops)                  # (Nexc, nset), relative to the engine's Amp()
    qm, qe = orc.virt_update(hops)                 # absolute, BigComplex mantissa / exponent
    am, ae = orc.amp()
    m, e = job.amplitude()
    qo = qm * 10.0 ** (qe - ae).astype(float) / am  # relative to the oracle's Amp()
    qg = qg * (m[0] * 10.0 ** float(e[0] - ae) / am)
    scale = np.abs(qo).max(axis=0)
    assert (np.abs(qg - qo) < 1e-9 * scale).all()


@pytest.mark.parametrize("L,q,seed,walker,steps", [(4, (2, 2), 7, 3, 2000), (8, (4, 4), 7, 3, 1500),
                                                   (8, (2, 0), 11, 0, 2500), (12, (6, 6), 5, 1, 1200),
                                                   (16, (4, 4), 7, 3, 1500)])
def test_trans_trace_parity(engine, oracle, L, q, seed, walker, steps):
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(steps, 0)
    to = orc.walk(steps, trace=True)
    orc2 = oracle.OracleChain(L, PHI, 0.1, channel=oracle.TRANS, q=q, seed=seed, walker=walker)
    orc2.random_start()

    def fresh():
        o = oracle.OracleChain(L, PHI, 0.1, channel=oracle.TRANS, q=q, seed=seed, walker=walker)
        o.random_start()
        return o
    ties = _compare_traces(orc2, tg, to, fresh)
    assert (job.config()[0] == orc.config()).all()
    # with every pick equal the Slater rows hold the same orbitals in the same
    # order as the oracle's; after a differently broken tie they may be permuted
    if _check_state(job, orc) and ties == 0:
        for fl in (0, 1):
            gi, oi = job.inverse(0, fl), orc.inverse(fl)
            assert np.abs(gi - oi).max() < 1e-9 * np.abs(oi).max()
    assert job.drift().max() < 1e-10
    c = job.counts()[0]
    assert c[0] == steps and c[1] == int((to["accepted"] & (to["kind"] == 1)).sum())


@pytest.mark.parametrize("L,q,seed,walker", [(4, (2, 2), 7, 3), (8, (4, 4), 7, 3), (16, (4, 4), 7, 3)])
def test_trans_measurements(engine, oracle, L, q, seed, walker):
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN | oracle.MEAS_STATSPIN
    job, orc = _pair(engine, oracle, L, q, seed, walker)
    job.set_measurements(mask)
    job.init_walkers()
    orc.random_start()
    job.walk(L * L * 4, 0)
    orc.walk(L * L * 4)
    assert (job.config()[0] == orc.config()).all()
    job.walk(L * L * 6, L * L)
    orc.walk(L * L * 6, meas=L * L, mask=mask)
    assert (job.config()[0] == orc.config()).all()
    pg, ng = job.projheis()
    po, no = orc.projheis()
    assert ng[0] == no == 6
    assert np.abs(pg[0] - po).max() < 1e-9 * np.abs(po).max()
    sg, nsg = job.stagmagn()
    so, nso = orc.stagmagn()
    assert nsg[0] == nso and abs(sg[0] - so) < 1e-12
    ssg, nssg = job.statspin()
    sso, nsso = orc.statspin()
    assert nssg == nsso
    # StatSpinStruct swaps particles within the current channel state
    # (StatSpinStruct.cpp:74, one state), so its sums depend on the picked
    # state: compare one measurement made where both codes hold the same state.
    if job.state_index()[0] == orc.current_state():
        job.reset_quantities()
        job.set_measurements(oracle.MEAS_STATSPIN)
        job.measure()
        orc.reset_quantities()
        orc.measure(oracle.MEAS_STATSPIN)
        ssg, _ = job.statspin()
        sso, _ = orc.statspin()
        assert np.abs(ssg - sso).max() < 1e-9 * max(1.0, np.abs(sso).max())


def test_trans_reinversion_cadence(engine, oracle):
    L, q, seed, walker = 8, (4, 4), 9, 2
    job, orc = _pair(engine, oracle, L, q, seed, walker, reinv=L * L)
    job.init_walkers()
    orc.random_start()
    tg = job.walk_traced(3000, 0)
    to = orc.walk(3000, reinv_every=L * L, trace=True)
    orc2 = oracle.OracleChain(L, PHI, 0.1, channel=oracle.TRANS, q=q, seed=seed, walker=walker)
    orc2.random_start()
    _compare_traces(orc2, tg, to)
    assert (job.config()[0] == orc.config()).all()
    assert job.counts()[0][4] == orc.counts()[3] > 0
    _check_state(job, orc)


@pytest.mark.parametrize("policy", ["cadence", "drift"])
def test_trans_mixed_vs_fp64(engine, policy):
    """Mixed-precision walk against the FP64 walk on the same walkers: the
    first steps agree, and after a walk the H and O matrices the mixed job
    measures on its configurations match an FP64 job started on the same
    configurations (H and O depend on the configuration only)."""
    L, q, W = 8, (4, 4), 64
    wav = engine.StagFluxTransExciton(L, PHI, 0.1, q=q)
    kw = dict(reinv_every=L * L)
    if policy == "drift":
        kw.update(drift_threshold=1e-5)
    mixed = engine.Job(wav, walkers=W, seed=21, precision="mixed", **kw)
    exact = engine.Job(wav, walkers=W, seed=21, precision="fp64", reinv_every=L * L)
    for j in (mixed, exact):
        j.set_measurements(1)
        j.init_walkers()
    # the mixed job redraws starts too ill-conditioned for FP32; the rest agree
    same_start = (mixed.config() == exact.config()).all(axis=1)
    assert same_start.mean() > 0.8
    w = int(np.flatnonzero(same_start)[0])
    tm = mixed.walk_traced(200, 0, walker=w)
    te = exact.walk_traced(200, 0, walker=w)
    assert (tm["accepted"][:50] == te["accepted"][:50]).all()
    real = te["kind"] == 1
    assert np.allclose(tm["ratio"][real][:40], te["ratio"][real][:40], rtol=1e-3, atol=1e-6)
    mixed.walk(L * L * 20, 0)
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
    print("H/O matrix error vs FP64: median %.2e max %.2e" % (np.median(err), err.max()))
    assert np.median(err) < 1e-4 and err.max() < 1e-2
    assert mixed.drift().max() < 1e-3
