"""Single-walker stepping: the reference's step-level API (Stepper::trystep /
step / weight, MetroMC::Step / YesNo, SlaterDeterminant::Update) through the
C ABI, against the oracle.

Bar (FP64): the same proposals, decisions up to flagged near-ties, ratios as
in test_gpu_parity.check_ratios, the same final configuration; stepping and
gv_job_walk share each walker's Philox stream, so they can be mixed; and
gv_job_update applies a move with the walk kernels' own update code, so
replaying a walk's accepted moves reproduces its inverses bit for bit.
"""
import math

import numpy as np
import pytest
from test_gpu_parity import check_ratios

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _wav(engine, channel, L, q):
    if channel == "trans":
        return engine.StagFluxTransExciton(L, PHI, 0.1, q=q)
    if channel == "long":
        return engine.StagFluxLongExciton(L, PHI, 0.1, q=q)
    return engine.StagFluxGroundState(L, PHI, 0.1)


def _oracle(oracle, channel, L, q, seed, walker):
    ch = {"gs": oracle.GROUNDSTATE, "trans": oracle.TRANS, "long": oracle.LONG}[channel]
    o = oracle.OracleChain(L, PHI, 0.1, channel=ch, q=q, seed=seed, walker=walker)
    assert o.random_start() == 0
    return o


def _step_trace(mc, stepper, n):
    """MetroMC::Step written out (MetroMC.cpp:90-103), one record per step."""
    rec = []
    sw = stepper.weight()
    for _ in range(n):
        new = stepper.trystep()
        ratio = math.ldexp(new[0] / sw[0], new[1] - sw[1])
        acc = mc.YesNo(ratio)
        v1, v2 = stepper.prev
        kind = int(stepper.khop >= 0)
        if acc:
            stepper.step()
            sw = new
        rec.append((v1, v2, kind, int(acc), ratio))
    t = np.zeros(n, dtype=[("v1", "<i4"), ("v2", "<i4"), ("kind", "<i4"), ("accepted", "<i4"), ("ratio", "<f8")])
    for i, r in enumerate(rec):
        t[i] = r
    return t


@pytest.mark.parametrize("channel,L,q,seed,steps", [("gs", 8, (0, 0), 77, 1200), ("gs", 16, (0, 0), 5, 600),
                                                    ("trans", 8, (4, 4), 7, 500), ("trans", 4, (2, 2), 7, 500),
                                                    ("long", 4, (2, 2), 7, 500), ("long", 8, (0, 0), 7, 400)])
def test_metromc_step_matches_oracle(engine, oracle, channel, L, q, seed, steps):
    job = engine.Job(_wav(engine, channel, L, q), walkers=1, seed=seed, precision="fp64")
    job.init_walkers()
    orc = _oracle(oracle, channel, L, q, seed, 0)
    assert (job.config()[0] == orc.config()).all()
    stepper = engine.LatticeStepper(job)
    mc = engine.MetroMC(stepper)
    t = _step_trace(mc, stepper, steps)
    to = orc.walk(steps, trace=True)
    assert (t["v1"] == to["v1"]).all() and (t["v2"] == to["v2"]).all()
    assert (t["kind"] == to["kind"]).all()
    tie = np.abs(to["u"][:, 3] - to["ratio"]) < 1e-9
    assert ((t["accepted"] == to["accepted"]) | tie).all()
    if not tie.any():

        def fresh():
            return _oracle(oracle, channel, L, q, seed, 0)
        check_ratios(t, to, fresh)
        assert (job.config()[0] == orc.config()).all()
        c = job.counts()[0]
        assert c[0] == steps and c[1] == int((to["accepted"] & (to["kind"] == 1)).sum())
    # MetroMC.Step itself continues the same chain
    for _ in range(100):
        mc.Step()
    orc.walk(100)
    if not tie.any():
        assert (job.config()[0] == orc.config()).all()


@pytest.mark.parametrize("channel,L,q", [("gs", 8, (0, 0)), ("gs", 12, (0, 0)), ("trans", 8, (4, 4)),
                                         ("long", 8, (2, 2))])
def test_update_replays_a_walk_bit_for_bit(engine, channel, L, q):
    """SlaterDeterminant::Update with the exchanges and channel states a walk
    accepted gives that walk's configuration, amplitude and inverses exactly."""
    wav = _wav(engine, channel, L, q)
    a = engine.Job(wav, walkers=2, seed=11, precision="fp64")
    b = engine.Job(wav, walkers=2, seed=11, precision="fp64")
    a.init_walkers()
    b.init_walkers()
    t = a.walk_traced(800, 0, walker=1)
    for r in t[(t["kind"] == 1) & (t["accepted"] == 1)]:
        v1, v2 = int(r["v1"]), int(r["v2"])
        up = b.config()[1].astype(bool)
        u, d = (v1, v2) if up[v1] else (v2, v1)
        b.update(1, (u, d, d, u), int(r["khop"]) if channel != "gs" else -1)
    assert (a.config()[1] == b.config()[1]).all()
    ma, ea = a.amplitude()
    mb, eb = b.amplitude()
    assert ea[1] == eb[1] and ma[1] == mb[1]
    for fl in (0, 1):
        assert np.array_equal(a.inverse(1, fl), b.inverse(1, fl))
    if channel != "gs":
        assert a.state_index()[1] == b.state_index()[1]
    # walker 0 untouched by the updates on walker 1
    c = engine.Job(wav, walkers=2, seed=11, precision="fp64")
    c.init_walkers()
    assert (b.config()[0] == c.config()[0]).all()
    with pytest.raises(engine.GvError):
        b.update(1, (0, 1, 2, 3), -1)                   # not an exchange


def test_stepping_and_walking_share_the_stream(engine):
    """Single steps of walker 2 followed by a walk of every walker equal a job
    that only walked (FP64, tie-free seed)."""
    L, W, n1, n2 = 8, 4, 200, 400
    wav = engine.StagFluxGroundState(L, PHI, 0.1)
    a = engine.Job(wav, walkers=W, seed=41, precision="fp64")
    b = engine.Job(wav, walkers=W, seed=41, precision="fp64")
    for j in (a, b):
        j.init_walkers()
    a.walk(n1, 0)
    stepper = engine.LatticeStepper(b, walker=2)
    mc = engine.MetroMC(stepper)
    for _ in range(n1):
        mc.Step()
    b.walk(n2, 0)
    a.walk(n2, 0)
    assert (a.config()[2] == b.config()[2]).all()
    ca, cb = a.counts()[2], b.counts()[2]
    assert ca[0] == cb[0] and ca[1] == cb[1]
