"""StagMagnTrack / OverlapTrack (GV_MEAS_STAGMAGN_TRACK, GV_MEAS_OVERLAP_TRACK):
per-measurement series whose sum is the StagMagnZ sum, whose last weight
entry after a measure() is the current |Amp|^2 (exciton: sigma |Amp|^2), and
which stop growing at the capacity."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi
TRACKS = 8 | 16


@pytest.mark.parametrize("precision,channel", [("fp64", "gs"), ("mixed", "gs"), ("mixed", "trans"), ("fp64", "trans")])
def test_tracks_follow_the_measurements(engine, oracle, precision, channel):
    L, W = 8, 6
    wav = (engine.StagFluxTransExciton(L, PHI, 0.1, q=(4, 4)) if channel == "trans"
           else engine.StagFluxGroundState(L, PHI, 0.1))
    j = engine.Job(wav, walkers=W, seed=13, precision=precision, reinv_every=64, deferred_reinversion=True)
    j.set_measurements(oracle.MEAS_STAGMAGN | oracle.MEAS_PROJHEIS | TRACKS)
    j.set_track_capacity(8)
    j.init_walkers()
    j.walk(L * L * 5, L * L)
    sm, lw, n = j.tracks()
    s, ns = j.stagmagn()
    assert (n == 5).all() and (ns == 5).all()
    assert np.allclose(sm[:, :5].sum(axis=1), s.real, rtol=0, atol=1e-12)
    assert np.isfinite(lw[:, :5]).all()
    # one more measurement without a step: the weight of the current state
    j.measure()
    sm, lw, n = j.tracks()
    assert (n == 6).all()
    m, e = j.amplitude()
    want = 2 * (np.log10(np.abs(m)) + e)
    if channel == "trans":
        want = want + np.log10(j.weight())
    assert np.allclose(lw[:, 5], want, rtol=0, atol=1e-9)
    # a new measuring walk restarts the tracks; they stop at the capacity
    j.walk(L * L * 10, L * L)
    sm, lw, n = j.tracks()
    assert (n == 8).all()


def test_track_quantities_through_metromc(engine):
    L = 8
    job = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=3, seed=5, precision="fp64")
    step = engine.LatticeStepper(job)
    mc = engine.MetroMC(step)
    st, ov, smz = engine.StagMagnTrack(step), engine.OverlapTrack(step), engine.StagMagnZ(step)
    for q in (st, ov, smz):
        mc.AddQuantity(q)
    job.init_walkers()
    mc.Walk(L * L * 7, L * L)
    series, rel = st.save(), ov.save()
    assert [len(x) for x in series] == [7, 7, 7] and [len(x) for x in rel] == [7, 7, 7]
    assert np.allclose([x.mean() for x in series], smz.save().real, atol=1e-12)
    assert np.allclose([x.mean() for x in rel], 1.0)
