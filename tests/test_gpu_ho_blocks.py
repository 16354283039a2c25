"""Exciton ProjHeis H / O sums of mixed jobs in blocks of measurements.

A mixed job keeps each measurement's FP32 factors (conj(a)/w, h, a) in one of
32 slots per walker and folds a full block into the FP64 sums: the block's
outer products are summed in FP32 and added to FP64 once per entry.  Reads
fold the waiting slots into a copy, so the sums a job accumulates do not
depend on when (or whether) it is read.

Bars, per walker, against the largest |entry| of one measurement times the
number of measurements:
  * repeated measurements of one configuration (two full blocks and six
    waiting) against that many times one measurement: 1e-5 (the FP32 block
    sum is off by at most 2 * 32 * 2^-24 = 4e-6 of the block's absolute sum);
  * against the FP64 job on the same configurations: 1e-3, the bar of a single
    mixed measurement (the FP32 bond ratios dominate);
  * a read in the middle of a block changes nothing, bit for bit;
  * reset_quantities empties the waiting slots.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _wav(engine, channel, L):
    if channel == "trans":
        return engine.StagFluxTransExciton(L, PHI, 0.1, q=(4, 4))
    return engine.StagFluxLongExciton(L, PHI, 0.1, q=(2, 2))


@pytest.mark.parametrize("channel", ["trans", "long"])
def test_block_sums_of_repeated_measurements(engine, oracle, channel):
    L, W, M = 8, 6, 70
    wav = _wav(engine, channel, L)
    mk = lambda prec: engine.Job(wav, walkers=W, seed=13, precision=prec, reinv_every=64,
                                 deferred_reinversion=True)
    j0 = mk("mixed")
    j0.init_walkers()
    j0.walk(L * L * 2, 0)
    cfg = j0.config()
    jobs = [mk("mixed") for _ in range(3)] + [mk("fp64")]
    for j in jobs:
        j.init_walkers(cfg)
        j.set_measurements(oracle.MEAS_PROJHEIS)
        j.reset_quantities()
    j1, jm, jr, j64 = jobs
    j1.measure()
    one, n1 = j1.projheis()
    assert (n1 == 1).all()
    scale = np.abs(one).max(axis=(1, 2), keepdims=True)
    assert (scale > 0).all()
    for i in range(M):
        for j in (jm, jr, j64):
            j.measure()
        if i == 39:
            mid, _ = jr.projheis()             # 32 folded + 8 waiting
            assert (np.abs(mid - 40 * one) / (40 * scale)).max() < 1e-5
    pm, nm = jm.projheis()
    pr, nr = jr.projheis()
    p64, n64 = j64.projheis()
    assert (nm == M).all() and (nr == M).all() and (n64 == M).all()
    assert np.array_equal(pm, pr)
    assert (np.abs(pm - M * one) / (M * scale)).max() < 1e-5
    assert (np.abs(pm - p64) / (M * scale)).max() < 1e-3
    # reading twice gives the same sums; a reset drops the waiting slots too
    assert np.array_equal(jm.projheis()[0], pm)
    jm.reset_quantities()
    for _ in range(3):
        jm.measure()
    p3, n3 = jm.projheis()
    assert (n3 == 3).all()
    assert (np.abs(p3 - 3 * one) / (3 * scale)).max() < 1e-5
    for j in jobs + [j0]:
        j.close()
