"""On-chip exciton walk (k_walk_trans_res: GupT and the flavour-1 inverse in
TMEM, the flavour-0 inverse in shared memory) against the streaming exciton
walk (k_walk_trans, selected with stream_inverses=True) and against FP64.

Both kernels run the same FP32 arithmetic in a different summation order, so
the bar is: the same proposals, the same accept decisions except near-ties
(|u4 - ratio| < 1e-4 relative), Metropolis ratios to 1e-4 relative, inverses
after a walk to 1e-3 of their largest entry on walkers whose chains stayed
together, and H / O measured on the final configurations within 1e-4 (median)
of an FP64 job started on the same configurations.  L = 16 puts row 128 of
GupT in its own TMEM columns (N0 = 129).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi
CASES = [(8, (4, 4), 64), (12, (6, 0), 32), (16, (8, 8), 32)]


def _jobs(engine, L, q, W, seed=5):
    wav = engine.StagFluxTransExciton(L, PHI, 0.1, q=q)
    kw = dict(walkers=W, seed=seed, precision="mixed", reinv_every=L * L, deferred_reinversion=True)
    onchip = engine.Job(wav, **kw)
    stream = engine.Job(wav, stream_inverses=True, **kw)
    for j in (onchip, stream):
        j.set_measurements(1)
        j.init_walkers()
    return wav, onchip, stream


@pytest.mark.parametrize("L,q,W", CASES)
def test_trans_onchip_trace(engine, L, q, W):
    _, onchip, stream = _jobs(engine, L, q, W)
    assert (onchip.config() == stream.config()).all()
    ta = onchip.walk_traced(400, 0, walker=1)
    tb = stream.walk_traced(400, 0, walker=1)
    # the chains agree up to the first near-tie decision
    tie = np.abs(tb["u4"] - tb["ratio"]) < 1e-4 * np.maximum(tb["ratio"], 1e-30)
    stop = int(np.flatnonzero(tie)[0]) if tie.any() else len(tie)
    assert stop > 50
    assert (ta["v1"][:stop] == tb["v1"][:stop]).all() and (ta["v2"][:stop] == tb["v2"][:stop]).all()
    assert (ta["accepted"][:stop] == tb["accepted"][:stop]).all()
    real = (tb["kind"] == 1)[:stop]
    assert real.sum() > 20
    assert np.allclose(ta["ratio"][:stop][real], tb["ratio"][:stop][real], rtol=1e-4, atol=1e-7)
    assert (onchip.status() == 0).all() and (stream.status() == 0).all()
    onchip.close()
    stream.close()


@pytest.mark.parametrize("L,q,W", CASES)
def test_trans_onchip_state(engine, L, q, W):
    """After a walk of 2 sweeps the counters of chains that stayed together
    agree with the streaming kernel's, and so do the H / O sums measured on
    them (independent of which of tied channel states each kernel picked);
    the inverses and weights agree where the picked states are the same too."""
    _, onchip, stream = _jobs(engine, L, q, W)
    n = 2 * L * L
    onchip.walk(n, 0)
    stream.walk(n, 0)
    assert (onchip.status() == 0).all() and (stream.status() == 0).all()
    same = (onchip.config() == stream.config()).all(axis=1)
    assert same.mean() > 0.7, same.mean()
    ca, cb = onchip.counts(), stream.counts()
    assert (ca[same][:, :4] == cb[same][:, :4]).all()
    pick = same & (onchip.state_index() == stream.state_index())
    for w in np.flatnonzero(pick)[:8]:
        w = int(w)
        if not all((onchip.orbitals(w, fl) == stream.orbitals(w, fl)).all() for fl in (0, 1)):
            continue
        for fl in (0, 1):
            a, b = onchip.inverse(w, fl), stream.inverse(w, fl)
            assert np.abs(a - b).max() < 1e-3 * np.abs(b).max(), (w, fl)
    assert np.allclose(onchip.weight()[pick], stream.weight()[pick], rtol=1e-3)
    for j in (onchip, stream):
        j.reset_quantities()
        j.measure()
    pa, pb = onchip.projheis()[0][same], stream.projheis()[0][same]
    err = np.abs(pa - pb).max(axis=(1, 2)) / np.abs(pb).max(axis=(1, 2))
    assert np.median(err) < 1e-4 and err.max() < 1e-2, (np.median(err), err.max())
    onchip.close()
    stream.close()


@pytest.mark.parametrize("L,q,W", CASES)
def test_trans_onchip_vs_fp64(engine, L, q, W):
    wav, onchip, stream = _jobs(engine, L, q, W)
    stream.close()
    onchip.walk(L * L * 6, 0)
    assert (onchip.status() == 0).all()
    cfg = onchip.config()
    onchip.reset_quantities()
    onchip.measure()
    pm, _ = onchip.projheis()
    ref = engine.Job(wav, walkers=W, seed=5, precision="fp64")
    ref.set_measurements(1)
    ref.init_walkers(cfg)
    ref.reset_quantities()
    ref.measure()
    pr, _ = ref.projheis()
    err = np.abs(pm - pr).max(axis=(1, 2)) / np.abs(pr).max(axis=(1, 2))
    print("L=%d H/O error vs FP64: median %.2e max %.2e" % (L, np.median(err), err.max()))
    assert np.median(err) < 1e-4 and err.max() < 1e-2
    onchip.close()
    ref.close()
