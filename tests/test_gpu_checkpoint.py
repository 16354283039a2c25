"""Checkpoint / resume (gv_job_checkpoint, gv_job_restore).

The reference resumes a chain from its saved lattice Fock state
(State::Save, State.cpp:117-166; vmc.cpp:178-220) with fresh random numbers
and a fresh inversion.  Here a checkpoint also carries the Philox counters,
counters, amplitude and quantity sums, so the bar is exact:
  * with stored inverses, a restored job continues bit for bit as the
    checkpointed job does (configurations, amplitudes, inverses, counters,
    quantity sums);
  * without them, the restored job equals the checkpointed job after an FP64
    re-inversion (gv_job_reinvert), again bit for bit from there on;
  * a blob from a job of another configuration, or a damaged blob, is refused
    and leaves the job untouched.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _gs(engine, precision, L=8, W=24, seed=5, **kw):
    kw.setdefault("reinv_every", 64)
    kw.setdefault("deferred_reinversion", True)
    return engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=W, seed=seed, precision=precision, **kw)


def _trans(engine, precision, L=8, W=8, seed=7, **kw):
    kw.setdefault("reinv_every", 64)
    kw.setdefault("deferred_reinversion", True)
    return engine.Job(engine.StagFluxTransExciton(L, PHI, 0.1, q=(4, 4)), walkers=W, seed=seed,
                      precision=precision, **kw)


def _long(engine, precision, L=8, W=8, seed=3, **kw):
    kw.setdefault("reinv_every", 64)
    kw.setdefault("deferred_reinversion", True)
    return engine.Job(engine.StagFluxLongExciton(L, PHI, 0.1, q=(2, 2)), walkers=W, seed=seed,
                      precision=precision, **kw)


def _snapshot(job, statspin=False):
    s = {
        "config": job.config(),
        "counts": job.counts(),
        "amp": job.amplitude(),
        "status": job.status(),
        "state": job.state_index(),
        "weight": job.weight(),
        "pj": job.projheis(),
        "sm": job.stagmagn(),
        "drift": job.drift_checks(),
        "inv": [job.inverse(w, fl) for w in (0, job.walkers - 1) for fl in (0, 1)],
    }
    if statspin:
        s["ss"] = job.statspin()
    return s


def _assert_same(a, b, ss_rtol=None):
    for k in a:
        if k == "ss":
            np.testing.assert_allclose(a[k][0], b[k][0], rtol=ss_rtol, atol=1e-12)
            assert a[k][1] == b[k][1]
            continue
        va, vb = a[k], b[k]
        if isinstance(va, tuple):
            for x, y in zip(va, vb):
                assert np.array_equal(x, y), k
        elif isinstance(va, list):
            for x, y in zip(va, vb):
                assert np.array_equal(x, y), k
        else:
            assert np.array_equal(va, vb), k


def _split_run(make, mask, inverses, statspin=False):
    """Walk A, checkpoint, continue A; restore into a fresh B and continue it
    the same way; return both snapshots."""
    a = make()
    a.set_measurements(mask)
    a.init_walkers()
    L2 = a.Ns
    a.walk(L2 * 6, 0)
    a.walk(L2 * 3, L2)
    blob = a.checkpoint(inverses=inverses)
    if not inverses:
        a.reinvert()
    a.walk_continue(L2 * 3, L2)
    a.walk(L2 * 2, 0)
    b = make()
    b.set_measurements(mask)
    b.restore(blob)
    b.walk_continue(L2 * 3, L2)
    b.walk(L2 * 2, 0)
    return _snapshot(a, statspin), _snapshot(b, statspin)


@pytest.mark.parametrize("inverses", [True, False])
def test_resident_walk_resumes_exactly(engine, oracle, inverses):
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN
    a, b = _split_run(lambda: _gs(engine, "mixed"), mask, inverses)
    _assert_same(a, b)
    assert (a["pj"][1] == 6).all()   # the sums ran on across the checkpoint


@pytest.mark.parametrize("inverses", [True, False])
def test_fp64_walk_resumes_exactly(engine, oracle, inverses):
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN | oracle.MEAS_STATSPIN
    a, b = _split_run(lambda: _gs(engine, "fp64", W=12), mask, inverses, statspin=True)
    # StatSpinStruct sums are job-wide atomics: equal up to summation order
    _assert_same(a, b, ss_rtol=1e-12)


def test_streaming_mixed_walk_resumes_exactly(engine, oracle):
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN
    a, b = _split_run(lambda: _gs(engine, "mixed", stream_inverses=True, drift_threshold=1e-5), mask, True)
    _assert_same(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("inverses", [True, False])
def test_exciton_walk_resumes_exactly(engine, oracle, precision, inverses):
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN
    a, b = _split_run(lambda: _trans(engine, precision), mask, inverses)
    _assert_same(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("inverses", [True, False])
def test_long_exciton_walk_resumes_exactly(engine, oracle, precision, inverses):
    """The longitudinal channel also carries its overlap tables R; without
    stored inverses the restore rebuilds them with the FP64 inversion."""
    mask = oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN
    a, b = _split_run(lambda: _long(engine, precision), mask, inverses)
    _assert_same(a, b)
    assert (a["pj"][1] == 6).all()


def test_restore_refuses_foreign_or_damaged_blobs(engine, tmp_path):
    a = _gs(engine, "mixed", W=8)
    a.init_walkers()
    a.walk(a.Ns * 2, 0)
    blob = a.checkpoint(inverses=True)
    light = a.checkpoint(inverses=False)
    assert len(blob) > len(light)

    b = _gs(engine, "mixed", W=8)
    b.init_walkers()
    before = _snapshot(b)

    def refused(job, data):
        with pytest.raises(engine.GvError) as e:
            job.restore(data)
        assert e.value.status == 1

    refused(_gs(engine, "mixed", W=8, seed=6), blob)          # another seed
    refused(_gs(engine, "mixed", W=9), blob)                  # another walker count
    refused(_gs(engine, "fp64", W=8), blob)                   # stored inverses of another precision
    bad = bytearray(blob)
    bad[len(bad) // 2] ^= 0x40
    refused(b, bytes(bad))                                    # damaged payload
    refused(b, blob[:-8])                                     # truncated
    refused(b, b"GVCKPT01" + blob[8:16])                      # header only
    _assert_same(before, _snapshot(b))                        # refusals left b as it was

    # without inverses the blob restores into a job of the other precision
    c = _gs(engine, "fp64", W=8)
    c.restore(light)
    assert np.array_equal(c.config(), a.config())
    assert np.array_equal(c.counts(), a.counts())
    assert c.drift().max() < 1e-9

    # file round trip
    p = tmp_path / "chain.ckpt"
    a.save_checkpoint(str(p), inverses=True)
    d = _gs(engine, "mixed", W=8)
    d.load_checkpoint(str(p))
    a.walk(a.Ns, 0)
    d.walk(d.Ns, 0)
    assert np.array_equal(a.config(), d.config())
    assert np.array_equal(a.inverse(3, 1), d.inverse(3, 1))
