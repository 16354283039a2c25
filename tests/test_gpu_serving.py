"""Serving loop (gv_server_*): continuous batching of heterogeneous requests.

Each request's results must be the same alone and in the mix: a job's chain
depends only on its own request (seed, walkers, chunking), so the steps,
accepted moves and quantity averages are compared exactly.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _requests(engine):
    gs, tr = engine.StagFluxGroundState, engine.StagFluxTransExciton
    return [
        dict(wav=gs(8, PHI, 0.1), walkers=48, sweeps=12, therm_sweeps=4, seed=1, precision="mixed"),
        dict(wav=tr(4, PHI, 0.1, q=(2, 2)), walkers=16, sweeps=10, therm_sweeps=2, seed=2, precision="mixed"),
        dict(wav=gs(12, 0.2 * math.pi, 0.05), walkers=32, sweeps=6, therm_sweeps=2, seed=3, precision="fp64",
             reinv_every=0),
        dict(wav=gs(16, PHI, 0.1), walkers=64, sweeps=4, therm_sweeps=2, seed=4, precision="mixed"),
        dict(wav=tr(8, PHI, 0.1, q=(4, 4)), walkers=24, sweeps=5, therm_sweeps=2, seed=5, precision="mixed"),
        dict(wav=gs(6, PHI, 0.1), walkers=8, sweeps=20, therm_sweeps=0, seed=6, precision="mixed",
             reinv_every=0),
    ]


def _run(engine, reqs, max_jobs, budget=0):
    with engine.Server(hbm_budget=budget, max_jobs=max_jobs, chunk_sweeps=2) as srv:
        tickets = [srv.submit(**r) for r in reqs]
        srv.drain(600)
        return [srv.poll(t) for t in tickets]


def test_results_same_alone_and_in_the_mix(engine):
    reqs = _requests(engine)
    mixed = _run(engine, reqs, max_jobs=8)
    for r in mixed:
        assert r["state"] == 2 and r["status"] == 0
        assert r["t_submit"] <= r["t_admit"] <= r["t_done"]
        assert r["t_admit"] <= r["t_started"] <= r["t_walked"] <= r["t_done"]
        assert np.isfinite(r["e_site"]) and r["steps"] > 0
    # jobs overlapped on the device: some job was admitted before another finished
    admits = sorted(r["t_admit"] for r in mixed)
    dones = sorted(r["t_done"] for r in mixed)
    assert admits[1] < dones[0]
    for i, r in enumerate(reqs):
        alone = _run(engine, [r], max_jobs=1)[0]
        for k in ("steps", "accepted", "e_site", "stagmagn"):
            assert alone[k] == mixed[i][k], (i, k, alone[k], mixed[i][k])


def test_admission_by_footprint(engine):
    gs = engine.StagFluxGroundState
    big = dict(wav=gs(16, PHI, 0.1), walkers=256, sweeps=2, therm_sweeps=0, seed=9)
    fp = engine.Job.footprint(big["wav"], 256, "mixed")
    with engine.Server(hbm_budget=int(fp * 1.5), max_jobs=8, chunk_sweeps=1) as srv:
        a = srv.submit(**big)
        b = srv.submit(**dict(big, seed=10))
        ra, rb = srv.wait(a), srv.wait(b)
    assert ra["footprint"] == fp
    assert rb["t_admit"] >= ra["t_done"]   # the budget holds one such job at a time


def test_validation_and_invalid_request(engine):
    gs = engine.StagFluxGroundState
    with engine.Server(max_jobs=4, chunk_sweeps=2) as srv:
        t = srv.submit(gs(8, PHI, 0.1), walkers=32, sweeps=4, therm_sweeps=4, seed=12, validate=True)
        u = srv.submit(engine.StagFluxTransExciton(8, PHI, 0.1, q=(4, 4)), walkers=16, sweeps=2, therm_sweeps=2,
                       seed=13, validate=True)
        r, s = srv.wait(t), srv.wait(u)
        with pytest.raises(engine.GvError):
            srv.submit(gs(8, PHI, 0.1), walkers=8, sweeps=4, meas=7)      # meas must divide L*L
    assert r["status"] == 0 and s["status"] == 0, (r, s)
    assert 0 <= r["validation_error"] < 1e-5
    assert 0 <= s["validation_error"] < 1e-3


def test_jobs_driven_from_concurrent_threads(engine):
    """Jobs of different sizes created, started and measured from several host
    threads at once (as the server's helper threads do): kernels shared by the
    jobs are launched with different shared-memory sizes from different
    threads, and every launch must succeed."""
    import concurrent.futures as cf

    def work(args):
        L, ch, seed = args
        wav = (engine.StagFluxTransExciton(L, PHI, 0.1, q=(L // 2, L // 2)) if ch == "trans"
               else engine.StagFluxGroundState(L, PHI, 0.1))
        for _ in range(6):
            j = engine.Job(wav, walkers=8, seed=seed, precision="fp64")
            j.set_measurements(1)
            j.init_walkers()
            j.walk(L * L, L * L)
            j.close()
        return True

    jobs = [(8, "gs", 1), (10, "gs", 2), (8, "trans", 3), (10, "trans", 4), (12, "gs", 5), (6, "trans", 6)]
    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        assert all(ex.map(work, jobs))
