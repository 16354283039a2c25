"""CUDA-graph replay of walk calls (GV_FLAG_CUDA_GRAPHS): the replayed kernels
are the directly enqueued ones, so the chains, amplitudes, inverses and
quantity sums are bit-identical with and without graphs."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _run(engine, make, mask, graphs):
    j = make(graphs)
    j.set_measurements(mask)
    j.init_walkers()
    L2 = j.Ns
    for _ in range(3):
        j.walk(L2, 0)
    j.walk(L2 * 2, L2)
    j.walk_continue(L2 * 2, L2)
    j.walk_continue(L2 * 2, L2)
    out = dict(config=j.config(), counts=j.counts(), amp=j.amplitude(), pj=j.projheis(), sm=j.stagmagn(),
               inv=j.inverse(1, 0), stats=j.graph_stats())
    if mask & 4:
        out["ss"] = j.statspin()
    j.close()
    return out


CASES = {
    "resident": (lambda e, g: e.Job(e.StagFluxGroundState(8, PHI, 0.1), walkers=16, seed=3, precision="mixed",
                                    reinv_every=32, deferred_reinversion=True, cuda_graphs=g), 7),
    "fp64": (lambda e, g: e.Job(e.StagFluxGroundState(8, PHI, 0.1), walkers=8, seed=4, precision="fp64",
                                reinv_every=64, cuda_graphs=g), 3),
    "exciton": (lambda e, g: e.Job(e.StagFluxTransExciton(8, PHI, 0.1, q=(4, 4)), walkers=8, seed=5,
                                   precision="mixed", reinv_every=32, drift_threshold=1e-5, cuda_graphs=g), 3),
    # longitudinal exciton: the measuring calls capture the tensor-core bond sums too
    "long": (lambda e, g: e.Job(e.StagFluxLongExciton(8, PHI, 0.1, q=(4, 4)), walkers=8, seed=6,
                                precision="mixed", reinv_every=32, drift_threshold=1e-5, cuda_graphs=g), 3),
}


@pytest.mark.parametrize("case", list(CASES))
def test_graph_replay_is_bit_identical(engine, case):
    make, mask = CASES[case]
    a = _run(engine, lambda g: make(engine, g), mask, False)
    b = _run(engine, lambda g: make(engine, g), mask, True)
    for k in a:
        if k == "stats":
            continue
        if k == "ss":
            # job-wide sums: the tensor-core pair products are added through FP32
            # staging atomics, so the two runs agree up to FP32 summation order
            np.testing.assert_allclose(a[k][0], b[k][0], rtol=1e-6, atol=1e-6 * np.abs(b[k][0]).max())
            continue
        va, vb = a[k], b[k]
        for x, y in (zip(va, vb) if isinstance(va, tuple) else [(va, vb)]):
            assert np.array_equal(x, y), k
    cached, replays = b["stats"]
    assert cached == 3 and replays == 6          # three distinct calls, six calls
    assert a["stats"] == (0, 0)


def test_autotune_times_the_variants_and_remembers(engine):
    wav = engine.StagFluxGroundState(8, PHI, 0.1)
    mk = lambda: engine.Job(wav, walkers=96, seed=11, precision="mixed", reinv_every=64,
                            deferred_reinversion=True)
    j = mk()
    name, times = j.autotune(steps=64)
    assert set(times) == {"streaming", "streaming-256", "streaming-delayed", "streaming-256-delayed", "on-chip"}
    assert name == min(times, key=times.get)
    j.init_walkers()
    j.walk(64 * 4, 0)
    assert (j.status() == 0).all() and j.drift().max() < 1e-3
    again, t2 = mk().autotune(steps=64)      # remembered for this shape: nothing timed
    assert again == name and t2 == {}
    # the plain form has no on-chip variant; the exciton channel has nothing to choose
    n64, t64 = engine.Job(wav, walkers=40, seed=11, precision="fp64").autotune(steps=32)
    assert "on-chip" not in t64 and n64 in t64
    assert engine.Job(engine.StagFluxTransExciton(8, PHI, 0.1, q=(4, 4)), walkers=8, seed=1,
                      precision="mixed").autotune() == (None, {})
