"""Result files from a real walk: vmc.cpp's sample loop (vmc.cpp:299-313:
Walk, every quantity's save, data attributes rej / time / statistics, Write)
through gpvmc_gb300.FileManager; every dataset equals the mean of the saves of
its sample, per walker (calc rank = walker + 1)."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("channel", ["groundstate", "trans"])
def test_sample_loop_files(engine, tmp_path, channel):
    from gpvmc_gb300 import output
    L, W, saves, stat = 8, 8, 2, 3
    if channel == "trans":
        wav = engine.StagFluxTransExciton(L, 0.25 * math.pi, 0.1, q=(4, 4))
    else:
        wav = engine.StagFluxGroundState(L, 0.25 * math.pi, 0.1)
    job = engine.Job(wav, walkers=W, seed=17, precision="mixed", reinv_every=L * L, drift_threshold=1e-5)
    st = engine.LatticeStepper(job)
    mc = engine.MetroMC(st)
    qs = [engine.ProjHeis(st), engine.StagMagnZ(st)]
    if channel == "groundstate":
        qs.append(engine.StatSpinStruct(st))
    for q in qs:
        mc.AddQuantity(q)
    job.init_walkers()
    fm = engine.FileManager(str(tmp_path), prefix=0, backend="tree")
    fm.StatPerSample(saves)
    fm.FileAttribute("L", L)
    fm.FileAttribute("channel", channel)
    mc.Walk(L * L * 4, 0)
    expect = {}
    for sample in range(2):
        for m in range(saves):
            job.reset_quantities()
            mc.Walk(L * L * stat, L * L)
            vals = {type(q).__name__: q.save() for q in qs}
            output.save_quantities(fm, qs)
            for k, v in vals.items():
                expect.setdefault((k, sample), []).append(np.asarray(v))
            fm.DataAttribute("rej", mc.Rejection())
            fm.DataAttribute("time", 0.0)
            fm.DataAttribute("statistics", (m + 1) * stat)
            fm.Write()
    assert (job.status() == 0).all()
    for q in qs:
        name = type(q).__name__
        fattrs, data = output.read_tree(fm.path(name))
        assert fattrs["type"] == name and fattrs["channel"] == channel
        ranks = [1] if name == "StatSpinStruct" else range(1, W + 1)
        for r in ranks:
            for sample in (0, 1):
                arr, attrs = data["/rank-%d/data-%d" % (r, sample)]
                assert np.allclose(attrs["statistics"], [saves * stat])
                z = arr[:, 0::2] + 1j * arr[:, 1::2]
                mean = np.mean(expect[(name, sample)], axis=0)
                ref = mean.reshape(5, -1) if name == "StatSpinStruct" else mean[r - 1]
                assert np.allclose(z.ravel(), np.ravel(ref), rtol=1e-12, atol=1e-15)
                assert np.isfinite(z).all()
    # E/site of the ground state is the real part of H / O (ProjHeis.cpp:143)
    if channel == "groundstate":
        arr, _ = output.read_tree(fm.path("ProjHeis"))[1]["/rank-1/data-1"]
        assert -1.0 < arr[0, 0] < 0.0
    job.close()
