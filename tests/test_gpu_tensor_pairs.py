"""StatSpinStruct pair ratios from the split-TF32 tensor-core G = Phi A^-1
products (k_statspin_tc) against the FP32 CUDA-core dot products
(scalar_pairs=True) and the FP64 engine on the same configurations.

Bars (stated against the largest entry of each sum):
  * szz and the occupation diagonals are integer counts: identical;
  * s+- / s-+ of the tensor-core form vs the FP32 dot products on the same
    FP32 inverses: 1e-5 (the split recovers FP32 accuracy; plain TF32 would
    sit near 1e-3);
  * vs FP64 inverses of the same configurations: 5e-5 (adds the FP32
    rounding of the inverses).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PHI = 0.25 * math.pi


def _mixed(engine, L, W, seed, **kw):
    return engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=W, seed=seed, precision="mixed",
                      reinv_every=64, deferred_reinversion=True, **kw)


def _measure(job, oracle):
    job.set_measurements(oracle.MEAS_STATSPIN)
    job.reset_quantities()
    job.measure()
    return job.statspin()


@pytest.mark.parametrize("L,W", [(4, 8), (8, 24), (12, 16), (16, 40)])
def test_tensor_core_pairs_match_scalar_and_fp64(engine, oracle, L, W):
    jt = _mixed(engine, L, W, 3)
    jt.init_walkers()
    jt.walk(L * L * 4, 0)
    jt.reinvert()                       # FP32 copies of fresh FP64 inverses
    cfg = jt.config()
    js = _mixed(engine, L, W, 3, scalar_pairs=True)
    js.init_walkers(cfg)
    j64 = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=W, seed=3, precision="fp64")
    j64.init_walkers(cfg)
    st, nt = _measure(jt, oracle)
    ss, ns = _measure(js, oracle)
    s64, n64 = _measure(j64, oracle)
    assert nt == ns == n64 == 1
    st, ss, s64 = (a.reshape(5, L * L, L * L) for a in (st, ss, s64))
    # szz (and every diagonal) are counts
    assert np.array_equal(st[0], s64[0]) and np.array_equal(st[0], ss[0])
    for a in (st, ss):
        for k in (1, 2):
            assert np.array_equal(np.diag(a[k]).real, np.diag(s64[k]).real)
    scale = np.abs(s64[1:3]).max()
    assert np.abs(st[1:3] - ss[1:3]).max() < 1e-5 * scale
    assert np.abs(st[1:3] - s64[1:3]).max() < 5e-5 * scale
    assert np.abs(ss[1:3] - s64[1:3]).max() < 5e-5 * scale
    assert not st[3:].any()


def test_tensor_core_pairs_inside_the_walk(engine, oracle):
    """A measuring walk with StatSpinStruct: same chain on both paths (the
    walk does not depend on how the pairs are summed), same counts, sums equal
    to FP32 accuracy."""
    L, W = 16, 24
    jobs = [_mixed(engine, L, W, 9), _mixed(engine, L, W, 9, scalar_pairs=True)]
    out = []
    for j in jobs:
        j.set_measurements(oracle.MEAS_STATSPIN | oracle.MEAS_PROJHEIS)
        j.init_walkers()
        j.walk(L * L * 2, 0)
        j.walk(L * L * 3, L * L)
        out.append((j.statspin(), j.projheis(), j.config()))
    (st, nt), (pt, _), ct = out[0]
    (ss, ns), (ps, _), cs = out[1]
    assert nt == ns == 3
    assert np.array_equal(ct, cs) and np.array_equal(pt, ps)
    st, ss = st.reshape(5, L * L, L * L), ss.reshape(5, L * L, L * L)
    assert np.array_equal(st[0], ss[0])
    assert np.abs(st[1:3] - ss[1:3]).max() < 1e-5 * np.abs(ss[1:3]).max()


@pytest.mark.parametrize("L,q", [(8, (4, 4)), (12, (2, 2)), (16, (4, 4))])
def test_exciton_overlap_rows_on_tensor_cores(engine, oracle, L, q):
    """Exciton ProjHeis with Z = GupT^T Phi_0 from split-TF32 tensor-core
    products (k_trans_z_tc) against the FP32 CUDA-core product on the same
    FP32 state (2e-5 of the largest H / O entry) and against the FP64 engine
    on the same configurations (H and O do not depend on the current state)."""
    W = 12
    wav = engine.StagFluxTransExciton(L, PHI, 0.1, q=q)
    mk = lambda prec, **kw: engine.Job(wav, walkers=W, seed=21, precision=prec, reinv_every=64,
                                       deferred_reinversion=True, **kw)
    j0 = mk("mixed")
    j0.init_walkers()
    j0.walk(L * L * 2, 0)
    cfg = j0.config()
    out = []
    for j in (mk("mixed"), mk("mixed", scalar_pairs=True), mk("fp64")):
        j.init_walkers(cfg)
        j.set_measurements(oracle.MEAS_PROJHEIS)
        j.reset_quantities()
        j.measure()
        pj, n = j.projheis()
        assert (n == 1).all()
        out.append(pj)
    pt, ps, p64 = out
    scale = np.abs(p64).max(axis=(1, 2), keepdims=True)
    assert (np.abs(pt - ps) / scale).max() < 2e-5
    assert (np.abs(pt - p64) / scale).max() < 1e-3


def test_bounded_wait_gives_up_with_a_status(engine, oracle):
    """The tensor-core kernel's mbarrier waits are bounded: with a poll budget
    of zero every wait gives up at once, the walker each CTA was on and those
    it did not reach report GV_ERR_TIMEOUT (host-visible status, no hang, no
    fault: the MMAs issued still finish before the kernel frees its tensor
    memory), and the same job then measures normally again with the default
    budget."""
    L, W = 8, 24
    job = _mixed(engine, L, W, 3)
    job.init_walkers()
    job.walk(L * L * 2, 0)
    job.reinvert()
    cfg = job.config()
    job.set_measurements(oracle.MEAS_STATSPIN)
    job.reset_quantities()
    job.set_wait_limit(0)
    with pytest.raises(engine.GvError) as err:
        job.measure()
    assert err.value.status == 6
    st = job.status()
    assert (st == 6).any() and set(st.tolist()) <= {0, 6}
    job.set_wait_limit(-1)
    job.init_walkers(cfg)                 # clears the statuses, fresh FP64 inverses
    ok, n = _measure(job, oracle)
    assert n == 1 and (job.status() == 0).all()
    ref = _mixed(engine, L, W, 3)
    ref.init_walkers(cfg)
    want, _ = _measure(ref, oracle)
    # the job-wide sums go through FP32 staging atomics over walkers (folded into
    # FP64 after each measurement): equal up to FP32 summation order
    assert np.abs(ok - want).max() <= 1e-6 * np.abs(want).max()


@pytest.mark.parametrize("L,W", [(8, 24), (16, 40)])
def test_tensor_core_projheis(engine, oracle, L, W):
    """GV_FLAG_TC_PROJHEIS: ProjHeis from the split-TF32 tensor-core pair
    products (G = Phi A^-1, nearest-neighbour pairs) equals the per-particle
    FP32 dot products on the same FP32 inverses to 5e-6 in E/site, and fresh
    FP64 inverses of the same configurations to 1e-5; in a walk it measures
    once per measurement point."""
    jt = _mixed(engine, L, W, 5, tc_projheis=True)
    jt.set_measurements(oracle.MEAS_PROJHEIS | oracle.MEAS_STAGMAGN)
    jt.init_walkers()
    jt.walk(L * L * 4, L * L)
    pj, n = jt.projheis()
    sm, ns = jt.stagmagn()
    assert (n == 4).all() and (ns == 4).all() and np.isfinite(pj).all()
    jt.reinvert()
    cfg = jt.config()
    jt.reset_quantities()
    jt.measure()
    e_tc = jt.projheis()[0][:, 0].real
    jc = _mixed(engine, L, W, 5)
    jc.set_measurements(oracle.MEAS_PROJHEIS)
    jc.init_walkers(cfg)
    jc.measure()
    e_cc = jc.projheis()[0][:, 0].real
    j64 = engine.Job(engine.StagFluxGroundState(L, PHI, 0.1), walkers=W, seed=5, precision="fp64")
    j64.set_measurements(oracle.MEAS_PROJHEIS)
    j64.init_walkers(cfg)
    j64.measure()
    e64 = j64.projheis()[0][:, 0].real
    assert np.abs(e_tc - e_cc).max() < 5e-6
    assert np.abs(e_tc - e64).max() < 1e-5


def test_tensor_core_projheis_rejected_where_it_does_not_apply(engine):
    with pytest.raises(engine.GvError):
        engine.Job(engine.StagFluxGroundState(8, PHI, 0.1), walkers=2, seed=1, precision="fp64", tc_projheis=True)
    with pytest.raises(engine.GvError):
        engine.Job(engine.StagFluxGroundState(20, PHI, 0.1), walkers=2, seed=1, precision="mixed", tc_projheis=True)


def test_exciton_overlap_rows_bounded_wait(engine, oracle):
    """The transverse exciton's tensor-core overlap rows (k_trans_z_tc) give up
    at a zero poll budget with GV_ERR_TIMEOUT on the walker each CTA was on and
    on those it did not reach, so the measurement reads no unwritten rows; the
    job measures as a fresh one afterwards."""
    L, W = 8, 12
    wav = engine.StagFluxTransExciton(L, PHI, 0.1, q=(4, 4))
    mk = lambda: engine.Job(wav, walkers=W, seed=31, precision="mixed", reinv_every=64, deferred_reinversion=True)
    job = mk()
    job.init_walkers()
    job.walk(L * L * 2, 0)
    cfg = job.config()
    job.set_measurements(oracle.MEAS_PROJHEIS)
    job.reset_quantities()
    job.set_wait_limit(0)
    with pytest.raises(engine.GvError) as err:
        job.measure()
    assert err.value.status == 6
    st = job.status()
    assert (st == 6).all()   # one walker per CTA here (W < SMs): every walker's wait ran out
    job.set_wait_limit(-1)
    job.init_walkers(cfg)
    job.reset_quantities()
    job.measure()
    got, n = job.projheis()
    assert (n == 1).all() and (job.status() == 0).all()
    ref = mk()
    ref.init_walkers(cfg)
    ref.set_measurements(oracle.MEAS_PROJHEIS)
    ref.reset_quantities()
    ref.measure()
    want, _ = ref.projheis()
    assert np.array_equal(got, want)
    job.close()
    ref.close()
