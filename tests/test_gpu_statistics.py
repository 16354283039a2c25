"""Statistical comparison for the plain method (L = 8, one walker, phi = 0.25 pi,
neel = 0.1, FP64 re-inversion every L^2 accepted exchanges): the GPU FP64
engine over 1e5 measured sweeps of ProjHeis, StagMagnZ and StatSpinStruct
(after 200 L^2 thermalisation steps) against the oracle over a shorter run of
the same chain.  Each run is cut into equal bins (one measuring
MetroMC::Walk each, so the quantities restart per bin); the estimate is the
mean of the bin averages and its error the standard error over bins, the
estimator of the reference's post-processing, which bunches samples of equal
statistics and averages within bunches (tools/vmc_postproc/load.py:58-94).
Bar: |mean_gpu - mean_oracle| <= 4 sqrt(err_gpu^2 + err_oracle^2) for E/site,
the staggered magnetisation and the staggered structure factor
S_zz(pi, pi) = sum_ij e_i e_j <S^z_i S^z_j> / Ns (e_i = (-1)^(x + y)).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

L, PHI, NEEL, SEED = 8, 0.25 * math.pi, 0.1, 1234
NS = L * L
EPS = np.array([(-1) ** ((v % L) + (v // L)) for v in range(NS)], dtype=float)


def _szz_pipi(ss):
    szz = ss.reshape(5, NS, NS)[0].real
    return float(EPS @ szz @ EPS) / NS


def _binned(x):
    x = np.asarray(x, dtype=float)
    return x.mean(), x.std(ddof=1) / math.sqrt(len(x))


def _gpu_bins(engine, nbins, sweeps):
    job = engine.Job(engine.StagFluxGroundState(L, PHI, NEEL), walkers=1, seed=SEED, precision="fp64",
                     reinv_every=NS)
    job.set_measurements(7)
    job.init_walkers()
    job.walk(200 * NS, 0)
    e, m, s = [], [], []
    for _ in range(nbins):
        job.walk(sweeps * NS, NS)
        pj, n = job.projheis()
        sm, nsm = job.stagmagn()
        ss, nss = job.statspin()
        assert n[0] == nsm[0] == nss == sweeps
        e.append(pj[0, 0].real / n[0])
        m.append(sm[0].real / nsm[0])
        s.append(_szz_pipi(ss / nss))
    return e, m, s


def _oracle_bins(oracle, nbins, sweeps):
    o = oracle.OracleChain(L, PHI, NEEL, seed=SEED, walker=0)
    assert o.random_start() == 0
    o.walk(200 * NS, reinv_every=NS)
    e, m, s = [], [], []
    for _ in range(nbins):
        o.walk(sweeps * NS, meas=NS, mask=7, reinv_every=NS)
        pj, n = o.projheis()
        sm, nsm = o.stagmagn()
        ss, nss = o.statspin()
        assert n == nsm == nss == sweeps
        e.append(pj[0, 0].real / n)
        m.append(sm.real / nsm)
        s.append(_szz_pipi(ss / nss))
    return e, m, s


def test_plain_method_statistics(engine, oracle):
    g = _gpu_bins(engine, 100, 1000)          # 1e5 measured sweeps
    o = _oracle_bins(oracle, 40, 250)         # 1e4 measured sweeps
    for name, a, b in zip(("E/site", "m_s", "S_zz(pi,pi)"), g, o):
        (ma, ea), (mb, eb) = _binned(a), _binned(b)
        print("%-12s GPU %.6f +- %.6f   oracle %.6f +- %.6f" % (name, ma, ea, mb, eb))
        assert ea > 0 and eb > 0
        assert abs(ma - mb) <= 4.0 * math.hypot(ea, eb), (name, ma, ea, mb, eb)
    # the GPU run's own precision on E/site (1e5 sweeps, one chain)
    assert _binned(g[0])[1] < 2e-3
