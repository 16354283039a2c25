#!/usr/bin/env python
"""Benchmark of the GB300 engine on the gpvmc sampling hot path.

Workload (one GPU): L = 16 square lattice (256 sites, 128 x 128 complex
Slater matrices per spin), staggered-flux ground state, 2048 independent
walkers with per-walker phi ~ U[0.1, 0.4) pi and neel ~ U[0, 0.15) (Philox
stream 2), ProjHeis measured once per sweep (every L^2 = 256 Metropolis
steps), FP64 re-inversion after every 128 accepted exchanges.  Inputs are
synthetic (seeded Philox start configurations); nothing is read from disk.

One bench "step" = one sweep of every walker = 2048 * 256 Metropolis steps
(MetroMC::Step).  value = Metropolis steps/s of the mixed-precision engine
(FP32 inverses and Sherman-Morrison updates, FP64 re-inversion), with the
plain FP64 engine measured on the same workload beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

For N > 1 (torchrun) every rank runs an independent replica of the workload
with its own walker ids (walkers are independent chains: no data-path
collective); value = all ranks' steps / max rank time.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Metropolis steps/s, L=16×2048 walkers, mixed vs FP64 on GB300 @ΔE≤1e-5; p99 lat"
L, WALKERS, SWEEP = 16, 2048, 256
PHI_RANGE = (0.1 * math.pi, 0.4 * math.pi)
NEEL_RANGE = (0.0, 0.15)
REINV = 128
DRIFT_THRESHOLD = 1e-5
THERM_SWEEPS = 16   # untimed thermalisation before the warm-up steps, every GPU arm alike
SEED = 20261203


PRECISION_MODES = {
    "mixed": "mixed: FP32 inverses, ratios and Sherman-Morrison updates; FP64 drift check every 128 accepted "
             "exchanges, FP64 re-inversion when ||A A^-1 - I||_max > %g" % DRIFT_THRESHOLD,
    "fp64": "fp64: FP64 inverses, ratios and Sherman-Morrison updates, no re-inversion (as the reference: "
            "vmc.cpp inverts only at the start)",
}


def workload_config(precision):
    """The bench configuration; arms differ only in `precision` (which names
    the re-inversion rule that belongs to each precision)."""
    return {"workload": "staggered-flux ground state L=16 (128x128 complex per spin), 2048 walkers, "
                        "phi~U[0.1,0.4)pi, neel~U[0,0.15), ProjHeis every sweep",
            "L": L, "walkers": WALKERS, "sweep_steps": SWEEP, "precision": PRECISION_MODES[precision],
            "thermalisation_sweeps": THERM_SWEEPS,
            "step": "one sweep of every walker (2048*256 Metropolis steps)",
            "l2": "inputs larger than L2: walker inverses >= 512 MiB"}


# ---------------------------------------------------------------------------
# CPU side: the oracle port (the reference's algorithm restated in C) timed on
# the host cores.  Runs in spawned processes before any GPU work.

def _cpu_chain(args):
    walker, sweeps, measure, reinv = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol   # the oracle's own Philox: no engine library in this process
    u_phi = ol.uniform_at(SEED, walker, 2, 0)
    u_neel = ol.uniform_at(SEED, walker, 2, 1)
    phi = PHI_RANGE[0] + (PHI_RANGE[1] - PHI_RANGE[0]) * u_phi
    neel = NEEL_RANGE[0] + (NEEL_RANGE[1] - NEEL_RANGE[0]) * u_neel
    o = ol.OracleChain(L, phi, neel, seed=SEED, walker=walker, timing_build=True)
    if o.random_start():
        return 0, 0.0
    t0 = time.perf_counter()
    o.walk(SWEEP * sweeps, meas=SWEEP if measure else 0, mask=ol.MEAS_PROJHEIS if measure else 0,
           reinv_every=reinv)
    return SWEEP * sweeps, time.perf_counter() - t0


def cpu_baseline(cores, sweeps, reinv=0):
    """The reference's CPU path (its algorithm restated in C, the timing build)
    on every host core: one single-threaded chain per core, concurrently, as
    the reference runs one chain per MPI rank; no re-inversion (reinv = 0), as
    the reference."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_chain, [(w, sweeps, True, reinv) for w in range(cores)])
        wall = time.perf_counter() - t0
    rates = [r[0] / r[1] for r in res if r[1] > 0]
    # chains run concurrently, one per core: aggregate = sum of per-chain rates
    return {"value": sum(rates), "unit": "steps/s", "cores": cores, "kind": "port",
            "per_core": statistics.mean(rates), "wall_s": wall,
            "sample": "%d independent L=16 chains (one per core, walkers 0..%d of the workload, the same Philox "
                      "streams), %d sweeps each with ProjHeis per sweep, %s; oracle/vmc_oracle.c timing build "
                      "(-O3, inline complex arithmetic)" % (cores, cores - 1, sweeps,
                                                            "no re-inversion" if not reinv else
                                                            "re-inversion every %d accepted moves" % reinv)}


# ---------------------------------------------------------------------------
# GPU side

class Clocks:
    """nvidia-smi samples (every 20 ms) kept when their timestamp falls inside
    the timed region [t0, t1] (time.time()); the sampler is started before the
    warm-up so that its own start-up does not eat the region."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        self.first = ""
        if self.proc:   # wait (3 s at most) until the sampler is producing
            import select
            r, _, _ = select.select([self.proc.stdout], [], [], 3.0)
            if r:
                self.first = self.proc.stdout.readline()
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()
            self.out = self.first + (self.out or "")

    @staticmethod
    def _epoch(ts):
        try:
            base, _, frac = ts.partition(".")
            return time.mktime(time.strptime(base, "%Y/%m/%d %H:%M:%S")) + (float("0." + frac) if frac else 0.0)
        except ValueError:
            return None

    def summary(self, t0=None, t1=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            t = self._epoch(f[0])
            if t0 is not None and t is not None and not (t0 - 0.01 <= t <= t1 + 0.01):
                continue
            try:
                sm.append(float(f[2]))
                mx.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[6:10]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons), "interval_ms": 20}


def block_measure_ms(job, nm):
    """Kernel time of one measurement, mean over nm back-to-back measure() calls
    (each launches the same kernels).  Each call ends with a synchronisation, so
    its first event is recorded on an idle stream: a host stall before the launch
    would be counted as kernel time.  Measurements above four times the median
    are such stalls (a block's fold adds under a factor two); they are left out
    and counted."""
    import numpy as np
    job.timer_start()
    for _ in range(nm):
        job.measure()
    job.timer_stop()
    per = job.kernel_times(2).reshape(nm, -1).sum(axis=1)
    keep = per <= 4.0 * np.median(per)
    return float(per[keep].mean()), int((~keep).sum())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_job(g, precision, rank, policy="drift"):
    from gpvmc_gb300.replicas import walker_base
    wav = g.StagFluxGroundState(L, 0.25 * math.pi, 0.0)
    job = g.Job(wav, walkers=WALKERS, seed=SEED, precision=precision, reinv_every=REINV if policy != "none" else 0,
                walker_base=walker_base(rank, WALKERS), phi_range=PHI_RANGE, neel_range=NEEL_RANGE,
                deferred_reinversion=True, drift_threshold=DRIFT_THRESHOLD if policy == "drift" else None,
                delayed_updates=False)
    job.set_measurements(1)
    return job


def delta_e(g, job, rank):
    """|E/site| difference between the engine's estimator on its own
    (drifted) inverses and the FP64 engine on fresh FP64 inverses of the
    same configurations, per walker."""
    import numpy as np
    job.reset_quantities()
    job.measure()
    pj, n = job.projheis()
    e_mixed = pj[:, 0].real / np.maximum(n, 1)
    ref = make_job(g, "fp64", rank, policy="none")
    ref.init_walkers(job.config())
    ref.measure()
    pr, nr = ref.projheis()
    e_ref = pr[:, 0].real / np.maximum(nr, 1)
    ref.close()
    d = np.abs(e_mixed - e_ref)
    return {"max": float(d.max()), "mean": float(d.mean()), "walkers": int(len(d)),
            "bar": 1e-5, "within_bar": bool(d.max() <= 1e-5),
            "note": "same configurations, ProjHeis E/site from the engine's inverses vs fresh FP64 inverses"}


def run_gpu(g, precision, steps, warmup, rank, clocks_index=None, policy="drift", check_delta=False):
    job = make_job(g, precision, rank, policy)
    job.init_walkers()
    clk = Clocks(clocks_index) if clocks_index is not None else None
    if clk:
        clk.__enter__()
    for _ in range(THERM_SWEEPS):
        job.walk(SWEEP, 0, sync=False)
    for _ in range(warmup):
        job.walk(SWEEP, SWEEP, sync=False)
    job.synchronize()
    c0 = job.counts().sum(axis=0)
    lat = []
    job.timer_start()
    e0 = time.time()
    t0 = time.perf_counter()
    for _ in range(steps):
        t = time.perf_counter()
        job.walk(SWEEP, SWEEP, sync=False)
        lat.append(t)
    ms, launches = job.timer_stop()
    wall = time.perf_counter() - t0
    e1 = time.time()
    walk_ms, walk_n = job.kernel_ms(0)
    inv_ms, inv_n = job.kernel_ms(1)
    import numpy as np
    sweep_each = np.array(job.kernel_times(0))
    if clk:
        clk.__exit__()
    job.synchronize()
    c1 = job.counts().sum(axis=0)
    pj, n = job.projheis()
    e_site = float((pj[:, 0].real / n).mean())
    d = (c1 - c0).astype(float)
    drift_seen, nchecks = job.drift_checks()
    res = {"ms": ms, "wall_s": wall, "launches": launches, "steps": float(d[0]), "walk_ms": walk_ms,
           "walk_launches": walk_n, "inv_ms": inv_ms, "inv_launches": inv_n,
           "sweep_p50_ms": float(np.percentile(sweep_each, 50)) if len(sweep_each) else None,
           "sweep_p99_ms": float(np.percentile(sweep_each, 99)) if len(sweep_each) else None,
           "checks_without_reinversion": int(nchecks.sum()), "max_drift_at_check": float(drift_seen.max()),
           "p_acc": d[1] / d[0], "p_ap": (d[1] + d[3]) / d[0], "reinv": float(d[4]), "e_site": e_site,
           "clocks": clk.summary(e0, e1) if clk else None}
    if check_delta:
        res["delta_e_site"] = delta_e(g, job, rank)
    job.close()
    return res


def run_e2e(g, precision, steps, rank):
    """Through the public API with host buffers: job creation (host tables ->
    device), host random start configurations -> device, FP64 LU start, then
    each step one sweep and a device->host read of the per-walker results.
    Bytes are the library's own count of the host<->device copies it issued
    inside the timed region (gv_transfer_bytes)."""
    import numpy as np
    from gpvmc_gb300 import _lib
    h0, d0 = _lib.transfer_bytes()
    t0 = time.perf_counter()
    job = make_job(g, precision, rank)
    job.init_walkers()
    results = []
    for _ in range(steps):
        job.walk(SWEEP, SWEEP, sync=False)
        pj, n = job.projheis()
        results.append(pj[:, 0].real / np.maximum(n, 1))
    wall = time.perf_counter() - t0
    h1, d1 = _lib.transfer_bytes()
    job.close()
    return {"value": WALKERS * SWEEP * steps / wall, "unit": "steps/s", "h2d_bytes_per_step": (h1 - h0) // steps,
            "d2h_bytes_per_step": (d1 - d0) // steps, "wall_s": wall,
            "h2d_bytes": h1 - h0, "d2h_bytes": d1 - d0,
            "includes": "job creation + start upload + FP64 LU start amortised over the steps; bytes counted "
                        "by the library at every copy it issued"}


# ---------------------------------------------------------------------------
# Batched FP64 vs FP32 Sherman-Morrison at L=12: 4096 walkers, phi = 0.25 pi,
# neel = 0.05, FP64 re-inversion every 64 accepted moves, ProjHeis every sweep.

C2_L, C2_WALKERS, C2_NEEL, C2_REINV = 12, 4096, 0.05, 64


def run_config2(g, sweeps=8):
    """Both precisions on the same seeds (kernel time between CUDA events):
    the plain FP64 engine without re-inversion, as the reference runs, and the
    mixed form with the specified cadence (FP64 re-inversion every 64 accepted
    moves) and with the drift-checked policy (every 64 accepted moves the
    residual is estimated and the walker re-inverted only above 1e-5); the
    mixed jobs' ||A A^-1 - I||_max at the end of the timed walk and their
    E/site against an FP64 job started on the same configurations."""
    import numpy as np
    sweep = C2_L * C2_L
    out = {"workload": "staggered-flux ground state L=12 (72x72 complex per spin), phi=0.25pi, neel=0.05, "
                       "4096 walkers, ProjHeis every sweep, FP64 re-inversion every 64 accepted moves",
           "unit": "steps/s", "sweeps": sweeps}
    wav = g.StagFluxGroundState(C2_L, 0.25 * math.pi, C2_NEEL)
    for key, prec, thr in (("mixed", "mixed", None), ("mixed_drift_checked", "mixed", DRIFT_THRESHOLD),
                           ("fp64", "fp64", None)):
        # the plain FP64 engine, as the headline's: no re-inversion (the reference never re-inverts)
        job = g.Job(wav, walkers=C2_WALKERS, seed=SEED, precision=prec, reinv_every=C2_REINV if prec == "mixed" else 0,
                    deferred_reinversion=True, drift_threshold=thr)
        job.set_measurements(1)
        job.init_walkers()
        for _ in range(4):
            job.walk(sweep, 0, sync=False)
        job.synchronize()
        c0 = job.counts().sum(axis=0)
        job.timer_start()
        for _ in range(sweeps):
            job.walk(sweep, sweep, sync=False)
        ms, _ = job.timer_stop()
        wk, _ = job.kernel_ms(0)
        rk, _ = job.kernel_ms(1)
        d = (job.counts().sum(axis=0) - c0).astype(float)
        out[key] = {"value": C2_WALKERS * sweep * sweeps / (ms * 1e-3), "ms_per_sweep": ms / sweeps,
                    "walk_ms_per_sweep": wk / sweeps, "reinversion_ms_per_sweep": rk / sweeps,
                    "reinversions_per_walker_sweep": d[4] / (C2_WALKERS * sweeps), "p_acc": d[1] / d[0]}
        if prec == "mixed":
            out[key]["inverse_residual_max"] = float(job.drift().max())
            cfg = job.config()
            job.reset_quantities()
            job.measure()
            pm, nm = job.projheis()
            ref = g.Job(wav, walkers=C2_WALKERS, seed=SEED, precision="fp64")
            ref.set_measurements(1)
            ref.init_walkers(cfg)
            ref.measure()
            pr, nr = ref.projheis()
            ref.close()
            dd = np.abs(pm[:, 0].real / np.maximum(nm, 1) - pr[:, 0].real / np.maximum(nr, 1))
            out[key]["delta_e_site_vs_fp64"] = {"max": float(dd.max()), "mean": float(dd.mean())}
        job.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["mixed_drift_checked_over_fp64"] = out["mixed_drift_checked"]["value"] / out["fp64"]["value"]
    return out


# ---------------------------------------------------------------------------
# Exciton channel: transverse exciton L=16, q = (n, n) for n = 0..7, 512 walkers
# per momentum (N0 = 129, N1 = 127, Nexc = 128), ProjHeis H / O every sweep.

EXC_QS = [(n, n) for n in range(8)]
EXC_WALKERS = 512
HO_BLOCK = 32        # measurements per FP32 H / O block of a mixed exciton job (kHoSlots in the engine)


def _cpu_exciton_chain(args):
    walker, sweeps = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol
    q = EXC_QS[walker % len(EXC_QS)]
    o = ol.OracleChain(L, 0.25 * math.pi, 0.1, channel=ol.TRANS, q=q, seed=SEED, walker=walker, timing_build=True)
    if o.random_start():
        return 0, 0.0
    t0 = time.perf_counter()
    o.walk(SWEEP * sweeps, meas=SWEEP, mask=ol.MEAS_PROJHEIS)
    return SWEEP * sweeps, time.perf_counter() - t0


def cpu_exciton_baseline(cores, sweeps):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_exciton_chain, [(w, sweeps) for w in range(cores)])
    rates = [r[0] / r[1] for r in res if r[1] > 0]
    return {"value": sum(rates), "unit": "steps/s", "cores": cores, "kind": "port", "per_core": statistics.mean(rates),
            "sample": "%d independent exciton chains L=16 (q=(n,n) round robin), %d sweeps each with ProjHeis "
                      "H/O per sweep" % (cores, sweeps)}


def exciton_jobs(g, precision, walkers=EXC_WALKERS, qs=EXC_QS):
    jobs = []
    for i, q in enumerate(qs):
        wav = g.StagFluxTransExciton(L, 0.25 * math.pi, 0.1, q=q)
        kw = dict(reinv_every=REINV)
        if precision == "mixed":
            kw["drift_threshold"] = DRIFT_THRESHOLD
        j = g.Job(wav, walkers=walkers, seed=SEED, precision=precision, walker_base=i * walkers, **kw)
        j.set_measurements(1)
        j.init_walkers()
        jobs.append(j)
    return jobs


def run_exciton(g, sweeps, fp64_sweeps):
    """All eight momenta at once (one stream per job), wall time between
    synchronisations; the walk-kernel roofline from the q=(4,4) job alone."""
    import numpy as np
    out = {"workload": "transverse exciton L=16 (129x129 / 127x127 complex per spin, Nexc=128), "
                       "q=(n,n) n=0..7, 512 walkers per q, ProjHeis H/O (128x128 each) every sweep",
           "unit": "steps/s"}
    for prec, n in (("mixed", sweeps), ("fp64", fp64_sweeps)):
        jobs = exciton_jobs(g, prec)
        for _ in range(THERM_SWEEPS):   # thermalised as the headline walk, both arms alike
            for j in jobs:
                j.walk(SWEEP, 0, sync=False)
        for j in jobs:
            j.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            for j in jobs:
                j.walk(SWEEP, SWEEP, sync=False)
        for j in jobs:
            j.synchronize()
        wall = time.perf_counter() - t0
        steps = len(jobs) * EXC_WALKERS * SWEEP * n
        out[prec] = {"value": steps / wall, "sweeps": n, "wall_s": wall}
        if prec == "mixed":
            # single job, kernel-timed, for the walk kernel's roofline
            j = jobs[4]
            c0 = j.counts().sum(axis=0)
            j.timer_start()
            for _ in range(n):
                j.walk(SWEEP, 0, sync=False)
            ms, _ = j.timer_stop()
            wk, wn = j.kernel_ms(0)
            mk, mn = j.kernel_ms(2)
            d = (j.counts().sum(axis=0) - c0).astype(float)
            p_acc, p_ap = d[1] / d[0], (d[1] + d[3]) / d[0]
            N0, N1, Nexc, sz = L * L // 2 + 1, L * L // 2 - 1, L * L // 2, 8
            bytes_step = p_ap * (Nexc * N0 + N0 + N1 + Nexc) * sz + p_acc * 2 * (N0 * N0 + N1 * N1 + N0 * Nexc) * sz
            # complex MACs: Z = GupT^T C and the two row dots per proposal; per accepted move the
            # rank-2 updates of both inverses (column product + two rank-1 passes) and of GupT
            flops_step = 8.0 * (p_ap * (Nexc * N0 + N0 + N1 + Nexc) + p_acc * (3 * (N0 * N0 + N1 * N1) + 3 * N0 * Nexc))
            launches = max(1, wn)
            steps_launch = d[0] / launches
            ms_launch = wk / launches
            res_bytes = EXC_WALKERS * 2 * (N0 * N0 + N1 * N1 + N0 * Nexc) * sz   # on-chip state in and out
            achieved = res_bytes / (ms_launch * 1e-3) / 1e9
            peak, kind = measured_peaks()
            # the same walk on the streaming kernel (inverses and overlap rows re-read from L2 / HBM)
            jst = g.Job(g.StagFluxTransExciton(L, 0.25 * math.pi, 0.1, q=(4, 4)), walkers=EXC_WALKERS, seed=SEED,
                        precision="mixed", reinv_every=REINV, drift_threshold=DRIFT_THRESHOLD, stream_inverses=True)
            jst.init_walkers()
            jst.walk(SWEEP, 0)
            s0 = jst.counts().sum(axis=0)
            jst.timer_start()
            for _ in range(n):
                jst.walk(SWEEP, 0, sync=False)
            jst.timer_stop()
            sk, _ = jst.kernel_ms(0)
            ds = (jst.counts().sum(axis=0) - s0).astype(float)
            jst.close()
            f32_peak, mhz = fp32_peak_tflops(None)
            f32 = flops_step * steps_launch / (ms_launch * 1e-3) / 1e12
            stream_gbs = bytes_step * steps_launch / (ms_launch * 1e-3) / 1e9
            out["roofline"] = {"kernel": "k_walk_trans_res", "bound": "hbm", "achieved": achieved, "peak": peak,
                               "unit": "GB/s", "frac": achieved / peak, "peak_kind": kind,
                               "algorithmic_bytes_per_launch": res_bytes,
                               "algorithmic_bytes_what": "both inverses and the overlap rows GupT loaded at launch "
                                                         "entry and stored at exit (FP32)",
                               "binding_resource": "on-chip latency (profiles/k_walk_trans_res_L16_512walkers.md: "
                                                   "issue-active 36 %, DRAM 0.9 % of peak)",
                               "fp32": {"achieved_tflops": f32, "peak_tflops": f32_peak, "frac": f32 / f32_peak,
                                        "flops_per_step": flops_step},
                               "streaming_equivalent": {"bytes_per_step": bytes_step, "gbs": stream_gbs,
                                                        "over_hbm_peak": stream_gbs / peak},
                               "walk_ms_per_launch": ms_launch, "kernel_steps_per_s": d[0] / (wk * 1e-3),
                               "streaming_kernel_steps_per_s": ds[0] / (sk * 1e-3),
                               "p_acc": p_acc, "p_ap": p_ap, "q": [4, 4], "walkers": EXC_WALKERS}
            # H / O accuracy of the mixed form against FP64 on the same configurations
            cfg = j.config()
            j.reset_quantities()
            j.measure()
            pm, _ = j.projheis()
            ref = g.Job(g.StagFluxTransExciton(L, 0.25 * math.pi, 0.1, q=(4, 4)), walkers=EXC_WALKERS, seed=SEED,
                        precision="fp64")
            ref.set_measurements(1)
            ref.init_walkers(cfg)
            ref.reset_quantities()
            ref.measure()
            pr, _ = ref.projheis()
            err = np.abs(pm - pr).max(axis=(1, 2)) / np.abs(pr).max(axis=(1, 2))
            out["ho_error_vs_fp64"] = {"median": float(np.median(err)), "max": float(err.max()),
                                       "what": "max |H,O mixed - H,O FP64| / max |H,O FP64| per walker, one measurement"}
            ref.close()

            js = g.Job(g.StagFluxTransExciton(L, 0.25 * math.pi, 0.1, q=(4, 4)), walkers=EXC_WALKERS, seed=SEED,
                       precision="mixed", scalar_pairs=True)
            js.set_measurements(1)
            js.init_walkers(cfg)
            # a whole block of HO_BLOCK measurements: exactly one of them folds the
            # block's FP32 outer products into the FP64 H / O sums
            (mt, dt), (mc, dc) = block_measure_ms(j, HO_BLOCK), block_measure_ms(js, HO_BLOCK)
            out["measure_ms"] = {"tensor_cores": mt, "cuda_cores": mc, "stalls_dropped": dt + dc,
                                 "what": "one ProjHeis H/O measurement of the q=(4,4) job's %d walkers (kernel time, "
                                         "mean over a block of %d, the block's FP64 fold included): overlap rows "
                                         "Z = GupT^T Phi as split-TF32 tcgen05 products vs FP32 dot products on the "
                                         "CUDA cores" % (EXC_WALKERS, HO_BLOCK)}
            js.close()
        for j in jobs:
            j.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


# ---------------------------------------------------------------------------
# Longitudinal exciton (StagFluxLongExciton): L=16, q = (0,0) and (8,8)
# (257 states each, the ground state included), N0 = N1 = 128.

LONG_QS = [(0, 0), (8, 8)]
LONG_WALKERS = 256


def _cpu_long_chain(args):
    walker, sweeps = args
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle_lib as ol
    q = LONG_QS[walker % len(LONG_QS)]
    o = ol.OracleChain(L, 0.25 * math.pi, 0.1, channel=ol.LONG, q=q, seed=SEED, walker=walker, timing_build=True)
    if o.random_start():
        return 0, 0.0
    t0 = time.perf_counter()
    o.walk(sweeps, meas=0)
    return sweeps, time.perf_counter() - t0


def cpu_long_baseline(cores, steps):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_long_chain, [(w, steps) for w in range(cores)])
    rates = [r[0] / r[1] for r in res if r[1] > 0]
    return {"value": sum(rates), "unit": "steps/s", "cores": cores, "kind": "port", "per_core": statistics.mean(rates),
            "sample": "%d independent longitudinal-exciton chains L=16 (q=(0,0), (8,8) alternating), %d Metropolis "
                      "steps each, no measurement; oracle timing build" % (cores, steps)}


def run_long(g, sweeps, fp64_sweeps):
    """Both momenta at once (one stream per job), wall time between
    synchronisations, ProjHeis H/O every sweep in the measured phase; the
    mixed form's H/O error against FP64 on the same configurations."""
    import numpy as np
    out = {"workload": "longitudinal exciton L=16 (128x128 complex per spin, 257 states incl. the ground state), "
                       "q=(0,0) and (8,8), %d walkers per q, ProjHeis H/O (257x257 each) every sweep" % LONG_WALKERS,
           "unit": "steps/s"}
    for prec, n in (("mixed", sweeps), ("fp64", fp64_sweeps)):
        jobs = []
        for i, q in enumerate(LONG_QS):
            kw = dict(reinv_every=REINV)
            if prec == "mixed":
                kw["drift_threshold"] = DRIFT_THRESHOLD
            j = g.Job(g.StagFluxLongExciton(L, 0.25 * math.pi, 0.1, q=q), walkers=LONG_WALKERS, seed=SEED,
                      precision=prec, walker_base=i * LONG_WALKERS, **kw)
            j.set_measurements(1)
            j.init_walkers()
            jobs.append(j)
        for _ in range(THERM_SWEEPS):   # thermalised as the headline walk, both arms alike
            for j in jobs:
                j.walk(SWEEP, 0, sync=False)
        for j in jobs:
            j.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            for j in jobs:
                j.walk(SWEEP, SWEEP, sync=False)   # ProjHeis H / O once per sweep
        for j in jobs:
            j.synchronize()
        wall = time.perf_counter() - t0
        steps = len(jobs) * LONG_WALKERS * SWEEP * n
        j = jobs[0]
        nm = HO_BLOCK if prec == "mixed" else 1   # a mixed job folds its FP32 H/O block once in HO_BLOCK
        j.reset_quantities()
        mk, _ = block_measure_ms(j, nm)
        out[prec] = {"value": steps / wall, "sweeps": n, "wall_s": wall, "measure_ms": mk,
                     "measure_what": "one ProjHeis H/O measurement of one job's %d walkers (kernel time%s)"
                                     % (LONG_WALKERS, ", mean over a block of %d, its fold included" % nm if nm > 1 else "")}
        if prec == "mixed":
            cfg = j.config()
            j.reset_quantities()
            j.measure()
            pm, _ = j.projheis()
            ref = g.Job(g.StagFluxLongExciton(L, 0.25 * math.pi, 0.1, q=LONG_QS[0]), walkers=LONG_WALKERS, seed=SEED,
                        precision="fp64")
            ref.set_measurements(1)
            ref.init_walkers(cfg)
            ref.reset_quantities()
            ref.measure()
            pr, _ = ref.projheis()
            err = np.abs(pm - pr).max(axis=(1, 2)) / np.abs(pr).max(axis=(1, 2))
            out["ho_error_vs_fp64"] = {"median": float(np.median(err)), "max": float(err.max()),
                                       "what": "max |H,O mixed - H,O FP64| / max |H,O FP64| per walker, q=(0,0)"}
            ref.close()
        for j in jobs:
            j.close()
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


# ---------------------------------------------------------------------------
# Serving stream: Poisson arrivals (20 jobs/s) of heterogeneous requests --
# L in {8,12,16,20,24}, phi ~ U[0,0.5) pi, neel ~ U[0,0.2), ground state 80% /
# transverse exciton 20% (q on the diagonal), 64-1024 walkers (log-uniform) --
# served by the engine's request loop with footprint admission.

SERVE_JOBS = 48
SERVE_RATE = 20.0          # jobs per second
SERVE_SWEEP_SCALE = 200    # sweeps per job: log-uniform [1e3, 1e4] / 200 = [5, 50]


PAIR_MEAS = 4


def run_pairs(g, walkers):
    """StatSpinStruct on the headline workload's configurations: every
    antiparallel pair ratio of every walker, as split-TF32 tensor-core
    G = Phi A^-1 products (k_statspin_tc) and, beside it, as FP32 dot products
    on the CUDA cores; both against fresh FP64 inverses of the same
    configurations."""
    import numpy as np
    job = make_job(g, "mixed", 0)
    job.init_walkers()
    for _ in range(4):
        job.walk(SWEEP, 0, sync=False)
    job.synchronize()
    cfg = job.config()
    job.set_measurements(4)

    def timed(j, n):
        j.reset_quantities()
        j.measure()   # warm-up
        j.reset_quantities()
        j.timer_start()
        for _ in range(n):
            j.measure()
        j.timer_stop()
        ms, launches = j.kernel_ms(2)
        return ms / max(1, launches), j.statspin()[0]

    ms_tc, ss_tc = timed(job, PAIR_MEAS)
    job.close()
    from gpvmc_gb300.replicas import walker_base
    wav = g.StagFluxGroundState(L, 0.25 * math.pi, 0.0)
    common = dict(walkers=walkers, seed=SEED, reinv_every=REINV, walker_base=walker_base(0, walkers),
                  phi_range=PHI_RANGE, neel_range=NEEL_RANGE, deferred_reinversion=True)
    js = g.Job(wav, precision="mixed", scalar_pairs=True, **common)
    js.init_walkers(cfg)
    js.set_measurements(4)
    ms_sc, ss_sc = timed(js, 1)
    js.close()
    j64 = g.Job(wav, precision="fp64", **common)
    j64.init_walkers(cfg)
    j64.set_measurements(4)
    j64.reset_quantities()
    j64.measure()
    ss64 = j64.statspin()[0]
    j64.close()
    # ss_tc holds PAIR_MEAS measurements of the same configurations, ss_sc one
    scale = np.abs(ss64[1:3]).max()
    err_tc = float(np.abs(ss_tc[1:3] / PAIR_MEAS - ss64[1:3]).max() / scale)
    err_sc = float(np.abs(ss_sc[1:3] - ss64[1:3]).max() / scale)
    N = L * L // 2
    useful = 2 * 8.0 * N ** 3 * walkers              # two complex N^3 products per walker
    executed = 2 * 3 * 4 * 2.0 * 128 * N * N * walkers   # 3 split terms x 4 real products, M padded to 128
    peak_tf32 = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak_tf32 = float(json.load(f)["bf16_tflops"]) / 2
    except Exception:
        peak_tf32 = 1900.0 / 2
    tens = executed / (ms_tc * 1e-3) / 1e12
    return {"workload": "StatSpinStruct of %d walkers at L=16 (all 128x128 antiparallel pair ratios per walker), "
                        "configurations of the headline workload after 4 sweeps" % walkers,
            "kernel": "k_statspin_tc (tcgen05.mma kind::tf32, split precision, FP32 accumulation in TMEM)",
            "ms_per_measurement": ms_tc, "scalar_ms_per_measurement": ms_sc,
            "speedup_over_cuda_cores": ms_sc / ms_tc,
            "useful_tflops": useful / (ms_tc * 1e-3) / 1e12,
            "tensor_tflops_executed": tens,
            "tensor_peak_tflops": peak_tf32,
            "tensor_frac": tens / peak_tf32,
            "tensor_peak_kind": "TF32 dense = half the measured bf16 dense burst (the nominal ratio)",
            "pair_error_vs_fp64": err_tc, "scalar_pair_error_vs_fp64": err_sc,
            "error_what": "max |s+-, s-+ (engine) - same from fresh FP64 inverses| / max |s+-, s-+|"}


def run_tc_projheis(g, walkers):
    """Config 3: every sweep's ProjHeis from the split-TF32 tensor-core products
    G = Phi A^-1 (GV_FLAG_TC_PROJHEIS; the nearest-neighbour pairs of G_up G_dn^T
    are the bond ratios): time per measurement of all walkers, executed
    tensor-pipe rate, and the E/site error against fresh FP64 inverses of the
    same configurations; and the headline walk with ProjHeis taken that way."""
    import numpy as np
    from gpvmc_gb300.replicas import walker_base
    wav = g.StagFluxGroundState(L, 0.25 * math.pi, 0.0)
    common = dict(walkers=walkers, seed=SEED, reinv_every=REINV, walker_base=walker_base(0, walkers),
                  phi_range=PHI_RANGE, neel_range=NEEL_RANGE, deferred_reinversion=True)
    job = g.Job(wav, precision="mixed", drift_threshold=DRIFT_THRESHOLD, tc_projheis=True, **common)
    job.set_measurements(1)
    job.init_walkers()
    for _ in range(THERM_SWEEPS):   # thermalised as the headline walk, so that the walks compare
        job.walk(SWEEP, 0, sync=False)
    job.synchronize()
    c0 = job.counts().sum(axis=0)
    job.timer_start()
    n = 8
    for _ in range(n):
        job.walk(SWEEP, SWEEP, sync=False)
    ms, _ = job.timer_stop()
    walk_steps = float((job.counts().sum(axis=0) - c0)[0])
    meas_ms, meas_n = job.kernel_ms(2)
    cfg = job.config()
    job.reset_quantities()
    job.measure()
    e_tc = job.projheis()[0][:, 0].real
    j64 = g.Job(wav, precision="fp64", **common)
    j64.set_measurements(1)
    j64.init_walkers(cfg)
    j64.measure()
    e64 = j64.projheis()[0][:, 0].real
    j64.close()
    job.close()
    N = L * L // 2
    per = meas_ms / max(1, meas_n)
    useful = 2 * 8.0 * N ** 3 * walkers                # the two complex N^3 products restricted to used columns
    full_g = 2 * 8.0 * (L * L) * N * N * walkers        # G = Phi(Ns x N) A^-1(N x N) per spin, in full
    executed = 2 * 3 * 4 * 2.0 * 128 * N * N * walkers
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak_tf32 = float(json.load(f)["bf16_tflops"]) / 2
    except Exception:
        peak_tf32 = 1900.0 / 2
    tens = executed / (per * 1e-3) / 1e12
    d = np.abs(e_tc - e64)
    return {"workload": "ProjHeis of %d walkers at L=16 from tensor-core pair products, per-walker phi/neel, "
                        "every sweep of the headline walk" % walkers,
            "kernel": "k_statspin_tc (mode ProjHeis): tcgen05.mma kind::tf32, split precision, FP32 accumulation",
            "ms_per_measurement": per, "walk_with_tc_projheis_steps_per_s": walk_steps / (ms * 1e-3),
            "useful_tflops": useful / (per * 1e-3) / 1e12,
            "full_g_equivalent_tflops": full_g / (per * 1e-3) / 1e12,
            "tensor_tflops_executed": tens, "tensor_peak_tflops": peak_tf32, "tensor_frac": tens / peak_tf32,
            "tensor_peak_kind": "TF32 dense = half the measured bf16 dense burst (the nominal ratio)",
            "e_site_error_vs_fp64": {"max": float(d.max()), "mean": float(d.mean()), "bar": 1e-5}}


def run_graphs(g, calls=200):
    """Walk calls of a small job (L=8, 64 walkers, one sweep per call with
    ProjHeis, StagMagnZ and StatSpinStruct measured), enqueued kernel by
    kernel and replayed as one CUDA graph per call (GV_FLAG_CUDA_GRAPHS);
    host wall time of `calls` back-to-back calls."""
    out = {}
    for graphs in (False, True):
        j = g.Job(g.StagFluxGroundState(8, 0.25 * math.pi, 0.1), walkers=64, seed=SEED, precision="mixed",
                  reinv_every=REINV, deferred_reinversion=True, drift_threshold=DRIFT_THRESHOLD, cuda_graphs=graphs)
        j.set_measurements(7)
        j.init_walkers()
        for _ in range(5):
            j.walk_continue(64, 64, sync=False)
        j.synchronize()
        t0 = time.perf_counter()
        for _ in range(calls):
            j.walk_continue(64, 64, sync=False)
        j.synchronize()
        dt = time.perf_counter() - t0
        _, launches = j.last_walk_ms()
        out["graphs" if graphs else "direct"] = {"calls_per_s": calls / dt, "us_per_call": dt / calls * 1e6,
                                                 "kernels_per_call": launches,
                                                 "graph_launches_per_call": 1 if graphs else 0}
        j.close()
    out["workload"] = ("L=8, 64 walkers, mixed, one sweep per walk call with ProjHeis, StagMagnZ and "
                       "StatSpinStruct measured, %d calls back to back (host wall time)" % calls)
    return out


def run_autotune(g):
    """The autotuner on the headline configuration: every walk-kernel variant
    timed on a scratch job (608 walkers), the fastest chosen."""
    job = make_job(g, "mixed", 0)
    name, times = job.autotune(steps=SWEEP)
    job.close()
    return {"choice": name, "us_per_step_all_scratch_walkers": times,
            "what": "gv_job_autotune on L=16 mixed ground state, drift-checked re-inversion; scratch job of "
                    "min(walkers, 4 x SMs) walkers, one timed sweep after one warm-up sweep"}


def serving_requests(g, n=SERVE_JOBS, scale=SERVE_SWEEP_SCALE):
    import numpy as np
    rng = np.random.default_rng(SEED)
    reqs, t = [], 0.0
    for i in range(n):
        t += rng.exponential(1.0 / SERVE_RATE)
        L = int(rng.choice([8, 12, 16, 20, 24]))
        phi, neel = math.pi * rng.uniform(0.0, 0.5), rng.uniform(0.0, 0.2)
        if rng.uniform() < 0.2:
            qn = int(rng.integers(0, L // 2))
            wav = g.StagFluxTransExciton(L, phi, neel, q=(qn, qn))
        else:
            wav = g.StagFluxGroundState(L, phi, neel)
        walkers = int(round(math.exp(rng.uniform(math.log(64), math.log(1024)))))
        sweeps = max(1, int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e4))) / scale)))
        reqs.append((t, dict(wav=wav, walkers=walkers, sweeps=sweeps, therm_sweeps=max(1, sweeps // 5),
                             seed=SEED + i, walker_base=0, precision="mixed", validate=True)))
    return reqs


def serving_phases(reqs, res):
    """Where each request's time went (host clock): queue (submitted ->
    admitted), start (job creation, walker start, FP64 start inversions),
    walk (the walk calls, sharing the device with the other admitted jobs),
    retire (final reads, summary, FP64 validation, teardown); means by L and
    channel over the requests that finished without error, and the share of
    the admitted time (start + walk + retire) each phase took overall."""
    phases = {}
    for (t, q), r in zip(reqs, res):
        if r["status"] != 0:
            continue
        key = "L%d_%s" % (q["wav"].L, "gs" if q["wav"].channel == "groundstate" else "trans")
        d = phases.setdefault(key, {"jobs": 0, "queue_s": 0.0, "start_s": 0.0, "walk_s": 0.0, "retire_s": 0.0,
                                    "steps": 0})
        d["jobs"] += 1
        d["queue_s"] += r["t_admit"] - r["t_submit"]
        d["start_s"] += r["t_started"] - r["t_admit"]
        d["walk_s"] += r["t_walked"] - r["t_started"]
        d["retire_s"] += r["t_done"] - r["t_walked"]
        d["steps"] += r["steps"]
    tot = {k: sum(d[k] for d in phases.values()) for k in ("queue_s", "start_s", "walk_s", "retire_s")}
    for d in phases.values():
        n = d["jobs"]
        d["walk_steps_per_s"] = d["steps"] / d["walk_s"] if d["walk_s"] > 0 else None
        for k in ("queue_s", "start_s", "walk_s", "retire_s"):
            d[k] /= n
        d["steps_per_job"] = d.pop("steps") / n
    busy = tot["start_s"] + tot["walk_s"] + tot["retire_s"]
    share = {k: tot[k] / busy for k in ("start_s", "walk_s", "retire_s")} if busy > 0 else None
    return phases, share


def run_serving(g):
    import numpy as np
    reqs = serving_requests(g)
    srv = g.Server(max_jobs=32, chunk_sweeps=4)
    tickets = []
    t0 = time.perf_counter()
    for t_arr, r in reqs:
        dt = t_arr - (time.perf_counter() - t0)
        if dt > 0:
            time.sleep(dt)
        tickets.append(srv.submit(**r))
    srv.drain(1800)
    res = [srv.poll(t) for t in tickets]
    srv.close()
    ok = [r for r in res if r["status"] == 0]
    lat = np.array([r["t_done"] - r["t_submit"] for r in ok])
    queue = np.array([r["t_admit"] - r["t_submit"] for r in ok])
    span = max(r["t_done"] for r in ok) - min(r["t_submit"] for r in res)
    steps = sum(r["steps"] for r in ok)
    gs_err = [r["validation_error"] for (t, q), r in zip(reqs, res)
              if r["status"] == 0 and r["validation_error"] >= 0 and q["wav"].channel == "groundstate"]
    tr_err = [r["validation_error"] for (t, q), r in zip(reqs, res)
              if r["status"] == 0 and r["validation_error"] >= 0 and q["wav"].channel == "trans"]
    # The sustained arrival rate for the unscaled request distribution (1e3-1e4
    # sweeps): the stream kept the device saturated (queue p99 above), so its
    # steps/s is the mix's service capacity, and a queue stays bounded while
    # rate x mean steps per request < capacity.
    phases, share = serving_phases(reqs, res)
    unscaled = serving_requests(g, n=4000, scale=1)
    mean_steps = float(np.mean([q["walkers"] * (q["sweeps"] + q["therm_sweeps"]) * q["wav"].L ** 2
                                for _, q in unscaled]))
    cap = steps / span
    return {"workload": "%d requests, Poisson arrivals at %g/s, L~U{8,12,16,20,24}, phi~U[0,0.5)pi, "
                        "neel~U[0,0.2), ground state 80%% / transverse exciton 20%% (q on the diagonal), "
                        "64-1024 walkers log-uniform, sweeps log-uniform [1e3,1e4] scaled by 1/%d, mixed "
                        "precision, drift-checked FP64 re-inversion every 128 accepted moves; ProjHeis and "
                        "StagMagnZ every sweep" % (SERVE_JOBS, SERVE_RATE, SERVE_SWEEP_SCALE),
            "jobs": len(res), "failed": len(res) - len(ok),
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "queue_p50_s": float(np.percentile(queue, 50)), "queue_p99_s": float(np.percentile(queue, 99)),
            "steps_per_s": steps / span, "wall_s": span, "steps": int(steps),
            "e_site_error_vs_fp64_max": max(gs_err) if gs_err else None,
            "exciton_ho_error_vs_fp64_max": max(tr_err) if tr_err else None,
            "validated_jobs": len(gs_err) + len(tr_err),
            "phases_by_L": phases,
            "admitted_time_share": share,
            "unscaled": {"mean_steps_per_request": mean_steps,
                         "sustained_rate_jobs_per_s": cap / mean_steps,
                         "rate_at_80pct_load_jobs_per_s": 0.8 * cap / mean_steps,
                         "requested_rate_jobs_per_s": SERVE_RATE,
                         "what": "the unscaled distribution (1e3-1e4 sweeps log-uniform, thermalisation a fifth of "
                                 "that) needs mean_steps_per_request Metropolis steps per request; at the stream's "
                                 "saturated service rate the queue stays bounded below sustained_rate"},
            "what": "latency = done - submitted (host clock, includes queueing, walker start and FP64 start "
                    "inversions); error: the job's final configurations measured with its own inverses and "
                    "with fresh FP64 inverses"}


# DRAM bytes per walker per walk launch of k_walk_gs_res (inverses in at entry,
# out at exit, plus tables): dram__bytes_read.sum + dram__bytes_write.sum of
# one measured sweep of the 2048-walker workload (557.59 MB + 478.38 MB, a
# one-pass ncu capture), summarised in
# profiles/k_walk_gs_res_L16_2048walkers_dram.md
RES_DRAM_BYTES_PER_WALKER = (557.59e6 + 478.38e6) / 2048


def sm_count():
    try:
        import torch
        return int(torch.cuda.get_device_properties(0).multi_processor_count)
    except Exception:
        return 152


def fp32_peak_tflops(clocks):
    """Nominal FP32 CUDA-core peak at the SM clock sampled during the timed
    region: SMs x 128 FP32 lanes x 2 flops (FMA) x clock."""
    mhz = (clocks or {}).get("sm_mhz")
    if not mhz:
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                mhz = float(json.load(f)["sm_max_mhz"])
        except Exception:
            mhz = 2070.0
    return sm_count() * 128 * 2 * mhz * 1e6 / 1e12, mhz


def walk_roofline(res, precision):
    """Roofline of the dominant kernel, the walk.

    The on-chip kernel (k_walk_gs_res, mixed, N <= 128) keeps both inverses in
    tensor memory for the whole launch: its algorithmic HBM bytes are the two
    FP32 inverses in at entry and out at exit, 2 * 2 * N^2 * 8 B per walker
    per launch, and it is bound by on-chip latency (one walker per SM), not by
    HBM: the report gives that HBM fraction, the FP32 CUDA-core fraction of
    its algorithmic flops, and the streaming formulation's bytes per step
    (what an HBM-resident walk would move) under its own name.
    The streaming kernel (k_walk_gs: FP64, or mixed with stream_inverses)
    moves p_ap * (2 * 2 * N * s) + p_acc * (2 * 3 * N^2 * s) bytes per step."""
    N, s_b = L * L // 2, (8 if precision == "mixed" else 16)
    nl = max(1, res["walk_launches"])
    ms_launch = res["walk_ms"] / nl
    steps_launch = res["steps"] / nl
    p_ap, p_acc = res["p_ap"], res["p_acc"]
    stream_bytes = p_ap * (2 * 2 * N * s_b) + p_acc * (2 * 3 * N * N * s_b)
    flops_step = p_ap * 2 * 8 * N + p_acc * 2 * 16 * N * N
    peak, peak_kind = measured_peaks()
    resident = precision == "mixed" and N <= 128
    if resident:
        alg = WALKERS * 2 * 2 * N * N * 8.0
        alg_what = "both FP32 inverses loaded at launch entry and stored at exit: 2 flavours x 2 x N^2 x 8 B per walker"
    else:
        alg = stream_bytes * steps_launch
        alg_what = "streaming formulation: p_ap*(2*2*N*s) + p_acc*(2*3*N^2*s) per Metropolis step"
    achieved = alg / (ms_launch * 1e-3) / 1e9
    f32_peak, mhz = fp32_peak_tflops(res.get("clocks"))
    f32 = flops_step * steps_launch / (ms_launch * 1e-3) / 1e12
    roof = {"bound": "hbm", "kernel": "k_walk_gs_res" if resident else "k_walk_gs",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "traffic": RES_DRAM_BYTES_PER_WALKER * WALKERS if resident else None,
            "algorithmic_bytes_per_launch": alg, "algorithmic_bytes_what": alg_what,
            "kernel_ms_per_launch": ms_launch, "steps_per_launch": steps_launch,
            "fp32": {"achieved_tflops": f32, "peak_tflops": f32_peak, "frac": f32 / f32_peak,
                     "flops_per_step": flops_step,
                     "flops_what": "p_ap*2*8N (two ratio dots) + p_acc*2*16N^2 (A^-1 u and the rank-1 update, "
                                   "both flavours)",
                     "peak_kind": "nominal: %d SMs x 128 FP32 lanes x 2 flops x %.0f MHz (median sampled SM clock)"
                                  % (sm_count(), mhz)},
            "streaming_equivalent": {"bytes_per_step": stream_bytes,
                                     "gbs": stream_bytes * steps_launch / (ms_launch * 1e-3) / 1e9,
                                     "over_hbm_peak": stream_bytes * steps_launch / (ms_launch * 1e-3) / 1e9 / peak,
                                     "what": "bytes an HBM-streaming walk would move per step, per second of this "
                                             "kernel: the speed-up over that formulation's HBM bound, not a "
                                             "bandwidth drawn"}}
    if resident:
        roof["binding_resource"] = ("instruction issue and short dependency chains with one walker (8 warps) per "
                                    "SM: ncu issue-active 53.8 %, ALU pipe 37.6 %, FMA pipe 25.5 %, stalls per "
                                    "issue wait 0.71 / short scoreboard 0.66 / not selected 0.48 "
                                    "(profiles/k_walk_gs_res_L16_304walkers.md)")
    return roof


def main():
    global WALKERS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--cpu-sweeps", type=int, default=300)
    ap.add_argument("--no-fp64-arm", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--walkers", type=int, default=WALKERS, help="walkers (profiling a smaller case)")
    ap.add_argument("--no-exciton", action="store_true", help="skip the exciton-channel section")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-stream section")
    ap.add_argument("--no-long", action="store_true", help="skip the longitudinal-exciton section")
    ap.add_argument("--serving-only", action="store_true", help="only the serving stream (profiling runs)")
    ap.add_argument("--no-pairs", action="store_true",
                    help="skip the StatSpinStruct tensor-core, graphs, autotune and L=12 sections")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        # The reference's CPU path (its algorithm restated in oracle/vmc_oracle.c;
        # the reference build itself needs its sources, absent on the GPU host).
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        v = cpu_baseline(cores, args.cpu_sweeps, reinv=0)
        out = {"metric": METRIC, "impl": "reference", "value": v["value"], "unit": "steps/s", "n_gpus": args.gpus,
               "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": workload_config("fp64"),
               "cpu_baseline": {"value": v["value"], "unit": "steps/s", "cores": v["cores"], "kind": v["kind"],
                                "sample": v["sample"]},
               "e2e": {"value": v["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return

    WALKERS = args.walkers
    if args.serving_only:
        import gpvmc_gb300 as g
        print(json.dumps({"serving": run_serving(g)}))
        return
    cpu = cpu_exc = cpu_lng = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(os.cpu_count() or 1, args.cpu_sweeps, reinv=0)
        if not args.no_exciton:
            cpu_exc = cpu_exciton_baseline(os.cpu_count() or 1, 4)
        if not args.no_long:
            cpu_lng = cpu_long_baseline(os.cpu_count() or 1, 2000)

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import gpvmc_gb300 as g

    if dist:
        dist.barrier()
    res = run_gpu(g, args.precision, args.steps, args.warmup, rank, clocks_index=local,
                  check_delta=(rank == 0 and args.precision == "mixed"))
    ms = res["ms"]
    if dist:
        import torch
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    total_steps = res["steps"] * world
    value = total_steps / (ms * 1e-3)

    fp64 = always = None
    if rank == 0 and not args.no_fp64_arm and args.precision == "mixed":
        k = max(2, args.steps // 4)
        r64 = run_gpu(g, "fp64", k, args.warmup, rank, policy="none")
        fp64 = {"value": r64["steps"] / (r64["ms"] * 1e-3), "ms_per_step": r64["ms"] / k,
                "p_acc": r64["p_acc"], "reinversion_policy": "none (the reference never re-inverts)",
                "steps": k}
        ra = run_gpu(g, "mixed", k, args.warmup, rank, policy="always")
        always = {"value": ra["steps"] / (ra["ms"] * 1e-3), "ms_per_step": ra["ms"] / k,
                  "walk_ms": ra["walk_ms"], "reinversion_ms": ra["inv_ms"], "reinversions": ra["reinv"],
                  "reinversion_policy": "FP64 re-inversion every 128 accepted exchanges", "steps": k}

    exc = run_exciton(g, 4, 1) if (rank == 0 and not args.no_exciton) else None
    lng = run_long(g, 2, 1) if (rank == 0 and not args.no_long) else None
    c2 = run_config2(g) if (rank == 0 and not args.no_pairs) else None
    serving = run_serving(g) if (rank == 0 and world == 1 and not args.no_serving) else None
    pairs = run_pairs(g, WALKERS) if (rank == 0 and not args.no_pairs) else None
    tcph = run_tc_projheis(g, WALKERS) if (rank == 0 and not args.no_pairs) else None
    graphs = run_graphs(g) if (rank == 0 and not args.no_pairs) else None
    tune = run_autotune(g) if (rank == 0 and not args.no_pairs) else None
    e2e = run_e2e(g, args.precision, args.steps, rank) if not args.no_e2e else None
    if dist and e2e:
        import torch
        t = torch.tensor([e2e["wall_s"]], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e["value"] = WALKERS * SWEEP * args.steps * world / float(t.item())

    if rank != 0:
        return
    roof = walk_roofline(res, args.precision)
    out = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
           "config": workload_config(args.precision),
           "e2e": ({k: e2e[k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step", "includes")}
                   if e2e else None),
           "gpu_launches": int(res["launches"]),
           "roofline": roof,
           "kernel_share": {"walk_ms": res["walk_ms"], "reinversion_ms": res["inv_ms"],
                            "reinversion_launches": res["inv_launches"], "total_ms": res["ms"]},
           "acceptance": {"p_acc": res["p_acc"], "p_ap": res["p_ap"], "reinversions": res["reinv"],
                          "checks_without_reinversion": res["checks_without_reinversion"],
                          "max_drift_at_check": res["max_drift_at_check"]},
           "latency": {"sweep_p50_ms": res["sweep_p50_ms"], "sweep_p99_ms": res["sweep_p99_ms"],
                       "what": "device time of one sweep of all walkers (walk kernel launch)"},
           "delta_e_site": res.get("delta_e_site"),
           "e_site_mean": res["e_site"],
           "clocks": res["clocks"]}
    if fp64:
        out["fp64_engine"] = fp64
        out["mixed_over_fp64"] = value / world / fp64["value"]
    if always:
        out["mixed_reinvert_every_128"] = always
    if cpu:
        out["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        out["cpu_baseline"]["per_core"] = cpu["per_core"]
    if exc:
        if cpu_exc:
            exc["cpu_baseline"] = {k: cpu_exc[k] for k in ("value", "unit", "cores", "kind", "sample", "per_core")}
        out["exciton"] = exc
    if lng:
        if cpu_lng:
            lng["cpu_baseline"] = {k: cpu_lng[k] for k in ("value", "unit", "cores", "kind", "sample", "per_core")}
        out["long_exciton"] = lng
    if serving:
        out["serving"] = serving
    if pairs:
        out["statspin_tensor_cores"] = pairs
    if tcph:
        out["projheis_tensor_cores"] = tcph
    if graphs:
        out["cuda_graphs"] = graphs
    if tune:
        out["autotune"] = tune
    if c2:
        out["l12_batched"] = c2
    print(json.dumps(out))


if __name__ == "__main__":
    main()
