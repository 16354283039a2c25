"""Serving loop over the engine (gv_server_* in include/gpvmc_gb300.h).

Requests -- a wavefunction, walker count, precision, seed and re-inversion
policy plus thermalisation and measured sweeps -- are queued as they arrive,
admitted by device footprint, and advanced concurrently on the GPU
(continuous batching).  Each result carries the request's timestamps
(submitted, admitted, done: seconds since the server started), so latency
percentiles come from the results themselves.

    srv = Server(max_jobs=16, chunk_sweeps=4)
    t = srv.submit(StagFluxGroundState(16, 0.25 * pi, 0.1), walkers=256, sweeps=100, meas=256)
    r = srv.wait(t)          # dict: e_site, stagmagn, steps, accepted, t_submit, t_admit, t_started, t_walked, t_done, ...
    srv.close()
"""
import ctypes

from . import _lib
from ._lib import check
from .vmc import CHANNELS, PRECISIONS


def _result_dict(r):
    return {k: getattr(r, k) for k, _ in _lib.Result._fields_}


class Server:
    def __init__(self, hbm_budget=0, max_jobs=16, chunk_sweeps=4):
        cfg = _lib.ServerConfig(hbm_budget, max_jobs, chunk_sweeps)
        h = ctypes.c_void_p()
        check(_lib.lib().gv_server_create(ctypes.byref(cfg), ctypes.byref(h)), "gv_server_create")
        self._h = h

    def submit(self, wav, walkers, sweeps, meas=None, therm_sweeps=0, seed=1234, precision="mixed", walker_base=0,
               reinv_every=128, drift_threshold=1e-5, meas_mask=_lib.GV_MEAS_PROJHEIS | _lib.GV_MEAS_STAGMAGN,
               validate=False, phi_range=None, neel_range=None):
        """Queue one request; returns its ticket."""
        req = _lib.Request()
        c = req.job
        c.L = wav.L
        c.channel = CHANNELS[wav.channel]
        c.q[0], c.q[1] = wav.q
        c.phi, c.neel, c.neel_exp = wav.phi, wav.neel, wav.neel_exp
        c.phase_shift[0], c.phase_shift[1] = wav.phase_shift
        if phi_range:
            c.phi_range[0], c.phi_range[1] = phi_range
        if neel_range:
            c.neel_range[0], c.neel_range[1] = neel_range
        c.n_walkers = walkers
        c.precision = PRECISIONS[precision]
        c.seed = seed
        c.walker_base = walker_base
        c.reinv_every = reinv_every
        c.meas_mask = meas_mask
        c.flags = 0
        if reinv_every:
            c.flags |= _lib.GV_FLAG_REINV_DEFERRED
            if drift_threshold:
                c.flags |= _lib.GV_FLAG_REINV_ON_DRIFT
                c.drift_threshold = drift_threshold
        req.therm_sweeps = therm_sweeps
        req.sweeps = sweeps
        req.meas = meas if meas is not None else wav.L * wav.L
        req.validate = 1 if validate else 0
        t = ctypes.c_uint64()
        check(_lib.lib().gv_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)), "gv_server_submit")
        return t.value

    def poll(self, ticket):
        r = _lib.Result()
        check(_lib.lib().gv_server_poll(self._h, ticket, ctypes.byref(r)), "gv_server_poll")
        return _result_dict(r)

    def wait(self, ticket, timeout=600.0):
        r = _lib.Result()
        check(_lib.lib().gv_server_wait(self._h, ticket, timeout, ctypes.byref(r)), "gv_server_wait")
        return _result_dict(r)

    def drain(self, timeout=3600.0):
        check(_lib.lib().gv_server_drain(self._h, timeout), "gv_server_drain")

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gv_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
