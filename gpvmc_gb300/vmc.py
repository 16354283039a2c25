"""Host-side mirror of the reference's sampling-path API over the C ABI.

The reference builds one Markov chain per process from SquareLattice,
LatticeState, a StagFlux* WaveFunction, SlaterDeterminant, LatticeStepper and
MetroMC, then attaches Quantity objects (vmc.cpp:140-285).  Here a ``Job``
holds ``walkers`` such chains on the GPU; the classes below keep the
reference's names and call semantics on top of it:

    wav = StagFluxGroundState(L=8, phi=0.25 * pi, neel=0.1)
    job = Job(wav, walkers=1, seed=1234)
    amp = SlaterDeterminant(job)             # amp.Init(), amp.Amp(), amp.VirtUpdate(...)
    step = LatticeStepper(job)
    mc = MetroMC(step)
    heis = ProjHeis(step); mc.AddQuantity(heis)
    mc.Walk(therm * L * L, 0); mc.Walk(meas * n, meas)
    heis.save()                               # m_vals / m_meas per walker

Errors are raised as ``GvError`` (the reference aborts, or throws under
-DEXCEPT).
"""
import ctypes
import math

import numpy as np

from . import _lib
from ._lib import GvError, check

CHANNELS = {"groundstate": _lib.GV_CH_GROUNDSTATE, "trans": _lib.GV_CH_TRANS, "long": _lib.GV_CH_LONG}
PRECISIONS = {"fp64": _lib.GV_PREC_FP64, "mixed": _lib.GV_PREC_MIXED}


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class SquareLattice:
    """Periodic L x L lattice (SquareLattice.cpp:9-28) with the reference's
    vertex numbering v = y*L + x and edge/neighbour order."""

    def __init__(self, Lx, Ly=None):
        if Ly is not None and Ly != Lx:
            raise ValueError("only square lattices are on this path")
        self.L = Lx
        self.Nv = Lx * Lx
        edges, nbr = [], [[] for _ in range(self.Nv)]
        for x in range(Lx):
            for y in range(Lx):
                a = y * Lx + x
                for b in (((y + 1) % Lx) * Lx + x, y * Lx + (x + 1) % Lx):
                    edges.append((a, b))
                    nbr[a].append(b)
                    nbr[b].append(a)
        self.edges = np.array(edges, dtype=np.int32)
        self.neighbours = np.array(nbr, dtype=np.int32)

    def GetNv(self):
        return self.Nv

    def GetLx(self):
        return self.L

    def GetLy(self):
        return self.L


class StagFluxWaveFunction:
    """Parameters of a staggered-flux (+Neel) trial state (StagFluxWaveFunction.cpp:8-43).
    ``phi`` is in radians, the value the reference's constructor receives."""

    channel = "groundstate"

    def __init__(self, L, phi, neel, neel_exp=0.0, phase_shift=(1.0, 1.0), q=(0, 0)):
        self.L, self.phi, self.neel, self.neel_exp = L, phi, neel, neel_exp
        self.phase_shift = tuple(phase_shift)
        self.q = tuple(q)


class StagFluxGroundState(StagFluxWaveFunction):
    channel = "groundstate"


class StagFluxTransExciton(StagFluxWaveFunction):
    channel = "trans"


class StagFluxLongExciton(StagFluxWaveFunction):
    """StagFluxLongExciton (StagFluxLongExciton.cpp:6-66): a particle-hole pair
    of momentum q in one flavour, L^2 states (+ the ground state at q = 0 or
    (pi, pi))."""
    channel = "long"


class Job:
    """A batch of independent chains of one wavefunction on the GPU (gv_job)."""

    def __init__(self, wav, walkers=1, seed=1234, precision="fp64", reinv_every=0, walker_base=0,
                 phi_range=None, neel_range=None, deferred_reinversion=False, drift_threshold=None,
                 delayed_updates=False, stream_inverses=False, scalar_pairs=False, cuda_graphs=False,
                 tc_projheis=False):
        L = _lib.lib()
        cfg = _lib.JobConfig()
        cfg.L = wav.L
        cfg.channel = CHANNELS[wav.channel]
        cfg.q[0], cfg.q[1] = wav.q
        cfg.phi, cfg.neel, cfg.neel_exp = wav.phi, wav.neel, wav.neel_exp
        cfg.phase_shift[0], cfg.phase_shift[1] = wav.phase_shift
        if phi_range:
            cfg.phi_range[0], cfg.phi_range[1] = phi_range
        if neel_range:
            cfg.neel_range[0], cfg.neel_range[1] = neel_range
        cfg.n_walkers = walkers
        cfg.precision = PRECISIONS[precision]
        cfg.seed = seed
        cfg.walker_base = walker_base
        cfg.reinv_every = reinv_every
        cfg.meas_mask = 0
        cfg.flags = _lib.GV_FLAG_REINV_DEFERRED if (deferred_reinversion or drift_threshold) else 0
        if drift_threshold:
            cfg.flags |= _lib.GV_FLAG_REINV_ON_DRIFT
            cfg.drift_threshold = drift_threshold
        if delayed_updates:
            cfg.flags |= _lib.GV_FLAG_DELAYED_UPDATES
        if stream_inverses:
            cfg.flags |= _lib.GV_FLAG_STREAM_INVERSES
        if scalar_pairs:
            cfg.flags |= _lib.GV_FLAG_SCALAR_PAIRS
        if cuda_graphs:
            cfg.flags |= _lib.GV_FLAG_CUDA_GRAPHS
        if tc_projheis:
            cfg.flags |= _lib.GV_FLAG_TC_PROJHEIS
        self.cfg = cfg
        self.wav = wav
        self.walkers = walkers
        self.precision = precision
        h = ctypes.c_void_p()
        check(L.gv_job_create(ctypes.byref(cfg), ctypes.byref(h)), "gv_job_create")
        self._h = h
        dims = [ctypes.c_int32() for _ in range(4)]
        check(L.gv_job_dims(h, *[ctypes.byref(d) for d in dims]), "gv_job_dims")
        self.Ns, Nup, Ndn, self.Nexc = (d.value for d in dims)
        self.N = (Nup, Ndn)
        self.lattice = SquareLattice(wav.L)

    @staticmethod
    def footprint(wav, walkers, precision="fp64"):
        cfg = _lib.JobConfig()
        cfg.L, cfg.channel = wav.L, CHANNELS[wav.channel]
        cfg.n_walkers, cfg.precision = walkers, PRECISIONS[precision]
        out = ctypes.c_uint64()
        check(_lib.lib().gv_job_footprint(ctypes.byref(cfg), ctypes.byref(out)), "gv_job_footprint")
        return out.value

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().gv_job_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- calls -----------------------------------------------------------
    def set_measurements(self, mask):
        check(_lib.lib().gv_job_set_meas_mask(self._h, mask), "gv_job_set_meas_mask")

    def init_walkers(self, up=None):
        if up is None:
            check(_lib.lib().gv_job_init_walkers(self._h, None), "gv_job_init_walkers")
        else:
            up = np.ascontiguousarray(up, dtype=np.int8).reshape(self.walkers, self.Ns)
            check(_lib.lib().gv_job_init_walkers(self._h, _p(up)), "gv_job_init_walkers")

    def walk(self, length, meas=0, sync=True):
        check(_lib.lib().gv_job_walk(self._h, length, meas), "gv_job_walk")
        if sync:
            self.synchronize()

    def walk_continue(self, length, meas=0, sync=True):
        """As walk, with the quantity sums carried over from the previous call."""
        check(_lib.lib().gv_job_walk_continue(self._h, length, meas), "gv_job_walk_continue")
        if sync:
            self.synchronize()

    TUNE_VARIANTS = ("streaming", "streaming-256", "streaming-delayed", "streaming-256-delayed", "on-chip")

    def autotune(self, steps=0):
        """gv_job_autotune: time the walk-kernel variants for this configuration
        on a scratch job, apply the fastest; returns (name or None, {name: us/step})."""
        c = ctypes.c_int32()
        t = np.zeros(5)
        check(_lib.lib().gv_job_autotune(self._h, steps, ctypes.byref(c), _p(t)), "gv_job_autotune")
        times = {n: float(x) for n, x in zip(self.TUNE_VARIANTS, t) if x >= 0}
        return (self.TUNE_VARIANTS[c.value] if c.value >= 0 else None), times

    track_capacity = 0

    def set_track_capacity(self, capacity):
        """Room for `capacity` track entries per walker (StagMagnTrack / OverlapTrack)."""
        check(_lib.lib().gv_job_set_track_capacity(self._h, capacity), "gv_job_set_track_capacity")
        self.track_capacity = capacity

    def tracks(self):
        """(stagmagn[W, cap], log10_weight[W, cap], n[W]) recorded since the last measuring walk."""
        cap = max(self.track_capacity, 1)
        sm = np.zeros(self.walkers * cap)
        lw = np.zeros(self.walkers * cap)
        n = np.zeros(self.walkers, dtype=np.int32)
        check(_lib.lib().gv_job_read_tracks(self._h, _p(sm), _p(lw), _p(n)), "gv_job_read_tracks")
        return sm.reshape(self.walkers, cap), lw.reshape(self.walkers, cap), n

    def graph_stats(self):
        """(graphs cached, replays) with cuda_graphs=True; cached = -1 if capture was refused."""
        c, r = ctypes.c_int32(), ctypes.c_int64()
        check(_lib.lib().gv_job_graph_stats(self._h, ctypes.byref(c), ctypes.byref(r)), "gv_job_graph_stats")
        return c.value, r.value

    # -- checkpoint / resume -------------------------------------------------
    def checkpoint(self, inverses=False):
        """The job's chain state as bytes (gv_job_checkpoint); with inverses the
        restored job continues bit for bit, without them it re-inverts in FP64."""
        flags = _lib.GV_CKPT_INVERSES if inverses else 0
        n = ctypes.c_uint64()
        check(_lib.lib().gv_job_checkpoint_size(self._h, flags, ctypes.byref(n)), "gv_job_checkpoint_size")
        buf = np.empty(n.value, dtype=np.uint8)
        check(_lib.lib().gv_job_checkpoint(self._h, flags, _p(buf), n.value, None), "gv_job_checkpoint")
        return buf.tobytes()

    def restore(self, blob):
        """Load a checkpoint taken from a job of the same configuration."""
        buf = np.frombuffer(blob, dtype=np.uint8)
        check(_lib.lib().gv_job_restore(self._h, _p(buf), buf.size), "gv_job_restore")

    def save_checkpoint(self, path, inverses=False):
        with open(path, "wb") as f:
            f.write(self.checkpoint(inverses))

    def load_checkpoint(self, path):
        with open(path, "rb") as f:
            self.restore(f.read())

    def walk_traced(self, length, meas=0, walker=0):
        buf = (_lib.Trace * max(length, 1))()
        check(_lib.lib().gv_job_walk_traced(self._h, length, meas, walker, buf), "gv_job_walk_traced")
        arr = np.frombuffer(bytes(buf), dtype=np.dtype([("v1", "<i4"), ("v2", "<i4"), ("kind", "<i4"),
                                                         ("accepted", "<i4"), ("khop", "<i4"), ("pad", "<i4"),
                                                         ("ratio", "<f8"), ("u4", "<f8")]))
        return arr[:length].copy()

    def measure(self):
        """Quantity::measure on the current configurations (no step)."""
        check(_lib.lib().gv_job_measure(self._h), "gv_job_measure")

    def reset_quantities(self):
        check(_lib.lib().gv_job_reset_quantities(self._h), "gv_job_reset_quantities")

    def drift_checks(self):
        d = np.zeros(self.walkers)
        n = np.zeros(self.walkers, dtype=np.uint64)
        check(_lib.lib().gv_job_read_drift_checks(self._h, _p(d), _p(n)), "gv_job_read_drift_checks")
        return d, n

    def synchronize(self):
        check(_lib.lib().gv_job_synchronize(self._h), "gv_job_synchronize")

    def set_wait_limit(self, polls):
        """Poll budget of the tensor-core kernels' bounded mbarrier waits
        (negative: the default)."""
        check(_lib.lib().gv_job_set_wait_limit(self._h, int(polls)), "gv_job_set_wait_limit")

    def reinvert(self):
        check(_lib.lib().gv_job_reinvert(self._h), "gv_job_reinvert")

    # ---- single-walker stepping (LatticeStepper::trystep / step, MetroMC::YesNo) ----
    def trystep(self, walker=0):
        """LatticeStepper::trystep on one walker: ((v1, v2), weight as
        (mantissa, base-2 exponent), arg-max channel state or -1 for a
        same-flavour proposal).  The proposal stays pending for step()."""
        v = np.zeros(2, dtype=np.int32)
        m, e, k = ctypes.c_double(), ctypes.c_int32(), ctypes.c_int32()
        check(_lib.lib().gv_job_trystep(self._h, walker, _p(v), ctypes.byref(m), ctypes.byref(e), ctypes.byref(k)),
              "gv_job_trystep")
        return (int(v[0]), int(v[1])), (m.value, e.value), k.value

    def yesno(self, walker, ratio):
        """MetroMC::YesNo with the walker's u4; moves its stream to the next step."""
        a = ctypes.c_int32()
        check(_lib.lib().gv_job_yesno(self._h, walker, float(ratio), ctypes.byref(a)), "gv_job_yesno")
        return bool(a.value)

    def step(self, walker=0):
        """LatticeStepper::step: apply the walker's pending proposal."""
        check(_lib.lib().gv_job_step(self._h, walker), "gv_job_step")

    def update(self, walker, hop, state=-1):
        """Lattice hop + wavefunction hop + SlaterDeterminant::Update for the
        exchange hop = (up_from, up_to, dn_from, dn_to) and channel state
        `state` (-1: the arg-max)."""
        h = np.ascontiguousarray(hop, dtype=np.int32)
        check(_lib.lib().gv_job_update(self._h, walker, _p(h), int(state)), "gv_job_update")

    def stepper_weight(self, walker=0):
        """LatticeStepper::weight of one walker as (mantissa, base-2 exponent)."""
        m, e = ctypes.c_double(), ctypes.c_int32()
        check(_lib.lib().gv_job_stepper_weight(self._h, walker, ctypes.byref(m), ctypes.byref(e)),
              "gv_job_stepper_weight")
        return m.value, e.value

    def drift(self):
        out = np.zeros(2 * self.walkers)
        check(_lib.lib().gv_job_drift(self._h, _p(out)), "gv_job_drift")
        return out.reshape(self.walkers, 2)

    def virt_update(self, walker, hops):
        hops = np.ascontiguousarray(hops, dtype=np.int32).reshape(-1, 4)
        out = np.zeros(2 * len(hops) * self.Nexc)
        check(_lib.lib().gv_job_virt_update(self._h, walker, len(hops), _p(hops), _p(out)), "gv_job_virt_update")
        return (out[0::2] + 1j * out[1::2]).reshape(self.Nexc, len(hops))

    def timer_start(self):
        check(_lib.lib().gv_job_timer_start(self._h), "gv_job_timer_start")

    def timer_stop(self):
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(_lib.lib().gv_job_timer_stop(self._h, ctypes.byref(ms), ctypes.byref(n)), "gv_job_timer_stop")
        return ms.value, n.value

    def kernel_ms(self, kind):
        """(ms, launches) of walk (0), re-inversion (1) or measurement (2) kernels in the last timer window."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(_lib.lib().gv_job_kernel_ms(self._h, kind, ctypes.byref(ms), ctypes.byref(n)), "gv_job_kernel_ms")
        return ms.value, n.value

    def kernel_times(self, kind):
        n = ctypes.c_int64()
        check(_lib.lib().gv_job_kernel_times(self._h, kind, None, 0, ctypes.byref(n)), "gv_job_kernel_times")
        out = np.zeros(n.value)
        check(_lib.lib().gv_job_kernel_times(self._h, kind, _p(out), n.value, ctypes.byref(n)), "gv_job_kernel_times")
        return out

    def last_walk_ms(self):
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(_lib.lib().gv_job_last_walk_ms(self._h, ctypes.byref(ms), ctypes.byref(n)), "gv_job_last_walk_ms")
        return ms.value, n.value

    # -- readers ---------------------------------------------------------
    def config(self):
        out = np.zeros(self.walkers * self.Ns, dtype=np.int8)
        check(_lib.lib().gv_job_read_config(self._h, _p(out)), "gv_job_read_config")
        return out.reshape(self.walkers, self.Ns)

    def particles(self, walker, fl):
        out = np.zeros(self.N[fl], dtype=np.int32)
        check(_lib.lib().gv_job_read_particles(self._h, walker, fl, _p(out)), "gv_job_read_particles")
        return out

    def amplitude(self):
        m = np.zeros(2 * self.walkers)
        e = np.zeros(self.walkers, dtype=np.int32)
        check(_lib.lib().gv_job_read_amplitude(self._h, _p(m), _p(e)), "gv_job_read_amplitude")
        return m[0::2] + 1j * m[1::2], e

    def inverse(self, walker, fl):
        n = self.N[fl]
        out = np.zeros(2 * n * n)
        check(_lib.lib().gv_job_read_inverse(self._h, walker, fl, _p(out)), "gv_job_read_inverse")
        return (out[0::2] + 1j * out[1::2]).reshape(n, n).T.copy()   # [p, f]

    def counts(self):
        out = np.zeros(5 * self.walkers, dtype=np.uint64)
        check(_lib.lib().gv_job_read_counts(self._h, _p(out)), "gv_job_read_counts")
        return out.reshape(self.walkers, 5)

    def orbitals(self, walker, fl):
        """Orbital of every Slater row of the walker's wavefunction Fock state."""
        out = np.zeros(self.N[fl], dtype=np.int32)
        check(_lib.lib().gv_job_read_orbitals(self._h, walker, fl, _p(out)), "gv_job_read_orbitals")
        return out

    def status(self):
        """Per-walker status codes (0 = running)."""
        out = np.zeros(self.walkers, dtype=np.int32)
        check(_lib.lib().gv_job_read_status(self._h, _p(out)), "gv_job_read_status")
        return out

    def state_index(self):
        """WaveFunction::m_c_exc of every walker (0 for the ground state)."""
        out = np.zeros(self.walkers, dtype=np.int32)
        check(_lib.lib().gv_job_read_state_index(self._h, _p(out)), "gv_job_read_state_index")
        return out

    def weight(self):
        """LatticeStepper weight over |Amp|^2 per walker: sum_k |q_k / Amp|^2 (1 for the ground state)."""
        out = np.zeros(self.walkers)
        check(_lib.lib().gv_job_read_weight(self._h, _p(out)), "gv_job_read_weight")
        return out

    def projheis(self):
        """Ground state: [E/site sum, count] per walker, shape (walkers, 2).  Exciton
        channel: m_vals = [H; O] per walker, shape (walkers, 2*Nexc, Nexc)."""
        n = np.zeros(self.walkers, dtype=np.int32)
        if self.Nexc > 1:
            vals = np.zeros(4 * self.walkers * self.Nexc * self.Nexc)
            check(_lib.lib().gv_job_read_projheis(self._h, _p(vals), _p(n)), "gv_job_read_projheis")
            return (vals[0::2] + 1j * vals[1::2]).reshape(self.walkers, 2 * self.Nexc, self.Nexc), n
        vals = np.zeros(4 * self.walkers)
        check(_lib.lib().gv_job_read_projheis(self._h, _p(vals), _p(n)), "gv_job_read_projheis")
        return (vals[0::2] + 1j * vals[1::2]).reshape(self.walkers, 2), n

    def stagmagn(self):
        vals = np.zeros(2 * self.walkers)
        n = np.zeros(self.walkers, dtype=np.int32)
        check(_lib.lib().gv_job_read_stagmagn(self._h, _p(vals), _p(n)), "gv_job_read_stagmagn")
        return vals[0::2] + 1j * vals[1::2], n

    def statspin(self):
        vals = np.zeros(10 * self.Ns * self.Ns)
        n = np.zeros(1, dtype=np.int32)
        check(_lib.lib().gv_job_read_statspin(self._h, _p(vals), _p(n)), "gv_job_read_statspin")
        return (vals[0::2] + 1j * vals[1::2]).reshape(5, self.Ns, self.Ns), int(n[0])


# ---------------------------------------------------------------------------
# Reference-named classes

class SlaterDeterminant:
    """SlaterDeterminant (SlaterDeterminant.h:44-71) over all walkers of a job."""

    def __init__(self, job):
        self.job = job

    def Init(self):
        self.job.reinvert()

    def Amp(self, walker=0):
        m, e = self.job.amplitude()
        return m[walker] * 10.0 ** float(e[walker])

    def VirtUpdate(self, rhop, walker=0):
        """rhop: list of (up_hop, dn_hop) with hop = (from_site, to_site) or None.
        Returns qs / Amp() for every set (ground state: one channel state)."""
        rows = []
        for up, dn in rhop:
            rows.append([*(up if up else (-1, -1)), *(dn if dn else (-1, -1))])
        return self.job.virt_update(walker, np.array(rows, dtype=np.int32))


class LatticeStepper:
    """LatticeStepper (LatticeStepper.h:16-37): nearest-neighbour exchanges.
    Step-level calls (Stepper.h:13-34) act on one walker of the job; weights
    are (mantissa, base-2 exponent) pairs (the reference's BigDouble)."""

    def __init__(self, job, walker=0):
        self.job = job
        self.walker = walker
        self.prev = None
        self.khop = -1

    def GetAmp(self):
        return SlaterDeterminant(self.job)

    def Reset(self):
        self.prev, self.khop = None, -1

    def trystep(self):
        self.prev, w, self.khop = self.job.trystep(self.walker)
        return w

    def step(self):
        self.job.step(self.walker)
        self.prev, self.khop = None, -1

    def weight(self):
        return self.job.stepper_weight(self.walker)

    def transprob(self):
        return 1.0


class Quantity:
    mask = 0

    def __init__(self, stepper):
        self.job = stepper.job

    def GetNmeas(self):
        return self._read()[1]


class ProjHeis(Quantity):
    """ProjHeis (ProjHeis.cpp:40-158), Bx = 0: for the ground state m_vals is
    [sum of E/site samples, count] per walker."""

    mask = _lib.GV_MEAS_PROJHEIS

    def _read(self):
        return self.job.projheis()

    def save(self):
        v, n = self._read()
        return v / np.maximum(n, 1).reshape((-1,) + (1,) * (v.ndim - 1))


class StagMagnZ(Quantity):
    mask = _lib.GV_MEAS_STAGMAGN

    def _read(self):
        return self.job.stagmagn()

    def save(self):
        v, n = self._read()
        return v / np.maximum(n, 1)


class StatSpinStruct(Quantity):
    """StatSpinStruct (StatSpinStruct.cpp:16-135): 5 x Ns x Ns sums over all walkers."""

    mask = _lib.GV_MEAS_STATSPIN

    def _read(self):
        return self.job.statspin()

    def GetNmeas(self):
        return self._read()[1]

    def save(self):
        v, n = self._read()
        return v / max(n, 1)


class StagMagnTrack(Quantity):
    """StagMagnTrack (StagMagnTrack.cpp:21-50): the staggered magnetisation of
    every measurement since the walk began, per walker (a list of arrays)."""

    mask = _lib.GV_MEAS_STAGMAGN_TRACK

    def _read(self):
        sm, _, n = self.job.tracks()
        return sm, n

    def save(self):
        sm, n = self._read()
        return [sm[w, :n[w]] for w in range(len(n))]


class OverlapTrack(Quantity):
    """OverlapTrack (OverlapTrack.cpp:26-29): the stepper weight of every
    measurement divided by their mean, per walker (as OverlapTrack::save)."""

    mask = _lib.GV_MEAS_OVERLAP_TRACK

    def _read(self):
        _, lw, n = self.job.tracks()
        return lw, n

    def save(self):
        lw, n = self._read()
        out = []
        for w in range(len(n)):
            x = lw[w, :n[w]]
            if len(x) == 0:
                out.append(x)
                continue
            m = x.max()
            rel = 10.0 ** (x - m)
            out.append(rel / rel.mean())
        return out


class MetroMC:
    """MetroMC (MetroMC.h:11-45): Walk(len, meas) on every walker of the job,
    Step(meas) / YesNo(ratio) on the stepper's walker, Rejection()."""

    def __init__(self, stepper):
        self.job = stepper.job
        self.stepper = stepper
        self.quantities = []
        self._state_weight = None

    def YesNo(self, ratio):
        return self.job.yesno(self.stepper.walker, ratio)

    def Step(self, meas=False):
        """MetroMC::Step (MetroMC.cpp:90-103)."""
        if self._state_weight is None:
            self._state_weight = self.stepper.weight()
        new = self.stepper.trystep()
        ratio = math.ldexp(new[0] / self._state_weight[0], new[1] - self._state_weight[1])
        if self.YesNo(ratio):
            self.stepper.step()
            self._state_weight = new

    def AddQuantity(self, q):
        self.quantities.append(q)
        mask = 0
        for x in self.quantities:
            mask |= x.mask
        self.job.set_measurements(mask)

    def GetQuantities(self):
        return self.quantities

    def Walk(self, length, meas):
        if meas and any(q.mask & (_lib.GV_MEAS_STAGMAGN_TRACK | _lib.GV_MEAS_OVERLAP_TRACK)
                        for q in self.quantities):
            need = -(-length // meas)   # measurements of this walk
            if self.job.track_capacity < need:
                self.job.set_track_capacity(need)
        self.job.walk(length, meas)
        self._state_weight = None   # the walk moved the stepper's walker too

    def Rejection(self):
        c = self.job.counts().astype(np.float64)
        return np.where(c[:, 0] > 0, c[:, 3] / np.maximum(c[:, 0], 1), 0.0)


def pi_phi(phi_over_pi):
    """The CLI's phi is in units of pi (vmc.cpp:120)."""
    return phi_over_pi * math.pi


__all__ = ["SquareLattice", "StagFluxGroundState", "StagFluxTransExciton", "StagFluxLongExciton", "Job",
           "SlaterDeterminant",
           "LatticeStepper", "MetroMC", "ProjHeis", "StagMagnZ", "StatSpinStruct", "GvError", "pi_phi"]
