"""ctypes access to the parity oracle (test infrastructure only).

Two back-ends with one surface:

* ``OracleChain`` -- the C restatement ``oracle/_build/liboracle.so``
  (oracle/vmc_oracle.c), buildable on every machine;
* ``RefChain`` -- the reference itself, compiled unmodified from its sources
  into ``oracle/_ref/libgpvmc_ref.so`` by ``make -C oracle ref`` (only where
  the reference sources are present).

A chain is one Markov chain of one channel (the reference's single-process
run: SquareLattice + LatticeState + StagFlux* + SlaterDeterminant +
LatticeStepper + MetroMC + quantities).
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
# the same source built for timing (-O3, inline complex arithmetic): CPU-baseline legs only
ORACLE_FAST_SO = os.path.join(ROOT, "oracle", "_build", "liboracle_fast.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libgpvmc_ref.so")

GROUNDSTATE, TRANS, LONG = 0, 1, 2
MEAS_PROJHEIS, MEAS_STAGMAGN, MEAS_STATSPIN = 1, 2, 4


class Trace(ctypes.Structure):
    _fields_ = [("v1", ctypes.c_int32), ("v2", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("accepted", ctypes.c_int32), ("khop", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("u", ctypes.c_double * 4), ("ratio", ctypes.c_double),
                ("w_new_c", ctypes.c_double), ("w_new_e", ctypes.c_int32), ("pad2", ctypes.c_int32)]


TRACE_DTYPE = np.dtype([("v1", "<i4"), ("v2", "<i4"), ("kind", "<i4"), ("accepted", "<i4"),
                        ("khop", "<i4"), ("pad", "<i4"), ("u", "<f8", (4,)), ("ratio", "<f8"),
                        ("w_new_c", "<f8"), ("w_new_e", "<i4"), ("pad2", "<i4")])
assert TRACE_DTYPE.itemsize == ctypes.sizeof(Trace)


def build_oracle():
    """Compile the C restatement (and the reference build when its sources exist)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    return ORACLE_SO


def reference_available():
    return os.path.exists(REF_SO)


_libs = {}


def _load(path, prefix):
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    P, D, I, U64, U32 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_uint64, ctypes.c_uint32
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)
    bp = ctypes.POINTER(ctypes.c_int8)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    tp = ctypes.POINTER(Trace)
    sigs = {
        "step": (I, [P, I, tp]),
        "walk": (I, [P, U64, U64, I, I, tp]),
        "measure": (I, [P, I]),
        "reset_quantities": (None, [P]),
        "reinit": (I, [P]),
        "config": (None, [P, bp]),
        "particles": (None, [P, I, ip]),
        "amp": (None, [P, dp, ip]),
        "weight": (None, [P, dp, ip]),
        "inverse": (None, [P, I, dp]),
        "current_state": (I, [P]),
        "counts": (None, [P, u64p, u64p, u64p, u64p]),
        "projheis": (I, [P, dp]),
        "stagmagn": (I, [P, dp]),
        "statspin": (I, [P, dp]),
        "virt_update": (I, [P, I, ip, dp]),
        "rng_seek": (None, [P, U64]),
    }
    wp = "orc_walker_" if prefix == "orc" else "ref_"
    for name, (res, args) in sigs.items():
        f = getattr(lib, wp + name)
        f.restype = res
        f.argtypes = args
    if prefix == "orc":
        lib.orc_job_create.restype = P
        lib.orc_job_create.argtypes = [I, D, D, D, D, D, I, I, I, ctypes.POINTER(I)]
        lib.orc_job_destroy.argtypes = [P]
        lib.orc_job_info.argtypes = [P, ctypes.POINTER(I)] + [ctypes.POINTER(I)] * 3
        lib.orc_job_phi.argtypes = [P, I, dp]
        lib.orc_job_neighbours.argtypes = [P, ip]
        lib.orc_job_orbitals.argtypes = [P, I, ip]
        lib.orc_walker_create.restype = P
        lib.orc_walker_create.argtypes = [P, U64, U32]
        lib.orc_walker_destroy.argtypes = [P]
        lib.orc_walker_set_config.restype = I
        lib.orc_walker_set_config.argtypes = [P, bp]
        lib.orc_walker_random_start.restype = I
        lib.orc_walker_random_start.argtypes = [P]
        lib.orc_uniform_at.restype = D
        lib.orc_uniform_at.argtypes = [U64, U32, U32, U64]
        lib.orc_philox4x32_10.argtypes = [ctypes.POINTER(U32), ctypes.POINTER(U32), ctypes.POINTER(U32)]
    else:
        lib.ref_create.restype = P
        lib.ref_create.argtypes = [I, D, D, D, D, D, I, I, I, ctypes.POINTER(I)]
        lib.ref_destroy.argtypes = [P]
        lib.ref_info.argtypes = [P] + [ctypes.POINTER(I)] * 4
        lib.ref_phi.argtypes = [P, I, dp]
        lib.ref_neighbours.argtypes = [P, ip]
        lib.ref_orbitals.argtypes = [P, I, ip]
        lib.ref_set_config.restype = I
        lib.ref_set_config.argtypes = [P, U64, U32, bp]
        lib.ref_random_start.restype = I
        lib.ref_random_start.argtypes = [P, U64, U32]
    lib._wp = wp
    _libs[path] = lib
    return lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


class _Chain:
    """Common methods over the walker-level entry points."""

    def _f(self, name):
        return getattr(self.lib, self.lib._wp + name)

    def info(self):
        return self.Ns, self.N, self.Nexc

    def step(self, meas=False):
        tr = Trace()
        rc = self._f("step")(self.h, int(meas), ctypes.byref(tr))
        if rc:
            raise RuntimeError("step failed: %d" % rc)
        return np.frombuffer(bytes(tr), dtype=TRACE_DTYPE)[0]

    def walk(self, length, meas=0, mask=0, reinv_every=0, trace=False):
        buf = np.zeros(length if trace else 0, dtype=TRACE_DTYPE)
        tp = buf.ctypes.data_as(ctypes.POINTER(Trace)) if trace else None
        rc = self._f("walk")(self.h, length, meas, mask, reinv_every, tp)
        if rc:
            raise RuntimeError("walk failed: %d" % rc)
        return buf if trace else None

    def measure(self, mask):
        rc = self._f("measure")(self.h, mask)
        if rc:
            raise RuntimeError("measure failed: %d" % rc)

    def reset_quantities(self):
        self._f("reset_quantities")(self.h)

    def reinit(self):
        return self._f("reinit")(self.h)

    def rng_seek(self, k):
        self._f("rng_seek")(self.h, k)

    def config(self):
        a = np.zeros(self.Ns, dtype=np.int8)
        self._f("config")(self.h, _ptr(a, ctypes.c_int8))
        return a

    def particles(self, fl):
        a = np.zeros(self.N[fl], dtype=np.int32)
        self._f("particles")(self.h, fl, _ptr(a, ctypes.c_int32))
        return a

    def amp(self):
        m = np.zeros(2)
        e = ctypes.c_int32()
        self._f("amp")(self.h, _ptr(m, ctypes.c_double), ctypes.byref(e))
        return complex(m[0], m[1]), int(e.value)

    def weight(self):
        m = ctypes.c_double()
        e = ctypes.c_int32()
        self._f("weight")(self.h, ctypes.byref(m), ctypes.byref(e))
        return float(m.value), int(e.value)

    def inverse(self, fl):
        n = self.N[fl]
        a = np.zeros(2 * n * n)
        self._f("inverse")(self.h, fl, _ptr(a, ctypes.c_double))
        # column-major (i + j*N) -> numpy [i, j]
        return (a[0::2] + 1j * a[1::2]).reshape(n, n).T.copy()

    def current_state(self):
        return self._f("current_state")(self.h)

    def counts(self):
        v = [ctypes.c_uint64() for _ in range(4)]
        self._f("counts")(self.h, *[ctypes.byref(x) for x in v])
        return tuple(int(x.value) for x in v)

    def projheis(self):
        a = np.zeros(2 * 2 * self.Nexc * self.Nexc)
        n = self._f("projheis")(self.h, _ptr(a, ctypes.c_double))
        return (a[0::2] + 1j * a[1::2]).reshape(2 * self.Nexc, self.Nexc), n

    def stagmagn(self):
        a = np.zeros(2)
        n = self._f("stagmagn")(self.h, _ptr(a, ctypes.c_double))
        return complex(a[0], a[1]), n

    def statspin(self):
        a = np.zeros(2 * 5 * self.Ns * self.Ns)
        n = self._f("statspin")(self.h, _ptr(a, ctypes.c_double))
        return (a[0::2] + 1j * a[1::2]).reshape(5, self.Ns, self.Ns), n

    def virt_update(self, hops):
        """hops: int array (nset, 4) of (up_from, up_to, dn_from, dn_to), -1 = none.
        Returns complex ratios qs/amp-style raw values as (mantissa, exp10) pairs:
        array (Nexc, nset) of complex mantissas and int exponents."""
        hops = np.ascontiguousarray(hops, dtype=np.int32).reshape(-1, 4)
        nset = hops.shape[0]
        out = np.zeros(3 * nset * self.Nexc)
        rc = self._f("virt_update")(self.h, nset, _ptr(hops, ctypes.c_int32), _ptr(out, ctypes.c_double))
        if rc:
            raise RuntimeError("virt_update failed: %d" % rc)
        out = out.reshape(self.Nexc, nset, 3)
        return out[..., 0] + 1j * out[..., 1], out[..., 2].astype(np.int64)


class OracleChain(_Chain):
    def __init__(self, L, phi, neel, neel_exp=0.0, bc=(1.0, 1.0), channel=GROUNDSTATE, q=(0, 0),
                 seed=1234, walker=0, timing_build=False):
        self.lib = _load(ORACLE_FAST_SO if timing_build else ORACLE_SO, "orc")
        st = ctypes.c_int()
        self.job = self.lib.orc_job_create(L, phi, neel, neel_exp, bc[0], bc[1], channel, q[0], q[1],
                                           ctypes.byref(st))
        if not self.job:
            raise RuntimeError("orc_job_create failed: %d" % st.value)
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        self.lib.orc_job_info(self.job, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
        self.L, self.Ns, self.N, self.Nexc = L, a.value, (b.value, c.value), d.value
        self.h = self.lib.orc_walker_create(self.job, seed, walker)

    def __del__(self):
        try:
            self.lib.orc_walker_destroy(self.h)
            self.lib.orc_job_destroy(self.job)
        except Exception:
            pass

    def phi_table(self, fl):
        a = np.zeros(2 * self.Ns * self.Ns)
        self.lib.orc_job_phi(self.job, fl, _ptr(a, ctypes.c_double))
        return (a[0::2] + 1j * a[1::2]).reshape(self.Ns, self.Ns)

    def neighbours(self):
        a = np.zeros(4 * self.Ns, dtype=np.int32)
        self.lib.orc_job_neighbours(self.job, _ptr(a, ctypes.c_int32))
        return a.reshape(self.Ns, 4)

    def orbitals(self, fl):
        a = np.zeros(self.N[fl], dtype=np.int32)
        self.lib.orc_job_orbitals(self.job, fl, _ptr(a, ctypes.c_int32))
        return a

    def set_config(self, up):
        up = np.ascontiguousarray(up, dtype=np.int8)
        return self.lib.orc_walker_set_config(self.h, _ptr(up, ctypes.c_int8))

    def random_start(self):
        return self.lib.orc_walker_random_start(self.h)


class RefChain(_Chain):
    def __init__(self, L, phi, neel, neel_exp=0.0, bc=(1.0, 1.0), channel=GROUNDSTATE, q=(0, 0),
                 seed=1234, walker=0):
        self.lib = _load(REF_SO, "ref")
        st = ctypes.c_int()
        self.h = self.lib.ref_create(L, phi, neel, neel_exp, bc[0], bc[1], channel, q[0], q[1],
                                     ctypes.byref(st))
        if not self.h:
            raise RuntimeError("ref_create failed: %d" % st.value)
        a, b, c, d = (ctypes.c_int() for _ in range(4))
        self.lib.ref_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
        self.L, self.Ns, self.N, self.Nexc = L, a.value, (b.value, c.value), d.value
        self.seed, self.walker = seed, walker

    def __del__(self):
        try:
            self.lib.ref_destroy(self.h)
        except Exception:
            pass

    def phi_table(self, fl):
        a = np.zeros(2 * self.Ns * self.Ns)
        self.lib.ref_phi(self.h, fl, _ptr(a, ctypes.c_double))
        return (a[0::2] + 1j * a[1::2]).reshape(self.Ns, self.Ns)

    def neighbours(self):
        a = np.zeros(4 * self.Ns, dtype=np.int32)
        self.lib.ref_neighbours(self.h, _ptr(a, ctypes.c_int32))
        return a.reshape(self.Ns, 4)

    def orbitals(self, fl):
        a = np.zeros(self.N[fl], dtype=np.int32)
        self.lib.ref_orbitals(self.h, fl, _ptr(a, ctypes.c_int32))
        return a

    def set_config(self, up):
        up = np.ascontiguousarray(up, dtype=np.int8)
        return self.lib.ref_set_config(self.h, self.seed, self.walker, _ptr(up, ctypes.c_int8))

    def random_start(self):
        return self.lib.ref_random_start(self.h, self.seed, self.walker)


def uniform_at(seed, walker, stream, k):
    lib = _load(ORACLE_SO, "orc")
    return lib.orc_uniform_at(seed, walker, stream, k)


def big_to_complex(mant, exp10):
    return mant * (10.0 ** exp10)
