"""ctypes binding of the engine's C ABI (include/gpvmc_gb300.h).

The shared library is built in-tree by ``python -m gpvmc_gb300.build``.  There
is no fallback: if the library is missing or a CUDA device is absent, the
calls fail with an explicit error.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgpvmc_gb300.so")

GV_OK = 0
GV_ERR_TIMEOUT, GV_ERR_OOM, GV_ERR_CUDA = 6, 7, 8
GV_REQ_PENDING, GV_REQ_RUNNING, GV_REQ_DONE = 0, 1, 2
STATUS_NAMES = {0: "ok", 1: "invalid", 2: "singular", 3: "nan", 4: "zero amplitude", 5: "drift",
                6: "timeout", 7: "out of memory", 8: "cuda error", 9: "not ready", 10: "too large"}

GV_CH_GROUNDSTATE, GV_CH_TRANS, GV_CH_LONG = 0, 1, 2
GV_PREC_FP64, GV_PREC_MIXED = 0, 1
GV_MEAS_PROJHEIS, GV_MEAS_STAGMAGN, GV_MEAS_STATSPIN = 1, 2, 4
GV_MEAS_STAGMAGN_TRACK, GV_MEAS_OVERLAP_TRACK = 8, 16
GV_FLAG_REINV_DEFERRED = 1
GV_FLAG_REINV_ON_DRIFT = 2
GV_FLAG_DELAYED_UPDATES = 4
GV_FLAG_STREAM_INVERSES = 8
GV_FLAG_SCALAR_PAIRS = 16
GV_FLAG_CUDA_GRAPHS = 32
GV_FLAG_TC_PROJHEIS = 64
GV_CKPT_INVERSES = 1


class GvError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        msg = "%s failed: %s (%d)" % (where, STATUS_NAMES.get(status, "?"), status)
        super().__init__(msg + (": " + detail if detail else ""))


class JobConfig(ctypes.Structure):
    _fields_ = [("L", ctypes.c_int32), ("channel", ctypes.c_int32), ("q", ctypes.c_int32 * 2),
                ("phi", ctypes.c_double), ("neel", ctypes.c_double), ("neel_exp", ctypes.c_double),
                ("phase_shift", ctypes.c_double * 2), ("phi_range", ctypes.c_double * 2),
                ("neel_range", ctypes.c_double * 2), ("n_walkers", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("seed", ctypes.c_uint64), ("walker_base", ctypes.c_uint32),
                ("reinv_every", ctypes.c_int32), ("meas_mask", ctypes.c_int32), ("flags", ctypes.c_int32),
                ("drift_threshold", ctypes.c_double)]

class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("max_jobs", ctypes.c_int32), ("chunk_sweeps", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("job", JobConfig), ("therm_sweeps", ctypes.c_uint64), ("sweeps", ctypes.c_uint64),
                ("meas", ctypes.c_uint64), ("validate", ctypes.c_int32), ("pad", ctypes.c_int32)]


class Result(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("status", ctypes.c_int32), ("steps", ctypes.c_uint64),
                ("accepted", ctypes.c_uint64), ("footprint", ctypes.c_uint64), ("e_site", ctypes.c_double),
                ("stagmagn", ctypes.c_double), ("validation_error", ctypes.c_double), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("t_started", ctypes.c_double),
                ("t_walked", ctypes.c_double)]



class Trace(ctypes.Structure):
    _fields_ = [("v1", ctypes.c_int32), ("v2", ctypes.c_int32), ("kind", ctypes.c_int32),
                ("accepted", ctypes.c_int32), ("khop", ctypes.c_int32), ("pad", ctypes.c_int32),
                ("ratio", ctypes.c_double), ("u4", ctypes.c_double)]


# name -> (argtypes); every function returns gv_status (int32) unless noted
_P = ctypes.c_void_p
_SIGS = {
    "gv_job_create": [ctypes.POINTER(JobConfig), ctypes.POINTER(ctypes.c_void_p)],
    "gv_job_destroy": [_P],
    "gv_job_dims": [_P] + [ctypes.POINTER(ctypes.c_int32)] * 4,
    "gv_job_footprint": [ctypes.POINTER(JobConfig), ctypes.POINTER(ctypes.c_uint64)],
    "gv_job_init_walkers": [_P, ctypes.c_void_p],
    "gv_job_set_meas_mask": [_P, ctypes.c_int32],
    "gv_job_measure": [_P],
    "gv_job_reset_quantities": [_P],
    "gv_job_read_drift_checks": [_P, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_set_wait_limit": [_P, ctypes.c_int32],
    "gv_transfer_bytes": [ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)],
    "gv_job_trystep": [_P, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                       ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)],
    "gv_job_yesno": [_P, ctypes.c_int32, ctypes.c_double, ctypes.POINTER(ctypes.c_int32)],
    "gv_job_step": [_P, ctypes.c_int32],
    "gv_job_update": [_P, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32],
    "gv_job_stepper_weight": [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)],
    "gv_slater_invert_noalloc": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_walk": [_P, ctypes.c_uint64, ctypes.c_uint64],
    "gv_job_walk_traced": [_P, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p],
    "gv_job_synchronize": [_P],
    "gv_job_reinvert": [_P],
    "gv_job_drift": [_P, ctypes.c_void_p],
    "gv_job_virt_update": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_read_config": [_P, ctypes.c_void_p],
    "gv_job_read_particles": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
    "gv_job_read_amplitude": [_P, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_read_inverse": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
    "gv_job_read_counts": [_P, ctypes.c_void_p],
    "gv_job_read_state_index": [_P, ctypes.c_void_p],
    "gv_job_read_weight": [_P, ctypes.c_void_p],
    "gv_job_read_status": [_P, ctypes.c_void_p],
    "gv_job_walk_continue": [_P, ctypes.c_uint64, ctypes.c_uint64],
    "gv_job_stream": [_P, ctypes.c_void_p],
    "gv_job_graph_stats": [_P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)],
    "gv_job_set_track_capacity": [_P, ctypes.c_int32],
    "gv_job_read_tracks": [_P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_autotune": [_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p],
    "gv_job_checkpoint_size": [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)],
    "gv_job_checkpoint": [_P, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "gv_job_restore": [_P, ctypes.c_void_p, ctypes.c_uint64],
    "gv_server_create": [ctypes.c_void_p, ctypes.c_void_p],
    "gv_server_submit": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "gv_server_poll": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p],
    "gv_server_wait": [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p],
    "gv_server_drain": [ctypes.c_void_p, ctypes.c_double],
    "gv_server_destroy": [ctypes.c_void_p],
    "gv_job_read_orbitals": [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p],
    "gv_job_read_projheis": [_P, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_read_stagmagn": [_P, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_read_statspin": [_P, ctypes.c_void_p, ctypes.c_void_p],
    "gv_job_last_walk_ms": [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)],
    "gv_job_timer_start": [_P],
    "gv_job_timer_stop": [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)],
    "gv_job_kernel_ms": [_P, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)],
    "gv_job_kernel_times": [_P, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)],
    "gv_phi_table": [ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                     ctypes.c_int32, ctypes.c_void_p],
    "gv_lattice_neighbours": [ctypes.c_int32, ctypes.c_void_p],
    "gv_channel_states": [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p],
    "gv_channel_orbitals": [ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "gv_fock_quantum_numbers": [ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p],
}
# exported names that take no status-returning signature above
EXTRA_SYMBOLS = ["gv_version", "gv_status_string", "gv_philox4x32_10", "gv_uniform_at"]

_lib = None


def lib():
    """Load libgpvmc_gb300.so (once).  Raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("gpvmc_gb300 native library missing (%s); build it with "
                           "`python -m gpvmc_gb300.build`" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    for name, args in _SIGS.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int32
    L.gv_version.restype = ctypes.c_char_p
    L.gv_version.argtypes = []
    L.gv_status_string.restype = ctypes.c_char_p
    L.gv_status_string.argtypes = [ctypes.c_int32]
    L.gv_last_cuda_error.restype = ctypes.c_char_p
    L.gv_last_cuda_error.argtypes = []
    L.gv_philox4x32_10.restype = None
    L.gv_philox4x32_10.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
    L.gv_uniform_at.restype = ctypes.c_double
    L.gv_uniform_at.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
    _lib = L
    return L


def transfer_bytes():
    """(host->device, device->host) bytes the library has copied so far."""
    h, d = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().gv_transfer_bytes(ctypes.byref(h), ctypes.byref(d)), "gv_transfer_bytes")
    return int(h.value), int(d.value)


def check(status, where):
    if status != GV_OK:
        detail = ""
        if status in (GV_ERR_CUDA, GV_ERR_OOM) and _lib is not None:
            detail = _lib.gv_last_cuda_error().decode()
        raise GvError(status, where, detail)
