"""Result files in the reference's HDF5 layout (FileManager.cpp:293-551,
FileManager.h:25-115, WaveFunction.cpp:85-137), so that the reference's
post-processing (tools/vmc_postproc: load.get_quantity / get_stat / get_attr /
get_wav) reads engine results unchanged.

Layout (one file per quantity, `<dir>/<prefix>-<Quantity>.h5`):
  /                 file attributes: every run parameter as a 1-element
                    float64 array (FileManager::FileAttribute(double)) or a
                    fixed-length byte string, plus `type` (the quantity) and
                    `date`;
  /rank-<r>/data-<i>  float64 [M, 2N]: the quantity's M x N complex m_vals /
                    m_meas, real and imaginary parts interleaved along a row
                    (MatrixQuantity::save, ScalarQuantity::save), running-
                    averaged over the saves of one sample (MatStream::Write),
                    with 1-element float64 attributes `rej`, `time`,
                    `statistics`.
The reference runs one Markov chain per MPI calc rank r = 1..n and its rank 0
writes `/rank-r`; here walker w of a job is calc rank r = w + 1.  Quantities
the engine sums over all walkers (StatSpinStruct) go to `/rank-1` once, as the
job-wide mean (the mean of all ranks' datasets, which is what
load.get_quantity forms from per-rank files).

Backends: h5py when it is importable; otherwise an incremental directory tree
`<prefix>-<Quantity>.h5.d/` (attrs.json per group, data-i.npy + data-i.json
per dataset) that `convert_tree(path)` turns into the .h5 file on a machine
that has h5py.  The datasets, attribute names and dtypes are the same.
"""
import json
import os
import time

import numpy as np

__all__ = ["FileManager", "MatStream", "convert_tree", "read_tree", "write_wavefunction", "save_quantities",
           "next_run_number"]


class MatStream:
    """FileManager.h:68-115: the running mean of the matrices written since the
    last dataset was closed (m_stat of them)."""

    def __init__(self):
        self.mat = None
        self.stat = 0

    def Write(self, mat):
        mat = np.asarray(mat, dtype=np.float64)
        if self.mat is None or not self.stat:
            self.mat = mat.copy()
            self.stat = 1
            return
        if mat.shape != self.mat.shape:
            raise ValueError("MatStream::Write: sizes must match.")
        self.mat = (self.stat * self.mat + mat) / (self.stat + 1)
        self.stat += 1


def _interleave(z):
    """M x N complex -> M x 2N float64 (re, im along each row)."""
    z = np.asarray(z, dtype=np.complex128)
    if z.ndim == 1:
        z = z.reshape(1, -1)
    out = np.empty((z.shape[0], 2 * z.shape[1]), dtype=np.float64)
    out[:, 0::2] = z.real
    out[:, 1::2] = z.imag
    return out


def _attr_value(v):
    if isinstance(v, (str, bytes)):
        return np.bytes_(v.encode("ascii") if isinstance(v, str) else v)
    return np.array([float(v)], dtype=np.float64)


# ---------------------------------------------------------------------------
# Backends: the same operations on an HDF5 file or on a directory tree.

class _TreeFile:
    """One quantity file as a directory: attrs.json, <group>/attrs.json,
    <group>/data-i.npy, <group>/data-i.json."""

    def __init__(self, path, create):
        self.root = path + ".d"
        if create:
            os.makedirs(self.root, exist_ok=False)
            self._save_attrs(self.root, {})

    @staticmethod
    def _load_attrs(p):
        with open(p) as f:
            return json.load(f)

    @staticmethod
    def _save_attrs(d, a):
        with open(os.path.join(d, "attrs.json"), "w") as f:
            json.dump(a, f, sort_keys=True)

    @staticmethod
    def _enc(v):
        if isinstance(v, np.bytes_):
            return {"s": v.decode("ascii")}
        return {"d": [float(x) for x in np.atleast_1d(v)]}

    def set_attr(self, obj, name, value):
        d = os.path.join(self.root, obj.strip("/"))
        p = os.path.join(d, "attrs.json") if os.path.isdir(d) else d + ".json"
        a = self._load_attrs(p) if os.path.exists(p) else {}
        a[name] = self._enc(value)
        with open(p, "w") as f:
            json.dump(a, f, sort_keys=True)

    def has(self, path):
        p = os.path.join(self.root, path.strip("/"))
        return os.path.isdir(p) or os.path.exists(p + ".npy")

    def create_group(self, path):
        os.makedirs(os.path.join(self.root, path.strip("/")))
        self._save_attrs(os.path.join(self.root, path.strip("/")), {})

    def nlinks(self, group):
        d = os.path.join(self.root, group.strip("/"))
        return sum(1 for n in os.listdir(d) if n.endswith(".npy"))

    def write_dataset(self, path, data):
        p = os.path.join(self.root, path.strip("/"))
        np.save(p + ".npy", np.ascontiguousarray(data))
        if not os.path.exists(p + ".json"):
            with open(p + ".json", "w") as f:
                json.dump({}, f)

    def close(self):
        pass


class _H5File:
    def __init__(self, path, create):
        import h5py
        self.f = h5py.File(path, "w-" if create else "r+")

    def set_attr(self, obj, name, value):
        self.f[obj].attrs[name] = value

    def has(self, path):
        return path in self.f

    def create_group(self, path):
        self.f.create_group(path)

    def nlinks(self, group):
        return len(self.f[group])

    def write_dataset(self, path, data):
        if path in self.f:
            self.f[path][...] = data
        else:
            self.f.create_dataset(path, data=data, dtype=np.float64)

    def close(self):
        self.f.close()


def _have_h5py():
    try:
        import h5py  # noqa: F401
        return True
    except ImportError:
        return False


# ---------------------------------------------------------------------------

def next_run_number(d):
    """FileManager(dir, num < 0): the run counter kept in <dir>/.runfile
    (FileManager.cpp:7-56)."""
    p = os.path.join(d, ".runfile")
    try:
        with open(p) as f:
            n = int(f.read().split()[0]) + 1
    except (OSError, ValueError, IndexError):
        n = 0
    with open(p, "w") as f:
        f.write("%d\n" % n)
    return n


class FileManager:
    """FileManager (FileManager.h:25-66) for a job's walkers.

    FileStream(name, rank) gives the MatStream of quantity `name` for calc rank
    `rank` (walker + 1); Write() writes every stream as FileManager::Write
    does in its MPI form: file created with the file attributes on first use,
    group /rank-r, dataset data-<nlinks> when the stream holds one matrix and
    data-<nlinks - 1> (rewritten) when it holds more, the data attributes set
    on it, and the stream restarted once it holds StatPerSample matrices.
    backend: "auto" (h5py if importable, else the directory tree), "h5" or
    "tree"."""

    def __init__(self, dir=".", prefix=-1, backend="auto"):
        self.dir = dir
        os.makedirs(dir, exist_ok=True)
        self.num = int(prefix) if (isinstance(prefix, int) and prefix >= 0) else None
        if isinstance(prefix, str):
            self.num_str = prefix
        else:
            self.num_str = str(self.num if self.num is not None else next_run_number(dir))
        if backend == "auto":
            backend = "h5" if _have_h5py() else "tree"
        if backend not in ("h5", "tree"):
            raise ValueError("backend must be 'auto', 'h5' or 'tree'")
        self.backend = backend
        self.streams = {}          # (name, rank) -> MatStream
        self.file_attr = {}
        self.data_attr = {}        # name -> scalar or per-rank array (indexed by rank - 1)
        self.stat_per_sample = 1

    # reference-named setters
    def FileAttribute(self, name, value):
        if isinstance(value, (bool, np.bool_)):
            value = float(value)
        self.file_attr[name] = value

    def DataAttribute(self, name, value):
        self.data_attr[name] = value

    def StatPerSample(self, n=None):
        if n is not None:
            self.stat_per_sample = int(n)
        return self.stat_per_sample

    def FileStream(self, name, rank=0):
        return self.streams.setdefault((name, int(rank)), MatStream())

    def path(self, name):
        return os.path.join(self.dir, "%s-%s.h5" % (self.num_str, name))

    def _open(self, name):
        p = self.path(name)
        exists = os.path.exists(p + ".d") if self.backend == "tree" else os.path.exists(p)
        f = (_TreeFile if self.backend == "tree" else _H5File)(p, not exists)
        if not exists:
            for k in sorted(self.file_attr):
                f.set_attr("/", k, _attr_value(self.file_attr[k]))
            f.set_attr("/", "type", _attr_value(name))
            f.set_attr("/", "date", _attr_value(time.asctime() + "\n"))
        return f

    def Write(self):
        by_name = {}
        for (name, rank), st in sorted(self.streams.items()):
            by_name.setdefault(name, []).append((rank, st))
        for name, items in by_name.items():
            f = self._open(name)
            try:
                for rank, st in items:
                    if st.mat is None:
                        continue
                    g = "/rank-%d" % rank
                    if not f.has(g):
                        f.create_group(g)
                        d = g + "/data-0"
                    else:
                        n = f.nlinks(g)
                        d = g + "/data-%d" % (n if st.stat == 1 else n - 1)
                    f.write_dataset(d, st.mat)
                    for k in sorted(self.data_attr):
                        v = self.data_attr[k]
                        if np.ndim(v) > 0:
                            v = np.asarray(v)[rank - 1] if rank >= 1 else np.asarray(v)[0]
                        f.set_attr(d, k, _attr_value(v))
                    if st.stat == self.stat_per_sample:
                        st.stat = 0
            finally:
                f.close()


def save_quantities(fm, quantities):
    """Quantity::save for every quantity of a MetroMC, per walker: each walker's
    m_vals / m_meas into its calc rank's stream (walker + 1).  Engine-wide
    quantities (StatSpinStruct) go to rank 1."""
    from . import vmc
    for q in quantities:
        name = type(q).__name__
        vals = q.save()
        if isinstance(q, vmc.StatSpinStruct):
            # MatrixQuantity(5, Ns*Ns) layout: row a = correlator a, Ns*Ns complex
            fm.FileStream(name, 1).Write(_interleave(np.asarray(vals).reshape(5, -1)))
            continue
        if isinstance(q, (vmc.StagMagnTrack, vmc.OverlapTrack)):
            for w, x in enumerate(vals):
                x = np.asarray(x)
                col = _interleave(x).reshape(-1, 1) if np.iscomplexobj(x) else x.astype(np.float64).reshape(-1, 1)
                fm.FileStream(name, w + 1).Write(col)
            continue
        vals = np.asarray(vals)
        for w in range(vals.shape[0]):
            v = vals[w]
            if v.ndim == 0:                 # ScalarQuantity: 1 x 1 complex
                v = v.reshape(1, 1)
            elif v.ndim == 1:               # ground-state ProjHeis [H; O]: 2 x 1
                v = v.reshape(-1, 1)
            fm.FileStream(name, w + 1).Write(_interleave(v))


def write_wavefunction(fm, L, phase_shift=(1.0, 1.0), channel=0, q=(0, 0)):
    """WaveFunction::Save (WaveFunction.cpp:85-137): `<prefix>-WaveFunction.h5`
    with the file attributes, `type` = WaveFunction, and per flavour an int32
    dataset states_<fl> [Nexc, L*L] (1 where channel state e occupies fock
    orbital f) whose attributes kx, ky, band (big-endian uint32, one per
    orbital) are the orbitals' quantum numbers."""
    import ctypes
    from . import _lib
    lib = _lib.lib()
    Ns = L * L
    bc = np.asarray(phase_shift, dtype=np.float64)
    qq = np.asarray(q, dtype=np.int32)
    qn = np.zeros(3 * Ns, dtype=np.int32)
    st = lib.gv_fock_quantum_numbers(L, bc.ctypes.data_as(ctypes.c_void_p), qn.ctypes.data_as(ctypes.c_void_p))
    if st:
        raise ValueError("gv_fock_quantum_numbers: status %d" % st)
    qn = qn.reshape(Ns, 3)
    states = []
    for fl in (0, 1):
        orb = np.zeros(Ns, dtype=np.int32)
        N = ctypes.c_int32()
        nexc = ctypes.c_int32()
        st = lib.gv_channel_orbitals(L, bc.ctypes.data_as(ctypes.c_void_p), channel,
                                     qq.ctypes.data_as(ctypes.c_void_p), fl, orb.ctypes.data_as(ctypes.c_void_p),
                                     ctypes.byref(N), ctypes.byref(nexc))
        if st:
            raise ValueError("gv_channel_orbitals: status %d" % st)
        occ = np.zeros(Ns, dtype=np.int32)
        occ[orb[:N.value]] = 1
        states.append(np.repeat(occ[None, :], nexc.value, axis=0))
    if channel != 0:
        nexc = states[0].shape[0]
        up = np.zeros(nexc, dtype=np.int32)
        dn = np.zeros(nexc, dtype=np.int32)
        st = lib.gv_channel_states(L, bc.ctypes.data_as(ctypes.c_void_p), channel,
                                   qq.ctypes.data_as(ctypes.c_void_p), up.ctypes.data_as(ctypes.c_void_p),
                                   dn.ctypes.data_as(ctypes.c_void_p))
        if st:
            raise ValueError("gv_channel_states: status %d" % st)
        # every state from the lower band: orbital up[e] added to flavour 0, dn[e] removed from flavour 1
        lower = np.zeros(Ns, dtype=np.int32)
        lower[0::2] = 1
        s0 = np.repeat(lower[None, :], nexc, axis=0)
        s1 = s0.copy()
        s0[np.arange(nexc), up] = 1
        s1[np.arange(nexc), dn] = 0
        states = [s0, s1]
    p = fm.path("WaveFunction")
    f = (_TreeFile if fm.backend == "tree" else _H5File)(p, True)
    try:
        for k in sorted(fm.file_attr):
            f.set_attr("/", k, _attr_value(fm.file_attr[k]))
        f.set_attr("/", "type", _attr_value("WaveFunction"))
        for fl in (0, 1):
            name = "/states_%d" % fl
            if fm.backend == "tree":
                np.save(os.path.join(f.root, name.strip("/") + ".npy"), states[fl].astype(np.int32))
                with open(os.path.join(f.root, name.strip("/") + ".json"), "w") as g:
                    json.dump({}, g)
            else:
                f.f.create_dataset(name, data=states[fl].astype(np.int32), dtype=np.int32)
            for j, key in enumerate(("kx", "ky", "band")):
                v = qn[:, j].astype(">u4")
                if fm.backend == "tree":
                    f.set_attr(name, key, np.asarray(v, dtype=np.float64))
                else:
                    f.set_attr(name, key, v)
    finally:
        f.close()
    return states, qn


def read_tree(path):
    """Directory tree of one file -> (file attrs, {"/rank-r/data-i": (array, attrs)}) with
    attribute values decoded (strings as str, numbers as float64 arrays)."""
    root = path if path.endswith(".d") else path + ".d"

    def dec(a):
        return {k: (v["s"] if "s" in v else np.asarray(v["d"], dtype=np.float64)) for k, v in a.items()}

    with open(os.path.join(root, "attrs.json")) as f:
        fattrs = dec(json.load(f))
    data = {}
    for dirpath, _, files in os.walk(root):
        for n in files:
            if not n.endswith(".npy"):
                continue
            rel = os.path.relpath(os.path.join(dirpath, n[:-4]), root).replace(os.sep, "/")
            arr = np.load(os.path.join(dirpath, n))
            aj = os.path.join(dirpath, n[:-4] + ".json")
            attrs = {}
            if os.path.exists(aj):
                with open(aj) as f:
                    attrs = dec(json.load(f))
            data["/" + rel] = (arr, attrs)
    return fattrs, data


def convert_tree(path, h5py_module=None):
    """Write the .h5 file of a directory tree (`<prefix>-<Quantity>.h5.d`)
    next to it, with h5py (on a machine that has it)."""
    if h5py_module is None:
        import h5py as h5py_module
    root = path if path.endswith(".d") else path + ".d"
    out = root[:-2]
    fattrs, data = read_tree(root)
    wavefile = fattrs.get("type") == "WaveFunction"
    with h5py_module.File(out, "w-") as f:
        for k, v in fattrs.items():
            f.attrs[k] = _attr_value(v) if isinstance(v, str) else np.asarray(v, dtype=np.float64)
        for p in sorted(data, key=_path_key):
            arr, attrs = data[p]
            parent = p.rsplit("/", 1)[0]
            if parent and parent not in f:
                f.create_group(parent)
            if wavefile:
                ds = f.create_dataset(p, data=arr.astype(np.int32), dtype=np.int32)
                for k, v in attrs.items():
                    ds.attrs[k] = np.asarray(v).astype(">u4")
            else:
                ds = f.create_dataset(p, data=arr.astype(np.float64), dtype=np.float64)
                for k, v in attrs.items():
                    ds.attrs[k] = _attr_value(v) if isinstance(v, str) else np.asarray(v, dtype=np.float64)
    return out


def _path_key(p):
    """Order /rank-r/data-i numerically (creation order in FileManager::Write)."""
    out = []
    for part in p.strip("/").split("/"):
        head, _, num = part.rpartition("-")
        out.append((head, int(num)) if num.isdigit() else (part, -1))
    return out
