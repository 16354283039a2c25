"""Result files in the reference's HDF5 layout (gpvmc_gb300.output), CPU only.

The reference's writer (FileManager.cpp:293-551) needs HDF5, which neither
machine has, so the layout is checked structurally: the MatStream running mean
and dataset rollover restated from FileManager.h:68-115 / FileManager.cpp:
361-392, the directory-tree backend, and its conversion through a recording
stand-in for h5py, read back with the access pattern of the reference's
post-processing (tools/vmc_postproc/load.py: get_stat, get_quantity, get_attr,
get_wav).
"""
import ctypes
import os
import types

import numpy as np
import pytest

import gpvmc_gb300 as g
from gpvmc_gb300 import output


# ---------------------------------------------------------------------------
# a recording stand-in for h5py (File / Group / Dataset / attrs)

class _Node(dict):
    def __init__(self):
        super().__init__()
        self.attrs = {}

    def _walk(self, path):
        node = self
        for part in [p for p in path.strip("/").split("/") if p]:
            node = dict.__getitem__(node, part)
        return node

    def __getitem__(self, path):
        return self._walk(path)

    def __contains__(self, path):
        try:
            self._walk(path)
            return True
        except KeyError:
            return False

    def create_group(self, path):
        parent, _, name = path.strip("/").rpartition("/")
        node = _Node()
        dict.__setitem__(self._walk(parent), name, node)
        return node

    def create_dataset(self, path, data, dtype):
        parent, _, name = path.strip("/").rpartition("/")
        ds = _Dataset(np.asarray(data, dtype=dtype))
        dict.__setitem__(self._walk(parent), name, ds)
        return ds


class _Dataset:
    def __init__(self, data):
        self.data = data
        self.attrs = {}
        self.shape = data.shape

    def __getitem__(self, idx):
        return self.data[idx]


class FakeH5py:
    files = {}

    class File(_Node):
        def __init__(self, path, mode="r"):
            super().__init__()
            if mode == "r":
                src = FakeH5py.files[path]
                self.update(src)
                self.attrs = src.attrs
            else:
                assert mode == "w-" and path not in FakeH5py.files
                FakeH5py.files[path] = self

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def close(self):
            pass


# load.py's access pattern (get_stat / get_quantity / get_attr), restated
def _postproc_read(h5, path):
    f = h5.File(path, "r")
    stats, paths = [], []
    for r in f:
        for d in f[r]:
            stats.append(int(f[r][d].attrs["statistics"][0]))
            paths.append("/{0}/{1}".format(r, d))
    out = {}
    for p in paths:
        dat = f[p]
        out[p] = dat[:, ::2] + 1j * dat[:, 1::2]
    attrs = dict(f.attrs)
    for k, v in attrs.items():
        if type(v) is np.bytes_:
            attrs[k] = str(v, encoding="ascii")
    return stats, out, attrs


# ---------------------------------------------------------------------------

def test_matstream_running_mean():
    ms = output.MatStream()
    a, b, c = np.ones((2, 2)), 3 * np.ones((2, 2)), 8 * np.ones((2, 2))
    ms.Write(a)
    ms.Write(b)
    assert ms.stat == 2 and np.allclose(ms.mat, 2.0)
    ms.Write(c)
    assert ms.stat == 3 and np.allclose(ms.mat, 4.0)
    ms.stat = 0          # what FileManager::Write does after StatPerSample matrices
    ms.Write(b)
    assert ms.stat == 1 and np.allclose(ms.mat, 3.0)
    with pytest.raises(ValueError):
        ms.Write(np.ones((3, 2)))


def _fake_job(W, Ns=16, Nexc=1, seed=0):
    rng = np.random.default_rng(seed)
    state = {"k": 0}

    class Job:
        walkers = W

        def projheis(self):
            state["k"] += 1
            if Nexc > 1:
                v = rng.normal(size=(W, 2 * Nexc, Nexc)) + 1j * rng.normal(size=(W, 2 * Nexc, Nexc))
            else:
                v = rng.normal(size=(W, 2)) + 1j * rng.normal(size=(W, 2))
            return v, np.full(W, 4, dtype=np.int32)

        def stagmagn(self):
            return rng.normal(size=W) + 1j * rng.normal(size=W), np.full(W, 4, dtype=np.int32)

        def statspin(self):
            return rng.normal(size=(5, Ns, Ns)) + 0j, 4 * W

        def set_measurements(self, mask):
            pass

    return types.SimpleNamespace(job=Job())


@pytest.mark.parametrize("Nexc", [1, 3])
def test_filemanager_layout_and_rollover(tmp_path, Nexc):
    """Two samples of three saves each (StatPerSample = 3, as vmc.cpp:301-313
    with samples_saves = 3): per rank data-0 and data-1, each the mean of its
    sample's three saves, attributes statistics = (m+1)*stat and per-rank rej."""
    W, stat = 3, 10
    st = _fake_job(W, Nexc=Nexc)
    qs = [g.ProjHeis(st), g.StagMagnZ(st), g.StatSpinStruct(st)]
    fm = g.FileManager(str(tmp_path), prefix=7, backend="tree")
    fm.StatPerSample(3)
    fm.FileAttribute("L", 4)
    fm.FileAttribute("channel", "groundstate")
    fm.FileAttribute("meas_projheis", True)
    expect = {}
    for sample in range(2):
        for m in range(3):
            saved = {type(q).__name__: q.save() for q in qs}
            # save_quantities reads each quantity once more: replay the same values
            for q in qs:
                q.save = (lambda v: (lambda: v))(saved[type(q).__name__])
            output.save_quantities(fm, qs)
            for q in qs:
                del q.save
            for name, v in saved.items():
                expect.setdefault((name, sample), []).append(v)
            fm.DataAttribute("rej", np.arange(W) * 0.1 + sample)
            fm.DataAttribute("time", 1.5)
            fm.DataAttribute("statistics", (m + 1) * stat)
            fm.Write()
    for name in ("ProjHeis", "StagMagnZ", "StatSpinStruct"):
        fattrs, data = output.read_tree(fm.path(name))
        assert fattrs["type"] == name and fattrs["channel"] == "groundstate"
        assert np.allclose(fattrs["L"], [4.0]) and np.allclose(fattrs["meas_projheis"], [1.0])
        assert "date" in fattrs
        ranks = [1] if name == "StatSpinStruct" else list(range(1, W + 1))
        assert sorted(data) == sorted("/rank-%d/data-%d" % (r, i) for r in ranks for i in (0, 1))
        for r in ranks:
            for sample in (0, 1):
                arr, attrs = data["/rank-%d/data-%d" % (r, sample)]
                assert np.allclose(attrs["statistics"], [3 * stat])
                assert np.allclose(attrs["time"], [1.5])
                assert np.allclose(attrs["rej"], [(r - 1) * 0.1 + sample])
                vals = np.mean(expect[(name, sample)], axis=0)
                z = arr[:, 0::2] + 1j * arr[:, 1::2]
                if name == "StatSpinStruct":
                    ref = vals.reshape(5, -1)
                elif name == "StagMagnZ":
                    ref = vals[r - 1].reshape(1, 1)
                elif Nexc > 1:
                    ref = vals[r - 1]
                else:
                    ref = vals[r - 1].reshape(2, 1)
                assert arr.dtype == np.float64 and arr.shape == (ref.shape[0], 2 * ref.shape[1])
                assert np.allclose(z, ref, rtol=1e-12, atol=1e-14)


def test_runfile_counter(tmp_path):
    a = g.FileManager(str(tmp_path), backend="tree")
    b = g.FileManager(str(tmp_path), backend="tree")
    assert (a.num_str, b.num_str) == ("0", "1")
    assert open(os.path.join(str(tmp_path), ".runfile")).read().split()[0] == "1"


def test_convert_and_postproc_read(tmp_path):
    """The tree converted through h5py's interface reads back, with load.py's
    access pattern, as the quantities the walkers saved."""
    W = 2
    st = _fake_job(W)
    q = g.ProjHeis(st)
    fm = g.FileManager(str(tmp_path), prefix="run", backend="tree")
    fm.FileAttribute("phi", 0.25)
    saved = []
    for m in range(2):
        v = q.save()
        q.save = (lambda x: (lambda: x))(v)
        output.save_quantities(fm, [q])
        del q.save
        saved.append(v)
        fm.DataAttribute("statistics", 100)
        fm.DataAttribute("rej", 0.3)
        fm.Write()
    FakeH5py.files = {}
    out = g.convert_tree(fm.path("ProjHeis"), h5py_module=FakeH5py)
    assert out == fm.path("ProjHeis")
    stats, data, attrs = _postproc_read(FakeH5py, out)
    assert stats == [100] * (2 * W)
    assert attrs["type"] == "ProjHeis" and np.allclose(attrs["phi"], [0.25])
    for w in range(W):
        for m in range(2):
            assert np.allclose(data["/rank-%d/data-%d" % (w + 1, m)], saved[m][w].reshape(2, 1))
    f = FakeH5py.files[out]
    assert f["/rank-1/data-0"].data.dtype == np.float64
    assert f["/rank-1/data-0"].attrs["statistics"].dtype == np.float64
    assert isinstance(f.attrs["type"], np.bytes_)


def _lib():
    from gpvmc_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    return g.lib()


@pytest.mark.parametrize("L", [4, 8, 16])
def test_fock_quantum_numbers(L):
    lib = _lib()
    qn = np.zeros(3 * L * L, dtype=np.int32)
    bc = np.array([1.0, 1.0])
    assert lib.gv_fock_quantum_numbers(L, bc.ctypes.data_as(ctypes.c_void_p), qn.ctypes.data_as(ctypes.c_void_p)) == 0
    qn = qn.reshape(-1, 3)
    assert (qn[0::2, 2] == 0).all() and (qn[1::2, 2] == 1).all()
    assert (qn[0::2, :2] == qn[1::2, :2]).all()
    k = set(map(tuple, qn[0::2, :2]))
    assert len(k) == L * L // 2          # the magnetic Brillouin zone: half the momenta, each once
    for kx, ky in k:                     # no two MBZ points differ by (pi, pi)
        assert ((kx + L // 2) % L, (ky + L // 2) % L) not in k


@pytest.mark.parametrize("channel,q", [(0, (0, 0)), (1, (2, 2)), (1, (4, 0))])
def test_wavefunction_file(tmp_path, channel, q):
    L = 8
    fm = g.FileManager(str(tmp_path), prefix=3, backend="tree")
    fm.FileAttribute("L", L)
    states, qn = g.write_wavefunction(fm, L, channel=channel, q=q)
    fattrs, data = output.read_tree(fm.path("WaveFunction"))
    assert fattrs["type"] == "WaveFunction" and np.allclose(fattrs["L"], [L])
    s0, a0 = data["/states_0"]
    s1, _ = data["/states_1"]
    assert s0.dtype == np.int32 and s0.shape == s1.shape
    assert np.allclose(a0["kx"], qn[:, 0]) and np.allclose(a0["band"], qn[:, 2])
    half = L * L // 2
    if channel == 0:
        assert s0.shape == (1, L * L) and s0.sum() == half and (s0 == s1).all()
        assert (s0[0, 0::2] == 1).all()
    else:
        assert s0.shape == (half, L * L)
        assert (s0.sum(axis=1) == half + 1).all() and (s1.sum(axis=1) == half - 1).all()
        for e in range(half):
            add = np.flatnonzero(s0[e, 1::2]) * 2 + 1         # the upper-band orbital of flavour 0
            hole = np.flatnonzero(s1[e, 0::2] == 0) * 2      # the lower-band hole of flavour 1
            assert len(add) == 1 and len(hole) == 1
            dk = (qn[add[0], :2] - qn[hole[0], :2]) % L
            # k(particle) - k(hole) = q up to the (pi, pi) folding of the magnetic zone
            assert tuple(dk) in {(q[0] % L, q[1] % L), ((q[0] + L // 2) % L, (q[1] + L // 2) % L)}
    FakeH5py.files = {}
    out = g.convert_tree(fm.path("WaveFunction"), h5py_module=FakeH5py)
    f = FakeH5py.files[out]
    assert f["/states_0"].data.dtype == np.int32
    assert f["/states_0"].attrs["kx"].dtype == np.dtype(">u4")
