"""gv_slater_invert_noalloc: the allocation-free inversion entry point.

It is for callers that cannot let a library allocate device memory (an
application that pre-allocates all of its HBM and forbids allocations later,
or a latency-critical loop that cannot afford cudaMalloc's implicit
synchronisation).  The test allocates the input and output buffers itself
(with torch), calls the entry point through the C ABI twice in a row, and
checks each result against the inverse and determinant the existing job
path (gv_job_init_walkers' FP64 inversion) produced for the same Slater
matrix, to the parity tolerance the other GPU tests use.  It sits in a file of
its own, collected last.
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-10
PHI, NEEL, L = 0.25 * math.pi, 0.1, 16


def slater_matrix(lib, job, walker, fl):
    """A(f, r) = phi_{2f}(site of particle r) in the reference's column-major
    m_mat layout, A[r*N + f] (SlaterDeterminant.cpp:64-70)."""
    Ns = L * L
    N = job.N[fl]
    out = np.zeros(2 * Ns * Ns)
    bc = (ctypes.c_double * 2)(1.0, 1.0)
    assert lib.gv_phi_table(L, PHI, NEEL, 0.0, bc, fl, out.ctypes.data_as(ctypes.c_void_p)) == 0
    phi = (out[0::2] + 1j * out[1::2]).reshape(Ns, Ns)          # [orbital, site]
    orb = 2 * np.arange(N)                                       # ground state: lower band
    sites = job.particles(walker, fl)
    return np.ascontiguousarray(phi[np.ix_(orb, sites)].T)      # [r, f] = A(f, r)


def test_noalloc_inverse_matches_job_path(engine):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = engine.lib()
    job = engine.Job(engine.StagFluxGroundState(L, PHI, NEEL), walkers=2, seed=97, precision="fp64")
    job.init_walkers()
    mant, exp10 = job.amplitude()
    stream = torch.cuda.current_stream().cuda_stream
    for walker in (0, 1):
        det = 1.0 + 0.0j
        det_log2 = 0.0
        for fl in (0, 1):                      # two calls in a row per walker
            A = slater_matrix(lib, job, walker, fl)
            N = A.shape[0]
            dA = torch.from_numpy(A.view(np.float64).copy()).cuda()
            dAi = torch.full((2 * N * N,), float("nan"), dtype=torch.float64, device="cuda")
            dinfo = torch.zeros(4, dtype=torch.float64, device="cuda")
            st = lib.gv_slater_invert_noalloc(ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dAi.data_ptr()), N,
                                              ctypes.c_void_p(dinfo.data_ptr()), ctypes.c_void_p(stream))
            assert st == 0
            torch.cuda.synchronize()
            info = dinfo.cpu().numpy()
            assert info[3] == 0
            got = dAi.cpu().numpy()
            got = (got[0::2] + 1j * got[1::2]).reshape(N, N).T       # column-major -> [p, f]
            want = job.inverse(walker, fl)
            assert np.abs(got - want).max() < RTOL * np.abs(want).max()
            # the input is untouched, and the inverse is one
            assert np.array_equal(dA.cpu().numpy().ravel(), A.view(np.float64).ravel())
            Amat = A.T                                                # [f, r]
            assert np.abs(got @ Amat - np.eye(N)).max() < 1e-9
            det *= complex(info[0], info[1])
            det_log2 += info[2]
        # amplitude = det_0 * det_1 (SlaterDeterminant.cpp:82-88)
        l10 = math.log10(abs(det)) + det_log2 * math.log10(2.0)
        l10_ref = math.log10(abs(mant[walker])) + exp10[walker]
        assert abs(l10 - l10_ref) < 1e-10
        ph_got = det / abs(det)
        ph_ref = mant[walker] / abs(mant[walker])
        assert abs(ph_got - ph_ref) < 1e-10
    job.close()


def test_noalloc_rejects_oversize(engine):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = engine.lib()
    buf = torch.zeros(2 * 129 * 129, dtype=torch.float64, device="cuda")
    info = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(buf.data_ptr())
    assert lib.gv_slater_invert_noalloc(p, p, 129, ctypes.c_void_p(info.data_ptr()), None) == 10
    assert b"N <= 128" in lib.gv_status_string(10)


def test_noalloc_singular_reports_zero_determinant(engine):
    """linalg::DetInv's singular rule (|det|^2 < 1e-9, linalg.cpp:23): status
    GV_ERR_SINGULAR with a zero mantissa; just above the bar the inverse and
    determinant come back."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = engine.lib()
    stream = torch.cuda.current_stream().cuda_stream
    for d4, want in ((1e-5, 2), (1e-4, 0), (0.0, 2)):
        A = np.diag([1.0 + 0.5j, 2.0, 1.0j, d4]).astype(np.complex128)
        A[0, 1] = 0.25
        dA = torch.from_numpy(np.ascontiguousarray(A.T).view(np.float64).ravel().copy()).cuda()
        dAi = torch.zeros(32, dtype=torch.float64, device="cuda")
        dinfo = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
        st = lib.gv_slater_invert_noalloc(ctypes.c_void_p(dA.data_ptr()), ctypes.c_void_p(dAi.data_ptr()), 4,
                                          ctypes.c_void_p(dinfo.data_ptr()), ctypes.c_void_p(stream))
        assert st == 0
        torch.cuda.synchronize()
        info = dinfo.cpu().numpy()
        assert info[3] == want, (d4, info)
        if want:
            assert info[0] == 0.0 and info[1] == 0.0
        else:
            det = complex(info[0], info[1]) * 2.0 ** info[2]
            assert abs(det - np.linalg.det(A)) < 1e-12 * abs(np.linalg.det(A))
