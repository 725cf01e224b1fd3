"""The allocation-free Chi3GNLSE batch entry point (nlm_batch_gnlse_noalloc).

It exists for callers that cannot allocate device memory where they propagate (memory owned by
another allocator with a fixed budget, or loops where a cudaMalloc/cudaFree would synchronise the
device).  It must give the same rows as the ordinary batch entry point, call after call, although
every call reuses the same file-scope scratch array.  Collected last (file name) so that a run
stopping at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _bind(nlm):
    fn = nlm._lib.nlm_batch_gnlse_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p]
    return fn


def test_noalloc_batch_matches_batch_entry_point(nlm):
    torch = pytest.importorskip("torch")
    fn = _bind(nlm)
    med = nlm.Chi3GNLSE(**cases.CASES["Chi3GNLSE"])
    n = med._dims["nFreqs"]
    rows = 5
    x = np.stack([cases.signal_input("Chi3GNLSE", n, 1, seed=20 + k) for k in range(rows)])
    stream = torch.cuda.current_stream()
    for in_time in (False, True):
        expected = med.batchSignalSimulation(x, in_time)   # existing entry point; builds the device tables
        xin = torch.from_numpy(x).to("cuda")
        for _ in range(2):                                  # two calls in a row on the shared scratch
            out = torch.full((rows, n), float("nan"), dtype=torch.complex128, device="cuda")
            status = fn(med._h(), ctypes.c_void_p(xin.data_ptr()), rows, int(in_time), ctypes.c_void_p(out.data_ptr()),
                        ctypes.c_void_p(stream.cuda_stream))
            assert status == 0, nlm._lib.nlm_last_error().decode()
            torch.cuda.synchronize()
            assert cases.rel_l2(out.cpu().numpy(), expected) < TOL


def test_noalloc_rounds_over_capped_grid(nlm):
    """At N=4096 the array holds 128 slots of 2N values, fewer than the SMs: the grid is capped at
    128 CTAs, and 300 rows make the CTAs walk several rows each in the static round robin, reusing
    their slot.  Two calls in a row must match the ordinary batch entry point.  The medium is the
    GNLSE batch workload's (N=4096, its z step) over 40 steps."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG
    fn = _bind(nlm)
    med = nlm.Chi3GNLSE(**dict(GNLSE_CONFIG, relativeLength=0.004))
    n = med._dims["nFreqs"]
    rows = 300
    t = np.fft.fftshift(np.linspace(-50, 50, n, endpoint=False))
    rng = np.random.default_rng(30)
    x = 3.0 / np.cosh(t)[None, :] + cases.noise(rng, rows * n, 1e-4).reshape(rows, n)
    expected = med.batchSignalSimulation(x, True)
    assert np.all(np.isfinite(expected))
    xin = torch.from_numpy(x).to("cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        out = torch.full((rows, n), float("nan"), dtype=torch.complex128, device="cuda")
        status = fn(med._h(), ctypes.c_void_p(xin.data_ptr()), rows, 1, ctypes.c_void_p(out.data_ptr()),
                    ctypes.c_void_p(stream.cuda_stream))
        assert status == 0, nlm._lib.nlm_last_error().decode()
        torch.cuda.synchronize()
        assert cases.rel_l2(out.cpu().numpy(), expected) < TOL


def test_noalloc_rejects_other_solvers(nlm):
    torch = pytest.importorskip("torch")
    fn = _bind(nlm)
    med = nlm.Chi2SHG(**cases.CASES["Chi2SHG"])
    buf = torch.zeros((1, 2 * med._dims["nFreqs"]), dtype=torch.complex128, device="cuda")
    status = fn(med._h(), ctypes.c_void_p(buf.data_ptr()), 1, 0, ctypes.c_void_p(buf.data_ptr()), None)
    assert status == 1
    assert "Chi3GNLSE" in nlm._lib.nlm_last_error().decode()


def test_noalloc_rejects_grids_of_the_cluster_kernels(nlm):
    """8192 points need more than the one-CTA kernel's 512 threads: rejected as unsupported
    (status 6) with the reason, before anything is launched."""
    torch = pytest.importorskip("torch")
    fn = _bind(nlm)
    med = nlm.Chi3GNLSE(**dict(cases.CASES["Chi3GNLSE"], tMax=40, tPrecision=8192, zPrecision=4))
    n = med._dims["nFreqs"]
    med.batchSignalSimulation(np.ones((1, n), dtype=np.complex128), False)
    buf = torch.zeros((1, n), dtype=torch.complex128, device="cuda")
    status = fn(med._h(), ctypes.c_void_p(buf.data_ptr()), 1, 0, ctypes.c_void_p(buf.data_ptr()), None)
    assert status == 6
    assert "8192" in nlm._lib.nlm_last_error().decode()
