"""Green's-function consumers on the GPU: the functions of the reference's ``multimode.py`` (quadrature
and a-basis transfer matrices, covariance matrices, local-oscillator squeezing, down-sampling,
Bloch-Messiah principal values and vectors, time/frequency conversion, photon statistics, losses),
under the same names and arguments.

The element-wise assembly of the transfer matrices from C and S is the engine's own kernel
(``nlm_quadrature_greens`` / ``nlm_abasis_greens``); products are cuBLAS GEMMs and decompositions
cuSOLVER, both through torch; everything stays in FP64 on the device.

Arguments may be numpy arrays (the result comes back as numpy, like the reference) or CUDA tensors
(the result stays on the device).  The reference's convention hbar = 2 applies: x = a^dagger + a,
p = i (a^dagger - a).
"""

import ctypes

import numpy as np
import torch

from . import nonlinearmedium as nlm

__all__ = ["calcQuadratureGreens", "calcCovarianceMtx", "calcCovarianceMtxABasis", "normalizedCov",
           "calcLOSqueezing", "downSampledCov", "downSampledCovABasis", "blochMessiahEigs", "blochMessiahVecs",
           "ftGreens", "basisTransforms", "combineGreens", "incoherentPowerGreens", "photonMean", "photonMeanA",
           "photonCov", "photonCovA", "parametricFluorescence", "effectiveAdjacencyMatrix",
           "fullEffectiveAdjacencyMatrix", "covLumpLoss"]


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("the Green's-function consumers run on a CUDA device; none is available")


def _numpy_in(*xs):
    return any(not isinstance(x, torch.Tensor) for x in xs if x is not None)


def _dev(x, dtype=None):
    """x as a contiguous CUDA tensor (of dtype when given)."""
    _require_cuda()
    if isinstance(x, torch.Tensor):
        t = x if x.is_cuda else x.cuda()
    else:
        t = torch.as_tensor(np.asarray(x), device="cuda")
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    return t.contiguous()


def _ret(t, as_numpy):
    if isinstance(t, tuple):
        return tuple(_ret(u, as_numpy) for u in t)
    return t.cpu().numpy() if as_numpy else t


def _eye(n, dtype=torch.float64):
    return torch.eye(n, dtype=dtype, device="cuda")


def _assemble(C, S, fn, out_dtype):
    if C.shape != S.shape or C.dim() != 2:
        raise ValueError("greenC and greenS must be matrices of the same shape")
    rows, cols = C.shape
    out = torch.empty((2 * rows, 2 * cols), dtype=out_dtype, device="cuda")
    nlm._check(fn(ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(S.data_ptr()), rows, cols,
                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def _quadrature(C, S):
    return _assemble(_dev(C, torch.complex128), _dev(S, torch.complex128), nlm._lib.nlm_quadrature_greens,
                     torch.float64)


def _abasis(C, S):
    return _assemble(_dev(C, torch.complex128), _dev(S, torch.complex128), nlm._lib.nlm_abasis_greens,
                     torch.complex128)


def calcQuadratureGreens(greenC, greenS):
    """Z = [[Re(C+S), -Im(C-S)], [Im(C+S), Re(C-S)]] in the x/p basis (multimode.py:15-24)."""
    return _ret(_quadrature(greenC, greenS), _numpy_in(greenC, greenS))


def _covariance(Z, tol):
    cov = Z @ Z.T
    d = float(torch.linalg.det(cov))
    if not abs(d - 1) < tol:
        raise AssertionError("det(C) = %f" % d)
    return cov


def calcCovarianceMtx(Z, tol=1e-4):
    """Z Z^T, asserting |det - 1| < tol (multimode.py:27-36)."""
    return _ret(_covariance(_dev(Z, torch.float64), tol), _numpy_in(Z))


def calcCovarianceMtxABasis(greenC, greenS):
    """Z Z^dagger with Z = sqrt(1/2) [[C, S], [S*, C*]] (multimode.py:39-47)."""
    za = _abasis(greenC, greenS)
    return _ret(za @ za.mH, _numpy_in(greenC, greenS))


def normalizedCov(Cov):
    """(Cov - I) / sqrt(d_i d_j) (multimode.py:50-56)."""
    c = _dev(Cov)
    d = torch.diagonal(c)
    return _ret((c - _eye(c.shape[0], c.dtype)) / torch.sqrt(torch.outer(d, d)), _numpy_in(Cov))


def calcLOSqueezing(C, pumpProf, tol=1e-4, inTimeDomain=True):
    """Quadrature variances [min, max] seen by a local oscillator with the pump's spectral profile
    (multimode.py:59-84); C is the quadrature covariance matrix."""
    cov = _dev(C, torch.float64)
    p = _dev(pumpProf, torch.complex128)
    spec = torch.fft.fftshift(torch.fft.fft(p)) if inTimeDomain else torch.fft.fftshift(p)
    nrm = torch.linalg.vector_norm(spec)
    lx = torch.cat([spec.real, spec.imag]) / nrm
    lp = torch.cat([spec.imag, -spec.real]) / nrm
    s = lx + lp
    xx, pp, ss = (float(v @ (cov @ v)) for v in (lx, lp, s))
    xp = (ss - xx - pp) / 2
    m = np.array([[xx, xp], [xp, pp]])
    var = np.linalg.eigvals(m).astype(np.complex128)
    if not abs(xx - 1) < tol:
        raise AssertionError("C_xx = %f" % xx)
    var = np.array([np.min(var), np.max(var)])
    return var if _numpy_in(C, pumpProf) else torch.as_tensor(var, device="cuda")


def _sampling(omega, measurements, freqCutoff):
    w = omega.cpu().numpy() if isinstance(omega, torch.Tensor) else np.asarray(omega)
    cut = np.abs(np.fft.fftshift(w)) < freqCutoff
    n_cut = int(np.sum(cut))
    start = int(np.argmax(cut))
    return np.round(np.linspace(start, start + n_cut - 1, measurements)).astype(np.int64)


def downSampledCov(Z, measurements, omega, freqCutoff, nModeClasses=1):
    """Covariance of the quadratures at `measurements` bins spread over |w| < freqCutoff, per mode
    class (multimode.py:87-110)."""
    z = _dev(Z, torch.float64)
    samp = _sampling(omega, measurements, freqCutoff)
    nt = z.shape[0] // 2 // nModeClasses
    subset = np.concatenate([samp + nt * i for i in range(nModeClasses)])
    idx = torch.as_tensor(np.concatenate([subset, nt * nModeClasses + subset]), device="cuda")
    return _ret(_covariance(z.index_select(0, idx), np.inf), _numpy_in(Z))


def downSampledCovABasis(C, S, measurements, omega, freqCutoff, nModeClasses=1):
    """The a-basis covariance of the same down-sampled rows (multimode.py:113-137)."""
    c, s = _dev(C, torch.complex128), _dev(S, torch.complex128)
    samp = _sampling(omega, measurements, freqCutoff)
    nt = c.shape[0] // nModeClasses
    idx = torch.as_tensor(np.concatenate([samp + nt * i for i in range(nModeClasses)]), device="cuda")
    za = _abasis(c.index_select(0, idx), s.index_select(0, idx))
    return _ret(za @ za.mH, _numpy_in(C, S))


def _gram_eigh(z):
    """Eigen-decomposition of the symmetric Z Z^T (ascending), with the square roots of its values:
    the eigenvalues and eigenvectors of the polar factor sqrtm(Z Z^T): a symmetric eigensolver after
    one GEMM, in place of the reference's sqrtm and general eigensolver (an SVD of Z, the other
    route, took 16.6 s at 2048 x 2048 on this device)."""
    lam, u = torch.linalg.eigh(z @ z.T)
    return torch.sqrt(torch.clamp(lam, min=0.0)), u


def blochMessiahEigs(Z):
    """Bloch-Messiah principal values, ascending (multimode.py:140-147): the eigenvalues of
    sqrtm(Z Z^T)."""
    z = _dev(Z, torch.float64)
    s = torch.sqrt(torch.clamp(torch.linalg.eigvalsh(z @ z.T), min=0.0))
    return _ret(s, _numpy_in(Z))


def blochMessiahVecs(Z):
    """(values, left vectors, right vectors) of Z = L diag(values) R (multimode.py:150-170), ordered
    as the N largest values descending then the N smallest ascending.  With sqrtm(Z Z^T) = U s U^T,
    the left vectors are U and the right vectors U^T sqrtm(Z Z^T)^-1 Z = s^-1 U^T Z.  Each vector is
    determined up to its sign (the reference's eigenvector normalisation)."""
    z = _dev(Z, torch.float64)
    s, u = _gram_eigh(z)
    n = z.shape[0] // 2
    idx = torch.cat([torch.arange(2 * n - 1, n - 1, -1, device="cuda"), torch.arange(n, device="cuda")])
    right = (u.T @ z)[idx] / s[idx][:, None]
    return _ret((s[idx], u[:, idx], right), _numpy_in(Z))


def ftGreens(greenC, greenS, toTime=True):
    """Green's matrices converted between the frequency and time domains (multimode.py:173-186)."""
    c, s = _dev(greenC, torch.complex128), _dev(greenS, torch.complex128)
    f = torch.fft
    if toTime:
        cc = f.fftshift(f.fft(f.ifft(f.ifftshift(c), dim=0), dim=1))
        cs = f.fftshift(f.ifft2(f.ifftshift(s))) * s.shape[0]
    else:
        cc = f.fftshift(f.ifft(f.fft(f.ifftshift(c), dim=0), dim=1))
        cs = f.fftshift(f.fft2(f.ifftshift(s))) / s.shape[0]
    return _ret((cc, cs), _numpy_in(greenC, greenS))


def basisTransforms(n):
    """(a -> xp, xp -> a) transformation matrices (multimode.py:189-196), as numpy arrays."""
    i = np.eye(n)
    to_xp = np.block([[i, i], [-1j * i, 1j * i]])
    from_xp = np.block([[i, 1j * i], [i, -1j * i]]) * 0.5
    return to_xp, from_xp


def combineGreens(Cfirst, Sfirst, Csecond, Ssecond):
    """C2 C1 + S2 S1*, C2 S1 + S2 C1* (multimode.py:199-205)."""
    c1, s1, c2, s2 = (_dev(x, torch.complex128) for x in (Cfirst, Sfirst, Csecond, Ssecond))
    return _ret((c2 @ c1 + s2 @ s1.conj(), c2 @ s1 + s2 @ c1.conj()), _numpy_in(Cfirst, Sfirst, Csecond, Ssecond))


def incoherentPowerGreens(Z):
    """Power transfer matrix for incoherent light (multimode.py:208-216)."""
    z = _dev(Z)
    n = z.shape[0] // 2
    return _ret(0.5 * (z[:n, :n] ** 2 + z[n:, n:] ** 2 + z[:n, n:] ** 2 + z[n:, :n] ** 2), _numpy_in(Z))


def photonMean(V):
    """Mean photon number per mode from the quadrature covariance (multimode.py:219-225)."""
    v = _dev(V)
    n = v.shape[0] // 2
    return _ret(0.25 * (torch.diagonal(v[:n, :n]) + torch.diagonal(v[n:, n:]) - 2), _numpy_in(V))


def photonMeanA(sigma):
    """Mean photon number per mode from the a-basis covariance (multimode.py:228-235)."""
    s = _dev(sigma)
    n = s.shape[0] // 2
    return _ret(torch.diagonal(s[:n, :n]).real - 0.5, _numpy_in(sigma))


def photonCov(V):
    """Photon-number covariance from the quadrature covariance (multimode.py:238-245)."""
    v = _dev(V)
    n = v.shape[0] // 2
    out = 0.125 * (v[:n, :n] ** 2 + v[:n, n:] ** 2 + v[n:, :n] ** 2 + v[n:, n:] ** 2) - 0.25 * _eye(n, v.dtype)
    return _ret(out, _numpy_in(V))


def photonCovA(sigma):
    """Photon-number covariance from the a-basis covariance (multimode.py:248-253).  The reference's
    body names undefined variables and raises NameError; this computes its evident formula
    |sigma_aa|^2 + |sigma_aa*|^2 - I/4 with n = half the matrix size."""
    s = _dev(sigma)
    n = s.shape[0] // 2
    out = torch.abs(s[:n, :n]) ** 2 + torch.abs(s[:n, n:]) ** 2 - 0.25 * _eye(n)
    return _ret(out, _numpy_in(sigma))


def parametricFluorescence(modes, diag):
    """Parametric fluorescence spectrum from a decomposition (multimode.py:256-261)."""
    m, d = _dev(modes), _dev(diag)
    return _ret(torch.sum(torch.abs(m) ** 2 * torch.sinh(torch.log(d[:, None])) ** 2, dim=0), _numpy_in(modes, diag))


def effectiveAdjacencyMatrix(modes, diag):
    """B = U^T tanh(|log d|) U (multimode.py:264-272)."""
    m, d = _dev(modes), _dev(diag)
    return _ret(m.T @ torch.diag(torch.tanh(torch.abs(torch.log(d)))).to(m.dtype) @ m, _numpy_in(modes, diag))


def fullEffectiveAdjacencyMatrix(cov):
    """[[0, I], [I, 0]] (I - (cov + I/2)^-1) (multimode.py:275-288)."""
    c = _dev(cov)
    n = c.shape[0]
    h = n // 2
    i = _eye(n, c.dtype)
    swap = torch.zeros((n, n), dtype=c.dtype, device="cuda")
    swap[:h, h:] = i[:h, :h]
    swap[h:, :h] = i[:h, :h]
    return _ret(swap @ (i - torch.linalg.inv(c + 0.5 * i)), _numpy_in(cov))


def covLumpLoss(cov, transmission, abasis=False):
    """A lumped loss of transmission t (scalar or per mode) on a covariance matrix (multimode.py:291-310)."""
    c = _dev(cov)
    vac = 0.5 if abasis else 1
    n = c.shape[0]
    if not np.shape(transmission):
        t = float(transmission)
        return _ret(t * c + ((1 - t) * vac) * _eye(n, c.dtype), _numpy_in(cov))
    t = _dev(transmission, torch.float64).repeat(2)
    st = torch.sqrt(t)
    out = torch.outer(st, st).to(c.dtype) * c + torch.diag((1 - t) * vac).to(c.dtype)
    return _ret(out, _numpy_in(cov))
