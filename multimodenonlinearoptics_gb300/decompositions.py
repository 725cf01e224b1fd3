"""Bloch-Messiah decomposition on the GPU: the functions of the reference's ``decompositions.py`` that
it needs (``sympmat``, ``leftPolar``, ``takagi``, ``bloch_messiah``; the reference's copy of the
Strawberry Fields decompositions), under the same names and arguments.

The SVDs and eigen-decompositions are cuSOLVER's through torch (FP64); the few host steps are the
degeneracy bookkeeping over the 2N singular values.  Arguments may be numpy arrays (numpy results)
or CUDA tensors (results on the device).  Singular vectors are determined up to signs and, inside
degenerate subspaces, up to rotations: the factors can differ from the reference's LAPACK ones by
such transformations, while the squeezing values and the products agree.
"""

import numpy as np
import torch

from .multimode import _dev, _numpy_in, _ret

__all__ = ["sympmat", "leftPolar", "takagi", "bloch_messiah"]


def sympmat(n):
    """[[0, I], [-I, 0]] of order 2n (decompositions.py:17-28), as a numpy array."""
    i = np.identity(n)
    z = np.zeros((n, n))
    return np.block([[z, i], [-i, z]])


_POLAR_EIGH_MIN = 512   # square matrices from this size: polar factor from a symmetric eigensolver


def _leftPolar(a):
    if a.shape[0] == a.shape[1] and a.shape[0] >= _POLAR_EIGH_MIN:
        # p = sqrtm(a a^dagger) = w s w^dagger, u = p^-1 a: one GEMM and a symmetric eigensolver in
        # place of the SVD (cuSOLVER's FP64 SVD of a 2048 x 2048 matrix took 16.6 s on GB300)
        lam, w = torch.linalg.eigh(a @ a.mH)
        s = torch.sqrt(torch.clamp(lam, min=0.0)).to(w.dtype)
        return (w / s) @ (w.mH @ a), (w * s) @ w.mH
    w, s, vh = torch.linalg.svd(a, full_matrices=False)
    return w @ vh, (w * s.to(w.dtype)) @ w.mH


def leftPolar(a):
    """Left polar decomposition a = p u: u unitary, p = w s w^dagger Hermitian positive
    semidefinite, returned as (u, p) (decompositions.py:48-64)."""
    return _ret(_leftPolar(_dev(a)), _numpy_in(a))


def _sqrtm(m):
    """Principal square root of a small diagonalisable matrix from its eigen-decomposition."""
    lam, v = torch.linalg.eig(m.to(torch.complex128))
    return v @ torch.diag(torch.sqrt(lam)) @ torch.linalg.inv(v)


def _takagi(N, tol, rounding):
    n = N.shape[0]
    if N.shape[0] != N.shape[1]:
        raise ValueError("The input matrix must be square")
    err = float(torch.linalg.matrix_norm(N - N.T)) / n
    if err >= tol:
        raise ValueError("The input matrix is not symmetric (error = %f)" % err)
    if not N.is_complex() or bool(torch.all(N.imag == 0)):
        l, U = torch.linalg.eigh(N.real if N.is_complex() else N)
        phase = torch.where(l < 0, torch.tensor(1j, dtype=torch.complex128, device=l.device),
                            torch.tensor(1 + 0j, dtype=torch.complex128, device=l.device))
        Uc = U.to(torch.complex128) * phase[None, :]
        l = torch.abs(l)
        perm = torch.argsort(l, descending=True, stable=True)
        return l[perm], Uc[:, perm]
    v, l, ws = torch.linalg.svd(N)
    rl = torch.round(l, decimals=rounding)
    counts = np.unique(np.round(rl.cpu().numpy(), rounding), return_counts=True)[1][::-1]
    w = ws.mH
    blocks, first = [], 0
    for c in counts:
        c = int(c)
        blocks.append(_sqrtm(v[:, first:first + c].T @ w[:, first:first + c]))
        first += c
    return rl, v @ torch.block_diag(*blocks).conj()


def takagi(N, tol=1e-13, rounding=13):
    """Autonne-Takagi decomposition N = U diag(l) U^T of a complex symmetric matrix, values
    descending (decompositions.py:67-136)."""
    return _ret(_takagi(_dev(N), tol, rounding), _numpy_in(N))


def bloch_messiah(S, tol=1e-10, rounding=9):
    """S = ut1 st1 v1 with ut1, v1 symplectic orthogonal and st1 = diag(s_1..s_n, 1/s_1..1/s_n) in
    the canonical order (decompositions.py:250-355)."""
    s = _dev(S)
    n2, m = s.shape
    if n2 != m:
        raise ValueError("The input matrix is not square")
    if n2 % 2 != 0:
        raise ValueError("The input matrix must have an even number of rows/columns")
    n = n2 // 2
    om = torch.as_tensor(sympmat(n), dtype=s.dtype, device="cuda")
    err = float(torch.linalg.matrix_norm(s.T @ om @ s - om)) / n
    if err >= tol:
        raise ValueError("The input matrix is not symplectic (error = %f)" % err)
    eye = torch.eye(2 * n, dtype=torch.float64, device="cuda")
    if float(torch.linalg.matrix_norm(s.T @ s - eye)) < tol:
        return _ret((s.real if s.is_complex() else s, eye, eye), _numpy_in(S))
    u, sigma = _leftPolar(s)
    ss, uss = _takagi(sigma, tol, rounding)
    z = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    i = torch.eye(n, dtype=torch.float64, device="cuda")
    pmat = torch.cat([torch.cat([i, z], 1), torch.cat([z, torch.flip(i, (0,))], 1)], 0)
    ut = uss @ pmat.to(uss.dtype)
    qom = ut.T @ om.to(ut.dtype) @ ut
    counts = np.unique(np.round(ss[:n].cpu().numpy(), rounding), return_counts=True)[1][::-1]
    if counts.size < n:
        ul, vl, first = [], [], 0
        for c in counts:
            c = int(c)
            last = first + c
            if c > 1:
                us, _, vs = torch.linalg.svd(qom[first:last, n + first:n + last].real)
                ul.append(us)
                vl.append(vs.T)
            else:
                one = torch.ones((1, 1), dtype=torch.float64, device="cuda")
                ul.append(torch.sign(qom[first, n + first].real) * one)
                vl.append(one)
            first = last
        pmat1 = torch.block_diag(*(ul + vl))
    else:
        sg = torch.diag(torch.sign(torch.diagonal(qom[:n, n:].real)))
        pmat1 = torch.cat([torch.cat([sg, z], 1), torch.cat([z, i], 1)], 0)
    perm = pmat @ pmat1
    st1 = perm.T @ torch.diag(ss.to(torch.float64)) @ perm
    ut1 = uss @ perm.to(uss.dtype)
    v1 = ut1.T @ u.to(ut1.dtype)
    return _ret((ut1.real, st1, v1.real), _numpy_in(S))
