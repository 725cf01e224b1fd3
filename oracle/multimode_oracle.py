"""CPU oracle for the Green's-function consumers of MultimodeNonlinearOptics.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module: only ``tests/`` and the CPU
legs of ``bench.py`` use it, as the checker and as the timed CPU baseline.

A numpy/scipy restatement of the reference's helpers that turn the Green's matrices (C, S) into
quadrature transfer matrices, covariance matrices, photon statistics and Bloch-Messiah
decompositions: ``multimode.py`` (the project's own module) and ``decompositions.py`` (the project's
copy of the Strawberry Fields decompositions, Apache-2.0).  Every function cites the reference
file:line it restates.  The reference modules predate numpy 2 (``np.float_``, ``np.int``); the
restatement uses float64 / int instead.

Parity status: PINNED.  ``tests/golden/make_golden.py`` imports the reference modules themselves
and stores their outputs on seeded inputs (``multimode_golden.npz``); ``tests/test_oracle.py``
checks this restatement against them.
"""

import numpy as np
from scipy.linalg import block_diag, det, eig, eigvals, inv, norm, sqrtm, svd


# ---- multimode.py --------------------------------------------------------------------------------
def quadrature_greens(C, S):
    """multimode.py:15-24 (calcQuadratureGreens): Z in the x/p basis from a_out = C a + S a^dagger."""
    top = np.hstack([(C + S).real, -(C - S).imag])
    bottom = np.hstack([(C + S).imag, (C - S).real])
    return np.vstack([top, bottom]).astype(np.float64)


def covariance(Z, tol=1e-4):
    """multimode.py:27-36 (calcCovarianceMtx): Z Z^T, with |det - 1| < tol asserted."""
    cov = Z @ Z.T
    d = det(cov)
    if not abs(d - 1) < tol:
        raise AssertionError("det(C) = %f" % d)
    return cov


def covariance_abasis(C, S):
    """multimode.py:39-47 (calcCovarianceMtxABasis): Z Z^dagger with Z = sqrt(1/2) [[C, S], [S*, C*]]."""
    Z = np.vstack([np.hstack([C, S]), np.hstack([S.conj(), C.conj()])]) * np.sqrt(1 / 2)
    return Z @ Z.T.conj()


def normalized_cov(cov):
    """multimode.py:50-56 (normalizedCov): (Cov - I) / sqrt(d_i d_j)."""
    d = np.diag(cov)
    return (cov - np.eye(cov.shape[0])) / np.sqrt(np.outer(d, d))


def lo_squeezing(cov, pump_prof, tol=1e-4, in_time_domain=True):
    """multimode.py:59-84 (calcLOSqueezing): quadrature variances seen by a local oscillator with the
    pump's spectral profile; returns [min, max] of the 2x2 covariance's eigenvalues."""
    spec = np.fft.fftshift(np.fft.fft(pump_prof)) if in_time_domain else np.fft.fftshift(pump_prof)
    nrm = norm(spec)
    lx = np.concatenate([spec.real, spec.imag]) / nrm
    lp = np.concatenate([spec.imag, -spec.real]) / nrm
    m = np.zeros((2, 2))
    m[0, 0] = lx @ cov @ lx
    m[1, 1] = lp @ cov @ lp
    m[0, 1] = m[1, 0] = ((lx + lp) @ cov @ (lx + lp) - m[0, 0] - m[1, 1]) / 2
    var = eigvals(m)
    if not abs(m[0, 0] - 1) < tol:
        raise AssertionError("C_xx = %f" % m[0, 0])
    var[0], var[1] = np.min(var), np.max(var)
    return var


def _sampling(omega, measurements, freq_cutoff):
    cut = np.abs(np.fft.fftshift(omega)) < freq_cutoff
    n_cut = int(np.sum(cut))
    start = int(np.argmax(cut))
    return np.round(np.linspace(start, start + n_cut - 1, measurements)).astype(int)


def downsampled_cov(Z, measurements, omega, freq_cutoff, n_mode_classes=1):
    """multimode.py:87-110 (downSampledCov): rows of Z at `measurements` bins spread over |w| < cutoff
    (per mode class), then Zcut Zcut^T."""
    samp = _sampling(omega, measurements, freq_cutoff)
    nt = Z.shape[0] // 2 // n_mode_classes
    subset = np.concatenate([samp + nt * i for i in range(n_mode_classes)])
    zcut = np.vstack([Z[subset], Z[nt * n_mode_classes + subset]])
    return covariance(zcut, np.inf)


def downsampled_cov_abasis(C, S, measurements, omega, freq_cutoff, n_mode_classes=1):
    """multimode.py:113-137 (downSampledCovABasis)."""
    samp = _sampling(omega, measurements, freq_cutoff)
    nt = C.shape[0] // n_mode_classes
    subset = np.concatenate([samp + nt * i for i in range(n_mode_classes)])
    return covariance_abasis(C[subset], S[subset])


def bloch_messiah_eigs(Z):
    """multimode.py:140-147 (blochMessiahEigs): sorted eigenvalues of sqrtm(Z Z^T), real parts."""
    return np.sort(eigvals(sqrtm(Z @ Z.T))).real


def bloch_messiah_vecs(Z):
    """multimode.py:150-170 (blochMessiahVecs): eigen-decomposition of the polar factor sqrtm(Z Z^T),
    ordered as the N largest values descending then the N smallest ascending, and the right vectors
    U^T polar^-1 Z in the same order."""
    polar = sqrtm(Z @ Z.T)
    diag, left = eig(polar)
    order = np.argsort(diag)
    n = Z.shape[0] // 2
    order = np.concatenate([order[-1:-n - 1:-1], order[:n]])
    right = left.T @ (inv(polar) @ Z)
    return diag[order].real, left[:, order], right[order]


def ft_greens(C, S, to_time=True):
    """multimode.py:173-186 (ftGreens): Green's matrices between the frequency and time domains."""
    if to_time:
        c = np.fft.fftshift(np.fft.fft(np.fft.ifft(np.fft.ifftshift(C), axis=0), axis=1))
        s = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(S))) * S.shape[0]
    else:
        c = np.fft.fftshift(np.fft.ifft(np.fft.fft(np.fft.ifftshift(C), axis=0), axis=1))
        s = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(S))) / S.shape[0]
    return c, s


def basis_transforms(n):
    """multimode.py:189-196 (basisTransforms): a basis -> xp basis and back."""
    i = np.eye(n)
    to_xp = np.block([[i, i], [-1j * i, 1j * i]])
    from_xp = np.block([[i, 1j * i], [i, -1j * i]]) * 0.5
    return to_xp, from_xp


def combine_greens(c1, s1, c2, s2):
    """multimode.py:199-205 (combineGreens): the second medium after the first."""
    return c2 @ c1 + s2 @ np.conjugate(s1), c2 @ s1 + s2 @ np.conjugate(c1)


def incoherent_power_greens(Z):
    """multimode.py:208-216 (incoherentPowerGreens)."""
    n = Z.shape[0] // 2
    return 0.5 * (Z[:n, :n] ** 2 + Z[n:, n:] ** 2 + Z[:n, n:] ** 2 + Z[n:, :n] ** 2)


def photon_mean(V):
    """multimode.py:219-225 (photonMean): (V_xx + V_pp - 2) / 4 on the diagonal."""
    n = V.shape[0] // 2
    return 0.25 * (V[:n, :n].diagonal() + V[n:, n:].diagonal() - 2)


def photon_mean_a(sigma):
    """multimode.py:228-235 (photonMeanA)."""
    n = sigma.shape[0] // 2
    return sigma[:n, :n].diagonal().real - 0.5


def photon_cov(V):
    """multimode.py:238-245 (photonCov)."""
    n = V.shape[0] // 2
    return 0.125 * (V[:n, :n] ** 2 + V[:n, n:] ** 2 + V[n:, :n] ** 2 + V[n:, n:] ** 2) - 0.25 * np.eye(n)


def photon_cov_a(sigma):
    """multimode.py:248-253 (photonCovA).  The reference body names undefined variables (V, nt) and
    raises NameError; this is its evident formula with n = half the matrix size."""
    n = sigma.shape[0] // 2
    return np.abs(sigma[:n, :n]).real ** 2 + np.abs(sigma[:n, n:]).real ** 2 - 0.25 * np.eye(n)


def parametric_fluorescence(modes, diag):
    """multimode.py:256-261 (parametricFluorescence)."""
    return np.sum(np.abs(modes) ** 2 * np.sinh(np.log(diag[:, np.newaxis])) ** 2, axis=0)


def effective_adjacency(modes, diag):
    """multimode.py:264-272 (effectiveAdjacencyMatrix): U^T tanh(|log d|) U."""
    return modes.T @ np.diag(np.tanh(np.abs(np.log(diag)))) @ modes


def full_effective_adjacency(cov):
    """multimode.py:275-288 (fullEffectiveAdjacencyMatrix): [[0, I], [I, 0]] (I - (cov + I/2)^-1)."""
    n = cov.shape[0]
    i = np.identity(n)
    h = n // 2
    swap = np.block([[np.zeros((h, h)), i[:h, :h]], [i[:h, :h], np.zeros((h, h))]])
    return swap @ (i - inv(cov + 0.5 * i))


def cov_lump_loss(cov, transmission, abasis=False):
    """multimode.py:291-310 (covLumpLoss): a beam splitter to vacuum with transmission t."""
    vac = 0.5 if abasis else 1
    if not np.shape(transmission):
        return transmission * cov + ((1 - transmission) * vac) * np.identity(cov.shape[0])
    t = np.tile(transmission, 2)
    st = np.sqrt(t)
    return np.outer(st, st) * cov + ((1 - t) * vac) * np.identity(cov.shape[0])


# ---- decompositions.py ---------------------------------------------------------------------------
def sympmat(n):
    """decompositions.py:17-28: [[0, I], [-I, 0]]."""
    i = np.identity(n)
    z = np.zeros((n, n))
    return np.block([[z, i], [-i, z]])


def left_polar(a):
    """decompositions.py:48-64 (leftPolar): a = u p with u unitary, p = w s w^dagger."""
    w, s, vh = svd(np.asarray(a), full_matrices=False)
    return w @ vh, (w * s) @ w.T.conj()


def takagi(N, tol=1e-13, rounding=13):
    """decompositions.py:67-136: N = U diag(l) U^T for complex symmetric N, values descending."""
    n = N.shape[0]
    if N.shape[0] != N.shape[1]:
        raise ValueError("The input matrix must be square")
    err = np.linalg.norm(N - N.T) / n
    if err >= tol:
        raise ValueError("The input matrix is not symmetric (error = %f)" % err)
    if np.isrealobj(N) or np.all(N.imag == 0):
        l, U = np.linalg.eigh(N.real)
        phase = np.where(l < 0, 1j, 1.0 + 0j)
        Uc = U * phase[np.newaxis, :]
        l = np.abs(l)
        perm = np.argsort(l)[::-1]
        return l[perm], Uc[:, perm]
    v, l, ws = svd(N)
    rl = np.round(l, rounding)
    counts = np.unique(np.round(rl, rounding), return_counts=True)[1][::-1]
    w = ws.T.conj()
    blocks, first = [], 0
    for c in counts:
        va, wa = v[:, first:first + c], w[:, first:first + c]
        blocks.append(sqrtm(va.T @ wa))
        first += c
    return rl, v @ np.conj(block_diag(*blocks))


def bloch_messiah(S, tol=1e-10, rounding=9):
    """decompositions.py:250-355: S = ut1 st1 v1 with ut1, v1 symplectic orthogonal and st1 =
    diag(s_1..s_n, 1/s_1..1/s_n) in canonical order."""
    n2, m = S.shape
    if n2 != m:
        raise ValueError("The input matrix is not square")
    if n2 % 2 != 0:
        raise ValueError("The input matrix must have an even number of rows/columns")
    n = n2 // 2
    om = sympmat(n)
    err = np.linalg.norm(S.T @ om @ S - om) / n
    if err >= tol:
        raise ValueError("The input matrix is not symplectic (error = %f)" % err)
    if np.linalg.norm(S.T @ S - np.eye(2 * n)) < tol:
        return S.real, np.eye(2 * n), np.eye(2 * n)
    u, sigma = left_polar(S)
    ss, uss = takagi(sigma, tol=tol, rounding=rounding)
    z = np.zeros((n, n))
    pmat = np.block([[np.identity(n), z], [z, np.identity(n)[::-1]]])
    ut = uss @ pmat
    qom = ut.T @ om @ ut
    counts = np.unique(np.round(ss[:n], rounding), return_counts=True)[1][::-1]
    if counts.size < n:
        ul, vl, first = [], [], 0
        for c in counts:
            last = first + c
            if c > 1:
                us, _, vs = svd(qom[first:last, n + first:n + last].real)
                ul.append(us)
                vl.append(vs.T)
            else:
                ul.append(np.sign(qom[first, n + first]))
                vl.append(1)
            first = last
        pmat1 = block_diag(*(ul + vl))
    else:
        pmat1 = np.block([[np.diag(np.sign(qom[:n, n:].real.diagonal())), z], [z, np.eye(n)]])
    perm = pmat @ pmat1
    st1 = perm.T @ np.diag(ss) @ perm
    ut1 = uss @ perm
    v1 = ut1.T @ u
    return ut1.real, st1.real, v1.real
