"""Poling-pattern helpers for chi(2) media (host side).

The functions return arrays of domain lengths, the format every solver's ``poling=`` argument and
``setPoling`` take (the engine turns them into per-step orientations, ``src/_NonlinearMedium.cpp:470-503``).
Here are the closed-form generators of the reference's ``poling.py`` (periodic, linearly chirped and
artanh-detuned patterns sampled on a grid, and the three-wave mismatch range), each written from its
formula, and ``domainsToSpace``, the vectorised twin of ``setPoling`` that the engine is checked
against bit for bit.  The reference's procedural pattern designers (``linearPolingContinuous``,
``dutyCyclePmf``, ``deletedDomainPmf``, ``combinePoling``) are plain numpy host code with no device
counterpart: use the reference's own ``poling.py`` for them, which runs beside this engine unchanged
and whose outputs feed ``poling=`` directly.  This is setup work on the host: it runs once per
design, before any propagation.
"""

import numpy as np

__all__ = ["periodicPoling", "linearPoling", "detunePoling", "threeWaveMismatchRange", "domainsToSpace"]


def _run_lengths(orientation):
    """Lengths of the maximal runs of equal values in a 1-D array of +/-1."""
    n = orientation.size
    if n == 0:
        return np.zeros(0, dtype=np.int64)
    flips = np.flatnonzero(orientation[1:] != orientation[:-1]) + 1
    return np.diff(np.concatenate(([0], flips, [n])))


def _sampled_domains(phase, dL):
    """Domain lengths of the orientation sign(sin(phase)) sampled every dL (zeros count as +1)."""
    orientation = np.sign(np.sin(phase))
    orientation[orientation == 0.] = 1.
    return _run_lengths(orientation) * dL


def periodicPoling(deltaBeta0, L):
    """Periodic poling that phase matches ``deltaBeta0`` over length L (poling.py:8-14).

    Domains are half a period 2 pi / |deltaBeta0| long, scaled so that they sum to L; the last one
    holds the fractional remainder.  As in the reference, a length that is a whole number of half
    periods leaves a last domain of length zero.
    """
    halfPeriods = 2 * L / (2 * np.pi / abs(deltaBeta0))
    remainder = halfPeriods % 1
    lengths = np.ones(int(halfPeriods) + int(remainder > 0))
    lengths[-1] = remainder
    return lengths * (L / np.sum(lengths))


def linearPoling(k0, kf, L, dL):
    """Chirped poling whose spatial frequency runs linearly from k0 at z=0 to kf at z=L, resolved on a
    grid of step dL (poling.py:17-29).  The orientation is the sign of sin(phi(z)) with
    phi(z) = (kf - k0) z^2 / (2L) + k0 z."""
    z = np.linspace(0, L, int(round(L / dL)))
    return _sampled_domains(0.5 * (kf - k0) * z**2 / L + k0 * z, dL)


def detunePoling(kMin, kMax, k0, ka, L, dL):
    """Poling whose spatial frequency follows k(z) = k0 + ka artanh(a (z - z0)), from kMin at z=0 to
    kMax at z=L, on a grid of step dL (poling.py:86-103).  The phase is the integral of k(z)."""
    z = np.linspace(0, L, int(round(L / dL)))
    a = (np.tanh((kMax - k0) / ka) + np.tanh((k0 - kMin) / ka)) / L
    z0 = np.tanh((k0 - kMin) / ka) / a
    phase = ka / (2 * a) * np.log(1 - a**2 * (z - z0)**2) + ka * (z - z0) * np.arctanh(a * (z - z0)) + k0 * z
    return _sampled_domains(phase - phase[0], dL)


def threeWaveMismatchRange(omega, domega, dbeta0, sign1, sign2,
                           beta1a=0, beta2a=0, beta3a=0,
                           beta1b=0, beta2b=0, beta3b=0,
                           beta1c=0, beta2c=0, beta3c=0):
    """Smallest and largest |wavenumber mismatch| of a three-wave process over a band (poling.py:292-315).

    mismatch(w) = dbeta0 + D_a(w) + sign1 D_b(w) + sign2 D_c(w), D(w) = b1 w + b2 w^2 / 2 + b3 w^3 / 6.
    ``domega`` is a half width (|w| < domega) or a pair (lower, upper) with -lower < w < upper.
    """
    assert abs(sign1) == 1 and abs(sign2) == 1, "Sign must be +/-1"

    def taylor(b1, b2, b3, w):
        return b1 * w + 0.5 * b2 * w**2 + 1/6 * b3 * w**3

    mismatch = dbeta0 + taylor(beta1a, beta2a, beta3a, omega) \
        + sign1 * taylor(beta1b, beta2b, beta3b, omega) \
        + sign2 * taylor(beta1c, beta2c, beta3c, omega)
    if isinstance(domega, (float, int)):
        band = np.abs(omega) < domega
    elif isinstance(domega, (tuple, list, np.ndarray)):
        band = np.logical_and(-domega[0] < omega, omega < domega[1])
    else:
        raise ValueError("unrecognized type for domega")
    inBand = np.abs(mismatch[band])
    return np.min(inBand), np.max(inBand)


def domainsToSpace(poling, nZSteps):
    """Orientation (+/-1) of each of nZSteps steps for the domain lengths ``poling`` (poling.py:439-471).

    The domains are scaled to nZSteps steps.  A step containing a wall takes the interpolated value
    orientation * (2 frac(wall) - 1), where the orientation is that of the domain the wall ends.
    Vectorised: each step belongs to the first domain whose wall index (the truncated wall position)
    is at or after it.
    """
    poling = np.array(poling)
    if np.any(poling <= 0):
        raise ValueError("Poling contains non-positive length domains")
    walls = np.cumsum(poling, dtype=np.float64)
    walls *= nZSteps / walls[-1]
    wallStep = walls.astype(np.int64)
    firstFree = np.concatenate(([0], wallStep[:-1] + 1))
    if np.any(walls < firstFree):
        raise ValueError("Poling period too small for given resolution")
    steps = np.arange(nZSteps)
    domain = np.searchsorted(wallStep, steps, side="left")
    orientation = np.where(domain % 2 == 0, 1.0, -1.0)
    onWall = wallStep[domain] == steps
    orientation[onWall] *= 2 * np.abs(np.fmod(walls[domain[onWall]], 1)) - 1
    return orientation
