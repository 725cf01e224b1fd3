"""Small seeded configurations of every solver, shared by the oracle, golden and GPU tests.

Sizes are chosen so the numpy oracle finishes each case in well under a second.
"""

import numpy as np

INF = float("inf")

# constructor keyword arguments per solver (names and meaning as in the reference's py::init lists)
CASES = {
    "Chi3": dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0.1, tMax=10, tPrecision=64,
                 zPrecision=20),
    "Chi2PDC": dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0.3, beta1s=2,
                    beta3=0.05, beta3s=0.1, diffBeta0=0.7, tMax=20, tPrecision=64, zPrecision=10,
                    poling=[1, 1, 1, 1, 2.5, 1, 1, 1, 1.3, 1]),
    "Chi2SFG": dict(relativeLength=1, nlLength=0.8, nlLengthOrig=1.2, beta2=0.5, beta2s=-0.3, beta2o=0.2,
                    pulseType=0, beta1=0.1, beta1s=1, beta1o=-0.5, beta3=0, beta3s=0.05, beta3o=0.02,
                    diffBeta0=1.3, tMax=10, tPrecision=32, zPrecision=10, poling=[2, 1, 3, 1, 1, 2]),
    "Chi2AFC": dict(relativeLength=1, nlLength=0.8, nlLengthOrig=1.2, beta2=0.5, beta2s=-0.3, beta2o=0.2,
                    pulseType=1, beta1=0.1, beta1s=1, beta1o=-0.5, diffBeta0Start=-2, diffBeta0End=3, tMax=10,
                    tPrecision=32, zPrecision=10),
    "Chi2SFGPDC": dict(relativeLength=1, nlLength=0.8, nlLengthOrig=1.2, beta2=0.5, beta2s=-0.3, beta2o=0.2,
                       beta1s=1, beta1o=-0.5, diffBeta0=1.3, diffBeta0o=-0.4, tMax=10, tPrecision=32,
                       zPrecision=10, poling=[1, 2, 1, 2]),
    "Chi2SFGII": dict(relativeLength=1, nlLengthZY=0.9, nlLengthZZ=1.3, beta2=0.5, beta2sz=-0.3, beta2sy=0.2,
                      beta2oz=0.1, beta2oy=-0.2, beta1=0.1, beta1sz=1, beta1sy=-0.5, beta1oz=0.3, beta1oy=0.2,
                      diffBeta0z=0.5, diffBeta0y=-0.7, diffBeta0=1.1, tMax=10, tPrecision=32,
                      poling=[1, 1, 2, 1, 1]),
    "Chi2PDCII": dict(relativeLength=1, nlLengthI=0.8, nlLengthII=1.2, beta2=0.5, beta2s=-0.3, beta2o=0.2,
                      beta1s=1, beta1o=-0.5, diffBeta0=0.9, tMax=10, tPrecision=32, zPrecision=10,
                      poling=[1, 1, 1, 2, 1]),
    "Chi2SFGOPA": dict(relativeLength=1, nlLengthSFGh=0.8, nlLengthSFGf=1.2, nlLengthDOPAh=0.9, nlLengthDOPAf=1.1,
                       beta2F=0.5, beta2H=-0.2, beta2h=0.3, beta2f=-0.4, beta1F=0.1, beta1H=0.2, beta1h=1,
                       beta1f=-0.5, diffBeta0SFG=1.3, diffBeta0DOPA=-0.6, tMax=10, tPrecision=32, zPrecision=10,
                       poling=[1, 1, 2, 1]),
    "Chi2SFGXPM": dict(relativeLength=1, nlLength=0.8, nlLengthOrig=1.2, nlLengthChi3=2.0, nlLengthChi3Orig=3.0,
                       beta2=0.5, beta2s=-0.3, beta2o=0.2, beta1s=1, beta1o=-0.5, diffBeta0=1.3, tMax=10,
                       tPrecision=32, zPrecision=10, poling=[1, 2, 1]),
    "Chi2SHG": dict(relativeLength=1, nlLengthH=0.9, nlLengthP=1.1, beta2h=0.3, beta2p=-0.2, beta1h=0.5,
                    beta1p=-0.1, diffBeta0=0.4, rayleighLength=0.8, tMax=10, tPrecision=32, zPrecision=10,
                    poling=[1, 1, 2]),
    "Chi2SHGOPA": dict(relativeLength=1, nlLengthP=0.9, nlLengthSH=1.1, nlLengthPA1=1.3, nlLengthPA2=1.2,
                       beta2p=0.3, beta2sh=-0.2, beta2pa1=0.1, beta2pa2=0.2, beta1sh=0.5, beta1pa1=-0.2,
                       diffBeta0shg=0.4, diffBeta0opa=-0.3, tMax=10, tPrecision=32, zPrecision=10,
                       intensityProfile=2, rayleighLength=0.7),
    "Chi2DSFG": dict(relativeLength=1, nlLengthP=0.9, nlLengthS=1.1, nlLengthD=1.3, beta2p=0.3, beta2s=-0.2,
                     beta2d=0.1, beta1s=0.5, beta1d=-0.2, diffBeta0=0.4, tMax=10, tPrecision=32, zPrecision=10,
                     poling=[2, 1, 1]),
    "Chi2SHGXPM": dict(relativeLength=1, nlLengthH=0.9, nlLengthP=1.1, nlLengthChi3=2.0, beta2h=0.3, beta2p=-0.2,
                       beta1h=0.5, diffBeta0=0.4, tMax=10, tPrecision=32, zPrecision=10),
    "Chi2ASHG": dict(relativeLength=1, nlLengthH=0.9, nlLengthP=1.1, beta2h=0.3, beta2p=-0.2, beta1h=0.5,
                     diffBeta0Start=-1, diffBeta0End=2, tMax=10, tPrecision=32, zPrecision=10),
    "Chi3GNLSE": dict(relativeLength=0.5, nlLength=1, selfSteepLength=5, fr=0.18, fb=0.21, tau1=0.0155,
                      tau2=0.2165, tau3=0.4, beta2=-1, beta3=0.05, tMax=10, tPrecision=64, zPrecision=20),
}

FULLY_NONLINEAR = {"Chi2SHG", "Chi2SHGOPA", "Chi2DSFG", "Chi2SHGXPM", "Chi2ASHG", "Chi3GNLSE"}

def oracle_kwargs(name):
    """Keyword arguments of the oracle's constructor (the same as the engine's for these cases)."""
    return dict(CASES[name])


def noise(rng, n, sigma):
    """Complex Gaussian noise of standard deviation sigma: (N(0,1) + i N(0,1)) sigma / sqrt(2)."""
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * sigma / np.sqrt(2)


def signal_input(name, n_freqs, n_modes, seed=0):
    """A seeded signal input filling every mode (amplitude large enough to exercise the nonlinear terms)."""
    rng = np.random.default_rng(seed)
    sigma = 0.5 if name in FULLY_NONLINEAR else 1.0
    if name == "Chi3GNLSE":
        t = np.fft.fftshift(np.linspace(-10, 10, n_freqs, endpoint=False))
        return 2.0 / np.cosh(t) + noise(rng, n_freqs, 1e-3)
    return noise(rng, n_freqs * n_modes, sigma)


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def rel_l2_pair(c, s, cr, sr):
    """Joint relative L2 error of a (C, S) pair: S vanishes identically for processes without
    conjugate coupling (sum-frequency generation), where a per-matrix ratio is meaningless."""
    num = np.linalg.norm(np.asarray(c) - cr) ** 2 + np.linalg.norm(np.asarray(s) - sr) ** 2
    den = np.linalg.norm(cr) ** 2 + np.linalg.norm(sr) ** 2
    return float(np.sqrt(num / (den if den > 0 else 1.0)))
