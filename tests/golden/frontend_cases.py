"""Seeded cases for the poling and material front ends, shared by the fixture script and the tests.

The Sellmeier expressions are synthetic: smooth index curves of the usual form with made-up
coefficients, chosen to exercise every derivative the material decorator takes (wavelength,
temperature, angle, a piecewise branch).  They describe no real crystal.
"""

import numpy as np


def gaussian_nlf(z):
    return np.exp(-((z - 5.0) / 2.0) ** 2)


def offset_gaussian_nlf(z):
    return 0.2 + 0.8 * np.exp(-((z - 3.0) / 1.5) ** 2)


def signed_nlf(z):
    # changes sign: negative duty cycles are wrapped by +1 in dutyCyclePmf
    return np.cos(0.6 * z) * np.exp(-((z - 5.0) / 3.0) ** 2)


def flat_nlf(z):
    return 0.9 * np.ones_like(z)


NLF = {"gaussian": gaussian_nlf, "offset_gaussian": offset_gaussian_nlf, "signed": signed_nlf,
       "flat": flat_nlf}


def poling_cases():
    """(name, function, args, kwargs); an ``nlf`` argument is given by its key in NLF."""
    c = []
    for k, (db, L) in enumerate([(2.0, 10.0), (np.pi, 10.0), (-3.7, 5.0), (40.0, 1.0), (0.3, 7.0)]):
        c.append(("periodic_%d" % k, "periodicPoling", (db, L), {}))
    for k, (k0, kf, L, dL) in enumerate([(10, 20, 5.0, 0.01), (-10, 20, 5.0, 0.01), (30, 5, 2.0, 0.002),
                                         (0.5, 60, 3.0, 0.001)]):
        c.append(("linear_%d" % k, "linearPoling", (k0, kf, L, dL), {}))
    for k, (k0, kf, L) in enumerate([(10, 20, 5.0), (-10, 20, 5.0), (20, 10, 5.0), (10, -20, 5.0),
                                     (-20, -10, 5.0), (3.0, 50.0, 2.0), (-7.0, 9.0, 4.0), (15.0, -4.0, 3.0)]):
        c.append(("continuous_%d" % k, "linearPolingContinuous", (k0, kf, L), {}))
    for k, args in enumerate([(5, 15, 10, 2, 5.0, 0.01), (20, 40, 30, 4, 2.0, 0.001), (8, 9, 8.5, 0.3, 10.0, 0.02)]):
        c.append(("detune_%d" % k, "detunePoling", args, {}))
    for k, (nlf, db, L, ms, kw) in enumerate([("gaussian", 20.0, 10.0, 0.01, {}),
                                              ("offset_gaussian", 31.0, 6.0, 0.005, {}),
                                              ("signed", 25.0, 10.0, 0.02, {}),
                                              ("gaussian", 20.0, 10.0, 0.05, {}),
                                              ("flat", 17.3, 4.0, 0.01, {"normalize": False})]):
        c.append(("dutycycle_%d" % k, "dutyCyclePmf", (nlf, db, L, ms), kw))
    for k, (nlf, db, L, kw) in enumerate([("gaussian", 20.0, 10.0, {}),
                                          ("gaussian", 20.0, 10.0, {"dutyCycle": 0.3, "normalize": False,
                                                                    "override": True}),
                                          ("offset_gaussian", 31.0, 6.0, {}),
                                          ("gaussian", 23.7, 10.0, {}),
                                          ("flat", 23.7, 10.0, {"dutyCycle": 0.7, "normalize": False}),
                                          ("offset_gaussian", 18.2, 6.0, {"dutyCycle": 0.2, "normalize": False,
                                                                          "override": True})]):
        c.append(("deleted_%d" % k, "deletedDomainPmf", (nlf, db, L), kw))
    w = np.linspace(-5, 5, 101)
    c.append(("mismatch_0", "threeWaveMismatchRange",
              (w, 2.0, 0.1, 1, -1, 0.1, 0.2, 0.0, 0.3, 0.1, 0.01, 0.0, 0.05, 0.0), {}))
    c.append(("mismatch_1", "threeWaveMismatchRange", (w, (1.0, 3.0), 0.1, -1, -1, 0.1, 0.2), {}))
    c.append(("mismatch_2", "threeWaveMismatchRange", (w, np.array([0.5, 4.0]), -0.4, 1, 1),
              {"beta1b": 0.7, "beta3c": -0.2}))
    return c


def combine_cases(periodic):
    """(name, polingA, polingB, minLength, tol) built from ``periodic`` (a periodicPoling function)."""
    rng = np.random.default_rng(11)
    out = [("combine_0", periodic(2.0, 10.0), periodic(3.1, 10.0), 0.2, 0.05),
           ("combine_1", periodic(20.0, 10.0), periodic(1.3, 10.0), 0.05, 0.01),
           ("combine_2", periodic(7.0, 6.0), periodic(7.2, 5.0), 0.1, 0.02)]
    for k in range(4):
        a = rng.uniform(0.05, 1.0, size=rng.integers(5, 40))
        b = rng.uniform(0.05, 1.0, size=rng.integers(5, 40))
        out.append(("combine_r%d" % k, a, b * (a.sum() / b.sum()) * rng.uniform(0.8, 1.2), 0.12, 0.03))
    return out


def sellmeier_cases(sym, angled):
    """Synthetic index expressions: (name, expression, decorator kwargs, argument grid).

    ``sym`` is the symbol namespace (l0, T, th and sqrt, Piecewise from sympy); ``angled`` is the
    module's angledRefractiveIndex."""
    l0, T, th, sqrt, Piecewise = sym["l0"], sym["T"], sym["th"], sym["sqrt"], sym["Piecewise"]
    base = sqrt(2.3 + 0.9 / (1 - 0.05 / l0**2) + 0.4 / (1 - 80.0 / l0**2) - 0.012 * l0**2)
    dn = (1.1e-5 + 3.0e-6 / l0 - 1.0e-6 / l0**2) * (T - 20.0) + (2.0e-8 + 4.0e-9 / l0) * (T - 20.0)**2
    n1 = sqrt(2.7 + 0.05 / (l0**2 - 0.02) - 0.015 * l0**2)
    n2 = sqrt(2.4 + 0.04 / (l0**2 - 0.018) - 0.011 * l0**2)
    hi = sqrt(2.1 + 0.9 / (1 - 0.047 / l0**2) - 0.014 * l0**2)
    lo = sqrt(2.2 + 0.8 / (1 - 0.05 / l0**2) - 0.016 * l0**2)
    lam = [0.8, 1.064, 1.55, 2.0]
    temp = [25.0, 60.0]
    ang = [0.3, 0.7]
    return [
        ("thermal", base + dn, {}, [(x, t) for x in lam for t in temp]),
        ("plain", base, {"temperatureTuning": False, "deleteInd": False}, [(x,) for x in lam]),
        ("angled", angled(n1, n2), {"angleTuning": True, "temperatureTuning": False},
         [(a, x) for a in ang for x in lam]),
        ("angled_thermal", angled(n1 + dn, n2), {"angleTuning": True}, [(a, x, t) for a in ang for x in lam for t in temp]),
        ("piecewise", Piecewise((hi, l0 > 1.2), (lo, l0 < 1.2)) + dn, {}, [(x, t) for x in lam for t in temp]),
    ]


MATERIAL_FUNCTIONS = ["n", "ng", "gvd", "beta2", "beta1", "beta0", "beta3"]
