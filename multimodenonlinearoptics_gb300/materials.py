"""Dispersion of nonlinear-optical materials from a symbolic Sellmeier expression (host side).

``nlMaterial`` is a class decorator with the reference's interface (materials/nlMaterial.py:14-71).
The class holds ``ind``, the refractive index as a sympy expression of the free-space wavelength
``l0`` in um and, when enabled, the temperature ``T`` in C and the tuning angle ``th``.  The decorator
adds static functions of (th, l0, T) (th and T only when enabled):

* ``n``: the index;
* ``ng``: the group index n - l0 dn/dl0;
* ``gvd`` and ``beta2``: -l0^2 / (2 pi c^2 1e6) dng/dl0;
* ``beta1`` = ng / c, ``beta0`` = 2 pi 1e6 n / l0;
* ``beta3``: the third derivative of ng with respect to w = 2 pi c 1e6 / l0, as the reference
  defines it (materials/nlMaterial.py:56-59);
* ``walkoff`` (angle tuning): Re atan(-(dn/dth) / n).

The outputs feed the solvers' beta arguments.  Material coefficient tables are not carried here: the
decorator takes any Sellmeier expression.  This module needs sympy and is imported on its own, not by
the package.
"""

import sympy

__all__ = ["l0", "T", "th", "nlMaterial", "angledRefractiveIndex", "C_LIGHT"]

C_LIGHT = 299792458  # m / s

l0 = sympy.symbols("l0", real=True)   # free-space wavelength, um
T = sympy.symbols("T", real=True)     # temperature, C
th = sympy.symbols("th", real=True)   # tuning angle, rad

_DOCS = {
    "n": "Calculate refractive index n from the Sellmeier equation",
    "ng": "Calculate the group index from the Sellmeier equation",
    "gvd": "Calculate 2nd order dispersion (group dispersion) from the Sellmeier equation",
    "beta1": "Calculate 1st order dispersion (inverse group velocity) from the Sellmeier equation",
    "beta0": "Calculate wavenumber (0th order dispersion) from the Sellmeier equation",
    "beta3": "Calculate 3rd order dispersion from the Sellmeier equation",
    "walkoff": "Calculate the spatial walk-off angle",
}


def _dispersion_expressions(index, angleTuning):
    """The derived quantities of a Sellmeier index, as sympy expressions."""
    pi, c, diff = sympy.pi, C_LIGHT, sympy.diff
    group = index - l0 * diff(index, l0)
    w = sympy.symbols("w")
    wavelengthOf = (2 * pi * c * 1e6) / w       # l0 in um at angular frequency w in rad/s
    exprs = {
        "n": index,
        "ng": group,
        "gvd": -l0**2 / (1e6 * 2 * pi * c**2) * diff(group, l0),
        "beta1": group / c,
        "beta0": 2 * pi * 1e6 / l0 * index,
        "beta3": diff(group.subs(l0, wavelengthOf), w, 3).subs(w, (2 * pi * c * 1e6) / l0),
    }
    if angleTuning:
        exprs["walkoff"] = sympy.re(sympy.atan(-diff(index, th) / index))
    return exprs


def _compile(args, expr, doc):
    fn = sympy.lambdify(args, expr)

    def evaluate(*values):
        return fn(*values)

    evaluate.__doc__ = doc
    return staticmethod(evaluate)


def nlMaterial(deleteInd=True, angleTuning=False, temperatureTuning=True):
    """Class decorator: derive the dispersion functions of the class's index expression ``ind``.

    deleteInd: remove ``ind`` from the class afterwards; angleTuning: the functions take the angle th
    first; temperatureTuning: the functions take the temperature T last.
    """
    def attach(cls):
        if not hasattr(cls, "ind"):
            raise AttributeError("Class does not have an index expression!")
        args = ([th] if angleTuning else []) + [l0] + ([T] if temperatureTuning else [])
        for name, expr in _dispersion_expressions(cls.ind, angleTuning).items():
            setattr(cls, name, _compile(args, expr, _DOCS[name]))
        cls.beta2 = cls.__dict__["gvd"]
        if deleteInd:
            del cls.ind
        return cls
    return attach


def angledRefractiveIndex(axisIndex1, axisIndex2):
    """Index at angle th between two crystal axes with indices axisIndex1, axisIndex2:
    [cos(th)^2 / n1^2 + sin(th)^2 / n2^2]^(-1/2) (materials/nlMaterial.py:74-80)."""
    return 1 / sympy.sqrt(sympy.cos(th)**2 / axisIndex1**2 + sympy.sin(th)**2 / axisIndex2**2)
