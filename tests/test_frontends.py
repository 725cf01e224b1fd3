"""Poling generators and the material decorator against the reference's own outputs.

The fixture (tests/golden/frontends_golden.npz) holds the outputs of the reference's poling.py and
materials/nlMaterial.py on the seeded cases of tests/golden/frontend_cases.py, or the error each case
raised.  Both are bit-identical with the numpy and sympy of this image; the tolerances (1e-12 of the
crystal length for domain lengths, 1e-11 relative for the material functions) leave room for another
build of numpy or sympy.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import frontend_cases as FC  # noqa: E402
from multimodenonlinearoptics_gb300 import poling  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "frontends_golden.npz"))


def _check(name, fn, args, kwargs):
    expected = GOLDEN["pol_" + name]
    if expected.dtype.kind in "US":
        kind, _, msg = str(expected).partition(": ")
        with pytest.raises(Exception) as info:
            fn(*args, **kwargs)
        assert type(info.value).__name__ == kind
        assert str(info.value) == msg
        return
    got = np.asarray(fn(*args, **kwargs), dtype=np.float64)
    assert got.shape == expected.shape, (name, got.shape, expected.shape)
    scale = max(1.0, float(np.sum(np.abs(expected))))
    assert np.max(np.abs(got - expected), initial=0.0) <= 1e-12 * scale, name


@pytest.mark.parametrize("case", [c for c in FC.poling_cases() if hasattr(poling, c[1])], ids=lambda c: c[0])
def test_poling_generators(case):
    name, fn, args, kwargs = case
    args = tuple(FC.NLF[a] if isinstance(a, str) else a for a in args)
    _check(name, getattr(poling, fn), args, kwargs)


def test_domains_to_space_matches_reference():
    """The vectorised domainsToSpace equals the reference's loop on the setPoling fixtures."""
    g = np.load(os.path.join(HERE, "golden", "poling_golden.npz"))
    for k in range(int(g["count"])):
        doms, nz = g["domains_%d" % k], int(g["nz_%d" % k])
        if doms.size <= 1:
            continue   # the engine's own one-domain rule; the Python function is not asked for it
        np.testing.assert_array_equal(poling.domainsToSpace(doms, nz), g["expected_%d" % k])


def test_domains_to_space_errors():
    with pytest.raises(ValueError, match="non-positive"):
        poling.domainsToSpace([1.0, 0.0, 2.0], 10)
    with pytest.raises(ValueError, match="too small"):
        poling.domainsToSpace(np.ones(50), 20)


def test_generated_poling_feeds_set_poling():
    """Generator outputs are valid setPoling inputs: positive lengths summing to the crystal length,
    and an orientation grid of +/-1 away from the walls."""
    for doms, L in ((poling.linearPoling(10, 20, 5.0, 0.001), 5.0),
                    (poling.detunePoling(5, 15, 10, 2, 5.0, 0.01), 5.0),
                    (poling.periodicPoling(20.0, 10.0), 10.0)):
        assert np.all(doms > 0)
        assert abs(np.sum(doms) - L) < 1e-9 * L
        space = poling.domainsToSpace(doms, 2000)
        assert space.shape == (2000,)
        assert np.all(np.abs(space) <= 1)
        assert np.mean(np.abs(space) == 1) > 0.9


def test_material_decorator():
    sympy = pytest.importorskip("sympy")
    from multimodenonlinearoptics_gb300 import materials as M
    sym = {"l0": M.l0, "T": M.T, "th": M.th, "sqrt": sympy.sqrt, "Piecewise": sympy.Piecewise}
    for name, expr, kw, grid in FC.sellmeier_cases(sym, M.angledRefractiveIndex):
        cls = M.nlMaterial(**kw)(type(name, (), {"ind": expr}))
        assert hasattr(cls, "ind") == (kw.get("deleteInd", True) is False)
        fns = FC.MATERIAL_FUNCTIONS + (["walkoff"] if kw.get("angleTuning") else [])
        for f in fns:
            got = np.array([float(getattr(cls, f)(*pt)) for pt in grid])
            expected = GOLDEN["mat_%s_%s" % (name, f)]
            np.testing.assert_allclose(got, expected, rtol=1e-11, atol=0, err_msg="%s.%s" % (name, f))
        assert not hasattr(cls, "walkoff") or kw.get("angleTuning")


def test_material_decorator_requires_index():
    pytest.importorskip("sympy")
    from multimodenonlinearoptics_gb300 import materials as M
    with pytest.raises(AttributeError, match="index expression"):
        M.nlMaterial()(type("Empty", (), {}))
