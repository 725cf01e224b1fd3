"""Generate the committed golden fixtures under tests/golden/.

1. ``poling_golden.npz`` -- pinned to the reference itself: the reference's Python twin of
   ``setPoling`` (poling.py:439-471, ``domainsToSpace``) is imported from a checkout of the
   reference and run on seeded domain-length arrays.  Run with REFERENCE_ROOT (environment) or
   --reference-root pointing at the reference checkout; without one only the oracle fixture below
   is regenerated.
2. ``multimode_golden.npz`` -- pinned to the reference itself: outputs of the reference's
   ``multimode.py`` and ``decompositions.py`` (imported from the checkout) on a Green's pair of the
   oracle and seeded matrices.
3. ``frontends_golden.npz`` -- pinned to the reference itself: the poling generators of the
   reference's ``poling.py`` and its ``nlMaterial`` decorator (applied to the synthetic Sellmeier
   expressions of frontend_cases.py), imported from the checkout and run on the seeded cases there.
4. ``oracle_golden.npz`` -- outputs of the numpy oracle (oracle/nlm_oracle.py) for the small
   configurations of tests/cases.py: pump grids, signal grids, Green's matrices and batch rows
   of every solver.  They pin the oracle over time and give the GPU tests fixed expectations.

Usage:  python tests/golden/make_golden.py
"""

import contextlib
import importlib.util
import io
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import nlm_oracle as O  # noqa: E402
import cases  # noqa: E402


def poling_cases():
    rng = np.random.default_rng(7)
    out = []
    out.append((np.ones(100), 1000))                   # the Green's-function benchmark poling (period 20 steps)
    out.append((np.ones(100), 997))                    # non-integer domain boundaries
    out.append((np.array([1.0, 2.5, 1.0, 1.3]), 37))
    out.append((np.array([3.0]), 10))                  # one domain: all +1
    for k in range(6):
        doms = rng.uniform(5, 50, size=rng.integers(3, 30))
        out.append((doms, int(doms.sum() * rng.uniform(0.5, 2.0))))
    doms = rng.integers(5, 51, size=40).astype(float)  # the ragged-batch domain lengths (5..50 steps)
    out.append((doms, int(doms.sum())))
    return out


def make_poling(ref_root):
    sys.path.insert(0, ref_root)
    if not hasattr(np, "float_"):
        np.float_ = np.float64  # the reference predates numpy 2
    import poling as ref_poling  # the reference's module
    data = {}
    for k, (doms, nz) in enumerate(poling_cases()):
        data["domains_%d" % k] = doms
        data["nz_%d" % k] = np.array(nz)
        if doms.size <= 1:
            data["expected_%d" % k] = np.ones(nz)   # src/_NonlinearMedium.cpp:471-472 (size <= 1 -> all +1)
        else:
            data["expected_%d" % k] = ref_poling.domainsToSpace(doms, nz)
    data["count"] = np.array(len(poling_cases()))
    np.savez_compressed(os.path.join(HERE, "poling_golden.npz"), **data)


def multimode_inputs():
    """A symplectic Green's pair (the Chi2PDC test medium, from the oracle), its pump profile, and
    seeded matrices for the decompositions."""
    kw = cases.oracle_kwargs("Chi2PDC")
    med = O.SOLVERS["Chi2PDC"](**kw)
    med.run_pump_simulation()
    C, S = med.compute_greens_function(False, False)
    rng = np.random.default_rng(21)
    n = C.shape[0]
    a = rng.standard_normal((6, 6)) + 1j * rng.standard_normal((6, 6))
    return {"C": C, "S": S, "omega": med.omega, "pump": med.pump_time[0][0],
            "sym_complex": a + a.T, "sym_real": (a + a.T).real, "polar_in": a,
            "modes": rng.standard_normal((n, n)), "diag": np.exp(rng.uniform(-1, 1, n)),
            "transmission": rng.uniform(0.2, 0.9, n)}


def make_multimode(ref_root):
    """Outputs of the reference's multimode.py and decompositions.py on multimode_inputs()."""
    sys.path.insert(0, ref_root)
    if not hasattr(np, "float_"):
        np.float_ = np.float64  # the reference predates numpy 2
    if not hasattr(np, "int"):
        np.int = int
    import multimode as mm  # the reference's modules
    import decompositions as dc
    x = multimode_inputs()
    C, S = x["C"], x["S"]
    out = dict(("in_" + k, v) for k, v in x.items())
    Z = mm.calcQuadratureGreens(C, S)
    out["Z"] = Z
    cov = mm.calcCovarianceMtx(Z)
    out["cov"] = cov
    out["cov_a"] = mm.calcCovarianceMtxABasis(C, S)
    out["normalized_cov"] = mm.normalizedCov(cov)
    out["lo_squeezing"] = mm.calcLOSqueezing(cov, x["pump"], tol=1.0)   # C_xx = 0.93 here
    out["downsampled_cov"] = mm.downSampledCov(Z, 12, x["omega"], 2.0)
    out["downsampled_cov_a"] = mm.downSampledCovABasis(C, S, 12, x["omega"], 2.0)
    out["bm_eigs"] = mm.blochMessiahEigs(Z)
    d, lv, rv = mm.blochMessiahVecs(Z)
    out["bm_diag"], out["bm_left"], out["bm_right"] = d, lv, rv
    out["ft_c_time"], out["ft_s_time"] = mm.ftGreens(C, S, True)
    out["ft_c_freq"], out["ft_s_freq"] = mm.ftGreens(C, S, False)
    out["to_xp"], out["from_xp"] = mm.basisTransforms(5)
    out["combined_c"], out["combined_s"] = mm.combineGreens(C, S, C.T, S.conj())
    out["incoherent"] = mm.incoherentPowerGreens(Z)
    out["photon_mean"] = mm.photonMean(cov)
    out["photon_mean_a"] = mm.photonMeanA(out["cov_a"])
    out["photon_cov"] = mm.photonCov(cov)
    out["fluorescence"] = mm.parametricFluorescence(x["modes"], x["diag"])
    out["adjacency"] = mm.effectiveAdjacencyMatrix(x["modes"], x["diag"])
    out["full_adjacency"] = mm.fullEffectiveAdjacencyMatrix(cov)
    out["lump_scalar"] = mm.covLumpLoss(cov, 0.7)
    out["lump_vector_a"] = mm.covLumpLoss(out["cov_a"], x["transmission"], abasis=True)
    out["polar_u"], out["polar_p"] = dc.leftPolar(x["polar_in"])
    out["takagi_c_l"], out["takagi_c_u"] = dc.takagi(x["sym_complex"])
    out["takagi_r_l"], out["takagi_r_u"] = dc.takagi(x["sym_real"])
    out["bm_ut"], out["bm_st"], out["bm_v"] = dc.bloch_messiah(Z, tol=1e-6)   # RK4: symplectic to 2.4e-7
    np.savez_compressed(os.path.join(HERE, "multimode_golden.npz"), **out)


class _Numpy2Shim(types.ModuleType):
    """numpy for the reference's poling module, as the numpy its code was written for behaves.

    Current numpy refuses to store a one-element array in a scalar slot, which poling.py:152-156 does
    with the rows of ``np.argwhere``; handing it each row as a tuple indexes a scalar instead, which is
    the value older numpy stored."""

    def __init__(self):
        super().__init__("numpy")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def argwhere(a):
        return [tuple(r) for r in np.argwhere(a)]


def _outcome(fn, args, kwargs):
    try:
        with contextlib.redirect_stdout(io.StringIO()):   # linearPolingContinuous prints a flag
            return np.asarray(fn(*args, **kwargs), dtype=np.float64), None
    except Exception as e:   # recorded: the front end must raise the same
        return None, "%s: %s" % (type(e).__name__, e)


def make_frontends(ref_root):
    """Outputs of the reference's poling generators and material decorator on frontend_cases.py."""
    import frontend_cases as FC
    sys.path.insert(0, ref_root)
    if not hasattr(np, "float_"):
        np.float_ = np.float64
    import poling as ref_poling  # the reference's module
    ref_poling.np = _Numpy2Shim()
    out = {}
    for name, fn, args, kwargs in FC.poling_cases():
        args = tuple(FC.NLF[a] if isinstance(a, str) else a for a in args)
        val, err = _outcome(getattr(ref_poling, fn), args, kwargs)
        out["pol_" + name] = val if err is None else np.array(err)
    for name, a, b, ml, tol in FC.combine_cases(ref_poling.periodicPoling):
        out["in_%s_a" % name], out["in_%s_b" % name] = a, b
        val, err = _outcome(ref_poling.combinePoling, (a, b, ml, tol), {})
        out["pol_" + name] = val if err is None else np.array(err)
    spec = importlib.util.spec_from_file_location("ref_nlMaterial", os.path.join(ref_root, "materials", "nlMaterial.py"))
    ref_mat = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ref_mat)
    import sympy
    sym = {"l0": ref_mat.l0, "T": ref_mat.T, "th": ref_mat.th, "sqrt": sympy.sqrt, "Piecewise": sympy.Piecewise}
    for name, expr, kw, grid in FC.sellmeier_cases(sym, ref_mat.angledRefractiveIndex):
        cls = ref_mat.nlMaterial(**kw)(type(name, (), {"ind": expr}))
        out["mat_%s_grid" % name] = np.array(grid, dtype=np.float64)
        fns = FC.MATERIAL_FUNCTIONS + (["walkoff"] if kw.get("angleTuning") else [])
        for f in fns:
            out["mat_%s_%s" % (name, f)] = np.array([float(getattr(cls, f)(*pt)) for pt in grid])
    np.savez_compressed(os.path.join(HERE, "frontends_golden.npz"), **out)


def oracle_case(name):
    kw = cases.oracle_kwargs(name)
    med = O.SOLVERS[name](**kw)
    res = {}
    n, nm = med.n_freqs, med.n_signal_modes
    rows = sorted({0, 1, med.n_z_steps // 2, med.n_z_steps - 1})
    res["rows"] = np.array(rows)
    if not med.fully_nonlinear:
        med.run_pump_simulation()
        prow = sorted({0, 1, med.n_z_steps_p // 2, med.n_z_steps_p - 1})
        res["pump_rows"] = np.array(prow)
        res["pump_time"] = np.stack([pt[prow] for pt in med.pump_time])
        res["pump_freq"] = np.stack([pf[prow] for pf in med.pump_freq])
    x = cases.signal_input(name, n, nm, seed=1)
    res["signal_in"] = x
    med.run_signal_simulation(x, True, 0)
    res["signal_time"] = np.stack([g[rows] for g in med.signal_time])
    res["signal_freq"] = np.stack([g[rows] for g in med.signal_freq])
    rng = np.random.default_rng(2)
    b = np.stack([cases.signal_input(name, n, 1, seed=10 + k) for k in range(3)])
    res["batch_in"] = b
    if med.fully_nonlinear:
        res["batch_out"] = med.batch_signal_simulation(b, False, 1, 0)
    else:
        res["batch_out"] = med.batch_signal_simulation(b, False, False)
        C, S = med.compute_greens_function(False, False)
        res["green_c"], res["green_s"] = C, S
        Ct, St = med.compute_greens_function(True, False)
        res["green_c_time"], res["green_s_time"] = Ct, St
    del rng
    return res


def make_oracle():
    data = {}
    for name in cases.CASES:
        for k, v in oracle_case(name).items():
            data["%s__%s" % (name, k)] = v
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **data)


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=os.environ.get("REFERENCE_ROOT"),
                    help="checkout of the reference (also REFERENCE_ROOT)")
    ref_root = ap.parse_args().reference_root
    if ref_root and os.path.exists(os.path.join(ref_root, "poling.py")):
        make_poling(ref_root)
        make_multimode(ref_root)
        make_frontends(ref_root)
    else:
        print("no reference checkout given (REFERENCE_ROOT or --reference-root); poling, multimode and "
              "front-end fixtures left unchanged",
              file=sys.stderr)
    make_oracle()
