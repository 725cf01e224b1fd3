"""Generate the committed golden fixtures under tests/golden/.

1. ``poling_golden.npz`` -- pinned to the reference itself: the reference's Python twin of
   ``setPoling`` (poling.py:439-471, ``domainsToSpace``) is imported from a checkout of the
   reference and run on seeded domain-length arrays.  Run with REFERENCE_ROOT pointing at the
   reference checkout (default: /root/reference).
2. ``oracle_golden.npz`` -- outputs of the numpy oracle (oracle/nlm_oracle.py) for the small
   configurations of tests/cases.py: pump grids, signal grids, Green's matrices and batch rows
   of every solver.  They pin the oracle over time and give the GPU tests fixed expectations.

Usage:  python tests/golden/make_golden.py
"""

import os
import sys

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
    ref_root = os.environ.get("REFERENCE_ROOT", "/root/reference")
    if os.path.exists(os.path.join(ref_root, "poling.py")):
        make_poling(ref_root)
    else:
        print("reference checkout not found; poling fixtures left unchanged", file=sys.stderr)
    make_oracle()
