"""Edges of the grid and step counts against the oracle: the largest grid of the single-mode kernels
(N=8192, sixteen points per thread), the smallest grids (N=8, 16) and a single z step (nZSteps=2)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9

PDC = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0.2, beta1s=2, beta3=0.05,
           beta3s=0.1, diffBeta0=0.4, tMax=40, zPrecision=10, poling=[1, 2, 1])


def _batch_pair(med, ref, rows, seed, fnl=False):
    n = med._dims["nFreqs"]
    x = cases.noise(np.random.default_rng(seed), rows * n, 0.5).reshape(rows, n)
    if fnl:
        return med.batchSignalSimulation(x, inTimeDomain=False), ref.batch_signal_simulation(x, False)
    return med.batchSignalSimulation(x, False, False), ref.batch_signal_simulation(x, False, False)


def test_largest_single_mode_grid(nlm, oracle):
    """The one-CTA kernels with sixteen points per thread (few propagations on this grid otherwise
    run on 4-CTA clusters, covered by test_gpu_cluster.py)."""
    kw = dict(PDC, tPrecision=8192)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    med._set_cluster(0)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    for use_prop in (1, 0):
        med._set_schedule(use_propagator=use_prop)
        out, want = _batch_pair(med, ref, 6, 3)
        assert med._last_schedule()["R"] == 16
        assert cases.rel_l2(out, want) < TOL
    a = cases.noise(np.random.default_rng(4), 8192, 1e-2)
    med.runSignalSimulation(a)
    ref.run_signal_simulation(a)
    assert cases.rel_l2(med.signalTime, ref.signal_time[0]) < TOL
    assert cases.rel_l2(med.signalFreq, ref.signal_freq[0]) < TOL


def test_largest_grid_chi3_pump_march(nlm, oracle):
    """The one-CTA march with sixteen points per thread (the cluster march is in test_gpu_cluster.py)."""
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0.02, tMax=40, tPrecision=8192, zPrecision=15)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med._set_cluster(0)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL


@pytest.mark.parametrize("n", [8, 16])
@pytest.mark.parametrize("name", ["Chi2PDC", "Chi2SFG", "Chi3"])
def test_smallest_grids(nlm, oracle, name, n):
    kw = dict(cases.CASES[name], tPrecision=n)
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    C, S = med.computeGreensFunction()
    Cr, Sr = ref.compute_greens_function()
    assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL
    out, want = _batch_pair(med, ref, 5, 6)
    assert cases.rel_l2(out, want) < TOL
    a = cases.noise(np.random.default_rng(8), n, 0.3)
    med.runSignalSimulation(a)
    ref.run_signal_simulation(a)
    for m in range(med._dims["nSignalModes"]):
        assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL


@pytest.mark.parametrize("name", ["Chi2PDC", "Chi2SFG", "Chi2SHG", "Chi3GNLSE"])
def test_single_z_step(nlm, oracle, name):
    """zPrecision chosen so that nZSteps = 2: one RK4 step between the two dispersion halves (without
    poling, whose domains would be shorter than the step)."""
    kw = dict(cases.CASES[name])
    kw.pop("poling", None)
    kw["zPrecision"] = 1 if name == "Chi2PDC" else 2
    if name == "Chi3GNLSE":
        kw["relativeLength"] = 1
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    fnl = name in cases.FULLY_NONLINEAR
    assert med._dims["nZSteps"] == 2
    if not fnl:
        med.runPumpSimulation()
        ref.run_pump_simulation()
        C, S = med.computeGreensFunction()
        Cr, Sr = ref.compute_greens_function()
        assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL
    out, want = _batch_pair(med, ref, 4, 9, fnl)
    assert cases.rel_l2(out, want) < TOL


def test_null_output_pointers(nlm):
    """C-ABI queries given a null output pointer return an error status and leave the handle usable."""
    import ctypes
    lib = nlm._lib
    med = nlm.Chi2PDC(**dict(PDC, tPrecision=64))
    rows, cols = ctypes.c_size_t(), ctypes.c_size_t()
    assert lib.nlm_green_dims(med._h(), 1, None, 0, None, 0, None, ctypes.byref(cols)) != 0
    assert "null output pointer" in lib.nlm_last_error().decode()
    data = ctypes.POINTER(ctypes.c_double)()
    assert lib.nlm_get_grid(med._h(), 0, 0, ctypes.byref(data), None, ctypes.byref(cols)) != 0
    assert lib.nlm_cascade_media(med._h(), None) != 0
    assert lib.nlm_fp64_peak(None) != 0
    assert lib.nlm_green_dims(med._h(), 1, None, 0, None, 0, ctypes.byref(rows), ctypes.byref(cols)) == 0
    assert rows.value == cols.value == 64
