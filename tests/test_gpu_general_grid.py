"""Grids that are not powers of two (the general plan: mixed-radix passes through shared memory,
padded thread ownership) against the oracle, through the drop-in API.

The reference accepts any even number of frequency bins (src/_NonlinearMedium.cpp:105-113) and its
FFT adapter any length (src/CustomEigenFFT.h:44-140).  The cases cover radix-3/5 products (96, 384,
1000, 1536, 6000), small and odd-factor grids (6, 10, 462), large prime factors (514 = 2 x 257,
8186 = 2 x 4093), the four-mode solvers, and power-of-two grids beyond the register plan of the
one-CTA kernels (two modes at 8192 points in a batch).  The time window grows with the grid so that
the RK4 step stays stable (grid spacing at least 0.078; 0.024 with the GNLSE workload's z step).
Tolerance: relative L2 error <= 1e-9 on every output.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9
GRIDS = [96, 384, 1000, 1536, 6000]


def _kw(name, n, **over):
    if name == "Chi3GNLSE":
        # the GNLSE workload's medium and z step (stable with self-steepening up to its highest
        # frequency) over 19 steps; the window keeps its grid spacing from 4096 points up
        from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG
        kw = dict(GNLSE_CONFIG, tPrecision=n, tMax=50 * max(1.0, n / 4096), relativeLength=0.002)
    else:
        kw = dict(cases.CASES[name], tPrecision=n)
        kw["tMax"] = kw["tMax"] * max(1.0, n / 256)
    kw.update(over)
    return kw


def _input(name, n, modes, seed, t_max):
    rng = np.random.default_rng(seed)
    if name == "Chi3GNLSE":
        t = np.fft.fftshift(np.linspace(-t_max, t_max, n, endpoint=False))
        return 3.0 / np.cosh(t) + cases.noise(rng, n, 1e-3)
    sigma = 0.5 if name in cases.FULLY_NONLINEAR else 1.0
    return cases.noise(rng, n * modes, sigma)


def _grids_match(med, ref, modes):
    for m in range(modes):
        f, t = med.signalFreqs(m), med.signalTimes(m)
        assert np.all(np.isfinite(f)) and np.all(np.isfinite(t))
        assert cases.rel_l2(f, ref.signal_freq[m]) < TOL, m
        assert cases.rel_l2(t, ref.signal_time[m]) < TOL, m


@pytest.mark.parametrize("n", GRIDS)
def test_chi2pdc_general_grid(nlm, oracle, n):
    kw = _kw("Chi2PDC", n)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    x = _input("Chi2PDC", n, 1, 1, kw["tMax"])
    med.runSignalSimulation(x)
    ref.run_signal_simulation(x)
    _grids_match(med, ref, 1)
    rows = np.stack([_input("Chi2PDC", n, 1, 10 + k, kw["tMax"]) for k in range(3)])
    for use_prop in (1, 0):   # the RK4 propagator (linear kernel) and the DiffEq (direct kernel)
        med._set_schedule(use_propagator=use_prop)
        out = med.batchSignalSimulation(rows, runPump=False)
        assert cases.rel_l2(out, ref.batch_signal_simulation(rows, run_pump=False)) < TOL
        if n <= 1000:
            C, S = med.computeGreensFunction(runPump=False)
            Cr, Sr = ref.compute_greens_function(run_pump=False, chunk=512)
            assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL


@pytest.mark.parametrize("n", GRIDS)
def test_chi3_general_grid(nlm, oracle, n):
    """The self-phase-modulation pump march (one CTA on the general plan) and a signal."""
    kw = _kw("Chi3", n)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med._set_cluster(0)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL
    x = _input("Chi3", n, 1, 2, kw["tMax"])
    med.runSignalSimulation(x)
    ref.run_signal_simulation(x)
    _grids_match(med, ref, 1)


@pytest.mark.parametrize("n", GRIDS)
def test_chi2sfg_general_grid(nlm, oracle, n):
    kw = _kw("Chi2SFG", n)
    med, ref = nlm.Chi2SFG(**kw), oracle.Chi2SFG(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    rows = np.stack([_input("Chi2SFG", n, 2, 20 + k, kw["tMax"]) for k in range(3)])
    out = med.batchSignalSimulation(rows, runPump=False)
    assert cases.rel_l2(out, ref.batch_signal_simulation(rows, run_pump=False)) < TOL
    x = _input("Chi2SFG", n, 2, 3, kw["tMax"])
    med.runSignalSimulation(x)
    ref.run_signal_simulation(x)
    _grids_match(med, ref, 2)
    if n <= 384:
        C, S = med.computeGreensFunction(runPump=False)
        Cr, Sr = ref.compute_greens_function(run_pump=False, chunk=512)
        assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL


@pytest.mark.parametrize("n", GRIDS)
def test_gnlse_general_grid(nlm, oracle, n):
    kw = _kw("Chi3GNLSE", n)
    med, ref = nlm.Chi3GNLSE(**kw), oracle.Chi3GNLSE(**kw)
    rows = np.stack([_input("Chi3GNLSE", n, 1, 30 + k, kw["tMax"]) for k in range(3)])
    for in_time in (True, False):
        out = med.batchSignalSimulation(rows, in_time)
        assert np.all(np.isfinite(out))
        assert cases.rel_l2(out, ref.batch_signal_simulation(rows, in_time)) < TOL
    med._set_cluster(0)
    x = rows[0]
    med.runSignalSimulation(x)
    ref.run_signal_simulation(x)
    _grids_match(med, ref, 1)


@pytest.mark.parametrize("n", [6, 10, 462, 514])
def test_small_and_odd_factor_grids(nlm, oracle, n):
    """2 x 3, 2 x 5, 2 x 3 x 7 x 11 and 2 x 257 (a radix-257 pass computed as 257-term sums)."""
    kw = _kw("Chi2PDC", n)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    C, S = med.computeGreensFunction()
    Cr, Sr = ref.compute_greens_function(chunk=512)
    assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL
    kwg = _kw("Chi3GNLSE", n)
    g, gr = nlm.Chi3GNLSE(**kwg), oracle.Chi3GNLSE(**kwg)
    rows = np.stack([_input("Chi3GNLSE", n, 1, 40 + k, kwg["tMax"]) for k in range(2)])
    assert cases.rel_l2(g.batchSignalSimulation(rows, True), gr.batch_signal_simulation(rows, True)) < TOL


def test_large_prime_factor_grid(nlm, oracle):
    """8186 = 2 x 4093: the radix-4093 pass runs as 4093-term sums (the cost class of a generic
    butterfly); four z steps."""
    kw = _kw("Chi2PDC", 8186, zPrecision=2, poling=[1, 1])
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    assert med._dims["nZSteps"] == ref.n_z_steps and ref.n_z_steps <= 6
    x = _input("Chi2PDC", 8186, 1, 5, kw["tMax"])
    med.runSignalSimulation(x)
    ref.run_signal_simulation(x)
    _grids_match(med, ref, 1)


@pytest.mark.parametrize("n", [1000, 6000])
def test_four_mode_general_grid(nlm, oracle, n):
    kw = _kw("Chi2SFGII", n)
    med, ref = nlm.Chi2SFGII(**kw), oracle.Chi2SFGII(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    rows = np.stack([_input("Chi2SFGII", n, 4, 50 + k, kw["tMax"]) for k in range(2)])
    out = med.batchSignalSimulation(rows, runPump=False)
    assert cases.rel_l2(out, ref.batch_signal_simulation(rows, run_pump=False)) < TOL


def test_two_mode_batch_at_8192_points(nlm, oracle):
    """A power-of-two grid beyond the register plan of the one-CTA two-mode kernels (8192 / 8 = 1024
    threads), with more rows than the cluster form takes: the general-plan kernel with R = 16."""
    kw = _kw("Chi2SFG", 8192, zPrecision=4, poling=[1, 1])
    med, ref = nlm.Chi2SFG(**kw), oracle.Chi2SFG(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    rows = np.stack([_input("Chi2SFG", 8192, 2, 60 + k, kw["tMax"]) for k in range(48)])
    out = med.batchSignalSimulation(rows, runPump=False)
    assert med._last_schedule()["R"] == 16
    assert cases.rel_l2(out, ref.batch_signal_simulation(rows, run_pump=False)) < TOL


def test_ragged_set_with_general_grids(nlm, oracle):
    """A ragged set mixing power-of-two and other grids: the others propagate one launch each."""
    media, refs, ins = [], [], []
    for k, n in enumerate((128, 96, 1000, 256)):
        kw = _kw("Chi2SFG", n)
        m, r = nlm.Chi2SFG(**kw), oracle.Chi2SFG(**kw)
        m.runPumpSimulation()
        r.run_pump_simulation()
        media.append(m)
        refs.append(r)
        ins.append(_input("Chi2SFG", n, 1, 70 + k, kw["tMax"]))
    outs = nlm.ragged_batch(media, ins)
    for r, x, o in zip(refs, ins, outs):
        f, _ = r.propagate(x[None, :], False, 0)
        assert cases.rel_l2(o, f[0]) < TOL


def test_general_grid_limits(nlm):
    """Past 8192 points there is no kernel; the adjoint takes power-of-two grids only."""
    big = nlm.Chi2PDC(**_kw("Chi2PDC", 8194, zPrecision=2, poling=[1, 1]))
    with pytest.raises(nlm.UnsupportedError):
        big.runSignalSimulation(np.ones(8194, dtype=np.complex128))
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_pdc
    med = nlm.Chi2PDC(**_kw("Chi2PDC", 96))
    nz = med._dims["nZSteps"]
    x = torch.zeros((1, 96), dtype=torch.complex128, device="cuda", requires_grad=True)
    f0 = torch.ones(96, dtype=torch.complex128, device="cuda", requires_grad=True)
    d = torch.ones(nz, dtype=torch.float64, requires_grad=True)
    with pytest.raises(nlm.UnsupportedError, match="power-of-two"):
        propagate_pdc(med, x, f0, d)
