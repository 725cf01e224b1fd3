"""The C++ restatement of the split-step loop (oracle/nlm_cpu.cpp, the timed CPU baseline) against
the numpy oracle: the same algorithm written twice must agree to rounding (1e-12 relative L2)."""

import numpy as np
import pytest

import cases
from oracle import cpu_port, nlm_oracle as O

TOL = 1e-12


def test_green_matches_oracle():
    med = O.Chi2PDC(**cases.oracle_kwargs("Chi2PDC"))
    C0, S0 = med.compute_greens_function()
    C1, S1 = cpu_port.chi2pdc_green(med, threads=3)
    assert cases.rel_l2_pair(C1, S1, C0, S0) < TOL


def test_green_with_intensity_profile_matches_oracle():
    kw = dict(cases.oracle_kwargs("Chi2PDC"), rayleighLength=0.7, intensityProfile=O.GAUSSIAN_APODIZATION)
    med = O.Chi2PDC(**kw)
    C0, S0 = med.compute_greens_function()
    C1, S1 = cpu_port.chi2pdc_green(med, threads=2)
    assert cases.rel_l2_pair(C1, S1, C0, S0) < TOL


def test_impulse_range_matches_oracle():
    med = O.Chi2PDC(**cases.oracle_kwargs("Chi2PDC"))
    med.run_pump_simulation()
    n, start, count = med.n_freqs, 37, 11
    got = cpu_port.chi2pdc_impulses(med, start, count, threads=4)
    prof = np.zeros((count, n), dtype=np.complex128)
    for q in range(count):
        inst = start + q
        prof[q, (inst >> 1) % n] = 1j if inst & 1 else 1.0
    expected, _ = med.propagate(prof, False, 0)
    assert cases.rel_l2(got, expected[:, 0]) < TOL


@pytest.mark.parametrize("in_time", [False, True])
def test_gnlse_batch_matches_oracle(in_time):
    med = O.Chi3GNLSE(**cases.oracle_kwargs("Chi3GNLSE"))
    n = med.n_freqs
    x = np.stack([cases.signal_input("Chi3GNLSE", n, 1, seed=k) for k in range(3)])
    expected = med.batch_signal_simulation(x, in_time)
    got = cpu_port.gnlse_batch(med, x, in_time, threads=2)
    assert cases.rel_l2(got, expected) < TOL


def test_rejects_grids_it_does_not_take():
    med = O.Chi2PDC(**dict(cases.oracle_kwargs("Chi2PDC"), tPrecision=48))
    with pytest.raises(ValueError, match="power-of-two"):
        cpu_port.chi2pdc_green(med)


def test_gnlse_record_matches_full_grid():
    """The recorded spectra are the rows of the oracle's full signalFreq grid (runSignalSimulation)."""
    med = O.Chi3GNLSE(**cases.oracle_kwargs("Chi3GNLSE"))
    n = med.n_freqs
    x = cases.signal_input("Chi3GNLSE", n, 1, seed=3)
    med.run_signal_simulation(x, True)
    rec, out = cpu_port.gnlse_record(med, x, True, 3)
    rows = np.arange(1, rec.shape[0] + 1) * 3
    assert rows[-1] < med.n_z_steps - 1
    assert cases.rel_l2(rec, med.signal_freq[0][rows]) < TOL
    assert cases.rel_l2(out, med.signal_time[0][-1]) < TOL
