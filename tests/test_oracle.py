"""The oracle against the reference's own golden vectors, its committed fixtures and the
known-answer properties of the reference's notebooks (CPU only)."""
import os

import numpy as np
import pytest

import cases

HERE = os.path.dirname(os.path.abspath(__file__))


def test_poling_matches_reference_domains_to_space(oracle):
    """setPoling restatement == reference poling.domainsToSpace (poling.py:439-471), bit for bit."""
    d = np.load(os.path.join(HERE, "golden", "poling_golden.npz"))
    for k in range(int(d["count"])):
        got = oracle.domains_to_space(d["domains_%d" % k], int(d["nz_%d" % k]))
        assert np.array_equal(got, d["expected_%d" % k]), k


def test_poling_errors(oracle):
    with pytest.raises(ValueError, match="invalid domain length"):
        oracle.domains_to_space([1, 0, 2], 10)
    with pytest.raises(ValueError, match="too small"):
        oracle.domains_to_space(np.ones(50), 10)


@pytest.mark.parametrize("name", ["Chi2PDC", "Chi2SFG", "Chi3", "Chi2SHG", "Chi3GNLSE"])
def test_oracle_reproduces_fixture(oracle, golden, name):
    """Regression pin: the oracle still produces the committed fixture."""
    med = oracle.SOLVERS[name](**cases.oracle_kwargs(name))
    if not med.fully_nonlinear:
        med.run_pump_simulation()
    x = golden[name + "__signal_in"]
    med.run_signal_simulation(x, True, 0)
    rows = golden[name + "__rows"]
    got = np.stack([g[rows] for g in med.signal_time])
    assert cases.rel_l2(got, golden[name + "__signal_time"]) < 1e-14


def test_axes_are_fft_ordered(oracle):
    """tau/omega in FFT order with omega opposite to numpy's fftfreq (src/_NonlinearMedium.cpp:121-124)."""
    m = oracle.Chi3(relativeLength=1, nlLength=1, beta2=-1, tMax=10, tPrecision=16, zPrecision=10)
    assert m.tau[0] == 0 and m.omega[0] == 0
    assert np.allclose(m.omega, -2 * np.pi * np.fft.fftfreq(16, d=2 * 10 / 16))


def test_soliton_is_stationary(oracle):
    """N=1 soliton keeps |A| (tests/03 - Nonlinear Propagation -- Solitons.py:42-48)."""
    m = oracle.Chi3(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, tMax=20, tPrecision=256, zPrecision=100)
    m.run_pump_simulation()
    assert np.max(np.abs(np.abs(m.pump_time[0][-1]) - np.abs(m.pump_time[0][0]))) < 1e-4


def test_green_consistency_and_symplectic(oracle):
    """a(L) = C a + S a* reproduces runSignalSimulation (tests/04 - Green's Function.py:98-111);
    C C^H - S S^H = I and C S^T = S C^T (tests/05 - Hosaka.py:115-121)."""
    m = oracle.Chi2PDC(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, beta1s=2, beta3s=0.1, tMax=20,
                       tPrecision=64, zPrecision=20, poling=np.ones(20))
    C, S = m.compute_greens_function()
    rng = np.random.default_rng(0)
    a = cases.noise(rng, 64, 1.0)
    m.run_signal_simulation(a, False)
    out = C @ np.fft.fftshift(a) + S @ np.fft.fftshift(a.conj())
    assert cases.rel_l2(out, np.fft.fftshift(m.signal_freq[0][-1])) < 1e-12
    eye = np.eye(64)
    assert np.abs(C @ C.conj().T - S @ S.conj().T - eye).max() < 1e-6
    assert np.abs(C @ S.T - S @ C.T).max() < 1e-9


def test_weak_gain_pdc_matches_pump_spectrum(oracle):
    """Weak-gain Chi2PDC: |S(w, -w)| follows the pump spectrum (tests/07 - Wasilewski.py:41-66)."""
    m = oracle.Chi2PDC(relativeLength=1, nlLength=100, beta2=1, beta2s=1, tMax=20, tPrecision=64, zPrecision=20)
    C, S = m.compute_greens_function()
    s_diag = np.abs(np.fliplr(S).diagonal())
    assert np.argmax(s_diag) in (31, 32, 33)
