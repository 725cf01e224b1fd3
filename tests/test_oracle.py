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


def test_gaussian_dispersion_known_answer(oracle):
    """Dispersion length (tests/01 - Dispersion.py, "Dispersion Length"): a Gaussian exp(-t^2/2) under
    beta2 = 1 with no nonlinearity keeps |A(z, t)| = (1 + z^2)^(-1/4) exp(-t^2 / (2 (1 + z^2))), whose
    width follows Agrawal's T(z) = T0 (1 + (z/L_d)^2)^(1/2); the last pump row (z = 5) to rounding,
    the rows at z = 1..4 to the sampling of the row grid."""
    m = oracle.Chi3(relativeLength=5, nlLength=np.inf, beta2=1, pulseType=0, tPrecision=2048, zPrecision=100,
                    tMax=50)
    m.run_pump_simulation()
    pt = np.asarray(m.pump_time[0])
    tau = m.tau

    def exact(z):
        return (1 + z * z) ** -0.25 * np.exp(-tau ** 2 / (2 * (1 + z * z)))
    assert np.max(np.abs(np.abs(pt[-1]) - exact(5.0))) < 1e-12
    for i in range(1, 5):
        r = int((pt.shape[0] - 1) * i / 5)
        assert np.max(np.abs(np.abs(pt[r]) - exact(5.0 * r / (pt.shape[0] - 1)))) < 2e-3


def test_group_delay_known_answer(oracle):
    """A group-velocity mismatch beta1 = 4 moves the pump by beta1 L = 20 over L = 5 (tests/01 -
    Dispersion.py, "Qualitative test"), its envelope unchanged by the walk-off."""
    m = oracle.Chi2PDC(relativeLength=5, nlLength=np.inf, beta2=1, beta2s=-1, pulseType=0, beta1=4, beta1s=-4,
                       tPrecision=2048, zPrecision=100, tMax=50)
    m.run_pump_simulation()
    p = np.abs(np.asarray(m.pump_time[0][-1])) ** 2
    assert abs(abs(np.sum(m.tau * p) / np.sum(p)) - 20.0) < 1e-9


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


def test_squeezing_known_answer(oracle):
    """Shirasaki notebook (tests/08 - Shirasaki.py): the squeezed quadrature of a Gaussian pulse in a
    Chi3 fibre over a nonlinear phase 0.1 follows Haus's formula (to 2e-4 here), through the Green's
    function and the restated consumers."""
    from oracle import multimode_oracle as M
    phi = 0.1
    m = oracle.Chi3(relativeLength=phi, nlLength=1, beta2=-1, pulseType=0, tPrecision=512, zPrecision=200)
    C, S = m.compute_greens_function()
    v = np.real(M.lo_squeezing(M.covariance(M.quadrature_greens(C, S)), m.pump_time[0][-1], tol=1e-2))
    haus = 1 + 2 * phi ** 2 / np.sqrt(3) - (2 * phi ** 3 / np.sqrt(3) + np.sqrt(2) * phi) / np.sqrt(1 + phi ** 2)
    assert abs(v[0] - haus) < 1e-3 * haus and v[1] > 1.0


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_multimode_oracle_matches_reference():
    """The restatement of the Green's-function consumers (multimode.py, decompositions.py) against
    the reference modules' own outputs (tests/golden/make_golden.py)."""
    from oracle import multimode_oracle as M
    g = np.load(os.path.join(HERE, "golden", "multimode_golden.npz"))
    C, S = g["in_C"], g["in_S"]
    Z = M.quadrature_greens(C, S)
    assert np.array_equal(Z, g["Z"])
    cov = M.covariance(Z)
    assert _rel(cov, g["cov"]) < 1e-14
    assert _rel(M.covariance_abasis(C, S), g["cov_a"]) < 1e-14
    assert _rel(M.normalized_cov(cov), g["normalized_cov"]) < 1e-14
    assert _rel(M.lo_squeezing(cov, g["in_pump"], tol=1.0), g["lo_squeezing"]) < 1e-13
    with pytest.raises(AssertionError, match="C_xx"):
        M.lo_squeezing(cov, g["in_pump"])
    assert _rel(M.downsampled_cov(Z, 12, g["in_omega"], 2.0), g["downsampled_cov"]) < 1e-14
    assert _rel(M.downsampled_cov_abasis(C, S, 12, g["in_omega"], 2.0), g["downsampled_cov_a"]) < 1e-14
    assert _rel(M.bloch_messiah_eigs(Z), g["bm_eigs"]) < 1e-13
    d, lv, rv = M.bloch_messiah_vecs(Z)
    assert _rel(d, g["bm_diag"]) < 1e-13 and _rel(lv, g["bm_left"]) < 1e-12 and _rel(rv, g["bm_right"]) < 1e-12
    for to_time, suffix in ((True, "time"), (False, "freq")):
        c, s = M.ft_greens(C, S, to_time)
        assert _rel(c, g["ft_c_" + suffix]) < 1e-14 and _rel(s, g["ft_s_" + suffix]) < 1e-14
    to_xp, from_xp = M.basis_transforms(5)
    assert np.array_equal(to_xp, g["to_xp"]) and np.array_equal(from_xp, g["from_xp"])
    cc, cs = M.combine_greens(C, S, C.T, S.conj())
    assert _rel(cc, g["combined_c"]) < 1e-14 and _rel(cs, g["combined_s"]) < 1e-14
    assert _rel(M.incoherent_power_greens(Z), g["incoherent"]) < 1e-15
    assert _rel(M.photon_mean(cov), g["photon_mean"]) < 1e-13
    assert _rel(M.photon_mean_a(g["cov_a"]), g["photon_mean_a"]) < 1e-13
    assert _rel(M.photon_cov(cov), g["photon_cov"]) < 1e-14
    assert _rel(M.parametric_fluorescence(g["in_modes"], g["in_diag"]), g["fluorescence"]) < 1e-14
    assert _rel(M.effective_adjacency(g["in_modes"], g["in_diag"]), g["adjacency"]) < 1e-14
    assert _rel(M.full_effective_adjacency(cov), g["full_adjacency"]) < 1e-13
    assert _rel(M.cov_lump_loss(cov, 0.7), g["lump_scalar"]) < 1e-15
    assert _rel(M.cov_lump_loss(g["cov_a"], g["in_transmission"], abasis=True), g["lump_vector_a"]) < 1e-15
    u, p = M.left_polar(g["in_polar_in"])
    assert _rel(u, g["polar_u"]) < 1e-13 and _rel(p, g["polar_p"]) < 1e-13
    for kind in ("c", "r"):
        src = g["in_sym_complex"] if kind == "c" else g["in_sym_real"]
        lam, U = M.takagi(src)
        assert _rel(lam, g["takagi_%s_l" % kind]) < 1e-13 and _rel(U, g["takagi_%s_u" % kind]) < 1e-12
    ut, st, v = M.bloch_messiah(Z, tol=1e-6)
    assert _rel(st, g["bm_st"]) < 1e-12
    assert _rel(ut, g["bm_ut"]) < 1e-10 and _rel(v, g["bm_v"]) < 1e-10
