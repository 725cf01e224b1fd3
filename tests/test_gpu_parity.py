"""Parity of the CUDA engine with the oracle, through the drop-in API and its C ABI.

Tolerance: relative L2 error <= 1e-9 over every output array (the required bound for FP64
propagation); the expected level is ~1e-13 since both sides compute in double precision.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9


def make(nlm, name, **over):
    return getattr(nlm, name)(**dict(cases.CASES[name], **over))


@pytest.mark.parametrize("name", [n for n in cases.CASES if n not in cases.FULLY_NONLINEAR])
def test_pump_grids_match_golden(nlm, golden, name):
    med = make(nlm, name)
    med.runPumpSimulation()
    rows = golden[name + "__pump_rows"]
    for m in range(golden[name + "__pump_time"].shape[0]):
        assert cases.rel_l2(med.pumpTimes(m)[rows], golden[name + "__pump_time"][m]) < TOL
        assert cases.rel_l2(med.pumpFreqs(m)[rows], golden[name + "__pump_freq"][m]) < TOL


@pytest.mark.parametrize("name", list(cases.CASES))
def test_signal_grids_match_golden(nlm, golden, name):
    med = make(nlm, name)
    if name not in cases.FULLY_NONLINEAR:
        med.runPumpSimulation()
    med.runSignalSimulation(golden[name + "__signal_in"], True, 0)
    rows = golden[name + "__rows"]
    for m in range(golden[name + "__signal_time"].shape[0]):
        assert cases.rel_l2(med.signalTimes(m)[rows], golden[name + "__signal_time"][m]) < TOL, m
        assert cases.rel_l2(med.signalFreqs(m)[rows], golden[name + "__signal_freq"][m]) < TOL, m


@pytest.mark.parametrize("name", list(cases.CASES))
def test_batch_matches_golden(nlm, golden, name):
    med = make(nlm, name)
    x = golden[name + "__batch_in"]
    if name in cases.FULLY_NONLINEAR:
        out = med.batchSignalSimulation(x, False, 1, 0)
    else:
        med.runPumpSimulation()
        out = med.batchSignalSimulation(x, False, False)
    assert out.shape == golden[name + "__batch_out"].shape
    assert cases.rel_l2(out, golden[name + "__batch_out"]) < TOL


@pytest.mark.parametrize("name", [n for n in cases.CASES if n not in cases.FULLY_NONLINEAR])
@pytest.mark.parametrize("use_prop", [1, 0])
def test_green_matches_golden(nlm, golden, name, use_prop):
    med = make(nlm, name)
    med._set_schedule(use_propagator=use_prop)
    med.runPumpSimulation()
    C, S = med.computeGreensFunction(False, False)
    assert cases.rel_l2_pair(C, S, golden[name + "__green_c"], golden[name + "__green_s"]) < TOL
    Ct, St = med.computeGreensFunction(True, False)
    assert cases.rel_l2_pair(Ct, St, golden[name + "__green_c_time"], golden[name + "__green_s_time"]) < TOL


def test_green_options_match_oracle(nlm, oracle):
    """normalize, useInput/useOutput masks on a two-mode solver (src/_NonlinearMedium.cpp:266-372)."""
    kw = dict(cases.CASES["Chi2SFG"])
    med, ref = nlm.Chi2SFG(**kw), oracle.Chi2SFG(**kw)
    for norm, ui, uo in ((True, [], []), (False, [1, 1], [1, 0]), (True, [1, 1], [0, 1]), (False, [], [1])):
        C, S = med.computeGreensFunction(False, True, 1, norm, ui, uo)
        Cr, Sr = ref.compute_greens_function(False, True, 1, norm, ui, uo)
        assert C.shape == Cr.shape
        assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL


def test_batch_options_match_oracle(nlm, oracle):
    kw = dict(cases.CASES["Chi2SFGII"])
    med, ref = nlm.Chi2SFGII(**kw), oracle.Chi2SFGII(**kw)
    n = med._dims["nFreqs"]
    rng = np.random.default_rng(5)
    x2 = cases.noise(rng, 4 * 2 * n, 1.0).reshape(4, 2 * n)
    x1 = cases.noise(rng, 4 * n, 1.0).reshape(4, n)
    for x, mode, uo, t in ((x2, 0, [1, 0, 1, 1], True), (x1, 3, [0, 1], False), (x1, 2, [], True)):
        out = med.batchSignalSimulation(x, t, True, 1, mode, uo)
        refo = ref.batch_signal_simulation(x, t, True, 1, mode, uo)
        assert cases.rel_l2(out, refo) < TOL


def test_chirp_delay_and_custom_pump(nlm, oracle):
    kw = dict(cases.CASES["Chi2PDC"], chirp=0.3, delay=0.2)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    assert cases.rel_l2(med._axis(4, 0, complex_=True), ref.envelope[0]) < 1e-13
    rng = np.random.default_rng(3)
    p = np.exp(-ref.tau ** 2 / 3) * (1 + 0.1 * rng.standard_normal(ref.n_freqs))
    med.setPump(p, chirp=-0.2, delay=0.1)
    ref.set_pump_custom(p, -0.2, 0.1)
    med.setPump(nlm.Sinc, 0.1)
    ref.set_pump_type(oracle.SINC, 0.1)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL


def test_gaussian_beam_profile_pump(nlm, oracle):
    kw = dict(cases.CASES["Chi2SFG"], rayleighLength=0.6, intensityProfile=0)
    med, ref = nlm.Chi2SFG(**kw), oracle.Chi2SFG(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    kw = dict(cases.CASES["Chi3"], rayleighLength=0.6, intensityProfile=2)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL


def test_set_pump_from_other_medium(nlm, oracle):
    """setPump(other) copies another medium's signal with the frame phase (src/_NonlinearMedium.cpp:506-534)."""
    kw1 = dict(cases.CASES["Chi2SFG"], zPrecision=20)
    kw2 = dict(cases.CASES["Chi2PDCII"])
    a, ra = nlm.Chi2SFG(**kw1), oracle.Chi2SFG(**kw1)
    b, rb = nlm.Chi2PDCII(**kw2), oracle.Chi2PDCII(**kw2)
    assert a._dims["nZSteps"] >= b._dims["nZSteps"]
    x = cases.signal_input("Chi2SFG", 32, 2, seed=4)
    a.runPumpSimulation()
    ra.run_pump_simulation()
    a.runSignalSimulation(x)
    ra.run_signal_simulation(x)
    b.runPumpSimulation()
    rb.run_pump_simulation()
    b.setPump(a, 1, 0.3)
    rb.set_pump_other(ra, 1, 0.3)
    assert cases.rel_l2(b.pumpFreq, rb.pump_freq[0]) < TOL
    assert cases.rel_l2(b.pumpTime, rb.pump_time[0]) < TOL
    C, S = b.computeGreensFunction(runPump=False)
    Cr, Sr = rb.compute_greens_function(run_pump=False)
    assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL
    with pytest.raises(ValueError, match="Mode index larger"):
        nlm.Chi2PDC(**dict(cases.CASES["Chi2PDC"], tPrecision=32, tMax=10)).setPump(a, 1)   # this medium's modes


@pytest.mark.parametrize("n", [16, 32, 128])
def test_cascade_matches_oracle(nlm, oracle, n):
    """Green's functions, signal and batch through a cascade of two media; the composition's 32 x 32
    tiles are partial (16), whole (32) and several (128)."""
    kwa = dict(cases.CASES["Chi2PDC"], tPrecision=n, tMax=10)
    kwb = dict(cases.CASES["Chi2PDC"], tPrecision=n, tMax=10, beta1s=-1, diffBeta0=0.2)
    a, b = nlm.Chi2PDC(**kwa), nlm.Chi2PDC(**kwb)
    ra, rb = oracle.Chi2PDC(**kwa), oracle.Chi2PDC(**kwb)
    c = nlm.Cascade([a, b], [{0: 0}], True)
    rc = oracle.Cascade([ra, rb], [{0: 0}], True)
    C, S = c.computeGreensFunction()
    Cr, Sr = rc.compute_greens_function()
    assert cases.rel_l2_pair(C, S, Cr, Sr) < TOL
    x = cases.signal_input("Chi2PDC", n, 1, seed=9)
    c.runSignalSimulation(x)
    rc.run_signal_simulation(x)
    assert cases.rel_l2(b.signalFreq, rb.signal_freq[0]) < TOL
    xb = np.stack([cases.signal_input("Chi2PDC", n, 1, seed=k) for k in range(3)])
    assert cases.rel_l2(c.batchSignalSimulation(xb), rc.batch_signal_simulation(xb)) < TOL


@pytest.mark.parametrize("rows,inner,cols", [(16, 16, 16), (40, 72, 24), (256, 256, 256)])
def test_cascade_compose_matches_torch(nlm, rows, inner, cols):
    """The composition kernel on its own (partial and whole 32 x 32 tiles, rectangular shapes) against
    torch's complex128 matmul: C2 C1 + S2 conj(S1), C2 S1 + S2 conj(C1)."""
    import ctypes
    torch = pytest.importorskip("torch")
    g = torch.Generator().manual_seed(rows + inner + cols)

    def mat(r, c):
        return torch.complex(torch.randn(r, c, generator=g, dtype=torch.float64),
                             torch.randn(r, c, generator=g, dtype=torch.float64)).cuda()
    c2, s2, c1, s1 = mat(rows, inner), mat(rows, inner), mat(inner, cols), mat(inner, cols)
    co = torch.empty(rows, cols, dtype=torch.complex128, device="cuda")
    so = torch.empty_like(co)
    vp = ctypes.c_void_p
    nlm._check(nlm._lib.nlm_cascade_compose(vp(c2.data_ptr()), vp(s2.data_ptr()), vp(c1.data_ptr()), vp(s1.data_ptr()),
                                            rows, inner, cols, vp(co.data_ptr()), vp(so.data_ptr()),
                                            vp(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    ce = c2 @ c1 + s2 @ s1.conj()
    se = c2 @ s1 + s2 @ c1.conj()
    assert cases.rel_l2(co.cpu().numpy(), ce.cpu().numpy()) < 1e-13
    assert cases.rel_l2(so.cpu().numpy(), se.cpu().numpy()) < 1e-13


def test_plain_equals_batched(nlm):
    med = make(nlm, "Chi2PDC")
    med.runPumpSimulation()
    C, S = med.computeGreensFunction(runPump=False)
    n = med._dims["nFreqs"]
    import ctypes
    Cp = np.empty_like(C)
    Sp = np.empty_like(S)
    nlm._check(nlm._lib.nlm_green_plain(med._h(), 0, 0, 0, nlm._dptr(Cp.view(np.float64)),
                                        nlm._dptr(Sp.view(np.float64))))
    assert med._launch_count() >= 2 * n
    assert cases.rel_l2(Cp, C) < 1e-12 and cases.rel_l2(Sp, S) < 1e-12
    del ctypes


def test_deterministic(nlm):
    med = make(nlm, "Chi2SFG")
    C1, S1 = med.computeGreensFunction()
    C2, S2 = med.computeGreensFunction()
    assert np.array_equal(C1, C2) and np.array_equal(S1, S2)


def test_green_benchmark_config_reduced_steps(nlm, oracle):
    """The Green's-function benchmark medium (N=1024) at 40 z steps against the oracle."""
    kw = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
              beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, zPrecision=20, poling=np.ones(4))
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    assert med._dims["nZSteps"] == 40
    C, S = med.computeGreensFunction()
    Cr, Sr = ref.compute_greens_function(chunk=512)
    assert cases.rel_l2(C, Cr) < TOL and cases.rel_l2(S, Sr) < TOL   # both matrices are O(1) for PDC


def test_green_benchmark_config_full_size_properties(nlm):
    """Full benchmark size (N=1024, nZSteps=1000): symplectic C/S and Green consistency with a direct run."""
    kw = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
              beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, zPrecision=500, poling=np.ones(100))
    med = nlm.Chi2PDC(**kw)
    C, S = med.computeGreensFunction()
    eye = np.eye(1024)
    assert np.abs(C @ C.conj().T - S @ S.conj().T - eye).max() < 1e-6
    assert np.abs(C @ S.T - S @ C.T).max() < 1e-8
    rng = np.random.default_rng(2)
    a = cases.noise(rng, 1024, 1e-3)
    med.runSignalSimulation(a, False)
    out = C @ np.fft.fftshift(a) + S @ np.fft.fftshift(a.conj())
    assert cases.rel_l2(out, np.fft.fftshift(med.signalFreq[-1])) < 1e-9


def test_dispersion_known_answers(nlm):
    """The reference's dispersion checks (tests/01 - Dispersion.py) on the engine: with no nonlinearity
    a Gaussian exp(-t^2/2) under beta2 = 1 keeps |A(z, t)| = (1 + z^2)^(-1/4) exp(-t^2 / (2 (1 + z^2)))
    (Agrawal's dispersion-length broadening), in the pump march and in the signal march (full grids
    of 2048 points on clusters); a group-velocity mismatch beta1 = 4 (beta1s = -4) moves the pump
    (signal) by 20 over L = 5."""
    m = nlm.Chi3(relativeLength=5, nlLength=np.inf, beta2=1, pulseType=0, tPrecision=2048, zPrecision=100, tMax=50)
    tau = m.tau

    def exact(z):
        return (1 + z * z) ** -0.25 * np.exp(-tau ** 2 / (2 * (1 + z * z)))
    m.runPumpSimulation()
    pt = m.pumpTime
    assert np.max(np.abs(np.abs(pt[-1]) - exact(5.0))) < 1e-12
    for i in range(1, 5):
        r = int((pt.shape[0] - 1) * i / 5)
        assert np.max(np.abs(np.abs(pt[r]) - exact(5.0 * r / (pt.shape[0] - 1)))) < 2e-3
    m.runSignalSimulation(np.exp(-0.5 * tau ** 2) + 0j)
    assert np.max(np.abs(np.abs(m.signalTime[-1]) - exact(5.0))) < 1e-12
    w = nlm.Chi2PDC(relativeLength=5, nlLength=np.inf, beta2=1, beta2s=-1, pulseType=0, beta1=4, beta1s=-4,
                    tPrecision=2048, zPrecision=100, tMax=50)
    w.runPumpSimulation()
    w.runSignalSimulation(np.exp(-0.5 * tau ** 2) + 0j)
    for grid, shift in ((w.pumpTime, 20.0), (w.signalTime, 20.0)):
        p = np.abs(grid[-1]) ** 2
        assert abs(abs(np.sum(tau * p) / np.sum(p)) - shift) < 1e-9
    # opposite walk-off: the pump and the signal move apart by 40
    pp, ps = np.abs(w.pumpTime[-1]) ** 2, np.abs(w.signalTime[-1]) ** 2
    assert abs(abs(np.sum(tau * pp) / np.sum(pp) - np.sum(tau * ps) / np.sum(ps)) - 40.0) < 1e-8


def test_soliton_and_green_known_answers(nlm):
    """On the engine: an N=1 soliton keeps |A| along the pump march (tests/03 - Nonlinear Propagation --
    Solitons.py:42-48); the Green's function of a Chi2PDC medium is symplectic, C C^H - S S^H = I and
    C S^T = S C^T (tests/05 - Hosaka.py:115-121), and reproduces a propagation through
    a(L) = C a + S a* (tests/04 - Green's Function.py:98-111)."""
    m = nlm.Chi3(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, tMax=20, tPrecision=256, zPrecision=100)
    m.runPumpSimulation()
    assert np.max(np.abs(np.abs(m.pumpTime[-1]) - np.abs(m.pumpTime[0]))) < 1e-4
    g = nlm.Chi2PDC(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, beta1s=2, beta3s=0.1, tMax=20,
                    tPrecision=256, zPrecision=20, poling=np.ones(20))
    C, S = g.computeGreensFunction()
    n = C.shape[0]
    # RK4 is symplectic only to its truncation error: 7.7e-9 and 1.4e-9 in the oracle at this size
    assert np.abs(C @ C.conj().T - S @ S.conj().T - np.eye(n)).max() < 1e-7
    assert np.abs(C @ S.T - S @ C.T).max() < 1e-7
    a = cases.noise(np.random.default_rng(0), n, 1.0)
    g.runSignalSimulation(a, False)
    out = C @ np.fft.fftshift(a) + S @ np.fft.fftshift(a.conj())
    assert cases.rel_l2(out, np.fft.fftshift(g.signalFreq[-1])) < 1e-12


def test_chi3_soliton_config(nlm, oracle):
    """Chi3 N=1 soliton pump + seeded-noise signal (N=512, nZSteps=200) against the oracle."""
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=512, zPrecision=200)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL
    a = cases.noise(np.random.default_rng(1), 512, 1e-3)
    med.runSignalSimulation(a)
    ref.run_signal_simulation(a)
    assert cases.rel_l2(med.signalTime, ref.signal_time[0]) < TOL
    assert cases.rel_l2(med.signalFreq, ref.signal_freq[0]) < TOL


@pytest.mark.parametrize("name", [n for n in cases.CASES if n != "Chi3GNLSE"])
def test_wide_and_narrow_direct_kernels(nlm, oracle, name):
    """The direct-DiffEq kernels in both launch forms: a batch with at least as many rows as SMs runs
    N/8 threads per propagation (N/4 for three and four modes), a batch of a few rows runs N/4."""
    med, ref = make(nlm, name), getattr(oracle, name)(**cases.oracle_kwargs(name))
    fnl = name in cases.FULLY_NONLINEAR
    if not fnl:
        med._set_schedule(use_propagator=0)
        med.runPumpSimulation()
        ref.run_pump_simulation()
    n = med._dims["nFreqs"]
    modes = med._dims["nSignalModes"]
    rng = np.random.default_rng(31)
    for rows, want_r in ((160, 8 if modes <= 2 else 4), (3, 4)):
        x = cases.noise(rng, rows * n, 0.5).reshape(rows, n)
        out = med.batchSignalSimulation(x, inTimeDomain=False) if fnl else \
            med.batchSignalSimulation(x, False, False)
        assert med._last_schedule()["R"] == want_r
        assert cases.rel_l2(out, ref.batch_signal_simulation(x, False) if fnl else
                            ref.batch_signal_simulation(x, False, False)) < TOL
