"""Propagations spread over a 4-CTA cluster (four-step FFT through distributed shared memory): the
full grids of runSignalSimulation and small batches on grids of 1024 to 8192 points with four points
per thread (cluster mode 2, and the default from 2048 points), the full grids and the Chi3 pump march
on grids of 256 to 1024 points with one point per thread (the default there), against the oracle and
against the one-CTA kernels."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9

PDC = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0.2, beta1s=2, beta3=0.05,
           beta3s=0.1, diffBeta0=0.4, tMax=40, zPrecision=8, poling=[1, 2, 1])
SFG = dict(relativeLength=1, nlLength=0.8, nlLengthOrig=1.2, beta2=0.5, beta2s=-0.3, beta2o=0.2, pulseType=0,
           beta1=0.1, beta1s=1, beta1o=-0.5, beta3=0, beta3s=0.05, beta3o=0.02, diffBeta0=1.3, tMax=20,
           zPrecision=8, poling=[2, 1, 3, 1])
CHI3 = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0.02, tMax=40, zPrecision=12)
SHG = dict(relativeLength=1, nlLengthH=0.9, nlLengthP=1.1, beta2h=0.3, beta2p=-0.2, beta1h=0.5, beta1p=-0.1,
           diffBeta0=0.4, tMax=20, zPrecision=8, poling=[1, 1, 2])
MEDIA = {"Chi2PDC": PDC, "Chi2SFG": SFG, "Chi3": CHI3, "Chi2SHG": SHG}


@pytest.mark.parametrize("n", [1024, 2048, 4096, 8192])
@pytest.mark.parametrize("name", ["Chi2PDC", "Chi3"])
def test_cluster_signal_grids_match_oracle(nlm, oracle, name, n):
    kw = dict(MEDIA[name], tPrecision=n)
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    med._set_cluster(2)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    a = cases.noise(np.random.default_rng(n), n, 0.2)
    for in_time in (True, False):
        med.runSignalSimulation(a, in_time)
        ref.run_signal_simulation(a, in_time)
        sched = med._last_schedule()
        assert sched["R"] == 4 and sched["grid"] == 4 and sched["block"] == n // 16
        assert cases.rel_l2(med.signalTime, ref.signal_time[0]) < TOL
        assert cases.rel_l2(med.signalFreq, ref.signal_freq[0]) < TOL


@pytest.mark.parametrize("name", ["Chi2SFG", "Chi2SHG"])
@pytest.mark.parametrize("n", [1024, 4096])
def test_cluster_two_modes_match_oracle(nlm, oracle, name, n):
    kw = dict(MEDIA[name], tPrecision=n)
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    fnl = name in cases.FULLY_NONLINEAR
    if not fnl:
        med.runPumpSimulation()
        ref.run_pump_simulation()
    a = cases.noise(np.random.default_rng(3), n, 0.2)
    med.runSignalSimulation(a)
    ref.run_signal_simulation(a)
    # full grids: eight CTAs (two modes fused; sixteen CTAs would not hold their buffers at 4096)
    assert med._last_schedule()["grid"] == 8
    for m in range(2):
        assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL
        assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL
    x = cases.noise(np.random.default_rng(4), 3 * n, 0.2).reshape(3, n)
    out = med.batchSignalSimulation(x, inTimeDomain=True) if fnl else med.batchSignalSimulation(x, True, False)
    want = ref.batch_signal_simulation(x, True) if fnl else ref.batch_signal_simulation(x, True, False)
    assert med._last_schedule()["grid"] == 12
    assert cases.rel_l2(out, want) < TOL


def test_cluster_equals_one_cta_kernels(nlm):
    kw = dict(PDC, tPrecision=2048, zPrecision=40)
    a = cases.noise(np.random.default_rng(9), 2048, 0.3)
    res = []
    for use in (2, 0):
        med = nlm.Chi2PDC(**kw)
        med._set_cluster(use)
        med.runPumpSimulation()
        med.runSignalSimulation(a)
        assert (med._last_schedule()["grid"] == 4) == bool(use)
        res.append((med.signalFreq.copy(), med.signalTime.copy()))
    assert cases.rel_l2(res[0][0], res[1][0]) < 1e-12 and cases.rel_l2(res[0][1], res[1][1]) < 1e-12


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("name", [n for n in cases.CASES if n != "Chi3GNLSE"])
def test_cluster_every_solver_matches_oracle(nlm, oracle, name, mode):
    """runSignalSimulation of each DiffEq solver on a 1024-point grid runs on a cluster: eight CTAs with
    one point per thread (mode 1, the default) or four CTAs with four (mode 2), and matches the oracle's
    full grids."""
    kw = dict(cases.CASES[name], tPrecision=1024)
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**cases.oracle_kwargs(name) | {"tPrecision": 1024})
    med._set_cluster(mode)
    if name not in cases.FULLY_NONLINEAR:
        med.runPumpSimulation()
        ref.run_pump_simulation()
    a = cases.noise(np.random.default_rng(5), 1024, 0.3)
    med.runSignalSimulation(a, True, 0)
    ref.run_signal_simulation(a, True, 0)
    if name == "Chi3" and mode == 1:
        # right after runPumpSimulation: the pump march and the signal side by side, four CTAs of 256
        # threads each; with the pump in place the signal alone takes the form below
        sched = med._last_schedule()
        assert sched["grid"] == 8 and sched["R"] == 1 and sched["block"] == 256
        first = med.signalTime.copy()
        med.runSignalSimulation(a, True, 0)
        assert cases.rel_l2(med.signalTime, first) < 1e-12
    sched = med._last_schedule()
    # full grids at 1024 points: eight CTAs of 128 threads (mode 1), four of 64 with four points each
    assert sched["grid"] == (8 if mode == 1 else 4) and sched["R"] == (1 if mode == 1 else 4)
    assert sched["block"] == (128 if mode == 1 else 64)
    for m in range(med._dims["nSignalModes"]):
        assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL, m
        assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL, m


@pytest.mark.parametrize("n,t_max", [(1024, 50), (4096, 50), (8192, 100)])
def test_cluster_gnlse_matches_oracle(nlm, oracle, n, t_max):
    """Chi3GNLSE on clusters (all 16 stage transforms and the dispersion pair as cluster FFTs): full
    grids of one propagation and a small batch (one point per thread on 8 or 16 CTAs per row; four
    points per thread on four at 8192), against the oracle and the one-CTA kernel (N=8192 has no
    one-CTA GNLSE kernel).  The medium is the GNLSE benchmark's (N=3 soliton, Raman,
    self-steepening) over 0.2 of its length with its z step (1999 steps); at N=8192 the time window
    doubles so that the RK4 step stays stable for the self-steepening term at the highest frequency."""
    from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG
    kw = dict(GNLSE_CONFIG, tPrecision=n, relativeLength=0.2, tMax=t_max)
    med, ref = nlm.Chi3GNLSE(**kw), oracle.Chi3GNLSE(**kw)
    t = np.fft.fftshift(np.linspace(-t_max, t_max, n, endpoint=False))
    a = 3.0 / np.cosh(t) + cases.noise(np.random.default_rng(n), n, 1e-4)
    med.runSignalSimulation(a)
    ref.run_signal_simulation(a)
    # full grids: one point per thread on eight CTAs at 1024 points, sixteen at 4096; four points per
    # thread on four CTAs at 8192
    s = med._last_schedule()
    assert (s["grid"], s["R"]) == {1024: (8, 1), 4096: (16, 1), 8192: (4, 4)}[n]
    assert cases.rel_l2(med.signalTime, ref.signal_time[0]) < TOL
    assert cases.rel_l2(med.signalFreq, ref.signal_freq[0]) < TOL
    x = np.fft.fft(a)[None, :] * np.exp(1j * np.arange(3))[:, None]
    out = med.batchSignalSimulation(x, inTimeDomain=False)
    s = med._last_schedule()
    # a small batch: one point per thread on eight CTAs per row at 1024 points, sixteen at 4096; four
    # points per thread on four CTAs at 8192
    assert (s["grid"], s["R"]) == {1024: (24, 1), 4096: (48, 1), 8192: (12, 4)}[n]
    assert cases.rel_l2(out, ref.batch_signal_simulation(x, False)) < TOL
    if n <= 4096:
        one = nlm.Chi3GNLSE(**kw)
        one._set_cluster(0)
        # soliton fission amplifies rounding differences between the two transform orders
        assert cases.rel_l2(one.batchSignalSimulation(x, inTimeDomain=False), out) < 1e-10


@pytest.mark.parametrize("n", [1024, 2048, 8192])
def test_cluster_chi3_pump_march(nlm, oracle, n):
    """The self-phase-modulation pump march on four SMs: both pump grids against the oracle, and
    against the one-CTA march (same arithmetic, other transform order)."""
    kw = dict(CHI3, tPrecision=n, zPrecision=15)
    med, ref, one = nlm.Chi3(**kw), oracle.Chi3(**kw), nlm.Chi3(**kw)
    one._set_cluster(0)
    for m in (med, one):
        m.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL
    assert cases.rel_l2(med.pumpTime, one.pumpTime) < 1e-12
    assert cases.rel_l2(med.pumpFreq, one.pumpFreq) < 1e-12


@pytest.mark.parametrize("name", [n for n in cases.CASES if n != "Chi3GNLSE" and n not in ("Chi3", "Chi2PDC")])
def test_wide_spread_every_multimode_solver(nlm, oracle, name):
    """runSignalSimulation of every multi-mode solver on 2048 points in cluster mode 3: eight CTAs with
    one point per thread, the modes in each transform together where their buffers fit (two modes), one after another
    otherwise (three and four), against the oracle's full grids."""
    kw = dict(cases.CASES[name], tPrecision=2048, tMax=cases.CASES[name]["tMax"] * 8)
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    med._set_cluster(3)                                  # eight CTAs (mode 1 takes sixteen where it can)
    if name not in cases.FULLY_NONLINEAR:
        med.runPumpSimulation()
        ref.run_pump_simulation()
    modes = med._dims["nSignalModes"]
    a = cases.noise(np.random.default_rng(7), 2048 * modes, 0.3)
    med.runSignalSimulation(a, True, 0)
    ref.run_signal_simulation(a, True, 0)
    sched = med._last_schedule()
    assert sched["grid"] == 8 and sched["R"] == 1 and sched["block"] == 256
    for m in range(modes):
        assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL, m
        assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL, m


@pytest.mark.parametrize("name", [n for n in cases.CASES if n != "Chi3GNLSE"])
def test_sixteen_cta_spread_every_solver(nlm, oracle, name):
    """runSignalSimulation on 2048 points over sixteen CTAs with one point per thread (the default for
    full grids; 128 threads each; multi-mode solvers with their modes in each transform together, up
    to three modes), against the oracle's full grids and the eight-CTA form (cluster mode 3)."""
    kw = dict(cases.CASES[name], tPrecision=2048, tMax=cases.CASES[name]["tMax"] * 8)
    med, ref, w8 = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw), getattr(nlm, name)(**kw)
    w8._set_cluster(3)
    if name not in cases.FULLY_NONLINEAR:
        for m in (med, w8):
            m.runPumpSimulation()
        ref.run_pump_simulation()
    modes = med._dims["nSignalModes"]
    a = cases.noise(np.random.default_rng(17), 2048 * modes, 0.3)
    for in_time in (True, False):
        med.runSignalSimulation(a, in_time, 0)
        w8.runSignalSimulation(a, in_time, 0)
        ref.run_signal_simulation(a, in_time, 0)
        sched = med._last_schedule()
        # four modes: the mode-fused buffers of sixteen CTAs do not fit, and eight CTAs run it
        ctas = 16 if modes <= 3 else 8
        assert sched["grid"] == ctas and sched["R"] == 1 and sched["block"] == 2048 // ctas
        assert w8._last_schedule()["grid"] == 8
        for m in range(modes):
            assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL, m
            assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL, m
            assert cases.rel_l2(med.signalTimes(m), w8.signalTimes(m)) < 1e-12, m


@pytest.mark.parametrize("name", ["Chi2PDC", "Chi2SFG"])
def test_eight_cta_spread_at_1024(nlm, oracle, name):
    """Full grids on 1024 points: eight CTAs of 128 threads (also the form a ragged plan gives its long
    1024-point marches), both input domains, against the oracle and the four-CTA form (mode 3)."""
    kw = dict(MEDIA[name], tPrecision=1024)
    med, ref, c4 = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw), getattr(nlm, name)(**kw)
    c4._set_cluster(3)
    for m in (med, c4):
        m.runPumpSimulation()
    ref.run_pump_simulation()
    modes = med._dims["nSignalModes"]
    a = cases.noise(np.random.default_rng(21), 1024, 0.2)
    for in_time in (True, False):
        med.runSignalSimulation(a, in_time)
        c4.runSignalSimulation(a, in_time)
        ref.run_signal_simulation(a, in_time)
        sched = med._last_schedule()
        assert sched["grid"] == 8 and sched["block"] == 128 and c4._last_schedule()["grid"] == 4
        for m in range(modes):
            assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL
            assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL
            assert cases.rel_l2(med.signalFreqs(m), c4.signalFreqs(m)) < 1e-12


@pytest.mark.parametrize("n", [2048, 4096])
def test_sixteen_cta_spread_single_mode(nlm, oracle, n):
    """Full grids of Chi2PDC at 2048 and 4096 points on sixteen CTAs (256 threads per CTA at 4096), both
    input domains, against the oracle; a 4096-point two-mode medium, whose mode-fused buffers do not
    fit, keeps eight CTAs."""
    kw = dict(MEDIA["Chi2PDC"], tPrecision=n)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    a = cases.noise(np.random.default_rng(n + 5), n, 0.2)
    for in_time in (True, False):
        med.runSignalSimulation(a, in_time)
        ref.run_signal_simulation(a, in_time)
        sched = med._last_schedule()
        assert sched["grid"] == 16 and sched["block"] == n // 16
        assert cases.rel_l2(med.signalTimes(0), ref.signal_time[0]) < TOL
        assert cases.rel_l2(med.signalFreqs(0), ref.signal_freq[0]) < TOL
    if n == 4096:
        kw2 = dict(MEDIA["Chi2SFG"], tPrecision=n)
        m2 = nlm.Chi2SFG(**kw2)
        m2.runPumpSimulation()
        m2.runSignalSimulation(cases.noise(np.random.default_rng(3), n, 0.2))
        assert m2._last_schedule()["grid"] == 8


@pytest.mark.parametrize("n", [128, 256, 512, 1024, 2048, 4096])
@pytest.mark.parametrize("name", ["Chi2PDC", "Chi3", "Chi2SFG"])
def test_spread_signal_grids_match_oracle(nlm, oracle, name, n):
    """runSignalSimulation on 128..4096 points: one point per thread on four SMs (eight from 2048
    points), both input domains, against the oracle and against the one-CTA kernels (same arithmetic,
    other transform order)."""
    kw = dict(MEDIA[name], tPrecision=n)
    med, ref, one = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw), getattr(nlm, name)(**kw)
    med._set_cluster(3)                                  # four CTAs to 1024 points, eight above
    one._set_cluster(0)
    for m in (med, one):
        m.runPumpSimulation()
    ref.run_pump_simulation()
    modes = 2 if name == "Chi2SFG" else 1
    a = cases.noise(np.random.default_rng(n + 1), n, 0.2)
    for in_time in (True, False):
        med.runSignalSimulation(a, in_time)
        one.runSignalSimulation(a, in_time)
        ref.run_signal_simulation(a, in_time)
        sched = med._last_schedule()
        ctas = 4 if n <= 1024 else 8
        assert sched["R"] == 1 and sched["grid"] == ctas and sched["block"] == n // ctas
        assert one._last_schedule()["grid"] == 1
        for m in range(modes):
            assert cases.rel_l2(med.signalTimes(m), ref.signal_time[m]) < TOL
            assert cases.rel_l2(med.signalFreqs(m), ref.signal_freq[m]) < TOL
            assert cases.rel_l2(med.signalTimes(m), one.signalTimes(m)) < 1e-12
            assert cases.rel_l2(med.signalFreqs(m), one.signalFreqs(m)) < 1e-12


@pytest.mark.parametrize("n", [128, 256, 512, 4096])
def test_spread_chi3_pump_march(nlm, oracle, n):
    """The self-phase-modulation pump march with one point per thread on four SMs (the default on 128
    to 1024 points) or eight (2048 and 4096 points; 1024 and 2048 are covered by
    test_cluster_chi3_pump_march)."""
    kw = dict(CHI3, tPrecision=n, zPrecision=15)
    med, ref, one = nlm.Chi3(**kw), oracle.Chi3(**kw), nlm.Chi3(**kw)
    one._set_cluster(0)
    for m in (med, one):
        m.runPumpSimulation()
    ref.run_pump_simulation()
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL
    assert cases.rel_l2(med.pumpTime, one.pumpTime) < 1e-12
    assert cases.rel_l2(med.pumpFreq, one.pumpFreq) < 1e-12


def test_spread_config_chi3_n512(nlm, oracle):
    """The Chi3 pump + signal configuration (N=512, nZSteps=200, nZStepsP=399): pump march and signal
    march both on the spread kernels, full grids against the oracle."""
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=512, zPrecision=200)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med.runPumpSimulation()
    ref.run_pump_simulation()
    a = cases.noise(np.random.default_rng(1), 512, 1e-3)
    med.runSignalSimulation(a, True)
    ref.run_signal_simulation(a, True)
    # the pump march and the signal side by side on one cluster of eight CTAs
    assert med._last_schedule()["R"] == 1 and med._last_schedule()["grid"] == 8
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(med.pumpFreq, ref.pump_freq[0]) < TOL
    assert cases.rel_l2(med.signalTime, ref.signal_time[0]) < TOL
    assert cases.rel_l2(med.signalFreq, ref.signal_freq[0]) < TOL


@pytest.mark.parametrize("n,z,in_time", [(512, 200, True), (128, 2, True), (256, 17, False), (1024, 30, True)])
def test_pipelined_chi3_pump_signal(nlm, oracle, n, z, in_time):
    """runPumpSimulation then runSignalSimulation runs both marches on one cluster of eight CTAs (the
    signal one pump step pair behind, with the solver's DiffEq).  Reading the pump grids between the
    calls runs the pump march alone first, and the signal then takes the four-CTA kernel with the RK4
    matrices.  Both orders: the pump grids alike to rounding (the same operations in both kernels; the
    compiler may pair their multiply-adds differently), the signal grids too, all against the oracle;
    from the two-step minimum (one phase) up to 1024 points."""
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=n, zPrecision=z)
    pipe, seq, ref = nlm.Chi3(**kw), nlm.Chi3(**kw), oracle.Chi3(**kw)
    a = cases.noise(np.random.default_rng(n + z), n, 1e-3)
    pipe.runPumpSimulation()
    pipe.runSignalSimulation(a, in_time)
    assert pipe._last_schedule()["grid"] == 8
    seq.runPumpSimulation()
    pump_t = seq.pumpTime                              # runs the march alone
    seq.runSignalSimulation(a, in_time)
    assert seq._last_schedule()["grid"] == (8 if n == 1024 else 4)   # eight CTAs of 128 at 1024 points
    ref.run_pump_simulation()
    ref.run_signal_simulation(a, in_time)
    assert cases.rel_l2(pipe.pumpTime, pump_t) < 1e-13 and cases.rel_l2(pipe.pumpFreq, seq.pumpFreq) < 1e-13
    assert cases.rel_l2(pipe.signalTime, seq.signalTime) < 1e-12
    assert cases.rel_l2(pipe.signalFreq, seq.signalFreq) < 1e-12
    assert cases.rel_l2(pipe.pumpTime, ref.pump_time[0]) < TOL
    assert cases.rel_l2(pipe.signalTime, ref.signal_time[0]) < TOL
    assert cases.rel_l2(pipe.signalFreq, ref.signal_freq[0]) < TOL


def test_deferred_chi3_pump_other_uses(nlm, oracle):
    """A pump march that runPumpSimulation deferred runs before anything else that reads the pump: a
    Green's function without rerunning the pump, a batch, and a second runPumpSimulation in between
    (which replaces the deferred march)."""
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=256, zPrecision=40)
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    ref.run_pump_simulation()
    med.runPumpSimulation()
    med.runPumpSimulation()
    C, S = med.computeGreensFunction(runPump=False)
    Cr, Sr = ref.compute_greens_function(run_pump=False)
    assert cases.rel_l2(C, Cr) < TOL and cases.rel_l2(S, Sr) < TOL
    med.runPumpSimulation()
    x = cases.noise(np.random.default_rng(3), 3 * 256, 1e-3).reshape(3, 256)
    out = med.batchSignalSimulation(x, inTimeDomain=True, runPump=False)
    want = ref.batch_signal_simulation(x, in_time_domain=True, run_pump=False)
    assert cases.rel_l2(out, want) < TOL
    assert cases.rel_l2(med.pumpTime, ref.pump_time[0]) < TOL
