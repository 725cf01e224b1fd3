"""Double-float kernel (pairs of FP32 values on the FP32 units) of the single-mode propagator path,
against the oracle, the golden fixtures and the FP64 kernel."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9

BENCH_KW = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
                beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, poling=np.ones(4))


def _pair(nlm, name, kw, fn):
    """fn(medium) with FP64 and with double-float arithmetic on two fresh media."""
    a = getattr(nlm, name)(**kw)
    b = getattr(nlm, name)(**kw)
    b._set_precision("ff")
    return fn(a), fn(b)


@pytest.mark.parametrize("name", ["Chi3", "Chi2PDC"])
def test_ff_green_matches_golden(nlm, golden, name):
    med = getattr(nlm, name)(**cases.CASES[name])
    med._set_precision("ff")
    med.runPumpSimulation()
    C, S = med.computeGreensFunction(False, False)
    assert cases.rel_l2_pair(C, S, golden[name + "__green_c"], golden[name + "__green_s"]) < TOL
    Ct, St = med.computeGreensFunction(True, False)
    assert cases.rel_l2_pair(Ct, St, golden[name + "__green_c_time"], golden[name + "__green_s_time"]) < TOL


def test_ff_green_benchmark_medium_matches_oracle(nlm, oracle):
    kw = dict(BENCH_KW, zPrecision=20)
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    med._set_precision("ff")
    assert med._dims["nZSteps"] == 40
    C, S = med.computeGreensFunction()
    Cr, Sr = ref.compute_greens_function(chunk=512)
    assert cases.rel_l2(C, Cr) < TOL and cases.rel_l2(S, Sr) < TOL


def test_ff_green_full_size_against_fp64(nlm):
    """N=1024, nZSteps=1000 (the benchmark medium): the two arithmetics agree to far below 1e-9
    (measured ~1e-11), and they are different computations (not bit-identical)."""
    kw = dict(BENCH_KW, zPrecision=500, poling=np.ones(100))
    (C64, S64), (Cff, Sff) = _pair(nlm, "Chi2PDC", kw, lambda m: m.computeGreensFunction())
    assert cases.rel_l2(Cff, C64) < 1e-10 and cases.rel_l2(Sff, S64) < 1e-10
    assert not np.array_equal(Cff, C64)


@pytest.mark.parametrize("n", [128, 256, 2048, 4096])
def test_ff_grid_sizes_against_fp64(nlm, n):
    """Several propagations per CTA (small grids) and the largest grid of the R=8 kernel."""
    kw = dict(BENCH_KW, tPrecision=n, zPrecision=30)
    (C64, S64), (Cff, Sff) = _pair(nlm, "Chi2PDC", kw, lambda m: m.computeGreensFunction(True))
    assert cases.rel_l2_pair(Cff, Sff, C64, S64) < 1e-11


@pytest.mark.parametrize("in_time", [False, True])
def test_ff_batch_matches_oracle(nlm, oracle, in_time):
    kw = dict(cases.CASES["Chi3"])
    med, ref = nlm.Chi3(**kw), oracle.Chi3(**kw)
    med._set_precision("ff")
    med._set_schedule(use_propagator=1)
    n = med._dims["nFreqs"]
    rng = np.random.default_rng(12)
    x = cases.noise(rng, 6 * n, 1.0).reshape(6, n)
    out = med.batchSignalSimulation(x, in_time, True)
    assert cases.rel_l2(out, ref.batch_signal_simulation(x, in_time, True)) < TOL


def test_ff_switch_back_is_fp64(nlm):
    """After switching back, the FP64 kernel runs again (bit-identical to a medium never switched),
    and a pump change rebuilds the double-float propagator."""
    kw = dict(cases.CASES["Chi2PDC"])
    ref = nlm.Chi2PDC(**kw)
    C0, S0 = ref.computeGreensFunction()
    med = nlm.Chi2PDC(**kw)
    med._set_precision("ff")
    Cf, _ = med.computeGreensFunction()
    med._set_precision("f64")
    C1, S1 = med.computeGreensFunction()
    assert np.array_equal(C1, C0) and np.array_equal(S1, S0)
    assert not np.array_equal(Cf, C0)
    tau = med.tau
    med._set_precision("ff")
    med.setPump(np.exp(-tau ** 2 / 1.5))
    ref.setPump(np.exp(-tau ** 2 / 1.5))
    C2, S2 = med.computeGreensFunction()
    C3, S3 = ref.computeGreensFunction()
    assert cases.rel_l2_pair(C2, S2, C3, S3) < 1e-12
