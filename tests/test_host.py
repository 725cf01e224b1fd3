"""Host-side logic of the engine (set-up, validation, errors) against the oracle; no GPU needed."""
import numpy as np
import pytest

import cases


@pytest.mark.parametrize("name", list(cases.CASES))
def test_setup_matches_oracle(nlm, oracle, name):
    kw = cases.CASES[name]
    med = getattr(nlm, name)(**kw)
    ref = oracle.SOLVERS[name](**cases.oracle_kwargs(name))
    d = med._dims
    assert d["nFreqs"] == ref.n_freqs
    assert d["nZSteps"] == ref.n_z_steps
    assert d["nSignalModes"] == ref.n_signal_modes
    assert np.array_equal(med.tau, ref.tau)
    assert np.array_equal(med.omega, ref.omega)
    assert np.array_equal(med.poling, ref.poling)
    ln = med._lengths
    assert ln["dz"] == ref.dz
    if not ref.fully_nonlinear:
        assert d["nZStepsP"] == ref.n_z_steps_p
        assert ln["dzp"] == ref.dzp


def test_green_benchmark_configuration_sizes(nlm):
    """Chi2PDC at nFreqs=1024: minLen 0.5 gives nZSteps = 1000 (src/_NonlinearMedium.cpp:87-91)."""
    m = nlm.Chi2PDC(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
                    beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, zPrecision=500, poling=np.ones(100))
    assert m._dims["nZSteps"] == 1000 and m._dims["nZStepsP"] == 1999
    pol = m.poling
    assert pol.size == 1000 and set(np.unique(pol)) <= {-1.0, 1.0}


def test_validation_errors(nlm):
    with pytest.raises(ValueError, match="Invalid number of Frequencies"):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, tPrecision=1023)
    with pytest.raises(ValueError, match="No unit length scale"):
        nlm.Chi2PDC(2, 0.5, 2, 0.5)
    with pytest.raises(ValueError, match="Non-positive length scale"):
        nlm.Chi2PDC(1, -0.5, 1, 0.5)
    with pytest.raises(ValueError, match="Negative time span"):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, tMax=-1)
    with pytest.raises(ValueError, match="Zero steps"):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, zPrecision=0)
    with pytest.raises(ValueError, match="invalid domain length"):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, poling=[1, -1, 2])
    with pytest.raises(ValueError, match="Custom pump array length"):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, customPump=np.ones(7))
    with pytest.raises(TypeError):
        nlm.Chi2PDC(1, 0.5)
    with pytest.raises(TypeError):
        nlm.Chi2PDC(1, 0.5, 1, 0.5, notAnArgument=3)


def test_precision_switch_validation(nlm):
    m = nlm.Chi2PDC(**cases.CASES["Chi2PDC"])
    m._set_precision("ff")
    m._set_precision("f64")
    with pytest.raises(ValueError):
        m._set_precision("f16")
    assert nlm._lib.nlm_set_precision(m._h(), 2) == 1   # NLM_ERR_INVALID_ARGUMENT


def test_method_validation_before_any_device_work(nlm):
    m = nlm.Chi2SFG(**cases.CASES["Chi2SFG"])
    n = m._dims["nFreqs"]
    with pytest.raises(ValueError, match="inputProf array size"):
        m.runSignalSimulation(np.ones(n + 1))
    with pytest.raises(ValueError, match="inputProf array size"):
        m.runSignalSimulation(np.ones(3 * n))
    with pytest.raises(ValueError, match="inputModes does not match"):
        m.runSignalSimulation(np.ones(n), inputMode=2)
    with pytest.raises(ValueError, match="Signals not of correct length"):
        m.batchSignalSimulation(np.ones((2, n + 2)))
    with pytest.raises(ValueError, match="Too many threads"):
        m.batchSignalSimulation(np.ones((2, n)), nThreads=3)
    with pytest.raises(ValueError, match="Too many threads"):
        m.batchSignalSimulation(np.zeros((0, n)))
    with pytest.raises(ValueError, match="Requested no outputs"):
        m.batchSignalSimulation(np.ones((2, n)), useOutput=[0, 0])
    with pytest.raises(ValueError, match="longer than number of modes"):
        m.computeGreensFunction(useInput=[1, 1, 1])
    with pytest.raises(ValueError, match="Too many threads"):
        m.computeGreensFunction(nThreads=2 * n + 1)
    with pytest.raises(ValueError, match="Invalid pump index"):
        m.setPump(0, pumpIndex=1)


def test_single_mode_use_input_follows_reference_count_rule(nlm):
    """For a one-mode solver the reference counts entries < nModes: [1] selects nothing (ValueError)."""
    m = nlm.Chi2PDC(**cases.CASES["Chi2PDC"])
    with pytest.raises(ValueError, match="Requested no valid inputs"):
        m.computeGreensFunction(useInput=[1])


def test_fully_nonlinear_disabled_methods(nlm):
    m = nlm.Chi2SHG(**cases.CASES["Chi2SHG"])
    for call in (lambda: m.runPumpSimulation(), lambda: m.computeGreensFunction(), lambda: m.setPump(0),
                 lambda: m.setPump(np.ones(32))):
        with pytest.raises(RuntimeError, match="Object does not have this method"):
            call()
    with pytest.raises(IndexError):
        m.pumpTime


def test_envelopes_match_oracle(nlm, oracle):
    for pt in (0, 1, 2):
        m = nlm.Chi2PDC(1, 0.5, 1, 0.5, pulseType=pt, tPrecision=64)
        o = oracle.Chi2PDC(1, 0.5, 1, 0.5, pulseType=pt, tPrecision=64)
        env = m._axis(4, 0, complex_=True)
        # libm and numpy may differ in the last bit of exp/cosh/sin (Eigen's own vectorised exp in
        # the reference differs from both at that level too)
        assert cases.rel_l2(env, o.envelope[0]) < 1e-15
    m = nlm.Chi2SFGOPA(**cases.CASES["Chi2SFGOPA"])
    assert np.all(m._axis(4, 1, complex_=True) == 0)


def test_cascade_construction_errors(nlm):
    a = nlm.Chi2PDC(1, 0.5, 1, 0.5, tPrecision=64)
    b = nlm.Chi2PDC(1, 0.5, 1, 0.5, tPrecision=32)
    c = nlm.Chi2SFG(**dict(cases.CASES["Chi2SFG"], tPrecision=64))
    with pytest.raises(ValueError, match="at least one medium"):
        nlm.Cascade([], [], True)
    with pytest.raises(ValueError, match="same time and frequency axes"):
        nlm.Cascade([a, b], [{0: 0}], True)
    with pytest.raises(ValueError, match="one connection per pair"):
        nlm.Cascade([a, a], [], True)
    with pytest.raises(ValueError, match="Connections missing"):
        nlm.Cascade([a, a], [{}], True)
    with pytest.raises(ValueError, match="out of range"):
        nlm.Cascade([a, c], [{0: 1}], True)
    casc = nlm.Cascade([a, c], [{1: 0}], False)
    assert casc.nMedia == 2 and casc[1] is c
    with pytest.raises(ValueError, match="No connection"):
        casc.addMedium(a, {})
    with pytest.raises(RuntimeError):
        casc.setPump(a)
    assert np.array_equal(casc.tau, a.tau)


def test_gpu_methods_fail_loudly_without_device(nlm):
    if nlm.device_available():
        pytest.skip("a device is present")
    m = nlm.Chi2PDC(**cases.CASES["Chi2PDC"])
    with pytest.raises(nlm.NoDeviceError):
        m.runPumpSimulation()
    with pytest.raises(nlm.NoDeviceError):
        m.computeGreensFunction()
