"""The schedule autotuner: it picks a launch shape by timing, caches it for the process, and the
shape it picks does not change the numbers."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

KW = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
          beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, zPrecision=20, poling=np.ones(4))


def test_tuned_schedule_gives_the_analytic_result(nlm):
    """A batch of 337 rows (a shape no other test uses, so this process has not tuned it yet)."""
    rng = np.random.default_rng(17)
    x = cases.noise(rng, 337 * 1024, 0.1).reshape(337, 1024)
    fixed = nlm.Chi2PDC(**KW)
    fixed._set_schedule(cta_per_sm=-1)
    ref = fixed.batchSignalSimulation(x)
    s0 = fixed._last_schedule()
    assert s0["tuned"] == 0 and s0["trials"] == 0
    med = nlm.Chi2PDC(**KW)
    out = med.batchSignalSimulation(x)
    s1 = med._last_schedule()
    assert s1["tuned"] == 1 and s1["trials"] > 0 and s1["R"] in (8, 16)
    assert s1["block"] == (1024 // s1["R"]) * s1["ipc"]
    assert cases.rel_l2(out, ref) < 1e-13
    # the choice is cached for the process: a second medium of the same shape runs no trial
    again = nlm.Chi2PDC(**KW)
    out2 = again.batchSignalSimulation(x)
    s2 = again._last_schedule()
    assert s2["tuned"] == 1 and s2["trials"] == 0
    assert {k: s2[k] for k in ("R", "ipc", "grid", "block")} == {k: s1[k] for k in ("R", "ipc", "grid", "block")}
    assert np.array_equal(out2, out)


def test_tuned_green_matches_oracle(nlm, oracle):
    med = nlm.Chi2PDC(**KW)
    C, S = med.computeGreensFunction()
    assert med._last_schedule()["tuned"] == 1
    Cr, Sr = oracle.Chi2PDC(**KW).compute_greens_function(chunk=512)
    assert cases.rel_l2(C, Cr) < 1e-9 and cases.rel_l2(S, Sr) < 1e-9


def test_forced_schedule_is_respected(nlm):
    med = nlm.Chi2PDC(**KW)
    med._set_schedule(cta_per_sm=1)
    C, S = med.computeGreensFunction()
    s = med._last_schedule()
    assert s["tuned"] == 0 and s["cta_per_sm"] == 1
    ref = nlm.Chi2PDC(**KW)
    ref._set_schedule(cta_per_sm=-1)
    C0, S0 = ref.computeGreensFunction()
    assert cases.rel_l2_pair(C, S, C0, S0) < 1e-13


def test_small_batches_are_not_tuned(nlm):
    med = nlm.Chi2PDC(**cases.CASES["Chi2PDC"])
    med.runPumpSimulation()
    n = med._dims["nFreqs"]
    med.batchSignalSimulation(np.ones((3, n)), runPump=False)
    assert med._last_schedule()["tuned"] == 0
