"""Batched propagations captured into CUDA graphs: a repeated call replays its graph and gives the
same numbers as direct launches; a change of arguments captures a new graph."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def test_green_replays_its_graph(nlm):
    kw = dict(cases.CASES["Chi2PDC"])
    med = nlm.Chi2PDC(**kw)
    direct = nlm.Chi2PDC(**kw)
    direct._set_schedule(use_graph=0)
    C0, S0 = direct.computeGreensFunction()
    assert direct._graph_stats() == (0, 0)
    C1, S1 = med.computeGreensFunction()
    assert med._graph_stats() == (1, 0)
    C2, S2 = med.computeGreensFunction()
    assert med._graph_stats() == (1, 1)
    for c, s in ((C1, S1), (C2, S2)):
        assert np.array_equal(c, C0) and np.array_equal(s, S0)
    # other arguments: a second graph; alternating calls replay both
    Ct0, St0 = direct.computeGreensFunction(True)
    Ct, St = med.computeGreensFunction(True)
    assert med._graph_stats() == (2, 1)
    med.computeGreensFunction()
    Ct2, St2 = med.computeGreensFunction(True)
    assert med._graph_stats() == (2, 3)
    assert np.array_equal(Ct, Ct0) and np.array_equal(Ct2, Ct0) and np.array_equal(St2, St0)


def test_green_replay_sees_new_pump(nlm, oracle):
    """The pump and the propagator are rebuilt before the replayed launch, which reads them."""
    kw = dict(cases.CASES["Chi2PDC"])
    med, ref = nlm.Chi2PDC(**kw), oracle.Chi2PDC(**kw)
    med.computeGreensFunction()
    tau = ref.tau
    for width in (1.5, 0.7):
        med.setPump(np.exp(-tau ** 2 / width))
        ref.set_pump_custom(np.exp(-tau ** 2 / width))
        C, S = med.computeGreensFunction()
        Cr, Sr = ref.compute_greens_function()
        assert cases.rel_l2_pair(C, S, Cr, Sr) < 1e-9
    assert med._graph_stats()[1] >= 2


@pytest.mark.parametrize("name", ["Chi2SFG", "Chi3GNLSE"])
def test_batch_replay_reads_new_inputs(nlm, oracle, name):
    kw = dict(cases.CASES[name])
    med, ref = getattr(nlm, name)(**kw), getattr(oracle, name)(**kw)
    if name != "Chi3GNLSE":
        med.runPumpSimulation()
    n = med._dims["nFreqs"]
    rng = np.random.default_rng(21)
    for _ in range(3):
        x = cases.noise(rng, 5 * n, 0.5).reshape(5, n)
        out = med.batchSignalSimulation(x, inTimeDomain=False)
        assert cases.rel_l2(out, ref.batch_signal_simulation(x, False)) < 1e-9
    captures, replays = med._graph_stats()
    assert captures == 1 and replays == 2
