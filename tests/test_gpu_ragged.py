"""One persistent launch over a ragged set of media against the oracle and against one batch per medium."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9


@pytest.mark.parametrize("use_prop", [1, -1, 0])
def test_ragged_launch_matches_oracle(nlm, oracle, use_prop):
    """All media on one SM each (clusters off): one ragged launch per solver and grid.  use_prop 1:
    every (pump-driven) medium's RK4 matrices are built before its launch (one build launch per
    medium); 0: the launches evaluate the DiffEq; -1 (the default): the DiffEq on the first call after a
    pump change, the matrices built on the second and reused from the third."""
    from multimodenonlinearoptics_gb300.workloads import ragged_media_params
    params = ragged_media_params(seed=11, count=6)
    media, refs, ins = [], [], []
    for kw, doms, pump, sig in params:
        kw = dict(kw, zPrecision=max(10, kw["zPrecision"] // 20))   # fewer steps for the oracle
        doms = doms[: max(2, doms.size // 20)]                      # keep domains longer than a step
        m = nlm.Chi2SFG(customPump=pump, poling=doms, **kw)
        r = oracle.Chi2SFG(customPump=pump, poling=doms, **kw)
        m.runPumpSimulation()
        r.run_pump_simulation()
        media.append(m)
        refs.append(r)
        ins.append(sig)
    # a Chi2PDC medium in the same call takes its own launch
    kw = dict(cases.CASES["Chi2PDC"])
    media.append(nlm.Chi2PDC(**kw))
    refs.append(oracle.Chi2PDC(**kw))
    media[-1].runPumpSimulation()
    refs[-1].run_pump_simulation()
    ins.append(cases.signal_input("Chi2PDC", 64, 1, seed=3))
    for m in media:
        m._set_schedule(use_propagator=use_prop)
        m._set_cluster(0)                                   # every medium in the ragged launch
    outs = nlm.ragged_batch(media, ins)
    # one ragged launch per solver and grid in the set (plus the propagator builds)
    classes = len({(type(m).__name__, m._dims["nFreqs"]) for m in media})
    assert sum(m._launch_count() for m in media) == classes + (len(media) if use_prop == 1 else 0)
    if use_prop == -1:
        again = nlm.ragged_batch(media, ins)
        assert sum(m._launch_count() for m in media) == classes + len(media)
        third = nlm.ragged_batch(media, ins)
        assert sum(m._launch_count() for m in media) == classes
        for o, o2, o3 in zip(outs, again, third):
            assert cases.rel_l2(o2, o) < 1e-13 and np.array_equal(o3, o2)
    for m, r, x, o in zip(media, refs, ins, outs):
        f, _ = r.propagate(x[None, :], False, 0)
        assert cases.rel_l2(o, f[0]) < TOL
        b = m.batchSignalSimulation(x[None, :], runPump=False)
        assert cases.rel_l2(o.reshape(1, -1), b) < 1e-13
    outs_t = nlm.ragged_batch(media[:3], ins[:3], True)
    for m, r, x, o in zip(media[:3], refs[:3], ins[:3], outs_t):
        _, t = r.propagate(x[None, :], True, 0)
        assert cases.rel_l2(o, t[0]) < TOL


def _sfg_set(nlm, oracle, shapes, seed=21):
    kw0 = dict(relativeLength=1, nlLength=1, nlLengthOrig=1, beta2=0.4, beta2s=-0.3, beta2o=0, beta1=0, beta1s=1.2,
               beta1o=0, beta3=0, beta3s=0.05, beta3o=0, diffBeta0=0, tMax=10)
    rng = np.random.default_rng(seed)
    media, refs, ins = [], [], []
    for n, zp in shapes:
        kw = dict(kw0, tPrecision=n, zPrecision=zp)
        t = np.fft.fftshift(np.linspace(-10, 10, n, endpoint=False))
        pump = np.exp(-t ** 2 / 2)
        m = nlm.Chi2SFG(customPump=pump, poling=[3, 4, 3], **kw)
        r = oracle.Chi2SFG(customPump=pump, poling=[3, 4, 3], **kw)
        m.runPumpSimulation()
        r.run_pump_simulation()
        media.append(m)
        refs.append(r)
        ins.append(cases.noise(rng, n, 1e-2))
    return media, refs, ins


def test_ragged_set_with_cluster_propagations(nlm, oracle):
    """The planner gives the longest march its fastest form (the 2048-point medium: one point per
    thread on sixteen CTAs, or eight where sixteen-CTA clusters do not fit) and every other medium the
    form of least SM time that finishes within the makespan; every output matches the oracle."""
    media, refs, ins = _sfg_set(nlm, oracle, ((2048, 14), (1024, 12), (256, 10), (128, 8), (1024, 6)))
    outs = nlm.ragged_batch(media, ins)
    plan = nlm.ragged_last_plan()
    assert plan["slots_w8"] + plan["slots_w16"] >= 1 and plan["makespan_estimate_ms"] > 0
    s = media[0]._last_schedule()
    assert s["grid"] in (8, 16) and s["R"] == 1 and s["block"] == 2048 // s["grid"]
    assert (s["grid"] == 16) == (plan["slots_w16"] >= 1)
    for r, x, o in zip(refs, ins, outs):
        f, _ = r.propagate(x[None, :], False, 0)
        assert cases.rel_l2(o, f[0]) < TOL


def test_ragged_call_replays_its_graph(nlm, oracle):
    """The whole call (input copy, cluster slots, ragged launch, output copy) is captured once its plan
    repeats and then replayed: the same outputs bit for bit, and a new pump is seen by the replay."""
    media, refs, ins = _sfg_set(nlm, oracle, ((2048, 10), (1024, 8), (512, 9), (256, 6), (128, 7), (128, 5)), seed=5)
    for m in media:
        m._set_schedule(use_propagator=0)   # the DiffEq in every call: one plan throughout
    first = nlm.ragged_batch(media, ins)
    before = nlm.ragged_last_plan()
    again = [nlm.ragged_batch(media, ins) for _ in range(3)]
    after = nlm.ragged_last_plan()
    assert after["graph_captures"] >= before["graph_captures"] + 1
    assert after["graph_replays"] >= before["graph_replays"] + 2
    for outs in again:
        for o, o1 in zip(outs, first):
            assert np.array_equal(o, o1)
    for r, x, o in zip(refs, ins, first):
        f, _ = r.propagate(x[None, :], False, 0)
        assert cases.rel_l2(o, f[0]) < TOL
    # a new pump (same buffers) is read by the replayed graph
    t = np.fft.fftshift(np.linspace(-10, 10, 1024, endpoint=False))
    media[1].setPump(np.exp(-t ** 2 / 3) + 0j)
    refs[1].set_pump_custom(np.exp(-t ** 2 / 3) + 0j)
    media[1].runPumpSimulation()
    refs[1].run_pump_simulation()
    outs = nlm.ragged_batch(media, ins)
    f, _ = refs[1].propagate(ins[1][None, :], False, 0)
    assert cases.rel_l2(outs[1], f[0]) < TOL
    assert nlm.ragged_last_plan()["graph_replays"] > after["graph_replays"]
