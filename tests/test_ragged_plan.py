"""The ragged-batch makespan planner on the CPU (nlm_ragged_plan: the planner of nlm_ragged_batch with
no device work).  Every plan is checked against its own constraints, restated here: each medium in an
available form that ends within the target, each cluster slot's media of one form and within the
target one after another, the slots within the cluster budget, slots and ragged CTAs within the SMs,
and per ragged-launch class the fewest CTAs whose largest-first schedule ends within the target."""
import math

import numpy as np
import pytest

FORM_SMS = np.array([1, 4, 8, 16])
RTOL = 1e-12


@pytest.fixture(scope="module")
def nlm():
    from multimodenonlinearoptics_gb300 import nonlinearmedium
    return nonlinearmedium


def lpt(times, m):
    """Makespan of the largest-first list schedule of `times` on m machines."""
    load = [0.0] * m
    for t in sorted(times, reverse=True):
        load[load.index(min(load))] += t
    return max(load)


def check_plan(r, forms, cls, cluster_sms, w16_slots, pool_sms, gran):
    T, form, slot, t = r["makespan_us"], r["form"], r["slot"], r["times_us"]
    assert T is not None
    n = len(form)
    for k in range(n):
        f = form[k]
        assert (forms[k] >> f) & 1 and t[k, f] >= 0
        assert t[k, f] <= T * (1 + RTOL)
        assert (slot[k] < 0) == (f == 0)
    used = 0
    w16 = 0
    for s in set(slot[slot >= 0].tolist()):
        members = np.flatnonzero(slot == s)
        fs = set(form[members].tolist())
        assert len(fs) == 1
        f = fs.pop()
        assert t[members, f].sum() <= T * (1 + RTOL)
        used += FORM_SMS[f]
        w16 += f == 3
    assert used <= cluster_sms and w16 <= w16_slots
    ctas = 0
    for c in set(np.asarray(cls)[form == 0].tolist()):
        pool = t[(form == 0) & (np.asarray(cls) == c), 0].tolist()
        m = max(1, math.ceil(sum(pool) / T))
        while m < len(pool) and lpt(pool, m) > T:
            m += 1
        assert lpt(pool, m) <= T * (1 + RTOL)
        ctas += -(-m // gran) * gran
    assert ctas == r["ragged_ctas"]
    assert used + ctas <= pool_sms
    # lower bounds: the longest medium in its fastest form; the SM time over all SMs
    avail = np.where(t >= 0, t, np.inf)
    lo = avail.min(axis=1).max()
    assert T >= lo * (1 - RTOL)
    assert T * pool_sms >= (avail * FORM_SMS).min(axis=1).sum() * (1 - RTOL)
    # the first target that fits on the 0.25 % grid from the bound, or the sum of the one-SM times
    hi = np.where(t[:, 0] >= 0, t[:, 0], avail.min(axis=1)).sum()
    k = math.log(T / lo) / math.log(1.0025)
    assert abs(k - round(k)) < 1e-6 or abs(T - hi) <= RTOL * hi


def test_one_sm_media_known_answer(nlm):
    """Four 128-point two-mode media of 200, 400, 800 and 1600 steps, one SM each: 26.4 us per step
    from the per-step table; the longest (42.24 ms) is the makespan, the other three share a CTA."""
    r = nlm.ragged_plan([128] * 4, [2] * 4, [201, 401, 801, 1601], [0] * 4, [7] * 4, [1] * 4)
    assert r["makespan_us"] == pytest.approx(1600 * 26.4)
    assert r["ragged_ctas"] == 2
    assert (r["form"] == 0).all() and (r["slot"] == -1).all()
    assert r["times_us"][:, 0] == pytest.approx(np.array([200, 400, 800, 1600]) * 26.4)
    assert (r["times_us"][:, 1:] == -1).all()


def test_cluster_forms_by_sm_time(nlm):
    """Within the target, a medium takes the form of least SM time: 1024 points on four SMs (33.8 ms,
    135 SM-ms) rather than eight (25.0 ms, 200 SM-ms); 2048 points on eight (the longest: 43.0 ms)."""
    r = nlm.ragged_plan([512, 2048, 1024], [2] * 3, [2000] * 3, [1] * 3, [7, 9, 10],
                        [0b11, 0b111, 0b111])
    assert r["makespan_us"] == pytest.approx(1999 * 21.5)
    assert list(r["form"]) == [1, 2, 1]
    check_plan(r, [0b11, 0b111, 0b111], [7, 9, 10], 128, 7, 152, 1)


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("gran", [1, 4])
def test_random_sets_satisfy_their_constraints(nlm, seed, gran):
    rng = np.random.default_rng(seed)
    n_media = int(rng.integers(5, 90))
    n = rng.choice([128, 256, 512, 1024, 2048], n_media)
    modes = rng.integers(1, 4, n_media)
    nz = rng.integers(200, 2001, n_media)
    prop = rng.integers(0, 2, n_media)
    solver = rng.integers(0, 3, n_media)
    cls = solver * 64 + np.log2(n).astype(int)
    forms = np.where(n >= 2048, 0b1111, np.where(n == 1024, 0b0111, 0b0011))
    forms = np.where(modes > 2, forms & 0b0111, forms)
    budgets = dict(cluster_sms=int(rng.choice([64, 128, 144])), w16_slots=int(rng.integers(0, 8)), pool_sms=152,
                   pool_granularity=gran)
    r = nlm.ragged_plan(n, modes, nz, prop, cls, forms, **budgets)
    check_plan(r, forms, cls, budgets["cluster_sms"], budgets["w16_slots"], 152, gran)


def test_benchmark_ragged_set(nlm):
    """The 64 Chi2SFG media of the ragged benchmark (workloads.ragged_media_params) with the forms the
    engine gives them in cluster mode 1 and a GB300's budgets (144 SMs for slots, 7 sixteen-SM slots,
    152 SMs): with new pumps (the DiffEq) the plan measured on the GPU (43.9 ms target; 25 media on one
    SM in 22 CTAs, 34 on four-SM slots, 5 on eight); with kept pumps (RK4 matrices) 35.1 ms."""
    from multimodenonlinearoptics_gb300 import workloads
    dims = []
    for kw, doms, pump, _ in workloads.ragged_media_params():
        d = nlm.Chi2SFG(customPump=pump, poling=doms, **kw)._dims
        dims.append((d["nFreqs"], d["nZSteps"], d["nSignalModes"]))
    n, nz, modes = (np.array(v) for v in zip(*dims))
    assert len(n) == 64 and (nz - 1).sum() + 64 == 77165
    cls = 3 * 64 + np.log2(n).astype(int)
    forms = np.where(n >= 2048, 0b1111, np.where(n == 1024, 0b0111, 0b0011))
    new = nlm.ragged_plan(n, modes, nz, [0] * 64, cls, forms, cluster_sms=144, w16_slots=7, pool_sms=152)
    check_plan(new, forms, cls, 144, 7, 152, 1)
    assert new["makespan_us"] / 1e3 == pytest.approx(43.9, abs=0.1)
    assert list(np.bincount(new["form"], minlength=4)) == [25, 34, 5, 0] and new["ragged_ctas"] == 22
    kept = nlm.ragged_plan(n, modes, nz, [1] * 64, cls, forms, cluster_sms=144, w16_slots=7, pool_sms=152)
    check_plan(kept, forms, cls, 144, 7, 152, 1)
    assert kept["makespan_us"] / 1e3 == pytest.approx(35.1, abs=0.1)


def test_no_plan_fits_then_fastest_forms(nlm):
    """Cluster-only media whose slots need more SMs than the budget: no target fits, and each medium
    takes its fastest form in a slot of its own (the slots then queue for SMs)."""
    r = nlm.ragged_plan([2048] * 3 + [128], [2] * 4, [500] * 4, [0] * 4, [11] * 3 + [7], [0b1000] * 3 + [1],
                        cluster_sms=8, w16_slots=7, pool_sms=152)
    assert r["makespan_us"] is None
    assert list(r["form"]) == [3, 3, 3, 0]
    assert sorted(r["slot"][:3].tolist()) == [0, 1, 2] and r["slot"][3] == -1
    assert r["ragged_ctas"] == 4          # one medium, in a group of four


def test_invalid_requests(nlm):
    with pytest.raises(ValueError):
        nlm.ragged_plan([1], [2], [10], [0], [0], [1])            # grid of one point
    with pytest.raises(ValueError):
        nlm.ragged_plan([128], [2], [10], [0], [0], [0])          # no form
    with pytest.raises(ValueError):
        nlm.ragged_plan([512], [2], [10], [0], [0], [0b100])      # eight CTAs at 512 points: not in the table
    with pytest.raises(ValueError):
        nlm.ragged_plan([128], [2], [10], [0], [0], [1], pool_sms=0)
    with pytest.raises(ValueError):
        nlm.ragged_plan([128, 256], [2], [10], [0], [0], [1])     # per-medium arrays of different lengths
