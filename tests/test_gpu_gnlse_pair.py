"""Chi3GNLSE batches of more rows than SMs run two rows per thread group, with the two rows' Raman
convolutions as one complex convolution (k_propagate_gnlse_pair, k_adjoint_gnlse_pair).  Against
the oracle, against the one-row kernels on the same rows, with an odd row count, and under the
adjoint."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
TOL = 1e-9


def _rows(n, rows, seed):
    t = np.fft.fftshift(np.linspace(-10, 10, n, endpoint=False))
    rng = np.random.default_rng(seed)
    base = 2.0 / np.cosh(t)
    return np.fft.fft(base[None, :] + cases.noise(rng, rows * n, 0.05).reshape(rows, n), axis=1)


@pytest.mark.parametrize("rows", [153, 320, 321])
def test_paired_rows_match_oracle_and_one_row_kernel(nlm, oracle, rows):
    kw = dict(cases.CASES["Chi3GNLSE"])
    med, ref = nlm.Chi3GNLSE(**kw), oracle.Chi3GNLSE(**kw)
    n = med._dims["nFreqs"]
    x = _rows(n, rows, rows)
    out = med.batchSignalSimulation(x, inTimeDomain=False)
    sched = med._last_schedule()
    assert sched["grid"] <= (rows + 1) // 2      # thread groups hold pairs of rows
    assert cases.rel_l2(out, ref.batch_signal_simulation(x, False)) < TOL
    # the same rows through the one-row kernel (fewer rows than SMs per launch)
    single = np.concatenate([med.batchSignalSimulation(x[k:k + 100], inTimeDomain=False)
                             for k in range(0, rows, 100)])
    assert cases.rel_l2(out, single) < 1e-12
    assert not np.array_equal(out, single)        # two kernels (the Raman result is taken real)
    # each row on its own: the unpaired last row of an odd count is computed like the others
    assert cases.rel_l2(out[-1], single[-1]) < 1e-12
    # time-domain inputs and outputs
    xt = np.fft.ifft(x, axis=1)
    out_t = med.batchSignalSimulation(xt, inTimeDomain=True)
    assert cases.rel_l2(out_t, ref.batch_signal_simulation(xt, True)) < TOL


def test_paired_forward_under_the_adjoint(nlm):
    """320 rows: the adjoint's checkpointed forward runs paired; the gradients of the first rows equal
    those of a 3-row problem (the loss is a sum over rows)."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    kw = dict(cases.CASES["Chi3GNLSE"])
    n = nlm.Chi3GNLSE(**kw)._dims["nFreqs"]
    x = _rows(n, 320, 5)
    weights = torch.linspace(0, 1, n, device="cuda", dtype=torch.float64)
    grads = {}
    for rows in (3, 320):
        for k in (1, 4):
            med = nlm.Chi3GNLSE(**kw)
            xt = torch.tensor(x[:rows], device="cuda", requires_grad=True)
            out = propagate_gnlse(med, xt, k)
            torch.sum(torch.abs(out) ** 2 * weights).backward()
            grads[rows, k] = xt.grad.cpu().numpy()
    for key in ((3, 4), (320, 1), (320, 4)):
        assert cases.rel_l2(grads[key][:3], grads[3, 1]) < 1e-11


@pytest.mark.parametrize("k", [1, 4])
def test_paired_reverse_sweep(nlm, k):
    """320 rows: the reverse sweep also runs two rows per thread group (shared Raman transforms in the
    stage recomputation and in the Raman adjoint); its gradients equal those of 100-row sweeps (one row
    per thread group) on the same rows, to rounding."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    kw = dict(cases.CASES["Chi3GNLSE"])
    n = nlm.Chi3GNLSE(**kw)._dims["nFreqs"]
    x = _rows(n, 320, 9)
    weights = torch.linspace(0, 1, n, device="cuda", dtype=torch.float64)

    def grad(rows_x):
        med = nlm.Chi3GNLSE(**kw)
        xt = torch.tensor(rows_x, device="cuda", requires_grad=True)
        torch.sum(torch.abs(propagate_gnlse(med, xt, k)) ** 2 * weights).backward()
        return xt.grad.cpu().numpy()

    paired = grad(x)
    single = np.concatenate([grad(x[q:q + 100]) for q in range(0, 320, 100)])
    assert cases.rel_l2(paired, single) < 1e-11
    assert not np.array_equal(paired, single)


def test_pair_waves_then_single_rows(nlm, oracle):
    """400 rows of 4096 points on 152 SMs: 152 pairs fill one wave of the paired kernel, and the 96
    rows left over run one per thread group in one wave of the single-row kernel (instead of a second,
    part-empty pair wave).  Against the oracle; the tail rows equal the single-row kernel's bit for bit."""
    from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG, gnlse_rows
    kw = dict(GNLSE_CONFIG, relativeLength=0.002)
    med, ref = nlm.Chi3GNLSE(**kw), oracle.Chi3GNLSE(**kw)
    torch = pytest.importorskip("torch")
    if torch.cuda.get_device_properties(0).multi_processor_count != 152:
        pytest.skip("the wave arithmetic below is for 4096 points on 152 SMs")
    x = gnlse_rows(400, seed=8)
    med.batchSignalSimulation(x[:1], inTimeDomain=True)             # device tables (the Raman transform)
    out = med.batchSignalSimulation(x, inTimeDomain=True)
    assert med._launch_count() == 2                                 # the pair wave and the single-row wave
    assert cases.rel_l2(out, ref.batch_signal_simulation(x, True)) < TOL
    tail = med.batchSignalSimulation(x[304:], inTimeDomain=True)   # fewer rows than SMs: one-row kernel
    assert np.array_equal(out[304:], tail)


@pytest.mark.parametrize("k", [1, 4])
def test_reverse_sweep_waves_then_single_rows(nlm, k):
    """400 rows of 4096 points: the reverse sweep too runs one wave of pairs and the 96 rows left over
    one per thread group; the gradients equal those of 100-row sweeps on the same rows, to rounding."""
    torch = pytest.importorskip("torch")
    if torch.cuda.get_device_properties(0).multi_processor_count != 152:
        pytest.skip("the wave arithmetic below is for 4096 points on 152 SMs")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG, gnlse_rows
    kw = dict(GNLSE_CONFIG, relativeLength=0.002)
    x = np.fft.fft(gnlse_rows(400, seed=12), axis=1)
    n = x.shape[1]
    weights = torch.linspace(0, 1, n, device="cuda", dtype=torch.float64)

    def grad(rows_x):
        med = nlm.Chi3GNLSE(**kw)
        xt = torch.tensor(rows_x, device="cuda", requires_grad=True)
        torch.sum(torch.abs(propagate_gnlse(med, xt, k)) ** 2 * weights).backward()
        return xt.grad.cpu().numpy()

    waves = grad(x)
    chunks = np.concatenate([grad(x[q:q + 100]) for q in range(0, 400, 100)])
    assert np.all(np.isfinite(waves))
    assert cases.rel_l2(waves, chunks) < 1e-11
    assert cases.rel_l2(waves[304:], chunks[304:]) < 1e-11
