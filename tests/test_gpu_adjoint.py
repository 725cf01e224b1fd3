"""Gradients of the reverse sweep (Chi2PDC) against central finite differences of the engine's own
forward and of the oracle's forward (the reference's algorithm with its poling array replaced by a
continuous profile)."""
import os

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

KW = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
          beta3s=0.1, diffBeta0=0.3, tMax=20, tPrecision=64, zPrecision=20)


def _problem(n, nz, rows, seed=4):
    rng = np.random.default_rng(seed)
    x = cases.noise(rng, rows * n, 0.3).reshape(rows, n)
    t = np.fft.fftshift(np.linspace(-KW["tMax"], KW["tMax"], n, endpoint=False))
    f0 = np.fft.fft(np.exp(-t ** 2 / 2)) * (1 + 0.05 * cases.noise(rng, n, 1.0))
    d = rng.uniform(-1, 1, nz)
    target = cases.noise(rng, rows * n, 1.0).reshape(rows, n)
    target /= np.linalg.norm(target)
    return x, f0, d, target


def _oracle_out(oracle, kw, x, f0, d):
    m = oracle.Chi2PDC(**kw)
    m.set_pump_custom(np.fft.ifft(f0))
    m.poling = np.asarray(d, dtype=np.float64)        # continuous profile in place of the domains
    m.run_pump_simulation()
    f, _ = m.propagate(x, False, 0)
    return f[:, 0]


def _loss(out, target):
    """||out - target||^2 without its constant ||target||^2 (same gradient): keeps the value at the
    scale of the field so the finite-difference round-off (~1e-16 |L| / h) stays below the gradients."""
    out = np.asarray(out)
    return float(np.sum(np.abs(out) ** 2) - 2 * np.real(np.vdot(target, out)))


def _engine_grads(nlm, kw, x, f0, d, target, interval=0, cluster=1):
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_pdc
    med = nlm.Chi2PDC(**kw)
    med._set_cluster(cluster)
    xt = torch.tensor(x, dtype=torch.complex128, device="cuda", requires_grad=True)
    ft = torch.tensor(f0, dtype=torch.complex128, device="cuda", requires_grad=True)
    dt = torch.tensor(d, dtype=torch.float64, requires_grad=True)
    tt = torch.tensor(target, dtype=torch.complex128, device="cuda")
    out = propagate_pdc(med, xt, ft, dt, interval)
    loss = torch.sum(torch.abs(out - tt) ** 2)
    loss.backward()
    return (out.detach().cpu().numpy(), xt.grad.cpu().numpy(), ft.grad.cpu().numpy(), dt.grad.numpy(), med)


def _fd(fun, base, idx, h, complex_part=None, relative=False):
    if relative:   # step relative to the parameter's magnitude
        h = h * max(1.0, abs(base.flat[idx]))
    p, m = base.copy(), base.copy()
    if complex_part == "im":
        p.flat[idx] += 1j * h
        m.flat[idx] -= 1j * h
    else:
        p.flat[idx] += h
        m.flat[idx] -= h
    return (fun(p) - fun(m)) / (2 * h)


def _significant(g, count, rng):
    """Indices of the largest components and of random ones above 5% of the largest: components far
    below the loss scale are dominated by the finite-difference round-off (~1e-16 L / h)."""
    mag = np.abs(g).ravel()
    top = list(np.argsort(mag)[::-1][:count])
    big = np.flatnonzero(mag >= 0.05 * mag.max())
    extra = list(rng.choice(big, min(count, big.size), replace=False))
    return sorted(set(top + extra))


def _rel_vec(adj, fd):
    adj, fd = np.asarray(adj), np.asarray(fd)
    return float(np.linalg.norm(adj - fd) / np.linalg.norm(fd))


def test_adjoint_matches_finite_differences_of_oracle_and_engine(nlm, oracle):
    kw = dict(KW)
    n = 64
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    x, f0, d, target = _problem(n, nz, rows=2)
    out, gx, gf, gd, med = _engine_grads(nlm, kw, x, f0, d, target)
    ref = _oracle_out(oracle, kw, x, f0, d)
    assert cases.rel_l2(out, ref) < 1e-9
    h = 1e-6
    rng = np.random.default_rng(0)

    def loss_x(v):
        return _loss(_oracle_out(oracle, kw, v, f0, d), target)

    def loss_f(v):
        return _loss(_oracle_out(oracle, kw, x, v, d), target)

    def loss_d(v):
        return _loss(_oracle_out(oracle, kw, x, f0, v), target)

    ga, gfd = [], []
    for idx in _significant(gx, 3, rng):
        ga += [gx.flat[idx].real, gx.flat[idx].imag]
        gfd += [_fd(loss_x, x, idx, h), _fd(loss_x, x, idx, h, "im")]
    assert _rel_vec(ga, gfd) < 1e-6
    ga, gfd = [], []
    for idx in _significant(gf, 3, rng):
        ga += [gf[idx].real, gf[idx].imag]
        gfd += [_fd(loss_f, f0, idx, h), _fd(loss_f, f0, idx, h, "im")]
    assert _rel_vec(ga, gfd) < 1e-6
    idx_d = _significant(gd, 4, rng)
    assert _rel_vec(gd[idx_d], [_fd(loss_d, d, i, h) for i in idx_d]) < 1e-6

    # central differences of the engine's own forward
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_pdc

    def eng_loss_d(v):
        o = propagate_pdc(med, torch.tensor(x, device="cuda"), torch.tensor(f0, device="cuda"),
                          torch.tensor(v), 0).cpu().numpy()
        return _loss(o, target)

    idx_d = _significant(gd, 3, rng)
    assert _rel_vec(gd[idx_d], [_fd(eng_loss_d, d, i, h) for i in idx_d]) < 1e-6


def test_checkpointed_sweep_equals_stored_states(nlm):
    kw = dict(KW)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    x, f0, d, target = _problem(64, nz, rows=3, seed=9)
    a = _engine_grads(nlm, kw, x, f0, d, target, interval=1)
    b = _engine_grads(nlm, kw, x, f0, d, target, interval=7)
    for ga, gb in zip(a[1:4], b[1:4]):
        assert cases.rel_l2(gb, ga) < 1e-12


def _dir_fd(fun, base, direction, h):
    """Central difference of fun along `direction` (fun(base + h direction) - fun(base - h direction)) / 2h."""
    return (fun(base + h * direction) - fun(base - h * direction)) / (2 * h)


def test_adjoint_config_size(nlm, oracle):
    """The gradient configuration: N=512, nZSteps=2000, one noise signal (1e-3), d(z) ~ U[-1, 1].

    The loss is ~1e-3 and single gradient components reach down to 1e-9, so componentwise finite
    differences at this size resolve only ~1e-4 (the forward's own round-off over 2000 steps, a few
    1e-13 of the loss, divided by the step).  The check therefore uses directional derivatives along
    random directions, which sum all components: Re<g, v> against the central difference of the oracle's
    forward along v.  Steps of 1e-4 to 1e-3 (relative) agree with each other to a few 1e-8 for the
    pump and poling directions; the loss is exactly quadratic in the input, so any step is exact there."""
    kw = dict(KW, tMax=40, tPrecision=512, zPrecision=1000, diffBeta0=0)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    assert nz == 2000
    rng = np.random.default_rng(4)
    x = cases.noise(rng, 512, 1e-3).reshape(1, 512)
    t = np.fft.fftshift(np.linspace(-40, 40, 512, endpoint=False))
    f0 = np.fft.fft(np.exp(-t ** 2 / 2))
    d = rng.uniform(-1, 1, nz)
    target = cases.noise(rng, 512, 1.0).reshape(1, 512)
    target /= np.linalg.norm(target)
    out, gx, gf, gd, _ = _engine_grads(nlm, kw, x, f0, d, target)
    assert cases.rel_l2(out, _oracle_out(oracle, kw, x, f0, d)) < 1e-9
    r2 = np.random.default_rng(11)
    # pump: a perturbation proportional to the spectrum with random phases
    v = f0 * np.exp(2j * np.pi * r2.uniform(size=512)) * r2.uniform(0.5, 1.5, 512)
    adj = float(np.sum(gf.real * v.real + gf.imag * v.imag))
    fd = _dir_fd(lambda f: _loss(_oracle_out(oracle, kw, x, f, d), target), f0, v, 5e-4)
    assert abs(adj - fd) < 1e-6 * abs(fd)
    # poling profile
    u = r2.uniform(-1, 1, nz)
    adj = float(np.dot(gd, u))
    fd = _dir_fd(lambda p: _loss(_oracle_out(oracle, kw, x, f0, p), target), d, u, 5e-4)
    assert abs(adj - fd) < 1e-6 * abs(fd)
    # input spectrum
    w = cases.noise(r2, 512, 1e-3).reshape(1, 512)
    adj = float(np.sum(gx.real * w.real + gx.imag * w.imag))
    fd = _dir_fd(lambda y: _loss(_oracle_out(oracle, kw, y, f0, d), target), x, w, 0.5)
    assert abs(adj - fd) < 1e-6 * abs(fd)


GN = dict(relativeLength=0.5, nlLength=1, selfSteepLength=5, fr=0.18, fb=0.21, tau1=0.0155, tau2=0.2165, tau3=0.4,
          beta2=-1, beta3=0.05, tMax=10, tPrecision=64, zPrecision=20)


def _oracle_gnlse(oracle, x):
    m = oracle.Chi3GNLSE(**GN)
    f, _ = m.propagate(x, False, 0)
    return f[:, 0]


def test_gnlse_adjoint_matches_finite_differences(nlm, oracle):
    """Gradient of the band energy with respect to the input spectrum, and of the spectral phase of the
    pump part of the input (the gradient configuration of the GNLSE batch, at small size)."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    med = nlm.Chi3GNLSE(**GN)
    n = 64
    rng = np.random.default_rng(5)
    t = np.fft.fftshift(np.linspace(-10, 10, n, endpoint=False))
    pump = np.fft.fft(2.0 / np.cosh(t))
    noise = np.fft.fft(cases.noise(rng, 2 * n, 1e-2).reshape(2, n), axis=1)
    w = med.omega
    band = ((w >= 2) & (w <= 4)).astype(float)
    phi0 = rng.uniform(-0.3, 0.3, n)

    def inputs(phi):
        return pump[None, :] * np.exp(1j * phi)[None, :] + noise

    phi = torch.tensor(phi0, dtype=torch.float64, device="cuda", requires_grad=True)
    a_in = torch.tensor(pump, device="cuda")[None, :] * torch.exp(1j * phi)[None, :] + torch.tensor(noise, device="cuda")
    out = propagate_gnlse(med, a_in)
    energy = torch.sum(torch.abs(out) ** 2 * torch.tensor(band, device="cuda"))
    energy.backward()
    gphi = phi.grad.cpu().numpy()
    ref_out = _oracle_gnlse(oracle, inputs(phi0))
    assert cases.rel_l2(out.detach().cpu().numpy(), ref_out) < 1e-9

    def e_oracle(p):
        return float(np.sum(np.abs(_oracle_gnlse(oracle, inputs(p))) ** 2 * band))

    h = 1e-6
    idx = _significant(gphi, 4, np.random.default_rng(0))
    assert _rel_vec(gphi[idx], [_fd(e_oracle, phi0, i, h) for i in idx]) < 1e-6


def test_gnlse_checkpointed_sweep(nlm):
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    med = nlm.Chi3GNLSE(**GN)
    rng = np.random.default_rng(8)
    x = np.fft.fft(cases.signal_input("Chi3GNLSE", 64, 1, seed=2))[None, :].repeat(3, 0)
    x = x + np.fft.fft(cases.noise(rng, 3 * 64, 1e-2).reshape(3, 64), axis=1)
    grads = []
    for k in (1, 6):
        xt = torch.tensor(x, device="cuda", requires_grad=True)
        out = propagate_gnlse(med, xt, k)
        torch.sum(torch.abs(out) ** 2 * torch.arange(64, device="cuda")).backward()
        grads.append(xt.grad.cpu().numpy())
    assert cases.rel_l2(grads[1], grads[0]) < 1e-12


@pytest.mark.parametrize("rows", [1, 80])
def test_checkpoint_paths_agree(nlm, rows):
    """Checkpoint interval > 1 with few rows runs the two-CTA pipelined sweep, with more rows than half
    the SMs the one-CTA sweep; both must give the stored-state (interval 1) gradients."""
    kw = dict(KW, zPrecision=60)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    x, f0, d, target = _problem(64, nz, rows=rows, seed=12)
    a = _engine_grads(nlm, kw, x, f0, d, target, interval=1)
    b = _engine_grads(nlm, kw, x, f0, d, target, interval=11)
    for ga, gb in zip(a[1:4], b[1:4]):
        assert cases.rel_l2(gb, ga) < 1e-12


def test_sqrt_checkpoints_at_config_size(nlm):
    """The gradient configuration with sqrt(nZSteps) checkpoints against all states stored."""
    kw = dict(KW, tMax=40, tPrecision=512, zPrecision=1000, diffBeta0=0)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    rng = np.random.default_rng(4)
    x = cases.noise(rng, 512, 1e-3).reshape(1, 512)
    t = np.fft.fftshift(np.linspace(-40, 40, 512, endpoint=False))
    f0 = np.fft.fft(np.exp(-t ** 2 / 2))
    d = rng.uniform(-1, 1, nz)
    target = cases.noise(rng, 512, 1.0).reshape(1, 512)
    target /= np.linalg.norm(target)
    a = _engine_grads(nlm, kw, x, f0, d, target, interval=1)
    k = int(np.ceil(np.sqrt(nz - 1)))
    b = _engine_grads(nlm, kw, x, f0, d, target, interval=k)
    assert b[4]._last_schedule()["grid"] == 12          # a stage-gradient group beside the sweep
    for ga, gb in zip(a[1:4], b[1:4]):
        assert cases.rel_l2(gb, ga) < 1e-11
    # two stage groups on sixteen CTAs; the two-group form on eight CTAs (the transposed stages inside
    # the reverse steps)
    for cap in (16, 8):
        os.environ["NLM_ADJOINT_CTAS"] = str(cap)
        try:
            c = _engine_grads(nlm, kw, x, f0, d, target, interval=k)
        finally:
            del os.environ["NLM_ADJOINT_CTAS"]
        assert c[4]._last_schedule()["grid"] == cap
        for gb, gc in zip(b[1:4], c[1:4]):
            assert cases.rel_l2(gb, gc) < 1e-11


@pytest.mark.parametrize("interval", [2, 13, 20, 40])
def test_stage_group_sweep_segment_counts(nlm, interval):
    """The sweeps with stage-gradient groups (sixteen and twelve CTAs) with one segment (interval 40 > nZSteps - 1), two, several, and the shortest
    interval, on 256 points and 3 rows (stage-factor gradients accumulated over rows): the gradients
    of every-state storage."""
    kw = dict(KW, tPrecision=256, zPrecision=15)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    assert 20 < nz - 1 < 40
    x, f0, d, target = _problem(256, nz, rows=3, seed=interval)
    a = _engine_grads(nlm, kw, x, f0, d, target, interval=1)
    b = _engine_grads(nlm, kw, x, f0, d, target, interval=interval)
    assert b[4]._last_schedule()["grid"] % 12 == 0
    for ga, gb in zip(a[1:4], b[1:4]):
        assert cases.rel_l2(gb, ga) < 1e-11
    os.environ["NLM_ADJOINT_CTAS"] = "16"
    try:
        c = _engine_grads(nlm, kw, x, f0, d, target, interval=interval)
    finally:
        del os.environ["NLM_ADJOINT_CTAS"]
    assert c[4]._last_schedule()["grid"] % 16 == 0
    for ga, gc in zip(a[1:4], c[1:4]):
        assert cases.rel_l2(gc, ga) < 1e-11


def test_gnlse_pipelined_and_one_cta_sweeps_agree(nlm):
    """3 rows run the two-CTA pipelined sweep, 80 rows (more than half the SMs) the one-CTA sweep;
    the loss is a sum over rows, so the first 3 rows' gradients must agree between the two."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    rng = np.random.default_rng(13)
    x80 = np.fft.fft(cases.noise(rng, 80 * 64, 0.5).reshape(80, 64), axis=1)
    weights = torch.arange(64, device="cuda", dtype=torch.float64)
    grads = {}
    for rows in (3, 80):
        for k in (1, 5):
            med = nlm.Chi3GNLSE(**GN)
            xt = torch.tensor(x80[:rows], device="cuda", requires_grad=True)
            torch.sum(torch.abs(propagate_gnlse(med, xt, k)) ** 2 * weights).backward()
            grads[rows, k] = xt.grad.cpu().numpy()
    for key in ((3, 5), (80, 1), (80, 5)):
        assert cases.rel_l2(grads[key][:3], grads[3, 1]) < 1e-12
    assert cases.rel_l2(grads[80, 5], grads[80, 1]) < 1e-12


@pytest.mark.parametrize("n", [1024, 4096])
def test_gnlse_cluster_sweep(nlm, n):
    """Few rows on grids of 1024+ points: the forward runs on clusters.  With the interval chosen by the
    engine (0) it stores the stage values of every step and the reverse sweep reads them on clusters of
    the same form (one point per thread on 8 or 16 CTAs; four points per thread on four in mode 2); with an explicit checkpoint interval the reverse sweep runs on clusters of eight CTAs
    (four reverse the current segment while four recompute the next).  Gradients agree with the one-CTA
    sweeps for intervals 1 and one that leaves a short last segment, and match a directional central
    difference of the engine's forward."""
    torch = pytest.importorskip("torch")
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    from multimodenonlinearoptics_gb300.workloads import GNLSE_CONFIG
    kw = dict(GNLSE_CONFIG, tPrecision=n, relativeLength=0.05, tMax=50)
    rows = 3
    rng = np.random.default_rng(n)
    t = np.fft.fftshift(np.linspace(-50, 50, n, endpoint=False))
    x = np.fft.fft(3.0 / np.cosh(t) + cases.noise(rng, rows * n, 1e-3).reshape(rows, n), axis=1)
    weights = torch.linspace(0, 1, n, device="cuda", dtype=torch.float64)
    nz = nlm.Chi3GNLSE(**kw)._dims["nZSteps"]
    k_short = 7 if (nz - 1) % 7 else 6

    def grad(cluster, k):
        med = nlm.Chi3GNLSE(**kw)
        med._set_cluster(cluster)
        xt = torch.tensor(x, device="cuda", requires_grad=True)
        torch.sum(torch.abs(propagate_gnlse(med, xt, k)) ** 2 * weights).backward()
        return xt.grad.cpu().numpy(), med._last_schedule()

    g = {}
    g[1, 0], sched = grad(1, 0)
    # stored stages: the forward and the reverse sweep with one point per thread on eight CTAs per row
    # at 1024 points, sixteen at 4096
    assert sched["grid"] == (8 if n == 1024 else 16) * rows and sched["R"] == 1
    g[2, 0], sched = grad(2, 0)                       # four points per thread on four CTAs per row
    assert sched["grid"] == 4 * rows and sched["R"] == 4
    for k in (1, k_short):
        g[1, k], sched = grad(1, k)
        assert sched["grid"] == 8 * rows and sched["R"] == 4
        g[0, k], sched = grad(0, k)
        assert sched["grid"] not in (4 * rows, 8 * rows)
    for key in ((2, 0), (1, 1), (1, k_short), (0, 1), (0, k_short)):
        assert cases.rel_l2(g[key], g[1, 0]) < 1e-10
    med = nlm.Chi3GNLSE(**kw)
    w = weights.cpu().numpy()

    def loss(y):
        return float(np.sum(np.abs(med.batchSignalSimulation(y, inTimeDomain=False)) ** 2 * w))

    d = cases.noise(np.random.default_rng(1), rows * n, 1.0).reshape(rows, n)
    adj = float(np.sum(np.real(np.conj(g[1, 0]) * d)))
    # the loss is ~1e7 at N=4096: a larger step keeps the difference's round-off (~1e-16 L / h) small
    fd = _dir_fd(loss, x, d, 1e-4)
    assert abs(adj - fd) < 1e-6 * abs(fd)


@pytest.mark.parametrize("n", [512, 1024, 2048, 4096])
def test_pdc_cluster_sweep(nlm, oracle, n):
    """Few rows on grids of 256+ points: the checkpointed forward runs on 4-CTA clusters (one point per
    thread up to 1024 points, four above; cluster mode 2 keeps four at 1024), and so does the reverse
    sweep for checkpoint interval 1; interval 7 (segments recomputed with the cluster transforms) runs
    pipelined on clusters of eight CTAs.  The input, pump and poling gradients agree with the one-CTA
    sweeps, and match directional central differences of the oracle's forward."""
    kw = dict(KW, tPrecision=n, zPrecision=30)
    nz = nlm.Chi2PDC(**kw)._dims["nZSteps"]
    x, f0, d, target = _problem(n, nz, rows=2, seed=n)
    res = {}
    for cluster in ((1, 2, 0) if n == 1024 else (1, 0)):
        for k in (1, 7):
            res[cluster, k] = _engine_grads(nlm, kw, x, f0, d, target, interval=k, cluster=cluster)
            if cluster:
                sched = res[cluster, k][4]._last_schedule()
                # interval 7 up to 2048 points in mode 1: three groups on twelve CTAs with one point per
                # thread (the propagator matrices are built), else two groups on eight
                staged = cluster == 1 and n <= 2048 and k > 1
                assert sched["grid"] == (8 if k == 1 else (24 if staged else 16))
                assert sched["R"] == (1 if (cluster == 1 and n <= 1024) or staged else 4)
    for key in [(1, 7), (0, 1), (0, 7)] + ([(2, 1), (2, 7)] if n == 1024 else []):
        for ga, gb in zip(res[1, 1][1:4], res[key][1:4]):
            assert cases.rel_l2(gb, ga) < 1e-11
    out, gx, gf, gd, _ = res[1, 1]
    assert cases.rel_l2(out, _oracle_out(oracle, kw, x, f0, d)) < 1e-9
    r2 = np.random.default_rng(5)
    v = f0 * np.exp(2j * np.pi * r2.uniform(size=n)) * r2.uniform(0.5, 1.5, n)
    adj = float(np.sum(gf.real * v.real + gf.imag * v.imag))
    fd = _dir_fd(lambda f: _loss(_oracle_out(oracle, kw, x, f, d), target), f0, v, 5e-4)
    assert abs(adj - fd) < 1e-6 * abs(fd)
    u = r2.uniform(-1, 1, nz)
    adj = float(np.dot(gd, u))
    fd = _dir_fd(lambda p: _loss(_oracle_out(oracle, kw, x, f0, p), target), d, u, 5e-4)
    assert abs(adj - fd) < 1e-6 * abs(fd)
