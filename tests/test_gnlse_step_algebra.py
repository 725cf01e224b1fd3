"""The algebra behind the Chi3GNLSE kernels' step forms, restated in numpy (solvers/Chi3GNLSE.cpp:39-92:
one RK4 step of the generalised NLSE, then the dispersion step).  Conventions of the kernels: F the
unscaled forward transform, B the unscaled inverse (B F = N), the per-point tables carry 1/N, and a
gradient is g = dL/dRe + i dL/dIm.

* The RK4 sum in the frequency domain (the stages' spectra added, the state's spectrum kept from the
  previous step) is the time-domain step.
* The reverse step in the frequency domain (the gradient kept as a spectrum) is the transform of the
  time-domain reverse step, and both are the transpose of the step: a dot-product test against central
  differences.
* Two rows' real Raman fields go through one complex transform pair."""
import numpy as np
import pytest

N = 64
W = np.array([1.0, 2.0, 2.0, 1.0]) / 6.0      # RK4 weights of the stages' k
FAC = np.array([0.0, 0.5, 0.5, 1.0])          # y_s = x + FAC_s k_{s-1}


def F(x):
    return np.fft.fft(x)


def B(x):
    return np.fft.ifft(x) * N


@pytest.fixture(scope="module")
def tables():
    rng = np.random.default_rng(11)
    w = 2 * np.pi * np.fft.fftfreq(N, d=0.3)
    resp = np.exp(-np.abs(np.arange(N) - 3) / 4.0) * np.sin(0.4 * np.arange(N))   # a real response
    return dict(
        raman=F(resp) / N,                                        # R~ / N (Hermitian: real in, real out)
        steep=(1j * 0.7 + 0.05 * w) / N,                          # (g0 + g1 w) / N
        disp=np.exp(1j * 0.02 * (0.5 * w ** 2 - 0.1 * w ** 3)) / N,   # one dispersion step, 1/N folded in
        rel=np.array([0.008, 0.009, 0.011]),                      # the step's nonlinear factors (s = 0, 1-2, 3)
        rng=rng)


def ri(t, s):
    return t["rel"][0 if s == 0 else (2 if s == 3 else 1)]


def stage(t, s, y):
    """k, and the stored u2, of stage s at its input y."""
    u2 = B(t["raman"] * F(ri(t, s) * np.abs(y) ** 2))
    return B(t["steep"] * F(u2 * y)), u2


def step_time(t, x):
    """The step as the one-CTA kernels ran it: time-domain RK4 sum, then F, dispersion, B."""
    k = np.zeros(N, complex)
    acc = np.zeros(N, complex)
    Y, U2 = [], []
    for s in range(4):
        y = x + FAC[s] * k
        k, u2 = stage(t, s, y)
        Y.append(y)
        U2.append(u2)
        acc += W[s] * 6 * k
    return B(t["disp"] * F(x + acc / 6)), Y, U2


def step_freq(t, x, xf):
    """The frequency-domain RK4 sum: the stages' spectra added; FFT[x + sum / 6] = N (xf + sum / 6),
    with xf the state's spectrum (B xf = x).  Returns the new time-domain state and spectrum."""
    k = np.zeros(N, complex)
    acc_f = np.zeros(N, complex)
    for s in range(4):
        y = x + FAC[s] * k
        u2 = B(t["raman"] * F(ri(t, s) * np.abs(y) ** 2))
        kf = t["steep"] * F(u2 * y)
        acc_f += W[s] * 6 * kf
        if s < 3:
            k = B(kf)
    xf_new = N * (xf + acc_f / 6) * t["disp"]
    return B(xf_new), xf_new


def reverse_time(t, g, Y, U2):
    """The time-domain reverse step (g: the gradient of the state after the step, time domain)."""
    g = B(np.conj(t["disp"]) * F(g))
    gx, gxp, gke = g.copy(), g.copy(), np.zeros(N, complex)
    for s in range(3, -1, -1):
        u = B(np.conj(t["steep"]) * F(gke + W[s] * gxp))                     # g_u3
        gy = np.conj(U2[s]) * u
        g1 = B(np.conj(t["raman"]) * F(np.conj(Y[s]) * u)).real             # g_u1
        gy = gy + 2 * ri(t, s) * g1 * Y[s]
        gx += gy
        gke = FAC[s] * gy
    return gx


def reverse_freq(t, G, Y, U2):
    """The frequency-domain reverse step (G = F g): h = N conj(D) G; stage s's spectrum gets W_s h plus
    F of the gradient its time-domain value takes through the next stage's input; the spectrum before
    the step gets h + F[the stage inputs' gradient]."""
    h = N * np.conj(t["disp"]) * G
    gx, gke = np.zeros(N, complex), np.zeros(N, complex)
    for s in range(3, -1, -1):
        u = (F(gke) + W[s] * h) if s < 3 else W[s] * h
        u = B(np.conj(t["steep"]) * u)                                       # g_u3
        gy = np.conj(U2[s]) * u
        g1 = B(np.conj(t["raman"]) * F(np.conj(Y[s]) * u)).real
        gy = gy + 2 * ri(t, s) * g1 * Y[s]
        gx += gy
        gke = FAC[s] * gy
    return F(gx) + h


def noise(rng, scale):
    return (rng.standard_normal(N) + 1j * rng.standard_normal(N)) * scale


def test_raman_field_is_real(tables):
    x = noise(tables["rng"], 1.0)
    u2 = B(tables["raman"] * F(np.abs(x) ** 2))
    assert np.abs(u2.imag).max() < 1e-12 * np.abs(u2.real).max()


def test_frequency_domain_sum_is_the_step(tables):
    rng = tables["rng"]
    x0 = noise(rng, 1.0)
    x, xf = x0.copy(), F(x0) / N
    xt = x0.copy()
    for _ in range(5):
        xt = step_time(tables, xt)[0]
        x, xf = step_freq(tables, x, xf)
    assert np.linalg.norm(x - xt) / np.linalg.norm(xt) < 1e-13


def test_frequency_domain_reverse_is_the_transform_of_the_time_domain_one(tables):
    rng = tables["rng"]
    x = noise(rng, 1.0)
    _, Y, U2 = step_time(tables, x)
    g = noise(rng, 1.0)
    gt = reverse_time(tables, g, Y, U2)
    gf = reverse_freq(tables, F(g), Y, U2)
    assert np.linalg.norm(gf - F(gt)) / np.linalg.norm(F(gt)) < 1e-13


@pytest.mark.parametrize("form", ["time", "freq"])
def test_reverse_step_is_the_transpose(tables, form):
    """Re <g_in, v> = Re <g_out, J v> with J v from central differences of the step (real-linear J)."""
    rng = tables["rng"]
    x, v, g = noise(rng, 1.0), noise(rng, 1.0), noise(rng, 1.0)
    _, Y, U2 = step_time(tables, x)
    gin = reverse_time(tables, g, Y, U2) if form == "time" else B(reverse_freq(tables, F(g), Y, U2)) / N
    eps = 1e-6
    jv = (step_time(tables, x + eps * v)[0] - step_time(tables, x - eps * v)[0]) / (2 * eps)
    lhs = np.vdot(gin, v).real
    rhs = np.vdot(g, jv).real
    assert abs(lhs - rhs) <= 1e-7 * abs(rhs)


def test_two_real_fields_share_one_transform_pair(tables):
    """L(a + i b) = L(a) + i L(b) for real a, b and a Hermitian response: the paired kernels' shared
    Raman transforms, forward and adjoint."""
    rng = tables["rng"]
    a, b = rng.standard_normal(N), rng.standard_normal(N)
    for resp in (tables["raman"], np.conj(tables["raman"])):
        pair = B(resp * F(a + 1j * b))
        la, lb = B(resp * F(a)), B(resp * F(b))
        assert np.allclose(pair.real, la.real, rtol=0, atol=1e-12 * np.abs(la).max())
        assert np.allclose(pair.imag, lb.real, rtol=0, atol=1e-12 * np.abs(lb).max())
