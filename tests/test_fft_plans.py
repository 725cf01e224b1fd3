"""The index arithmetic of the general-plan transform (csrc/nlm_device.cuh, fft_general), emulated
in numpy on the CPU: padded ownership (thread j of T = ceil(N/R) owns the points j + v T below N),
radix-8/4/2 passes as butterflies held ceil(R/r) per thread, any other radix as r-term sums held one
per owned index, and the plan's factor order (make_plan_gen in csrc/engine.h).  Every pass must write
each point exactly once and the result must be the DFT."""
import numpy as np
import pytest


def plan_radices(n):
    """make_plan_gen's passes: radix 8 while three factors of two remain, then 4 or 2, then the odd
    prime factors in ascending order."""
    twos = 0
    while n % 2 == 0:
        n //= 2
        twos += 1
    rad = [8] * (twos // 3) + ([1 << (twos % 3)] if twos % 3 else [])
    q = 3
    while n > 1:
        while n % q == 0:
            rad.append(q)
            n //= q
        q += 2
    return rad


def general_fft(x, R, inverse=False):
    n = x.size
    T = -(-n // R)
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    if inverse:
        tw = tw.conj()
    buf = np.zeros(n, dtype=np.complex128)
    owned = np.zeros(n, dtype=int)
    for j in range(T):
        for v in range(R):
            t = j + v * T
            if t < n:
                buf[t] = x[t]
                owned[t] += 1
    assert np.all(owned == 1)
    L = 1
    for r in plan_radices(n):
        nb, stride = n // r, n // (L * r)
        out = np.zeros(n, dtype=np.complex128)
        hits = np.zeros(n, dtype=int)
        if r in (2, 4, 8):
            for j in range(T):
                for u in range(-(-R // r)):
                    b = j + u * T
                    if b >= nb:
                        continue
                    k = b % L
                    a = np.array([buf[b + q * nb] * (tw[k * q * stride] if L > 1 else 1) for q in range(r)])
                    y = np.fft.ifft(a) * r if inverse else np.fft.fft(a)
                    for s in range(r):
                        out[(b - k) * r + k + s * L] = y[s]
                        hits[(b - k) * r + k + s * L] += 1
        else:
            for j in range(T):
                for v in range(R):
                    o = j + v * T
                    if o >= n:
                        continue
                    b, s = o % nb, o // nb
                    k = b % L
                    step = (k * stride + s * nb) % n
                    acc, e = 0j, 0
                    for q in range(r):
                        acc += buf[b + q * nb] * tw[e]
                        e = (e + step) % n
                    out[(b - k) * r + k + s * L] = acc
                    hits[(b - k) * r + k + s * L] += 1
        assert np.all(hits == 1), (n, R, r, L)
        buf = out
        L *= r
    return buf


@pytest.mark.parametrize("n", [2, 6, 10, 12, 24, 96, 100, 462, 514, 1000, 1002, 1536, 4098])
@pytest.mark.parametrize("R", [4, 8, 16])
def test_general_plan_is_the_dft(n, R):
    if -(-n // R) > 512:
        pytest.skip("no CTA of more than 512 threads")
    rng = np.random.default_rng(n * R)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    np.testing.assert_allclose(general_fft(x, R), np.fft.fft(x), rtol=0, atol=1e-9 * np.abs(x).sum())
    np.testing.assert_allclose(general_fft(x, R, True), np.fft.ifft(x) * n, rtol=0, atol=1e-9 * np.abs(x).sum())


def test_plan_radices():
    assert plan_radices(1000) == [8, 5, 5, 5]
    assert plan_radices(6000) == [8, 2, 3, 5, 5, 5]
    assert plan_radices(8190) == [2, 3, 3, 5, 7, 13]
    assert plan_radices(8186) == [2, 4093]
    assert len(plan_radices(2 * 3 ** 7)) <= 16
