"""The index arithmetic of the cluster transforms, replayed in numpy.

One point per thread (`nlm_spread.cuh`):

multimodenonlinearoptics_gb300/csrc/nlm_spread.cuh spreads an N-point transform over C = 4 or 8 CTAs
of M = N / C threads: thread j of CTA c holds time point c + C j and frequency bin j + M c.  The local
M-point DFT is a radix-2 Stockham pass per stage (output t = e + W o with e = y[k + L p], o = e's
partner M/2 further, W = twM[k' M / 2L]); the C-point DFT across the CTAs combines the received
column per output row (4 points: a + W_4^r b; 8 points: v0 + W_8^r v1).  This test executes exactly
those index expressions for every thread, checks every shared-memory index against its buffer, and
compares the result with numpy's FFT: forward, and the unscaled inverse round trip.

Four points per thread (`nlm_cluster.cuh`, C = R = 4): thread j of CTA c, register v holds time point
c + C (j + v T) and frequency bin j + c T + M v (T = M / C).  The local M-point transform is the one-CTA
register FFT, which keeps the ownership j + v T of its input for its output (tested against the oracle
by the one-CTA kernels' own parity tests; here an exact DFT).  The test replays the twiddle
exp(-2 pi i c k2 / N), the transpose through distributed shared memory (thread j of CTA c writes its
register v to slot c T + j of CTA v's receive half; thread j then reads register c' from slot
c' T + j) and the C-point DFT over the registers.  No GPU needed.
"""
import numpy as np
import pytest


def _local(x, tw_m, inverse):
    """spread_local: thread t holds element t on entry and bin t on return."""
    m = x.size
    half = m >> 1
    t = np.arange(m)
    p = t >> 1
    assert p.max() + half < m
    x = x[p] + np.where(t & 1, -1.0, 1.0) * x[p + half]
    big_l, shift = 2, 1
    while big_l < m:
        kp = t & (2 * big_l - 1)
        src = (kp & (big_l - 1)) + big_l * (t >> (shift + 1))
        widx = kp * (half >> shift)
        assert src.min() >= 0 and src.max() < half and widx.max() < m
        w = np.conj(tw_m[widx]) if inverse else tw_m[widx]
        x = x[src] + w * x[src + half]
        big_l <<= 1
        shift += 1
    return x


def _quarter(q, b):
    return (b, -1j * b, -b, 1j * b)[q]


def _exchange(rows, tw_m, inverse):
    """spread_exchange: rows[c] is the column pushed by CTA c; returns CTA r's output per row r."""
    c_count, m = rows.shape
    out = np.empty_like(rows)
    for r in range(c_count):
        sg = -1.0 if r & 1 else 1.0
        q = (4 - (r & 3)) & 3 if inverse else r & 3
        if c_count == 4:
            out[r] = rows[0] + sg * rows[2] + _quarter(q, rows[1] + sg * rows[3])
        else:
            u = [rows[c] + sg * rows[c + 4] for c in range(4)]
            v0, v1 = u[0] + _quarter(q, u[2]), u[1] + _quarter(q, u[3])
            w = tw_m[r * (m // 8)]
            out[r] = v0 + (np.conj(w) if inverse else w) * v1
    return out


def _tables(n, c_count):
    tw = np.exp(-2j * np.pi * np.arange(n) / n)         # the engine's N-point table
    m = n // c_count
    return tw, tw[np.arange(m) * c_count], m


def spread_forward(x, c_count):
    n = x.size
    tw, tw_m, m = _tables(n, c_count)
    j = np.arange(m)
    rows = np.array([_local(x[c + c_count * j], tw_m, False) * tw[c * j] for c in range(c_count)])
    y = _exchange(rows, tw_m, False)
    out = np.empty(n, complex)
    for c in range(c_count):
        out[j + m * c] = y[c]
    return out


def spread_inverse(xf, c_count):
    n = xf.size
    tw, tw_m, m = _tables(n, c_count)
    j = np.arange(m)
    y = _exchange(np.array([xf[j + m * c] for c in range(c_count)]), tw_m, True)
    out = np.empty(n, complex)
    for c in range(c_count):
        out[c + c_count * j] = _local(y[c] * np.conj(tw[c * j]), tw_m, True)
    return out


@pytest.mark.parametrize("c_count,n", [(4, 128), (4, 256), (4, 512), (4, 1024), (8, 2048), (8, 4096), (8, 256)])
def test_spread_transform_matches_numpy(c_count, n):
    rng = np.random.default_rng(n + c_count)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    got = spread_forward(x, c_count)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    back = spread_inverse(got, c_count) / n
    assert np.max(np.abs(back - x)) <= 1e-12 * np.max(np.abs(x))


def test_shared_memory_layout():
    """Twiddles (M), two exchange buffers (2M) and two halves of C receive rows (2CM) per CTA, as
    spread_smem_per_point in nlm_kernels.h; within 227 KB for the largest launch (N=4096 on 8 CTAs)."""
    for c_count, n in ((4, 1024), (8, 4096)):
        m = n // c_count
        values = m * (1 + 2 + 2 * c_count)
        assert values * 16 <= 227 * 1024


def _four_point_forward(x, c_count=4):
    n = x.size
    m = n // c_count
    t = m // c_count                                    # threads per CTA
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    j = np.arange(t)
    # regs[c][v][j]: register v of thread j in CTA c after the local transform and the twiddle
    regs = np.empty((c_count, c_count, t), complex)
    for c in range(c_count):
        local = np.fft.fft(x[c + c_count * np.arange(m)])   # bin k2 at ownership k2 = j + v T
        for v in range(c_count):
            k2 = j + v * t
            regs[c, v] = local[k2] * tw[c * k2]
    recv = np.full((c_count, c_count * t), np.nan + 0j)   # one receive half per CTA
    for c in range(c_count):
        for v in range(c_count):
            dst = c * t + j
            assert dst.max() < c_count * t
            recv[v, dst] = regs[c, v]
    assert not np.isnan(recv).any()                       # every slot written exactly by the plan
    out = np.empty(n, complex)
    w_c = np.exp(-2j * np.pi / c_count)
    for v in range(c_count):                               # CTA v after the barrier
        r = np.array([recv[v, cp * t + j] for cp in range(c_count)])
        for k1 in range(c_count):
            out[j + v * t + m * k1] = sum(w_c ** (cp * k1) * r[cp] for cp in range(c_count))
    return out


@pytest.mark.parametrize("n", [1024, 2048, 8192])
def test_four_point_cluster_transform_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.max(np.abs(_four_point_forward(x) - ref)) <= 1e-12 * np.max(np.abs(ref))
