"""The index arithmetic of the cluster transforms, replayed in numpy.

One point per thread (`nlm_spread.cuh`):

multimodenonlinearoptics_gb300/csrc/nlm_spread.cuh spreads an N-point transform over C = 4, 8 or 16
CTAs of M = N / C threads: thread j of CTA c (lane l = j mod 32, warp g = j / 32, G = M / 32 warps)
holds time point c + C (g + G l) and frequency bin j + M c.  The local M-point DFT is 32 x G: a 32-point
DFT in each warp (the lanes take their bit-reversed lane's element by a shuffle, then five radix-2
decimation-in-time stages pair lane l with l ^ s through shuffles, each lane computing A + (+-W) B),
the twiddle W_M^(g l), then a G-point radix-2 Stockham DFT across the warps through shared memory; the
C-point DFT across the CTAs combines the received column per output row (4 points: a + W_4^r b; 8
points: v0 + W_8^r v1; 16 points: y0 + W_16^r y1).  This test executes exactly those index
expressions for every thread, checks every shared-memory and table index against its buffer, and
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


def _brev5(lane):
    return int(format(lane, "05b")[::-1], 2)


def _warp_dft(vals, tw_m, inverse):
    """spread_warp_dft: lane l holds element l on entry and bin l on return."""
    m = tw_m.size
    x = np.array([vals[_brev5(lane)] for lane in range(32)])
    s = 1
    while s < 32:
        p = x[np.arange(32) ^ s]
        out = np.empty(32, complex)
        for lane in range(32):
            up = (lane & s) != 0
            if s == 1:                                  # W = 1: own + partner, partner - own
                out[lane] = p[lane] + (-1 if up else 1) * x[lane]
                continue
            a, b = (p[lane], x[lane]) if up else (x[lane], p[lane])
            if s == 2:                                  # W = 1 or -i (i inverse) as a component swap
                if lane & 1:
                    b = complex(-b.imag, b.real) if inverse else complex(b.imag, -b.real)
                out[lane] = a + (-1 if up else 1) * b
                continue
            idx = (lane & (s - 1)) * (m // (2 * s))
            assert idx < m
            w = np.conj(tw_m[idx]) if inverse else tw_m[idx]
            out[lane] = a + (-w if up else w) * b
        x = out
        s *= 2
    return x


def _cross_warp(vals, tw_m, inverse):
    """spread_cross_warp: vals[g][l]; the G-point DFT over g for every lane (Stockham, shared memory
    element e of lane l at e 32 + l)."""
    g_count, m = vals.shape[0], tw_m.size
    y = vals.copy()
    big_l, shift = 1, 0
    g = np.arange(g_count)
    while big_l < g_count:
        kp = g & (2 * big_l - 1)
        src = (kp & (big_l - 1)) + big_l * (g >> (shift + 1))
        assert (src + g_count // 2).max() * 32 + 31 < m
        if big_l <= 2:                                   # W = (-i)^q as a swap and signs
            q = (2 * kp if big_l == 1 else kp) & 3
            qq = (4 - q) & 3 if inverse else q
            o = y[src + g_count // 2]
            swap = (q & 1)[:, None] != 0
            ox = np.where(swap, o.imag, o.real)
            oy = np.where(swap, o.real, o.imag)
            sx = np.where((qq == 2) | (qq == 3), -1.0, 1.0)[:, None]
            sy = np.where((qq == 1) | (qq == 2), -1.0, 1.0)[:, None]
            y = y[src] + sx * ox + 1j * sy * oy
        else:
            w = tw_m[kp * (m // (2 * big_l))]
            w = np.conj(w) if inverse else w
            y = y[src] + w[:, None] * y[src + g_count // 2]
        big_l <<= 1
        shift += 1
    return y


def _local(x, tw_m, inverse):
    """spread_local: x[j] is thread j's value; forward: thread j holds element t(j), returns bin j."""
    m = tw_m.size
    g_count = m // 32
    gl = np.array([[tw_m[g * lane] for lane in range(32)] for g in range(g_count)])
    v = x.reshape(g_count, 32)
    if not inverse:
        w = np.array([_warp_dft(v[g], tw_m, False) for g in range(g_count)]) * gl
        return _cross_warp(w, tw_m, False).reshape(m)
    z = _cross_warp(v, tw_m, True) * np.conj(gl)
    return np.array([_warp_dft(z[g], tw_m, True) for g in range(g_count)]).reshape(m)


def _time_index(j, m):
    """spread_time_index: the local time element of thread j."""
    return (j >> 5) + (m >> 5) * (j & 31)


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
        elif c_count == 8:
            u = [rows[c] + sg * rows[c + 4] for c in range(4)]
            v0, v1 = u[0] + _quarter(q, u[2]), u[1] + _quarter(q, u[3])
            w = tw_m[r * (m // 8)]
            out[r] = v0 + (np.conj(w) if inverse else w) * v1
        else:
            u = [rows[c] + sg * rows[c + 8] for c in range(8)]
            w4 = [u[c] + _quarter(q, u[c + 4]) for c in range(4)]
            w8 = tw_m[(r & 7) * (m // 8)]
            w8 = np.conj(w8) if inverse else w8
            y = [w4[c] + w8 * w4[c + 2] for c in range(2)]
            w16 = tw_m[r * (m // 16)]
            out[r] = y[0] + (np.conj(w16) if inverse else w16) * y[1]
    return out


def _tables(n, c_count):
    tw = np.exp(-2j * np.pi * np.arange(n) / n)         # the engine's N-point table
    m = n // c_count
    return tw, tw[np.arange(m) * c_count], m


def spread_forward(x, c_count):
    n = x.size
    tw, tw_m, m = _tables(n, c_count)
    j = np.arange(m)
    t = _time_index(j, m)
    rows = np.array([_local(x[c + c_count * t], tw_m, False) * tw[c * j] for c in range(c_count)])
    y = _exchange(rows, tw_m, False)
    out = np.empty(n, complex)
    for c in range(c_count):
        out[j + m * c] = y[c]
    return out


def spread_inverse(xf, c_count):
    n = xf.size
    tw, tw_m, m = _tables(n, c_count)
    j = np.arange(m)
    t = _time_index(j, m)
    y = _exchange(np.array([xf[j + m * c] for c in range(c_count)]), tw_m, True)
    out = np.empty(n, complex)
    for c in range(c_count):
        out[c + c_count * t] = _local(y[c] * np.conj(tw[c * j]), tw_m, True)
    return out


@pytest.mark.parametrize("c_count,n", [(4, 128), (4, 256), (4, 512), (4, 1024), (4, 2048), (8, 1024), (8, 2048),
                                       (8, 4096), (16, 2048), (16, 4096)])
def test_spread_transform_matches_numpy(c_count, n):
    rng = np.random.default_rng(n + c_count)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    got = spread_forward(x, c_count)
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    back = spread_inverse(got, c_count) / n
    assert np.max(np.abs(back - x)) <= 1e-12 * np.max(np.abs(x))


def test_time_ownership_is_a_permutation():
    """Every local time element is held by exactly one thread (M = 32 .. 512)."""
    for m in (32, 64, 128, 256, 512):
        assert np.array_equal(np.sort(_time_index(np.arange(m), m)), np.arange(m))


def test_shared_memory_layout():
    """Twiddles (M), two exchange buffers (2M) and two halves of C receive rows (2CM) per CTA, as
    spread_smem_per_point in nlm_kernels.h; within 227 KB for the largest launches (N=4096 on 8 and
    16 CTAs)."""
    for c_count, n in ((4, 1024), (8, 4096), (16, 4096)):
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
