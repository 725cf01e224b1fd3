"""CPU oracle for the split-step propagation path of MultimodeNonlinearOptics.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module: only
``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it,
as the checker and as the timed CPU baseline ("port").

This is a numpy restatement of the reference's double-precision algorithm,
vectorised over a leading batch axis so that Green's-function and batch runs
finish in seconds at test sizes.  Every function cites the reference file:line
it restates (paths are relative to the reference project root).

Parity status
-------------
* ``set_poling`` is PINNED: it is checked bit-for-bit against golden vectors
  produced by the reference's own Python twin ``poling.py:439-471``
  (``domainsToSpace``), see ``tests/golden/make_golden.py``.
* Everything that goes through a DFT is PARITY UNPINNED: the reference's C++
  engine cannot be built on this image (it needs the Eigen 3 headers,
  ``CMakeLists.txt:12``, which are absent) and the reference ships no golden
  vectors.  The DFT convention is the one of ``src/CustomEigenFFT.h:91-101``
  (forward unscaled, inverse scaled by 1/N), which is numpy.fft's convention.
  The restatement is additionally anchored on the known-answer properties of
  the reference's notebooks (soliton stationarity, Green's-function
  consistency, symplectic C/S), which the tests assert.
"""

import math

import numpy as np

INF = float("inf")

GAUSSIAN, SECH, SINC = 0, 1, 2                      # PulseType, src/_NonlinearMedium.hpp:25-29
GAUSSIAN_BEAM, CONSTANT, GAUSSIAN_APODIZATION = 0, 1, 2   # IntensityProfile, src/_NonlinearMedium.hpp:30-34


def fft(x):
    """Unscaled forward DFT along the last axis (src/CustomEigenFFT.h:59-63)."""
    return np.fft.fft(x, axis=-1)


def ifft(x):
    """Inverse DFT scaled by 1/N along the last axis (src/CustomEigenFFT.h:91-101)."""
    return np.fft.ifft(x, axis=-1)


def fftshift1(x):
    """Half swap of a 1-D array (src/_NonlinearMedium.cpp:447-453)."""
    half = x.shape[-1] // 2
    return np.concatenate([x[..., half:], x[..., :half]], axis=-1)


def fftshift2(block):
    """Quadrant swap of a 2-D block (src/_NonlinearMedium.cpp:456-467)."""
    hr, hc = block.shape[0] // 2, block.shape[1] // 2
    out = np.empty_like(block)
    out[:hr, :hc] = block[-hr:, -hc:] if hr and hc else out[:hr, :hc]
    out[:hr, -hc:] = block[-hr:, :hc] if hr and hc else out[:hr, -hc:]
    out[-hr:, :hc] = block[:hr, -hc:] if hr and hc else out[-hr:, :hc]
    out[-hr:, -hc:] = block[:hr, :hc] if hr and hc else out[-hr:, -hc:]
    return out


def linspaced(n, low, high):
    """Evenly spaced samples low..high inclusive (used at src/_NonlinearMedium.cpp:240)."""
    if n == 1:
        return np.array([high], dtype=np.float64)
    step = (high - low) / (n - 1)
    out = low + np.arange(n, dtype=np.float64) * step
    out[-1] = high
    return out


def domains_to_space(poling, n_z_steps):
    """Domain lengths -> per-z-step poling direction (src/_NonlinearMedium.cpp:470-503)."""
    poling = np.asarray(poling, dtype=np.float64).ravel()
    if poling.size <= 1:
        return np.ones(n_z_steps)
    if np.any(poling <= 0):
        raise ValueError("Poling contains invalid domain length")
    pole = np.cumsum(poling)
    pole = pole * (n_z_steps / pole[-1])
    out = np.empty(n_z_steps)
    prev = 0
    direction = 1
    for cur in pole:
        cur_round = int(cur)
        if cur < prev:
            raise ValueError("Poling period too small for simulation resolution")
        out[prev:cur_round] = direction
        if cur_round < n_z_steps:
            out[cur_round] = direction * (2 * abs(math.fmod(cur, 1)) - 1)
        direction *= -1
        prev = cur_round + 1
    return out


def _maxabs(values):
    """Element of largest magnitude (signed), 0 when empty (src/_NonlinearMedium.cpp:78-84)."""
    if len(values) == 0:
        return 0.0
    best = values[0]
    for v in values[1:]:
        if abs(best) < abs(v):
            best = v
    return best


class Medium:
    """Restatement of ``_NonlinearMedium`` (src/_NonlinearMedium.hpp:20-142, src/_NonlinearMedium.cpp:8-40)."""

    n_signal_modes = 1
    fully_nonlinear = False
    name = "_NonlinearMedium"

    def __init__(self, n_pump_modes, can_be_poled, relative_length, nl_length, beta2, beta2s,
                 custom_pump, pulse_type, beta1, beta1s, beta3, beta3s, diff_beta0,
                 rayleigh_length, t_max, t_precision, z_precision, intensity_profile,
                 chirp, delay, poling=None):
        self.n_pump_modes = n_pump_modes
        if intensity_profile == CONSTANT:
            rayleigh_length = INF
        self.set_lengths(relative_length, list(nl_length), z_precision, rayleigh_length,
                         list(beta2), list(beta2s), list(beta1), list(beta1s), list(beta3), list(beta3s))
        self.reset_grids(t_precision, t_max)
        self.set_dispersion(list(beta2), list(beta2s), list(beta1), list(beta1s), list(beta3), list(beta3s),
                            list(diff_beta0))
        if can_be_poled:
            self.set_poling(np.zeros(0) if poling is None else poling)
        else:
            self.poling = np.zeros(0)
        self.intensity_profile = intensity_profile if self.rayleigh_length != INF else CONSTANT
        self.envelope = []
        if self.n_pump_modes > 0:
            self.envelope = [np.zeros(self.n_freqs, dtype=np.complex128) for _ in range(self.n_pump_modes)]
            if custom_pump is not None and np.asarray(custom_pump).size != 0:
                Medium.set_pump_custom(self, custom_pump, chirp, delay)
            else:
                Medium.set_pump_type(self, pulse_type, chirp, delay)

    # -- setup (src/_NonlinearMedium.cpp:43-177) ---------------------------------------------
    def set_lengths(self, relative_length, nl_length, z_precision, rayleigh_length,
                    beta2, beta2s, beta1, beta1s, beta3, beta3s):
        """src/_NonlinearMedium.cpp:43-102."""
        negative = relative_length <= 0 or rayleigh_length <= 0 or any(nl <= 0 for nl in nl_length)
        if negative:
            raise ValueError("Non-positive length scale")
        all_non_unit = True
        for group in (beta1, beta2, beta3, beta1s, beta2s, beta3s):
            for b in group:
                all_non_unit &= abs(b) != 1
        for nl in nl_length:
            all_non_unit &= nl != 1
        all_non_unit &= relative_length != 1
        all_non_unit &= rayleigh_length != 1
        if all_non_unit:
            raise ValueError("No unit length scale provided: please normalize variables")
        self.z = float(relative_length)
        extremes = [_maxabs(g) for g in (beta2, beta2s, beta1, beta1s, beta3, beta3s)]
        big = _maxabs(extremes)
        min_disp_length = 1.0 / abs(big) if big != 0 else INF
        min_nl = min(nl_length) if nl_length else 0.0
        denom = min(1.0, min_disp_length, rayleigh_length, min_nl)
        steps = z_precision * self.z / denom if denom != 0 else INF
        self.n_z_steps = int(steps) if math.isfinite(steps) and steps < 2**32 else 0
        self.n_z_steps_p = max(2 * self.n_z_steps - 1, 0)
        self.dz = self.z / (self.n_z_steps - 1) if self.n_z_steps > 1 else INF
        self.dzp = self.z / (self.n_z_steps_p - 1) if self.n_z_steps_p > 1 else INF
        self.nl_step = [complex(0.0, 1.0 / nl) * self.dz for nl in nl_length]
        self.rayleigh_length = float(rayleigh_length)

    def reset_grids(self, n_freqs, t_max):
        """src/_NonlinearMedium.cpp:105-145 (tau and omega in FFT order)."""
        if n_freqs % 2 != 0 or n_freqs == 0:
            raise ValueError("Invalid number of Frequencies")
        if self.n_z_steps == 0:
            raise ValueError("Zero steps")
        if t_max <= 0:
            raise ValueError("Negative time span")
        self.n_freqs = int(n_freqs)
        self.t_max = float(t_max)
        nt = self.n_freqs
        ramp = np.arange(-nt // 2, nt // 2, dtype=np.float64)
        self.tau = fftshift1((2 * t_max / nt) * ramp)
        self.omega = fftshift1((-math.pi / t_max) * ramp)
        self.pump_freq = [np.zeros((self.n_z_steps_p, nt), dtype=np.complex128) for _ in range(self.n_pump_modes)]
        self.pump_time = [np.zeros((self.n_z_steps_p, nt), dtype=np.complex128) for _ in range(self.n_pump_modes)]
        self.signal_freq = [np.zeros((self.n_z_steps, nt), dtype=np.complex128) for _ in range(self.n_signal_modes)]
        self.signal_time = [np.zeros((self.n_z_steps, nt), dtype=np.complex128) for _ in range(self.n_signal_modes)]

    def set_dispersion(self, beta2, beta2s, beta1, beta1s, beta3, beta3s, diff_beta0):
        """src/_NonlinearMedium.cpp:148-177."""
        w = self.omega
        self.beta2, self.beta1, self.diff_beta0 = beta2, beta1, diff_beta0
        self.disp_pump = [w * (beta1[m] + w * (0.5 * beta2[m] + w * beta3[m] / 6)) for m in range(self.n_pump_modes)]
        self.disp_sign = [w * (beta1s[m] + w * (0.5 * beta2s[m] + w * beta3s[m] / 6))
                          for m in range(self.n_signal_modes)]
        self.disp_step_pump = [np.exp(1j * self.dzp * d) for d in self.disp_pump]
        self.disp_step_sign = [np.exp(1j * self.dz * d) for d in self.disp_sign]

    def set_poling(self, poling):
        """src/_NonlinearMedium.cpp:470-503."""
        self.poling = domains_to_space(poling, self.n_z_steps)

    # -- pump (src/_NonlinearMedium.cpp:180-250, 506-534) ---------------------------------------
    def _chirp_delay(self, idx, chirp, delay):
        """Chirp and delay applied through the frequency domain (src/_NonlinearMedium.cpp:198-203)."""
        if chirp != 0 or delay != 0:
            w = self.omega
            spec = fft(self.envelope[idx])
            spec = spec * np.exp(1j * (self.beta1[idx] * delay + 0.5 * self.beta2[idx] * chirp * w) * w)
            self.envelope[idx] = ifft(spec)

    def set_pump_type(self, pulse_type, chirp=0.0, delay=0.0, pump_index=0):
        """src/_NonlinearMedium.cpp:180-204."""
        if pump_index >= self.n_pump_modes:
            raise ValueError("Invalid pump index")
        tau = self.tau
        if pulse_type == SECH:
            env = 1 / np.cosh(tau)
        elif pulse_type == SINC:
            with np.errstate(invalid="ignore", divide="ignore"):
                env = np.sin(tau) / tau
            env[0] = 1
        else:
            env = np.exp(-0.5 * tau ** 2)
        self.envelope[pump_index] = env.astype(np.complex128)
        self._chirp_delay(pump_index, chirp, delay)

    def set_pump_custom(self, custom_pump, chirp=0.0, delay=0.0, pump_index=0):
        """src/_NonlinearMedium.cpp:207-222."""
        custom_pump = np.asarray(custom_pump, dtype=np.complex128).ravel()
        if custom_pump.size != self.n_freqs:
            raise ValueError("Custom pump array length does not match number of frequency/time bins")
        if pump_index >= self.n_pump_modes:
            raise ValueError("Invalid pump index")
        self.envelope[pump_index] = custom_pump.copy()
        self._chirp_delay(pump_index, chirp, delay)

    def set_pump_other(self, other, mode_index=0, delay=0.0, pump_index=0):
        """Pump copied from another medium's signal (src/_NonlinearMedium.cpp:506-534)."""
        if other.n_freqs != self.n_freqs or other.t_max != self.t_max:
            raise ValueError("Medium does not have same time and frequency axes as this one")
        if mode_index >= self.n_signal_modes:
            raise ValueError("Mode index larger than number of modes in medium")
        if pump_index >= self.n_pump_modes:
            raise ValueError("Invalid pump index")
        if other.n_z_steps < self.n_z_steps:
            raise ValueError("Medium does not have sufficient resolution to be used with this one")
        dl = 1j * self.beta1[pump_index] * delay * self.omega
        src = other.signal_freq[mode_index]
        pf, pt = self.pump_freq[pump_index], self.pump_time[pump_index]
        ratio = float(other.n_z_steps - 1) / (self.n_z_steps_p - 1)
        for i in range(self.n_z_steps_p - 1):
            jf = i * ratio
            j = int(jf)
            frac = jf - j
            pf[i] = ((1 - frac) * src[j] + frac * src[j + 1]) * np.exp(
                (1j * (i * self.dzp)) * self.disp_pump[pump_index]
                - (1j * (jf + 0.5) * other.dz) * other.disp_sign[mode_index] + dl)
            pt[i] = ifft(pf[i])
        pf[-1] = src[-1] * np.exp((1j * self.z) * self.disp_pump[pump_index]
                                  - (1j * other.z) * other.disp_sign[mode_index] + dl)
        # the reference transforms row nZSteps-1 here, not the last row (src/_NonlinearMedium.cpp:533)
        pt[self.n_z_steps - 1] = ifft(pf[self.n_z_steps - 1])

    def run_pump_simulation(self):
        """Linear pump: dispersion phase per row, then the z profile (src/_NonlinearMedium.cpp:225-250)."""
        for m in range(self.n_pump_modes):
            pf, pt = self.pump_freq[m], self.pump_time[m]
            pf[0] = fft(self.envelope[m])
            pt[0] = self.envelope[m]
            rows = np.arange(1, self.n_z_steps_p, dtype=np.float64)
            pf[1:] = pf[0][None, :] * np.exp((1j * (rows * self.dzp))[:, None] * self.disp_pump[m][None, :])
            pt[1:] = ifft(pf[1:])
            if self.intensity_profile != CONSTANT:
                zl = linspaced(self.n_z_steps_p, -0.5 * self.z, 0.5 * self.z) / self.rayleigh_length
                if self.intensity_profile == GAUSSIAN_APODIZATION:
                    strength = np.exp(-0.5 * zl ** 2)
                else:
                    strength = 1 / np.sqrt(1 + zl ** 2)
                pf *= strength[:, None]
                pt *= strength[:, None]

    # -- z profile of fully nonlinear media (src/_FullyNonlinearMedium.hpp:40-63) ----------------
    def relative_amplitude(self, i):
        x = (i * self.dz - 0.5 * self.z) / self.rayleigh_length
        if self.intensity_profile == GAUSSIAN_BEAM:
            return math.sqrt(1 / (1 + x ** 2))
        if self.intensity_profile == GAUSSIAN_APODIZATION:
            return math.exp(-0.5 * x ** 2)
        return 1.0

    def relative_intensity(self, i):
        x = (i * self.dz - 0.5 * self.z) / self.rayleigh_length
        if self.intensity_profile == GAUSSIAN_BEAM:
            return 1 / (1 + x ** 2)
        if self.intensity_profile == GAUSSIAN_APODIZATION:
            return math.exp(-x ** 2)
        return 1.0

    # -- helpers for DiffEq -----------------------------------------------------------------
    def pump_rows(self, i, p=0):
        pt = self.pump_time[p]
        return pt[2 * i - 2], pt[2 * i - 1], pt[2 * i]

    def pol(self, i):
        prev, curr = self.poling[i - 1], self.poling[i]
        return prev, 0.5 * (prev + curr), curr

    def mismatch(self, i, db):
        """exp(i·Δβ·z) at the three RK4 sub-steps (e.g. solvers/Chi2PDC.cpp:36-38)."""
        return (np.exp(1j * db * ((i - 1) * self.dz)), np.exp(1j * db * ((i - .5) * self.dz)),
                np.exp(1j * db * (i * self.dz)))

    def diff_eq(self, i, a):
        raise NotImplementedError

    # -- the split-step template (src/_NonlinearMedium.hpp:160-239) -----------------------------
    def propagate(self, inputs, in_time_domain, input_mode, keep_grid=False):
        """Propagate a batch of inputs.

        ``inputs`` has shape (B, k·N).  Returns (freq, time): each a list over modes of arrays of
        shape (B, N) holding the last row, or (B, nZSteps, N) when ``keep_grid`` (the
        non-optimised path that fills the full grids).
        """
        inputs = np.asarray(inputs, dtype=np.complex128)
        if inputs.ndim == 1:
            inputs = inputs[None, :]
        nb, n, nm = inputs.shape[0], self.n_freqs, self.n_signal_modes
        n_in = inputs.shape[1] // n
        if n_in > 1:
            input_mode = 0
        if nm <= 1:
            input_mode = 0
        half = [np.exp((0.5j * self.dz) * d) for d in self.disp_sign]
        freq = np.zeros((nb, nm, n), dtype=np.complex128)
        for m in range(nm):
            if m == input_mode:
                seg = inputs[:, 0:n]
            elif input_mode < 1 and m < n_in:
                seg = inputs[:, m * n:(m + 1) * n]
            else:
                continue
            freq[:, m] = (fft(seg) if in_time_domain else seg) * half[m]
        time = np.zeros_like(freq)
        for m in range(nm):
            if m == input_mode or m < n_in:
                time[:, m] = ifft(freq[:, m])
        if keep_grid:
            grid_f = np.zeros((nb, nm, self.n_z_steps, n), dtype=np.complex128)
            grid_t = np.zeros_like(grid_f)
            grid_f[:, :, 0], grid_t[:, :, 0] = freq, time
        step = np.stack(self.disp_step_sign)[None]
        for i in range(1, self.n_z_steps):
            k1, k2, k3, k4 = self.diff_eq(i, time)
            time = time + (k1 + 2 * k2 + 2 * k3 + k4) * (1. / 6.)
            freq = fft(time) * step
            time = ifft(freq)
            if keep_grid:
                grid_f[:, :, i], grid_t[:, :, i] = freq, time
        back = np.stack([np.exp((-0.5j * self.dz) * d) for d in self.disp_sign])[None]
        freq = freq * back
        time = ifft(freq)
        if keep_grid:
            grid_f[:, :, -1], grid_t[:, :, -1] = freq, time
            return grid_f, grid_t
        return freq, time

    # -- public methods (src/_NonlinearMedium.cpp:253-444) --------------------------------------
    def run_signal_simulation(self, input_prof, in_time_domain=True, input_mode=0):
        """src/_NonlinearMedium.cpp:253-260."""
        input_prof = np.asarray(input_prof, dtype=np.complex128).ravel()
        n, nm = self.n_freqs, self.n_signal_modes
        if input_prof.size % n != 0 or input_prof.size // n == 0 or input_prof.size // n > nm:
            raise ValueError("inputProf array size does not match number of frequency/time bins")
        if input_mode >= nm:
            raise ValueError("inputModes does not match any mode in the system")
        gf, gt = self.propagate(input_prof[None], in_time_domain, input_mode, keep_grid=True)
        for m in range(nm):
            self.signal_freq[m] = gf[0, m].copy()
            self.signal_time[m] = gt[0, m].copy()

    @staticmethod
    def mode_mask(mask, n_modes):
        """Mode selection of a useInput/useOutput list, read as a 0/1 mask (src/_NonlinearMedium.cpp:292-299)."""
        if mask is None or len(mask) == 0:
            return list(range(n_modes))
        return [m for m in range(n_modes) if m < len(mask) and mask[m]]

    def compute_greens_function(self, in_time_domain=False, run_pump=True, n_threads=1, normalize=False,
                                use_input=(), use_output=(), chunk=None):
        """Green's matrices from 2·N·nIn impulse propagations (src/_NonlinearMedium.cpp:263-375)."""
        nm, n = self.n_signal_modes, self.n_freqs
        if len(use_input) > nm:
            raise ValueError("List of requested inputs indices longer than number of modes!")
        if len(use_output) > nm:
            raise ValueError("List of requested output indices longer than number of modes!")
        # The reference counts entries whose value is < nModes (src/_NonlinearMedium.cpp:274-290) but selects
        # modes by reading the list as a 0/1 mask (:294-299).  Where the two disagree the reference is undefined;
        # the count rule still decides when it raises, the mask decides the selection.
        if len(use_input) and sum(1 for v in use_input if v < nm) == 0:
            raise ValueError("Requested no valid inputs!")
        if len(use_output) and sum(1 for v in use_output if v < nm) == 0:
            raise ValueError("Requested no valid outputs!")
        inputs = self.mode_mask(use_input, nm)
        outputs = self.mode_mask(use_output, nm)
        if not inputs:
            raise ValueError("Requested no valid inputs!")
        if not outputs:
            raise ValueError("Requested no valid outputs!")
        n_in, n_out = len(inputs), len(outputs)
        if n_threads > n * n_in or n_threads < 1:
            raise ValueError("Too many threads requested!")
        if run_pump:
            self.run_pump_simulation()
        rows = n_in * n
        green_c = np.zeros((rows, n_out * n), dtype=np.complex128)
        green_s = np.zeros_like(green_c)
        chunk = chunk or max(1, min(rows, 256))
        for start in range(0, rows, chunk):
            idx = np.arange(start, min(rows, start + chunk))
            for value, sign in ((1.0, None), (1j, 1j)):
                outs = np.zeros((idx.size, n_out * n), dtype=np.complex128)
                for im in sorted(set((idx // n).tolist())):
                    sel = idx[idx // n == im]
                    prof = np.zeros((sel.size, n), dtype=np.complex128)
                    prof[np.arange(sel.size), sel % n] = value
                    f, t = self.propagate(prof, in_time_domain, inputs[im])
                    g = t if in_time_domain else f
                    pos = np.searchsorted(idx, sel)
                    for om, mo in enumerate(outputs):
                        outs[pos, om * n:(om + 1) * n] = g[:, mo]
                if sign is None:
                    green_c[idx] += 0.5 * outs
                    green_s[idx] += 0.5 * outs
                else:
                    green_c[idx] -= 0.5j * outs
                    green_s[idx] += 0.5j * outs
        green_c = green_c.T.copy()
        green_s = green_s.T.copy()
        for mat in (green_c, green_s):
            # the reference iterates im over nOutputModes here (src/_NonlinearMedium.cpp:361,368)
            for im in range(min(n_out, n_in)):
                for om in range(n_out):
                    blk = mat[om * n:(om + 1) * n, im * n:(im + 1) * n]
                    shifted = fftshift2(blk)
                    if normalize and im != om:
                        shifted = shifted * np.sqrt(self.nl_step[im] / self.nl_step[om])
                    mat[om * n:(om + 1) * n, im * n:(im + 1) * n] = shifted
        return green_c, green_s

    def batch_signal_simulation(self, input_profs, in_time_domain=False, run_pump=True, n_threads=1,
                                input_mode=0, use_output=(), chunk=None):
        """Independent propagations, one per input row (src/_NonlinearMedium.cpp:378-444)."""
        input_profs = np.asarray(input_profs, dtype=np.complex128)
        if input_profs.ndim == 1:
            input_profs = input_profs[None, :]
        n_inputs, in_cols = input_profs.shape
        nm, n = self.n_signal_modes, self.n_freqs
        if in_cols % n != 0 or in_cols // n == 0 or in_cols // n > nm:
            raise ValueError("Signals not of correct length!")
        if n_threads > n_inputs or n_threads < 1:
            raise ValueError("Too many threads requested!")
        if input_mode >= nm:
            raise ValueError("inputModes does not match any mode in the system")
        if len(use_output) > 0 and sum(1 for v in use_output if v != 0) == 0:
            raise ValueError("Requested no outputs!")
        outputs = self.mode_mask(use_output, nm)
        if run_pump:
            self.run_pump_simulation()
        out = np.zeros((n_inputs, len(outputs) * n), dtype=np.complex128)
        chunk = chunk or max(1, min(n_inputs, 256))
        for start in range(0, n_inputs, chunk):
            sl = slice(start, min(n_inputs, start + chunk))
            f, t = self.propagate(input_profs[sl], in_time_domain, input_mode)
            g = t if in_time_domain else f
            for om, mo in enumerate(outputs):
                out[sl, om * n:(om + 1) * n] = g[:, mo]
        return out


class FullyNonlinearMedium(Medium):
    """Restatement of ``_FullyNonlinearMedium`` (src/_FullyNonlinearMedium.hpp:6-69)."""

    fully_nonlinear = True

    def __init__(self, can_be_poled, relative_length, nl_length, beta2s, beta1s, beta3s, diff_beta0,
                 rayleigh_length, t_max, t_precision, z_precision, intensity_profile, poling=None):
        super().__init__(0, can_be_poled, relative_length, nl_length, [], beta2s, None, GAUSSIAN, [], beta1s, [],
                         beta3s, diff_beta0, rayleigh_length, t_max, t_precision, z_precision, intensity_profile,
                         0, 0, poling)
        self.dzp = 0.0
        self.n_z_steps_p = 0

    def run_pump_simulation(self):
        raise RuntimeError("Object does not have this method.")

    def compute_greens_function(self, *a, **k):
        raise RuntimeError("Object does not have this method.")

    def batch_signal_simulation(self, input_profs, in_time_domain=False, n_threads=1, input_mode=0,
                                use_output=(), chunk=None):
        """src/_FullyNonlinearMedium.hpp:8-11 (runPump forced off)."""
        return Medium.batch_signal_simulation(self, input_profs, in_time_domain, False, n_threads, input_mode,
                                              use_output, chunk)


# ------------------------------------------------------------------------------------------------
# Solvers (solvers/*.cpp).  Each diff_eq receives the batch of previous time-domain fields
# a[:, mode, :] and returns k1..k4 of the same shape.
# ------------------------------------------------------------------------------------------------

def _c(x):
    return np.conj(x)


class Chi3(Medium):
    """solvers/Chi3.cpp:22-85."""
    n_signal_modes = 1
    name = "Chi3"

    def __init__(self, relativeLength, nlLength, beta2, customPump=None, pulseType=GAUSSIAN, beta3=0.0,
                 rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100, intensityProfile=GAUSSIAN_BEAM,
                 chirp=0.0):
        super().__init__(1, False, relativeLength, [nlLength], [beta2], [beta2], customPump, pulseType, [0], [0],
                         [beta3], [beta3], [], rayleighLength, tMax, tPrecision, zPrecision, intensityProfile,
                         chirp, 0)

    def run_pump_simulation(self):
        """Self-phase-modulated pump march (solvers/Chi3.cpp:41-70)."""
        pf, pt = self.pump_freq[0], self.pump_time[0]
        d = self.disp_pump[0]
        pf[0] = fft(self.envelope[0]) * np.exp((0.5j * self.dzp) * d)
        pt[0] = ifft(pf[0])
        scale = (self.dzp / self.dz) * self.nl_step[0]
        if self.intensity_profile == GAUSSIAN_BEAM:
            zl = linspaced(self.n_z_steps_p, -0.5 * self.z, 0.5 * self.z) / self.rayleigh_length
            rel = scale / (1 + zl ** 2)
        elif self.intensity_profile == GAUSSIAN_APODIZATION:
            zl = linspaced(self.n_z_steps_p, -0.5 * self.z, 0.5 * self.z) / self.rayleigh_length
            rel = scale * np.exp(-zl ** 2)
        else:
            rel = scale * np.ones(self.n_z_steps_p)
        for i in range(1, self.n_z_steps_p):
            row = pt[i - 1] * np.exp(rel[i - 1] * np.abs(pt[i - 1]) ** 2)
            pf[i] = fft(row) * self.disp_step_pump[0]
            pt[i] = ifft(pf[i])
        pf[-1] = pf[-1] * np.exp((-0.5j * self.dzp) * d)
        pt[-1] = ifft(pf[-1])

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        g = self.nl_step[0]
        x = a[:, 0]
        k1 = g * (2 * np.abs(p0) ** 2 * x + p0 ** 2 * _c(x))
        y = x + 0.5 * k1
        k2 = g * (2 * np.abs(p1) ** 2 * y + p1 ** 2 * _c(y))
        y = x + 0.5 * k2
        k3 = g * (2 * np.abs(p1) ** 2 * y + p1 ** 2 * _c(y))
        y = x + k3
        k4 = g * (2 * np.abs(p2) ** 2 * y + p2 ** 2 * _c(y))
        return k1[:, None], k2[:, None], k3[:, None], k4[:, None]


class Chi2PDC(Medium):
    """solvers/Chi2PDC.cpp:6-44."""
    n_signal_modes = 1
    name = "Chi2PDC"

    def __init__(self, relativeLength, nlLength, beta2, beta2s, customPump=None, pulseType=GAUSSIAN, beta1=0.0,
                 beta1s=0.0, beta3=0.0, beta3s=0.0, diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512,
                 zPrecision=100, intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLength], [beta2], [beta2s], customPump, pulseType, [beta1],
                         [beta1s], [beta3], [beta3s], [diffBeta0], rayleighLength, tMax, tPrecision, zPrecision,
                         intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        s0, s1, s2 = self.pol(i)
        m0, m1, m2 = self.mismatch(i, self.diff_beta0[0])
        g = self.nl_step[0]
        x = a[:, 0]
        k1 = (s0 * g * m0) * p0 * _c(x)
        k2 = (s1 * g * m1) * p1 * _c(x + 0.5 * k1)
        k3 = (s1 * g * m1) * p1 * _c(x + 0.5 * k2)
        k4 = (s2 * g * m2) * p2 * _c(x + k3)
        return k1[:, None], k2[:, None], k3[:, None], k4[:, None]


class _TwoModeSFGLike(Medium):
    n_signal_modes = 2


class Chi2SFG(Medium):
    """solvers/Chi2SFG.cpp:6-57."""
    n_signal_modes = 2
    name = "Chi2SFG"

    def __init__(self, relativeLength, nlLength, nlLengthOrig, beta2, beta2s, beta2o, customPump=None,
                 pulseType=GAUSSIAN, beta1=0.0, beta1s=0.0, beta1o=0.0, beta3=0.0, beta3s=0.0, beta3o=0.0,
                 diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100,
                 intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLength, nlLengthOrig], [beta2], [beta2s, beta2o], customPump,
                         pulseType, [beta1], [beta1s, beta1o], [beta3], [beta3s, beta3o], [diffBeta0],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        s = self.pol(i)
        m = self.mismatch(i, self.diff_beta0[0])
        g0, g1 = self.nl_step
        xs, xo = a[:, 0], a[:, 1]
        ps = (p0, p1, p1, p2)
        ss = (s[0], s[1], s[1], s[2])
        ms = (m[0], m[1], m[1], m[2])
        ks, ko = [], []
        ds, do = 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            ys = xs + fac * ds
            yo = xo + fac * do
            a0 = (ss[st] * g0 * ms[st]) * ps[st] * yo
            a1 = (ss[st] * g1 * (1. / ms[st])) * _c(ps[st]) * ys
            ks.append(a0)
            ko.append(a1)
            ds, do = a0, a1
        return tuple(np.stack([ks[j], ko[j]], axis=1) for j in range(4))


class Chi2AFC(Medium):
    """solvers/Chi2AFC.cpp:6-51 (chirped mismatch, no poling)."""
    n_signal_modes = 2
    name = "Chi2AFC"

    def __init__(self, relativeLength, nlLength, nlLengthOrig, beta2, beta2s, beta2o, customPump=None,
                 pulseType=GAUSSIAN, beta1=0.0, beta1s=0.0, beta1o=0.0, beta3=0.0, beta3s=0.0, beta3o=0.0,
                 diffBeta0Start=0.0, diffBeta0End=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512,
                 zPrecision=100, intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0):
        super().__init__(1, False, relativeLength, [0.5 * math.pi * nlLength, 0.5 * math.pi * nlLengthOrig], [beta2],
                         [beta2s, beta2o], customPump, pulseType, [beta1], [beta1s, beta1o], [beta3],
                         [beta3s, beta3o], [diffBeta0Start, diffBeta0End], rayleighLength, tMax, tPrecision,
                         zPrecision, intensityProfile, chirp, delay)

    def chirped(self, i):
        """solvers/Chi2AFC.cpp:35-38."""
        arg = 0.5 * (self.diff_beta0[1] - self.diff_beta0[0]) / self.z
        d0, dz = self.diff_beta0[0], self.dz
        f = lambda s: np.exp(0.5j * ((d0 + s * dz * arg) * s * dz))
        return f(i - 1), f(i - .5), f(i)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        m = self.chirped(i)
        g0, g1 = self.nl_step
        xs, xo = a[:, 0], a[:, 1]
        ps, ms = (p0, p1, p1, p2), (m[0], m[1], m[1], m[2])
        out, ds, do = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            a0 = (g0 * ms[st]) * ps[st] * (xo + fac * do)
            a1 = (g1 * (1. / ms[st])) * _c(ps[st]) * (xs + fac * ds)
            out.append(np.stack([a0, a1], axis=1))
            ds, do = a0, a1
        return tuple(out)


class Chi2SFGPDC(Medium):
    """solvers/Chi2SFGPDC.cpp:6-59."""
    n_signal_modes = 2
    name = "Chi2SFGPDC"

    def __init__(self, relativeLength, nlLength, nlLengthOrig, beta2, beta2s, beta2o, customPump=None,
                 pulseType=GAUSSIAN, beta1=0.0, beta1s=0.0, beta1o=0.0, beta3=0.0, beta3s=0.0, beta3o=0.0,
                 diffBeta0=0.0, diffBeta0o=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100,
                 intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLength, nlLengthOrig], [beta2], [beta2s, beta2o], customPump,
                         pulseType, [beta1], [beta1s, beta1o], [beta3], [beta3s, beta3o], [diffBeta0, diffBeta0o],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        s = self.pol(i)
        m = self.mismatch(i, self.diff_beta0[0])
        mo = self.mismatch(i, self.diff_beta0[1])
        g0, g1 = self.nl_step
        xs, xo = a[:, 0], a[:, 1]
        ps, ss = (p0, p1, p1, p2), (s[0], s[1], s[1], s[2])
        ms, mos = (m[0], m[1], m[1], m[2]), (mo[0], mo[1], mo[1], mo[2])
        out, ds, do = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            ys, yo = xs + fac * ds, xo + fac * do
            a0 = (ss[st] * g0 * ms[st]) * ps[st] * yo
            a1 = (ss[st] * g1) * ((1. / ms[st]) * _c(ps[st]) * ys + mos[st] * ps[st] * _c(yo))
            out.append(np.stack([a0, a1], axis=1))
            ds, do = a0, a1
        return tuple(out)


class Chi2PDCII(Medium):
    """solvers/Chi2PDCII.cpp:6-55."""
    n_signal_modes = 2
    name = "Chi2PDCII"

    def __init__(self, relativeLength, nlLengthI, nlLengthII, beta2, beta2s, beta2o, customPump=None,
                 pulseType=GAUSSIAN, beta1=0.0, beta1s=0.0, beta1o=0.0, beta3=0.0, beta3s=0.0, beta3o=0.0,
                 diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100,
                 intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLengthI, nlLengthII], [beta2], [beta2s, beta2o], customPump,
                         pulseType, [beta1], [beta1s, beta1o], [beta3], [beta3s, beta3o], [diffBeta0],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        s = self.pol(i)
        m = self.mismatch(i, self.diff_beta0[0])
        g0, g1 = self.nl_step
        xs, xo = a[:, 0], a[:, 1]
        ps, ss, ms = (p0, p1, p1, p2), (s[0], s[1], s[1], s[2]), (m[0], m[1], m[1], m[2])
        out, ds, do = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            a0 = (ss[st] * g0 * ms[st]) * ps[st] * _c(xo + fac * do)
            a1 = (ss[st] * g1 * ms[st]) * ps[st] * _c(xs + fac * ds)
            out.append(np.stack([a0, a1], axis=1))
            ds, do = a0, a1
        return tuple(out)


class Chi2SFGII(Medium):
    """solvers/Chi2SFGII.cpp:6-90 (note: k4 uses prevPolDir, solvers/Chi2SFGII.cpp:86-89)."""
    n_signal_modes = 4
    name = "Chi2SFGII"

    def __init__(self, relativeLength, nlLengthZY, nlLengthZZ, beta2, beta2sz, beta2sy, beta2oz, beta2oy,
                 customPump=None, pulseType=GAUSSIAN, beta1=0.0, beta1sz=0.0, beta1sy=0.0, beta1oz=0.0, beta1oy=0.0,
                 beta3=0.0, beta3sz=0.0, beta3sy=0.0, beta3oz=0.0, beta3oy=0.0, diffBeta0z=0.0, diffBeta0y=0.0,
                 diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100,
                 intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLengthZY, nlLengthZZ], [beta2], [beta2sz, beta2sy, beta2oz, beta2oy],
                         customPump, pulseType, [beta1], [beta1sz, beta1sy, beta1oz, beta1oy], [beta3],
                         [beta3sz, beta3sy, beta3oz, beta3oy], [diffBeta0z, diffBeta0y, diffBeta0],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p0, p1, p2 = self.pump_rows(i)
        s = self.pol(i)
        mcz = self.mismatch(i, self.diff_beta0[0])
        mcy = self.mismatch(i, self.diff_beta0[1])
        msz = self.mismatch(i, self.diff_beta0[2])
        g0, g1 = self.nl_step
        x = [a[:, j] for j in range(4)]
        ps = (p0, p1, p1, p2)
        ss = (s[0], s[1], s[1], s[0])       # k4 uses the previous poling direction
        sel = (0, 1, 1, 2)
        out, d = [], [0, 0, 0, 0]
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            y = [x[j] + fac * d[j] for j in range(4)]
            q = sel[st]
            p, sd = ps[st], ss[st]
            k0 = sd * p * (g0 * mcz[q] * y[3] + g1 * msz[q] * y[2])
            k1 = (sd * g0 * mcy[q]) * p * y[2]
            k2 = sd * _c(p) * (g0 * (1. / mcy[q]) * y[1] + g1 * (1. / msz[q]) * y[0])
            k3 = (sd * g0 * (1. / mcz[q])) * _c(p) * y[0]
            d = [k0, k1, k2, k3]
            out.append(np.stack(d, axis=1))
        return tuple(out)


class Chi2SFGOPA(Medium):
    """solvers/Chi2SFGOPA.cpp:6-77 (two pumps)."""
    n_signal_modes = 2
    name = "Chi2SFGOPA"

    def __init__(self, relativeLength, nlLengthSFGh, nlLengthSFGf, nlLengthDOPAh, nlLengthDOPAf, beta2F, beta2H,
                 beta2h, beta2f, customPump=None, pulseType=GAUSSIAN, beta1F=0.0, beta1H=0.0, beta1h=0.0, beta1f=0.0,
                 beta3F=0.0, beta3H=0.0, beta3h=0.0, beta3f=0.0, diffBeta0SFG=0.0, diffBeta0DOPA=0.0,
                 rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100, intensityProfile=GAUSSIAN_BEAM,
                 chirp=0.0, delay=0.0, poling=None):
        super().__init__(2, True, relativeLength, [nlLengthSFGh, nlLengthSFGf, nlLengthDOPAh, nlLengthDOPAf],
                         [beta2F, beta2H], [beta2h, beta2f], customPump, pulseType, [beta1F, beta1H], [beta1h, beta1f],
                         [beta3F, beta3H], [beta3h, beta3f], [diffBeta0SFG, diffBeta0DOPA], rayleighLength, tMax,
                         tPrecision, zPrecision, intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        q0 = self.pump_rows(i, 0)
        q1 = self.pump_rows(i, 1)
        s = self.pol(i)
        msfg = self.mismatch(i, self.diff_beta0[0])
        mopa = self.mismatch(i, self.diff_beta0[1])
        g = self.nl_step
        xh, xf = a[:, 0], a[:, 1]
        sel = (0, 1, 1, 2)
        out, dh, df = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            yh, yf = xh + fac * dh, xf + fac * df
            sd = s[q]
            kh = (sd * g[0] * msfg[q]) * q0[q] * yf + (sd * g[2] * mopa[q]) * q1[q] * _c(yf)
            kf = (sd * g[1] * (1. / msfg[q])) * _c(q0[q]) * yh + (sd * g[3] * mopa[q]) * q1[q] * _c(yh)
            out.append(np.stack([kh, kf], axis=1))
            dh, df = kh, kf
        return tuple(out)


class Chi2SFGXPM(Medium):
    """solvers/Chi2SFGXPM.cpp:6-58 (XPM lengths halved, solvers/Chi2SFGXPM.cpp:24)."""
    n_signal_modes = 2
    name = "Chi2SFGXPM"

    def __init__(self, relativeLength, nlLength, nlLengthOrig, nlLengthChi3, nlLengthChi3Orig, beta2, beta2s,
                 beta2o, customPump=None, pulseType=GAUSSIAN, beta1=0.0, beta1s=0.0, beta1o=0.0, beta3=0.0,
                 beta3s=0.0, beta3o=0.0, diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512,
                 zPrecision=100, intensityProfile=GAUSSIAN_BEAM, chirp=0.0, delay=0.0, poling=None):
        super().__init__(1, True, relativeLength, [nlLength, nlLengthOrig, nlLengthChi3 / 2, nlLengthChi3Orig / 2],
                         [beta2], [beta2s, beta2o], customPump, pulseType, [beta1], [beta1s, beta1o], [beta3],
                         [beta3s, beta3o], [diffBeta0], rayleighLength, tMax, tPrecision, zPrecision,
                         intensityProfile, chirp, delay, poling)

    def diff_eq(self, i, a):
        p = self.pump_rows(i)
        s = self.pol(i)
        m = self.mismatch(i, self.diff_beta0[0])
        g = self.nl_step
        xs, xo = a[:, 0], a[:, 1]
        sel = (0, 1, 1, 2)
        out, ds, do = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            pp = p[q]
            ks = ((s[q] * g[0] * m[q]) * pp + g[2] * np.abs(pp) ** 2) * (xo + fac * do)
            ko = ((s[q] * g[1] * (1. / m[q])) * _c(pp) + g[3] * np.abs(pp) ** 2) * (xs + fac * ds)
            out.append(np.stack([ks, ko], axis=1))
            ds, do = ks, ko
        return tuple(out)


class Chi2SHG(FullyNonlinearMedium):
    """solvers/Chi2SHG.cpp:6-60 (modes reordered to {P, SH}, solvers/Chi2SHG.cpp:20)."""
    n_signal_modes = 2
    name = "Chi2SHG"

    def __init__(self, relativeLength, nlLengthH, nlLengthP, beta2h, beta2p, beta1h=0.0, beta1p=0.0, beta3h=0.0,
                 beta3p=0.0, diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100,
                 intensityProfile=GAUSSIAN_BEAM, poling=None):
        super().__init__(True, relativeLength, [nlLengthP, nlLengthH], [beta2p, beta2h], [beta1p, beta1h],
                         [beta3p, beta3h], [diffBeta0], rayleighLength, tMax, tPrecision, zPrecision,
                         intensityProfile, poling)

    def diff_eq(self, i, a):
        s = self.pol(i)
        r = (self.relative_amplitude(i - 1), self.relative_amplitude(i - .5), self.relative_amplitude(i))
        m = self.mismatch(i, self.diff_beta0[0])
        g = self.nl_step
        xp, xh = a[:, 0], a[:, 1]
        sel = (0, 1, 1, 2)
        out, dp, dh = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            rel = s[q] * r[q]
            yp, yh = xp + fac * dp, xh + fac * dh
            kp = (rel * g[0] * m[q]) * _c(yp) * yh
            kh = (rel * g[1] * (1. / m[q]) * .5) * yp ** 2
            out.append(np.stack([kp, kh], axis=1))
            dp, dh = kp, kh
        return tuple(out)


class Chi2SHGOPA(FullyNonlinearMedium):
    """solvers/Chi2SHGOPA.cpp:6-84."""
    n_signal_modes = 4
    name = "Chi2SHGOPA"

    def __init__(self, relativeLength, nlLengthP, nlLengthSH, nlLengthPA1, nlLengthPA2, beta2p, beta2sh, beta2pa1,
                 beta2pa2, beta1p=0.0, beta1sh=0.0, beta1pa1=0.0, beta1pa2=0.0, beta3p=0.0, beta3sh=0.0,
                 beta3pa1=0.0, beta3pa2=0.0, diffBeta0shg=0.0, diffBeta0opa=0.0, rayleighLength=INF, tMax=10.0,
                 tPrecision=512, zPrecision=100, intensityProfile=GAUSSIAN_BEAM, poling=None):
        super().__init__(True, relativeLength, [nlLengthP, nlLengthSH, nlLengthPA1, nlLengthPA2],
                         [beta2p, beta2sh, beta2pa1, beta2pa2], [beta1p, beta1sh, beta1pa1, beta1pa2],
                         [beta3p, beta3sh, beta3pa1, beta3pa2], [diffBeta0shg, diffBeta0opa], rayleighLength, tMax,
                         tPrecision, zPrecision, intensityProfile, poling)

    def diff_eq(self, i, a):
        s = self.pol(i)
        r = (self.relative_amplitude(i - 1), self.relative_amplitude(i - .5), self.relative_amplitude(i))
        ms = self.mismatch(i, self.diff_beta0[0])
        mo = self.mismatch(i, self.diff_beta0[1])
        g = self.nl_step
        x = [a[:, j] for j in range(4)]
        sel = (0, 1, 1, 2)
        out, d = [], [0, 0, 0, 0]
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            rel = s[q] * r[q]
            yp, yh, y1, y2 = (x[j] + fac * d[j] for j in range(4))
            k0 = (rel * g[0] * ms[q]) * _c(yp) * yh
            k1 = (rel * g[1]) * (mo[q] * y2 * y1 + (1. / ms[q]) * .5 * yp ** 2)
            k2 = (rel * g[2] * (1. / mo[q])) * yh * _c(y2)
            k3 = (rel * g[3] * (1. / mo[q])) * yh * _c(y1)
            d = [k0, k1, k2, k3]
            out.append(np.stack(d, axis=1))
        return tuple(out)


class Chi2DSFG(FullyNonlinearMedium):
    """solvers/Chi2DSFG.cpp:6-67."""
    n_signal_modes = 3
    name = "Chi2DSFG"

    def __init__(self, relativeLength, nlLengthP, nlLengthS, nlLengthD, beta2p, beta2s, beta2d, beta1p=0.0,
                 beta1s=0.0, beta1d=0.0, beta3p=0.0, beta3s=0.0, beta3d=0.0, diffBeta0=0.0, rayleighLength=INF,
                 tMax=10.0, tPrecision=512, zPrecision=100, intensityProfile=GAUSSIAN_BEAM, poling=None):
        super().__init__(True, relativeLength, [nlLengthP, nlLengthS, nlLengthD], [beta2p, beta2s, beta2d],
                         [beta1p, beta1s, beta1d], [beta3p, beta3s, beta3d], [diffBeta0], rayleighLength, tMax,
                         tPrecision, zPrecision, intensityProfile, poling)

    def diff_eq(self, i, a):
        s = self.pol(i)
        r = (self.relative_amplitude(i - 1), self.relative_amplitude(i - .5), self.relative_amplitude(i))
        m = self.mismatch(i, self.diff_beta0[0])
        g = self.nl_step
        x = [a[:, j] for j in range(3)]
        sel = (0, 1, 1, 2)
        out, d = [], [0, 0, 0]
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            rel = s[q] * r[q]
            yp, ys, yd = (x[j] + fac * d[j] for j in range(3))
            k0 = (rel * g[0] * m[q]) * ys * _c(yd)
            k1 = (rel * g[1] * (1. / m[q])) * yp * yd
            k2 = (rel * g[2] * m[q]) * ys * _c(yp)
            d = [k0, k1, k2]
            out.append(np.stack(d, axis=1))
        return tuple(out)


class Chi2SHGXPM(FullyNonlinearMedium):
    """solvers/Chi2SHGXPM.cpp:6-65."""
    n_signal_modes = 2
    name = "Chi2SHGXPM"

    def __init__(self, relativeLength, nlLengthH, nlLengthP, nlLengthChi3, beta2h, beta2p, beta1h=0.0, beta1p=0.0,
                 beta3h=0.0, beta3p=0.0, diffBeta0=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512,
                 zPrecision=100, intensityProfile=GAUSSIAN_BEAM, poling=None):
        super().__init__(True, relativeLength, [nlLengthP, nlLengthH, nlLengthChi3], [beta2p, beta2h],
                         [beta1p, beta1h], [beta3p, beta3h], [diffBeta0], rayleighLength, tMax, tPrecision,
                         zPrecision, intensityProfile, poling)

    def diff_eq(self, i, a):
        s = self.pol(i)
        r = (self.relative_amplitude(i - 1), self.relative_amplitude(i - .5), self.relative_amplitude(i))
        m = self.mismatch(i, self.diff_beta0[0])
        g = self.nl_step
        xp, xh = a[:, 0], a[:, 1]
        sel = (0, 1, 1, 2)
        out, dp, dh = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            rel = s[q] * r[q]
            chi3 = (r[q] ** 2) * g[2]
            yp, yh = xp + fac * dp, xh + fac * dh
            kp = (rel * g[0] * m[q]) * _c(yp) * yh + chi3 * (np.abs(yp) ** 2 + 2 * np.abs(yh) ** 2) * yp
            kh = (rel * g[1] * (1. / m[q]) * .5) * yp ** 2 + 2. * chi3 * (np.abs(yh) ** 2 + 2 * np.abs(yp) ** 2) * yh
            out.append(np.stack([kp, kh], axis=1))
            dp, dh = kp, kh
        return tuple(out)


class Chi2ASHG(FullyNonlinearMedium):
    """solvers/Chi2ASHG.cpp:6-56 (chirped mismatch, no poling)."""
    n_signal_modes = 2
    name = "Chi2ASHG"

    def __init__(self, relativeLength, nlLengthH, nlLengthP, beta2h, beta2p, beta1h=0.0, beta1p=0.0, beta3h=0.0,
                 beta3p=0.0, diffBeta0Start=0.0, diffBeta0End=0.0, rayleighLength=INF, tMax=10.0, tPrecision=512,
                 zPrecision=100, intensityProfile=GAUSSIAN_BEAM):
        super().__init__(False, relativeLength, [0.5 * math.pi * nlLengthP, 0.5 * math.pi * nlLengthH],
                         [beta2p, beta2h], [beta1p, beta1h], [beta3p, beta3h], [diffBeta0Start, diffBeta0End],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile)

    chirped = Chi2AFC.chirped

    def diff_eq(self, i, a):
        r = (self.relative_amplitude(i - 1), self.relative_amplitude(i - .5), self.relative_amplitude(i))
        m = self.chirped(i)
        g = self.nl_step
        xp, xh = a[:, 0], a[:, 1]
        sel = (0, 1, 1, 2)
        out, dp, dh = [], 0, 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            q = sel[st]
            yp, yh = xp + fac * dp, xh + fac * dh
            kp = (r[q] * g[0] * m[q]) * _c(yp) * yh
            kh = (r[q] * g[1] * (1. / m[q]) * .5) * yp ** 2
            out.append(np.stack([kp, kh], axis=1))
            dp, dh = kp, kh
        return tuple(out)


class Chi3GNLSE(FullyNonlinearMedium):
    """solvers/Chi3GNLSE.cpp:6-92 (Raman convolution and self-steepening)."""
    n_signal_modes = 1
    name = "Chi3GNLSE"

    def __init__(self, relativeLength, nlLength, selfSteepLength, fr, fb, tau1, tau2, tau3, beta2, beta3=0.0,
                 rayleighLength=INF, tMax=10.0, tPrecision=512, zPrecision=100, intensityProfile=GAUSSIAN_BEAM):
        super().__init__(False, relativeLength, [nlLength, selfSteepLength], [beta2], [0], [beta3], [],
                         rayleighLength, tMax, tPrecision, zPrecision, intensityProfile)
        n = self.n_freqs
        c1 = fr * (1. - fb) * (tau1 / (tau2 * tau2) + 1. / tau1)
        c2 = fr * fb / (tau3 * tau3)
        t = self.tau[:n // 2]
        rt = np.zeros(n, dtype=np.complex128)
        rt[:n // 2] = c1 * np.exp(-t / tau2) * np.sin(t / tau1) + c2 * np.exp(-t / tau3) * (2 * tau3 - t)
        rt[0] += 1. - fr
        self.raman_response = fft(rt)

    def diff_eq(self, i, a):
        r = (self.relative_intensity(i - 1), self.relative_intensity(i - .5), self.relative_intensity(i))
        steep = self.nl_step[0] + self.nl_step[1] * self.omega
        x = a[:, 0]
        sel = (0, 1, 1, 2)
        out, d = [], 0
        for st in range(4):
            fac = 0.0 if st == 0 else (1.0 if st == 3 else 0.5)
            y = x + fac * d
            conv = ifft(fft(r[sel[st]] * np.abs(y) ** 2) * self.raman_response)
            k = ifft(fft(conv * y) * steep)
            out.append(k[:, None])
            d = k
        return tuple(out)


SOLVERS = {cls.name: cls for cls in (Chi3, Chi2PDC, Chi2SFG, Chi2AFC, Chi2SFGPDC, Chi2SFGII, Chi2PDCII, Chi2SFGOPA,
                                     Chi2SFGXPM, Chi2SHG, Chi2SHGOPA, Chi2DSFG, Chi2SHGXPM, Chi2ASHG, Chi3GNLSE)}


class Cascade:
    """Restatement of ``Cascade`` (src/Cascade.cpp:3-167)."""

    def __init__(self, media, connections, share_pump):
        if len(media) == 0:
            raise ValueError("Cascade must contain at least one medium")
        n, t = media[0].n_freqs, media[0].t_max
        for med in media:
            if med.n_freqs != n or med.t_max != t:
                raise ValueError("Medium does not have same time and frequency axes as the first")
        if len(connections) != len(media) - 1:
            raise ValueError("Must have one connection per pair of adjacent media")
        for i, conn in enumerate(connections):
            if len(conn) == 0:
                raise ValueError("Connections missing between media!")
            for k, v in conn.items():
                if v >= media[i].n_signal_modes or k >= media[i + 1].n_signal_modes:
                    raise ValueError("Invalid connections, out of range")
        self.media = list(media)
        self.connections = [dict(c) for c in connections]
        self.shared = bool(share_pump)
        self.n_freqs = n

    def run_pump_simulation(self):
        """src/Cascade.cpp:75-88."""
        if not self.shared:
            for med in self.media:
                med.run_pump_simulation()
        else:
            self.media[0].run_pump_simulation()
            for i in range(1, len(self.media)):
                self.media[i].envelope[0] = self.media[i - 1].pump_time[0][-1].copy()
                self.media[i].run_pump_simulation()

    def run_signal_simulation(self, input_prof, in_time_domain=True, input_mode=0):
        """src/Cascade.cpp:91-107."""
        n = self.n_freqs
        self.media[0].run_signal_simulation(input_prof, in_time_domain, input_mode)
        for i in range(1, len(self.media)):
            conn = self.connections[i - 1]
            nxt = np.zeros(n * (max(conn.keys()) + 1), dtype=np.complex128)
            for k, v in conn.items():
                nxt[k * n:(k + 1) * n] = self.media[i - 1].signal_freq[v][-1]
            self.media[i].run_signal_simulation(nxt, False)

    def compute_greens_function(self, in_time_domain=False, run_pump=True, n_threads=1, normalize=False,
                                use_input=(), use_output=()):
        """src/Cascade.cpp:110-135 (connections are not used by the composition)."""
        if run_pump:
            self.run_pump_simulation()
        last = len(self.media) - 1
        c, s = self.media[0].compute_greens_function(in_time_domain, False, n_threads, normalize, use_input,
                                                     use_output if last == 0 else ())
        for i in range(1, len(self.media)):
            ci, si = self.media[i].compute_greens_function(in_time_domain, False, n_threads, normalize, (),
                                                           use_output if i == last else ())
            c, s = ci @ c + si @ np.conj(s), ci @ s + si @ np.conj(c)
        return c, s

    def batch_signal_simulation(self, input_profs, in_time_domain=False, run_pump=True, n_threads=1, input_mode=0,
                                use_output=()):
        """src/Cascade.cpp:138-167."""
        if run_pump:
            self.run_pump_simulation()
        out = Medium.batch_signal_simulation(self.media[0], input_profs, in_time_domain, False, n_threads, input_mode)
        last = len(self.media) - 1
        for i in range(1, len(self.media)):
            if i != last:
                out = Medium.batch_signal_simulation(self.media[i], out, in_time_domain, False, n_threads)
            else:
                out = Medium.batch_signal_simulation(self.media[i], out, in_time_domain, False, n_threads, 0,
                                                     use_output)
        return out
