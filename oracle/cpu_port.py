"""Python front of the C++ restatement (oracle/nlm_cpu.cpp): the timed CPU baseline.

TEST INFRASTRUCTURE ONLY.  The set-up of a medium (lengths, grids, dispersion, poling, envelope) comes
from the numpy oracle (oracle/nlm_oracle.py), which restates src/_NonlinearMedium.cpp:43-222; the
C++ library then runs what the reference spends its time on: the pump grid, the impulse or row
propagations over std::threads, and the Green's-function assembly.
"""

import numpy as np

from oracle import build_oracle


def _ptr(a):
    return a.ctypes.data if a is not None else None


def _c128(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _strength(med):
    """Row factors of the pump's intensity profile (src/_NonlinearMedium.cpp:236-248), or None."""
    from oracle import nlm_oracle as O
    if med.intensity_profile == O.CONSTANT:
        return None
    zl = O.linspaced(med.n_z_steps_p, -0.5 * med.z, 0.5 * med.z) / med.rayleigh_length
    if med.intensity_profile == O.GAUSSIAN_APODIZATION:
        return _f64(np.exp(-0.5 * zl ** 2))
    return _f64(1 / np.sqrt(1 + zl ** 2))


def chi2pdc_green(med, threads=1):
    """computeGreensFunction() of an oracle Chi2PDC medium (defaults: frequency domain, pump run,
    no normalisation): returns (C, S), N x N complex128."""
    n = med.n_freqs
    env, dp, ds, pol = _c128(med.envelope[0]), _f64(med.disp_pump[0]), _f64(med.disp_sign[0]), _f64(med.poling)
    strength = _strength(med)
    C = np.empty((n, n), dtype=np.complex128)
    S = np.empty_like(C)
    rc = build_oracle.load().nlmcpu_chi2pdc_green(n, med.n_z_steps, med.n_z_steps_p, med.dz, med.dzp, _ptr(env),
                                                  _ptr(dp), _ptr(ds), _ptr(pol), med.nl_step[0].imag,
                                                  float(med.diff_beta0[0]), _ptr(strength), int(threads),
                                                  _ptr(C), _ptr(S))
    if rc != 0:
        raise ValueError("the CPU restatement takes power-of-two grids and at least two z steps")
    return C, S


def chi2pdc_impulses(med, start, count, threads=1):
    """Output spectra of the impulse propagations [start, start + count) of the Green's function
    (instance 2 b + {0: 1, 1: i} at bin b) with the medium's current pump grid: count x N."""
    n = med.n_freqs
    pt = _c128(med.pump_time[0])
    out = np.empty((count, n), dtype=np.complex128)
    rc = build_oracle.load().nlmcpu_chi2pdc_impulses(n, med.n_z_steps, med.n_z_steps_p, med.dz, med.dzp, _ptr(pt),
                                                     _ptr(_f64(med.disp_sign[0])), _ptr(_f64(med.poling)),
                                                     med.nl_step[0].imag, float(med.diff_beta0[0]), int(start),
                                                     int(count), int(threads), _ptr(out))
    if rc != 0:
        raise ValueError("the CPU restatement takes power-of-two grids and at least two z steps")
    return out


def _gnlse_tables(med):
    rel = np.array([[med.relative_intensity(i - 1), med.relative_intensity(i - .5), med.relative_intensity(i)]
                    for i in range(1, med.n_z_steps)], dtype=np.float64).reshape(-1)
    return _f64(med.disp_sign[0]), _c128(med.raman_response), _c128(med.nl_step[0] + med.nl_step[1] * med.omega), rel


def gnlse_record(med, x, in_time_domain, every):
    """One Chi3GNLSE propagation of x (N values) recording the spectrum after steps every, 2 every,
    ... (< nZSteps-1): returns (rows x N recorded spectra, the last row in the input's domain)."""
    n = med.n_freqs
    disp, raman, steep, rel = _gnlse_tables(med)
    x = _c128(x).reshape(-1)
    rec = np.empty(((med.n_z_steps - 2) // every, n), dtype=np.complex128)
    out = np.empty(n, dtype=np.complex128)
    rc = build_oracle.load().nlmcpu_gnlse_record(n, med.n_z_steps, med.dz, _ptr(disp), _ptr(raman), _ptr(steep),
                                                 _ptr(rel), _ptr(x), int(bool(in_time_domain)), int(every),
                                                 _ptr(rec), _ptr(out))
    if rc != 0:
        raise ValueError("the CPU restatement takes power-of-two grids and at least two z steps")
    return rec, out


def gnlse_batch(med, inputs, in_time_domain=False, threads=1):
    """batchSignalSimulation of an oracle Chi3GNLSE medium: rows x N inputs, rows x N outputs."""
    n = med.n_freqs
    x = _c128(np.atleast_2d(inputs))
    rel = np.array([[med.relative_intensity(i - 1), med.relative_intensity(i - .5), med.relative_intensity(i)]
                    for i in range(1, med.n_z_steps)], dtype=np.float64).reshape(-1)
    steep = _c128(med.nl_step[0] + med.nl_step[1] * med.omega)
    raman = _c128(med.raman_response)
    out = np.empty_like(x)
    rc = build_oracle.load().nlmcpu_gnlse_batch(n, med.n_z_steps, med.dz, _ptr(_f64(med.disp_sign[0])), _ptr(raman),
                                                _ptr(steep), _ptr(rel), x.shape[0], _ptr(x), int(bool(in_time_domain)),
                                                int(threads), _ptr(out))
    if rc != 0:
        raise ValueError("the CPU restatement takes power-of-two grids and at least two z steps")
    return out
