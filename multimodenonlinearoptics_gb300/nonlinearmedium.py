"""Drop-in Python API of the reference's ``nonlinearmedium`` module, on the GB300 engine.

Same class names, constructor keywords and defaults, method names, keyword arguments,
return types and exception types as the pybind11 module of MultimodeNonlinearOptics
(src/nlmModulePy.cpp:12-217 and the ``#ifdef NLMMODULE`` block of every solvers/*.cpp).
This file is only the binding: every method is one call into the C ABI of
``libnlm_gb300.so`` (include/nlm_capi.h), where the host engine and the CUDA kernels live.

Differences a user can observe, all deliberate:
* ``nThreads`` is validated like the reference but the work runs on the GPU.
* The grid properties (``pumpTime``, ``signalFreq`` ...) are read-only views of a host
  mirror that is refreshed from the GPU each time the property is read.
* ``useInput``/``useOutput`` are read as 0/1 masks (the reference's own selection rule);
  combinations for which the reference reads past its mode list raise nothing here.
"""

import ctypes
import enum
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBPATH = os.path.join(_HERE, "libnlm_gb300.so")


class NoDeviceError(RuntimeError):
    """No CUDA device is usable; this engine has no CPU fallback."""


class UnsupportedError(RuntimeError):
    """The requested grid is outside what the fused kernels implement."""


def _load():
    if not os.path.exists(_LIBPATH):
        raise ImportError("libnlm_gb300.so is not built: run multimodenonlinearoptics_gb300.build_ext.build()")
    lib = ctypes.CDLL(_LIBPATH)
    P = ctypes.POINTER
    d, u8, sz, i, u = ctypes.c_double, ctypes.c_uint8, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint
    vp = ctypes.c_void_p
    sigs = {
        "nlm_last_error": (ctypes.c_char_p, []),
        "nlm_version": (ctypes.c_char_p, []),
        "nlm_solver_count": (i, []),
        "nlm_solver_name": (ctypes.c_char_p, [i]),
        "nlm_solver_signature": (ctypes.c_char_p, [ctypes.c_char_p]),
        "nlm_create": (i, [ctypes.c_char_p, P(d), sz, P(d), sz, P(d), sz, P(vp)]),
        "nlm_destroy": (i, [vp]),
        "nlm_info": (i, [vp, P(i), P(i), P(i), P(i), P(i), P(i), P(i)]),
        "nlm_lengths": (i, [vp, P(d), P(d), P(d), P(d)]),
        "nlm_set_pump_type": (i, [vp, i, d, d, u]),
        "nlm_set_pump_custom": (i, [vp, P(d), sz, d, d, u]),
        "nlm_set_pump_from": (i, [vp, vp, u, d, u]),
        "nlm_run_pump": (i, [vp]),
        "nlm_run_signal": (i, [vp, P(d), sz, i, u]),
        "nlm_green_dims": (i, [vp, u, P(u8), sz, P(u8), sz, P(sz), P(sz)]),
        "nlm_green": (i, [vp, i, i, u, i, P(u8), sz, P(u8), sz, P(d), P(d)]),
        "nlm_green_device": (i, [vp, i, i, u, i, P(u8), sz, P(u8), sz, vp, vp]),
        "nlm_green_plain": (i, [vp, i, i, sz, P(d), P(d)]),
        "nlm_batch_dims": (i, [vp, sz, sz, u, u, P(u8), sz, P(sz)]),
        "nlm_batch": (i, [vp, P(d), sz, sz, i, i, u, u, P(u8), sz, P(d)]),
        "nlm_batch_device": (i, [vp, vp, sz, sz, i, i, u, u, P(u8), sz, vp]),
        "nlm_ragged_batch": (i, [P(vp), sz, P(P(d)), i, P(P(d))]),
        "nlm_ragged_last_plan": (i, [P(d), P(i), P(i), P(i), P(i), P(ctypes.c_long), P(ctypes.c_long), P(i), P(i),
                                     P(d)]),
        "nlm_ragged_plan": (i, [sz, P(u), P(u), P(u), P(i), P(i), P(u), i, i, i, i, P(d), P(i), P(i), P(i), P(d)]),
        "nlm_get_grid": (i, [vp, i, u, P(P(d)), P(sz), P(sz)]),
        "nlm_get_axis": (i, [vp, i, u, P(P(d)), P(sz)]),
        "nlm_cascade_create": (i, [P(vp), sz, P(u), P(sz), sz, i, P(vp)]),
        "nlm_cascade_add": (i, [vp, vp, P(u), sz]),
        "nlm_cascade_media": (i, [vp, P(sz)]),
        "nlm_set_stream": (i, [vp, vp]),
        "nlm_synchronize": (i, [vp]),
        "nlm_device_available": (i, []),
        "nlm_set_schedule": (i, [vp, i, i, i]),
        "nlm_set_precision": (i, [vp, i]),
        "nlm_set_cluster": (i, [vp, i]),
        "nlm_graph_stats": (i, [vp, P(ctypes.c_long), P(ctypes.c_long)]),
        "nlm_last_schedule": (i, [vp, P(i)]),
        "nlm_last_launch_count": (i, [vp, P(ctypes.c_long)]),
        "nlm_kernel_timing": (i, [vp, i, P(d), P(ctypes.c_long)]),
        "nlm_set_poling_profile": (i, [vp, P(d), sz]),
        "nlm_green_rows": (i, [vp, i, i, sz, sz, P(d)]),
        "nlm_green_finish": (i, [vp, P(d), i, P(d), P(d)]),
        "nlm_green_rows_device": (i, [vp, i, i, sz, sz, vp]),
        "nlm_green_finish_device": (i, [vp, vp, i, vp, vp]),
        "nlm_adjoint_forward": (i, [vp, vp, sz, vp, i, P(i)]),
        "nlm_adjoint_backward": (i, [vp, vp, vp, vp, P(d)]),
        "nlm_fp64_peak": (i, [P(d)]),
        "nlm_fp64_mma_peak": (i, [P(d)]),
        "nlm_fp64_warps_rate": (i, [i, P(d)]),
        "nlm_quadrature_greens": (i, [vp, vp, sz, sz, vp, vp]),
        "nlm_abasis_greens": (i, [vp, vp, sz, sz, vp, vp]),
        "nlm_cascade_compose": (i, [vp, vp, vp, vp, sz, sz, sz, vp, vp, vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_lib = _load()

_ERRORS = {1: ValueError, 2: RuntimeError, 3: IndexError, 4: RuntimeError, 5: NoDeviceError, 6: UnsupportedError,
           7: RuntimeError}


def _check(status):
    if status != 0:
        msg = _lib.nlm_last_error().decode()
        raise _ERRORS.get(status, RuntimeError)(msg)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _complex1d(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))


def _mask(v):
    v = [] if v is None else list(v)
    arr = (ctypes.c_uint8 * max(1, len(v)))(*[int(x) & 0xFF for x in v])
    return arr, len(v)


def device_available():
    """True when a CUDA device is usable by this process."""
    return bool(_lib.nlm_device_available())


def ragged_batch(media, inputs, inTimeDomain=False):
    """Propagate one signal through each medium of a ragged set in one persistent launch.

    No counterpart in the reference, which would call batchSignalSimulation once per medium
    (src/_NonlinearMedium.cpp:378-444).  media: list of media (pumps already run); inputs: one
    N-point spectrum (or time profile) per medium for its first mode.  Returns, per medium, the last
    row of all its signal modes (nSignalModes x N).
    """
    media = list(media)
    ins = [_complex1d(x) for x in inputs]
    if len(ins) != len(media):
        raise ValueError("one input per medium")
    outs = []
    for m, x in zip(media, ins):
        d = m._dims
        if x.size != d["nFreqs"]:
            raise ValueError("input length does not match the medium's nFreqs")
        outs.append(np.empty((d["nSignalModes"], d["nFreqs"]), dtype=np.complex128))
    P = ctypes.POINTER(ctypes.c_double)
    hs = (ctypes.c_void_p * len(media))(*[m._h() for m in media])
    ip = (P * len(media))(*[_dptr(x.view(np.float64)) for x in ins])
    op = (P * len(media))(*[_dptr(o.view(np.float64)) for o in outs])
    _check(_lib.nlm_ragged_batch(hs, len(media), ip, int(bool(inTimeDomain)), op))
    return outs


def ragged_last_plan():
    """The plan of the last ragged_batch call (no counterpart in the reference): estimated makespan
    (ms), cluster slots of four, eight and sixteen SMs, CTAs of the one-SM ragged launches, the
    CUDA-graph captures and replays of ragged calls so far, the SMs the plan could use, the
    sixteen-SM slots that can run at once and the call's device time (ms)."""
    ms, c4, w8, w16, ctas = ctypes.c_double(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    cap, rep, budget, w16cap = ctypes.c_long(), ctypes.c_long(), ctypes.c_int(), ctypes.c_int()
    gpu = ctypes.c_double()
    _check(_lib.nlm_ragged_last_plan(ctypes.byref(ms), ctypes.byref(c4), ctypes.byref(w8), ctypes.byref(w16),
                                     ctypes.byref(ctas), ctypes.byref(cap), ctypes.byref(rep), ctypes.byref(budget),
                                     ctypes.byref(w16cap), ctypes.byref(gpu)))
    return {"makespan_estimate_ms": ms.value / 1e3, "slots_c4": c4.value, "slots_w8": w8.value,
            "slots_w16": w16.value, "ragged_ctas": ctas.value, "graph_captures": cap.value,
            "graph_replays": rep.value, "sm_budget": budget.value, "w16_capacity": w16cap.value,
            "gpu_ms": gpu.value}


def ragged_plan(n_freqs, n_modes, n_z_steps, propagator, launch_class, forms, cluster_sms=128, w16_slots=7,
                pool_sms=152, pool_granularity=1):
    """ragged_batch's makespan planner alone, with no device work (no counterpart in the reference).

    Per medium: its grid, signal mode count, nZSteps, whether its RK4 matrices are used, its
    ragged-launch class (one solver and one grid) and a mask of its available forms (bit 0 one SM,
    bits 1-3 clusters of 4, 8 and 16 SMs).  The budgets default to a GB300's.  Returns the plan's
    makespan in microseconds (None when no plan fits the SMs at once), each medium's form and cluster
    slot (-1: a ragged launch), the ragged launches' CTAs and each medium's estimated march time per
    form (microseconds, n x 4; -1 where the form is not available)."""
    n = len(n_freqs)
    arrs = [np.ascontiguousarray(v, dtype=t) for v, t in
            ((n_freqs, np.uint32), (n_modes, np.uint32), (n_z_steps, np.uint32), (propagator, np.int32),
             (launch_class, np.int32), (forms, np.uint32))]
    if any(a.shape != (n,) for a in arrs):
        raise ValueError("every per-medium array needs one entry per medium")
    ms, ctas = ctypes.c_double(), ctypes.c_int()
    form, slot, times = np.empty(n, np.int32), np.empty(n, np.int32), np.empty((n, 4), np.float64)
    ptr = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))
    _check(_lib.nlm_ragged_plan(n, ptr(arrs[0], ctypes.c_uint), ptr(arrs[1], ctypes.c_uint),
                                ptr(arrs[2], ctypes.c_uint), ptr(arrs[3], ctypes.c_int), ptr(arrs[4], ctypes.c_int),
                                ptr(arrs[5], ctypes.c_uint), int(cluster_sms), int(w16_slots), int(pool_sms),
                                int(pool_granularity), ctypes.byref(ms), ptr(form, ctypes.c_int),
                                ptr(slot, ctypes.c_int), ctypes.byref(ctas), ptr(times, ctypes.c_double)))
    return {"makespan_us": ms.value if ms.value >= 0 else None, "form": form, "slot": slot,
            "ragged_ctas": ctas.value, "times_us": times}


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s, FMA = 2 flops)."""
    v = ctypes.c_double()
    _check(_lib.nlm_fp64_peak(ctypes.byref(v)))
    return v.value


def fp64_warps_rate_tflops(warps_per_sm):
    """Measured FP64 FMA throughput (TFLOP/s) with one CTA of `warps_per_sm` warps on every SM."""
    v = ctypes.c_double()
    _check(_lib.nlm_fp64_warps_rate(int(warps_per_sm), ctypes.byref(v)))
    return v.value


def fp64_mma_peak_tflops():
    """Measured FP64 tensor-core (DMMA) throughput of the current device (TFLOP/s)."""
    v = ctypes.c_double()
    _check(_lib.nlm_fp64_mma_peak(ctypes.byref(v)))
    return v.value


class PulseType(enum.IntEnum):
    """Pump envelope shape (src/_NonlinearMedium.hpp:25-29)."""
    Gaussian = 0
    Sech = 1
    Sinc = 2


class IntensityProfile(enum.IntEnum):
    """Pump intensity along z (src/_NonlinearMedium.hpp:30-34)."""
    GaussianBeam = 0
    Constant = 1
    GaussianApodization = 2


Gaussian, Sech, Sinc = PulseType.Gaussian, PulseType.Sech, PulseType.Sinc
GaussianBeam, Constant, GaussianApodization = (IntensityProfile.GaussianBeam, IntensityProfile.Constant,
                                                IntensityProfile.GaussianApodization)


class _NonlinearMedium:
    """Base class for nonlinear medium solvers (src/_NonlinearMedium.hpp:20-142)."""

    _handle = None

    def _h(self):
        if self._handle is None:
            raise RuntimeError("medium is not initialised")
        return self._handle

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and _lib is not None:
            _lib.nlm_destroy(h)
            self._handle = None

    def _info(self):
        vals = [ctypes.c_int() for _ in range(7)]
        _check(_lib.nlm_info(self._h(), *[ctypes.byref(v) for v in vals]))
        return [v.value for v in vals]

    # -- setPump (src/nlmModulePy.cpp:33-59) ------------------------------------------------
    def setPump(self, *args, **kwargs):
        """Set the input shape of the pump.

        setPump(pulseType, chirp=0, delay=0, pumpIndex=0)
        setPump(customPump, chirp=0, delay=0, pumpIndex=0)
        setPump(other, modeIndex=0, delay=0, pumpIndex=0)
        """
        first = args[0] if args else kwargs.pop("pulseType", kwargs.pop("customPump", kwargs.pop("other", None)))
        rest = list(args[1:])
        if isinstance(first, _NonlinearMedium):
            names, defaults = ["modeIndex", "delay", "pumpIndex"], [0, 0.0, 0]
        else:
            names, defaults = ["chirp", "delay", "pumpIndex"], [0.0, 0.0, 0]
        vals = _bind(names, defaults, rest, kwargs, "setPump")
        if isinstance(first, _NonlinearMedium):
            _check(_lib.nlm_set_pump_from(self._h(), first._h(), int(vals[0]), float(vals[1]), int(vals[2])))
        elif isinstance(first, (PulseType, int, np.integer)) and not isinstance(first, bool):
            _check(_lib.nlm_set_pump_type(self._h(), int(first), float(vals[0]), float(vals[1]), int(vals[2])))
        else:
            p = _complex1d(first)
            _check(_lib.nlm_set_pump_custom(self._h(), _dptr(p.view(np.float64)), p.size, float(vals[0]),
                                            float(vals[1]), int(vals[2])))

    def runPumpSimulation(self):
        """Simulate propagation of the pump field."""
        _check(_lib.nlm_run_pump(self._h()))

    def runSignalSimulation(self, inputProf, inTimeDomain=True, inputMode=0):
        """Simulate propagation of the signal field(s) (src/_NonlinearMedium.cpp:253-260)."""
        p = _complex1d(inputProf)
        _check(_lib.nlm_run_signal(self._h(), _dptr(p.view(np.float64)), p.size, int(bool(inTimeDomain)),
                                   int(inputMode)))

    def computeGreensFunction(self, inTimeDomain=False, runPump=True, nThreads=1, normalize=False, useInput=(),
                              useOutput=()):
        """Green's function matrices C, S with a(L) = C a(0) + S a(0)^* (src/_NonlinearMedium.cpp:263-375)."""
        mi, ni = _mask(useInput)
        mo, no = _mask(useOutput)
        rows, cols = ctypes.c_size_t(), ctypes.c_size_t()
        _check(_lib.nlm_green_dims(self._h(), int(nThreads), mi, ni, mo, no, ctypes.byref(rows), ctypes.byref(cols)))
        C = np.empty((rows.value, cols.value), dtype=np.complex128)
        S = np.empty_like(C)
        _check(_lib.nlm_green(self._h(), int(bool(inTimeDomain)), int(bool(runPump)), int(nThreads),
                              int(bool(normalize)), mi, ni, mo, no, _dptr(C.view(np.float64)),
                              _dptr(S.view(np.float64))))
        return C, S

    def batchSignalSimulation(self, inputProfs, inTimeDomain=False, runPump=True, nThreads=1, inputMode=0,
                              useOutput=()):
        """Run multiple signal simulations (src/_NonlinearMedium.cpp:378-444)."""
        return self._batch(inputProfs, inTimeDomain, runPump, nThreads, inputMode, useOutput)

    def _batch(self, inputProfs, inTimeDomain, runPump, nThreads, inputMode, useOutput):
        x = np.asarray(inputProfs, dtype=np.complex128)
        if x.ndim == 1:
            x = x.reshape(1, -1)
        x = np.ascontiguousarray(x)
        rows, cols = x.shape
        mo, no = _mask(useOutput)
        oc = ctypes.c_size_t()
        _check(_lib.nlm_batch_dims(self._h(), rows, cols, int(nThreads), int(inputMode), mo, no, ctypes.byref(oc)))
        out = np.empty((rows, oc.value), dtype=np.complex128)
        _check(_lib.nlm_batch(self._h(), _dptr(x.view(np.float64)), rows, cols, int(bool(inTimeDomain)),
                              int(bool(runPump)), int(nThreads), int(inputMode), mo, no, _dptr(out.view(np.float64))))
        return out

    # -- getters (src/nlmModulePy.cpp:100-123) ----------------------------------------------
    def _grid(self, which, i):
        ptr = ctypes.POINTER(ctypes.c_double)()
        rows, cols = ctypes.c_size_t(), ctypes.c_size_t()
        _check(_lib.nlm_get_grid(self._h(), which, int(i), ctypes.byref(ptr), ctypes.byref(rows), ctypes.byref(cols)))
        n = rows.value * cols.value
        if n == 0:
            return np.zeros((rows.value, cols.value), dtype=np.complex128)
        arr = np.ctypeslib.as_array(ptr, shape=(2 * n,)).view(np.complex128).reshape(rows.value, cols.value)
        arr.flags.writeable = False
        return arr

    def _axis(self, which, i=0, complex_=False):
        ptr = ctypes.POINTER(ctypes.c_double)()
        n = ctypes.c_size_t()
        _check(_lib.nlm_get_axis(self._h(), which, int(i), ctypes.byref(ptr), ctypes.byref(n)))
        if n.value == 0:
            return np.zeros(0, dtype=np.complex128 if complex_ else np.float64)
        if complex_:
            arr = np.ctypeslib.as_array(ptr, shape=(2 * n.value,)).view(np.complex128)
        else:
            arr = np.ctypeslib.as_array(ptr, shape=(n.value,))
        arr.flags.writeable = False
        return arr

    omega = property(lambda self: self._axis(1), doc="Read-only frequency axis of the system.")
    tau = property(lambda self: self._axis(0), doc="Read-only time axis of the system")
    signalFreq = property(lambda self: self._grid(2, 0),
                          doc="Read-only array of the signal frequency profile along the length of the medium.")
    signalTime = property(lambda self: self._grid(3, 0),
                          doc="Read-only array of a signal time profile along the length of the medium.")
    pumpFreq = property(lambda self: self._grid(0, 0),
                        doc="Read-only array of the pump frequency profile along the length of the medium.")
    pumpTime = property(lambda self: self._grid(1, 0),
                        doc="Read-only array of the pump time profile along the length of the medium.")
    poling = property(lambda self: self._axis(2),
                      doc="Read-only array of the domain poling along the length of a Chi(2) medium.")

    def signalFreqs(self, i=0):
        return self._grid(2, i)

    def signalTimes(self, i=0):
        return self._grid(3, i)

    def pumpFreqs(self, i=0):
        return self._grid(0, i)

    def pumpTimes(self, i=0):
        return self._grid(1, i)

    def field(self, i=0):
        return self._grid(4, i)

    # -- engine controls (no counterpart in the reference) ------------------------------------
    def _set_schedule(self, cta_per_sm=0, use_propagator=-1, use_graph=1):
        _check(_lib.nlm_set_schedule(self._h(), int(cta_per_sm), int(use_propagator), int(use_graph)))

    def _set_cluster(self, enable):
        """Spread each propagation of small launches over a 4-CTA cluster: 1 (default) with one point
        per thread on 128..1024-point grids (and the Chi3 pump march there), full grids in the widest
        form (eight CTAs at 1024 points, sixteen at 2048 and 4096 where the solver has it), and a Chi3
        runPumpSimulation followed by runSignalSimulation as one launch of both marches side by side on
        eight CTAs; 3 the same without the widest forms (full grids on four CTAs up to 1024 points,
        eight above) and with the two Chi3 marches one after the other; 2 four
        points per thread only (grids of 1024 points and more); 0 one CTA per propagation."""
        _check(_lib.nlm_set_cluster(self._h(), int(enable)))

    def _set_precision(self, precision):
        """"f64" (default) or "ff": double-float arithmetic (FP32 pairs, ~48-bit significand) for the
        single-mode precomputed-propagator kernel; every other path stays FP64."""
        code = {"f64": 0, "ff": 1}.get(precision)
        if code is None:
            raise ValueError("precision must be 'f64' or 'ff'")
        _check(_lib.nlm_set_precision(self._h(), code))

    def _kernel_timing(self, enable):
        ms, cnt = ctypes.c_double(), ctypes.c_long()
        _check(_lib.nlm_kernel_timing(self._h(), int(enable), ctypes.byref(ms), ctypes.byref(cnt)))
        return ms.value, cnt.value

    def _set_poling_profile(self, profile):
        """Continuous poling d(z) on the nZSteps grid in place of the domain pattern (no reference counterpart)."""
        p = np.ascontiguousarray(np.asarray(profile, dtype=np.float64).ravel())
        _check(_lib.nlm_set_poling_profile(self._h(), _dptr(p), p.size))

    def _set_stream(self, stream_handle):
        _check(_lib.nlm_set_stream(self._h(), ctypes.c_void_p(stream_handle)))

    def _last_schedule(self):
        """Launch shape of the last propagation (R, ipc, grid, block, CTAs per SM, tuned, trials,
        registers per thread of the kernel variant)."""
        v = (ctypes.c_int * 8)()
        _check(_lib.nlm_last_schedule(self._h(), v))
        return dict(zip(("R", "ipc", "grid", "block", "cta_per_sm", "tuned", "trials", "registers"), list(v)))

    def _graph_stats(self):
        """(captures, replays) of the CUDA graphs of this medium's batched propagations."""
        c, r = ctypes.c_long(), ctypes.c_long()
        _check(_lib.nlm_graph_stats(self._h(), ctypes.byref(c), ctypes.byref(r)))
        return c.value, r.value

    def _launch_count(self):
        v = ctypes.c_long()
        _check(_lib.nlm_last_launch_count(self._h(), ctypes.byref(v)))
        return v.value

    @property
    def _dims(self):
        nsig, npump, n, nz, nzp, fnl, casc = self._info()
        return {"nSignalModes": nsig, "nPumpModes": npump, "nFreqs": n, "nZSteps": nz, "nZStepsP": nzp,
                "fullyNonlinear": bool(fnl), "cascade": bool(casc)}

    @property
    def _lengths(self):
        v = [ctypes.c_double() for _ in range(4)]
        _check(_lib.nlm_lengths(self._h(), *[ctypes.byref(x) for x in v]))
        return {"z": v[0].value, "dz": v[1].value, "dzp": v[2].value, "tMax": v[3].value}


class _FullyNonlinearMedium(_NonlinearMedium):
    """Base class for fully nonlinear medium solvers (src/_FullyNonlinearMedium.hpp:6-69)."""

    def batchSignalSimulation(self, inputProfs, inTimeDomain=False, nThreads=1, inputMode=0, useOutput=()):
        """Run multiple signal simulations (src/_FullyNonlinearMedium.hpp:8-11)."""
        return self._batch(inputProfs, inTimeDomain, False, nThreads, inputMode, useOutput)

    def setPump(self, *args, **kwargs):
        raise RuntimeError("Object does not have this method.")

    def runPumpSimulation(self):
        raise RuntimeError("Object does not have this method.")

    def computeGreensFunction(self, inTimeDomain=False, runPump=True, nThreads=1, normalize=False, useInput=(),
                              useOutput=()):
        raise RuntimeError("Object does not have this method.")


def _bind(names, defaults, args, kwargs, fname):
    """Positional + keyword binding with pybind11's error type (TypeError)."""
    if len(args) > len(names):
        raise TypeError("%s(): incompatible function arguments" % fname)
    vals = list(args) + [None] * (len(names) - len(args))
    for k, v in kwargs.items():
        if k not in names:
            raise TypeError("%s(): incompatible function arguments (unexpected keyword %r)" % (fname, k))
        idx = names.index(k)
        if idx < len(args):
            raise TypeError("%s(): got multiple values for argument %r" % (fname, k))
        vals[idx] = v
    for idx, v in enumerate(vals):
        if v is None:
            if defaults[idx] is _REQUIRED:
                raise TypeError("%s(): missing required argument %r" % (fname, names[idx]))
            vals[idx] = defaults[idx]
    return vals


_REQUIRED = object()


def _parse_signature(sig):
    names, defaults = [], []
    for tok in sig.split(","):
        if "=" in tok:
            k, v = tok.split("=")
            names.append(k)
            defaults.append(float("inf") if v == "inf" else float(v))
        else:
            names.append(tok)
            defaults.append(None if tok.startswith("@") else _REQUIRED)
    return names, defaults


def _make_solver(name, base, doc):
    sig = _lib.nlm_solver_signature(name.encode()).decode()
    names, defaults = _parse_signature(sig)
    kw = [n.lstrip("@") for n in names]

    def __init__(self, *args, **kwargs):
        vals = _bind(kw, [d if d is not None else _ARRAY_DEFAULT for d in defaults], list(args), dict(kwargs), name)
        if name == "Chi2SFGII":
            # the reference binds the keyword "intensityProfile" to the zPrecision slot and "zPrecision"
            # to the intensityProfile slot (solvers/Chi2SFGII.cpp:98-106)
            iz, ip = kw.index("zPrecision"), kw.index("intensityProfile")
            if "intensityProfile" in kwargs or "zPrecision" in kwargs:
                zval = kwargs.get("intensityProfile", 100)
                pval = kwargs.get("zPrecision", IntensityProfile.GaussianBeam)
                vals[iz], vals[ip] = zval, pval
        scalars, pump, poling = [], None, None
        for k, v in zip(kw, vals):
            if k == "customPump":
                pump = None if v is _ARRAY_DEFAULT else _complex1d(v)
            elif k == "poling":
                poling = None if v is _ARRAY_DEFAULT else np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
            else:
                if isinstance(v, (np.ndarray, list, tuple)):
                    raise TypeError("%s(): incompatible constructor arguments (%s)" % (name, k))
                scalars.append(float(v))
        a = (ctypes.c_double * max(1, len(scalars)))(*scalars)
        h = ctypes.c_void_p()
        pp = _dptr(pump.view(np.float64)) if pump is not None and pump.size else None
        pl = _dptr(poling) if poling is not None and poling.size else None
        _check(_lib.nlm_create(name.encode(), a, len(scalars), pp, 0 if pump is None else pump.size, pl,
                               0 if poling is None else poling.size, ctypes.byref(h)))
        self._handle = h
        self._keep = None

    cls = type(name, (base,), {"__init__": __init__, "__doc__": doc, "_signature": kw})
    return cls


_ARRAY_DEFAULT = object()

_DOCS = {
    "Chi3": ("Single mode self phase modulation", _NonlinearMedium),
    "Chi2PDC": ("Degenerate optical parametric amplification", _NonlinearMedium),
    "Chi2SFG": ("Sum (or difference) frequency generation", _NonlinearMedium),
    "Chi2AFC": ("Adiabatic sum (or difference) frequency generation, in a rotating frame with linearly varying poling "
                "frequency built into the solver", _NonlinearMedium),
    "Chi2SFGPDC": ("Simultaneous sum frequency generation and parametric amplification", _NonlinearMedium),
    "Chi2SFGII": ("Type II or simultaneous 2-mode sum frequency generation with parametric amplification",
                  _NonlinearMedium),
    "Chi2PDCII": ("Type II or nondegenerate optical parametric amplification", _NonlinearMedium),
    "Chi2SFGOPA": ("Simultaneous sum frequency generation and non-degenerate optical parametric amplification with "
                   "two pumps", _NonlinearMedium),
    "Chi2SFGXPM": ("Sum (or difference) frequency generation with cross phase modulation", _NonlinearMedium),
    "Chi2SHG": ("Fully nonlinear second harmonic generation", _FullyNonlinearMedium),
    "Chi2SHGOPA": ("Fully nonlinear OPA driven by the second harmonic of the pump", _FullyNonlinearMedium),
    "Chi2DSFG": ("Sum (or difference) frequency generation with pump depletion (fully nonlinear)",
                 _FullyNonlinearMedium),
    "Chi2SHGXPM": ("Fully nonlinear second harmonic generation with self and cross phase modulation",
                   _FullyNonlinearMedium),
    "Chi2ASHG": ("Fully nonlinear adiabatic second harmonic generation", _FullyNonlinearMedium),
    "Chi3GNLSE": ("Fully nonlinear general nonlinear Schrodinger equation", _FullyNonlinearMedium),
}

SOLVERS = []
for _i in range(_lib.nlm_solver_count()):
    _name = _lib.nlm_solver_name(_i).decode()
    _doc, _base = _DOCS[_name]
    globals()[_name] = _make_solver(_name, _base, _doc)
    SOLVERS.append(_name)


def _raman(self):
    return self._axis(3, complex_=True)


globals()["Chi3GNLSE"].ramanResponse = property(_raman, doc="Read-only array of the Raman response function in the "
                                                            "frequency domain.")


class Cascade(_NonlinearMedium):
    """Chain of media (src/Cascade.hpp:6-45): outputs of one feed the inputs of the next."""

    def __init__(self, inputMedia, modeConnections, sharePump):
        media = list(inputMedia)
        conns = [dict(c) for c in modeConnections]
        flat, counts = [], []
        for c in conns:
            counts.append(len(c))
            for k, v in c.items():
                flat += [int(k), int(v)]
        hs = (ctypes.c_void_p * max(1, len(media)))(*[m._h() for m in media])
        cf = (ctypes.c_uint * max(1, len(flat)))(*flat)
        cc = (ctypes.c_size_t * max(1, len(counts)))(*counts)
        h = ctypes.c_void_p()
        if len(media) == 0:
            hs = None
        _check(_lib.nlm_cascade_create(hs, len(media), cf, cc, len(conns), int(bool(sharePump)), ctypes.byref(h)))
        self._handle = h
        self._media = media   # keeps the media alive, like py::keep_alive<1, 2>

    def addMedium(self, medium, connection):
        flat = []
        for k, v in dict(connection).items():
            flat += [int(k), int(v)]
        cf = (ctypes.c_uint * max(1, len(flat)))(*flat)
        _check(_lib.nlm_cascade_add(self._h(), medium._h(), cf, len(flat) // 2))
        self._media.append(medium)

    def setPump(self, *args, **kwargs):
        first = args[0] if args else kwargs.get("other")
        if isinstance(first, _NonlinearMedium):
            raise RuntimeError("Object does not have this method.")
        return _NonlinearMedium.setPump(self, *args, **kwargs)

    def __getitem__(self, i):
        return self._media[i]

    @property
    def media(self):
        return list(self._media)

    @property
    def nMedia(self):
        return len(self._media)
