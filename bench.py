"""Benchmark of the split-step propagation engine on the Green's-function workload.

Workload (one step): computeGreensFunction of Chi2PDC with nFreqs=1024, nZSteps=1000,
relativeLength=1, nlLength=0.5, Gaussian pump (beta2=1), signal beta2s=0.5, beta1s=2,
beta3s=0.1, poling period 20 z steps: 2*1024 impulse propagations, C and S 1024x1024 complex128.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is the device-resident throughput (propagations/s,
C and S left in HBM); `e2e` is the same metric through the public drop-in API
(computeGreensFunction returning numpy arrays, C/S copied to host every step).  The CPU
baseline is the numpy oracle (a restatement of the reference's algorithm: the reference's
C++ engine cannot be built without the Eigen headers) on a bounded sample of the same
impulses.  Under torchrun every rank computes its own copy of the workload (weak scaling).
"""

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Green's-fn propagations/s at 1e-9 rel err: batched vs plain GPU; grad/fwd cost"
UNIT = "propagations/s"
from multimodenonlinearoptics_gb300.workloads import (GNLSE_CONFIG, GREEN_CONFIG as CONFIG,  # noqa: E402
                                                     GREEN_DOMAINS as N_DOMAINS, ragged_media_params)

C_SOLVER = 80          # point-wise flops per mode per step of Chi2PDC's DiffEq (fixed, not tuned)


def algorithmic_flops(n_inst, n_z, n, modes=1, c_solver=C_SOLVER):
    """F = n_inst (nZ-1) modes (10 N log2 N + c N): two FFTs of 5 N log2 N plus the point-wise work."""
    return n_inst * (n_z - 1) * modes * (10 * n * math.log2(n) + c_solver * n)


# ----------------------------------------------------------------------------------------------
# clocks sampled during the timed region
# ----------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------------------------
# oracle: impulse propagations of the workload (CPU baseline and the parity sample)
# ----------------------------------------------------------------------------------------------
def _oracle_medium():
    from oracle import nlm_oracle as O
    med = O.Chi2PDC(poling=np.ones(N_DOMAINS), **CONFIG)
    med.run_pump_simulation()
    return med


def oracle_columns(med, bins):
    """Columns b' = (b + N/2) mod N of C and S for impulse bins b, from 2 propagations per bin."""
    n = med.n_freqs
    bins = np.asarray(bins)
    prof = np.zeros((bins.size, n), dtype=np.complex128)
    prof[np.arange(bins.size), bins] = 1.0
    f1, _ = med.propagate(prof, False, 0)
    fi, _ = med.propagate(1j * prof, False, 0)
    o1, oi = f1[:, 0], fi[:, 0]
    pre_c = 0.5 * o1 - 0.5j * oi
    pre_s = 0.5 * o1 + 0.5j * oi
    return np.fft.fftshift(pre_c, axes=1).T, np.fft.fftshift(pre_s, axes=1).T


_WORKER_MEDIUM = None


def _init_worker():
    global _WORKER_MEDIUM
    _WORKER_MEDIUM = _oracle_medium()


def _oracle_worker(bins):
    med = _WORKER_MEDIUM if _WORKER_MEDIUM is not None else _oracle_medium()
    t0 = time.perf_counter()
    oracle_columns(med, bins)
    return time.perf_counter() - t0


class OraclePool:
    """Oracle impulse propagations on every host core (spawned processes, one medium each)."""

    def __init__(self, processes):
        self.processes = processes
        self.pool = mp.get_context("spawn").Pool(processes, initializer=_init_worker)
        self.pool.map(_oracle_worker, [np.array([0])] * processes)   # imports and pump done

    def rate(self, n_bins, seed=0):
        rng = np.random.default_rng(seed)
        bins = rng.choice(CONFIG["tPrecision"], size=n_bins, replace=False)
        chunks = [c for c in np.array_split(bins, self.processes) if c.size]
        t0 = time.perf_counter()
        self.pool.map(_oracle_worker, chunks)
        dt = time.perf_counter() - t0
        return 2 * n_bins / dt, dt

    def close(self):
        self.pool.close()
        self.pool.join()


def _ragged_oracle_output(index):
    """Oracle output (all signal modes, last row) of ragged medium `index` at its full step count."""
    from oracle import nlm_oracle as O
    kw, doms, pump, sig = ragged_media_params()[index]
    t0 = time.perf_counter()
    o = O.Chi2SFG(customPump=pump, poling=doms, **kw)
    o.run_pump_simulation()
    f, _ = o.propagate(sig[None, :], False, 0)
    return index, f[0], o.n_z_steps, time.perf_counter() - t0


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


# ----------------------------------------------------------------------------------------------
def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_profile_value(key):
    """A figure of the committed ncu summary of the benchmark kernel (a line `key: value ...`)."""
    path = os.path.join(ROOT, "profiles", "k_propagate_linear_green_n1024.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def measured_hbm_gbs():
    """The measured HBM copy bandwidth of this machine's GPUs (MEASURED_PEAKS.json), when present."""
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs")
    except (OSError, ValueError):
        return None


def read_profile_traffic():
    return read_profile_value("dram_bytes_per_launch_full")


WORKLOAD = "Chi2PDC computeGreensFunction N=1024 nZSteps=1000 (2048 impulse propagations, C and S 1024x1024 complex128)"


def bench_config():
    """The config object of both arms' JSON lines (identical, so the two lines compare)."""
    return {"workload": WORKLOAD, "global_batch": 2 * CONFIG["tPrecision"], "seq_len": 2 * CONFIG["zPrecision"],
            "parallelism": "2048 independent impulse propagations per step",
            "l2": "inputs and outputs of a step: 2048 propagations x 1024 points; the GPU arm writes a 256 MB "
                  "buffer between timed steps"}


def run_reference(args):
    """The reference arm: the whole workload (one full computeGreensFunction of 2048 propagations per
    step) with the CPU restatement of the reference's C++ engine (oracle/nlm_cpu.cpp: the optimised
    split-step loop, a radix-4 FFT of its own, std::threads over contiguous impulse ranges) on every
    host core.  The reference's own engine needs the Eigen 3 headers, absent on this host."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import build_oracle, cpu_port
    build_oracle.build()
    cores = os.cpu_count() or 1
    med = _oracle_medium()
    for _ in range(args.warmup):
        cpu_port.chi2pdc_green(med, cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        C, S = cpu_port.chi2pdc_green(med, cores)
        times.append(time.perf_counter() - t0)
    n_inst = 2 * CONFIG["tPrecision"]
    value = n_inst * args.steps / float(np.sum(times))
    if not (np.all(np.isfinite(C)) and np.all(np.isfinite(S))):
        raise RuntimeError("the CPU restatement produced non-finite C/S")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "the whole workload every step: computeGreensFunction with the pump grid, "
                                   "2048 impulse propagations and the C/S assembly, on %d std::threads; C++ "
                                   "restatement of the reference's loop (oracle/nlm_cpu.cpp; the reference's "
                                   "engine needs Eigen, absent)" % cores},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _adjoint_costs(nlm, torch, n, cluster=1, reps=3, check=False):
    """fwd / grad times (ms) of the gradient configuration at n frequency bins: Chi2PDC with
    nZSteps=2000, one seeded noise signal (sigma 1e-3), continuous poling d(z) ~ U[-1, 1] (seed 4),
    loss ||X(L) - target||^2.  fwd = one forward propagation with the pump run
    (batchSignalSimulation); grad = forward with checkpoints + reverse sweep with the pump-spectrum
    and poling-profile reductions; with the engine's checkpoint interval and with sqrt(nZSteps)."""
    import ctypes
    kw = dict(CONFIG, tPrecision=n, zPrecision=1000)
    med = nlm.Chi2PDC(**kw)
    med._set_cluster(cluster)
    n, nz = med._dims["nFreqs"], med._dims["nZSteps"]
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-3 / np.sqrt(2)
    d = rng.uniform(-1, 1, nz)
    target = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    target /= np.linalg.norm(target)
    stream = torch.cuda.Stream()
    med._set_stream(stream.cuda_stream)
    med._set_poling_profile(d)
    xin = torch.tensor(x.reshape(1, n), dtype=torch.complex128, device="cuda")
    out = torch.empty_like(xin)
    gin = torch.empty_like(xin)
    gp = torch.empty(n, dtype=torch.complex128, device="cuda")
    gpol = np.zeros(nz)
    tt = torch.tensor(target.reshape(1, n), dtype=torch.complex128, device="cuda")
    used = ctypes.c_int()

    def fwd():
        nlm._check(nlm._lib.nlm_batch_device(med._h(), ctypes.c_void_p(xin.data_ptr()), 1, n, 0, 1, 1, 0, None, 0,
                                             ctypes.c_void_p(out.data_ptr())))

    def grad(interval):
        nlm._check(nlm._lib.nlm_run_pump(med._h()))
        nlm._check(nlm._lib.nlm_adjoint_forward(med._h(), ctypes.c_void_p(xin.data_ptr()), 1,
                                                ctypes.c_void_p(out.data_ptr()), interval, ctypes.byref(used)))
        with torch.cuda.stream(stream):
            g = (2 * (out - tt)).contiguous()
        nlm._check(nlm._lib.nlm_adjoint_backward(med._h(), ctypes.c_void_p(g.data_ptr()),
                                                 ctypes.c_void_p(gin.data_ptr()), ctypes.c_void_p(gp.data_ptr()),
                                                 nlm._dptr(gpol)))

    def timed(fn):
        best = float("inf")
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    fwd()
    grad(0)
    parity = None
    if check:
        # the forward of the gradient configuration (nZSteps=2000) against the numpy oracle with the
        # same continuous poling profile in place of the domains
        from oracle import nlm_oracle as O
        o = O.Chi2PDC(**kw)
        o.poling = np.asarray(d, dtype=np.float64)
        o.run_pump_simulation()
        f, _ = o.propagate(x[None, :], False, 0)
        fwd()
        torch.cuda.synchronize()
        parity = {"rel_l2_forward": rel_l2(out.cpu().numpy()[0], f[0, 0]), "against": "numpy oracle",
                  "tolerance": 1e-9}
    t_fwd = timed(fwd)
    t_grad = timed(lambda: grad(0))
    k_auto = used.value
    k_sqrt = int(math.ceil(math.sqrt(nz - 1)))
    t_grad_sqrt = timed(lambda: grad(k_sqrt))
    res = {"grad_fwd_cost": t_grad / t_fwd, "fwd_ms": t_fwd, "grad_ms": t_grad, "checkpoint_interval": k_auto,
           "grad_fwd_cost_sqrt_checkpoints": t_grad_sqrt / t_fwd, "sqrt_checkpoint_interval": k_sqrt, "nz": nz}
    if parity:
        res["parity"] = parity
    return res


def measure_adjoint(nlm, torch, reps=3, check=True):
    """grad/fwd cost on the gradient configuration (Chi2PDC N=512, nZSteps=2000), and the same
    problem on a 2048-point grid, where one propagation runs on a 4-CTA cluster, with the reverse
    sweep on clusters and on one CTA."""
    res = _adjoint_costs(nlm, torch, 512, 1, reps, check=check)
    nz = res.pop("nz")
    res["workload"] = ("Chi2PDC N=512 nZSteps=%d, gradients wrt input spectrum, pump spectrum (512 bins) and "
                       "poling profile (%d values)" % (nz, nz))
    big = {"n_freqs": 2048}
    for cluster, label in ((1, "cluster"), (0, "one_cta")):
        r = _adjoint_costs(nlm, torch, 2048, cluster, reps)
        r.pop("nz")
        big[label] = r
    res["n2048"] = big
    return res


def measure_configs(nlm, torch, cpu=True):
    """The other workloads of the benchmark configuration list, each bounded to a few seconds."""
    import ctypes
    res = {}
    # 1. Chi3 N=1 soliton pump + seeded-noise signal, N=512, nZSteps=200: latency through the API
    kw1 = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=512, zPrecision=200)
    rng = np.random.default_rng(1)
    sig = (rng.standard_normal(512) + 1j * rng.standard_normal(512)) * 1e-3 / np.sqrt(2)

    def chi3_latency(mode):
        # mode 1 (default): the pump march and the signal side by side on one cluster of eight CTAs (four
        # SMs each, one point per thread); 3: the same two marches one after the other on four SMs; 0:
        # one CTA each
        m1 = nlm.Chi3(**kw1)
        m1._set_cluster(mode)
        m1.runPumpSimulation()
        m1.runSignalSimulation(sig)
        lat = []
        for _ in range(5):
            t0 = time.perf_counter()
            m1.runPumpSimulation()
            m1.runSignalSimulation(sig)
            _ = m1.signalTime
            lat.append(time.perf_counter() - t0)
        return 1e3 * min(lat), m1

    lat1, m1 = chi3_latency(1)
    res["chi3_pump_signal_n512"] = {"gpu_latency_ms": lat1, "form": "pump and signal pipelined on 8 CTAs",
                                    "gpu_latency_ms_sequential_spread": chi3_latency(3)[0],
                                    "gpu_latency_ms_one_cta": chi3_latency(0)[0]}
    if cpu:
        from oracle import nlm_oracle as O
        o1 = O.Chi3(**kw1)
        t0 = time.perf_counter()
        o1.run_pump_simulation()
        o1.run_signal_simulation(sig)
        res["chi3_pump_signal_n512"]["cpu_oracle_latency_ms"] = 1e3 * (time.perf_counter() - t0)
        # parity of every full grid of the configuration (pump 399 x 512, signal 200 x 512)
        res["chi3_pump_signal_n512"]["parity"] = {
            "rel_l2_pump_time": rel_l2(m1.pumpTime, o1.pump_time[0]),
            "rel_l2_pump_freq": rel_l2(m1.pumpFreq, o1.pump_freq[0]),
            "rel_l2_signal_time": rel_l2(m1.signalTime, o1.signal_time[0]),
            "rel_l2_signal_freq": rel_l2(m1.signalFreq, o1.signal_freq[0]),
            "against": "numpy oracle, full grids", "tolerance": 1e-9}
    # single propagations (runSignalSimulation, full grids): one CTA against a cluster per propagation;
    # at 1024 and 2048 points with one point per thread (the default) and with four
    single = {}
    for n in (1024, 2048, 8192):
        kw = dict(CONFIG, tPrecision=n, zPrecision=500)
        a = (np.random.default_rng(n).standard_normal(n) + 0j) * 0.1
        row = {"n_freqs": n}
        # mode 1 (default): one point per thread in the widest form (eight CTAs at 1024 points, sixteen
        # at 2048); mode 3: one point per thread on four CTAs at 1024 points, eight at 2048; mode 2:
        # four points per thread on four CTAs, the only cluster form at 8192 points
        forms = ((0, "one_cta_ms"), (1, "spread_ms"), (3, "spread_half_ctas_ms"), (2, "cluster_ms")) \
            if n <= 2048 else ((0, "one_cta_ms"), (1, "cluster_ms"))
        for use, label in forms:
            m = nlm.Chi2PDC(poling=np.ones(N_DOMAINS), **kw)
            m._set_cluster(use)
            m.runPumpSimulation()
            m.runSignalSimulation(a)
            best = float("inf")
            for _ in range(3):
                t0 = time.perf_counter()
                m.runSignalSimulation(a)
                best = min(best, time.perf_counter() - t0)
            row[label] = 1e3 * best
            row["z_steps"] = m._dims["nZSteps"]
        if cpu and n == 2048:
            from oracle import nlm_oracle as O
            o = O.Chi2PDC(poling=np.ones(N_DOMAINS), **kw)
            o.run_pump_simulation()
            t0 = time.perf_counter()
            o.run_signal_simulation(a)
            row["cpu_oracle_ms"] = 1e3 * (time.perf_counter() - t0)
        single["chi2pdc_run_signal_n%d" % n] = row
    # one Chi3GNLSE propagation (the GNLSE medium, N=4096, 999 steps): 18 transforms per step
    kw = dict(GNLSE_CONFIG, zPrecision=111)
    t = np.fft.fftshift(np.linspace(-50, 50, 4096, endpoint=False))
    a = 3 / np.cosh(t) + 0j
    row = {"n_freqs": 4096}
    # mode 1: one point per thread on sixteen CTAs; mode 2: four points per thread on four CTAs
    for use, label in ((0, "one_cta_ms"), (1, "spread_ms"), (2, "cluster_ms")):
        m = nlm.Chi3GNLSE(**kw)
        m._set_cluster(use)
        m.runSignalSimulation(a)
        t0 = time.perf_counter()
        m.runSignalSimulation(a)
        row[label] = 1e3 * (time.perf_counter() - t0)
        row["z_steps"] = m._dims["nZSteps"]
    if cpu:
        # the same propagation (999 steps of the medium's own z step) with the C++ restatement, one thread
        from oracle import build_oracle, cpu_port
        from oracle import nlm_oracle as O
        build_oracle.build()
        o = O.Chi3GNLSE(**kw)
        t0 = time.perf_counter()
        out = cpu_port.gnlse_batch(o, a[None, :], True, 1)
        row["cpu_port_ms"] = 1e3 * (time.perf_counter() - t0)
        if not np.all(np.isfinite(out)):
            raise RuntimeError("the CPU restatement diverged on the GNLSE medium")
    single["gnlse_run_signal_n4096"] = row
    # the Chi3 self-phase-modulation pump march (runPumpSimulation) on 8192 points, 1000 rows
    kw = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0.02, tMax=40, tPrecision=8192,
              zPrecision=500)
    row = {"n_freqs": 8192}
    for use, label in ((0, "one_cta_ms"), (1, "cluster_ms")):
        m = nlm.Chi3(**kw)
        m._set_cluster(use)
        m.runPumpSimulation()
        best = float("inf")
        for _ in range(3):
            t0 = time.perf_counter()
            m.runPumpSimulation()
            best = min(best, time.perf_counter() - t0)
        row[label] = 1e3 * best
        row["z_steps"] = m._dims["nZSteps"]
    single["chi3_run_pump_n8192"] = row
    res["single_propagation"] = single
    # Cascade of two Chi2PDC media (N=1024, 200 steps each): the two Green's functions and their
    # composition C2 C1 + S2 conj(S1), C2 S1 + S2 conj(C1) on the FP64 pipe (k_cgemm_compose), against
    # cuBLAS ZGEMMs of the same composition (measurement only)
    kwa = dict(CONFIG, zPrecision=100)
    kwb = dict(kwa, beta1s=-1, diffBeta0=0.2)
    ma, mb = nlm.Chi2PDC(poling=np.ones(N_DOMAINS), **kwa), nlm.Chi2PDC(poling=np.ones(N_DOMAINS), **kwb)
    casc = nlm.Cascade([ma, mb], [{0: 0}], False)
    casc.computeGreensFunction()
    ma.computeGreensFunction()
    mb.computeGreensFunction()

    def best_of(fn, reps=3):
        b = float("inf")
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            b = min(b, time.perf_counter() - t0)
        return b, out
    t_c, (Cc, Sc) = best_of(lambda: casc.computeGreensFunction())
    t_a, (Ca, Sa) = best_of(lambda: ma.computeGreensFunction())
    t_b, (Cb, Sb) = best_of(lambda: mb.computeGreensFunction())
    g = [torch.tensor(x, device="cuda") for x in (Ca, Sa, Cb, Sb)]

    def zgemm():
        return g[2] @ g[0] + g[3] @ g[1].conj(), g[2] @ g[1] + g[3] @ g[0].conj()
    co = torch.empty_like(g[0])
    so = torch.empty_like(g[0])

    def compose():
        nlm._check(nlm._lib.nlm_cascade_compose(*[ctypes.c_void_p(x.data_ptr()) for x in (g[2], g[3], g[0], g[1])],
                                                1024, 1024, 1024, ctypes.c_void_p(co.data_ptr()),
                                                ctypes.c_void_p(so.data_ptr()),
                                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        return co, so

    def event_ms(fn, reps=5):
        fn()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best
    t_k = event_ms(compose)
    t_z = event_ms(zgemm)
    Cz, Sz = zgemm()
    compose()
    torch.cuda.synchronize()
    res["cascade_green_n1024"] = {"media": 2, "n_freqs": 1024, "z_steps_each": ma._dims["nZSteps"],
                                  "cascade_ms": 1e3 * t_c, "media_green_ms": 1e3 * (t_a + t_b),
                                  "composition_kernel_ms": t_k,
                                  "composition_kernel_tflops": 32 * 1024 ** 3 / (t_k * 1e-3) / 1e12,
                                  "cublas_zgemm_composition_ms": t_z,
                                  "timing": "CUDA events on the current stream, best of 5, the four 1024 x 1024 "
                                            "operands resident: k_cgemm_compose against torch's four complex128 "
                                            "matmuls (cuBLAS ZGEMM) and two additions",
                                  "composition_flops": 32 * 1024 ** 3,
                                  "rel_diff_vs_cublas": float(torch.linalg.norm(co - Cz) / torch.linalg.norm(Cz)),
                                  "cascade_rel_diff_vs_cublas": float(np.linalg.norm(Cc - Cz.cpu().numpy()) /
                                                                      np.linalg.norm(Cc))}
    # 3. 64 ragged Chi2SFG media in one launch
    params = ragged_media_params()
    media = []
    for kw, doms, pump, _ in params:
        m = nlm.Chi2SFG(customPump=pump, poling=doms, **kw)
        m.runPumpSimulation()
        media.append(m)
    ins = [p[3] for p in params]
    nlm.ragged_batch(media, ins)
    wall, wall_kept, wall_direct = [], [], []
    dev, dev_kept = [], []         # the calls' device time (CUDA events on the engine's stream)
    for _ in range(3):
        for m in media:            # new pumps before every timed call
            m.runPumpSimulation()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nlm.ragged_batch(media, ins)
        wall.append(time.perf_counter() - t0)
        dev.append(nlm.ragged_last_plan()["gpu_ms"])
    for _ in range(3):             # the same pumps again: the RK4 matrices are built, then reused
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ragged_out = nlm.ragged_batch(media, ins)
        wall_kept.append(time.perf_counter() - t0)
        dev_kept.append(nlm.ragged_last_plan()["gpu_ms"])
    wall_one = []
    for m in media:
        m._set_cluster(0)
    nlm.ragged_batch(media, ins)
    for _ in range(2):
        t0 = time.perf_counter()
        nlm.ragged_batch(media, ins)
        wall_one.append(time.perf_counter() - t0)
    for m in media:
        m._set_schedule(use_propagator=0)
    nlm.ragged_batch(media, ins)
    for _ in range(2):
        t0 = time.perf_counter()
        nlm.ragged_batch(media, ins)
        wall_direct.append(time.perf_counter() - t0)
    steps = sum(m._dims["nZSteps"] for m in media)
    for m in media:
        m._set_cluster(1)
        m._set_schedule(use_propagator=-1)
    for m in media:
        m.runPumpSimulation()
    nlm.ragged_batch(media, ins)
    plan = nlm.ragged_last_plan()
    res["ragged_chi2sfg_64_media"] = {"gpu_wall_ms": 1e3 * min(wall), "media": len(media), "total_z_steps": steps,
                                      "n_freqs": sorted({m._dims["nFreqs"] for m in media}),
                                      "pumps": "rerun before each call: every medium propagates with its DiffEq "
                                               "(RK4 matrices are built only for a pump used again)",
                                      "gpu_wall_ms_pumps_kept": 1e3 * min(wall_kept),
                                      "device_ms": min(dev), "device_ms_pumps_kept": min(dev_kept),
                                      "timing": "wall: the API call (host conversion, one input and one output "
                                                "copy, the graph); device: CUDA events on the engine's stream "
                                                "around the enqueued work",
                                      "form": "each medium on one SM in a ragged launch or on a 4-, 8- or 16-SM "
                                              "cluster slot, planned for the makespan; the call replayed as a CUDA "
                                              "graph",
                                      "plan": plan,
                                      "gpu_wall_ms_one_cta_per_medium": 1e3 * min(wall_one),
                                      "gpu_wall_ms_one_cta_diffeq_form": 1e3 * min(wall_direct)}
    # the oracle of configuration 3 (all 64 media at their full step counts) in spawned processes, and
    # the C++ restatement of configuration 5 (four rows at the full 9999 steps, one of them recording
    # its spectrum every 1000 steps) in threads: both run on the host while the GPU runs configuration 5
    pool, ragged_async, gn_jobs = None, None, {}
    kw5 = dict(GNLSE_CONFIG)
    t = np.fft.fftshift(np.linspace(-50, 50, 4096, endpoint=False))
    rows = 1024
    rng = np.random.default_rng(5)
    x5 = 3 / np.cosh(t)[None, :] + (rng.standard_normal((rows, 4096)) + 1j * rng.standard_normal((rows, 4096))) \
        * 1e-4 / np.sqrt(2)
    if cpu:
        from oracle import build_oracle, cpu_port
        from oracle import nlm_oracle as O
        build_oracle.build()
        cores = os.cpu_count() or 1
        pool = mp.get_context("spawn").Pool(max(1, min(len(media), cores - 5)))
        ragged_async = pool.map_async(_ragged_oracle_output, range(len(media)))
        o5 = O.Chi3GNLSE(**kw5)

        def run_batch():
            t0 = time.perf_counter()
            gn_jobs["batch"] = cpu_port.gnlse_batch(o5, x5[:4], True, 4)
            gn_jobs["batch_s"] = time.perf_counter() - t0

        def run_record():
            gn_jobs["record"] = cpu_port.gnlse_record(o5, x5[0], True, 1000)

        gn_threads = [threading.Thread(target=run_batch), threading.Thread(target=run_record)]
        for th in gn_threads:
            th.start()
    # 5. Chi3GNLSE batch of 1024 seeded noise realisations of 3 sech(t), N=4096, nZSteps=9999: the whole
    # configuration in one call (schedule and kernels warmed up on the same rows over 99 steps)
    m5 = nlm.Chi3GNLSE(**kw5)
    nz5 = m5._dims["nZSteps"]
    x5t = torch.tensor(x5, device="cuda")
    o5d = torch.empty_like(x5t)

    def gn(med):
        nlm._check(nlm._lib.nlm_batch_device(med._h(), ctypes.c_void_p(x5t.data_ptr()), rows, 4096, 1, 0, 1, 0, None,
                                             0, ctypes.c_void_p(o5d.data_ptr())))
    gn(nlm.Chi3GNLSE(**dict(kw5, relativeLength=0.01)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gn(m5)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    flops5 = rows * (nz5 - 1) * (18 * 5 * 4096 * 12 + 120 * 4096)
    res["gnlse_batch_n4096"] = {"rows": rows, "z_steps": nz5, "wall_s": dt, "propagations_per_s": rows / dt,
                                "row_steps_per_s": rows * (nz5 - 1) / dt,
                                "algorithmic_tflops": flops5 / dt / 1e12,
                                "flops_model": "per row-step 18 transforms x 5 N log2 N + 120 N",
                                "schedule": m5._last_schedule()}
    # error growth over the 9999 steps: one propagation's full grids (runSignalSimulation) against the
    # restatement's spectrum every 1000 steps
    m5.runSignalSimulation(x5[0])
    grid = m5.signalFreq if cpu else None
    # gradient of the band energy (w in [2, 4]) with respect to the input spectral phase, on 16 rows (a
    # propagation per 4-CTA cluster) and on all 1024 rows, over 999 steps (the gradient-over-forward
    # ratio does not depend on the step count)
    from multimodenonlinearoptics_gb300.autograd import propagate_gnlse
    m6 = nlm.Chi3GNLSE(**dict(kw5, zPrecision=111))
    nz6 = m6._dims["nZSteps"]
    w = torch.tensor(m6.omega, device="cuda")
    band = ((w >= 2) & (w <= 4)).to(torch.float64)
    p0 = torch.fft.fft(torch.tensor(3 / np.cosh(t), device="cuda"))
    phi = torch.zeros(4096, dtype=torch.float64, device="cuda", requires_grad=True)
    grads = {}
    for nrows in (16, 1024):
        noise = torch.fft.fft(x5t[:nrows] - torch.tensor(3 / np.cosh(t), device="cuda")[None, :], dim=1)

        def fwd_only():
            with torch.no_grad():
                xa = (p0[None, :] * torch.exp(1j * phi)[None, :] + noise).contiguous()
                out = torch.empty_like(xa)
                nlm._check(nlm._lib.nlm_batch_device(m6._h(), ctypes.c_void_p(xa.data_ptr()), nrows, 4096, 0, 0, 1, 0,
                                                     None, 0, ctypes.c_void_p(out.data_ptr())))
                torch.cuda.synchronize()

        def grad():
            a = p0[None, :] * torch.exp(1j * phi)[None, :] + noise
            e = torch.sum(torch.abs(propagate_gnlse(m6, a)) ** 2 * band)
            phi.grad = None
            e.backward()
            torch.cuda.synchronize()
        fwd_only()
        grad()
        t0 = time.perf_counter()
        fwd_only()
        t_f = time.perf_counter() - t0
        t0 = time.perf_counter()
        grad()
        t_g = time.perf_counter() - t0
        grads[nrows] = {"rows": nrows, "z_steps": nz6, "fwd_ms": 1e3 * t_f, "grad_ms": 1e3 * t_g,
                        "grad_fwd_cost": t_g / t_f}
    res["gnlse_phase_gradient"] = dict(grads[16], rows_1024=grads[1024])
    if cpu:
        for th in gn_threads:
            th.join()
        got = o5d[:4].cpu().numpy()
        rec, last = gn_jobs["record"]
        steps = np.arange(1, rec.shape[0] + 1) * 1000
        res["gnlse_batch_n4096"]["parity"] = {
            "rel_l2_rows_0_3_full_steps": rel_l2(got, gn_jobs["batch"]),
            "rel_l2_by_step": {str(int(k)): rel_l2(grid[k], r) for k, r in zip(steps, rec)},
            "rel_l2_run_signal_last_row": rel_l2(m5.signalTime[-1], last),
            "against": "C++ restatement (agrees with the numpy oracle to 1e-15)", "tolerance": 1e-9}
        res["gnlse_batch_n4096"]["cpu_port_row_steps_per_s"] = 4 * (nz5 - 1) / gn_jobs["batch_s"]
        res["gnlse_batch_n4096"]["cpu_port_sample"] = "rows 0-3 of the configuration at 9999 steps, 4 threads"
        outs = ragged_async.get()
        pool.close()
        pool.join()
        errs = [rel_l2(ragged_out[i], f) for i, f, _, _ in outs]
        res["ragged_chi2sfg_64_media"]["parity"] = {
            "media": len(errs), "max_rel_l2": max(errs), "median_rel_l2": float(np.median(errs)),
            "z_steps": int(sum(nz for _, _, nz, _ in outs)),
            "against": "numpy oracle, every medium at its full step count", "tolerance": 1e-9}
        res["ragged_chi2sfg_64_media"]["cpu_oracle_sequential_ms"] = 1e3 * sum(dt for _, _, _, dt in outs)
        res["ragged_chi2sfg_64_media"]["cpu_sample"] = ("every medium (pump and propagation), numpy oracle, one "
                                                        "process per medium; the sum of their times")
    return res


def measure_consumers(nlm, torch, green_device, C, S, cpu=True):
    """Green's-function consumers on the benchmark's C and S (N=1024, left in HBM by the engine):
    the quadrature matrix Z (engine kernel), the covariance Z Z^T with its determinant check
    (cuBLAS, cuSOLVER) and the Bloch-Messiah principal values (cuSOLVER SVD); against the oracle
    (numpy / scipy, the reference's own method) on the host."""
    from multimodenonlinearoptics_gb300 import multimode as mm
    green_device()
    torch.cuda.synchronize()
    n = C.shape[0]
    Z = mm.calcQuadratureGreens(C, S)
    mm.calcCovarianceMtx(Z, tol=1e-6)
    mm.blochMessiahEigs(Z)            # warm-up: library handles and workspaces
    torch.cuda.synchronize()
    res = {"n_modes": n, "z_shape": list(Z.shape)}
    # the element-wise kernel, CUDA events on the current stream.  The L2 is flushed by reading a
    # 256 MB buffer: a written flush would leave ~129 MB of dirty lines to be written back during
    # the timed kernel.
    flush = torch.ones(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    best = float("inf")
    for _ in range(5):
        flush.sum()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        mm.calcQuadratureGreens(C, S)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    bytes_moved = 2 * n * n * 16 + 4 * n * n * 8          # C and S read, Z written
    res["quadrature_z_ms"] = best
    res["quadrature_z_gbs"] = bytes_moved / (best * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    res["hbm_peak_gbs"] = peaks.get("hbm_gbs")
    if res["hbm_peak_gbs"]:
        res["quadrature_z_frac_of_measured_hbm"] = res["quadrature_z_gbs"] / res["hbm_peak_gbs"]
    for name, fn in (("covariance_ms", lambda: mm.calcCovarianceMtx(Z, tol=1e-6)),
                     ("bloch_messiah_eigs_ms", lambda: mm.blochMessiahEigs(Z)),
                     ("bloch_messiah_vecs_ms", lambda: mm.blochMessiahVecs(Z))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        res[name] = 1e3 * (time.perf_counter() - t0)
    if cpu:
        from oracle import multimode_oracle as M
        Ch, Sh = C.cpu().numpy(), S.cpu().numpy()
        t0 = time.perf_counter()
        Zh = M.quadrature_greens(Ch, Sh)
        M.covariance(Zh, 1e-6)
        res["cpu_oracle_z_and_covariance_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        M.bloch_messiah_eigs(Zh)
        res["cpu_oracle_bloch_messiah_eigs_ms"] = 1e3 * (time.perf_counter() - t0)
        res["cpu_threads"] = os.cpu_count()
    return res


def measure_ff(nlm, torch, args, stream, flush, C64, S64, f64_value, f64_kernel_ms):
    """The same Green's function with the double-float kernel (FP32 pairs on the FP32 units): device
    throughput over the same steps, kernel time, and its distance from the FP64 result."""
    med = nlm.Chi2PDC(poling=np.ones(N_DOMAINS if CONFIG["zPrecision"] == 500 else 5), **CONFIG)
    med._set_stream(stream.cuda_stream)
    med._set_precision("ff")
    n = med._dims["nFreqs"]
    C = torch.empty_like(C64)
    S = torch.empty_like(S64)

    def green_device():
        nlm._check(nlm._lib.nlm_green_device(med._h(), 0, 1, 1, 0, None, 0, None, 0, C.data_ptr(), S.data_ptr()))

    for _ in range(args.warmup):
        green_device()
    torch.cuda.synchronize()
    med._kernel_timing(1)
    elapsed = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        green_device()
        e1.record(stream)
        e1.synchronize()
        elapsed += e0.elapsed_time(e1) / 1e3
    kernel_ms, kernel_count = med._kernel_timing(0)
    sched = med._last_schedule()
    value = 2 * n * args.steps / elapsed
    err = max(float(torch.linalg.norm(C - C64) / torch.linalg.norm(C64)),
              float(torch.linalg.norm(S - S64) / torch.linalg.norm(S64)))
    return {"value": value, "unit": UNIT, "kernel": "k_propagate_linear_ff<8>",
            "kernel_ms": kernel_ms / max(kernel_count, 1), "speedup_vs_f64": value / f64_value,
            "kernel_speedup_vs_f64": f64_kernel_ms / max(kernel_ms / max(kernel_count, 1), 1e-12),
            "rel_err_vs_f64": err, "dtype": "f32x2 (double-float, ~48-bit significand)",
            "schedule": {"cta_per_sm": sched["cta_per_sm"], "registers_per_thread": sched["registers"],
                         "chosen_by": "autotuner" if sched["tuned"] else "occupancy"}}


def _over_spread(value, configs):
    """Batched throughput over the fastest one-propagation form: one runSignalSimulation of the same
    medium (N=1024, 1000 steps) spread over an 8-CTA cluster, which also writes both full grids."""
    try:
        ms = configs["single_propagation"]["chi2pdc_run_signal_n1024"]["spread_ms"]
    except (KeyError, TypeError):
        return None
    return {"value": value / (1e3 / ms), "plain_spread_propagations_per_s": 1e3 / ms,
            "form": "runSignalSimulation on an 8-CTA cluster, one point per thread (full grids written)"}


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from multimodenonlinearoptics_gb300 import build_ext
    build_ext.build()
    from multimodenonlinearoptics_gb300 import nonlinearmedium as nlm

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if world == 1:
            return x
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    med = nlm.Chi2PDC(poling=np.ones(N_DOMAINS if CONFIG["zPrecision"] == 500 else 5), **CONFIG)
    n = med._dims["nFreqs"]
    n_z = med._dims["nZSteps"]
    n_inst = 2 * n
    stream = torch.cuda.Stream()
    med._set_stream(stream.cuda_stream)
    peak = nlm.fp64_peak_tflops()
    peak_mma = nlm.fp64_mma_peak_tflops()
    per_warps = {str(w): nlm.fp64_warps_rate_tflops(w) for w in (1, 2, 4, 8)}
    C = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    S = torch.empty_like(C)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")   # > 129 MB L2

    def green_local():
        nlm._check(nlm._lib.nlm_green_device(med._h(), 0, 1, 1, 0, None, 0, None, 0, C.data_ptr(), S.data_ptr()))

    def green_device():
        if world > 1:
            # one Green's function split over the ranks (strong scaling): rows on each GPU, one NCCL
            # gather of device buffers, C and S on rank 0's GPU
            from multimodenonlinearoptics_gb300 import sharding
            sharding.green_sharded_device(med, C, S)
            return
        nlm._check(nlm._lib.nlm_green_device(med._h(), 0, 1, 1, 0, None, 0, None, 0, C.data_ptr(), S.data_ptr()))

    # warm-up (also builds the kernel schedule and the propagator)
    for _ in range(args.warmup):
        green_device()
    torch.cuda.synchronize()

    # device-resident throughput
    barrier()
    med._kernel_timing(1)
    launches = 0
    elapsed = 0.0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            green_device()
            e1.record(stream)
            e1.synchronize()
            elapsed += e0.elapsed_time(e1) / 1e3
            launches += med._launch_count()
    kernel_ms, kernel_count = med._kernel_timing(0)
    sched = med._last_schedule()
    barrier()
    t_dev = max_over_ranks(elapsed)
    value = n_inst * args.steps / t_dev   # the whole Green's function per step, over all ranks

    # end to end through the public API: numpy C and S on the host every step
    barrier()
    e2e_elapsed = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if world > 1:
            from multimodenonlinearoptics_gb300 import sharding
            res = sharding.compute_greens_function_sharded(med)
            Ch, Sh = res if res is not None else (None, None)
        else:
            Ch, Sh = med.computeGreensFunction()
        e1.record(stream)
        e1.synchronize()
        e2e_elapsed += e0.elapsed_time(e1) / 1e3
    barrier()
    t_e2e = max_over_ranks(e2e_elapsed)
    e2e_value = n_inst * args.steps / t_e2e

    # plain form: one propagation per kernel launch, on a sample of the impulses
    plain = None
    if args.plain_sample > 0 and rank == 0:
        Cp = np.empty((n, n), dtype=np.complex128)
        Sp = np.empty_like(Cp)
        nlm._check(nlm._lib.nlm_green_plain(med._h(), 0, 0, 2, nlm._dptr(Cp.view(np.float64)),
                                            nlm._dptr(Sp.view(np.float64))))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nlm._check(nlm._lib.nlm_green_plain(med._h(), 0, 0, args.plain_sample, nlm._dptr(Cp.view(np.float64)),
                                            nlm._dptr(Sp.view(np.float64))))
        t_plain = time.perf_counter() - t0
        plain = args.plain_sample / t_plain

    # the secondary measurements run on rank 0 only (the other ranks wait at the final barrier)
    main = rank == 0
    ff = measure_ff(nlm, torch, args, stream, flush, C, S, value, kernel_ms / max(kernel_count, 1)) \
        if args.ff and main and world == 1 else None
    adjoint = measure_adjoint(nlm, torch, check=args.cpu_bins > 0) if args.adjoint and main else None
    configs = measure_configs(nlm, torch, cpu=args.cpu_bins > 0) if args.configs and main else None
    if configs is not None:
        with torch.cuda.stream(stream):
            configs["green_consumers_n1024"] = measure_consumers(nlm, torch, green_local, C, S,
                                                                 cpu=args.cpu_bins > 0)

    line = None
    if rank == 0:
        # CPU baseline and parity sample: oracle impulse propagations of the same workload
        cpu = None
        parity = None
        if args.cpu_bins > 0:
            from oracle import build_oracle, cpu_port
            build_oracle.build()
            ref = _oracle_medium()
            # parity sample against the numpy oracle (columns of C and S from impulse pairs)
            rng = np.random.default_rng(0)
            bins = rng.choice(n, size=args.cpu_bins, replace=False)
            cc, ss = oracle_columns(ref, bins)
            cols = (bins + n // 2) % n
            parity_numpy = max(np.linalg.norm(Ch[:, cols] - cc) / np.linalg.norm(cc),
                               np.linalg.norm(Sh[:, cols] - ss) / np.linalg.norm(ss))
            # the whole C and S (all 1024 columns) against the C++ restatement on every host core; the
            # restatement agrees with the numpy oracle to 1e-15 (tests/test_cpu_port.py)
            cores = os.cpu_count() or 1
            t0 = time.perf_counter()
            Cc, Sc = cpu_port.chi2pdc_green(ref, cores)
            t_all = time.perf_counter() - t0
            parity = {"rel_l2_full_c_s_vs_cpp_port": max(np.linalg.norm(Ch - Cc) / np.linalg.norm(Cc),
                                                         np.linalg.norm(Sh - Sc) / np.linalg.norm(Sc)),
                      "rel_l2_sample_vs_numpy_oracle": parity_numpy, "sample_columns": int(args.cpu_bins),
                      "tolerance": 1e-9}
            # one-core rate of the C++ restatement on a sample of the impulses
            ref.run_pump_simulation()
            t0 = time.perf_counter()
            cpu_port.chi2pdc_impulses(ref, 0, 2 * args.cpu_bins, 1)
            t_one = time.perf_counter() - t0
            cpu = {"value": n_inst / t_all, "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": "one whole computeGreensFunction (pump grid, 2048 impulse propagations, C/S "
                             "assembly) on %d std::threads; C++ restatement of the reference's loop "
                             "(oracle/nlm_cpu.cpp)" % cores,
                   "one_core": {"value": 2 * args.cpu_bins / t_one, "unit": UNIT, "cores": 1,
                                "sample": "%d impulse propagations, 1 thread" % (2 * args.cpu_bins)}}
        config = bench_config()
        if world > 1:
            config = dict(config, parallelism="2048 impulse propagations split over %d GPUs in contiguous row "
                                              "blocks, one NCCL gather to rank 0" % world)
        flops = algorithmic_flops(n_inst // world, n_z, n)   # one launch: this rank's share of the rows
        avg_kernel_s = kernel_ms / max(kernel_count, 1) / 1e3
        achieved = flops / avg_kernel_s / 1e12
        traffic = read_profile_traffic()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * 16,
                    "d2h_bytes_per_step": 2 * n * n * 16,
                    "api": "nonlinearmedium.Chi2PDC.computeGreensFunction() -> numpy C, S"},
            "gpu_launches": int(launches),
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None, "traffic": traffic,
                         "kernel": "k_propagate_linear<1,8>", "kernel_ms": 1e3 * avg_kernel_s,
                         "algorithmic_flops_per_launch": flops,
                         "traffic_source": "profile: dram__bytes_read.sum + write.sum of one ncu --set full capture "
                                           "of this kernel on the same workload at nZSteps=50, scaled by 999/49 "
                                           "(profiles/k_propagate_linear_green_n1024.md); not measured in this run",
                         "ncu_fp64_pipe_active_pct": read_profile_value("fp64_pipe_active_pct"),
                         "ncu_fp64_pipe_active_pct_source": "profile: the same nZSteps=50 capture; not measured in "
                                                            "this run",
                         "peak_source": "FP64 FMA chains measured in this run (MEASURED_PEAKS.json has no FP64 entry)",
                         "secondary": {
                             "l2_gbs": (read_profile_value("l2_bytes_per_launch_full") or 0) / avg_kernel_s / 1e9
                             if avg_kernel_s and read_profile_value("l2_bytes_per_launch_full") else None,
                             "dram_gbs": traffic / avg_kernel_s / 1e9 if (traffic and avg_kernel_s) else None,
                             "hbm_peak_gbs": measured_hbm_gbs(),
                             "source": "L2 and DRAM bytes per launch from the committed ncu summary "
                                       "(small-case capture scaled to the full step count) over the "
                                       "kernel's CUDA-event time"},
                         "fp64_tflops_by_warps_per_sm": per_warps,
                         "fp64_tensor_peak": peak_mma,
                         "fp64_tensor_peak_source": "m16n8k16 f64 MMAs (DMMA) measured in this run: the rate a "
                                                    "DFT-as-GEMM schedule could draw on"},
            "cpu_baseline": cpu,
            "plain": {"value": plain, "unit": UNIT, "sample": args.plain_sample,
                      "form": "one propagation per kernel launch"},
            "batched_over_plain": (value / plain) if plain else None,
            "batched_over_plain_spread": _over_spread(value, configs),
            "parity": parity,
            "schedule": {"points_per_thread": sched["R"], "propagations_per_cta": sched["ipc"], "grid": sched["grid"],
                         "block": sched["block"], "cta_per_sm": sched["cta_per_sm"],
                         "registers_per_thread": sched["registers"],
                         "chosen_by": "autotuner" if sched["tuned"] else "occupancy"},
            "cuda_graphs": dict(zip(("captures", "replays"), med._graph_stats())),
            "variant_ff": ff,
            "adjoint": adjoint,
            "other_configs": configs,
            "clocks": clocks.summary(),
        }
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-sample", type=int, default=16)
    ap.add_argument("--cpu-bins", type=int, default=64)
    ap.add_argument("--ref-bins", type=int, default=0)
    ap.add_argument("--ff", type=int, default=1, help="measure the double-float variant (1) or not (0)")
    ap.add_argument("--adjoint", type=int, default=1, help="measure the grad/fwd cost (1) or not (0)")
    ap.add_argument("--configs", type=int, default=1, help="measure the other workloads (1) or not (0)")
    ap.add_argument("--zprecision", type=int, default=0,
                    help="override zPrecision (smaller captures for the profiler; the benchmark uses 500)")
    args = ap.parse_args()
    if args.zprecision:
        CONFIG["zPrecision"] = args.zprecision
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
