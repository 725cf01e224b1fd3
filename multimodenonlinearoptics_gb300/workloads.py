"""The benchmark workloads of the split-step path, as seeded synthetic inputs.

Each one is defined here once, so that the benchmark (bench.py) and the profiler commands of the
committed profile summaries run the same media and inputs.  `python -m
multimodenonlinearoptics_gb300.workloads <name>` runs one workload once on cuda:0: a small,
self-contained command for ncu.

* green       Chi2PDC computeGreensFunction, N=1024, nZSteps = 2 zPrecision (1000 by default)
* chi3        Chi3 N=1 soliton pump + seeded-noise signal, N=512, nZSteps=200
* ragged      64 Chi2SFG media with N in {128..2048} and nZSteps in [200, 2000], one ragged launch
* adjoint     Chi2PDC gradient (input, pump spectrum, poling profile), N=512, nZSteps=2000
* gnlse       Chi3GNLSE batch of 3 sech(t) + noise rows, N=4096
* gnlse_grad  gradient of the band energy (omega in [2, 4]) with respect to the input spectral phase
* signal      one Chi2PDC runSignalSimulation (full grids) on the Green's medium at N=2048
* gnlse_signal  one Chi3GNLSE runSignalSimulation (full grids) on the GNLSE medium at N=4096
* ragged_wide  one 2048-point Chi2SFG runSignalSimulation with the ragged set's parameters (DiffEq form):
               the march of the ragged set's longest media, on sixteen CTAs (--cluster 1, the
               default for full grids) or eight (--cluster 3)
"""

import argparse
import ctypes
import math

import numpy as np

# Chi2PDC Green's function: nlLength=0.5 gives nZSteps = 2 zPrecision; 100 equal poling domains of
# 10 steps (period 20 steps) at zPrecision=500
GREEN_CONFIG = dict(relativeLength=1, nlLength=0.5, beta2=1, beta2s=0.5, pulseType=0, beta1=0, beta1s=2, beta3=0,
                    beta3s=0.1, diffBeta0=0, tMax=40, tPrecision=1024, zPrecision=500)
GREEN_DOMAINS = 100

CHI3_CONFIG = dict(relativeLength=1, nlLength=1, beta2=-1, pulseType=1, beta3=0, tMax=20, tPrecision=512,
                   zPrecision=200)

# Chi3GNLSE: nlLength=1/9 is the N=3 soliton with beta2=-1; the parameters the configuration leaves
# open (selfSteepLength, fb, tau1..3, zPrecision) are chosen so that nZSteps = 9999
GNLSE_CONFIG = dict(relativeLength=1, nlLength=1.0 / 9, selfSteepLength=6.5, fr=0.18, fb=0.21, tau1=0.244,
                    tau2=0.64, tau3=1.92, beta2=-1, beta3=0.05, tMax=50, tPrecision=4096, zPrecision=1111)


def green_medium(nlm, z_precision=500):
    return nlm.Chi2PDC(poling=np.ones(GREEN_DOMAINS if z_precision == 500 else 5),
                       **dict(GREEN_CONFIG, zPrecision=z_precision))


def chi3_signal(n=512, seed=1):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-3 / np.sqrt(2)


def ragged_media_params(seed=3, count=64):
    """The ragged workload: Chi2SFG media with N in {128..2048}, beta1s ~ U[-3,3], beta2, beta2s ~ U[-1,1],
    beta3s ~ U[-0.2,0.2], Gaussian pump of width U[0.5,3], poling domains of U{5..50} z steps with
    alternating sign, nZSteps ~ U[200,2000] (realised through zPrecision), relativeLength=1,
    nlLength=nlLengthOrig=1, beta2o=beta1o=beta3o=0, diffBeta0=0, tMax=10."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice([128, 256, 512, 1024, 2048]))
        b1s, b2, b2s, b3s = rng.uniform(-3, 3), rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-0.2, 0.2)
        w = rng.uniform(0.5, 3)
        target = int(rng.integers(200, 2001))
        min_len = min(1.0, 1.0 / max(abs(b1s), abs(b2), abs(b2s), abs(b3s)))
        zp = int(math.ceil(target * min_len))
        kw = dict(relativeLength=1, nlLength=1, nlLengthOrig=1, beta2=b2, beta2s=b2s, beta2o=0, beta1=0, beta1s=b1s,
                  beta1o=0, beta3=0, beta3s=b3s, beta3o=0, diffBeta0=0, tMax=10, tPrecision=n, zPrecision=zp)
        doms, total = [], 0
        while total < target:
            d = int(rng.integers(5, 51))
            doms.append(d)
            total += d
        t = np.fft.fftshift(np.linspace(-10, 10, n, endpoint=False))
        pump = np.exp(-t ** 2 / (2 * w * w))
        sig = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-3 / np.sqrt(2)
        out.append((kw, np.array(doms, dtype=float), pump, sig))
    return out


def ragged_media(nlm, seed=3, count=64):
    """The ragged media with their pumps run, and one input spectrum per medium."""
    params = ragged_media_params(seed, count)
    media = []
    for kw, doms, pump, _ in params:
        m = nlm.Chi2SFG(customPump=pump, poling=doms, **kw)
        m.runPumpSimulation()
        media.append(m)
    return media, [p[3] for p in params]


def adjoint_problem(nlm, z_precision=1000, n=512):
    """The gradient configuration: Chi2PDC as the Green's workload but N=512 (or n), nZSteps=2 zPrecision
    (2000), one seeded noise signal (sigma 1e-3), continuous poling d(z) ~ U[-1, 1] (seed 4), a
    unit-energy seeded target spectrum."""
    med = nlm.Chi2PDC(**dict(GREEN_CONFIG, tPrecision=n, zPrecision=z_precision))
    n, nz = med._dims["nFreqs"], med._dims["nZSteps"]
    rng = np.random.default_rng(4)
    x = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 1e-3 / np.sqrt(2)
    d = rng.uniform(-1, 1, nz)
    target = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    target /= np.linalg.norm(target)
    return med, x, d, target


def gnlse_rows(rows, n=4096, seed=5):
    """3 sech(t) + complex Gaussian noise of std 1e-4 (time domain), one row per realisation."""
    t = np.fft.fftshift(np.linspace(-50, 50, n, endpoint=False))
    rng = np.random.default_rng(seed)
    return 3 / np.cosh(t)[None, :] + (rng.standard_normal((rows, n)) + 1j * rng.standard_normal((rows, n))) \
        * 1e-4 / np.sqrt(2)


def _run(name, z_precision, rows, reps, cluster=1):
    import torch
    from . import nonlinearmedium as nlm
    from .autograd import propagate_gnlse

    def c(m):   # the cluster mode of every medium of the workload
        m._set_cluster(cluster)
        return m
    for _ in range(reps):
        if name == "green":
            c(green_medium(nlm, z_precision or 500)).computeGreensFunction()
        elif name == "chi3":
            m = c(nlm.Chi3(**CHI3_CONFIG))
            m.runPumpSimulation()
            m.runSignalSimulation(chi3_signal())
        elif name == "ragged":
            media, inputs = ragged_media(nlm)
            nlm.ragged_batch([c(m) for m in media], inputs)
        elif name == "adjoint":
            med, x, d, target = adjoint_problem(nlm, z_precision or 1000)
            c(med)
            nz = med._dims["nZSteps"]
            med._set_poling_profile(d)
            xin = torch.tensor(x.reshape(1, -1), dtype=torch.complex128, device="cuda")
            out = torch.empty_like(xin)
            used = ctypes.c_int()
            nlm._check(nlm._lib.nlm_run_pump(med._h()))
            nlm._check(nlm._lib.nlm_adjoint_forward(med._h(), ctypes.c_void_p(xin.data_ptr()), 1,
                                                    ctypes.c_void_p(out.data_ptr()),
                                                    int(math.ceil(math.sqrt(nz - 1))), ctypes.byref(used)))
            g = (2 * (out - torch.tensor(target.reshape(1, -1), device="cuda"))).contiguous()
            gin = torch.empty_like(xin)
            gp = torch.empty(x.size, dtype=torch.complex128, device="cuda")
            gpol = np.zeros(nz)
            nlm._check(nlm._lib.nlm_adjoint_backward(med._h(), ctypes.c_void_p(g.data_ptr()),
                                                     ctypes.c_void_p(gin.data_ptr()), ctypes.c_void_p(gp.data_ptr()),
                                                     nlm._dptr(gpol)))
        elif name == "cascade":
            kwa = dict(GREEN_CONFIG, zPrecision=z_precision or 100)
            kwb = dict(kwa, beta1s=-1, diffBeta0=0.2)
            ma = c(nlm.Chi2PDC(poling=np.ones(GREEN_DOMAINS), **kwa))
            mb = c(nlm.Chi2PDC(poling=np.ones(GREEN_DOMAINS), **kwb))
            nlm.Cascade([ma, mb], [{0: 0}], False).computeGreensFunction()
        elif name == "chi3_pump":
            m = c(nlm.Chi3(**dict(CHI3_CONFIG, tPrecision=8192, tMax=40, beta3=0.02, zPrecision=z_precision or 500)))
            m.runPumpSimulation()
        elif name == "adjoint_cluster":
            med, x, d, target = adjoint_problem(nlm, z_precision or 1000, n=2048)
            c(med)
            nz = med._dims["nZSteps"]
            med._set_poling_profile(d)
            xin = torch.tensor(x.reshape(1, -1), dtype=torch.complex128, device="cuda")
            out = torch.empty_like(xin)
            used = ctypes.c_int()
            nlm._check(nlm._lib.nlm_run_pump(med._h()))
            nlm._check(nlm._lib.nlm_adjoint_forward(med._h(), ctypes.c_void_p(xin.data_ptr()), 1,
                                                    ctypes.c_void_p(out.data_ptr()), 0, ctypes.byref(used)))
            g = (2 * (out - torch.tensor(target.reshape(1, -1), device="cuda"))).contiguous()
            gin = torch.empty_like(xin)
            gp = torch.empty(x.size, dtype=torch.complex128, device="cuda")
            gpol = np.zeros(nz)
            nlm._check(nlm._lib.nlm_adjoint_backward(med._h(), ctypes.c_void_p(g.data_ptr()),
                                                     ctypes.c_void_p(gin.data_ptr()), ctypes.c_void_p(gp.data_ptr()),
                                                     nlm._dptr(gpol)))
        elif name == "signal":
            m = c(nlm.Chi2PDC(poling=np.ones(GREEN_DOMAINS),
                              **dict(GREEN_CONFIG, tPrecision=2048, zPrecision=z_precision or 500)))
            m.runPumpSimulation()
            m.runSignalSimulation((np.random.default_rng(2048).standard_normal(2048) + 0j) * 0.1)
        elif name == "ragged_wide":
            kw = dict(relativeLength=1, nlLength=1, nlLengthOrig=1, beta2=0.4, beta2s=-0.3, beta2o=0, beta1=0,
                      beta1s=1.2, beta1o=0, beta3=0, beta3s=0.05, beta3o=0, diffBeta0=0, tMax=10, tPrecision=2048,
                      zPrecision=z_precision or 200)
            t = np.fft.fftshift(np.linspace(-10, 10, 2048, endpoint=False))
            m = nlm.Chi2SFG(customPump=np.exp(-t ** 2 / 2), poling=[3, 4, 3], **kw)
            m._set_schedule(use_propagator=0)
            c(m)
            m.runPumpSimulation()
            m.runSignalSimulation((np.random.default_rng(1).standard_normal(2048) + 0j) * 1e-3)
        elif name == "gnlse_signal":
            m = c(nlm.Chi3GNLSE(**dict(GNLSE_CONFIG, zPrecision=z_precision or 111)))
            m.runSignalSimulation(gnlse_rows(1)[0])
        elif name == "gnlse":
            m = c(nlm.Chi3GNLSE(**dict(GNLSE_CONFIG, zPrecision=z_precision or 111)))
            m.batchSignalSimulation(gnlse_rows(rows or 304), inTimeDomain=True)
        elif name == "gnlse_grad":
            m = c(nlm.Chi3GNLSE(**dict(GNLSE_CONFIG, zPrecision=z_precision or 111)))
            x = torch.tensor(gnlse_rows(rows or 16), device="cuda")
            w = torch.tensor(m.omega, device="cuda")
            band = ((w >= 2) & (w <= 4)).to(torch.float64)
            phi = torch.zeros(x.shape[1], dtype=torch.float64, device="cuda", requires_grad=True)
            spec = torch.fft.fft(x, dim=1) * torch.exp(1j * phi)[None, :]
            torch.sum(torch.abs(propagate_gnlse(m, spec)) ** 2 * band).backward()
        else:
            raise ValueError("unknown workload %r" % name)
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser(description="run one benchmark workload on cuda:0")
    ap.add_argument("name", choices=["green", "cascade", "chi3", "chi3_pump", "ragged", "adjoint", "adjoint_cluster", "gnlse",
                                     "gnlse_grad", "signal", "gnlse_signal", "ragged_wide"])
    ap.add_argument("--zprecision", type=int, default=0, help="zPrecision override (0: the workload's own)")
    ap.add_argument("--rows", type=int, default=0, help="rows of the GNLSE workloads (0: the workload's own)")
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--cluster", type=int, default=1,
                    help="cluster mode of the workload's media (nlm_set_cluster: 1 default, 3 narrower "
                         "one-point-per-thread forms, 2 four points per thread only, 0 one CTA)")
    args = ap.parse_args()
    from . import build_ext
    build_ext.build()
    _run(args.name, args.zprecision, args.rows, args.reps, args.cluster)


if __name__ == "__main__":
    main()
