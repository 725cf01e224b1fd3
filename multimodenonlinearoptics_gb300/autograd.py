"""Differentiable propagation: a torch.autograd.Function over the engine's adjoint.

``propagate_pdc(medium, signal_in, pump_spectrum, poling)`` returns the output spectra of a Chi2PDC
medium for a batch of input spectra; gradients flow to the input spectra, to the pump spectrum
F0 = FFT(envelope) and to a continuous poling profile d(z) (nZSteps values).  The backward pass is
the engine's hand-written reverse sweep (nlm_adjoint_backward), which uses the forward states
checkpointed by the forward pass.  The reference has no gradient; its forward model is reproduced
exactly (solvers/Chi2PDC.cpp:27-44 with the poling array replaced by d(z)).
"""

import ctypes

import numpy as np
import torch

from . import nonlinearmedium as nlm


class Chi2PDCPropagation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, medium, signal_in, pump_spectrum, poling, checkpoint_interval):
        if signal_in.dtype != torch.complex128 or not signal_in.is_cuda:
            raise TypeError("signal_in must be a complex128 CUDA tensor")
        x = signal_in.detach().reshape(-1, signal_in.shape[-1]).contiguous()
        env = torch.fft.ifft(pump_spectrum.detach().to(torch.complex128)).cpu().numpy()
        medium.setPump(env)
        medium._set_poling_profile(poling.detach().to(torch.float64).cpu().numpy())
        medium.runPumpSimulation()
        out = torch.empty_like(x)
        used = ctypes.c_int()
        nlm._check(nlm._lib.nlm_adjoint_forward(medium._h(), ctypes.c_void_p(x.data_ptr()), x.shape[0],
                                                ctypes.c_void_p(out.data_ptr()), int(checkpoint_interval),
                                                ctypes.byref(used)))
        medium._adjoint_generation = getattr(medium, "_adjoint_generation", 0) + 1
        ctx.medium = medium
        ctx.generation = medium._adjoint_generation
        ctx.shape = signal_in.shape
        ctx.pump_device = pump_spectrum.device
        ctx.poling_device = poling.device
        ctx.checkpoint_interval = used.value
        return out.reshape(signal_in.shape)

    @staticmethod
    def backward(ctx, grad_out):
        med = ctx.medium
        if getattr(med, "_adjoint_generation", None) != ctx.generation:
            raise RuntimeError("the medium ran another differentiable forward pass before this backward pass")
        g = grad_out.detach().to(torch.complex128).reshape(-1, ctx.shape[-1]).contiguous()
        gin = torch.empty_like(g)
        gpump = torch.empty(ctx.shape[-1], dtype=torch.complex128, device=g.device)
        gpol = np.zeros(med._dims["nZSteps"])
        nlm._check(nlm._lib.nlm_adjoint_backward(med._h(), ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(gin.data_ptr()),
                                                 ctypes.c_void_p(gpump.data_ptr()), nlm._dptr(gpol)))
        return (None, gin.reshape(ctx.shape), gpump.to(ctx.pump_device),
                torch.from_numpy(gpol).to(ctx.poling_device), None)


def propagate_pdc(medium, signal_in, pump_spectrum, poling, checkpoint_interval=0):
    """Output spectra (last z row, FFT order) of a Chi2PDC medium; differentiable in all three inputs.

    checkpoint_interval: 0 chooses (every step when the trajectory fits in 40 % of the free device
    memory, at most 96 GB, else every ceil(sqrt(nZSteps-1)) steps with recomputation of the segments
    in the reverse sweep).
    """
    return Chi2PDCPropagation.apply(medium, signal_in, pump_spectrum, poling, checkpoint_interval)


class Chi3GNLSEPropagation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, medium, signal_in, checkpoint_interval):
        if signal_in.dtype != torch.complex128 or not signal_in.is_cuda:
            raise TypeError("signal_in must be a complex128 CUDA tensor")
        x = signal_in.detach().reshape(-1, signal_in.shape[-1]).contiguous()
        out = torch.empty_like(x)
        used = ctypes.c_int()
        nlm._check(nlm._lib.nlm_adjoint_forward(medium._h(), ctypes.c_void_p(x.data_ptr()), x.shape[0],
                                                ctypes.c_void_p(out.data_ptr()), int(checkpoint_interval),
                                                ctypes.byref(used)))
        medium._adjoint_generation = getattr(medium, "_adjoint_generation", 0) + 1
        ctx.medium = medium
        ctx.generation = medium._adjoint_generation
        ctx.shape = signal_in.shape
        return out.reshape(signal_in.shape)

    @staticmethod
    def backward(ctx, grad_out):
        med = ctx.medium
        if getattr(med, "_adjoint_generation", None) != ctx.generation:
            raise RuntimeError("the medium ran another differentiable forward pass before this backward pass")
        g = grad_out.detach().to(torch.complex128).reshape(-1, ctx.shape[-1]).contiguous()
        gin = torch.empty_like(g)
        nlm._check(nlm._lib.nlm_adjoint_backward(med._h(), ctypes.c_void_p(g.data_ptr()), ctypes.c_void_p(gin.data_ptr()),
                                                 None, None))
        return None, gin.reshape(ctx.shape), None


def propagate_gnlse(medium, signal_in, checkpoint_interval=0):
    """Output spectra of a Chi3GNLSE medium for a batch of input spectra (FFT order), differentiable in
    the input spectra (solvers/Chi3GNLSE.cpp:39-92: Raman response and self-steepening)."""
    return Chi3GNLSEPropagation.apply(medium, signal_in, checkpoint_interval)
