"""Noise-rate gradients of a detector error model through ``torch.autograd``.

``NoiseRateDEM(circuit)`` prepares the circuit as a template on the GPU;
calling it with a FP64 CUDA tensor ``noise[num_ticks, 4]`` (see
``greenpeas_gb300.noise`` for ticks and classes) returns the merged
mechanisms' probabilities as a differentiable tensor.  The backward pass is
the FP64 adjoint kernel of the C ABI (``gpc_param_backward``): prefix and
suffix products of (1 - 2 q) along each merged run, the channel-split
derivatives, and a fixed-order reduction into the rate tensor.

The symptoms of the merged mechanisms (which do not depend on the rates) are
in ``last_dem()``, in the same order as the returned probabilities.
"""

from __future__ import annotations

import ctypes

from . import _native
from .error_analysis import _text, dem_from_handle

__all__ = ["NoiseRateDEM"]


def _torch():
    import torch
    return torch


class _Rates:
    """torch.autograd.Function over one NoiseRateDEM (built lazily so torch stays optional)."""

    fn = None

    @classmethod
    def get(cls):
        if cls.fn is None:
            torch = _torch()

            class DemProbabilities(torch.autograd.Function):
                @staticmethod
                def forward(ctx, noise, model):
                    out = model._forward(noise)
                    ctx.model = model
                    ctx.run = model._runs
                    ctx.save_for_backward(noise)
                    return out

                @staticmethod
                def backward(ctx, grad):
                    (noise,) = ctx.saved_tensors
                    if ctx.run != ctx.model._runs:
                        raise RuntimeError("NoiseRateDEM: backward needs its own forward to be the model's latest")
                    return ctx.model._backward(noise, grad), None

            cls.fn = DemProbabilities
        return cls.fn


class NoiseRateDEM:
    """A circuit template whose noise rates come from a [num_ticks, 4] FP64 CUDA tensor."""

    def __init__(self, circuit, correlation_level: int = 2, device: int = 0):
        L = _native.lib()
        text = _text(circuit)
        opts = _native.Options(device=device, sort_bits=64, global_sort=0)
        h = ctypes.c_void_p()
        _native.check(L.gpc_get_driver(text, len(text), int(correlation_level), ctypes.byref(opts), ctypes.byref(h)))
        self._h = h
        nt = ctypes.c_uint32()
        _native.check(L.gpc_param_prepare(self._h, text, len(text), ctypes.byref(nt)))
        self.num_ticks = int(nt.value)
        self.device = device
        self._runs = 0
        self._n = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                _native.lib().gpc_driver_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def shape(self):
        return (self.num_ticks, 4)

    def _check_noise(self, noise):
        torch = _torch()
        if noise.dtype != torch.float64 or not noise.is_cuda or tuple(noise.shape) != self.shape:
            raise ValueError(f"noise must be a float64 CUDA tensor of shape {self.shape}")
        return noise.contiguous()

    def _forward(self, noise):
        torch = _torch()
        noise = self._check_noise(noise)
        stream = ctypes.c_void_p(torch.cuda.current_stream(noise.device).cuda_stream)
        n = ctypes.c_uint32()
        L = _native.lib()
        _native.check(L.gpc_param_forward(self._h, ctypes.c_void_p(noise.data_ptr()), stream, ctypes.byref(n)))
        self._n = int(n.value)
        self._runs += 1
        out = torch.empty(self._n, dtype=torch.float64, device=noise.device)
        if self._n:
            _native.check(L.gpc_param_probs(self._h, ctypes.c_void_p(out.data_ptr()), stream))
        return out

    def _backward(self, noise, grad):
        torch = _torch()
        grad = grad.to(torch.float64).contiguous()
        g = torch.empty(self.shape, dtype=torch.float64, device=noise.device)
        stream = ctypes.c_void_p(torch.cuda.current_stream(noise.device).cuda_stream)
        _native.check(_native.lib().gpc_param_backward(self._h, ctypes.c_void_p(grad.data_ptr()),
                                                        ctypes.c_void_p(g.data_ptr()), stream))
        return g

    def __call__(self, noise):
        """Merged probabilities (DEM order) for the rates in ``noise``, differentiable in ``noise``."""
        return _Rates.get().apply(noise, self)

    def last_dem(self):
        """The DEM of the latest call (host arrays: symptoms and probabilities)."""
        out = ctypes.c_void_p()
        _native.check(_native.lib().gpc_fetch(self._h, ctypes.byref(out)))
        return dem_from_handle(out)
