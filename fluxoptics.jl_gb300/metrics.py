"""SquaredIntensityDifference on the GPU (metrics/squared_intensity_difference.jl:58-90)."""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _capi
from .components import OpticalSystem, _ptr, _stream
from .fields import ScalarField


class SquaredIntensityDifference:
    """c_t = sum (I_t - target_t)^2 with I_t = sum of |u_b|^2 over the fields b mapped
    to target slice t.

    ``target`` has shape (ny, nx) or (T, ny, nx) (the C view of the reference's
    (nx, ny[, T]) target).  By default field b maps to slice b % T, the broadcast of an
    (nx, ny, T) target over (nx, ny, T, M) fields; ``target_index`` overrides it."""

    def __init__(self, pair, target_index=None):
        u0, target = pair
        t = torch.as_tensor(target.detach().cpu().numpy() if isinstance(target, torch.Tensor) else np.asarray(target),
                            dtype=torch.float32)
        if t.dim() == 2:
            t = t[None]
        if tuple(t.shape[1:]) != (u0.ny, u0.nx):
            raise ValueError("target must have the field's (ny, nx) shape")
        self.target = t.cuda().contiguous()
        self.T = int(t.shape[0])
        self.nx, self.ny, self.batch = u0.nx, u0.ny, u0.batch
        self.handle = C.c_void_p()
        tidx = None if target_index is None else _capi.ivec(target_index)
        _capi.call("fo_sid_create", C.byref(self.handle), self.nx, self.ny, self.batch, self.T, tidx)
        self.loss = torch.zeros(self.T, dtype=torch.float32, device="cuda")

    def __call__(self, u: ScalarField):
        """Per-slice losses (device tensor of T floats)."""
        _capi.call("fo_sid_forward", self.handle, _ptr(u.electric), _ptr(self.target), _ptr(self.loss), _stream())
        return self.loss

    def backpropagate_into(self, u: ScalarField, du: ScalarField, dc=None):
        _capi.call("fo_sid_backward", self.handle, _ptr(u.electric), _ptr(dc), _ptr(du.electric), _stream())
        return du

    def backpropagate(self, u: ScalarField, dc=None):
        du = u.similar()
        return self.backpropagate_into(u, du, dc)

    def __del__(self):
        lib = _capi._LIB
        if lib is not None and getattr(self, "handle", None):
            lib.fo_sid_destroy(self.handle)


def withgradient(metric: SquaredIntensityDifference, system: OpticalSystem, x=None):
    """Loss sum_t c_t and the gradients of every trainable component, through
    the hand-written adjoint (the GPU counterpart of Zygote.withgradient over
    the reference's rrules, src/ChainRulesCoreExt.jl:21-111)."""
    src = system.source.u0 if x is None else x
    u = src.similar()
    tape = []
    system.forward(u, tape, src=src)
    loss = metric(u)
    du = u.similar()
    grads = system.backward(du, tape, seed=(metric, u))
    return loss.sum(), grads
