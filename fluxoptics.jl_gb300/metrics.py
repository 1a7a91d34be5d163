"""Metrics on the GPU: SquaredIntensityDifference
(metrics/squared_intensity_difference.jl:58-90), SquaredFieldDifference
(metrics/squared_field_difference.jl:35-61), DotProduct (metrics/dot_product.jl:47-100)
and PowerCoupling (metrics/power_coupling.jl:48-66)."""

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

    # OpticalSystem.forward(..., metric=m) evaluates it inside the last fused pass
    fuses_into_chain = True

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


class SquaredFieldDifference:
    """c_b = sum |u_b - v_b|^2 over the field's pixels (no dx dy factor), against
    reference fields v of the same grid and batch; pull-back 2 dc_b (u_b - v_b)."""

    def __init__(self, v: ScalarField):
        self.v = v
        self.nx, self.ny, self.batch = v.nx, v.ny, v.batch
        self.handle = C.c_void_p()
        _capi.call("fo_sfd_create", C.byref(self.handle), v.nx, v.ny, v.batch)
        self.out = torch.zeros(self.batch, dtype=torch.float32, device="cuda")

    def _check(self, u: ScalarField):
        if (u.nx, u.ny, u.batch) != (self.nx, self.ny, self.batch):
            raise ValueError("SquaredFieldDifference: the field's grid and batch must match the reference fields")

    def __call__(self, u: ScalarField):
        """Per-field values (device tensor of batch floats)."""
        self._check(u)
        _capi.call("fo_sfd_forward", self.handle, _ptr(u.electric), _ptr(self.v.electric), _ptr(self.out), _stream())
        return self.out

    def backpropagate_into(self, u: ScalarField, du: ScalarField, dc=None):
        self._check(u)
        if dc is not None:
            dc = dc.to(torch.float32).reshape(-1).contiguous()
            if dc.numel() != self.batch:
                raise ValueError("dc must hold one value per field")
        _capi.call("fo_sfd_backward", self.handle, _ptr(u.electric), _ptr(self.v.electric), _ptr(dc),
                   _ptr(du.electric), _stream())
        return du

    def backpropagate(self, u: ScalarField, dc=None):
        du = u.similar()
        return self.backpropagate_into(u, du, dc)

    def __del__(self):
        lib = _capi._LIB
        if lib is not None and getattr(self, "handle", None):
            lib.fo_sfd_destroy(self.handle)


class _Overlap:
    """Common part of DotProduct and PowerCoupling: fields v of the same grid and
    batch as the fields the metric is applied to (one reference field per field)."""

    power = 0

    def __init__(self, v: ScalarField, mode_selective=True):
        self.v = v
        self.mode_selective = bool(mode_selective)
        self.nx, self.ny, self.batch = v.nx, v.ny, v.batch
        self.handle = C.c_void_p()
        _capi.call("fo_overlap_create", C.byref(self.handle), v.nx, v.ny, v.batch, v.ds[0], v.ds[1],
                   _ptr(v.electric), int(self.mode_selective), self.power)
        shape = (self.batch,) if self.mode_selective else (self.batch, self.batch)
        self.out = torch.zeros(shape, dtype=torch.float32 if self.power else torch.complex64, device="cuda")

    def __call__(self, u: ScalarField):
        """Per-field values (mode selective) or the batch x batch matrix; for the
        matrix, out[j, i] is the reference's c[i, j] (column-major storage)."""
        _capi.call("fo_overlap_forward", self.handle, _ptr(u.electric), _ptr(self.out), _stream())
        return self.out

    def backpropagate_into(self, u: ScalarField, du: ScalarField, dc=None):
        if dc is None:
            dc = torch.ones_like(self.out)
        dc = dc.to(self.out.dtype).contiguous()
        _capi.call("fo_overlap_backward", self.handle, _ptr(dc), _ptr(du.electric), _stream())
        return du

    def backpropagate(self, u: ScalarField, dc=None):
        du = u.similar()
        return self.backpropagate_into(u, du, dc)

    def __del__(self):
        lib = _capi._LIB
        if lib is not None and getattr(self, "handle", None):
            lib.fo_overlap_destroy(self.handle)


class DotProduct(_Overlap):
    """c_b = dx dy sum u_b conj(v_b) (or the matrix v' u with mode_selective=False)."""

    power = 0


class PowerCoupling(_Overlap):
    """|DotProduct(u, v_hat)|^2 against unit-power copies v_hat of v."""

    power = 1


def compute_metric(metric, u: ScalarField):
    """The metric's values on u (metrics/Metrics.jl: compute_metric, the callable form)."""
    return metric(u)


def backpropagate_metric(metric, u: ScalarField, dc=None):
    """The metric's pull-back: the gradient with respect to u of sum(dc * c)
    (metrics/Metrics.jl: backpropagate_metric), as a new field."""
    return metric.backpropagate(u, dc)


def withgradient(metric, system: OpticalSystem, x=None, dc=None):
    """Loss sum(dc * c) (dc = 1 by default) and the gradients of every trainable
    component, through the hand-written adjoint (the GPU counterpart of
    Zygote.withgradient over the reference's rrules, src/ChainRulesCoreExt.jl:21-111).
    SquaredIntensityDifference and SquaredFieldDifference seed the adjoint inside the
    first fused pass; the overlap metrics write their pull-back first."""
    src = system.source.u0 if x is None else x
    du = src.similar()

    def with_source(grads):
        # a trainable source's gradient is the adjoint sweep's input gradient
        # (trainable(::ScalarSource), sources/scalar_source.jl:65)
        if system.source is not None and getattr(system.source, "trainable", False):
            grads[system.source] = {"u0": du.electric}
        return grads

    if isinstance(metric, SquaredIntensityDifference) and dc is None:
        # one fused chain ending in a propagator: forward, metric and adjoint in one call
        grads = system.forward_backward_sid(du, src, metric)
        if grads is not None:
            return metric.loss.sum(), with_source(grads)
    if isinstance(metric, SquaredFieldDifference):
        w = None if dc is None else dc.to(device=metric.out.device, dtype=torch.float32).reshape(-1).contiguous()
        # one fused chain: forward, metric, pull-back and adjoint in one call
        grads = system.forward_backward_sfd(du, src, metric, dc=w)
        if grads is not None:
            c = metric.out
            return (c.sum() if w is None else (w * c).sum()), with_source(grads)
    u = src.similar()
    tape = []
    if isinstance(metric, SquaredIntensityDifference):
        system.forward(u, tape, src=src, metric=metric)
        c = metric.loss
    else:
        system.forward(u, tape, src=src)
        c = metric(u)
    du.tilts = u.tilts  # the adjoint sweep starts at the output's tilts (a TiltAnchor may have changed them)
    if isinstance(metric, SquaredIntensityDifference) and dc is None:
        grads = system.backward(du, tape, seed=(metric, u))
        return c.sum(), with_source(grads)
    metric.backpropagate_into(u, du, dc)
    grads = system.backward(du, tape)
    w = torch.ones_like(c) if dc is None else dc.to(c.dtype)
    return (w * c).sum().real if c.is_complex() else (w * c).sum(), with_source(grads)
