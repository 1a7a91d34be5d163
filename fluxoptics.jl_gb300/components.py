"""Optical components of the hot path and the fused system executor.

Mirrors the reference's component API (src/optical_components/OpticalComponents.jl,
freespace_propagators/*, modulators/phasemask.jl, modulators/mask.jl,
bulk_propagators/bpm.jl, sources/scalar_source.jl, system/optical_system.jl):
``propagate_`` is Julia's ``propagate!``, ``backpropagate_with_gradient_`` is
``backpropagate_with_gradient!``, and ``a | b`` builds an ``OpticalSystem`` like
``a |> b``.  Every component executes on the GPU through libfluxoptics_gb300;
there is no CPU fallback.

When a system runs, maximal runs ``[mod] prop [mod] prop ... [mod]`` on one grid
are executed as one fused chain (fo_chain_*): the inverse row transform of each
propagator, the modulation after it and the next forward row transform share one
pass over the field, which is the GPU counterpart of the reference's merge rules
that cancel adjacent ift/ft pairs (system/merge_rules.jl:45-52).
"""

from __future__ import annotations

import ctypes as C
import math
import warnings

import numpy as np
import torch

from . import _capi
from ._capi import FO_BACKWARD, FO_FORWARD, fo_mod
from .fields import ScalarField, per_field

Forward = FO_FORWARD
Backward = FO_BACKWARD


def reverse(direction):
    return -direction


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def spatial_vectors(ns, ds, offset=None):
    """Centred grid vectors (src/GridUtils.jl:56-60), Julia order (x, y)."""
    if offset is None:
        offset = (0.0,) * len(ns)
    return tuple((np.arange(n) - (n - 1) / 2.0) * d - c for n, d, c in zip(ns, ds, offset))


def function_to_array(f, ns, ds, isfourier=False):
    """Evaluate f(x, y) on the spatial grid, or on the FFT-ordered frequency grid
    (fftfreq) when ``isfourier``; returns an (ny, nx) array (OpticalComponents.jl:927-935)."""
    if isfourier:
        x, y = np.fft.fftfreq(ns[0], ds[0]), np.fft.fftfreq(ns[1], ds[1])
    else:
        x, y = spatial_vectors(ns, ds)
    xv = x[None, :]
    yv = y[:, None]
    out = np.vectorize(f, otypes=[np.complex128])(np.broadcast_to(xv, (len(y), len(x))),
                                                  np.broadcast_to(yv, (len(y), len(x))))
    return out


class Component:
    """Base of all pipe components.  OpticalSystem drives any component through the
    protocol of the reference's AbstractCustomComponent (OpticalComponents.jl:751-816):
    ``propagate_(u, d)`` in place and its adjoint ``backpropagate_(dv, d)``; a trainable
    component also gives ``params()`` ({name: tensor}), ``propagate_and_save_(u, saved,
    d)`` (``saved`` from ``get_saved_buffer(u)`` when it defines one),
    ``get_gradient_buffer()`` and ``backpropagate_with_gradient_(dv, saved, grad, d)``,
    which returns (dv, {name: grad})."""

    trainable = False
    buffered = False

    def propagate_(self, u: ScalarField, direction=Forward):
        raise NotImplementedError

    def propagate(self, u: ScalarField, direction=Forward):
        return self.propagate_(u.copy(), direction)

    def backpropagate_(self, dv: ScalarField, direction=Forward):
        raise NotImplementedError

    def params(self):
        """Trainable arrays, the reference's ``trainable(p)``."""
        return {}

    def __or__(self, other):
        return OpticalSystem(None, [self]) | other

    def istrainable(self):
        return self.trainable

    def isbuffered(self):
        return self.trainable and self.buffered


# ---------------------------------------------------------------------------
# Propagators
# ---------------------------------------------------------------------------

class _Propagator(Component):
    kind = None
    autotune = True  # time the launch shapes of the passes at plan creation (cached per grid)

    def __init__(self, u: ScalarField, z, ds=None):
        self.z = float(z)
        self.ds = tuple(float(d) for d in (ds if ds is not None else u.ds))
        self._plans = {}
        self.plan_for(u)

    def _create(self, u, lam):
        raise NotImplementedError

    def plan_for(self, u: ScalarField):
        lam = tuple(float(v) for v in u.lambdas_per_field())
        key = (u.nx, u.ny, u.batch, lam, tuple(map(float, u.tilts_per_field().ravel())))
        p = self._plans.get(key)
        if p is None:
            p = self._create(u, lam)
            self._plans[key] = p
        return p

    def layout(self, u: ScalarField):
        h = self.plan_for(u)
        fx, fy = C.c_int(), C.c_int()
        _capi.call("fo_prop_info", h, C.byref(fx), C.byref(fy), None)
        return (self.kind, u.nx, u.ny, u.batch, fx.value, fy.value)

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_propagate", self.plan_for(u), _ptr(u.electric), int(direction), _stream())
        return u

    def backpropagate_(self, dv, direction=Forward):
        # backpropagate! = propagate!(reverse(direction)) (freespace.jl:61-63)
        return self.propagate_(dv, reverse(direction))

    def __del__(self):
        lib = _capi._LIB
        if lib is None:
            return
        for h in getattr(self, "_plans", {}).values():
            lib.fo_prop_destroy(h)


class ASProp(_Propagator):
    """Angular-spectrum propagation (angular_spectrum.jl:193-234)."""

    kind = "AS"

    def __init__(self, u, z, ds=None, n0=1.0, use_cache=True, double_precision_kernel=True,
                 filter=None, paraxial=False, track_tilts=False):
        self.n0 = float(n0)
        self.filter = filter              # (fx, fy) -> transmission, numpy-vectorised
        self.paraxial = bool(paraxial)
        self.track_tilts = bool(track_tilts)
        super().__init__(u, z, ds)

    def _create(self, u, lam):
        h = C.c_void_p()
        tilts = u.tilts_per_field()
        if not (self.paraxial or self.track_tilts or self.filter is not None or np.any(tilts != 0.0)):
            _capi.call("fo_asprop_create", C.byref(h), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                       _capi.dvec(lam), len(lam), self.z, self.n0, int(self.autotune))
            return h
        opt, keep = _as_options(self.paraxial, self.track_tilts, tilts, self.filter)
        _capi.call("fo_asprop_create_ex", C.byref(h), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                   _capi.dvec(lam), len(lam), self.z, self.n0, C.byref(opt), int(self.autotune))
        del keep
        return h


def _as_options(paraxial, track_tilts, tilts, filt):
    """fo_as_options for fo_asprop_create_ex, and the objects that must stay alive
    until the call returns (the tilt array and the filter callback)."""
    opt = _capi.fo_as_options()
    opt.paraxial = int(paraxial)
    opt.track_tilts = int(track_tilts)
    tv = _capi.dvec(np.asarray(tilts).ravel())
    opt.tilts = C.cast(tv, C.POINTER(C.c_double))
    opt.n_tilts = len(tilts)
    cb = None
    if filt is not None:
        def _eval(fx, fy, n, re, im, _ctx):
            fxv = np.ctypeslib.as_array(fx, shape=(n,))
            fyv = np.ctypeslib.as_array(fy, shape=(n,))
            val = np.broadcast_to(np.asarray(filt(fxv, fyv), dtype=np.complex128), (n,))
            np.ctypeslib.as_array(re, shape=(n,))[:] = val.real
            np.ctypeslib.as_array(im, shape=(n,))[:] = val.imag

        cb = _capi.fo_filter_fn(_eval)
        opt.filter = cb
    return opt, (tv, cb)


def ParaxialProp(u, z, ds=None, n0=1.0, filter=None, track_tilts=False, **kw):
    """Fresnel (paraxial) angular-spectrum propagation: ASProp(paraxial=true)
    (angular_spectrum.jl:27-44)."""
    return ASProp(u, z, ds=ds, n0=n0, filter=filter, paraxial=True, track_tilts=track_tilts)


def rs_valid_distance(nx, ny, dx, dy, lam):
    """rayleigh_sommerfeld.jl:29-36."""
    if dx < lam / 2 and dy < lam / 2:
        return 0.0
    zx = 0.0 if dx < lam / 2 else (nx * dx / 2) * math.sqrt(4 * dx ** 2 / lam ** 2 - 1)
    zy = 0.0 if dy < lam / 2 else (ny * dy / 2) * math.sqrt(4 * dy ** 2 / lam ** 2 - 1)
    return max(zx, zy)


class RSProp(_Propagator):
    """Rayleigh-Sommerfeld propagation as a zero-padded FFT convolution
    (rayleigh_sommerfeld.jl:128-169)."""

    kind = "RS"

    def __init__(self, u, z, ds=None, use_cache=True, double_precision_kernel=True, track_tilts=False):
        if track_tilts or not u.is_on_axis():
            raise NotImplementedError("tilted fields in RSProp are not in the GB300 path")
        dsv = tuple(ds) if ds is not None else u.ds
        zc = rs_valid_distance(u.nx, u.ny, dsv[0], dsv[1], float(np.min(u.lambdas_per_field())))
        if abs(z) < zc:
            warnings.warn(f"RSProp: propagation distance z={z} is below critical distance zc={zc}. "
                          "Numerical artifacts expected.")
        super().__init__(u, z, ds)

    def _create(self, u, lam):
        h = C.c_void_p()
        _capi.call("fo_rsprop_create", C.byref(h), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                   _capi.dvec(lam), len(lam), self.z, int(self.autotune))
        return h


# ---------------------------------------------------------------------------
# Modulators
# ---------------------------------------------------------------------------

class _Modulator(Component):
    mod_kind = None
    pname = None

    def _alloc_buffers(self, u):
        if self.trainable and self.buffered:
            self.grad_buffer = torch.empty_like(self.param)
            self.saved_buffer = torch.empty_like(u.electric)
        else:
            self.grad_buffer = None
            self.saved_buffer = None

    @property
    def param(self):
        return getattr(self, self.pname)

    def params(self):
        return {self.pname: self.param} if self.trainable else {}

    def get_data(self):
        return self.param

    def fo_mod(self, saved=None, grad=None, u=None):
        return fo_mod(self.mod_kind, self.param.data_ptr(), saved.data_ptr() if saved is not None else None,
                      grad.data_ptr() if grad is not None else None, 1.0, None)

    def alloc_saved_buffer(self, u):
        return torch.empty_like(u.electric)

    def get_saved_buffer(self, u):
        if self.saved_buffer is not None and self.saved_buffer.shape == u.electric.shape:
            return self.saved_buffer
        return self.alloc_saved_buffer(u)

    def alloc_gradient(self):
        return torch.empty_like(self.param)

    def get_gradient_buffer(self):
        return self.grad_buffer if self.grad_buffer is not None else self.alloc_gradient()


class Phase(_Modulator):
    """u -> u * cis(s*phi) (modulators/phasemask.jl:38-150)."""

    mod_kind = _capi.FO_MOD_PHASE
    pname = "phi"

    def __init__(self, u, f=None, ds=None, trainable=False, buffered=False):
        ds = tuple(ds) if ds is not None else u.ds
        if f is None:
            arr = np.zeros((u.ny, u.nx))
        elif callable(f):
            arr = np.real(function_to_array(f, (u.nx, u.ny), ds))
        else:
            arr = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
            if arr.shape != (u.ny, u.nx):
                raise ValueError(f"phase array must have shape (ny, nx) = {(u.ny, u.nx)}")
        self.phi = torch.as_tensor(np.asarray(arr, dtype=np.float32)).cuda().contiguous()
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)
        self._alloc_buffers(u)

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_phase_forward", _ptr(u.electric), _ptr(self.phi), None, u.nx, u.ny, u.batch,
                   int(direction), _stream())
        return u

    def propagate_and_save_(self, u, saved, direction=Forward):
        _capi.call("fo_phase_forward", _ptr(u.electric), _ptr(self.phi), _ptr(saved), u.nx, u.ny,
                   u.batch, int(direction), _stream())
        return u

    def backpropagate_(self, dv, direction=Forward):
        _capi.call("fo_phase_backward", _ptr(dv.electric), _ptr(self.phi), None, None, dv.nx, dv.ny,
                   dv.batch, int(direction), _stream())
        return dv

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_phase_backward", _ptr(dv.electric), _ptr(self.phi), _ptr(saved), _ptr(grad),
                   dv.nx, dv.ny, dv.batch, int(direction), _stream())
        return dv, {"phi": grad}


class TeaDOE(_Modulator):
    """Thin-element DOE: u -> r(λ) cis(2π dn(λ) h / λ) u, conj(r) and the opposite
    phase backward (modulators/tea_doe.jl:38-215).  ``dn`` and ``r`` are numbers
    or functions of the wavelength; the trainable parameter is the height ``h``."""

    mod_kind = _capi.FO_MOD_TEA
    pname = "h"

    def __init__(self, u, dn, f=None, ds=None, r=1.0, trainable=False, buffered=False):
        ds = tuple(ds) if ds is not None else u.ds
        if f is None:
            arr = np.zeros((u.ny, u.nx))
        elif callable(f):
            arr = np.real(function_to_array(f, (u.nx, u.ny), ds))
        else:
            arr = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
            if arr.shape != (u.ny, u.nx):
                raise ValueError(f"height array must have shape (ny, nx) = {(u.ny, u.nx)}")
        self.h = torch.as_tensor(np.asarray(arr, dtype=np.float32)).cuda().contiguous()
        self.dn = dn if callable(dn) else (lambda lam, _v=float(dn): _v)
        self.r = r if callable(r) else (lambda lam, _v=complex(r): _v)
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)
        self._coefs = {}
        self._alloc_buffers(u)

    def field_coef(self, u: ScalarField):
        """Device float[batch][4] = {2π dn(λ_b)/λ_b, Re r(λ_b), Im r(λ_b), 0}, per field."""
        lams = tuple(float(v) for v in u.lambdas_per_field())
        c = self._coefs.get(lams)
        if c is None:
            rows = []
            for lam in lams:
                rv = complex(self.r(lam))
                rows.append([2.0 * math.pi * float(self.dn(lam)) / lam, rv.real, rv.imag, 0.0])
            c = torch.tensor(np.asarray(rows, dtype=np.float32)).cuda().contiguous()
            self._coefs[lams] = c
        return c

    def fo_mod(self, saved=None, grad=None, u=None):
        if u is None:
            raise ValueError("TeaDOE needs the field to build its per-wavelength coefficients")
        return fo_mod(self.mod_kind, self.h.data_ptr(), saved.data_ptr() if saved is not None else None,
                      grad.data_ptr() if grad is not None else None, 1.0, self.field_coef(u).data_ptr())

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_tea_forward", _ptr(u.electric), _ptr(self.h), _ptr(self.field_coef(u)), None, u.nx,
                   u.ny, u.batch, int(direction), _stream())
        return u

    def propagate_and_save_(self, u, saved, direction=Forward):
        _capi.call("fo_tea_forward", _ptr(u.electric), _ptr(self.h), _ptr(self.field_coef(u)), _ptr(saved),
                   u.nx, u.ny, u.batch, int(direction), _stream())
        return u

    def backpropagate_(self, dv, direction=Forward):
        _capi.call("fo_tea_backward", _ptr(dv.electric), _ptr(self.h), _ptr(self.field_coef(dv)), None, None,
                   dv.nx, dv.ny, dv.batch, int(direction), _stream())
        return dv

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_tea_backward", _ptr(dv.electric), _ptr(self.h), _ptr(self.field_coef(dv)), _ptr(saved),
                   _ptr(grad), dv.nx, dv.ny, dv.batch, int(direction), _stream())
        return dv, {"h": grad}


def TeaReflector(u, f=None, ds=None, r=1.0, trainable=False, buffered=False):
    """Reflective thin element: TeaDOE with dn = 2 (phase 4π h / λ) (tea_doe.jl:84-127)."""
    return TeaDOE(u, 2.0, f, ds=ds, r=r, trainable=trainable, buffered=buffered)


class ASPropZ(_Modulator):
    """Angular-spectrum propagation with a trainable distance z
    (angular_spectrum.jl:236-344), with the on-axis, tilted (fields with tilts,
    ``track_tilts``) or ``paraxial`` kernel and an optional frequency ``filter``, like
    the reference's.  z lives in device memory; every forward rebuilds the transfer
    functions from it in FP64, and the adjoint sweep gets dL/dz from fo_prop_z_gradient."""

    pname = "z"

    def __init__(self, u, z, ds=None, n0=1.0, trainable=False, track_tilts=False, paraxial=False,
                 filter=None, double_precision_kernel=False):
        self.ds = tuple(float(d) for d in (ds if ds is not None else u.ds))
        self.n0 = float(n0)
        self.paraxial = bool(paraxial)
        self.track_tilts = bool(track_tilts)
        self.filter = filter
        self.z = torch.tensor([float(z)], dtype=torch.float32, device="cuda")
        self.trainable = bool(trainable)
        self.buffered = False
        self.grad_buffer = None
        self.saved_buffer = None
        self._plans = {}
        self.plan_for(u)

    def plan_for(self, u: ScalarField):
        lam = tuple(float(v) for v in u.lambdas_per_field())
        tilts = u.tilts_per_field()
        key = (u.nx, u.ny, u.batch, lam, tuple(tilts.ravel()))
        p = self._plans.get(key)
        if p is None:
            p = C.c_void_p()
            flags = 1 | _capi.FO_FLAG_DEVICE_Z | (_capi.FO_FLAG_GRAD_SPECTRA if self.trainable else 0)
            if not (self.paraxial or self.track_tilts or self.filter is not None or np.any(tilts != 0.0)):
                _capi.call("fo_asprop_create", C.byref(p), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                           _capi.dvec(lam), len(lam), float(self.z.item()), self.n0, flags)
            else:
                opt, keep = _as_options(self.paraxial, self.track_tilts, tilts, self.filter)
                _capi.call("fo_asprop_create_ex", C.byref(p), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                           _capi.dvec(lam), len(lam), float(self.z.item()), self.n0, C.byref(opt), flags)
                del keep
            self._plans[key] = p
        return p

    def propagate_(self, u, direction=Forward):
        h = self.plan_for(u)
        _capi.call("fo_prop_set_z", h, _ptr(self.z), _stream())
        _capi.call("fo_propagate", h, _ptr(u.electric), int(direction), _stream())
        return u

    def propagate_and_save_(self, u, saved, direction=Forward):
        saved.copy_(u.electric)
        return self.propagate_(u, direction)

    def backpropagate_(self, dv, direction=Forward):
        _capi.call("fo_propagate", self.plan_for(dv), _ptr(dv.electric), int(reverse(direction)), _stream())
        return dv

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_prop_z_gradient", self.plan_for(dv), _ptr(self.z), _ptr(saved), _ptr(dv.electric),
                   int(direction), _ptr(grad), _stream())
        self.backpropagate_(dv, direction)
        return dv, {"z": grad}

    def __del__(self):
        lib = _capi._LIB
        if lib is None:
            return
        for h in getattr(self, "_plans", {}).values():
            lib.fo_prop_destroy(h)


class _FourierModulator(_Modulator):
    """u -> IFFT2(w FFT2(u)), w = cis(phi) or m on the FFT-ordered frequency grid
    (FourierWrapper(ft, Phase|Mask, ift), fourier/fourier_wrapper.jl:1-5).  A static
    one is a propagator of the fused chains (the multiplier rides in the column pass);
    a trainable one runs on its own and gets its gradient from fo_fourier_gradient."""

    kind = "AS"  # unpadded pass layout: chains with ASProps

    def _init_param(self, u, arr, dtype, trainable, buffered):
        setattr(self, self.pname, torch.as_tensor(np.asarray(arr, dtype=dtype)).cuda().contiguous())
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)
        self._plans = {}
        self._alloc_buffers(u)
        self.plan_for(u)

    def plan_for(self, u: ScalarField):
        key = (u.nx, u.ny, u.batch)
        p = self._plans.get(key)
        if p is None:
            p = C.c_void_p()
            flags = 1 | (_capi.FO_FOURIER_TRAINABLE if self.trainable else 0)
            _capi.call("fo_fourier_create", C.byref(p), u.nx, u.ny, u.batch, flags)
            self._plans[key] = p
        return p

    def layout(self, u: ScalarField):
        h = self.plan_for(u)
        fx, fy = C.c_int(), C.c_int()
        _capi.call("fo_prop_info", h, C.byref(fx), C.byref(fy), None)
        return (self.kind, u.nx, u.ny, u.batch, fx.value, fy.value)

    def refresh(self, u: ScalarField):
        """Rebuild the multiplier from the current parameter (stream-ordered)."""
        _capi.call("fo_fourier_set", self.plan_for(u), self.mod_kind, _ptr(self.param), _stream())

    def propagate_(self, u, direction=Forward):
        self.refresh(u)
        _capi.call("fo_propagate", self.plan_for(u), _ptr(u.electric), int(direction), _stream())
        return u

    def propagate_and_save_(self, u, saved, direction=Forward):
        saved.copy_(u.electric)
        return self.propagate_(u, direction)

    def backpropagate_(self, dv, direction=Forward):
        _capi.call("fo_propagate", self.plan_for(dv), _ptr(dv.electric), int(reverse(direction)), _stream())
        return dv

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_fourier_gradient", self.plan_for(dv), self.mod_kind, _ptr(self.param), _ptr(saved),
                   _ptr(dv.electric), _ptr(grad), int(direction), _stream())
        self.backpropagate_(dv, direction)
        return dv, {self.pname: grad}

    def __del__(self):
        lib = _capi._LIB
        if lib is None:
            return
        for h in getattr(self, "_plans", {}).values():
            lib.fo_prop_destroy(h)


class FourierPhase(_FourierModulator):
    """Phase mask applied in the Fourier domain (fourier/fourier_phase.jl:29-65); ``f``
    is a function of (fx, fy) or an (ny, nx) array on the FFT-ordered frequency grid."""

    mod_kind = _capi.FO_MOD_PHASE
    pname = "phi"

    def __init__(self, u, f=None, ds=None, trainable=False, buffered=False):
        ds = tuple(ds) if ds is not None else u.ds
        if f is None:
            arr = np.zeros((u.ny, u.nx))
        elif callable(f):
            arr = np.real(function_to_array(f, (u.nx, u.ny), ds, isfourier=True))
        else:
            arr = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
        self._init_param(u, arr, np.float32, trainable, buffered)


class FourierMask(_FourierModulator):
    """Complex mask applied in the Fourier domain (fourier/fourier_mask.jl)."""

    mod_kind = _capi.FO_MOD_MASK
    pname = "m"

    def __init__(self, u, f=None, ds=None, trainable=False, buffered=False):
        ds = tuple(ds) if ds is not None else u.ds
        if f is None:
            arr = np.ones((u.ny, u.nx), dtype=np.complex128)
        elif callable(f):
            arr = function_to_array(f, (u.nx, u.ny), ds, isfourier=True)
        else:
            arr = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
        self._init_param(u, arr, np.complex64, trainable, buffered)


class Mask(_Modulator):
    """u -> u * m (conj(m) backward) (modulators/mask.jl:39-142)."""

    mod_kind = _capi.FO_MOD_MASK
    pname = "m"

    def __init__(self, u, f=None, ds=None, trainable=False, buffered=False):
        ds = tuple(ds) if ds is not None else u.ds
        if f is None:
            arr = np.ones((u.ny, u.nx), dtype=np.complex128)
        elif callable(f):
            arr = function_to_array(f, (u.nx, u.ny), ds)
        else:
            arr = f.detach().cpu().numpy() if isinstance(f, torch.Tensor) else np.asarray(f)
            if arr.shape != (u.ny, u.nx):
                raise ValueError(f"mask array must have shape (ny, nx) = {(u.ny, u.nx)}")
        self.m = torch.as_tensor(np.asarray(arr, dtype=np.complex64)).cuda().contiguous()
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)
        self._alloc_buffers(u)

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_mask_forward", _ptr(u.electric), _ptr(self.m), None, u.nx, u.ny, u.batch,
                   int(direction), _stream())
        return u

    def propagate_and_save_(self, u, saved, direction=Forward):
        _capi.call("fo_mask_forward", _ptr(u.electric), _ptr(self.m), _ptr(saved), u.nx, u.ny, u.batch,
                   int(direction), _stream())
        return u

    def backpropagate_(self, dv, direction=Forward):
        _capi.call("fo_mask_backward", _ptr(dv.electric), _ptr(self.m), None, None, dv.nx, dv.ny,
                   dv.batch, int(direction), _stream())
        return dv

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_mask_backward", _ptr(dv.electric), _ptr(self.m), _ptr(saved), _ptr(grad), dv.nx,
                   dv.ny, dv.batch, int(direction), _stream())
        return dv, {"m": grad}


# ---------------------------------------------------------------------------
# AS_BPM
# ---------------------------------------------------------------------------

class AS_BPM(Component):
    """Split-step beam propagation with angular-spectrum steps (bpm.jl:130-142).

    ``dn0`` has shape (n_slices, ny, nx) -- the C view of the reference's
    (nx, ny, n_slices) array.  The adjoint keeps every ``checkpoint_every``-th
    slice input and recomputes the rest (0: round(sqrt(n_slices)); 1: keep all).
    ``paraxial`` selects the Fresnel steps; fields with tilts take the tilted steps
    and the per-field kdz = 2 pi dz / (cos theta_x cos theta_y) (bpm.jl:3-6).  The
    reference computes but never applies its ``aperture`` mask, so it is accepted
    and ignored here too."""

    def __init__(self, u, thickness, n0, dn0, use_cache=True, paraxial=False, trainable=False,
                 buffered=False, aperture=None, double_precision_kernel=True, checkpoint_every=0):
        self.paraxial = bool(paraxial)
        dn = dn0.detach().cpu().numpy() if isinstance(dn0, torch.Tensor) else np.asarray(dn0)
        if dn.ndim != 3 or dn.shape[1:] != (u.ny, u.nx):
            raise ValueError("dn0 must have shape (n_slices, ny, nx)")
        if dn.shape[0] < 2:
            raise ValueError("AS_BPM needs at least 2 slices")
        self.dn = torch.as_tensor(np.asarray(dn, dtype=np.float32)).cuda().contiguous()
        self.thickness = float(thickness)
        self.n0 = float(n0)
        self.n_slices = dn.shape[0]
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)
        self.checkpoint_every = int(checkpoint_every)
        self.ds = u.ds
        self._bpms = {}
        self.grad_buffer = torch.empty_like(self.dn) if (self.trainable and self.buffered) else None
        self.handle(u)

    def handle(self, u):
        lam = tuple(float(v) for v in u.lambdas_per_field())
        tilts = u.tilts_per_field()
        key = (u.nx, u.ny, u.batch, lam, tuple(map(float, tilts.ravel())))
        h = self._bpms.get(key)
        if h is None:
            h = C.c_void_p()
            if self.paraxial or np.any(tilts != 0.0):
                opt, keep = _as_options(self.paraxial, False, tilts, None)
                _capi.call("fo_bpm_create_ex", C.byref(h), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                           _capi.dvec(lam), len(lam), self.thickness, self.n0, self.n_slices,
                           self.checkpoint_every, C.byref(opt), 1)
                del keep
            else:
                _capi.call("fo_bpm_create", C.byref(h), u.nx, u.ny, u.batch, self.ds[0], self.ds[1],
                           _capi.dvec(lam), len(lam), self.thickness, self.n0, self.n_slices,
                           self.checkpoint_every, 1.0, 1)
            self._bpms[key] = h
        return h

    def params(self):
        return {"dn": self.dn} if self.trainable else {}

    def get_data(self):
        return self.dn

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_bpm_forward", self.handle(u), _ptr(u.electric), _ptr(self.dn), int(direction), 0,
                   _stream())
        return u

    def propagate_and_save_(self, u, saved=None, direction=Forward):
        _capi.call("fo_bpm_forward", self.handle(u), _ptr(u.electric), _ptr(self.dn), int(direction), 1,
                   _stream())
        return u

    def backpropagate_with_gradient_(self, dv, saved, grad, direction=Forward):
        _capi.call("fo_bpm_backward", self.handle(dv), _ptr(dv.electric), _ptr(self.dn), _ptr(grad),
                   int(direction), _stream())
        return dv, {"dn": grad}

    def get_gradient_buffer(self):
        return self.grad_buffer if self.grad_buffer is not None else torch.empty_like(self.dn)

    def __del__(self):
        lib = _capi._LIB
        if lib is None:
            return
        for h in getattr(self, "_bpms", {}).values():
            lib.fo_bpm_destroy(h)


# ---------------------------------------------------------------------------
# Source and system
# ---------------------------------------------------------------------------

class ScalarSource:
    """Holds the input field (sources/scalar_source.jl:39-106)."""

    def __init__(self, u: ScalarField, trainable=False, buffered=False):
        self.u0 = u.copy()
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)

    def propagate(self):
        return self.u0.copy()

    def params(self):
        return {"u0": self.u0.electric} if self.trainable else {}

    def get_source(self):
        return self.u0

    def __or__(self, other):
        return OpticalSystem(self, []) | other


class FourierOperator(Component):
    """In-place 2-D FFT (``direct=True``) or inverse FFT (``direct=False``) of every
    field, FFTW's unnormalised fft and 1/(nx ny)-normalised ifft; the Backward direction
    swaps the two (fourier/fourier_operator.jl:37-83).  Its pull-back is the exact
    adjoint of the transform it applied: F^H for the FFT, F / (nx ny) for the inverse."""

    def __init__(self, u, direct):
        self.direct = bool(direct)
        self._plans = {}

    def _plan(self, u):
        key = (u.nx, u.ny, u.batch)
        h = self._plans.get(key)
        if h is None:
            h = C.c_void_p()
            # a z = 0 ASProp plan gives the grid's transform layout and twiddles
            _capi.call("fo_asprop_create", C.byref(h), u.nx, u.ny, u.batch, u.ds[0], u.ds[1], _capi.dvec([1.0]), 1,
                       0.0, 1.0, 0)
            self._plans[key] = h
        return h

    def _is_fft(self, direction):
        return self.direct == (int(direction) == int(Forward))

    def propagate_(self, u, direction=Forward):
        _capi.call("fo_fft2", self._plan(u), _ptr(u.electric),
                   _capi.FO_FFT_FORWARD if self._is_fft(direction) else _capi.FO_FFT_INVERSE, _stream())
        return u

    def backpropagate_(self, dv, direction=Forward):
        mode = _capi.FO_FFT_FORWARD_ADJOINT if self._is_fft(direction) else _capi.FO_FFT_INVERSE_ADJOINT
        _capi.call("fo_fft2", self._plan(dv), _ptr(dv.electric), mode, _stream())
        return dv

    def __del__(self):
        lib = _capi._LIB
        if lib is not None:
            for h in getattr(self, "_plans", {}).values():
                lib.fo_prop_destroy(h)


class TiltAnchor(Component):
    """Resets the field's tilts to the ones of the template field it was built from,
    moving the difference of the carriers into the envelope with offset_tilts_
    (utilities/tilt_anchor.jl:1-84).  In a system its pull-back restores the tilts the
    field had on entry (the exact adjoint of the offset, as the reference's trainable
    form computes it); the standalone ``backpropagate_`` offsets to the anchor's tilts
    like the reference's static form.  It has no trainable parameters."""

    def __init__(self, u, trainable=False, buffered=False):
        tc = u.tilts_per_field()
        shape = u.julia_batch_shape
        self.tilts = tuple(tc[:, k].reshape(shape, order="F") if shape else float(tc[0, k]) for k in range(2))
        self.trainable = bool(trainable)
        self.buffered = bool(buffered)

    def params(self):
        return {}

    def propagate_(self, u, direction=Forward):
        return u.offset_tilts_(self.tilts)

    def backpropagate_(self, dv, direction=Forward):
        return dv.offset_tilts_(self.tilts)


class OpticalSequence(Component):
    """Components applied as one (system/optical_sequence.jl:54-137): in order for the
    Forward direction and in reverse order for the Backward direction, each with that
    direction.  Inside an OpticalSystem the sequence is expanded that way before the
    components are fused, so it costs nothing over listing its components."""

    def __init__(self, *components):
        self.components = list(components)
        self.trainable = any(getattr(c, "trainable", False) for c in self.components)
        self._systems = {}

    def get_sequence(self):
        return tuple(self.components)

    def expanded(self, direction=Forward):
        seq = self.components if int(direction) == int(Forward) else list(reversed(self.components))
        out = []
        for c in seq:
            out.extend(c.expanded(direction) if isinstance(c, OpticalSequence) else [c])
        return out

    def __len__(self):
        return len(self.expanded())

    def propagate_(self, u, direction=Forward):
        s = self._systems.get(int(direction))
        if s is None:
            s = OpticalSystem(None, [self], direction=direction)
            self._systems[int(direction)] = s
        return s.forward(u)

    def backpropagate_(self, dv, direction=Forward):
        for c in reversed(self.expanded(direction)):
            c.backpropagate_(dv, direction)
        return dv


def get_sequence(p):
    """The components of a sequence (optical_sequence.jl: get_sequence)."""
    return p.get_sequence()


def FourierWrapper(u, *components):
    """FFT, the components on the spectrum, inverse FFT (fourier/fourier_wrapper.jl:1-42),
    as an OpticalSequence (reversed, with each part's Backward form, in the Backward
    direction)."""
    return OpticalSequence(FourierOperator(u, True), *components, FourierOperator(u, False))


class FieldProbe(Component):
    """Records the field where it sits (system/field_probe.jl:31-43): calling the
    system returns a copy of the field at every probe in ``result["probes"][probe]``
    (system/optical_system.jl:194-214).  Inside a fused chain the copy is written by
    the row pass that produces that plane, so a probe costs no extra pass; the field
    itself is unchanged."""

    def propagate_(self, u, direction=Forward):
        return u


# ---------------------------------------------------------------------------
# Padding and cropping
# ---------------------------------------------------------------------------

def _grid_of(u):
    """(tensor, rebuild) for a ScalarField or a CUDA complex tensor of shape (..., ny, nx)."""
    if isinstance(u, ScalarField):
        return u.electric, lambda t: u.set_field_data(t)
    if isinstance(u, torch.Tensor) and u.is_cuda and u.dtype == torch.complex64:
        return u.contiguous(), lambda t: t
    raise TypeError("pad / crop take a ScalarField or a CUDA complex64 tensor")


def _pad_into(src, dst, offset, fill):
    ny, nx = src.shape[-2:]
    py, px = dst.shape[-2:]
    batch = src.numel() // (nx * ny)
    fill = complex(fill)
    _capi.call("fo_pad", _ptr(src), nx, ny, _ptr(dst), px, py, batch, int(offset[0]), int(offset[1]), fill.real,
               fill.imag, _stream())


def _crop_into(src, dst, offset):
    py, px = src.shape[-2:]
    ny, nx = dst.shape[-2:]
    batch = dst.numel() // (nx * ny)
    _capi.call("fo_crop", _ptr(src), px, py, _ptr(dst), nx, ny, batch, int(offset[0]), int(offset[1]), _stream())


def pad(u, ns, offset=(0, 0), pad_val=0):
    """A new field of size ns = (px, py) (Julia order) holding pad_val, with u placed at
    the 0-based offset (ox, oy) (utilities/pad_crop_operators.jl:18-59)."""
    t, rebuild = _grid_of(u)
    out = torch.empty(tuple(t.shape[:-2]) + (int(ns[1]), int(ns[0])), dtype=torch.complex64, device=t.device)
    _pad_into(t, out, offset, pad_val)
    return rebuild(out)


def crop(u, ns, offset=(0, 0)):
    """The block of size ns = (nx, ny) at the 0-based offset (ox, oy) of u
    (utilities/pad_crop_operators.jl:81-120)."""
    t, rebuild = _grid_of(u)
    out = torch.empty(tuple(t.shape[:-2]) + (int(ns[1]), int(ns[0])), dtype=torch.complex64, device=t.device)
    _crop_into(t, out, offset)
    return rebuild(out)


def _padded_size(u_tmp):
    if isinstance(u_tmp, ScalarField):
        return (u_tmp.nx, u_tmp.ny)
    if isinstance(u_tmp, (tuple, list)) and len(u_tmp) == 2 and all(isinstance(v, (int, np.integer)) for v in u_tmp):
        return (int(u_tmp[0]), int(u_tmp[1]))
    shape = tuple(u_tmp.shape)
    if len(shape) < 2:
        raise ValueError("the padded template needs two spatial dims")
    return (int(shape[-1]), int(shape[-2]))


class PadCropOperator(Component):
    """Reversible padding of a field into a larger grid (pad_crop_operators.jl:122-356).

    ``PadCropOperator(u, u_tmp; offset, pad_val)`` pads fields of u's grid to the grid of
    ``u_tmp`` (a ScalarField, an array of shape (..., py, px), or (px, py)) with u at the
    0-based ``offset`` (ox, oy); ``adjoint()`` gives the operator that crops back.  In the
    Backward direction the two swap roles, and the pull-back of either is the operation
    of the reversed direction, as in the reference (for pad_val = 0 this is the exact
    adjoint).  Inside an OpticalSystem, the components between a padding operator and
    its cropping partner run on the padded grid (they are built on it, as the reference's
    ``ASProp(set_field_data(u, u_tmp), z)``).  ``store_ref`` is accepted for the
    reference's signature; the padded buffers are owned by the system either way."""

    def __init__(self, u, u_tmp, offset=(0, 0), pad_val=0, store_ref=False):
        self.n = (u.nx, u.ny)
        self.p = _padded_size(u_tmp)
        self.offset = (int(offset[0]), int(offset[1]))
        self.pad_val = complex(pad_val)
        self.store_ref = bool(store_ref)
        self.ispad = True
        if min(self.offset) < 0:
            raise ValueError("offsets must be non-negative")
        if self.offset[0] + self.n[0] > self.p[0] or self.offset[1] + self.n[1] > self.p[1]:
            raise ValueError(f"a {self.n} field at offset {self.offset} does not fit in {self.p}")

    def adjoint(self):
        c = PadCropOperator.__new__(PadCropOperator)
        c.__dict__.update(self.__dict__)
        c.ispad = not self.ispad
        return c

    def pads(self, direction=Forward):
        return self.ispad == (int(direction) == int(Forward))

    def pairs_with(self, other):
        return isinstance(other, PadCropOperator) and (self.n, self.p, self.offset) == (other.n, other.p,
                                                                                         other.offset)

    def _apply(self, u, padding):
        want = self.n if padding else self.p
        if (u.nx, u.ny) != want:
            raise ValueError(f"PadCropOperator: a {'padding' if padding else 'cropping'} step takes a {want} grid, "
                             f"got {(u.nx, u.ny)}")
        return pad(u, self.p, self.offset, self.pad_val) if padding else crop(u, self.n, self.offset)

    def propagate(self, u, direction=Forward):
        return self._apply(u, self.pads(direction))

    def propagate_(self, u, direction=Forward):
        raise TypeError("PadCropOperator changes the grid: use propagate, or place it in an OpticalSystem")

    def backpropagate(self, dv, direction=Forward):
        return self._apply(dv, not self.pads(direction))


def adjoint(p):
    """The reference's ``adjoint(p)`` / ``p'`` for PadCropOperator."""
    return p.adjoint()


class _PaddedSpan:
    """The components between a padding PadCropOperator and its cropping partner, run
    as a system on the padded grid: pad u into a padded buffer, run the components in
    place there, crop back into u.  The adjoint pads the incoming gradient (the crop's
    pull-back), runs the components' adjoint sweep and crops (the pad's pull-back)."""

    trainable = False

    def __init__(self, pad_op, inner, crop_op, direction, merge):
        self.pad_op, self.crop_op = pad_op, crop_op
        self.inner = OpticalSystem(None, inner, direction=direction, merge_components=merge)
        self._bufs = {}

    def _buf(self, u, key):
        px, py = self.pad_op.p
        shape = tuple(u.electric.shape[:-2]) + (py, px)
        t = self._bufs.get((key, shape))
        if t is None:
            t = torch.empty(shape, dtype=torch.complex64, device=u.electric.device)
            self._bufs[(key, shape)] = t
        return u.set_field_data(t)

    def forward(self, u, tape, probes):
        w = self._buf(u, "fwd")
        _pad_into(u.electric, w.electric, self.pad_op.offset, self.pad_op.pad_val)
        inner_tape = [] if tape is not None else None
        self.inner.forward(w, inner_tape, probes=probes)
        _crop_into(w.electric, u.electric, self.crop_op.offset)
        if tape is not None:
            tape.append((self, inner_tape))

    def backward(self, du, inner_tape):
        dw = self._buf(du, "bwd")
        _pad_into(du.electric, dw.electric, self.crop_op.offset, self.crop_op.pad_val)
        grads = self.inner.backward(dw, inner_tape, input_grad=True)
        _crop_into(dw.electric, du.electric, self.pad_op.offset)
        return grads


def _is_mod(c):
    return isinstance(c, (Phase, Mask, TeaDOE))


def _is_prop(c):
    return isinstance(c, _Propagator) or (isinstance(c, _FourierModulator) and not c.trainable)


class _Chain:
    def __init__(self, props, mods, probes=()):
        self.props = props
        self.mods = mods  # len(props) + 1, entries None or modulators
        # (("pre" | "post", slot k), FieldProbe): the plane entering / leaving modulation slot k
        self.probes = list(probes)


def _merge_pair(a, b, u):
    """The merge of two adjacent components (system/merge_rules.jl:1-80), or None."""
    if getattr(a, "trainable", False) or getattr(b, "trainable", False):
        return None
    if type(a) is ASProp and type(b) is ASProp:
        # one ASProp over z1 + z2 is the product of the two kernels when the distances
        # have the same sign (for opposite signs the evanescent parts of the reference's
        # kernels, conjugated for z < 0, do not combine that way)
        if (a.filter is None and b.filter is None and a.n0 == b.n0 and a.paraxial == b.paraxial
                and a.track_tilts == b.track_tilts and a.ds == b.ds and (a.z >= 0) == (b.z >= 0)):
            return ASProp(u, a.z + b.z, ds=a.ds, n0=a.n0, paraxial=a.paraxial, track_tilts=a.track_tilts)
        return None
    if type(a) is Phase and type(b) is Phase and a.phi.shape == b.phi.shape:
        return Phase(u, a.phi + b.phi)
    if type(a) in (Phase, Mask) and type(b) in (Phase, Mask) and (Mask in (type(a), type(b))):
        fa = a.m if type(a) is Mask else torch.polar(torch.ones_like(a.phi), a.phi)
        fb = b.m if type(b) is Mask else torch.polar(torch.ones_like(b.phi), b.phi)
        if fa.shape == fb.shape:
            return Mask(u, fa * fb)
    return None


class OpticalSystem:
    """Source + pipe components (system/optical_system.jl:60-214)."""

    def __init__(self, source, components, direction=Forward, inplace=True, merge_components=True):
        self.source = source
        self.components = list(components)
        self.direction = direction
        self.inplace = inplace
        self.merge_components = merge_components
        self._chains = {}

    def __or__(self, other):
        if isinstance(other, OpticalSystem):
            if other.source is not None:
                raise ValueError("the right-hand system must not have a source")
            return OpticalSystem(self.source, self.components + other.components, self.direction)
        if isinstance(other, Component):
            return OpticalSystem(self.source, self.components + [other], self.direction)
        raise TypeError(f"cannot pipe {type(other)}")

    def __len__(self):
        return len(self.components)

    def get_components(self):
        return list(self.components)

    def leaf_components(self):
        """The components with every OpticalSequence expanded for the system's direction:
        the order in which they are applied."""
        out = []
        for c in self.components:
            out.extend(c.expanded(self.direction) if isinstance(c, OpticalSequence) else [c])
        return out

    # -- planning ---------------------------------------------------------------
    def merged_components(self, u: ScalarField):
        """The components after the reference's merge rules (system/merge_rules.jl:1-80),
        applied to directly adjacent static components: two ASProps with the same
        options and no filter become one ASProp over the summed distance (the product of
        their transfer functions, so the FFT pair between them cancels as ift * ft does);
        two phases add; masks and phases multiply into one mask.  Merged components are
        new objects; the caller's own components are left unchanged.  The list is cached
        per field shape."""
        key = (u.nx, u.ny, u.batch, tuple(float(v) for v in u.lambdas_per_field()),
               tuple(map(float, u.tilts_per_field().ravel())))
        cache = self.__dict__.setdefault("_merged", {})
        if key in cache:
            return cache[key]
        out = []
        depth = 0  # inside a padded span the components live on another grid: not merged here
        for c in self.leaf_components():
            if isinstance(c, PadCropOperator):
                depth += 1 if c.pads(self.direction) else -1
                out.append(c)
                continue
            prev = out[-1] if out else None
            m = _merge_pair(prev, c, u) if (prev is not None and depth == 0) else None
            if m is not None:
                out[-1] = m
            else:
                out.append(c)
        cache[key] = out
        return out

    def _padded_span(self, comps, i):
        """The span that starts with the padding operator comps[i]: (span, index of its
        cropping partner).  Spans nest; each is built once and kept with the system."""
        depth = 0
        for k in range(i, len(comps)):
            c = comps[k]
            if isinstance(c, PadCropOperator):
                depth += 1 if c.pads(self.direction) else -1
                if depth == 0:
                    if not comps[i].pairs_with(c):
                        raise ValueError("a PadCropOperator span must end with the operator that undoes its pad")
                    spans = self.__dict__.setdefault("_spans", {})
                    key = tuple(id(x) for x in comps[i:k + 1])
                    sp = spans.get(key)
                    if sp is None:
                        sp = _PaddedSpan(comps[i], comps[i + 1:k], c, self.direction, self.merge_components)
                        spans[key] = sp
                    return sp, k
        raise ValueError("a padding PadCropOperator has no cropping partner later in the system")

    def segments(self, u: ScalarField):
        """Split the components into fused chains and single components."""
        comps = self.merged_components(u) if self.merge_components else self.leaf_components()
        segs = []
        i, n = 0, len(comps)
        fuse = self.merge_components
        while i < n:
            if isinstance(comps[i], PadCropOperator):
                if not comps[i].pads(self.direction):
                    raise ValueError("a cropping PadCropOperator without a padding one before it")
                sp, k = self._padded_span(comps, i)
                segs.append(sp)
                i = k + 1
                continue
            if fuse and (_is_mod(comps[i]) or _is_prop(comps[i]) or isinstance(comps[i], FieldProbe)):
                j = i
                mods = [None]
                props = []
                probes = []
                lay = None

                def take_probes(plane):
                    nonlocal j
                    while j < n and isinstance(comps[j], FieldProbe):
                        probes.append((plane, comps[j]))
                        j += 1

                take_probes(("pre", 0))
                if j < n and _is_mod(comps[j]):
                    mods[0] = comps[j]
                    j += 1
                    take_probes(("post", 0))
                while j < n and _is_prop(comps[j]):
                    lj = comps[j].layout(u)
                    if lay is not None and lj != lay:
                        break
                    lay = lj
                    props.append(comps[j])
                    mods.append(None)
                    j += 1
                    k = len(props)
                    take_probes(("pre", k))
                    if j < n and _is_mod(comps[j]):
                        mods[-1] = comps[j]
                        j += 1
                        take_probes(("post", k))
                if props:
                    # a probe after the chain's last propagator or modulator stays in the chain;
                    # one that is followed by a propagator the chain could not take is left out
                    segs.append(_Chain(props, mods, probes))
                    i = j
                    continue
            segs.append(comps[i])
            i += 1
        return segs

    def _set_chain_probes(self, seg: _Chain, u: ScalarField, probes):
        """Points the chain's probe planes at fresh fields (collected into ``probes``)
        or clears them."""
        if not seg.probes:
            return
        h = self._chain_handle(seg, u)
        if probes is None:
            _capi.call("fo_chain_set_probes", h, None, None)
            return
        K = len(seg.props)
        pre = (C.c_void_p * (K + 1))()
        post = (C.c_void_p * (K + 1))()
        by_plane = {}
        for (side, k), pr in seg.probes:
            f = by_plane.get((side, k))
            if f is None:
                f = u.similar()
                by_plane[(side, k)] = f
                (pre if side == "pre" else post)[k] = f.electric.data_ptr()
            # several probes on one plane share one copy, like the reference's copies of one field
            probes[pr] = f
        _capi.call("fo_chain_set_probes", h, pre, post)

    def _chain_handle(self, ch: _Chain, u: ScalarField):
        plans = tuple(p.plan_for(u).value for p in ch.props)
        h = self._chains.get(plans)
        if h is None:
            h = C.c_void_p()
            arr = (C.c_void_p * len(plans))(*plans)
            _capi.call("fo_chain_create", C.byref(h), len(plans), arr)
            self._chains[plans] = h
        return h

    def __del__(self):
        lib = _capi._LIB
        if lib is None:
            return
        for h in getattr(self, "_chains", {}).values():
            lib.fo_chain_destroy(h)

    # -- execution ----------------------------------------------------------------
    def forward(self, u: ScalarField, tape=None, src: ScalarField = None, metric=None, probes=None):
        """Runs the system in place on u (or from ``src`` into u).  With a tape,
        trainable components save their inputs and the tape records what the
        adjoint sweep needs.  A trainable modulator that directly follows the
        source of an out-of-place run saves nothing: the tape refers to ``src``,
        which must stay unchanged until the adjoint sweep has run.

        With ``metric``, the metric is evaluated on the result (its ``loss`` holds
        the values afterwards); SquaredIntensityDifference is then computed inside
        the last pass when the system ends with a fused chain.

        With a ``probes`` dict, every FieldProbe's copy of the field is stored in it."""
        d = self.direction
        segs = self.segments(u)
        metric_done = False
        for i, seg in enumerate(segs):
            from_src = src is not None and i == 0
            if src is not None and i == 0 and not isinstance(seg, _Chain):
                u.electric.copy_(src.electric)
                from_src = False
            if isinstance(seg, _Chain):
                for p in seg.props:
                    if isinstance(p, _FourierModulator):
                        p.refresh(u)
                self._set_chain_probes(seg, u, probes)
                mods = (fo_mod * len(seg.mods))()
                saved = []
                # The first modulator of a chain that reads the system input out of place
                # sees that input unchanged, so its adjoint reads it there: no copy is saved.
                src_is_input = from_src and src.electric.data_ptr() != u.electric.data_ptr()
                for k, m in enumerate(seg.mods):
                    if m is None:
                        mods[k] = fo_mod(_capi.FO_MOD_NONE, None, None, None, 0.0, None)
                        saved.append(None)
                        continue
                    if tape is not None and m.trainable and k == 0 and src_is_input:
                        mods[k] = m.fo_mod(saved=None, u=u)
                        saved.append(src.electric)
                        continue
                    sv = m.get_saved_buffer(u) if (tape is not None and m.trainable) else None
                    mods[k] = m.fo_mod(saved=sv, u=u)
                    saved.append(sv)
                if metric is not None and getattr(metric, "fuses_into_chain", False) and i == len(segs) - 1:
                    _capi.call("fo_chain_forward_sid", self._chain_handle(seg, u),
                               _ptr(src.electric) if from_src else None, _ptr(u.electric), mods, int(d),
                               metric.handle, _ptr(metric.target), _ptr(metric.loss), _stream())
                    metric_done = True
                elif from_src:
                    _capi.call("fo_chain_forward_from", self._chain_handle(seg, u), _ptr(src.electric),
                               _ptr(u.electric), mods, int(d), _stream())
                else:
                    _capi.call("fo_chain_forward", self._chain_handle(seg, u), _ptr(u.electric), mods, int(d),
                               _stream())
                if tape is not None:
                    tape.append((seg, saved))
            elif isinstance(seg, _PaddedSpan):
                seg.forward(u, tape, probes)
            else:
                c = seg
                if isinstance(c, TiltAnchor):
                    entry = u.tilts
                    c.propagate_(u, d)
                    if tape is not None:
                        tape.append((c, entry))
                elif tape is not None and c.trainable and isinstance(c, AS_BPM):
                    c.propagate_and_save_(u, None, d)
                    tape.append((c, None))
                elif tape is not None and c.trainable and hasattr(c, "propagate_and_save_"):
                    # the component protocol (OpticalComponents.jl:751-816): a trainable
                    # component saves what its adjoint needs into its saved buffer
                    sv = c.get_saved_buffer(u) if hasattr(c, "get_saved_buffer") else None
                    c.propagate_and_save_(u, sv, d)
                    tape.append((c, sv))
                elif isinstance(c, FieldProbe):
                    if probes is not None:
                        probes[c] = u.copy()
                    if tape is not None:
                        tape.append((c, None))
                else:
                    c.propagate_(u, d)
                    if tape is not None:
                        tape.append((c, None))
        if src is not None and not self.components:
            u.electric.copy_(src.electric)
        if metric is not None and not metric_done:
            metric(u)
        return u

    def _fused_chain_mods(self, src: ScalarField, input_grad):
        """The single fused chain of a system for the withgradient entry points, with its
        forward and adjoint modulation slots and gradient buffers; None when the system
        has another shape."""
        if src is None:
            return None
        segs = self.segments(src)
        if len(segs) != 1 or not isinstance(segs[0], _Chain):
            return None
        seg = segs[0]
        if seg.probes or any(isinstance(p, _FourierModulator) for p in seg.props):
            return None
        if input_grad is None:
            input_grad = self.source is None or getattr(self.source, "trainable", False)
        n = len(seg.mods)
        mf, mb = (fo_mod * n)(), (fo_mod * n)()
        grads = {}
        saves = []  # kept with the system until the next call: the stream may still use them
        for k, m in enumerate(seg.mods):
            if m is None:
                mf[k] = fo_mod(_capi.FO_MOD_NONE, None, None, None, 0.0, None)
                mb[k] = fo_mod(_capi.FO_MOD_NONE, None, None, None, 0.0, None)
                continue
            if not m.trainable:
                mf[k] = m.fo_mod(saved=None, u=src)
                mb[k] = m.fo_mod(saved=None, grad=None, u=src)
                continue
            # the first slot reads the unchanged input in the adjoint instead of a saved copy
            sv = None if k == 0 else m.get_saved_buffer(src)
            g = m.get_gradient_buffer()
            saves.append(sv)
            mf[k] = m.fo_mod(saved=sv, u=src)
            mb[k] = m.fo_mod(saved=src.electric if k == 0 else sv, grad=g, u=src)
            grads[m] = {m.pname: g}
        return seg, mf, mb, grads, saves, (0 if input_grad else 1)

    def forward_backward_sid(self, du: ScalarField, src: ScalarField, metric, u_out: ScalarField = None,
                             input_grad=None):
        """Forward sweep from ``src``, SquaredIntensityDifference and its seeded adjoint
        sweep in one library call (fo_chain_withgradient_sid), for a system that is one
        fused chain; when it ends in a propagator, the chain's last forward row pass and
        the adjoint's first row pass run as one pass.  ``metric.loss`` holds the
        per-slice losses afterwards; ``u_out`` (optional) receives the output field.
        Returns {component: {name: grad}}, or None when the system has another shape
        (callers then run forward and backward)."""
        if not getattr(metric, "fuses_into_chain", False):
            return None
        fm = self._fused_chain_mods(src, input_grad)
        if fm is None:
            return None
        seg, mf, mb, grads, saves, flags = fm
        _capi.call("fo_chain_withgradient_sid", self._chain_handle(seg, src), _ptr(src.electric),
                   _ptr(u_out.electric) if u_out is not None else None, _ptr(du.electric), mf, mb, int(self.direction),
                   metric.handle, _ptr(metric.target), _ptr(metric.loss), flags, _stream())
        self._fused_saves = saves
        return grads

    def forward_backward_sfd(self, du: ScalarField, src: ScalarField, metric, dc=None, u_out: ScalarField = None,
                             input_grad=None):
        """The same for SquaredFieldDifference (fo_chain_withgradient_sfd): ``metric.out``
        holds the per-field values c afterwards and ``du`` the gradient of sum(dc * c)
        (dc: one value per field, or None for ones).  Returns
        {component: {name: grad}}, or None when the system is not one fused chain."""
        if (src.nx, src.ny, src.batch) != (metric.nx, metric.ny, metric.batch):
            return None
        if dc is not None:
            dc = dc.to(device=metric.out.device, dtype=torch.float32).reshape(-1).contiguous()
            if dc.numel() != metric.batch:
                raise ValueError("dc must hold one value per field")
        fm = self._fused_chain_mods(src, input_grad)
        if fm is None:
            return None
        seg, mf, mb, grads, saves, flags = fm
        _capi.call("fo_chain_withgradient_sfd", self._chain_handle(seg, src), _ptr(src.electric),
                   _ptr(u_out.electric) if u_out is not None else None, _ptr(du.electric), mf, mb, int(self.direction),
                   metric.handle, _ptr(metric.v.electric), _ptr(dc), _ptr(metric.out), flags, _stream())
        self._fused_saves = (saves, dc)
        return grads

    def backward(self, du: ScalarField, tape, seed=None, input_grad=None):
        """Adjoint sweep over a tape; returns {component: {name: grad}}.

        ``input_grad=False`` skips writing the gradient with respect to the system
        input when a fused chain ends the sweep (default: only when the source is
        not trainable)."""
        d = self.direction
        if input_grad is None:
            input_grad = self.source is None or getattr(self.source, "trainable", False)
        grads = {}
        first = True
        n_seg = len(tape)
        for idx, (seg, saved) in enumerate(reversed(tape)):
            last = idx == n_seg - 1
            if isinstance(seg, _Chain):
                mods = (fo_mod * len(seg.mods))()
                for k, m in enumerate(seg.mods):
                    if m is None:
                        mods[k] = fo_mod(_capi.FO_MOD_NONE, None, None, None, 0.0, None)
                        continue
                    g = m.get_gradient_buffer() if m.trainable else None
                    mods[k] = m.fo_mod(saved=saved[k], grad=g, u=du)
                    if g is not None:
                        grads[m] = {m.pname: g}
                flags = 0 if (input_grad or not last) else 1  # FO_BWD_DISCARD_INPUT_GRAD
                if first and seed is not None:
                    sid, u_out = seed
                    _capi.call("fo_chain_backward_ex", self._chain_handle(seg, du), _ptr(du.electric), mods,
                               int(d), sid.handle, _ptr(u_out.electric), flags, _stream())
                else:
                    _capi.call("fo_chain_backward_ex", self._chain_handle(seg, du), _ptr(du.electric), mods,
                               int(d), None, None, flags, _stream())
            else:
                if first and seed is not None:
                    sid, u_out = seed
                    sid.backpropagate_into(u_out, du)
                c = seg
                if isinstance(c, _PaddedSpan):
                    grads.update(c.backward(du, saved))
                elif isinstance(c, TiltAnchor):
                    du.offset_tilts_(saved)  # back to the tilts the field had on entry
                elif c.trainable and hasattr(c, "backpropagate_with_gradient_"):
                    g = c.get_gradient_buffer()
                    _, gd = c.backpropagate_with_gradient_(du, saved, g, d)
                    grads[c] = gd
                elif isinstance(c, AS_BPM):
                    c.backpropagate_with_gradient_(du, None, None, d)
                elif isinstance(c, FieldProbe):
                    pass
                elif type(c).backpropagate_ is not Component.backpropagate_:
                    c.backpropagate_(du, d)
                else:
                    raise NotImplementedError(f"no adjoint for {type(c).__name__}")
            first = False
        if first and seed is not None:  # empty system
            sid, u_out = seed
            sid.backpropagate_into(u_out, du)
        return grads

    def __call__(self, x=None):
        if (x is None) == (self.source is None):
            raise ValueError("give exactly one of a source or an input field")
        src = self.source.u0 if x is None else x
        u = src.similar()
        probes = {}
        self.forward(u, src=src, probes=probes)
        return {"out": u, "probes": probes}


def propagate(u, p, direction=Forward):
    """Out-of-place propagate (the reference's ``propagate``)."""
    return p.propagate(u, direction)


def propagate_(u, p, direction=Forward):
    """In-place propagate (the reference's ``propagate!``)."""
    return p.propagate_(u, direction)


def backpropagate_(dv, p, direction=Forward):
    return p.backpropagate_(dv, direction)


def backpropagate(dv, p, direction=Forward):
    """Out-of-place adjoint (the reference's ``backpropagate``): a new field."""
    if isinstance(p, PadCropOperator):
        return p.backpropagate(dv, direction)
    out = dv.copy()
    p.backpropagate_(out, direction)
    return out


# Accessors of the reference's component API (OpticalComponents.jl:277-340,
# system/optical_system.jl), as free functions over the objects above.

def trainable(p):
    """The trainable arrays of a component, {name: tensor} ({} when static); of a
    system, {component: {name: tensor}} over its source and components."""
    if isinstance(p, (OpticalSystem, OpticalSequence)):
        leaves = p.leaf_components() if isinstance(p, OpticalSystem) else p.expanded()
        parts = ([p.source] if getattr(p, "source", None) is not None else []) + leaves
        return {c: c.params() for c in parts if c.params()}
    return p.params()


def istrainable(p):
    return bool(getattr(p, "trainable", False))


def isbuffered(p):
    return bool(getattr(p, "trainable", False) and getattr(p, "buffered", False))


def get_data(p):
    """A component's parameter array (Phase: phi, Mask: m, TeaDOE: h, AS_BPM: dn, ...)."""
    return p.get_data()


def get_source(p):
    """The system's ScalarSource, or a source's field."""
    return p.source if isinstance(p, OpticalSystem) else p.get_source()


def get_components(system):
    return system.get_components()
