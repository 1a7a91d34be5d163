"""Fista, Descent, Momentum, Nesterov, ProxRule, ClampProx, IstaProx, PositiveProx and
TVProx on the GPU (src/OptimisersExt.jl, src/proximal_operators/*)."""

from __future__ import annotations

import ctypes as C

import torch

from . import _capi
from .components import OpticalSystem, _ptr, _stream


class Fista:
    """Fista(eta): the rule keeps eta^2 (OptimisersExt.jl:33-54)."""

    def __init__(self, eta):
        self.eta = float(eta)

    def init(self, x):
        return {"t": torch.ones(1, dtype=torch.float64, device=x.device), "xk": x.detach().clone(),
                "newdx": torch.zeros_like(x)}

    def apply_(self, state, x, dx):
        # the update is real-linear in x and dx, so a complex parameter (a trainable
        # source field) is updated as its interleaved real and imaginary parts
        xf, xk, nd = _float_view(x), _float_view(state["xk"]), _float_view(state["newdx"])
        d = _float_view(dx.to(x.dtype).contiguous())
        _capi.call("fo_fista_step", _ptr(xf), _ptr(xk), _ptr(nd), _ptr(d), xf.numel(), self.eta, _ptr(state["t"]),
                   _stream())


class _PlainRule:
    """Descent / Momentum / Nesterov of Optimisers.jl 0.4 (re-exported by the reference,
    OptimisersExt.jl:9) as one elementwise FP32 kernel (fo_rule_step)."""

    kind = _capi.FO_RULE_DESCENT
    eta = 0.1
    rho = 0.0

    def init(self, x):
        return None if self.kind == _capi.FO_RULE_DESCENT else torch.zeros_like(x)

    def apply_(self, state, x, dx):
        xf = _float_view(x)
        d = _float_view(dx.to(x.dtype).contiguous())
        v = None if state is None else _float_view(state)
        _capi.call("fo_rule_step", _ptr(xf), _ptr(v), _ptr(d), xf.numel(), self.kind, self.eta, self.rho, _stream())


class Descent(_PlainRule):
    """x <- x - eta dx."""

    def __init__(self, eta=0.1):
        self.eta = float(eta)


class Momentum(_PlainRule):
    """v <- rho v + eta dx; x <- x - v."""

    kind = _capi.FO_RULE_MOMENTUM

    def __init__(self, eta=0.01, rho=0.9):
        self.eta, self.rho = float(eta), float(rho)


class Nesterov(_PlainRule):
    """newdx = -rho^2 v + (1 + rho) eta dx; v <- rho v - eta dx; x <- x - newdx."""

    kind = _capi.FO_RULE_NESTEROV

    def __init__(self, eta=0.001, rho=0.9):
        self.eta, self.rho = float(eta), float(rho)


class NoDescent:
    def init(self, x):
        return {}

    def apply_(self, state, x, dx):
        pass


class ClampProx:
    """clamp(x, lo, hi) (proximal_operators/clamp_prox.jl:35-37)."""

    def __init__(self, lo, hi):
        self.lo, self.hi = float(lo), float(hi)

    def init(self, x):
        return None

    def apply_(self, state, x):
        _capi.call("fo_clamp", _ptr(x), x.numel(), self.lo, self.hi, _stream())


def _float_view(x):
    """The float values of a float32 or complex64 parameter (a complex one as its
    interleaved real and imaginary parts)."""
    if x.dtype == torch.complex64:
        return torch.view_as_real(x)
    if x.dtype != torch.float32:
        raise NotImplementedError("the GPU proximal operators update float32 or complex64 parameters")
    return x


class PointwiseProx:
    """PointwiseProx(f) (proximal_operators/pointwise_prox.jl:1-46): x <- f.(x) for a
    user function of the parameter tensor (a torch expression evaluated on the device,
    e.g. ``lambda x: torch.where(x < 0, 0, x)``).  The built-in operators below are
    PointwiseProx of fixed functions with their own kernels."""

    def __init__(self, f):
        self.f = f

    def init(self, x):
        return None

    def apply_(self, state, x):
        x.copy_(self.f(x))


class IstaProx:
    """Soft threshold towards c (proximal_operators/ista_prox.jl:1-56); a complex
    parameter has its real and imaginary parts shrunk separately, each towards c."""

    def __init__(self, s, c=0.0):
        if s < 0:
            raise ValueError("IstaProx threshold must be non-negative")
        self.s, self.c = float(s), float(c)

    def init(self, x):
        return None

    def apply_(self, state, x):
        f = _float_view(x)
        _capi.call("fo_ista", _ptr(f), f.numel(), self.s, self.c, _stream())


class PositiveProx:
    """max(x, 0) (proximal_operators/positive_prox.jl:1-40); real parameters only, as
    the reference's comparison x < 0 is defined for real values only."""

    def init(self, x):
        return None

    def apply_(self, state, x):
        if x.is_complex():
            raise TypeError("PositiveProx applies to real parameters")
        f = _float_view(x)
        _capi.call("fo_positive", _ptr(f), f.numel(), _stream())


class TVProx:
    """TVProx(lambda, n_iter; tol, isotropic, rule=Fista(eta)) (tv_prox.jl:94-195) on 1-, 2-
    or 3-D parameters.
    ``tol`` stops the dual iterations once the primal iterate changes by less than tol
    (tested on the device); a complex parameter has its real and imaginary parts
    denoised separately, each with its own dual state, as the reference does."""

    def __init__(self, lam, n_iter=50, tol=None, isotropic=True, eta=None):
        self.lam = float(lam)
        self.n_iter = int(n_iter)
        self.tol = None if tol is None else float(tol)
        self.isotropic = bool(isotropic)
        self.eta = float(eta if eta is not None else (0.25 if isotropic else 2.5))

    def _handle(self, x):
        h = C.c_void_p()
        dims = list(reversed(x.shape))  # x (the last axis) fastest, as in the reference's arrays
        _capi.call("fo_tv_create_nd", C.byref(h), len(dims), _capi.ivec(dims), self.lam, self.n_iter,
                   int(self.isotropic), self.eta, 0.0 if self.tol is None else self.tol)
        return _TvHandle(h)

    def init(self, x):
        if x.dim() not in (1, 2, 3):
            raise NotImplementedError("TVProx on the GPU path takes 1-, 2- or 3-D parameters")
        if x.is_complex():
            return (self._handle(x), self._handle(x))
        return self._handle(x)

    def apply_(self, state, x):
        if x.is_complex():
            re, im = x.real.contiguous(), x.imag.contiguous()
            _capi.call("fo_tv_apply", state[0].h, _ptr(re), _stream())
            _capi.call("fo_tv_apply", state[1].h, _ptr(im), _stream())
            x.copy_(torch.complex(re, im))
            return
        _capi.call("fo_tv_apply", state.h, _ptr(x), _stream())


def tv_denoise_(x, lam, n_iter=50, tol=None, isotropic=True, eta=None):
    """TV_denoise!(x, lambda, n_iter; tol, isotropic) (tv_prox.jl:197-258): TVProx applied
    once, in place."""
    tv = TVProx(lam, n_iter, tol=tol, isotropic=isotropic, eta=eta)
    tv.apply_(tv.init(x), x)
    return x


class _TvHandle:
    def __init__(self, h):
        self.h = h

    def __del__(self):
        lib = _capi._LIB
        if lib is not None:
            lib.fo_tv_destroy(self.h)


class ProxRule:
    """Rule step, then the proximal operator (OptimisersExt.jl:222-244)."""

    def __init__(self, rule, prox):
        self.rule = rule
        self.prox = prox

    def init(self, x):
        return {"rule": self.rule.init(x), "prox": self.prox.init(x)}

    def apply_(self, state, x, dx):
        if isinstance(self.rule, Fista) and isinstance(self.prox, ClampProx) and x.dtype == torch.float32:
            # the clamp rides in the Fista pass (fo_fista_clamp_step)
            r = state["rule"]
            _capi.call("fo_fista_clamp_step", _ptr(x), _ptr(r["xk"]), _ptr(r["newdx"]), _ptr(dx), x.numel(),
                       self.rule.eta, _ptr(r["t"]), self.prox.lo, self.prox.hi, _stream())
            return
        self.rule.apply_(state["rule"], x, dx)
        self.prox.apply_(state["prox"], x)


def make_rules(*pairs):
    """{parameter data_ptr: rule} from (component-or-tensor, rule) pairs
    (OptimisersExt.jl:195-214)."""
    rules = {}
    for obj, rule in pairs:
        if isinstance(obj, torch.Tensor):
            rules[obj.data_ptr()] = rule
        else:
            for t in obj.params().values():
                rules[t.data_ptr()] = rule
    return rules


class OptState:
    def __init__(self):
        self.leaves = []  # (component, name, tensor, rule, state)


def setup(rules, model_or_default=None, model=None):
    """setup(rule, system) / setup(rules, system) / setup(rules, default_rule, system)."""
    if model is None:
        model, default = model_or_default, None
    else:
        default = model_or_default
    if not isinstance(rules, dict):
        default, rules = rules, {}
    st = OptState()
    comps = model.leaf_components()
    if model.source is not None:
        comps = [model.source] + comps
    for c in comps:
        for name, t in c.params().items():
            rule = rules.get(t.data_ptr(), default if default is not None else NoDescent())
            st.leaves.append((c, name, t, rule, rule.init(t)))
    return st


def update_(state: OptState, system: OpticalSystem, grads):
    """Apply each rule to its parameter in place (Optimisers.update!)."""
    for c, name, t, rule, s in state.leaves:
        g = grads.get(c)
        if g is None or name not in g:
            continue
        rule.apply_(s, t, g[name])
    return state
