"""ScalarField: the field container of the hot path.

Mirrors ``ScalarField`` of FluxOptics.jl (src/Fields.jl:118-149).  Storage is a
CUDA complex64 tensor; the Julia column-major array ``(nx, ny, d3, d4, ...)``
is the C-ordered tensor ``(..., d4, d3, ny, nx)``, so the two share one memory
layout: x fastest, then y, then the trailing dims in Julia order.  Wavelengths
(and tilts) are given in Julia order over the trailing dims and broadcast like
the reference's ``parse_lambdas`` (src/Fields.jl:18-38).
"""

from __future__ import annotations

import numpy as np
import torch


def _as_device_field(data):
    if isinstance(data, torch.Tensor):
        t = data
    else:
        t = torch.as_tensor(np.asarray(data))
    if not t.is_complex():
        t = t.to(torch.complex64)
    if t.dtype != torch.complex64:
        t = t.to(torch.complex64)
    if t.device.type != "cuda":
        t = t.to("cuda")
    return t.contiguous()


def per_field(values, julia_batch_shape):
    """Broadcast a scalar or a Julia-ordered array over the trailing dims and
    return one float64 value per field, in memory (column-major) order."""
    nb = int(np.prod(julia_batch_shape)) if len(julia_batch_shape) else 1
    v = np.asarray(values, dtype=np.float64)
    if v.ndim == 0:
        return np.full(nb, float(v))
    if len(julia_batch_shape) == 0:
        if v.size != 1:
            raise ValueError("per-field values given for a single field")
        return v.reshape(1)
    shape = tuple(v.shape) + (1,) * (len(julia_batch_shape) - v.ndim)
    b = np.broadcast_to(v.reshape(shape, order="F"), tuple(julia_batch_shape))
    return np.asarray(b).reshape(-1, order="F")


class ScalarField:
    """A batch of scalar fields on a regular grid.

    ``data``: complex tensor/array of shape ``(..., ny, nx)``; ``ds = (dx, dy)``;
    ``lambdas``: a wavelength or an array broadcast over the trailing dims
    (Julia order); ``tilts = (theta_x, theta_y)`` in radians, each a number or an
    array broadcast the same way (src/Fields.jl:34-38, :130-141)."""

    def __init__(self, data, ds, lambdas, tilts=None):
        if isinstance(data, tuple) and data and all(isinstance(n, (int, np.integer)) for n in data):
            # ScalarField(nd::NTuple, ds, lambdas; tilts): zeros of the Julia size nd (src/Fields.jl:143-148)
            data = torch.zeros(tuple(int(n) for n in reversed(data)), dtype=torch.complex64)
        self.electric = _as_device_field(data)
        if self.electric.dim() < 2:
            raise ValueError("a field needs two spatial dims")
        self.ds = (float(ds[0]), float(ds[1]))
        self.lambdas = lambdas
        self.tilts = (0.0, 0.0) if tilts is None else (tilts[0], tilts[1])

    # -- shape -------------------------------------------------------------
    @property
    def nx(self):
        return int(self.electric.shape[-1])

    @property
    def ny(self):
        return int(self.electric.shape[-2])

    @property
    def julia_batch_shape(self):
        return tuple(int(s) for s in reversed(self.electric.shape[:-2]))

    @property
    def batch(self):
        return int(np.prod(self.julia_batch_shape)) if self.electric.dim() > 2 else 1

    def size(self):
        """Size in Julia order (nx, ny, trailing...)."""
        return (self.nx, self.ny) + self.julia_batch_shape

    def ndims(self, spatial=False):
        """Number of dimensions, or of spatial ones (src/Fields.jl:360-362)."""
        return 2 if spatial else self.electric.dim()

    def copyto_(self, v):
        """Copy another field's data in (src/Fields.jl:433-436)."""
        self.electric.copy_(v.electric)
        return self

    def lambdas_per_field(self):
        return per_field(self.lambdas, self.julia_batch_shape)

    def tilts_per_field(self):
        """(batch, 2) array of (theta_x, theta_y) per field."""
        tx = per_field(self.tilts[0], self.julia_batch_shape)
        ty = per_field(self.tilts[1], self.julia_batch_shape)
        return np.stack([np.broadcast_to(tx, (self.batch,)), np.broadcast_to(ty, (self.batch,))], axis=1)

    # -- helpers of the reference API -------------------------------------------
    def copy(self):
        return ScalarField(self.electric.clone(), self.ds, self.lambdas, self.tilts)

    def similar(self):
        return ScalarField(torch.empty_like(self.electric), self.ds, self.lambdas, self.tilts)

    def set_field_data(self, data):
        """New field sharing grid, wavelengths and tilts (src/Fields.jl:213-215)."""
        return ScalarField(data, self.ds, self.lambdas, self.tilts)

    def is_on_axis(self):
        return not bool(np.any(self.tilts_per_field() != 0.0))

    # -- accessors of the reference (src/Fields.jl:153-300) ----------------------
    def get_lambdas(self):
        """The wavelengths as given at construction."""
        return self.lambdas

    def get_lambdas_collection(self):
        """One wavelength per field, in memory order."""
        return self.lambdas_per_field()

    def get_tilts(self):
        return self.tilts

    def get_tilts_collection(self):
        """(batch, 2) array of (theta_x, theta_y) per field."""
        return self.tilts_per_field()

    def select_lambdas(self):
        """A function of is_collection giving the per-field wavelengths or the
        wavelengths as given (src/Fields.jl:161-166)."""
        return lambda is_collection: self.get_lambdas_collection() if is_collection else self.get_lambdas()

    def select_tilts(self):
        """(select_x, select_y): each a function of is_collection giving the per-field
        tilt angles or the angles as given (src/Fields.jl:176-180)."""
        tc = self.get_tilts_collection()
        return tuple((lambda is_collection, k=k: tc[:, k] if is_collection else self.tilts[k]) for k in range(2))

    def set_field_ds_(self, ds):
        """In-place change of the sampling steps (src/Fields.jl:182-185)."""
        self.ds = (float(ds[0]), float(ds[1]))
        return self

    def set_field_tilts(self, tilts):
        """New field sharing the data with other tilts (src/Fields.jl:243-245)."""
        return ScalarField(self.electric, self.ds, self.lambdas, tilts)

    def offset_tilts_(self, tilts):
        """Change the tilts to ``tilts`` and multiply the field by the linear phase
        cis(2 pi / lambda ((sin tx0 - sin tx) x + (sin ty0 - sin ty) y)) that keeps the
        physical field unchanged (src/Fields.jl:280-301)."""
        new = ScalarField(self.electric[..., :1, :1], self.ds, self.lambdas, tilts)
        t0, t1 = self.tilts_per_field(), new.tilts_per_field()
        if np.array_equal(t0, t1):
            return self
        lam = self.lambdas_per_field()
        dev = self.electric.device
        ax = torch.as_tensor(2 * np.pi / lam * (np.sin(t0[:, 0]) - np.sin(t1[:, 0])), device=dev)
        ay = torch.as_tensor(2 * np.pi / lam * (np.sin(t0[:, 1]) - np.sin(t1[:, 1])), device=dev)
        x = (torch.arange(self.nx, dtype=torch.float64, device=dev) - (self.nx - 1) / 2.0) * self.ds[0]
        y = (torch.arange(self.ny, dtype=torch.float64, device=dev) - (self.ny - 1) / 2.0) * self.ds[1]
        # the phase is separable: one factor along x and one along y per field, formed in
        # float64 and rounded once each
        fx = torch.polar(torch.ones_like(x)[None, :].expand(len(lam), -1), ax[:, None] * x[None, :])
        fy = torch.polar(torch.ones_like(y)[None, :].expand(len(lam), -1), ay[:, None] * y[None, :])
        v = self.electric.view(-1, self.ny, self.nx)
        v.mul_(fx.to(torch.complex64)[:, None, :]).mul_(fy.to(torch.complex64)[:, :, None])
        self.tilts = new.tilts
        return self

    # -- arithmetic (src/Fields.jl:315-337, 392-400, 899-901) --------------------
    def __add__(self, v):
        return self.set_field_data(self.electric + v.electric)

    def __sub__(self, v):
        return self.set_field_data(self.electric - v.electric)

    def __neg__(self):
        return self.set_field_data(-self.electric)

    def __mul__(self, a):
        return self.set_field_data(self.electric * a)

    __rmul__ = __mul__

    def __truediv__(self, a):
        return self.set_field_data(self.electric / a)

    def conj(self):
        return self.set_field_data(self.electric.conj().resolve_conj())

    def fill_(self, v):
        """Fill with a number, or copy an array of the field's shape in (src/Fields.jl:392-400)."""
        if isinstance(v, (int, float, complex)):
            self.electric.fill_(v)
        else:
            self.electric.copy_(torch.as_tensor(np.asarray(v) if not isinstance(v, torch.Tensor) else v))
        return self


def power(u: ScalarField):
    """sum |u|^2 dx dy per field (src/Fields.jl:843-846)."""
    return (u.electric.abs() ** 2).sum(dim=(-2, -1)) * (u.ds[0] * u.ds[1])


def normalize_power_(u: ScalarField, target_power=1.0):
    """In-place normalisation (src/Fields.jl:889-892)."""
    p = power(u)
    u.electric.mul_(torch.sqrt(target_power / p)[..., None, None].to(u.electric.dtype))
    return u


def intensity(u: ScalarField):
    """sum over the trailing dims of |u|^2 (src/Fields.jl:608-616)."""
    i = u.electric.abs() ** 2
    return i.reshape(-1, u.ny, u.nx).sum(0)


def coupling_efficiency(u: ScalarField, v: ScalarField):
    """|<u, v>|^2 / (|u|^2 |v|^2) per field (src/Fields.jl:748-756)."""
    a = u.electric.reshape(-1, u.ny * u.nx)
    b = v.electric.reshape(-1, v.ny * v.nx)
    num = (a.conj() * b).sum(-1).abs() ** 2
    den = (a.abs() ** 2).sum(-1) * (b.abs() ** 2).sum(-1)
    return num / den


def phase(u):
    """angle(u) of a field or an array (src/Fields.jl:667-673)."""
    return torch.angle(u.electric) if isinstance(u, ScalarField) else torch.angle(torch.as_tensor(u))


def dot(u: ScalarField, v: ScalarField):
    """<u, v> = sum conj(u) v per field, without dx dy (src/Fields.jl:810-815)."""
    a = u.electric.reshape(-1, u.ny * u.nx)
    b = v.electric.reshape(-1, v.ny * v.nx)
    return (a.conj() * b).sum(-1)


def get_lambdas(u: ScalarField):
    return u.get_lambdas()


def get_lambdas_collection(u: ScalarField):
    return u.get_lambdas_collection()


def get_tilts(u: ScalarField):
    return u.get_tilts()


def get_tilts_collection(u: ScalarField):
    return u.get_tilts_collection()


def select_lambdas(u: ScalarField):
    return u.select_lambdas()


def select_tilts(u: ScalarField):
    return u.select_tilts()


def set_field_data(u: ScalarField, data):
    return u.set_field_data(data)


def set_field_ds_(u: ScalarField, ds):
    return u.set_field_ds_(ds)


def set_field_tilts(u: ScalarField, tilts):
    return u.set_field_tilts(tilts)


def offset_tilts_(u: ScalarField, tilts):
    return u.offset_tilts_(tilts)


def is_on_axis(u: ScalarField):
    return u.is_on_axis()
