"""Ragged batch: independent Phase -> ASProp -> SquaredIntensityDifference problems
on grids of different sizes, forward + adjoint of all of them in one persistent
launch (fo_ragged_create / fo_ragged_batch).

Per problem this is what the reference computes with
``Zygote.withgradient(ϕ -> SquaredIntensityDifference((u, t))(propagate(u, Phase(ϕ) |> ASProp(z))), ϕ)``
(modulators/phasemask.jl:90-150, freespace_propagators/angular_spectrum.jl:193-234,
metrics/squared_intensity_difference.jl:58-90, src/ChainRulesCoreExt.jl:21-111),
batched over problems that share nothing.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _capi
from .fields import ScalarField


def _dev(x, dtype):
    t = torch.as_tensor(x, dtype=dtype)
    return t.to("cuda").contiguous()


class RaggedBatch:
    """``problems``: a list of dicts with keys ``u`` (a single-field ScalarField on
    an n x n grid, n a power of two from 256 to 4096), ``phase`` (n x n), ``target``
    (n x n intensity), ``z`` and optionally ``n0``.  ``run()`` launches the batch on
    the current stream and returns (losses, outputs, grads): a CUDA tensor of one
    loss per problem, and per problem the propagated field and d loss / d phase."""

    def __init__(self, problems):
        if not problems:
            raise ValueError("RaggedBatch needs at least one problem")
        self.inputs, self.phases, self.targets, self.outputs, self.grads = [], [], [], [], []
        self.losses = torch.zeros(len(problems), dtype=torch.float32, device="cuda")
        descs = (_capi.fo_ragged_problem * len(problems))()
        for i, pr in enumerate(problems):
            u: ScalarField = pr["u"]
            if u.batch != 1 or u.nx != u.ny:
                raise ValueError("each ragged problem is one field on a square grid")
            lam = float(np.asarray(u.lambdas_per_field()).ravel()[0])
            uin = u.electric.reshape(u.ny, u.nx).contiguous()
            ph = _dev(pr["phase"], torch.float32).reshape(u.ny, u.nx)
            tg = _dev(pr["target"], torch.float32).reshape(u.ny, u.nx)
            out = torch.empty_like(uin)
            g = torch.empty((u.ny, u.nx), dtype=torch.float32, device="cuda")
            self.inputs.append(uin)
            self.phases.append(ph)
            self.targets.append(tg)
            self.outputs.append(out)
            self.grads.append(g)
            d = descs[i]
            d.n = u.nx
            d.dx, d.dy = float(u.ds[0]), float(u.ds[1])
            d.lam = lam
            d.z = float(pr["z"])
            d.n0 = float(pr.get("n0", 1.0))
            d.u_in, d.phase, d.target = uin.data_ptr(), ph.data_ptr(), tg.data_ptr()
            d.u_out, d.grad_phase = out.data_ptr(), g.data_ptr()
            d.loss = self.losses.data_ptr() + 4 * i
        self._h = C.c_void_p()
        _capi.call("fo_ragged_create", C.byref(self._h), descs, len(problems), 0)

    def info(self):
        grid, ws = C.c_int(), C.c_size_t()
        _capi.call("fo_ragged_info", self._h, C.byref(grid), C.byref(ws))
        return {"grid_ctas": grid.value, "workspace_bytes": ws.value}

    def pass_ms(self):
        """Device milliseconds of the five passes of the last run (synchronizes)."""
        ms = (C.c_double * 5)()
        _capi.call("fo_ragged_pass_ms", self._h, ms)
        return list(ms)

    def run(self):
        _capi.call("fo_ragged_batch", self._h, C.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self.losses, self.outputs, self.grads

    def __del__(self):
        lib = _capi._LIB
        h = getattr(self, "_h", None)
        if lib is not None and h is not None and h.value:
            lib.fo_ragged_destroy(h)
