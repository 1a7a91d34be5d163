"""ctypes binding of libfluxoptics_gb300 (the C ABI declared in include/fluxoptics_gb300.h)."""

from __future__ import annotations

import ctypes as C
import os

from . import build as _build

FO_OK = 0
FO_FORWARD = 1
FO_BACKWARD = -1
FO_MOD_NONE, FO_MOD_PHASE, FO_MOD_MASK, FO_MOD_DN, FO_MOD_TEA = 0, 1, 2, 3, 4
FO_FOURIER_TRAINABLE = 2
FO_FLAG_GRAD_SPECTRA = 2
FO_FLAG_DEVICE_Z = 4
FO_FFT_FORWARD, FO_FFT_INVERSE, FO_FFT_FORWARD_ADJOINT, FO_FFT_INVERSE_ADJOINT = 0, 1, 2, 3
FO_RULE_DESCENT, FO_RULE_MOMENTUM, FO_RULE_NESTEROV = 0, 1, 2

ERROR_NAMES = {1: "FO_ERR_ARG", 2: "FO_ERR_SHAPE", 3: "FO_ERR_ALLOC", 4: "FO_ERR_CUDA",
               5: "FO_ERR_TIMEOUT", 6: "FO_ERR_UNSUPPORTED"}


class FluxOpticsError(RuntimeError):
    """Raised when a C-ABI call returns a non-zero status."""

    def __init__(self, code, msg):
        super().__init__(f"{ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class fo_mod(C.Structure):
    _fields_ = [("kind", C.c_int), ("param", C.c_void_p), ("saved", C.c_void_p),
                ("grad", C.c_void_p), ("scale", C.c_double), ("field_coef", C.c_void_p)]


fo_filter_fn = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_longlong,
                           C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


class fo_as_options(C.Structure):
    _fields_ = [("paraxial", C.c_int), ("track_tilts", C.c_int), ("tilts", C.POINTER(C.c_double)),
                ("n_tilts", C.c_int), ("filter", fo_filter_fn), ("filter_ctx", C.c_void_p)]


class fo_ragged_problem(C.Structure):
    _fields_ = [("n", C.c_int), ("dx", C.c_double), ("dy", C.c_double), ("lam", C.c_double), ("z", C.c_double),
                ("n0", C.c_double), ("u_in", C.c_void_p), ("phase", C.c_void_p), ("target", C.c_void_p),
                ("u_out", C.c_void_p), ("grad_phase", C.c_void_p), ("loss", C.c_void_p)]


_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_ll = C.c_longlong
_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "fo_version": (_i, []),
    "fo_last_error": (C.c_char_p, []),
    "fo_stream_synchronize": (_i, [_vp]),
    "fo_device_status": (_i, [_vp]),
    "fo_profile_begin": (_i, []),
    "fo_profile_end": (_i, [_pd, _pi]),
    "fo_asprop_create": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _pd, _i, _d, _d, _i]),
    "fo_rsprop_create": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _pd, _i, _d, _i]),
    "fo_prop_destroy": (_i, [_vp]),
    "fo_prop_info": (_i, [_vp, _pi, _pi, C.POINTER(C.c_size_t)]),
    "fo_fourier_create": (_i, [C.POINTER(_vp), _i, _i, _i, _i]),
    "fo_prop_set_z": (_i, [_vp, _vp, _vp]),
    "fo_prop_z_gradient": (_i, [_vp, _vp, _vp, _vp, _i, _vp, _vp]),
    "fo_fourier_set": (_i, [_vp, _i, _vp, _vp]),
    "fo_fourier_gradient": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _i, _vp]),
    "fo_asprop_create_ex": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _pd, _i, _d, _d,
                                 C.POINTER(fo_as_options), _i]),
    "fo_fft2": (_i, [_vp, _vp, _i, _vp]),
    "fo_prop_variants": (_i, [_vp, _pi, _pi, C.c_char_p, C.c_char_p, _i]),
    "fo_propagate": (_i, [_vp, _vp, _i, _vp]),
    "fo_phase_forward": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_phase_backward": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_mask_forward": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_mask_backward": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_chain_create": (_i, [C.POINTER(_vp), _i, C.POINTER(_vp)]),
    "fo_chain_destroy": (_i, [_vp]),
    "fo_chain_forward": (_i, [_vp, _vp, C.POINTER(fo_mod), _i, _vp]),
    "fo_chain_set_probes": (_i, [_vp, _vp, _vp]),
    "fo_chain_forward_from": (_i, [_vp, _vp, _vp, C.POINTER(fo_mod), _i, _vp]),
    "fo_chain_forward_sid": (_i, [_vp, _vp, _vp, C.POINTER(fo_mod), _i, _vp, _vp, _vp, _vp]),
    "fo_chain_backward": (_i, [_vp, _vp, C.POINTER(fo_mod), _i, _vp, _vp, _vp]),
    "fo_chain_backward_ex": (_i, [_vp, _vp, C.POINTER(fo_mod), _i, _vp, _vp, _i, _vp]),
    "fo_chain_withgradient_sid": (_i, [_vp, _vp, _vp, _vp, C.POINTER(fo_mod), C.POINTER(fo_mod), _i, _vp, _vp, _vp,
                                       _i, _vp]),
    "fo_chain_withgradient_sfd": (_i, [_vp, _vp, _vp, _vp, C.POINTER(fo_mod), C.POINTER(fo_mod), _i, _vp, _vp, _vp,
                                       _vp, _i, _vp]),
    "fo_bpm_create": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _pd, _i, _d, _d, _i, _i, _d, _i]),
    "fo_bpm_create_ex": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _pd, _i, _d, _d, _i, _i,
                              C.POINTER(fo_as_options), _i]),
    "fo_bpm_destroy": (_i, [_vp]),
    "fo_bpm_info": (_i, [_vp, _pi, C.POINTER(C.c_size_t)]),
    "fo_bpm_forward": (_i, [_vp, _vp, _vp, _i, _i, _vp]),
    "fo_bpm_backward": (_i, [_vp, _vp, _vp, _vp, _i, _vp]),
    "fo_sid_create": (_i, [C.POINTER(_vp), _i, _i, _i, _i, _pi]),
    "fo_sid_destroy": (_i, [_vp]),
    "fo_sid_forward": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "fo_sid_backward": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "fo_sid_loss_noalloc": (_i, [_vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp]),
    "fo_fista_step": (_i, [_vp, _vp, _vp, _vp, _ll, _d, _vp, _vp]),
    "fo_copy": (_i, [_vp, _vp, C.c_size_t, _vp]),
    "fo_fista_clamp_step": (_i, [_vp, _vp, _vp, _vp, _ll, _d, _vp, _d, _d, _vp]),
    "fo_clamp": (_i, [_vp, _ll, _d, _d, _vp]),
    "fo_ista": (_i, [_vp, C.c_longlong, C.c_double, C.c_double, _vp]),
    "fo_positive": (_i, [_vp, C.c_longlong, _vp]),
    "fo_rule_step": (_i, [_vp, _vp, _vp, C.c_longlong, _i, C.c_double, C.c_double, _vp]),
    "fo_pad": (_i, [_vp, _i, _i, _vp, _i, _i, _i, _i, _i, C.c_double, C.c_double, _vp]),
    "fo_crop": (_i, [_vp, _i, _i, _vp, _i, _i, _i, _i, _i, _vp]),
    "fo_sfd_create": (_i, [C.POINTER(_vp), _i, _i, _i]),
    "fo_sfd_forward": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "fo_sfd_backward": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fo_sfd_destroy": (_i, [_vp]),
    "fo_tv_create": (_i, [C.POINTER(_vp), _i, _i, _d, _i, _i, _d]),
    "fo_tv_create_ex": (_i, [C.POINTER(_vp), _i, _i, _d, _i, _i, _d, _d]),
    "fo_tv_create_nd": (_i, [C.POINTER(_vp), _i, _pi, _d, _i, _i, _d, _d]),
    "fo_tv_destroy": (_i, [_vp]),
    "fo_tv_apply": (_i, [_vp, _vp, _vp]),
    "fo_graph_begin": (_i, [_vp]),
    "fo_graph_end": (_i, [_vp, C.POINTER(_vp)]),
    "fo_graph_launch": (_i, [_vp, _vp]),
    "fo_graph_info": (_i, [_vp, _pi]),
    "fo_graph_destroy": (_i, [_vp]),
    "fo_ragged_create": (_i, [C.POINTER(_vp), C.POINTER(fo_ragged_problem), _i, _i]),
    "fo_tea_forward": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_overlap_create": (_i, [C.POINTER(_vp), _i, _i, _i, _d, _d, _vp, _i, _i]),
    "fo_overlap_forward": (_i, [_vp, _vp, _vp, _vp]),
    "fo_overlap_backward": (_i, [_vp, _vp, _vp, _vp]),
    "fo_overlap_destroy": (_i, [_vp]),
    "fo_tea_backward": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp]),
    "fo_ragged_batch": (_i, [_vp, _vp]),
    "fo_ragged_info": (_i, [_vp, _pi, C.POINTER(C.c_size_t)]),
    "fo_ragged_destroy": (_i, [_vp]),
    "fo_ragged_pass_ms": (_i, [_vp, _pd]),
}

_LIB = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the shared library (building it first when missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = lib_path()
    if build_if_missing and (_build.is_stale() or not os.path.exists(path)):
        _build.build()
    if not os.path.exists(path):
        raise FluxOpticsError(6, f"{path} is missing; run build() first")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(rc: int) -> None:
    if rc != FO_OK:
        msg = _LIB.fo_last_error().decode() if _LIB is not None else ""
        raise FluxOpticsError(rc, msg)


def call(name, *args):
    lib = load()
    check(getattr(lib, name)(*args))


def dvec(values):
    arr = (C.c_double * len(values))(*[float(v) for v in values])
    return arr


def ivec(values):
    return (C.c_int * len(values))(*[int(v) for v in values])
