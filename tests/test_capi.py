"""The C-ABI library loads, exports every symbol of include/*.h, and rejects bad
arguments before touching the GPU (CPU only: argument validation runs first)."""

import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def capi():
    from __graft_entry__ import build, load_package
    build()
    pkg = load_package()
    return pkg._capi


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names |= set(re.findall(r"FO_API\s+[\w\s\*]+?\b(fo_\w+)\s*\(", txt))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "fo_asprop_create" in names and "fo_chain_backward" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(capi):
    lib = capi.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the header exactly
    assert set(capi.SIGNATURES) == set(declared_symbols())


def test_version(capi):
    assert capi.load().fo_version() == 10000


def _err(capi, rc):
    assert rc != 0
    return capi.load().fo_last_error().decode()


def test_bad_shapes_are_rejected(capi):
    lib = capi.load()
    h = C.c_void_p()
    lam = capi.dvec([1.064])
    rc = lib.fo_asprop_create(C.byref(h), 0, 64, 1, 1.0, 1.0, lam, 1, 100.0, 1.0, 0)
    assert rc == 2 and "positive" in _err(capi, rc)
    rc = lib.fo_asprop_create(C.byref(h), 100, 64, 1, 1.0, 1.0, lam, 1, 100.0, 1.0, 0)
    assert rc == 2 and "not supported" in _err(capi, rc)
    rc = lib.fo_rsprop_create(C.byref(h), 4000, 64, 1, 1.0, 1.0, lam, 1, 100.0, 0)
    assert rc == 2
    rc = lib.fo_asprop_create(C.byref(h), 64, 64, 2, 1.0, 1.0, lam, 3, 100.0, 1.0, 0)
    assert rc == 1 and "lambdas" in _err(capi, rc)
    rc = lib.fo_asprop_create(C.byref(h), 64, 64, 1, -1.0, 1.0, lam, 1, 100.0, 1.0, 0)
    assert rc == 1
    rc = lib.fo_bpm_create(C.byref(h), 64, 64, 1, 1.0, 1.0, lam, 1, 10.0, 1.45, 1, 0, 1.0, 0)
    assert rc == 2 and "2 slices" in _err(capi, rc)


def test_bad_arguments_are_rejected(capi):
    lib = capi.load()
    assert lib.fo_propagate(None, None, 1, None) == 1
    assert lib.fo_phase_forward(C.c_void_p(16), C.c_void_p(16), None, 8, 8, 1, 3, None) == 1
    assert "direction" in lib.fo_last_error().decode()
    assert lib.fo_phase_backward(C.c_void_p(16), C.c_void_p(16), None, C.c_void_p(16), 8, 8, 1, 1, None) == 1
    assert lib.fo_clamp(C.c_void_p(16), 10, 1.0, 0.0, None) == 1
    assert lib.fo_ista(C.c_void_p(16), 10, -0.1, 0.0, None) == 1
    assert "non-negative" in lib.fo_last_error().decode()
    assert lib.fo_ista(None, 10, 0.1, 0.0, None) == 1
    assert lib.fo_positive(C.c_void_p(16), 0, None) == 2
    assert lib.fo_sfd_create(C.byref(C.c_void_p()), 8, 0, 2) == 2
    assert lib.fo_sfd_forward(None, None, None, None, None) == 1
    assert lib.fo_sfd_backward(None, None, None, None, None, None) == 1
    assert lib.fo_sfd_destroy(None) == 0
    p16 = C.c_void_p(16)
    assert lib.fo_rule_step(p16, None, p16, 10, 1, 0.1, 0.9, None) == 1
    assert "velocity" in lib.fo_last_error().decode()
    assert lib.fo_rule_step(p16, p16, p16, 10, 7, 0.1, 0.9, None) == 1
    assert lib.fo_fft2(None, None, 0, None) == 1
    assert lib.fo_chain_create(C.byref(C.c_void_p()), 0, None) == 1
    assert lib.fo_sid_create(C.byref(C.c_void_p()), 8, 8, 2, 2, capi.ivec([0, 5])) == 1
    assert lib.fo_tv_create(C.byref(C.c_void_p()), 1, 8, 0.1, 10, 1, 0.25) == 2
    # ragged batch: sizes and aliasing are checked before anything touches the GPU
    probs = (capi.fo_ragged_problem * 2)()
    for i, q in enumerate(probs):
        q.n, q.dx, q.dy, q.lam, q.z, q.n0 = 256, 1.0, 1.0, 1.064, 100.0, 1.0
        q.u_in, q.phase, q.target, q.u_out, q.grad_phase, q.loss = 16, 32, 48, 64 + 16 * i, 96, 112
    probs[1].n = 300
    h = C.c_void_p()
    assert lib.fo_ragged_create(C.byref(h), probs, 2, 0) == 2
    assert "power of two" in lib.fo_last_error().decode()
    probs[1].n = 256
    probs[1].u_out = probs[1].u_in
    assert lib.fo_ragged_create(C.byref(h), probs, 2, 0) == 1
    assert "alias" in lib.fo_last_error().decode()
    assert lib.fo_ragged_create(C.byref(h), probs, 0, 0) == 1
    assert lib.fo_fista_step(None, None, None, None, 10, 0.1, None, None) == 1
    assert lib.fo_fista_clamp_step(None, None, None, None, 10, 0.1, None, 0.0, 1.0, None) == 1
    p = C.c_void_p(16)
    assert lib.fo_fista_clamp_step(p, p, p, p, 10, 0.1, p, 1.0, 0.0, None) == 1
    assert "lo must not exceed hi" in lib.fo_last_error().decode()
    assert lib.fo_chain_forward_sid(None, None, None, None, 1, None, None, None, None) == 1
    m = (capi.fo_mod * 1)()
    p32, p48 = C.c_void_p(32), C.c_void_p(48)
    # pad / crop: NULL, aliasing, a block that does not fit, negative offsets
    assert lib.fo_pad(None, 8, 8, p32, 16, 16, 1, 0, 0, 0.0, 0.0, None) == 1
    assert lib.fo_pad(p32, 8, 8, p32, 16, 16, 1, 0, 0, 0.0, 0.0, None) == 1
    assert lib.fo_pad(p, 8, 8, p32, 16, 16, 1, 9, 0, 0.0, 0.0, None) == 2
    assert "does not fit" in lib.fo_last_error().decode()
    assert lib.fo_crop(p, 16, 16, p32, 8, 8, 1, -1, 0, None) == 1
    assert lib.fo_crop(p, 16, 16, p32, 8, 8, 0, 0, 0, None) == 2
    # the fused withgradient calls reject aliased fields before touching the chain
    assert lib.fo_chain_withgradient_sid(p, p, p32, p32, m, m, 1, p, p, p, 0, None) == 1
    assert lib.fo_chain_withgradient_sid(p, p32, p32, p48, m, m, 1, p, p, p, 0, None) == 1
    assert "alias" in lib.fo_last_error().decode()
    assert lib.fo_chain_withgradient_sfd(p, p32, None, p32, m, m, 1, p, p48, None, p, 0, None) == 1
    assert "alias" in lib.fo_last_error().decode()
    assert lib.fo_chain_withgradient_sfd(p, p32, None, p48, m, m, 1, p, p48, None, p, 0, None) == 1
    assert "v must not alias" in lib.fo_last_error().decode()
    assert lib.fo_copy(None, None, 16, None) == 1
    assert lib.fo_copy(None, None, 0, None) == 0  # nothing to copy


def _header_decls():
    import importlib.util
    spec = importlib.util.spec_from_file_location("_shim_test", os.path.join(os.path.dirname(__file__),
                                                                              "test_julia_shim.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.header_decls()


def _is_c_pointer(ct, handles):
    return ct.endswith("*") or ct in handles or ct.endswith("_fn")


def test_ctypes_signatures_match_the_header():
    """Every ctypes binding of the Python mirror has the header's argument count and,
    argument by argument, the same kind (pointer, int, long long, double), so a call
    through ctypes passes what the C function reads."""
    import ctypes as C
    from __graft_entry__ import load_package
    capi = load_package()._capi
    decls, handles = _header_decls()
    scalar = {"int": C.c_int, "long long": C.c_longlong, "double": C.c_double, "size_t": C.c_size_t,
              "unsigned": C.c_uint, "unsigned int": C.c_uint}
    pointee = {"double*": C.c_double, "const double*": C.c_double, "int*": C.c_int, "const int*": C.c_int,
               "float*": C.c_float, "const float*": C.c_float}
    for name, (res, args) in capi.SIGNATURES.items():
        assert name in decls, f"{name} is bound but not declared"
        cret, cargs = decls[name]
        assert len(args) == len(cargs), f"{name}: ctypes has {len(args)} arguments, the header {len(cargs)}"
        for k, (ct, pt) in enumerate(zip(cargs, args)):
            is_ptr_type = (pt in (C.c_void_p, C.c_char_p)
                           or (isinstance(pt, type) and issubclass(pt, C._Pointer))  # POINTER(T)
                           or bool(getattr(pt, "_flags_", 0) & C._FUNCFLAG_CDECL))  # a CFUNCTYPE
            if _is_c_pointer(ct, handles):
                assert is_ptr_type, f"{name} argument {k + 1}: header {ct!r}, ctypes {pt}"
                if ct in pointee and pt is not C.c_void_p:
                    assert pt._type_ is pointee[ct], f"{name} argument {k + 1}: header {ct!r}, ctypes {pt}"
            else:
                assert ct in scalar, f"{name} argument {k + 1}: unexpected header type {ct!r}"
                assert pt is scalar[ct], f"{name} argument {k + 1}: header {ct!r}, ctypes {pt}"
        if cret == "const char*":
            assert res is C.c_char_p, name
        else:
            assert res is C.c_int, f"{name} returns {cret}"
