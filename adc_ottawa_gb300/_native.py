"""ctypes binding of libadcgpu.so (include/adcgpu.h).

The library is loaded from the package's in-tree _lib/ folder.  If it is
missing, loading raises: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libadcgpu.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_vp = C.c_void_p


class DavParams(C.Structure):
    _fields_ = [
        ("davstates", C.c_int),
        ("dmain", C.c_int),
        ("maxsubdim", C.c_int),
        ("maxiter", C.c_int),
        ("precon", C.c_int),
        ("ldfl", C.c_int),
        ("lsubdiag", C.c_int),
        ("guessdim", C.c_int),
        ("davtol", C.c_double),
        ("precision", C.c_int),
        ("refine", C.c_int),
        ("tol_bf16", C.c_double),
        ("tol_fp32", C.c_double),
        ("refine_block", C.c_int),
    ]


class DavInfo(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("nmult", C.c_int64),
        ("nconv", C.c_int),
        ("seconds", C.c_double),
        ("sigma_seconds", C.c_double),
        ("max_residual", C.c_double),
        ("iters_bf16", C.c_int),
        ("iters_fp32", C.c_int),
        ("iters_fp64", C.c_int),
        ("nmult_reference", C.c_int64),
    ]


class SilState(C.Structure):
    _fields_ = [("old_order", C.c_int), ("old_error", C.c_double), ("old_stepsize", C.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "adcgpu_synth_orbitals": (C.c_int, [C.c_int, C.c_int, C.c_uint64, _dp]),
    "adcgpu_eri_packed_size": (C.c_int64, [C.c_int]),
    "adcgpu_synth_eri_packed": (C.c_int, [C.c_int, C.c_uint64, _dp, C.c_int]),
    "adcgpu_synth_uniform_block": (C.c_int, [C.c_int64, C.c_int, C.c_uint64, _dp]),
    "adcgpu_synth_dipole": (C.c_int, [C.c_int, C.c_uint64, _dp]),
    "adcgpu_set_dipole": (C.c_int, [_vp, _dp]),
    "adcgpu_modified_tm_adc2": (C.c_int, [_vp, C.c_int, _ip, _dp]),
    "adcgpu_fill_stvc": (C.c_int, [C.c_int, _dp, C.c_int, _ip]),
    "adcgpu_cvs_dim": (C.c_int64, [C.c_int, C.c_int, C.c_int, _ip, _ip]),
    "adcgpu_select_adc2s_cvs": (C.c_int, [C.c_int, C.c_int, C.c_int, _ip, _ip]),
    "adcgpu_build_adc2s_cvs": (C.c_int, [_vp, C.c_int, _ip, C.c_int, _ip, _i64p, C.c_char]),
    "adcgpu_adc2s_dim": (C.c_int64, [C.c_int, C.c_int, _ip]),
    "adcgpu_select_adc2s": (C.c_int, [C.c_int, C.c_int, _ip]),
    "adcgpu_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "adcgpu_ctx_destroy": (C.c_int, [_vp]),
    "adcgpu_last_error": (C.c_char_p, [_vp]),
    "adcgpu_set_orbitals": (C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    "adcgpu_set_eri_packed": (C.c_int, [_vp, _dp]),
    "adcgpu_set_eri_mo_complex": (C.c_int, [_vp, _dp]),
    "adcgpu_build_adc2s": (C.c_int, [_vp, C.c_int, _ip, _i64p, C.c_char, C.c_int]),
    "adcgpu_get_diag": (C.c_int, [_vp, _dp]),
    "adcgpu_export_coo": (C.c_int, [_vp, C.c_int64, _dp, _ip, _ip]),
    "adcgpu_write_hmlt_files": (C.c_int, [_vp, C.c_char_p, C.c_char]),
    "adcgpu_sigma": (C.c_int, [_vp, C.c_int, _dp, _dp]),
    "adcgpu_sigma_device": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int64]),
    "adcgpu_sigma_device_noalloc": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_int64]),
    "adcgpu_kernel_launches": (C.c_uint64, []),
    "adcgpu_davidson": (C.c_int, [_vp, C.POINTER(DavParams), _dp, _dp, C.POINTER(DavInfo)]),
    "adcgpu_write_davidson_file": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp, _dp]),
    "adcgpu_block_lanczos": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp]),
    "adcgpu_silstep": (C.c_int, [_vp, _dp, _dp, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int,
                                 C.c_int, C.c_int, _dp, C.POINTER(C.c_int), C.POINTER(SilState)]),
    "adcgpu_autocorr": (C.c_int, [_vp, C.c_int, _dp, C.c_double, C.c_double, C.c_int, C.c_double, _dp,
                                  C.POINTER(C.c_int), _i64p]),
    "adcgpu_chebyshev_auto": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_int, C.c_int, _dp, _dp, C.POINTER(C.c_int)]),
    "adcgpu_chebyshev_project": (C.c_int, [_vp, C.c_int, _dp, _dp, C.c_int, C.c_double, C.c_int]),
    "adcgpu_spectral_bounds": (C.c_int, [_vp, C.POINTER(DavParams), _dp]),
    "adcgpu_last_sigma_ms": (C.c_double, [_vp]),
    "adcgpu_device_bytes": (C.c_int64, [_vp]),
    "adcgpu_set_fp64_arith": (C.c_int, [_vp, C.c_int]),
    "adcgpu_sigma_stats": (C.c_int, [_vp, _dp, C.c_int]),
    "adcgpu_sigma_stats_by_store": (C.c_int, [_vp, _dp, C.c_int]),
    "adcgpu_mlp_num_params": (C.c_int64, []),
    "adcgpu_mlp_set_params": (C.c_int, [_vp, C.POINTER(C.c_float), C.c_int64]),
    "adcgpu_mlp_get_params": (C.c_int, [_vp, C.POINTER(C.c_float), C.c_int64]),
    "adcgpu_mlp_train_step": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "adcgpu_mlp_infer": (C.c_int, [_vp, C.c_int, _dp, _dp, C.POINTER(C.c_float), _dp, C.POINTER(C.c_float)]),
    "adcgpu_davidson_trace": (C.c_int, [_vp, C.POINTER(DavParams), C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp,
                                        C.POINTER(C.c_int)]),
    "adcgpu_sigma_autotune": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _dp]),
    "adcgpu_sigma_set_shape": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "adcgpu_gram_f32": (C.c_int, [_vp, C.c_int64, C.c_int, C.c_int, _vp, C.c_int64, _vp, C.c_int64, _vp, C.c_int]),
}

_lib = None


def lib():
    """Load libadcgpu.so; raises if it is absent or lacks a declared symbol."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libadcgpu.so not built ({LIB_PATH}); run __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)
