"""ctypes binding of libmkgpu.so (declared in include/mkgpu.h).

Loading order mirrors the reference's minkasi/lib/_minkasi_init.py:9-16: the
in-package library first, then ``libmkgpu.so`` on the loader path.  There is
no CPU fallback: if neither loads, importing a kernel raises.
"""
from __future__ import annotations

import ctypes
import os
import re
from typing import Optional

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libmkgpu.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "mkgpu.h")

MK_OK, MK_ERR_ARG, MK_ERR_CUDA, MK_ERR_CUFFT, MK_ERR_CUBLAS, MK_ERR_RANGE, MK_ERR_NOMEM, MK_ERR_NUMERIC = range(8)
MK_F64, MK_F32 = 0, 1
(MK_S_ZR, MK_S_PAP, MK_S_ALPHA, MK_S_ZRNEW, MK_S_BETA, MK_S_RR, MK_S_FLAG, MK_S_ITER,
 MK_PCG_NSCALAR) = range(9)


class MkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[mkgpu error {code}] {msg}")
        self.code = code


_vp, _i64, _i32, _sz = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_size_t
_dbl = ctypes.c_double
_pp = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes)
SIGNATURES = {
    "mk_last_error": (ctypes.c_char_p, []),
    "mk_version": (_i32, []),
    "mk_map2tod": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp]),
    "mk_tod2map": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _vp]),
    "mk_tod2map_staged": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _vp]),
    "mk_tod2map_status": (_i32, [ctypes.POINTER(ctypes.c_int), _vp]),
    "mk_tod2map_rows": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _vp]),
    "mk_pix_car": (_i32, [_vp, _vp, _vp, _i64, _dbl, _dbl, _dbl, _dbl, _i64, _i32, _vp]),
    "mk_pix_wcs_car": (_i32, [_vp, _vp, _vp, _i64, _vp, _i64, _vp]),
    "mk_cuts_gather": (_i32, [_vp, _vp, _vp, _i64, _i64, _i32, _i32, _vp]),
    "mk_cuts_scatter": (_i32, [_vp, _vp, _vp, _i64, _i64, _i32, _i32, _vp]),
    "mk_stripes_map2tod": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp]),
    "mk_stripes_tod2map": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp]),
    "mk_binned_map2tod": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _dbl, _dbl, _i32, _i32, _i32, _vp]),
    "mk_binned_tod2map": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _dbl, _dbl, _i32, _i32, _i32, _vp]),
    "mk_pol_npol": (_i32, [_i32]),
    "mk_pol_sincos": (_i32, [_vp, _vp, _vp, _i64, _i32, _vp]),
    "mk_polmap2tod": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _i32, _vp]),
    "mk_tod2polmap": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i64, _i64, _i32, _i32, _vp, _vp]),
    "mk_pol_precon_mul": (_i32, [_vp, _vp, _vp, _i64, _i32, _i32, _vp]),
    "mk_check_pix": (_i32, [_vp, _i64, _i64, ctypes.POINTER(ctypes.c_int64), _vp]),
    "mk_tod2map_fixed_scratch_bytes": (_sz, [_i64]),
    "mk_tod2map_fixed": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i32, _vp, _vp]),
    "mk_tod2map_fixed_noalloc": (_i32, [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i32, _vp]),
    "mk_pixplan_create": (_i32, [_pp, _vp, _i64, _i64, _vp]),
    "mk_tod2map_sorted": (_i32, [_vp, _vp, _vp, _i32, _vp]),
    "mk_pixplan_destroy": (_i32, [_vp]),
    "mk_dct1_workspace_bytes": (_i32, [_i64, _i64, _i32, ctypes.POINTER(ctypes.c_size_t)]),
    "mk_dct1_plan_create": (_i32, [_pp, _i64, _i64, _i32, _vp, _sz]),
    "mk_dct1_exec": (_i32, [_vp, _vp, _vp, _vp]),
    "mk_dct1_plan_destroy": (_i32, [_vp]),
    "mk_noise_workspace_bytes": (_i32, [_i64, _i64, _i32, ctypes.POINTER(ctypes.c_size_t)]),
    "mk_noise_plan_create": (_i32, [_pp, _i64, _i64, _i32, _vp, _sz]),
    "mk_apply_noise": (_i32, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _i32, _vp]),
    "mk_noise_plan_destroy": (_i32, [_vp]),
    "mk_rotate": (_i32, [_vp, _vp, _vp, _vp, _i32, _vp]),
    "mk_noise_status": (_i32, [_vp, ctypes.POINTER(ctypes.c_int), _vp]),
    "mk_reduce_scratch_bytes": (_sz, []),
    "mk_dot": (_i32, [_vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mk_axpy": (_i32, [_vp, _vp, ctypes.c_double, _i64, _i32, _vp]),
    "mk_mul": (_i32, [_vp, _vp, _vp, _i64, _i32, _vp]),
    "mk_pcg_update": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mk_pcg_init": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mk_pcg_step_xr": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mk_pcg_step_zp": (_i32, [_vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp]),
    "mk_scale_add": (_i32, [_vp, _vp, _vp, _vp, _i64, _i32, _vp]),
    "mk_conv3x3_fwd": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "mk_conv3x3_adj": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp]),
    "mk_conv3x3_wgrad_scratch_bytes": (_sz, [_i32, _i32, _i32, _i32, _i32]),
    "mk_conv3x3_wgrad": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _vp, _sz, _vp]),
    "mk_set_dct_engine": (_i32, [_i32]),
    "mk_get_dct_engine": (_i32, []),
    "mk_dct1_engine": (_i32, [_vp]),
    "mk_dct1_describe": (_i32, [_i64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64),
                                ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "mk_noise_engine": (_i32, [_vp]),
    "mk_noise_group_create": (_i32, [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "mk_noise_group_exec": (_i32, [_vp, _vp]),
    "mk_noise_group_status": (_i32, [_vp, ctypes.POINTER(ctypes.c_int), _vp]),
    "mk_noise_group_destroy": (_i32, [_vp]),
    "mk_noise_split": (_i32, [_vp, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "mk_set_fft4_split": (_i32, [_i32]),
    "mk_get_fft4_split": (_i32, []),
    "mk_learned_precon_work_bytes": (_sz, [_i32, _i32, _i32, _vp]),
    "mk_learned_precon_apply": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _sz, _i32, _vp]),
    "mk_learned_precon_stencil": (_i32, [_vp, _vp, _vp, _i32, _i32, _i32, _vp, _i32, _vp, _sz, _i32, _vp]),
    "mk_learned_precon_stencil_work_bytes": (_sz, [_i32, _i32, _i32]),
}

_lib: Optional[ctypes.CDLL] = None


def header_symbols() -> list:
    """Function names declared in include/mkgpu.h."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mk_[a-z0-9_]+)\s*\(", txt)))


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Load and bind libmkgpu.so.  Raises OSError if it cannot be found."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    errors = []
    h = None
    for cand in ([path] if path else [LIB_PATH, "libmkgpu.so"]):
        try:
            h = ctypes.CDLL(cand)
            break
        except OSError as e:  # pragma: no cover - depends on the machine
            errors.append(f"{cand}: {e}")
    if h is None:
        raise OSError("libmkgpu.so not found; build it with `python minkasi_gb300/build.py` "
                      "(or __graft_entry__.build()).\n" + "\n".join(errors))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(h, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = h
    return h


def check(rc: int, what: str = "") -> None:
    if rc != MK_OK:
        msg = load().mk_last_error().decode(errors="replace")
        raise MkError(rc, f"{what}: {msg}" if what else msg)
