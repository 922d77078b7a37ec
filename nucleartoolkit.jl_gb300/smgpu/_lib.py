"""ctypes binding of libsmgpu.so (the C ABI in include/smgpu.h).

The library is the only compute path: there is no CPU fallback, and loading
fails loudly when the shared object has not been built.
"""
import ctypes as C
import os

from . import build as _build

# Status codes (include/smgpu.h)
OK = 0
ERR_ARG = -1
ERR_IO = -2
ERR_PARSE = -3
ERR_NUCLEUS = -4
ERR_CUDA = -5
ERR_NOMEM = -6
ERR_LIMIT = -7
ERR_NOCONV = -8
ERR_EMPTY = -9
ERR_DEVICE = -10

FP64 = 0
MIXED = 1      # FP32 H·v and Krylov storage, FP64 Lanczos arithmetic
MIXED_DF = 2   # as MIXED, with the residual and re-orthogonalisation in double-float

# Every symbol include/smgpu.h declares, with its ctypes signature.
_vp = C.c_void_p
SIGNATURES = {
    "smgpu_problem_create_from_snt": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(_vp)]),
    "smgpu_problem_create_from_snt_J": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.POINTER(_vp)]),
    "smgpu_problem_create": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "smgpu_problem_destroy": (C.c_int, [_vp]),
    "smgpu_last_error": (C.c_char_p, [_vp]),
    "smgpu_dims": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int), _vp]),
    "smgpu_blocks": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "smgpu_export_basis": (C.c_int, [_vp, _vp, _vp]),
    "smgpu_export_jumps": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_longlong), _vp, _vp]),
    "smgpu_matvec": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int]),
    "smgpu_solve": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp, _vp]),
    "smgpu_jj": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "smgpu_obtr": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int, _vp, C.c_int, _vp]),
    "smgpu_ec_td_length": (C.c_int, [_vp, _vp]),
    "smgpu_ec_td": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "smgpu_wigner3j": (C.c_double, [C.c_int] * 6),
    "smgpu_wigner6j": (C.c_double, [C.c_int] * 6),
    "smgpu_solve_block": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp,
                                    _vp]),
    "smgpu_solve_J": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp, _vp]),
    "smgpu_timings": (C.c_int, [_vp, _vp]),
    "smgpu_stats": (C.c_int, [_vp, _vp]),
    "smgpu_time_matvec": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "smgpu_tune_report": (C.c_int, [_vp, C.c_int, _vp, _vp, C.POINTER(C.c_int)]),
    "smgpu_matvec_noalloc": (C.c_int, [_vp, _vp, _vp, _vp]),
    "smgpu_l2_read_bandwidth": (C.c_int, [C.c_longlong, C.c_int, C.POINTER(C.c_double)]),
    "smgpu_write_wav": (C.c_int, [C.c_char_p, C.c_longlong, C.c_int, C.c_int, _vp, _vp, _vp]),
    "smgpu_read_wav_header": (C.c_int, [C.c_char_p, C.c_longlong, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "smgpu_read_wav": (C.c_int, [C.c_char_p, C.c_longlong, C.c_int, _vp, _vp, _vp]),
    "smgpu_wav_last_error": (C.c_char_p, []),
    "smgpu_multi_create_from_snt": (C.c_int, [C.POINTER(C.c_char_p), C.c_int, C.c_char_p, C.POINTER(_vp)]),
    "smgpu_multi_destroy": (C.c_int, [_vp]),
    "smgpu_multi_last_error": (C.c_char_p, [_vp]),
    "smgpu_multi_dims": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "smgpu_multi_matvec": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "smgpu_multi_solve": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp, _vp]),
    "smgpu_multi_stats": (C.c_int, [_vp, _vp]),
    "smgpu_multi_timings": (C.c_int, [_vp, _vp]),
    "smgpu_multi_time_matvec": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "smgpu_batch_create_from_snt": (C.c_int, [C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.c_int,
                                              C.POINTER(_vp)]),
    "smgpu_batch_destroy": (C.c_int, [_vp]),
    "smgpu_batch_last_error": (C.c_char_p, [_vp]),
    "smgpu_batch_dims": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int), _vp]),
    "smgpu_batch_matvec": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "smgpu_batch_solve": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp, _vp]),
    "smgpu_batch_stats": (C.c_int, [_vp, _vp]),
    "smgpu_batch_timings": (C.c_int, [_vp, _vp]),
    "smgpu_batch_time_matvec": (C.c_int, [_vp, C.c_int, C.c_int, C.POINTER(C.c_double)]),
}

_lib = None


class SmgpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"smgpu error {code}: {msg}")
        self.code = code


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libsmgpu.so (building it in-tree first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"libsmgpu.so is not built ({path})")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code: int, handle=None):
    if code != OK:
        msg = load().smgpu_last_error(handle)
        raise SmgpuError(code, (msg or b"").decode(errors="replace"))


def check_multi(code: int, handle=None):
    """check() for smgpu_multi handles."""
    if code != OK:
        msg = load().smgpu_multi_last_error(handle)
        raise SmgpuError(code, (msg or b"").decode(errors="replace"))


def check_batch(code: int, handle=None):
    """check() for smgpu_batch handles."""
    if code != OK:
        msg = load().smgpu_batch_last_error(handle)
        raise SmgpuError(code, (msg or b"").decode(errors="replace"))


def check_wav(code: int):
    """check() for the .wav calls."""
    if code != OK:
        msg = load().smgpu_wav_last_error()
        raise SmgpuError(code, (msg or b"").decode(errors="replace"))
