"""ctypes binding of ``libmrsr.so`` (declarations in ``include/mrsr.h``).

Loading fails loudly: there is no CPU implementation behind this package.
"""
import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmrsr.so"

MRSR_OK, MRSR_ERR_ARG, MRSR_ERR_CUDA, MRSR_ERR_ALLOC, MRSR_ERR_UNSUPPORTED, MRSR_ERR_STATE, MRSR_ERR_DEVICE = range(7)
PREC_FP32, PREC_FP16, PREC_FP16_TC = 0, 1, 3
DCF_NONE, DCF_RADIAL_2D, DCF_RADIAL_3D, DCF_ARRAY = range(4)
KIND_NFFT, KIND_FFT = 0, 1

p = C.c_void_p
i64p = C.POINTER(C.c_int64)
i32 = C.c_int
i64 = C.c_int64
f32 = C.c_float
f64 = C.c_double

# name -> argtypes (all return int unless listed in _VOID / _STR)
SIGNATURES = {
    "mrsr_last_error": [],
    "mrsr_version": [],
    "mrsr_nfft_normalop_create": [i32, i64p, i64, i64, p, p, p, i32, i32, p, i32, i32, p, C.POINTER(p)],
    "mrsr_nfft_normalop_from_lambda": [i32, i64p, i32, p, i32, p, i64, p, i32, i32, p, C.POINTER(p)],
    "mrsr_fft_normalop_create": [i32, i64p, i64, i64, p, p, p, i32, i32, i32, p, i32, i32, p, C.POINTER(p)],
    "mrsr_fft_normalop_create_from_mask": [i32, i64p, i64, p, p, i32, i32, p, i32, i32, p, C.POINTER(p)],
    "mrsr_fft_normalop_from_lambda": [i32, i64p, i32, p, p, i32, i32, p, C.POINTER(p)],
    "mrsr_normalop_apply": [p, p, p, f32, f32, f32, f32, p],
    "mrsr_normalop_apply_host": [p, p, p, f32, f32, f32, f32, p],
    "mrsr_normalop_info": [p, i64p],
    "mrsr_normalop_get_kmask": [p, p, p],
    "mrsr_normalop_get_lambda": [p, p, p],
    "mrsr_normalop_profile": [p, p, p, i32, C.POINTER(f32), p],
    "mrsr_normalop_check": [p, p],
    "mrsr_normalop_destroy": [p],
    "mrsr_backprojection": [i32, i64p, i64, i64, i32, p, p, p, p, i32, i32, p, i32, p, p, p],
    "mrsr_backprojection_cartesian": [i32, i64p, i64, i64, i32, i32, p, p, p, p, i32, i32, p, p, p],
    "mrsr_forward_model": [i32, i64p, i64, i64, i32, p, p, p, i32, i32, p, p, p],
    "mrsr_grog_calib": [i32, i64, i64, i64, i32, i32, p, p, p, p],
    "mrsr_espirit": [i32, i64p, i64p, i32, p, i64p, f64, f64, i32, p, p, p],
    "mrsr_grog_gridding": [i32, i64p, i64, i64, i64, i32, i32, p, p, p, p, p],
    "mrsr_cg": [p, p, p, i32, f64, f64, C.POINTER(i32), C.POINTER(f64), p],
    "mrsr_cg_refined": [p, p, p, p, i32, i32, f64, C.POINTER(i32), C.POINTER(f64), p],
    "mrsr_cg_noalloc": [p, p, p, i32, f64, f64, C.POINTER(i32), C.POINTER(f64), p],
    "mrsr_cg_relaxed": [p, p, p, p, i32, f64, f64, f64, C.POINTER(i32), C.POINTER(i32), C.POINTER(f64), p],
    "mrsr_normalop_stack": [p, i32, p, C.POINTER(p)],
    "mrsr_cg_stacked": [p, p, p, i32, f64, f64, C.POINTER(i32), C.POINTER(f64), p],
    "mrsr_normalop_share": [p, p, i32, i32, p, C.POINTER(p)],
    "mrsr_cg_batch_create": [C.POINTER(p), C.POINTER(p), C.POINTER(p), C.POINTER(p), i32, i32, i32, p, C.POINTER(p)],
    "mrsr_cg_batch_create_relaxed": [C.POINTER(p), C.POINTER(p), C.POINTER(p), C.POINTER(p), i32, i32, i32, p,
                                     C.POINTER(p)],
    "mrsr_cg_batch_launch": [p, p],
    "mrsr_cg_batch_result": [p, i32, C.POINTER(i32), C.POINTER(f64)],
    "mrsr_cg_batch_destroy": [p],
    # internal test hook (include/mrsr_test.h), not part of the product ABI
    "mrsr_test_set_device_error": [p, i32, p],
}
_VOID = {"mrsr_normalop_destroy", "mrsr_cg_batch_destroy"}
_STR = {"mrsr_last_error"}

_lib = None


def load():
    """Load (and type) the library; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"{LIB_PATH.name} is not built; run __graft_entry__.build() (nvcc, sm_103a). "
            "This package has no CPU implementation.")
    lib = C.CDLL(str(LIB_PATH))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = None if name in _VOID else (C.c_char_p if name in _STR else C.c_int)
    _lib = lib
    return lib


class MrsrError(RuntimeError):
    pass


def check(status):
    """Map a status code to the exception type the reference raises."""
    if status == MRSR_OK:
        return
    msg = load().mrsr_last_error().decode(errors="replace")
    if status == MRSR_ERR_ARG:
        if msg.startswith("AssertionError"):
            raise AssertionError(msg)
        raise ValueError(msg)
    if status == MRSR_ERR_ALLOC:
        raise MemoryError(msg)
    if status == MRSR_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise MrsrError(f"status {status}: {msg}")


def int64_array(vals):
    arr = (C.c_int64 * len(vals))(*[int(v) for v in vals])
    return arr
