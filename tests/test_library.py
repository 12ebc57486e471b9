"""The C-ABI library loads and exports every entry point ``include/mrsr.h`` declares (CPU only)."""
import ctypes as C
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "mrsr.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mrsr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("mrsr_normalop_apply", "mrsr_nfft_normalop_create", "mrsr_backprojection", "mrsr_grog_gridding",
              "mrsr_cg"):
        assert s in syms


def test_library_exports_all_declared_symbols(mr):
    lib = mr.library()
    for s in declared_symbols():
        assert hasattr(lib, s), f"libmrsr.so does not export {s}"


def test_python_binding_covers_header(mr):
    from importlib import import_module
    _lib = import_module("mrsr_gb300._lib")
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_version_and_error_string(mr):
    lib = mr.library()
    assert lib.mrsr_version() >= 100
    assert isinstance(lib.mrsr_last_error(), bytes)


def test_invalid_arguments_are_rejected_without_a_device(mr):
    """Argument checks run on the host before any CUDA call."""
    lib = mr.library()
    h = C.c_void_p()
    shape = (C.c_int64 * 2)(16, 16)
    # ndims = 4 is rejected
    st = lib.mrsr_nfft_normalop_from_lambda(4, shape, 2, None, 1, None, 0, None, 1, 0, None, C.byref(h))
    assert st != 0
    assert b"ndims" in lib.mrsr_last_error()
    # rank above the compiled maximum is rejected
    st = lib.mrsr_nfft_normalop_from_lambda(2, shape, 99, None, 1, None, 0, None, 1, 0, None, C.byref(h))
    assert st != 0
