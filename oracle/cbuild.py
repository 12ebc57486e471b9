"""Builds and loads the oracle's C restatement (``grog_index.c``) with gcc.

Test infrastructure only (see ``oracle/__init__.py``).
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle_grog.so"
SRC = HERE / "grog_index.c"


def build():
    OUT.mkdir(exist_ok=True)
    if LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-o", str(LIB), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def grog_index_c(trj, img_shape, Nr):
    """(idx int32, shift float64), arrays (d, Ns, Nt) like ``trj``."""
    lib = C.CDLL(str(build()))
    f = lib.oracle_grog_index
    f.restype = None
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    t = np.asfortranarray(np.asarray(trj, dtype=np.float32))
    d = t.shape[0]
    n = int(np.prod(t.shape[1:]))
    idx = np.empty(t.shape, dtype=np.int32, order="F")
    shift = np.empty(t.shape, dtype=np.float64, order="F")
    shp = np.asarray(img_shape, dtype=np.int64)
    f(t.ctypes.data, d, n, shp.ctypes.data, int(Nr), idx.ctypes.data, shift.ctypes.data)
    return idx, shift
