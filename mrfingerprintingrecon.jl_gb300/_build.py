"""In-tree build of ``libmrsr.so`` (the sm_103a C-ABI library) with nvcc.

Every ``csrc/*.cu`` is compiled in parallel for ``sm_103a`` only and linked
into ``libmrsr.so`` next to this file.  Objects go to ``_build/``; a source
is recompiled when it or any header is newer than its object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OBJDIR = PKG / "_build"
LIB = PKG / "libmrsr.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmrsr.so")


def _headers_mtime():
    hs = list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def build(verbose=False, jobs=None, extra_flags=()):
    nvcc = nvcc_path()
    OBJDIR.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    hdr = _headers_mtime()
    todo = []
    for s in srcs:
        o = OBJDIR / (s.stem + ".o")
        if not o.exists() or o.stat().st_mtime < max(s.stat().st_mtime, hdr):
            todo.append((s, o))

    def compile_one(so):
        s, o = so
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", str(s), "-o", str(o)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {s.name}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return s.name

    if todo:
        jobs = jobs or min(len(todo), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for name in ex.map(compile_one, todo):
                if verbose:
                    print("compiled", name)
    objs = [str(OBJDIR / (s.stem + ".o")) for s in srcs]
    if todo or not LIB.exists() or LIB.stat().st_mtime < max(Path(o).stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
