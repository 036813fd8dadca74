"""ctypes binding of oracle/ref_thrust.cu: the reference's thrust call sites.

TEST INFRASTRUCTURE ONLY (tests/ and bench.py's reference legs).  The library
is compiled with nvcc for this GPU into oracle/_build/libref_thrust.so with the
flags the reference programs are built with (-O3 -arch=sm_103a).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libref_thrust.so"


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return "nvcc"


def build(force: bool = False) -> Path:
    src = HERE / "ref_thrust.cu"
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.so")
    subprocess.run([_nvcc(), "-std=c++17", "-O3", "-arch=sm_103a", "-shared", "-Xcompiler", "-fPIC", str(src),
                    "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.ref_thrust_mean_r.restype = C.c_int
        _lib.ref_thrust_mean_r.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        _lib.ref_thrust_sort_unique.restype = C.c_int64
        _lib.ref_thrust_sort_unique.argtypes = [C.c_void_p, C.c_int64]
    return _lib


def mean_r(r_complex) -> tuple[float, float]:
    """(sum, mean) of the real parts of a complex64 CUDA tensor (or K x 2 float32),
    thrust::transform_reduce as shade1M.cu:219-220 calls it."""
    import torch
    torch.cuda.synchronize()
    s, m = C.c_float(), C.c_float()
    n = r_complex.numel() if r_complex.dtype == torch.complex64 else r_complex.numel() // 2
    if lib().ref_thrust_mean_r(C.c_void_p(r_complex.data_ptr()), n, C.byref(s), C.byref(m)) != 0:
        raise RuntimeError("ref_thrust_mean_r failed")
    return s.value, m.value


def sort_unique(rows) -> int:
    """Sort + unique in place on an (n, 3) float32 CUDA tensor (SortCompare /
    UniqueCompare, MIncline_generate_uvw_float.cu:374-378); returns the unique count."""
    import torch
    assert rows.dtype == torch.float32 and rows.is_contiguous() and rows.shape[-1] == 3
    torch.cuda.synchronize()
    n = lib().ref_thrust_sort_unique(C.c_void_p(rows.data_ptr()), rows.shape[0])
    if n < 0:
        raise RuntimeError("ref_thrust_sort_unique failed")
    return int(n)
