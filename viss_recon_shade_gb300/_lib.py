"""ctypes binding of libvissgb.so (declarations in include/viss_gb300.h).

The library is built in-tree by ``viss_recon_shade_gb300.build`` (or
``__graft_entry__.build()``).  Importing this module loads it; a missing
library raises ImportError -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvissgb.so"

# status codes
VISS_OK = 0
VISS_ERR_INVALID = -1
VISS_ERR_WORKSPACE = -2
VISS_ERR_CUDA = -3
VISS_ERR_RANGE = -4
VISS_ERR_TIMEOUT = -5
VISS_ERR_UNSUPPORTED = -6
VISS_ERR_IO = -7
VISS_ERR_FORMAT = -8

MASK_NONE, MASK_REF_QUIRK, MASK_REF_INTENDED, MASK_GEOMETRIC = 0, 1, 2, 3
RECON_MASK_NONE, RECON_MASK_REF, RECON_MASK_GEOMETRIC = 0, 1, 2
PREC_PLAIN, PREC_FAST, PREC_COMPENSATED, PREC_F64_PHASE = 0, 1, 2, 3
VARIANT_PLAIN, VARIANT_OPTIM = 0, 1


class DftCfg(C.Structure):
    _fields_ = [("mask_mode", C.c_int32), ("recon_mask", C.c_int32), ("precision", C.c_int32),
                ("res", C.c_int32), ("trunc_brightness", C.c_int32), ("occluded_value", C.c_float),
                ("phase_scale", C.c_double), ("n_offset", C.c_double), ("moon_radius_km", C.c_double),
                ("norm", C.c_double)]


class Sky(C.Structure):
    _fields_ = [("l", C.c_void_p), ("m", C.c_void_p), ("n", C.c_void_p), ("bright", C.c_void_p),
                ("J", C.c_int64)]


class VisSet(C.Structure):
    _fields_ = [("u", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p), ("wgt", C.c_void_p),
                ("shade", C.c_void_p), ("snap", C.c_void_p), ("pair", C.c_void_p), ("K", C.c_int64)]


class Geometry(C.Structure):
    _fields_ = [("sat_pos", C.c_void_p), ("S", C.c_int64), ("nsat", C.c_int32), ("reserved", C.c_int32)]


class FineMap(C.Structure):
    _fields_ = [("FF", C.c_void_p), ("NXq_f", C.c_void_p), ("NXq_i", C.c_void_p), ("countLoc", C.c_void_p),
                ("X", C.c_int64)]


MAX_CHANNELS = 64


class Batch(C.Structure):
    _fields_ = [("nch", C.c_int32), ("reserved", C.c_int32), ("row_off", C.POINTER(C.c_int64)),
                ("bright", C.c_void_p), ("norm", C.POINTER(C.c_double))]


class Tuning(C.Structure):
    _fields_ = [("ctas_per_sm", C.c_int32), ("vis_split", C.c_int32), ("rec_items", C.c_int32),
                ("tile", C.c_int32)]


class OrbitCfg(C.Structure):
    _fields_ = [("nsat", C.c_int32), ("orbit_res", C.c_int32), ("orbit_counts", C.c_int32),
                ("index", C.c_int32), ("a_km", C.c_double), ("e", C.c_double), ("incl_deg", C.c_double),
                ("argp_deg", C.c_double), ("raan_step_deg", C.c_double), ("r1_m", C.c_void_p),
                ("r2_m", C.c_void_p), ("fp64", C.c_int32), ("reserved", C.c_int32)]


_P = C.c_void_p
_SIGS = {
    "viss_status_str": (C.c_char_p, [C.c_int]),
    "viss_last_error": (C.c_char_p, []),
    "viss_version": (C.c_int, []),
    "viss_launch_count": (C.c_uint64, []),
    "viss_vis_dft_workspace": (C.c_size_t, [C.POINTER(DftCfg), C.c_int64, C.c_int64, C.POINTER(Geometry)]),
    "viss_vis_dft": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(VisSet), C.POINTER(Geometry), _P, _P,
                               C.c_size_t, _P]),
    "viss_vis_dft_noalloc": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(VisSet), C.POINTER(Geometry), _P,
                                       _P]),
    "viss_recon_workspace": (C.c_size_t, [C.POINTER(DftCfg), C.c_int64, C.c_int64, C.POINTER(Geometry)]),
    "viss_recon": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(VisSet), C.POINTER(Geometry), _P, _P,
                             _P, C.c_size_t, _P]),
    "viss_vis_dft_batch_workspace": (C.c_size_t, [C.POINTER(DftCfg), C.POINTER(Batch), C.c_int64, C.c_int64,
                                                  C.POINTER(Geometry), C.POINTER(Tuning)]),
    "viss_vis_dft_batch": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(VisSet), C.POINTER(Batch),
                                     C.POINTER(Geometry), C.POINTER(Tuning), _P, _P, C.c_size_t, _P]),
    "viss_recon_batch_workspace": (C.c_size_t, [C.POINTER(DftCfg), C.POINTER(Batch), C.c_int64, C.c_int64,
                                                C.POINTER(Geometry), C.POINTER(Tuning)]),
    "viss_recon_batch": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(VisSet), C.POINTER(Batch),
                                   C.POINTER(Geometry), C.POINTER(Tuning), _P, _P, _P, C.c_size_t, _P]),
    "viss_vis_dft_map_workspace": (C.c_size_t, [C.POINTER(DftCfg), C.c_int64, C.c_int64, C.POINTER(FineMap),
                                                C.POINTER(Geometry)]),
    "viss_vis_dft_map": (C.c_int, [C.POINTER(DftCfg), C.POINTER(Sky), C.POINTER(FineMap), C.POINTER(VisSet),
                                   C.POINTER(Geometry), _P, _P, C.c_size_t, _P]),
    "viss_workspace_flags": (C.c_int, [_P, C.POINTER(C.c_int32), _P]),
    "viss_workspace_limb_count": (C.c_int, [_P, C.POINTER(C.c_int64), _P]),
    "viss_vis_dft_windowed_workspace": (C.c_size_t, [_P, C.c_int64, C.c_int64]),
    "viss_vis_dft_windowed": (C.c_int, [_P, _P, _P, _P, _P, _P, C.c_size_t, _P]),
    "viss_nxq_workspace": (C.c_size_t, [C.c_int64, C.c_int64]),
    "viss_nxq": (C.c_int, [_P, C.c_int64, C.c_int64, _P, _P, _P, C.c_size_t, _P]),
    "viss_visscal": (C.c_int, [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                               C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, _P]),
    "viss_imagerecon": (C.c_int, [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                  C.c_float, C.c_float, C.c_float, C.c_int, _P]),
    "viss_orbit_snapshots": (C.c_int64, [C.POINTER(OrbitCfg)]),
    "viss_orbit_positions": (C.c_int, [C.POINTER(OrbitCfg), _P, _P, _P]),
    "viss_baseline_uvw": (C.c_int, [_P, _P, C.c_int64, C.c_int32, C.c_int, C.c_double, C.c_int, _P, _P, _P, _P, _P,
                                    _P]),
    "viss_dedup_uvw_workspace": (C.c_size_t, [C.c_int64]),
    "viss_dedup_uvw": (C.c_int, [_P, _P, _P, C.c_int64, C.POINTER(C.c_int64), _P, C.c_size_t, _P]),
    "viss_unique_uvw_workspace": (C.c_size_t, [C.c_int64, C.c_int32, C.c_int]),
    "viss_unique_uvw": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_int, C.c_double, _P, _P, _P, C.c_int64,
                                  C.POINTER(C.c_int64), _P, C.c_size_t, _P]),
    "viss_shade_windows_workspace": (C.c_size_t, [C.c_int64]),
    "viss_shade_windows": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int, C.c_double, _P, C.POINTER(C.c_double), _P,
                                     C.c_size_t, _P]),
    "viss_normalise_shade": (C.c_int, [_P, C.c_int64, _P, _P]),
    "viss_sfu_probe": (C.c_int, [C.c_int, C.c_int, _P, C.POINTER(C.c_int64), _P]),
    "viss_text_read_floats": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _P, C.c_int64, C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]),
    "viss_text_read_ints": (C.c_int, [C.c_char_p, C.c_int, _P, C.c_int64, C.POINTER(C.c_int64)]),
    "viss_text_write_floats": (C.c_int, [C.c_char_p, C.c_int, _P, C.c_int64, C.c_int64]),
    "viss_text_write_ints": (C.c_int, [C.c_char_p, C.c_int, _P, C.c_int64]),
}


def declared_symbols() -> list[str]:
    """The entry points include/viss_gb300.h declares."""
    import re
    hdr = (Path(__file__).resolve().parents[1] / "include" / "viss_gb300.h").read_text()
    return sorted(set(re.findall(r"VISS_API\s+[\w\s\*]+?\b(viss_\w+)\s*\(", hdr)))


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"libvissgb.so not built ({LIB_PATH}); run `python viss_recon_shade_gb300/build.py` "
            "or __graft_entry__.build() -- there is no CPU fallback")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


class VissError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib.viss_last_error().decode(errors="replace")
        super().__init__(f"{where}: {lib.viss_status_str(status).decode()} ({status}): {msg}")


def check(status: int, where: str) -> None:
    if status != VISS_OK:
        raise VissError(status, where)
