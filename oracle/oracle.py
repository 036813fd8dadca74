"""ctypes binding of the CPU oracle (viss_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline / reference legs, as the checker.  The product
package never imports this module.

Every function restates a reference routine; the C++ source cites the
reference file:line for each.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

MASK_NONE, MASK_REF_QUIRK, MASK_REF_INTENDED, MASK_GEOMETRIC = 0, 1, 2, 3


def build(force: bool = False) -> Path:
    """Compile viss_oracle.cpp with g++/OpenMP into oracle/_build/liboracle.so."""
    src = HERE / "viss_oracle.cpp"
    BUILD.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", str(src), "-o", str(tmp)]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class DftCfg(C.Structure):
    _fields_ = [("mask_mode", C.c_int32), ("res", C.c_int32), ("trunc_brightness", C.c_int32),
                ("recon_ref_mask", C.c_int32), ("occluded_value", C.c_float), ("pad0", C.c_float),
                ("phase_scale", C.c_double), ("n_offset", C.c_double),
                ("moon_radius_km", C.c_double), ("norm", C.c_double)]


class Geo(C.Structure):
    _fields_ = [("sat_pos", C.c_void_p), ("snap", C.c_void_p), ("pair", C.c_void_p),
                ("nsat", C.c_int32), ("pad", C.c_int32), ("S", C.c_int64)]


class OrbitCfg(C.Structure):
    _fields_ = [("nsat", C.c_int32), ("orbit_res", C.c_int32), ("orbit_counts", C.c_int32),
                ("index", C.c_int32), ("a_km", C.c_double), ("e", C.c_double),
                ("incl_deg", C.c_double), ("argp_deg", C.c_double), ("raan_step_deg", C.c_double),
                ("r1_m", C.c_void_p), ("r2_m", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        for name in ("oracle_vis_dft", "oracle_vis_dft_windex", "oracle_vis_dft_nxq", "oracle_recon", "oracle_vis_plain_f32",
                     "oracle_recon_plain_f32", "oracle_geo_mask", "oracle_orbit_positions",
                     "oracle_orbit_positions_f64"):
            getattr(_lib, name).restype = C.c_int
        _lib.oracle_uvw.restype = C.c_int64
        _lib.oracle_uvw_f64.restype = C.c_int64
        _lib.oracle_dedup_uvw.restype = C.c_int64
        _lib.oracle_text_read_stream.restype = C.c_int64
        _lib.oracle_text_write_stream.restype = C.c_int64
        _lib.oracle_shade_windows.restype = C.c_double
        _lib.oracle_max_threads.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def make_cfg(mask_mode=MASK_NONE, res=1, trunc=False, recon_ref_mask=False, occluded_value=240.0,
             phase_scale=0.5, n_offset=0.0, moon_radius_km=1737.4, norm=1.0) -> DftCfg:
    return DftCfg(int(mask_mode), int(res), int(bool(trunc)), int(bool(recon_ref_mask)),
                  float(occluded_value), 0.0, float(phase_scale), float(n_offset),
                  float(moon_radius_km), float(norm))


def make_geo(sat_pos, snap, pair):
    sat_pos = _f32(sat_pos)
    snap, pair = _i32(snap), _i32(pair)
    g = Geo(sat_pos.ctypes.data, snap.ctypes.data, pair.ctypes.data, int(sat_pos.shape[1]), 0,
            int(sat_pos.shape[0]))
    g._keep = (sat_pos, snap, pair)
    return g


def vis_dft(cfg: DftCfg, u, v, w, l, m, n, bright, shade=None, geo=None, nthreads=0):
    """FP64 shaded vis DFT; returns complex128[K]."""
    u, v, w, l, m, n, bright = map(_f32, (u, v, w, l, m, n, bright))
    shade = _i32(shade)
    K, J = u.size, l.size
    out = np.zeros((K, 2), np.float64)
    lib().oracle_vis_dft(C.byref(cfg), _p(u), _p(v), _p(w), C.c_int64(K), _p(shade),
                         C.byref(geo) if geo is not None else None, _p(l), _p(m), _p(n), _p(bright),
                         C.c_int64(J), _p(out), C.c_int(nthreads))
    return out[:, 0] + 1j * out[:, 1]


def vis_dft_windex(cfg: DftCfg, u, v, w, l, m, n, bright, shade, widx, nthreads=0):
    """vis_dft with the REF window tested on widx[j] instead of j; complex128[K]."""
    u, v, w, l, m, n, bright = map(_f32, (u, v, w, l, m, n, bright))
    shade, widx = _i32(shade), _i32(widx)
    K, J = u.size, l.size
    out = np.zeros((K, 2), np.float64)
    lib().oracle_vis_dft_windex(C.byref(cfg), _p(u), _p(v), _p(w), C.c_int64(K), _p(shade), _p(widx), _p(l), _p(m),
                                _p(n), _p(bright), C.c_int64(J), _p(out), C.c_int(nthreads))
    return out[:, 0] + 1j * out[:, 1]


def vis_dft_nxq(cfg: DftCfg, u, v, w, l, m, n, FF, NXq, countLoc, shade=None, nthreads=0):
    u, v, w, l, m, n, FF, NXq = map(_f32, (u, v, w, l, m, n, FF, NXq))
    countLoc, shade = _i32(countLoc), _i32(shade)
    K, J = u.size, l.size
    out = np.zeros((K, 2), np.float64)
    lib().oracle_vis_dft_nxq(C.byref(cfg), _p(u), _p(v), _p(w), C.c_int64(K), _p(shade), _p(l), _p(m),
                             _p(n), C.c_int64(J), _p(FF), _p(NXq), _p(countLoc), _p(out),
                             C.c_int(nthreads))
    return out[:, 0] + 1j * out[:, 1]


def recon(cfg: DftCfg, u, v, w, wgt, V, l, m, n, shade=None, geo=None, nthreads=0):
    """FP64 direct-DFT reconstruction; V complex[K]; returns complex128[J]."""
    u, v, w, l, m, n = map(_f32, (u, v, w, l, m, n))
    wgt = None if wgt is None else _f32(wgt)
    Vf = np.ascontiguousarray(np.stack([np.real(V), np.imag(V)], -1), dtype=np.float32)
    shade = _i32(shade)
    K, J = u.size, l.size
    out = np.zeros((J, 2), np.float64)
    lib().oracle_recon(C.byref(cfg), _p(u), _p(v), _p(w), _p(wgt), _p(Vf), C.c_int64(K), _p(shade),
                       C.byref(geo) if geo is not None else None, _p(l), _p(m), _p(n), C.c_int64(J),
                       _p(out), C.c_int(nthreads))
    return out[:, 0] + 1j * out[:, 1]


def vis_plain_f32(cfg: DftCfg, u, v, w, l, m, n, FF, d=2.0, shade=None, nthreads=0, optim=False):
    u, v, w, l, m, n, FF = map(_f32, (u, v, w, l, m, n, FF))
    shade = _i32(shade)
    K, J = u.size, l.size
    out = np.zeros((K, 2), np.float32)
    lib().oracle_vis_plain_f32(C.byref(cfg), _p(u), _p(v), _p(w), C.c_int64(K), _p(shade), _p(l),
                               _p(m), _p(n), _p(FF), C.c_int64(J), C.c_float(d), _p(out),
                               C.c_int(nthreads), C.c_int(int(optim)))
    return out[:, 0] + 1j * out[:, 1]


def recon_plain_f32(cfg: DftCfg, u, v, w, wgt, V, l, m, n, d=2.0, shade=None, nthreads=0, optim=False):
    u, v, w, wgt, l, m, n = map(_f32, (u, v, w, wgt, l, m, n))
    Vf = np.ascontiguousarray(np.stack([np.real(V), np.imag(V)], -1), dtype=np.float32)
    shade = _i32(shade)
    K, J = u.size, l.size
    out = np.zeros((J, 2), np.float32)
    lib().oracle_recon_plain_f32(C.byref(cfg), _p(u), _p(v), _p(w), _p(wgt), _p(Vf), C.c_int64(K),
                                 _p(shade), _p(l), _p(m), _p(n), C.c_int64(J), C.c_float(d), _p(out),
                                 C.c_int(nthreads), C.c_int(int(optim)))
    return out[:, 0] + 1j * out[:, 1]


def geo_mask(geo: Geo, R, l, m, n, K, J, nthreads=0):
    l, m, n = map(_f32, (l, m, n))
    mask = np.zeros((K, J), np.uint8)
    margin = np.zeros((K, J), np.float64)
    lib().oracle_geo_mask(C.byref(geo), C.c_double(R), _p(l), _p(m), _p(n), C.c_int64(K), C.c_int64(J),
                          _p(mask), _p(margin), C.c_int(nthreads))
    return mask.astype(bool), margin


def make_orbit_cfg(nsat, orbit_res, orbit_counts, index=1, a_km=2038.14, e=0.0, incl_deg=30.0,
                   argp_deg=0.0, raan_step_deg=0.08, r1_m=None, r2_m=None) -> OrbitCfg:
    r1 = _f32(r1_m)
    r2 = _f32(r2_m)
    c = OrbitCfg(int(nsat), int(orbit_res), int(orbit_counts), int(index), float(a_km), float(e),
                 float(incl_deg), float(argp_deg), float(raan_step_deg), r1.ctypes.data, r2.ctypes.data)
    c._keep = (r1, r2)
    return c


def orbit_positions(cfg: OrbitCfg, mode=1, nthreads=0):
    """Positions [S][nsat][3] float32 (km); mode 1 = reference FP32 mimic, 0 = FP64."""
    S = cfg.orbit_counts * (cfg.orbit_res // 3)
    pos = np.zeros((S, cfg.nsat, 3), np.float32)
    lib().oracle_orbit_positions(C.byref(cfg), C.c_int(mode), _p(pos), C.c_int(nthreads))
    return pos


def orbit_positions_f64(cfg: OrbitCfg, nthreads=0):
    S = cfg.orbit_counts * (cfg.orbit_res // 3)
    pos = np.zeros((S, cfg.nsat, 3), np.float64)
    lib().oracle_orbit_positions_f64(C.byref(cfg), _p(pos), C.c_int(nthreads))
    return pos


def uvw(pos, lambda_m, ordered=True, rounding=True):
    pos = _f32(pos)
    S, nsat = pos.shape[0], pos.shape[1]
    P = nsat * (nsat - 1) // (1 if ordered else 2)
    K = S * P
    u, v, w = (np.zeros(K, np.float32) for _ in range(3))
    snap = np.zeros(K, np.int32)
    pair = np.zeros(K, np.int32)
    lib().oracle_uvw(_p(pos), C.c_int64(S), C.c_int32(nsat), C.c_int(int(ordered)),
                     C.c_double(lambda_m), C.c_int(int(rounding)), _p(u), _p(v), _p(w), _p(snap), _p(pair))
    return u, v, w, snap, pair


def uvw_f64(pos64, lambda_m, ordered=False):
    pos64 = np.ascontiguousarray(pos64, dtype=np.float64)
    S, nsat = pos64.shape[0], pos64.shape[1]
    P = nsat * (nsat - 1) // (1 if ordered else 2)
    u, v, w = (np.zeros(S * P, np.float32) for _ in range(3))
    lib().oracle_uvw_f64(_p(pos64), C.c_int64(S), C.c_int32(nsat), C.c_int(int(ordered)),
                         C.c_double(lambda_m), _p(u), _p(v), _p(w))
    return u, v, w


def dedup_uvw(u, v, w):
    u, v, w = (np.array(x, dtype=np.float32, copy=True) for x in (u, v, w))
    n = lib().oracle_dedup_uvw(_p(u), _p(v), _p(w), C.c_int64(u.size))
    return u[:n], v[:n], w[:n]


def shade_windows(u, v, w, RES, mean_r=0.0, mode=1):
    """Raw shadeM (1-based thetaS, thetaE, phiS, phiE) int32[K,4] and the mean radius used."""
    u, v, w = map(_f32, (u, v, w))
    out = np.zeros((u.size, 4), np.int32)
    mr = lib().oracle_shade_windows(_p(u), _p(v), _p(w), C.c_int64(u.size), C.c_int(RES),
                                    C.c_double(mean_r), C.c_int(mode), _p(out))
    return out, mr


def normalise_shade(raw):
    raw = _i32(raw)
    M = np.zeros_like(raw)
    lib().oracle_normalise_shade(_p(raw), C.c_int64(raw.shape[0]), _p(M))
    return M


def nxq(NX, J):
    NX = _f32(NX)
    countLoc = np.zeros(J, np.int32)
    NXq = np.zeros(NX.size, np.int32)
    lib().oracle_nxq(_p(NX), C.c_int64(NX.size), C.c_int64(J), _p(countLoc), _p(NXq))
    return countLoc, NXq


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def text_read_stream(path, ncols, cap):
    """The reference's single-threaded `ifstream >>` reading loop; columns [ncols, rows]."""
    out = np.zeros((ncols, cap), np.float32)
    n = lib().oracle_text_read_stream(str(path).encode(), C.c_int(ncols), _p(out), C.c_int64(cap))
    return out[:, :min(n, cap)], n


def text_write_stream(path, values):
    """The reference's `file << value << std::endl` writing loop."""
    values = np.ascontiguousarray(values, dtype=np.float32)
    return lib().oracle_text_write_stream(str(path).encode(), _p(values), C.c_int64(values.size))
