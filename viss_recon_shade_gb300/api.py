"""Torch-tensor interface over the C ABI (include/viss_gb300.h).

Operator names and argument meanings follow the reference programs:
``visscal`` / ``imagerecon`` take the argument lists of the reference kernels
(vissGen10M_shade.cu:108-116, 149-154); ``vis_dft`` / ``recon`` are the general
forms with explicit mask, precision and phase conventions.  Device tensors are
used in place; the work is enqueued on torch's current CUDA stream.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, replace
from typing import Optional

import torch

from . import _lib as L
from ._lib import (MASK_GEOMETRIC, MASK_NONE, MASK_REF_INTENDED, MASK_REF_QUIRK, PREC_COMPENSATED,  # noqa: F401
                   PREC_FAST, PREC_PLAIN, RECON_MASK_GEOMETRIC, RECON_MASK_NONE, RECON_MASK_REF, VARIANT_OPTIM,
                   VARIANT_PLAIN, VissError)

MOON_RADIUS_KM = 1737.4


def reference_d(res: int) -> int:
    """dl = dm = dn = 2*RES/(RES-1) in integer arithmetic (vissGen10M_shade.cu:183-185): 2."""
    return (2 * res) // (res - 1)


@dataclass(frozen=True)
class DftConfig:
    """One DFT pass.  Phase turns t = phase_scale * (u l + v m + w (n + n_offset))."""
    mask: int = MASK_NONE
    recon_mask: int = RECON_MASK_NONE
    precision: int = PREC_FAST
    res: int = 0
    trunc_brightness: bool = False
    occluded_value: float = 240.0
    phase_scale: float = 0.5
    n_offset: float = 0.0
    moon_radius_km: float = MOON_RADIUS_KM
    norm: Optional[float] = None  # recon scale; None -> 1/K as the reference

    @staticmethod
    def reference(res: int, variant: int = VARIANT_OPTIM, precision: int = PREC_FAST,
                  mask: int = MASK_REF_QUIRK) -> "DftConfig":
        """The reference's conventions: d = 2*RES/(RES-1) (int), REF windows, 240 inside
        the window, reference recon mask, F / K."""
        return DftConfig(mask=mask, recon_mask=RECON_MASK_REF, precision=precision, res=res,
                         trunc_brightness=variant == VARIANT_PLAIN, occluded_value=240.0,
                         phase_scale=1.0 / reference_d(res), n_offset=0.0)

    @staticmethod
    def north_star(precision: int = PREC_FAST, occluded_value: float = 0.0) -> "DftConfig":
        """V_k = sum_j I_j mask_kj exp(-2 pi i (u l + v m + w (n - 1))) with the geometric mask."""
        return DftConfig(mask=MASK_GEOMETRIC, recon_mask=RECON_MASK_GEOMETRIC, precision=precision, res=0,
                         occluded_value=occluded_value, phase_scale=1.0, n_offset=-1.0)

    def with_(self, **kw) -> "DftConfig":
        return replace(self, **kw)

    def c(self, K: int) -> L.DftCfg:
        norm = self.norm if self.norm is not None else (1.0 / K if K > 0 else 1.0)
        return L.DftCfg(int(self.mask), int(self.recon_mask), int(self.precision), int(self.res),
                        int(bool(self.trunc_brightness)), float(self.occluded_value), float(self.phase_scale),
                        float(self.n_offset), float(self.moon_radius_km), float(norm))


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else C.c_void_p(t.data_ptr())


def _dev(t: Optional[torch.Tensor], dtype, name: str, n: Optional[int] = None, cols: int = 0):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    t = t.contiguous()
    if n is not None:
        want = n * cols if cols else n
        if t.numel() != want:
            raise ValueError(f"{name} has {t.numel()} elements, expected {want}")
    return t


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _workspace(nbytes: int, device) -> Optional[torch.Tensor]:
    if nbytes == 0:
        return None
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def _geometry(sat_pos: Optional[torch.Tensor]):
    if sat_pos is None:
        return None, None
    sp = _dev(sat_pos, torch.float32, "sat_pos")
    if sp.dim() != 3 or sp.shape[2] != 3:
        raise ValueError("sat_pos must be [S, nsat, 3]")
    return sp, L.Geometry(sp.data_ptr(), sp.shape[0], sp.shape[1], 0)


def vis_dft(cfg: DftConfig, u, v, w, l, m, n, bright, shade=None, snap=None, pair=None, sat_pos=None,
            out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Shaded visibility DFT; returns complex64 V[K] (replaces visscal)."""
    K, J = u.numel(), l.numel()
    u, v, w = (_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    l, m, n, bright = (_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n"), (bright, "bright")))
    shade = _dev(shade, torch.int32, "shade", K, 4)
    snap = _dev(snap, torch.int32, "snap", K)
    pair = _dev(pair, torch.int32, "pair", K)
    sp, geo = _geometry(sat_pos)
    if out is None:
        out = torch.empty(K, dtype=torch.complex64, device=u.device)
    c = cfg.c(K)
    ws_bytes = L.lib.viss_vis_dft_workspace(C.byref(c), K, J, C.byref(geo) if geo else None)
    ws = _workspace(ws_bytes, u.device)
    sky = L.Sky(l.data_ptr(), m.data_ptr(), n.data_ptr(), bright.data_ptr(), J)
    vs = L.VisSet(u.data_ptr(), v.data_ptr(), w.data_ptr(), None, _ptr(shade), _ptr(snap), _ptr(pair), K)
    L.check(L.lib.viss_vis_dft(C.byref(c), C.byref(sky), C.byref(vs), C.byref(geo) if geo else None,
                               C.c_void_p(out.data_ptr()), _ptr(ws), ws_bytes, _stream()), "viss_vis_dft")
    return out


def recon(cfg: DftConfig, u, v, w, V, l, m, n, wgt=None, shade=None, snap=None, pair=None, sat_pos=None,
          out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Direct-DFT reconstruction; returns complex64 F[J] (replaces imagerecon)."""
    K, J = u.numel(), l.numel()
    u, v, w = (_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    V = _dev(V, torch.complex64, "V", K)
    l, m, n = (_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n")))
    wgt = _dev(wgt, torch.float32, "wgt", K)
    shade = _dev(shade, torch.int32, "shade", K, 4)
    snap = _dev(snap, torch.int32, "snap", K)
    pair = _dev(pair, torch.int32, "pair", K)
    sp, geo = _geometry(sat_pos)
    if out is None:
        out = torch.empty(J, dtype=torch.complex64, device=u.device)
    c = cfg.c(K)
    ws_bytes = L.lib.viss_recon_workspace(C.byref(c), K, J, C.byref(geo) if geo else None)
    ws = _workspace(ws_bytes, u.device)
    sky = L.Sky(l.data_ptr(), m.data_ptr(), n.data_ptr(), None, J)
    vs = L.VisSet(u.data_ptr(), v.data_ptr(), w.data_ptr(), _ptr(wgt), _ptr(shade), _ptr(snap), _ptr(pair), K)
    L.check(L.lib.viss_recon(C.byref(c), C.byref(sky), C.byref(vs), C.byref(geo) if geo else None,
                             C.c_void_p(V.data_ptr()), C.c_void_p(out.data_ptr()), _ptr(ws), ws_bytes, _stream()),
            "viss_recon")
    return out


# ---------------------------------------------------------------- reference-shaped
def visscal(uvws_index: int, lmnC_index: int, res: int, FF, viss, u, v, w, l, m, n, shadeM1, shadeM2, shadeM3,
            shadeM4, NXq=None, countLoc=None, dl: float = 2.0, dm: float = 2.0, dn: float = 2.0,
            variant: int = VARIANT_OPTIM, mask: int = MASK_REF_QUIRK, precision: int = PREC_FAST):
    """visscal(...) with the reference's arguments (vissGen10M_shade.cu:108-116); writes viss
    (complex64[K]) in place.  NXq/countLoc None = identity fine->coarse map."""
    K, J = int(uvws_index), int(lmnC_index)
    args = [_dev(x, torch.float32, nm, J) for x, nm in ((FF, "FF"),)]
    viss = _dev(viss, torch.complex64, "viss", K)
    uu = [_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w"))]
    pix = [_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n"))]
    sh = [_dev(x, torch.int32, f"shadeM{i + 1}", K) for i, x in enumerate((shadeM1, shadeM2, shadeM3, shadeM4))]
    L.check(L.lib.viss_visscal(K, J, int(res), _ptr(args[0]), _ptr(viss), *map(_ptr, uu), *map(_ptr, pix),
                               *map(_ptr, sh), _ptr(NXq), _ptr(countLoc), float(dl), float(dm), float(dn),
                               int(variant), int(mask), int(precision), _stream()), "viss_visscal")
    return viss


def imagerecon(uvw_index: int, lmnC_index: int, res: int, F, viss, u, v, w, l, m, n, uvwFrequencyMap, thetaP0=None,
               phiP0=None, dtheta=None, dphi=None, dl: float = 2.0, dm: float = 2.0, dn: float = 2.0,
               precision: int = PREC_FAST):
    """imagerecon(...) with the reference's arguments (vissGen10M_shade.cu:149-154); writes F
    (complex64[J]) in place."""
    K, J = int(uvw_index), int(lmnC_index)
    F = _dev(F, torch.complex64, "F", J)
    viss = _dev(viss, torch.complex64, "viss", K)
    uu = [_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w"))]
    pix = [_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n"))]
    wg = _dev(uvwFrequencyMap, torch.float32, "uvwFrequencyMap", K)
    rat = [_dev(x, torch.float32, nm, K) for x, nm in ((thetaP0, "thetaP0"), (phiP0, "phiP0"), (dtheta, "dtheta"),
                                                      (dphi, "dphi"))]
    L.check(L.lib.viss_imagerecon(K, J, int(res), _ptr(F), _ptr(viss), *map(_ptr, uu), *map(_ptr, pix), _ptr(wg),
                                  *map(_ptr, rat), float(dl), float(dm), float(dn), int(precision), _stream()),
            "viss_imagerecon")
    return F


def recon_ratios(shade: torch.Tensor):
    """thetaP0 = dtheta = M1/M2, phiP0 = dphi = M3/M4 as float (vissGen10M_shade.cu:514-517)."""
    s = shade.view(-1, 4)
    return s[:, 0].float() / s[:, 1].float(), s[:, 2].float() / s[:, 3].float()


# ---------------------------------------------------------------- orbit + uvw
REF_R1 = (0.0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3)      # MIncline_generate_uvw_float.cu:29
REF_R2 = (0.0, 0.1e3, 0.445e3, 0.6e3, 0.91e3, 1.62e3, 3.53e3, 10e3)  # :30


@dataclass(frozen=True)
class OrbitConfig:
    nsat: int = 8
    orbit_res: int = 864000
    orbit_counts: int = 140
    index: int = 1
    a_km: float = 2038.14
    e: float = 0.0
    incl_deg: float = 30.0
    argp_deg: float = 0.0
    raan_step_deg: float = 0.08
    r1_m: tuple = REF_R1
    r2_m: tuple = REF_R2
    fp64: bool = False

    def c(self):
        import numpy as np
        r1 = np.ascontiguousarray(self.r1_m, dtype=np.float32)
        r2 = np.ascontiguousarray(self.r2_m, dtype=np.float32)
        if r1.size < self.nsat or r2.size < self.nsat:
            raise ValueError("r1_m / r2_m need nsat entries")
        cfg = L.OrbitCfg(self.nsat, self.orbit_res, self.orbit_counts, self.index, self.a_km, self.e, self.incl_deg,
                         self.argp_deg, self.raan_step_deg, r1.ctypes.data, r2.ctypes.data, int(self.fp64), 0)
        cfg._keep = (r1, r2)
        return cfg

    @property
    def snapshots(self) -> int:
        return self.orbit_counts * (self.orbit_res // 3)


def orbit_positions(cfg: OrbitConfig, device="cuda", want_f64: bool = False):
    """Satellite positions [S, nsat, 3] (km) at the windowed snapshots; with want_f64 also the
    double positions."""
    c = cfg.c()
    S = L.lib.viss_orbit_snapshots(C.byref(c))
    pos = torch.empty(S, cfg.nsat, 3, dtype=torch.float32, device=device)
    pos64 = torch.empty(S, cfg.nsat, 3, dtype=torch.float64, device=device) if want_f64 else None
    L.check(L.lib.viss_orbit_positions(C.byref(c), _ptr(pos), _ptr(pos64), _stream()), "viss_orbit_positions")
    return (pos, pos64) if want_f64 else pos


def baseline_uvw(pos: torch.Tensor, lambda_m: float, ordered: bool = True, rounding: bool = True,
                 pos64: Optional[torch.Tensor] = None):
    """uvw per (snapshot, pair), snapshot-major; returns u, v, w, snap, pair."""
    S, nsat = pos.shape[0], pos.shape[1]
    P = nsat * (nsat - 1) // (1 if ordered else 2)
    K = S * P
    dev = pos.device
    u, v, w = (torch.empty(K, dtype=torch.float32, device=dev) for _ in range(3))
    snap = torch.empty(K, dtype=torch.int32, device=dev)
    pair = torch.empty(K, dtype=torch.int32, device=dev)
    L.check(L.lib.viss_baseline_uvw(_ptr(pos.contiguous()), _ptr(pos64), S, nsat, int(ordered), float(lambda_m),
                                    int(rounding), _ptr(u), _ptr(v), _ptr(w), _ptr(snap), _ptr(pair), _stream()),
            "viss_baseline_uvw")
    return u, v, w, snap, pair


def dedup_uvw(u: torch.Tensor, v: torch.Tensor, w: torch.Tensor):
    """Sort + unique of integer-valued uvw (copies); returns (u, v, w) of the unique count."""
    u, v, w = (x.clone().contiguous() for x in (u, v, w))
    K = u.numel()
    nb = L.lib.viss_dedup_uvw_workspace(K)
    ws = _workspace(nb, u.device)
    cnt = C.c_int64(0)
    L.check(L.lib.viss_dedup_uvw(_ptr(u), _ptr(v), _ptr(w), K, C.byref(cnt), _ptr(ws), nb, _stream()),
            "viss_dedup_uvw")
    n = cnt.value
    return u[:n], v[:n], w[:n]


def shade_windows(u, v, w, RES: int, mean_r_km: float = 0.0):
    """Raw shadeM windows int32[K, 4] (1-based) and the mean radius used."""
    K = u.numel()
    out = torch.empty(K, 4, dtype=torch.int32, device=u.device)
    nb = L.lib.viss_shade_windows_workspace(K)
    ws = _workspace(nb, u.device)
    mr = C.c_double(0.0)
    L.check(L.lib.viss_shade_windows(_ptr(u.contiguous()), _ptr(v.contiguous()), _ptr(w.contiguous()), K, int(RES),
                                     float(mean_r_km), _ptr(out), C.byref(mr), _ptr(ws), nb, _stream()),
            "viss_shade_windows")
    return out, mr.value


def normalise_shade(raw: torch.Tensor) -> torch.Tensor:
    raw = _dev(raw, torch.int32, "raw").view(-1, 4)
    M = torch.empty_like(raw)
    L.check(L.lib.viss_normalise_shade(_ptr(raw), raw.shape[0], _ptr(M), _stream()), "viss_normalise_shade")
    return M
