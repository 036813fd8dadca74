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
                   PREC_F64_PHASE, PREC_FAST, PREC_PLAIN, RECON_MASK_GEOMETRIC, RECON_MASK_NONE, RECON_MASK_REF, VARIANT_OPTIM,
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
    def geometric(precision: int = PREC_FAST, occluded_value: float = 0.0) -> "DftConfig":
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


def _need(t, dtype, name: str, n: Optional[int] = None) -> torch.Tensor:
    """A required tensor argument: as _dev, and None is refused."""
    if t is None:
        raise TypeError(f"{name} is required")
    return _dev(t, dtype, name, n)


def _positions(pos: torch.Tensor, dtype=torch.float32, name: str = "pos") -> torch.Tensor:
    """Satellite positions [S, nsat, 3] on the GPU, contiguous."""
    pos = _need(pos, dtype, name)
    if pos.dim() != 3 or pos.shape[2] != 3:
        raise ValueError(f"{name} must be [S, nsat, 3], got {list(pos.shape)}")
    return pos


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


def vis_dft_windowed(cfg: DftConfig, u, v, w, l, m, n, bright, win_index, shade,
                     out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """vis_dft with a REF mask whose window tests win_index[j] for pixel j (the appro
    program's NX[j] - 1); returns complex64 V[K]."""
    K, J = u.numel(), l.numel()
    u, v, w = (_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    l, m, n, bright = (_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n"), (bright, "bright")))
    win_index = _dev(win_index, torch.int32, "win_index", J)
    shade = _dev(shade, torch.int32, "shade", K, 4)
    if out is None:
        out = torch.empty(K, dtype=torch.complex64, device=u.device)
    c = cfg.c(K)
    ws_bytes = L.lib.viss_vis_dft_windowed_workspace(C.byref(c), K, J)
    ws = _workspace(ws_bytes, u.device)
    sky = L.Sky(l.data_ptr(), m.data_ptr(), n.data_ptr(), bright.data_ptr(), J)
    vs = L.VisSet(u.data_ptr(), v.data_ptr(), w.data_ptr(), None, _ptr(shade), None, None, K)
    L.check(L.lib.viss_vis_dft_windowed(C.byref(c), C.byref(sky), _ptr(win_index), C.byref(vs),
                                        C.c_void_p(out.data_ptr()), _ptr(ws), ws_bytes, _stream()),
            "viss_vis_dft_windowed")
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


# ---------------------------------------------------------------- fine->coarse sky maps
def nxq(NX: torch.Tensor, J: int):
    """NX (1-based coarse pixel per fine pixel, float32[X]) -> (countLoc int32[J], NXq int32[X]):
    the fine pixels of every coarse pixel, ascending (computeLocCount / computeLocViss,
    vissGen1M_shade_optim1.cu:54-115)."""
    NX = _dev(NX, torch.float32, "NX")
    X = NX.numel()
    countLoc = torch.empty(int(J), dtype=torch.int32, device=NX.device)
    NXq = torch.empty(X, dtype=torch.int32, device=NX.device)
    nb = L.lib.viss_nxq_workspace(X, int(J))
    ws = _workspace(nb, NX.device)
    L.check(L.lib.viss_nxq(_ptr(NX), X, int(J), _ptr(countLoc), _ptr(NXq), _ptr(ws), nb, _stream()), "viss_nxq")
    return countLoc, NXq


def vis_dft_map(cfg: DftConfig, u, v, w, l, m, n, FF, NXq, countLoc, shade=None, snap=None, pair=None, sat_pos=None,
                out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Shaded visibility DFT over a fine->coarse map (visscal with NXq/countLoc,
    vissGen10M_shade.cu:120-136): coarse pixel j's brightness for row k is the mean of its
    fine pixels' FF, the occluded value inside k's REF window.  NXq float32 (the 10M files)
    or int32 (nxq())."""
    K, J = u.numel(), l.numel()
    u, v, w = (_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    l, m, n = (_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n")))
    FF = _dev(FF, torch.float32, "FF")
    if NXq.dtype not in (torch.float32, torch.int32):
        raise TypeError("NXq must be float32 or int32")
    NXq = _dev(NXq, NXq.dtype, "NXq")
    countLoc = _dev(countLoc, torch.int32, "countLoc", J)
    shade = _dev(shade, torch.int32, "shade", K, 4)
    snap = _dev(snap, torch.int32, "snap", K)
    pair = _dev(pair, torch.int32, "pair", K)
    sp, geo = _geometry(sat_pos)
    X = FF.numel()
    if NXq.numel() < X:
        raise ValueError("NXq needs an entry per fine pixel")
    fm = L.FineMap(FF.data_ptr(), NXq.data_ptr() if NXq.dtype == torch.float32 else None,
                   NXq.data_ptr() if NXq.dtype == torch.int32 else None, countLoc.data_ptr(), X)
    if out is None:
        out = torch.empty(K, dtype=torch.complex64, device=u.device)
    c = cfg.c(K)
    ws_bytes = L.lib.viss_vis_dft_map_workspace(C.byref(c), K, J, C.byref(fm), C.byref(geo) if geo else None)
    ws = _workspace(ws_bytes, u.device)
    sky = L.Sky(l.data_ptr(), m.data_ptr(), n.data_ptr(), None, J)
    vs = L.VisSet(u.data_ptr(), v.data_ptr(), w.data_ptr(), None, _ptr(shade), _ptr(snap), _ptr(pair), K)
    L.check(L.lib.viss_vis_dft_map(C.byref(c), C.byref(sky), C.byref(fm), C.byref(vs), C.byref(geo) if geo else None,
                                   C.c_void_p(out.data_ptr()), _ptr(ws), ws_bytes, _stream()), "viss_vis_dft_map")
    return out


# ---------------------------------------------------------------- batched channels
@dataclass(frozen=True)
class Tuning:
    """Launch choices of the persistent passes (viss_tuning); zeros are the defaults."""
    ctas_per_sm: int = 0
    vis_split: int = 0
    rec_items: int = 0
    tile: int = 0  # bit 0: vis sky tiles of 256 pixels (else 512); bit 1 / 3: recon row tiles of 128 / 256
    # rows (else 512, 1,024 with the geometric mask at FAST precision; bit 2 asks for that default)

    def c(self) -> L.Tuning:
        return L.Tuning(int(self.ctas_per_sm), int(self.vis_split), int(self.rec_items), int(self.tile))


class ChannelBatch:
    """Many frequency channels through one persistent vis launch and one persistent
    recon launch (viss_vis_dft_batch / viss_recon_batch).

    u, v, w (and snap, pair, wgt, shade) hold every channel's rows back to back;
    channel c owns rows [row_off[c], row_off[c+1]).  bright is [nch, J]: each
    channel's sky brightness.  Outputs: V complex64[K] and F complex64[nch, J],
    allocated once with the workspaces, so that a pass can be captured in a CUDA
    graph (:meth:`graph`) and replayed.  norm: per-channel recon scale, default
    1/K_c (the reference's F / amount)."""

    def __init__(self, cfg: DftConfig, u, v, w, row_off, l, m, n, bright, snap=None, pair=None, sat_pos=None,
                 wgt=None, shade=None, norm=None, tuning: Optional[Tuning] = None):
        import numpy as np
        self.K, self.J = u.numel(), l.numel()
        K, J = self.K, self.J
        ro = np.ascontiguousarray(np.asarray(row_off, dtype=np.int64))
        self.nch = ro.size - 1
        if not (1 <= self.nch <= L.MAX_CHANNELS) or ro[0] != 0 or ro[-1] != K or np.any(np.diff(ro) < 0):
            raise ValueError("row_off must be 0 = r_0 <= ... <= r_nch = K with 1 <= nch <= 64")
        self.row_off = ro
        kc = np.diff(ro)
        if norm is None:
            norm = [cfg.norm if cfg.norm is not None else (1.0 / k if k > 0 else 1.0) for k in kc]
        self.norm = np.ascontiguousarray(np.asarray(norm, dtype=np.float64))
        if self.norm.size != self.nch:
            raise ValueError("norm needs one value per channel")
        self.cfg = cfg
        self.u, self.v, self.w = (_dev(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
        self.l, self.m, self.n = (_dev(x, torch.float32, nm, J) for x, nm in ((l, "l"), (m, "m"), (n, "n")))
        self.bright = _dev(bright, torch.float32, "bright", self.nch * J)
        self.wgt = _dev(wgt, torch.float32, "wgt", K)
        self.shade = _dev(shade, torch.int32, "shade", K, 4)
        self.snap = _dev(snap, torch.int32, "snap", K)
        self.pair = _dev(pair, torch.int32, "pair", K)
        self.sp, self.geo = _geometry(sat_pos)
        dev = self.u.device
        self.V = torch.zeros(K, dtype=torch.complex64, device=dev)
        self.F = torch.zeros(self.nch, J, dtype=torch.complex64, device=dev)
        self._c = cfg.c(K)
        self._batch = L.Batch(self.nch, 0, self.row_off.ctypes.data_as(C.POINTER(C.c_int64)), self.bright.data_ptr(),
                              self.norm.ctypes.data_as(C.POINTER(C.c_double)))
        self._sky = L.Sky(self.l.data_ptr(), self.m.data_ptr(), self.n.data_ptr(), None, J)
        self._vs = L.VisSet(self.u.data_ptr(), self.v.data_ptr(), self.w.data_ptr(), _ptr(self.wgt), _ptr(self.shade),
                            _ptr(self.snap), _ptr(self.pair), K)
        self.set_tuning(tuning or Tuning())

    def _geo(self):
        return C.byref(self.geo) if self.geo else None

    def set_tuning(self, tuning: Tuning) -> None:
        """Choose launch parameters and (re)size the workspaces for them."""
        self.tuning = tuning
        self._t = tuning.c()
        self._vis_ws_bytes = L.lib.viss_vis_dft_batch_workspace(C.byref(self._c), C.byref(self._batch), self.K, self.J,
                                                                self._geo(), C.byref(self._t))
        self._rec_ws_bytes = L.lib.viss_recon_batch_workspace(C.byref(self._c), C.byref(self._batch), self.K, self.J,
                                                              self._geo(), C.byref(self._t))
        # one buffer serves both passes (they run in order on one stream)
        self._ws = _workspace(max(self._vis_ws_bytes, self._rec_ws_bytes), self.u.device)

    def vis(self) -> torch.Tensor:
        """Enqueue the batched vis DFT on the current stream; returns V."""
        self._sky.bright = None
        L.check(L.lib.viss_vis_dft_batch(C.byref(self._c), C.byref(self._sky), C.byref(self._vs), C.byref(self._batch),
                                         self._geo(), C.byref(self._t), C.c_void_p(self.V.data_ptr()), _ptr(self._ws),
                                         self._vis_ws_bytes, _stream()), "viss_vis_dft_batch")
        return self.V

    def recon(self, V: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Enqueue the batched reconstruction of V (default: this batch's V); returns F [nch, J]."""
        V = self.V if V is None else _dev(V, torch.complex64, "V", self.K)
        L.check(L.lib.viss_recon_batch(C.byref(self._c), C.byref(self._sky), C.byref(self._vs), C.byref(self._batch),
                                       self._geo(), C.byref(self._t), C.c_void_p(V.data_ptr()),
                                       C.c_void_p(self.F.data_ptr()), _ptr(self._ws), self._rec_ws_bytes, _stream()),
                "viss_recon_batch")
        return self.F

    def step(self):
        """vis then recon of every channel."""
        self.vis()
        return self.recon()

    def graph(self) -> "torch.cuda.CUDAGraph":
        """Capture :meth:`step` in a CUDA graph (after one eager warm-up run); replay() re-runs the
        whole batched pass with one launch call."""
        s = torch.cuda.Stream(device=self.u.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.step()
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
        return g


def tuning_candidates() -> list:
    """Launch choices the autotuner times: tile shapes (sky tile of the vis kernel, row tile
    of the recon kernel), persistent CTAs per SM, recon items per CTA, sky split."""
    out = []
    for tile in (0, 1, 2, 3, 8, 9):
        for items in (16, 32):
            out.append(Tuning(tile=tile, rec_items=items))
    out.append(Tuning(rec_items=8))
    out.append(Tuning(rec_items=64))
    out.append(Tuning(ctas_per_sm=2))
    out.append(Tuning(vis_split=1))
    out.append(Tuning(vis_split=2))
    return out


_TUNED: dict = {}


def autotune(batch: ChannelBatch, candidates=None, reps: int = 1, use_cache: bool = True) -> Tuning:
    """Time vis + recon of ``batch`` under each candidate Tuning (CUDA events on the current
    stream, after one warm-up run each) and keep the fastest on the batch.  Results are cached
    per device and batch shape (channel row counts, J, mask and precision)."""
    key = (torch.cuda.get_device_name(batch.u.device), tuple(batch.row_off.tolist()), batch.J, batch.cfg.mask,
           batch.cfg.recon_mask, batch.cfg.precision)
    if use_cache and key in _TUNED:
        batch.set_tuning(_TUNED[key][0])
        return _TUNED[key][0]
    cands = list(candidates) if candidates is not None else tuning_candidates()
    times = []
    for t in cands:
        batch.set_tuning(t)
        batch.step()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            batch.step()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / reps)
    best = cands[min(range(len(cands)), key=times.__getitem__)]
    _TUNED[key] = (best, list(zip(cands, times)))
    batch.set_tuning(best)
    return best


def autotune_report(batch: ChannelBatch):
    """(tuning, ms) pairs of the last autotune of this batch shape, or None."""
    key = (torch.cuda.get_device_name(batch.u.device), tuple(batch.row_off.tolist()), batch.J, batch.cfg.mask,
           batch.cfg.recon_mask, batch.cfg.precision)
    return _TUNED.get(key, (None, None))[1]


# ---------------------------------------------------------------- reference-shaped
def visscal(uvws_index: int, lmnC_index: int, res: int, FF, viss, u, v, w, l, m, n, shadeM1, shadeM2, shadeM3,
            shadeM4, NXq=None, countLoc=None, dl: float = 2.0, dm: float = 2.0, dn: float = 2.0,
            variant: int = VARIANT_OPTIM, mask: int = MASK_REF_QUIRK, precision: int = PREC_FAST):
    """visscal(...) with the reference's arguments (vissGen10M_shade.cu:108-116); writes viss
    (complex64[K]) in place.  NXq/countLoc None = identity fine->coarse map; else NXq float32
    (as the 10M files) and countLoc int32[J], with FF the fine brightness."""
    K, J = int(uvws_index), int(lmnC_index)
    # FF: J coarse values for the identity map, else the fine grid
    args = [_dev(FF, torch.float32, "FF", J if NXq is None else None)]
    NXq = _dev(NXq, torch.float32, "NXq")
    countLoc = _dev(countLoc, torch.int32, "countLoc", J)
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
from .synth import REF_R1, REF_R2  # noqa: E402  (MIncline_generate_uvw_float.cu:29-30)


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
    if torch.device(device).type != "cuda":
        raise TypeError("orbit_positions computes on a CUDA device")
    c = cfg.c()
    S = L.lib.viss_orbit_snapshots(C.byref(c))
    pos = torch.empty(S, cfg.nsat, 3, dtype=torch.float32, device=device)
    pos64 = torch.empty(S, cfg.nsat, 3, dtype=torch.float64, device=device) if want_f64 else None
    L.check(L.lib.viss_orbit_positions(C.byref(c), _ptr(pos), _ptr(pos64), _stream()), "viss_orbit_positions")
    return (pos, pos64) if want_f64 else pos


def baseline_uvw(pos: torch.Tensor, lambda_m: float, ordered: bool = True, rounding: bool = True,
                 pos64: Optional[torch.Tensor] = None):
    """uvw per (snapshot, pair), snapshot-major; returns u, v, w, snap, pair."""
    pos = _positions(pos)
    pos64 = None if pos64 is None else _positions(pos64, torch.float64, "pos64")
    if pos64 is not None and pos64.shape != pos.shape:
        raise ValueError("pos64 must have the shape of pos")
    S, nsat = pos.shape[0], pos.shape[1]
    P = nsat * (nsat - 1) // (1 if ordered else 2)
    K = S * P
    dev = pos.device
    u, v, w = (torch.empty(K, dtype=torch.float32, device=dev) for _ in range(3))
    snap = torch.empty(K, dtype=torch.int32, device=dev)
    pair = torch.empty(K, dtype=torch.int32, device=dev)
    L.check(L.lib.viss_baseline_uvw(_ptr(pos), _ptr(pos64), S, nsat, int(ordered), float(lambda_m),
                                    int(rounding), _ptr(u), _ptr(v), _ptr(w), _ptr(snap), _ptr(pair), _stream()),
            "viss_baseline_uvw")
    return u, v, w, snap, pair


def dedup_uvw(u: torch.Tensor, v: torch.Tensor, w: torch.Tensor):
    """Sort + unique of integer-valued uvw (copies); returns (u, v, w) of the unique count."""
    K = u.numel() if isinstance(u, torch.Tensor) else 0
    u, v, w = (_need(x, torch.float32, nm, K).clone() for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    nb = L.lib.viss_dedup_uvw_workspace(K)
    ws = _workspace(nb, u.device)
    cnt = C.c_int64(0)
    L.check(L.lib.viss_dedup_uvw(_ptr(u), _ptr(v), _ptr(w), K, C.byref(cnt), _ptr(ws), nb, _stream()),
            "viss_dedup_uvw")
    n = cnt.value
    return u[:n], v[:n], w[:n]


def unique_uvw(pos: torch.Tensor, lambda_m: float, ordered: bool = True, capacity: int = 1 << 22):
    """baseline_uvw (ceil) + dedup_uvw fused: the unique uvw rows of all (snapshot, pair)
    baselines of float positions [S, nsat, 3], sorted, with the values of each key's first
    occurrence in pair-major order (the reference's concatenation of per-pair lists).  Starts
    with room for `capacity` rows and repeats the pass once with the exact count if that
    is short."""
    pos = _positions(pos)
    S, nsat = pos.shape[0], pos.shape[1]
    nb = L.lib.viss_unique_uvw_workspace(S, nsat, int(ordered))
    ws = _workspace(nb, pos.device)
    cnt = C.c_int64(0)
    for _ in range(2):
        u, v, w = (torch.empty(max(capacity, 1), dtype=torch.float32, device=pos.device) for _ in range(3))
        rc = L.lib.viss_unique_uvw(_ptr(pos), S, nsat, int(ordered), float(lambda_m), _ptr(u), _ptr(v), _ptr(w),
                                   capacity, C.byref(cnt), _ptr(ws), nb, _stream())
        if rc == L.VISS_ERR_RANGE and cnt.value > capacity:
            capacity = cnt.value
            continue
        L.check(rc, "viss_unique_uvw")
        n = cnt.value
        return u[:n], v[:n], w[:n]
    raise RuntimeError("viss_unique_uvw: unique count changed between passes")


def shade_windows(u, v, w, RES: int, mean_r_km: float = 0.0):
    """Raw shadeM windows int32[K, 4] (1-based) and the mean radius used."""
    K = u.numel() if isinstance(u, torch.Tensor) else 0
    u, v, w = (_need(x, torch.float32, nm, K) for x, nm in ((u, "u"), (v, "v"), (w, "w")))
    out = torch.empty(K, 4, dtype=torch.int32, device=u.device)
    nb = L.lib.viss_shade_windows_workspace(K)
    ws = _workspace(nb, u.device)
    mr = C.c_double(0.0)
    L.check(L.lib.viss_shade_windows(_ptr(u), _ptr(v), _ptr(w), K, int(RES),
                                     float(mean_r_km), _ptr(out), C.byref(mr), _ptr(ws), nb, _stream()),
            "viss_shade_windows")
    return out, mr.value


def normalise_shade(raw: torch.Tensor) -> torch.Tensor:
    raw = _dev(raw, torch.int32, "raw").view(-1, 4)
    M = torch.empty_like(raw)
    L.check(L.lib.viss_normalise_shade(_ptr(raw), raw.shape[0], _ptr(M), _stream()), "viss_normalise_shade")
    return M
