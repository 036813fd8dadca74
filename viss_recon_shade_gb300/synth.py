"""Seeded synthetic inputs with the shapes of the simulator's workloads.

The reference reads MATLAB-generated sky and uvw files that are not part of
it; these generators stand in for them: Fibonacci-sphere pixels, log-normal or
power-law diffuse skies with point sources deposited on the nearest pixel,
and lunar orbits driven through the product's own orbit/uvw kernels.

Everything above make_orbit_cfg needs numpy only (the module also loads on its
own, by path, without the product library).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

MOON_R = 1737.4
# along-track separation ramps of the reference's 8 satellites, r1 -> r2 -> r1 (m)
REF_R1 = (0.0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3)      # MIncline_generate_uvw_float.cu:29
REF_R2 = (0.0, 0.1e3, 0.445e3, 0.6e3, 0.91e3, 1.62e3, 3.53e3, 10e3)  # :30


def fibonacci_sphere(J: int):
    """J unit vectors (l, m, n) on a Fibonacci spiral, float32."""
    i = np.arange(J, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / J
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.pi * (3.0 - np.sqrt(5.0)) * i
    return (r * np.cos(phi)).astype(np.float32), (r * np.sin(phi)).astype(np.float32), z.astype(np.float32)


def lognormal_sky(J: int, seed: int = 0, sigma: float = 1.0, n_points: int = 20):
    rng = np.random.default_rng(seed)
    b = rng.lognormal(0.0, sigma, J)
    idx = rng.choice(J, n_points, replace=False)
    b[idx] += rng.uniform(20.0, 200.0, n_points)
    return b.astype(np.float32)


def powerlaw_sky(n: np.ndarray, freq_mhz: float, seed: int = 0, n_points: int = 500, index: float = -2.5):
    """Smooth (1 + cos theta)^2 field (theta from +z) with spectral index `index`
    relative to 1 MHz, plus point sources."""
    rng = np.random.default_rng(seed)
    J = n.size
    b = (1.0 + n.astype(np.float64)) ** 2 * 100.0 * freq_mhz ** index
    idx = rng.choice(J, n_points, replace=False)
    b[idx] += rng.uniform(5.0, 50.0, n_points) * b.mean()
    return b.astype(np.float32)


def log_separations(nsat: int, dmax_m: float = 100e3):
    """Along-track separation ramps for nsat satellites, 0 .. dmax (r1) and dmax/10 (r2),
    log-spaced like the reference's 8 (MIncline_generate_uvw_float.cu:29-30)."""
    if nsat == 8:
        return tuple(REF_R1), tuple(REF_R2)
    r1 = np.concatenate([[0.0], np.geomspace(1e3, dmax_m, nsat - 1)])
    return tuple(float(x) for x in r1), tuple(float(x) / 10.0 for x in r1)


@dataclass(frozen=True)
class Workload:
    name: str
    nsat: int
    orbit_res: int
    orbit_counts: int
    freq_hz: float
    J: int
    sky: str           # "lognormal" | "powerlaw"
    n_points: int
    a_km: float = MOON_R + 300.0
    incl_deg: float = 30.0
    ordered: bool = False
    rounding: bool = False

    @property
    def lambda_m(self) -> float:
        return 3e8 / self.freq_hz

    @property
    def snapshots(self) -> int:
        return self.orbit_counts * (self.orbit_res // 3)

    @property
    def npairs(self) -> int:
        return self.nsat * (self.nsat - 1) // (1 if self.ordered else 2)

    @property
    def K(self) -> int:
        return self.snapshots * self.npairs


# The simulator's configurations (1 MHz small; 10 MHz inclined; differentiable
# 10 MHz; 30 MHz with 16 satellites).  orbit_res/orbit_counts are chosen so that
# counts * res/3 gives the snapshot counts.
WORKLOADS = {
    "cfg1_1MHz": Workload("cfg1_1MHz", 8, 768, 4, 1e6, 12288, "lognormal", 20),
    "cfg2_10MHz": Workload("cfg2_10MHz", 8, 12288, 16, 1e7, 196608, "powerlaw", 500),
    "cfg4_10MHz": Workload("cfg4_10MHz", 8, 3072, 16, 1e7, 49152, "lognormal", 20),
    "cfg5_30MHz": Workload("cfg5_30MHz", 16, 12288, 16, 3e7, 786432, "powerlaw", 5000),
}


def make_sky(wl: Workload, seed: int = 0):
    l, m, n = fibonacci_sphere(wl.J)
    if wl.sky == "lognormal":
        b = lognormal_sky(wl.J, seed=seed, n_points=wl.n_points)
    else:
        b = powerlaw_sky(n, wl.freq_hz / 1e6, seed=seed, n_points=wl.n_points)
    return l, m, n, b


def make_orbit_cfg(wl: Workload, fp64: bool = True):
    from .api import OrbitConfig
    r1, r2 = log_separations(wl.nsat)
    return OrbitConfig(nsat=wl.nsat, orbit_res=wl.orbit_res, orbit_counts=wl.orbit_counts, index=1, a_km=wl.a_km,
                       incl_deg=wl.incl_deg, r1_m=r1, r2_m=r2, fp64=fp64)


def make_uvw(wl: Workload, device="cuda"):
    """Positions and uvw on the GPU through the product kernels.  Continuous
    uvw come from FP64 positions; reference-compatible (ceil) uvw from the FP32
    arithmetic.  Returns dict of device tensors."""
    from .api import baseline_uvw, orbit_positions
    cfg = make_orbit_cfg(wl, fp64=not wl.rounding)
    if wl.rounding:
        pos = orbit_positions(cfg, device=device)
        u, v, w, snap, pair = baseline_uvw(pos, wl.lambda_m, ordered=wl.ordered, rounding=True)
    else:
        pos, pos64 = orbit_positions(cfg, device=device, want_f64=True)
        u, v, w, snap, pair = baseline_uvw(pos, wl.lambda_m, ordered=wl.ordered, rounding=False, pos64=pos64)
    return dict(u=u, v=v, w=w, snap=snap, pair=pair, sat_pos=pos)


@dataclass(frozen=True)
class BatchWorkload:
    """Many frequency channels in one pass: nch channels log-spaced over
    [fmin, fmax], each with its own snapshot count (uniform in [smin, smax],
    multiples of 16, at least 128, seeded) and orbit phase (the period index, which moves the
    orbit's node and window start), and a power-law brightness per channel."""
    name: str = "batch64"
    nch: int = 64
    fmin_hz: float = 1e6
    fmax_hz: float = 30e6
    smin: int = 4096
    smax: int = 65536
    J: int = 49152
    nsat: int = 8
    n_points: int = 500
    seed: int = 0
    a_km: float = MOON_R + 300.0
    incl_deg: float = 30.0

    def freqs(self) -> np.ndarray:
        return np.geomspace(self.fmin_hz, self.fmax_hz, self.nch)

    def snapshots(self) -> np.ndarray:
        rng = np.random.default_rng(self.seed)
        return rng.integers(self.smin // 16, self.smax // 16 + 1, self.nch) * 16

    @property
    def npairs(self) -> int:
        return self.nsat * (self.nsat - 1) // 2


BATCH_WORKLOADS = {
    "batch64": BatchWorkload(),
    "batch5_small": BatchWorkload(name="batch5_small", nch=5, smin=128, smax=512, J=12288, n_points=20),
}


def make_batch(bw: BatchWorkload, device="cuda"):
    """Rows of every channel back to back (uvw, snap into one satellite-position
    array, pair), row offsets, per-channel brightness [nch, J] and the sky."""
    import torch

    from .api import OrbitConfig, baseline_uvw, orbit_positions
    l, m, n = fibonacci_sphere(bw.J)
    r1, r2 = log_separations(bw.nsat)
    us, vs, ws, snaps, pairs, poss = [], [], [], [], [], []
    row_off = [0]
    s_off = 0
    bright = np.empty((bw.nch, bw.J), dtype=np.float32)
    for c, (f, S) in enumerate(zip(bw.freqs(), bw.snapshots())):
        counts = 16 if 3 * int(S) // 16 >= 360 else 1  # the orbit kernel wants >= 360 samples per orbit
        cfg = OrbitConfig(nsat=bw.nsat, orbit_res=3 * int(S) // counts, orbit_counts=counts, index=1 + c,
                          a_km=bw.a_km, incl_deg=bw.incl_deg, r1_m=r1, r2_m=r2, fp64=True)
        pos, pos64 = orbit_positions(cfg, device=device, want_f64=True)
        u, v, w, snap, pair = baseline_uvw(pos, 3e8 / f, ordered=False, rounding=False, pos64=pos64)
        us.append(u); vs.append(v); ws.append(w); pairs.append(pair); poss.append(pos)
        snaps.append(snap + s_off)
        s_off += pos.shape[0]
        row_off.append(row_off[-1] + u.numel())
        bright[c] = powerlaw_sky(n, f / 1e6, seed=bw.seed, n_points=bw.n_points)
    cat = torch.cat
    return dict(u=cat(us), v=cat(vs), w=cat(ws), snap=cat(snaps), pair=cat(pairs), sat_pos=cat(poss),
                row_off=np.asarray(row_off, dtype=np.int64), bright=torch.from_numpy(bright).to(device),
                l=l, m=m, n=n, freqs=bw.freqs())
