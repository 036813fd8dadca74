"""Run the reference's own CUDA kernels (built by oracle/build_ref.sh) on a GPU.

TEST INFRASTRUCTURE ONLY (the checker and the reference arm of the bench).
The device images in oracle/_ref/ are compiled, unmodified, from the reference
sources; this module replaces only the reference's host code: it loads the
image through the CUDA driver API, looks kernels up by name and launches them
with the argument lists of the reference's own launch sites.  Device memory
comes from torch tensors (torch owns the primary context).

Kernel argument lists (reference file:line):
  vissGen10M_shade.cu:108-116    visscal(int K, int J, int res, float* FF, Complex* viss,
                                 float* u,v,w, float* l,m,n, int* shadeM1..4, float* NXq,
                                 int* countLoc, Complex I1, CPI, zero, two, float dl, dm, dn)
  vissGen10M_shade.cu:149-154    imagerecon(int K, int J, int res, Complex* F, Complex* viss,
                                 float* u,v,w, float* l,m,n, float* uvwFrequencyMap,
                                 float* thetaP0, phiP0, dtheta, dphi, Complex I1, CPI, zero,
                                 two, float dl, dm, dn)
  MIncline_generate_uvw_float.cu:83,113,153   calculateOrbit / uvwPosition / computeUVW
  shade1M.cu:63,74               Cart2SphKernel / ShadeMatrix
  vissGen1M_shade_optim1.cu:54,82  computeLocCount / computeLocViss
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

REF_DIR = Path(__file__).resolve().parent / "_ref"

_cuda = None


def _drv():
    global _cuda
    if _cuda is None:
        _cuda = C.CDLL("libcuda.so.1")
    return _cuda


def _check(rc, what):
    if rc != 0:
        msg = C.c_char_p()
        _drv().cuGetErrorString(rc, C.byref(msg))
        raise RuntimeError(f"{what} failed: {rc} {msg.value.decode() if msg.value else ''}")


def available() -> bool:
    return (REF_DIR / "vissGen10M_shade.cubin").exists()


class RefModule:
    """A reference device image with its kernels indexed by source name."""

    def __init__(self, name: str):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make torch's primary context current on this thread
        d = _drv()
        _check(d.cuInit(0), "cuInit")
        self.mod = C.c_void_p()
        cubin = REF_DIR / f"{name}.cubin"
        _check(d.cuModuleLoad(C.byref(self.mod), str(cubin).encode()), f"cuModuleLoad({name})")
        cnt = C.c_uint()
        _check(d.cuModuleGetFunctionCount(C.byref(cnt), self.mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * cnt.value)()
        _check(d.cuModuleEnumerateFunctions(funcs, cnt, self.mod), "cuModuleEnumerateFunctions")
        self.funcs = {}
        for f in funcs:
            nm = C.c_char_p()
            _check(d.cuFuncGetName(C.byref(nm), C.c_void_p(f)), "cuFuncGetName")
            mangled = nm.value.decode()
            m = re.match(r"_Z(\d+)", mangled)
            base = mangled[m.end():m.end() + int(m.group(1))] if m else mangled
            # free __global__ functions only (thrust's kernels live in namespaces: _ZN...)
            if m and base not in self.funcs:
                self.funcs[base] = C.c_void_p(f)

    def kernel(self, name: str):
        return self.funcs[name]

    def occupancy_block(self, name: str) -> int:
        """Block size the reference picks with cudaOccupancyMaxPotentialBlockSize(f, 0, 0)."""
        mg, bs = C.c_int(), C.c_int()
        _check(_drv().cuOccupancyMaxPotentialBlockSize(C.byref(mg), C.byref(bs), self.funcs[name], None,
                                                       C.c_size_t(0), C.c_int(0)),
               "cuOccupancyMaxPotentialBlockSize")
        return bs.value

    def launch(self, name: str, grid: int, block: int, args, shmem: int = 0, stream: int = 0):
        """args: list of ctypes scalars / arrays (device pointers as c_void_p)."""
        ptrs = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        _check(_drv().cuLaunchKernel(self.funcs[name], C.c_uint(grid), C.c_uint(1), C.c_uint(1),
                                     C.c_uint(block), C.c_uint(1), C.c_uint(1), C.c_uint(shmem),
                                     C.c_void_p(stream), ptrs, None), f"cuLaunchKernel({name})")


def ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def cplx(re_: float, im_: float):
    """thrust::complex<float> passed by value (8 bytes)."""
    return (C.c_float * 2)(re_, im_)


def i32(x):
    return C.c_int(int(x))


def f32(x):
    return C.c_float(float(x))


_MODS: dict[str, RefModule] = {}


def module(name: str) -> RefModule:
    if name not in _MODS:
        _MODS[name] = RefModule(name)
    return _MODS[name]


# ---------------------------------------------------------------------------
# Reference launch sequences (host logic restated from the reference mains)
# ---------------------------------------------------------------------------

def visscal(variant: str, K, J, res, FF, u, v, w, l, m, n, M1, M2, M3, M4, NXq, countLoc, d=2.0,
            block=None, stream=0):
    """Reference visscal of `variant` (e.g. 'vissGen10M_shade'); returns complex64 viss[K].
    NXq is float32 for the 10M files and int32 for the 1M files (as in the reference)."""
    import torch
    mod = module(variant)
    viss = torch.zeros(K, 2, dtype=torch.float32, device="cuda")
    bs = block or mod.occupancy_block("visscal")
    grid = (K + bs - 1) // bs
    args = [i32(K), i32(J), i32(res), ptr(FF), ptr(viss), ptr(u), ptr(v), ptr(w), ptr(l), ptr(m),
            ptr(n), ptr(M1), ptr(M2), ptr(M3), ptr(M4), ptr(NXq), ptr(countLoc),
            cplx(0, 1), cplx(3.14159265358979, 0), cplx(0, 0), cplx(2, 0), f32(d), f32(d), f32(d)]
    mod.launch("visscal", grid, bs, args, stream=stream)
    return viss


def recon_ratios(M1, M2, M3, M4):
    """thetaP0 = dtheta = M1/M2 and phiP0 = dphi = M3/M4 as float (vissGen10M_shade.cu:514-517)."""
    r1 = M1.float() / M2.float()
    r2 = M3.float() / M4.float()
    return r1, r2


def imagerecon(variant: str, K, J, res, viss, u, v, w, l, m, n, wgt, M1, M2, M3, M4, d=2.0,
               block=None, stream=0):
    import torch
    mod = module(variant)
    F = torch.zeros(J, 2, dtype=torch.float32, device="cuda")
    r1, r2 = recon_ratios(M1, M2, M3, M4)
    if variant.endswith("optim2"):
        # launch_imagerecon (vissGen10M_shade_optim2.cu:320-389): block from the
        # occupancy of visscal, dynamic smem argument, static 128-entry tiles.
        bs = block or mod.occupancy_block("visscal")
        shmem = 128 * (4 * 8 + 8)
        # its threads past J return before __syncthreads (:257 vs :294) and
        # leave their share of the tile unloaded: only whole blocks are run.
        if J % bs:
            raise ValueError(f"optim2 imagerecon needs J % {bs} == 0")
    else:
        bs = block or mod.occupancy_block("imagerecon")
        shmem = 0
    grid = (J + bs - 1) // bs
    args = [i32(K), i32(J), i32(res), ptr(F), ptr(viss), ptr(u), ptr(v), ptr(w), ptr(l), ptr(m),
            ptr(n), ptr(wgt), ptr(r1), ptr(r2), ptr(r1), ptr(r2),
            cplx(0, 1), cplx(3.14159265358979, 0), cplx(0, 0), cplx(2, 0), f32(d), f32(d), f32(d)]
    mod.launch("imagerecon", grid, bs, args, shmem=shmem, stream=stream)
    return F


def mincline_unique(nsat, orbit_res, orbit_counts, index, frequency, r1, r2, a=2038.14, e=0.0, incl_deg=30.0,
                    argp_deg=0.0, mu=4.902793455e3, timed=False):
    """The reference's whole uvw stage (MIncline_generate_uvw_float.cu:215-397): its
    calculateOrbit / uvwPosition kernels per satellite, then per ordered pair its
    computeUVW kernel followed by thrust::sort + thrust::unique (restated in
    oracle/ref_thrust.cu) and the append to a global list, which is sorted and
    uniqued at the end.  Returns the unique rows [n, 3] (float32, CUDA) and, with
    timed=True, a dict of CUDA-event milliseconds {positions, pairs, global, total}."""
    import torch
    from oracle import ref_thrust
    ref_thrust.lib()  # load (and build) before the timed region
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    st = torch.cuda.current_stream()
    ev[0].record(st)
    mod, (xt, yt, zt), S, nblk, bs3, lam = _positions(nsat, orbit_res, orbit_counts, index, frequency, r1, r2, a, e,
                                                      incl_deg, argp_deg, mu)
    ev[1].record(st)
    hash_ = torch.zeros(nblk * bs3, 3, dtype=torch.float32, device="cuda")
    parts = []
    for mm in range(nsat):
        for nn in range(nsat):
            if mm == nn:
                continue
            mod.launch("computeUVW", nblk, bs3, [ptr(xt), ptr(yt), ptr(zt), ptr(hash_), i32(orbit_counts),
                                                 i32(orbit_res), f32(lam), i32(mm), i32(nn)])
            rows = hash_[:S]
            parts.append(rows[:ref_thrust.sort_unique(rows)].clone())
    glob = torch.cat(parts)
    del parts
    ev[2].record(st)
    glob = glob[:ref_thrust.sort_unique(glob)]
    ev[3].record(st)
    torch.cuda.synchronize()
    if not timed:
        return glob
    ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(3)]
    return glob, {"positions": ms[0], "pairs": ms[1], "global": ms[2], "total": sum(ms)}


def _positions(nsat, orbit_res, orbit_counts, index, frequency, r1, r2, a, e, incl_deg, argp_deg, mu):
    """calculateOrbit + uvwPosition per satellite (MIncline_generate_uvw_float.cu:215-330):
    windowed positions xt, yt, zt [nsat * S (+ a block of padding)]."""
    import math
    import numpy as np
    import torch
    mod = module("MIncline_generate_uvw_float")
    N = orbit_res * orbit_counts
    interval = orbit_res // 360 * 10
    span = orbit_res // 3
    lam = int(3e8 / frequency)
    fl = lambda x: float(np.float32(x))  # noqa: E731
    d2r = fl(math.pi / 180)
    # one satellite of zeros beyond the last: uvwPosition reads one element past it
    x = torch.zeros(N * (nsat + 1), dtype=torch.float32, device="cuda")
    y = torch.zeros_like(x)
    z = torch.zeros_like(x)
    S = N // 3
    bs3 = mod.occupancy_block("computeUVW")
    xt = torch.zeros(S * nsat + bs3, dtype=torch.float32, device="cuda")
    yt = torch.zeros_like(xt)
    zt = torch.zeros_like(xt)
    step = fl(fl(2 * math.pi) / fl(orbit_res - 1))
    seq = np.arange(orbit_res, dtype=np.float32).astype(np.float64)
    Mt = torch.from_numpy((step * seq).astype(np.float32)).cuda()
    for ss in range(nsat):
        h = N // 2
        s1 = fl(fl(fl(r2[ss]) - fl(r1[ss])) / fl(h - 1))
        s2 = fl(fl(fl(r1[ss]) - fl(r2[ss])) / fl(h - 1))
        sq = np.arange(h, dtype=np.float32).astype(np.float64)  # thrust::sequence into a float vector
        d1 = (s1 * sq + fl(r1[ss])).astype(np.float32)
        d2 = (s2 * sq + fl(r2[ss])).astype(np.float32)
        dd = np.concatenate([d1, d2]).astype(np.float64)
        dM = torch.from_numpy((np.arcsin(dd / (fl(2 * fl(a)) * 1e3)) * 2).astype(np.float32)).cuda()
        bs = mod.occupancy_block("calculateOrbit")
        args = [ptr(dM), ptr(x), ptr(y), ptr(z), ptr(Mt), i32(orbit_counts), i32(orbit_res), f32(d2r),
                f32(e), f32(a), f32(mu), f32(fl(argp_deg) * d2r), f32(fl(incl_deg) * d2r), i32(index), i32(ss)]
        mod.launch("calculateOrbit", (N + bs - 1) // bs, bs, args)
        bs2 = mod.occupancy_block("uvwPosition")
        args = [ptr(x), ptr(y), ptr(z), ptr(xt), ptr(yt), ptr(zt), i32(orbit_counts), i32(orbit_res),
                i32(interval), i32(span), i32(ss)]
        mod.launch("uvwPosition", (N // 3 + bs2 - 1) // bs2, bs2, args)
    nblk = (S + bs3 - 1) // bs3
    return mod, (xt, yt, zt), S, nblk, bs3, lam


def orbit_uvw(nsat, orbit_res, orbit_counts, index, frequency, r1, r2, a=2038.14, e=0.0,
              incl_deg=30.0, argp_deg=0.0, mu=4.902793455e3):
    """calculateOrbit + uvwPosition per satellite, then computeUVW per ordered
    pair (MIncline_generate_uvw_float.cu:215-368).  Returns xt,yt,zt [nsat][S]
    and uvw [pairs][S][3] (before the thrust sort/unique).

    Host-side arrays are built as the reference's thrust code builds them
    (linspace `a + step*x` contracted to one FMA, x the float sequence value;
    dM in double, :42-58).  Two reference reads run past their buffers:
    uvwPosition reads x[sat*total + total] when a window ends exactly at the
    end (for the last satellite one element past the array), and computeUVW
    has no bounds check on its rounded-up grid.  The buffers here are padded
    (one extra satellite of zeros; one extra block of xt and of the output) so
    both stay inside their allocations; the padding reads as zero."""
    import torch
    mod, (xt, yt, zt), S, nblk, bs3, lam = _positions(nsat, orbit_res, orbit_counts, index, frequency, r1, r2, a, e,
                                                      incl_deg, argp_deg, mu)
    uvws = []
    hash_ = torch.zeros(nblk * bs3, 3, dtype=torch.float32, device="cuda")
    for mm in range(nsat):
        for nn in range(nsat):
            if mm == nn:
                continue
            args = [ptr(xt), ptr(yt), ptr(zt), ptr(hash_), i32(orbit_counts), i32(orbit_res),
                    f32(lam), i32(mm), i32(nn)]
            mod.launch("computeUVW", nblk, bs3, args)
            uvws.append(hash_[:S].clone())
    torch.cuda.synchronize()
    return (xt[:S * nsat].view(nsat, S), yt[:S * nsat].view(nsat, S), zt[:S * nsat].view(nsat, S)), torch.stack(uvws)


def host_r0(mean_r: float) -> float:
    """r0 = atanf(1737.74f / (mean_r + 1737.74f)) with the host's float arithmetic and
    libm's atanf, as the reference's host code computes it (shade1M.cu:222).  The
    float sum and quotient are evaluated in double and rounded once, which gives the
    correctly rounded float results that the host's float operations give."""
    f = lambda x: C.c_float(x).value  # noqa: E731
    libm = C.CDLL("libm.so.6")
    libm.atanf.restype = C.c_float
    libm.atanf.argtypes = [C.c_float]
    return float(libm.atanf(f(f(1737.74) / f(f(mean_r) + f(1737.74)))))


def cart2sph_r(u, v, w):
    """The r array of the reference's Cart2SphKernel (shade1M.cu:63-70): K complex<float>
    (imaginary parts 0) as a K x 2 float32 tensor."""
    import torch
    mod = module("shade1M")
    K = u.numel()
    cu = torch.stack([u, torch.zeros_like(u)], -1).contiguous()
    cv = torch.stack([v, torch.zeros_like(v)], -1).contiguous()
    cw = torch.stack([w, torch.zeros_like(w)], -1).contiguous()
    th = torch.zeros(K, 2, dtype=torch.float32, device="cuda")
    ph = torch.zeros_like(th)
    r = torch.zeros_like(th)
    bs = mod.occupancy_block("Cart2SphKernel")
    mod.launch("Cart2SphKernel", (K + bs - 1) // bs, bs, [ptr(cu), ptr(cv), ptr(cw), ptr(th), ptr(ph), ptr(r), i32(K)])
    torch.cuda.synchronize()
    return r


def shade_windows(u, v, w, RES, mean_r):
    """Cart2SphKernel + ShadeMatrix (shade1M.cu:63-105) on complex<float> arrays
    with zero imaginary parts; mean_r is supplied by the caller."""
    import math
    import torch
    mod = module("shade1M")
    K = u.numel()
    cu = torch.stack([u, torch.zeros_like(u)], -1).contiguous()
    cv = torch.stack([v, torch.zeros_like(v)], -1).contiguous()
    cw = torch.stack([w, torch.zeros_like(w)], -1).contiguous()
    th = torch.zeros(K, 2, dtype=torch.float32, device="cuda")
    ph = torch.zeros_like(th)
    r = torch.zeros_like(th)
    bs = mod.occupancy_block("Cart2SphKernel")
    mod.launch("Cart2SphKernel", (K + bs - 1) // bs, bs, [ptr(cu), ptr(cv), ptr(cw), ptr(th), ptr(ph), ptr(r), i32(K)])
    mean_rf = C.c_float(mean_r).value
    r0 = host_r0(mean_rf)
    dtheta = C.c_float(2 * math.pi / RES).value
    dphi = C.c_float(math.pi / RES).value
    sh = torch.zeros(K * 4, 2, dtype=torch.float32, device="cuda")
    bs = mod.occupancy_block("ShadeMatrix")
    mod.launch("ShadeMatrix", (K + bs - 1) // bs, bs,
               [ptr(cu), ptr(cv), ptr(cw), ptr(th), ptr(ph), ptr(r), ptr(sh), i32(K), i32(RES), f32(mean_rf),
                f32(r0), f32(dtheta), f32(dphi)])
    torch.cuda.synchronize()
    return sh[:, 0].view(K, 4).round().int(), r[:, 0].clone()


def nxq(NX, J):
    """computeLocCount + computeLocViss (vissGen1M_shade_optim1.cu:54-115)."""
    import torch
    mod = module("vissGen1M_shade_optim1")
    X = NX.numel()
    countLoc = torch.zeros(J, dtype=torch.int32, device="cuda")
    NXq = torch.zeros(X, dtype=torch.int32, device="cuda")
    bs = mod.occupancy_block("computeLocCount")
    mod.launch("computeLocCount", (J + bs - 1) // bs, bs, [ptr(NX), ptr(countLoc), i32(J), i32(X)])
    bs = mod.occupancy_block("computeLocViss")
    mod.launch("computeLocViss", (J + bs - 1) // bs, bs, [ptr(NX), ptr(NXq), ptr(countLoc), i32(J), i32(X)])
    torch.cuda.synchronize()
    return countLoc, NXq
