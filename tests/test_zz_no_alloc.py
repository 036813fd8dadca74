"""viss_vis_dft_noalloc: the vis DFT for callers that cannot allocate device
memory (hosts that own a fixed GPU memory budget or pool, and loops that cannot
absorb cudaMalloc's synchronisation).  It must give the same visibilities as
viss_vis_dft with a caller workspace, call after call on its one built-in
scratch buffer, refuse passes larger than that buffer, and report the input
problems its pass records (the caller cannot read the scratch).

Collected last on purpose (file name): a failure here comes after every other
test has run.  Works alone in a fresh process and after the other tests."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5  # the parity tolerance of the other DFT tests
SCRATCH = 32 << 20  # VISS_NOALLOC_SCRATCH_BYTES
VIS_ROWS, VIS_MINB = 1024, 3  # visibilities per vis block; resident vis CTAs per SM


def _case(seed, J=49152, orbit_counts=2, rows=None):
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import fibonacci_sphere, lognormal_sky, log_separations
    r1, r2 = log_separations(8)
    oc = V.OrbitConfig(nsat=8, orbit_res=6144, orbit_counts=orbit_counts, index=1 + seed, a_km=2037.4, r1_m=r1,
                       r2_m=r2, fp64=True)
    pos, pos64 = V.orbit_positions(oc, want_f64=True)
    u, v, w, snap, pair = V.baseline_uvw(pos, 30.0, ordered=False, rounding=False, pos64=pos64)
    if rows is not None:
        u, v, w, snap, pair = (x[:rows].contiguous() for x in (u, v, w, snap, pair))
    l, m, n = (torch.from_numpy(a).cuda() for a in fibonacci_sphere(J))
    b = torch.from_numpy(lognormal_sky(J, seed=seed)).cuda()
    return dict(u=u, v=v, w=w, snap=snap, pair=pair, pos=pos, l=l, m=m, n=n, b=b)


def _structs(L, d, cfg_py):
    K, J = d["u"].numel(), d["l"].numel()
    cfg = cfg_py.c(K)
    sky = L.Sky(d["l"].data_ptr(), d["m"].data_ptr(), d["n"].data_ptr(), d["b"].data_ptr(), J)
    vis = L.VisSet(d["u"].data_ptr(), d["v"].data_ptr(), d["w"].data_ptr(), None, None, d["snap"].data_ptr(),
                   d["pair"].data_ptr(), K)
    geo = L.Geometry(d["pos"].data_ptr(), d["pos"].shape[0], d["pos"].shape[1], 0)
    return cfg, sky, vis, geo


def _noalloc_tuning(L, K):
    """The sky split the entry point plans with: ~4 work items per resident CTA."""
    slots = torch.cuda.get_device_properties(0).multi_processor_count * VIS_MINB
    nrb = (K + VIS_ROWS - 1) // VIS_ROWS
    split = -(-4 * slots // nrb) if 0 < nrb < 4 * slots else 1
    return L.Tuning(0, split, 0, 0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _both(L, d, cfg_py):
    cfg, sky, vis, geo = _structs(L, d, cfg_py)
    K = vis.K
    ref = torch.empty(K, dtype=torch.complex64, device="cuda")
    nbytes = L.lib.viss_vis_dft_workspace(C.byref(cfg), K, sky.J, C.byref(geo))
    ws = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    L.check(L.lib.viss_vis_dft(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(geo), C.c_void_p(ref.data_ptr()),
                               C.c_void_p(ws.data_ptr()), nbytes, _stream()), "viss_vis_dft")
    out = torch.full((K,), float("nan"), dtype=torch.complex64, device="cuda")
    L.check(L.lib.viss_vis_dft_noalloc(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(geo),
                                       C.c_void_p(out.data_ptr()), _stream()), "viss_vis_dft_noalloc")
    torch.cuda.synchronize()
    return ref.cpu().numpy(), out.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_twice():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    cfg_py = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    for seed in (0, 1):  # two calls in a row on the shared scratch, different inputs
        r, o = _both(L, _case(seed), cfg_py)
        assert np.isfinite(o).all()
        err = np.linalg.norm(o - r) / np.linalg.norm(r)
        assert err <= TOL, (seed, err)


def test_noalloc_largest_documented_pass():
    """131,072 visibilities x 196,608 pixels with the geometric mask: the size the
    header states fits the built-in scratch."""
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    d = _case(2, J=196608, orbit_counts=3, rows=131072)
    cfg_py = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    cfg, sky, vis, geo = _structs(L, d, cfg_py)
    tn = _noalloc_tuning(L, vis.K)
    assert L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), None, vis.K, sky.J, C.byref(geo), C.byref(tn)) <= SCRATCH
    r, o = _both(L, d, cfg_py)
    err = np.linalg.norm(o - r) / np.linalg.norm(r)
    assert np.isfinite(o).all() and err <= TOL, err


def test_noalloc_rejects_passes_beyond_its_scratch():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    d = _case(0, orbit_counts=24)  # 28 x 49,152 visibilities: needs more than the built-in scratch
    cfg, sky, vis, geo = _structs(L, d, V.DftConfig.geometric())
    tn = _noalloc_tuning(L, vis.K)
    assert L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), None, vis.K, sky.J, C.byref(geo), C.byref(tn)) > SCRATCH
    out = torch.empty(vis.K, dtype=torch.complex64, device="cuda")
    rc = L.lib.viss_vis_dft_noalloc(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(geo),
                                    C.c_void_p(out.data_ptr()), _stream())
    assert rc == L.VISS_ERR_RANGE
    assert b"scratch" in L.lib.viss_last_error()


def test_noalloc_reports_bad_snapshot_index():
    """A snapshot index beyond the geometry is recorded by the pass (which then
    tests that row against an in-range satellite instead of reading out of
    bounds); the entry point returns it as VISS_ERR_INVALID."""
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    d = _case(3, J=4096, orbit_counts=1)
    d["snap"][5] = d["pos"].shape[0] + 10
    cfg, sky, vis, geo = _structs(L, d, V.DftConfig.geometric())
    out = torch.empty(vis.K, dtype=torch.complex64, device="cuda")
    rc = L.lib.viss_vis_dft_noalloc(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(geo),
                                    C.c_void_p(out.data_ptr()), _stream())
    assert rc == L.VISS_ERR_INVALID
    assert b"snapshot or satellite" in L.lib.viss_last_error()
    d["snap"][5] = 0  # the next call on the same scratch starts from clean flags
    cfg, sky, vis, geo = _structs(L, d, V.DftConfig.geometric())
    L.check(L.lib.viss_vis_dft_noalloc(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(geo),
                                       C.c_void_p(out.data_ptr()), _stream()), "viss_vis_dft_noalloc")
