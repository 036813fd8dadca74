"""Inputs a pass cannot use are recorded, not read out of bounds: a snapshot index
outside the geometry and a fine-map index outside the fine grid set flag bits that
viss_workspace_flags returns after the pass; clean inputs leave them zero."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _vis_flags(V, d, snap):
    from viss_recon_shade_gb300 import _lib as L
    cfg = V.DftConfig.geometric().c(d["u"].numel())
    K, J = d["u"].numel(), d["l"].numel()
    sp = d["sat_pos"]
    geo = L.Geometry(sp.data_ptr(), sp.shape[0], sp.shape[1], 0)
    nb = L.lib.viss_vis_dft_workspace(C.byref(cfg), K, J, C.byref(geo))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = torch.empty(K, dtype=torch.complex64, device="cuda")
    sky = L.Sky(d["l"].data_ptr(), d["m"].data_ptr(), d["n"].data_ptr(), d["b"].data_ptr(), J)
    vs = L.VisSet(d["u"].data_ptr(), d["v"].data_ptr(), d["w"].data_ptr(), None, None, snap.data_ptr(),
                  d["pair"].data_ptr(), K)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(L.lib.viss_vis_dft(C.byref(cfg), C.byref(sky), C.byref(vs), C.byref(geo), C.c_void_p(out.data_ptr()),
                               C.c_void_p(ws.data_ptr()), nb, st), "viss_vis_dft")
    f = C.c_int32(-1)
    L.check(L.lib.viss_workspace_flags(C.c_void_p(ws.data_ptr()), C.byref(f), st), "viss_workspace_flags")
    return f.value, out


def test_snapshot_out_of_range_is_flagged():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    import dataclasses
    wl = dataclasses.replace(WORKLOADS["cfg1_1MHz"], orbit_counts=1)
    d = make_uvw(wl)
    l, m, n, b = (torch.from_numpy(a).cuda() for a in make_sky(wl))
    d.update(l=l, m=m, n=n, b=b)
    f0, v0 = _vis_flags(V, d, d["snap"])
    assert f0 == 0
    bad = d["snap"].clone()
    bad[7] = d["sat_pos"].shape[0] + 5
    f1, v1 = _vis_flags(V, d, bad)
    assert f1 & 2
    # only the bad row changes (the others up to summation order: their block's sky
    # tiles are compacted against a cone that now includes satellite 0 of snapshot 0)
    same = torch.ones_like(v0, dtype=torch.bool)
    same[7] = False
    a, b = v0[same].cpu().numpy(), v1[same].cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(a)


def test_fine_map_index_out_of_range_is_nan():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import fibonacci_sphere
    rng = np.random.default_rng(0)
    res, J = 32, 256
    X = res * res
    cl = np.full(J, X // J, np.int32)
    nq = np.arange(X, dtype=np.float32)
    nq[10] = X + 3  # pixel 2's third member points outside the fine grid
    l, m, n = fibonacci_sphere(J)
    FF = rng.lognormal(size=X).astype(np.float32)
    u, v, w = (np.ceil(rng.normal(0, 20, 64)).astype(np.float32) for _ in range(3))
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    cfg = V.DftConfig.reference(res, mask=V.MASK_NONE)
    Vg = V.vis_dft_map(cfg, cu(u), cu(v), cu(w), cu(l), cu(m), cu(n), cu(FF), cu(nq), cu(cl)).cpu().numpy()
    assert np.all(np.isnan(Vg))  # the NaN pixel reaches every visibility, as a NaN brightness would
