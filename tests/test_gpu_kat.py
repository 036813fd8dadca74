"""Known-answer tests of the DFT kernels (closed forms, no oracle):

- a point source at the phase centre (l, m, n) = (0, 0, 1): every visibility is
  its brightness, for integer and fractional uvw and every precision;
- one visibility V = 1: the reconstructed image is exp(+2 pi i (u l + v m + w (n-1))),
  a pure cosine in its real part;
- the geometric mask in its limits: satellites so far away that the Moon hides
  no pixel give the unmasked result (pixels near the anti-satellite direction
  fall in the float test's band there and are decided, unoccluded, in double);
  an orbit at 300 km hides pixels and decides some tests near the limb in double,
  which viss_workspace_limb_count counts; an unmasked pass counts none."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def sphere(J, seed):
    x = np.random.default_rng(seed).normal(size=(J, 3))
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return [np.ascontiguousarray(x[:, i]).astype(np.float32) for i in range(3)]


PRECS = ["fast", "comp", "plain"]


def prec(V, name):
    return {"fast": V.PREC_FAST, "comp": V.PREC_COMPENSATED, "plain": V.PREC_PLAIN}[name]


@pytest.mark.parametrize("p", PRECS)
@pytest.mark.parametrize("integer", [True, False])
def test_point_source_at_phase_centre(V, p, integer):
    rng = np.random.default_rng(1)
    K, J = 3000, 700
    l, m, n = sphere(J, 2)
    l[5], m[5], n[5] = 0.0, 0.0, 1.0
    b = np.zeros(J, np.float32)
    b[5] = 3.5
    u, v, w = (rng.normal(0, 3000, K).astype(np.float32) for _ in range(3))
    if integer:
        u, v, w = np.ceil(u), np.ceil(v), np.ceil(w)
    cfg = V.DftConfig.geometric(precision=prec(V, p)).with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE)
    Vg = V.vis_dft(cfg, cu(u), cu(v), cu(w), cu(l), cu(m), cu(n), cu(b)).cpu().numpy()
    assert np.abs(Vg - 3.5).max() <= 3.5 * 1e-6


@pytest.mark.parametrize("p", PRECS)
def test_single_visibility_gives_cosine_image(V, p):
    J = 5000
    l, m, n = sphere(J, 3)
    u, v, w = (np.array([x], np.float32) for x in (1234.25, -777.5, 310.0))
    Vis = torch.ones(1, dtype=torch.complex64, device="cuda")
    cfg = V.DftConfig.geometric(precision=prec(V, p)).with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE,
                                                            norm=1.0)
    F = V.recon(cfg, cu(u), cu(v), cu(w), Vis, cu(l), cu(m), cu(n)).cpu().numpy()
    ph = 2 * np.pi * (1234.25 * l.astype(np.float64) - 777.5 * m.astype(np.float64)
                      + 310.0 * (n.astype(np.float64) - 1.0))
    tol = 5e-3 if p == "plain" else 2e-6  # plain: the reference's FP32 phase of |u| ~ 1e3
    assert np.abs(F.real - np.cos(ph)).max() <= tol
    assert np.abs(F.imag - np.sin(ph)).max() <= tol


def vis_pass(V, cfg, d, sat_pos):
    """One vis pass through the C ABI; returns (V, near-limb decision count)."""
    from viss_recon_shade_gb300 import _lib as L
    c = cfg.c(d["u"].numel())
    K, J = d["u"].numel(), d["l"].numel()
    geo = L.Geometry(sat_pos.data_ptr(), sat_pos.shape[0], sat_pos.shape[1], 0)
    nb = L.lib.viss_vis_dft_workspace(C.byref(c), K, J, C.byref(geo))
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    out = torch.empty(K, dtype=torch.complex64, device="cuda")
    sky = L.Sky(d["l"].data_ptr(), d["m"].data_ptr(), d["n"].data_ptr(), d["b"].data_ptr(), J)
    vs = L.VisSet(d["u"].data_ptr(), d["v"].data_ptr(), d["w"].data_ptr(), None, None, d["snap"].data_ptr(),
                  d["pair"].data_ptr(), K)
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(L.lib.viss_vis_dft(C.byref(c), C.byref(sky), C.byref(vs), C.byref(geo), C.c_void_p(out.data_ptr()),
                               C.c_void_p(ws.data_ptr()), nb, st), "viss_vis_dft")
    cnt = C.c_int64(-1)
    L.check(L.lib.viss_workspace_limb_count(C.c_void_p(ws.data_ptr()), C.byref(cnt), st),
            "viss_workspace_limb_count")
    return out, cnt.value


@pytest.fixture(scope="module")
def orbit_case(V):
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = dataclasses.replace(WORKLOADS["cfg1_1MHz"], orbit_counts=1)
    d = make_uvw(wl)
    l, m, n, b = (torch.from_numpy(a).cuda() for a in make_sky(wl))
    d.update(l=l, m=m, n=n, b=b)
    return d


@pytest.mark.parametrize("p", PRECS)
def test_geometric_mask_limits_and_limb_count(V, orbit_case, p):
    d = orbit_case
    geo_cfg = V.DftConfig.geometric(precision=prec(V, p))
    none_cfg = geo_cfg.with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE)
    v_none, c_none = vis_pass(V, none_cfg, d, d["sat_pos"])
    assert c_none == 0
    # satellites 1e9 times farther out: the Moon subtends ~1e-9 rad and hides no pixel
    v_far, _ = vis_pass(V, geo_cfg, d, (d["sat_pos"].double() * 1e9).float())
    a, b = v_far.cpu().numpy(), v_none.cpu().numpy()
    assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(b)
    # the 300 km orbit: some tests land within the limb band and are counted
    v_geo, c_geo = vis_pass(V, geo_cfg, d, d["sat_pos"])
    assert c_geo > 0
    assert np.linalg.norm(v_geo.cpu().numpy() - b) > 1e-3 * np.linalg.norm(b)  # the Moon does hide pixels
