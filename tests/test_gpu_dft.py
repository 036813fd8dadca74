"""Parity of the CUDA vis-DFT / recon kernels against the FP64 oracle.

Tolerances (normwise relative error ||x - x_ref|| / ||x_ref|| and the max
form max|x - x_ref| / max|x_ref|) against the FP64 oracle on the same float
inputs:
  FAST / COMPENSATED: rms <= 1e-5, max <= 3e-5 (the target is 1e-5)
  PLAIN (the reference's FP32 phase): rms <= 5e-3 -- its error grows with |uvw|
Occlusion masks are compared exactly through zero-phase counting passes.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_RMS = 1e-5
TOL_MAX = 3e-5


def errs(x, ref):
    x = np.asarray(x, np.complex128)
    ref = np.asarray(ref, np.complex128)
    d = x - ref
    return (np.linalg.norm(d) / max(np.linalg.norm(ref), 1e-300),
            np.abs(d).max() / max(np.abs(ref).max(), 1e-300))


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


def cu(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def sky(J, seed=0):
    from viss_recon_shade_gb300.synth import fibonacci_sphere, lognormal_sky
    l, m, n = fibonacci_sphere(J)
    return l, m, n, lognormal_sky(J, seed=seed, n_points=min(20, J))


def uvw_int(K, sigma, seed=1):
    rng = np.random.default_rng(seed)
    return [np.ceil(rng.normal(0, sigma, K)).astype(np.float32) for _ in range(3)]


def uvw_frac(K, sigma, seed=2):
    rng = np.random.default_rng(seed)
    return [rng.normal(0, sigma, K).astype(np.float32) for _ in range(3)]


def shade_windows_synth(K, res, seed=3):
    rng = np.random.default_rng(seed)
    M1 = rng.integers(0, res - 1, K)
    M2 = np.minimum(res - 1, M1 + rng.integers(0, res // 2, K))
    M3 = np.where(rng.random(K) < 0.4, 0, rng.integers(0, 6, K))
    M4 = M3 + rng.integers(0, 6, K)
    return np.stack([M1, M2, M3, M4], -1).astype(np.int32)


# ------------------------------------------------------------------ no mask
@pytest.mark.parametrize("prec", ["fast", "comp"])
@pytest.mark.parametrize("kind,sigma", [("int", 300.0), ("int", 3000.0), ("frac", 300.0), ("frac", 3000.0)])
def test_vis_recon_nomask(V, oracle, prec, kind, sigma):
    K, J = 3000, 2500
    u, v, w = uvw_int(K, sigma) if kind == "int" else uvw_frac(K, sigma)
    l, m, n, b = sky(J)
    p = V.PREC_FAST if prec == "fast" else V.PREC_COMPENSATED
    for scale, noff in ((0.5, 0.0), (1.0, -1.0)):
        cfg = V.DftConfig(mask=V.MASK_NONE, precision=p, phase_scale=scale, n_offset=noff)
        Vg = V.vis_dft(cfg, *map(cu, (u, v, w, l, m, n, b))).cpu().numpy()
        ocfg = oracle.make_cfg(phase_scale=scale, n_offset=noff)
        Vo = oracle.vis_dft(ocfg, u, v, w, l, m, n, b)
        rms, mx = errs(Vg, Vo)
        assert rms <= TOL_RMS and mx <= TOL_MAX, (prec, kind, sigma, scale, rms, mx)
        wgt = np.random.default_rng(5).uniform(0.2, 1.0, K).astype(np.float32)
        Fg = V.recon(cfg, *map(cu, (u, v, w)), cu(Vg.astype(np.complex64)), *map(cu, (l, m, n)),
                     wgt=cu(wgt)).cpu().numpy()
        Fo = oracle.recon(oracle.make_cfg(phase_scale=scale, n_offset=noff, norm=1.0 / K), u, v, w, wgt,
                          Vg.astype(np.complex64), l, m, n)
        rms, mx = errs(Fg, Fo)
        assert rms <= TOL_RMS and mx <= TOL_MAX, ("recon", prec, kind, sigma, scale, rms, mx)


def test_plain_precision_matches_reference_formula(V, oracle):
    K, J = 1024, 1536
    u, v, w = uvw_int(K, 2000.0)
    l, m, n, b = sky(J)
    cfg = V.DftConfig(mask=V.MASK_NONE, precision=V.PREC_PLAIN, phase_scale=0.5, n_offset=0.0)
    Vg = V.vis_dft(cfg, *map(cu, (u, v, w, l, m, n, b))).cpu().numpy()
    Vo = oracle.vis_dft(oracle.make_cfg(phase_scale=0.5), u, v, w, l, m, n, b)
    Vm = oracle.vis_plain_f32(oracle.make_cfg(), u, v, w, l, m, n, b, d=2.0)
    rms_o, _ = errs(Vg, Vo)
    rms_m, _ = errs(Vg, Vm)
    assert rms_o < 5e-3          # FP32 phase: far from 1e-5 at |uvw| ~ 2000
    assert rms_m < rms_o / 3     # and much closer to the FP32 restatement of the reference


# ------------------------------------------------------------------ edge sizes
@pytest.mark.parametrize("K,J", [(0, 10), (10, 0), (1, 1), (1, 513), (1025, 1), (1023, 1025), (2049, 511)])
def test_edge_sizes(V, oracle, K, J):
    u, v, w = uvw_int(max(K, 1), 500.0)
    u, v, w = u[:K], v[:K], w[:K]
    l, m, n, b = sky(max(J, 1))
    l, m, n, b = l[:J], m[:J], n[:J], b[:J]
    cfg = V.DftConfig(mask=V.MASK_NONE, precision=V.PREC_FAST)
    Vg = V.vis_dft(cfg, *map(cu, (u, v, w, l, m, n, b))).cpu().numpy()
    assert Vg.shape == (K,)
    if K and J:
        rms, mx = errs(Vg, oracle.vis_dft(oracle.make_cfg(), u, v, w, l, m, n, b))
        assert rms <= TOL_RMS and mx <= TOL_MAX
    elif K:
        assert np.all(Vg == 0)
    Fg = V.recon(cfg, *map(cu, (u, v, w)), cu(Vg.astype(np.complex64)), *map(cu, (l, m, n))).cpu().numpy()
    assert Fg.shape == (J,)
    if K and J:
        Fo = oracle.recon(oracle.make_cfg(norm=1.0 / K), u, v, w, None, Vg.astype(np.complex64), l, m, n)
        rms, mx = errs(Fg, Fo)
        assert rms <= TOL_RMS and mx <= TOL_MAX
    elif J:
        assert np.all(Fg == 0)


# ------------------------------------------------------------------ REF masks
@pytest.mark.parametrize("mode", ["quirk", "intended"])
@pytest.mark.parametrize("trunc", [False, True])
@pytest.mark.parametrize("prec", ["fast", "plain"])
def test_vis_ref_masks(V, oracle, mode, trunc, prec):
    K, J, res = 2048, 1536, 256
    u, v, w = uvw_int(K, 800.0)
    l, m, n, b = sky(J)
    shade = shade_windows_synth(K, res)
    mm = V.MASK_REF_QUIRK if mode == "quirk" else V.MASK_REF_INTENDED
    p = V.PREC_FAST if prec == "fast" else V.PREC_PLAIN
    cfg = V.DftConfig(mask=mm, precision=p, res=res, trunc_brightness=trunc, occluded_value=240.0)
    Vg = V.vis_dft(cfg, *map(cu, (u, v, w, l, m, n, b)), shade=cu(shade)).cpu().numpy()
    Vo = oracle.vis_dft(oracle.make_cfg(mask_mode=mm, res=res, trunc=trunc, occluded_value=240.0), u, v, w, l, m, n,
                        b, shade=shade)
    rms, mx = errs(Vg, Vo)
    tol = (TOL_RMS, TOL_MAX) if prec == "fast" else (5e-4, 5e-3)
    assert rms <= tol[0] and mx <= tol[1], (mode, trunc, prec, rms, mx)


@pytest.mark.parametrize("mode", ["quirk", "intended"])
def test_vis_ref_mask_counts_exact(V, oracle, mode):
    """u = v = w = 0, brightness 0, occluded value 1: V_k counts the masked pixels exactly."""
    K, J, res = 4096, 3000, 300
    z = np.zeros(K, np.float32)
    l, m, n, _ = sky(J)
    shade = shade_windows_synth(K, res, seed=9)
    mm = V.MASK_REF_QUIRK if mode == "quirk" else V.MASK_REF_INTENDED
    cfg = V.DftConfig(mask=mm, precision=V.PREC_FAST, res=res, occluded_value=1.0)
    Vg = V.vis_dft(cfg, cu(z), cu(z), cu(z), *map(cu, (l, m, n)), cu(np.zeros(J, np.float32)),
                   shade=cu(shade)).cpu().numpy()
    counts = np.array([sum(oracle_hit(j, res, *shade[k], mm) for j in range(J)) for k in range(0, K, 97)])
    # zero phase: V_k = number of masked pixels (up to the SFU's cos(0) rounding)
    assert np.array_equal(np.round(Vg.real[::97]).astype(np.int64), counts)
    assert np.all(np.abs(Vg.imag) <= 1e-5 * np.maximum(1, np.abs(Vg.real)))
    assert counts.max() > 0


def oracle_hit(i, res, M1, M2, M3, M4, mode):
    if mode == 1:
        if M3 > 0 or M4 < 0:
            return False
        lo_a, lo_b = 0, M4
    else:
        lo_a, lo_b = M3, M4
    return any(lo * res + M1 + 1 <= i < lo * res + M2 for lo in range(lo_a, lo_b + 1))


def test_recon_ref_mask(V, oracle):
    K, J, res = 2048, 1536, 256
    u, v, w = uvw_int(K, 800.0)
    l, m, n, _ = sky(J)
    shade = shade_windows_synth(K, res)
    # ratios > 0.5 for a third of the rows so pixel res+1 is masked
    sel = np.random.default_rng(4).random(K) < 0.33
    shade[sel, 1] = 100; shade[sel, 0] = 80; shade[sel, 3] = 9; shade[sel, 2] = 7
    Vin = (np.random.default_rng(6).normal(size=K) + 1j * np.random.default_rng(7).normal(size=K)).astype(np.complex64)
    wgt = np.random.default_rng(8).uniform(0.2, 1.0, K).astype(np.float32)
    for p in (V.PREC_FAST, V.PREC_PLAIN):
        cfg = V.DftConfig(recon_mask=V.RECON_MASK_REF, precision=p, res=res)
        Fg = V.recon(cfg, *map(cu, (u, v, w)), cu(Vin), *map(cu, (l, m, n)), wgt=cu(wgt), shade=cu(shade)).cpu().numpy()
        Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, wgt, Vin, l, m, n,
                          shade=shade)
        rms, mx = errs(Fg, Fo)
        tol = (TOL_RMS, TOL_MAX) if p == V.PREC_FAST else (5e-4, 5e-3)
        assert rms <= tol[0] and mx <= tol[1], (p, rms, mx)
        # the masked pixel differs from the unmasked result
        Fu = oracle.recon(oracle.make_cfg(res=res, norm=1.0 / K), u, v, w, wgt, Vin, l, m, n)
        assert abs(Fu[res + 1] - Fo[res + 1]) > 1e3 * abs(Fg[res + 1] - Fo[res + 1])


def test_reference_shaped_entry_points(V, oracle):
    K, J, res = 2048, 1536, 256
    u, v, w = uvw_int(K, 800.0)
    l, m, n, b = sky(J)
    shade = shade_windows_synth(K, res)
    wgt = np.random.default_rng(8).uniform(0.2, 1.0, K).astype(np.float32)
    t = {k: cu(x) for k, x in dict(u=u, v=v, w=w, l=l, m=m, n=n, b=b, wgt=wgt).items()}
    M = [cu(shade[:, i].copy()) for i in range(4)]
    for variant in (V.VARIANT_PLAIN, V.VARIANT_OPTIM):
        viss = torch.zeros(K, dtype=torch.complex64, device="cuda")
        V.visscal(K, J, res, t["b"], viss, t["u"], t["v"], t["w"], t["l"], t["m"], t["n"], *M, variant=variant)
        Vo = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=res, trunc=variant == V.VARIANT_PLAIN), u, v, w, l, m, n,
                            b, shade=shade)
        rms, mx = errs(viss.cpu().numpy(), Vo)
        assert rms <= TOL_RMS and mx <= TOL_MAX
        r1, r2 = V.recon_ratios(cu(shade))
        F = torch.zeros(J, dtype=torch.complex64, device="cuda")
        V.imagerecon(K, J, res, F, viss, t["u"], t["v"], t["w"], t["l"], t["m"], t["n"], t["wgt"], r1, r2, r1, r2)
        Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, wgt,
                          viss.cpu().numpy(), l, m, n, shade=shade)
        rms, mx = errs(F.cpu().numpy(), Fo)
        assert rms <= TOL_RMS and mx <= TOL_MAX


# ------------------------------------------------------------------ geometric
def small_geometry(V, nsat=8, orbit_res=360, orbit_counts=2, freq=1e7):
    from viss_recon_shade_gb300.synth import log_separations
    r1, r2 = log_separations(nsat)
    cfg = V.OrbitConfig(nsat=nsat, orbit_res=orbit_res, orbit_counts=orbit_counts, a_km=2037.4, r1_m=r1, r2_m=r2,
                        fp64=True)
    pos, pos64 = V.orbit_positions(cfg, want_f64=True)
    u, v, w, snap, pair = V.baseline_uvw(pos, 3e8 / freq, ordered=False, rounding=False, pos64=pos64)
    return pos, u, v, w, snap, pair


@pytest.mark.parametrize("occ", [0.0, 240.0])
@pytest.mark.parametrize("prec", ["fast", "comp", "plain"])
def test_vis_recon_geometric(V, oracle, occ, prec):
    pos, u, v, w, snap, pair = small_geometry(V)
    K = u.numel()
    J = 3000
    l, m, n, b = sky(J)
    p = {"fast": V.PREC_FAST, "comp": V.PREC_COMPENSATED, "plain": V.PREC_PLAIN}[prec]
    cfg = V.DftConfig.geometric(precision=p, occluded_value=occ)
    Vg = V.vis_dft(cfg, u, v, w, *map(cu, (l, m, n, b)), snap=snap, pair=pair, sat_pos=pos).cpu().numpy()
    hn = lambda t: t.cpu().numpy()  # noqa: E731
    geo = oracle.make_geo(hn(pos), hn(snap), hn(pair))
    ocfg = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=occ, norm=1.0 / K)
    Vo = oracle.vis_dft(ocfg, hn(u), hn(v), hn(w), l, m, n, b, geo=geo)
    rms, mx = errs(Vg, Vo)
    tol = (TOL_RMS, TOL_MAX) if prec != "plain" else (5e-4, 5e-3)
    assert rms <= tol[0] and mx <= tol[1], (occ, prec, rms, mx)
    Fg = V.recon(cfg, u, v, w, cu(Vg.astype(np.complex64)), *map(cu, (l, m, n)), snap=snap, pair=pair,
                 sat_pos=pos).cpu().numpy()
    ocfg2 = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, norm=1.0 / K)
    Fo = oracle.recon(ocfg2, hn(u), hn(v), hn(w), None, Vg.astype(np.complex64), l, m, n, geo=geo)
    rms, mx = errs(Fg, Fo)
    assert rms <= tol[0] and mx <= tol[1], ("recon", occ, prec, rms, mx)


@pytest.mark.parametrize("order", ["snapshot", "shuffled"])
def test_geometric_mask_exact_counts(V, oracle, order):
    """Zero phase, brightness 0, occluded value 1: V_k = number of occluded pixels of row k;
    recon of V = 1 gives K * F_j = number of rows that see pixel j.  Both exact integers,
    compared with the FP64 oracle mask; decisions within 1e-9 rad of a limb are counted
    and excluded.  In snapshot order a block of 1,024 visibilities uses ~300 satellites and
    the vis kernel decides each (straddling pixel, satellite) once per tile; shuffled, a
    block spans the whole orbit (~5,760 satellites), the vis kernel tests each term's two
    satellites instead and the recon sees snapshot runs of one row."""
    pos, u, v, w, snap, pair = small_geometry(V)
    K = u.numel()
    if order == "shuffled":
        perm = torch.from_numpy(np.random.default_rng(11).permutation(K)).cuda()
        u, v, w, snap, pair = (t[perm].contiguous() for t in (u, v, w, snap, pair))
    J = 4000
    l, m, n, _ = sky(J)
    z = torch.zeros(K, dtype=torch.float32, device="cuda")
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=1.0)
    Vg = V.vis_dft(cfg, z, z, z, *map(cu, (l, m, n)), cu(np.zeros(J, np.float32)), snap=snap, pair=pair,
                   sat_pos=pos).cpu().numpy()
    hn = lambda t: t.cpu().numpy()  # noqa: E731
    geo = oracle.make_geo(hn(pos), hn(snap), hn(pair))
    mask, margin = oracle.geo_mask(geo, 1737.4, l, m, n, K, J)
    limb = margin < 1e-9
    cnt = mask.sum(1)
    ok_rows = ~limb.any(1)
    assert ok_rows.mean() > 0.99
    assert np.array_equal(np.round(Vg.real[ok_rows]).astype(np.int64), cnt[ok_rows])
    ones = torch.ones(K, dtype=torch.complex64, device="cuda")
    Fg = V.recon(cfg.with_(norm=1.0), z, z, z, ones, *map(cu, (l, m, n)), snap=snap, pair=pair,
                 sat_pos=pos).cpu().numpy()
    vis_cnt = (~mask).sum(0)
    ok_pix = ~limb.any(0)
    assert np.array_equal(np.round(Fg.real[ok_pix]).astype(np.int64), vis_cnt[ok_pix])
    assert 0.05 < mask.mean() < 0.6


# ------------------------------------------------------------------ properties at size
@pytest.mark.parametrize("workload", ["cfg4_10MHz", "cfg2_10MHz"])
def test_linearity_and_adjoint_large(V, workload):
    """Full-size properties (the 10 MHz workloads up to the headline's 1,835,008 x
    196,608): linearity of V in the brightness and the adjoint identity
    Re<A x, y> = <x, Re(A^H y)> with the geometric mask."""
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS[workload]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    J = l.size
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    rng = np.random.default_rng(11)
    x1 = rng.uniform(0, 1, J).astype(np.float32)
    x2 = rng.uniform(0, 1, J).astype(np.float32)
    args = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    L = lambda x: V.vis_dft(cfg, d["u"], d["v"], d["w"], *map(cu, (l, m, n)), cu(x), **args)  # noqa: E731
    A1, A2, A12 = L(x1), L(x2), L((2 * x1 + x2).astype(np.float32))
    lin = (A12 - (2 * A1 + A2)).abs().max() / A12.abs().max()
    assert lin.item() < 1e-5
    K = d["u"].numel()
    y = torch.complex(torch.randn(K, device="cuda"), torch.randn(K, device="cuda"))
    AH = V.recon(cfg.with_(norm=1.0), d["u"], d["v"], d["w"], y, *map(cu, (l, m, n)), **args)
    lhs = (A1.conj() * y).real.double().sum().item()
    rhs = (cu(x1).double() * AH.real.double()).sum().item()
    # scale of the identity: |<Ax, y>| <= ||Ax|| ||y|| (the sum itself cancels heavily)
    scale = A1.abs().double().norm().item() * y.abs().double().norm().item()
    assert abs(lhs - rhs) / scale < 1e-5


@pytest.mark.parametrize("mode", ["quirk", "intended"])
@pytest.mark.parametrize("prec", ["fast", "plain"])
def test_vis_windowed_index(V, oracle, mode, prec):
    """viss_vis_dft_windowed: the REF window tests win_index[j] (a shuffled grid index,
    some negative or past the grid) instead of j; exact counts with zero phase and the
    FP64 oracle otherwise.  An identity index reproduces viss_vis_dft."""
    K, J, res = 2048, 3000, 300
    rng = np.random.default_rng(21)
    widx = rng.permutation(J).astype(np.int32)
    widx[::37] = -1 - rng.integers(0, 5, widx[::37].size)
    widx[5::41] = J + rng.integers(0, 900, widx[5::41].size)
    l, m, n, b = sky(J)
    shade = shade_windows_synth(K, res, seed=10)
    mm = V.MASK_REF_QUIRK if mode == "quirk" else V.MASK_REF_INTENDED
    p = V.PREC_FAST if prec == "fast" else V.PREC_PLAIN
    # zero phase, brightness 0, occluded 1: V_k counts the pixels whose index the window holds
    z = np.zeros(K, np.float32)
    cfg0 = V.DftConfig(mask=mm, precision=p, res=res, occluded_value=1.0)
    Vc = V.vis_dft_windowed(cfg0, cu(z), cu(z), cu(z), *map(cu, (l, m, n)), cu(np.zeros(J, np.float32)), cu(widx),
                            cu(shade)).cpu().numpy()
    ks = range(0, K, 61)
    counts = np.array([sum(oracle_hit(int(widx[j]), res, *shade[k], mm) for j in range(J)) for k in ks])
    assert np.array_equal(np.round(Vc.real[::61]).astype(np.int64), counts)
    assert counts.max() > 0
    # brightness and phase against FP64
    u, v, w = uvw_int(K, 800.0)
    cfg = V.DftConfig(mask=mm, precision=p, res=res, occluded_value=240.0)
    Vg = V.vis_dft_windowed(cfg, *map(cu, (u, v, w, l, m, n, b)), cu(widx), cu(shade)).cpu().numpy()
    Vo = oracle.vis_dft_windex(oracle.make_cfg(mask_mode=mm, res=res, occluded_value=240.0), u, v, w, l, m, n, b,
                               shade, widx)
    rms, mx = errs(Vg, Vo)
    tol = (TOL_RMS, TOL_MAX) if prec == "fast" else (5e-4, 5e-3)
    assert rms <= tol[0] and mx <= tol[1], (mode, prec, rms, mx)
    # identity index: the ordinary pass
    Vi = V.vis_dft_windowed(cfg, *map(cu, (u, v, w, l, m, n, b)), cu(np.arange(J, dtype=np.int32)),
                            cu(shade)).cpu().numpy()
    Vn = V.vis_dft(cfg, *map(cu, (u, v, w, l, m, n, b)), shade=cu(shade)).cpu().numpy()
    assert np.abs(Vi - Vn).max() <= 1e-6 * np.abs(Vn).max()
