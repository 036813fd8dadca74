"""The simulator's configurations at their stated sizes.

  cfg1  1 MHz, 28 baselines x 1,024 snapshots = 28,672 uvw, 12,288 pixels:
        REF_QUIRK windows -- ours against the reference's own visscal/imagerecon
        (vissGen10M_shade, _optim1, _optim2, run from its sources) and against the
        FP64 oracle on every term; GEOMETRIC -- ours against the full FP64 oracle,
        and the occlusion mask itself exactly (integer counts).
  cfg2  10 MHz, 1,835,008 uvw x 196,608 pixels, REF_QUIRK windows: ours against the
        reference kernels' full-size outputs, both against FP64 on sampled rows and
        pixels.
  cfg3  64 channels (1-30 MHz, 28 x U[4096, 65536] snapshots, 49,152 pixels) in one
        batched pass: sampled channels against FP64 and against their solo runs.
(cfg4 is covered at its size by test_gpu_autograd.py, cfg5 by test_gpu_precision.py.)

Tolerances: 1e-5 normwise relative error against FP64 for the fast path; against a
reference kernel, within 1.5x of that kernel's own FP32 error from FP64."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-5


def nerr(x, ref):
    return float(np.linalg.norm(np.asarray(x) - ref) / np.linalg.norm(ref))


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def h(t):
    return t.detach().cpu().numpy()


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


@pytest.fixture(scope="module")
def refk():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    return ref_cuda


def synth_windows(K, res, seed):
    """Normalised shade windows [K, 4] (M1 <= M2, M3 <= M4, 0-based) that exercise both
    reference masks: a third with M3 == 0, so the quirk's window-row loop
    (vissGen10M_shade.cu:130) runs, and some with both ratios M1/M2, M3/M4 above 1/2,
    so the recon mask (:166) fires on pixel res + 1.  (Windows computed from orbit uvw
    keep M3 > 0 for a 30 degree orbit, where the quirk's loop never runs.)"""
    rng = np.random.default_rng(seed)
    M1 = rng.integers(0, res - 1, K)
    M2 = np.minimum(res - 1, M1 + rng.integers(0, res // 2, K))
    M3 = np.where(rng.random(K) < 0.35, 0, rng.integers(0, res - 1, K))
    M4 = np.minimum(res - 1, M3 + rng.integers(0, 8, K))
    sel = rng.random(K) < 0.15
    M2[sel] = rng.integers(2, res - 1, sel.sum())
    M1[sel] = M2[sel] - rng.integers(0, 1 + M2[sel] // 3, sel.sum())
    M4[sel] = rng.integers(2, res - 1, sel.sum())
    M3[sel] = M4[sel] - rng.integers(0, 1 + M4[sel] // 3, sel.sum())
    return np.stack([M1, M2, M3, M4], -1).astype(np.int32)


@pytest.fixture(scope="module")
def cfg1():
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS["cfg1_1MHz"]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    assert d["u"].numel() == 28672 and l.size == 12288
    d.update(l=l, m=m, n=n, b=b)
    return d


VARIANTS = [("vissGen10M_shade", True), ("vissGen10M_shade_optim1", False), ("vissGen10M_shade_optim2", False)]


@pytest.mark.parametrize("variant,trunc", VARIANTS)
def test_cfg1_ref_quirk_vs_reference_kernels(V, oracle, refk, cfg1, variant, trunc):
    d = cfg1
    K, J, RES = d["u"].numel(), d["l"].size, 111  # 111 x 111 ~ 12,288: about 110 window rows
    u, v, w = d["u"], d["v"], d["w"]
    l, m, n, FF = (cu(d[k]) for k in ("l", "m", "n", "b"))
    shade = synth_windows(K, RES, 11)
    M = cu(shade)
    Ms = [M[:, i].contiguous() for i in range(4)]
    wgt = cu((1.0 / np.random.default_rng(1).integers(1, 6, K)).astype(np.float32))
    nxq = torch.arange(J, dtype=torch.float32, device="cuda")
    cl = torch.ones(J, dtype=torch.int32, device="cuda")
    ref_v = refk.visscal(variant, K, J, RES, FF, u, v, w, l, m, n, *Ms, nxq, cl)
    ours = torch.zeros(K, dtype=torch.complex64, device="cuda")
    V.visscal(K, J, RES, FF, ours, u, v, w, l, m, n, *Ms, variant=V.VARIANT_PLAIN if trunc else V.VARIANT_OPTIM)
    hu, hv, hw = h(u), h(v), h(w)
    f64 = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=RES, trunc=trunc, occluded_value=240.0), hu, hv, hw,
                         d["l"], d["m"], d["n"], d["b"], shade=shade)
    rv = h(ref_v)[:, 0] + 1j * h(ref_v)[:, 1]
    assert nerr(h(ours), f64) < TOL
    assert nerr(h(ours), rv) < 1.5 * nerr(rv, f64) + TOL
    # recon of the reference kernel's visibilities, both ways
    ref_f = refk.imagerecon(variant, K, J, RES, ref_v, u, v, w, l, m, n, wgt, *Ms)
    r1, r2 = V.recon_ratios(M.contiguous())
    F = torch.zeros(J, dtype=torch.complex64, device="cuda")
    V.imagerecon(K, J, RES, F, ref_v.view(torch.complex64).view(-1), u, v, w, l, m, n, wgt, r1, r2, r1, r2)
    f64r = oracle.recon(oracle.make_cfg(res=RES, recon_ref_mask=True, norm=1.0 / K), hu, hv, hw, h(wgt),
                        rv.astype(np.complex64), d["l"], d["m"], d["n"], shade=shade)
    rf = h(ref_f)[:, 0] + 1j * h(ref_f)[:, 1]
    assert nerr(h(F), f64r) < TOL
    assert nerr(h(F), rf) < 1.5 * nerr(rf, f64r) + TOL


def test_cfg1_geometric_vs_full_fp64(V, oracle, cfg1):
    """Every term of both passes against the FP64 oracle (3.5e8 terms each)."""
    d = cfg1
    K = d["u"].numel()
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    Vg = V.vis_dft(cfg, d["u"], d["v"], d["w"], *(cu(d[k]) for k in ("l", "m", "n", "b")), **geo)
    Fg = V.recon(cfg, d["u"], d["v"], d["w"], Vg, *(cu(d[k]) for k in ("l", "m", "n")), **geo)
    hu, hv, hw, snap, pair, pos = (h(d[k]) for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    g = oracle.make_geo(pos, snap, pair)
    Vo = oracle.vis_dft(oc, hu, hv, hw, d["l"], d["m"], d["n"], d["b"], geo=g)
    Fo = oracle.recon(oc, hu, hv, hw, None, h(Vg), d["l"], d["m"], d["n"], geo=g)
    assert nerr(h(Vg), Vo) < TOL and nerr(h(Fg), Fo) < TOL


def test_cfg1_geometric_mask_exact(V, oracle, cfg1):
    """The occlusion mask of all 28,672 x 12,288 terms, read out exactly: with zero uvw
    every phase is 0, so V_k = sum over pixel weights (visible: brightness, occluded:
    the occluded value) and F_j = sum over row weights of the rows that see j, all
    small integers.  Per row: the occluded count and a weighted visible sum; per
    pixel: the visible count and a weighted sum -- all equal to the FP64 oracle's mask.
    Decisions within 1e-9 rad of a limb are counted and their rows / pixels left out."""
    d = cfg1
    K, J = d["u"].numel(), d["l"].size
    z = torch.zeros(K, dtype=torch.float32, device="cuda")
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    lmn = [cu(d[k]) for k in ("l", "m", "n")]
    wj = ((np.arange(J) % 509) + 1).astype(np.float32)
    wk = ((np.arange(K) % 509) + 1).astype(np.float32)
    base = V.DftConfig.geometric(precision=V.PREC_FAST)
    occ_cnt = h(V.vis_dft(base.with_(occluded_value=1.0), z, z, z, *lmn, cu(np.zeros(J, np.float32)), **geo)).real
    vis_w = h(V.vis_dft(base.with_(occluded_value=0.0), z, z, z, *lmn, cu(wj), **geo)).real
    ones = torch.ones(K, dtype=torch.complex64, device="cuda")
    see_cnt = h(V.recon(base.with_(norm=1.0), z, z, z, ones, *lmn, **geo)).real
    see_w = h(V.recon(base.with_(norm=1.0), z, z, z, cu(wk.astype(np.complex64)), *lmn, **geo)).real
    snap, pair, pos = (h(d[k]) for k in ("snap", "pair", "sat_pos"))
    o_occ = np.zeros(K, np.int64)
    o_visw = np.zeros(K, np.int64)
    o_see = np.zeros(J, np.int64)
    o_seew = np.zeros(J, np.int64)
    limb_row = np.zeros(K, bool)
    limb_pix = np.zeros(J, bool)
    for r0 in range(0, K, 2048):
        rows = np.arange(r0, min(K, r0 + 2048))
        g = oracle.make_geo(pos, snap[rows], pair[rows])
        mask, margin = oracle.geo_mask(g, 1737.4, d["l"], d["m"], d["n"], rows.size, J)
        limb = margin < 1e-9
        limb_row[rows] = limb.any(1)
        limb_pix |= limb.any(0)
        o_occ[rows] = mask.sum(1)
        o_visw[rows] = (~mask * wj.astype(np.int64)).sum(1)
        o_see += (~mask).sum(0)
        o_seew += ((~mask) * wk[rows, None].astype(np.int64)).sum(0)
    assert limb_row.mean() < 0.01 and limb_pix.mean() < 0.01
    ok, okp = ~limb_row, ~limb_pix
    assert np.array_equal(np.round(occ_cnt[ok]).astype(np.int64), o_occ[ok])
    assert np.array_equal(np.round(vis_w[ok]).astype(np.int64), o_visw[ok])
    assert np.array_equal(np.round(see_cnt[okp]).astype(np.int64), o_see[okp])
    assert np.array_equal(np.round(see_w[okp]).astype(np.int64), o_seew[okp])
    assert 0.02 < o_occ.sum() / (K * J) < 0.6


def test_cfg2_ref_quirk_full_size_vs_reference_kernels(V, oracle, refk):
    """1,835,008 x 196,608 with the reference's window mask (RES 443: 443 rows of the
    sky index; windows as in the cfg1 test), the reference's plain kernel and its optim2 rewrite at full size; ours
    and theirs against FP64 on 48 visibilities (all pixels) and 12 pixels (all
    visibilities, the reference kernel's visibilities as input)."""
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS["cfg2_10MHz"]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    u, v, w = d["u"], d["v"], d["w"]
    K, J, RES = u.numel(), l.size, 443
    shade = synth_windows(K, RES, 12)
    M = cu(shade)
    Ms = [M[:, i].contiguous() for i in range(4)]
    tl, tm, tn, FF = cu(l), cu(m), cu(n), cu(b)
    wgt = torch.ones(K, dtype=torch.float32, device="cuda")
    nxq = torch.arange(J, dtype=torch.float32, device="cuda")
    cl = torch.ones(J, dtype=torch.int32, device="cuda")
    hu, hv, hw = h(u), h(v), h(w)
    rows = np.linspace(0, K - 1, 48).astype(np.int64)
    # the reference's recon mask can only fire on pixel RES + 1 (thetaP = phiP = 1); the
    # oracle indexes the pixels it is given from 0, so the sample starts with pixels
    # 0 .. RES + 1 (their own indices) and adds 12 beyond (never at local index RES + 1)
    pix = np.concatenate([np.arange(RES + 2), np.linspace(RES + 2, J - 1, 12).astype(np.int64)])
    for variant, trunc in (VARIANTS[0], VARIANTS[2]):
        ref_v = refk.visscal(variant, K, J, RES, FF, u, v, w, tl, tm, tn, *Ms, nxq, cl)
        ours = torch.zeros(K, dtype=torch.complex64, device="cuda")
        V.visscal(K, J, RES, FF, ours, u, v, w, tl, tm, tn, *Ms,
                  variant=V.VARIANT_PLAIN if trunc else V.VARIANT_OPTIM)
        f64 = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=RES, trunc=trunc, occluded_value=240.0), hu[rows],
                             hv[rows], hw[rows], l, m, n, b, shade=shade[rows])
        rv = h(ref_v)[:, 0] + 1j * h(ref_v)[:, 1]
        assert nerr(h(ours)[rows], f64) < TOL, variant
        assert nerr(h(ours)[rows], rv[rows]) < 1.5 * nerr(rv[rows], f64) + TOL, variant
        ref_f = refk.imagerecon(variant, K, J, RES, ref_v, u, v, w, tl, tm, tn, wgt, *Ms)
        r1, r2 = V.recon_ratios(M.contiguous())
        F = torch.zeros(J, dtype=torch.complex64, device="cuda")
        V.imagerecon(K, J, RES, F, ref_v.view(torch.complex64).view(-1), u, v, w, tl, tm, tn, wgt, r1, r2, r1, r2)
        f64r = oracle.recon(oracle.make_cfg(res=RES, recon_ref_mask=True, norm=1.0 / K), hu, hv, hw, None,
                            rv.astype(np.complex64), l[pix], m[pix], n[pix], shade=shade)
        rf = h(ref_f)[:, 0] + 1j * h(ref_f)[:, 1]
        assert nerr(h(F)[pix], f64r) < TOL, variant
        assert nerr(h(F)[pix], rf[pix]) < 1.5 * nerr(rf[pix], f64r) + TOL, variant


def test_cfg3_all_64_channels(V, oracle):
    """The batched workload at its size (63.5M visibilities over 64 channels, one
    persistent launch per pass, graph-replayed): three channels spread over the band
    against FP64 (16 visibilities x all pixels, 16 pixels x all the channel's
    visibilities) and against the same channel run alone."""
    from viss_recon_shade_gb300.synth import BATCH_WORKLOADS, make_batch
    bw = BATCH_WORKLOADS["batch64"]
    d = make_batch(bw)
    ro = d["row_off"]
    lg, mg, ng = cu(d["l"]), cu(d["m"]), cu(d["n"])
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    b = V.ChannelBatch(cfg, d["u"], d["v"], d["w"], ro, lg, mg, ng, d["bright"], snap=d["snap"], pair=d["pair"],
                       sat_pos=d["sat_pos"])
    g = b.graph()
    g.replay()
    torch.cuda.synchronize()
    assert b.nch == 64 and int(ro[-1]) > 60_000_000
    pos = h(d["sat_pos"])
    for c in (0, 31, 63):
        r0, r1 = int(ro[c]), int(ro[c + 1])
        u, v, w, snap, pair = (h(d[k][r0:r1]) for k in ("u", "v", "w", "snap", "pair"))
        Kc = r1 - r0
        oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=float(b.norm[c]))
        rows = np.linspace(0, Kc - 1, 16).astype(np.int64)
        Vo = oracle.vis_dft(oc, u[rows], v[rows], w[rows], d["l"], d["m"], d["n"], h(d["bright"][c]),
                            geo=oracle.make_geo(pos, snap[rows], pair[rows]))
        Vb = h(b.V[r0:r1])
        assert nerr(Vb[rows], Vo) < TOL, c
        pix = np.linspace(0, bw.J - 1, 16).astype(np.int64)
        Fo = oracle.recon(oc, u, v, w, None, Vb, d["l"][pix], d["m"][pix], d["n"][pix],
                          geo=oracle.make_geo(pos, snap, pair))
        Fb = h(b.F[c])
        assert nerr(Fb[pix], Fo) < TOL, c
        # the channel alone (its own launches) gives the same result
        sl = slice(r0, r1)
        Vs = V.vis_dft(cfg, d["u"][sl], d["v"][sl], d["w"][sl], lg, mg, ng, d["bright"][c], snap=d["snap"][sl],
                       pair=d["pair"][sl], sat_pos=d["sat_pos"])
        assert nerr(Vb, h(Vs).astype(np.complex128)) < 1e-6, c
