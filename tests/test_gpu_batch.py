"""Batched multi-channel passes (viss_vis_dft_batch / viss_recon_batch): five
channels log-spaced over 1-30 MHz with uneven snapshot counts and orbit phases,
12,288 pixels, per-channel power-law brightness.  Every channel of the one
persistent launch must match the same channel run alone, and one small channel
the FP64 oracle; graph replay and every tuning candidate give the same result."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def data():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import BATCH_WORKLOADS, make_batch
    d = make_batch(BATCH_WORKLOADS["batch5_small"])
    t = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    d.update(lg=t(d["l"]), mg=t(d["m"]), ng=t(d["n"]))
    return V, d


def rel(a, b):
    a, b = a.detach().cpu().numpy().astype(np.complex128), b.detach().cpu().numpy().astype(np.complex128)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def channel(d, c, V=None):
    r0, r1 = int(d["row_off"][c]), int(d["row_off"][c + 1])
    sl = slice(r0, r1)
    return dict(u=d["u"][sl], v=d["v"][sl], w=d["w"][sl], snap=d["snap"][sl], pair=d["pair"][sl],
                V=None if V is None else V[sl])


@pytest.mark.parametrize("prec", ["fast", "comp", "plain"])
@pytest.mark.parametrize("mask", ["geo", "none"])
def test_batch_matches_channels_run_alone(data, prec, mask):
    V, d = data
    p = {"fast": V.PREC_FAST, "comp": V.PREC_COMPENSATED, "plain": V.PREC_PLAIN}[prec]
    cfg = V.DftConfig.geometric(precision=p)
    if mask == "none":
        cfg = cfg.with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE)
    b = V.ChannelBatch(cfg, d["u"], d["v"], d["w"], d["row_off"], d["lg"], d["mg"], d["ng"], d["bright"],
                       snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    Vb = b.vis().clone()
    Fb = b.recon().clone()
    tol = 0.0 if prec == "plain" else 2e-6  # plain: the same per-channel launches
    for c in range(b.nch):
        ch = channel(d, c)
        K = ch["u"].numel()
        Vc = V.vis_dft(cfg, ch["u"], ch["v"], ch["w"], d["lg"], d["mg"], d["ng"], d["bright"][c], snap=ch["snap"],
                       pair=ch["pair"], sat_pos=d["sat_pos"])
        r0 = int(d["row_off"][c])
        assert rel(Vb[r0:r0 + K], Vc) <= tol, (c, rel(Vb[r0:r0 + K], Vc))
        Fc = V.recon(cfg.with_(norm=1.0 / K), ch["u"], ch["v"], ch["w"], Vb[r0:r0 + K], d["lg"], d["mg"], d["ng"],
                     snap=ch["snap"], pair=ch["pair"], sat_pos=d["sat_pos"])
        assert rel(Fb[c], Fc) <= tol, (c, rel(Fb[c], Fc))


def test_batch_channel_against_fp64_oracle(data, oracle):
    V, d = data
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST)
    b = V.ChannelBatch(cfg, d["u"], d["v"], d["w"], d["row_off"], d["lg"], d["mg"], d["ng"], d["bright"],
                       snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    Vb = b.vis()
    Fb = b.recon()
    h = lambda t: t.detach().cpu().numpy()  # noqa: E731
    c = int(np.argmin(np.diff(d["row_off"])))
    ch = channel(d, c)
    K = ch["u"].numel()
    r0 = int(d["row_off"][c])
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    geo = oracle.make_geo(h(d["sat_pos"]), h(ch["snap"]), h(ch["pair"]))
    rows = np.linspace(0, K - 1, 64).astype(np.int64)
    Vo = oracle.vis_dft(oc, h(ch["u"])[rows], h(ch["v"])[rows], h(ch["w"])[rows], d["l"], d["m"], d["n"],
                        h(d["bright"][c]), geo=oracle.make_geo(h(d["sat_pos"]), h(ch["snap"])[rows],
                                                               h(ch["pair"])[rows]))
    assert np.linalg.norm(h(Vb[r0:r0 + K])[rows] - Vo) / np.linalg.norm(Vo) <= 1e-5
    pix = np.linspace(0, d["l"].size - 1, 256).astype(np.int64)
    Fo = oracle.recon(oc, h(ch["u"]), h(ch["v"]), h(ch["w"]), None, h(Vb[r0:r0 + K]), d["l"][pix], d["m"][pix],
                      d["n"][pix], geo=geo)
    assert np.linalg.norm(h(Fb[c])[pix] - Fo) / np.linalg.norm(Fo) <= 1e-5


def test_graph_replay_and_tunings_agree(data):
    V, d = data
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST)
    b = V.ChannelBatch(cfg, d["u"], d["v"], d["w"], d["row_off"], d["lg"], d["mg"], d["ng"], d["bright"],
                       snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    b.step()
    V0, F0 = b.V.clone(), b.F.clone()
    # the same tuning again: work items are summed in a fixed order whichever CTA runs them
    b.step()
    assert torch.equal(b.V, V0) and torch.equal(b.F, F0)
    g = b.graph()
    b.V.zero_()
    b.F.zero_()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(b.V, V0) and torch.equal(b.F, F0)
    for t in V.tuning_candidates():
        b.set_tuning(t)
        b.step()
        assert rel(b.V, V0) <= 2e-6 and rel(b.F, F0) <= 2e-6, t
    best = V.autotune(b, use_cache=False)
    assert best in V.tuning_candidates()
    assert len(V.autotune_report(b)) == len(V.tuning_candidates())


def test_empty_channel_and_ref_masks(data):
    V, d = data
    # channel 1 without visibilities; REF windows from the shade kernel
    ro = d["row_off"].copy()
    keep = np.r_[0:ro[1], ro[2]:ro[-1]]
    sel = torch.from_numpy(keep).cuda()
    ro2 = np.concatenate([[0, ro[1], ro[1]], ro[3:] - (ro[2] - ro[1])]).astype(np.int64)
    u, v, w = d["u"][sel], d["v"][sel], d["w"][sel]
    raw, _ = V.shade_windows(u, v, w, 64)
    shade = V.normalise_shade(raw)
    res = 64
    J = res * res  # REF masks index pixels on a res x res grid
    cfg = V.DftConfig.reference(res).with_(norm=None)
    lg, mg, ng = d["lg"][:J], d["mg"][:J], d["ng"][:J]
    bright = d["bright"][:, :J].contiguous()
    b = V.ChannelBatch(cfg, u, v, w, ro2, lg, mg, ng, bright, shade=shade)
    b.step()
    assert torch.count_nonzero(b.F[1]) == 0
    for c in (0, 2):
        r0, r1 = int(ro2[c]), int(ro2[c + 1])
        Vc = V.vis_dft(cfg, u[r0:r1], v[r0:r1], w[r0:r1], lg, mg, ng, bright[c], shade=shade[r0:r1])
        assert rel(b.V[r0:r1], Vc) <= 2e-6
        Fc = V.recon(cfg, u[r0:r1], v[r0:r1], w[r0:r1], b.V[r0:r1], lg, mg, ng, shade=shade[r0:r1])
        assert rel(b.F[c], Fc) <= 2e-6
