"""Adjoint / autograd: the gradient of a visibility loss through the CUDA
forward (viss_vis_dft) and adjoint (viss_recon) agrees with central finite
differences on 64 random pixels and with the FP64 oracle gradient; a sky +
per-baseline-gain fit recovers the seeded sky and gains (differentiable imaging
at 10 MHz, 28 baselines x 16,384 snapshots, 49,152 pixels, SNR 20)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS["cfg4_10MHz"]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    t = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    d.update(l=t(l), m=t(m), n=t(n), truth=t(b / b.max()))
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    return V, wl, d, cfg


def forward(V, d, cfg, x):
    from viss_recon_shade_gb300.autograd import vis_dft_autograd
    return vis_dft_autograd(x, cfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["snap"], d["pair"], d["sat_pos"])


def test_gradient_vs_finite_differences_and_fp64(setup, oracle):
    V, wl, d, cfg = setup
    J = d["l"].numel()
    gen = torch.Generator(device="cuda").manual_seed(0)
    Vt = forward(V, d, cfg, d["truth"])
    noise = (torch.randn(Vt.shape, generator=gen, device="cuda") + 1j * torch.randn(Vt.shape, generator=gen,
                                                                                        device="cuda")) / np.sqrt(2)
    V_obs = (Vt + noise.to(torch.complex64) * Vt.abs().mean() / 20).detach()
    x0 = (d["truth"] * 0.5 + 0.1).requires_grad_(True)
    loss = ((forward(V, d, cfg, x0) - V_obs).abs() ** 2).sum()
    loss.backward()
    grad = x0.grad.double().cpu().numpy()

    # FP64 oracle gradient: 2 Re(A^H r), r = A x0 - V_obs
    h = lambda t: t.detach().cpu().numpy()  # noqa: E731
    r = h(forward(V, d, cfg, x0.detach()) - V_obs).astype(np.complex128)
    K = r.size
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0)
    geo = oracle.make_geo(h(d["sat_pos"]), h(d["snap"]), h(d["pair"]))
    pix = np.random.default_rng(1).choice(J, 64, replace=False)
    g64 = 2 * oracle.recon(oc, h(d["u"]), h(d["v"]), h(d["w"]), None, r.astype(np.complex64), h(d["l"])[pix],
                           h(d["m"])[pix], h(d["n"])[pix], geo=geo).real
    e64 = np.linalg.norm(grad[pix] - g64) / np.linalg.norm(g64)
    assert e64 < 1e-4, e64

    # central finite differences on the same 64 pixels (the loss is quadratic in x,
    # so the only error is float rounding of the forward passes)
    x = x0.detach()
    fd = np.zeros(64)
    step = 0.05
    for i, j in enumerate(pix):
        e = torch.zeros_like(x)
        e[j] = step
        lp = ((forward(V, d, cfg, x + e) - V_obs).abs().double() ** 2).sum().item()
        lm = ((forward(V, d, cfg, x - e) - V_obs).abs().double() ** 2).sum().item()
        fd[i] = (lp - lm) / (2 * step)
    efd = np.linalg.norm(grad[pix] - fd) / np.linalg.norm(fd)
    assert efd < 1e-4, efd


def test_fit_recovers_sky_and_gains(setup):
    """The cfg4 fit (100 Adam steps, non-negative sky + 28 complex baseline gains) recovers
    the seeded truth.  The model g_b A(x) is invariant under x -> a x, g -> g / a, so the
    gains are compared after the best complex scale c (c g closest to the true gains):
    their error must be well below the spread of the true gains (i.e. the fit finds each
    baseline's own gain, not just the mean), the sky must correlate with the truth, and
    the misfit must sit at the noise level (SNR 20: |noise|^2 / |V|^2 ~ 1/400)."""
    V, wl, d, cfg = setup
    from viss_recon_shade_gb300.autograd import fit_sky_and_gains
    gen = torch.Generator(device="cuda").manual_seed(2)
    nb = wl.npairs
    true_g = ((1 + 0.05 * torch.randn(nb, generator=gen, device="cuda")) * torch.exp(
        1j * 0.05 * torch.randn(nb, generator=gen, device="cuda"))).to(torch.complex64)
    baseline = torch.arange(d["u"].numel(), device="cuda") % nb
    Vt = forward(V, d, cfg, d["truth"]).detach() * true_g[baseline]
    noise = (torch.randn(Vt.shape, generator=gen, device="cuda") + 1j * torch.randn(Vt.shape, generator=gen,
                                                                                        device="cuda")) / np.sqrt(2)
    V_obs = Vt + noise.to(torch.complex64) * Vt.abs().mean() / 20
    res = fit_sky_and_gains(V_obs, cfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["snap"], d["pair"],
                            d["sat_pos"], baseline, nb, steps=100)
    assert torch.all(res.sky >= 0)
    assert res.losses[-1] < 4.0 / 400 and res.losses[-1] < 0.01 * res.losses[0], res.losses[-1]
    g = res.gains
    c = (g.conj() * true_g).sum() / (g.abs() ** 2).sum()
    err = ((c * g - true_g).abs() ** 2).mean().sqrt().item()
    spread = ((true_g - true_g.mean()).abs() ** 2).mean().sqrt().item()
    assert err < 0.3 * spread, (err, spread)
    corr = torch.corrcoef(torch.stack([res.sky, d["truth"]]))[0, 1].item()
    assert corr > 0.999, corr
