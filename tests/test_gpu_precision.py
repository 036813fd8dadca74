"""Precision sweep at 30 MHz (|uvw| up to ~1e4 wavelengths): 16 satellites on a
300 km lunar orbit, 120 baselines, 786,432 Fibonacci pixels.  Against the FP64
oracle on a 1% pixel subsample (recon) and sampled visibilities (vis):
  PLAIN       -- the reference's FP32 phase: error grows with |uvw|, ~1e-3..1e-2
  FAST        -- 32-bit fixed-point phase: <= 1e-5
  COMPENSATED -- fixed point + FP32 correction of the pixel rounding: <= 1e-5, not above FAST
The snapshot count is reduced (2,048) so the FP64 oracle finishes in seconds; the
error does not depend on it."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_precision_sweep_30MHz(oracle):
    import dataclasses
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = dataclasses.replace(WORKLOADS["cfg5_30MHz"], orbit_res=3072, orbit_counts=2)
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    cu = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    h = lambda t: t.cpu().numpy()  # noqa: E731
    K, J = d["u"].numel(), l.size
    umax = max(float(d[k].abs().max()) for k in "uvw")
    assert umax > 5000  # the long-baseline regime
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    u, v, w, snap, pair, pos = (h(d[k]) for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    rows = np.linspace(0, K - 1, 32).astype(np.int64)
    Vo = oracle.vis_dft(oc, u[rows], v[rows], w[rows], l, m, n, b, geo=oracle.make_geo(pos, snap[rows], pair[rows]))
    pix = np.linspace(0, J - 1, J // 100).astype(np.int64)  # 1% subsample
    errs = {}
    Vref = None
    for name, prec in (("plain", V.PREC_PLAIN), ("fast", V.PREC_FAST), ("comp", V.PREC_COMPENSATED)):
        cfg = V.DftConfig.geometric(precision=prec)
        Vg = V.vis_dft(cfg, d["u"], d["v"], d["w"], cu(l), cu(m), cu(n), cu(b), **geo)
        if Vref is None:
            # recon errors are measured on the same input visibilities for every mode
            Vref = V.vis_dft(V.DftConfig.geometric(precision=V.PREC_COMPENSATED), d["u"], d["v"], d["w"], cu(l),
                             cu(m), cu(n), cu(b), **geo)
            Fo = oracle.recon(oc, u, v, w, None, h(Vref), l[pix], m[pix], n[pix], geo=oracle.make_geo(pos, snap, pair))
        Fg = V.recon(cfg, d["u"], d["v"], d["w"], Vref, cu(l), cu(m), cu(n), **geo)
        ev = np.linalg.norm(h(Vg)[rows] - Vo) / np.linalg.norm(Vo)
        ef = np.linalg.norm(h(Fg)[pix] - Fo) / np.linalg.norm(Fo)
        errs[name] = (ev, ef)
    print("precision sweep (vis rms, recon rms):", {k: (f"{a:.2e}", f"{b:.2e}") for k, (a, b) in errs.items()})
    assert errs["fast"][0] <= 1e-5 and errs["fast"][1] <= 1e-5
    assert errs["comp"][0] <= 1e-5 and errs["comp"][1] <= 1e-5
    # at |uvw| ~ 1e4 the fixed-point rounding of the pixels (|U| 2^-33 turns) is already
    # below the float angle's own rounding: the compensation must not make things worse
    assert errs["comp"][0] <= 1.05 * errs["fast"][0] and errs["comp"][1] <= 1.05 * errs["fast"][1]
    assert errs["plain"][0] > 30 * errs["comp"][0]
