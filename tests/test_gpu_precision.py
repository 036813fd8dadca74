"""Precision sweep of the largest configuration at its size: 30 MHz, 16 satellites on
a 300 km lunar orbit, 120 baselines x 65,536 snapshots = 7,864,320 visibilities,
786,432 Fibonacci pixels (|uvw| up to ~1e4 wavelengths), geometric occlusion.

Arms (phase arithmetic; all evaluate sin/cos in FP32):
  PLAIN        the reference's FP32 phase u*l/d + v*m/d + w*n/d
  F64_PHASE    the phase in FP64, range-reduced in FP64
  FAST         32-bit fixed-point phase (the chosen path)
  COMPENSATED  fixed point + FP32 correction of the pixel rounding (a double-word phase)
Errors against the FP64 oracle: vis on 32 sampled visibilities (all pixels), recon on
a 1% pixel subsample (all visibilities, the same input visibilities for every arm);
each as RMS (||gpu - fp64|| / ||fp64||) and max (max |gpu - fp64| / max |fp64|).
FAST and COMPENSATED run the full passes; PLAIN and F64_PHASE (one thread per
visibility / pixel) run on the sampled visibilities and pixels only.
With VISS_SWEEP_OUT set, the table is also written there as JSON."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_precision_sweep_30MHz(oracle):
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS["cfg5_30MHz"]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    h = lambda t: t.cpu().numpy()  # noqa: E731
    K, J = d["u"].numel(), l.size
    assert K == 7864320 and J == 786432 and wl.snapshots == 65536
    umax = max(float(d[k].abs().max()) for k in "uvw")
    assert umax > 5000  # the long-baseline regime
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    u, v, w, snap, pair, pos = (h(d[k]) for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    rows = np.linspace(0, K - 1, 32).astype(np.int64)
    Vo = oracle.vis_dft(oc, u[rows], v[rows], w[rows], l, m, n, b, geo=oracle.make_geo(pos, snap[rows], pair[rows]))
    pix = np.linspace(0, J - 1, J // 100).astype(np.int64)  # 1% subsample
    lg, mg, ng, bg = cu(l), cu(m), cu(n), cu(b)
    lp, mp, np_ = cu(l[pix]), cu(m[pix]), cu(n[pix])
    rsel = torch.from_numpy(rows).cuda()
    grow = dict(snap=d["snap"][rsel], pair=d["pair"][rsel], sat_pos=d["sat_pos"])
    # the recon input, the same for every arm
    Vin = V.vis_dft(V.DftConfig.geometric(precision=V.PREC_COMPENSATED), d["u"], d["v"], d["w"], lg, mg, ng, bg, **geo)
    Fo = oracle.recon(oc, u, v, w, None, h(Vin), l[pix], m[pix], n[pix], geo=oracle.make_geo(pos, snap, pair))

    def errs(x, ref):
        return (float(np.linalg.norm(x - ref) / np.linalg.norm(ref)), float(np.abs(x - ref).max() / np.abs(ref).max()))

    table = {}
    for name, prec in (("plain", V.PREC_PLAIN), ("f64_phase", V.PREC_F64_PHASE), ("fast", V.PREC_FAST),
                       ("compensated", V.PREC_COMPENSATED)):
        cfg = V.DftConfig.geometric(precision=prec)
        if prec in (V.PREC_PLAIN, V.PREC_F64_PHASE):
            Vg = h(V.vis_dft(cfg, d["u"][rsel], d["v"][rsel], d["w"][rsel], lg, mg, ng, bg, **grow))
            Fg = h(V.recon(cfg, d["u"], d["v"], d["w"], Vin, lp, mp, np_, **geo))
        else:
            Vg = h(V.vis_dft(cfg, d["u"], d["v"], d["w"], lg, mg, ng, bg, **geo))[rows]
            Fg = h(V.recon(cfg, d["u"], d["v"], d["w"], Vin, lg, mg, ng, **geo))[pix]
        (vr, vm), (fr, fm) = errs(Vg, Vo), errs(Fg, Fo)
        table[name] = {"vis_rms": vr, "vis_max": vm, "recon_rms": fr, "recon_max": fm}
    print("precision sweep:", json.dumps(table))
    if os.environ.get("VISS_SWEEP_OUT"):
        with open(os.environ["VISS_SWEEP_OUT"], "w") as f:
            json.dump({"workload": wl.name, "K": K, "J": J, "umax": umax, "vis_rows": int(rows.size),
                       "recon_pixels": int(pix.size), "arms": table}, f, indent=1)
    for name in ("fast", "compensated", "f64_phase"):
        assert table[name]["vis_rms"] <= 1e-5 and table[name]["recon_rms"] <= 1e-5, (name, table[name])
    # FP64 phase: only the FP32 sincos and sums are left
    assert table["f64_phase"]["vis_rms"] <= table["fast"]["vis_rms"]
    # at |uvw| ~ 1e4 the fixed-point rounding of the pixels (|U| 2^-33 turns) is already
    # below the float angle's own rounding: the compensation must not make things worse
    assert table["compensated"]["vis_rms"] <= 1.05 * table["fast"]["vis_rms"]
    assert table["compensated"]["recon_rms"] <= 1.05 * table["fast"]["recon_rms"]
    assert table["plain"]["vis_rms"] > 30 * table["compensated"]["vis_rms"]
