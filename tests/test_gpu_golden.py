"""The CUDA path against the reference's own kernel outputs (tests/golden/*.npz,
generated by tests/golden/make_golden.py from the reference's sources), and the
bench workload's accuracy against the FP64 oracle on sampled rows / pixels."""
from pathlib import Path

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"


def load(name):
    p = G / name
    if not p.exists():
        pytest.skip(f"{name} not generated")
    return np.load(p)


def cplx(a):
    return a[..., 0].astype(np.float64) + 1j * a[..., 1].astype(np.float64)


def nerr(x, ref):
    return np.linalg.norm(np.asarray(x) - ref) / np.linalg.norm(ref)


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


VARIANTS = [("vissGen10M_shade", True), ("vissGen10M_shade_optim1", False), ("vissGen10M_shade_optim2", False)]


@pytest.mark.parametrize("case", ["lo", "hi"])
@pytest.mark.parametrize("variant,trunc", VARIANTS)
def test_visscal_imagerecon_vs_reference_kernels(V, oracle, case, variant, trunc):
    z = load("ref_vis_recon.npz")
    g = {k[len(case) + 4:]: z[k] for k in z.files if k.startswith(f"{case}_in_")}
    K, J, res = g["u"].size, g["l"].size, int(g["res"])
    t = {k: cu(g[k]) for k in ("u", "v", "w", "l", "m", "n", "FF", "wgt")}
    M = [cu(g["shade"][:, i].copy()) for i in range(4)]
    viss = torch.zeros(K, dtype=torch.complex64, device="cuda")
    V.visscal(K, J, res, t["FF"], viss, t["u"], t["v"], t["w"], t["l"], t["m"], t["n"], *M,
              variant=V.VARIANT_PLAIN if trunc else V.VARIANT_OPTIM)
    ref_v = cplx(z[f"{case}_{variant}_viss"])
    f64 = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=res, trunc=trunc, occluded_value=240.0), g["u"], g["v"],
                         g["w"], g["l"], g["m"], g["n"], g["FF"], shade=g["shade"])
    ours = viss.cpu().numpy()
    assert nerr(ours, f64) < 1e-5
    # the reference kernel sits at its own FP32 error from FP64; ours is within that of it
    assert nerr(ours, ref_v) < 1.5 * nerr(ref_v, f64) + 1e-5
    r1, r2 = V.recon_ratios(cu(g["shade"]))
    F = torch.zeros(J, dtype=torch.complex64, device="cuda")
    viss_ref = cu(z[f"{case}_{variant}_viss"]).view(torch.complex64).view(-1)
    V.imagerecon(K, J, res, F, viss_ref, t["u"], t["v"], t["w"], t["l"], t["m"], t["n"], t["wgt"], r1, r2, r1, r2)
    ref_f = cplx(z[f"{case}_{variant}_F"])
    f64r = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), g["u"], g["v"], g["w"], g["wgt"],
                        z[f"{case}_{variant}_viss"].view(np.complex64).reshape(-1), g["l"], g["m"], g["n"],
                        shade=g["shade"])
    oursf = F.cpu().numpy()
    assert nerr(oursf, f64r) < 1e-5
    assert nerr(oursf, ref_f) < 1.5 * nerr(ref_f, f64r) + 1e-5


@pytest.mark.parametrize("tag", ["a", "b"])
def test_orbit_uvw_vs_reference_kernels(V, tag):
    """FP32 positions evaluate the reference's formulas with the same CUDA math
    functions in the same expression shapes; they match the reference kernels'
    positions to the last bit (all samples of both cases on GB300; the bound
    leaves room for a rare ulp), and uvw (ceil) follow."""
    z = load("ref_orbit.npz")
    nsat, orbit_res, orbit_counts, index, freq = z[f"{tag}_cfg"]
    cfg = V.OrbitConfig(nsat=int(nsat), orbit_res=int(orbit_res), orbit_counts=int(orbit_counts), index=int(index),
                        r1_m=tuple(z["r1"].tolist()), r2_m=tuple(z["r2"].tolist()), fp64=False)
    pos = V.orbit_positions(cfg).cpu().numpy()
    ref = z[f"{tag}_pos"]
    exact = np.all(pos == ref, axis=2)
    assert exact.mean() >= 0.999, exact.mean()
    assert np.abs(pos - ref).max() / 2038.14 < 2e-6
    u, v, w, snap, pair = V.baseline_uvw(torch.from_numpy(pos).cuda(), float(int(3e8 / freq)), ordered=True,
                                         rounding=True)
    S = pos.shape[0]
    ours = torch.stack([u, v, w], -1).cpu().numpy().reshape(S, -1, 3).transpose(1, 0, 2)
    assert np.array_equal(ours.astype(np.int64), z[f"{tag}_uvw"].astype(np.int64))


def test_shade_windows_vs_reference_kernels(V):
    """Given the mean radius the fixture's reference run used, every window end equals
    the reference kernels' (integers: no mismatch allowed)."""
    z = load("ref_shade.npz")
    u, v, w = (cu(z[k]) for k in ("u", "v", "w"))
    for RES in (2094, 20940, 62820):
        ours, _ = V.shade_windows(u, v, w, RES, mean_r_km=float(z["mean_r"]))
        assert np.array_equal(ours.cpu().numpy(), z[f"shade_{RES}"]), RES


def test_bench_workload_accuracy(V, oracle):
    """The bench configuration (10 MHz, 1.84M uvw x 196,608 pixels, geometric mask)
    against FP64 on 48 sampled visibilities (all pixels) and 12 sampled pixels
    (all visibilities): <= 1e-5 normwise relative error."""
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS["cfg2_10MHz"]
    d = make_uvw(wl)
    l, m, n, b = make_sky(wl)
    cfg = V.DftConfig.geometric(precision=V.PREC_FAST, occluded_value=0.0)
    args = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    Vg = V.vis_dft(cfg, d["u"], d["v"], d["w"], cu(l), cu(m), cu(n), cu(b), **args)
    Fg = V.recon(cfg, d["u"], d["v"], d["w"], Vg, cu(l), cu(m), cu(n), **args)
    h = lambda x: x.cpu().numpy()  # noqa: E731
    u, v, w, snap, pair, pos = (h(d[k]) for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    K, J = u.size, l.size
    oc = oracle.make_cfg(mask_mode=3, phase_scale=1.0, n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    rows = np.linspace(0, K - 1, 48).astype(np.int64)
    Vo = oracle.vis_dft(oc, u[rows], v[rows], w[rows], l, m, n, b, geo=oracle.make_geo(pos, snap[rows], pair[rows]))
    ev = nerr(h(Vg)[rows], Vo)
    pix = np.linspace(0, J - 1, 12).astype(np.int64)
    Fo = oracle.recon(oc, u, v, w, None, h(Vg), l[pix], m[pix], n[pix], geo=oracle.make_geo(pos, snap, pair))
    ef = nerr(h(Fg)[pix], Fo)
    assert ev < 1e-5 and ef < 1e-5, (ev, ef)
