"""Generate the golden fixtures that pin the oracle to the reference.

Runs the reference's own CUDA kernels (built unmodified from the reference
sources by oracle/build_ref.sh; launched by oracle/ref_cuda.py) on seeded
synthetic inputs and stores inputs + outputs as .npz next to this script:

  ref_vis_recon.npz  visscal / imagerecon of vissGen10M_shade (plain),
                     vissGen10M_shade_optim1/_optim2 and vissGen1M_shade_optim1
  ref_orbit.npz      calculateOrbit + uvwPosition + computeUVW (MIncline)
  ref_shade.npz      Cart2SphKernel + ShadeMatrix (shade1M)
  ref_nxq.npz        computeLocCount + computeLocViss (vissGen1M_shade_optim1)

Usage (needs a GPU and the images in oracle/_ref):
    python tests/golden/make_golden.py [outdir]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_cuda  # noqa: E402

R1 = [0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3]   # MIncline_generate_uvw_float.cu:29
R2 = [0, 0.1e3, 0.445e3, 0.6e3, 0.91e3, 1.62e3, 3.53e3, 10e3]  # :30


def fibonacci_sphere(J: int):
    i = np.arange(J, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / J
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = np.pi * (3.0 - np.sqrt(5.0)) * i
    return (r * np.cos(phi)).astype(np.float32), (r * np.sin(phi)).astype(np.float32), z.astype(np.float32)


def synth_vis_case(seed: int, K: int, J: int, res: int, sigma: float):
    rng = np.random.default_rng(seed)
    u, v, w = (np.ceil(rng.normal(0.0, sigma, K)).astype(np.float32) for _ in range(3))
    l, m, n = fibonacci_sphere(J)
    FF = rng.lognormal(0.0, 1.0, J).astype(np.float32) * 50.0
    freq = rng.integers(1, 6, K).astype(np.float32)
    wgt = (1.0 / freq).astype(np.float32)
    # normalised shade windows (M1 <= M2, M3 <= M4, 0-based): a third with
    # M3 == 0 so the reference's window loop runs; some with both ratios > 0.5
    # so the reference recon mask fires on pixel res + 1.
    M1 = rng.integers(0, res - 1, K)
    M2 = np.minimum(res - 1, M1 + rng.integers(0, res // 2, K))
    M3 = np.where(rng.random(K) < 0.35, 0, rng.integers(0, res - 1, K))
    M4 = np.minimum(res - 1, M3 + rng.integers(0, 8, K))
    sel = rng.random(K) < 0.15
    M2[sel] = rng.integers(2, res - 1, sel.sum())
    M1[sel] = M2[sel] - rng.integers(0, 1 + M2[sel] // 3, sel.sum())
    M4[sel] = rng.integers(2, res - 1, sel.sum())
    M3[sel] = M4[sel] - rng.integers(0, 1 + M4[sel] // 3, sel.sum())
    shade = np.stack([M1, M2, M3, M4], -1).astype(np.int32)
    return dict(u=u, v=v, w=w, l=l, m=m, n=n, FF=FF, wgt=wgt, shade=shade, res=np.int32(res))


def run_vis_recon(case: dict, prefix: str, out: dict):
    import torch
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in case.items() if isinstance(v, np.ndarray) and v.ndim}
    K, J, res = case["u"].size, case["l"].size, int(case["res"])
    M = [t["shade"][:, i].contiguous() for i in range(4)]
    countLoc = torch.ones(J, dtype=torch.int32, device="cuda")
    nxq_f = torch.arange(J, dtype=torch.float32, device="cuda")
    nxq_i = torch.arange(J, dtype=torch.int32, device="cuda")
    for variant, nxq in (("vissGen10M_shade", nxq_f), ("vissGen10M_shade_optim1", nxq_f),
                         ("vissGen10M_shade_optim2", nxq_f), ("vissGen1M_shade_optim1", nxq_i)):
        viss = ref_cuda.visscal(variant, K, J, res, t["FF"], t["u"], t["v"], t["w"], t["l"], t["m"], t["n"],
                                *M, nxq, countLoc)
        # optim2's recon is launched with 128-thread blocks (J is a multiple of
        # 128) so none of its threads leaves before the tile barrier.
        F = ref_cuda.imagerecon(variant, K, J, res, viss, t["u"], t["v"], t["w"], t["l"], t["m"], t["n"],
                                t["wgt"], *M, block=128 if variant.endswith("optim2") else None)
        torch.cuda.synchronize()
        out[f"{prefix}_{variant}_viss"] = viss.cpu().numpy()
        out[f"{prefix}_{variant}_F"] = F.cpu().numpy()
    for k, v in case.items():
        out[f"{prefix}_in_{k}"] = v


def main(outdir: Path):
    import torch
    outdir.mkdir(parents=True, exist_ok=True)
    assert torch.cuda.is_available()

    # -- vis / recon ---------------------------------------------------------
    out = {}
    run_vis_recon(synth_vis_case(1, 1024, 384, 64, 300.0), "lo", out)     # 1 MHz-like |uvw|
    run_vis_recon(synth_vis_case(2, 1024, 1536, 256, 2000.0), "hi", out)  # 10 MHz-like |uvw|
    np.savez_compressed(outdir / "ref_vis_recon.npz", **out)

    # -- orbit / uvw -----------------------------------------------------------
    out = {}
    for tag, (orbit_res, orbit_counts, index, freq) in {"a": (360, 30, 2, 1e7), "b": (360, 40, 1, 1e6)}.items():
        (xt, yt, zt), uvw = ref_cuda.orbit_uvw(8, orbit_res, orbit_counts, index, freq, R1, R2)
        out[f"{tag}_cfg"] = np.array([8, orbit_res, orbit_counts, index, freq], np.float64)
        out[f"{tag}_pos"] = torch.stack([xt, yt, zt], -1).permute(1, 0, 2).contiguous().cpu().numpy()
        out[f"{tag}_uvw"] = uvw.cpu().numpy().astype(np.int32)
    out["r1"] = np.array(R1, np.float32)
    out["r2"] = np.array(R2, np.float32)
    np.savez_compressed(outdir / "ref_orbit.npz", **out)

    # -- shade windows ---------------------------------------------------------
    out = {}
    rng = np.random.default_rng(3)
    u, v, w = (np.ceil(rng.normal(0.0, 2000.0, 4096)).astype(np.float32) for _ in range(3))
    r = np.sqrt(u.astype(np.float64) ** 2 + v.astype(np.float64) ** 2 + w.astype(np.float64) ** 2)
    mean_r = float(np.float32(r.mean()))
    for RES in (2094, 20940, 62820):
        tu, tv, tw = (torch.from_numpy(x).cuda() for x in (u, v, w))
        sh, rr = ref_cuda.shade_windows(tu, tv, tw, RES, mean_r)
        out[f"shade_{RES}"] = sh.cpu().numpy()
        out["r_f32"] = rr.cpu().numpy()
    out.update(u=u, v=v, w=w, mean_r=np.float64(mean_r))
    np.savez_compressed(outdir / "ref_shade.npz", **out)

    # -- NX -> countLoc / NXq ---------------------------------------------------
    rng = np.random.default_rng(4)
    J, X = 300, 2400
    NX = (rng.integers(0, J, X) + 1).astype(np.float32)
    cl, nq = ref_cuda.nxq(torch.from_numpy(NX).cuda(), J)
    np.savez_compressed(outdir / "ref_nxq.npz", NX=NX, J=np.int32(J), countLoc=cl.cpu().numpy(),
                        NXq=nq.cpu().numpy())
    print("golden fixtures written to", outdir)


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
