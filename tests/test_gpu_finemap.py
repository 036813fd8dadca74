"""Non-identity fine->coarse sky maps (vissGen10M_shade.cu:120-136 with
countLoc/NXq; vissGen1M_shade_optim1.cu:54-115 for NX -> NXq).

A 96 x 96 fine grid (X = 9,216) is mapped onto 2,304 coarse pixels, mostly
2 x 2 blocks with a few fine pixels moved to other blocks and one coarse pixel
of a single member.  Checked against the oracle:
  viss_nxq:       countLoc and NXq bit-exact (the oracle is pinned to the
                  reference's computeLocCount / computeLocViss outputs)
  FAST map path:  <= 1e-5 normwise relative to FP64 (REF quirk and intended
                  windows, float brightness and the int-truncated variant)
  PLAIN map path: the reference's FP32 member loop, <= 5e-3 (FP32 phase)
The windows cut through coarse pixels, so the exact member loop runs as well as
the box decisions."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RES = 96


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def fmap():
    rng = np.random.default_rng(11)
    q, r = np.divmod(np.arange(RES * RES), RES)
    coarse = (q // 2) * (RES // 2) + (r // 2)
    J = (RES // 2) ** 2
    moved = rng.choice(RES * RES, 200, replace=False)
    coarse[moved] = rng.integers(0, J, moved.size)
    coarse[coarse == 5] = 6
    coarse[17] = 5  # coarse pixel 5: a single member
    assert np.all(np.bincount(coarse, minlength=J) > 0)
    NX = (coarse + 1).astype(np.float32)
    FF = rng.lognormal(3.0, 1.0, RES * RES).astype(np.float32)
    from viss_recon_shade_gb300.synth import fibonacci_sphere
    l, m, n = fibonacci_sphere(J)
    K = 1500
    u, v, w = (np.ceil(rng.normal(0, 40, K)).astype(np.float32) for _ in range(3))
    M1 = rng.integers(-1, RES - 2, K)
    M2 = np.minimum(RES, M1 + rng.integers(2, RES // 2, K))
    M3 = rng.integers(-RES // 4, RES // 2, K)
    M4 = M3 + rng.integers(0, RES // 3, K)
    shade = np.stack([M1, M2, M3, M4], 1).astype(np.int32)
    return dict(NX=NX, FF=FF, J=J, l=l, m=m, n=n, u=u, v=v, w=w, shade=shade)


def test_nxq_matches_oracle(fmap, oracle):
    import viss_recon_shade_gb300 as V
    NX = fmap["NX"].copy()
    NX[[3, 40]] = [0.0, 1e9]  # no coarse pixel: excluded, as the reference's float test does
    cl, nq = V.nxq(cu(NX), fmap["J"])
    cl_o, nq_o = oracle.nxq(NX, fmap["J"])
    cl, nq = cl.cpu().numpy(), nq.cpu().numpy()
    assert np.array_equal(cl, cl_o)
    tot = int(cl_o.sum())
    assert tot == NX.size - 2
    assert np.array_equal(nq[:tot], nq_o[:tot])


@pytest.mark.parametrize("mask", ["quirk", "intended"])
@pytest.mark.parametrize("trunc", [False, True])
def test_map_vis_fast_and_plain(fmap, oracle, mask, trunc):
    import viss_recon_shade_gb300 as V
    mm = {"quirk": V.MASK_REF_QUIRK, "intended": V.MASK_REF_INTENDED}[mask]
    cl_o, nq_o = oracle.nxq(fmap["NX"], fmap["J"])
    oc = oracle.make_cfg(mask_mode=mm, res=RES, trunc=trunc, occluded_value=240.0, phase_scale=0.5, n_offset=0.0)
    Vo = oracle.vis_dft_nxq(oc, fmap["u"], fmap["v"], fmap["w"], fmap["l"], fmap["m"], fmap["n"], fmap["FF"],
                            nq_o.astype(np.float32), cl_o, shade=fmap["shade"])
    args = [cu(fmap[k]) for k in ("u", "v", "w", "l", "m", "n", "FF")]
    variant = V.VARIANT_PLAIN if trunc else V.VARIANT_OPTIM
    for prec, tol in ((V.PREC_FAST, 1e-5), (V.PREC_COMPENSATED, 1e-5), (V.PREC_PLAIN, 5e-3)):
        cfg = V.DftConfig.reference(RES, variant=variant, precision=prec, mask=mm)
        for nxq_dev in (cu(nq_o.astype(np.float32)), cu(nq_o)):  # 10M float files / in-program int
            Vg = V.vis_dft_map(cfg, *args, nxq_dev, cu(cl_o), shade=cu(fmap["shade"])).cpu().numpy()
            e = np.linalg.norm(Vg - Vo) / np.linalg.norm(Vo)
            assert e <= tol, (prec, nxq_dev.dtype, e)


def test_visscal_with_map(fmap, oracle):
    """viss_visscal with the reference's NXq (float) / countLoc arguments."""
    import viss_recon_shade_gb300 as V
    cl_o, nq_o = oracle.nxq(fmap["NX"], fmap["J"])
    K, J = fmap["u"].size, fmap["J"]
    oc = oracle.make_cfg(mask_mode=1, res=RES, trunc=False, occluded_value=240.0, phase_scale=0.5, n_offset=0.0)
    Vo = oracle.vis_dft_nxq(oc, fmap["u"], fmap["v"], fmap["w"], fmap["l"], fmap["m"], fmap["n"], fmap["FF"],
                            nq_o.astype(np.float32), cl_o, shade=fmap["shade"])
    viss = torch.zeros(K, dtype=torch.complex64, device="cuda")
    sh = [cu(fmap["shade"][:, i].copy()) for i in range(4)]
    V.visscal(K, J, RES, cu(fmap["FF"]), viss, cu(fmap["u"]), cu(fmap["v"]), cu(fmap["w"]), cu(fmap["l"]),
              cu(fmap["m"]), cu(fmap["n"]), *sh, NXq=cu(nq_o.astype(np.float32)), countLoc=cu(cl_o))
    Vg = viss.cpu().numpy()
    assert np.linalg.norm(Vg - Vo) / np.linalg.norm(Vo) <= 1e-5
