"""Shade windows (stage 2: Cart2SphKernel + mean radius + ShadeMatrix) bit for bit
against the reference's own kernels, run live from its sources (oracle/ref_cuda.py),
and its FP32 mean-radius sum restated with the same thrust call (oracle/ref_thrust.cu).

Windows are integers: no mismatch is allowed.  The mean radius is the reference's
order-dependent FP32 sum; the product reproduces its order, so it is compared exactly
too, in a test of its own."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refk():
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    return ref_cuda


@pytest.fixture(scope="module")
def RT():
    from oracle import ref_thrust
    ref_thrust.build()
    return ref_thrust


def _uvw_sets():
    """(name, u, v, w): integer-valued uvw from the product's stage 1 (the rows the
    reference's shade programs read) and the continuous 10 MHz bench uvw."""
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300.synth import WORKLOADS, make_uvw
    cfg = V.OrbitConfig(orbit_res=86400, orbit_counts=20)  # the MIncline constants, 576,000 snapshots
    pos = V.orbit_positions(cfg)
    uu, vv, ww = V.unique_uvw(pos, 30.0, ordered=True)
    yield "mincline_unique_10MHz", uu, vv, ww
    d = make_uvw(WORKLOADS["cfg2_10MHz"])
    yield "cfg2_10MHz", d["u"], d["v"], d["w"]


def test_shade_mean_radius_is_the_reference_fp32_sum(refk, RT):
    """The reference sums r in FP32 with thrust (shade1M.cu:219); the sum depends on the
    order.  Ours uses the same reduction and must give the same float, at sizes from one
    tile to tens of millions of rows."""
    import viss_recon_shade_gb300 as V
    g = torch.Generator(device="cuda").manual_seed(5)
    for K in (1, 777, 4096, 100_003, 1 << 20, 14_336_001):
        u, v, w = (torch.randn(K, device="cuda", generator=g).mul_(3000).ceil_() for _ in range(3))
        r = refk.cart2sph_r(u, v, w)
        s_ref, m_ref = RT.mean_r(r)
        _, m_ours = V.shade_windows(u, v, w, 20940)
        assert np.float32(m_ours) == np.float32(m_ref), (K, m_ours, m_ref, s_ref)


def test_shade_windows_bit_exact_vs_reference_kernels(refk, RT):
    """Whole pipelines side by side on millions of rows: the reference's Cart2SphKernel,
    thrust mean and ShadeMatrix (r0 by the host's atanf) against viss_shade_windows
    computing its own mean radius.  Every window end must be equal."""
    import viss_recon_shade_gb300 as V
    for name, u, v, w in _uvw_sets():
        r = refk.cart2sph_r(u, v, w)
        _, mean_r = RT.mean_r(r)
        for RES in (2094, 20940, 62820):
            ref = refk.shade_windows(u, v, w, RES, mean_r)[0].cpu().numpy()
            ours, m = V.shade_windows(u, v, w, RES)
            assert np.float32(m) == np.float32(mean_r), (name, m, mean_r)
            ours = ours.cpu().numpy()
            bad = np.flatnonzero(np.any(ours != ref, axis=1))
            assert bad.size == 0, (name, RES, u.numel(), bad.size, bad[:5], ours[bad[:5]], ref[bad[:5]])


def test_normalised_windows_bit_exact(refk, RT):
    """shadeM normalisation on load (vissGen10M_shade.cu:383-399) of the reference's windows."""
    import viss_recon_shade_gb300 as V
    from oracle import oracle as O
    _, u, v, w = next(_uvw_sets())
    _, mean_r = RT.mean_r(refk.cart2sph_r(u, v, w))
    raw = refk.shade_windows(u, v, w, 20940, mean_r)[0]
    M = V.normalise_shade(raw.contiguous()).cpu().numpy()
    assert np.array_equal(M, O.normalise_shade(raw.cpu().numpy()))
