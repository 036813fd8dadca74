"""The Python layer refuses tensors the kernels cannot take (host memory, wrong
dtype or shape, missing) before calling into the library: no GPU needed."""
import pytest

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


def test_stage1_entry_points_refuse_host_tensors(V):
    pos = torch.zeros(4, 8, 3)
    with pytest.raises(TypeError, match="CUDA"):
        V.baseline_uvw(pos, 30.0)
    with pytest.raises(TypeError, match="CUDA"):
        V.unique_uvw(pos, 30.0)
    x = torch.zeros(10)
    with pytest.raises(TypeError, match="CUDA"):
        V.dedup_uvw(x, x, x)
    with pytest.raises(TypeError, match="CUDA"):
        V.shade_windows(x, x, x, 64)
    with pytest.raises(TypeError, match="CUDA"):
        V.orbit_positions(V.OrbitConfig(orbit_res=3600, orbit_counts=1), device="cpu")


def test_missing_and_misshapen_arguments(V):
    with pytest.raises(TypeError, match="required"):
        V.dedup_uvw(None, None, None)
    with pytest.raises(TypeError, match="required"):
        V.unique_uvw(None, 30.0)
    with pytest.raises(TypeError, match="required"):
        V.shade_windows(None, None, None, 64)


def test_dft_entry_points_refuse_host_tensors(V):
    x = torch.zeros(8)
    cfg = V.DftConfig.geometric().with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE)
    with pytest.raises(TypeError, match="CUDA"):
        V.vis_dft(cfg, x, x, x, x, x, x, x)
    with pytest.raises(TypeError, match="CUDA"):
        V.recon(cfg, x, x, x, torch.zeros(8, dtype=torch.complex64), x, x, x)
