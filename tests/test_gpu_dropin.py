"""The drop-in programs (bin/vissGen10M_shade, vissGen1M_shade_optim1, shade10M,
MIncline_generate_uvw_float) on a synthetic tree in the reference's layout:
outputs land where the reference writes them and match the oracle and, where
the reference's kernels can run (oracle/_ref), the reference's own results on
the same inputs (integer outputs byte for byte)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
BIN = Path(__file__).resolve().parents[1] / "viss_recon_shade_gb300" / "_lib" / "bin"


def write_col(path, vals, header=None):
    with open(path, "w") as f:
        if header is not None:
            f.write(f"{header}\n")
        for x in vals:
            f.write(f"{np.float32(x):g}\n")


def read_col(path):
    return np.loadtxt(path, dtype=np.float64, ndmin=1)


def make_sky_dir(d, J, seed=0):
    from viss_recon_shade_gb300.synth import fibonacci_sphere, lognormal_sky
    l, m, n = fibonacci_sphere(J)
    FF = lognormal_sky(J, seed=seed) * 10
    d.mkdir(parents=True, exist_ok=True)
    write_col(d / "l.txt", l, header=J)
    write_col(d / "m.txt", m)
    write_col(d / "n.txt", n)
    write_col(d / "C.txt", FF)
    write_col(d / "NX.txt", np.arange(1, J + 1))
    write_col(d / "FF.txt", FF, header=J)
    # values as the programs read them back (6 significant digits)
    return [read_col(d / f).astype(np.float32)[1 if f in ("l.txt", "FF.txt") else 0:]
            for f in ("l.txt", "m.txt", "n.txt", "FF.txt")]


def synth_uvw_shade(K, res, seed=1):
    rng = np.random.default_rng(seed)
    u, v, w = (np.ceil(rng.normal(0, 500, K)).astype(np.float32) for _ in range(3))
    raw = np.stack([rng.integers(1, res, K), rng.integers(1, res, K), np.where(rng.random(K) < 0.4, 1, rng.integers(1, 6, K)),
                    rng.integers(1, 8, K)], -1).astype(np.int32)
    return u, v, w, raw


def read_sidecar(path):
    """The drop-in programs' binary sidecar: 'VISS', version, type (1 = complex64), reserved, int64 count."""
    raw = Path(path).read_bytes()
    hdr = np.frombuffer(raw[:16], np.uint32)
    assert hdr[0] == 0x53534956 and hdr[1] == 1 and hdr[2] == 1
    n = int(np.frombuffer(raw[16:24], np.int64)[0])
    return np.frombuffer(raw[24:], np.complex64, count=n)


def run(args, cwd):
    r = subprocess.run([str(a) for a in args], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_vissGen10M_shade_dropin(oracle, tmp_path):
    J, K, res = 1536, 2048, 256
    l, m, n, FF = make_sky_dir(tmp_path / "lmn10M", J)
    write_col(tmp_path / "lmn10M" / "countLoc.txt", np.ones(J))
    write_col(tmp_path / "lmn10M" / "NXq.txt", np.arange(J))
    u, v, w, raw = synth_uvw_shade(K, res)
    freq = np.random.default_rng(2).integers(1, 5, K).astype(np.float32)
    fd = tmp_path / "frequency_10M"
    fd.mkdir()
    np.savetxt(fd / "updated_uvw1frequency10M.txt", np.stack([u, v, w, freq], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency10M.txt", raw, fmt="%d")
    out = run([BIN / "vissGen10M_shade", "--res", res, "--sidecar"], tmp_path)
    assert "Compute Viss Cost Time" in out
    F = read_col(tmp_path / "F_recon_10M" / "F1period10M.txt")
    Fs = read_sidecar(tmp_path / "F_recon_10M" / "F1period10M.F.c64")
    Vs = read_sidecar(tmp_path / "F_recon_10M" / "F1period10M.V.c64")
    assert Fs.shape == (J,) and Vs.shape == (K,)
    assert np.abs(F - Fs.real).max() <= 1e-5 * np.abs(Fs.real).max()  # the text keeps 6 digits
    M = oracle.normalise_shade(raw)
    ncl = np.clip(n, -1, 1)
    V = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=res, trunc=True, occluded_value=240.0), u, v, w, l, m, ncl, FF,
                       shade=M)
    Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, 1.0 / freq,
                      V.astype(np.complex64), l, m, ncl, shade=M)
    assert F.shape == (J,)
    assert np.abs(F - Fo.real).max() / np.abs(Fo.real).max() < 2e-5
    assert np.abs(Fs - Fo).max() / np.abs(Fo).max() < 2e-5
    # the reference's own kernels on the inputs its main would pass them (the files as
    # parsed, n clipped to [-1, 1] (:308), normalised windows, 1/freq weights): our F
    # file is as close to FP64 as theirs, value for value
    from oracle import ref_cuda
    if ref_cuda.available():
        import torch
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
        Ms = [torch.from_numpy(np.ascontiguousarray(M[:, i])).cuda() for i in range(4)]
        args = (t(u), t(v), t(w), t(l), t(m), t(ncl))
        viss = ref_cuda.visscal("vissGen10M_shade", K, J, res, t(FF), *args, *Ms,
                                torch.arange(J, dtype=torch.float32, device="cuda"),
                                torch.ones(J, dtype=torch.int32, device="cuda"))
        Fr = ref_cuda.imagerecon("vissGen10M_shade", K, J, res, viss, *args, t(1.0 / freq), *Ms)[:, 0].cpu().numpy()
        scale = np.abs(Fo.real).max()
        assert np.abs(F - Fo.real).max() / scale <= 1.5 * np.abs(Fr - Fo.real).max() / scale + 1e-5
    # optim2 naming and period loop (days/start-period flags as in its main)
    run([BIN / "vissGen10M_shade_optim2", "--res", res, "--start-period", 0, "--days", 1], tmp_path)
    assert (tmp_path / "F_recon_10M" / "F1period10M_optim2.txt").exists()


def test_vissGen10M_resume_skips_complete_periods(tmp_path):
    """--resume: periods whose F_recon file already holds all J lines are skipped;
    a truncated file (an interrupted run elsewhere) is recomputed, to the same bytes."""
    J, K, res = 1024, 1024, 128
    make_sky_dir(tmp_path / "lmn10M", J)
    write_col(tmp_path / "lmn10M" / "countLoc.txt", np.ones(J))
    write_col(tmp_path / "lmn10M" / "NXq.txt", np.arange(J))
    fd = tmp_path / "frequency_10M"
    fd.mkdir()
    for p in (1, 2, 3):
        u, v, w, raw = synth_uvw_shade(K, res, seed=10 + p)
        np.savetxt(fd / f"updated_uvw{p}frequency10M.txt", np.stack([u, v, w, np.ones(K)], -1), fmt="%g")
        np.savetxt(fd / f"shadeM{p}frequency10M.txt", raw, fmt="%d")
    args = [BIN / "vissGen10M_shade", "--res", res, "--days", 3]
    run(args, tmp_path)
    outs = [tmp_path / "F_recon_10M" / f"F{p}period10M.txt" for p in (1, 2, 3)]
    full = [o.read_bytes() for o in outs]
    assert not list((tmp_path / "F_recon_10M").glob("*.part"))
    outs[1].write_bytes(full[1][: len(full[1]) // 2])  # period 2 interrupted half way
    outs[2].unlink()                                   # period 3 never written
    log = run(args + ["--resume", 1], tmp_path)
    assert "F1period10M.txt complete, skipped" in log and log.count("complete, skipped") == 1
    assert [o.read_bytes() for o in outs] == full


def test_vissGen1M_dropin_weights_and_expansion(oracle, tmp_path):
    J, K, res = 1024, 1024, 128
    fd = tmp_path / "frequency_1M"
    l, m, n, FF = make_sky_dir(fd, J, seed=3)
    u, v, w, raw = synth_uvw_shade(K, res, seed=4)
    np.savetxt(fd / "uvw1frequency1M.txt", np.stack([u, v, w], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency1M.txt", raw, fmt="%d")
    cnt = np.random.default_rng(5).integers(1, 6, K)
    keep = np.arange(K) % 3 != 0  # a third of the uvw are absent from the map: weight 1
    with open(fd / "uvwMap130.txt", "w") as f:
        f.write(f"{keep.sum()}\n")
        for k in np.nonzero(keep)[0]:
            f.write(f"{int(u[k])} {int(v[k])} {int(w[k])} {cnt[k]}\n")
    run([BIN / "vissGen1M_shade_optim1", "--res", res], tmp_path)
    F = read_col(tmp_path / "F_recon_1M" / "F1_optim1.txt")
    M = oracle.normalise_shade(raw)
    wgt = np.where(keep, 1.0 / cnt, 1.0).astype(np.float32)
    V = oracle.vis_dft(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0), u, v, w, l, m, n, FF, shade=M)
    Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, wgt, V.astype(np.complex64),
                      l, m, n, shade=M)
    assert np.abs(F - Fo.real).max() / np.abs(Fo.real).max() < 2e-5


def _ref_kernels():
    from oracle import ref_cuda, ref_thrust
    if not ref_cuda.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    ref_thrust.build()
    return ref_cuda, ref_thrust


def test_shade10M_dropin(tmp_path):
    """shade10M on a file tree: the shadeM file equals, window end for window end, what
    the reference's pipeline gives on the same rows (its Cart2SphKernel and ShadeMatrix
    from its sources, its thrust mean restated, r0 by the host's atanf)."""
    import torch
    refk, RT = _ref_kernels()
    K = 40000
    u, v, w, _ = synth_uvw_shade(K, 100, seed=6)
    fd = tmp_path / "frequency_10M"
    fd.mkdir()
    np.savetxt(fd / "updated_uvw2frequency10M.txt", np.stack([u, v, w, np.ones(K)], -1), fmt="%g")
    run([BIN / "shade10M", "--last", 2], tmp_path)
    ours = np.loadtxt(fd / "shadeM2frequency10M.txt", dtype=np.int64)
    tu, tv, tw = (torch.from_numpy(x).cuda() for x in (u, v, w))
    _, mean_r = RT.mean_r(refk.cart2sph_r(tu, tv, tw))
    ref = refk.shade_windows(tu, tv, tw, 20940, mean_r)[0].cpu().numpy()
    assert np.array_equal(ours, ref)


def test_mincline_dropin(tmp_path):
    """MIncline_generate_uvw_float on a small orbit grid: the uvw file equals, byte for
    byte, the reference's rows written as its writer writes them (`u v w`, std::ostream
    default format, MIncline_generate_uvw_float.cu:421-427).  Reference rows: its
    calculateOrbit / uvwPosition / computeUVW kernels from its sources, then its
    per-pair sort + unique, concatenation and global sort + unique (thrust, restated)."""
    refk, _ = _ref_kernels()
    run([BIN / "MIncline_generate_uvw_float", "--periods", 1, "--orbit-res", 720, "--orbit-counts", 3], tmp_path)
    ours = (tmp_path / "frequency_10M" / "uvw1frequency10M.txt").read_text()
    r1 = [0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3]
    r2 = [0, 0.1e3, 0.445e3, 0.6e3, 0.91e3, 1.62e3, 3.53e3, 10e3]
    glob = refk.mincline_unique(8, 720, 3, 1, 1e7, r1, r2).cpu().numpy()
    ref = "".join(f"{np.float32(a):g} {np.float32(b):g} {np.float32(c):g}\n" for a, b, c in glob.tolist())
    assert ours == ref


def make_map_sky_dir(d, res, seed=7):
    """A res x res fine grid (FF) mapped onto (res/2)^2 coarse pixels (2 x 2 blocks,
    some fine pixels moved): NX plus, for the 10M layout, countLoc and NXq."""
    from viss_recon_shade_gb300.synth import fibonacci_sphere
    rng = np.random.default_rng(seed)
    X = res * res
    q, r = np.divmod(np.arange(X), res)
    coarse = (q // 2) * (res // 2) + (r // 2)
    J = (res // 2) ** 2
    moved = rng.choice(X, X // 40, replace=False)
    coarse[moved] = rng.integers(0, J, moved.size)
    coarse[coarse == 0] = 1
    coarse[5] = 0
    l, m, n = fibonacci_sphere(J)
    FF = rng.lognormal(3.0, 1.0, X).astype(np.float32)
    d.mkdir(parents=True, exist_ok=True)
    write_col(d / "l.txt", l, header=J)
    write_col(d / "m.txt", m)
    write_col(d / "n.txt", n)
    write_col(d / "C.txt", np.zeros(J))
    write_col(d / "NX.txt", coarse + 1)
    write_col(d / "FF.txt", FF, header=X)
    l, m, n = (read_col(d / f).astype(np.float32) for f in ("l.txt", "m.txt", "n.txt"))
    return l[1:], m, n, read_col(d / "FF.txt").astype(np.float32)[1:], (coarse + 1).astype(np.float32), J


def test_vissGen10M_shade_fine_map(oracle, tmp_path):
    res, K = 64, 1024
    l, m, n, FF, NX, J = make_map_sky_dir(tmp_path / "lmn10M", res)
    cl, nq = oracle.nxq(NX, J)
    write_col(tmp_path / "lmn10M" / "countLoc.txt", cl)
    write_col(tmp_path / "lmn10M" / "NXq.txt", nq)
    u, v, w, raw = synth_uvw_shade(K, res, seed=8)
    fd = tmp_path / "frequency_10M"
    fd.mkdir()
    np.savetxt(fd / "updated_uvw1frequency10M.txt", np.stack([u, v, w, np.full(K, 2.0)], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency10M.txt", raw, fmt="%d")
    run([BIN / "vissGen10M_shade", "--res", res], tmp_path)
    F = read_col(tmp_path / "F_recon_10M" / "F1period10M.txt")
    M = oracle.normalise_shade(raw)
    ncl = np.clip(n, -1, 1)
    V = oracle.vis_dft_nxq(oracle.make_cfg(mask_mode=1, res=res, trunc=True, occluded_value=240.0), u, v, w, l, m, ncl,
                           FF, nq.astype(np.float32), cl, shade=M)
    Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, np.full(K, 0.5, np.float32),
                      V.astype(np.complex64), l, m, ncl, shade=M)
    assert F.shape == (J,)
    assert np.abs(F - Fo.real).max() / np.abs(Fo.real).max() < 2e-5


def test_vissGen1M_fine_map(oracle, tmp_path):
    res, K = 64, 1024
    fd = tmp_path / "frequency_1M"
    l, m, n, FF, NX, J = make_map_sky_dir(fd, res, seed=9)
    u, v, w, raw = synth_uvw_shade(K, res, seed=10)
    np.savetxt(fd / "uvw1frequency1M.txt", np.stack([u, v, w], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency1M.txt", raw, fmt="%d")
    run([BIN / "vissGen1M_shade_optim1", "--res", res], tmp_path)
    F = read_col(tmp_path / "F_recon_1M" / "F1_optim1.txt")
    cl, nq = oracle.nxq(NX, J)
    M = oracle.normalise_shade(raw)
    V = oracle.vis_dft_nxq(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0), u, v, w, l, m, n, FF,
                           nq.astype(np.float32), cl, shade=M)
    Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, None,
                      V.astype(np.complex64), l, m, n, shade=M)
    Ffine = Fo.real[NX.astype(np.int64) - 1]  # expanded to the fine grid
    assert F.shape == (res * res,)
    assert np.abs(F - Ffine).max() / np.abs(Ffine).max() < 2e-5


def test_vissGen1M_shade_accurate_dropin(oracle, tmp_path):
    """vissGen1M_shade_accurate: the 1M fine-map flow with the fine brightness truncated
    to int (vissGen1M_shade_accurate.cu:115), written expanded as
    F_recon_1M_accu/Ex{p}frequency1M.txt (:571-585)."""
    res, K = 64, 1024
    fd = tmp_path / "frequency_1M"
    l, m, n, FF, NX, J = make_map_sky_dir(fd, res, seed=13)
    u, v, w, raw = synth_uvw_shade(K, res, seed=14)
    np.savetxt(fd / "uvw1frequency1M.txt", np.stack([u, v, w], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency1M.txt", raw, fmt="%d")
    run([BIN / "vissGen1M_shade_accurate", "--res", res], tmp_path)
    F = read_col(tmp_path / "F_recon_1M_accu" / "Ex1frequency1M.txt")
    cl, nq = oracle.nxq(NX, J)
    M = oracle.normalise_shade(raw)
    V = oracle.vis_dft_nxq(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0, trunc=True), u, v, w, l, m, n,
                           FF, nq.astype(np.float32), cl, shade=M)
    Fo = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0 / K), u, v, w, None,
                      V.astype(np.complex64), l, m, n, shade=M)
    Ffine = Fo.real[NX.astype(np.int64) - 1]
    assert F.shape == (res * res,)
    assert np.abs(F - Ffine).max() / np.abs(Ffine).max() < 2e-5
    # the truncation matters on this sky: the untruncated brightness gives another image
    V2 = oracle.vis_dft_nxq(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0), u, v, w, l, m, n, FF,
                            nq.astype(np.float32), cl, shade=M)
    assert np.abs(V2 - V).max() > 1e-3 * np.abs(V).max()


def test_vissGen1M_shade_appro_dropin(oracle, tmp_path):
    """vissGen1M_shade_appro: coarse brightness C_j = mean of FF over NX == j + 1
    (computeC), the window tested on NX[j] - 1 (the fine-array entry at the coarse
    index, vissGen1M_shade_appro.cu:113-118; the 240 replaces C_j for that term only,
    the reference's shared write being a race), d = (float)2 RES / (RES - 1), no recon
    mask, F / K expanded as F_recon_1M_appro/Ex{p}frequency1M.txt."""
    res, K = 64, 1024
    fd = tmp_path / "frequency_1M"
    l, m, n, FF, NX, J = make_map_sky_dir(fd, res, seed=15)
    u, v, w, raw = synth_uvw_shade(K, res, seed=16)
    np.savetxt(fd / "uvw1frequency1M.txt", np.stack([u, v, w], -1), fmt="%g")
    np.savetxt(fd / "shadeM1frequency1M.txt", raw, fmt="%d")
    run([BIN / "vissGen1M_shade_appro", "--res", res], tmp_path)
    F = read_col(tmp_path / "F_recon_1M_appro" / "Ex1frequency1M.txt")
    csum = np.zeros(J, np.float32)
    cnt = np.zeros(J, np.int64)
    for i in range(NX.size):  # float sums in fine-index order, as computeC
        q = int(NX[i]) - 1
        csum[q] = np.float32(csum[q] + FF[i])
        cnt[q] += 1
    C = np.where(cnt > 0, csum / np.maximum(cnt, 1).astype(np.float32), 0).astype(np.float32)
    widx = (NX[:J].astype(np.int64) - 1).astype(np.int32)
    d = float(np.float32(2 * res) / np.float32(res - 1))
    M = oracle.normalise_shade(raw)
    Vo = oracle.vis_dft_windex(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0, phase_scale=1.0 / d,
                                               n_offset=0.0), u, v, w, l, m, n, C, M, widx)
    Fo = oracle.recon(oracle.make_cfg(phase_scale=1.0 / d, n_offset=0.0, norm=1.0 / K), u, v, w, None,
                      Vo.astype(np.complex64), l, m, n)
    Ffine = Fo.real[NX.astype(np.int64) - 1]
    assert F.shape == (res * res,)
    assert np.abs(F - Ffine).max() / np.abs(Ffine).max() < 2e-5
    # the window on NX[j] - 1 is not the window on j: the masks differ on this sky
    Vj = oracle.vis_dft_windex(oracle.make_cfg(mask_mode=1, res=res, occluded_value=240.0, phase_scale=1.0 / d,
                                               n_offset=0.0), u, v, w, l, m, n, C, M, np.arange(J, dtype=np.int32))
    assert np.abs(Vj - Vo).max() > 1e-3 * np.abs(Vo).max()
