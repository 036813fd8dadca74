"""CPU checks of the oracle itself: brute-force numpy on small cases, the
reference's loop semantics written out literally, and internal identities."""
import numpy as np


def d64(x):
    return np.asarray(x, np.float64)


def small_case(K=40, J=35, sigma=200.0, seed=0):
    rng = np.random.default_rng(seed)
    u, v, w = (np.ceil(rng.normal(0, sigma, K)).astype(np.float32) for _ in range(3))
    l, m, n = (rng.uniform(-1, 1, J).astype(np.float32) for _ in range(3))
    b = rng.uniform(0, 20, J).astype(np.float32)
    return u, v, w, l, m, n, b


def test_vis_matches_bruteforce(oracle):
    u, v, w, l, m, n, b = small_case()
    for s, noff in ((0.5, 0.0), (1.0, -1.0)):
        V = oracle.vis_dft(oracle.make_cfg(phase_scale=s, n_offset=noff), u, v, w, l, m, n, b)
        ph = s * (d64(u)[:, None] * d64(l) + d64(v)[:, None] * d64(m) + d64(w)[:, None] * (d64(n) + noff))
        ref = (d64(b) * np.exp(-2j * np.pi * ph)).sum(1)
        assert np.abs(V - ref).max() / np.abs(ref).max() < 1e-12


def test_reference_trailing_factor_identity(oracle):
    """visscal accumulates exp(-2 pi i (u l + v m + w (n-1))/d) and multiplies by
    exp(-2 pi i w/d) (vissGen10M_shade.cu:137-143): equal to n_offset = 0."""
    u, v, w, l, m, n, b = small_case(seed=1)
    V = oracle.vis_dft(oracle.make_cfg(phase_scale=0.5, n_offset=0.0), u, v, w, l, m, n, b)
    ph = 0.5 * (d64(u)[:, None] * d64(l) + d64(v)[:, None] * d64(m) + d64(w)[:, None] * (d64(n) - 1))
    lit = (d64(b) * np.exp(-2j * np.pi * ph)).sum(1) * np.exp(-2j * np.pi * 0.5 * d64(w))
    assert np.abs(V - lit).max() / np.abs(lit).max() < 1e-12


def test_recon_matches_bruteforce(oracle):
    u, v, w, l, m, n, _ = small_case(seed=2)
    K = u.size
    rng = np.random.default_rng(3)
    Vin = (rng.normal(size=K) + 1j * rng.normal(size=K)).astype(np.complex64)
    wgt = rng.uniform(0.1, 1, K).astype(np.float32)
    F = oracle.recon(oracle.make_cfg(phase_scale=0.5, norm=1.0 / K), u, v, w, wgt, Vin, l, m, n)
    ph = 0.5 * (d64(u)[:, None] * d64(l) + d64(v)[:, None] * d64(m) + d64(w)[:, None] * d64(n))
    ref = ((d64(wgt) * Vin.astype(np.complex128))[:, None] * np.exp(2j * np.pi * ph)).sum(0) / K
    assert np.abs(F - ref).max() / np.abs(ref).max() < 1e-12


def literal_window(i, res, M1, M2, M3, M4):
    """for (lo = 0; lo >= M3 && lo <= M4; ++lo) if (i >= lo*res+M1+1 && i < lo*res+M2) hit
    (vissGen10M_shade.cu:130-134), executed literally."""
    lo = 0
    hit = False
    while lo >= M3 and lo <= M4:
        if lo * res + M1 + 1 <= i < lo * res + M2:
            hit = True
        lo += 1
    return hit


def test_ref_quirk_window_is_the_literal_loop(oracle):
    """The oracle's REF_QUIRK vis mask equals the reference loop run literally,
    including windows that fall outside one row and negative M values."""
    rng = np.random.default_rng(4)
    res = 17
    K, J = 300, 120
    M1 = rng.integers(-5, res + 3, K)
    M2 = M1 + rng.integers(-2, 2 * res, K)
    M3 = rng.integers(-3, 3, K)
    M4 = M3 + rng.integers(-1, 8, K)
    shade = np.stack([M1, M2, M3, M4], -1).astype(np.int32)
    z = np.zeros(K, np.float32)
    l, m, n = (np.zeros(J, np.float32) for _ in range(3))
    V = oracle.vis_dft(oracle.make_cfg(mask_mode=oracle.MASK_REF_QUIRK, res=res, occluded_value=1.0), z, z, z, l, m,
                       n, np.zeros(J, np.float32), shade=shade)
    counts = np.array([sum(literal_window(j, res, *shade[k]) for j in range(J)) for k in range(K)])
    assert np.array_equal(np.round(V.real).astype(int), counts)
    assert counts.max() > 0 and (counts == 0).any()


def test_recon_ref_mask_only_pixel_res_plus_1(oracle):
    """With windows normalised from 1-based files (0 <= M1 <= M2), the reference's
    recon mask (vissGen10M_shade.cu:166) can only skip pixel res + 1."""
    rng = np.random.default_rng(5)
    res, K = 20, 200
    M1 = rng.integers(0, res, K); M2 = M1 + rng.integers(0, res, K)
    M3 = rng.integers(0, res, K); M4 = M3 + rng.integers(0, res, K)
    shade = np.stack([M1, M2, M3, M4], -1).astype(np.int32)
    J = 3 * res
    z = np.zeros(K, np.float32)
    pix = np.zeros(J, np.float32)
    F = oracle.recon(oracle.make_cfg(res=res, recon_ref_mask=True, norm=1.0), z, z, z, None,
                     np.ones(K, np.complex64), pix, pix, pix, shade=shade)
    skipped = K - np.round(F.real).astype(int)
    with np.errstate(invalid="ignore", divide="ignore"):  # 0/0 = NaN never passes > 0.5, as in the reference
        r1 = M1.astype(np.float32) / M2.astype(np.float32)
        r2 = M3.astype(np.float32) / M4.astype(np.float32)
    expect = np.zeros(J, int)
    expect[res + 1] = int(np.sum((r1 > 0.5) & (r2 > 0.5)))
    assert np.array_equal(skipped, expect)


def test_normalise_shade(oracle):
    raw = np.array([[5, 3, 1, 9], [2, 2, 7, 4]], np.int32)
    M = oracle.normalise_shade(raw)
    assert M.tolist() == [[2, 4, 0, 8], [1, 1, 3, 6]]


def test_nxq_inversion(oracle):
    rng = np.random.default_rng(6)
    J, X = 50, 400
    NX = (rng.integers(0, J, X) + 1).astype(np.float32)
    cl, nq = oracle.nxq(NX, J)
    assert cl.sum() == X
    start = np.concatenate([[0], np.cumsum(cl)])
    for q in range(J):
        idx = nq[start[q]:start[q + 1]]
        assert np.array_equal(idx, np.nonzero(NX - 1 == q)[0])


def test_window_index_quirks(oracle):
    """uvwPosition windows (MIncline:113-151) at 360 samples x 30 orbits: the last
    window runs past the end (49 zero-filled samples and one read of the next
    satellite's first sample); at 40 orbits the reset path starts over."""
    r1 = np.array([0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3], np.float32)
    r2 = r1 / 10
    cfg = oracle.make_orbit_cfg(8, 360, 30, r1_m=r1, r2_m=r2)
    pos = oracle.orbit_positions(cfg, mode=1)
    zero = np.all(pos == 0, axis=2)
    # 49 zero-filled samples plus the one-past-the-end read, which lands in the
    # next satellite's slot before the reference has computed it: zero as well
    assert np.all(zero.sum(0) == 50)
    cfg40 = oracle.make_orbit_cfg(8, 360, 40, r1_m=r1, r2_m=r2)
    assert not np.all(oracle.orbit_positions(cfg40, mode=1) == 0, axis=2).any()


def test_orbit_fp32_mimic_close_to_fp64(oracle):
    r1 = np.array([0, 1e3, 4.45e3, 6e3, 9.1e3, 16.2e3, 35.3e3, 100e3], np.float32)
    cfg = oracle.make_orbit_cfg(8, 720, 4, r1_m=r1, r2_m=r1 / 10)
    p32 = oracle.orbit_positions(cfg, mode=1)
    p64 = oracle.orbit_positions_f64(cfg)
    rel = np.abs(p32 - p64).max() / 2038.14
    assert rel < 2e-6
    r = np.linalg.norm(p64, axis=2)
    assert np.allclose(r, 2038.14, rtol=1e-12)


def test_uvw_ceil_and_pairs(oracle):
    rng = np.random.default_rng(7)
    pos = rng.normal(0, 1000, (5, 4, 3)).astype(np.float32)
    u, v, w, snap, pair = oracle.uvw(pos, 30.0, ordered=True, rounding=True)
    assert u.size == 5 * 12
    k = 7
    g, pr = snap[k], pair[k]
    a, b = pr & 0xffff, pr >> 16
    exp = np.ceil((pos[g, b, 0] - pos[g, a, 0]).astype(np.float64) * 1e3 / 30.0)
    assert u[k] == np.float32(exp)
    u2, *_ = oracle.uvw(pos, 30.0, ordered=False, rounding=False)
    assert u2.size == 5 * 6


def test_dedup(oracle):
    u = np.array([3, 1, 3, 1, -0.0, 0.0], np.float32)
    v = np.array([1, 2, 1, 2, 5, 5], np.float32)
    w = np.array([0, 0, 0, 1, 1, 1], np.float32)
    uu, vv, ww = oracle.dedup_uvw(u, v, w)
    assert list(zip(uu.tolist(), vv.tolist(), ww.tolist())) == [(0.0, 5.0, 1.0), (1.0, 2.0, 0.0), (1.0, 2.0, 1.0),
                                                               (3.0, 1.0, 0.0)]


def test_shade_windows_modes_agree(oracle):
    rng = np.random.default_rng(8)
    u, v, w = (np.ceil(rng.normal(0, 2000, 3000)).astype(np.float32) for _ in range(3))
    for RES in (2094, 20940):
        a, mr = oracle.shade_windows(u, v, w, RES, mode=1)
        b, _ = oracle.shade_windows(u, v, w, RES, mean_r=mr, mode=0)
        diff = np.abs(a - b)
        diff = np.minimum(diff, RES - diff)  # wrapped indices
        assert (diff > 1).sum() == 0
        assert (diff == 1).mean() < 0.01
