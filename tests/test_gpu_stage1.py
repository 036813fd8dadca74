"""Stage 1 of the path, the inputs of the DFT: baseline uvw
(MIncline_generate_uvw_float.cu:149-164, computeUVW: ceil((x_n - x_m) * 1e3 / lambda)
in double) and the sort + unique of the uvw rows (:60-71 SortCompare, :352-356).

baseline_uvw: bit-exact against the oracle's double arithmetic, on positions
  chosen so that many quotients land within a few ulp of an integer (where the
  kernel's reciprocal product has to give way to the division).
dedup_uvw: the same unique rows, in the same order, as the oracle's sort +
  unique, on the hash path (many repeats), on the sort fallback (a table that
  fills up) and on small inputs; the first occurrence's values are kept
  (-0 before +0 stays -0); non-integer input is rejected on both paths."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import viss_recon_shade_gb300 as V
    return V


@pytest.mark.parametrize("lam", [10.0, 29.0, 1.0 / 3.0])
@pytest.mark.parametrize("rounding", [True, False])
def test_baseline_uvw_bit_exact(V, oracle, lam, rounding):
    rng = np.random.default_rng(int(lam * 7) + rounding)
    S, nsat = 400, 8
    # positions on a 0.01 km (10 m) grid: (x_n - x_m) * 1e3 / lambda sits near integers
    pos = (rng.integers(-300000, 300000, (S, nsat, 3)) * 0.01).astype(np.float32)
    pos[::7] = rng.normal(0, 2000, (len(pos[::7]), nsat, 3)).astype(np.float32)
    u, v, w, snap, pair = V.baseline_uvw(torch.from_numpy(pos).cuda(), lam, ordered=True, rounding=rounding)
    uo, vo, wo, so, po = oracle.uvw(pos, lam, ordered=True, rounding=rounding)
    for g, o in ((u, uo), (v, vo), (w, wo)):
        assert np.array_equal(g.cpu().numpy().view(np.int32), o.view(np.int32))
    assert np.array_equal(snap.cpu().numpy(), so) and np.array_equal(pair.cpu().numpy(), po)


def dedup_case(rng, K, nkeys, span=3000):
    keys = rng.integers(-span, span, (nkeys, 3)).astype(np.float32)
    pick = rng.integers(0, nkeys, K)
    return [np.ascontiguousarray(keys[pick, i]) for i in range(3)]


@pytest.mark.parametrize("K,nkeys", [(300_000, 5_000), (2_000_000, 400_000), (5_000, 50_000), (3_000, 800),
                                     (1, 1)])
def test_dedup_matches_oracle(V, oracle, K, nkeys):
    rng = np.random.default_rng(K + nkeys)
    u, v, w = dedup_case(rng, K, nkeys)
    g = V.dedup_uvw(*(torch.from_numpy(x).cuda() for x in (u, v, w)))
    o = oracle.dedup_uvw(u, v, w)
    for a, b in zip(g, o):
        assert np.array_equal(a.cpu().numpy(), b)


@pytest.mark.parametrize("K", [8_000, 600])  # hash path, sort path
def test_dedup_keeps_first_occurrence(V, K):
    rng = np.random.default_rng(3)
    u, v, w = dedup_case(rng, K, 200)
    u[:4] = [-0.0, 0.0, 0.0, -0.0]  # rows (+-0, 1, 2) then (+-0, 5, 5)
    v[:4] = [1, 1, 5, 5]
    w[:4] = [2, 2, 5, 5]
    uu, vv, ww = (x.cpu().numpy() for x in V.dedup_uvw(*(torch.from_numpy(x).cuda() for x in (u, v, w))))
    i = np.nonzero((uu == 0) & (vv == 1) & (ww == 2))[0]
    j = np.nonzero((uu == 0) & (vv == 5) & (ww == 5))[0]
    assert len(i) == 1 and len(j) == 1
    assert np.signbit(uu[i[0]]) and not np.signbit(uu[j[0]])


@pytest.mark.parametrize("K", [8_000, 600])
def test_dedup_rejects_non_integer(V, K):
    u, v, w = dedup_case(np.random.default_rng(4), K, 100)
    u[K // 2] = 0.5
    with pytest.raises(RuntimeError):
        V.dedup_uvw(*(torch.from_numpy(x).cuda() for x in (u, v, w)))


def pair_major(pos, x):
    """snapshot-major rows [S * P] -> the reference's pair-major concatenation"""
    return x.view(pos.shape[0], -1).t().reshape(-1)


@pytest.mark.parametrize("ordered", [True, False])
def test_unique_uvw_equals_two_calls(V, oracle, ordered):
    """The fused pass against baseline_uvw + the pair-major concatenation +
    dedup_uvw (bit-exact, sign of zero included) and the oracle (values), on
    windowed orbit positions whose pairs repeat keys over runs of snapshots, with
    run boundaries inside the data."""
    cfg = V.OrbitConfig(orbit_res=7200, orbit_counts=3)
    pos = V.orbit_positions(cfg)
    for lam in (30.0, 3.0):
        u, v, w, _, _ = V.baseline_uvw(pos, lam, ordered=ordered, rounding=True)
        ref = V.dedup_uvw(*(pair_major(pos, x) for x in (u, v, w)))
        got = V.unique_uvw(pos, lam, ordered=ordered, capacity=64)  # short capacity: the retry path
        for a, b in zip(got, ref):
            assert np.array_equal(a.cpu().numpy().view(np.int32), b.cpu().numpy().view(np.int32))
        o = oracle.dedup_uvw(u.cpu().numpy(), v.cpu().numpy(), w.cpu().numpy())
        for a, b in zip(got, o):
            assert np.array_equal(a.cpu().numpy(), b)


def test_unique_uvw_random_positions(V):
    """Positions without run structure (every row inserts) and S not a multiple of
    the run length."""
    rng = np.random.default_rng(9)
    pos = torch.from_numpy(rng.normal(0, 50, (1003, 6, 3)).astype(np.float32)).cuda()
    u, v, w, _, _ = V.baseline_uvw(pos, 10.0, ordered=True, rounding=True)
    ref = V.dedup_uvw(*(pair_major(pos, x) for x in (u, v, w)))
    got = V.unique_uvw(pos, 10.0, ordered=True)
    for a, b in zip(got, ref):
        assert np.array_equal(a.cpu().numpy().view(np.int32), b.cpu().numpy().view(np.int32))


@pytest.mark.parametrize("nsat,ordered", [(16, True), (32, False), (32, True), (2, True)])
def test_unique_uvw_other_formation_sizes(V, nsat, ordered):
    """Other satellite counts (120 and 496 pairs a snapshot, and a single pair):
    slowly drifting positions, so runs of repeated keys cross chunk boundaries."""
    rng = np.random.default_rng(nsat)
    S = 700
    base = rng.normal(0, 30, (1, nsat, 3))
    drift = rng.normal(0, 0.02, (1, nsat, 3))
    pos = (base + drift * np.arange(S)[:, None, None]).astype(np.float32)
    pos_t = torch.from_numpy(pos).cuda()
    u, v, w, _, _ = V.baseline_uvw(pos_t, 3.0, ordered=ordered, rounding=True)
    ref = V.dedup_uvw(*(pair_major(pos_t, x) for x in (u, v, w)))
    got = V.unique_uvw(pos_t, 3.0, ordered=ordered)
    assert got[0].numel() == ref[0].numel() > 0
    for a, b in zip(got, ref):
        assert np.array_equal(a.cpu().numpy().view(np.int32), b.cpu().numpy().view(np.int32))


def test_unique_uvw_count_only_and_short_capacity(V):
    """Through the C ABI: capacity 0 only counts; a nonzero capacity below the count
    returns VISS_ERR_RANGE with the count set; the exact capacity then succeeds."""
    import ctypes as C
    from viss_recon_shade_gb300 import _lib as L
    pos = V.orbit_positions(V.OrbitConfig(orbit_res=3600, orbit_counts=2)).contiguous()
    S, nsat = pos.shape[0], pos.shape[1]
    nb = L.lib.viss_unique_uvw_workspace(S, nsat, 1)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cnt = C.c_int64(-1)
    rc = L.lib.viss_unique_uvw(C.c_void_p(pos.data_ptr()), S, nsat, 1, 30.0, None, None, None, 0, C.byref(cnt),
                               C.c_void_p(ws.data_ptr()), nb, st)
    assert rc == L.VISS_OK and cnt.value > 1
    n = cnt.value
    u, v, w = (torch.empty(n, dtype=torch.float32, device="cuda") for _ in range(3))
    ptrs = [C.c_void_p(x.data_ptr()) for x in (u, v, w)]
    rc = L.lib.viss_unique_uvw(C.c_void_p(pos.data_ptr()), S, nsat, 1, 30.0, *ptrs, n - 1, C.byref(cnt),
                               C.c_void_p(ws.data_ptr()), nb, st)
    assert rc == L.VISS_ERR_RANGE and cnt.value == n
    rc = L.lib.viss_unique_uvw(C.c_void_p(pos.data_ptr()), S, nsat, 1, 30.0, *ptrs, n, C.byref(cnt),
                               C.c_void_p(ws.data_ptr()), nb, st)
    assert rc == L.VISS_OK and cnt.value == n
    ref = V.unique_uvw(pos, 30.0, ordered=True)
    for a, b in zip((u, v, w), ref):
        assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    # a workspace one byte short is refused
    rc = L.lib.viss_unique_uvw(C.c_void_p(pos.data_ptr()), S, nsat, 1, 30.0, *ptrs, n, C.byref(cnt),
                               C.c_void_p(ws.data_ptr()), nb - 1, st)
    assert rc == L.VISS_ERR_WORKSPACE


@pytest.mark.parametrize("orbit_res,orbit_counts,index", [(86400, 10, 1), (8640, 140, 3)])
def test_unique_uvw_bitwise_vs_reference_pipeline(V, orbit_res, orbit_counts, index):
    """The whole stage against the reference's own: its orbit, window and computeUVW
    kernels (from its sources) + per-pair thrust sort/unique with its comparators and
    the global sort/unique (restated) -- the same rows, bit for bit (signs of zero
    included), as positions + viss_unique_uvw at 10 MHz, on millions of snapshots."""
    from oracle import ref_cuda
    if not ref_cuda.available():
        pytest.skip("reference kernels not built (oracle/_ref)")
    from viss_recon_shade_gb300.synth import REF_R1, REF_R2
    ref = ref_cuda.mincline_unique(8, orbit_res, orbit_counts, index, 1e7, REF_R1, REF_R2)
    pos = V.orbit_positions(V.OrbitConfig(orbit_res=orbit_res, orbit_counts=orbit_counts, index=index))
    u, v, w = V.unique_uvw(pos, 30.0, ordered=True)
    ours = torch.stack([u, v, w], 1)
    assert ours.shape == ref.shape
    assert torch.equal(ours.view(torch.int32), ref.view(torch.int32))
