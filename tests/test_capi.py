"""The C ABI library: loads, exports every declared entry point, and rejects bad
arguments with status codes before touching a GPU."""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def L():
    from viss_recon_shade_gb300 import _lib
    return _lib


def test_exports_every_declared_symbol(L):
    declared = L.declared_symbols()
    assert len(declared) >= 18
    for name in declared:
        assert hasattr(L.lib, name), name
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(declared) <= exported


def test_every_declared_symbol_has_a_ctypes_signature(L):
    # a symbol without argtypes would pass 64-bit and double arguments as C int
    assert set(L.declared_symbols()) == set(L._SIGS)


def test_status_strings(L):
    for s in (0, -1, -2, -3, -4, -5, -6, -7, -8):
        assert L.lib.viss_status_str(s)
    assert L.lib.viss_status_str(0) == b"ok"
    assert L.lib.viss_version() >= 10000


def test_invalid_arguments_fail_without_gpu(L):
    # NULL config, bad modes and bad sizes are rejected on the host
    assert L.lib.viss_vis_dft(None, None, None, None, None, None, 0, None) == L.VISS_ERR_INVALID
    cfg = L.DftCfg(9, 0, 1, 0, 0, 0.0, 0.5, 0.0, 1737.4, 1.0)
    sky = L.Sky(None, None, None, None, 0)
    vis = L.VisSet(None, None, None, None, None, None, None, 0)
    assert L.lib.viss_vis_dft(C.byref(cfg), C.byref(sky), C.byref(vis), None, None, None, 0, None) == \
        L.VISS_ERR_INVALID
    cfg.mask_mode = 0
    cfg.phase_scale = 2.0
    assert L.lib.viss_vis_dft(C.byref(cfg), C.byref(sky), C.byref(vis), None, None, None, 0, None) == L.VISS_ERR_RANGE
    assert b"phase_scale" in L.lib.viss_last_error()
    cfg.phase_scale = 0.5
    cfg.mask_mode = 3  # geometric without geometry
    vis.K = 5
    sky.J = 3
    dummy = C.c_void_p(16)
    vis.u = vis.v = vis.w = dummy
    sky.l = sky.m = sky.n = sky.bright = dummy
    assert L.lib.viss_vis_dft(C.byref(cfg), C.byref(sky), C.byref(vis), None, dummy, None, 0, None) == \
        L.VISS_ERR_INVALID
    assert L.lib.viss_visscal(-1, 3, 10, *([None] * 14), 2.0, 2.0, 2.0, 0, 1, 1, None) == L.VISS_ERR_RANGE
    assert L.lib.viss_dedup_uvw(None, None, None, 5, None, None, 0, None) == L.VISS_ERR_INVALID
    oc = L.OrbitCfg(1, 360, 1, 1, 2038.14, 0.0, 30.0, 0.0, 0.08, None, None, 0, 0)
    assert L.lib.viss_orbit_positions(C.byref(oc), dummy, None, None) == L.VISS_ERR_RANGE


def test_workspace_queries_are_consistent(L):
    cfg = L.DftCfg(3, 2, 1, 0, 0, 0.0, 1.0, -1.0, 1737.4, 1.0)
    geo = L.Geometry(None, 100, 8, 0)
    a = L.lib.viss_vis_dft_workspace(C.byref(cfg), 10000, 5000, C.byref(geo))
    b = L.lib.viss_recon_workspace(C.byref(cfg), 10000, 5000, C.byref(geo))
    assert a > 0 and b > 0 and a % 256 == 0 and b % 256 == 0
    cfg.precision = 0  # plain needs no records
    assert L.lib.viss_vis_dft_workspace(C.byref(cfg), 10000, 5000, C.byref(geo)) < a


def _batch(L, row_off, norm=None):
    import numpy as np
    ro = np.ascontiguousarray(row_off, dtype=np.int64)
    nb = None if norm is None else np.ascontiguousarray(norm, dtype=np.float64)
    b = L.Batch(ro.size - 1, 0, ro.ctypes.data_as(C.POINTER(C.c_int64)), None,
                None if nb is None else nb.ctypes.data_as(C.POINTER(C.c_double)))
    b._keep = (ro, nb)
    return b


def test_batch_arguments_checked_on_host(L):
    cfg = L.DftCfg(0, 0, 1, 0, 0, 0.0, 1.0, -1.0, 1737.4, 1.0)
    dummy = C.c_void_p(16)
    sky = L.Sky(dummy, dummy, dummy, dummy, 3)
    vis = L.VisSet(dummy, dummy, dummy, None, None, None, None, 10)
    t = L.Tuning(0, 0, 0, 0)
    for bad in ([1, 10], [0, 4, 3, 10], [0, 4, 9]):  # not from 0, decreasing, not ending at K
        b = _batch(L, bad)
        assert L.lib.viss_vis_dft_batch(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(b), None, C.byref(t),
                                        dummy, None, 0, None) == L.VISS_ERR_INVALID
        assert L.lib.viss_recon_batch(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(b), None, C.byref(t),
                                      dummy, dummy, None, 0, None) == L.VISS_ERR_INVALID
        assert L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), C.byref(b), 10, 3, None, None) == 0
    b = _batch(L, [0] * 66)  # 65 channels
    assert L.lib.viss_vis_dft_batch(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(b), None, None, dummy, None, 0,
                                    None) == L.VISS_ERR_RANGE
    # trunc_brightness cannot combine with per-channel brightness
    b = _batch(L, [0, 4, 10])
    b.bright = dummy
    cfg.trunc_brightness = 1
    assert L.lib.viss_vis_dft_batch(C.byref(cfg), C.byref(sky), C.byref(vis), C.byref(b), None, None, dummy, None, 0,
                                    None) == L.VISS_ERR_UNSUPPORTED


def test_batch_workspace_grows_with_channel_padding(L):
    # every channel is padded to whole blocks of 1024 visibilities in the vis pass
    cfg = L.DftCfg(3, 2, 1, 0, 0, 0.0, 1.0, -1.0, 1737.4, 1.0)
    geo = L.Geometry(None, 100, 8, 0)
    one = L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), None, 10000, 5000, C.byref(geo), None)
    assert one == L.lib.viss_vis_dft_workspace(C.byref(cfg), 10000, 5000, C.byref(geo))
    b = _batch(L, [0, 1, 2, 3, 10000])
    t = L.Tuning(0, 1, 0, 0)  # one sky chunk: no partial sums
    many = L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), C.byref(b), 10000, 5000, C.byref(geo), C.byref(t))
    single = L.lib.viss_vis_dft_batch_workspace(C.byref(cfg), None, 10000, 5000, C.byref(geo), C.byref(t))
    assert many > single
    r = L.lib.viss_recon_batch_workspace(C.byref(cfg), C.byref(b), 10000, 5000, C.byref(geo), None)
    assert r > 0 and r % 256 == 0


def test_stage1_and_window_entry_points_check_arguments(L):
    """viss_unique_uvw, viss_vis_dft_windowed and viss_workspace_limb_count reject
    bad arguments on the host; an empty snapshot set is a valid no-op."""
    dummy = C.c_void_p(16)
    cnt = C.c_int64(-1)
    unique = L.lib.viss_unique_uvw
    assert unique(dummy, 10, 8, 1, 30.0, None, None, None, 0, None, None, 0, None) == L.VISS_ERR_INVALID
    assert unique(dummy, 10, 1, 1, 30.0, None, None, None, 0, C.byref(cnt), None, 0, None) == L.VISS_ERR_RANGE
    assert cnt.value == 0
    assert unique(dummy, 10, 8, 1, 0.0, None, None, None, 0, C.byref(cnt), None, 0, None) == L.VISS_ERR_RANGE
    assert unique(dummy, 10, 8, 1, float("nan"), None, None, None, 0, C.byref(cnt), None, 0, None) == \
        L.VISS_ERR_RANGE
    assert unique(dummy, -1, 8, 1, 30.0, None, None, None, 0, C.byref(cnt), None, 0, None) == L.VISS_ERR_RANGE
    assert unique(dummy, 10, 8, 1, 30.0, None, None, None, -1, C.byref(cnt), None, 0, None) == L.VISS_ERR_RANGE
    cnt.value = -1
    assert unique(None, 0, 8, 1, 30.0, None, None, None, 0, C.byref(cnt), None, 0, None) == L.VISS_OK
    assert cnt.value == 0
    assert unique(None, 10, 8, 1, 30.0, None, None, None, 0, C.byref(cnt), None, 0, None) == L.VISS_ERR_INVALID
    assert unique(dummy, 10, 8, 1, 30.0, None, None, None, 5, C.byref(cnt), None, 0, None) == L.VISS_ERR_INVALID
    nb = L.lib.viss_unique_uvw_workspace(10, 8, 1)
    assert nb > 0 and L.lib.viss_unique_uvw_workspace(0, 8, 1) == 0 and L.lib.viss_unique_uvw_workspace(10, 1, 1) == 0
    assert unique(dummy, 10, 8, 1, 30.0, None, None, None, 0, C.byref(cnt), None, nb, None) == L.VISS_ERR_WORKSPACE
    assert unique(dummy, 10, 8, 1, 30.0, None, None, None, 0, C.byref(cnt), C.c_void_p(16), nb, None) == \
        L.VISS_ERR_WORKSPACE  # not 256-byte aligned
    assert L.lib.viss_unique_uvw_workspace(10, 8, 1) > L.lib.viss_unique_uvw_workspace(10, 8, 0)

    cfg = L.DftCfg(1, 0, 1, 8, 0, 240.0, 0.5, 0.0, 1737.4, 1.0)  # REF_QUIRK, res 8
    sky = L.Sky(dummy, dummy, dummy, dummy, 3)
    vis = L.VisSet(dummy, dummy, dummy, None, None, None, None, 5)
    win = L.lib.viss_vis_dft_windowed
    assert win(C.byref(cfg), C.byref(sky), dummy, C.byref(vis), dummy, None, 0, None) == L.VISS_ERR_INVALID
    assert b"shade windows" in L.lib.viss_last_error()
    vis.shade = dummy
    assert win(C.byref(cfg), C.byref(sky), None, C.byref(vis), dummy, None, 0, None) == L.VISS_ERR_INVALID
    assert b"win_index" in L.lib.viss_last_error()
    cfg.mask_mode = 0
    assert win(C.byref(cfg), C.byref(sky), dummy, C.byref(vis), dummy, None, 0, None) == L.VISS_ERR_INVALID
    assert b"REF mask" in L.lib.viss_last_error()
    assert L.lib.viss_workspace_limb_count(None, C.byref(cnt), None) == L.VISS_ERR_INVALID
    assert L.lib.viss_workspace_limb_count(dummy, None, None) == L.VISS_ERR_INVALID


def test_vis_split_beyond_int_work_items_is_refused(L):
    """A caller's vis_split that would make more than 2^31 - 1 work items (visibility
    blocks x sky chunks) is refused on the host, before the workspace is looked at."""
    dummy = C.c_void_p(16)
    cfg = L.DftCfg(0, 0, 1, 0, 0, 0.0, 1.0, -1.0, 1737.4, 1.0)  # no mask, FAST
    sky = L.Sky(dummy, dummy, dummy, dummy, 1 << 30)
    vis = L.VisSet(dummy, dummy, dummy, None, None, None, None, 1 << 31)
    t = L.Tuning(0, 1 << 21, 0, 0)  # 2^21 sky chunks x 2^21 visibility blocks
    rc = L.lib.viss_vis_dft_batch(C.byref(cfg), C.byref(sky), C.byref(vis), None, None, C.byref(t), dummy, None, 0,
                                  None)
    assert rc == L.VISS_ERR_RANGE
    assert b"vis_split" in L.lib.viss_last_error()
    t.vis_split = 4  # a sane split reaches the workspace check instead
    rc = L.lib.viss_vis_dft_batch(C.byref(cfg), C.byref(sky), C.byref(vis), None, None, C.byref(t), dummy, None, 0,
                                  None)
    assert rc == L.VISS_ERR_WORKSPACE
