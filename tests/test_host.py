"""Host-side logic of the product, checked without a GPU: the C ABI library
loads and exports every declared symbol, the plan geometry and tables equal
the oracle's, and the rand() stream matches."""
import ctypes
import os
import re

import numpy as np

from tests.conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "mrg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mrg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(mrg_lib):
    lib = ctypes.CDLL(mrg_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers the same set
    from mri_recon_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == names


def _geometry(L, N, kernel=1, overgrid=1.5, dwin=-1.0):
    from mri_recon_gb300._lib import MrgConfig, _fp, _ip
    cfg = MrgConfig()
    L.mrg_config_default(ctypes.byref(cfg))
    cfg.kernel_type, cfg.overgrid, cfg.dwin = kernel, overgrid, dwin
    S = (ctypes.c_int * 3)()
    og = (ctypes.c_int * 3)()
    gr = (ctypes.c_float * 3)()
    be = (ctypes.c_float * 3)()
    ll = ctypes.c_int()
    assert L.mrg_plan_geometry(ctypes.byref(cfg), N, N, N, S, og, gr, be, ctypes.byref(ll), None, None) == 0
    lut = np.zeros(3 * ll.value, np.float32)
    win = np.zeros(sum(S), np.float32)
    assert L.mrg_plan_geometry(ctypes.byref(cfg), N, N, N, S, og, gr, be, ctypes.byref(ll),
                               lut.ctypes.data_as(_fp), win.ctypes.data_as(_fp)) == 0
    return tuple(S), tuple(og), tuple(be), lut.reshape(3, -1), win


def test_geometry_tables_equal_oracle(mrg_lib, oracle_lib):
    L = mrg_lib.load()
    for N in (32, 64, 96, 128, 256):
        S, og, beta, lut, win = _geometry(L, N)
        p = oracle_lib.Plan(N)
        olut, owin = p.tables()
        assert S == p.S and og == p.og
        assert np.array_equal(lut, olut)
        assert np.array_equal(win, np.concatenate(owin))
        assert beta == p.beta


def test_geometry_other_kernels(mrg_lib, oracle_lib):
    L = mrg_lib.load()
    for k in (0, 2, 3):
        S, og, beta, lut, win = _geometry(L, 64, kernel=k)
        p = oracle_lib.Plan(64, kernel=k)
        olut, owin = p.tables()
        assert np.array_equal(lut, olut)
        assert np.array_equal(win, np.concatenate(owin))


def test_rand_stream_matches_oracle(mrg_lib, oracle_lib):
    """The library's glibc random() stream against the oracle's draw-by-draw one at short and
    long skips (long skips jump ahead through the recurrence's characteristic polynomial), and
    a skip of 10^15 draws that only a jump can make, checked against a nearby skip."""
    L = mrg_lib.load()

    def stream(skip, n):
        out = (ctypes.c_int * n)()
        assert L.mrg_rand_stream(skip, n, out) == 0
        return np.array(out[:])

    rng = np.random.default_rng(0)
    for skip in list(range(0, 130)) + [int(v) for v in rng.integers(130, 200000, 20)]:
        assert np.array_equal(stream(skip, 25), oracle_lib.glibc_rand(skip, 25)), skip
    far = stream(10 ** 15, 20)
    assert np.array_equal(far, stream(10 ** 15 - 7, 27)[7:])
    edge = stream(2 ** 63 - 40, 30)  # the largest skips do not overflow the stream position
    assert np.array_equal(edge[10:], stream(2 ** 63 - 30, 20))


def test_errors_are_reported_not_fatal(mrg_lib):
    from mri_recon_gb300._lib import MrgConfig
    L = mrg_lib.load()
    h = ctypes.c_void_p()
    assert L.mrg_plan_create(None, 0, 64, 64, 1, 1, ctypes.byref(h)) == 1
    assert b"positive" in L.mrg_last_error()
    assert L.mrg_rand_stream(-1, 3, None) == 1
    cfg = MrgConfig()
    L.mrg_config_default(ctypes.byref(cfg))
    assert abs(cfg.overgrid - 1.5) < 1e-7 and cfg.kernel_type == 1 and abs(cfg.k_rad - 9999.0) < 1e-3
    assert cfg.fft_norm == 0  # gridFFT's normalised transforms unless asked
    S, og, ll = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), ctypes.c_int()
    gr, be = (ctypes.c_float * 3)(), (ctypes.c_float * 3)()
    for field, bad in (("fft_norm", 2), ("fft_norm", -1), ("grid_mode", 4), ("kernel_type", 5), ("dwin", 1e9),
                       ("dwin", -2.0), ("dwin", 0.0), ("dwin", float("nan")), ("overgrid", float("nan")),
                       ("overgrid", 100.0), ("overgrid", 0.5)):
        c2 = MrgConfig()
        L.mrg_config_default(ctypes.byref(c2))
        setattr(c2, field, bad)
        # rejected with a status before any table is sized from it (no exception, no exit)
        assert L.mrg_plan_create(ctypes.byref(c2), 32, 32, 32, 1, 1, ctypes.byref(h)) == 1, field
        assert b"bad config" in L.mrg_last_error()
        assert L.mrg_plan_geometry(ctypes.byref(c2), 32, 32, 32, S, og, gr, be, ctypes.byref(ll), None, None) == 1
        assert b"bad config" in L.mrg_last_error()
    assert L.mrg_plan_geometry(None, 70000, 32, 32, S, og, gr, be, ctypes.byref(ll), None, None) == 1
    assert b"65536" in L.mrg_last_error()
    # density-compensation parameters are checked before any device work
    from mri_recon_gb300._lib import MrgDcfParams
    k = np.zeros(8, np.float32)
    kp = k.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    for field, bad in (("overgrid", 1e6), ("dwin", 1e9), ("dwin", 0.0), ("iters", -1), ("kernel", 2)):
        q = MrgDcfParams()
        L.mrg_dcf_params_default(ctypes.byref(q))
        setattr(q, field, bad)
        assert L.mrg_dcf_pipe(kp, kp, kp, 8, 16, 16, 16, ctypes.byref(q), kp, None) == 1, field
    c3 = MrgConfig()
    L.mrg_config_default(ctypes.byref(c3))
    c3.dwin, c3.overgrid = 16.0, 8.0  # the edges of the accepted ranges
    assert L.mrg_plan_geometry(ctypes.byref(c3), 16, 16, 16, S, og, gr, be, ctypes.byref(ll), None, None) == 0


def test_loop_parameter_defaults_are_the_references(mrg_lib):
    """FISTA (src/recon_lib.cpp:83-133), CLEAR (src/clear.cpp:47-61) and SPIRIT
    (src/spirit.cpp:9-34) defaults, and the DCF flags (src/recon_lib.cpp), set without a GPU;
    the Python structures match the C layout."""
    from mri_recon_gb300 import _lib
    L = mrg_lib.load()
    f = _lib.MrgFistaParams()
    L.mrg_fista_params_default(ctypes.byref(f))
    assert f.max_iter == 50 and f.max_eig_iter == 30 and f.cycle_spins == 4 and list(f.wave_levels) == [4, 4, 4]
    assert f.wave_type == 1 and list(f.llr_block) == [4, 4, 4] and f.llr_block_iter == 4 and f.llr_alpha == 0.0
    c = _lib.MrgClearParams()
    L.mrg_clear_params_default(ctypes.byref(c))
    assert c.max_iter == 50 and list(c.block) == [4, 4, 4] and c.block_iter == 4
    assert abs(c.alpha_coil - 0.01) < 1e-9 and c.clear_amp == 4.0 and c.clear_t2 == 6.0
    assert c.early_stop_thresh == 0.0 and c.early_stop_range == 5 and c.rand_skip == 0
    assert c.use_threshold == 0 and c.cycle_spins == 4 and list(c.wave_levels) == [4, 4, 4] and c.wave_type == 1
    e = _lib.MrgEspiritParams()
    L.mrg_espirit_params_default(ctypes.byref(e))
    assert list(e.kernel_radius) == [3.0, 3.0, 3.0] and list(e.calib_radius) == [12, 12, 12]
    assert abs(e.svd_thresh - 0.01) < 1e-9 and e.square == 0
    d = _lib.MrgDcfParams()
    L.mrg_dcf_params_default(ctypes.byref(d))
    assert d.iters == 20 and abs(d.dwin - 2.1) < 1e-6
    # the Python wrappers fill the same structures
    assert list(mrg_lib.espirit_params(kernel_radius=2.5, calib_radius=9).kernel_radius) == [2.5, 2.5, 2.5]
    assert list(mrg_lib.clear_params(block=(8, 8, 2), wave_levels=(3, 3, 3)).block) == [8, 8, 2]


def test_new_entry_points_reject_bad_arguments_without_a_gpu(mrg_lib):
    """Argument checks of the CLEAR, ESPIRiT and FFT entry points run before any CUDA call."""
    from mri_recon_gb300 import _lib
    L = mrg_lib.load()
    ip3 = (ctypes.c_int * 3)
    buf = np.zeros(64, np.complex64)
    ptr = ctypes.c_void_p(buf.ctypes.data)
    cp = _lib.MrgClearParams()
    L.mrg_clear_params_default(ctypes.byref(cp))
    assert L.mrg_clear(None, ctypes.byref(cp), ptr, None, None, None, None) == 1
    assert L.mrg_clear_thresh(ptr, 1, 4, 4, 4, 4, ip3(0, 4, 4), 4, 0.1, 1.0, 0, None) == 1
    assert L.mrg_clear_thresh(ptr, 1, 4, 4, 4, 4, ip3(4, 4, 4), 0, 0.1, 1.0, 0, None) == 1
    assert L.mrg_clear_combine(ptr, 0, 4, 4, 4, 4, ip3(4, 4, 4), ptr, None) == 1
    assert L.mrg_clear_update_threshold(ptr, 1, 4, 4, 4, 4, ip3(4, 4, 4), 4.0, 6.0, 0, None, None) == 1
    ep = _lib.MrgEspiritParams()
    L.mrg_espirit_params_default(ctypes.byref(ep))
    ep.kernel_radius[0] = 8.0
    assert L.mrg_espirit(ptr, 4, 4, 4, 4, ctypes.byref(ep), ptr, None, None, 0, None) == 1
    assert b"radius" in L.mrg_last_error()
    assert L.mrg_espirit(None, 4, 4, 4, 4, ctypes.byref(ep), ptr, None, None, 0, None) == 1
    assert L.mrg_espirit_smaps(None, 0, ptr, 0, ctypes.byref(ep), None, None, 0, None, None) == 1
    assert L.mrg_fft3(None, ptr, -1, None) == 1


def test_low_rank_entry_points_reject_empty_blocks_without_a_gpu(mrg_lib):
    """A block edge below 1 is an argument error (status 1), not an integer division by
    zero in the block count or the shift draw (src/clear.cpp:408-410 takes rand() % block)."""
    L = mrg_lib.load()
    ip3 = (ctypes.c_int * 3)
    buf = np.zeros(2 * 8 ** 3, np.complex64)
    ptr = ctypes.c_void_p(buf.ctypes.data)
    v = ctypes.c_float()
    for block in [(0, 8, 8), (8, 0, 8), (8, 8, -1)]:
        assert L.mrg_llr_update_threshold(ptr, 2, 8, 8, 8, ip3(*block), 4.0, 6.0, 0, ctypes.byref(v), None) == 1
        assert L.mrg_llr_thresh(ptr, 2, 8, 8, 8, ip3(*block), 4, 0.1, 1.0, 0, None) == 1
        assert L.mrg_llr_update_threshold_noalloc(ptr, 2, 8, 8, 8, ip3(*block), 4.0, 6.0, 0, ctypes.byref(v),
                                                  None) == 1


def test_plan_calls_reject_a_null_plan_without_a_gpu(mrg_lib):
    L = mrg_lib.load()
    n = ctypes.c_int()
    assert L.mrg_set_wait_limit(None, 1.0) == 1
    assert L.mrg_plan_check(None, None) == 1
    assert L.mrg_last_iterations(None, ctypes.byref(n)) == 1
    from mri_recon_gb300 import _lib
    f = _lib.MrgFistaParams()
    L.mrg_fista_params_default(ctypes.byref(f))
    assert f.early_stop_thresh == 0.0 and f.early_stop_range == 5  # src/recon_lib.cpp:84-85


def test_gating_weights_and_pregate_match_oracle(mrg_lib, oracle_lib):
    """GATING::hist_weight with the respiratory factor, and RECON::pregate_data for each
    frame, from the library's host code against the oracle's restatement: bit for bit."""
    from mri_recon_gb300 import synth
    rng = np.random.default_rng(21)
    nproj, nread, T = 700, 16, 10
    kx, ky, kz, kw = synth.radial_trajectory(32, nproj, nread)
    gate = rng.uniform(0, T, nproj)
    gate[:7] = [0.0, 1.0, 2.999999, 9.0, 9.999, -0.5, 10.0]   # integers, edges, outside [0, T)
    rweight = rng.uniform(0, 1, nproj).astype(np.float32)
    rweight[::9] = 0.0
    data = (rng.standard_normal((3, kx.size)) + 1j * rng.standard_normal((3, kx.size))).astype(np.complex64)
    total = 0
    for rw in (None, rweight):
        for reset in (False, True):
            for t in list(range(T)) + [T, -1]:
                got = mrg_lib.pregate(gate, nread, t, kx, ky, kz, kw, data, rweight=rw, reset_dens=reset)
                want = oracle_lib.pregate(gate, nread, t, kx, ky, kz, kw, data, rweight=rw, reset_dens=reset)
                for g_, w_ in zip(got, want):
                    assert g_.shape == w_.shape and np.array_equal(g_, w_)
                if rw is None and not reset and 0 <= t < T:
                    total += got[0].size
    # without respiratory weights every readout in [0, T) lands in exactly one frame
    assert total == nread * int(np.sum((np.floor(gate) >= 0) & (np.floor(gate) < T)))
    # the time weight of the non-pregated loops
    for t in (0, 3):
        w = mrg_lib.gate_weights(gate, kw, nread, t, rweight=rweight)
        mask = np.repeat(rweight * (np.floor(gate) == t), nread).astype(np.float32)
        assert np.array_equal(w, kw * mask)
    # sizes whose product would overflow are rejected before anything is read
    L = mrg_lib.load()
    n = ctypes.c_int64()
    g1 = np.zeros(1, np.float64)
    assert L.mrg_pregate(g1.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, 2 ** 62, 4, 0, 0, None, None, None,
                         None, None, 0, 0, None, None, None, None, None, 0, ctypes.byref(n)) == 1
