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
    L = mrg_lib.load()
    out = (ctypes.c_int * 25)()
    assert L.mrg_rand_stream(1000, 25, out) == 0
    assert np.array_equal(np.array(out[:]), oracle_lib.glibc_rand(1000, 25))


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
