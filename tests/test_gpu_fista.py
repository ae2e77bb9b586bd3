"""GPU parity of the FISTA building blocks and of whole FISTA / FISTA+LLR runs
against the oracle."""
import ctypes

import numpy as np
import pytest

from tests.helpers import case, rel

pytestmark = pytest.mark.gpu


def _lib():
    import mri_recon_gb300 as m
    return m.load()


def _ip(v):
    return (ctypes.c_int * 3)(*v)


def _vols(n, N, seed):
    rng = np.random.default_rng(seed)
    return np.stack([(rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))) for _ in range(n)]).astype(np.complex64)


@pytest.mark.parametrize("shift", [(0, 0, 0), (1, 2, 3), (3, 0, 2)])
@pytest.mark.parametrize("wtype", [1, 0])
def test_wavelet_matches_oracle(mrg_lib, oracle_lib, shift, wtype):
    import torch
    X = _vols(2, 32, 4)
    d = torch.from_numpy(X).cuda()
    L = _lib()
    assert L.mrg_wavelet(ctypes.c_void_p(d.data_ptr()), 2, 32, 32, 32, _ip((3, 3, 3)), _ip(shift), wtype, 0, None) == 0
    ref = np.stack([oracle_lib.wavelet(X[t], (3, 3, 3), shift, wtype) for t in range(2)])
    assert rel(d.cpu().numpy(), ref) < 1e-6
    assert L.mrg_wavelet(ctypes.c_void_p(d.data_ptr()), 2, 32, 32, 32, _ip((3, 3, 3)), _ip(shift), wtype, 1, None) == 0
    assert rel(d.cpu().numpy(), X) < 1e-6


def test_wavelet_anisotropic_levels(mrg_lib, oracle_lib):
    rng = np.random.default_rng(9)
    X = (rng.standard_normal((16, 40, 48)) + 1j * rng.standard_normal((16, 40, 48))).astype(np.complex64)
    L = _lib()
    Y = X.copy()
    assert L.mrg_wavelet(ctypes.c_void_p(Y.ctypes.data), 1, 48, 40, 16, _ip((4, 4, 4)), _ip((1, 2, 3)), 1, 0, None) == 0
    assert rel(Y, oracle_lib.wavelet(X, (4, 4, 4), (1, 2, 3))) < 1e-6


def test_fraction_and_soft_threshold(mrg_lib, oracle_lib):
    X = _vols(3, 24, 8)
    L = _lib()
    v = ctypes.c_float()
    assert L.mrg_fraction_threshold(ctypes.c_void_p(X.ctypes.data), 3, 24 ** 3, 0.1, ctypes.byref(v), None) == 0
    ref = oracle_lib.fraction_threshold([X[t] for t in range(3)], 0.1)
    assert abs(v.value - ref) <= 1e-6 * ref
    Y = X[0].copy()
    assert L.mrg_soft_threshold(ctypes.c_void_p(Y.ctypes.data), Y.size, ctypes.c_float(ref), None) == 0
    assert rel(Y, oracle_lib.soft_threshold(X[0], ref)) < 1e-6


def test_llr_blocks_match_oracle(mrg_lib, oracle_lib):
    X = _vols(6, 32, 12)
    L = _lib()
    sm = ctypes.c_float()
    assert L.mrg_llr_update_threshold(ctypes.c_void_p(X.ctypes.data), 6, 32, 32, 32, _ip((8, 8, 8)), 4.0, 6.0, 2,
                                      ctypes.byref(sm), None) == 0
    ref = oracle_lib.llr_update_threshold([X[t] for t in range(6)], (8, 8, 8), 4.0, 6.0, 2)
    assert abs(sm.value - ref) / ref < 1e-5
    Y = X.copy()
    assert L.mrg_llr_thresh(ctypes.c_void_p(Y.ctypes.data), 6, 32, 32, 32, _ip((8, 8, 8)), 4, 0.3, ref, 1000, None) == 0
    refY = oracle_lib.llr_thresh([X[t] for t in range(6)], (8, 8, 8), 4, 0.3, ref, 1000)
    assert rel(Y, np.stack(refY)) < 1e-5


def _fista_inputs(N, C, T, nproj, seed):
    from mri_recon_gb300 import synth
    frames = []
    smaps = synth.coil_maps(N, C, seed=seed)
    for t in range(T):
        kx, ky, kz, kw = synth.radial_trajectory(N, nproj, N, start=t * nproj)
        img = synth.phantom(N, 6, seed=seed, frame=t, nframes=max(T, 1))
        frames.append(dict(kx=kx, ky=ky, kz=kz, kw=kw, img=img))
    return frames, smaps


def _run_fista(mrg_lib, oracle_lib, N, C, T, nproj, iters, llr_alpha=0.0, use_graph=True, seed=21):
    import torch
    from mri_recon_gb300 import synth
    frames, smaps = _fista_inputs(N, C, T, nproj, seed)
    O64 = oracle_lib.Plan(N, prec=1)
    for fr in frames:
        a = (fr["kx"], fr["ky"], fr["kz"], fr["kw"])
        y = np.stack([O64.forward(fr["img"], smaps[c], *a) for c in range(C)]).astype(np.complex64)
        fr["data"] = synth.add_noise(y, 0.01, seed)
    p = mrg_lib.Plan(N, C, T)
    for t, fr in enumerate(frames):
        p.set_traj(t, fr["kx"], fr["ky"], fr["kz"], fr["kw"])
        p.set_data(t, torch.from_numpy(fr["data"]).cuda())
    p.set_smaps(torch.from_numpy(smaps).cuda())
    kw = dict(max_iter=iters, max_eig_iter=30, cycle_spins=4, wave_levels=(3, 3, 3), wave_type=1, thresh=0.1,
              use_threshold=1, llr_block=(8, 8, 8), llr_block_iter=4, llr_alpha=llr_alpha)
    X, resid, step = p.fista(mrg_lib.fista_params(**kw), use_graph=use_graph)
    q = oracle_lib.FistaParams()
    q.max_iter, q.max_eig_iter, q.cycle_spins = iters, 30, 4
    q.wave_levels[:] = [3, 3, 3]
    q.wave_type, q.thresh, q.use_threshold = 1, 0.1, 1
    q.llr_bs[:] = [8, 8, 8]
    q.llr_block_iter, q.llr_alpha, q.clear_amp, q.clear_t2 = 4, llr_alpha, 4.0, 6.0
    q.rand_skip = 2 * N ** 3 * T
    X32, r32, s32, _ = oracle_lib.Plan(N, prec=0).fista(frames, smaps, q)
    X64, r64, s64, _ = O64.fista(frames, smaps, q)
    return X.cpu().numpy(), resid, step, np.stack(X32), r32, s32, np.stack(X64), r64, s64


@pytest.mark.parametrize("use_graph", [True, False])
def test_fista_l1_wavelet_matches_oracle(mrg_lib, oracle_lib, use_graph):
    X, r, s, X32, r32, s32, X64, r64, s64 = _run_fista(mrg_lib, oracle_lib, 32, 4, 1, 1200, 12, use_graph=use_graph)
    assert abs(s - s64) / s64 < 1e-5
    print("fista rel-L2 vs FP64 %.3g vs FP32 %.3g" % (rel(X, X64), rel(X, X32)))
    assert rel(X, X64) < 1e-4
    assert rel(X, X32) < 1e-4


def test_fista_with_llr_matches_oracle(mrg_lib, oracle_lib):
    X, r, s, X32, r32, s32, X64, r64, s64 = _run_fista(mrg_lib, oracle_lib, 32, 3, 4, 700, 6, llr_alpha=0.05)
    print("fista+llr rel-L2 vs FP64 %.3g vs FP32 %.3g" % (rel(X, X64), rel(X, X32)))
    assert rel(X, X64) < 1e-4
    assert rel(X, X32) < 1e-4
