"""GPU parity of CLEAR (coil low rank, src/clear.cpp:99-232, :561-914 with dim = 2, and
the CLEAR loop of src/recon_lib.cpp:1025-1238) against the oracle, through the C ABI."""
import ctypes

import numpy as np
import pytest

from tests.helpers import rel

pytestmark = pytest.mark.gpu


def _ip(v):
    return (ctypes.c_int * 3)(*v)


def _stack(T, C, N, seed):
    """Coil stack in the library's layout (T, Nz, Ny, Nx, C) complex64."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((T, N, N, N, C)) + 1j * rng.standard_normal((T, N, N, N, C))).astype(np.complex64)


def _oracle_layout(XX):
    return np.ascontiguousarray(XX.transpose(0, 4, 1, 2, 3)).astype(np.complex128)


# (2, 8, 16, 4): block matrix in shared memory; (4, 16, 16, 8): 2048 x 16 matrix read from
# global memory; (1, 32, 16, 4): 32 coils; (3, 5, 12, (4, 3, 4)): anisotropic blocks
@pytest.mark.parametrize("T,C,N,bs", [(2, 8, 16, (4, 4, 4)), (4, 16, 16, (8, 8, 8)), (1, 32, 16, (4, 4, 4)),
                                      (3, 5, 12, (4, 3, 4)), (1, 1, 8, (4, 4, 4))])
@pytest.mark.parametrize("device", [True, False])
def test_coil_lowrank_blocks_match_oracle(mrg_lib, oracle_lib, T, C, N, bs, device):
    import torch
    XX = _stack(T, C, N, 3 + C)
    ref = _oracle_layout(XX)
    arg = torch.from_numpy(XX).cuda() if device else XX.copy()
    smax = mrg_lib.clear_update_threshold(arg, bs, 4.0, 6.0, 1)
    smax_ref = oracle_lib.clear_update_threshold(ref, bs, 4.0, 6.0, 1)
    assert abs(smax - smax_ref) <= 1e-5 * smax_ref
    Y = mrg_lib.clear_thresh(arg, smax_ref, bs, 4, 0.05, 100)
    Yref = oracle_lib.clear_thresh(ref, bs, 4, 0.05, smax_ref, 100).transpose(0, 2, 3, 4, 1)
    Y = Y.cpu().numpy() if device else Y
    assert rel(Y, Yref) < 1e-5
    assert rel(Y, XX) > 1e-3  # the threshold changed the stack
    im = mrg_lib.clear_combine(torch.from_numpy(XX).cuda() if device else XX, bs)
    im = im.cpu().numpy() if device else im
    imref = oracle_lib.clear_combine(ref, bs)
    assert rel(np.abs(im), np.abs(imref)) < 1e-5
    assert rel(im, imref) < 1e-5  # same phase convention for v1


def test_combine_leaves_partial_blocks(mrg_lib, oracle_lib):
    """N not a multiple of the block: voxels outside whole blocks keep the output's values."""
    rng = np.random.default_rng(1)
    XX = (rng.standard_normal((1, 10, 10, 10, 3)) + 1j * rng.standard_normal((1, 10, 10, 10, 3))).astype(np.complex64)
    out0 = np.full((1, 10, 10, 10), 7.0 + 1.0j, np.complex64)
    im = mrg_lib.clear_combine(XX, (4, 4, 4), out=out0.copy())
    imref = oracle_lib.clear_combine(_oracle_layout(XX), (4, 4, 4), out=out0)
    assert rel(im, imref) < 1e-5
    assert np.all(im[:, 8:, :, :] == out0[:, 8:, :, :])


def test_clear_thresh_alpha_zero_and_bad_args(mrg_lib):
    XX = _stack(1, 4, 8, 2)
    Y = mrg_lib.clear_thresh(XX.copy(), 10.0, (4, 4, 4), 4, 0.0, 0)
    assert np.array_equal(Y, XX)
    L = mrg_lib.load()
    assert L.mrg_clear_thresh(ctypes.c_void_p(XX.ctypes.data), 1, 4, 8, 8, 8, _ip((0, 4, 4)), 4, 0.1, 1.0, 0, None) != 0
    XX33 = np.zeros((1, 4, 4, 4, 33), np.complex64)
    assert L.mrg_clear_combine(ctypes.c_void_p(XX33.ctypes.data), 1, 33, 4, 4, 4, _ip((4, 4, 4)),
                               ctypes.c_void_p(XX33.ctypes.data), None) != 0


def _inputs(oracle_lib, N, C, T, nproj, seed):
    from mri_recon_gb300 import synth
    smaps = synth.coil_maps(N, C, seed=seed)
    O64 = oracle_lib.Plan(N, prec=1)
    frames = []
    for t in range(T):
        kx, ky, kz, kw = synth.radial_trajectory(N, nproj, N, start=t * nproj)
        img = synth.phantom(N, 6, seed=seed, frame=t, nframes=max(T, 1))
        y = np.stack([O64.forward(img, smaps[c], kx, ky, kz, kw) for c in range(C)]).astype(np.complex64)
        frames.append(dict(kx=kx, ky=ky, kz=kz, kw=kw, data=synth.add_noise(y, 0.01, seed)))
    return frames


def _plan(mrg_lib, N, C, T, frames, device=True):
    import torch
    p = mrg_lib.Plan(N, C, T)
    for t, fr in enumerate(frames):
        p.set_traj(t, fr["kx"], fr["ky"], fr["kz"], fr["kw"])
        p.set_data(t, torch.from_numpy(fr["data"]).cuda() if device else fr["data"])
    return p


# the last two cases add the loop's L1-wavelet soft threshold (cycle spinning, DB4 and DB2)
@pytest.mark.parametrize("N,C,T,nproj,iters,alpha,l1", [
    (16, 4, 1, 300, 4, 0.01, None), (16, 3, 2, 200, 3, 0.01, None), (16, 1, 1, 300, 3, 0.01, None),
    (20, 6, 1, 400, 3, 0.0, None),
    (16, 4, 1, 300, 3, 0.01, dict(use_threshold=1, thresh=0.2, cycle_spins=3, wave_levels=(2, 2, 2), wave_type=1)),
    (16, 3, 2, 200, 2, 0.0, dict(use_threshold=1, thresh=0.1, cycle_spins=2, wave_levels=(3, 3, 3), wave_type=0,
                                 rand_skip=5))])
def test_clear_matches_oracle(mrg_lib, oracle_lib, N, C, T, nproj, iters, alpha, l1):
    import torch
    frames = _inputs(oracle_lib, N, C, T, nproj, 9)
    p = _plan(mrg_lib, N, C, T, frames)
    X = torch.zeros((T, N, N, N), dtype=torch.complex64, device="cuda")
    extra = l1 or {}
    X, resid, XX = p.clear(mrg_lib.clear_params(max_iter=iters, alpha_coil=alpha, **extra), X=X, coil_images=True)
    q = oracle_lib.clear_params(max_iter=iters, alpha_coil=alpha, **extra)
    XX64, im64, r64, d64 = oracle_lib.Plan(N, prec=1).clear(frames, q)
    XX32, im32, r32, d32 = oracle_lib.Plan(N, prec=0).clear(frames, q)
    XX = XX.cpu().numpy().transpose(0, 4, 1, 2, 3)
    X = X.cpu().numpy()
    print("clear rel-L2 coils vs FP64 %.3g vs FP32 %.3g; combined %.3g" % (rel(XX, XX64), rel(XX, XX32), rel(X, im64)))
    assert len(resid) == iters == d64
    assert np.max(np.abs(resid - r64) / r64) < 1e-4
    assert rel(XX, XX64) < 1e-4
    assert rel(XX, XX32) < 1e-4
    assert rel(X, im64) < 1e-4


def test_clear_host_buffers_and_early_stop(mrg_lib, oracle_lib):
    N, C, T = 16, 3, 1
    frames = _inputs(oracle_lib, N, C, T, 250, 5)
    p = _plan(mrg_lib, N, C, T, frames, device=False)
    kw = dict(max_iter=8, early_stop_thresh=1e9, early_stop_range=3)
    X, resid = p.clear(mrg_lib.clear_params(**kw))
    assert isinstance(X, np.ndarray) and len(resid) == 3  # stdev < thresh as soon as 3 residuals exist
    XX64, im64, r64, d64 = oracle_lib.Plan(N, prec=1).clear(frames, oracle_lib.clear_params(**kw))
    assert d64 == 3
    assert rel(X, im64) < 1e-4


def test_clear_needs_data_and_few_coils(mrg_lib):
    from mri_recon_gb300 import synth
    p = mrg_lib.Plan(8, 2, 1)
    kx, ky, kz, kw = synth.radial_trajectory(8, 40, 8)
    p.set_traj(0, kx, ky, kz, kw)
    with pytest.raises(mrg_lib.MrgError, match="low-rank"):
        p.clear(mrg_lib.clear_params(max_iter=1, alpha_coil=0.01, block_iter=65))  # checked before the data
    with pytest.raises(mrg_lib.MrgError):
        p.clear(mrg_lib.clear_params(max_iter=1))  # no k-space data
    p33 = mrg_lib.Plan(8, 33, 1)
    p33.set_traj(0, kx, ky, kz, kw)
    p33.set_data(0, np.zeros((33, kx.size), np.complex64))
    with pytest.raises(mrg_lib.MrgError):
        p33.clear(mrg_lib.clear_params(max_iter=1))
