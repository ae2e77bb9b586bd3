"""The oracle's CLEAR restatement (coil low rank, src/clear.cpp:99-232, :561-914 with
dim = 2; the loop of src/recon_lib.cpp:1025-1238) checked on the CPU: the block
operations against numpy's LAPACK SVD written out from the reference's gather /
threshold / scatter loops, and the loop's first iteration against the oracle's own
operators."""
import numpy as np
import pytest

from tests.helpers import case, rel


def _coils(T, C, N, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((T, C) + N) + 1j * rng.standard_normal((T, C) + N)).astype(np.complex128)


def _blocks(shape, bs, sh=(0, 0, 0)):
    """Voxel index arrays (z, y, x) of each block, shifted and wrapped (clear.cpp:629-648)."""
    Nz, Ny, Nx = shape
    for bk in range(Nz // bs[2]):
        for bj in range(Ny // bs[1]):
            for bi in range(Nx // bs[0]):
                xs = (np.arange(bs[0]) + bi * bs[0] + sh[0]) % Nx
                ys = (np.arange(bs[1]) + bj * bs[1] + sh[1]) % Ny
                zs = (np.arange(bs[2]) + bk * bs[2] + sh[2]) % Nz
                yield np.ix_(zs, ys, xs)


def _matrix(XX, ix):
    """Block matrix: rows (frame, z, y, x), columns coils."""
    T, C = XX.shape[:2]
    return np.stack([XX[t, c][ix].reshape(-1) for c in range(C) for t in range(T)]).reshape(C, T, -1) \
        .transpose(1, 2, 0).reshape(-1, C)


def _np_thresh(XX, bs, block_iter, alpha, smax, skip, oracle_lib):
    XX = XX.copy()
    T, C = XX.shape[:2]
    r = oracle_lib.glibc_rand(skip, 3 * block_iter)
    for it in range(block_iter):
        sh = [int(r[3 * it + d]) % bs[d] - bs[d] // 2 for d in range(3)]
        for ix in _blocks(XX.shape[2:], bs, sh):
            A = _matrix(XX, ix)
            U, s, Vh = np.linalg.svd(A, full_matrices=False)
            A2 = (U * np.maximum(s - np.float64(np.float32(alpha)) * smax / block_iter, 0)) @ Vh
            A2 = A2.reshape(T, -1, C)
            for t in range(T):
                for c in range(C):
                    XX[t, c][ix] = A2[t, :, c].reshape(XX[t, c][ix].shape)
    return XX


@pytest.mark.parametrize("T,C,N,bs", [(2, 6, (8, 8, 8), (4, 4, 4)), (1, 4, (12, 8, 10), (4, 4, 4)),
                                      (3, 3, (6, 6, 6), (2, 3, 4))])
def test_coil_lowrank_blocks_vs_numpy_svd(oracle_lib, T, C, N, bs):
    XX = _coils(T, C, N, 5)
    # update_threshold: sigma_1 of the last coil's block per frame (column t), max over t
    sig = [max(np.linalg.norm(XX[t, C - 1][ix]) for t in range(T)) for ix in _blocks(N, bs)]
    smax = oracle_lib.clear_update_threshold(XX, bs, 4.0, 6.0, 3)
    amp = np.float32(1 + 4.0 * np.exp(np.float32(-3.0 / 6.0)))
    assert abs(smax - np.median(sig) * amp) <= 1e-6 * smax
    for block_iter, alpha, skip in ((1, 0.25, 0), (4, 0.125, 11), (3, 0.0625, 1000)):
        got = oracle_lib.clear_thresh(XX, bs, block_iter, alpha, smax, skip)
        ref = _np_thresh(XX, bs, block_iter, alpha, smax, skip, oracle_lib)
        assert np.abs(got - ref).max() < 1e-12 * np.abs(XX).max()
        assert np.abs(got - XX).max() > 1e-3  # the threshold did something
    # combine: A v1 with v1's largest component real positive
    im = oracle_lib.clear_combine(XX, bs)
    for ix in _blocks(N, bs):
        A = _matrix(XX, ix)
        _, _, Vh = np.linalg.svd(A, full_matrices=False)
        v = Vh[0].conj()
        m = np.argmax(np.abs(v))
        v = v * np.conj(v[m]) / abs(v[m])
        ref = (A @ v).reshape(T, -1)
        got = np.stack([im[t][ix].reshape(-1) for t in range(T)])
        assert np.abs(got - ref).max() < 1e-12 * np.abs(A).max()


def test_coil_thresh_alpha_zero_is_identity(oracle_lib):
    XX = _coils(1, 4, (8, 8, 8), 2)
    assert np.array_equal(oracle_lib.clear_thresh(XX, (4, 4, 4), 4, 0.0, 10.0, 0), XX)


def test_clear_first_iteration_by_hand(oracle_lib):
    """One iteration without the threshold: X_c = -scale E_c^H W (0 - d_c) with
    scale = sum |R|^2 / sum P conj(R), from the oracle's single-coil operators."""
    cs = case(N=12, C=3, nproj=120, seed=4)
    O = oracle_lib.Plan(12, prec=1)
    a = (cs["kx"], cs["ky"], cs["kz"], cs["kw"])
    frames = [dict(kx=cs["kx"], ky=cs["ky"], kz=cs["kz"], kw=cs["kw"], data=cs["data"])]
    XX, im, resid, done = O.clear(frames, oracle_lib.clear_params(max_iter=1, alpha_coil=0.0))
    assert done == 1
    zero = np.zeros(O.ishape, np.complex128)
    R, P = [], []
    for c in range(3):
        r = O.adjoint(np.zeros(O.ishape), None, O.forward(zero, None, *a, diff=cs["data"][c]), *a)
        R.append(r)
        P.append(O.adjoint(np.zeros(O.ishape), None, O.forward(r, None, *a), *a))
    rr = sum(np.vdot(r, r).real for r in R)
    pr = sum(np.sum(p * np.conj(r)) for p, r in zip(P, R))
    ref = np.stack([-(rr / pr) * r for r in R])
    assert rel(XX[0], ref) < 1e-12
    assert abs(resid[0] - rr) <= 1e-12 * rr


def test_clear_loop_reduces_data_error(oracle_lib):
    cs = case(N=12, C=3, nproj=200, seed=6, nudft=True)
    O = oracle_lib.Plan(12, prec=1)
    a = (cs["kx"], cs["ky"], cs["kz"], cs["kw"])
    frames = [dict(kx=cs["kx"], ky=cs["ky"], kz=cs["kz"], kw=cs["kw"], data=cs["data"])]

    def err(XX):
        return sum(np.linalg.norm((O.forward(XX[0, c], None, *a) - cs["data"][c]) * np.sqrt(cs["kw"])) ** 2
                   for c in range(3))
    XX1, _, _, _ = O.clear(frames, oracle_lib.clear_params(max_iter=1, bs=(4, 4, 4)))
    XX6, im, resid, done = O.clear(frames, oracle_lib.clear_params(max_iter=6, bs=(4, 4, 4)))
    e0 = sum(np.linalg.norm(d * np.sqrt(cs["kw"])) ** 2 for d in cs["data"])
    assert done == 6 and err(XX6) < err(XX1) < e0
    assert np.all(np.isfinite(im)) and np.abs(im).max() > 0


def test_clear_l1_threshold_by_hand(oracle_lib):
    """One iteration with the loop's L1 threshold and no coil threshold: the gradient step,
    then on frame 0's coil images the DB4 wavelet at the glibc rand() shifts after rand_skip
    draws, the fraction threshold over all coils, the soft threshold, the inverse wavelet."""
    cs = case(N=16, C=3, nproj=200, seed=8)
    O = oracle_lib.Plan(16, prec=1)
    frames = [dict(kx=cs["kx"], ky=cs["ky"], kz=cs["kz"], kw=cs["kw"], data=cs["data"])]
    plain, _, _, _ = O.clear(frames, oracle_lib.clear_params(max_iter=1, alpha_coil=0.0))
    q = oracle_lib.clear_params(max_iter=1, alpha_coil=0.0, use_threshold=1, thresh=0.3, cycle_spins=1,
                                wave_levels=(2, 2, 2), wave_type=1, rand_skip=7)
    got, _, _, _ = O.clear(frames, q)
    r = oracle_lib.glibc_rand(7, 3)
    shift = tuple(int(v) % 4 for v in r)
    W = [oracle_lib.wavelet(plain[0, c], (2, 2, 2), shift, 1) for c in range(3)]
    thr = oracle_lib.fraction_threshold(W, 0.3)
    ref = np.stack([oracle_lib.wavelet(oracle_lib.soft_threshold(w, thr), (2, 2, 2), shift, 1, inverse=True)
                    for w in W])
    assert rel(got[0], ref) < 1e-12
    assert rel(got[0], plain[0]) > 1e-3
