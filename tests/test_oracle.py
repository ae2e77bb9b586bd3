"""The oracle (CPU restatement of the reference) checked against independent
implementations: numpy's FFT, scipy's I0, libc's rand(), the closed-form
Daubechies-4 filters and the reference's literal filter values, and the
adjoint identity of its own E / E^H."""
import ctypes
import subprocess
import sys

import numpy as np
import pytest

from tests.helpers import case, rel


@pytest.mark.parametrize("n", [24, 48, 96, 144, 192, 384, 160])
def test_fft1d_vs_numpy(oracle_lib, n):
    O = oracle_lib
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    assert rel(O.fft1d(x, -1, 1), np.fft.fft(x)) < 1e-13
    assert rel(O.fft1d(x, +1, 1), np.fft.ifft(x) * n) < 1e-13
    assert rel(O.fft1d(x, -1, 0), np.fft.fft(x)) < 5e-7


def test_fft3_pruned_equals_full(oracle_lib):
    """do_fft prunes lines that are zero; the result equals the full 3D FFT."""
    O = oracle_lib
    p = O.Plan(32, prec=1)
    rng = np.random.default_rng(0)
    X = rng.standard_normal(p.ishape) + 1j * rng.standard_normal(p.ishape)
    g = p.set_image(X, None)
    S3 = np.prod(p.S)
    ref = np.fft.fftn(g) / np.sqrt(S3)
    assert rel(p.fft3(g, -1), ref) < 1e-12
    ref_b = np.fft.ifftn(g) * S3 / np.sqrt(S3)
    assert rel(p.fft3(g, +1), ref_b) < 1e-12


def test_kaiser_lut_vs_scipy_i0(oracle_lib):
    scipy_special = pytest.importorskip("scipy.special")
    p = oracle_lib.Plan(64, prec=0)
    lut, _ = p.tables()
    beta = p.beta[0]
    glen = int(round(p.dwin[0] * 600))
    u = np.arange(glen + 1) / glen
    ref = scipy_special.i0(beta * np.sqrt(1 - u * u)) / scipy_special.i0(beta)
    got = lut[0, :glen + 1] / lut[0, 0]
    assert np.max(np.abs(got - ref / ref[0])) < 2e-6
    assert np.all(lut[0, glen + 1:] == 0)
    assert abs(lut[0].sum(dtype=np.float64) - 300.0) < 1e-3


def test_geometry_sizes(oracle_lib):
    for N, S, og in [(64, 96, 16), (96, 144, 24), (128, 192, 32), (256, 384, 64), (32, 48, 8)]:
        p = oracle_lib.Plan(N)
        assert p.S == (S, S, S) and p.og == (og, og, og)


def test_fp32_vs_fp64_operators(oracle_lib):
    O = oracle_lib
    c = case(N=32, C=1, nproj=400)
    p32, p64 = O.Plan(32, prec=0), O.Plan(32, prec=1)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    e32 = p32.forward(c["X"], c["smaps"][0], *a)
    e64 = p64.forward(c["X"], c["smaps"][0], *a)
    assert rel(e32, e64) < 1e-5
    h32 = p32.adjoint(np.zeros(p32.ishape, np.complex64), c["smaps"][0], c["data"][0], *a)
    h64 = p64.adjoint(np.zeros(p64.ishape, np.complex128), c["smaps"][0], c["data"][0], *a)
    assert rel(h32, h64) < 1e-5


def test_adjoint_identity_fp64(oracle_lib):
    """<E x, W d> == <x, E^H d> with W = kw * taper (E^H applies kw, E does not)."""
    O = oracle_lib
    c = case(N=32, C=1, nproj=300)
    p = O.Plan(32, prec=1)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    Ex = p.forward(c["X"], c["smaps"][0], *a)
    EHd = p.adjoint(np.zeros(p.ishape, np.complex128), c["smaps"][0], c["data"][0], *a)
    k2 = c["kx"].astype(np.float64) ** 2 + c["ky"].astype(np.float64) ** 2 + c["kz"].astype(np.float64) ** 2
    W = c["kw"] * np.exp(-k2 / (2 * 9999.0 ** 2))
    lhs = np.vdot(Ex, W * c["data"][0].astype(np.complex128))
    rhs = np.vdot(c["X"].astype(np.complex128), EHd)
    assert abs(lhs - rhs) / abs(lhs) < 1e-11


def test_gridding_approximates_nudft(oracle_lib):
    """Approximation accuracy of the reference algorithm against a direct NUDFT
    (reported, not a parity criterion): a 5-point Kaiser-Bessel kernel at 1.5x."""
    from mri_recon_gb300 import synth
    O = oracle_lib
    N = 32
    c = case(N=N, C=1, nproj=200)
    p = O.Plan(N, prec=1)
    a = (c["kx"], c["ky"], c["kz"], np.ones_like(c["kw"]))
    Ex = p.forward(c["img"], None, *a)
    y = synth.nudft(c["img"], c["kx"], c["ky"], c["kz"])
    scale = np.vdot(y, Ex) / np.vdot(y, y)
    err = rel(Ex, scale * y)
    assert err < 5e-3, err


def test_glibc_rand_stream(oracle_lib):
    libc = ctypes.CDLL(None)
    if not hasattr(libc, "rand"):
        pytest.skip("no libc rand")
    # a fresh process: rand() without srand() starts from seed 1
    code = "import ctypes; L=ctypes.CDLL(None); print(' '.join(str(L.rand()) for _ in range(40)))"
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, check=True).stdout.split()
    ref = np.array([int(v) for v in out])
    assert np.array_equal(oracle_lib.glibc_rand(0, 40), ref)
    assert np.array_equal(oracle_lib.glibc_rand(7, 10), ref[7:17])


def test_db4_filters_match_reference_values(oracle_lib):
    # the reference's DB4 literals (src/wavelet3D.cpp:168-186), as float32
    ref_lpf = np.float32([-0.1294095225509214500000, 0.2241438680418573500000, 0.8365163037374689900000,
                          0.4829629131446902500000])
    L, f = oracle_lib.wavelet_info((64, 64, 64), (3, 3, 3), 1)
    assert np.array_equal(f[0], ref_lpf)
    assert np.array_equal(f[1], np.float32([-ref_lpf[3], ref_lpf[2], -ref_lpf[1], ref_lpf[0]]))
    assert np.array_equal(f[2], ref_lpf[::-1])
    assert np.array_equal(f[3], np.float32([ref_lpf[0], -ref_lpf[1], ref_lpf[2], -ref_lpf[3]]))
    assert L == (3, 3, 3)
    L2, _ = oracle_lib.wavelet_info((48, 40, 64), (4, 4, 4), 1)
    assert L2 == (4, 3, 4)


def test_wavelet_perfect_reconstruction(oracle_lib):
    rng = np.random.default_rng(3)
    X = rng.standard_normal((32, 32, 32)) + 1j * rng.standard_normal((32, 32, 32))
    # the filters are the reference's float32 values, orthonormal to ~1e-8
    for shift in ((0, 0, 0), (1, 2, 3), (3, 3, 1)):
        W = oracle_lib.wavelet(X, (3, 3, 3), shift)
        assert abs(np.linalg.norm(W) - np.linalg.norm(X)) / np.linalg.norm(X) < 1e-6
        assert rel(oracle_lib.wavelet(W, (3, 3, 3), shift, inverse=True), X) < 1e-6


def test_fraction_threshold_hits_target(oracle_lib):
    rng = np.random.default_rng(5)
    vols = [(rng.standard_normal((16, 16, 16)) + 1j * rng.standard_normal((16, 16, 16))).astype(np.complex64)
            for _ in range(2)]
    t = oracle_lib.fraction_threshold(vols, 0.3)
    frac = np.mean(np.abs(np.concatenate([v.ravel() for v in vols])) < t)
    assert abs(frac - 0.3) <= 0.0011
    y = oracle_lib.soft_threshold(vols[0], t)
    mag = np.abs(vols[0])
    expect = np.where(mag <= t, 0, vols[0] * (1 - t / np.maximum(mag, 1e-30)))
    assert rel(y, expect) < 1e-6


def test_llr_jacobi_svd_vs_numpy(oracle_lib):
    rng = np.random.default_rng(11)
    Nt, N = 5, 16
    vols = [(rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))) for _ in range(Nt)]
    smax = oracle_lib.llr_update_threshold(vols, (8, 8, 8), amp=4.0, t2=6.0, iteration=0)
    s1 = []
    for bz in range(2):
        for by in range(2):
            for bx in range(2):
                A = np.stack([v[bz * 8:(bz + 1) * 8, by * 8:(by + 1) * 8, bx * 8:(bx + 1) * 8].ravel() for v in vols], 1)
                s1.append(np.linalg.svd(A, compute_uv=False)[0])
    assert abs(smax - np.median(s1) * (1 + 4.0)) / smax < 1e-5
    # thresholding with block_iter = 1 (no shift): singular values shrink by alpha*smax
    out = oracle_lib.llr_thresh(vols, (8, 8, 8), 1, 0.5, smax, 0)
    A = np.stack([v[:8, :8, :8].ravel() for v in vols], 1)
    U, s, Vh = np.linalg.svd(A, full_matrices=False)
    ref = (U * np.maximum(s - 0.5 * smax, 0)) @ Vh
    got = np.stack([v[:8, :8, :8].ravel() for v in out], 1)
    assert rel(got, ref) < 1e-10


def _blur_literal(X, sigma):
    """gaussian_blur_template written out loop by loop in numpy (float32 taps)."""
    X = X.astype(np.complex128).copy()
    for d, s in enumerate(sigma):  # axes x, y, z of a [z][y][x] array
        if s <= 0:
            continue
        w = int(5 * s)
        t = np.arange(2 * w + 1, dtype=np.float32) - np.float32(w)
        k = np.exp(-(t * t).astype(np.float64) / (2.0 * np.float64(np.float32(s) * np.float32(s)))).astype(np.float32)
        k = (k / k.astype(np.float64).sum()).astype(np.float32)
        ax = 2 - d
        Y = np.moveaxis(X, ax, -1).copy()
        out = np.zeros_like(Y)
        n = Y.shape[-1]
        for i in range(n):
            for ii in range(max(i - w, 0), min(i + w, n)):
                out[..., i] += k[ii - (i - w)] * Y[..., ii]
        X = np.moveaxis(out, -1, ax)
    return X


def test_gaussian_blur_vs_literal(oracle_lib):
    rng = np.random.default_rng(1)
    X = (rng.standard_normal((9, 10, 11)) + 1j * rng.standard_normal((9, 10, 11))).astype(np.complex64)
    for sigma in [(1.0, 0.0, 0.0), (0.0, 0.6, 0.0), (0.0, 0.0, 1.4), (0.8, 1.1, 0.5)]:
        got = oracle_lib.gaussian_blur(X.astype(np.complex128), sigma)
        assert np.max(np.abs(got - _blur_literal(X, sigma))) < 1e-12
    # the upper tap ii = i + w is excluded, as in the reference's loop bound
    e = np.zeros((1, 1, 9), np.complex128)
    e[0, 0, 4] = 1.0
    out = oracle_lib.gaussian_blur(e, (1.0, 0.0, 0.0))
    # w = 5: output i reads ii in [i - 5, i + 5) through tap ii - i + 5, so an impulse
    # at ii = 4 shows tap 9 - i at output i; tap 10 (ii = i + 5) never contributes
    k = np.exp(-(np.arange(11, dtype=np.float32) - 5) ** 2 / 2.0).astype(np.float32)
    k = (k / k.astype(np.float64).sum()).astype(np.float32)
    for i in range(9):
        t = 4 - (i - 5)
        expect = k[t] if 0 <= t < 10 else 0.0
        assert abs(out[0, 0, i] - expect) < 1e-7


def test_sos_normalize_vs_numpy(oracle_lib):
    rng = np.random.default_rng(2)
    A = (rng.standard_normal((4, 6, 7, 8)) + 1j * rng.standard_normal((4, 6, 7, 8))).astype(np.complex128)
    got = oracle_lib.sos_normalize(A)
    ref = A / np.sqrt(np.sum(np.abs(A) ** 2, 0))
    assert np.max(np.abs(got - ref)) < 1e-12


def test_adjoint_sos_is_squared_map_free_adjoint(oracle_lib):
    c = case(N=24, C=2, nproj=300)
    p = oracle_lib.Plan(24)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    X = np.zeros(p.ishape, np.complex64)
    ref = np.zeros(p.ishape, np.float32)
    for k in range(2):
        X = p.adjoint_sos(X, c["data"][k], *a)
        im = p.adjoint(np.zeros(p.ishape, np.complex64), None, c["data"][k], *a)
        ref = ref + (im.real * im.real + im.imag * im.imag)
    # the oracle's gridding adds with OpenMP atomics, so two runs differ in the last bits
    assert rel(X.real, ref) < 1e-6 and np.all(X.imag == 0)


def test_lowres_smaps_unit_sos_and_taper(oracle_lib):
    c = case(N=24, C=3, nproj=400, nudft=True)
    p = oracle_lib.Plan(24)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    maps = oracle_lib.lowres_smaps(p, c["data"], *a, smap_res=8.0)
    assert np.allclose(np.sqrt(np.sum(np.abs(maps.astype(np.complex128)) ** 2, 0)), 1.0, atol=1e-5)
    # k_rad 8 is a strong low-pass: the map images are smoother than the full-resolution ones
    full = p.adjoint(np.zeros(p.ishape, np.complex64), None, c["data"][0], *a)
    p.set_k_rad(8.0)
    low = p.adjoint(np.zeros(p.ishape, np.complex64), None, c["data"][0], *a)
    p.set_k_rad(9999.0)
    def hf(v):
        return np.linalg.norm(np.diff(v, axis=2)) / np.linalg.norm(v)
    assert hf(low) < 0.8 * hf(full)


def test_dcf_table_and_weights(oracle_lib):
    """The polynomial kernel table (length (int)(2.1*600)+100, sum 0.5*600) and the Pipe
    weights: FP32 restatement close to FP64, growing with |k| on a radial trajectory."""
    from mri_recon_gb300 import synth
    t = oracle_lib.dcf_table(2.1, 0)
    assert t.size == 1360 and abs(float(t.astype(np.float64).sum()) - 300.0) < 1e-3
    assert t[0] > t[600] > t[1200]
    kx, ky, kz, _ = synth.radial_trajectory(20, 300, 20, seed=2)
    w32 = oracle_lib.dcf_pipe(kx, ky, kz, 20, iters=8)
    w64 = oracle_lib.dcf_pipe(kx, ky, kz, 20, iters=8, prec=1)
    assert rel(w32, w64) < 1e-5
    prof = w64.reshape(300, 20).mean(0)
    assert np.all(np.diff(prof[2:15]) > 0)
