"""The oracle restatement (and the library's host-side tables) against the reference's own
code: src/gridFFT.cpp, src/ArrayTemplates.cpp, src/wavelet3D.cpp, src/threshold.cpp and
src/clear.cpp compiled unmodified into oracle/_ref/libref.so (``make -C oracle ref``,
stand-in headers for Blitz++ / FFTW / Armadillo / HDF5 in oracle/refshim).

Tolerances: tables bit for bit; operators and stages at relative L2 <= 1e-6 (both sides
FP32; the reference adds its gridding with unordered OpenMP atomics and its stand-in FFT
rounds a double-precision transform, so the last bits differ); wavelets and thresholds
at 1e-6; the low-rank block operations of LOWRANKCOIL (SVDs in double on both sides, a
one-sided Jacobi here and in the Armadillo stand-in) at 1e-6.  These tests need the reference sources and are skipped where they are absent
(the GPU host).
"""
import ctypes

import numpy as np
import pytest

from tests.helpers import align_block_phases, aniso_case, case, edge_trajectory, low_rank_frames, rel

R = pytest.importorskip("oracle.ref")
if not R.available():
    pytest.skip("reference sources not present: oracle/_ref cannot be built here", allow_module_level=True)

TOL = 1e-6


@pytest.fixture(scope="module")
def O():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.mark.parametrize("kernel", [1, 0, 2, 3])
@pytest.mark.parametrize("N,overgrid", [(32, 1.5), (64, 1.5), (96, 1.5), ((40, 48, 24), 1.5), (64, 1.375),
                                        (32, 2.0)])
def test_tables_equal_reference(O, mrg_lib, kernel, N, overgrid):
    """precalc_gridding / precalc_kernel: S, crop, beta, kernel tables and deapodisation
    windows, bit for bit, from the oracle and from the library's host code."""
    g = R.Gridder(N, overgrid=overgrid, kernel=kernel)
    o = O.Plan(N, overgrid=overgrid, kernel=kernel)
    lut, win = o.tables()
    assert g.S == o.S and g.og == o.og
    assert g.beta == o.beta
    assert np.array_equal(g.lut, lut)
    for a, b in zip(g.win, win):
        assert np.array_equal(a, b)
    # the library's tables (mrg_plan_geometry, no GPU needed)
    from mri_recon_gb300._lib import MrgConfig, _fp
    L = mrg_lib.load()
    cfg = MrgConfig()
    L.mrg_config_default(ctypes.byref(cfg))
    cfg.kernel_type, cfg.overgrid = kernel, overgrid
    Nx, Ny, Nz = (N, N, N) if np.isscalar(N) else N
    S, og, gr, be, ll = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), (ctypes.c_float * 3)(), (ctypes.c_float * 3)(), \
        ctypes.c_int()
    assert L.mrg_plan_geometry(ctypes.byref(cfg), Nx, Ny, Nz, S, og, gr, be, ctypes.byref(ll), None, None) == 0
    mlut = np.zeros(3 * ll.value, np.float32)
    mwin = np.zeros(sum(S), np.float32)
    assert L.mrg_plan_geometry(ctypes.byref(cfg), Nx, Ny, Nz, S, og, gr, be, ctypes.byref(ll),
                               mlut.ctypes.data_as(_fp), mwin.ctypes.data_as(_fp)) == 0
    assert tuple(S) == g.S and tuple(og) == g.og and tuple(be) == g.beta
    assert np.array_equal(mlut.reshape(3, -1), g.lut)
    assert np.array_equal(mwin, np.concatenate(g.win))


@pytest.mark.parametrize("kernel", [1, 0, 2, 3])
@pytest.mark.parametrize("N,overgrid", [(32, 1.375), (64, 1.5), ((40, 48, 24), 1.375), (32, 2.0)])
def test_coil_threaded_tables_equal_gridfft(kernel, N, overgrid):
    """gridFFT_CoilThreaded::precalc_gridding builds the same S, crop, beta, kernel tables and
    windows as gridFFT::precalc_gridding, bit for bit (so a plan's tables serve both)."""
    g = R.Gridder(N, overgrid=overgrid, kernel=kernel)
    S, og, be, lut, win = g.coils_tables(C=3)
    assert S == g.S and og == g.og and be == g.beta
    assert np.array_equal(lut, g.lut)
    assert np.array_equal(win, np.concatenate(g.win))


def _traj(N, nproj, seed=3):
    c = case(N=N, C=1, nproj=nproj, seed=seed)
    return c, (c["kx"], c["ky"], c["kz"], c["kw"])


def test_gridding_and_ungridding_match_reference(O):
    """chop_grid_forward and chop_grid_backward on the 64^3 SENSE-CG geometry (4096 x 64
    radial), and on samples at the grid edge, outside it, at kw == 0 and at half-integer
    positions."""
    c, a = _traj(64, 4096)
    g, o = R.Gridder(64), O.Plan(64)
    d = c["data"][0]
    assert rel(o.grid(d, *a), g.grid(d, *a)) < TOL
    rng = np.random.default_rng(4)
    grid = (rng.standard_normal(g.gshape) + 1j * rng.standard_normal(g.gshape)).astype(np.complex64)
    assert rel(o.ungrid(grid, *a), g.ungrid(grid, *a)) < TOL
    assert rel(o.ungrid(grid, *a, diff=d), g.ungrid(grid, *a, diff=d)) < TOL
    e = edge_trajectory(32)
    g32, o32 = R.Gridder(32), O.Plan(32)
    de = (rng.standard_normal(e[0].size) + 1j * rng.standard_normal(e[0].size)).astype(np.complex64)
    assert rel(o32.grid(de, *e), g32.grid(de, *e)) < TOL
    grid32 = (rng.standard_normal(g32.gshape) + 1j * rng.standard_normal(g32.gshape)).astype(np.complex64)
    ue, ur = o32.ungrid(grid32, *e), g32.ungrid(grid32, *e)
    assert rel(ue, ur) < TOL
    assert np.array_equal(ue == 0, ur == 0)  # the same samples are dropped


@pytest.mark.parametrize("N", [32, (40, 24, 56)])
def test_fft_passes_match_reference(O, N):
    """do_fft (pruned: only the crop is read) and do_ifft."""
    g, o = R.Gridder(N), O.Plan(N)
    rng = np.random.default_rng(6)
    grid = (rng.standard_normal(g.gshape) + 1j * rng.standard_normal(g.gshape)).astype(np.complex64)
    assert rel(o.fft3(grid, +1), g.fft(grid, inverse=True)) < TOL
    # the forward transform of a grid holding an image in its crop, as set_image leaves it
    img = np.zeros(g.gshape, np.complex64)
    Nx, Ny, Nz = g.N
    sx, sy, sz = g.og
    img[sz:sz + Nz, sy:sy + Ny, sx:sx + Nx] = grid[sz:sz + Nz, sy:sy + Ny, sx:sx + Nx]
    assert rel(o.fft3(img, -1), g.fft(img, inverse=False)) < TOL


@pytest.mark.parametrize("kernel", [1, 0, 2, 3])
def test_operators_match_reference(O, kernel):
    """gridFFT::backward (E), backward_residual and forward (E^H) with a coil map."""
    N = 64 if kernel == 1 else 32
    c, a = _traj(N, 4096 if N == 64 else 800, seed=9)
    g, o = R.Gridder(N, kernel=kernel), O.Plan(N, kernel=kernel)
    sm = c["smaps"][0]
    assert rel(o.forward(c["img"], sm, *a), g.forward(c["img"], sm, *a)) < TOL
    d = c["data"][0]
    assert rel(o.forward(c["img"], sm, *a, diff=d), g.forward(c["img"], sm, *a, diff=d)) < TOL
    X0 = c["X"] * np.complex64(0.1)
    assert rel(o.adjoint(X0.copy(), sm, d, *a), g.adjoint(X0, sm, d, *a)) < TOL


@pytest.mark.parametrize("N,overgrid,kernel,dwin", [((40, 24, 32), 1.375, 1, -1.0), ((24, 32, 16), 2.0, 1, 2.0),
                                                     ((32, 24, 24), 1.5, 0, 1.5), ((16, 24, 32), 1.5, 2, -1.0)])
def test_anisotropic_operators_match_reference(O, N, overgrid, kernel, dwin):
    """gridFFT's E, residual E and E^H on anisotropic images at other overgrid factors and
    kernel widths (each axis has its own S, crop and window)."""
    c = aniso_case(N, 2, 300, seed=60)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    g = R.Gridder(N, overgrid=overgrid, kernel=kernel, dwin=dwin)
    o = O.Plan(N, overgrid=overgrid, kernel=kernel, dwin=dwin)
    assert g.gshape == o.gshape
    for k in range(2):
        sm, d = c["smaps"][k], c["data"][k]
        assert rel(o.forward(c["img"], sm, *a), g.forward(c["img"], sm, *a)) < TOL
        assert rel(o.forward(c["img"], sm, *a, diff=d), g.forward(c["img"], sm, *a, diff=d)) < TOL
        X0 = np.zeros(g.ishape, np.complex64)
        assert rel(o.adjoint(X0.copy(), sm, d, *a), g.adjoint(X0, sm, d, *a)) < TOL


def test_sum_of_squares_adjoint_matches_reference(O):
    """gridFFT::forward_sos (the map-free E^H whose squared magnitude is summed over coils,
    src/gridFFT.cpp:722-748, :960-970), three coils accumulated into one image, with a taper."""
    c = aniso_case((32, 24, 20), 3, 400, seed=61)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    g, o = R.Gridder((32, 24, 20), k_rad=10.0), O.Plan((32, 24, 20), k_rad=10.0)
    Xr = np.zeros(g.ishape, np.complex64)
    Xo = np.zeros(o.ishape, np.complex64)
    for k in range(3):
        Xr = g.adjoint_sos(Xr, c["data"][k], *a)
        Xo = o.adjoint_sos(Xo, c["data"][k], *a)
    assert rel(Xo, Xr) < TOL


def test_taper_radius_matches_reference(O):
    """E^H with the Gaussian taper of a small k_rad (the coil-map estimate's smap_res)."""
    c, a = _traj(32, 800, seed=10)
    g, o = R.Gridder(32, k_rad=8.0), O.Plan(32, k_rad=8.0)
    X0 = np.zeros(g.ishape, np.complex64)
    assert rel(o.adjoint(X0.copy(), c["smaps"][0], c["data"][0], *a), g.adjoint(X0, c["smaps"][0], c["data"][0], *a)) < TOL


def test_fp64_oracle_against_reference(O):
    """The FP64 twin is as close to the FP32 reference as FP32 rounding allows."""
    c, a = _traj(64, 4096, seed=11)
    g, o64 = R.Gridder(64), O.Plan(64, prec=1)
    X0 = np.zeros(g.ishape, np.complex64)
    d = c["data"][0]
    assert rel(o64.adjoint(X0.astype(np.complex128), c["smaps"][0], d, *a), g.adjoint(X0, c["smaps"][0], d, *a)) < 1e-5


@pytest.mark.parametrize("wtype", [1, 0])
@pytest.mark.parametrize("shape,levels,shift", [((32, 32, 32), (3, 3, 3), (0, 0, 0)), ((32, 32, 32), (3, 3, 3), (1, 2, 3)),
                                                ((16, 40, 48), (4, 4, 4), (3, 0, 2)), ((24, 24, 24), (2, 3, 4), (1, 1, 0))])
def test_wavelet_matches_reference(O, wtype, shape, levels, shift):
    """WAVELET3D forward3D / backward3D with the shifts random_shift would set."""
    rng = np.random.default_rng(12)
    X = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    f = R.wavelet(X, levels, shift, wtype)
    assert rel(O.wavelet(X, levels, shift, wtype), f) < TOL
    assert rel(O.wavelet(f, levels, shift, wtype, inverse=True), R.wavelet(f, levels, shift, wtype, inverse=True)) < TOL


@pytest.mark.parametrize("fraction", [0.1, 0.5, 0.9])
def test_fraction_threshold_matches_reference(O, fraction):
    """THRESHOLD::get_threshold (bisection, its thresh * max starting bound) and the
    grouped-complex soft threshold over several frames."""
    rng = np.random.default_rng(13)
    vols = [(rng.standard_normal((24, 24, 24)) + 1j * rng.standard_normal((24, 24, 24))).astype(np.complex64)
            for _ in range(3)]
    t_ref, out_ref = R.fraction_threshold(vols, fraction, apply=True)
    t = O.fraction_threshold(vols, fraction)
    assert abs(t - t_ref) <= 1e-6 * t_ref
    for v, r in zip(vols, out_ref):
        assert rel(O.soft_threshold(v, t), r) < TOL


# (frames, (Nx, Ny, Nz), block, iteration): cubic and anisotropic blocks, blocks that do not
# divide the image, a block larger than the image (update_threshold clamps it)
LLR_CASES = [(6, (16, 12, 8), (4, 4, 4), 2), (10, (16, 16, 16), (8, 8, 8), 0), (4, (12, 8, 8), (8, 4, 2), 7),
             (5, (8, 8, 4), (16, 16, 16), 1)]


@pytest.mark.parametrize("T,N,bs,it", LLR_CASES)
def test_time_low_rank_threshold_matches_reference(O, T, N, bs, it):
    """LOWRANKCOIL::update_threshold(image, 0, iteration) (src/clear.cpp:233-351): the median
    of the blocks' sigma_1 times the amplitude schedule."""
    X = low_rank_frames(np.random.default_rng(21 + T), T, N[::-1])
    vols = [X[t] for t in range(T)]
    r = R.llr_update_threshold(vols, bs, 4.0, 6.0, it)
    assert abs(O.llr_update_threshold(vols, bs, 4.0, 6.0, it) - r) <= TOL * r
    assert abs(O.llr_update_threshold([v.astype(np.complex128) for v in vols], bs, 4.0, 6.0, it) - r) <= TOL * r


@pytest.mark.parametrize("T,N,bs,it", LLR_CASES)
@pytest.mark.parametrize("block_iter,rand_skip", [(4, 0), (4, 1000), (1, 5)])
def test_time_low_rank_thresh_matches_reference(O, T, N, bs, it, block_iter, rand_skip):
    """LOWRANKCOIL::thresh(image, 0) (src/clear.cpp:356-556): rand() block shifts (none when
    block_iter is 1), per block A <- U max(s - alpha smax / block_iter, 0) V^H, in place."""
    X = low_rank_frames(np.random.default_rng(31 + T), T, N[::-1])
    vols = [X[t] for t in range(T)]
    bsc = tuple(min(b, n) for b, n in zip(bs, N))
    smax = R.llr_update_threshold(vols, bsc, 4.0, 6.0, it)
    r = np.stack(R.llr_thresh(vols, bsc, block_iter, 0.1, smax, rand_skip))
    assert rel(r, X) > 1e-2  # the threshold changed the frames
    assert rel(np.stack(O.llr_thresh(vols, bs, block_iter, 0.1, smax, rand_skip)), r) < TOL
    assert rel(np.stack(O.llr_thresh([v.astype(np.complex128) for v in vols], bs, block_iter, 0.1, smax,
                                     rand_skip)), r) < TOL


# (frames, coils, (Nx, Ny, Nz), block): frames <= coils, as the reference's update_threshold
# with dim = 2 requires
COIL_CASES = [(2, 6, (8, 8, 8), (4, 4, 4)), (1, 8, (12, 8, 8), (4, 4, 2)), (3, 5, (10, 12, 8), (4, 3, 4)),
              (1, 16, (8, 8, 8), (8, 8, 8))]


def _coil_stack(T, C, N, seed):
    rng = np.random.default_rng(seed)
    return np.stack([low_rank_frames(rng, C, N[::-1]) for _ in range(T)])  # (T, C, Nz, Ny, Nx)


@pytest.mark.parametrize("T,C,N,bs", COIL_CASES)
def test_coil_low_rank_matches_reference(O, T, C, N, bs):
    """LOWRANKCOIL in the coil dimension: update_threshold(image, 2) (src/clear.cpp:99-232,
    the column index t quirk included), thresh(image, 2) (:561-813, full SVDs) and combine
    (:815-914) against the reference.  combine is compared after giving each block the
    unit phase of the oracle's (its first right singular vector's phase is free)."""
    XX = _coil_stack(T, C, N, 41 + C)
    r = R.clear_update_threshold(XX, bs, 4.0, 6.0, 1)
    assert abs(O.clear_update_threshold(XX, bs, 4.0, 6.0, 1) - r) <= TOL * r
    for block_iter, skip in [(4, 5), (1, 0)]:
        Y = R.clear_thresh(XX, bs, block_iter, 0.05, r, skip)
        assert rel(Y, XX) > 1e-3
        assert rel(O.clear_thresh(XX, bs, block_iter, 0.05, r, skip), Y) < TOL
        assert rel(O.clear_thresh(XX.astype(np.complex128), bs, block_iter, 0.05, r, skip), Y) < TOL
    im_ref = R.clear_combine(XX, bs)
    im = O.clear_combine(XX, bs)
    assert rel(np.abs(im), np.abs(im_ref)) < TOL
    assert rel(im, align_block_phases(im, im_ref, bs)) < TOL


@pytest.mark.parametrize("N,C,overgrid,kernel", [((20, 24, 16), 3, 1.375, 1), ((24, 24, 24), 2, 1.5, 1),
                                                 ((16, 16, 24), 4, 1.5, 0), ((16, 16, 16), 2, 1.5, 3)])
def test_coil_threaded_matches_oracle(O, N, C, overgrid, kernel):
    """gridFFT_CoilThreaded::backward (E of every coil), backward_residual and forward (E^H
    summed over the coils) (src/gridFFT_CoilThreaded.cpp:965-1120, its default overgrid
    1.375 in the first case) equal the oracle's per-coil gridFFT operators times
    sqrt(Sx Sy Sz): the class's FFTW transforms are unnormalised (:570-893) where gridFFT's
    fft3 scales each axis by 1/sqrt(S)."""
    c = aniso_case(N, C, 150, seed=50 + C)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    g, o = R.Gridder(N, overgrid=overgrid, kernel=kernel), O.Plan(N, overgrid=overgrid, kernel=kernel)
    f = np.sqrt(float(np.prod(g.S)))
    E = np.stack([o.forward(c["img"], c["smaps"][k], *a) for k in range(C)])
    assert rel(g.coils_forward(c["img"], c["smaps"], *a), f * E) < TOL
    d = c["data"]
    # residual: f E - d, and 0 at the samples with kw == 0 (src/gridFFT_CoilThreaded.cpp chop_grid_backward)
    Er = np.stack([o.forward(c["img"], c["smaps"][k], *a, diff=(d[k] / np.float32(f)).astype(np.complex64))
                   for k in range(C)])
    assert rel(g.coils_forward(c["img"], c["smaps"], *a, diff=d), f * Er) < TOL
    EH = sum(o.adjoint(np.zeros(o.ishape, np.complex64), c["smaps"][k], d[k], *a) for k in range(C))
    assert rel(g.coils_adjoint(np.zeros(g.ishape, np.complex64), c["smaps"], d, *a), f * EH) < TOL


@pytest.mark.parametrize("kernel", [0, 1])
@pytest.mark.parametrize("dwin", [2.1, 1.8, 2.5, 3.0])
def test_dcf_table_equals_reference(O, kernel, dwin):
    """DCFgridFFT::precalc_kernel's polynomial table (POLY_KERNEL, POLY_KERNEL2), its length
    (int)(dwin * 600) + 100 and its normalisation to sum 300, bit for bit."""
    assert np.array_equal(O.dcf_table(dwin, kernel), R.dcf_table(dwin, kernel))


@pytest.mark.parametrize("N,params", [(32, dict()), (48, dict(iters=5, dwin=2.5, overgrid=2.0)),
                                      (40, dict(kernel=1, acc=1.5, scale=0.9)),
                                      ((40, 32, 24), dict(iters=10)), ((24, 32, 40), dict(kernel=1, acc=1.5))])
def test_dcf_matches_reference(O, N, params):
    """RECON::dcf_calc's Pipe iteration around the reference's own DCFgridFFT (forward,
    backward, scale_kw; src/DCFgridFFT.cpp), including anisotropic matrices, whose DCF image
    recon_lib allocates with the x and z extents swapped (src/recon_lib.cpp:873-875)."""
    m = N if np.isscalar(N) else max(N)
    c = case(N=m, C=1, nproj=800, seed=3)
    Nt = (N, N, N) if np.isscalar(N) else N
    kx, ky, kz = (c[k] * np.float32(Nt[d] / m) for d, k in enumerate(("kx", "ky", "kz")))
    r = R.dcf_pipe(kx, ky, kz, N, **params)
    assert rel(O.dcf_pipe(kx, ky, kz, N, **params), r) < TOL
    assert rel(O.dcf_pipe(kx, ky, kz, N, prec=1, **params), r) < TOL


@pytest.mark.parametrize("N,C,kr,cr,square", [((12, 12, 12), 3, (2.0, 2.0, 2.0), (5, 5, 5), False),
                                              ((12, 10, 8), 2, (1.5, 2.0, 1.0), (4, 4, 3), False),
                                              ((16, 16, 16), 4, (2.0, 2.0, 2.0), (6, 6, 6), True),
                                              ((24, 20, 1), 3, (2.0, 2.0, 0.0), (6, 5, 0), False)])
def test_espirit_matches_reference(O, N, C, kr, cr, square):
    """SPIRIT::generateEigenCoils (src/spirit.cpp:137-550: ifft to k-space, the calibration
    matrix and its SVD, the kernels in image space, per-voxel dominant vectors,
    phase_correct) compiled unmodified, against the oracle, where the dominant vector is
    well defined ((s2/s1)^2 < 0.9; elsewhere any vector of the top pair is a valid answer)."""
    from mri_recon_gb300 import synth
    Nx, Ny, Nz = N
    n = max(N)
    cut = tuple(slice(n // 2 - m // 2, n // 2 - m // 2 + m) for m in (Nz, Ny, Nx))  # central block
    img = synth.phantom(n, 6, seed=3)[cut]
    sm = synth.coil_maps(n, C, seed=4)[(slice(None),) + cut]
    imgs = (img[None] * sm).astype(np.complex64)
    r = R.espirit(imgs, kr, cr, square=square)
    o, _, _, ratio = O.espirit(imgs, kr_f=kr, cr=cr, square=square)
    m = ratio < 0.9
    assert m.mean() > 0.5
    assert rel(o[:, m], r[:, m]) < TOL


@pytest.mark.parametrize("shape,sigma", [((16, 20, 24), (1.0, 1.0, 1.0)), ((12, 16, 20), (0.5, 2.0, 0.0)),
                                         ((20, 12, 16), (3.0, 0.7, 1.3))])
def test_gaussian_blur_matches_reference(O, shape, sigma):
    """NDarray::gaussian_blur (src/ArrayTemplates.cpp:489-608: taps [max(i - w, 0),
    min(i + w, n)) with w = (int)(5 sigma), normalised by their sum, an axis with sigma 0
    skipped), the blur of the low-resolution coil-map estimate."""
    rng = np.random.default_rng(62)
    X = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    assert rel(O.gaussian_blur(X, sigma), R.gaussian_blur(X, sigma)) < TOL


@pytest.mark.parametrize("wtype", [0, 1])
@pytest.mark.parametrize("skip", [0, 7, 1000])
def test_cycle_spin_shifts_match_reference(mrg_lib, wtype, skip):
    """The wavelet shifts of L1_threshold's cycle spins: WAVELET3D::random_shift's rand() % wN
    (src/wavelet3D.cpp:443-448, wN 2 for DB2 and 4 for DB4 from its constructor) against the
    library's host stream (mrg_rand_stream) taken modulo the same wN."""
    n = 40
    ref = R.wavelet_shifts((32, 24, 16), (3, 3, 3), wtype, skip, n)
    out = (ctypes.c_int * (3 * n))()
    assert mrg_lib.load().mrg_rand_stream(skip, 3 * n, out) == 0
    wN = 2 if wtype == 0 else 4
    assert np.array_equal(np.array(out[:]).reshape(n, 3) % wN, ref)
