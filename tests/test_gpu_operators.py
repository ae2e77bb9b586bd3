"""GPU parity of the gridFFT operators against the oracle (relative L2 <= 1e-5
per operator application, the FP32 tolerance of the hot path)."""
import numpy as np
import pytest

from tests.helpers import case, edge_trajectory, rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


def fp64_bound(ref32, ref64):
    """Against the FP64 twin the GPU may not be closer than the reference's own
    FP32 arithmetic is: when the grid ratio S/N is not representable in float
    (e.g. 80/48) the FP32 reference itself sits ~1.7e-5 from FP64."""
    return max(TOL, 1.25 * rel(ref32, ref64))


def _torch():
    import torch
    return torch


def _plan(m, c, nframes=1, **kw):
    p = m.Plan(c["N"], c["C"], nframes, **kw)
    p.set_traj(0, c["kx"], c["ky"], c["kz"], c["kw"])
    p.set_smaps(c["smaps"])
    return p


def _oracle_E(O, c, prec, diff=None):
    p = O.Plan(c["N"], prec=prec)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    return np.stack([p.forward(c["X"], c["smaps"][k], *a, diff=None if diff is None else diff[k]) for k in range(c["C"])])


def _oracle_EH(O, c, prec):
    p = O.Plan(c["N"], prec=prec)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    X = np.zeros(p.ishape, p.cdt)
    for k in range(c["C"]):
        X = p.adjoint(X, c["smaps"][k], c["data"][k], *a)
    return X


# N = 8, 16, 40, 80: oversampled lines of 16, 32, 64 and 128 points
@pytest.mark.parametrize("N,C,nproj", [(32, 4, 700), (64, 8, 1500), (48, 3, 500), (8, 2, 60), (16, 4, 200),
                                       (40, 3, 600), (80, 2, 1500)])
def test_forward_E_matches_oracle(mrg_lib, oracle_lib, N, C, nproj):
    torch = _torch()
    c = case(N=N, C=C, nproj=nproj)
    p = _plan(mrg_lib, c)
    X = torch.from_numpy(c["X"]).cuda()
    y = p.forward(0, X).cpu().numpy()
    r32, r64 = _oracle_E(oracle_lib, c, 0), _oracle_E(oracle_lib, c, 1)
    assert rel(y, r32) < TOL
    assert rel(y, r64) < fp64_bound(r32, r64)


# line lengths with a prime factor >= 7 (direct prime DFTs): 112 = 16*7, 176 = 16*11, 208 = 16*13
# at the default overgrid; 272 = 16*17, 304 = 16*19, 336 = 48*7, 352 = 32*11, 368 = 16*23 via
# a large overgrid on a 32^3 image
@pytest.mark.parametrize("N,overgrid,C,nproj", [(70, 1.5, 2, 800), (112, 1.5, 1, 1200), (136, 1.5, 1, 1200),
                                                (32, 8.4, 2, 300), (32, 9.4, 1, 300), (32, 10.4, 1, 300),
                                                (32, 10.9, 1, 300), (32, 11.3, 2, 300)])
def test_prime_factor_lengths_match_oracle(mrg_lib, oracle_lib, N, overgrid, C, nproj):
    torch = _torch()
    c = case(N=N, C=C, nproj=nproj)
    p = _plan(mrg_lib, c, overgrid=overgrid)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    o32 = oracle_lib.Plan(N, overgrid=overgrid, prec=0)
    assert tuple(p.S) == tuple(o32.S)
    y = p.forward(0, torch.from_numpy(c["X"]).cuda()).cpu().numpy()
    ref = np.stack([o32.forward(c["X"], c["smaps"][k], *a) for k in range(C)])
    assert rel(y, ref) < TOL
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    refX = np.zeros(o32.ishape, o32.cdt)
    for k in range(C):
        refX = o32.adjoint(refX, c["smaps"][k], c["data"][k], *a)
    assert rel(X.cpu().numpy(), refX) < TOL


def test_forward_residual_matches_oracle(mrg_lib, oracle_lib):
    torch = _torch()
    c = case(N=32, C=4, nproj=700)
    p = _plan(mrg_lib, c)
    y = p.forward(0, torch.from_numpy(c["X"]).cuda(), diff=torch.from_numpy(c["data"]).cuda()).cpu().numpy()
    assert rel(y, _oracle_E(oracle_lib, c, 0, diff=c["data"])) < TOL


@pytest.mark.parametrize("N,C,nproj", [(32, 4, 700), (64, 8, 1500), (48, 3, 500), (32, 20, 400), (8, 2, 60),
                                       (16, 4, 200), (40, 3, 600), (80, 2, 1500), (168, 1, 1500)])
def test_adjoint_EH_matches_oracle(mrg_lib, oracle_lib, N, C, nproj):
    torch = _torch()
    c = case(N=N, C=C, nproj=nproj)
    p = _plan(mrg_lib, c)
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    got = X.cpu().numpy()
    r32, r64 = _oracle_EH(oracle_lib, c, 0), _oracle_EH(oracle_lib, c, 1)
    assert rel(got, r32) < TOL
    assert rel(got, r64) < fp64_bound(r32, r64)


def test_adjoint_accumulates_into_X(mrg_lib, oracle_lib):
    torch = _torch()
    c = case(N=32, C=2, nproj=300)
    p = _plan(mrg_lib, c)
    X0 = torch.from_numpy(c["X"]).cuda()
    X = X0.clone()
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    ref = c["X"].astype(np.complex128) + _oracle_EH(oracle_lib, c, 1)
    assert rel(X.cpu().numpy(), ref) < TOL


def test_normal_operator_matches_oracle(mrg_lib, oracle_lib):
    torch = _torch()
    c = case(N=32, C=4, nproj=700)
    p = _plan(mrg_lib, c)
    got = p.normal(0, torch.from_numpy(c["X"]).cuda()).cpu().numpy()
    O = oracle_lib.Plan(32, prec=1)
    fr = [dict(kx=c["kx"], ky=c["ky"], kz=c["kz"], kw=c["kw"], data=c["data"])]
    ref = O.normal(fr, c["smaps"], 0, c["X"])
    assert rel(got, ref) < TOL


def test_host_pointers_are_staged(mrg_lib, oracle_lib):
    """numpy (host) buffers go through the same path as device tensors."""
    c = case(N=32, C=2, nproj=300)
    p = _plan(mrg_lib, c)
    y = p.forward(0, c["X"])
    assert isinstance(y, np.ndarray)
    assert rel(y, _oracle_E(oracle_lib, c, 1)) < TOL
    X = np.zeros(c["X"].shape, np.complex64)
    p.adjoint(0, c["data"], X)
    assert rel(X, _oracle_EH(oracle_lib, c, 1)) < TOL


def test_edge_samples(mrg_lib, oracle_lib):
    """kw == 0, samples outside the grid, clipped taps at the grid edge, six-tap
    half-integer positions: E writes 0 where the reference does."""
    torch = _torch()
    N, C = 32, 2
    c = case(N=N, C=C, nproj=10)
    c["kx"], c["ky"], c["kz"], c["kw"] = edge_trajectory(N)
    M = c["kx"].size
    rng = np.random.default_rng(1)
    c["data"] = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    p = _plan(mrg_lib, c)
    y = p.forward(0, torch.from_numpy(c["X"]).cuda()).cpu().numpy()
    ref = _oracle_E(oracle_lib, c, 1)
    assert rel(y, ref) < TOL
    assert np.all(y[:, 5] == 0) and np.all(y[:, 20] == 0)     # kw == 0
    assert np.all(y[:, 5:8] == 0)                               # outside the grid
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    assert rel(X.cpu().numpy(), _oracle_EH(oracle_lib, c, 1)) < TOL


def test_per_coil_drop_in_matches_oracle(mrg_lib, oracle_lib):
    """The reference's per-coil gridFFT surface (plain path, one coil per call)."""
    torch = _torch()
    c = case(N=32, C=3, nproj=500)
    g = mrg_lib.gridFFT()
    g.precalc_gridding(32, 32, 32)
    assert (g.Sx, g.og_sx, g.og_ex) == (48, 8, 40)
    a = [torch.from_numpy(v).cuda() for v in (c["kx"], c["ky"], c["kz"], c["kw"])]
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    Xin = torch.from_numpy(c["X"]).cuda()
    ys = []
    for k in range(c["C"]):
        sm = torch.from_numpy(c["smaps"][k]).cuda()
        d = torch.empty(c["kx"].size, dtype=torch.complex64, device="cuda")
        g.backward(Xin, sm, d, *a)
        ys.append(d.cpu().numpy())
        g.forward(X, sm, torch.from_numpy(c["data"][k]).cuda(), *a)
    assert rel(np.stack(ys), _oracle_E(oracle_lib, c, 1)) < TOL
    assert rel(X.cpu().numpy(), _oracle_EH(oracle_lib, c, 1)) < TOL
    # residual form and the no-smap overloads
    d = torch.empty(c["kx"].size, dtype=torch.complex64, device="cuda")
    g.backward_residual(Xin, None, d, *a, torch.from_numpy(c["data"][0]).cuda())
    O = oracle_lib.Plan(32, prec=1)
    ref = O.forward(c["X"], None, c["kx"], c["ky"], c["kz"], c["kw"], diff=c["data"][0])
    assert rel(d.cpu().numpy(), ref) < TOL


def test_errors_do_not_exit(mrg_lib):
    import mri_recon_gb300 as m
    c = case(N=32, C=2, nproj=50)
    p = m.Plan(32, 2, 1)
    with pytest.raises(m.MrgError, match="STATE"):
        p.forward(0, c["X"])                       # no trajectory yet
    with pytest.raises(m.MrgError, match="UNSUPPORTED"):
        m.Plan(300, 1, 1)                           # S = 464 = 16*29: a prime factor above 23, not built
    with pytest.raises(m.MrgError, match="UNSUPPORTED"):
        m.Plan(520, 1, 1)                           # S = 784: lines above 768 points not built


@pytest.mark.parametrize("grid_mode", [1, 2, 3])
@pytest.mark.parametrize("N,C,nproj,max_pairs", [(32, 4, 700, 0), (48, 3, 500, 0), (32, 20, 400, 0),
                                                  (32, 32, 300, 0), (32, 1, 600, 0), (32, 8, 700, 96),
                                                  (48, 9, 500, 0), (32, 16, 900, 200)])
def test_adjoint_each_gridding_kernel(mrg_lib, oracle_lib, grid_mode, N, C, nproj, max_pairs):
    """Every gridding kernel (FP32 CUDA cores; TF32 tensor cores with the hi/lo split
    through mma.sync and through tcgen05 / tensor memory), odd and partial coil chunks,
    and dense blocks split into work items that flush with atomics (small max_pairs)."""
    if grid_mode == 3 and C < 8:
        pytest.skip("the tcgen05 kernel needs >= 8 coils")
    torch = _torch()
    c = case(N=N, C=C, nproj=nproj)
    p = mrg_lib.Plan(N, C, 1, grid_mode=grid_mode, max_pairs=max_pairs)
    p.set_traj(0, c["kx"], c["ky"], c["kz"], c["kw"])
    p.set_smaps(c["smaps"])
    tun = p.frame_tuning(0)
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    got = X.cpu().numpy()
    r32, r64 = _oracle_EH(oracle_lib, c, 0), _oracle_EH(oracle_lib, c, 1)
    assert rel(got, r32) < TOL, tun
    assert rel(got, r64) < fp64_bound(r32, r64), tun


def test_edge_samples_tensor_core_gridding(mrg_lib, oracle_lib):
    torch = _torch()
    N, C = 32, 4
    c = case(N=N, C=C, nproj=10)
    c["kx"], c["ky"], c["kz"], c["kw"] = edge_trajectory(N)
    M = c["kx"].size
    rng = np.random.default_rng(2)
    c["data"] = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    p = mrg_lib.Plan(N, C, 1, grid_mode=2)
    p.set_traj(0, c["kx"], c["ky"], c["kz"], c["kw"])
    p.set_smaps(c["smaps"])
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    assert rel(X.cpu().numpy(), _oracle_EH(oracle_lib, c, 1)) < TOL


@pytest.mark.parametrize("C,G,cpl,uy", [(32, 8, 4, 1), (32, 4, 4, 1), (20, 16, 4, 1), (32, 16, 2, 3),
                                        (12, 4, 1, 2), (32, 32, 1, 1), (6, 8, 4, 1),
                                        (32, -8, 1, 1), (32, -4, 1, 1), (64, -8, 1, 1), (16, -4, 1, 1),
                                        (8, -2, 1, 1), (20, -1, 1, 1)])
def test_forward_each_ungrid_shape(mrg_lib, oracle_lib, C, G, cpl, uy):
    """Every ungridding variant, fixed through mrg_frame_set_tuning: lanes per sample,
    1, 2 or 4 coils per lane (8-, 16- and 32-byte gathers) and tap rows per step; with
    6 coils the 4-per-lane request falls back to 2 per lane.  Negative lanes: the
    tensor-core kernel with 4 |G| coils per pass (one or more passes)."""
    torch = _torch()
    c = case(N=32, C=C, nproj=500)
    p = _plan(mrg_lib, c)
    t = p.frame_tuning(0)
    p.set_frame_tuning(0, G, 128 if G > 0 else 256, t["grid_coils_per_pass"], cpl, uy)
    assert p.frame_tuning(0)["ungrid_lanes"] == G
    y = p.forward(0, torch.from_numpy(c["X"]).cuda()).cpu().numpy()
    r32, r64 = _oracle_E(oracle_lib, c, 0), _oracle_E(oracle_lib, c, 1)
    assert rel(y, r32) < TOL
    assert rel(y, r64) < fp64_bound(r32, r64)


@pytest.mark.parametrize("spb", [16, 100, 1024])
def test_tensor_core_ungrid_residual_and_normal(mrg_lib, oracle_lib, spb):
    """The tensor-core ungridding kernel on the residual (E x - data) and inside the
    normal operator (samples weighted by kw and the taper), with sample ranges per CTA
    that end inside a 16-sample group."""
    torch = _torch()
    c = case(N=32, C=8, nproj=700)
    p = _plan(mrg_lib, c)
    t = p.frame_tuning(0)
    p.set_frame_tuning(0, -2, spb, t["grid_coils_per_pass"], 1, 1)
    y = p.forward(0, torch.from_numpy(c["X"]).cuda(), diff=torch.from_numpy(c["data"]).cuda()).cpu().numpy()
    assert rel(y, _oracle_E(oracle_lib, c, 0, diff=c["data"])) < TOL
    got = p.normal(0, torch.from_numpy(c["X"]).cuda()).cpu().numpy()
    O = oracle_lib.Plan(32, prec=1)
    fr = [dict(kx=c["kx"], ky=c["ky"], kz=c["kz"], kw=c["kw"], data=c["data"])]
    assert rel(got, O.normal(fr, c["smaps"], 0, c["X"])) < TOL


def test_set_frame_tuning_rejects_unavailable_shapes(mrg_lib):
    c = case(N=32, C=4, nproj=300)
    p = _plan(mrg_lib, c)
    t = p.frame_tuning(0)
    for bad in [(3, 128, 0, 1, 1), (8, 0, 0, 1, 1), (8, 128, 0, 3, 1), (8, 128, 0, 1, 4), (-2, 128, 0, 1, 1),
                (8, 128, -8, 1, 1), (8, 128, -116, 1, 1), (8, 128, 12, 1, 1)]:
        with pytest.raises(mrg_lib.MrgError):
            p.set_frame_tuning(0, *bad)
    assert p.frame_tuning(0) == t


# Every line length the default geometry reaches, against cuFFT (torch.fft on the device) in
# single and double precision: 16, 32, 48, 64, 112 (7), 176 (11), 192, 256, 304 (19), 368 (23), 384
@pytest.mark.parametrize("N", [8, 16, 32, 40, 70, 112, 128, 168, 200, 236, 256])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft3_against_cufft(mrg_lib, N, sign):
    torch = _torch()
    C = 2
    p = mrg_lib.Plan(N, C, 1)
    Sx, Sy, Sz = p.S
    g = torch.randn((Sz, Sy, Sx, C), dtype=torch.complex64, device="cuda", generator=torch.Generator("cuda").manual_seed(N))
    f = torch.fft.fftn if sign < 0 else torch.fft.ifftn  # FFTW_FORWARD e^{-i}, FFTW_BACKWARD e^{+i}
    ref64 = f(g.to(torch.complex128), dim=(0, 1, 2), norm="ortho")
    ref32 = f(g, dim=(0, 1, 2), norm="ortho")
    got = p.fft3(g.clone(), sign)
    e64 = float(torch.linalg.norm(got - ref64) / torch.linalg.norm(ref64))
    e32 = float(torch.linalg.norm(ref32 - ref64) / torch.linalg.norm(ref64))
    assert e64 < max(1e-6, 2 * e32), (e64, e32)


@pytest.mark.parametrize("sign", [-1, 1])
def test_fft3_unnormalised_plan(mrg_lib, sign):
    """mrg_fft3 on a plan with fft_norm = 1 (gridFFT_CoilThreaded's FFTW transforms) is
    sqrt(Sx Sy Sz) times the normalised transform of fft_norm = 0."""
    torch = _torch()
    N, C = (40, 32, 24), 2
    p0, p1 = mrg_lib.Plan(N, C, 1), mrg_lib.Plan(N, C, 1, fft_norm=1)
    Sx, Sy, Sz = p0.S
    g = torch.randn((Sz, Sy, Sx, C), dtype=torch.complex64, device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    want = p0.fft3(g.clone(), sign) * float(np.sqrt(float(Sx * Sy * Sz)))
    got = p1.fft3(g.clone(), sign)
    assert float(torch.linalg.norm(got - want) / torch.linalg.norm(want)) < 1e-6


@pytest.mark.parametrize("kernel,overgrid,dwin,N,C", [(1, 1.5, -1.0, 32, 4), (0, 1.0, 1.0, 32, 2), (1, 1.5, -1.0, 24, 8)])
def test_grid_and_ungrid_on_a_caller_grid(mrg_lib, oracle_lib, kernel, overgrid, dwin, N, C):
    """chop_grid_forward / chop_grid_backward on a caller grid (mrg_grid / mrg_ungrid), per
    coil against the oracle; the triangle kernel at overgrid 1.0 and half width 1 is the
    setting of RECON::kspace_residual (src/recon_lib.cpp:2218-2252)."""
    import torch
    c = case(N=N, C=C, nproj=500, seed=41)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    p = mrg_lib.Plan(N, C, 2, kernel_type=kernel, overgrid=overgrid, dwin=dwin)
    e = edge_trajectory(N)
    p.set_traj(0, *a)
    p.set_traj(1, *e)
    o = oracle_lib.Plan(N, kernel=kernel, overgrid=overgrid, dwin=dwin)
    G = p.grid(0, torch.from_numpy(c["data"]).cuda()).cpu().numpy()
    for k in range(C):
        assert rel(G[..., k], o.grid(c["data"][k], *a)) < 1e-5
    Gh = p.grid(0, c["data"])  # host buffers
    assert rel(Gh, G) < 1e-6
    rng = np.random.default_rng(42)
    grid = (rng.standard_normal(G.shape) + 1j * rng.standard_normal(G.shape)).astype(np.complex64)
    y = p.ungrid(0, torch.from_numpy(grid).cuda()).cpu().numpy()
    yd = p.ungrid(0, grid, diff=c["data"])
    for k in range(C):
        ref = o.ungrid(np.ascontiguousarray(grid[..., k]), *a)
        assert rel(y[k], ref) < 1e-5
        assert rel(yd[k], o.ungrid(np.ascontiguousarray(grid[..., k]), *a, diff=c["data"][k])) < 1e-5
    # edge samples: outside the grid, kw == 0, half-integer positions
    de = (rng.standard_normal((C, e[0].size)) + 1j * rng.standard_normal((C, e[0].size))).astype(np.complex64)
    Ge = p.grid(1, de)
    ye = p.ungrid(1, grid)
    for k in range(C):
        assert rel(Ge[..., k], o.grid(de[k], *e)) < 1e-5
        r = o.ungrid(np.ascontiguousarray(grid[..., k]), *e)
        assert rel(ye[k], r) < 1e-5
        assert np.array_equal(ye[k] == 0, r == 0)


@pytest.mark.parametrize("n", [257, 264, 320, 340, 384, 448, 512])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_long_lines_against_cufft(mrg_lib, n, axis):
    """Lines above 384 points (N > 256 at the default 1.5x: 16 threads per line) along each
    axis of the grid, forward and inverse, against cuFFT in double precision."""
    torch = _torch()
    N = [16, 24, 20]
    N[axis] = n
    C = 2
    p = mrg_lib.Plan(tuple(N), C, 1)
    assert p.S[axis] > 384
    Sx, Sy, Sz = p.S
    g = torch.randn((Sz, Sy, Sx, C), dtype=torch.complex64, device="cuda", generator=torch.Generator("cuda").manual_seed(n))
    for sign in (-1, 1):
        f = torch.fft.fftn if sign < 0 else torch.fft.ifftn
        ref64 = f(g.to(torch.complex128), dim=(0, 1, 2), norm="ortho")
        ref32 = f(g, dim=(0, 1, 2), norm="ortho")
        got = p.fft3(g.clone(), sign)
        e64 = float(torch.linalg.norm(got - ref64) / torch.linalg.norm(ref64))
        e32 = float(torch.linalg.norm(ref32 - ref64) / torch.linalg.norm(ref64))
        assert e64 < max(1e-6, 2 * e32), (n, axis, sign, e64, e32)


@pytest.mark.parametrize("N,C", [((320, 24, 16), 3), ((16, 272, 24), 2), ((20, 16, 384), 9), ((400, 32, 32), 1)])
def test_long_lines_operators_match_oracle(mrg_lib, oracle_lib, N, C):
    """E and E^H with a grid axis above 384 points against the oracle (one coil: the
    single-coil pass order; nine coils: the tensor-core gridding)."""
    import torch
    from mri_recon_gb300 import synth
    rng = np.random.default_rng(3)
    M = 30000
    kx, ky, kz = [rng.uniform(-n / 2, n / 2, M).astype(np.float32) for n in N]
    kw = (kx.astype(np.float64) ** 2 + ky ** 2 + kz ** 2).astype(np.float32)
    ishape = (N[2], N[1], N[0])
    X = (rng.standard_normal(ishape) + 1j * rng.standard_normal(ishape)).astype(np.complex64)
    smaps = (rng.standard_normal((C,) + ishape) + 1j * rng.standard_normal((C,) + ishape)).astype(np.complex64)
    d = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    p = mrg_lib.Plan(N, C, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_smaps(torch.from_numpy(smaps).cuda())
    o = oracle_lib.Plan(N)
    y = p.forward(0, torch.from_numpy(X).cuda()).cpu().numpy()
    Xh = p.adjoint(0, d, np.zeros(ishape, np.complex64))
    ref_h = np.zeros(ishape, np.complex64)
    for k in range(C):
        assert rel(y[k], o.forward(X, smaps[k], kx, ky, kz, kw)) < 1e-5
        ref_h = o.adjoint(ref_h, smaps[k], d[k], kx, ky, kz, kw)
    assert rel(Xh, ref_h) < 1e-5


@pytest.mark.parametrize("N,C", [((128, 16, 24), 32), ((128, 24, 16), 16), ((256, 16, 8), 32), ((160, 8, 16), 16),
                                 ((192, 8, 8), 16), ((208, 8, 8), 32), ((128, 16, 16), 8), ((240, 8, 8), 20),
                                 ((16, 256, 16), 16), ((8, 16, 208), 32)])
@pytest.mark.parametrize("ib", [0, 16])
def test_persistent_x_passes_match_oracle(mrg_lib, oracle_lib, N, C, ib):
    """The set_image and accumulate x passes run by the persistent kernels (xp = 1; x lines
    of 192..384 points, 16 or 32 coils per CTA; xp = 2: 16 threads per line for 288, 320
    and 384 points, also in the plain y and z passes: the last two shapes; xp | 4: the
    plain persistent passes' tiles copied by tensor maps) and by the one-tile kernels (xp =
    0) give the oracle's E and E^H; 8 and 20 coils check the fall-back to the one-tile
    kernels."""
    import torch
    rng = np.random.default_rng(5)
    M = 20000
    kx, ky, kz = [rng.uniform(-n / 2, n / 2, M).astype(np.float32) for n in N]
    kw = (kx.astype(np.float64) ** 2 + ky ** 2 + kz ** 2).astype(np.float32)
    ishape = (N[2], N[1], N[0])
    X = (rng.standard_normal(ishape) + 1j * rng.standard_normal(ishape)).astype(np.complex64)
    smaps = (rng.standard_normal((C,) + ishape) + 1j * rng.standard_normal((C,) + ishape)).astype(np.complex64)
    d = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    p = mrg_lib.Plan(N, C, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_smaps(torch.from_numpy(smaps).cuda())
    o = oracle_lib.Plan(N)
    ref_e = np.stack([o.forward(X, smaps[k], kx, ky, kz, kw) for k in range(C)])
    ref_h = np.zeros(ishape, np.complex64)
    for k in range(C):
        ref_h = o.adjoint(ref_h, smaps[k], d[k], kx, ky, kz, kw)
    X0 = (rng.standard_normal(ishape) + 1j * rng.standard_normal(ishape)).astype(np.complex64)
    out = {}
    for xp in (0, 1, 2, 4, 5, 6):
        p.set_fft_tuning(ib=[ib] * 6, xp=[xp] * 6)
        assert p.fft_tuning() == dict(ib=[ib] * 6, xp=[xp] * 6)
        y = p.forward(0, torch.from_numpy(X).cuda()).cpu().numpy()
        Xh = p.adjoint(0, d, X0.copy())  # accumulates into X
        assert rel(y, ref_e) < 1e-5
        assert rel(Xh - X0, ref_h) < 1e-5
        out[xp] = (y, Xh)
    for xp in (1, 2, 4, 5, 6):
        assert rel(out[xp][0], out[0][0]) < 1e-6
        assert rel(out[xp][1], out[0][1]) < 1e-6


def test_set_fft_tuning_rejects_bad_values(mrg_lib):
    p = mrg_lib.Plan(16, 2, 1)
    with pytest.raises(mrg_lib.MrgError):
        p.set_fft_tuning(ib=[33] * 6)
    with pytest.raises(mrg_lib.MrgError):
        p.set_fft_tuning(xp=[3] * 6)
    with pytest.raises(mrg_lib.MrgError):
        p.set_fft_tuning(xp=[7] * 6)


@pytest.mark.parametrize("N,C", [((20, 16, 384), 9), ((16, 24, 400), 16)])
def test_tensor_core_gridding_on_long_z_axes(mrg_lib, oracle_lib, N, C):
    """The tcgen05 gridding (grid_mode 3) on z axes of 576 and 608 points: region origins
    at z >= 512 set the top bit of the packed work-item field, which must unpack unsigned."""
    import torch
    rng = np.random.default_rng(11)
    M = 30000
    kx, ky, kz = [rng.uniform(-n / 2, n / 2, M).astype(np.float32) for n in N]
    kw = (kx.astype(np.float64) ** 2 + ky ** 2 + kz ** 2).astype(np.float32)
    ishape = (N[2], N[1], N[0])
    smaps = (rng.standard_normal((C,) + ishape) + 1j * rng.standard_normal((C,) + ishape)).astype(np.complex64)
    d = (rng.standard_normal((C, M)) + 1j * rng.standard_normal((C, M))).astype(np.complex64)
    p = mrg_lib.Plan(N, C, 1, grid_mode=3)
    p.set_traj(0, kx, ky, kz, kw)
    assert p.frame_tuning(0)["grid_coils_per_pass"] <= -100  # the tcgen05 kernel
    p.set_smaps(torch.from_numpy(smaps).cuda())
    Xh = p.adjoint(0, d, np.zeros(ishape, np.complex64))
    o = oracle_lib.Plan(N)
    ref = np.zeros(ishape, np.complex64)
    for k in range(C):
        ref = o.adjoint(ref, smaps[k], d[k], kx, ky, kz, kw)
    assert rel(Xh, ref) < 1e-5


def test_large_pinned_host_input_matches_device_input(mrg_lib):
    """Host inputs of 64 MB or more in pinned memory are read by the GPU through their
    device-side alias (an SM copy); the result is the one from the same data on the device."""
    import torch
    from mri_recon_gb300 import synth
    N, C = 32, 8
    kx, ky, kz, kw = synth.radial_trajectory(N, 4096, 260)  # 1.06 M samples: 68 MB of k-space
    g = torch.Generator().manual_seed(4)
    d = torch.complex(torch.randn((C, kx.size), generator=g), torch.randn((C, kx.size), generator=g))
    p = mrg_lib.Plan(N, C, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_smaps(torch.from_numpy(synth.coil_maps(N, C, seed=3)).cuda())
    X_dev = p.adjoint(0, d.cuda(), torch.zeros(p.ishape, dtype=torch.complex64, device="cuda")).cpu()
    pinned = d.pin_memory()
    assert pinned.numel() * 8 >= 64 << 20
    X_pin = p.adjoint(0, pinned, torch.zeros(p.ishape, dtype=torch.complex64, device="cuda")).cpu()
    # the dense centre's split regions add with atomics in no fixed order: equal to rounding
    assert rel(X_pin.numpy(), X_dev.numpy()) < 1e-6
    p.set_data(0, pinned)
    X_cg, _ = p.cg(2)
    p.set_data(0, d.cuda())
    X_cg2, _ = p.cg(2)
    assert rel(X_cg.cpu().numpy(), X_cg2.cpu().numpy()) < 1e-6
