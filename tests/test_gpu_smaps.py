"""GPU parity of the coil-map path against the oracle: map-free per-coil adjoints,
the sum-of-squares adjoint, the k_rad taper, the Gaussian blur, SOS normalisation
and the whole low-resolution map estimate (relative L2 <= 1e-5 per operator)."""
import numpy as np
import pytest

from tests.helpers import case, rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _torch():
    import torch
    return torch


def _args(c):
    return (c["kx"], c["ky"], c["kz"], c["kw"])


@pytest.mark.parametrize("N,C", [(32, 4), (48, 3)])
def test_adjoint_coils_matches_oracle(mrg_lib, oracle_lib, N, C):
    torch = _torch()
    c = case(N=N, C=C, nproj=600)
    p = mrg_lib.Plan(N, C)
    p.set_traj(0, *_args(c))
    imgs = p.adjoint_coils(0, torch.from_numpy(c["data"]).cuda()).cpu().numpy()
    o = oracle_lib.Plan(N)
    for k in range(C):
        ref = o.adjoint(np.zeros(o.ishape, np.complex64), None, c["data"][k], *_args(c))
        assert rel(imgs[k], ref) < TOL


def test_adjoint_coils_host_buffers_accumulate(mrg_lib, oracle_lib):
    c = case(N=32, C=2, nproj=400)
    p = mrg_lib.Plan(32, 2)
    p.set_traj(0, *_args(c))
    start = np.stack([c["X"], 2 * c["X"]])
    got = p.adjoint_coils(0, c["data"], start.copy())
    o = oracle_lib.Plan(32)
    for k in range(2):
        ref = o.adjoint(start[k].copy(), None, c["data"][k], *_args(c))
        assert rel(got[k], ref) < TOL


def test_adjoint_sos_matches_oracle(mrg_lib, oracle_lib):
    torch = _torch()
    c = case(N=32, C=4, nproj=600)
    p = mrg_lib.Plan(32, 4)
    p.set_traj(0, *_args(c))
    X = p.adjoint_sos(0, torch.from_numpy(c["data"]).cuda()).cpu().numpy()
    o = oracle_lib.Plan(32)
    ref = np.zeros(o.ishape, np.complex64)
    for k in range(4):
        ref = o.adjoint_sos(ref, c["data"][k], *_args(c))
    assert rel(X, ref) < TOL
    assert np.all(X.imag == 0)


def test_k_rad_taper_matches_oracle(mrg_lib, oracle_lib):
    torch = _torch()
    c = case(N=32, C=4, nproj=600)
    p = mrg_lib.Plan(32, 4)
    p.set_traj(0, *_args(c))
    p.set_smaps(c["smaps"])
    p.set_k_rad(6.0)
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    o = oracle_lib.Plan(32, k_rad=6.0)
    ref = np.zeros(o.ishape, np.complex64)
    for k in range(4):
        ref = o.adjoint(ref, c["smaps"][k], c["data"][k], *_args(c))
    assert rel(X.cpu().numpy(), ref) < TOL
    # back to the default radius: same as a fresh plan
    p.set_k_rad(9999.0)
    X2 = torch.zeros_like(X)
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X2)
    o2 = oracle_lib.Plan(32)
    ref2 = np.zeros(o2.ishape, np.complex64)
    for k in range(4):
        ref2 = o2.adjoint(ref2, c["smaps"][k], c["data"][k], *_args(c))
    assert rel(X2.cpu().numpy(), ref2) < TOL


@pytest.mark.parametrize("sigma", [(1.0, 0.0, 0.0), (0.0, 2.0, 0.0), (0.0, 0.0, 1.5), (1.2, 0.7, 2.0)])
def test_gaussian_blur_matches_oracle(mrg_lib, oracle_lib, sigma):
    rng = np.random.default_rng(5)
    X = (rng.standard_normal((3, 20, 24, 28)) + 1j * rng.standard_normal((3, 20, 24, 28))).astype(np.complex64)
    got = mrg_lib.gaussian_blur(X.copy(), sigma)
    for v in range(3):
        ref = oracle_lib.gaussian_blur(X[v], sigma)
        assert rel(got[v], ref) < 1e-6


def test_sos_normalize_matches_oracle_bitwise(mrg_lib, oracle_lib):
    rng = np.random.default_rng(6)
    A = (rng.standard_normal((5, 16, 16, 16)) + 1j * rng.standard_normal((5, 16, 16, 16))).astype(np.complex64)
    got = mrg_lib.sos_normalize(A.copy())
    ref = oracle_lib.sos_normalize(A)
    assert np.array_equal(got.view(np.float32), ref.view(np.float32))


@pytest.mark.parametrize("blur", [(0.0, 0.0, 0.0), (1.0, 1.0, 0.5)])
def test_lowres_smaps_matches_oracle(mrg_lib, oracle_lib, blur):
    torch = _torch()
    c = case(N=32, C=4, nproj=800, nudft=True)
    p = mrg_lib.Plan(32, 4)
    p.set_traj(0, *_args(c))
    maps = p.lowres_smaps(0, torch.from_numpy(c["data"]).cuda(), smap_res=8.0, blur=blur).cpu().numpy()
    ref = oracle_lib.lowres_smaps(oracle_lib.Plan(32), c["data"], *_args(c), smap_res=8.0, blur=blur)
    # dividing by the root sum of squares turns an image error e into e / |sos| on the maps,
    # large where there is almost no signal; weighted by the local signal level |sos| (how
    # SENSE uses the maps) the error is that of the coil images again
    o = oracle_lib.Plan(32, k_rad=8.0)
    imgs = [o.adjoint(np.zeros(o.ishape, np.complex64), None, c["data"][k], *_args(c)) for k in range(4)]
    if any(b > 0 for b in blur):
        imgs = [oracle_lib.gaussian_blur(im, blur) for im in imgs]
    sos = np.sqrt(np.sum(np.abs(np.stack(imgs).astype(np.complex128)) ** 2, 0))
    assert rel(maps * sos, ref * sos) < TOL
    assert rel(maps, ref) < 1e-4
    sos = np.sqrt(np.sum(np.abs(maps.astype(np.complex128)) ** 2, 0))
    assert np.allclose(sos, 1.0, atol=1e-5)
    # the maps are now the plan's maps, and the plan's k_rad is back at 9999
    assert p.k_rad == 9999.0
    X = torch.zeros(c["X"].shape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, torch.from_numpy(c["data"]).cuda(), X)
    o = oracle_lib.Plan(32)
    r = np.zeros(o.ishape, np.complex64)
    for k in range(4):
        r = o.adjoint(r, ref[k], c["data"][k], *_args(c))
    assert rel(X.cpu().numpy(), r) < 1e-4
