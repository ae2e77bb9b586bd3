"""GPU parity of the ESPIRiT coil maps (src/spirit.cpp:137-550) against the oracle, through
the C ABI: standalone from coil images, and on a plan from k-space (the ESPIRIT branch of
calc_sensitivity_maps, src/recon_lib.cpp:2892-2899)."""
import numpy as np
import pytest

from tests.helpers import rel

pytestmark = pytest.mark.gpu


def _images(N, C, seed=3):
    from mri_recon_gb300 import synth
    Nx, Ny, Nz = N
    n = max(N)
    cut = tuple(slice(n // 2 - m // 2, n // 2 - m // 2 + m) for m in (Nz, Ny, Nx))  # central block
    img = synth.phantom(n, 6, seed=seed)[cut]
    sm = synth.coil_maps(n, C, seed=seed + 1)[(slice(None),) + cut]
    return (img[None] * sm).astype(np.complex64)  # (C, Nz, Ny, Nx)


def _compare(maps, ref, ratio, tol):
    """maps (Nz, Ny, Nx, C) against the oracle's (C, Nz, Ny, Nx) where the dominant vector is
    well defined (eigenvalue ratio below 0.9)."""
    mask = ratio < 0.9
    assert mask.mean() > 0.5
    got = np.moveaxis(np.asarray(maps), -1, 0)[:, mask]
    err = rel(got, ref[:, mask])
    print("espirit maps rel-L2 %.3g over %.1f%% of the voxels" % (err, 100 * mask.mean()))
    assert err < tol
    # phase_correct: unit sum of squares, coil 0 real and non-negative
    assert np.abs((np.abs(got) ** 2).sum(0) - 1).max() < 1e-4
    assert np.abs(got[0].imag).max() < 1e-4 and got[0].real.min() >= -1e-6


# (N, C, kernel radius, calibration radius, square):
#   A taller than wide (Jacobi on A's columns), and wider (Jacobi on A^H's), a square region,
#   an anisotropic grid and kernel, 2D (Nz = 1)
@pytest.mark.parametrize("N,C,kr,cr,square", [((32, 32, 32), 4, (2.0, 2.0, 2.0), (8, 8, 8), 0),
                                              ((32, 32, 32), 16, (2.0, 2.0, 2.0), (6, 6, 6), 0),
                                              ((32, 32, 32), 12, (3.0, 3.0, 3.0), (5, 5, 5), 0),
                                              ((24, 24, 24), 6, (2.0, 2.0, 2.0), (5, 5, 5), 1),
                                              ((32, 28, 24), 5, (2.5, 2.0, 1.5), (8, 7, 6), 0),
                                              ((48, 40, 1), 6, (3.0, 3.0, 0.0), (12, 10, 0), 0)])
@pytest.mark.parametrize("device", [True, False])
def test_espirit_matches_oracle(mrg_lib, oracle_lib, N, C, kr, cr, square, device):
    import torch
    imgs = _images(N, C)
    ref, nV, sv, ratio = oracle_lib.espirit(imgs, kr_f=kr, cr=cr, square=bool(square))
    x = np.ascontiguousarray(np.moveaxis(imgs, 0, -1))  # (Nz, Ny, Nx, C)
    if device:
        x = torch.from_numpy(x).cuda()
    p = mrg_lib.espirit_params(kernel_radius=kr, calib_radius=cr, square=square)
    maps, kept, svg = mrg_lib.espirit(x, p, sv_cap=len(sv))
    maps = maps.cpu().numpy() if device else maps
    assert kept == nV
    assert np.abs(svg[:nV] - sv[:nV]).max() < 1e-5 * sv[0]
    _compare(maps, ref, ratio, 1e-4)


def test_espirit_smaps_on_plan_then_cg(mrg_lib, oracle_lib):
    import torch
    from mri_recon_gb300 import synth
    N, C = 32, 6
    kx, ky, kz, kw = synth.radial_trajectory(N, 1200, N)
    img = synth.phantom(N, 6, seed=5)
    sm = synth.coil_maps(N, C, seed=6)
    O64 = oracle_lib.Plan(N, prec=1)
    a = (kx, ky, kz, kw)
    data = np.stack([O64.forward(img, sm[c], *a) for c in range(C)]).astype(np.complex64)
    # the oracle's coil images (gridding.forward per coil, no maps), then its ESPIRiT
    imgs = np.stack([O64.adjoint(np.zeros(O64.ishape), None, data[c], *a) for c in range(C)]).astype(np.complex64)
    ref, nV, sv, ratio = oracle_lib.espirit(imgs, kr_f=(3.0,) * 3, cr=(10,) * 3)
    p = mrg_lib.Plan(N, C, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_data(0, torch.from_numpy(data).cuda())
    maps, kept = p.espirit_smaps(0, torch.from_numpy(data).cuda(), mrg_lib.espirit_params(3.0, 10))
    assert kept == nV
    _compare(np.moveaxis(maps.cpu().numpy(), 0, -1), ref, ratio, 1e-3)
    X, resid = p.cg(5)  # the plan's maps are now the ESPIRiT maps
    assert resid[-1] < resid[0]


def test_espirit_one_coil_and_bad_arguments(mrg_lib):
    from mri_recon_gb300 import synth
    kx, ky, kz, kw = synth.radial_trajectory(16, 100, 16)
    p = mrg_lib.Plan(16, 1, 1)
    p.set_traj(0, kx, ky, kz, kw)
    maps, kept = p.espirit_smaps(0, np.ones((1, kx.size), np.complex64))
    assert np.all(maps == 1)  # one coil: the map is 1
    imgs = np.ones((16, 16, 16, 4), np.complex64)
    for kw_ in (dict(kernel_radius=8.0), dict(kernel_radius=3.0, calib_radius=3), dict(calib_radius=9)):
        with pytest.raises(mrg_lib.MrgError):
            mrg_lib.espirit(imgs, mrg_lib.espirit_params(**kw_))
    with pytest.raises(mrg_lib.MrgError):
        mrg_lib.espirit(np.ones((16, 16, 16, 33), np.complex64))
    with pytest.raises(mrg_lib.MrgError):  # all-zero calibration data: no kernel to keep
        mrg_lib.espirit(np.zeros((32, 32, 32, 4), np.complex64))
