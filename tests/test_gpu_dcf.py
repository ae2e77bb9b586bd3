"""GPU parity of the Pipe density compensation (RECON::dcf_calc with the DCFgridFFT
gridder) against the oracle: relative L2 <= 1e-5 on the weights after the stated
iterations (the gridding adds with atomics in both, so the order of the sums differs)."""
import numpy as np
import pytest

from mri_recon_gb300 import synth
from tests.helpers import rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.mark.parametrize("N,nproj,params", [
    (24, 500, dict(iters=20)),
    (32, 800, dict(iters=10, kernel=1)),
    (24, 400, dict(iters=8, acc=1.5, scale=0.8, dwin=1.8, overgrid=2.0)),
])
def test_dcf_matches_oracle(mrg_lib, oracle_lib, N, nproj, params):
    import torch
    kx, ky, kz, _ = synth.radial_trajectory(N, nproj, N, seed=3)
    got = mrg_lib.dcf_pipe(*[torch.from_numpy(v).cuda() for v in (kx, ky, kz)], N, **params).cpu().numpy()
    ref32 = oracle_lib.dcf_pipe(kx, ky, kz, N, prec=0, **params)
    ref64 = oracle_lib.dcf_pipe(kx, ky, kz, N, prec=1, **params)
    assert rel(got, ref32) < TOL
    assert rel(got, ref64) < max(TOL, 1.25 * rel(ref32, ref64))


def test_dcf_anisotropic_matrix(mrg_lib, oracle_lib):
    """An anisotropic matrix: the grid's x extent comes from Nz and its z extent from Nx, as
    recon_lib allocates the DCF image (src/recon_lib.cpp:873-875, read by DCFgridFFT as x
    first); many samples then fall outside the grid and get weight 0."""
    import torch
    N = (40, 32, 24)
    kx, ky, kz, _ = synth.radial_trajectory(40, 600, 40, seed=6)
    kx, ky, kz = kx, (ky * 0.8).astype(np.float32), (kz * 0.6).astype(np.float32)
    got = mrg_lib.dcf_pipe(*[torch.from_numpy(v).cuda() for v in (kx, ky, kz)], N, iters=10).cpu().numpy()
    ref = oracle_lib.dcf_pipe(kx, ky, kz, N, iters=10)
    assert rel(got, ref) < TOL
    assert np.array_equal(got == 0, ref == 0) and (ref == 0).sum() > 0


def test_dcf_host_arrays_and_edges(mrg_lib, oracle_lib):
    """numpy input, samples outside the grid (their weight goes to 0), default parameters."""
    N = 24
    kx, ky, kz, _ = synth.radial_trajectory(N, 300, N, seed=4)
    kx = kx.copy()
    kx[:5] = 3 * N  # far outside the (int)(2.1 N + 16) grid
    got = mrg_lib.dcf_pipe(kx, ky, kz, N, iters=6)
    assert isinstance(got, np.ndarray)
    ref = oracle_lib.dcf_pipe(kx, ky, kz, N, iters=6)
    assert rel(got, ref) < TOL
    assert np.all(got[:5] == 0)
