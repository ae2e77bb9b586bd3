"""SENSE-CG on the GPU against the oracle's FP32 and FP64 CG
(relative L2 <= 1e-4 after the stated iterations)."""
import numpy as np
import pytest

from tests.helpers import case, rel

pytestmark = pytest.mark.gpu
TOL_ITER = 1e-4


def _cg_case(N, C, nproj, nread, seed):
    c = case(N=N, C=C, nproj=nproj, nread=nread, seed=seed)
    # data from the FP64 oracle E on the phantom plus 1% noise (the CG input)
    return c


def _run(mrg_lib, oracle_lib, N, C, nproj, nread, iters, seed=5, use_graph=True, nudft=False):
    import torch
    from mri_recon_gb300 import synth
    c = case(N=N, C=C, nproj=nproj, nread=nread, seed=seed, nudft=nudft, ellipsoids=10 if nudft else 6)
    O64 = oracle_lib.Plan(N, prec=1)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    if nudft:  # FP64 direct NUDFT of the phantom times each map, 1% noise (helpers.case)
        y = c["data"]
    else:
        y = np.stack([O64.forward(c["img"], c["smaps"][k], *a) for k in range(C)]).astype(np.complex64)
        y = synth.add_noise(y, 0.01, seed)
    p = mrg_lib.Plan(N, C, 1)
    p.set_traj(0, *a)
    p.set_smaps(torch.from_numpy(c["smaps"]).cuda())
    p.set_data(0, torch.from_numpy(y).cuda())
    X, resid = p.cg(iters, use_graph=use_graph)
    fr = [dict(kx=c["kx"], ky=c["ky"], kz=c["kz"], kw=c["kw"], data=y)]
    X32, r32 = oracle_lib.Plan(N, prec=0).cg(fr, c["smaps"], iters)
    X64, r64 = O64.cg(fr, c["smaps"], iters)
    return X[0].cpu().numpy(), resid, X32[0], r32, X64[0], r64


@pytest.mark.parametrize("use_graph", [True, False])
def test_cg_small_matches_oracle(mrg_lib, oracle_lib, use_graph):
    X, r, X32, r32, X64, r64 = _run(mrg_lib, oracle_lib, 32, 4, 800, 32, 8, use_graph=use_graph)
    assert rel(X, X64) < TOL_ITER
    assert rel(X, X32) < TOL_ITER
    assert np.max(np.abs(r - r64) / r64) < 1e-3


def test_cg_64cube_8coils_20iters(mrg_lib, oracle_lib):
    """The SENSE-CG configuration at its stated size and iteration count: 64^3 x 8 coils,
    4096 x 64 radial, 20 iterations, k-space from an FP64 direct NUDFT of a 10-ellipsoid
    phantom times Gaussian coil maps plus 1% noise."""
    X, r, X32, r32, X64, r64 = _run(mrg_lib, oracle_lib, 64, 8, 4096, 64, 20, nudft=True)
    e64, e32 = rel(X, X64), rel(X, X32)
    print("cg64 rel-L2 vs FP64 oracle %.3g, vs FP32 oracle %.3g, FP32 oracle vs FP64 %.3g" % (e64, e32, rel(X32, X64)))
    assert e64 < TOL_ITER
    assert e32 < TOL_ITER
