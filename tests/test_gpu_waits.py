"""Bounded device-side waits reach the caller.

The tensor-core gridding kernel synchronises its warps through shared-memory barriers,
and every wait on them gives up after the plan's limit.  With the limit at 0 a wait
gives up after its first unsuccessful try: the kernel records the failure and returns,
the call reports MRG_ERR_TIMEOUT, and the next call with the default limit is correct
again.  Nothing here faults or hangs the GPU: every wait ends, the kernel frees what it
holds and the context stays usable.
"""
import numpy as np
import pytest

from tests.helpers import case, rel

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_returns_timeout(mrg_lib, oracle_lib):
    import torch
    from mri_recon_gb300 import _lib
    c = case(N=32, C=8, nproj=1200, seed=17)
    p = mrg_lib.Plan(32, 8, 1, grid_mode=3)  # the tcgen05 gridding kernel, the one with barrier waits
    p.set_traj(0, c["kx"], c["ky"], c["kz"], c["kw"])
    p.set_smaps(torch.from_numpy(c["smaps"]).cuda())
    assert p.frame_tuning(0)["grid_coils_per_pass"] <= -100
    ref = p.adjoint(0, c["data"], np.zeros(p.ishape, np.complex64))  # host buffers: the call waits and checks

    p.set_wait_limit(0.0)
    with pytest.raises(_lib.MrgError) as e:
        p.adjoint(0, c["data"], np.zeros(p.ishape, np.complex64))
    assert "MRG_ERR_TIMEOUT" in str(e.value)
    p.check()  # the record was cleared when it was reported

    # device buffers: the call returns without waiting; the plan check reports it
    d = torch.from_numpy(c["data"]).cuda()
    Xd = torch.zeros(p.ishape, dtype=torch.complex64, device="cuda")
    p.adjoint(0, d, Xd)
    with pytest.raises(_lib.MrgError) as e:
        p.check()
    assert "MRG_ERR_TIMEOUT" in str(e.value)

    p.set_wait_limit(2.0)
    again = p.adjoint(0, c["data"], np.zeros(p.ishape, np.complex64))
    assert rel(again, ref) < 1e-6
    Xd.zero_()
    p.adjoint(0, d, Xd)
    p.check()
    assert rel(Xd.cpu().numpy(), ref) < 1e-6
    # and the operator is still the reference's
    o = oracle_lib.Plan(32, prec=1)
    want = np.zeros(o.ishape, np.complex128)
    for k in range(8):
        want = o.adjoint(want, c["smaps"][k], c["data"][k], c["kx"], c["ky"], c["kz"], c["kw"])
    assert rel(again, want) < 1e-5


def test_wait_limit_arguments(mrg_lib):
    from mri_recon_gb300 import _lib
    p = mrg_lib.Plan(16, 1, 1)
    with pytest.raises(_lib.MrgError):
        p.set_wait_limit(-1.0)
    with pytest.raises(_lib.MrgError):
        p.set_wait_limit(float("nan"))
    p.set_wait_limit(0.5)
    p.check()
