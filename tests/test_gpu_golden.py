"""The CUDA path against outputs of the reference's own code.

tests/golden/ref_ops.npz holds seeded inputs and the outputs of the reference's gridFFT
(E, the residual E, E^H per coil), WAVELET3D and THRESHOLD, computed by the reference
sources compiled unmodified (oracle/_ref; tests/golden/make_ref_golden.py).  The GPU runs
the same inputs through the C ABI.  Bound: relative L2 <= 1e-5 per operator application
(FP32 on both sides; summation orders differ), 1e-6 for the wavelet and threshold.
"""
import ctypes
import os

import numpy as np
import pytest

from tests.helpers import rel

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ops.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def test_oracle_reproduces_the_reference_fixture(oracle_lib, gold):
    """CPU: the oracle restatement gives the fixture's reference outputs (so the fixture,
    the oracle and the reference agree wherever the reference sources are absent)."""
    g = gold
    o = oracle_lib.Plan(24)
    a = (g["kx"], g["ky"], g["kz"], g["kw"])
    for k in range(2):
        assert rel(o.forward(g["img"], g["smaps"][k], *a), g["E"][k]) < 1e-6
        assert rel(o.adjoint(np.zeros(o.ishape, np.complex64), g["smaps"][k], g["data"][k], *a), g["EH"][k]) < 1e-6
    assert rel(oracle_lib.wavelet(g["wave_in"], (3, 3, 3), (1, 2, 3), 1), g["wave_db4"]) < 1e-6
    t = oracle_lib.fraction_threshold([g["thr_in"][0], g["thr_in"][1]], 0.1)
    assert abs(t - float(g["thr_value"])) <= 1e-6 * float(g["thr_value"])


@pytest.mark.gpu
def test_operators_match_reference_outputs(mrg_lib, gold):
    import torch
    g = gold
    a = (g["kx"], g["ky"], g["kz"], g["kw"])
    p = mrg_lib.Plan(24, 2, 1)
    p.set_traj(0, *a)
    p.set_smaps(torch.from_numpy(g["smaps"]).cuda())
    y = p.forward(0, torch.from_numpy(g["img"]).cuda()).cpu().numpy()
    assert rel(y, g["E"]) < 1e-5
    yr = p.forward(0, torch.from_numpy(g["img"]).cuda(), diff=torch.from_numpy(g["data"]).cuda()).cpu().numpy()
    assert rel(yr, g["E_resid"]) < 1e-5
    X = p.adjoint(0, g["data"], np.zeros(p.ishape, np.complex64))
    assert rel(X, g["EH"].sum(0)) < 1e-5
    # the per-coil surface (a single-coil plan, explicit maps) and the edge samples
    q = mrg_lib.Plan(24, 1, 2)
    q.set_traj(0, *a)
    q.set_traj(1, g["ekx"], g["eky"], g["ekz"], g["ekw"])
    for k in range(2):
        out = np.zeros(g["kx"].size, np.complex64)
        q.forward_coil(0, g["img"], g["smaps"][k], out)
        assert rel(out, g["E"][k]) < 1e-5
        Xk = q.adjoint_coil(0, g["smaps"][k], g["data"][k], np.zeros(q.ishape, np.complex64))
        assert rel(Xk, g["EH"][k]) < 1e-5
    oe = np.zeros(g["ekx"].size, np.complex64)
    q.forward_coil(1, g["img"], g["smaps"][0], oe)
    assert rel(oe, g["edge_E"]) < 1e-5
    assert np.array_equal(oe == 0, g["edge_E"] == 0)
    Xe = q.adjoint_coil(1, g["smaps"][0], g["edata"], np.zeros(q.ishape, np.complex64))
    assert rel(Xe, g["edge_EH"]) < 1e-5


@pytest.mark.gpu
def test_wavelet_and_threshold_match_reference_outputs(mrg_lib, gold):
    g = gold
    L = mrg_lib.load()
    ip = lambda v: (ctypes.c_int * 3)(*v)  # noqa: E731
    for wtype, shift, key in [(1, (1, 2, 3), "wave_db4"), (0, (1, 0, 1), "wave_db2")]:
        Y = g["wave_in"].copy()
        assert L.mrg_wavelet(ctypes.c_void_p(Y.ctypes.data), 1, 32, 24, 16, ip((3, 3, 3)), ip(shift), wtype, 0,
                             None) == 0
        assert rel(Y, g[key]) < 1e-6
    V = np.ascontiguousarray(g["thr_in"])
    v = ctypes.c_float()
    assert L.mrg_fraction_threshold(ctypes.c_void_p(V.ctypes.data), 2, V[0].size, 0.1, ctypes.byref(v), None) == 0
    assert abs(v.value - float(g["thr_value"])) <= 1e-6 * float(g["thr_value"])
    W = V.copy()
    assert L.mrg_soft_threshold(ctypes.c_void_p(W.ctypes.data), W.size, ctypes.c_float(float(g["thr_value"])),
                                None) == 0
    assert rel(W, g["thr_out"]) < 1e-6
