"""The CUDA path against outputs of the reference's own code.

tests/golden/ref_ops.npz holds seeded inputs and the outputs of the reference's gridFFT
(E, the residual E, E^H per coil), WAVELET3D and THRESHOLD, tests/golden/ref_lowrank.npz
those of LOWRANKCOIL in time and in the coil dimension, tests/golden/ref_coils.npz those
of gridFFT_CoilThreaded (its default overgrid 1.375, unnormalised FFTs), and
tests/golden/ref_dcf.npz the Pipe density compensation around DCFgridFFT, and
tests/golden/ref_espirit.npz SPIRIT's ESPIRiT maps, computed by the reference sources
compiled unmodified (oracle/_ref; tests/golden/make_ref_golden.py).  The GPU runs the same
inputs through the C ABI.  Bound: relative L2 <= 1e-5 per operator application (FP32 on
both sides; summation orders differ), 1e-6 for the wavelet and threshold, 1e-5 for the
low-rank blocks (the GPU's Jacobi SVDs run in FP32 up to 16 coils).
"""
import ctypes
import os

import numpy as np
import pytest

from tests.helpers import align_block_phases, rel

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_ops.npz")
LOWRANK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_lowrank.npz")
COILS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_coils.npz")
DCF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_dcf.npz")
ESPIRIT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_espirit.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.fixture(scope="module")
def lowrank():
    return dict(np.load(LOWRANK))


@pytest.fixture(scope="module")
def coils():
    return dict(np.load(COILS))


@pytest.fixture(scope="module")
def dcf():
    return dict(np.load(DCF))


@pytest.fixture(scope="module")
def espirit():
    return dict(np.load(ESPIRIT))


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


def test_oracle_reproduces_the_low_rank_fixture(oracle_lib, lowrank):
    """CPU: the oracle gives the low-rank fixture's reference outputs (6 frames of 12^3 in
    4^3 blocks; 2 frames x 6 coils of 8^3)."""
    g = lowrank
    X = g["llr_in"]
    vols = [X[t] for t in range(X.shape[0])]
    smax = float(g["llr_smax"])
    assert abs(oracle_lib.llr_update_threshold(vols, (4, 4, 4), 4.0, 6.0, 2) - smax) <= 1e-6 * smax
    assert rel(np.stack(oracle_lib.llr_thresh(vols, (4, 4, 4), 4, 0.1, smax, 11)), g["llr_out"]) < 1e-6
    assert rel(np.stack(oracle_lib.llr_thresh(vols, (4, 4, 4), 1, 0.1, smax, 0)), g["llr_out_iter1"]) < 1e-6
    XX, sc = g["coil_in"], float(g["coil_smax"])
    assert abs(oracle_lib.clear_update_threshold(XX, (4, 4, 4), 4.0, 6.0, 1) - sc) <= 1e-6 * sc
    assert rel(oracle_lib.clear_thresh(XX, (4, 4, 4), 4, 0.05, sc, 5), g["coil_out"]) < 1e-6
    im = oracle_lib.clear_combine(XX, (4, 4, 4))
    assert rel(im, align_block_phases(im, g["coil_combine"], (4, 4, 4))) < 1e-6


@pytest.mark.gpu
def test_low_rank_blocks_match_reference_outputs(mrg_lib, lowrank):
    """mrg_llr_update_threshold / mrg_llr_thresh (time) and mrg_clear_update_threshold /
    mrg_clear_thresh / mrg_clear_combine (coils) on the fixture's inputs against the
    reference's outputs; combine after turning each reference block to the library's phase
    of v1 (its largest-magnitude component real and positive)."""
    g = lowrank
    L = mrg_lib.load()
    ip = lambda v: (ctypes.c_int * 3)(*v)  # noqa: E731
    X = np.ascontiguousarray(g["llr_in"])
    T, Nz, Ny, Nx = X.shape
    sm = ctypes.c_float()
    assert L.mrg_llr_update_threshold(ctypes.c_void_p(X.ctypes.data), T, Nx, Ny, Nz, ip((4, 4, 4)), 4.0, 6.0, 2,
                                      ctypes.byref(sm), None) == 0
    smax = float(g["llr_smax"])
    assert abs(sm.value - smax) <= 1e-5 * smax
    for block_iter, skip, key in [(4, 11, "llr_out"), (1, 0, "llr_out_iter1")]:
        Y = X.copy()
        assert L.mrg_llr_thresh(ctypes.c_void_p(Y.ctypes.data), T, Nx, Ny, Nz, ip((4, 4, 4)), block_iter, 0.1, smax,
                                skip, None) == 0
        assert rel(Y, g[key]) < 1e-5
    XX = np.ascontiguousarray(g["coil_in"].transpose(0, 2, 3, 4, 1))  # the library's (T, Nz, Ny, Nx, C)
    sc = float(g["coil_smax"])
    assert abs(mrg_lib.clear_update_threshold(XX, (4, 4, 4), 4.0, 6.0, 1) - sc) <= 1e-5 * sc
    Y = mrg_lib.clear_thresh(XX.copy(), sc, (4, 4, 4), 4, 0.05, 5)
    assert rel(Y, g["coil_out"].transpose(0, 2, 3, 4, 1)) < 1e-5
    im = mrg_lib.clear_combine(XX, (4, 4, 4))
    assert rel(im, align_block_phases(im, g["coil_combine"], (4, 4, 4))) < 1e-5


def test_oracle_reproduces_the_coil_threaded_fixture(oracle_lib, coils):
    """CPU: gridFFT_CoilThreaded's outputs (overgrid 1.375, 3 coils of 20 x 24 x 16) are the
    oracle's gridFFT operators times sqrt(Sx Sy Sz), its transforms being unnormalised."""
    g = coils
    a = (g["kx"], g["ky"], g["kz"], g["kw"])
    o = oracle_lib.Plan((20, 24, 16), overgrid=1.375)
    f = np.sqrt(float(np.prod(o.gshape)))
    E = np.stack([o.forward(g["img"], g["smaps"][k], *a) for k in range(3)])
    assert rel(f * E, g["E"]) < 1e-6
    EH = sum(o.adjoint(np.zeros(o.ishape, np.complex64), g["smaps"][k], g["data"][k], *a) for k in range(3))
    assert rel(f * EH, g["EH"]) < 1e-6


@pytest.mark.gpu
def test_coil_threaded_plan_matches_reference_outputs(mrg_lib, coils):
    """A plan with fft_norm = 1 at overgrid 1.375 (the gridFFT_CoilThreaded drop-in's
    settings) against the reference class's E, residual E and E^H."""
    import torch
    g = coils
    p = mrg_lib.Plan((20, 24, 16), 3, 1, overgrid=1.375, fft_norm=1)
    p.set_traj(0, g["kx"], g["ky"], g["kz"], g["kw"])
    p.set_smaps(torch.from_numpy(g["smaps"]).cuda())
    img = torch.from_numpy(g["img"]).cuda()
    assert rel(p.forward(0, img).cpu().numpy(), g["E"]) < 1e-5
    assert rel(p.forward(0, img, diff=torch.from_numpy(g["data"]).cuda()).cpu().numpy(), g["E_resid"]) < 1e-5
    X = p.adjoint(0, g["data"], np.zeros(p.ishape, np.complex64))
    assert rel(X, g["EH"]) < 1e-5


def test_oracle_reproduces_the_dcf_fixture(oracle_lib, dcf):
    """CPU: the oracle's Pipe density compensation gives the reference's weights (24^3 and the
    anisotropic 32 x 24 x 16, whose DCF grid has x and z extents swapped as recon_lib's)."""
    for key in ("iso", "aniso"):
        N = tuple(int(v) for v in dcf[key + "_N"])
        kw = oracle_lib.dcf_pipe(dcf[key + "_kx"], dcf[key + "_ky"], dcf[key + "_kz"], N, iters=10)
        assert rel(kw, dcf[key + "_kw"]) < 1e-6


@pytest.mark.gpu
def test_dcf_matches_reference_outputs(mrg_lib, dcf):
    """mrg_dcf_pipe on the fixture's trajectories against the reference's weights (the
    gridding adds with atomics on both sides, so the sums' order differs)."""
    for key in ("iso", "aniso"):
        N = tuple(int(v) for v in dcf[key + "_N"])
        kw = mrg_lib.dcf_pipe(dcf[key + "_kx"], dcf[key + "_ky"], dcf[key + "_kz"], N, iters=10)
        assert rel(kw, dcf[key + "_kw"]) < 1e-5
        assert np.array_equal(kw == 0, dcf[key + "_kw"] == 0)


def _espirit_defined(oracle_lib, g):
    """Voxels whose dominant vector is well defined ((s2/s1)^2 < 0.9 by the oracle)."""
    _, _, _, ratio = oracle_lib.espirit(g["imgs"], kr_f=tuple(float(v) for v in g["kr"]),
                                        cr=tuple(int(v) for v in g["cr"]))
    return ratio < 0.9


def test_oracle_reproduces_the_espirit_fixture(oracle_lib, espirit):
    """CPU: the oracle's ESPIRiT maps against SPIRIT::generateEigenCoils's (16 x 12 x 10, 4 coils)."""
    g = espirit
    m = _espirit_defined(oracle_lib, g)
    maps, _, _, _ = oracle_lib.espirit(g["imgs"], kr_f=tuple(float(v) for v in g["kr"]),
                                       cr=tuple(int(v) for v in g["cr"]))
    assert m.mean() > 0.5
    assert rel(maps[:, m], g["maps"][:, m]) < 1e-6


@pytest.mark.gpu
def test_espirit_matches_reference_outputs(mrg_lib, oracle_lib, espirit):
    """mrg_espirit on the fixture's coil images against SPIRIT's maps where the dominant
    vector is well defined (1e-4, the bound of the GPU tests against the FP64 oracle)."""
    g = espirit
    m = _espirit_defined(oracle_lib, g)
    p = mrg_lib.espirit_params(kernel_radius=tuple(float(v) for v in g["kr"]), calib_radius=tuple(int(v) for v in g["cr"]),
                               square=0)
    maps, kept, _ = mrg_lib.espirit(np.ascontiguousarray(np.moveaxis(g["imgs"], 0, -1)), p)
    got = np.moveaxis(np.asarray(maps), -1, 0)
    assert rel(got[:, m], g["maps"][:, m]) < 1e-4
