"""Writes inputs and outputs of the reference's own code (oracle/_ref/libref.so, built from
the reference sources by `make -C oracle ref`) on small seeded cases, so that the GPU tests
can check the CUDA path against the reference directly on a machine without the reference
sources:

  tests/golden/ref_ops.npz      gridFFT (E, residual E, E^H, edge samples), WAVELET3D, THRESHOLD
  tests/golden/ref_lowrank.npz  LOWRANKCOIL in time (update_threshold, thresh) and in the coil
                                dimension (update_threshold, thresh, combine)
  tests/golden/ref_coils.npz    gridFFT_CoilThreaded at its default overgrid 1.375 (E, residual
                                E, E^H over 3 coils of a 20 x 24 x 16 image)
  tests/golden/ref_dcf.npz      the Pipe density compensation around DCFgridFFT (10 iterations,
                                an isotropic 24^3 and an anisotropic 32 x 24 x 16 matrix)
  tests/golden/ref_espirit.npz  SPIRIT::generateEigenCoils on 4 coil images of 16 x 12 x 10
                                (anisotropic kernel and calibration radii)

Run from the repository root:
  python tests/golden/make_ref_golden.py [ops] [lowrank] [coils] [dcf] [espirit]
(both when no argument is given).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref as R  # noqa: E402
from tests.helpers import aniso_case, case, edge_trajectory, low_rank_frames  # noqa: E402


def lowrank():
    out = {}
    rng = np.random.default_rng(211)
    # time low rank: 6 frames of 12^3, 4^3 blocks (27 per shift), iteration 2 of the schedule
    X = low_rank_frames(rng, 6, (12, 12, 12))
    vols = [X[t] for t in range(6)]
    smax = R.llr_update_threshold(vols, (4, 4, 4), 4.0, 6.0, 2)
    out.update(llr_in=X, llr_smax=np.float32(smax))
    out["llr_out"] = np.stack(R.llr_thresh(vols, (4, 4, 4), 4, 0.1, smax, 11))
    out["llr_out_iter1"] = np.stack(R.llr_thresh(vols, (4, 4, 4), 1, 0.1, smax, 0))  # no shift
    # coil low rank: 2 frames x 6 coils of 8^3 (the reference's layout (T, C, Nz, Ny, Nx))
    XX = np.stack([low_rank_frames(rng, 6, (8, 8, 8)) for _ in range(2)])
    smax_c = R.clear_update_threshold(XX, (4, 4, 4), 4.0, 6.0, 1)
    out.update(coil_in=XX, coil_smax=np.float32(smax_c))
    out["coil_out"] = R.clear_thresh(XX, (4, 4, 4), 4, 0.05, smax_c, 5)
    out["coil_combine"] = R.clear_combine(XX, (4, 4, 4))
    path = os.path.join(ROOT, "tests", "golden", "ref_lowrank.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def coils():
    N, C = (20, 24, 16), 3
    c = aniso_case(N, C, 150, seed=301)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    g = R.Gridder(N, overgrid=1.375)
    out = dict(c)
    out["E"] = g.coils_forward(c["img"], c["smaps"], *a)
    out["E_resid"] = g.coils_forward(c["img"], c["smaps"], *a, diff=c["data"])
    out["EH"] = g.coils_adjoint(np.zeros(g.ishape, np.complex64), c["smaps"], c["data"], *a)
    path = os.path.join(ROOT, "tests", "golden", "ref_coils.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def dcf():
    out = {}
    for key, N in (("iso", (24, 24, 24)), ("aniso", (32, 24, 16))):
        m = max(N)
        c = case(N=m, C=1, nproj=300, seed=401)
        kx, ky, kz = (c[k] * np.float32(N[d] / m) for d, k in enumerate(("kx", "ky", "kz")))
        out.update({key + "_kx": kx, key + "_ky": ky, key + "_kz": kz, key + "_N": np.array(N, np.int32)})
        out[key + "_kw"] = R.dcf_pipe(kx, ky, kz, N, iters=10)
    path = os.path.join(ROOT, "tests", "golden", "ref_dcf.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def espirit():
    from mri_recon_gb300 import synth
    N, C = (16, 12, 10), 4
    Nx, Ny, Nz = N
    img = synth.phantom(16, 6, seed=7)[:Nz, :Ny, :Nx]
    sm = synth.coil_maps(16, C, seed=8)[:, :Nz, :Ny, :Nx]
    imgs = (img[None] * sm).astype(np.complex64)
    kr, cr = (2.0, 1.5, 1.5), (6, 5, 4)
    out = dict(imgs=imgs, kr=np.array(kr, np.float32), cr=np.array(cr, np.int32))
    out["maps"] = R.espirit(imgs, kr, cr)
    path = os.path.join(ROOT, "tests", "golden", "ref_espirit.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def ops():
    out = {}
    # two coils, 24^3 image, 400 x 24 radial: E, E residual, E^H per coil
    N, C = 24, 2
    c = case(N=N, C=C, nproj=400, seed=101)
    a = (c["kx"], c["ky"], c["kz"], c["kw"])
    g = R.Gridder(N)
    out.update(kx=c["kx"], ky=c["ky"], kz=c["kz"], kw=c["kw"], img=c["img"], smaps=c["smaps"], data=c["data"])
    out["E"] = np.stack([g.forward(c["img"], c["smaps"][k], *a) for k in range(C)])
    out["E_resid"] = np.stack([g.forward(c["img"], c["smaps"][k], *a, diff=c["data"][k]) for k in range(C)])
    out["EH"] = np.stack([g.adjoint(np.zeros(g.ishape, np.complex64), c["smaps"][k], c["data"][k], *a)
                          for k in range(C)])
    # edge samples (outside the grid, kw == 0, half-integer positions, the grid boundary)
    e = edge_trajectory(N, seed=102)
    rng = np.random.default_rng(103)
    de = (rng.standard_normal(e[0].size) + 1j * rng.standard_normal(e[0].size)).astype(np.complex64)
    out.update(ekx=e[0], eky=e[1], ekz=e[2], ekw=e[3], edata=de)
    out["edge_E"] = g.forward(c["img"], c["smaps"][0], *e)
    out["edge_EH"] = g.adjoint(np.zeros(g.ishape, np.complex64), c["smaps"][0], de, *e)
    # wavelet (DB4, 3 levels, shifts (1, 2, 3)) and the fraction threshold over two volumes
    V = (rng.standard_normal((2, 16, 24, 32)) + 1j * rng.standard_normal((2, 16, 24, 32))).astype(np.complex64)
    out["wave_in"] = V[0]
    out["wave_db4"] = R.wavelet(V[0], (3, 3, 3), (1, 2, 3), 1)
    out["wave_db2"] = R.wavelet(V[0], (3, 3, 3), (1, 0, 1), 0)
    out["thr_in"] = V
    t, vols = R.fraction_threshold([V[0], V[1]], 0.1, apply=True)
    out["thr_value"] = np.float32(t)
    out["thr_out"] = np.stack(vols)
    path = os.path.join(ROOT, "tests", "golden", "ref_ops.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


def main(which):
    assert R.available(), "oracle/_ref needs the reference sources"
    for name in which or ("ops", "lowrank", "coils", "dcf", "espirit"):
        {"ops": ops, "lowrank": lowrank, "coils": coils, "dcf": dcf, "espirit": espirit}[name]()


if __name__ == "__main__":
    main(sys.argv[1:])
