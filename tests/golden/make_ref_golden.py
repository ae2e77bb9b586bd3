"""Writes tests/golden/ref_ops.npz: inputs and outputs of the reference's own gridFFT,
WAVELET3D and THRESHOLD code (oracle/_ref/libref.so, built from the reference sources by
`make -C oracle ref`) on small seeded cases, so that the GPU tests can check the CUDA path
against the reference directly on a machine without the reference sources.

Run from the repository root: python tests/golden/make_ref_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref as R  # noqa: E402
from tests.helpers import case, edge_trajectory  # noqa: E402


def main():
    assert R.available(), "oracle/_ref needs the reference sources"
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


if __name__ == "__main__":
    main()
