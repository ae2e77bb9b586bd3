"""The oracle's ESPIRiT restatement (src/spirit.cpp:137-550) checked on the CPU against a
numpy restatement written from the reference's loops: the centred inverse FFT
(numpy.fft), the calibration matrix in the reference's row / column order, LAPACK's SVD
for the calibration and for every voxel, and phase_correct."""
import numpy as np
import pytest

from mri_recon_gb300 import synth


def _np_espirit(imgs, kr_f, cr, svd_thresh=0.01):
    C, Nz, Ny, Nx = imgs.shape
    N = (Nx, Ny, Nz)
    s = 2 * ((np.arange(Nz)[:, None, None] + np.arange(Ny)[None, :, None] + np.arange(Nx)[None, None, :]) % 2) - 1
    scale = np.float64(np.float32(1.0 / np.sqrt(np.float32(Nz) * np.float32(Ny) * np.float32(Nx))))
    K = np.stack([np.fft.ifftn(imgs[c].astype(np.complex128) * s) * (Nx * Ny * Nz) * s * scale for c in range(C)])
    kr = [int(np.ceil(v)) for v in kr_f]
    ce = [cr[d] - kr[d] for d in range(3)]
    rows = [(ix, iy, iz) for iz in range(-ce[2], ce[2] + 1) for iy in range(-ce[1], ce[1] + 1)
            for ix in range(-ce[0], ce[0] + 1)
            if not (np.float32(ix * ix) / (ce[0] ** 2) + np.float32(iy * iy) / (ce[1] ** 2)
                    + np.float32(iz * iz) / (ce[2] ** 2) > 1)]
    kp = [(jx, jy, jz) for jz in range(-kr[2], kr[2] + 1) for jy in range(-kr[1], kr[1] + 1)
          for jx in range(-kr[0], kr[0] + 1)
          if np.float32(jx * jx) / np.float32(kr_f[0] ** 2) + np.float32(jy * jy) / np.float32(kr_f[1] ** 2)
          + np.float32(jz * jz) / np.float32(kr_f[2] ** 2) <= 1]
    cz, cy, cx = Nz // 2, Ny // 2, Nx // 2
    A = np.array([[K[c, kz + iz + cz, ky + iy + cy, kx + ix + cx] for c in range(C) for (kx, ky, kz) in kp]
                  for (ix, iy, iz) in rows])
    _, sv, Vh = np.linalg.svd(A, full_matrices=False)
    nv = int((sv >= np.float32(sv[0] * np.sqrt(np.float32(svd_thresh)))).sum())
    V = Vh.conj().T[:, :nv]
    nk = len(kp)

    def H(x, j, n):
        nn = n // 2 + j
        sc = np.float64(np.float32(1.0 / np.sqrt(np.float32(n))))
        return (2 * (x % 2) - 1) * (2 * (nn % 2) - 1) * np.exp(2j * np.pi * ((nn * x) % n) / n) * sc
    maps = np.zeros(imgs.shape, np.complex128)
    for z in range(Nz):
        for y in range(Ny):
            for x in range(Nx):
                g = np.array([H(x, jx, Nx) * H(y, jy, Ny) * H(z, jz, Nz) for (jx, jy, jz) in kp])
                Ax = np.stack([g @ V[c * nk:(c + 1) * nk, :] for c in range(C)])
                m = np.conj(np.linalg.svd(Ax)[0][:, 0])
                maps[:, z, y, x] = m * np.exp(-1j * np.angle(m[0])) / np.sqrt((np.abs(m) ** 2).sum())
    return maps, nv, sv


@pytest.mark.parametrize("N,C,kr,cr", [((12, 12, 12), 3, (2.0, 2.0, 2.0), (5, 5, 5)),
                                       ((12, 10, 8), 2, (1.5, 2.0, 1.0), (4, 4, 3))])
def test_espirit_vs_numpy(oracle_lib, N, C, kr, cr):
    Nx, Ny, Nz = N
    img = synth.phantom(max(N), 6, seed=3)[:Nz, :Ny, :Nx]
    sm = synth.coil_maps(max(N), C, seed=4)[:, :Nz, :Ny, :Nx]
    imgs = (img[None] * sm).astype(np.complex64)
    maps, nV, sv, ratio = oracle_lib.espirit(imgs, kr_f=kr, cr=cr)
    ref, nv, svr = _np_espirit(imgs, kr, cr)
    assert nV == nv
    assert np.abs(sv[:len(svr)] - svr[:len(sv)]).max() < 1e-12 * svr[0]
    assert np.abs(maps - ref).max() < 1e-10
    # phase_correct: unit sum of squares, coil 0 real and non-negative
    assert np.abs((np.abs(maps) ** 2).sum(0) - 1).max() < 1e-12
    assert np.abs(maps[0].imag).max() < 1e-12 and maps[0].real.min() >= 0
    assert ratio.min() >= 0 and ratio.max() <= 1
