"""Seeded test cases shared by the CPU and GPU tests."""
import numpy as np

from mri_recon_gb300 import synth


def rel(a, b):
    a = np.asarray(a).astype(np.complex128)
    b = np.asarray(b).astype(np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def case(N=32, C=4, nproj=600, nread=None, seed=7, jitter=0.0, noise=0.01, ellipsoids=6, nudft=False):
    """Phantom, coil maps, radial trajectory and k-space for one frame.  With nudft the
    k-space is the FP64 direct NUDFT of the phantom times each map plus noise (evaluated
    with torch on the GPU when there is one, else with numpy)."""
    nread = nread or N
    kx, ky, kz, kw = synth.radial_trajectory(N, nproj, nread, jitter_grid=jitter, seed=seed)
    img = synth.phantom(N, ellipsoids, seed=seed)
    smaps = synth.coil_maps(N, C, seed=seed + 1)
    rng = np.random.default_rng(seed)
    if nudft:
        try:
            import torch
            gpu = torch.cuda.is_available()
        except ImportError:
            gpu = False
        if gpu:
            data = synth.nudft_torch(img[None] * smaps, kx, ky, kz, "cuda").astype(np.complex64)
        else:
            data = np.stack([synth.nudft(img * smaps[c], kx, ky, kz) for c in range(C)]).astype(np.complex64)
        data = synth.add_noise(data, noise, seed + 2)
    else:
        data = (rng.standard_normal((C, kx.size)) + 1j * rng.standard_normal((C, kx.size))).astype(np.complex64)
    X = (rng.standard_normal(img.shape) + 1j * rng.standard_normal(img.shape)).astype(np.complex64)
    return dict(N=N, C=C, kx=kx, ky=ky, kz=kz, kw=kw, img=img, smaps=smaps, data=data, X=X)


def edge_trajectory(N, seed=3):
    """Samples that exercise the reference's edge rules: kw == 0, outside the grid,
    on the grid boundary (clipped taps), exactly half-integer grid positions (a
    sixth tap), and the k-space centre."""
    rng = np.random.default_rng(seed)
    S = 16 * int(np.ceil(1.5 * N / 16))
    g = S / N
    pts = []
    pts += [(0.0, 0.0, 0.0)]
    half = N / 2
    pts += [(half, 0, 0), (-half, 0, 0), (0, half * 0.999, 0), (0, 0, -half)]          # near/at the edge
    pts += [(half * 1.2, 0, 0), (0, -half * 1.6, 0), (0, 0, 3 * half)]                  # outside the grid
    # with g = 1.5, odd integer k puts dk = k*g + S/2 exactly on x.5, where
    # ceil(dk - 2.5) .. floor(dk + 2.5) spans six taps
    pts += [(1.0, 5.0, -3.0), (7.0, -1.0, 3.0), (-5.0, 1.0, 9.0)]
    pts += [tuple(rng.uniform(-half, half, 3)) for _ in range(200)]
    k = np.array(pts, np.float32)
    kw = np.sum(k.astype(np.float64) ** 2, 1).astype(np.float32)
    kw[5] = 0.0
    kw[20] = 0.0
    return k[:, 0].copy(), k[:, 1].copy(), k[:, 2].copy(), kw


def low_rank_frames(rng, T, shape_zyx, rank=2, noise=0.3):
    """T frames (T, Nz, Ny, Nx) complex64 that share `rank` spatial components with smooth
    temporal weights, plus noise: blocks whose leading singular values stand out, as in a
    gated series, so a low-rank threshold keeps some and removes others."""
    comps = rng.standard_normal((rank,) + tuple(shape_zyx)) + 1j * rng.standard_normal((rank,) + tuple(shape_zyx))
    t = np.arange(T)[:, None]
    w = np.cos(np.pi * (np.arange(rank)[None, :] + 1) * (t + 0.5) / T) + 1.0
    X = np.tensordot(w, comps, axes=1)
    X += noise * (rng.standard_normal(X.shape) + 1j * rng.standard_normal(X.shape))
    return X.astype(np.complex64)


def align_block_phases(got, ref, bs):
    """ref (T, Nz, Ny, Nx) with each whole unshifted block of bs = (bx, by, bz) voxels turned
    by the unit phase that brings it closest to got: LOWRANKCOIL::combine's output per
    block carries the phase of a singular vector, which an SVD leaves free."""
    out = np.array(ref, copy=True)
    Nz, Ny, Nx = ref.shape[1:]
    bx, by, bz = bs
    for k in range(0, Nz - bz + 1, bz):
        for j in range(0, Ny - by + 1, by):
            for i in range(0, Nx - bx + 1, bx):
                sl = (slice(None), slice(k, k + bz), slice(j, j + by), slice(i, i + bx))
                z = np.vdot(ref[sl], got[sl])
                if abs(z) > 0:
                    out[sl] = ref[sl] * (z / abs(z))
    return out


def aniso_case(N, C, nproj, seed):
    """A multi-coil case on an anisotropic image N = (Nx, Ny, Nz): the radial trajectory of
    the largest edge scaled to each axis's extent, random complex image, maps and k-space."""
    Nx, Ny, Nz = N
    m = max(N)
    c = case(N=m, C=1, nproj=nproj, seed=seed)
    rng = np.random.default_rng(seed)

    def cz(*s):
        return (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)

    return dict(kx=(c["kx"] * (Nx / m)).astype(np.float32), ky=(c["ky"] * (Ny / m)).astype(np.float32),
                kz=(c["kz"] * (Nz / m)).astype(np.float32), kw=c["kw"].astype(np.float32), img=cz(Nz, Ny, Nx),
                smaps=cz(C, Nz, Ny, Nx), data=cz(C, c["kx"].size))
