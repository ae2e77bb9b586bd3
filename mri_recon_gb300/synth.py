"""Seeded synthetic inputs for the gridFFT / SENSE workloads.

No public dataset is used.  The inputs stand in for the reference's example
runs with the same shapes and value ranges:

* ellipsoid phantom with seeded centres, semi-axes and intensities in [0, 1];
* smooth Gaussian coil maps (sigma 0.4 FOV) centred on a sphere of radius
  0.6 FOV (Fibonacci points), uniform random phase, normalised to unit
  sum-of-squares;
* 3D radial centre-out trajectory whose directions follow the golden-means
  pair used by the reference (test_voronoi.cpp:40-53), |k| = 0.5*i/R in
  normalised units scaled by N to the reference's units (k in [-N/2, N/2],
  as in commandline_recon.cxx:68-72), density compensation kw = |k|^2;
* k-space data from an FP64 direct NUDFT (small cases) or from a supplied
  forward operator (large cases), plus complex Gaussian noise.

Images are C-ordered (Nz, Ny, Nx) arrays: x fastest, as the reference's
column-major Blitz arrays.
"""
import numpy as np

PHI1 = 0.465571231876768  # golden-means pair, test_voronoi.cpp:43-44
PHI2 = 0.682327803828019


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def radial_directions(nproj, start=0):
    """Unit directions of golden-means radial projections start..start+nproj-1."""
    p = np.arange(start, start + nproj, dtype=np.float64)
    m1 = p * PHI1
    m2 = p * PHI2
    m1 -= np.floor(m1)
    m2 -= np.floor(m2)
    kz = 2.0 * m1 - 1.0
    r = np.sqrt(np.maximum(1.0 - kz * kz, 0.0))
    kx = r * np.cos(2.0 * np.pi * m2)
    ky = r * np.sin(2.0 * np.pi * m2)
    return kx, ky, kz


def radial_trajectory(N, nproj, nread, start=0, jitter_grid=0.0, grid_ratio=1.5, seed=0):
    """3D radial centre-out trajectory in reference units.

    Returns float32 arrays kx, ky, kz, kw of shape (nproj, nread) flattened in
    the reference's (readout, projection) column-major order: readout fastest.
    ``jitter_grid`` adds seeded Gaussian jitter with that standard deviation in
    grid units (divided by the grid ratio to reference units).
    """
    dx, dy, dz = radial_directions(nproj, start)
    r = 0.5 * np.arange(nread, dtype=np.float64) / nread * N
    kx = dx[:, None] * r[None, :]
    ky = dy[:, None] * r[None, :]
    kz = dz[:, None] * r[None, :]
    if jitter_grid > 0:
        g = _rng(seed + 7)
        s = jitter_grid / grid_ratio
        kx = kx + g.normal(0, s, kx.shape)
        ky = ky + g.normal(0, s, ky.shape)
        kz = kz + g.normal(0, s, kz.shape)
    kw = kx * kx + ky * ky + kz * kz
    f = lambda a: np.ascontiguousarray(a.reshape(-1), dtype=np.float32)
    return f(kx), f(ky), f(kz), f(kw)


def ellipsoid_params(n, seed):
    g = _rng(seed)
    centres = g.uniform(-0.25, 0.25, (n, 3))
    axes = g.uniform(0.05, 0.22, (n, 3))
    inten = g.uniform(0.0, 1.0, n)
    phase = g.uniform(0.0, 2 * np.pi, n)
    return centres, axes, inten, phase


def phantom(N, n_ellipsoids=10, seed=1234, frame=None, nframes=1, mod_amp=0.2):
    """Ellipsoid phantom, complex64 (Nz, Ny, Nx).  With ``frame`` set, each
    ellipsoid intensity is modulated by 1 + mod_amp*sin(2*pi*frame/nframes + phi)."""
    c, a, inten, ph = ellipsoid_params(n_ellipsoids, seed)
    x = (np.arange(N, dtype=np.float32) - N / 2) / N
    img = np.zeros((N, N, N), np.float32)
    for e in range(n_ellipsoids):
        w = inten[e]
        if frame is not None:
            w = w * (1.0 + mod_amp * np.sin(2 * np.pi * frame / nframes + ph[e]))
        # bounding box keeps the 256^3 case cheap
        lo = [max(0, int(np.floor((c[e, d] - a[e, d] + 0.5) * N)) - 1) for d in range(3)]
        hi = [min(N, int(np.ceil((c[e, d] + a[e, d] + 0.5) * N)) + 2) for d in range(3)]
        xs, ys, zs = x[lo[0]:hi[0]], x[lo[1]:hi[1]], x[lo[2]:hi[2]]
        q = (((xs[None, None, :] - c[e, 0]) / a[e, 0]) ** 2 + ((ys[None, :, None] - c[e, 1]) / a[e, 1]) ** 2
             + ((zs[:, None, None] - c[e, 2]) / a[e, 2]) ** 2)
        img[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] += np.where(q <= 1.0, np.float32(w), np.float32(0))
    return img.astype(np.complex64)


def fibonacci_sphere(n):
    i = np.arange(n, dtype=np.float64) + 0.5
    z = 1 - 2 * i / n
    r = np.sqrt(1 - z * z)
    th = np.pi * (1 + 5 ** 0.5) * i
    return np.stack([r * np.cos(th), r * np.sin(th), z], 1)


def coil_maps(N, ncoils, seed=99, sigma=0.4, radius=0.6):
    """Gaussian coil maps (C, Nz, Ny, Nx) complex64, unit sum-of-squares."""
    g = _rng(seed)
    centres = fibonacci_sphere(ncoils) * radius
    phases = g.uniform(0, 2 * np.pi, ncoils)
    x = (np.arange(N, dtype=np.float64) - N / 2) / N
    out = np.zeros((ncoils, N, N, N), np.complex64)
    sos = np.zeros((N, N, N), np.float64)
    for c in range(ncoils):
        gx = np.exp(-((x - centres[c, 0]) ** 2) / (2 * sigma ** 2))
        gy = np.exp(-((x - centres[c, 1]) ** 2) / (2 * sigma ** 2))
        gz = np.exp(-((x - centres[c, 2]) ** 2) / (2 * sigma ** 2))
        m = gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
        sos += m * m
        out[c] = (m * np.exp(1j * phases[c])).astype(np.complex64)
    out /= np.sqrt(sos)[None].astype(np.float32)
    return out


def coil_map(N, ncoils, c, seed=99, sigma=0.4, radius=0.6, normalise=True):
    """Coil c of coil_maps(N, ncoils, seed), computed alone (complex64 (N, N, N))."""
    g = _rng(seed)
    centres = fibonacci_sphere(ncoils) * radius
    phases = g.uniform(0, 2 * np.pi, ncoils)
    x = (np.arange(N, dtype=np.float64) - N / 2) / N
    sos = np.zeros((N, N, N), np.float64) if normalise else None
    m_c = None
    for k in range(ncoils) if normalise else [c]:
        gx = np.exp(-((x - centres[k, 0]) ** 2) / (2 * sigma ** 2))
        gy = np.exp(-((x - centres[k, 1]) ** 2) / (2 * sigma ** 2))
        gz = np.exp(-((x - centres[k, 2]) ** 2) / (2 * sigma ** 2))
        m = gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
        if normalise:
            sos += m * m
        if k == c:
            m_c = m
    out = (m_c * np.exp(1j * phases[c])).astype(np.complex64)
    if normalise:
        out /= np.sqrt(sos).astype(np.float32)
    return out


def coil_maps_torch(N, ncoils, device, seed=99, sigma=0.4, radius=0.6):
    """coil_maps() evaluated on a torch device (same formula and seed)."""
    import torch
    g = _rng(seed)
    centres = torch.tensor(fibonacci_sphere(ncoils) * radius, dtype=torch.float64, device=device)
    phases = torch.tensor(g.uniform(0, 2 * np.pi, ncoils), dtype=torch.float64, device=device)
    x = (torch.arange(N, dtype=torch.float64, device=device) - N / 2) / N
    gx = torch.exp(-((x[None, :] - centres[:, 0:1]) ** 2) / (2 * sigma ** 2))   # (C, N)
    gy = torch.exp(-((x[None, :] - centres[:, 1:2]) ** 2) / (2 * sigma ** 2))
    gz = torch.exp(-((x[None, :] - centres[:, 2:3]) ** 2) / (2 * sigma ** 2))
    sos = torch.zeros((N, N, N), dtype=torch.float64, device=device)
    for c in range(ncoils):
        sos += (gz[c][:, None, None] * gy[c][None, :, None] * gx[c][None, None, :]) ** 2
    rs = (1.0 / torch.sqrt(sos)).to(torch.float32)
    out = torch.empty((ncoils, N, N, N), dtype=torch.complex64, device=device)
    for c in range(ncoils):
        m = (gz[c][:, None, None] * gy[c][None, :, None] * gx[c][None, None, :]).to(torch.float32) * rs
        ph = torch.polar(torch.ones((), dtype=torch.float64, device=device), phases[c]).to(torch.complex64)
        out[c] = m.to(torch.complex64) * ph
    return out


def nudft(img, kx, ky, kz, chunk=8192):
    """FP64 direct NUDFT y(k) = sum_r img(r) exp(-2 pi i k.(r - N/2)/N).

    Separable: contracted one axis at a time per chunk of samples.
    """
    Nz, Ny, Nx = img.shape
    im = img.astype(np.complex128)
    M = kx.size
    out = np.zeros(M, np.complex128)
    rx = (np.arange(Nx) - Nx / 2) / Nx
    ry = (np.arange(Ny) - Ny / 2) / Ny
    rz = (np.arange(Nz) - Nz / 2) / Nz
    imz = im.reshape(Nz, Ny * Nx)
    for s in range(0, M, chunk):
        e = min(M, s + chunk)
        ez = np.exp(-2j * np.pi * np.outer(kz[s:e].astype(np.float64), rz))  # (m, Nz)
        ey = np.exp(-2j * np.pi * np.outer(ky[s:e].astype(np.float64), ry))
        ex = np.exp(-2j * np.pi * np.outer(kx[s:e].astype(np.float64), rx))
        a = (ez @ imz).reshape(e - s, Ny, Nx)          # sum over z
        b = np.einsum("myx,my->mx", a, ey)              # sum over y
        out[s:e] = np.einsum("mx,mx->m", b, ex)         # sum over x
    return out


def nudft_torch(imgs, kx, ky, kz, device, chunk=16384):
    """nudft() of several images at once, evaluated in FP64 with torch on `device` (the same
    separable contraction as nudft; used to synthesise test data quickly).  imgs: (C, Nz, Ny,
    Nx).  Returns (C, M) complex128 numpy."""
    import torch
    im = torch.as_tensor(np.asarray(imgs), device=device).to(torch.complex128)
    C, Nz, Ny, Nx = im.shape
    M = kx.size
    out = torch.zeros((C, M), dtype=torch.complex128, device=device)
    r = [(torch.arange(n, dtype=torch.float64, device=device) - n / 2) / n for n in (Nx, Ny, Nz)]
    imz = im.permute(1, 0, 2, 3).reshape(Nz, C * Ny * Nx)
    k = [torch.as_tensor(np.asarray(v, dtype=np.float64), device=device) for v in (kx, ky, kz)]
    for s in range(0, M, chunk):
        e = min(M, s + chunk)
        ph = [torch.exp(-2j * np.pi * torch.outer(k[d][s:e], r[d])) for d in range(3)]  # (m, N_d)
        a = (ph[2] @ imz).reshape(e - s, C, Ny, Nx)           # sum over z
        b = torch.einsum("mcyx,my->mcx", a, ph[1])             # sum over y
        out[:, s:e] = torch.einsum("mcx,mx->cm", b, ph[0])     # sum over x
    return out.cpu().numpy()


def add_noise(y, level, seed):
    """Complex Gaussian noise with standard deviation level*max|y| per component."""
    g = _rng(seed)
    s = level * float(np.max(np.abs(y)))
    return (y + s * (g.standard_normal(y.shape) + 1j * g.standard_normal(y.shape))).astype(y.dtype)


# ---------------------------------------------------------------------------
# Workload configurations.  Sizes follow the five benchmark configurations:
# SENSE-CG 64^3 x 8, FISTA 128^3 x 16, gated LLR 128^3 x 20 x 10 frames,
# differentiable 96^3 x 8 x batch 4, SENSE-CG 256^3 x 32.
# ---------------------------------------------------------------------------
CONFIGS = {
    "cg64": dict(N=64, coils=8, nproj=4096, nread=64, ellipsoids=10, noise=0.01, iters=20, seed=1235),
    "fista128": dict(N=128, coils=16, nproj=16384, nread=128, ellipsoids=10, noise=0.01, iters=100, seed=1236),
    "llr128": dict(N=128, coils=20, nread=128, frames=10, proj_lo=1500, proj_hi=3500, ellipsoids=10, noise=0.01,
                   seed=1237),
    "grad96": dict(N=96, coils=8, nproj=6000, nread=96, batch=4, jitter=0.05, ellipsoids=10, noise=0.01, seed=1238),
    "cg256": dict(N=256, coils=32, nproj=65536, nread=256, ellipsoids=200, noise=0.005, iters=30, seed=1239),
    # the 256^3 x 32 kernels at 1/8 of the volume (~2 GB on the device): the case ncu profiles run on
    "prof128": dict(N=128, coils=32, nproj=16384, nread=128, ellipsoids=50, noise=0.005, iters=5, seed=1240),
}


def frame_projection_counts(frames, lo, hi, seed):
    g = _rng(seed + 3)
    return g.integers(lo, hi + 1, frames)
