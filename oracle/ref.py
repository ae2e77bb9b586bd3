"""REFERENCE CHECKER -- TEST INFRASTRUCTURE ONLY.

ctypes front end for ``oracle/_ref/libref.so``: the reference's own gridFFT.cpp,
gridFFT_CoilThreaded.cpp, DCFgridFFT.cpp, ArrayTemplates.cpp, wavelet3D.cpp, threshold.cpp,
clear.cpp and spirit.cpp compiled unmodified (``make -C oracle ref``) against the stand-in Blitz++ / FFTW / Armadillo / HDF5 headers of
``oracle/refshim`` and driven by ``oracle/ref_driver.cpp``.  The tests use it to pin the
oracle restatement (and, through committed fixtures, the CUDA path) to the reference's
code.  It can only be built where the reference sources are present; ``available()``
says whether it is.

Conventions as in ``oracle.py``: images C-ordered (Nz, Ny, Nx) complex64, k-space flat
complex64 arrays of M samples, trajectories float32, grids (Sz, Sy, Sx).
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "libref.so")
REF_SRC = os.environ.get("MRG_REFERENCE_SRC", "/root/reference/src")
_lib = None


def build():
    """Compile oracle/_ref/libref.so from the reference sources (no-op when they are absent)."""
    if not os.path.isdir(REF_SRC):
        return False
    subprocess.run(["make", "-s", "-C", _HERE, "ref", "REF_SRC=" + REF_SRC], check=True)
    return os.path.exists(LIB_PATH)


def available():
    return os.path.exists(LIB_PATH) or build()


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise RuntimeError("oracle/_ref/libref.so is not built and the reference sources are not present")
        L = ctypes.CDLL(LIB_PATH)
        vp, i, f, l = ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_long
        ip, fp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)
        geo = [i, i, i, f, f, i]
        L.ref_tables.argtypes = geo + [ip, ip, fp, ip, fp, fp]
        L.ref_coils_tables.argtypes = geo + [i, ip, ip, fp, ip, fp, fp]
        L.ref_forward.argtypes = geo + [f, vp, vp, fp, fp, fp, fp, l, vp, vp]
        L.ref_adjoint.argtypes = geo + [f, vp, vp, vp, fp, fp, fp, fp, l]
        L.ref_grid.argtypes = geo + [f, vp, fp, fp, fp, fp, l, vp]
        L.ref_ungrid.argtypes = geo + [vp, fp, fp, fp, fp, l, vp, vp]
        L.ref_fft.argtypes = [i, i, i, f, i, vp]
        L.ref_wavelet.argtypes = [i, i, i, ip, ip, i, i, vp]
        L.ref_fraction_threshold.restype = ctypes.c_float
        L.ref_fraction_threshold.argtypes = [i, i, i, i, ctypes.POINTER(vp), f, i]
        pv = ctypes.POINTER(vp)
        L.ref_adjoint_sos.argtypes = geo + [f, vp, vp, fp, fp, fp, fp, l]
        L.ref_gaussian_blur.argtypes = [vp, i, i, i, fp]
        L.ref_wavelet_shifts.argtypes = [i, i, i, ip, i, l, i, ip]
        L.ref_dcf_table.argtypes = [f, i, fp, ip]
        L.ref_coils_forward.argtypes = geo + [f, i, vp, pv, fp, fp, fp, fp, l, pv, pv]
        L.ref_coils_adjoint.argtypes = geo + [f, i, vp, pv, pv, fp, fp, fp, fp, l]
        L.ref_dcf_pipe.argtypes = [fp, fp, fp, l, i, i, i, i, f, f, f, f, i, fp]
        L.ref_espirit.argtypes = [pv, i, i, i, i, fp, ip, f, i, pv]
        L.ref_llr_update_threshold.restype = ctypes.c_float
        L.ref_llr_update_threshold.argtypes = [pv, i, i, i, i, ip, f, f, i]
        L.ref_llr_thresh.argtypes = [pv, i, i, i, i, ip, i, f, f, l]
        L.ref_clear_update_threshold.restype = ctypes.c_float
        L.ref_clear_update_threshold.argtypes = [pv, i, i, i, i, i, ip, f, f, i]
        L.ref_clear_thresh.argtypes = [pv, i, i, i, i, i, ip, i, f, f, l]
        L.ref_clear_combine.argtypes = [pv, i, i, i, i, i, ip, pv]
        _lib = L
    return _lib


def _c64(a):
    return np.ascontiguousarray(a, dtype=np.complex64)


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


class Gridder:
    """A reference gridFFT set up by precalc_gridding for an Nx x Ny x Nz 3D non-Cartesian
    acquisition (a new object per call, as the driver builds one per call)."""

    def __init__(self, N, overgrid=1.5, dwin=-1.0, kernel=1, k_rad=9999.0):
        self.N = (N, N, N) if np.isscalar(N) else tuple(N)  # (Nx, Ny, Nz)
        self.geo = (self.N[0], self.N[1], self.N[2], float(overgrid), float(dwin), int(kernel))
        self.k_rad = float(k_rad)
        self.S, self.og, self.beta, lut, win = self.tables()
        self.lut, self.win = lut, win

    @property
    def ishape(self):
        return (self.N[2], self.N[1], self.N[0])

    @property
    def gshape(self):
        return (self.S[2], self.S[1], self.S[0])

    def tables(self):
        S, og, ll = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), ctypes.c_int()
        be = (ctypes.c_float * 3)()
        fp = ctypes.POINTER(ctypes.c_float)
        assert lib().ref_tables(*self.geo, S, og, be, ctypes.byref(ll), None, None) == 0
        lut = np.zeros(3 * ll.value, np.float32)
        win = np.zeros(sum(S), np.float32)
        assert lib().ref_tables(*self.geo, S, og, be, ctypes.byref(ll), lut.ctypes.data_as(fp),
                                win.ctypes.data_as(fp)) == 0
        s0, s1 = S[0], S[0] + S[1]
        return tuple(S), tuple(og), tuple(be), lut.reshape(3, -1), (win[:s0], win[s0:s1], win[s1:])

    def forward(self, X, smap, kx, ky, kz, kw, diff=None):
        """gridFFT::backward (E), or backward_residual when diff is given."""
        X, smap = _c64(X), _c64(smap)
        diff = None if diff is None else _c64(diff)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        out = np.zeros(kx.size, np.complex64)
        assert lib().ref_forward(*self.geo, self.k_rad, _p(X), _p(smap), px, py, pz, pw, kx.size, _p(out),
                                 _p(diff)) == 0
        return out

    def adjoint(self, X, smap, data, kx, ky, kz, kw):
        """gridFFT::forward (E^H): X += ..."""
        X = _c64(X).copy()
        smap, data = _c64(smap), _c64(data)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        assert lib().ref_adjoint(*self.geo, self.k_rad, _p(X), _p(smap), _p(data), px, py, pz, pw, kx.size) == 0
        return X

    def grid(self, data, kx, ky, kz, kw):
        """chop_grid_forward into a zeroed grid."""
        data = _c64(data)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        g = np.zeros(self.gshape, np.complex64)
        assert lib().ref_grid(*self.geo, self.k_rad, _p(data), px, py, pz, pw, kx.size, _p(g)) == 0
        return g

    def ungrid(self, grid, kx, ky, kz, kw, diff=None):
        """chop_grid_backward from a grid."""
        grid = _c64(grid).reshape(self.gshape)
        diff = None if diff is None else _c64(diff)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        out = np.zeros(kx.size, np.complex64)
        assert lib().ref_ungrid(*self.geo, _p(grid), px, py, pz, pw, kx.size, _p(out), _p(diff)) == 0
        return out

    def adjoint_sos(self, X, data, kx, ky, kz, kw):
        """gridFFT::forward_sos: X += |deapodised E^H data|^2 (the map-free coil image)."""
        X, data = _c64(X).copy(), _c64(data)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        assert lib().ref_adjoint_sos(*self.geo, self.k_rad, _p(X), _p(data), px, py, pz, pw, kx.size) == 0
        return X

    def coils_tables(self, C=2):
        """S, og, beta, kernel tables and windows from gridFFT_CoilThreaded::precalc_gridding."""
        S, og, ll = (ctypes.c_int * 3)(), (ctypes.c_int * 3)(), ctypes.c_int()
        be = (ctypes.c_float * 3)()
        fp = ctypes.POINTER(ctypes.c_float)
        assert lib().ref_coils_tables(*self.geo, C, S, og, be, ctypes.byref(ll), None, None) == 0
        lut = np.zeros(3 * ll.value, np.float32)
        win = np.zeros(sum(S), np.float32)
        assert lib().ref_coils_tables(*self.geo, C, S, og, be, ctypes.byref(ll), lut.ctypes.data_as(fp),
                                      win.ctypes.data_as(fp)) == 0
        return tuple(S), tuple(og), tuple(be), lut.reshape(3, -1), win

    def coils_forward(self, X, smaps, kx, ky, kz, kw, diff=None):
        """gridFFT_CoilThreaded::backward (E of every coil of smaps (C, Nz, Ny, Nx)), or
        backward_residual when diff (C, M) is given: (C, M)."""
        X = _c64(X)
        smaps = [_c64(m) for m in smaps]
        C = len(smaps)
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        out = np.zeros((C, kx.size), np.complex64)
        dif = None if diff is None else [_c64(d) for d in diff]
        assert lib().ref_coils_forward(*self.geo, self.k_rad, C, _p(X), _ptrs(smaps), px, py, pz, pw, kx.size,
                                       _ptrs([out[c] for c in range(C)]), None if dif is None else _ptrs(dif)) == 0
        return out

    def coils_adjoint(self, X, smaps, data, kx, ky, kz, kw):
        """gridFFT_CoilThreaded::forward (E^H with maps, summed over the coils): X += ..."""
        X = _c64(X).copy()
        smaps, data = [_c64(m) for m in smaps], [_c64(d) for d in data]
        (kx, px), (ky, py), (kz, pz), (kw, pw) = _f32(kx), _f32(ky), _f32(kz), _f32(kw)
        assert lib().ref_coils_adjoint(*self.geo, self.k_rad, len(smaps), _p(X), _ptrs(smaps), _ptrs(data), px, py,
                                       pz, pw, kx.size) == 0
        return X

    def fft(self, grid, inverse):
        """do_fft (pruned to the crop) or do_ifft."""
        g = _c64(grid).reshape(self.gshape).copy()
        assert lib().ref_fft(self.N[0], self.N[1], self.N[2], self.geo[3], int(bool(inverse)), _p(g)) == 0
        return g


def wavelet(X, levels, shift, wtype=1, inverse=False):
    """WAVELET3D forward / backward of one (Nz, Ny, Nx) volume with shifts (x, y, z)."""
    X = _c64(X).copy()
    Nz, Ny, Nx = X.shape
    assert lib().ref_wavelet(Nx, Ny, Nz, (ctypes.c_int * 3)(*levels), (ctypes.c_int * 3)(*shift), int(wtype),
                             int(bool(inverse)), _p(X)) == 0
    return X


def fraction_threshold(vols, fraction, apply=False):
    """THRESHOLD -threshold_type fraction: (threshold, thresholded volumes or None)."""
    vols = [_c64(v).copy() for v in vols]
    Nz, Ny, Nx = vols[0].shape
    arr = (ctypes.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    t = lib().ref_fraction_threshold(Nx, Ny, Nz, len(vols), arr, float(fraction), int(bool(apply)))
    return float(t), (vols if apply else None)


def _vols(arrs):
    return (ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])


def llr_update_threshold(vols, bs, amp=4.0, t2=6.0, iteration=0):
    """LOWRANKCOIL::update_threshold(image, 0, iteration) over frames (Nz, Ny, Nx): smax."""
    vols = [_c64(v) for v in vols]
    Nz, Ny, Nx = vols[0].shape
    return float(lib().ref_llr_update_threshold(_vols(vols), len(vols), Nx, Ny, Nz, (ctypes.c_int * 3)(*bs),
                                                float(amp), float(t2), int(iteration)))


def llr_thresh(vols, bs, block_iter, alpha, smax, rand_skip):
    """LOWRANKCOIL::thresh(image, 0) on copies of the frames, clear_alpha_time = alpha, rand()
    seeded with srand(1) and advanced rand_skip draws."""
    vols = [_c64(v).copy() for v in vols]
    Nz, Ny, Nx = vols[0].shape
    assert lib().ref_llr_thresh(_vols(vols), len(vols), Nx, Ny, Nz, (ctypes.c_int * 3)(*bs), int(block_iter),
                                float(alpha), float(smax), int(rand_skip)) == 0
    return vols


def _coil_vols(XX):
    T, C = XX.shape[:2]
    return [XX[t, c] for t in range(T) for c in range(C)]


def clear_update_threshold(XX, bs, amp=4.0, t2=6.0, iteration=0):
    """LOWRANKCOIL::update_threshold(image, 2, iteration) on coil images (T, C, Nz, Ny, Nx)."""
    XX = _c64(XX)
    T, C, Nz, Ny, Nx = XX.shape
    return float(lib().ref_clear_update_threshold(_vols(_coil_vols(XX)), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*bs),
                                                  float(amp), float(t2), int(iteration)))


def clear_thresh(XX, bs, block_iter, alpha, smax, rand_skip):
    """LOWRANKCOIL::thresh(image, 2) on a copy of coil images (T, C, Nz, Ny, Nx)."""
    XX = _c64(XX).copy()
    T, C, Nz, Ny, Nx = XX.shape
    assert lib().ref_clear_thresh(_vols(_coil_vols(XX)), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*bs), int(block_iter),
                                  float(alpha), float(smax), int(rand_skip)) == 0
    return XX


def clear_combine(XX, bs):
    """LOWRANKCOIL::combine of coil images (T, C, Nz, Ny, Nx) into (T, Nz, Ny, Nx) (zero where
    no block covers a voxel).  Each block's result carries the unit phase of its first right
    singular vector, which the SVD leaves free."""
    XX = _c64(XX)
    T, C, Nz, Ny, Nx = XX.shape
    im = np.zeros((T, Nz, Ny, Nx), np.complex64)
    assert lib().ref_clear_combine(_vols(_coil_vols(XX)), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*bs),
                                   _vols([im[t] for t in range(T)])) == 0
    return im


def dcf_pipe(kx, ky, kz, N, iters=20, dwin=2.1, scale=1.0, overgrid=2.1, acc=1.0, kernel=0):
    """RECON::dcf_calc's Pipe iteration around the reference's DCFgridFFT; returns kw (float32)."""
    if np.isscalar(N):
        N = (N, N, N)
    (kx, px), (ky, py), (kz, pz) = _f32(kx), _f32(ky), _f32(kz)
    out = np.zeros(kx.size, np.float32)
    assert lib().ref_dcf_pipe(px, py, pz, kx.size, N[0], N[1], N[2], int(iters), float(dwin), float(scale),
                              float(overgrid), float(acc), int(kernel),
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == 0
    return out


def espirit(images, kr_f=(3.0, 3.0, 3.0), cr=(12, 12, 12), svd_thresh=0.01, square=False):
    """SPIRIT::generateEigenCoils on coil images (C, Nz, Ny, Nx): the maps (C, Nz, Ny, Nx)
    complex64."""
    imgs = [_c64(x).copy() for x in images]
    C = len(imgs)
    Nz, Ny, Nx = imgs[0].shape
    maps = np.zeros((C, Nz, Ny, Nx), np.complex64)
    assert lib().ref_espirit(_ptrs(imgs), C, Nx, Ny, Nz, (ctypes.c_float * 3)(*kr_f), (ctypes.c_int * 3)(*cr),
                             float(svd_thresh), int(bool(square)), _ptrs([maps[c] for c in range(C)])) == 0
    return maps


def gaussian_blur(X, sigma):
    """NDarray::gaussian_blur of one (Nz, Ny, Nx) complex volume (a copy), sigma = (x, y, z)."""
    X = _c64(X).copy()
    Nz, Ny, Nx = X.shape
    assert lib().ref_gaussian_blur(_p(X), Nx, Ny, Nz, (ctypes.c_float * 3)(*[float(v) for v in sigma])) == 0
    return X


def wavelet_shifts(shape_xyz, levels, wtype, skip, n):
    """WAVELET3D::random_shift called n times after srand(1) and `skip` draws: (n, 3) shifts."""
    out = (ctypes.c_int * (3 * n))()
    assert lib().ref_wavelet_shifts(*[int(v) for v in shape_xyz], (ctypes.c_int * 3)(*levels), int(wtype), int(skip),
                                    int(n), out) == 0
    return np.array(out[:], dtype=np.int64).reshape(n, 3)


def dcf_table(dwin=2.1, kernel=0):
    """DCFgridFFT::precalc_kernel's normalised polynomial table (float32)."""
    n = ctypes.c_int()
    assert lib().ref_dcf_table(float(dwin), int(kernel), None, ctypes.byref(n)) == 0
    out = np.zeros(n.value, np.float32)
    assert lib().ref_dcf_table(float(dwin), int(kernel), out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                               ctypes.byref(n)) == 0
    return out
