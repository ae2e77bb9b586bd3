"""ORACLE -- TEST INFRASTRUCTURE ONLY.

ctypes front end for ``oracle/_build/liboracle.so``, the CPU restatement of the
uwmri/mri_recon gridFFT / recon_lib hot path (see ``oracle.cpp``).  Only the
tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module, and only as the checker.  Parity unpinned: the reference has no golden
vectors for this path and cannot be built here.

Array conventions follow the reference: images are C-ordered (Nz, Ny, Nx)
complex arrays (column-major x-fastest in the reference's terms), k-space data
are flat complex arrays of M samples, trajectories are float32.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

KAISER, TRIANGLE, SINC, POLY = 1, 0, 2, 3


def build():
    """Compile the oracle shared library (make, in oracle/)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, fp, ip, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)
        L.orc_plan_create.restype = vp
        L.orc_plan_create.argtypes = [ctypes.c_int] * 3 + [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                                             ctypes.c_int, ctypes.c_int]
        L.orc_plan_destroy.argtypes = [vp]
        L.orc_plan_info.argtypes = [vp, ip, ip, fp, fp, fp, ip]
        L.orc_get_tables.argtypes = [vp, fp, fp]
        L.orc_adjoint.argtypes = [vp, vp, vp, vp, fp, fp, fp, fp, ctypes.c_long]
        L.orc_forward.argtypes = [vp, vp, vp, vp, fp, fp, fp, fp, ctypes.c_long, vp]
        L.orc_adjoint_sos.argtypes = [vp, vp, vp, fp, fp, fp, fp, ctypes.c_long]
        L.orc_set_k_rad.argtypes = [vp, ctypes.c_float]
        L.orc_gaussian_blur.argtypes = [vp] + [ctypes.c_int] * 3 + [fp, ctypes.c_int]
        L.orc_sos_normalize.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_long, ctypes.c_int]
        L.orc_dcf_pipe.argtypes = [fp, fp, fp, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, fp,
                                   ctypes.c_int]
        L.orc_dcf_table.argtypes = [ctypes.c_float, ctypes.c_int, fp, ip]
        L.orc_get_grid.argtypes = [vp, vp]
        L.orc_set_grid.argtypes = [vp, vp]
        L.orc_grid.argtypes = [vp, vp, fp, fp, fp, fp, ctypes.c_long]
        L.orc_ungrid.argtypes = [vp, vp, fp, fp, fp, fp, ctypes.c_long, vp]
        L.orc_set_image.argtypes = [vp, vp, vp]
        L.orc_values_at.argtypes = [vp, dp, dp, dp, ctypes.c_long, vp]
        L.orc_accumulate.argtypes = [vp, vp, vp]
        L.orc_fft3.argtypes = [vp, ctypes.c_int]
        L.orc_fft1d.argtypes = [ctypes.c_int, vp, ctypes.c_int, ctypes.c_int]
        L.orc_cg.argtypes = [vp, vp, ctypes.c_int, ctypes.POINTER(vp), dp]
        L.orc_fista.argtypes = [vp, vp, vp, ctypes.POINTER(vp), dp, fp, fp]
        L.orc_normal.argtypes = [vp, vp, ctypes.c_int, vp, vp]
        L.orc_wavelet.argtypes = [ctypes.c_int] * 3 + [ip, ip, ctypes.c_int, vp, ctypes.c_int, ctypes.c_int]
        L.orc_wavelet_info.argtypes = [ctypes.c_int] * 3 + [ip, ctypes.c_int, ip, fp]
        L.orc_fraction_threshold.restype = ctypes.c_float
        L.orc_fraction_threshold.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_int]
        L.orc_soft_threshold.argtypes = [vp, ctypes.c_long, ctypes.c_float, ctypes.c_int]
        L.orc_llr_update_threshold.restype = ctypes.c_float
        L.orc_llr_update_threshold.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ip, ip, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int]
        L.orc_llr_thresh.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ip, ip, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_long, ctypes.c_int]
        L.orc_clear_update_threshold.restype = ctypes.c_float
        L.orc_clear_update_threshold.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_float,
                                                 ctypes.c_float, ctypes.c_int, ctypes.c_int]
        L.orc_clear_thresh.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int,
                                       ctypes.c_float, ctypes.c_float, ctypes.c_long, ctypes.c_int]
        L.orc_clear_combine.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ctypes.c_int, ip, ip, ctypes.POINTER(vp),
                                        ctypes.c_int]
        L.orc_clear.restype = ctypes.c_int
        L.orc_clear.argtypes = [vp, vp, vp, ctypes.POINTER(vp), ctypes.POINTER(vp), dp]
        L.orc_espirit.restype = ctypes.c_int
        L.orc_espirit.argtypes = [ctypes.POINTER(vp), ctypes.c_int, ip, fp, ip, ctypes.c_float, ctypes.c_int,
                                  ctypes.POINTER(vp), dp, dp]
        L.orc_glibc_rand.argtypes = [ctypes.c_long, ctypes.c_int, ip]
        L.orc_pregate.restype = ctypes.c_long
        L.orc_pregate.argtypes = [vp, vp, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int] + [vp] * 5 + \
            [ctypes.c_int, ctypes.c_long] + [vp] * 5 + [ctypes.c_long]
        L.orc_cg_vectors.restype = ctypes.c_double
        L.orc_cg_vectors.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_int] + [ctypes.POINTER(vp)] * 4 + [ctypes.c_int]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _ip(vals):
    arr = (ctypes.c_int * len(vals))(*[int(v) for v in vals])
    return arr


class _Frames(ctypes.Structure):
    _fields_ = [("Nt", ctypes.c_int), ("C", ctypes.c_int),
                ("kx", ctypes.c_void_p), ("ky", ctypes.c_void_p), ("kz", ctypes.c_void_p), ("kw", ctypes.c_void_p),
                ("M", ctypes.c_void_p), ("data", ctypes.c_void_p), ("smaps", ctypes.c_void_p)]


class FistaParams(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("max_eig_iter", ctypes.c_int), ("cycle_spins", ctypes.c_int),
                ("wave_levels", ctypes.c_int * 3), ("wave_type", ctypes.c_int), ("thresh", ctypes.c_float),
                ("use_threshold", ctypes.c_int), ("llr_bs", ctypes.c_int * 3), ("llr_block_iter", ctypes.c_int),
                ("llr_alpha", ctypes.c_float), ("clear_amp", ctypes.c_float), ("clear_t2", ctypes.c_float),
                ("rand_skip", ctypes.c_long)]


class ClearParams(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("bs", ctypes.c_int * 3), ("block_iter", ctypes.c_int),
                ("alpha_coil", ctypes.c_float), ("clear_amp", ctypes.c_float), ("clear_t2", ctypes.c_float),
                ("early_stop_thresh", ctypes.c_float), ("early_stop_range", ctypes.c_int), ("rand_skip", ctypes.c_long),
                ("use_threshold", ctypes.c_int), ("thresh", ctypes.c_float), ("cycle_spins", ctypes.c_int),
                ("wave_levels", ctypes.c_int * 3), ("wave_type", ctypes.c_int)]


def clear_params(max_iter=50, bs=(4, 4, 4), block_iter=4, alpha_coil=0.01, clear_amp=4.0, clear_t2=6.0,
                 early_stop_thresh=0.0, early_stop_range=5, rand_skip=0, use_threshold=0, thresh=0.0,
                 cycle_spins=4, wave_levels=(4, 4, 4), wave_type=1):
    """The CLEAR loop's parameters with the reference's defaults (clear.cpp:47-61, recon_lib.cpp:83-85)."""
    return ClearParams(max_iter, (ctypes.c_int * 3)(*bs), block_iter, alpha_coil, clear_amp, clear_t2,
                       early_stop_thresh, early_stop_range, rand_skip, use_threshold, thresh, cycle_spins,
                       (ctypes.c_int * 3)(*wave_levels), wave_type)


class Plan:
    """One gridFFT operator (one coil at a time), FP32 (prec=0) or FP64 (prec=1)."""

    def __init__(self, N, overgrid=1.5, dwin=-1.0, kernel=KAISER, k_rad=9999.0, prec=0, analytic=False):
        if np.isscalar(N):
            N = (N, N, N)
        self.N = tuple(int(n) for n in N)  # (Nx, Ny, Nz)
        self.prec = prec
        self.cdt = np.complex128 if prec else np.complex64
        self.h = lib().orc_plan_create(self.N[0], self.N[1], self.N[2], overgrid, dwin, kernel, k_rad, prec,
                                       1 if analytic else 0)
        S = (ctypes.c_int * 3)()
        og = (ctypes.c_int * 3)()
        gr = (ctypes.c_float * 3)()
        be = (ctypes.c_float * 3)()
        dw = (ctypes.c_float * 3)()
        ll = ctypes.c_int()
        lib().orc_plan_info(self.h, S, og, gr, be, dw, ctypes.byref(ll))
        self.S = tuple(S)
        self.og = tuple(og)
        self.grid_ratio = tuple(gr)
        self.beta = tuple(be)
        self.dwin = tuple(dw)
        self.lut_len = ll.value

    def __del__(self):
        try:
            lib().orc_plan_destroy(self.h)
        except Exception:
            pass

    @property
    def ishape(self):
        return (self.N[2], self.N[1], self.N[0])

    @property
    def gshape(self):
        return (self.S[2], self.S[1], self.S[0])

    def tables(self):
        lut = np.zeros(3 * self.lut_len, np.float32)
        win = np.zeros(sum(self.S), np.float32)
        lib().orc_get_tables(self.h, lut.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), win.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        s0, s1 = self.S[0], self.S[0] + self.S[1]
        return lut.reshape(3, self.lut_len), (win[:s0], win[s0:s1], win[s1:])

    def _c(self, a):
        return None if a is None else np.ascontiguousarray(a, dtype=self.cdt)

    def adjoint(self, X, smap, data, kx, ky, kz, kw):
        """gridFFT::forward (E^H): X += accumulate(ifft(grid(data*kw)))."""
        X = self._c(X)
        assert X.flags.writeable
        smap, data = self._c(smap), self._c(data)
        kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz); kw, pw = _f32(kw)
        lib().orc_adjoint(self.h, _ptr(X), _ptr(smap), _ptr(data), px, py, pz, pw, kx.size)
        return X

    def adjoint_sos(self, X, data, kx, ky, kz, kw):
        """gridFFT::forward_sos: X += |deapp(ifft(grid(data*kw)))|^2."""
        X = self._c(X)
        assert X.flags.writeable
        data = self._c(data)
        kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz); kw, pw = _f32(kw)
        lib().orc_adjoint_sos(self.h, _ptr(X), _ptr(data), px, py, pz, pw, kx.size)
        return X

    def set_k_rad(self, k_rad):
        """The public gridFFT::k_rad field (taper radius of E^H)."""
        lib().orc_set_k_rad(self.h, k_rad)

    def forward(self, X, smap, kx, ky, kz, kw, diff=None):
        """gridFFT::backward (E), or backward_residual when diff is given."""
        X, smap, diff = self._c(X), self._c(smap), self._c(diff)
        kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz); kw, pw = _f32(kw)
        out = np.zeros(kx.size, self.cdt)
        lib().orc_forward(self.h, _ptr(X), _ptr(smap), _ptr(out), px, py, pz, pw, kx.size, _ptr(diff))
        return out

    # stage access
    def grid(self, data, kx, ky, kz, kw):
        data = self._c(data)
        kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz); kw, pw = _f32(kw)
        lib().orc_grid(self.h, _ptr(data), px, py, pz, pw, kx.size)
        return self.get_grid()

    def ungrid(self, grid, kx, ky, kz, kw, diff=None):
        self.set_grid(grid)
        diff = self._c(diff)
        kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz); kw, pw = _f32(kw)
        out = np.zeros(kx.size, self.cdt)
        lib().orc_ungrid(self.h, _ptr(out), px, py, pz, pw, kx.size, _ptr(diff))
        return out

    def get_grid(self):
        g = np.zeros(self.gshape, self.cdt)
        lib().orc_get_grid(self.h, _ptr(g))
        return g

    def set_grid(self, g):
        g = self._c(g).reshape(self.gshape)
        lib().orc_set_grid(self.h, _ptr(g))

    def set_image(self, X, smap):
        X, smap = self._c(X), self._c(smap)
        lib().orc_set_image(self.h, _ptr(X), _ptr(smap))
        return self.get_grid()

    def values_at(self, X, smap, kx, ky, kz):
        """FP64 plans: E X (one coil, no kw test) at float64 positions, for finite differences."""
        assert self.prec == 1
        self.set_image(X, smap)
        lib().orc_fft3(self.h, -1)
        k = [np.ascontiguousarray(v, dtype=np.float64) for v in (kx, ky, kz)]
        out = np.zeros(k[0].size, np.complex128)
        dp = ctypes.POINTER(ctypes.c_double)
        lib().orc_values_at(self.h, k[0].ctypes.data_as(dp), k[1].ctypes.data_as(dp), k[2].ctypes.data_as(dp),
                            k[0].size, _ptr(out))
        return out

    def accumulate(self, grid, X, smap):
        self.set_grid(grid)
        X, smap = self._c(X), self._c(smap)
        lib().orc_accumulate(self.h, _ptr(X), _ptr(smap))
        return X

    def fft3(self, grid, direction):
        self.set_grid(grid)
        lib().orc_fft3(self.h, int(direction))
        return self.get_grid()

    # solvers ---------------------------------------------------------------
    def _frames(self, frames, smaps, ncoil=None):
        """frames: list of dicts with kx, ky, kz, kw (float32, M) and data (C, M); smaps None
        (no maps, ncoil coils) or a list of C maps."""
        C = len(smaps) if smaps is not None else ncoil
        keep = []
        Nt = len(frames)
        arrs = {k: (ctypes.c_void_p * Nt)() for k in ("kx", "ky", "kz", "kw")}
        Ms = (ctypes.c_long * Nt)()
        datas = (ctypes.c_void_p * (Nt * C))()
        for t, fr in enumerate(frames):
            for k in ("kx", "ky", "kz", "kw"):
                a = np.ascontiguousarray(fr[k], dtype=np.float32)
                keep.append(a)
                arrs[k][t] = a.ctypes.data
            Ms[t] = keep[-1].size
            for c in range(C):
                d = self._c(fr["data"][c])
                keep.append(d)
                datas[t * C + c] = d.ctypes.data
        sm = (ctypes.c_void_p * C)()
        for c in range(C if smaps is not None else 0):
            s = self._c(smaps[c])
            keep.append(s)
            sm[c] = s.ctypes.data
        F = _Frames(Nt, C, ctypes.cast(arrs["kx"], ctypes.c_void_p), ctypes.cast(arrs["ky"], ctypes.c_void_p),
                    ctypes.cast(arrs["kz"], ctypes.c_void_p), ctypes.cast(arrs["kw"], ctypes.c_void_p),
                    ctypes.cast(Ms, ctypes.c_void_p), ctypes.cast(datas, ctypes.c_void_p), ctypes.cast(sm, ctypes.c_void_p))
        keep += [arrs, Ms, datas, sm]
        return F, keep

    def normal(self, frames, smaps, t, X):
        F, keep = self._frames(frames, smaps)
        X = self._c(X)
        out = np.zeros(self.ishape, self.cdt)
        lib().orc_normal(self.h, ctypes.byref(F), t, _ptr(X), _ptr(out))
        return out

    def cg(self, frames, smaps, iters):
        F, keep = self._frames(frames, smaps)
        Nt = len(frames)
        X = [np.zeros(self.ishape, self.cdt) for _ in range(Nt)]
        Xp = (ctypes.c_void_p * Nt)(*[x.ctypes.data for x in X])
        resid = np.zeros(max(iters, 1), np.float64)
        lib().orc_cg(self.h, ctypes.byref(F), iters, Xp, resid.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return X, resid[:iters]

    def fista(self, frames, smaps, params):
        F, keep = self._frames(frames, smaps)
        Nt = len(frames)
        X = [np.zeros(self.ishape, self.cdt) for _ in range(Nt)]
        Xp = (ctypes.c_void_p * Nt)(*[x.ctypes.data for x in X])
        n = max(params.max_iter, 1)
        resid = np.zeros(n, np.float64)
        thr = np.zeros(n, np.float32)
        step = ctypes.c_float()
        lib().orc_fista(self.h, ctypes.byref(F), ctypes.byref(params), Xp, resid.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                        ctypes.byref(step), thr.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return X, resid[:params.max_iter], step.value, thr[:params.max_iter]


    def clear(self, frames, params):
        """CLEAR (recon_lib.cpp:1025-1238) without coil maps: returns the coil images
        (T, C, Nz, Ny, Nx), the combined images (T, Nz, Ny, Nx), sum |R|^2 per iteration
        and the number of iterations run."""
        C = len(frames[0]["data"])
        F, keep = self._frames(frames, None, C)
        Nt = len(frames)
        XX = np.zeros((Nt, C) + self.ishape, self.cdt)
        im = np.zeros((Nt,) + self.ishape, self.cdt)
        xp = (ctypes.c_void_p * (Nt * C))(*[XX[t, c].ctypes.data for t in range(Nt) for c in range(C)])
        ip_ = (ctypes.c_void_p * Nt)(*[im[t].ctypes.data for t in range(Nt)])
        resid = np.zeros(max(params.max_iter, 1), np.float64)
        done = lib().orc_clear(self.h, ctypes.byref(F), ctypes.byref(params), xp, ip_,
                               resid.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return XX, im, resid[:done], done


def _coil_ptrs(XX):
    T, C = XX.shape[:2]
    return (ctypes.c_void_p * (T * C))(*[XX[t, c].ctypes.data for t in range(T) for c in range(C)])


def clear_update_threshold(XX, bs, amp=4.0, t2=6.0, iteration=0):
    """LOWRANKCOIL::update_threshold(image, 2, iteration) on coil images (T, C, Nz, Ny, Nx)."""
    XX = np.ascontiguousarray(XX)
    T, C, Nz, Ny, Nx = XX.shape
    prec = 1 if XX.dtype == np.complex128 else 0
    return lib().orc_clear_update_threshold(_coil_ptrs(XX), T, C, _ip((Nx, Ny, Nz)), _ip(bs), amp, t2, iteration, prec)


def clear_thresh(XX, bs, block_iter, alpha, smax, rand_skip):
    """LOWRANKCOIL::thresh(image, 2) on a copy of coil images (T, C, Nz, Ny, Nx)."""
    XX = np.ascontiguousarray(XX).copy()
    T, C, Nz, Ny, Nx = XX.shape
    prec = 1 if XX.dtype == np.complex128 else 0
    lib().orc_clear_thresh(_coil_ptrs(XX), T, C, _ip((Nx, Ny, Nz)), _ip(bs), block_iter, alpha, smax, rand_skip, prec)
    return XX


def clear_combine(XX, bs, out=None):
    """LOWRANKCOIL::combine of coil images (T, C, Nz, Ny, Nx) into (T, Nz, Ny, Nx)."""
    XX = np.ascontiguousarray(XX)
    T, C, Nz, Ny, Nx = XX.shape
    prec = 1 if XX.dtype == np.complex128 else 0
    im = np.zeros((T, Nz, Ny, Nx), XX.dtype) if out is None else np.ascontiguousarray(out, XX.dtype).copy()
    ip_ = (ctypes.c_void_p * T)(*[im[t].ctypes.data for t in range(T)])
    lib().orc_clear_combine(_coil_ptrs(XX), T, C, _ip((Nx, Ny, Nz)), _ip(bs), ip_, prec)
    return im


def espirit(images, kr_f=(3.0, 3.0, 3.0), cr=(12, 12, 12), svd_thresh=0.01, square=False):
    """ESPIRiT maps (spirit.cpp) from coil images (C, Nz, Ny, Nx) complex64: returns the maps
    (C, Nz, Ny, Nx) complex128, the number of kernel vectors kept, the calibration
    singular values (descending) and per voxel (s_2 / s_1)^2 of A_x (how well defined
    the dominant vector is)."""
    images = np.ascontiguousarray(images, dtype=np.complex64)
    C, Nz, Ny, Nx = images.shape
    maps = np.zeros(images.shape, np.complex128)
    ip_ = (ctypes.c_void_p * C)(*[images[c].ctypes.data for c in range(C)])
    mp = (ctypes.c_void_p * C)(*[maps[c].ctypes.data for c in range(C)])
    sv = np.zeros(200000, np.float64)
    kf = (ctypes.c_float * 3)(*kr_f)
    ratio = np.zeros((Nz, Ny, Nx), np.float64)
    nV = lib().orc_espirit(ip_, C, _ip((Nx, Ny, Nz)), kf, _ip(cr), svd_thresh, int(bool(square)), mp,
                           sv.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                           ratio.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return maps, nV, sv[sv > 0], ratio


def fft1d(x, sign, prec=1):
    x = np.ascontiguousarray(x, dtype=np.complex128 if prec else np.complex64).copy()
    lib().orc_fft1d(x.size, _ptr(x), int(sign), prec)
    return x


def wavelet(X, levels, shift, wtype=1, inverse=False):
    X = np.ascontiguousarray(X).copy()
    prec = 1 if X.dtype == np.complex128 else 0
    Nz, Ny, Nx = X.shape
    lib().orc_wavelet(Nx, Ny, Nz, _ip(levels), _ip(shift), wtype, _ptr(X), int(inverse), prec)
    return X


def wavelet_info(shape_xyz, levels, wtype=1):
    L = (ctypes.c_int * 3)()
    f = np.zeros(16, np.float32)
    lib().orc_wavelet_info(shape_xyz[0], shape_xyz[1], shape_xyz[2], _ip(levels), wtype, L, f.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    return tuple(L), f.reshape(4, 4)


def fraction_threshold(vols, fraction):
    prec = 1 if vols[0].dtype == np.complex128 else 0
    arr = (ctypes.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    return lib().orc_fraction_threshold(arr, len(vols), vols[0].size, fraction, prec)


def soft_threshold(X, value):
    X = np.ascontiguousarray(X).copy()
    prec = 1 if X.dtype == np.complex128 else 0
    lib().orc_soft_threshold(_ptr(X), X.size, value, prec)
    return X


def llr_update_threshold(vols, bs, amp=4.0, t2=6.0, iteration=0):
    prec = 1 if vols[0].dtype == np.complex128 else 0
    Nz, Ny, Nx = vols[0].shape
    arr = (ctypes.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    return lib().orc_llr_update_threshold(arr, len(vols), _ip((Nx, Ny, Nz)), _ip(bs), amp, t2, iteration, prec)


def llr_thresh(vols, bs, block_iter, alpha, smax, rand_skip):
    vols = [np.ascontiguousarray(v).copy() for v in vols]
    prec = 1 if vols[0].dtype == np.complex128 else 0
    Nz, Ny, Nx = vols[0].shape
    arr = (ctypes.c_void_p * len(vols))(*[v.ctypes.data for v in vols])
    lib().orc_llr_thresh(arr, len(vols), _ip((Nx, Ny, Nz)), _ip(bs), block_iter, alpha, smax, rand_skip, prec)
    return vols


def gaussian_blur(X, sigma):
    """gaussian_blur_template on one [Nz][Ny][Nx] complex volume (copy), sigma = (x, y, z)."""
    X = np.ascontiguousarray(X).copy()
    prec = 1 if X.dtype == np.complex128 else 0
    Nz, Ny, Nx = X.shape
    sig = (ctypes.c_float * 3)(*[float(v) for v in sigma])
    lib().orc_gaussian_blur(_ptr(X), Nx, Ny, Nz, sig, prec)
    return X


def sos_normalize(maps):
    """RECON::sos_normalize (smap_thresh == 0) on a [C][Nz][Ny][Nx] array (copy)."""
    maps = np.ascontiguousarray(maps).copy()
    prec = 1 if maps.dtype == np.complex128 else 0
    C = maps.shape[0]
    arr = (ctypes.c_void_p * C)(*[maps[c].ctypes.data for c in range(C)])
    lib().orc_sos_normalize(arr, C, maps[0].size, prec)
    return maps


def lowres_smaps(plan, data, kx, ky, kz, kw, smap_res=8.0, blur=(0.0, 0.0, 0.0)):
    """The LOWRES coil-map estimate with SOS normalisation (recon_lib.cpp:2694-2950):
    per coil, E^H without maps at k_rad = smap_res, Gaussian blur, then sos_normalize.
    data is [C][M]; returns [C][Nz][Ny][Nx] and restores k_rad = 9999."""
    plan.set_k_rad(smap_res)
    imgs = np.zeros((len(data),) + plan.ishape, plan.cdt)
    for c in range(len(data)):
        plan.adjoint(imgs[c], None, data[c], kx, ky, kz, kw)
        if any(b > 0 for b in blur):
            imgs[c] = gaussian_blur(imgs[c], blur)
    plan.set_k_rad(9999.0)
    return sos_normalize(imgs)


class DcfParams(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("dwin", ctypes.c_float), ("scale", ctypes.c_float),
                ("overgrid", ctypes.c_float), ("acc", ctypes.c_float), ("kernel", ctypes.c_int)]


def dcf_pipe(kx, ky, kz, N, iters=20, dwin=2.1, scale=1.0, overgrid=2.1, acc=1.0, kernel=0, prec=0):
    """RECON::dcf_calc (Pipe iteration with the DCFgridFFT polynomial kernel); returns kw (float32)."""
    if np.isscalar(N):
        N = (N, N, N)
    kx, px = _f32(kx); ky, py = _f32(ky); kz, pz = _f32(kz)
    q = DcfParams(iters, dwin, scale, overgrid, acc, kernel)
    out = np.zeros(kx.size, np.float32)
    lib().orc_dcf_pipe(px, py, pz, kx.size, N[0], N[1], N[2], ctypes.byref(q),
                       out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), prec)
    return out


def dcf_table(dwin=2.1, kernel=0):
    n = ctypes.c_int()
    lib().orc_dcf_table(dwin, kernel, None, ctypes.byref(n))
    out = np.zeros(n.value, np.float32)
    lib().orc_dcf_table(dwin, kernel, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), ctypes.byref(n))
    return out


def glibc_rand(skip, n):
    out = (ctypes.c_int * n)()
    lib().orc_glibc_rand(skip, n, out)
    return np.array(out[:], dtype=np.int64)


def pregate(gate_times, nread, t, kx, ky, kz, kw, data, rweight=None, reset_dens=False):
    """RECON::pregate_data for one frame (see orc_pregate): (kx, ky, kz, kw, data)."""
    gt = np.ascontiguousarray(gate_times, np.float64)
    rw = None if rweight is None else np.ascontiguousarray(rweight, np.float32)
    ks = [np.ascontiguousarray(v, np.float32) for v in (kx, ky, kz, kw)]
    d = np.ascontiguousarray(data, np.complex64).reshape(-1, ks[0].size)
    P = ctypes.c_void_p
    rwp = None if rw is None else P(rw.ctypes.data)
    n = lib().orc_pregate(P(gt.ctypes.data), rwp, gt.size, nread, t, int(reset_dens), *[P(k.ctypes.data) for k in ks],
                          P(d.ctypes.data), d.shape[0], ks[0].size, None, None, None, None, None, 0)
    outs = [np.empty(n, np.float32) for _ in range(4)]
    od = np.empty((d.shape[0], n), np.complex64)
    lib().orc_pregate(P(gt.ctypes.data), rwp, gt.size, nread, t, int(reset_dens), *[P(k.ctypes.data) for k in ks],
                      P(d.ctypes.data), d.shape[0], ks[0].size, *[P(o.ctypes.data) for o in outs], P(od.ctypes.data), n)
    return tuple(outs) + (od,)


def cg_vectors(X, R, P, L):
    """One CG iteration's vector updates (X, R, P updated in place; L read) on lists of
    (Nz, Ny, Nx) complex64 frames; returns sum |r|^2 after the update."""
    Nz = X[0].shape[0]
    n = X[0].size
    arr = lambda vs: (ctypes.c_void_p * len(vs))(*[v.ctypes.data for v in vs])
    prec = 1 if X[0].dtype == np.complex128 else 0
    return lib().orc_cg_vectors(len(X), n, Nz, arr(X), arr(R), arr(P), arr(L), prec)


def num_threads():
    return lib().orc_num_threads()
