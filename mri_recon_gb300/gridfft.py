"""Python mirror of the reference's gridFFT / RECON call surface over libmrg.

``Plan`` is the coil-batched operator (the reference's gridFFT_CoilThreaded plus
the CG / FISTA loops of RECON::full_recon); by default its transforms are normalised as
gridFFT's, and ``fft_norm=1`` with ``overgrid=1.375`` gives gridFFT_CoilThreaded's own
unnormalised transforms and default grid.  ``gridFFT`` keeps the per-coil
member functions and public fields of the reference class
(src/gridFFT.h:28-194) so code written against it ports line for line:

    g = gridFFT(); g.overgrid = 1.5; g.kernel_type = KAISER_KERNEL
    g.precalc_gridding(Nz, Ny, Nx)
    g.forward(X, smap, data, kx, ky, kz, kw)    # X += E^H (data * kw)
    g.backward(X, smap, data, kx, ky, kz, kw)   # data = E X

Arrays may be torch tensors (CUDA or CPU) or numpy arrays: complex64 images of
shape (Nz, Ny, Nx), complex64 k-space of M samples, float32 trajectories.
Device tensors are used in place; host arrays are staged by the library.
"""
import ctypes

import numpy as np

from . import _lib

TRIANGLE_KERNEL, KAISER_KERNEL, SINC_KERNEL, POLY_KERNEL = 0, 1, 2, 3

try:  # torch is plumbing for device memory and streams
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_tensor(a):
    return torch is not None and isinstance(a, torch.Tensor)


class _Args:
    """Keeps host arrays alive for the duration of a call and yields raw pointers."""

    def __init__(self):
        self.keep = []

    def ptr(self, a, dtype=None):
        if a is None:
            return None
        if _is_tensor(a):
            if not a.is_contiguous():
                a = a.contiguous()
                self.keep.append(a)
            return a.data_ptr()
        arr = np.ascontiguousarray(a, dtype=dtype) if dtype is not None else np.ascontiguousarray(a)
        self.keep.append(arr)
        return arr.ctypes.data


def _stream(stream=None):
    if stream is not None:
        return stream
    if torch is not None and torch.cuda.is_available():
        return torch.cuda.current_stream().cuda_stream
    return None


def _numel(a):
    return a.numel() if _is_tensor(a) else int(np.asarray(a).size)


class Plan:
    """Coil-batched gridFFT plan with ``ncoils`` coils and ``nframes`` trajectories.
    fft_norm=1: unnormalised FFT passes (gridFFT_CoilThreaded), E and E^H sqrt(Sx Sy Sz)
    times those of the default."""

    def __init__(self, N, ncoils=1, nframes=1, overgrid=1.5, dwin=-1.0, kernel_type=KAISER_KERNEL, k_rad=9999.0,
                 tile=0, max_pairs=0, time_grid=0, analytic_kernel=False, grid_mode=0, fft_norm=0):
        L = _lib.load()
        if np.isscalar(N):
            N = (N, N, N)
        self.N = tuple(int(n) for n in N)  # (Nx, Ny, Nz)
        self.ncoils, self.nframes = int(ncoils), int(nframes)
        cfg = _lib.MrgConfig()
        L.mrg_config_default(ctypes.byref(cfg))
        cfg.overgrid, cfg.dwin, cfg.kernel_type, cfg.k_rad = overgrid, dwin, kernel_type, k_rad
        cfg.tile, cfg.max_pairs, cfg.time_grid = tile, max_pairs, time_grid
        cfg.kernel_eval = 1 if analytic_kernel else 0
        cfg.grid_mode = grid_mode
        cfg.fft_norm = fft_norm
        h = ctypes.c_void_p()
        _lib.check(L.mrg_plan_create(ctypes.byref(cfg), self.N[0], self.N[1], self.N[2], self.ncoils, self.nframes,
                                     ctypes.byref(h)))
        self._h = h
        S = (ctypes.c_int * 3)()
        og = (ctypes.c_int * 3)()
        gr = (ctypes.c_float * 3)()
        be = (ctypes.c_float * 3)()
        dw = (ctypes.c_float * 3)()
        ll = ctypes.c_int()
        _lib.check(L.mrg_plan_info(h, S, og, gr, be, dw, ctypes.byref(ll)))
        self.S, self.og, self.grid_ratio, self.beta, self.dwin = tuple(S), tuple(og), tuple(gr), tuple(be), tuple(dw)
        self.lut_len = ll.value
        self.M = [0] * self.nframes
        self.k_rad = float(k_rad)

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mrg_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ishape(self):
        return (self.N[2], self.N[1], self.N[0])

    def tables(self):
        lut = np.zeros(3 * self.lut_len, np.float32)
        win = np.zeros(sum(self.S), np.float32)
        _lib.check(_lib.load().mrg_get_tables(self._h, lut.ctypes.data_as(_lib._fp), win.ctypes.data_as(_lib._fp)))
        s0, s1 = self.S[0], self.S[0] + self.S[1]
        return lut.reshape(3, self.lut_len), (win[:s0], win[s0:s1], win[s1:])

    # -- inputs ---------------------------------------------------------------
    def set_smaps(self, smaps, stream=None):
        """smaps: (C, Nz, Ny, Nx) complex64."""
        a = _Args()
        stride = _numel(smaps) // self.ncoils
        _lib.check(_lib.load().mrg_set_smaps(self._h, a.ptr(smaps, np.complex64), stride, _stream(stream)))

    def set_traj(self, frame, kx, ky, kz, kw, stream=None):
        a = _Args()
        M = _numel(kx)
        _lib.check(_lib.load().mrg_set_traj(self._h, frame, a.ptr(kx, np.float32), a.ptr(ky, np.float32),
                                            a.ptr(kz, np.float32), a.ptr(kw, np.float32), M, _stream(stream)))
        self.M[frame] = M

    def frame_info(self, frame, taps=False):
        """dict(M, nvalid, npairs, nitems[, ntaps]) of a frame after set_traj."""
        v = [ctypes.c_int64() for _ in range(5)]
        refs = [ctypes.byref(x) for x in v[:4]] + [ctypes.byref(v[4]) if taps else None]
        _lib.check(_lib.load().mrg_frame_info(self._h, frame, *refs))
        keys = ("M", "nvalid", "npairs", "nitems") + (("ntaps",) if taps else ())
        return dict(zip(keys, (x.value for x in v)))

    def frame_tuning(self, frame):
        out = (ctypes.c_int * 5)()
        ms = (ctypes.c_float * 2)()
        _lib.check(_lib.load().mrg_frame_tuning(self._h, frame, out, ms))
        return dict(ungrid_lanes=out[0], ungrid_samples_per_cta=out[1], grid_coils_per_pass=out[2],
                    ungrid_coils_per_lane=out[3], ungrid_rows_per_step=out[4], ungrid_ms=ms[0], grid_ms=ms[1])

    def set_frame_tuning(self, frame, ungrid_lanes, ungrid_samples_per_cta, grid_coils_per_pass,
                         ungrid_coils_per_lane, ungrid_rows_per_step=1):
        """Fixes a frame's launch shapes (the fields of frame_tuning) in place of the autotuner's."""
        v = (ctypes.c_int * 5)(ungrid_lanes, ungrid_samples_per_cta, grid_coils_per_pass, ungrid_coils_per_lane,
                               ungrid_rows_per_step)
        _lib.check(_lib.load().mrg_frame_set_tuning(self._h, frame, v))

    def fft_tuning(self):
        """Per FFT pass (E x, z, y; E^H y, z, x): lines per CTA and the persistent x-pass flag."""
        ib, xp = (ctypes.c_int * 6)(), (ctypes.c_int * 6)()
        _lib.check(_lib.load().mrg_fft_tuning(self._h, ib, xp))
        return dict(ib=list(ib), xp=list(xp))

    def set_fft_tuning(self, ib=None, xp=None):
        """Fixes the FFT launch shapes (see fft_tuning); None leaves that field as it is."""
        a = None if ib is None else (ctypes.c_int * 6)(*ib)
        b = None if xp is None else (ctypes.c_int * 6)(*xp)
        _lib.check(_lib.load().mrg_set_fft_tuning(self._h, a, b))

    def set_data(self, frame, data, stream=None):
        """data: (C, M) complex64."""
        a = _Args()
        stride = _numel(data) // self.ncoils
        _lib.check(_lib.load().mrg_set_data(self._h, frame, a.ptr(data, np.complex64), stride, _stream(stream)))

    # -- operators ------------------------------------------------------------
    def adjoint(self, frame, data, X, stream=None):
        """X += sum_c E_c^H (data_c * kw)   (gridFFT::forward).  Returns X."""
        a = _Args()
        stride = _numel(data) // self.ncoils
        if not _is_tensor(X):
            X = np.ascontiguousarray(X, dtype=np.complex64)
        _lib.check(_lib.load().mrg_adjoint(self._h, frame, a.ptr(data, np.complex64), stride, a.ptr(X),
                                           _stream(stream)))
        return X

    def forward(self, frame, X, out=None, diff=None, stream=None):
        """data_c = E_c X (- diff_c)   (gridFFT::backward / backward_residual).  Returns (C, M)."""
        a = _Args()
        M = self.M[frame]
        if out is None:
            if _is_tensor(X) and X.is_cuda:
                out = torch.empty((self.ncoils, M), dtype=torch.complex64, device=X.device)
            else:
                out = np.zeros((self.ncoils, M), np.complex64)
        _lib.check(_lib.load().mrg_forward(self._h, frame, a.ptr(X, np.complex64), a.ptr(out), M,
                                           a.ptr(diff, np.complex64), _stream(stream)))
        return out

    def normal(self, frame, X, out=None, stream=None):
        a = _Args()
        if out is None:
            if _is_tensor(X) and X.is_cuda:
                out = torch.empty(self.ishape, dtype=torch.complex64, device=X.device)
            else:
                out = np.zeros(self.ishape, np.complex64)
        _lib.check(_lib.load().mrg_normal(self._h, frame, a.ptr(X, np.complex64), a.ptr(out), _stream(stream)))
        return out

    def adjoint_coil(self, frame, smap, data, X, stream=None):
        a = _Args()
        _lib.check(_lib.load().mrg_adjoint_coil(self._h, frame, a.ptr(smap, np.complex64), a.ptr(data, np.complex64),
                                                a.ptr(X), _stream(stream)))
        return X

    def forward_coil(self, frame, X, smap, out, diff=None, stream=None):
        a = _Args()
        _lib.check(_lib.load().mrg_forward_coil(self._h, frame, a.ptr(X, np.complex64), a.ptr(smap, np.complex64),
                                                a.ptr(out), a.ptr(diff, np.complex64), _stream(stream)))
        return out

    def grid(self, frame, data, out=None, stream=None):
        """chop_grid_forward of data_c * kw onto a (Sz, Sy, Sx, C) grid (every point written)."""
        a = _Args()
        stride = _numel(data) // self.ncoils
        gshape = (self.S[2], self.S[1], self.S[0], self.ncoils)
        if out is None:
            if _is_tensor(data) and data.is_cuda:
                out = torch.empty(gshape, dtype=torch.complex64, device=data.device)
            else:
                out = np.zeros(gshape, np.complex64)
        _lib.check(_lib.load().mrg_grid(self._h, frame, a.ptr(data, np.complex64), stride, a.ptr(out),
                                        _stream(stream)))
        return out

    def ungrid(self, frame, grid, out=None, diff=None, stream=None):
        """chop_grid_backward from a (Sz, Sy, Sx, C) grid: (C, M) samples (minus diff)."""
        a = _Args()
        M = self.M[frame]
        if out is None:
            if _is_tensor(grid) and grid.is_cuda:
                out = torch.empty((self.ncoils, M), dtype=torch.complex64, device=grid.device)
            else:
                out = np.zeros((self.ncoils, M), np.complex64)
        _lib.check(_lib.load().mrg_ungrid(self._h, frame, a.ptr(grid, np.complex64), a.ptr(out), M,
                                          a.ptr(diff, np.complex64), _stream(stream)))
        return out

    def set_k_rad(self, k_rad, stream=None):
        """The public gridFFT::k_rad field: radius of E^H's Gaussian taper, every frame."""
        _lib.check(_lib.load().mrg_set_k_rad(self._h, float(k_rad), _stream(stream)))
        self.k_rad = float(k_rad)

    def _new_images(self, like, n):
        shape = ((n,) if n else ()) + self.ishape
        if _is_tensor(like) and like.is_cuda:
            return torch.zeros(shape, dtype=torch.complex64, device=like.device)
        return np.zeros(shape, np.complex64)

    def adjoint_coils(self, frame, data, images=None, stream=None):
        """images[c] += E_c^H (data_c * kw) without maps, one image per coil
        (gridFFT::forward without smap).  data is (C, M); returns (C,) + ishape."""
        a = _Args()
        if images is None:
            images = self._new_images(data, self.ncoils)
        elif not _is_tensor(images):
            images = np.ascontiguousarray(images, dtype=np.complex64)
        stride = _numel(data) // self.ncoils
        _lib.check(_lib.load().mrg_adjoint_coils(self._h, frame, a.ptr(data, np.complex64), stride, a.ptr(images),
                                                 _numel(images) // self.ncoils, _stream(stream)))
        return images

    def adjoint_sos(self, frame, data, X=None, stream=None):
        """X += sum_c |deapp(E_c^H (data_c * kw))|^2 (gridFFT::forward_sos over coils)."""
        a = _Args()
        if X is None:
            X = self._new_images(data, 0)
        elif not _is_tensor(X):
            X = np.ascontiguousarray(X, dtype=np.complex64)
        stride = _numel(data) // self.ncoils
        _lib.check(_lib.load().mrg_adjoint_sos(self._h, frame, a.ptr(data, np.complex64), stride, a.ptr(X),
                                               _stream(stream)))
        return X

    def lowres_smaps(self, frame, data, smap_res=8.0, blur=(0.0, 0.0, 0.0), stream=None):
        """Low-resolution, SOS-normalised coil maps from this frame's data; they become the
        plan's maps and are returned as (C,) + ishape."""
        a = _Args()
        out = self._new_images(data, self.ncoils)
        b = (ctypes.c_float * 3)(*[float(v) for v in blur])
        stride = _numel(data) // self.ncoils
        _lib.check(_lib.load().mrg_lowres_smaps(self._h, frame, a.ptr(data, np.complex64), stride, float(smap_res), b,
                                                a.ptr(out), _numel(out) // self.ncoils, _stream(stream)))
        return out

    def fft3(self, grid, sign=-1, stream=None):
        """do_fft (sign -1) / do_ifft (sign +1) of a grid (Sz, Sy, Sx, ncoils), unpruned, in place."""
        a = _Args()
        _lib.check(_lib.load().mrg_fft3(self._h, a.ptr(grid), int(sign), _stream(stream)))
        return grid

    def espirit_smaps(self, frame, data, params=None, blur=None, stream=None):
        """ESPIRiT maps from one frame's k-space (the ESPIRIT branch of calc_sensitivity_maps);
        they become the plan's maps.  Returns (maps (ncoils, Nz, Ny, Nx), kernel vectors kept)."""
        a = _Args()
        params = params if params is not None else espirit_params()
        d = data if _is_tensor(data) else np.ascontiguousarray(data, dtype=np.complex64)
        M = _numel(d) // self.ncoils
        out = self._new_images(d, self.ncoils)
        bl = (ctypes.c_float * 3)(*blur) if blur is not None else None
        kept = ctypes.c_int()
        _lib.check(_lib.load().mrg_espirit_smaps(self._h, frame, a.ptr(d), M, ctypes.byref(params), bl, a.ptr(out),
                                                 _numel(out) // self.ncoils, ctypes.byref(kept), _stream(stream)))
        return out, kept.value

    def grad(self, frame, X, y, stream=None):
        """loss = sum_c ||E_c X - y_c||^2, grad_x = 2 E^*(E X - y), grad_k = dloss/dk [3, M].

        Device tensors in, device tensors out (host arrays in, numpy out)."""
        a = _Args()
        M = self.M[frame]
        if _is_tensor(X) and X.is_cuda:
            gx = torch.empty(self.ishape, dtype=torch.complex64, device=X.device)
            gk = torch.empty((3, M), dtype=torch.float32, device=X.device)
        else:
            gx = np.zeros(self.ishape, np.complex64)
            gk = np.zeros((3, M), np.float32)
        loss = ctypes.c_double()
        gkp = gk.data_ptr() if _is_tensor(gk) else gk.ctypes.data
        _lib.check(_lib.load().mrg_grad(self._h, frame, a.ptr(X, np.complex64), a.ptr(y, np.complex64), M,
                                        ctypes.byref(loss), a.ptr(gx), ctypes.cast(gkp, _lib._fp), _stream(stream)))
        return loss.value, gx, gk

    # -- solvers --------------------------------------------------------------
    def cg(self, iters, X=None, use_graph=True, stream=None):
        """SENSE-CG from x0 = 0.  Returns (X (nframes, Nz, Ny, Nx), residual history)."""
        a = _Args()
        if X is None:
            if torch is not None and torch.cuda.is_available():
                X = torch.empty((self.nframes,) + self.ishape, dtype=torch.complex64, device="cuda")
            else:
                X = np.zeros((self.nframes,) + self.ishape, np.complex64)
        resid = np.zeros(max(iters, 1), np.float64)
        _lib.check(_lib.load().mrg_cg(self._h, iters, a.ptr(X), resid.ctypes.data_as(_lib._dp), int(bool(use_graph)),
                                      _stream(stream)))
        return X, resid[:iters]

    def cg_init(self, max_iter, X, stream=None):
        """X (device tensor, nframes images) = 0; R = P = E^H W d."""
        _lib.check(_lib.load().mrg_cg_init(self._h, max_iter, X.data_ptr(), _stream(stream)))

    def cg_iterate(self, n, X, use_graph=True, stream=None):
        _lib.check(_lib.load().mrg_cg_iterate(self._h, n, X.data_ptr(), int(bool(use_graph)), _stream(stream)))

    def cg_residuals(self, n, stream=None):
        r = np.zeros(max(n, 1), np.float64)
        _lib.check(_lib.load().mrg_cg_residuals(self._h, r.ctypes.data_as(_lib._dp), n, _stream(stream)))
        return r[:n]

    def set_timing(self, on):
        _lib.check(_lib.load().mrg_set_timing(self._h, int(bool(on))))

    def timings(self):
        """Accumulated per-stage ms since the last read: (E[4], E^H[4]), number of E calls."""
        out = np.zeros(8, np.float32)
        calls = ctypes.c_int()
        _lib.check(_lib.load().mrg_last_timings(self._h, out.ctypes.data_as(_lib._fp), ctypes.byref(calls)))
        return out, calls.value

    def fista(self, params, X=None, use_graph=True, stream=None):
        a = _Args()
        if X is None:
            if torch is not None and torch.cuda.is_available():
                X = torch.empty((self.nframes,) + self.ishape, dtype=torch.complex64, device="cuda")
            else:
                X = np.zeros((self.nframes,) + self.ishape, np.complex64)
        n = max(params.max_iter, 1)
        resid = np.zeros(n, np.float64)
        step = ctypes.c_float()
        _lib.check(_lib.load().mrg_fista(self._h, ctypes.byref(params), a.ptr(X), resid.ctypes.data_as(_lib._dp),
                                         ctypes.byref(step), int(bool(use_graph)), _stream(stream)))
        return X, resid[:self.last_iterations()], step.value

    def last_iterations(self):
        """Iterations the last cg / fista / clear call ran (fewer than max_iter after an early stop)."""
        n = ctypes.c_int()
        _lib.check(_lib.load().mrg_last_iterations(self._h, ctypes.byref(n)))
        return n.value

    def set_wait_limit(self, seconds):
        """Limit of each bounded device-side wait (default 2 s); 0 gives up after the first try."""
        _lib.check(_lib.load().mrg_set_wait_limit(self._h, float(seconds)))

    def check(self, stream=None):
        """Waits for the stream; raises MrgError (MRG_ERR_TIMEOUT) if a bounded wait ran out since
        the last report."""
        _lib.check(_lib.load().mrg_plan_check(self._h, _stream(stream)))


    def clear(self, params, X=None, coil_images=None, stream=None):
        """CLEAR (RECON CLEAR recon_type): returns the combined images X (nframes, Nz, Ny, Nx),
        the residual energy per iteration run, and coil_images (nframes, Nz, Ny, Nx, ncoils)
        when an array or True is passed for it (None: not returned)."""
        a = _Args()
        if X is None:
            X = self._new_images(None, self.nframes)
        if coil_images is True:
            shape = (self.nframes,) + self.ishape + (self.ncoils,)
            if _is_tensor(X) and X.is_cuda:
                coil_images = torch.empty(shape, dtype=torch.complex64, device=X.device)
            else:
                coil_images = np.zeros(shape, np.complex64)
        resid = np.zeros(max(params.max_iter, 1), np.float64)
        iters = ctypes.c_int()
        _lib.check(_lib.load().mrg_clear(self._h, ctypes.byref(params), a.ptr(X),
                                         a.ptr(coil_images) if coil_images is not None else None,
                                         resid.ctypes.data_as(_lib._dp), ctypes.byref(iters), _stream(stream)))
        if coil_images is None:
            return X, resid[:iters.value]
        return X, resid[:iters.value], coil_images


if torch is not None:
    class NufftLoss(torch.autograd.Function):
        """loss = sum_c ||E_c(x, k) - y_c||^2 as a torch autograd function of the image x
        (complex64, (Nz, Ny, Nx)) and the trajectory k (float32, (3, M)); gradients from
        mrg_grad.  `plan` is a Plan whose frame 0 is re-pointed at k on every call with
        unit weights (kw = 1)."""

        @staticmethod
        def forward(ctx, x, k, y, plan):
            kw = torch.ones(k.shape[1], dtype=torch.float32, device=k.device)
            plan.set_traj(0, k[0].contiguous(), k[1].contiguous(), k[2].contiguous(), kw)
            loss, gx, gk = plan.grad(0, x.contiguous(), y.contiguous())
            ctx.save_for_backward(gx, gk)
            return torch.tensor(loss, dtype=torch.float64, device=x.device)

        @staticmethod
        def backward(ctx, g):
            gx, gk = ctx.saved_tensors
            gf = g.to(torch.float32)
            return gx * gf, gk * gf, None, None


def gaussian_blur(X, sigma, stream=None):
    """gaussian_blur of one volume (Nz, Ny, Nx) or a stack (n, Nz, Ny, Nx), in place; returns X."""
    a = _Args()
    if not _is_tensor(X):
        X = np.ascontiguousarray(X, dtype=np.complex64)
    shape = tuple(X.shape)
    nvol = 1 if len(shape) == 3 else int(np.prod(shape[:-3]))
    Nz, Ny, Nx = shape[-3:]
    sig = (ctypes.c_float * 3)(*[float(v) for v in sigma])
    _lib.check(_lib.load().mrg_gaussian_blur(a.ptr(X), nvol, Nx, Ny, Nz, Nx * Ny * Nz, sig, _stream(stream)))
    return X


def sos_normalize(maps, stream=None):
    """RECON::sos_normalize on (C, Nz, Ny, Nx) maps, in place; returns maps."""
    a = _Args()
    if not _is_tensor(maps):
        maps = np.ascontiguousarray(maps, dtype=np.complex64)
    C = int(maps.shape[0])
    n = _numel(maps) // C
    _lib.check(_lib.load().mrg_sos_normalize(a.ptr(maps), C, n, n, _stream(stream)))
    return maps


def dcf_pipe(kx, ky, kz, N, stream=None, **params):
    """Pipe density compensation (RECON::dcf_calc) for one encode's trajectory; returns kw
    (a device tensor for device input, numpy otherwise).  params: iters, dwin, scale,
    overgrid, acc, kernel (the reference's -dcf_* flags)."""
    a = _Args()
    if np.isscalar(N):
        N = (N, N, N)
    q = _lib.MrgDcfParams()
    _lib.load().mrg_dcf_params_default(ctypes.byref(q))
    for k, v in params.items():
        setattr(q, k, v)
    M = _numel(kx)
    if _is_tensor(kx) and kx.is_cuda:
        out = torch.empty(M, dtype=torch.float32, device=kx.device)
    else:
        out = np.zeros(M, np.float32)
    _lib.check(_lib.load().mrg_dcf_pipe(a.ptr(kx, np.float32), a.ptr(ky, np.float32), a.ptr(kz, np.float32), M,
                                        int(N[0]), int(N[1]), int(N[2]), ctypes.byref(q), a.ptr(out),
                                        _stream(stream)))
    return out


def _coil_stack(XX):
    """(nframes, Nz, Ny, Nx, ncoils) complex64 stack -> (array, nframes, ncoils, Nx, Ny, Nz)."""
    if not _is_tensor(XX):
        XX = np.ascontiguousarray(XX, dtype=np.complex64)
    T, Nz, Ny, Nx, C = (int(v) for v in XX.shape)
    return XX, T, C, Nx, Ny, Nz


def clear_update_threshold(XX, block=(4, 4, 4), clear_amp=4.0, clear_t2=6.0, iteration=0, stream=None):
    """LOWRANKCOIL::update_threshold(image, 2, iteration) on a coil stack (nframes, Nz, Ny, Nx, ncoils)."""
    a = _Args()
    XX, T, C, Nx, Ny, Nz = _coil_stack(XX)
    smax = ctypes.c_float()
    _lib.check(_lib.load().mrg_clear_update_threshold(a.ptr(XX), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*block),
                                                      clear_amp, clear_t2, iteration, ctypes.byref(smax),
                                                      _stream(stream)))
    return smax.value


def clear_thresh(XX, smax, block=(4, 4, 4), block_iter=4, alpha=0.01, rand_skip=0, stream=None):
    """LOWRANKCOIL::thresh(image, 2) in place on a coil stack (nframes, Nz, Ny, Nx, ncoils); returns it."""
    a = _Args()
    XX, T, C, Nx, Ny, Nz = _coil_stack(XX)
    _lib.check(_lib.load().mrg_clear_thresh(a.ptr(XX), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*block), block_iter,
                                            alpha, smax, rand_skip, _stream(stream)))
    return XX


def clear_combine(XX, block=(4, 4, 4), out=None, stream=None):
    """LOWRANKCOIL::combine of a coil stack (nframes, Nz, Ny, Nx, ncoils) into (nframes, Nz, Ny, Nx)."""
    a = _Args()
    XX, T, C, Nx, Ny, Nz = _coil_stack(XX)
    if out is None:
        if _is_tensor(XX):
            out = torch.zeros(XX.shape[:-1], dtype=torch.complex64, device=XX.device)
        else:
            out = np.zeros(XX.shape[:-1], np.complex64)
    _lib.check(_lib.load().mrg_clear_combine(a.ptr(XX), T, C, Nx, Ny, Nz, (ctypes.c_int * 3)(*block), a.ptr(out),
                                             _stream(stream)))
    return out


def espirit_params(kernel_radius=None, calib_radius=None, svd_thresh=None, square=None):
    """SPIRIT options (-sp_kr_f / -sp_cr as scalars set all three axes)."""
    p = _lib.MrgEspiritParams()
    _lib.load().mrg_espirit_params_default(ctypes.byref(p))
    if kernel_radius is not None:
        p.kernel_radius[:] = [float(v) for v in (kernel_radius if not np.isscalar(kernel_radius) else (kernel_radius,) * 3)]
    if calib_radius is not None:
        p.calib_radius[:] = [int(v) for v in (calib_radius if not np.isscalar(calib_radius) else (calib_radius,) * 3)]
    if svd_thresh is not None:
        p.svd_thresh = svd_thresh
    if square is not None:
        p.square = int(bool(square))
    return p


def espirit(images, params=None, sv_cap=0, stream=None):
    """ESPIRiT maps from coil images (Nz, Ny, Nx, ncoils) complex64, coil innermost: returns
    (maps of the same shape, kernel vectors kept, the first sv_cap calibration singular values)."""
    a = _Args()
    if not _is_tensor(images):
        images = np.ascontiguousarray(images, dtype=np.complex64)
    Nz, Ny, Nx, C = (int(v) for v in images.shape)
    params = params if params is not None else espirit_params()
    if _is_tensor(images):
        maps = torch.empty_like(images)
    else:
        maps = np.zeros(images.shape, np.complex64)
    kept = ctypes.c_int()
    sv = np.zeros(max(sv_cap, 1), np.float64)
    _lib.check(_lib.load().mrg_espirit(a.ptr(images), C, Nx, Ny, Nz, ctypes.byref(params), a.ptr(maps),
                                       ctypes.byref(kept), sv.ctypes.data_as(_lib._dp) if sv_cap else None, sv_cap,
                                       _stream(stream)))
    return maps, kept.value, sv[:sv_cap]


def clear_params(**kw):
    p = _lib.MrgClearParams()
    _lib.load().mrg_clear_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("block", "wave_levels"):
            getattr(p, k)[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def gate_weights(gate_times, kw, nread, frame, rweight=None):
    """kw times the frame weight rweight * (floor(gate_time) == frame) of each sample's readout
    (GATING::hist_weight); gate_times / rweight: one value per readout of nread samples."""
    gt = np.ascontiguousarray(gate_times, np.float64)
    rw = None if rweight is None else np.ascontiguousarray(rweight, np.float32)
    kw = np.ascontiguousarray(kw, np.float32)
    out = np.empty_like(kw)
    _lib.check(_lib.load().mrg_gate_weights(gt.ctypes.data, None if rw is None else rw.ctypes.data, gt.size, int(nread),
                                            int(frame), kw.ctypes.data, out.ctypes.data))
    return out


def pregate(gate_times, nread, frame, kx, ky, kz, kw, data=None, rweight=None, reset_dens=False):
    """RECON::pregate_data for one frame: (kx, ky, kz, kw, data) of the frame's samples, kw scaled
    by 1e6 / count (or 1 with reset_dens); data (C, M) complex64 or None."""
    L = _lib.load()
    gt = np.ascontiguousarray(gate_times, np.float64)
    rw = None if rweight is None else np.ascontiguousarray(rweight, np.float32)
    rwp = None if rw is None else rw.ctypes.data
    ks = [np.ascontiguousarray(v, np.float32) for v in (kx, ky, kz, kw)]
    n = ctypes.c_int64()
    _lib.check(L.mrg_pregate(gt.ctypes.data, rwp, gt.size, int(nread), int(frame), int(bool(reset_dens)), None, None,
                             None, None, None, 0, 0, None, None, None, None, None, 0, ctypes.byref(n)))
    outs = [np.empty(n.value, np.float32) for _ in range(4)]
    if data is not None:
        d = np.ascontiguousarray(data, np.complex64).reshape(-1, ks[0].size)
        od = np.empty((d.shape[0], n.value), np.complex64)
        dp, odp, C = d.ctypes.data, od.ctypes.data, d.shape[0]
    else:
        d = od = None
        dp = odp = None
        C = 0
    _lib.check(L.mrg_pregate(gt.ctypes.data, rwp, gt.size, int(nread), int(frame), int(bool(reset_dens)),
                             *[k.ctypes.data for k in ks], dp, C, ks[0].size, *[o.ctypes.data for o in outs], odp,
                             n.value, ctypes.byref(n)))
    return tuple(outs) + (od,)


class H5File:
    """The reference's k-space file (MRI_DATA::read_external_data layout) through the library's
    own HDF5 reader: attributes, datasets, and whole encodes loaded into a plan frame."""

    def __init__(self, path):
        h = ctypes.c_void_p()
        _lib.check(_lib.load().mrg_h5_open(str(path).encode(), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mrg_h5_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def attr_int(self, group, name):
        v = ctypes.c_int()
        _lib.check(_lib.load().mrg_h5_attr_int(self._h, group.encode(), name.encode(), ctypes.byref(v)))
        return v.value

    def info(self, path):
        """(dims in HDF5 order, is_complex)."""
        r, cx = ctypes.c_int(), ctypes.c_int()
        dims = (ctypes.c_int64 * 8)()
        _lib.check(_lib.load().mrg_h5_dataset_info(self._h, path.encode(), ctypes.byref(r), dims, ctypes.byref(cx)))
        return tuple(dims[:r.value]), bool(cx.value)

    def read(self, path):
        dims, cx = self.info(path)
        out = np.empty(dims, np.complex64 if cx else np.float32)
        _lib.check(_lib.load().mrg_h5_read(self._h, path.encode(), int(cx), out.ctypes.data, out.size))
        return out

    def mri_info(self):
        ne, nc = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().mrg_h5_mri_info(self._h, ctypes.byref(ne), ctypes.byref(nc), None, 0))
        m = (ctypes.c_int64 * max(ne.value, 1))()
        _lib.check(_lib.load().mrg_h5_mri_info(self._h, None, None, m, ne.value))
        return ne.value, nc.value, list(m[:ne.value])

    def load_encode(self, encode, plan, frame, stream=None):
        """KX/KY/KZ/KW_E<encode> and KData_E<encode>_C* into plan frame `frame` through pinned memory."""
        _lib.check(_lib.load().mrg_h5_load_encode(self._h, int(encode), plan._h, int(frame), _stream(stream)))
        plan.M[frame] = self.mri_info()[2][encode]


def fista_params(**kw):
    p = _lib.MrgFistaParams()
    _lib.load().mrg_fista_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k in ("wave_levels", "llr_block"):
            getattr(p, k)[:] = list(v)
        else:
            setattr(p, k, v)
    return p


class gridFFT:
    """Per-coil drop-in for the reference class gridFFT (src/gridFFT.h:28-194).

    Public fields set before precalc_gridding keep the reference names and
    defaults (src/gridFFT.cpp:28-60).  The trajectory passed to each call is
    uploaded and sorted once and re-used while the same arrays are passed.
    """

    def __init__(self):
        self.overgrid = 1.5
        self.kernel_type = KAISER_KERNEL
        self.dwinX = self.dwinY = self.dwinZ = -1.0
        self.k_rad = 9999.0
        self.time_grid = 0
        self._plan = None
        self._traj_key = None

    def precalc_gridding(self, Nz, Ny, Nx, data=None):
        if not (self.dwinX == self.dwinY == self.dwinZ):
            raise ValueError("anisotropic kernel widths are not supported")
        self._plan = Plan((Nx, Ny, Nz), 1, 1, overgrid=self.overgrid, dwin=self.dwinX, kernel_type=self.kernel_type,
                          k_rad=self.k_rad, time_grid=self.time_grid)
        p = self._plan
        self.Sx, self.Sy, self.Sz = p.S
        self.og_sx, self.og_sy, self.og_sz = p.og
        self.og_ex, self.og_ey, self.og_ez = (p.og[0] + Nx, p.og[1] + Ny, p.og[2] + Nz)
        self.grid_x, self.grid_y, self.grid_z = p.grid_ratio
        self.betaX, self.betaY, self.betaZ = p.beta
        self.dwinX, self.dwinY, self.dwinZ = p.dwin
        self.Nx, self.Ny, self.Nz = Nx, Ny, Nz

    def _traj(self, kx, ky, kz, kw):
        key = tuple((id(a), _numel(a)) for a in (kx, ky, kz, kw))
        if key != self._traj_key:
            self._plan.set_traj(0, kx, ky, kz, kw)
            self._traj_key = key
            self._traj_refs = (kx, ky, kz, kw)

    def _sync_k_rad(self):
        if self.k_rad != self._plan.k_rad:
            self._plan.set_k_rad(self.k_rad)

    def forward(self, X, smap, data, kx, ky, kz, kw):
        """X += E^H data (gridFFT::forward, src/gridFFT.cpp:791-812).  smap may be None."""
        self._traj(kx, ky, kz, kw)
        self._sync_k_rad()
        return self._plan.adjoint_coil(0, smap, data, X)

    def forward_sos(self, X, data, kx, ky, kz, kw):
        """X += |deapp(E^H data)|^2 (gridFFT::forward_sos, src/gridFFT.cpp:722-757)."""
        self._traj(kx, ky, kz, kw)
        self._sync_k_rad()
        return self._plan.adjoint_sos(0, data, X)

    def backward(self, X, smap, data, kx, ky, kz, kw):
        """data = E X (gridFFT::backward, src/gridFFT.cpp:824-844)."""
        self._traj(kx, ky, kz, kw)
        return self._plan.forward_coil(0, X, smap, data)

    def backward_residual(self, X, smap, data, kx, ky, kz, kw, diff_data):
        """data = E X - diff_data (gridFFT::backward_residual, src/gridFFT.cpp:856-876)."""
        self._traj(kx, ky, kz, kw)
        return self._plan.forward_coil(0, X, smap, data, diff=diff_data)
