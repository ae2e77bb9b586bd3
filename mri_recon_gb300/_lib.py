"""ctypes binding of libmrg.so (include/mrg.h).

There is no fallback: if the CUDA library is missing or fails to load, every
entry point raises.  Build it with ``python -m mri_recon_gb300.build`` or
``__graft_entry__.build()``.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmrg.so")

MRG_OK = 0
STATUS = {0: "MRG_OK", 1: "MRG_ERR_INVALID", 2: "MRG_ERR_CUDA", 3: "MRG_ERR_NOMEM", 4: "MRG_ERR_STATE",
          5: "MRG_ERR_TIMEOUT", 6: "MRG_ERR_UNSUPPORTED"}

# Every function declared in include/mrg.h: name -> (restype, argtypes)
_vp = ctypes.c_void_p
_i = ctypes.c_int
_i64 = ctypes.c_int64
_f = ctypes.c_float
_ip = ctypes.POINTER(ctypes.c_int)
_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)


class MrgConfig(ctypes.Structure):
    _fields_ = [("overgrid", ctypes.c_float), ("dwin", ctypes.c_float), ("kernel_type", ctypes.c_int),
                ("k_rad", ctypes.c_float), ("time_grid", ctypes.c_int), ("tile", ctypes.c_int),
                ("max_pairs", ctypes.c_int), ("kernel_eval", ctypes.c_int), ("grid_mode", ctypes.c_int),
                ("fft_norm", ctypes.c_int)]


class MrgDcfParams(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_int), ("dwin", ctypes.c_float), ("scale", ctypes.c_float),
                ("overgrid", ctypes.c_float), ("acc", ctypes.c_float), ("kernel", ctypes.c_int)]


class MrgFistaParams(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("max_eig_iter", ctypes.c_int), ("fista", ctypes.c_int),
                ("cycle_spins", ctypes.c_int), ("wave_levels", ctypes.c_int * 3), ("wave_type", ctypes.c_int),
                ("thresh", ctypes.c_float), ("use_threshold", ctypes.c_int), ("llr_block", ctypes.c_int * 3),
                ("llr_block_iter", ctypes.c_int), ("llr_alpha", ctypes.c_float), ("clear_amp", ctypes.c_float),
                ("clear_t2", ctypes.c_float), ("rand_skip", ctypes.c_int64), ("early_stop_thresh", ctypes.c_float),
                ("early_stop_range", ctypes.c_int)]


class MrgClearParams(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("block", ctypes.c_int * 3), ("block_iter", ctypes.c_int),
                ("alpha_coil", ctypes.c_float), ("clear_amp", ctypes.c_float), ("clear_t2", ctypes.c_float),
                ("early_stop_thresh", ctypes.c_float), ("early_stop_range", ctypes.c_int), ("rand_skip", ctypes.c_int64),
                ("use_threshold", ctypes.c_int), ("thresh", ctypes.c_float), ("cycle_spins", ctypes.c_int),
                ("wave_levels", ctypes.c_int * 3), ("wave_type", ctypes.c_int)]


class MrgEspiritParams(ctypes.Structure):
    _fields_ = [("kernel_radius", ctypes.c_float * 3), ("calib_radius", ctypes.c_int * 3),
                ("svd_thresh", ctypes.c_float), ("square", ctypes.c_int)]


SIGNATURES = {
    "mrg_config_default": (None, [ctypes.POINTER(MrgConfig)]),
    "mrg_last_error": (ctypes.c_char_p, []),
    "mrg_plan_create": (_i, [ctypes.POINTER(MrgConfig), _i, _i, _i, _i, _i, ctypes.POINTER(_vp)]),
    "mrg_plan_destroy": (_i, [_vp]),
    "mrg_plan_info": (_i, [_vp, _ip, _ip, _fp, _fp, _fp, _ip]),
    "mrg_get_tables": (_i, [_vp, _fp, _fp]),
    "mrg_set_smaps": (_i, [_vp, _vp, _i64, _vp]),
    "mrg_set_traj": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _i64, _vp]),
    "mrg_set_data": (_i, [_vp, _i, _vp, _i64, _vp]),
    "mrg_frame_tuning": (_i, [_vp, _i, _ip, _fp]),
    "mrg_frame_set_tuning": (_i, [_vp, _i, _ip]),
    "mrg_fft_tuning": (_i, [_vp, _ip, _ip]),
    "mrg_set_fft_tuning": (_i, [_vp, _ip, _ip]),
    "mrg_frame_info": (_i, [_vp, _i] + [ctypes.POINTER(_i64)] * 5),
    "mrg_adjoint": (_i, [_vp, _i, _vp, _i64, _vp, _vp]),
    "mrg_forward": (_i, [_vp, _i, _vp, _vp, _i64, _vp, _vp]),
    "mrg_normal": (_i, [_vp, _i, _vp, _vp, _vp]),
    "mrg_adjoint_coil": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "mrg_forward_coil": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp]),
    "mrg_set_k_rad": (_i, [_vp, _f, _vp]),
    "mrg_adjoint_coils": (_i, [_vp, _i, _vp, _i64, _vp, _i64, _vp]),
    "mrg_adjoint_sos": (_i, [_vp, _i, _vp, _i64, _vp, _vp]),
    "mrg_lowres_smaps": (_i, [_vp, _i, _vp, _i64, _f, _fp, _vp, _i64, _vp]),
    "mrg_gaussian_blur": (_i, [_vp, _i, _i, _i, _i, _i64, _fp, _vp]),
    "mrg_sos_normalize": (_i, [_vp, _i, _i64, _i64, _vp]),
    "mrg_dcf_params_default": (None, [ctypes.POINTER(MrgDcfParams)]),
    "mrg_dcf_pipe": (_i, [_vp, _vp, _vp, _i64, _i, _i, _i, ctypes.POINTER(MrgDcfParams), _vp, _vp]),
    "mrg_cg": (_i, [_vp, _i, _vp, _dp, _i, _vp]),
    "mrg_fista_params_default": (None, [ctypes.POINTER(MrgFistaParams)]),
    "mrg_fista": (_i, [_vp, ctypes.POINTER(MrgFistaParams), _vp, _dp, _fp, _i, _vp]),
    "mrg_fft3": (_i, [_vp, _vp, _i, _vp]),
    "mrg_espirit_params_default": (None, [ctypes.POINTER(MrgEspiritParams)]),
    "mrg_espirit": (_i, [_vp, _i, _i, _i, _i, ctypes.POINTER(MrgEspiritParams), _vp, _ip, _dp, _i, _vp]),
    "mrg_espirit_smaps": (_i, [_vp, _i, _vp, _i64, ctypes.POINTER(MrgEspiritParams), _fp, _vp, _i64, _ip, _vp]),
    "mrg_clear_params_default": (None, [ctypes.POINTER(MrgClearParams)]),
    "mrg_clear": (_i, [_vp, ctypes.POINTER(MrgClearParams), _vp, _vp, _dp, _ip, _vp]),
    "mrg_clear_update_threshold": (_i, [_vp, _i, _i, _i, _i, _i, _ip, _f, _f, _i, _fp, _vp]),
    "mrg_clear_thresh": (_i, [_vp, _i, _i, _i, _i, _i, _ip, _i, _f, _f, _i64, _vp]),
    "mrg_clear_combine": (_i, [_vp, _i, _i, _i, _i, _i, _ip, _vp, _vp]),
    "mrg_wavelet": (_i, [_vp, _i, _i, _i, _i, _ip, _ip, _i, _i, _vp]),
    "mrg_fraction_threshold": (_i, [_vp, _i, _i64, _f, _fp, _vp]),
    "mrg_soft_threshold": (_i, [_vp, _i64, _f, _vp]),
    "mrg_llr_update_threshold": (_i, [_vp, _i, _i, _i, _i, _ip, _f, _f, _i, _fp, _vp]),
    "mrg_llr_thresh": (_i, [_vp, _i, _i, _i, _i, _ip, _i, _f, _f, _i64, _vp]),
    "mrg_llr_update_threshold_noalloc": (_i, [_vp, _i, _i, _i, _i, _ip, _f, _f, _i, _fp, _vp]),
    "mrg_plan_geometry": (_i, [ctypes.POINTER(MrgConfig), _i, _i, _i, _ip, _ip, _fp, _fp, _ip, _fp, _fp]),
    "mrg_rand_stream": (_i, [_i64, _i, _ip]),
    "mrg_grad": (_i, [_vp, _i, _vp, _vp, _i64, _dp, _vp, _fp, _vp]),
    "mrg_cg_init": (_i, [_vp, _i, _vp, _vp]),
    "mrg_cg_iterate": (_i, [_vp, _i, _vp, _i, _vp]),
    "mrg_cg_residuals": (_i, [_vp, _dp, _i, _vp]),
    "mrg_set_timing": (_i, [_vp, _i]),
    "mrg_last_timings": (_i, [_vp, _fp, _ip]),
    "mrg_kernel_launches": (_i64, []),
    "mrg_gate_weights": (_i, [_vp, _vp, _i64, _i, _i, _vp, _vp]),
    "mrg_pregate": (_i, [_vp, _vp, _i64, _i, _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _i64, _vp, _vp, _vp, _vp, _vp,
                         _i64, ctypes.POINTER(_i64)]),
    "mrg_h5_open": (_i, [ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "mrg_h5_close": (_i, [_vp]),
    "mrg_h5_attr_int": (_i, [_vp, ctypes.c_char_p, ctypes.c_char_p, _ip]),
    "mrg_h5_dataset_info": (_i, [_vp, ctypes.c_char_p, _ip, ctypes.POINTER(_i64), _ip]),
    "mrg_h5_read": (_i, [_vp, ctypes.c_char_p, _i, _vp, _i64]),
    "mrg_h5_mri_info": (_i, [_vp, _ip, _ip, ctypes.POINTER(_i64), _i]),
    "mrg_h5_load_encode": (_i, [_vp, _i, _vp, _i, _vp]),
    "mrg_grid": (_i, [_vp, _i, _vp, _i64, _vp, _vp]),
    "mrg_ungrid": (_i, [_vp, _i, _vp, _vp, _i64, _vp, _vp]),
    "mrg_set_wait_limit": (_i, [_vp, ctypes.c_double]),
    "mrg_plan_check": (_i, [_vp, _vp]),
    "mrg_last_iterations": (_i, [_vp, _ip]),
}

_lib = None


class MrgError(RuntimeError):
    pass


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MrgError("libmrg.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status):
    if status != MRG_OK:
        msg = load().mrg_last_error().decode(errors="replace")
        raise MrgError("%s: %s" % (STATUS.get(status, str(status)), msg))
