"""GB300-native gridFFT / SENSE hot path of uwmri/mri_recon.

The compute path is libmrg.so (hand-written sm_103a CUDA kernels behind the C ABI
of include/mrg.h); this package is its Python binding and a mirror of the
reference's gridFFT / RECON call surface.
"""
from . import synth  # noqa: F401
from ._lib import LIB_PATH, MrgError, load  # noqa: F401
from .gridfft import (KAISER_KERNEL, POLY_KERNEL, SINC_KERNEL, TRIANGLE_KERNEL, Plan, clear_combine,  # noqa: F401
                      clear_params, clear_thresh, clear_update_threshold, dcf_pipe, espirit, espirit_params,
                      fista_params, gate_weights, gaussian_blur, gridFFT, H5File, pregate, sos_normalize)
