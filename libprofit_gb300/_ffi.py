"""ctypes binding of include/pf_cuda.h (the C ABI of libpfcuda.so).

The structures below mirror pf_profile_desc / pf_model_desc field for field.
Loading fails loudly when the CUDA library has not been built: there is no
CPU fallback behind this binding.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# PF_CUDA_LIBRARY: another build of the library to load (one with a
# user-defined profile compiled in, libprofit_gb300/build.py --out)
LIB_PATH = os.environ.get("PF_CUDA_LIBRARY") or os.path.join(HERE, "libpfcuda.so")

NPAR = 12

PF_OK = 0
PF_ERR_INVALID_PARAMETER = 1
PF_ERR_UNKNOWN_PARAMETER = 2
PF_ERR_CUDA = 3
PF_ERR_NO_MEMORY = 4
PF_ERR_DEVICE_LIMIT = 5
PF_ERR_UNSUPPORTED = 6
PF_ERR_INTERNAL = 7
PF_ERR_INVALID_FILE = 8

PF_ENV_DOUBLE = 0x1

PF_CONV_AUTO = 0
PF_CONV_BRUTE = 1
PF_CONV_FFT = 2

KINDS = {"sersic": 0, "coresersic": 1, "moffat": 2, "ferrer": 3, "king": 4,
         "brokenexp": 5, "sky": 6, "psf": 7, "null": 8}


class ProfileDesc(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("convolve", ctypes.c_int32), ("rough", ctypes.c_int32),
                ("adjust", ctypes.c_int32), ("rescale_flux", ctypes.c_int32),
                ("resolution", ctypes.c_uint32), ("max_recursions", ctypes.c_uint32),
                ("acc", ctypes.c_double), ("rscale_switch", ctypes.c_double),
                ("rscale_max", ctypes.c_double), ("par", ctypes.c_double * NPAR)]


class ModelDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("scale_x", ctypes.c_double), ("scale_y", ctypes.c_double),
                ("magzero", ctypes.c_double), ("finesampling", ctypes.c_uint32),
                ("return_finesampled", ctypes.c_int32), ("first_profile", ctypes.c_uint32),
                ("n_profiles", ctypes.c_uint32), ("psf_offset", ctypes.c_int64),
                ("psf_w", ctypes.c_uint32), ("psf_h", ctypes.c_uint32),
                ("psf_scale_x", ctypes.c_double), ("psf_scale_y", ctypes.c_double),
                ("convolver", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("mask_offset", ctypes.c_int64), ("adjust_mask", ctypes.c_int32), ("no_crop", ctypes.c_int32),
                ("mask_w", ctypes.c_uint32), ("mask_h", ctypes.c_uint32)]


class StageTimes(ctypes.Structure):
    _fields_ = [("setup_ms", ctypes.c_double), ("eval_ms", ctypes.c_double), ("finish_ms", ctypes.c_double),
                ("chi2_ms", ctypes.c_double), ("adjoint_conv_ms", ctypes.c_double),
                ("backward_ms", ctypes.c_double), ("forward_calls", ctypes.c_uint64),
                ("backward_calls", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64)]


PF_ENV_PROFILE = 0x2
PF_ENV_NO_AUTOTUNE = 0x4
PF_ENV_NO_SPLIT = 0x8

_P = ctypes.c_void_p
_SIGNATURES = {
    "pf_batch_stats": (ctypes.c_int, [_P, ctypes.POINTER(StageTimes), ctypes.c_int]),
    "pf_last_error": (ctypes.c_char_p, []),
    "pf_version": (ctypes.c_char_p, []),
    "pf_env_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(_P)]),
    "pf_env_destroy": (None, [_P]),
    "pf_model_output_dims": (ctypes.c_int, [ctypes.POINTER(ModelDesc), ctypes.POINTER(ProfileDesc),
                                            ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "pf_model_output_offset": (ctypes.c_int, [ctypes.POINTER(ModelDesc), ctypes.POINTER(ProfileDesc),
                                              ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "pf_model_evaluate": (ctypes.c_int, [_P, ctypes.POINTER(ModelDesc), ctypes.POINTER(ProfileDesc), _P, _P,
                                         ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]),
    "pf_model_evaluate_masked": (ctypes.c_int, [_P, ctypes.POINTER(ModelDesc), ctypes.POINTER(ProfileDesc), _P,
                                                _P, _P, ctypes.POINTER(ctypes.c_uint32),
                                                ctypes.POINTER(ctypes.c_uint32)]),
    "pf_convolve": (ctypes.c_int, [_P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_uint32,
                                   ctypes.c_uint32, _P, _P]),
    "pf_convolve_crop": (ctypes.c_int, [_P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_uint32,
                                        ctypes.c_uint32, _P, ctypes.c_int, _P, _P, _P]),
    "pf_convolve_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_uint32,
                                           ctypes.c_uint32, _P, _P]),
    "pf_batch_create": (ctypes.c_int, [_P, ctypes.POINTER(ModelDesc), ctypes.c_size_t,
                                       ctypes.POINTER(ProfileDesc), ctypes.c_size_t, _P, ctypes.c_size_t,
                                       ctypes.POINTER(_P)]),
    "pf_batch_create_masked": (ctypes.c_int, [_P, ctypes.POINTER(ModelDesc), ctypes.c_size_t,
                                              ctypes.POINTER(ProfileDesc), ctypes.c_size_t, _P, ctypes.c_size_t,
                                              _P, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "pf_batch_destroy": (None, [_P]),
    "pf_batch_layout": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(ctypes.c_uint64)]),
    "pf_batch_set_params": (ctypes.c_int, [_P, _P]),
    "pf_batch_set_params_dev": (ctypes.c_int, [_P, _P, _P]),
    "pf_forward": (ctypes.c_int, [_P, _P, _P, _P]),
    "pf_batch_check": (ctypes.c_int, [_P, _P]),
    "pf_batch_enable_adjoint": (ctypes.c_int, [_P]),
    "pf_backward": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "pf_forward_backward": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "pf_step_graph": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "pf_batch_record_depth": (ctypes.c_int, [_P, ctypes.c_int]),
    "pf_batch_depth": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "pf_batch_drawing_dims": (ctypes.c_int, [_P, _P]),
    "pf_batch_conv_info": (ctypes.c_int, [_P, _P, _P, _P]),
    "pf_user_profile_info": (ctypes.c_int, [ctypes.POINTER(ctypes.c_char_p),
                                            ctypes.POINTER(ctypes.POINTER(ctypes.c_char_p)),
                                            ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                            ctypes.POINTER(ctypes.c_uint32)]),
    "pf_env_last_model_stats": (ctypes.c_int, [_P, _P, _P, ctypes.c_size_t]),
    "pf_env_autotune_counts": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "pf_batch_split_info": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "pf_fits_write": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_double, ctypes.c_double]),
    "pf_fits_read": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_size_t, _P, _P, _P, _P]),
}

_lib = None


class LibraryMissing(RuntimeError):
    pass


def load():
    """Loads libpfcuda.so (built by libprofit_gb300/build.py or
    __graft_entry__.build()); raises LibraryMissing if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryMissing("libprofit_gb300/libpfcuda.so is not built; run "
                             "`python -c 'import __graft_entry__ as g; g.build()'` first "
                             "(the CUDA backend has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGNATURES)
