"""GB300-native backend for libprofit's image-generation path.

The host-side classes mirror libprofit's C++ interface for this path so that
code written against it reads the same:

    profit::Model            -> Model (add_profile, set_psf, set_image_pixel_scale,
                                set_psf_pixel_scale, set_magzero, set_finesampling,
                                set_return_finesampled, set_cuda_env, evaluate)
    Profile::parameter       -> Profile.parameter(name, value) / parameter("name=value")
                                (src/profile.cpp:84-163: same names, types, messages)
    get_opencl_environment   -> get_cuda_environment(device, use_double)
    create_convolver("cuda") -> create_convolver("cuda").convolve(src, krn, mask)
    exceptions               -> InvalidParameter, UnknownParameter, CudaError
                                (include/profit/exceptions.h:41-104)

Everything computes on the GPU through the C ABI of include/pf_cuda.h
(libpfcuda.so); Batch exposes the batched path (many models per launch).
"""
import ctypes
import os

import numpy as np

from . import _ffi
from ._ffi import KINDS, NPAR

__all__ = ["Model", "Profile", "CUDAEnv", "get_cuda_environment", "create_convolver", "Batch",
           "from_fits", "to_fits",
           "ProfitError", "InvalidParameter", "UnknownParameter", "CudaError", "InvalidFile", "version"]


class ProfitError(RuntimeError):
    """profit::exception"""


class InvalidParameter(ProfitError):
    """profit::invalid_parameter"""


class UnknownParameter(ProfitError):
    """profit::unknown_parameter"""


class CudaError(ProfitError):
    """A CUDA runtime failure (the role profit::opencl_error plays for OpenCL)."""


class DeviceLimit(ProfitError):
    """A bounded device-side resource was exceeded."""


class Unsupported(ProfitError):
    """A parameter combination the CUDA backend does not support."""


class InvalidFile(ProfitError):
    """profit::invalid_file (include/profit/fits_utils.h:34-43)"""


_ERRORS = {
    _ffi.PF_ERR_INVALID_PARAMETER: InvalidParameter,
    _ffi.PF_ERR_UNKNOWN_PARAMETER: UnknownParameter,
    _ffi.PF_ERR_CUDA: CudaError,
    _ffi.PF_ERR_NO_MEMORY: CudaError,
    _ffi.PF_ERR_DEVICE_LIMIT: DeviceLimit,
    _ffi.PF_ERR_UNSUPPORTED: Unsupported,
    _ffi.PF_ERR_INTERNAL: ProfitError,
    _ffi.PF_ERR_INVALID_FILE: InvalidFile,
}


def _check(status):
    if status != _ffi.PF_OK:
        msg = _ffi.load().pf_last_error().decode()
        raise _ERRORS.get(status, ProfitError)(msg)


def version():
    return _ffi.load().pf_version().decode()


# Parameter registry per profile kind: name -> (type, slot). Slots index
# pf_profile_desc.par; the control parameters live in named fields.
_RADIAL_COMMON = {"xcen": 0, "ycen": 1, "mag": 2, "ang": 3, "axrat": 4, "box": 5}
_SPECIFIC = {
    "sersic": {"re": 6, "nser": 7},
    "coresersic": {"re": 6, "nser": 7, "rb": 8, "a": 9, "b": 10},
    "moffat": {"fwhm": 6, "con": 7},
    "ferrer": {"rout": 6, "a": 7, "b": 8},
    "king": {"rc": 6, "rt": 7, "a": 8},
    "brokenexp": {"h1": 6, "h2": 7, "rb": 8, "a": 9},
    "sky": {"bg": 6},
    "psf": {"xcen": 0, "ycen": 1, "mag": 2},
    "null": {},
}
# constructor defaults (src/radial.cpp:724-752 and each profile's constructor)
_DEFAULTS = {
    "sersic": {"re": 1.0, "nser": 1.0},
    "coresersic": {"re": 1.0, "rb": 1.0, "nser": 4.0, "a": 1.0, "b": 1.0},
    "moffat": {"fwhm": 3.0, "con": 2.0},
    "ferrer": {"rout": 3.0, "a": 1.0, "b": 1.0},
    "king": {"rc": 1.0, "rt": 3.0, "a": 2.0},
    "brokenexp": {"h1": 1.0, "h2": 1.0, "rb": 1.0, "a": 1.0},
    "sky": {"bg": 0.0},
    "psf": {"xcen": 0.0, "ycen": 0.0, "mag": 0.0},
    "null": {},
}
_RADIAL = ["sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp"]
PF_USER = 9


def _user_profile():
    """The user-defined radial profile compiled into the loaded library
    (pf_user_profile_info): registered under its name, with its parameters
    and defaults, the first time an unknown profile name is asked for."""
    name, names, defaults, n = ctypes.c_char_p(), ctypes.POINTER(ctypes.c_char_p)(), \
        ctypes.POINTER(ctypes.c_double)(), ctypes.c_uint32()
    if _ffi.load().pf_user_profile_info(ctypes.byref(name), ctypes.byref(names), ctypes.byref(defaults),
                                        ctypes.byref(n)) != _ffi.PF_OK:
        return None
    kind = name.value.decode()
    if kind not in KINDS:
        KINDS[kind] = PF_USER
        _SPECIFIC[kind] = {names[i].decode(): 6 + i for i in range(n.value)}
        _DEFAULTS[kind] = {names[i].decode(): defaults[i] for i in range(n.value)}
        _RADIAL.append(kind)
    return kind


class Profile:
    """A profile of a Model; parameters are set with parameter()."""

    def __init__(self, name):
        kind = "ferrer" if name == "ferrers" else name
        if kind not in KINDS and _user_profile() != kind:
            raise InvalidParameter("Unknown profile name: %s" % name)
        self.name = name
        self.kind = kind
        d = _ffi.ProfileDesc()
        d.kind = KINDS[kind]
        d.convolve = 0
        d.rough = 0
        d.adjust = 1
        d.rescale_flux = 0
        d.resolution = 9
        d.max_recursions = 2
        d.acc = 1.0 if kind == "ferrer" else 0.1
        d.rscale_switch = 1.0
        d.rscale_max = 0.0
        vals = [0.0] * NPAR
        if kind in _RADIAL:
            vals[:6] = [0.0, 0.0, 15.0, 0.0, 1.0, 0.0]
        for k, v in _DEFAULTS[kind].items():
            vals[_SPECIFIC[kind][k]] = v
        d.par[:] = vals
        self.desc = d

    # name -> type ("bool", "unsigned int", "double") for this kind
    def _types(self):
        t = {"convolve": "bool"}
        if self.kind in _RADIAL:
            t.update({"rough": "bool", "adjust": "bool", "force_cpu": "bool",
                      "max_recursions": "unsigned int", "resolution": "unsigned int",
                      "acc": "double", "rscale_switch": "double", "rscale_max": "double"})
            t.update({k: "double" for k in _RADIAL_COMMON})
        if self.kind == "sersic":
            t["rescale_flux"] = "bool"
        t.update({k: "double" for k in _SPECIFIC[self.kind]})
        return t

    def parameter(self, name, value=None):
        """parameter(name, value) or parameter("name=value")
        (Profile::parameter, src/profile.cpp:84-163)."""
        if value is None:
            parts = name.split("=")
            if len(parts) != 2:
                raise InvalidParameter("missing = in parameter: %s" % name)
            pname, sval = parts[0].strip(), parts[1].strip()
            t = self._types().get(pname)
            try:
                if t == "bool":
                    conv = bool(int(sval, 10))
                elif t == "unsigned int":
                    conv = int(sval, 10)
                    if conv < 0:
                        raise ValueError(sval)
                elif t == "double":
                    conv = float(sval)
                else:
                    raise KeyError(pname)
            except (KeyError, ValueError):
                raise UnknownParameter("Profile %s doesn't support parameter %s, or parameter has invalid "
                                       "value: %s" % (self.name, pname, sval))
            return self._set(pname, conv, t)
        if isinstance(value, bool):
            t = "bool"
        elif isinstance(value, (int, np.integer)):
            t = "unsigned int"
        else:
            t = "double"
        known = self._types()
        if known.get(name) != t:
            # an int given for a double parameter is accepted as a double
            if t == "unsigned int" and known.get(name) == "double":
                t = "double"
                value = float(value)
            else:
                raise InvalidParameter("Unknown %s parameter in profile %s: %s" % (t, self.name, name))
        return self._set(name, value, t)

    def _set(self, name, value, t):
        d = self.desc
        if name in ("convolve", "rough", "adjust", "rescale_flux"):
            setattr(d, name, int(bool(value)))
        elif name == "force_cpu":
            pass  # no CPU path exists behind the CUDA backend
        elif name in ("resolution", "max_recursions"):
            setattr(d, name, int(value))
        elif name in ("acc", "rscale_switch", "rscale_max"):
            setattr(d, name, float(value))
        elif self.kind in _RADIAL and name in _RADIAL_COMMON:
            d.par[_RADIAL_COMMON[name]] = float(value)
        else:
            d.par[_SPECIFIC[self.kind][name]] = float(value)
        return self

    def get(self, name):
        d = self.desc
        if name in ("convolve", "rough", "adjust", "rescale_flux", "resolution", "max_recursions",
                    "acc", "rscale_switch", "rscale_max"):
            return getattr(d, name)
        if self.kind in _RADIAL and name in _RADIAL_COMMON:
            return d.par[_RADIAL_COMMON[name]]
        return d.par[_SPECIFIC[self.kind][name]]


class CUDAEnv:
    """A CUDA environment (get_opencl_environment analogue). use_double selects
    the plain FP64 path (the reference's arithmetic and subsampling decisions);
    profile, per-stage CUDA-event timing; autotune=False, the fixed cost model
    for the automatic convolution choice of large single-precision batches;
    split=False, every subsampled pixel's tree walked by the warp that meets
    it (PF_ENV_NO_SPLIT)."""

    def __init__(self, device=0, use_double=True, profile=False, autotune=True, split=True):
        lib = _ffi.load()
        h = ctypes.c_void_p()
        flags = (_ffi.PF_ENV_DOUBLE if use_double else 0) | (_ffi.PF_ENV_PROFILE if profile else 0) | \
            (0 if autotune else _ffi.PF_ENV_NO_AUTOTUNE) | (0 if split else _ffi.PF_ENV_NO_SPLIT)
        _check(lib.pf_env_create(int(device), flags, ctypes.byref(h)))
        self._h = h
        self.device = device
        self.use_double = use_double

    @property
    def handle(self):
        return self._h

    def autotune_counts(self):
        """{"timed", "reused"}: the autotuner's decisions made by timing in
        this environment and those taken from its cache (the same batch
        layout seen before, or the PF_AUTOTUNE_CACHE file read at its
        creation) (pf_env_autotune_counts)."""
        t, r = ctypes.c_uint64(), ctypes.c_uint64()
        _check(_ffi.load().pf_env_autotune_counts(self._h, ctypes.byref(t), ctypes.byref(r)))
        return {"timed": t.value, "reused": r.value}

    def close(self):
        if self._h:
            _ffi.load().pf_env_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_cuda_environment(device=0, use_double=True, profile=False, autotune=True, split=True):
    return CUDAEnv(device, use_double, profile, autotune, split)


_default_env = None


def _env_or_default(env):
    global _default_env
    if env is not None:
        return env
    if _default_env is None:
        _default_env = CUDAEnv(0, True)
    return _default_env


class Model:
    """profit::Model for the CUDA backend (include/profit/model.h)."""

    def __init__(self, width=0, height=0):
        self.width = int(width)
        self.height = int(height)
        self.profiles = []
        self.psf = None
        self.scale = (1.0, 1.0)
        self.psf_scale = (1.0, 1.0)
        self.magzero = 0.0
        self.finesampling = 1
        self.return_finesampled = True
        self.env = None
        self.convolver = _ffi.PF_CONV_AUTO
        self.mask = None
        self.adjust_mask = True
        self.crop = True

    def add_profile(self, name):
        p = Profile(name)
        self.profiles.append(p)
        return p

    def set_dimensions(self, dims):
        self.width, self.height = int(dims[0]), int(dims[1])

    def set_psf(self, psf):
        self.psf = None if psf is None else np.ascontiguousarray(psf, dtype=np.float64)

    def set_image_pixel_scale(self, scale):
        self.scale = (float(scale[0]), float(scale[1]))

    def set_psf_pixel_scale(self, scale):
        self.psf_scale = (float(scale[0]), float(scale[1]))

    def set_magzero(self, magzero):
        self.magzero = float(magzero)

    def set_finesampling(self, fs):
        if int(fs) == 0:
            raise InvalidParameter("finesampling must be > 0")
        self.finesampling = int(fs)

    def set_return_finesampled(self, flag):
        self.return_finesampled = bool(flag)

    def set_cuda_env(self, env):
        self.env = env

    def set_mask(self, mask):
        """Model::set_mask: a boolean (height, width) calculation mask (True =
        evaluate), of the model's dimensions (or of the drawing dimensions when
        set_adjust_mask(False)); None removes it."""
        self.mask = None if mask is None else np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8)

    def set_adjust_mask(self, adjust):
        """Model::set_adjust_mask (default True)."""
        self.adjust_mask = bool(adjust)

    def set_crop(self, crop):
        """Model::set_crop (default True). The direct convolutions add no
        padding, so their uncropped image is the cropped one at offset (0, 0);
        the FFT convolution with crop False gives its uncropped frame less the
        PSF padding, and the offset of the requested area in it
        (evaluate_with_offset; double precision only)."""
        self.crop = bool(crop)

    def set_convolver(self, convolver):
        """A Convolver from create_convolver, or "auto", "brute" or "fft"."""
        names = {"auto": _ffi.PF_CONV_AUTO, "brute": _ffi.PF_CONV_BRUTE, "cuda": _ffi.PF_CONV_BRUTE,
                 "cuda-brute": _ffi.PF_CONV_BRUTE, "fft": _ffi.PF_CONV_FFT, "cuda-fft": _ffi.PF_CONV_FFT}
        if isinstance(convolver, Convolver):
            self.convolver = convolver.kind
        elif isinstance(convolver, str):
            if convolver not in names:
                raise InvalidParameter("Unsupported convolver type: %s" % convolver)
            self.convolver = names[convolver]
        else:
            self.convolver = int(convolver)

    def _descs(self, first_profile=0, psf_offset=None, mask_offset=None):
        m = _ffi.ModelDesc()
        m.width, m.height = self.width, self.height
        m.scale_x, m.scale_y = self.scale
        m.magzero = self.magzero
        m.finesampling = self.finesampling
        m.return_finesampled = int(self.return_finesampled)
        m.first_profile = first_profile
        m.n_profiles = len(self.profiles)
        if self.psf is not None:
            m.psf_h, m.psf_w = self.psf.shape
            m.psf_offset = 0 if psf_offset is None else psf_offset
        else:
            m.psf_offset = -1
        m.psf_scale_x, m.psf_scale_y = self.psf_scale
        m.convolver = self.convolver
        m.mask_offset = -1 if self.mask is None else (0 if mask_offset is None else mask_offset)
        m.adjust_mask = int(self.adjust_mask)
        if self.mask is not None:
            m.mask_h, m.mask_w = self.mask.shape
        m.no_crop = int(not self.crop)
        profs = (_ffi.ProfileDesc * max(1, len(self.profiles)))()
        for i, p in enumerate(self.profiles):
            profs[i] = p.desc
        return m, profs

    def output_dims(self):
        m, profs = self._descs()
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        _check(_ffi.load().pf_model_output_dims(ctypes.byref(m), profs, ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value

    def output_offset(self):
        """The offset Model::evaluate reports (pf_model_output_offset): (0, 0)
        unless set_crop(False) with the FFT convolver."""
        m, profs = self._descs()
        x, y = ctypes.c_uint32(), ctypes.c_uint32()
        _check(_ffi.load().pf_model_output_offset(ctypes.byref(m), profs, ctypes.byref(x), ctypes.byref(y)))
        return x.value, y.value

    def evaluate_with_offset(self):
        """Model::evaluate(Point &offset): (image, (x, y)) with the offset of
        the requested area in the returned image (see set_crop)."""
        return self.evaluate(), self.output_offset()

    def evaluate(self):
        """Model::evaluate: returns the image as a (height, width) float64 array."""
        env = _env_or_default(self.env)
        m, profs = self._descs()
        w, h = self.output_dims()
        out = np.zeros(w * h, dtype=np.float64)
        ow, oh = ctypes.c_uint32(), ctypes.c_uint32()
        psf_ptr = None if self.psf is None else self.psf.ctypes.data_as(ctypes.c_void_p)
        mask_ptr = None if self.mask is None else self.mask.ctypes.data_as(ctypes.c_void_p)
        _check(_ffi.load().pf_model_evaluate_masked(env.handle, ctypes.byref(m), profs, psf_ptr, mask_ptr,
                                                    out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ow),
                                                    ctypes.byref(oh)))
        return out.reshape(oh.value, ow.value)

    def get_stats(self):
        """Model::get_stats (src/model.cpp:362-368): {profile name: stats} of
        the last evaluate() on this model's environment, keyed by name as the
        reference's map is (a later profile of the same name replaces an
        earlier one). Needs an environment created with profile=True (an
        empty dict otherwise). This backend evaluates all of a model's
        profiles in fused passes timed as a whole, so each entry holds the
        passes' device times ("pass_*_ms") and the profile's own counts --
        subsample_pixel calls per recursion level ("integrations", as
        get_profile_integrations) and evaluate_at calls ("evaluations") --
        and "total_ms", the setup pass split evenly plus the evaluation pass
        split by evaluations (pf_env_last_model_stats)."""
        env = _env_or_default(self.env)
        n = len(self.profiles)
        t = _ffi.StageTimes()
        counts = np.zeros(max(1, n) * 32, dtype=np.int64)
        _check(_ffi.load().pf_env_last_model_stats(env.handle, ctypes.byref(t),
                                                    counts.ctypes.data_as(ctypes.c_void_p), n))
        if t.forward_calls == 0 or n == 0:
            return {}
        counts = counts.reshape(-1, 32)[:n]
        evals = counts[:, 30] + counts[:, 31]
        all_evals = int(evals.sum())
        out = {}
        for i, p in enumerate(self.profiles):
            share = evals[i] / all_evals if all_evals else 1.0 / n
            out[p.name] = {
                "total_ms": t.setup_ms / n + t.eval_ms * share,
                "pass_setup_ms": t.setup_ms, "pass_evaluation_ms": t.eval_ms, "pass_convolution_ms": t.finish_ms,
                "evaluations": int(evals[i]),
                "integrations": {lvl: int(c) for lvl, c in enumerate(counts[i, :16]) if c},
            }
        return out

    def get_profile_integrations(self):
        """Model::get_profile_integrations (src/model.cpp:370-381, a
        PROFIT_DEBUG build): per radial profile name, {recursion level:
        subsample_pixel calls at that level} for one evaluation of the model
        (src/radial.cpp:71-79); a later profile of the same name replaces an
        earlier one, as in the reference's map. Evaluates the model once
        through a one-model batch with depth recording on."""
        import torch
        env = _env_or_default(self.env)
        b = Batch([self], env)
        try:
            b.record_depth(True)
            out = torch.zeros(b.total_pixels, dtype=torch.float64 if env.use_double else torch.float32,
                              device="cuda:%d" % env.device)
            b.forward(out)
            b.check()
            res = {}
            for prof, (_, counts) in zip(self.profiles, b.depth()):
                if prof.kind in _RADIAL:
                    # slots 0-15 of the depth recording's counts are the levels
                    res[prof.kind] = {lvl: int(c) for lvl, c in enumerate(counts[:16]) if c > 0}
            return res
        finally:
            b.close()


class Convolver:
    """A ConvolverType::CUDA convolver (create_convolver, src/convolve.cpp:521-584)."""

    def __init__(self, kind=_ffi.PF_CONV_BRUTE, env=None):
        self.kind = kind
        self.env = env

    def convolve(self, src, krn, mask=None, crop=True, offset_out=None):
        """Convolver::convolve (include/profit/convolve.h:65-99). The CUDA
        convolver adds no padding: crop=False gives the same image, and
        offset_out (a list, optional) receives the offset [0, 0]."""
        env = _env_or_default(self.env)
        src = np.ascontiguousarray(src, dtype=np.float64)
        krn = np.ascontiguousarray(krn, dtype=np.float64)
        out = np.zeros_like(src)
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        ox, oy = ctypes.c_uint32(), ctypes.c_uint32()
        _check(_ffi.load().pf_convolve_crop(env.handle, src.ctypes.data_as(ctypes.c_void_p), src.shape[1],
                                            src.shape[0], krn.ctypes.data_as(ctypes.c_void_p), krn.shape[1],
                                            krn.shape[0], None if mk is None else mk.ctypes.data_as(ctypes.c_void_p),
                                            int(bool(crop)), out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ox),
                                            ctypes.byref(oy)))
        if offset_out is not None:
            offset_out[:] = [ox.value, oy.value]
        return out


def create_convolver(kind="cuda", env=None):
    names = {"cuda": _ffi.PF_CONV_BRUTE, "cuda-brute": _ffi.PF_CONV_BRUTE, "cuda-fft": _ffi.PF_CONV_FFT}
    if kind not in names:
        raise InvalidParameter("Unsupported convolver type: %s" % kind)
    return Convolver(names[kind], env)


def from_fits(filename):
    """profit::from_fits (src/fits_utils.cpp:60-126) through pf_fits_read:
    the image of a FITS file written as to_fits writes (BITPIX -64, NAXIS 2)
    as a float64 array of shape (height, width), and its pixel scale
    (CDELT1, CDELT2; 1 where absent). Raises InvalidFile with the
    reference's messages."""
    lib = _ffi.load()
    name = os.fsencode(filename)
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    sx, sy = ctypes.c_double(), ctypes.c_double()
    _check(lib.pf_fits_read(name, None, 0, ctypes.byref(w), ctypes.byref(h), ctypes.byref(sx), ctypes.byref(sy)))
    img = np.zeros((h.value, w.value), dtype=np.float64)
    _check(lib.pf_fits_read(name, img.ctypes.data_as(ctypes.c_void_p), img.size, ctypes.byref(w),
                            ctypes.byref(h), ctypes.byref(sx), ctypes.byref(sy)))
    return img, (sx.value, sy.value)


def to_fits(image, offset, pixel_scale, filename):
    """profit::to_fits (src/fits_utils.cpp:150-205) through pf_fits_write:
    writes `image` (2-D, rows = height) with the origin's `offset` (x, y;
    whole pixels, as Model.evaluate_with_offset returns it) and `pixel_scale`
    (x, y) into `filename`, ".fits" appended unless it ends in it; the bytes
    are the reference's."""
    img = np.ascontiguousarray(image, dtype=np.float64)
    if img.ndim != 2:
        raise InvalidParameter("to_fits: the image must be 2-D")
    ox, oy = (int(v) for v in offset)
    if ox != offset[0] or oy != offset[1] or ox < 0 or oy < 0 or max(ox, oy) >= 1 << 32:
        raise InvalidParameter("to_fits: the offset must be a pair of non-negative whole pixels")
    h, w = img.shape
    _check(_ffi.load().pf_fits_write(os.fsencode(filename), img.ctypes.data_as(ctypes.c_void_p), w, h, ox, oy,
                                     float(pixel_scale[0]), float(pixel_scale[1])))


class Batch:
    """Many models rendered by one launch sequence (pf_batch_* / pf_forward).

    Device buffers are torch tensors (or any object with data_ptr()); the
    batch sizes all its scratch once at construction."""

    def __init__(self, models, env=None):
        self.env = _env_or_default(env)
        self.models = list(models)
        n_prof = sum(len(m.profiles) for m in self.models)
        mds = (_ffi.ModelDesc * max(1, len(self.models)))()
        pds = (_ffi.ProfileDesc * max(1, n_prof))()
        psfs, masks = [], []
        first, psf_off, mask_off = 0, 0, 0
        for i, m in enumerate(self.models):
            md, pd = m._descs(first_profile=first, psf_offset=psf_off if m.psf is not None else None,
                              mask_offset=mask_off if m.mask is not None else None)
            mds[i] = md
            for j in range(len(m.profiles)):
                pds[first + j] = pd[j]
            first += len(m.profiles)
            if m.psf is not None:
                psfs.append(m.psf.ravel())
                psf_off += m.psf.size
            if m.mask is not None:
                masks.append(m.mask.ravel())
                mask_off += m.mask.size
        self.psf_pool = np.ascontiguousarray(np.concatenate(psfs) if psfs else np.zeros(0), dtype=np.float64)
        self.mask_pool = np.ascontiguousarray(np.concatenate(masks) if masks else np.zeros(0), dtype=np.uint8)
        self.n_profiles = n_prof
        h = ctypes.c_void_p()
        lib = _ffi.load()
        _check(lib.pf_batch_create_masked(
            self.env.handle, mds, len(self.models), pds, n_prof,
            self.psf_pool.ctypes.data_as(ctypes.c_void_p) if self.psf_pool.size else None, self.psf_pool.size,
            self.mask_pool.ctypes.data_as(ctypes.c_void_p) if self.mask_pool.size else None, self.mask_pool.size,
            ctypes.byref(h)))
        self._h = h
        n = len(self.models)
        offs = (ctypes.c_uint64 * (n + 1))()
        dims = (ctypes.c_uint32 * max(1, 2 * n))()
        total = ctypes.c_uint64()
        _check(lib.pf_batch_layout(h, offs, dims, ctypes.byref(total)))
        self.offsets = [int(offs[i]) for i in range(n + 1)]
        self.dims = [(int(dims[2 * i]), int(dims[2 * i + 1])) for i in range(n)]
        self.total_pixels = int(total.value)

    @property
    def handle(self):
        return self._h

    def _check_buffers(self, params=None, images=None, data=None, sigma=None, cotangent=None, chi2=None,
                       grad=None):
        pix = 8 if self.env.use_double else 4
        dev = self.env.device
        _need(params, self.n_profiles * NPAR, 8, "params", dev)
        for name, buf in (("images", images), ("data", data), ("sigma", sigma), ("cotangent", cotangent)):
            _need(buf, self.total_pixels, pix, name, dev)
        _need(chi2, len(self.models), 8, "chi2", dev)
        _need(grad, self.n_profiles * NPAR, 8, "grad", dev)

    def forward(self, images, flux=None, stream=None):
        """Renders into `images` (device buffer of total_pixels elements,
        float64 for a use_double environment), on `stream` (a cudaStream_t
        handle; by default torch's current stream)."""
        self._check_buffers(images=images)
        _need(flux, len(self.models), 8, "flux", self.env.device)
        _check(_ffi.load().pf_forward(self._h, ctypes.c_void_p(images.data_ptr()),
                                      None if flux is None else ctypes.c_void_p(flux.data_ptr()),
                                      _stream_arg(stream)))

    def check(self, stream=None):
        _check(_ffi.load().pf_batch_check(self._h, _stream_arg(stream)))

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(self.n_profiles, NPAR)
        _check(_ffi.load().pf_batch_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p)))

    def set_params_dev(self, params, stream=None):
        self._check_buffers(params=params)
        _check(_ffi.load().pf_batch_set_params_dev(self._h, ctypes.c_void_p(params.data_ptr()),
                                                   _stream_arg(stream)))

    def stats(self, reset=False):
        """Per-stage device milliseconds (environment created with profile=True)."""
        t = _ffi.StageTimes()
        _check(_ffi.load().pf_batch_stats(self._h, ctypes.byref(t), int(bool(reset))))
        return {name: getattr(t, name) for name, _ in _ffi.StageTimes._fields_}

    def conv_info(self):
        """The convolution plan: {"forward_shape", "adjoint_shape" (-1 before
        enable_adjoint), "fft_models"} (pf_batch_conv_info)."""
        f, a, n = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_uint32()
        _check(_ffi.load().pf_batch_conv_info(self._h, ctypes.byref(f), ctypes.byref(a), ctypes.byref(n)))
        return {"forward_shape": f.value, "adjoint_shape": a.value, "fft_models": n.value}

    def split_info(self, stream=None):
        """How the last forward pass spread its subsampling trees: {"boxes",
        "roots", "pixels", "refused"} (pf_batch_split_info)."""
        v = [ctypes.c_uint32() for _ in range(4)]
        _check(_ffi.load().pf_batch_split_info(self._h, _stream_arg(stream), *[ctypes.byref(x) for x in v]))
        return dict(zip(("boxes", "roots", "pixels", "refused"), (x.value for x in v)))

    def enable_adjoint(self):
        """Sizes the adjoint's device buffers (pf_batch_enable_adjoint)."""
        _check(_ffi.load().pf_batch_enable_adjoint(self._h))

    def backward(self, images, data=None, sigma=None, cotangent=None, chi2=None, grad=None, stream=None):
        """chi^2 per model and d chi^2 / d par (or, with a cotangent, the
        vector-Jacobian product of the images) into the given device buffers."""
        self._check_buffers(images=images, data=data, sigma=sigma, cotangent=cotangent, chi2=chi2, grad=grad)
        _check(_ffi.load().pf_backward(self._h, _ptr(images), _ptr(data), _ptr(sigma), _ptr(cotangent),
                                       _ptr(chi2), _ptr(grad), _stream_arg(stream)))

    def forward_backward(self, images, data, sigma=None, chi2=None, grad=None, stream=None):
        """One model + VJP evaluation: render, then chi^2 and its gradient."""
        self._check_buffers(images=images, data=data, sigma=sigma, chi2=chi2, grad=grad)
        _check(_ffi.load().pf_forward_backward(self._h, _ptr(images), _ptr(data), _ptr(sigma), _ptr(chi2),
                                               _ptr(grad), _stream_arg(stream)))

    def step_graph(self, params, images, data, sigma=None, chi2=None, grad=None, stream=None):
        """set_params_dev(params) (if given) + forward_backward, captured once
        into a CUDA graph and replayed (pf_step_graph); `stream` must be a
        created stream (torch.cuda.Stream().cuda_stream)."""
        self._check_buffers(params=params, images=images, data=data, sigma=sigma, chi2=chi2, grad=grad)
        _check(_ffi.load().pf_step_graph(self._h, _ptr(params), _ptr(images), _ptr(data), _ptr(sigma),
                                         _ptr(chi2), _ptr(grad), _stream_arg(stream)))

    def record_depth(self, enable=True):
        _check(_ffi.load().pf_batch_record_depth(self._h, int(bool(enable))))

    def depth(self):
        """Per profile: (depth map over its model's drawing area, 32 counts:
        slots 0-15 the subsample_pixel calls per recursion level, slot 30 the
        evaluate_at calls on pixel centres, slot 31 those inside
        subsample_pixel)."""
        dims = np.zeros(2 * max(1, len(self.models)), dtype=np.uint32)
        _check(_ffi.load().pf_batch_drawing_dims(self._h, dims.ctypes.data_as(ctypes.c_void_p)))
        sizes = []
        for m_idx, m in enumerate(self.models):
            w, h = int(dims[2 * m_idx]), int(dims[2 * m_idx + 1])
            sizes += [(h, w)] * len(m.profiles)
        total = sum(h * w for h, w in sizes)
        buf = np.zeros(max(1, total), dtype=np.int8)
        counts = np.zeros(max(1, self.n_profiles) * 32, dtype=np.int64)
        _check(_ffi.load().pf_batch_depth(self._h, buf.ctypes.data_as(ctypes.c_void_p), total,
                                          counts.ctypes.data_as(ctypes.c_void_p)))
        out, off = [], 0
        for i, (h, w) in enumerate(sizes):
            out.append((buf[off:off + h * w].reshape(h, w), counts[32 * i:32 * (i + 1)]))
            off += h * w
        return out

    def close(self):
        if getattr(self, "_h", None):
            _ffi.load().pf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _need(buf, count, itemsize, what, device=None):
    """The C ABI takes raw device pointers and reads or writes `count`
    elements through them as one dense array on the environment's device: a
    tensor that is smaller, of another element size, not contiguous, in host
    memory or on another device is refused here instead of being overrun or
    misread on the device."""
    if buf is None or not hasattr(buf, "numel"):
        return
    if buf.element_size() != itemsize or buf.numel() < count:
        raise InvalidParameter("%s: %d elements of %d bytes needed, the buffer has %d of %d" %
                               (what, count, itemsize, buf.numel(), buf.element_size()))
    if hasattr(buf, "is_cuda"):
        if not buf.is_cuda:
            raise InvalidParameter("%s: a device (CUDA) buffer is needed, the tensor is in host memory" % what)
        if device is not None and buf.device.index is not None and buf.device.index != device:
            raise InvalidParameter("%s: the buffer is on device %d, the environment on device %d" %
                                   (what, buf.device.index, device))
    if hasattr(buf, "is_contiguous") and not buf.is_contiguous():
        raise InvalidParameter("%s: the buffer must be contiguous" % what)


def _stream_arg(stream):
    """The cudaStream_t to pass: the given handle, else torch's current
    stream (its legacy default stream is handle 0, passed as cudaStreamLegacy
    because NULL selects the environment's own stream in the C ABI)."""
    if stream is None:
        try:
            import torch
            stream = torch.cuda.current_stream().cuda_stream
        except Exception:
            return None
    if hasattr(stream, "cuda_stream"):
        stream = stream.cuda_stream
    return ctypes.c_void_p(stream if stream else _CUDA_STREAM_LEGACY)
