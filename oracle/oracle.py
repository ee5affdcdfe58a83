"""ctypes access to the CPU oracle: TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the plain-C restatement of libprofit's
``Model::evaluate`` path, src/model.cpp:259-360 and the files listed in
profit_oracle.h) and, where it was built, ``oracle/_ref/libprofit_ref.so``
(the unmodified libprofit sources driven through their public C++ API).

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module; the CUDA product never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libprofit_ref.so")

KINDS = {"sersic": 0, "coresersic": 1, "moffat": 2, "ferrer": 3, "king": 4,
         "brokenexp": 5, "sky": 6, "psf": 7, "null": 8}
NPAR = 12

# parameter slots, identical to the product's descriptor layout
SPECIFIC = {
    "sersic": ["re", "nser"],
    "coresersic": ["re", "nser", "rb", "a", "b"],
    "moffat": ["fwhm", "con"],
    "ferrer": ["rout", "a", "b"],
    "king": ["rc", "rt", "a"],
    "brokenexp": ["h1", "h2", "rb", "a"],
    "sky": ["bg"],
    "psf": [],
    "null": [],
}
COMMON = ["xcen", "ycen", "mag", "ang", "axrat", "box"]

# defaults of the reference constructors (src/radial.cpp:724-752 and each profile's ctor)
DEFAULTS = {
    "sersic": dict(re=1.0, nser=1.0),
    "coresersic": dict(re=1.0, rb=1.0, nser=4.0, a=1.0, b=1.0),
    "moffat": dict(fwhm=3.0, con=2.0),
    "ferrer": dict(rout=3.0, a=1.0, b=1.0, acc=1.0),
    "king": dict(rc=1.0, rt=3.0, a=2.0),
    "brokenexp": dict(h1=1.0, h2=1.0, rb=1.0, a=1.0),
    "sky": dict(bg=0.0),
    "psf": dict(xcen=0.0, ycen=0.0, mag=0.0),
    "null": dict(),
}


class OrcProfile(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("convolve", ctypes.c_int), ("rough", ctypes.c_int),
                ("adjust", ctypes.c_int), ("rescale_flux", ctypes.c_int),
                ("resolution", ctypes.c_uint), ("max_recursions", ctypes.c_uint),
                ("acc", ctypes.c_double), ("rscale_switch", ctypes.c_double),
                ("rscale_max", ctypes.c_double), ("par", ctypes.c_double * NPAR)]


class OrcModel(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint), ("height", ctypes.c_uint),
                ("scale_x", ctypes.c_double), ("scale_y", ctypes.c_double),
                ("magzero", ctypes.c_double), ("finesampling", ctypes.c_uint),
                ("return_finesampled", ctypes.c_int),
                ("psf", ctypes.POINTER(ctypes.c_double)), ("psf_w", ctypes.c_uint),
                ("psf_h", ctypes.c_uint), ("psf_scale_x", ctypes.c_double),
                ("psf_scale_y", ctypes.c_double), ("mask", ctypes.POINTER(ctypes.c_ubyte)),
                ("adjust_mask", ctypes.c_int), ("mask_w", ctypes.c_uint), ("mask_h", ctypes.c_uint),
                ("convolver", ctypes.c_int), ("omp_threads", ctypes.c_int)]


class OrcConstants(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("rscale", "ie", "bn", "lumtot", "rescale_factor", "rscale_switch", "rscale_max", "acc")] + \
               [("resolution", ctypes.c_uint), ("cos_ang", ctypes.c_double),
                ("sin_ang", ctypes.c_double), ("flux_scale", ctypes.c_double)]


def build(with_ref=None):
    """Compiles liboracle.so (always) and the reference library when the
    environment variable PF_REFERENCE_DIR names a libprofit source tree
    (with_ref None), or must (with_ref True)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_dir = os.environ.get("PF_REFERENCE_DIR", "")
    if with_ref or (with_ref is None and ref_dir and os.path.isdir(os.path.join(ref_dir, "src"))):
        subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "REF=" + ref_dir], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.orc_evaluate.restype = ctypes.c_int
        _lib.orc_last_error.restype = ctypes.c_char_p
        for name in ("orc_api_qgamma", "orc_api_pgamma", "orc_api_beta"):
            getattr(_lib, name).restype = ctypes.c_double
            getattr(_lib, name).argtypes = [ctypes.c_double, ctypes.c_double]
        _lib.orc_api_gammafn.restype = ctypes.c_double
        _lib.orc_api_gammafn.argtypes = [ctypes.c_double]
    return _lib


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_PATH)
        _ref.ref_evaluate.restype = ctypes.c_int
    return _ref


def ref_to_fits(image, offset, scale, fname):
    """profit::to_fits of the compiled reference (oracle/_ref)."""
    R = ref()
    img = np.ascontiguousarray(image, dtype=np.float64)
    err = ctypes.create_string_buffer(512)
    rc = R.ref_to_fits(img.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint(img.shape[1]), ctypes.c_uint(img.shape[0]),
                       ctypes.c_uint(offset[0]), ctypes.c_uint(offset[1]), ctypes.c_double(scale[0]),
                       ctypes.c_double(scale[1]), os.fsencode(fname), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())


def ref_from_fits(fname, cap=1 << 22):
    """profit::from_fits of the compiled reference: (image (h, w), (sx, sy))."""
    R = ref()
    out = np.zeros(cap, dtype=np.float64)
    w, h = ctypes.c_uint(), ctypes.c_uint()
    sx, sy = ctypes.c_double(), ctypes.c_double()
    err = ctypes.create_string_buffer(512)
    rc = R.ref_from_fits(os.fsencode(fname), out.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(cap),
                         ctypes.byref(w), ctypes.byref(h), ctypes.byref(sx), ctypes.byref(sy), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return out[:w.value * h.value].reshape(h.value, w.value).copy(), (sx.value, sy.value)


def make_profile(kind, **params):
    """Builds an OrcProfile with the reference defaults, overridden by params."""
    p = OrcProfile()
    p.kind = KINDS[kind]
    p.convolve = int(params.pop("convolve", False))
    p.rough = int(params.pop("rough", False))
    p.adjust = int(params.pop("adjust", True))
    p.rescale_flux = int(params.pop("rescale_flux", False))
    p.resolution = int(params.pop("resolution", 9))
    p.max_recursions = int(params.pop("max_recursions", 2))
    merged = dict(DEFAULTS[kind])
    merged.update(params)
    p.acc = float(merged.pop("acc", 0.1))
    p.rscale_switch = float(merged.pop("rscale_switch", 1.0))
    p.rscale_max = float(merged.pop("rscale_max", 0.0))
    vals = [0.0] * NPAR
    base = dict(xcen=0.0, ycen=0.0, mag=15.0, ang=0.0, axrat=1.0, box=0.0)
    if kind == "psf":
        base["mag"] = 0.0
    base.update({k: v for k, v in merged.items() if k in COMMON})
    for i, name in enumerate(COMMON):
        vals[i] = float(base[name])
    for i, name in enumerate(SPECIFIC[kind]):
        vals[6 + i] = float(merged[name])
    unknown = set(merged) - set(COMMON) - set(SPECIFIC[kind])
    if unknown:
        raise KeyError("unknown parameters for %s: %s" % (kind, sorted(unknown)))
    p.par[:] = vals
    return p


class Case:
    """A model: dims, scale, psf, and a list of (kind, params) profiles."""

    def __init__(self, width, height, profiles, psf=None, scale=(1.0, 1.0), magzero=0.0,
                 finesampling=1, return_finesampled=True, convolver="brute", psf_scale=(1.0, 1.0),
                 mask=None, adjust_mask=True):
        self.width, self.height = width, height
        self.profiles = profiles
        self.psf = None if psf is None else np.ascontiguousarray(psf, dtype=np.float64)
        self.scale = scale
        self.magzero = magzero
        self.finesampling = finesampling
        self.return_finesampled = return_finesampled
        self.convolver = convolver
        self.psf_scale = psf_scale
        # adjust_mask (the reference's default): mask of the model's dimensions,
        # adjusted as Model::evaluate does; otherwise used as given (drawing
        # dimensions, padded only if the mask is larger than the model)
        self.mask = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        self.adjust_mask = adjust_mask

    def c_model(self, threads=1):
        m = OrcModel()
        m.width, m.height = self.width, self.height
        m.scale_x, m.scale_y = self.scale
        m.magzero = self.magzero
        m.finesampling = self.finesampling
        m.return_finesampled = int(self.return_finesampled)
        if self.psf is not None:
            m.psf = self.psf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            m.psf_h, m.psf_w = self.psf.shape
        m.psf_scale_x, m.psf_scale_y = self.psf_scale
        if self.mask is not None:
            m.mask = self.mask.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte))
            m.mask_h, m.mask_w = self.mask.shape
        m.adjust_mask = int(bool(self.adjust_mask))
        m.convolver = 1 if self.convolver == "brute_old" else 0
        m.omp_threads = threads
        return m

    def c_profiles(self):
        arr = (OrcProfile * max(1, len(self.profiles)))()
        for i, (kind, params) in enumerate(self.profiles):
            arr[i] = make_profile(kind, **dict(params))
        return arr


class OracleError(RuntimeError):
    pass


def evaluate(case, threads=1, want_depth=False):
    """Runs the C restatement. Returns (image, depth_maps or None, level_counts)."""
    L = lib()
    m = case.c_model(threads)
    profs = case.c_profiles()
    n = len(case.profiles)
    ow, oh, dw, dh = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint()
    if L.orc_output_dims(ctypes.byref(m), profs, n, ctypes.byref(ow), ctypes.byref(oh),
                         ctypes.byref(dw), ctypes.byref(dh)) != 0:
        raise OracleError(L.orc_last_error().decode())
    out = np.zeros(ow.value * oh.value, dtype=np.float64)
    depth = np.zeros(max(1, n) * dw.value * dh.value, dtype=np.int8) if want_depth else None
    counts = np.zeros(max(1, n) * 32, dtype=np.int64)
    rc = L.orc_evaluate(ctypes.byref(m), profs, n, out.ctypes.data_as(ctypes.c_void_p),
                        ctypes.byref(ow), ctypes.byref(oh),
                        depth.ctypes.data_as(ctypes.c_void_p) if want_depth else None,
                        counts.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise OracleError(L.orc_last_error().decode())
    img = out.reshape(oh.value, ow.value)
    if want_depth:
        depth = depth[: n * dw.value * dh.value].reshape(n, dh.value, dw.value)
    return img, depth, counts[: n * 32].reshape(n, 32)


def evaluate_reference(case, threads=1):
    """Runs the unmodified libprofit (built into oracle/_ref). Returns (image, level_counts)."""
    R = ref()
    m = case.c_model(threads)
    profs = case.c_profiles()
    n = len(case.profiles)
    cap = (case.width * max(1, case.finesampling) + 512) * (case.height * max(1, case.finesampling) + 512)
    out = np.zeros(cap, dtype=np.float64)
    ow, oh = ctypes.c_uint(), ctypes.c_uint()
    counts = np.zeros(max(1, n) * 32, dtype=np.int64)
    err = ctypes.create_string_buffer(512)
    rc = R.ref_evaluate(ctypes.byref(m), profs, n, out.ctypes.data_as(ctypes.c_void_p),
                        ctypes.c_size_t(cap), ctypes.byref(ow), ctypes.byref(oh),
                        counts.ctypes.data_as(ctypes.c_void_p), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return out[: ow.value * oh.value].reshape(oh.value, ow.value).copy(), counts[: n * 32].reshape(n, 32)


def constants(case, index):
    L = lib()
    m = case.c_model()
    profs = case.c_profiles()
    c = OrcConstants()
    if L.orc_profile_constants(ctypes.byref(m), ctypes.byref(profs[index]), ctypes.byref(c)) != 0:
        raise OracleError(L.orc_last_error().decode())
    return {name: getattr(c, name) for name, _ in OrcConstants._fields_}


def convolve_brute(src, krn, mask=None, old=False, threads=1):
    L = lib()
    src = np.ascontiguousarray(src, dtype=np.float64)
    krn = np.ascontiguousarray(krn, dtype=np.float64)
    out = np.zeros_like(src)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    L.orc_convolve_brute(src.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint(src.shape[1]),
                         ctypes.c_uint(src.shape[0]), krn.ctypes.data_as(ctypes.c_void_p),
                         ctypes.c_uint(krn.shape[1]), ctypes.c_uint(krn.shape[0]),
                         None if mk is None else mk.ctypes.data_as(ctypes.c_void_p),
                         out.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(int(old)), ctypes.c_int(threads))
    return out


def fft_convolve_reference_math(src, krn):
    """The FFTConvolver's arithmetic (src/convolve.cpp:233-312) in numpy: ext =
    2*max(src,krn) with the x-only max() of include/profit/image.h:204-207, src
    at (0,0), kernel at (src-krn)/2, a 1-D real FFT of the flattened ext image,
    pointwise product, inverse, and the crop at offset_after_convolution."""
    sh, sw = src.shape
    kh, kw = krn.shape
    m = max(sw, kw)
    ext_w, ext_h = 2 * m, 2 * m
    ext_src = np.zeros((ext_h, ext_w))
    ext_src[:sh, :sw] = src
    ext_krn = np.zeros((ext_h, ext_w))
    ky, kx = (sh - kh) // 2, (sw - kw) // 2
    ext_krn[ky:ky + kh, kx:kx + kw] = krn
    n = ext_w * ext_h
    res = np.fft.irfft(np.fft.rfft(ext_src.ravel()) * np.fft.rfft(ext_krn.ravel()), n=n).reshape(ext_h, ext_w)
    ox = sw // 2 - (1 if (sw % 2 == 0 or kw % 2 == 0) else 0)
    oy = sh // 2 - (1 if (sh % 2 == 0 or kh % 2 == 0) else 0)
    return res[oy:oy + sh, ox:ox + sw]


def fft_convolve_uncropped(src, krn, mask=None):
    """The FFTConvolver's uncropped result (crop = false): the whole ext frame
    of fft_convolve_reference_math, masked by the mask extended over it at
    the offset (mask_and_crop, src/convolve.cpp:81-94), and that offset."""
    sh, sw = src.shape
    kh, kw = krn.shape
    m = max(sw, kw)
    ext_w, ext_h = 2 * m, 2 * m
    ext_src = np.zeros((ext_h, ext_w))
    ext_src[:sh, :sw] = src
    ext_krn = np.zeros((ext_h, ext_w))
    ky, kx = (sh - kh) // 2, (sw - kw) // 2
    ext_krn[ky:ky + kh, kx:kx + kw] = krn
    n = ext_w * ext_h
    res = np.fft.irfft(np.fft.rfft(ext_src.ravel()) * np.fft.rfft(ext_krn.ravel()), n=n).reshape(ext_h, ext_w)
    ox = sw // 2 - (1 if (sw % 2 == 0 or kw % 2 == 0) else 0)
    oy = sh // 2 - (1 if (sh % 2 == 0 or kh % 2 == 0) else 0)
    if mask is not None:
        ext_mask = np.zeros((ext_h, ext_w), dtype=bool)
        ext_mask[oy:oy + sh, ox:ox + sw] = np.asarray(mask) != 0
        res = np.where(ext_mask, res, 0.0)
    return res, (ox, oy)


def evaluate_uncropped_fft(case):
    """Model::evaluate with set_crop(false) and the FFT convolver
    (src/model.cpp:259-360), finesampling 1 and no calculation mask: the
    profiles drawn on the padded drawing area (the oracle's own drawing, the
    centres moved by the PSF padding as RadialProfile::evaluate moves them),
    the convolved ones through fft_convolve_uncropped, the others extended to
    its frame at its offset and added, then only the PSF padding removed with
    FFTConvolver::padding's offset and dimension differences (the x component
    of max() for both sides, include/profit/image.h:204-207). Returns (image,
    (offset_x, offset_y)) as Model::evaluate(Point &) does."""
    psf = np.asarray(case.psf, dtype=np.float64)
    psf = psf / psf.sum()
    kh, kw = psf.shape
    conv = [(k, p) for k, p in case.profiles if p.get("convolve", False)]
    rest = [(k, p) for k, p in case.profiles if not p.get("convolve", False)]
    px, py = kw // 2, kh // 2
    sx, sy = case.scale if hasattr(case, "scale") else (1.0, 1.0)
    dw, dh = case.width + 2 * px, case.height + 2 * py

    def draw(profiles):
        if not profiles:
            return np.zeros((dh, dw))
        moved = []
        for k, p in profiles:
            q = dict(p, convolve=False)
            if "xcen" in q:
                q["xcen"] = q["xcen"] + px * sx
                q["ycen"] = q["ycen"] + py * sy
            moved.append((k, q))
        img, _, _ = evaluate(Case(dw, dh, moved, scale=(sx, sy), magzero=case.magzero))
        return img

    conv_img, (ox, oy) = fft_convolve_uncropped(draw(conv), psf)
    direct = np.zeros_like(conv_img)
    direct[oy:oy + dh, ox:ox + dw] = draw(rest)
    image = direct + conv_img
    e = conv_img.shape[0]

    def off(a, k):
        return a // 2 - (1 if (a % 2 == 0 or k % 2 == 0) else 0)

    if px > 0 and py > 0:
        d2w, d2h = dw - 2 * px, dh - 2 * py
        shrink = max(dw, kw) - max(d2w, kw)
        cw, ch = e - 2 * px - shrink, e - 2 * py - shrink
        cx, cy = px + off(dw, kw) - off(d2w, kw), py + off(dh, kh) - off(d2h, kh)
        return image[cy:cy + ch, cx:cx + cw], (off(d2w, kw), off(d2h, kh))
    return image, (ox, oy)


def moffat_psf(size, fwhm, con, threads=1):
    """A size x size Moffat PSF rendered by the oracle's moffat profile,
    centred, normalised to unit sum (as Model::set_psf does)."""
    c = Case(size, size, [("moffat", dict(xcen=size / 2.0, ycen=size / 2.0, fwhm=fwhm, con=con, mag=0.0))])
    img, _, _ = evaluate(c, threads)
    return img / img.sum()
