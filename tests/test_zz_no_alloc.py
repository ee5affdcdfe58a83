"""pf_convolve_noalloc (GPU): pf_convolve with its device scratch in static
device data, called through the C ABI and compared with pf_convolve.

The file name puts it last in collection: it must give pf_convolve's results
both alone and after every other test has used the device. Each case makes two
calls in a row on different inputs, so a result that depended on what an
earlier call left in the shared scratch would show. Tolerance: 1e-13 relative,
as for pf_convolve against the brute-force oracle (both run the same kernel).
Two tests check the property the entry point exists for: 100 calls leave the
device's free memory unchanged, and with the device's memory taken by
torch's caching allocator (pf_convolve on a new environment, which must
allocate its buffers, then fails) the call still succeeds.
"""
import ctypes

import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


@pytest.fixture(scope="module")
def abi():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    from libprofit_gb300 import _ffi
    env = pg.get_cuda_environment(0, use_double=True)
    yield _ffi, _ffi.load(), env
    env.close()


def _call(lib, name, env, src, krn, mask=None):
    out = np.full(src.shape, np.nan)
    status = getattr(lib, name)(env.handle, _ptr(src), src.shape[1], src.shape[0], _ptr(krn), krn.shape[1],
                                krn.shape[0], _ptr(mask), _ptr(out))
    return status, out


# (image h, w), (kernel h, w), masked; the 10 x 10 images with a 15 x 15
# kernel take the extend-convolve-crop path; 1024 x 1024 is the largest image
CASES = [((100, 100), (25, 25), False), ((101, 99), (24, 25), True), ((10, 10), (15, 15), True),
         ((10, 10), (15, 15), False), ((37, 64), (15, 16), True), ((1024, 1024), (9, 9), True)]


@pytest.mark.parametrize("shape,kshape,masked", CASES)
def test_noalloc_matches_pf_convolve(abi, shape, kshape, masked):
    ffi, lib, env = abi
    rng = np.random.default_rng(hash((shape, kshape, masked)) % (1 << 32))
    for _ in range(2):
        src, krn = rng.random(shape), rng.random(kshape)
        mask = (rng.random(shape) > 0.3).astype(np.uint8) if masked else None
        st_ref, ref = _call(lib, "pf_convolve", env, src, krn, mask)
        assert st_ref == ffi.PF_OK, lib.pf_last_error()
        st, got = _call(lib, "pf_convolve_noalloc", env, src, krn, mask)
        assert st == ffi.PF_OK, lib.pf_last_error()
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)
        if masked:
            assert np.all(got[mask == 0] == 0)


def test_noalloc_refuses_beyond_scratch(abi):
    ffi, lib, env = abi
    rng = np.random.default_rng(5)
    limit = 1 << 20
    krn_limit = 1 << 16
    for shape, kshape in [((1024, 1025), (3, 3)),      # one row of pixels too many
                          ((1000, 1000), (5, 1100)),   # fits, but not once extended to 1100 x 1100
                          ((300, 300), (256, 257))]:   # kernel too large
        assert shape[0] * shape[1] > limit or kshape[0] * kshape[1] > krn_limit or max(shape[1], kshape[1]) ** 2 > limit
        st, out = _call(lib, "pf_convolve_noalloc", env, rng.random(shape), rng.random(kshape))
        assert st == ffi.PF_ERR_DEVICE_LIMIT
        assert b"use pf_convolve" in lib.pf_last_error()
        assert np.all(np.isnan(out))  # nothing was written
    # the reference's extension refusal is kept
    st, _ = _call(lib, "pf_convolve_noalloc", env, rng.random((40, 10)), rng.random((15, 15)))
    assert st == ffi.PF_ERR_INVALID_PARAMETER
    # and a call after the refusals still works
    src, krn = rng.random((64, 64)), rng.random((7, 7))
    _, ref = _call(lib, "pf_convolve", env, src, krn)
    st, got = _call(lib, "pf_convolve_noalloc", env, src, krn)
    assert st == ffi.PF_OK
    np.testing.assert_allclose(got, ref, rtol=RTOL, atol=0)


def test_noalloc_allocates_no_device_memory(abi):
    """The property the entry point exists for. After a first call on the
    device (which may load the library's device code), 100 calls leave the
    device's free memory exactly as it was."""
    import torch
    ffi, lib, env = abi
    rng = np.random.default_rng(11)
    src, krn = rng.random((512, 512)), rng.random((25, 25))
    mask = (rng.random(src.shape) > 0.2).astype(np.uint8)
    st, first = _call(lib, "pf_convolve_noalloc", env, src, krn, mask)
    assert st == ffi.PF_OK, lib.pf_last_error()
    gc.collect()  # earlier objects freed now, not during the measurement
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(100):
        st, out = _call(lib, "pf_convolve_noalloc", env, src, krn, mask)
        assert st == ffi.PF_OK, lib.pf_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    np.testing.assert_array_equal(out, first)


def test_noalloc_works_on_a_full_device(abi):
    """A caller whose caching allocator holds nearly all of the device's
    memory: pf_convolve on an environment that has not yet grown its buffers
    cannot allocate them there, while pf_convolve_noalloc still gives the
    same result as on an empty device."""
    import torch
    import libprofit_gb300 as pg
    ffi, lib, env = abi
    rng = np.random.default_rng(12)
    src, krn = rng.random((1024, 1024)), rng.random((15, 15))
    st, want = _call(lib, "pf_convolve_noalloc", env, src, krn)
    assert st == ffi.PF_OK, lib.pf_last_error()
    fresh = pg.get_cuda_environment(0, use_double=True)  # no convolution buffers yet
    held = []
    try:
        # take the device's memory through torch until 8 to 10 MiB are free
        # (pf_convolve needs 2 x 8 MiB for this image)
        for chunk in (1 << 34, 1 << 30, 1 << 26, 1 << 21):
            while torch.cuda.mem_get_info(0)[0] > chunk + (8 << 20):
                try:
                    held.append(torch.empty(chunk, dtype=torch.uint8, device="cuda:0"))
                except torch.cuda.OutOfMemoryError:
                    break
        assert torch.cuda.mem_get_info(0)[0] < 16 << 20
        st_alloc, _ = _call(lib, "pf_convolve", fresh, src, krn)
        assert st_alloc != ffi.PF_OK
        st, got = _call(lib, "pf_convolve_noalloc", env, src, krn)
        assert st == ffi.PF_OK, lib.pf_last_error()
        np.testing.assert_array_equal(got, want)
    finally:
        del held
        torch.cuda.empty_cache()
        fresh.close()
