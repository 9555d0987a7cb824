"""The allocation-free error norm, b200_errest_static_f64.

It exists for callers that cannot give the library scratch memory when
they evaluate the PI controller's error norm.  An integrator that keeps
its step loop asynchronous cannot afford cudaFree's device-wide
synchronisation.  An application whose own pool allocator owns all device
memory cannot make a raw allocation.  The test calls it through the C ABI
and checks it against b200_errest_f64, which takes caller-provided
scratch, and against a numpy restatement of the norm.  It makes two calls in a row: the second is smaller, so stale
partials left by the first call must not leak into its result.  The file
is collected last, so a run that stops at the first failure has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BLOCKS = 4096
RTOL = 1e-12


@pytest.fixture(scope='module')
def lib():
    import __graft_entry__ as ge
    ge.build_library()
    from pyfr_gb300.backend.lib import LIBPATH

    lib = C.CDLL(str(LIBPATH))
    vp, i32, i64, f64 = C.c_void_p, C.c_int, C.c_int64, C.c_double
    lib.b200_errest_f64.argtypes = [i32, i32, i64, i64, vp, vp, vp, f64, i32,
                                    vp, i32, vp, vp]
    lib.b200_errest_static_f64.argtypes = [i32, i32, i64, i64, vp, vp, vp,
                                           f64, i32, i32, vp, vp]
    lib.b200_malloc.argtypes = [C.POINTER(vp), C.c_size_t]
    lib.b200_free.argtypes = [vp]
    lib.b200_memcpy_htod.argtypes = [vp, vp, C.c_size_t, vp]
    lib.b200_memcpy_dtoh.argtypes = [vp, vp, C.c_size_t, vp]
    lib.b200_device_sync.argtypes = []
    lib.b200_get_last_error.argtypes = [C.c_char_p, C.c_size_t]
    assert lib.b200_init(0) == 0
    return lib


def _dev(lib, arr):
    p = C.c_void_p()
    assert lib.b200_malloc(C.byref(p), arr.nbytes) == 0
    assert lib.b200_memcpy_htod(p, arr.ctypes.data, arr.nbytes, None) == 0
    return p


def _get(lib, p, n):
    out = np.empty(n)
    assert lib.b200_memcpy_dtoh(out.ctypes.data, p, out.nbytes, None) == 0
    assert lib.b200_device_sync() == 0
    return out


def _case(lib, nupts, nvars, neles, seed):
    rng = np.random.default_rng(seed)
    ld = nvars*(neles + (-neles % 32))
    curr = rng.normal(size=nupts*ld)
    err = 1e-6*rng.normal(size=nupts*ld)
    atol = np.linspace(1e-6, 4e-6, nvars)
    host = (curr, err, atol)
    return ld, host, [_dev(lib, a) for a in host]


def _norm_numpy(curr, err, atol, rtol, uniform, nupts, nvars, neles, ld):
    """The error norm restated with numpy: over the valid elements of
    each point and variable (AoSoA, blocks of 32 elements), the sum of
    (err/(atol_v + rtol |curr|))^2, or the largest |.| when uniform."""
    e = np.arange(neles)
    idx = ((e // 32)*32*nvars + e % 32)[None, :] + \
        (32*np.arange(nvars))[:, None]              # (nvars, neles)
    idx = np.arange(nupts)[:, None, None]*ld + idx[None]
    q = err[idx]/(atol[None, :, None] + rtol*np.abs(curr[idx]))
    return np.abs(q).max() if uniform else np.sum(q*q)


@pytest.mark.parametrize('uniform', [0, 1])
def test_static_errest_matches_scratch_errest(lib, uniform):
    # (nupts, nvars, neles, seed, nblocks): the second call is smaller than
    # the first; nblocks = 4096 fills the whole static array; the last case
    # has fewer work items (nupts x element blocks) than partial sums
    cases = [(64, 5, 20000, 11, 1000), (16, 4, 333, 12, 7),
             (27, 5, 40000, 13, MAX_BLOCKS), (8, 5, 100, 14, 1000)]
    out = _dev(lib, np.zeros(2))
    scratch = _dev(lib, np.zeros(MAX_BLOCKS))
    bufs = []
    try:
        for nupts, nvars, neles, seed, nblocks in cases:
            ld, host, (curr, err, atol) = _case(lib, nupts, nvars, neles,
                                                seed)
            bufs += [curr, err, atol]
            want = _norm_numpy(*host, 1e-5, uniform, nupts, nvars, neles, ld)

            assert lib.b200_errest_f64(nupts, nvars, neles, ld, curr, err,
                                       atol, 1e-5, uniform, scratch, nblocks,
                                       out, None) == 0
            ref = _get(lib, out, 1)[0]

            assert lib.b200_errest_static_f64(nupts, nvars, neles, ld, curr,
                                              err, atol, 1e-5, uniform,
                                              nblocks, out, None) == 0
            got = _get(lib, out, 1)[0]

            assert ref > 0
            assert abs(got - ref) <= RTOL*abs(ref)
            assert abs(got - want) <= RTOL*abs(want), (got, want)
    finally:
        for p in bufs + [out, scratch]:
            lib.b200_free(p)


def test_static_errest_rejects_too_many_blocks(lib):
    out = _dev(lib, np.zeros(1))
    try:
        rc = lib.b200_errest_static_f64(4, 4, 32, 128, None, None, None, 1e-5,
                                        0, MAX_BLOCKS + 1, out, None)
        assert rc != 0
        buf = C.create_string_buffer(512)
        lib.b200_get_last_error(buf, 512)
        assert b'nblocks' in buf.value
    finally:
        lib.b200_free(out)
