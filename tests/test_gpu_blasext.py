"""The blasext kernels against numpy: axnpby with run-time coefficients,
in its plain and scaled forms (pyfr/backends/base/blasext.py:9-19 with the
arithmetic of pyfr/backends/cuda/kernels/axnpby.mako and
pyfr/backends/base/makoutil.py:43-58), and the generic reduction entry
point in the forms PyFR's explicit path makes (the PI controller's l2 and
uniform error norms, pyfr/integrators/controllers.py:105-117, and the
maximum of one variable)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def be():
    import __graft_entry__ as ge
    ge.build_library()
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    return B200Backend(Inifile())


def _regs(be, rng, n, shape=(8, 5, 77)):
    xs = [rng.normal(size=shape) for _ in range(n)]
    ms = [be.matrix(shape, x, tags={'align'}) for x in xs]
    be.commit()
    return xs, ms


@pytest.mark.parametrize('a0', [0.0, 1.0, 0.7])
def test_axnpby(be, a0):
    rng = np.random.default_rng(1)
    xs, ms = _regs(be, rng, 3)
    k = be.kernel('axnpby', *ms)
    k.bind(a0, -0.5, 2.0)
    be.run_kernels([k], wait=True)
    want = a0*xs[0] - 0.5*xs[1] + 2.0*xs[2]
    np.testing.assert_allclose(ms[0].get(), want, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize('a0', [0.0, 1.0, 0.7])
@pytest.mark.parametrize('idxs', [(1,), (0, 2)])
@pytest.mark.parametrize('out', [True, False])
def test_axnpby_scaled(be, a0, idxs, out):
    rng = np.random.default_rng(2)
    xs, ms = _regs(be, rng, 3)
    nvars = 5
    insc = rng.uniform(0.5, 2.0, nvars)
    outsc = rng.uniform(0.5, 2.0, nvars) if out else None
    k = be.kernel('axnpby', *ms, in_scale=tuple(insc), in_scale_idxs=idxs,
                  out_scale=tuple(outsc) if out else ())
    a = [a0, -0.5, 2.0]
    k.bind(*a)
    be.run_kernels([k], wait=True)

    first = 1 if a0 in (0.0, 1.0) else 0
    s = sum(a[i]*(insc[None, :, None] if i in idxs else 1)*xs[i]
            for i in range(first, 3))
    if out:
        s = outsc[None, :, None]*s
    want = xs[0] + s if a0 == 1.0 else s
    np.testing.assert_allclose(ms[0].get(), want, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize('norm', ['l2', 'uniform'])
def test_reduction_error_norm(be, norm):
    rng = np.random.default_rng(3)
    shape = (8, 5, 77)
    cur, err = rng.normal(size=shape), 1e-6*rng.normal(size=shape)
    C_ = be.matrix(shape, cur, tags={'align'})
    E = be.matrix(shape, err, tags={'align'})
    be.commit()
    atols = np.array([1e-6, 2e-6, 3e-6, 4e-6, 5e-6])
    q = 'err / (atol + rtol*fabs(curr))'
    expr, rop = (f'({q})*({q})', 'sum') if norm == 'l2' else \
        (f'fabs({q})', 'max')
    k = be.kernel('reduction', rop, [expr], {'curr': C_, 'err': E},
                  svars=['rtol'], pvars={'atol': atols})
    k.bind(1e-5)
    be.run_kernels([k], wait=True)
    x = err/(atols[None, :, None] + 1e-5*np.abs(cur))
    want = np.sum(x*x) if norm == 'l2' else np.abs(x).max()
    assert abs(k.retval[0] - want) <= 1e-12*want


def test_reduction_max(be):
    rng = np.random.default_rng(4)
    x = rng.uniform(0, 3, size=(1, 333))
    X = be.matrix(x.shape, x, tags={'align'})
    be.commit()
    k = be.kernel('reduction', 'max', ['x'], {'x': X})
    be.run_kernels([k], wait=True)
    assert k.retval[0] == x.max()


def test_reduction_other_forms_refused(be):
    X = be.matrix((1, 32), tags={'align'})
    be.commit()
    with pytest.raises(NotImplementedError):
        be.kernel('reduction', 'sum', ['x*x'], {'x': X})


@pytest.mark.parametrize('chunks,streams', [(1, 1), (16, 1), (7, 2),
                                            (16, -1), (5, -2)])
def test_memcpy_roundtrip(be, chunks, streams):
    """The pipelined host round trip of the end-to-end loop: a device array
    goes down to page-locked host memory and back into another (or the
    same) device array, by the copy engines or by kernels through the
    buffer's device mapping; an odd byte count exercises the last piece
    and the kernels' byte tail."""
    import ctypes as C
    rng = np.random.default_rng(chunks + 10*abs(streams))
    x = rng.normal(size=(8, 5, 77))
    a = be.matrix(x.shape, x, tags={'align'})
    b = be.matrix(x.shape, tags={'align'})
    be.commit()
    lib, st = be.lib, be.stream
    nbytes = a.nbytes - 3
    h = C.c_void_p()
    lib.host_alloc(C.byref(h), a.nbytes)
    try:
        lib.memcpy_roundtrip(h.value, a.data, b.data, nbytes, chunks, streams,
                             st)
        be.wait()
        got = np.frombuffer((C.c_char*nbytes).from_address(h.value),
                            dtype=np.uint8)
        want = np.empty(a.nbytes, dtype=np.uint8)
        lib.memcpy_dtoh(want.ctypes.data, a.data, a.nbytes, st)
        back = np.empty(a.nbytes, dtype=np.uint8)
        lib.memcpy_dtoh(back.ctypes.data, b.data, a.nbytes, st)
        be.wait()
        np.testing.assert_array_equal(got, want[:nbytes])
        np.testing.assert_array_equal(back[:nbytes], want[:nbytes])
        assert not back[nbytes:].any()
        # In place, down only
        lib.memcpy_roundtrip(h.value, a.data, None, a.nbytes, chunks, streams,
                             st)
        lib.memcpy_roundtrip(h.value, a.data, a.data, a.nbytes, chunks,
                             streams, st)
        be.wait()
        np.testing.assert_array_equal(a.get(), x)
    finally:
        lib.host_free(h.value)
