"""A stand-in for the pyfrb200 library with no GPU behind it (test
infrastructure): every entry point of the C ABI exists with its name, takes
its arguments and returns success; allocations return distinct fake device
addresses, handle and event outputs are set, and nothing is computed.  It
lets the host side of the backend (allocation, views, kernel construction,
graphs) run on a machine without a GPU, to check that callers drive the
backend interface correctly.  Results are meaningless."""

import ctypes as C
import itertools as it

from pyfr_gb300.backend import lib as liblib


class FakeLib:
    version = 'fake pyfrb200 (no GPU)'

    def __init__(self):
        self._addr = it.count(1 << 40, 1 << 20)
        self.calls = []
        for name in liblib._SIGS:
            setattr(self, name.removeprefix('b200_'), self._stub(name))
        self.malloc = self._malloc
        self.host_alloc = self._malloc
        self.device_info = self._device_info

    def _stub(self, name):
        def call(*args):
            self.calls.append(name)
            for a in args:
                obj = getattr(a, '_obj', None)
                if isinstance(obj, C.c_void_p) and not obj.value:
                    obj.value = next(self._addr)
                elif isinstance(obj, (C.c_int, C.c_size_t)) and not obj.value:
                    obj.value = 4
                elif isinstance(obj, C.c_float):
                    obj.value = 1.0
                elif isinstance(obj, C.c_double):
                    obj.value = 1.0
        call.__name__ = name
        return call

    def _malloc(self, ptr, nbytes):
        self.calls.append('b200_malloc')
        ptr._obj.value = next(self._addr)
        n = (nbytes + (1 << 20) - 1) >> 20
        for _ in range(n):
            next(self._addr)

    def _device_info(self, sms, major, minor, free, total, name, namelen):
        for p, v in ((sms, 152), (major, 10), (minor, 3), (free, 1 << 38),
                     (total, 1 << 38)):
            if p is not None:
                p._obj.value = v
        if name is not None:
            name.value = b'fake GB300'

    def last_error(self):
        return ''


def install():
    """Make the backend load the stand-in instead of the library."""
    liblib._LIB = FakeLib()
    return liblib._LIB
