"""ctypes binding of the pyfrb200 C ABI (``include/pyfrb200.h``).

Follows the pattern of ``pyfr/ctypesutil.py:8-40`` (LibWrapper): every
function is declared once with its argument types, and a nonzero status is
raised as a Python exception carrying the library's last error message.
There is no fallback: if the shared library is missing or cannot be
loaded, construction fails.
"""

import ctypes as C
from pathlib import Path

LIBPATH = Path(__file__).resolve().parent.parent / '_lib' / 'libpyfrb200.so'

vp, i32, i64, f64, f32, sz = (C.c_void_p, C.c_int, C.c_int64, C.c_double,
                              C.c_float, C.c_size_t)
pd, pf = C.POINTER(C.c_double), C.POINTER(C.c_float)


class B200Error(RuntimeError):
    pass


class MulArgs(C.Structure):
    """``b200_mul_bf16x3_args_t``"""
    _fields_ = [('b1', C.c_void_p), ('b2', C.c_void_p),
                ('ldb1', C.c_int64), ('ldb2', C.c_int64),
                ('c', C.c_void_p), ('ldc', C.c_int64), ('ncol', C.c_int64),
                ('nbatch', C.c_int), ('bstride1', C.c_int64),
                ('bstride2', C.c_int64), ('cstride', C.c_int64),
                ('alpha', C.c_float), ('beta', C.c_float),
                ('rowscale', C.c_void_p), ('ldr', C.c_int64),
                ('nvars', C.c_int), ('products', C.c_int),
                ('err', C.c_void_p), ('rk_acc', C.c_void_p),
                ('rk_u', C.c_void_p), ('rk_dt_dev', C.c_void_p),
                ('rk_dt', C.c_double), ('rk_a', C.c_double),
                ('rk_b', C.c_double), ('rk_stage', C.c_int)]


class Gas(C.Structure):
    _fields_ = [('gamma', f64), ('mu', f64), ('pr', f64), ('cpTref', f64),
                ('cpTs', f64), ('sutherland', i32), ('shifted', i32),
                ('rho_ref', f64), ('p_ref', f64), ('p_min', f64),
                ('v_ref', f64*3)]


# Boundary-condition types and constants (b200_bc_t)
BC_TYPES = {'sup-in-fa': 1, 'sup-out-fn': 2, 'slp-adia-wall': 3,
            'char-riem-inv': 4, 'no-slp-adia-wall': 5, 'no-slp-isot-wall': 6,
            'sub-in-frv': 7, 'sub-in-ftpttang': 8, 'sub-out-fp': 9,
            'char-riem-inv-mass-flow': 10, 'char-riem-inv-pressure': 10}


class BCOp(C.Structure):
    """``b200_bcop_t``"""
    _fields_ = [('op', i32), ('pad', i32), ('val', f64)]


class BC(C.Structure):
    _fields_ = [('type', i32), ('rho', f64), ('p', f64), ('u', f64*3),
                ('cpTw', f64), ('cpTt', f64), ('pt', f64), ('vc', f64*3),
                ('prog', C.c_void_p), ('expr_start', i32*6),
                ('expr_len', i32*6), ('ploc', C.c_void_p), ('ldp', i64),
                ('t_dev', C.c_void_p), ('t', f64), ('ic', f64), ('im', f64),
                ('ctrl', C.c_void_p)]


class Src(C.Structure):
    """``b200_src_t``"""
    _fields_ = [('prog', C.c_void_p), ('expr_start', i32*8),
                ('expr_len', i32*8), ('ploc', C.c_void_p), ('ldp', i64),
                ('u', C.c_void_p), ('ldu', i64), ('t', f64),
                ('t_dev', C.c_void_p)]


# Source-term kernel modes (B200_SRC_*)
SRC_NEGDIVCONF, SRC_ADD, SRC_EVAL = 0, 1, 2


class EF(C.Structure):
    """``b200_ef_t``"""
    _fields_ = [('ndims', i32), ('nupts', i32), ('nfpts', i32),
                ('nefpts', i32), ('nfaces', i32), ('order', i32),
                ('fpts_in_upts', i32), ('linearise', i32), ('niters', i32),
                ('gamma', f64), ('d_min', f64), ('p_min', f64), ('e_tol', f64),
                ('f_tol', f64)]


class AV(C.Structure):
    """``b200_av_t``"""
    _fields_ = [('nupts', i32), ('nvars', i32), ('svar', i32), ('nverts', i32),
                ('nmodes', i32), ('ndeg', i32), ('kwh', i32), ('kappa', f64),
                ('max_av', f64), ('se0', f64), ('s_weights', f64*16),
                ('baseline', f64*16)]


def _sig_pointwise(fp):
    return {
        'tflux_euler': [i32, i32, i64, i32, f64, vp, i64, vp, i64, vp, i64, vp,
                        i64, vp, i64, vp],
        'tflux_ns': [i32, i32, i64, i32, C.POINTER(Gas), vp, i64, vp, i64, vp,
                     i64, vp, i64, vp, i64, vp, i64, vp, i64, vp],
        'gradcoru': [i32, i32, i64, i32, vp, i64, vp, i64, vp, i64, vp, i64,
                     vp, i64, vp],
        'negdivconf': [i32, i32, i64, vp, i64, vp, i64, vp],
        'srcterms': [i32, i32, i32, i32, i64, vp, i64, vp, i64,
                     C.POINTER(Src), vp],
        'pack_view': [i64, i32, i32, vp, vp, vp, i32, vp, i64, vp],
        'intcflux_euler': [i32, i64, i32, f64, f64, vp, vp, vp, vp, i32, vp,
                           i64, i32, vp],
        'intcflux_ns': [i32, i64, i32, C.POINTER(Gas), f64, f64, vp, vp, vp,
                        vp, vp, vp, vp, vp, vp, vp, i32, vp, i64, i32, vp],
        'intconu': [i32, i64, f64, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp],
        'intconu_both': [i32, i64, f64, vp, vp, vp, vp, vp, vp, vp, vp, i32,
                         vp],
        'rkvdh2': [i64, i32, i32, i32, f64, f64, f64, f64, vp, vp, vp, vp, vp],
        'rkvdh2_dt': [i64, i32, i32, i32, vp, f64, f64, f64, vp, vp, vp, vp,
                      vp],
        'axnpby': [i64, i32, vp, C.POINTER(vp), C.POINTER(f64), vp],
        'axnpby_scaled': [i64, i32, i32, vp, C.POINTER(vp), C.POINTER(f64),
                          C.POINTER(f64), C.c_uint, C.POINTER(f64), vp],
        'errest': [i32, i32, i64, i64, vp, vp, vp, f64, i32, vp, i32, vp, vp],
        'mul': [vp, vp, i64, vp, i64, i64, fp, fp, vp],
        'wavespeed': [i32, i32, i64, i32, C.POINTER(Gas), vp, i64, vp, i64,
                      vp, i64, vp, i64, vp, i64, vp, vp],
        'bccflux_euler': [i32, i64, i32, f64, f64, C.POINTER(BC), vp, vp, i32,
                          vp, i64, vp],
        'bcconu': [i32, i64, f64, C.POINTER(BC), vp, vp, vp, vp, i32, vp, i64,
                   vp],
        'bccflux_ns': [i32, i64, i32, C.POINTER(Gas), f64, C.POINTER(BC), vp,
                       vp, vp, vp, vp, i32, vp, i64, vp],
        'bccflux_ns_av': [i32, i64, i32, C.POINTER(Gas), f64, C.POINTER(BC),
                          vp, vp, vp, vp, vp, i32, vp, i64, vp, vp, vp],
        'tflux_euler_shift': [i32, i32, i64, i32, C.POINTER(Gas), vp, i64, vp,
                              i64, vp, i64, vp, i64, vp, i64, vp],
        'intcflux_euler_shift': [i32, i64, C.POINTER(Gas), vp, vp, vp, vp, i32,
                                 vp, i64, i32, vp],
        'tflux_ns_refgrad': [i32, i32, i64, i32, C.POINTER(Gas), vp, i64, vp,
                             i64, vp, i64, vp, i64, vp, i64, vp, i64, vp, i64,
                             vp],
        'intcflux_ns_refgrad': [i32, i64, i32, C.POINTER(Gas), f64, f64, vp,
                                vp, vp, vp, vp, vp, vp, vp, vp, vp, i32, vp,
                                i64, i32, vp, i64, vp, vp, vp],
        'tflux_ns_av': [i32, i32, i64, i32, C.POINTER(Gas), vp, i64, vp, i64,
                        vp, i64, vp, i64, vp, i64, vp, i64, vp, i64, vp, i64,
                        vp],
        'intcflux_ns_av': [i32, i64, i32, C.POINTER(Gas), f64, f64, vp, vp,
                           vp, vp, vp, vp, vp, vp, vp, vp, i32, vp, i64, i32,
                           vp, vp, vp],
        'shocksensor': [C.POINTER(AV), i64, vp, i64, vp, i64, vp, vp, vp, i64,
                        vp, vp],
        'avfill': [i32, i32, i64, vp, vp, i64, vp, i64, vp, i64, vp],
        'bccent': [i32, i64, f64, C.POINTER(BC), vp, vp, vp, vp, i32, vp, i64,
                   vp],
        'entropyfilter': [C.POINTER(EF), i64, vp, i64, vp, i64, vp, vp, i64,
                          vp, i64, vp, i64, vp, i64, vp, vp],
        'entropylocal': [C.POINTER(EF), i64, vp, i64, vp, i64, vp, i64, vp],
        'intcent': [i64, vp, vp, vp, vp, i32, vp],
        'reduce_max': [i64, vp, vp, vp, vp],
    }


_SIGS = {
    'b200_init': [i32],
    'b200_get_last_error': [C.c_char_p, sz],
    'b200_device_info': [C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                         C.POINTER(sz), C.POINTER(sz), C.c_char_p, sz],
    'b200_malloc': [C.POINTER(vp), sz],
    'b200_free': [vp],
    'b200_host_alloc': [C.POINTER(vp), sz],
    'b200_host_free': [vp],
    'b200_memset': [vp, i32, sz, vp],
    'b200_stage_time': [vp, vp, f64, f64, vp],
    'b200_ef_merge_f64f32': [i32, i32, i64, vp, vp, i64, vp, i64, vp],
    'b200_memcpy_htod': [vp, vp, sz, vp],
    'b200_memcpy_dtoh': [vp, vp, sz, vp],
    'b200_memcpy_dtod': [vp, vp, sz, vp],
    'b200_memcpy_roundtrip': [vp, vp, vp, sz, C.c_int, C.c_int, vp],
    'b200_stream_create': [C.POINTER(vp)],
    'b200_stream_destroy': [vp],
    'b200_stream_sync': [vp],
    'b200_device_sync': [],
    'b200_event_create': [C.POINTER(vp)],
    'b200_event_destroy': [vp],
    'b200_event_record': [vp, vp],
    'b200_event_sync': [vp],
    'b200_event_elapsed': [C.POINTER(f32), vp, vp],
    'b200_probe_fp64_fma': [i32, C.POINTER(f64), vp],
    'b200_graph_begin_capture': [vp],
    'b200_graph_end_capture': [vp, C.POINTER(vp)],
    'b200_graph_launch': [vp, vp],
    'b200_graph_destroy': [vp],
    'b200_mul_create': [pd, i32, i32, C.POINTER(vp)],
    'b200_mul_nnz': [vp, C.POINTER(i32)],
    'b200_mul_destroy': [vp],
    'b200_rkmixed_f64f32': [i64, i32, i32, i32, f64, f64, f64, f64, vp, vp,
                            vp, vp, vp, vp],
    'b200_rkmixed_dt_f64f32': [i64, i32, i32, i32, vp, f64, f64, f64, vp, vp,
                               vp, vp, vp, vp],
    'b200_cast_f64_f32': [i64, vp, vp, i32, vp, vp],
    'b200_integrals_f64': [i32, i32, i64, vp, i64, vp, i64, vp, i64, vp, i32,
                           vp, vp],
    'b200_integrals_f64f32': [i32, i32, i64, vp, i64, vp, i64, vp, i64, vp,
                              vp, i32, vp, vp],
    'b200_errest_shifted_f64': [i32, i32, i64, i64, vp, vp, vp, f64, i32, vp,
                                f64, vp, i32, vp, vp],
    'b200_errest_static_f64': [i32, i32, i64, i64, vp, vp, vp, f64, i32, i32,
                               vp, vp],
    'b200_mul_bf16x3_create': [pd, i32, i32, C.POINTER(vp), C.POINTER(sz)],
    'b200_mul_bf16x3_destroy': [vp],
    'b200_mul_bf16x3': [vp, vp, i64, vp, i64, i64, f32, f32, vp, vp],
    'b200_mul_bf16x3_create_cat': [pd, i32, pd, i32, i32, C.POINTER(vp),
                                   C.POINTER(sz)],
    'b200_mul_bf16x3_apply': [vp, C.c_void_p, vp],
    'b200_mul_tf32_create': [pd, i32, i32, C.POINTER(vp), C.POINTER(sz)],
    'b200_mul_tc_create_plan': [pd, i32, pd, i32, i32, i32, i32, i32,
                                C.POINTER(vp), C.POINTER(sz)],
    'b200_mul_tc_plan': [vp, C.POINTER(i32), C.POINTER(i32)],
    'b200_mul_tc_create_terms': [pd, i32, pd, i32, i32, i32, i32, i32, i32,
                                 C.POINTER(vp), C.POINTER(sz)],
    'b200_mul_tc_terms': [vp, C.POINTER(i32)],
    'b200_mul_tf32_create_cat': [pd, i32, pd, i32, i32, C.POINTER(vp),
                                 C.POINTER(sz)],
}

for _fp, _suf in ((f64, 'f64'), (f32, 'f32')):
    for _name, _args in _sig_pointwise(_fp).items():
        _SIGS[f'b200_{_name}_{_suf}'] = _args


def exported_symbols():
    """Names of every entry point the Python side binds."""
    return sorted(_SIGS) + ['b200_version']


class Lib:
    """Loaded library with status-checked entry points as attributes
    (``lib.mul_f64(...)`` calls ``b200_mul_f64``)."""

    def __init__(self, path=LIBPATH):
        if not Path(path).exists():
            raise B200Error(f'pyfrb200 library not built: {path} is missing '
                            '(run __graft_entry__.build())')

        self._lib = lib = C.CDLL(str(path))
        lib.b200_version.restype = C.c_char_p
        lib.b200_version.argtypes = []
        self.version = lib.b200_version().decode()

        for name, args in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_int
            setattr(self, name.removeprefix('b200_'), self._wrap(name, fn))

    def _wrap(self, name, fn):
        def call(*args):
            rc = fn(*args)
            if rc:
                raise B200Error(f'{name} failed (status {rc}): '
                                f'{self.last_error()}')
        call.__name__ = name
        return call

    def last_error(self):
        buf = C.create_string_buffer(512)
        self._lib.b200_get_last_error(buf, 512)
        return buf.value.decode(errors='replace')


_LIB = None


def get_lib():
    global _LIB
    if _LIB is None:
        _LIB = Lib()
    return _LIB
