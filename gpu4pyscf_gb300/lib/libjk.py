"""ctypes binding of libgb300jk.so (C ABI declared in include/gb300jk.h).

The library is built in-tree by gpu4pyscf_gb300/csrc/build.py.  There is no
fallback: if the library is missing or fails to load, every entry point
raises.
"""
import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libgb300jk.so')

JK_PREC_FP64 = 0
JK_PREC_MIXED = 1
JK_PREC_MIXED_FP32ROOTS = 2
PRECISIONS = {'fp64': JK_PREC_FP64, 'mixed': JK_PREC_MIXED, 'mixed-fp32roots': JK_PREC_MIXED_FP32ROOTS}


class JKStats(ctypes.Structure):
    _fields_ = [('quartets_fp64', ctypes.c_int64),
                ('quartets_fp32', ctypes.c_int64),
                ('prim_quartets_fp64', ctypes.c_int64),
                ('prim_quartets_fp32', ctypes.c_int64),
                ('flops_fp64', ctypes.c_int64),
                ('flops_fp32', ctypes.c_int64),
                ('kernel_launches', ctypes.c_int32),
                ('n_classes', ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_lock = threading.Lock()

EXPORTS = ('jk_opt_create', 'jk_opt_destroy', 'jk_opt_nao', 'jk_opt_npairs',
           'jk_opt_get_qcond', 'jk_build', 'jk_last_error', 'jk_n_quartet_classes',
           'jk_opt_time_classes', 'jk_opt_class_times', 'jk_probe_fma', 'jk_int1e',
           'jk_int1e_last_error', 'jk_opt_create_batch', 'jk_build_batch', 'jk_opt_ntot',
           'jk_opt_tune', 'jk_opt_set_variant', 'jk_opt_get_variant', 'jk_opt_set_mol_ndm',
           'jk_build_rsh', 'jk_opt_set_deterministic', 'jk_energy_grad', 'jk_opt_natm', 'jk_sparse_mm')


def load(path=None):
    """Load the library (building it first if it does not exist)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            from ..csrc import build as _build
            _build.build()
        lib = ctypes.CDLL(path)
        vp, i32, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        lib.jk_opt_create.argtypes = [vp, i32, vp, i32, vp, i32, dp, i32, ctypes.POINTER(vp)]
        lib.jk_opt_create.restype = i32
        lib.jk_opt_destroy.argtypes = [vp]
        lib.jk_opt_destroy.restype = None
        lib.jk_opt_nao.argtypes = [vp]
        lib.jk_opt_nao.restype = i32
        lib.jk_opt_npairs.argtypes = [vp]
        lib.jk_opt_npairs.restype = i32
        lib.jk_opt_get_qcond.argtypes = [vp, vp]
        lib.jk_opt_get_qcond.restype = i32
        lib.jk_build.argtypes = [vp, vp, i32, i32, i32, i32, i32, i32, dp, vp, vp, vp,
                                 ctypes.POINTER(JKStats)]
        lib.jk_build.restype = i32
        lib.jk_last_error.argtypes = []
        lib.jk_last_error.restype = ctypes.c_char_p
        lib.jk_n_quartet_classes.argtypes = []
        lib.jk_n_quartet_classes.restype = i32
        lib.jk_opt_time_classes.argtypes = [vp, i32]
        lib.jk_opt_time_classes.restype = i32
        lib.jk_opt_class_times.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
        lib.jk_opt_class_times.restype = i32
        lib.jk_probe_fma.argtypes = [vp, i32, i32, i32, vp]
        lib.jk_probe_fma.restype = i32
        lib.jk_int1e.argtypes = [vp, i32, vp, i32, vp, i32, vp, vp, vp, vp]
        lib.jk_int1e.restype = i32
        lib.jk_int1e_last_error.argtypes = []
        lib.jk_int1e_last_error.restype = ctypes.c_char_p
        lib.jk_opt_create_batch.argtypes = [vp, i32, vp, i32, vp, i32, vp, vp, i32, vp, dp, i32,
                                            ctypes.POINTER(vp)]
        lib.jk_opt_create_batch.restype = i32
        lib.jk_build_batch.argtypes = [vp, vp, i32, i32, i32, i32, i32, dp, vp, vp, vp,
                                       ctypes.POINTER(JKStats)]
        lib.jk_build_batch.restype = i32
        lib.jk_build_rsh.argtypes = [vp, vp, i32, i32, i32, i32, i32, dp, dp, dp, i32, dp, vp, vp, vp,
                                     ctypes.POINTER(JKStats)]
        lib.jk_build_rsh.restype = i32
        lib.jk_opt_ntot.argtypes = [vp]
        lib.jk_opt_ntot.restype = ctypes.c_longlong
        lib.jk_opt_tune.argtypes = [vp, vp, i32, i32, i32, dp, vp, i32]
        lib.jk_opt_tune.restype = i32
        lib.jk_opt_set_variant.argtypes = [vp, i32, i32, i32, i32]
        lib.jk_opt_set_variant.restype = i32
        lib.jk_opt_get_variant.argtypes = [vp, i32, i32, vp, vp]
        lib.jk_opt_get_variant.restype = i32
        lib.jk_opt_set_mol_ndm.argtypes = [vp, vp]
        lib.jk_opt_set_mol_ndm.restype = i32
        lib.jk_opt_set_deterministic.argtypes = [vp, i32]
        lib.jk_opt_set_deterministic.restype = i32
        lib.jk_energy_grad.argtypes = [vp, vp, i32, i32, dp, dp, dp, dp, dp, vp, vp, vp]
        lib.jk_energy_grad.restype = i32
        lib.jk_opt_natm.argtypes = [vp]
        lib.jk_opt_natm.restype = i32
        lib.jk_sparse_mm.argtypes = [i32, vp, vp, vp, i32, i32, i32, i32, vp, vp, vp]
        lib.jk_sparse_mm.restype = i32
        _lib = lib
        return lib


def check(code, what):
    if code != 0:
        msg = load().jk_last_error().decode(errors='replace')
        raise RuntimeError('%s failed (%d): %s' % (what, code, msg))
