"""ctypes binding of liborbkit_gb300.so (the C ABI in include/orbkit_gb300.h).

There is no CPU fallback: if the library is missing or no GB300 is visible the
calls raise.  Device buffers are torch tensors (plumbing only); their data
pointers and torch's current CUDA stream are handed to the C ABI.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborbkit_gb300.so")

OKG_OK = 0


class OkgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("orbkit_gb300: %s (status %d): %s" % (_status_name(status), status, msg))
        self.status = status


class OkgGrid(ctypes.Structure):
    _fields_ = [("d_x", ctypes.c_void_p), ("d_y", ctypes.c_void_p), ("d_z", ctypes.c_void_p),
                ("npts", ctypes.c_int64), ("offset", ctypes.c_int64),
                ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("regular", ctypes.c_int32)]


_lib = None
_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

# name -> (restype, argtypes); every compute entry point returns an int status
SIGNATURES = {
    "okg_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "okg_last_error": (ctypes.c_char_p, []),
    "okg_version": (ctypes.c_int, []),
    "okg_basis_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _c_int_p, _c_int_p, _c_int_p, _c_int_p,
                                        ctypes.c_int, _c_dbl_p, ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p,
                                        ctypes.POINTER(_vp)]),
    "okg_basis_destroy": (ctypes.c_int, [_vp]),
    "okg_basis_info": (ctypes.c_int, [_vp, _c_int_p, _c_int_p, _c_int_p, _c_int_p, _c_int_p]),
    "okg_basis_set_params": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "okg_basis_set_mixed_order": (ctypes.c_int, [_vp, _vp]),
    "okg_eval_ao": (ctypes.c_int, [_vp, ctypes.POINTER(OkgGrid), ctypes.c_int, _c_int_p, ctypes.c_int, _vp,
                                   ctypes.c_int64, _vp]),
    "okg_eval_mo": (ctypes.c_int, [_vp, ctypes.POINTER(OkgGrid), ctypes.c_int, _vp, ctypes.c_int, _c_int_p,
                                   ctypes.c_int, _vp, ctypes.c_int64, _vp]),
    "okg_rho": (ctypes.c_int, [_vp, ctypes.POINTER(OkgGrid), ctypes.c_int, _vp, _vp, ctypes.c_int, _c_int_p,
                               ctypes.c_int, _vp, _vp, ctypes.c_int64, _vp, _vp]),
    "okg_mixed_plan_create": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(_vp)]),
    "okg_mixed_plan_destroy": (ctypes.c_int, [_vp]),
    "okg_mixed_set_coeffs": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "okg_rho_mixed": (ctypes.c_int, [_vp, ctypes.POINTER(OkgGrid), ctypes.c_int, _vp, _vp, ctypes.c_int64, _vp]),
    "okg_mixed_status": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "okg_diag_fp64_fma_rate": (ctypes.c_int, [ctypes.c_longlong, ctypes.POINTER(ctypes.c_double)]),
    "okg_mo_from_ao": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int64, ctypes.c_int64, _vp,
                                      ctypes.c_int64, _vp]),
    "okg_cart2sph": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_int64,
                                    _vp, ctypes.c_int64, _vp]),
    "okg_mo_products": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_int64, _vp,
                                       ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int64, _vp]),
    "okg_mo_pair_flux": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_int64, _vp,
                                        ctypes.c_int64, ctypes.c_int64, _vp, ctypes.c_int64, _vp]),
}


def _status_name(s):
    return {0: "ok", -1: "invalid argument", -2: "unsupported angular momentum", -3: "invalid derivative code",
            -4: "CUDA error", -5: "allocation failed", -6: "device wait timed out", -7: "unsupported shape",
            -8: "no usable device"}.get(s, "unknown status")


def load(path=None):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OkgError(-8, "%s not built; run `python -m orbkit_gb300.build`" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        if hasattr(L, name):
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
    _lib = L
    return L


def check(status):
    if status != OKG_OK:
        msg = load().okg_last_error()
        raise OkgError(status, msg.decode() if msg else "")
    return status


def ptr(t):
    """Device pointer of a torch tensor (or None)."""
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def int_array(vals):
    arr = (ctypes.c_int * max(1, len(vals)))(*[int(v) for v in vals])
    return arr
