"""ctypes binding of the engine's C ABI (include/pam.h).

The library is built in-tree by ``pseudoacousticmodeling_gb300.build``; this
module never falls back to anything else: if the shared library is missing or
fails to load, importing the engine raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libpam_gb300.so")

PAM_OK = 0
ERRORS = {-1: "PAM_E_ARG", -2: "PAM_E_CUDA", -3: "PAM_E_STATE", -4: "PAM_E_UNSUPPORTED", -5: "PAM_E_NUMERIC"}

# Every symbol include/pam.h declares, with (restype, argtypes).
_p = ctypes.c_void_p
_i = ctypes.c_int
_f = ctypes.c_float
_pi = ctypes.POINTER(ctypes.c_int)
_pf = ctypes.POINTER(ctypes.c_float)
_pd = ctypes.POINTER(ctypes.c_double)


class PamConfig(ctypes.Structure):
    _fields_ = [("nz", _i), ("nx", _i), ("n_abc", _i), ("dz", _f), ("dx", _f), ("dt", _f), ("nt", _i),
                ("itlag", _i), ("fcut", _f), ("approximation", _i), ("boundary", _i), ("max_shots", _i)]


SIGNATURES = {
    "pam_create": (_i, [ctypes.POINTER(PamConfig), _i, ctypes.POINTER(_p)]),
    "pam_destroy": (None, [_p]),
    "pam_last_error": (ctypes.c_char_p, [_p]),
    "pam_set_models": (_i, [_p, _p, _p, _p, _p]),
    "pam_set_wavelet": (_i, [_p, _p]),
    "pam_set_receivers": (_i, [_p, _i, _p, _p, _i]),
    "pam_forward": (_i, [_p, _i, _p, _p, _p, _p]),
    "pam_forward_device": (_i, [_p, _i, _p, _p, _p, _p]),
    "pam_begin": (_i, [_p, _i, _p, _p]),
    "pam_step": (_i, [_p, _i]),
    "pam_read_seismograms": (_i, [_p, _p]),
    "pam_read_wavefield": (_i, [_p, _i, _p]),
    "pam_rtm": (_i, [_p, _i, _p, _p, _p, _i, _i, _p]),
    "pam_rtm_result": (_i, [_p, _p, _p, _i]),
    "pam_rtm_reset": (_i, [_p]),
    "pam_fwi_gradient": (_i, [_p, _i, _p, _p, _p, _i, _i, _pd, _p]),
    "pam_fwi_result": (_i, [_p, _p, _p]),
    "pam_misfit_gradient": (_i, [_p, _i, _p, _p, _p, _i, _i, _pd, _p, _p]),
    "pam_adjoint_gradient": (_i, [_p, _i, _p, _p, _p, _i, _i, _p, _p]),
    "pam_check_stability": (_i, [_p, _pf, _pf]),
    "pam_grid_info": (_i, [_p, _pi, _pi, _pi]),
    "pam_autotune": (_i, [_p, _i]),
    "pam_smooth_model": (_i, [_p, _i, _i, ctypes.c_float, _i, _p]),
    "pam_stability_limits": (_i, [_i, _i, _i, _p, _p, _p, _p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, _p, _p]),
    "pam_set_mute": (_i, [_p, _i, _p, _p, _i, _p, _p, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "pam_set_multiparameter": (_i, [_p, _i]),
    "pam_fwi_multiparameter_result": (_i, [_p, _p, _p, _p]),
    "pam_set_random_boundary": (_i, [_p, ctypes.c_float, ctypes.c_float, ctypes.c_ulonglong]),
    "pam_random_boundary": (_i, [_p, _i, _i, _i, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 ctypes.c_float, ctypes.c_ulonglong, _p]),
    "pam_segment_height": (_i, [_p, _i]),
    "pam_profile_enable": (_i, [_p, _i]),
    "pam_profile_read": (_i, [_p, _pd, _pi, _i]),
    "pam_misfit_noalloc": (_i, [_p, _p, ctypes.c_longlong, _pd, _p]),
    "pam_plan_checkpoints": (_i, [_p, ctypes.c_longlong, _i, _pi, _pi]),
    "pam_set_damping": (_i, [_p, _p]),
    "pam_laplacian_filter": (_i, [_p, _i, _i, ctypes.c_float, ctypes.c_float, _p]),
}

_LIB = None


def load(path=LIB_PATH):
    """Load the engine library (building is the caller's job: build.build())."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"engine library not built: {path} is missing "
                           "(run pseudoacousticmodeling_gb300.build.build())")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class PamError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code
