"""ctypes binding of libcrs.so (include/crs.h).

The library is built in-tree by ``create_rate_subs_gb300.build``.  Loading
fails loudly when it is missing and cannot be built: there is no CPU
fallback for the batched evaluation.
"""

import ctypes
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None

CRS_OK = 0
ERRORS = {1: "bad argument", 2: "bad mechanism tables", 3: "CUDA error",
          4: "unsupported", 5: "timeout", 6: "no mechanism bound"}

MODES = {"fp64": 0, "fp64_strict": 1, "mixed": 2, "fp64_tps": 3, "mixed_tps": 4,
         "fp64_warp": 5, "mixed_warp": 6, "gemm": 7, "mixed_tile": 8,
         "fp64_tile": 9}

_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int


class CRSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("libcrs error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


def _sig(lib):
    s = {
        "crs_mech_load": [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_vp)],
        "crs_mech_load_file": [ctypes.c_char_p, ctypes.POINTER(_vp)],
        "crs_mech_inspect": [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_i64)],
        "crs_mech_free": [_vp],
        "crs_mech_dims": [_vp, ctypes.POINTER(_i64)],
        "crs_status": [_vp, _vp, ctypes.POINTER(ctypes.c_int32)],
        "crs_status_reset": [_vp, _vp],
        "crs_eval_conc_batch": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp],
        "crs_eval_rxn_rates_batch": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp],
        "crs_get_rxn_pres_mod_batch": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp],
        "crs_eval_spec_rates_batch": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp],
        "crs_wdot": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _i32, _vp],
        "crs_wdot_host": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _i32],
        "crs_eval_thermo_batch": [_vp, _i64, _vp, _i64, _i32, _vp, _vp],
        "crs_eval_conc_rho_batch": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp],
        "crs_dydt": [_vp, _i64, _vp, _vp, _i64, _vp, _i32, _i32, _vp],
        "crs_dydt_form": [_i32],
        "crs_wdot_stages": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp,
                            _vp, _i32, _vp],
        "crs_bind": [_vp],
        "crs_bind_thread": [_vp],
        "crs_mech_load_host": [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(_vp)],
        "crs_mech_image": [ctypes.c_char_p, ctypes.c_size_t, _vp, ctypes.c_size_t, _vp,
                           ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
        "crs_state_eval_conc": [_vp, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp,
                                _vp],
        "crs_state_eval_rxn_rates": [_vp, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp],
        "crs_state_get_rxn_pres_mod": [_vp, ctypes.c_double, ctypes.c_double, _vp, _vp],
        "crs_state_eval_spec_rates": [_vp, _vp, _vp, _vp, _vp, _vp],
        "crs_state_eval_thermo": [_vp, _i32, ctypes.c_double, _vp],
        "crs_state_eval_conc_rho": [_vp, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp,
                                    _vp, _vp],
        "crs_state_dydt": [_vp, _i32, ctypes.c_double, _vp, _vp],
        "crs_wdot_gemm_noalloc": [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp],
        "crs_gemm_bf16": [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i32, _vp, _vp],
        "crs_mlp_forward": [_vp, _vp, _vp, _i64, _i64, _i64, _i64, _i64, _i32, _vp, _i64,
                            _vp, _i64, _vp, _i64, _vp, _i64, _vp],
        "crs_mlp_infer": [_vp, _i64, _i64, _i32, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _vp],
        "crs_mlp_backward_data": [_vp, _vp, _i64, _i64, _i64, _i64, _i64, _vp, _i64, _vp,
                                  _i64, _vp, _i64, _vp],
        "crs_mlp_backward_weight": [_vp, _vp, _i64, _i64, _i64, _i64, _i64, _i32, _vp, _vp,
                                    _vp],
        "crs_mlp_row_sums": [_vp, _i64, _i64, _i64, _vp, _vp],
        "crs_mlp_loss_grad": [_vp, _i64, _vp, _i64, _i64, _i64, _i64, ctypes.c_float, _vp,
                              _i64, _vp, _i64, _vp, _vp],
        "crs_adam_step": [_vp, _vp, _vp, _vp, _i64, _i64, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, ctypes.c_float, _i32, _vp, _i64, _vp, _i64, _vp],
        "crs_surrogate_features": [_i64, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _vp, _vp,
                                   _i64, _vp, _i64, _i32, _vp, _vp, _vp],
        "crs_surrogate_output": [_i64, _vp, _i64, _i32, _vp, _vp, _vp, _i32, ctypes.c_float,
                                 _vp, _vp, _i64, _vp, _vp],
        "crs_surrogate_output2": [_i64, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _i32,
                                  ctypes.c_float, ctypes.c_float, _vp, _i64, ctypes.c_float,
                                  _vp, _vp, _i64, _vp, _vp, _vp],
        "crs_surrogate_disagreement": [_i64, _vp, _vp, _i64, _i32, ctypes.c_float,
                                       ctypes.c_float, _vp, _i64, _i32, _vp],
        "crs_select": [_i64, _vp, _vp, _vp, _vp],
        "crs_gather_states": [_i64, _vp, _vp, _vp, _vp, _i64, _i32, _vp, _vp, _vp, _i64, _vp],
        "crs_scatter_wdot": [_i64, _vp, _vp, _i64, _i32, _vp, _i64, _vp],
        "eval_conc": [ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _vp],
        "eval_rxn_rates": [ctypes.c_double, ctypes.c_double, _vp, _vp, _vp],
        "get_rxn_pres_mod": [ctypes.c_double, ctypes.c_double, _vp, _vp],
        "eval_spec_rates": [_vp, _vp, _vp, _vp, _vp],
        "eval_h": [ctypes.c_double, _vp],
        "eval_u": [ctypes.c_double, _vp],
        "eval_cv": [ctypes.c_double, _vp],
        "eval_cp": [ctypes.c_double, _vp],
        "eval_conc_rho": [ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _vp],
        "dydt": [ctypes.c_double, ctypes.c_double, _vp, _vp],
    }
    for name, args in s.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = None if name in ("eval_conc", "eval_rxn_rates", "get_rxn_pres_mod",
                                     "eval_spec_rates", "eval_h", "eval_u", "eval_cv",
                                     "eval_cp", "eval_conc_rho", "dydt") else ctypes.c_int
    lib.crs_last_error.argtypes = []
    lib.crs_last_error.restype = ctypes.c_char_p
    return lib


def load(build_if_missing=True):
    """The loaded libcrs (built first if missing and nvcc is available)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise OSError("libcrs.so is not built (%s); run "
                              "python -m create_rate_subs_gb300.build" % path)
            _build.build()
        _lib = _sig(ctypes.CDLL(path))
        return _lib


def check(rc):
    if rc != CRS_OK:
        msg = load().crs_last_error().decode(errors="replace")
        raise CRSError(rc, msg)
    return rc


def last_error():
    return load().crs_last_error().decode(errors="replace")
