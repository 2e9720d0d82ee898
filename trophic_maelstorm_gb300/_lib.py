"""ctypes bindings of include/tm.h (libtm.so).

The library is the product: there is no CPU fallback.  Importing the bindings
without a built libtm.so raises, and every call that fails raises TMError.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libtm.so")

TM_OK, TM_ERR_INVALID, TM_ERR_CUDA, TM_ERR_NOMEM, TM_ERR_STATE, TM_ERR_TIMEOUT = 0, -1, -2, -3, -4, -5
TM_MLP_NPARAMS = 33794
TM_STATUS_NAN, TM_STATUS_NEGATIVE, TM_STATUS_SAMPLER_CAP, TM_STATUS_WAIT_TIMEOUT = 0x1, 0x2, 0x4, 0x8
TM_PROBE_SAMPLER_CAP1, TM_PROBE_TILE_WAIT, TM_PROBE_MLP_WAIT = 0x1, 0x2, 0x4
TM_FP64, TM_FP32 = 0, 1
TM_REM_EULER_EXACT, TM_REM_RK4 = 0, 1
TM_SAMPLER_EXACT, TM_SAMPLER_REF_GAUSS100, TM_SAMPLER_OFF = 0, 1, 2
TM_STENCIL_5, TM_STENCIL_9 = 5, 9
TM_FKE_WS_MAX_RADIUS = 127

# every symbol include/tm.h declares
EXPORTS = (
    "tm_abi_version", "tm_error_string", "tm_create", "tm_destroy", "tm_stream", "tm_sync",
    "tm_batch_create_dp", "tm_batch_create_rietkerk", "tm_batch_destroy", "tm_batch_total_elems",
    "tm_batch_instance_offset", "tm_batch_field_stride", "tm_batch_num_fields", "tm_batch_obs_width",
    "tm_batch_step", "tm_batch_upload", "tm_batch_download", "tm_batch_upload_device",
    "tm_batch_download_device", "tm_batch_snapshot", "tm_batch_advance", "tm_batch_enqueue_steps",
    "tm_batch_set_launch", "tm_batch_get_launch", "tm_batch_autotune", "tm_run_dp", "tm_run_rietkerk",
    "tm_layout", "tm_observe_noalloc", "tm_power_spectrum_device", "tm_batch_power_spectrum",
    "tm_batch_set_site_coeff", "tm_batch_box_means", "tm_fke_advdiff_device",
    "tm_mlp_create", "tm_mlp_destroy", "tm_mlp_set_params", "tm_mlp_get_params", "tm_mlp_set_data",
    "tm_mlp_loss_grad", "tm_mlp_train", "tm_mlp_predict", "tm_set_test_probe",
    "tm_fke_workspace_bytes", "tm_fke_advdiff_device_ws", "tm_batch_set_spreading",
)


class TMError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__(f"{what}: {error_string(code)} ({code})" if what else f"{error_string(code)} ({code})")


class Instance(C.Structure):
    _fields_ = [("L", C.c_int32), ("reserved", C.c_int32), ("seed", C.c_uint64), ("a", C.c_double),
                ("a_step", C.c_double)]


class DPModel(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("b", "c", "D", "sigma", "dt", "dx", "clamp_lo", "clamp_eps")] + \
               [(n, C.c_int32) for n in ("remainder", "sampler", "deterministic", "stencil", "integrator",
                                         "reserved")]


class RietkerkModel(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("alpha", "k2", "W0", "gmax", "k1", "c", "d", "rW", "DP", "DW", "DO",
                                          "sigma", "dt", "dx", "clamp_lo", "clamp_eps")] + \
               [("sampler", C.c_int32), ("deterministic", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -m trophic_maelstorm_gb300.build` "
                               "(the integrator has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp, i64, u32p, dp = C.c_void_p, C.c_int64, C.POINTER(C.c_uint32), C.POINTER(C.c_double)
        i64p = C.POINTER(C.c_int64)
        fp = C.POINTER(C.c_float)
        sig = {
            "tm_abi_version": ([], C.c_int),
            "tm_error_string": ([C.c_int], C.c_char_p),
            "tm_create": ([C.POINTER(vp), C.c_int], C.c_int),
            "tm_destroy": ([vp], C.c_int),
            "tm_stream": ([vp], vp),
            "tm_sync": ([vp], C.c_int),
            "tm_batch_create_dp": ([vp, C.POINTER(DPModel), C.POINTER(Instance), C.c_int, C.c_int, C.POINTER(vp)],
                                   C.c_int),
            "tm_batch_create_rietkerk": ([vp, C.POINTER(RietkerkModel), C.POINTER(Instance), C.c_int, C.c_int,
                                          C.POINTER(vp)], C.c_int),
            "tm_batch_destroy": ([vp], C.c_int),
            "tm_batch_total_elems": ([vp], i64),
            "tm_batch_instance_offset": ([vp, C.c_int], i64),
            "tm_batch_field_stride": ([vp, C.c_int], i64),
            "tm_batch_num_fields": ([vp], C.c_int),
            "tm_batch_obs_width": ([vp], C.c_int),
            "tm_batch_step": ([vp], i64),
            "tm_batch_upload": ([vp, vp, i64], C.c_int),
            "tm_batch_download": ([vp, vp], C.c_int),
            "tm_batch_upload_device": ([vp, vp, i64], C.c_int),
            "tm_batch_download_device": ([vp, vp], C.c_int),
            "tm_batch_snapshot": ([vp, C.c_int, vp], C.c_int),
            "tm_batch_advance": ([vp, i64, i64p, C.c_int, dp, u32p], C.c_int),
            "tm_batch_enqueue_steps": ([vp, i64], C.c_int),
            "tm_batch_set_launch": ([vp, C.c_int, C.c_int], C.c_int),
            "tm_batch_get_launch": ([vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
            "tm_batch_autotune": ([vp, C.c_int], C.c_int),
            "tm_run_dp": ([vp, C.POINTER(DPModel), C.POINTER(Instance), C.c_int, C.c_int, vp, i64, i64p, C.c_int,
                           dp, u32p, vp], C.c_int),
            "tm_run_rietkerk": ([vp, C.POINTER(RietkerkModel), C.POINTER(Instance), C.c_int, C.c_int, vp, i64, i64p,
                                 C.c_int, dp, u32p, vp], C.c_int),
            "tm_layout": ([C.POINTER(Instance), C.c_int, C.c_int, i64p, i64p], i64),
            "tm_observe_noalloc": ([vp, C.c_int, C.POINTER(C.c_int32), i64p, C.c_int, vp, vp], C.c_int),
            "tm_power_spectrum_device": ([vp, C.c_int, C.c_int, C.c_double, vp, dp, dp, C.c_int,
                                          C.POINTER(C.c_int)], C.c_int),
            "tm_batch_power_spectrum": ([vp, C.c_int, C.c_int, C.c_double, dp, dp, C.c_int, C.POINTER(C.c_int)],
                                        C.c_int),
            "tm_batch_set_site_coeff": ([vp, vp], C.c_int),
            "tm_batch_box_means": ([vp, C.c_int, C.c_int, C.c_int, dp], C.c_int),
            "tm_fke_advdiff_device": ([vp, vp, vp, vp, C.c_int, C.c_int, C.c_double, C.c_double, dp, C.c_int, dp,
                                       C.c_int, vp, vp], C.c_int),
            "tm_mlp_create": ([vp, fp, C.POINTER(vp)], C.c_int),
            "tm_mlp_destroy": ([vp], C.c_int),
            "tm_mlp_set_params": ([vp, fp], C.c_int),
            "tm_mlp_get_params": ([vp, fp], C.c_int),
            "tm_mlp_set_data": ([vp, fp, fp, fp, C.c_int], C.c_int),
            "tm_mlp_loss_grad": ([vp, C.c_float, dp, fp], C.c_int),
            "tm_mlp_train": ([vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, dp], C.c_int),
            "tm_mlp_predict": ([vp, fp, C.c_int, fp], C.c_int),
            "tm_set_test_probe": ([vp, C.c_uint32], C.c_int),
            "tm_batch_set_spreading": ([vp, C.c_int, C.c_int, C.c_int], C.c_int),
            "tm_fke_workspace_bytes": ([C.c_int, C.c_int], C.c_size_t),
            "tm_fke_advdiff_device_ws": ([vp, vp, vp, vp, C.c_int, C.c_int, C.c_double, C.c_double, dp, C.c_int, dp,
                                          C.c_int, vp, vp, C.c_size_t, vp], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def error_string(code):
    try:
        return lib().tm_error_string(code).decode()
    except Exception:  # noqa: BLE001 - message only
        return "error"


def check(code, what=""):
    if code != TM_OK:
        raise TMError(code, what)
    return code
