"""ctypes binding of the C ABI in include/fdas_gb300.h.

The shared library is built in-tree (``python -m fdas_gb300.build`` or
``__graft_entry__.build()``).  There is no fallback: if the library is missing
or cannot be loaded, every entry point raises.
"""

import ctypes
import pathlib

_PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = _PKG / "libfdas_gb300.so"

# fdas_status
OK, ERR_INVALID_ARG, ERR_OUT_OF_MEMORY, ERR_CUDA, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_CAPACITY, ERR_STATE, \
    ERR_NO_DEVICE = range(9)
STATUS_NAMES = ["OK", "INVALID_ARG", "OUT_OF_MEMORY", "CUDA", "TIMEOUT", "UNSUPPORTED", "CAPACITY", "STATE",
                "NO_DEVICE"]

# fdas_set_fault_injection flags
INJECT_FTC_STALL = 1
INJECT_HSUM_STALL = 2

# fdas_template_layout
TEMPLATES_FFT_P4, TEMPLATES_FFT_NATURAL, TEMPLATES_TIME_DOMAIN = 0, 1, 2


LOG_FN = ctypes.CFUNCTYPE(None, ctypes.c_char_p, ctypes.c_void_p)


class FdasConfig(ctypes.Structure):
    _fields_ = [
        ("n_frequency_bins", ctypes.c_uint32),
        ("n_templates", ctypes.c_uint32),
        ("max_template_len", ctypes.c_uint32),
        ("tile_overlap", ctypes.c_uint32),
        ("n_planes", ctypes.c_uint32),
        ("candidate_capacity", ctypes.c_uint32),
        ("candidates_per_plane_compat", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        ("buffer_mode", ctypes.c_uint32),
        ("sync_pipeline", ctypes.c_uint32),
        ("recheck", ctypes.c_uint32),
        ("recheck_band", ctypes.c_float),
        ("overlap", ctypes.c_uint32),
        ("precision", ctypes.c_uint32),
        ("trace_enqueue", ctypes.c_uint32),
        ("log_fn", LOG_FN),
        ("log_user", ctypes.c_void_p),
        ("stream_priority", ctypes.c_int32),
    ]


class FdasCandidate(ctypes.Structure):
    _fields_ = [("harmonic", ctypes.c_uint32), ("template_num", ctypes.c_int32), ("bin", ctypes.c_uint32),
                ("power", ctypes.c_float)]


_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int32
_INT = ctypes.c_int

# name -> (restype, argtypes); the exported symbols of include/fdas_gb300.h
SIGNATURES = {
    "fdas_default_config": (None, [ctypes.POINTER(FdasConfig), _U32]),
    "fdas_initialise_accelerator": (_INT, [ctypes.POINTER(FdasConfig), ctypes.POINTER(_P)]),
    "fdas_destroy": (None, [_P]),
    "fdas_last_error": (ctypes.c_char_p, [_P]),
    "fdas_upload_templates": (_INT, [_P, _P, _INT, _INT]),
    "fdas_upload_thresholds": (_INT, [_P, _P, _INT]),
    "fdas_perform_input_tiling": (_INT, [_P, _P, _INT]),
    "fdas_perform_ft_convolution": (_INT, [_P, _INT, _INT]),
    "fdas_perform_harmonic_summing": (_INT, [_P, _P, _INT, _INT]),
    "fdas_launch": (_INT, [_P, _P, _P, _P, _P, _INT, _INT]),
    "fdas_wait": (_INT, [_P, _INT]),
    "fdas_end_pipeline": (_INT, [_P, _INT]),
    "fdas_retrieve_tiles": (_INT, [_P, _P, _INT]),
    "fdas_retrieve_fop": (_INT, [_P, _P, _INT]),
    "fdas_inject_fop": (_INT, [_P, _P, _INT]),
    "fdas_retrieve_candidates": (_INT, [_P, _P, _P, _INT]),
    "fdas_retrieve_candidate_list": (_INT, [_P, _P, _U32, ctypes.POINTER(_U32), ctypes.POINTER(_U32), _INT]),
    "fdas_print_stats": (None, [_P, _INT, _INT]),
    "fdas_print_events": (None, [_P, _INT]),
    "fdas_set_log": (None, [_P, LOG_FN, _P]),
    "fdas_set_wait_timeout": (_INT, [_P, ctypes.c_int64]),
    "fdas_set_fault_injection": (_INT, [_P, _U32]),
    "fdas_get_stage_times": (_INT, [_P, _INT, _P]),
    "fdas_get_input_sz": (_U32, [_P]),
    "fdas_get_tiles_sz": (_U32, [_P]),
    "fdas_get_templates_sz": (_U32, [_P]),
    "fdas_get_thresholds_sz": (_U32, [_P]),
    "fdas_get_fop_sz": (_U32, [_P]),
    "fdas_get_candidate_list_sz": (_U32, [_P]),
    "fdas_host_alloc": (_INT, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "fdas_host_free": (None, [_P]),
    "fdas_host_register": (_INT, [_P, ctypes.c_size_t]),
    "fdas_host_unregister": (_INT, [_P]),
    "fdas_enqueue_search_device": (_INT, [_P, _P, _P, _INT, _INT]),
    "fdas_synchronize": (_INT, [_P, _INT]),
    "fdas_get_stream": (_P, [_P, _INT]),
    "fdas_get_counters": (_INT, [_P, _INT, _P, _U32]),
    "fdas_retrieve_candidates_ring": (_INT, [_P, _P, _P, _INT, _INT]),
    "fdas_server_default_config": (None, [_P]),
    "fdas_server_create": (_INT, [_P, _P, _INT, _U32, _U32, _P]),
    "fdas_server_submit": (_INT, [_P, _P, _U32, _U32, _U32, _U32, _P, _P]),
    "fdas_server_wait": (_INT, [_P, ctypes.c_uint64, ctypes.c_int32, _P, _U32, _P, _P, _P]),
    "fdas_server_stats": (_INT, [_P, _P, _U32]),
    "fdas_server_last_error": (ctypes.c_char_p, [_P]),
    "fdas_server_destroy": (None, [_P]),
    "fdas_batch_default_config": (None, [_P]),
    "fdas_batch_create": (_INT, [_P, _P, _INT, _U32, _U32, _U32, _P, _P]),
    "fdas_batch_set_inputs": (_INT, [_P, _P, _INT]),
    "fdas_batch_input": (_P, [_P]),
    "fdas_batch_run": (_INT, [_P, _P, _INT]),
    "fdas_batch_wait": (_INT, [_P]),
    "fdas_batch_trial": (_P, [_P, _U32]),
    "fdas_batch_info": (_INT, [_P, _P, _U32, _P, _U32]),
    "fdas_batch_set_tuning": (_INT, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "fdas_batch_set_groups": (_INT, [_P, ctypes.c_int32]),
    "fdas_batch_last_error": (ctypes.c_char_p, [_P]),
    "fdas_batch_destroy": (None, [_P]),
    "fdas_reshape": (_INT, [_P, _U32, _U32, _U32, _U32, _U32]),
    "fdas_series_to_spectrum": (_INT, [_P, _P, ctypes.c_uint64, _INT, ctypes.c_float, _P, _INT]),
    "fdas_ft_convolution_noalloc": (_INT, [_P, _U32, _P, _INT, _U32, _U32, _INT, _P, ctypes.c_uint64, _P, _P]),
    "fdas_version": (ctypes.c_char_p, []),
}

_lib = None


def load():
    """Load the in-tree library (raises if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is not built; run __graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib
