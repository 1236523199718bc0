"""Batched form: Python view of fdas_batch_* (include/fdas_gb300.h).

    b = Batch(bank, n_bins=[...])       # one allocation for all trials
    b.set_inputs(spectra)               # list of complex64 arrays (or one concatenated array)
    b.run(thresholds)                   # autotune + CUDA-graph capture on the first call
    rec, n_total, n_dropped = b.trial(i).retrieve_candidate_list(FDAS.A)
"""
import ctypes

import numpy as np

from . import _lib
from .fdas import FDAS


class BatchConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("n_planes", ctypes.c_uint32), ("candidate_capacity", ctypes.c_uint32),
                ("candidates_per_plane_compat", ctypes.c_uint32), ("autotune", ctypes.c_uint32),
                ("recheck", ctypes.c_uint32)]


class Batch:
    def __init__(self, bank, n_bins, n_planes=8, device=0, candidate_capacity=1 << 18, autotune=True, layout=None):
        self._lib = _lib.load()
        bank = np.ascontiguousarray(bank, dtype=np.complex64)
        if layout is None:
            layout = FDAS.TemplatesFFTP4 if bank.shape[1] == 2048 else FDAS.TemplatesTimeDomain
        self.n_bins = np.ascontiguousarray(n_bins, dtype=np.uint32)
        cfg = BatchConfig()
        self._lib.fdas_batch_default_config(ctypes.byref(cfg))
        cfg.device, cfg.n_planes, cfg.candidate_capacity, cfg.autotune = device, n_planes, candidate_capacity, \
            int(bool(autotune))
        self.n_planes = n_planes
        self._b = ctypes.c_void_p()
        st = self._lib.fdas_batch_create(ctypes.byref(cfg), ctypes.c_void_p(bank.ctypes.data), int(layout),
                                         bank.shape[0], bank.shape[1], self.n_bins.size,
                                         ctypes.c_void_p(self.n_bins.ctypes.data), ctypes.byref(self._b))
        if st != _lib.OK:
            raise RuntimeError(f"fdas_batch_create failed ({st}): {self.last_error()}")
        self._keep = None

    def last_error(self):
        return (self._lib.fdas_batch_last_error(self._b if self._b else None) or b"").decode()

    def _ok(self, st, what):
        if st != _lib.OK:
            raise RuntimeError(f"{what} failed ({_lib.STATUS_NAMES[st]}): {self.last_error()}")

    def set_inputs(self, spectra):
        """Host spectra: a list of per-trial complex64 arrays, or one concatenated array."""
        x = spectra if isinstance(spectra, np.ndarray) else np.concatenate(spectra)
        x = np.ascontiguousarray(x, dtype=np.complex64)
        if x.size != int(self.n_bins.sum()):
            raise ValueError("the spectra must hold sum(n_bins) values")
        self._keep = x  # the copy is asynchronous
        self._ok(self._lib.fdas_batch_set_inputs(self._b, ctypes.c_void_p(x.ctypes.data), 0), "set_inputs")

    def set_inputs_device(self, ptr):
        self._ok(self._lib.fdas_batch_set_inputs(self._b, ctypes.c_void_p(ptr), 1), "set_inputs")

    def run(self, thresholds, wait=True):
        thr = np.ascontiguousarray(thresholds, dtype=np.float32)
        if thr.size != self.n_planes:
            raise ValueError("one threshold per plane")
        self._thr = thr
        self._ok(self._lib.fdas_batch_run(self._b, ctypes.c_void_p(thr.ctypes.data), int(bool(wait))), "run")

    def wait(self):
        self._ok(self._lib.fdas_batch_wait(self._b), "wait")

    def trial(self, i):
        h = self._lib.fdas_batch_trial(self._b, int(i))
        if not h:
            raise IndexError(i)
        return FDAS.view(h)

    def info(self):
        v = (ctypes.c_int32 * 7)()
        ms = (ctypes.c_float * 16)()
        self._lib.fdas_batch_info(self._b, v, 7, ms, 16)
        return {"ftc_split": "warp pair 32x64" if v[0] == 2 else "one warp 64x32", "ftc_ctas_per_sm": v[1],
                "hsum_lean": bool(v[2]), "tuned": bool(v[3]), "tiles": v[4], "tune_ms": list(ms)[:v[5]],
                "ftc_launches": v[6]}

    def set_tuning(self, ftc_split, ftc_ctas_per_sm, hsum_lean):
        self._ok(self._lib.fdas_batch_set_tuning(self._b, int(ftc_split), int(ftc_ctas_per_sm), int(bool(hsum_lean))),
                 "set_tuning")

    def set_groups(self, groups):
        """FT-convolution launches the trials are grouped into (1..16; 1: one
        persistent launch over the whole queue); skips the autotuner."""
        self._ok(self._lib.fdas_batch_set_groups(self._b, int(groups)), "set_groups")

    def close(self):
        if self._b:
            self._lib.fdas_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
