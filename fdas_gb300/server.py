"""Served form: Python view of the request server (fdas_server_* in
include/fdas_gb300.h).

    srv = Server(bank)                      # bank resident on the device
    rid = srv.submit(spectrum, thresholds)  # copies the spectrum to the device, returns
    rec, n_total, n_dropped, latency_ms = srv.result(rid)

Requests of any length up to ``max_bins``, with the full bank or a contiguous
odd range of its rows (``HALF_BANK`` = the z = -21..+21 rows of the 85-row
bank), and 1..``max_planes`` planes, run concurrently on the device.
"""
import ctypes

import numpy as np

from . import _lib
from .fdas import FDAS

HALF_BANK = (21, 43)


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_bins", ctypes.c_uint32), ("min_class_bins", ctypes.c_uint32),
                ("max_planes", ctypes.c_uint32), ("max_slots", ctypes.c_uint32),
                ("hbm_budget_bytes", ctypes.c_uint64), ("candidate_capacity", ctypes.c_uint32)]


class Server:
    def __init__(self, bank, layout=None, device=0, max_bins=1 << 21, max_slots=8, max_planes=16,
                 hbm_budget_bytes=0, candidate_capacity=1 << 20, min_class_bins=1 << 15):
        self._lib = _lib.load()
        bank = np.ascontiguousarray(bank, dtype=np.complex64)
        if bank.ndim != 2:
            raise ValueError("bank must be a 2-D complex64 array")
        if layout is None:
            layout = FDAS.TemplatesFFTP4 if bank.shape[1] == 2048 else FDAS.TemplatesTimeDomain
        cfg = ServerConfig()
        self._lib.fdas_server_default_config(ctypes.byref(cfg))
        cfg.device, cfg.max_bins, cfg.max_slots, cfg.max_planes = device, max_bins, max_slots, max_planes
        cfg.hbm_budget_bytes, cfg.candidate_capacity, cfg.min_class_bins = hbm_budget_bytes, candidate_capacity, \
            min_class_bins
        self._bank = bank
        self.n_rows = bank.shape[0]
        self._s = ctypes.c_void_p()
        st = self._lib.fdas_server_create(ctypes.byref(cfg), ctypes.c_void_p(bank.ctypes.data), int(layout),
                                          bank.shape[0], bank.shape[1], ctypes.byref(self._s))
        if st != _lib.OK:
            raise RuntimeError(f"fdas_server_create failed with status {st}")

    def submit(self, spectrum, thresholds, template_rows=None):
        x = np.ascontiguousarray(spectrum, dtype=np.complex64)
        thr = np.ascontiguousarray(thresholds, dtype=np.float32)
        r0, nt = (0, self.n_rows) if template_rows is None else template_rows
        rid = ctypes.c_uint64()
        st = self._lib.fdas_server_submit(self._s, ctypes.c_void_p(x.ctypes.data), x.size, r0, nt, thr.size,
                                          ctypes.c_void_p(thr.ctypes.data), ctypes.byref(rid))
        if st != _lib.OK:
            raise ValueError(f"fdas_server_submit rejected the request (status {st})")
        return rid.value

    def result(self, rid, timeout_ms=-1, capacity=None):
        """(records, n_total, n_dropped, latency_ms); records sorted by
        (harmonic, template, bin).  Raises on a failed request."""
        n_total, n_dropped, lat = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
        st = self._lib.fdas_server_wait(self._s, rid, timeout_ms, None, 0, ctypes.byref(n_total),
                                        ctypes.byref(n_dropped), ctypes.byref(lat))
        if st == _lib.ERR_TIMEOUT:
            raise TimeoutError(f"request {rid} not finished")
        cap = n_total.value if capacity is None else capacity
        out = np.zeros(max(cap, 1), dtype=FDAS.CANDIDATE_DTYPE)
        st = self._lib.fdas_server_wait(self._s, rid, timeout_ms, ctypes.c_void_p(out.ctypes.data), max(cap, 1),
                                        ctypes.byref(n_total), ctypes.byref(n_dropped), ctypes.byref(lat))
        if st == _lib.ERR_TIMEOUT:
            raise TimeoutError(f"request {rid} not finished")
        if st != _lib.OK:
            raise RuntimeError(f"request {rid} failed ({st}): {self._lib.fdas_server_last_error(self._s).decode()}")
        return out[:min(n_total.value, cap)], n_total.value, n_dropped.value, lat.value

    def stats(self):
        v = (ctypes.c_uint64 * 6)()
        self._lib.fdas_server_stats(self._s, v, 6)
        return dict(zip(["completed", "queued", "in_flight", "slots", "slot_bytes", "peak_in_flight"], list(v)))

    def close(self):
        if self._s:
            self._lib.fdas_server_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
