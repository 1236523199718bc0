"""Python mirror of the reference's host class ``FDAS`` (fdas/src/host/FDAS.h:36-187).

Same method names, argument meaning and error behaviour: every method returns
``True`` on success and ``False`` after logging ``[ERROR] ...`` (FDAS.cpp:34-52);
the message is also in ``last_error``.  The work runs in the CUDA library
``libfdas_gb300.so`` through its C ABI; there is no CPU fallback.

Arrays are NumPy: complex64 for spectra / tiles / templates, float32 for the
FOP, thresholds and powers, uint32 for locations.
"""

import ctypes
import sys

import numpy as np

from . import _lib

N_TMPL_PER_ACCEL_SIGN = 42


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _require(a, dtype, size=None, name="array"):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous numpy {np.dtype(dtype).name} array")
    if size is not None and a.size < size:
        raise ValueError(f"{name} must hold at least {size} elements")
    return a


class FDAS:
    # FDAS.h:38-40
    NegativeAccelerations, PositiveAccelerations, AllAccelerations = 0, 1, 2
    A, B = 0, 1
    PerSet, PerStage, Crossed = 0, 1, 2
    # template layouts accepted by upload_templates
    TemplatesFFTP4, TemplatesFFTNatural, TemplatesTimeDomain = (
        _lib.TEMPLATES_FFT_P4, _lib.TEMPLATES_FFT_NATURAL, _lib.TEMPLATES_TIME_DOMAIN)

    def __init__(self, log=None):
        """``log``: a writable text stream (default sys.stderr), like FDAS(std::ostream &)."""
        self._lib = _lib.load()
        self.log = log if log is not None else sys.stderr
        self._h = ctypes.c_void_p()
        self._keep = {0: [], 1: []}
        self.last_error = ""
        self._log_cb = _lib.LOG_FN(self._on_log)
        self.config = None
        self._borrowed = False

    @classmethod
    def view(cls, handle, log=None):
        """An FDAS over a handle owned elsewhere (a trial of a batch); never destroyed here."""
        f = cls(log)
        f._h = ctypes.c_void_p(handle)
        f._borrowed = True
        return f

    # ----------------------------------------------------------- plumbing
    def _on_log(self, line, _user):
        try:
            self.log.write(line.decode() + "\n")
        except Exception:
            pass

    def _check(self, st, what):
        if st == _lib.OK:
            return True
        msg = self._lib.fdas_last_error(self._h if self._h else None)
        self.last_error = (msg or b"").decode()
        self.log.write(f"[ERROR] {what} failed ({_lib.STATUS_NAMES[st]}): {self.last_error}\n")
        self.last_status = st
        return False

    def __del__(self):
        try:
            if self._h and not self._borrowed:
                self._lib.fdas_destroy(self._h)
                self._h = ctypes.c_void_p()
        except Exception:
            pass

    def close(self):
        self.__del__()

    # -------------------------------------------------------- the class API
    def initialise_accelerator(self, input_sz, mode=PerSet, sync_pipeline=False, device=0, n_templates=85,
                               max_template_len=421, tile_overlap=0, n_planes=8, candidate_capacity=0,
                               candidates_per_plane_compat=0, recheck=True, recheck_band=0.0, overlap=False,
                               precision=0, trace_enqueue=False, stream_priority=0):
        """FDAS::initialise_accelerator (FDAS.h:44-49).  The bitstream and the
        OpenCL platform / device selectors become a CUDA device ordinal.
        ``trace_enqueue``: log the reference's per-launch "[INFO] Enqueueing" and
        "%%%" lines (FDAS.cpp:556-575).  ``stream_priority``: CUDA priority of
        the buffer sets' streams (0 default, negative higher)."""
        cfg = _lib.FdasConfig()
        self._lib.fdas_default_config(ctypes.byref(cfg), int(input_sz))
        cfg.n_templates = n_templates
        cfg.max_template_len = max_template_len
        cfg.tile_overlap = tile_overlap
        cfg.n_planes = n_planes
        cfg.candidate_capacity = candidate_capacity
        cfg.candidates_per_plane_compat = candidates_per_plane_compat
        cfg.device = device
        cfg.buffer_mode = int(mode)
        cfg.sync_pipeline = int(bool(sync_pipeline))
        cfg.recheck = int(bool(recheck))
        cfg.recheck_band = float(recheck_band)
        cfg.overlap = int(bool(overlap))
        cfg.precision = int(precision)
        cfg.trace_enqueue = int(bool(trace_enqueue))
        cfg.stream_priority = int(stream_priority)
        cfg.log_fn = self._log_cb  # the "^^^" line of initialisation goes to this log too
        cfg.log_user = None
        if self._h:
            self._lib.fdas_destroy(self._h)
            self._h = ctypes.c_void_p()
        st = self._lib.fdas_initialise_accelerator(ctypes.byref(cfg), ctypes.byref(self._h))
        if st != _lib.OK:
            self._h = ctypes.c_void_p()
            return self._check(st, "initialise_accelerator")
        self._lib.fdas_set_log(self._h, self._log_cb, None)
        self.config = cfg
        return True

    def reshape(self, n_frequency_bins, template_row_begin=0, n_templates=None, tile_overlap=0, n_planes=None):
        """Re-size the idle handle within its initialised sizes (fdas_reshape):
        fewer bins, a contiguous odd range of the uploaded bank's rows (the
        z = -21..+21 half bank is rows 21..63 of the 85-row bank), fewer planes."""
        n_templates = self.config.n_templates if n_templates is None else n_templates
        n_planes = self.config.n_planes if n_planes is None else n_planes
        return self._check(self._lib.fdas_reshape(self._h, int(n_frequency_bins), int(template_row_begin),
                                                  int(n_templates), int(tile_overlap), int(n_planes)), "reshape")

    def upload_templates(self, templates, ab, layout=None):
        """FDAS::upload_templates.  ``templates`` complex64, n_templates x 2048
        spectra in p4 FFT order (the reference's ``..._ft_p4.npy``) unless
        ``layout`` says otherwise; n_templates x max_template_len arrays are
        taken as time-domain taps."""
        t = _require(np.ascontiguousarray(templates), np.complex64, name="templates")
        if layout is None:
            layout = self.TemplatesFFTP4 if t.shape[-1] == 2048 else self.TemplatesTimeDomain
        return self._check(self._lib.fdas_upload_templates(self._h, _ptr(t), int(layout), int(ab)),
                           "upload_templates")

    def upload_thresholds(self, thresholds, ab):
        thr = _require(np.ascontiguousarray(thresholds, dtype=np.float32), np.float32,
                       self.get_thresholds_sz(), "thresholds")
        return self._check(self._lib.fdas_upload_thresholds(self._h, _ptr(thr), int(ab)), "upload_thresholds")

    def perform_input_tiling(self, input, ab):
        """``input`` None: tile the spectrum series_to_spectrum made on ``ab``."""
        x = None if input is None else _require(np.ascontiguousarray(input), np.complex64, self.get_input_sz(),
                                                "input")
        return self._check(self._lib.fdas_perform_input_tiling(self._h, _ptr(x), int(ab)), "perform_input_tiling")

    def series_to_spectrum(self, samples, ab, scale=None, spectrum=None):
        """Upstream step of ft_conv.py:134-143 on the GPU: the N-bin spectrum of
        the first 2N samples, ``fft(samples) * scale`` with the reference's
        ``scale = 1 / (2N)`` by default.  ``samples`` is a float32 numpy array or
        a CUDA tensor (anything with ``data_ptr()``).  The spectrum stays on
        buffer set ``ab`` for perform_input_tiling / launch with input None and
        is copied into ``spectrum`` (complex64[N]) when given."""
        n = self.get_input_sz()
        scale = 1.0 / (2 * n) if scale is None else float(scale)
        out = None if spectrum is None else _require(spectrum, np.complex64, n, "spectrum")
        if hasattr(samples, "data_ptr"):
            if samples.dtype.__str__() != "torch.float32" or not samples.is_cuda or not samples.is_contiguous():
                raise TypeError("samples must be a contiguous float32 CUDA tensor")
            ptr, count, on_dev = ctypes.c_void_p(samples.data_ptr()), samples.numel(), 1
        else:
            x = _require(np.ascontiguousarray(samples), np.float32, None, "samples")
            ptr, count, on_dev = _ptr(x), x.size, 0
        return self._check(self._lib.fdas_series_to_spectrum(self._h, ptr, count, on_dev, scale, _ptr(out), int(ab)),
                           "series_to_spectrum")

    def perform_ft_convolution(self, which, ab):
        return self._check(self._lib.fdas_perform_ft_convolution(self._h, int(which), int(ab)),
                           "perform_ft_convolution")

    def perform_harmonic_summing(self, thresholds, which, ab):
        thr = None
        if thresholds is not None:
            thr = _require(np.ascontiguousarray(thresholds, dtype=np.float32), np.float32,
                           self.get_thresholds_sz(), "thresholds")
        return self._check(self._lib.fdas_perform_harmonic_summing(self._h, _ptr(thr), int(which), int(ab)),
                           "perform_harmonic_summing")

    def launch(self, input, thresholds, detection_location, detection_power, which, ab):
        """FDAS::launch: asynchronous; the arrays must stay alive until wait()."""
        x = None if input is None else _require(input, np.complex64, self.get_input_sz(), "input")
        thr = None
        if thresholds is not None:
            thr = _require(np.ascontiguousarray(thresholds, dtype=np.float32), np.float32,
                           self.get_thresholds_sz(), "thresholds")
        n = self.get_candidate_list_sz()
        loc = _require(detection_location, np.uint32, n, "detection_location")
        pwr = _require(detection_power, np.float32, n, "detection_power")
        self._keep[int(ab)] = [x, thr, loc, pwr]
        return self._check(self._lib.fdas_launch(self._h, _ptr(x), _ptr(thr), _ptr(loc), _ptr(pwr), int(which),
                                                 int(ab)), "launch")

    def wait(self, ab):
        ok = self._check(self._lib.fdas_wait(self._h, int(ab)), "wait")
        if ok:
            self._keep[int(ab)] = []
        return ok

    def end_pipeline(self, ab):
        return self._check(self._lib.fdas_end_pipeline(self._h, int(ab)), "end_pipeline")

    def retrieve_tiles(self, tiles, ab):
        t = _require(tiles, np.complex64, self.get_tiles_sz(), "tiles")
        return self._check(self._lib.fdas_retrieve_tiles(self._h, _ptr(t), int(ab)), "retrieve_tiles")

    def retrieve_FOP(self, fop, ab):
        f = _require(fop, np.float32, self.get_fop_sz(), "fop")
        return self._check(self._lib.fdas_retrieve_fop(self._h, _ptr(f), int(ab)), "retrieve_FOP")

    def inject_FOP(self, fop, ab):
        f = _require(np.ascontiguousarray(fop, dtype=np.float32), np.float32, self.get_fop_sz(), "fop")
        return self._check(self._lib.fdas_inject_fop(self._h, _ptr(f), int(ab)), "inject_FOP")

    def retrieve_candidates(self, detection_location, detection_power, ab):
        n = self.get_candidate_list_sz()
        loc = _require(detection_location, np.uint32, n, "detection_location")
        pwr = _require(detection_power, np.float32, n, "detection_power")
        return self._check(self._lib.fdas_retrieve_candidates(self._h, _ptr(loc), _ptr(pwr), int(ab)),
                           "retrieve_candidates")

    def print_stats(self, ab, reset=False):
        self._lib.fdas_print_stats(self._h, int(ab), int(bool(reset)))

    def print_events(self, ab):
        self._lib.fdas_print_events(self._h, int(ab))

    def get_input_sz(self):
        return int(self._lib.fdas_get_input_sz(self._h))

    def get_tiles_sz(self):
        return int(self._lib.fdas_get_tiles_sz(self._h))

    def get_templates_sz(self):
        return int(self._lib.fdas_get_templates_sz(self._h))

    def get_thresholds_sz(self):
        return int(self._lib.fdas_get_thresholds_sz(self._h))

    def get_fop_sz(self):
        return int(self._lib.fdas_get_fop_sz(self._h))

    def get_candidate_list_sz(self):
        return int(self._lib.fdas_get_candidate_list_sz(self._h))

    # ------------------------------------------------------------- extras
    CANDIDATE_DTYPE = np.dtype([("harmonic", np.uint32), ("template_num", np.int32), ("bin", np.uint32),
                                ("power", np.float32)])

    def retrieve_candidate_list(self, ab, capacity=None):
        """All hits of the last harmonic summing, sorted like hsum.py's list.

        Returns (records, n_total, n_dropped); records has fields harmonic,
        template_num, bin, power."""
        n_total, n_dropped = ctypes.c_uint32(), ctypes.c_uint32()
        if capacity is None:  # exactly the stored records
            if not self._check(self._lib.fdas_retrieve_candidate_list(self._h, None, 0, ctypes.byref(n_total),
                                                                      ctypes.byref(n_dropped), int(ab)),
                               "retrieve_candidate_list"):
                return None, 0, 0
            capacity = int(n_total.value) - int(n_dropped.value)
        out = np.zeros(capacity, dtype=self.CANDIDATE_DTYPE)
        ok = self._check(self._lib.fdas_retrieve_candidate_list(self._h, _ptr(out), capacity, ctypes.byref(n_total),
                                                                ctypes.byref(n_dropped), int(ab)),
                         "retrieve_candidate_list")
        if not ok:
            return None, 0, 0
        kept = min(int(n_total.value) - int(n_dropped.value), capacity)
        return out[:kept], int(n_total.value), int(n_dropped.value)

    def retrieve_candidates_ring(self, detection_location, detection_power, which, ab):
        """The FPGA's 64-slot candidate ring of one sign half, reproduced from
        the hits (for side-by-side comparison with FPGA logs)."""
        n = self.config.n_planes * 64 * 8
        loc = _require(detection_location, np.uint32, n, "detection_location")
        pwr = _require(detection_power, np.float32, n, "detection_power")
        return self._check(self._lib.fdas_retrieve_candidates_ring(self._h, _ptr(loc), _ptr(pwr), int(which), int(ab)),
                           "retrieve_candidates_ring")

    def counters(self, ab):
        """Device counters of the last harmonic summing: dict with status,
        recheck (cells sent to the FP64 recheck), records and per-plane hits."""
        out = np.zeros(35, dtype=np.uint32)
        if not self._check(self._lib.fdas_get_counters(self._h, int(ab), _ptr(out), out.size), "get_counters"):
            return None
        n = self.config.n_planes
        return {"status": int(out[0]), "recheck": int(out[1]), "records": int(out[2]),
                "per_plane": [int(x) for x in out[3:3 + n]], "selected": [int(x) for x in out[19:19 + n]]}

    def stage_times(self, ab):
        ms = np.zeros(6, dtype=np.float32)
        ok = self._check(self._lib.fdas_get_stage_times(self._h, int(ab), _ptr(ms)), "get_stage_times")
        return ms if ok else None

    def enqueue_search_device(self, d_input_ptr, thresholds, which, ab):
        thr = np.ascontiguousarray(thresholds, dtype=np.float32)
        self._keep[int(ab)] = [thr]
        return self._check(self._lib.fdas_enqueue_search_device(self._h, ctypes.c_void_p(int(d_input_ptr)),
                                                                _ptr(thr), int(which), int(ab)),
                           "enqueue_search_device")

    def set_wait_timeout(self, ns):
        """Bound (ns) on every wait inside the kernels; <= 0 restores 2 s.  A
        search that runs into it stops and reports FDAS_ERR_TIMEOUT."""
        return self._check(self._lib.fdas_set_wait_timeout(self._h, int(ns)), "set_wait_timeout")

    def set_fault_injection(self, flags):
        """Test hook of the timeout path (``_lib.INJECT_FTC_STALL``; 0 = off)."""
        return self._check(self._lib.fdas_set_fault_injection(self._h, int(flags)), "set_fault_injection")

    def synchronize(self, ab):
        return self._check(self._lib.fdas_synchronize(self._h, int(ab)), "synchronize")

    def stream(self, ab):
        return int(self._lib.fdas_get_stream(self._h, int(ab)) or 0)


def encode_location(harm, tmpl, freq, half=N_TMPL_PER_ACCEL_SIGN):
    """gen_info.h:62-64."""
    return ((((int(harm) - 1) & 0x7) << 29) | (((int(tmpl) + half) & 0x7F) << 22) | (int(freq) & 0x3FFFFF))


INVALID_LOCATION = encode_location(1, N_TMPL_PER_ACCEL_SIGN + 1, 0)


class PinnedArray:
    """A NumPy array backed by pinned host memory (fdas_host_alloc)."""

    def __init__(self, shape, dtype):
        lib = _lib.load()
        self._lib = lib
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self._p = ctypes.c_void_p()
        st = lib.fdas_host_alloc(ctypes.byref(self._p), max(nbytes, 1))
        if st != _lib.OK:
            raise MemoryError(lib.fdas_last_error(None).decode())
        buf = (ctypes.c_byte * max(nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def __del__(self):
        try:
            if self._p:
                self._lib.fdas_host_free(self._p)
                self._p = ctypes.c_void_p()
        except Exception:
            pass
