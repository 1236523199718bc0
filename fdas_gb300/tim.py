"""SIGPROC ``.tim`` time series: the input format of the reference's test-data
script (ft_conv.py:30-64), read on the host.

A ``.tim`` file is an optional SIGPROC header followed by float32 samples.
The header is a sequence of keywords, each a 4-byte little-endian length
followed by the keyword text, and each keyword followed by its binary value;
it opens with ``HEADER_START`` and closes with ``HEADER_END``.  The reader
follows the reference's rules: the header is looked for in the first 512
bytes, it counts only if ``HEADER_START`` sits right after its 4-byte length,
``data_type`` must be 2 and ``nbits`` 32 (32-bit float time series), and the
sampling time comes from ``tsamp``; without a header the whole file is samples
and the sampling time is unknown (None).
"""
import struct

import numpy as np

HEADER_PROBE = 512  # bytes searched for the header, as ft_conv.py:46


def _field(buf, tag, fmt):
    i = buf.find(tag)
    if i < 0:
        raise RuntimeError(f"Header field ({tag}) not found")
    return struct.unpack_from(fmt, buf, i + len(tag))[0]


def read_tim(path, read_header=True):
    """(samples float32[n], t_samp or None) -- ft_conv.py:39-64."""
    offset, t_samp = 0, None
    if read_header:
        with open(path, "rb") as f:
            head = f.read(HEADER_PROBE)
        if head.find(b"HEADER_START") == 4:
            end = head.find(b"HEADER_END")
            if end < 0:
                raise RuntimeError("Header end tag (b'HEADER_END') not found")
            offset = end + len(b"HEADER_END")
            if _field(head, b"data_type", "<i") != 2 or _field(head, b"nbits", "<i") != 32:
                raise RuntimeError("Format mismatch: Expecting 32-bit FP time series data")
            t_samp = _field(head, b"tsamp", "<d")
    return np.fromfile(path, dtype=np.float32, offset=offset), t_samp


def _kw(name):
    b = name.encode()
    return struct.pack("<i", len(b)) + b


def write_tim(path, samples, t_samp=None, header=True, source_name="fdas_gb300"):
    """Write a float32 series, with a minimal SIGPROC header (data_type 2,
    nbits 32, nchans 1, tsamp) unless ``header`` is False."""
    x = np.ascontiguousarray(samples, dtype=np.float32)
    with open(path, "wb") as f:
        if header:
            h = _kw("HEADER_START")
            h += _kw("source_name") + _kw(source_name)
            h += _kw("data_type") + struct.pack("<i", 2)
            h += _kw("nchans") + struct.pack("<i", 1)
            h += _kw("nbits") + struct.pack("<i", 32)
            h += _kw("tsamp") + struct.pack("<d", 6.4e-5 if t_samp is None else float(t_samp))
            h += _kw("HEADER_END")
            f.write(h)
        f.write(x.tobytes())
