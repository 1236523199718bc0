#!/usr/bin/env python3
"""Generate the ``.tim`` reader fixtures in this directory.

Writes small SIGPROC ``.tim`` files -- headers packed here byte by byte, not
with the library's writer -- and records what the reference's own reader,
``read_tim_file`` of ``fdas/test/ft_conv.py`` (UOA-PARC-SKA/FDAS, imported
unmodified from a local checkout given by ``--reference``), returns for each:
sample count, sampling time, a few samples and their float64 sum, or the
error it raises.  ``tests/test_tim.py`` checks the library's reader against it.

Usage:  python tests/golden/make_tim_golden.py --reference /path/to/FDAS
"""
import argparse
import importlib.util
import json
import pathlib
import struct

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent


def kw(s):
    b = s.encode()
    return struct.pack("<i", len(b)) + b


def header(data_type=2, nbits=32, tsamp=6.4e-5, extra=b""):
    h = kw("HEADER_START") + kw("source_name") + kw("J0000+0000_test")
    h += kw("telescope_id") + struct.pack("<i", 0)
    h += kw("data_type") + struct.pack("<i", data_type)
    h += kw("refdm") + struct.pack("<d", 12.5)
    h += kw("nchans") + struct.pack("<i", 1)
    h += kw("nbits") + struct.pack("<i", nbits)
    h += kw("tstart") + struct.pack("<d", 60000.0)
    h += kw("tsamp") + struct.pack("<d", tsamp)
    h += extra + kw("HEADER_END")
    return h


CASES = {
    # name: (header bytes or None, number of samples, read_header)
    "tim_header": (lambda: header(), 1000, True),
    "tim_header_t128": (lambda: header(tsamp=1.28e-4), 333, True),
    "tim_headerless": (lambda: b"", 777, False),
    "tim_header_read_as_raw": (lambda: header(), 64, False),
    "tim_no_header_probe": (lambda: b"", 50, True),
    "tim_bad_type": (lambda: header(data_type=1), 16, True),
    "tim_bad_nbits": (lambda: header(nbits=8), 16, True),
    "tim_no_end": (lambda: header(extra=kw("x" * 600))[:-len(kw("HEADER_END"))], 16, True),
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, type=pathlib.Path)
    args = ap.parse_args()
    spec = importlib.util.spec_from_file_location("ft_conv", args.reference / "fdas/test/ft_conv.py")
    ft_conv = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ft_conv)
    rng = np.random.default_rng(2024)
    out = {}
    for name, (hdr, n, read_header) in CASES.items():
        path = HERE / f"{name}.tim"
        samples = rng.standard_normal(n).astype(np.float32)
        path.write_bytes(hdr() + samples.tobytes())
        try:
            x, t = ft_conv.read_tim_file(str(path), read_header=read_header)
            out[name] = dict(read_header=read_header, n=int(x.size), t_samp=t, first=[float(v) for v in x[:4]],
                             sum=float(np.sum(x.astype(np.float64))), error=None)
        except RuntimeError as e:
            out[name] = dict(read_header=read_header, error=str(e))
    (HERE / "tim_golden.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
