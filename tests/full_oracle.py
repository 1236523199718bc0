"""FP64 oracle of full-size (2^21-bin) searches for the GPU tests, computed
once per test session and spread over the host's threads (SciPy's FFT
convolution and NumPy's loops release the GIL).

Semantics are those of oracle/fdas_oracle.py: the FOP by direct linear
convolution with each template's non-zero taps in complex128
(ft_conv.py:199-205) and harmonic summing with HP_k = HP_{k-1} +
FOP[trunc(t/k)][f // k] and strict '>' (hsum.py:95-140) in float64."""
import functools
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from fdas_gb300 import synth
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O


def _workers():
    return os.cpu_count() or 1


def fop64(x, bank):
    """FP64 FOP of spectrum ``x`` with template taps ``bank`` (rows x taps)."""
    w = _workers()
    out = np.empty((bank.shape[0], x.size), dtype=np.float64)

    def rows(rs):
        out[rs] = O.fop(x, bank, rows=rs)

    with ThreadPoolExecutor(w) as ex:
        list(ex.map(rows, [list(c) for c in np.array_split(np.arange(bank.shape[0]), w) if len(c)]))
    return out


def candidate_keys(fop, thr, n_planes):
    """Sorted keys (plane << 48 | row << 32 | bin), plane 0-based, of the FP64
    oracle's candidates over all rows of ``fop``, and their powers."""
    n = fop.shape[1]
    w = _workers()
    edges = np.linspace(0, n, 4 * w + 1).astype(np.int64)

    def part(b):
        _, pwr, plane, row, fbin = O.detections_streaming(fop, thr, n_planes, bins=(int(b[0]), int(b[1])))
        return (plane.astype(np.int64) << 48) | (row.astype(np.int64) << 32) | fbin.astype(np.int64), pwr

    with ThreadPoolExecutor(w) as ex:
        res = list(ex.map(part, list(zip(edges[:-1], edges[1:]))))
    keys = np.concatenate([r[0] for r in res])
    pwr = np.concatenate([r[1] for r in res])
    order = np.argsort(keys, kind="stable")
    return keys[order], pwr[order]


def record_keys(rec, half):
    """The same keys for the library's candidate records (template number t
    is FOP row t + half)."""
    return ((rec["harmonic"].astype(np.int64) - 1) << 48) | ((rec["template_num"].astype(np.int64) + half) << 32) | \
        rec["bin"].astype(np.int64)


@functools.lru_cache(maxsize=None)
def full_case():
    """The 2^21-bin benchmark workload: spectrum, injected signals, bank, FP64 FOP."""
    samples, sig = synth.full_case()
    x, _ = synth.spectrum(samples)
    bank = template_bank()
    return x, sig, bank, fop64(x, bank)


@functools.lru_cache(maxsize=None)
def full_case_candidates(n_planes=8):
    x, _, _, f = full_case()
    return candidate_keys(f, O.chi2_thresholds(1e-6, n_planes), n_planes)
