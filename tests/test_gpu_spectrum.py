"""Upstream step on the GPU (fdas_series_to_spectrum): the spectrum of a real
series against the reference's own complex64 spectra (ft_conv.py output in
the golden fixtures) and the FP64 oracle, and a search started from the
series against the same search from the host spectrum."""
import io

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import make_pipeline
from fdas_gb300 import synth
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

# FP32 mixed-radix FFT with FP64-rounded twiddles: every bin within 2e-6 of
# the spectrum's rms (about log2(N) single-precision roundings of the rms)
SPEC_TOL = 3e-6


def gpu_spectrum(samples, n, scale=None):
    p = make_pipeline(n, log=io.StringIO())
    out = np.zeros(n, dtype=np.complex64)
    assert p.series_to_spectrum(samples, FDAS.A, scale=scale, spectrum=out), p.last_error
    return p, out


@pytest.mark.parametrize("name", ["n1000", "n4096", "n32768"])
def test_spectrum_matches_reference(name):
    g = load_golden(name)
    n = g["input"].size
    _, x = gpu_spectrum(g["samples"], n)
    ref64 = O.spectrum(g["samples"], n).astype(np.complex128)  # FP64 FFT, rounded once
    exact = np.fft.fft(g["samples"][:2 * n].astype(np.float64))[:n] / (2 * n)
    rms = np.sqrt(np.mean(np.abs(exact) ** 2))
    assert np.abs(x - exact).max() <= SPEC_TOL * rms
    # the reference's own float32 spectrum (scipy in single precision) is no closer
    assert np.abs(g["input"] - exact).max() <= SPEC_TOL * rms
    assert np.abs(x - g["input"]).max() <= 2 * SPEC_TOL * rms
    assert np.abs(ref64 - exact).max() <= 1e-6 * rms


@pytest.mark.parametrize("n", [1, 7, 12, 1680, 1 << 21])
def test_spectrum_sizes(n):
    rng = np.random.default_rng(n)
    s = rng.standard_normal(2 * n + 5).astype(np.float32)  # extra samples are ignored
    _, x = gpu_spectrum(s, n, scale=1.0)
    exact = np.fft.fft(s[:2 * n].astype(np.float64))[:n]
    rms = np.sqrt(np.mean(np.abs(exact) ** 2))
    assert np.abs(x - exact).max() <= SPEC_TOL * rms * max(1.0, np.log2(max(n, 2)) / 11)


def test_spectrum_from_device_samples():
    import torch
    n = 4096
    s = np.random.default_rng(9).standard_normal(2 * n).astype(np.float32)
    _, x_host = gpu_spectrum(s, n)
    _, x_dev = gpu_spectrum(torch.from_numpy(s).cuda(), n)
    assert np.array_equal(x_host, x_dev)


def test_spectrum_rejections():
    p = make_pipeline(1100, log=io.StringIO())  # 1100 = 2^2 5^2 11
    s = np.zeros(2200, dtype=np.float32)
    assert not p.series_to_spectrum(s, FDAS.A)
    assert "factor" in p.last_error
    p = make_pipeline(1000, log=io.StringIO())
    assert not p.series_to_spectrum(np.zeros(1999, dtype=np.float32), FDAS.A)
    assert "2 x n_frequency_bins" in p.last_error
    # NULL input without a spectrum on the set is an error
    assert not p.perform_input_tiling(None, FDAS.B)


def test_search_from_series_equals_search_from_spectrum():
    samples, _ = synth.small_case(32768, seed=4, n_signals=2)
    n = 32768
    bank = template_bank()
    p = make_pipeline(n, log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A)
    spec = np.zeros(n, dtype=np.complex64)
    assert p.series_to_spectrum(samples, FDAS.A, scale=1.0 / np.sqrt(2 * n), spectrum=spec), p.last_error
    thr = O.chi2_thresholds(1e-6)
    nc = p.get_candidate_list_sz()
    loc_a, pwr_a = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert p.launch(None, thr, loc_a, pwr_a, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A), p.last_error
    rec_a, _, _ = p.retrieve_candidate_list(FDAS.A)
    loc_b, pwr_b = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert p.launch(spec, thr, loc_b, pwr_b, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A), p.last_error
    rec_b, _, _ = p.retrieve_candidate_list(FDAS.A)
    assert rec_a.size > 0
    assert np.array_equal(rec_a, rec_b)
    assert np.array_equal(loc_a, loc_b) and np.array_equal(pwr_a, pwr_b)
