"""Seeded synthetic inputs: white Gaussian time series with accelerated pulsars.

The reference builds its test vectors from SIGPROC ``.tim`` files written by
the SKA PSS test-vector generator (README.md:46-59, fdas/test/configs/*.yaml),
which is not available here.  These seeded series stand in for them with the
same shapes: float32 samples, sigma = 1, plus periodic signals whose frequency
drifts linearly (constant acceleration) over the observation.

A signal with starting frequency ``r0`` (in Fourier bins of the full series)
and drift ``z`` bins has phase ``2 pi (r0 u + z u^2 / 2)`` at normalised time
``u = n / n_samp``; harmonic ``h`` has ``h`` times that phase, hence drift
``h z``.  The acceleration template whose drift is closest to ``z`` is the one
expected to respond (template spacing is ``drift_bins()`` of the bank).
"""

import numpy as np

from .templates import drift_bins


def timeseries(n_samp, signals=(), seed=0, sigma=1.0):
    """float32 samples: N(0, sigma^2) noise + sum of accelerated periodic signals.

    ``signals`` is a sequence of dicts with keys ``r0`` (bins), ``z`` (drift in
    bins), ``n_harm`` (number of harmonics) and ``amp`` (amplitude of each
    harmonic, in units of sigma).
    """
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(n_samp) * sigma
    u = np.arange(n_samp, dtype=np.float64) / n_samp
    for s in signals:
        phase = 2 * np.pi * (s['r0'] * u + 0.5 * s['z'] * u * u)
        for h in range(1, int(s['n_harm']) + 1):
            x += s['amp'] * sigma * np.cos(h * phase + s.get('phi', 0.0) * h)
    return x.astype(np.float32)


def spectrum(samples, n_freq=None, unit_power=True):
    """Complex64 spectrum: first ``n_freq`` bins of the FFT of the series.

    ``unit_power`` scales by 1/sqrt(n_samp) so unit-variance noise has unit mean
    power per bin; otherwise by 1/n_samp as the reference's ft_conv.py:136 does.
    Returns (spectrum, scale).
    """
    samples = np.asarray(samples, dtype=np.float32)
    n_samp = samples.size if n_freq is None else 2 * n_freq
    n_freq = n_samp // 2 if n_freq is None else n_freq
    ft = np.fft.rfft(samples[:n_samp].astype(np.float64))[:n_freq]
    scale = 1.0 / np.sqrt(n_samp) if unit_power else 1.0 / n_samp
    return (ft * scale).astype(np.complex64), scale


def expected_template(z, n_templates=85, max_accel=350.0):
    """Template number whose drift is nearest to ``z`` bins."""
    d = drift_bins(n_templates, max_accel)
    return int(np.argmin(np.abs(d - z))) - n_templates // 2


# --- named workloads -------------------------------------------------------

def emulator_case(seed=42):
    """65536 samples -> 32768 bins, one signal (bin ~4000, z = +20, 4 harmonics, 0.05 sigma)."""
    sig = [dict(r0=4000.0, z=20.0, n_harm=4, amp=0.05)]
    return timeseries(1 << 16, sig, seed=seed), sig


def full_case(seed=7):
    """2^22 samples -> 2^21 bins, three signals with z in {-30, 0, +35}."""
    sig = [dict(r0=150000.5, z=-30.0, n_harm=2, amp=0.1),
           dict(r0=420000.25, z=0.0, n_harm=8, amp=0.02),
           dict(r0=777777.0, z=35.0, n_harm=5, amp=0.05)]
    return timeseries(1 << 22, sig, seed=seed), sig


def small_case(n_freq, seed=1, n_signals=1):
    """Small seeded case for parity tests at ``n_freq`` bins."""
    rng = np.random.default_rng(seed + 1000)
    sig = []
    for _ in range(n_signals):
        sig.append(dict(r0=float(rng.uniform(0.05, 0.5) * n_freq),
                        z=float(rng.uniform(-60, 60)),
                        n_harm=int(rng.integers(1, 9)),
                        amp=float(rng.uniform(0.1, 0.3))))
    return timeseries(2 * n_freq, sig, seed=seed), sig


def batch_mix(n_trials=256, seed=4242, device="cuda"):
    """The batched workload: ``n_trials`` dedispersed trials of uneven length,
    samples drawn log-uniformly from 2^18 to 2^22 (2^17 .. 2^21 bins), each
    with 0-2 accelerated signals (random z in [-42, 42], 1-8 harmonics,
    amplitude 0.05 sigma x sqrt(2^15 / bins)), unit-power spectra made on the
    GPU with torch (input preparation only).  Returns (n_bins uint32 array,
    bin offsets int64 array of n_trials + 1, device float32 tensor holding all
    spectra back to back as (re, im) pairs)."""
    import torch
    rng = np.random.default_rng(seed)
    n_samp = np.exp(rng.uniform(np.log(2 ** 18), np.log(2 ** 22), n_trials)).astype(np.int64) // 2 * 2
    n_bins = (n_samp // 2).astype(np.uint32)
    g = torch.Generator(device=device).manual_seed(7)
    specs = []
    for i in range(n_trials):
        ns = int(n_samp[i])
        x = torch.randn(ns, device=device, generator=g, dtype=torch.float64)
        u = torch.arange(ns, device=device, dtype=torch.float64) / ns
        for _ in range(int(rng.integers(0, 3))):
            r0, z, nh = rng.uniform(0.05, 0.45) * ns / 2, rng.uniform(-42, 42), int(rng.integers(1, 9))
            amp = 0.05 * np.sqrt((1 << 15) / (ns / 2))
            ph = 2 * np.pi * (r0 * u + 0.5 * z * u * u)
            for h in range(1, nh + 1):
                x += amp * torch.cos(h * ph)
        X = torch.fft.rfft(x.float().double())[: ns // 2] / np.sqrt(ns)
        specs.append(torch.view_as_real(X.to(torch.complex64)).contiguous().reshape(-1))
    offsets = np.concatenate([[0], np.cumsum(n_bins.astype(np.int64))])
    return n_bins, offsets, torch.cat(specs)
