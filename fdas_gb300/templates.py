"""Acceleration template bank (constant-acceleration Fresnel response).

Restates the published formula behind the reference's ``fdas/tmpl/tmpl-gen.py``
(``generate_templates``, tmpl-gen.py:45-78, itself a port of the SKA-TDT
``templateGenerator.m``) in float64, written for NumPy 2 (the reference script
uses ``np.complex``, removed in NumPy 2, tmpl-gen.py:64-76).

Template ``t`` (t = -42..42 for 85 templates) models a signal whose frequency
drifts by ``z_t = (t * step) * f0 * T^2 / c`` bins over the observation
(``step = 2 * max_accel / (n_templates - 1)``).  Its taps are

    h(x) = (2 z)^-1/2 * exp(i pi x^2 / z) * (S(Z) - S(Y) - i (C(Y) - C(Z)))

with ``x = arange(-|z|, |z|) - z/2``, ``Y = x sqrt(2/z)``, ``Z = (x + z) sqrt(2/z)``
and S, C the Fresnel integrals; for z = 0 the template is a single unit tap.
For z < 0 the square roots are imaginary and S(iy) = -i S(y), C(iy) = i C(y).
"""

import numpy as np
import scipy.special

SPEED_OF_LIGHT = 299792458.0


def _fresnel_sc(a):
    """Fresnel S, C for an array that is purely real or purely imaginary."""
    a = np.asarray(a, dtype=np.complex128)
    if np.any(a.real) and not np.any(a.imag):
        s, c = scipy.special.fresnel(a.real)
        return s.astype(np.complex128), c.astype(np.complex128)
    if np.any(a.imag) and not np.any(a.real):
        s, c = scipy.special.fresnel(a.imag)
        return -1j * s, 1j * c
    raise ValueError("argument must be purely real or purely imaginary")


def drift_bins(n_templates=85, max_accel=350.0, f0=500.0, t_obs=600.0, c=SPEED_OF_LIGHT):
    """Frequency drift in bins of each template (tmpl-gen.py:52-56)."""
    n = n_templates - 1
    step = 2 * max_accel / n
    return np.array([(step * i - max_accel) * f0 * np.square(t_obs) / c for i in range(n + 1)])


def generate_templates(n_templates=85, max_accel=350.0, f0=500.0, t_obs=600.0, c=SPEED_OF_LIGHT):
    """List of complex128 tap arrays, one per template (index = t + n_templates//2)."""
    if n_templates % 2 == 0:
        raise ValueError("number of templates must be odd")
    out = []
    for z in drift_bins(n_templates, max_accel, f0, t_obs, c):
        if z == 0:
            out.append(np.ones(1, dtype=np.complex128))
            continue
        x = np.arange(-np.abs(z), np.abs(z)) - z / 2
        root = np.sqrt(complex(2 / z))
        sy, cy = _fresnel_sc(x * root)
        sz, cz = _fresnel_sc((x + z) * root)
        out.append(1 / np.sqrt(complex(2 * z)) * np.exp(1j * np.pi * np.square(x) / z)
                   * (sz - sy - 1j * (cy - cz)))
    return out


def template_bank(n_templates=85, max_accel=350.0, dtype=np.complex64, **kw):
    """Rows of left-aligned taps, zero padded to the longest template (tmpl-gen.py:155-159)."""
    tmpls = generate_templates(n_templates, max_accel, **kw)
    width = max(t.size for t in tmpls)
    bank = np.zeros((len(tmpls), width), dtype=dtype)
    for i, t in enumerate(tmpls):
        bank[i, :t.size] = t
    return bank


def template_spectra(bank, fft_size=2048):
    """FFT of each template, natural bin order, computed in float64."""
    return np.fft.fft(np.asarray(bank, dtype=np.complex128), fft_size, axis=1)


def tile_overlap_for(bank, pack=4):
    """Overlap needed by overlap-save for this bank: taps-1 rounded up to ``pack``."""
    bank = np.asarray(bank)
    taps = max(int(np.count_nonzero(r)) for r in bank) if bank.ndim == 2 else len(bank)
    return -(-(taps - 1) // pack) * pack
