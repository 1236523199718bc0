"""CPU oracle for the FDAS hot path -- TEST INFRASTRUCTURE ONLY.

This module restates, in vectorised NumPy/SciPy and by default in float64, the
reference's own CPU path for the FT convolution and harmonic summing:

* ``fdas/test/ft_conv.py``  (spectrum, overlap-save tiles, filter-output plane)
* ``fdas/test/hsum.py``     (harmonic planes, thresholds, candidate list)
* ``fdas/src/host/gen_info.h`` (candidate location codec)

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import it, and only to check results (or as the timed CPU
baseline).  The product path (``fdas_gb300``) never calls into it.

Parity is pinned: ``tests/golden/make_golden.py`` runs the unmodified
reference scripts on seeded synthetic inputs and stores their outputs as
fixtures; ``tests/test_oracle_golden.py`` checks this restatement against them.
"""

import numpy as np
import scipy.fft
import scipy.signal

# gen_info.h:29-30 -- n_tmpl_per_accel_sign; template number t is row t + 42
N_TMPL_PER_ACCEL_SIGN = 42


# ---------------------------------------------------------------------------
# Stage 0: spectrum (ft_conv.py:134-143)
# ---------------------------------------------------------------------------
def spectrum(samples, n_freq, scale=None):
    """Normalised spectrum of a real time series, first ``n_freq`` bins.

    ft_conv.py:136 divides the full complex FFT by ``n_samp``; ``scale``
    overrides that factor (the synthetic generator uses 1/sqrt(n_samp) to get
    unit mean power).  Returned as complex64 like ft_conv.py:143.
    """
    samples = np.asarray(samples)
    n_samp = 2 * n_freq
    if samples.size < n_samp:
        raise ValueError("not enough samples")
    samples = samples[:n_samp]
    ft = scipy.fft.fft(samples.astype(np.float64))
    s = (1.0 / n_samp) if scale is None else scale
    return np.asarray(ft[:n_freq] * s, dtype=np.complex64)


# ---------------------------------------------------------------------------
# Stage 1: overlap-save tiles (ft_conv.py:159-197)
# ---------------------------------------------------------------------------
def tile_overlap(max_tmpl_len, pack=4):
    """ft_conv.py:161 / cl_codegen.py:99 -- overlap rounded up to the pack size."""
    return int(np.ceil((max_tmpl_len - 1) / pack)) * pack


def n_tiles(n_freq, tile_sz=2048, overlap=420):
    """FDAS.cpp:177-183 -- number of tiles; equals ceil(n_freq / payload)."""
    payload = tile_sz - overlap
    return -(-n_freq // payload)


def tiles(ft, tile_sz=2048, overlap=420, dtype=np.complex128):
    """Tiled, Fourier-transformed input in natural bin order (ft_conv.py:159-183).

    Tile i holds ``ft[i*P - O : i*P + P]`` with zeros before bin 0 (tile 0) and
    after the last bin (last tile); each tile is FFT'd (unnormalised).
    """
    ft = np.asarray(ft)
    n_freq = ft.size
    payload = tile_sz - overlap
    nt = n_tiles(n_freq, tile_sz, overlap)
    padded = np.zeros(overlap + nt * payload, dtype=dtype)
    padded[overlap:overlap + n_freq] = ft
    idx = np.arange(nt)[:, None] * payload + np.arange(tile_sz)[None, :]
    return scipy.fft.fft(padded[idx], axis=1)


def bit_rev(x, bits):
    """ft_conv.py:70-76 / utils.cl.mako bit_reversed."""
    y = 0
    for _ in range(bits):
        y = (y << 1) | (x & 1)
        x >>= 1
    return y


def p4_permutation(n=2048, n_par=4):
    """Index map of the reference's 'FFT order' (ft_conv.py:186-194, tmpl-gen.py:145-153).

    ``p4[j::n_par] = natural[bitrev(j) * n/n_par : (bitrev(j)+1) * n/n_par]``,
    i.e. position ``n_par*s + j`` holds natural bin ``bitrev(j)*(n/n_par) + s``.
    Returns ``perm`` with ``p4 = natural[..., perm]``.
    """
    bits = int(np.log2(n_par))
    chunk = n // n_par
    perm = np.empty(n, dtype=np.int64)
    for j in range(n_par):
        perm[j::n_par] = bit_rev(j, bits) * chunk + np.arange(chunk)
    return perm


def to_p4(arr, n_par=4):
    arr = np.asarray(arr)
    return arr[..., p4_permutation(arr.shape[-1], n_par)]


def from_p4(arr, n_par=4):
    arr = np.asarray(arr)
    out = np.empty_like(arr)
    out[..., p4_permutation(arr.shape[-1], n_par)] = arr
    return out


# ---------------------------------------------------------------------------
# Stage 2: filter-output plane (ft_conv.py:199-207)
# ---------------------------------------------------------------------------
def template_taps(templates):
    """Non-zero taps of each template row (ft_conv.py:203)."""
    return [row[np.nonzero(row)] for row in np.asarray(templates)]


def fop(ft, templates, dtype=np.float64, rows=None):
    """Filter-output plane by direct linear convolution, trimmed to N bins.

    ft_conv.py:201-205: ``conv = convolve(ft, tmpl[nonzero])[:n_freq]``,
    ``fop = |conv|^2``.  Computed in complex128 (``dtype`` float64) for the
    FP64 oracle, or complex64 to mirror the reference's own precision.
    """
    cdt = np.complex128 if dtype == np.float64 else np.complex64
    ft = np.asarray(ft).astype(cdt)
    taps = template_taps(templates)
    n_freq = ft.size
    rows = range(len(taps)) if rows is None else rows
    out = np.empty((len(list(rows)), n_freq), dtype=dtype)
    for i, r in enumerate(rows):
        conv = scipy.signal.convolve(ft, taps[r].astype(cdt))[:n_freq]
        out[i] = (conv.real * conv.real + conv.imag * conv.imag).astype(dtype)
    return out


def fop_cells(ft, templates, rows, bins):
    """FP64 FOP at individual cells (row, bin) by direct summation."""
    ft = np.asarray(ft).astype(np.complex128)
    taps = template_taps(templates)
    out = np.empty(len(rows), dtype=np.float64)
    for i, (r, f) in enumerate(zip(rows, bins)):
        h = taps[r].astype(np.complex128)
        j = np.arange(min(h.size, f + 1))
        y = np.sum(ft[f - j] * h[j])
        out[i] = y.real * y.real + y.imag * y.imag
    return out


# ---------------------------------------------------------------------------
# Stage 3: harmonic summing (hsum.py:95-151)
# ---------------------------------------------------------------------------
def subharmonic_row(row, k, n_tmpl):
    """hsum.py:107-113 -- row of template trunc(t / k), t = row - n_tmpl//2."""
    half = n_tmpl // 2
    t = np.asarray(row) - half
    return np.trunc(t / k).astype(np.int64) + half if np.ndim(t) else int(np.trunc(t / k)) + half


def harmonic_planes(fop_plane, n_planes=8, dtype=None):
    """HP_1..HP_n (hsum.py:95-120), vectorised.

    ``HP_k[t][f] = HP_{k-1}[t][f] + FOP[trunc(t/k)][f // k]``, accumulated
    in ``dtype`` (float32 reproduces hsum.py bit for bit; float64 is the oracle).
    """
    fop_plane = np.asarray(fop_plane)
    dtype = fop_plane.dtype if dtype is None else dtype
    f = fop_plane.astype(dtype)
    n_tmpl, n_freq = f.shape
    rows = np.arange(n_tmpl)
    hps = np.empty((n_planes, n_tmpl, n_freq), dtype=dtype)
    hps[0] = f
    freqs = np.arange(n_freq)
    for h in range(1, n_planes):
        k = h + 1
        sp_rows = subharmonic_row(rows, k, n_tmpl)
        hps[h] = hps[h - 1] + f[sp_rows][:, freqs // k]
    return hps


def mockup_thresholds(hps, n_cand_per_plane=64):
    """hsum.py:125-131 -- quantile thresholds giving ~n candidates per plane."""
    n_planes = hps.shape[0]
    size = hps[0].size
    thr = np.zeros(n_planes, dtype=np.float32)
    for h in range(n_planes):
        thr[h] = np.quantile(hps[h], q=1 - n_cand_per_plane / size)
    return thr


def chi2_thresholds(far=1e-6, n_planes=8, mean_power=1.0):
    """Per-plane thresholds for a false-alarm rate under chi-square noise.

    For unit-mean exponential FOP cells HP_k ~ Gamma(k, 1), so the threshold
    for FAR p is ``gamma.isf(p, k)`` scaled by the mean cell power.
    """
    from scipy.stats import gamma
    return np.array([gamma.isf(far, k) * mean_power for k in range(1, n_planes + 1)],
                    dtype=np.float32)


def encode_location(harm, tmpl, freq):
    """gen_info.h:62-64 / hsum.py:147 -- 32-bit candidate location."""
    harm = np.asarray(harm, dtype=np.int64)
    tmpl = np.asarray(tmpl, dtype=np.int64)
    freq = np.asarray(freq, dtype=np.int64)
    code = (((harm - 1) & 0x7) << 29) | (((tmpl + N_TMPL_PER_ACCEL_SIGN) & 0x7F) << 22) | (freq & 0x3FFFFF)
    return code.astype(np.uint32)


def decode_location(loc):
    """gen_info.h:65-67."""
    loc = np.asarray(loc, dtype=np.uint32).astype(np.int64)
    return ((loc >> 29) & 0x7) + 1, ((loc >> 22) & 0x7F) - N_TMPL_PER_ACCEL_SIGN, loc & 0x3FFFFF


INVALID_LOCATION = int(encode_location(1, N_TMPL_PER_ACCEL_SIGN + 1, 0))  # gen_info.h:69
INVALID_POWER = -1.0  # detect.cl.mako:139


def part_rows(part, n_tmpl):
    """Template rows covered by a FOP part (FDAS.cpp:333-346).

    part: 'neg' -> t in [-42, 0], 'pos' -> [0, 42], 'all' -> [-42, 42].
    """
    half = n_tmpl // 2
    if part == 'neg':
        return np.arange(0, half + 1)
    if part == 'pos':
        return np.arange(half, n_tmpl)
    return np.arange(n_tmpl)


def detections(hps, thresholds, rows=None):
    """Candidates ``HP_k > thr_k`` (strict, hsum.py:134-148; hms_baseline.cl.mako:74).

    Returns (location u32, power, plane, row, bin) sorted by location, which is
    hsum.py's emission order (plane-major, then row-major over the plane).
    Powers are returned in the planes' dtype.
    """
    n_planes, n_tmpl, n_freq = hps.shape
    rows = np.arange(n_tmpl) if rows is None else np.asarray(rows)
    locs, pwrs, ps, rs, fs = [], [], [], [], []
    for h in range(n_planes):
        sub = hps[h][rows]
        ri, fi = np.nonzero(sub > np.asarray(thresholds[h], dtype=hps.dtype))
        r = rows[ri]
        locs.append(encode_location(h + 1, r - n_tmpl // 2, fi))
        pwrs.append(sub[ri, fi])
        ps.append(np.full(ri.size, h, dtype=np.int64))
        rs.append(r)
        fs.append(fi)
    loc = np.concatenate(locs)
    order = np.argsort(loc, kind='stable')
    return (loc[order], np.concatenate(pwrs)[order], np.concatenate(ps)[order],
            np.concatenate(rs)[order], np.concatenate(fs)[order])


def compat_list(loc, pwr, plane, n_planes=8, per_plane=512):
    """Deterministic fixed-size candidate list (n_planes * per_plane entries).

    The reference keeps a 64-slot x 8-lane ring per plane (detect.cl.mako:32-115,
    store_cands.cl.mako:21-33), i.e. 512 entries per plane and 4096 in total,
    overwriting the oldest slots on overflow.  fdas_gb300 uses a deterministic
    rule instead: per plane, if more than ``per_plane`` hits exist keep the
    strongest (power descending, location ascending on ties); the kept entries
    are listed in location order and the rest of the plane's block is padded
    with (INVALID_LOCATION, -1.0).
    """
    out_loc = np.full(n_planes * per_plane, INVALID_LOCATION, dtype=np.uint32)
    out_pwr = np.full(n_planes * per_plane, INVALID_POWER, dtype=np.float32)
    for h in range(n_planes):
        sel = np.nonzero(plane == h)[0]
        l, p = loc[sel], np.asarray(pwr[sel], dtype=np.float32)
        if l.size > per_plane:
            keep = np.lexsort((l, -p))[:per_plane]
            l, p = l[keep], p[keep]
            o = np.argsort(l, kind='stable')
            l, p = l[o], p[o]
        out_loc[h * per_plane:h * per_plane + l.size] = l
        out_pwr[h * per_plane:h * per_plane + l.size] = p
    return out_loc, out_pwr


# ---------------------------------------------------------------------------
# Whole search (both stages)
# ---------------------------------------------------------------------------
def search(ft, templates, thresholds, n_planes=8, part='all', dtype=np.float64):
    """FOP -> harmonic planes -> candidates for one spectrum.

    For part 'all' template 0 is reported once; for 'neg'/'pos' the rows of
    that half only (as FDAS::launch does per half, FDAS.cpp:548).
    """
    plane = fop(ft, templates, dtype=dtype)
    hps = harmonic_planes(plane, n_planes, dtype=dtype)
    rows = part_rows(part, plane.shape[0])
    return plane, hps, detections(hps, thresholds, rows)


def detections_streaming(fop_plane, thresholds, n_planes=8, part='all', dtype=np.float64, bins=None):
    """Candidates of a whole search without materialising all harmonic planes.

    Same semantics as ``harmonic_planes`` + ``detections`` (sequential
    accumulation HP_k = HP_{k-1} + FOP[trunc(t/k)][f//k] in ``dtype``), one
    plane at a time, for full-size (2^21-bin) checks.  ``bins`` = (b0, b1)
    restricts the search to those frequency bins (the sums read the whole
    FOP), so bin ranges can be searched in parallel.
    Returns (location, power, plane, row, bin) sorted by location.
    """
    f = np.asarray(fop_plane).astype(dtype, copy=False)
    n_tmpl, n_freq = f.shape
    b0, b1 = (0, n_freq) if bins is None else bins
    rows = part_rows(part, n_tmpl)
    hp = f[rows, b0:b1].copy()
    freqs = np.arange(b0, b1)
    out = ([], [], [], [], [])
    for h in range(n_planes):
        k = h + 1
        if k > 1:
            hp += f[subharmonic_row(rows, k, n_tmpl)[:, None], (freqs // k)[None, :]]
        ri, fi = np.nonzero(hp > np.asarray(thresholds[h], dtype=dtype))
        fi = fi + b0
        out[0].append(encode_location(k, rows[ri] - n_tmpl // 2, fi))
        out[1].append(hp[ri, fi - b0])
        out[2].append(np.full(ri.size, h, dtype=np.int64))
        out[3].append(rows[ri])
        out[4].append(fi)
    loc = np.concatenate(out[0])
    order = np.argsort(loc, kind='stable')
    return tuple(np.concatenate(o)[order] for o in out)


def hp_cells(fop_plane, plane, rows, bins, dtype=np.float64):
    """HP_{plane+1} at individual cells (sequential accumulation)."""
    f = np.asarray(fop_plane)
    n_tmpl = f.shape[0]
    out = np.zeros(len(rows), dtype=dtype)
    for i, (p, r, b) in enumerate(zip(plane, rows, bins)):
        acc = dtype(0)
        for k in range(1, int(p) + 2):
            acc = dtype(acc + dtype(f[subharmonic_row(int(r), k, n_tmpl), int(b) // k]))
        out[i] = acc
    return out


def harmonic_planes_streaming_error(fop32, fop64, thresholds, n_planes=8, window=(0.5, 2.0)):
    """max |HP32 - HP64| / thr over cells whose FP64 harmonic sum lies within
    ``window`` x thr, with HP32 accumulated in float32 from ``fop32`` in the
    kernel's order and HP64 in float64 from ``fop64`` (full-size, streaming)."""
    f32 = np.asarray(fop32, dtype=np.float32)
    f64 = np.asarray(fop64, dtype=np.float64)
    n_tmpl, n_freq = f32.shape
    rows = np.arange(n_tmpl)
    freqs = np.arange(n_freq)
    h32 = f32.copy()
    h64 = f64.copy()
    worst = 0.0
    for h in range(n_planes):
        k = h + 1
        if k > 1:
            sr = subharmonic_row(rows, k, n_tmpl)
            h32 += f32[sr][:, freqs // k]
            h64 += f64[sr][:, freqs // k]
        thr = float(thresholds[h])
        sel = (h64 > window[0] * thr) & (h64 < window[1] * thr)
        if sel.any():
            worst = max(worst, float(np.max(np.abs(h32[sel].astype(np.float64) - h64[sel])) / thr))
    return worst


def ring_list(loc, pwr, part, n_planes=8, group_sz=4, bundle_sz=2, detection_sz=64):
    """The FPGA detectors' candidate ring, reproduced from a hit list.

    detect.cl.mako:141-216 scans one sign half in template groups of
    ``group_sz`` (|t| = group_sz*g + p) and bins in bundles of ``bundle_sz``
    (f = bundle_sz*b + q), group-major; every (g, b) with at least one hit is
    an event written to slot ``next`` (next = (next + 1) mod detection_sz) with
    lane p*bundle_sz + q.  Older events are overwritten, so the last
    ``detection_sz`` events survive.  store_cands.cl.mako:21-33 emits plane-major
    [plane][slot][lane] (the drain of detect.cl.mako:220-243); empty lanes and
    slots hold (INVALID_LOCATION, -1).  ``part``: 'neg' or 'pos'.
    """
    slot_sz = 1 << int(np.ceil(np.log2(group_sz * bundle_sz)))
    out_loc = np.full((n_planes, detection_sz, slot_sz), INVALID_LOCATION, dtype=np.uint32)
    out_pwr = np.full((n_planes, detection_sz, slot_sz), INVALID_POWER, dtype=np.float32)
    h, t, f = decode_location(loc)
    sel = (t <= 0) if part == 'neg' else (t >= 0)
    for k in range(1, n_planes + 1):
        m = sel & (h == k)
        if not m.any():
            continue
        tt, ff, ll, pp = np.abs(t[m]), f[m], np.asarray(loc)[m], np.asarray(pwr, dtype=np.float32)[m]
        g, p = tt // group_sz, tt % group_sz
        b, q = ff // bundle_sz, ff % bundle_sz
        ev = g.astype(np.int64) * (int(ff.max()) // bundle_sz + 2) + b  # scan order
        uniq, rank = np.unique(ev, return_inverse=True)
        n_ev = uniq.size
        keep = rank >= n_ev - detection_sz
        slot = rank[keep] % detection_sz
        lane = (p * bundle_sz + q)[keep]
        out_loc[k - 1, slot, lane] = ll[keep]
        out_pwr[k - 1, slot, lane] = pp[keep]
    return out_loc.reshape(-1), out_pwr.reshape(-1)
