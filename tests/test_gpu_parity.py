"""GPU parity tests: the CUDA path through the C ABI against the oracle.

Checks follow the reference's gtest (fdas/src/host/main_gtest.cpp:173-228) and
add the stricter FP64 criteria: FOP within 1e-5 of the plane's mean power of
the FP64 oracle, candidate sets identical to the FP64 oracle's (near-threshold
cells are decided by the FP64 recheck), and harmonic summing of an injected FOP
bit-exact with hsum.py.
"""
import io

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import make_pipeline, candidates_as_arrays, validate_harmonic_summing
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from fdas_gb300 import synth
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

# FOP tolerance against the FP64 oracle: 1e-5 of the plane's mean power, plus
# 1e-6 of the cell's own power.  The second term only matters at strong
# signals: there a float32 FOP value cannot be stored closer than half an ulp
# (3e-8 relative), which for a cell 300x the mean is already 1e-5 of the mean.
FOP_REL_TOL = 1e-5
FOP_VALUE_TOL = 1e-6


def fop_within(fop, ref, x=None, bank=None):
    """|fop - ref| <= 1e-5 x plane power + 1e-6 x |ref|.  The plane power is
    the row mean; for spectra shorter than a template (a few bins) the row
    keeps only a fraction of the filtered power, so the power entering the
    filter, mean|x|^2 x sum|h_t|^2, is used when larger."""
    scale = ref.mean(axis=-1, keepdims=True)
    if x is not None:
        energy = np.sum(np.abs(np.asarray(bank, dtype=np.complex128)) ** 2, axis=1)[:, None]
        scale = np.maximum(scale, np.mean(np.abs(x.astype(np.complex128)) ** 2) * energy)
    return np.abs(fop - ref) <= FOP_REL_TOL * scale + FOP_VALUE_TOL * np.abs(ref)


@pytest.fixture(scope="module")
def bank64():
    return template_bank()


@pytest.fixture(scope="module")
def bank_p4(bank64):
    return O.to_p4(np.fft.fft(bank64.astype(np.complex128), 2048, axis=1)).astype(np.complex64)


def run_ftc(g_input, bank, layout, part=FDAS.AllAccelerations):
    n = g_input.size
    p = make_pipeline(n, log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A, layout=layout), p.last_error
    assert p.perform_input_tiling(g_input, FDAS.A), p.last_error
    assert p.perform_ft_convolution(part, FDAS.A), p.last_error
    tiles = np.zeros(p.get_tiles_sz(), dtype=np.complex64)
    assert p.retrieve_tiles(tiles, FDAS.A)
    fop = np.zeros(p.get_fop_sz(), dtype=np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    return p, tiles.reshape(-1, 2048), fop.reshape(85, n)


@pytest.mark.parametrize("name", ["n1000", "n4096", "n32768"])
def test_tiles_match_reference(name, bank_p4):
    g = load_golden(name)
    _, tiles, _ = run_ftc(g["input"], bank_p4, FDAS.TemplatesFFTP4)
    assert tiles.shape[0] == int(g["n_tiles"])
    # main_gtest.cpp:173-181: |d re|, |d im| < 1e-5 against input_tiled_p4_ref
    d = tiles[g["tile_idx"]] - g["tiles_p4_ref"]
    assert np.abs(d.real).max() < 1e-5 and np.abs(d.imag).max() < 1e-5
    # and against the FP64 tiles, relative to the tile rms
    ref = O.to_p4(O.tiles(g["input"]))
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    assert np.abs(tiles - ref).max() < 1e-5 * rms


@pytest.mark.parametrize("name", ["n1000", "n4096", "n32768"])
@pytest.mark.parametrize("layout", ["p4", "time"])
def test_fop_vs_fp64_oracle(name, layout, bank64, bank_p4):
    g = load_golden(name)
    bank = bank_p4 if layout == "p4" else bank64
    lay = FDAS.TemplatesFFTP4 if layout == "p4" else FDAS.TemplatesTimeDomain
    _, _, fop = run_ftc(g["input"], bank, lay)
    ref = O.fop(g["input"], bank64)
    assert fop_within(fop, ref).all()
    # the plain 1e-5-of-mean bound holds for every cell below 30x the mean power
    mean = ref.mean(axis=1, keepdims=True)
    weak = ref < 30 * mean
    assert (np.abs(fop - ref)[weak] <= FOP_REL_TOL * np.broadcast_to(mean, ref.shape)[weak]).all()
    # main_gtest.cpp:183-190 absolute check against the reference's own FOP
    assert np.abs(fop[g["fop_rows"]] - g["fop_ref"]).max() < 1e-5


@pytest.mark.parametrize("part", [FDAS.NegativeAccelerations, FDAS.PositiveAccelerations])
def test_fop_part_rows_only(part, bank_p4):
    g = load_golden("n4096")
    _, _, fop = run_ftc(g["input"], bank_p4, FDAS.TemplatesFFTP4, part=part)
    rows = np.arange(0, 43) if part == FDAS.NegativeAccelerations else np.arange(42, 85)
    other = np.setdiff1d(np.arange(85), rows)
    ref = O.fop(g["input"], template_bank(), rows=rows)
    assert fop_within(fop[rows], ref).all()
    assert np.all(fop[other] == 0)  # untouched rows of a fresh buffer set


@pytest.mark.parametrize("name", ["n1000", "n4096"])
@pytest.mark.parametrize("thr_key", ["", "_chi2"])
def test_hsum_injected_fop_bit_exact(name, thr_key):
    """inject_FOP(fop_ref) -> harmonic summing: identical to hsum.py's list."""
    g = load_golden(name)
    n = g["input"].size
    p = make_pipeline(n, log=io.StringIO())
    thr = g["thresholds" + thr_key]
    assert p.inject_FOP(g["fop_ref"], FDAS.A)
    assert p.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A), p.last_error
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    assert dropped == 0
    loc, pwr = candidates_as_arrays(rec)
    assert np.array_equal(loc, g["det_loc_ref" + thr_key])
    assert np.array_equal(pwr, g["det_pwr_ref" + thr_key])


@pytest.mark.parametrize("n_templates,n_planes", [(101, 16), (85, 16), (101, 8)])
def test_hsum_injected_wide_bank_dense_hits(n_templates, n_planes):
    """Banks wider than 88 rows (the 16-warp harmonic-summing variant) and 16
    planes, on an injected FOP with patches that make most cells of some tiles
    hits in every plane (the emission path at full load) and a ragged last
    block: every hit and its power equal hsum.py's recurrence in float32."""
    n = 6000
    rng = np.random.default_rng(n_templates + n_planes)
    fop = rng.exponential(1.0, size=(n_templates, n)).astype(np.float32)
    half = n_templates // 2
    fop[half - 12:half + 13, 300:340] *= np.float32(6.0)
    fop[half - 4:half + 5, 2000:2012] = np.float32(300.0)
    fop[:, n - 3:] = np.float32(90.0)  # the last bins, partly in the ragged block
    k = np.arange(1, n_planes + 1)
    thr = (k + 6.0 * np.sqrt(k) + 10.0).astype(np.float32)
    p = make_pipeline(n, log=io.StringIO(), n_templates=n_templates, n_planes=n_planes)
    assert p.inject_FOP(fop, FDAS.A), p.last_error
    assert p.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A), p.last_error
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    assert dropped == 0
    hps = O.harmonic_planes(fop, n_planes=n_planes, dtype=np.float32)
    _, pwr, plane, row, fbin = O.detections(hps, thr)
    assert total == pwr.size and pwr.size > 10000
    got = sorted(zip(rec["harmonic"].tolist(), rec["template_num"].tolist(), rec["bin"].tolist(),
                     rec["power"].astype(np.float32).tolist()))
    want = sorted(zip((plane + 1).tolist(), (row - half).tolist(), fbin.tolist(), pwr.tolist()))
    assert got == want


@pytest.mark.parametrize("part", [FDAS.NegativeAccelerations, FDAS.PositiveAccelerations])
def test_hsum_injected_half_gtest_check(part):
    """The reference's Harmonic_Summing test (main_gtest.cpp:261-283)."""
    g = load_golden("n4096")
    p = make_pipeline(4096, log=io.StringIO())
    assert p.inject_FOP(g["fop_ref"], FDAS.A)
    assert p.perform_harmonic_summing(g["thresholds"], part, FDAS.A)
    n = p.get_candidate_list_sz()
    assert n == 4096
    loc = np.zeros(n, dtype=np.uint32)
    pwr = np.zeros(n, dtype=np.float32)
    assert p.retrieve_candidates(loc, pwr, FDAS.A)
    validate_harmonic_summing(loc, pwr, g["det_loc_ref"], g["det_pwr_ref"])
    # every hit of the half is present (the list holds up to 512 per plane)
    h, t, f = O.decode_location(g["det_loc_ref"])
    want = (t <= 0) if part == FDAS.NegativeAccelerations else (t >= 0)
    got = set(loc[loc != O.INVALID_LOCATION].tolist())
    assert got == set(g["det_loc_ref"][want].tolist())


@pytest.mark.parametrize("name,thr_key", [("n4096", ""), ("n4096", "_chi2"), ("n32768", ""),
                                          ("n32768", "_chi2")])
@pytest.mark.parametrize("layout", ["time", "p4"])
def test_search_candidates_equal_fp64_oracle(name, thr_key, layout, bank64, bank_p4):
    """Full search (launch/wait): candidate set identical to the FP64 oracle's."""
    g = load_golden(name)
    n = g["input"].size
    thr = g["thresholds" + thr_key]
    p = make_pipeline(n, log=io.StringIO())
    bank = bank64 if layout == "time" else bank_p4
    assert p.upload_templates(bank, FDAS.A)
    loc = np.zeros(p.get_candidate_list_sz(), dtype=np.uint32)
    pwr = np.zeros_like(loc, dtype=np.float32)
    assert p.launch(g["input"], thr, loc, pwr, FDAS.AllAccelerations, FDAS.A), p.last_error
    assert p.wait(FDAS.A), p.last_error
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    assert dropped == 0
    gl, gp = candidates_as_arrays(rec)
    fop64 = O.fop(g["input"], bank64)
    ol, op, *_ = O.detections(O.harmonic_planes(fop64, 8, dtype=np.float64), thr)
    if layout == "time":
        assert np.array_equal(gl, ol)
    else:
        # FP32 template spectra: the recheck's filter differs from the
        # time-domain taps by ~1e-7 relative; allow cells that close
        diff = set(gl.tolist()) ^ set(ol.tolist())
        hps = O.harmonic_planes(fop64, 8, dtype=np.float64)
        for d in diff:
            hh, tt, ff = O.decode_location(d)
            assert abs(hps[hh - 1][tt + 42][ff] - thr[hh - 1]) <= 1e-6 * thr[hh - 1]
    common = np.isin(gl, ol)
    ref_p = dict(zip(ol.tolist(), op.tolist()))
    rp = np.array([ref_p[x] for x in gl[common].tolist()])
    assert np.all(np.abs(gp[common] - rp) <= 8 * FOP_REL_TOL * fop64.mean() + 8 * FOP_VALUE_TOL * np.abs(rp))
    # the fixed-size list holds the strongest per plane, as the oracle's rule says
    cl, cp = O.compat_list(ol, op.astype(np.float32), (ol >> 29).astype(np.int64))
    if layout == "time":
        assert np.array_equal(loc, cl)


def test_candidate_capacity_and_compat_overflow():
    """More hits than the fixed list holds: strongest 512 per plane, in location order."""
    g = load_golden("n4096")
    thr = np.full(8, 0.0, dtype=np.float32)
    thr[:] = np.quantile(g["fop_ref"], 0.99)  # thousands of hits per plane
    p = make_pipeline(4096, log=io.StringIO())
    assert p.inject_FOP(g["fop_ref"], FDAS.A)
    assert p.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A)
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    hps = O.harmonic_planes(g["fop_ref"].astype(np.float32), 8, dtype=np.float32)
    ol, op, opl, *_ = O.detections(hps, thr)
    assert total == ol.size and dropped == 0
    loc, pwr = candidates_as_arrays(rec)
    assert np.array_equal(loc, ol) and np.array_equal(pwr, op)
    cloc = np.zeros(4096, dtype=np.uint32)
    cpwr = np.zeros(4096, dtype=np.float32)
    assert p.retrieve_candidates(cloc, cpwr, FDAS.A)
    el, ep = O.compat_list(ol, op, opl)
    assert np.array_equal(cloc, el) and np.array_equal(cpwr, ep)
    # a capacity below the number of hits is reported, not silently truncated
    q = make_pipeline(4096, log=io.StringIO(), candidate_capacity=1000)
    assert q.inject_FOP(g["fop_ref"], FDAS.A)
    assert q.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A)
    rec, total, dropped = q.retrieve_candidate_list(FDAS.A)
    assert total == ol.size and dropped == ol.size - 1000 and rec.size == 1000


def _drive(sync_pipeline, n_runs=4):
    """main_gtest.cpp drive_serially / drive_pipelined with the p4 bank."""
    g = load_golden("n4096")
    bank_p4 = O.to_p4(np.fft.fft(template_bank().astype(np.complex128), 2048, axis=1)).astype(np.complex64)
    p = make_pipeline(4096, log=io.StringIO(), sync_pipeline=sync_pipeline)
    assert p.upload_templates(bank_p4, FDAS.A)
    assert p.upload_templates(bank_p4, FDAS.B)
    n = p.get_candidate_list_sz()
    loc = {ab: np.zeros(n, dtype=np.uint32) for ab in (FDAS.A, FDAS.B)}
    pwr = {ab: np.zeros(n, dtype=np.float32) for ab in (FDAS.A, FDAS.B)}
    thr = g["thresholds"]
    if not sync_pipeline:
        for i in range(n_runs):
            which = FDAS.PositiveAccelerations if i % 2 == 0 else FDAS.NegativeAccelerations
            assert p.launch(g["input"], thr, loc[FDAS.A], pwr[FDAS.A], which, FDAS.A)
            assert p.wait(FDAS.A), p.last_error
            p.print_stats(FDAS.A, i == 0)
            p.print_events(FDAS.A)
        sets = [FDAS.A]
    else:
        which = {FDAS.A: FDAS.PositiveAccelerations, FDAS.B: FDAS.NegativeAccelerations}
        for i in range(n_runs + 1):
            ab, prev = (FDAS.A, FDAS.B) if i % 2 == 0 else (FDAS.B, FDAS.A)
            if i < n_runs:
                assert p.launch(g["input"], thr, loc[ab], pwr[ab], which[ab], ab), p.last_error
            else:
                assert p.end_pipeline(ab)
            if i > 0:
                assert p.wait(prev), p.last_error
                p.print_stats(prev, i - 1 == 0)
                p.print_events(prev)
        sets = [FDAS.A, FDAS.B]
    for ab in sets:
        validate_harmonic_summing(loc[ab], pwr[ab], g["det_loc_ref"], g["det_pwr_ref"], tol=1e-5 * 8)
    return p


def test_drive_serially():
    _drive(False)


def test_drive_pipelined():
    p = _drive(True)
    # a set whose harmonic summing is held back cannot be waited on
    g = load_golden("n4096")
    loc = np.zeros(p.get_candidate_list_sz(), dtype=np.uint32)
    pwr = np.zeros_like(loc, dtype=np.float32)
    assert p.launch(g["input"], g["thresholds"], loc, pwr, FDAS.AllAccelerations, FDAS.A)
    assert not p.wait(FDAS.A)
    assert p.end_pipeline(FDAS.B)
    assert p.wait(FDAS.A)


def test_alternating_host_and_device_inputs():
    """The A/B driver loop (launch one set, wait for the other) over different
    spectra, host-memory launches (whose FT convolution is ordered after the
    other set's harmonic summing) mixed with device-resident ones (unordered)
    on one handle: every search's candidate list equals the same spectrum's
    searched alone."""
    import torch
    n = 1 << 16
    bank = template_bank()
    thr = O.chi2_thresholds(1e-6)
    specs = []
    for i in range(9):
        rng = np.random.default_rng(100 + i)
        sig = [dict(r0=float(rng.uniform(0.05, 0.45) * n), z=float(rng.uniform(-40, 40)),
                    n_harm=int(rng.integers(1, 9)), amp=0.02) for _ in range(2)]
        specs.append(synth.spectrum(synth.timeseries(2 * n, sig, seed=100 + i), n)[0])
    alone = make_pipeline(n, log=io.StringIO())
    assert alone.upload_templates(bank, FDAS.A)
    nc = alone.get_candidate_list_sz()
    want = []
    for x in specs:
        loc, pwr = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
        assert alone.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and alone.wait(FDAS.A)
        rec, _, dropped = alone.retrieve_candidate_list(FDAS.A)
        assert dropped == 0 and rec.size > 0
        want.append((rec, loc, pwr))
    alone.close()

    p = make_pipeline(n, log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A) and p.upload_templates(bank, FDAS.B)
    on_device = [i % 3 == 2 for i in range(len(specs))]
    d_specs = [torch.from_numpy(x.view(np.float32)).cuda() if dev else None for x, dev in zip(specs, on_device)]
    outs = [(np.zeros(nc, np.uint32), np.zeros(nc, np.float32)) for _ in specs]

    def finish(j):
        ab = j & 1
        assert (p.synchronize(ab) if on_device[j] else p.wait(ab)), p.last_error
        rec, _, dropped = p.retrieve_candidate_list(ab)
        assert dropped == 0
        assert np.array_equal(rec, want[j][0]), j
        if not on_device[j]:
            assert np.array_equal(outs[j][0], want[j][1]) and np.array_equal(outs[j][1], want[j][2]), j

    for i, x in enumerate(specs):
        ab = i & 1
        if on_device[i]:
            assert p.enqueue_search_device(d_specs[i].data_ptr(), thr, FDAS.AllAccelerations, ab), p.last_error
        else:
            assert p.launch(x, thr, outs[i][0], outs[i][1], FDAS.AllAccelerations, ab), p.last_error
        if i > 0:
            finish(i - 1)
    finish(len(specs) - 1)
    p.close()


@pytest.mark.parametrize("n_bins", [1, 7, 1627, 1628, 1629, 3001, 2 * 1628 + 1])
def test_edge_sizes(n_bins, bank64):
    """Ragged sizes: a single bin, a partial first tile, exact tile multiples."""
    rng = np.random.default_rng(n_bins)
    x = ((rng.standard_normal(n_bins) + 1j * rng.standard_normal(n_bins)) / np.sqrt(2)).astype(np.complex64)
    p = make_pipeline(n_bins, log=io.StringIO())
    assert p.upload_templates(bank64, FDAS.A)
    thr = O.chi2_thresholds(1e-3)
    loc = np.zeros(p.get_candidate_list_sz(), dtype=np.uint32)
    pwr = np.zeros_like(loc, dtype=np.float32)
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A)
    assert p.wait(FDAS.A)
    fop = np.zeros(p.get_fop_sz(), dtype=np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    ref = O.fop(x, bank64)
    assert fop_within(fop.reshape(85, n_bins), ref, x, bank64).all()
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    gl, _ = candidates_as_arrays(rec)
    ol, *_ = O.detections(O.harmonic_planes(ref, 8, dtype=np.float64), thr)
    assert np.array_equal(gl, ol)


def test_invalid_arguments_fail_loudly():
    p = FDAS(io.StringIO())
    assert not p.initialise_accelerator(0)
    assert not p.initialise_accelerator(4096, n_templates=84)
    assert not p.initialise_accelerator(4096, n_planes=17)
    assert not p.initialise_accelerator(4096, tile_overlap=100)  # < 421 - 1
    p = make_pipeline(4096, log=io.StringIO())
    # no templates uploaded yet
    assert p.perform_input_tiling(np.zeros(4096, np.complex64), FDAS.A)
    assert not p.perform_ft_convolution(FDAS.AllAccelerations, FDAS.A)
    assert "templates" in p.last_error
    assert not p.wait(FDAS.B)  # nothing launched
    assert not p.launch(np.zeros(4096, np.complex64), None, np.zeros(4096, np.uint32), np.zeros(4096, np.float32),
                        FDAS.AllAccelerations, FDAS.A)  # no thresholds given or uploaded


def test_full_size_properties(bank64):
    """2^21 bins: FOP rows against the FP64 oracle and the candidate set vs FP64."""
    import full_oracle as F
    x, sig, _, fop64 = F.full_case()  # the FP64 oracle, computed once per session
    n = x.size
    assert n == 1 << 21
    thr = O.chi2_thresholds(1e-6)
    p = make_pipeline(n, log=io.StringIO())
    assert p.upload_templates(bank64, FDAS.A)
    loc = np.zeros(p.get_candidate_list_sz(), dtype=np.uint32)
    pwr = np.zeros_like(loc, dtype=np.float32)
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A)
    assert p.wait(FDAS.A)
    fop = np.zeros(p.get_fop_sz(), dtype=np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    fop = fop.reshape(85, n)
    assert fop_within(fop, fop64).all()
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    assert dropped == 0
    gl, gp = candidates_as_arrays(rec)
    want, _ = F.full_case_candidates(8)
    assert np.array_equal(F.record_keys(rec, 42), want)
    cnt = p.counters(FDAS.A)
    assert cnt["status"] == 0 and cnt["records"] == total
    # margin of the FP32 harmonic sums against the FP64 ones, relative to the
    # threshold, over all cells near a threshold: the recheck band must cover it
    hp32 = O.harmonic_planes_streaming_error(fop, fop64, thr)
    print("max |HP32 - HP64| / thr near thresholds:", hp32, "recheck cells:", cnt["recheck"])
    assert hp32 < 1e-4
    # every injected signal is detected near its starting bin
    h, t, f = O.decode_location(gl)
    for s in sig:
        assert (np.abs(f - s["r0"]) < 1000).any(), s


@pytest.mark.parametrize("part,name", [(FDAS.NegativeAccelerations, "neg"), (FDAS.PositiveAccelerations, "pos")])
@pytest.mark.parametrize("thr_key", ["", "_chi2"])
def test_fpga_ring_list(part, name, thr_key):
    """The reference detectors' 64-slot ring, from an injected FOP (FP32, bit-exact)."""
    g = load_golden("n4096")
    thr = g["thresholds" + thr_key]
    p = make_pipeline(4096, log=io.StringIO())
    assert p.inject_FOP(g["fop_ref"], FDAS.A)
    assert p.perform_harmonic_summing(thr, part, FDAS.A)
    loc = np.zeros(4096, dtype=np.uint32)
    pwr = np.zeros(4096, dtype=np.float32)
    assert p.retrieve_candidates_ring(loc, pwr, part, FDAS.A)
    el, ep = O.ring_list(g["det_loc_ref" + thr_key], g["det_pwr_ref" + thr_key], name)
    assert np.array_equal(loc, el) and np.array_equal(pwr, ep)
    # every ring entry is a reference candidate (main_gtest.cpp:192-228)
    if (loc != O.INVALID_LOCATION).any():
        validate_harmonic_summing(loc, pwr, g["det_loc_ref" + thr_key], g["det_pwr_ref" + thr_key])
    assert not p.retrieve_candidates_ring(loc, pwr, FDAS.AllAccelerations, FDAS.A)
