"""Pin the CPU oracle against outputs of the reference's own scripts.

The fixtures in tests/golden were produced by tests/golden/make_golden.py,
which runs the unmodified ft_conv.py and hsum.py on seeded inputs.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import fdas_oracle as O
from fdas_gb300.templates import template_bank

CASES = ["n1000", "n4096", "n32768"]


def test_template_generator_matches_shipped_bank():
    g = np.load("tests/golden/template_bank.npz")
    bank = template_bank()
    assert tuple(bank.shape) == tuple(g["bank_shape"])
    assert np.array_equal(bank[g["rows"]], g["bank_rows"])
    assert np.array_equal(np.count_nonzero(bank, axis=1), g["bank_nnz"])
    # p4-ordered 2048-point spectra (tmpl-gen.py -f -p) from the same taps
    ft = O.to_p4(np.fft.fft(bank.astype(np.complex128), 2048, axis=1))
    assert np.abs(ft[g["rows"]] - g["ft_p4_rows"]).max() < 1e-6


def test_p4_permutation_roundtrip():
    x = np.arange(2048)
    p = O.to_p4(x)
    # position 4s+j holds natural bin bitrev2(j)*512 + s
    assert p[0] == 0 and p[1] == 1024 and p[2] == 512 and p[3] == 1536 and p[4] == 1
    assert np.array_equal(O.from_p4(p), x)


@pytest.mark.parametrize("name", CASES)
def test_spectrum(name):
    g = load_golden(name)
    x = O.spectrum(g["samples"], g["input"].size)
    assert np.abs(x - g["input"]).max() <= 1e-6 * np.abs(g["input"]).max()


@pytest.mark.parametrize("name", CASES)
def test_tiles(name):
    g = load_golden(name)
    t = O.to_p4(O.tiles(g["input"]))
    assert t.shape[0] == int(g["n_tiles"]) == O.n_tiles(g["input"].size)
    # main_gtest.cpp:173-181 checks |d re|, |d im| < 1e-5
    d = t[g["tile_idx"]] - g["tiles_p4_ref"]
    assert np.abs(d.real).max() < 1e-5 and np.abs(d.imag).max() < 1e-5


@pytest.mark.parametrize("name", CASES)
def test_fop_fp64_vs_reference(name, bank):
    g = load_golden(name)
    f = O.fop(g["input"], bank)
    mean = f.mean(axis=1)
    rows = g["fop_rows"]
    # the reference FOP is float32 (scipy in single precision): 1e-5 of the row mean
    err = np.abs(f[rows] - g["fop_ref"]).max(axis=1) / mean[rows]
    assert err.max() < 1e-5
    # main_gtest.cpp:183-190 absolute criterion
    assert np.abs(f[rows] - g["fop_ref"]).max() < 1e-5
    assert np.allclose(f.sum(axis=1), g["fop_row_sum"], rtol=1e-6)


@pytest.mark.parametrize("name", ["n1000", "n4096"])
@pytest.mark.parametrize("thr_key", ["", "_chi2"])
def test_hsum_fp32_bit_exact(name, thr_key):
    """The float32 restatement reproduces hsum.py's candidate list bit for bit."""
    g = load_golden(name)
    hps = O.harmonic_planes(g["fop_ref"].astype(np.float32), 8, dtype=np.float32)
    thr = g["thresholds" + ("_chi2" if thr_key else "")]
    loc, pwr, *_ = O.detections(hps, thr)
    assert np.array_equal(loc, g["det_loc_ref" + thr_key])
    assert np.array_equal(pwr, g["det_pwr_ref" + thr_key])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("thr_key", ["", "_chi2"])
def test_fp64_candidates_vs_reference(name, thr_key, bank):
    """FP64 oracle candidates equal hsum.py's except cells within 1e-6 of the threshold."""
    g = load_golden(name)
    f = O.fop(g["input"], bank)
    hps = O.harmonic_planes(f, 8, dtype=np.float64)
    thr = g["thresholds" + thr_key]
    loc, pwr, plane, row, fq = O.detections(hps, thr)
    ref = g["det_loc_ref" + thr_key]
    diff = set(loc.tolist()) ^ set(ref.tolist())
    for d in diff:
        h, t, fb = O.decode_location(d)
        margin = abs(hps[h - 1][t + 42][fb] - thr[h - 1]) / thr[h - 1]
        assert margin < 1e-6, (h, t, fb, margin)
    common = np.isin(ref, loc)
    ref_pwr = g["det_pwr_ref" + thr_key][common]
    ours = dict(zip(loc.tolist(), pwr.tolist()))
    mine = np.array([ours[l] for l in ref[common].tolist()])
    mean = f.mean()
    if mine.size:
        assert np.abs(mine - ref_pwr).max() < 8 * 1e-5 * mean


def test_location_codec():
    loc = O.encode_location(np.array([1, 8, 3]), np.array([-42, 42, 0]), np.array([0, 0x3FFFFF, 12345]))
    h, t, f = O.decode_location(loc)
    assert list(h) == [1, 8, 3] and list(t) == [-42, 42, 0] and list(f) == [0, 0x3FFFFF, 12345]
    assert O.INVALID_LOCATION == (43 + 42) << 22


def test_compat_list_rule():
    rng = np.random.default_rng(0)
    n = 700
    loc = np.sort(rng.choice(1 << 22, n, replace=False)).astype(np.uint32)
    pwr = rng.random(n).astype(np.float32)
    plane = np.zeros(n, dtype=np.int64)
    L, P = O.compat_list(loc, pwr, plane, n_planes=2, per_plane=512)
    kept = L[:512]
    assert np.all(np.diff(kept.astype(np.int64)) > 0)
    assert P[:512].min() >= np.sort(pwr)[-512]
    assert np.all(L[512:] == O.INVALID_LOCATION) and np.all(P[512:] == -1.0)


def test_ring_list_matches_fpga_scan_order():
    """ring_list keeps the last 64 (group, bundle) events of the scan, slot = index mod 64."""
    # 70 events on plane 1 in the negative half: template 0, bins 0, 2, 4, ... (one hit per bundle)
    f = np.arange(70) * 2
    loc = O.encode_location(np.ones(70, dtype=np.int64), np.zeros(70, dtype=np.int64), f)
    pwr = np.arange(70, dtype=np.float32)
    L, P = O.ring_list(loc, pwr, "neg")
    L = L.reshape(8, 64, 8)
    # events 6..69 survive; event e sits in slot e % 64, lane 0
    h, t, fb = O.decode_location(L[0, :, 0])
    assert sorted(fb.tolist()) == sorted((np.arange(6, 70) * 2).tolist())
    assert L[0, 6 % 64, 0] == loc[6] and L[0, 69 % 64, 0] == loc[69]
    assert np.all(L[1:] == O.INVALID_LOCATION)
