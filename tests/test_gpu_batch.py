"""Batched form (fdas_batch_*): trials of uneven length searched in one pass
(one tiling launch, persistent FT-convolution launches over all trials'
(tile, template) items -- one, or one per group of trials, as tuned --
per-trial harmonic summing on branch streams, all in one CUDA graph) against
plain searches of each trial on its own handle."""
import io

import numpy as np
import pytest

from gpu_util import make_pipeline
from fdas_gb300 import synth
from fdas_gb300.batch import Batch
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

N_BINS = [32768, 40000, 65536, 100003, 20000, 131072]


def spectrum(n, seed):
    rng = np.random.default_rng(seed)
    amp = 0.05 * np.sqrt((1 << 15) / n)
    sig = [dict(r0=float(rng.uniform(0.05, 0.45) * n), z=float(rng.uniform(-42, 42)), n_harm=int(rng.integers(1, 9)),
                amp=amp) for _ in range(int(rng.integers(0, 3)))]
    return synth.spectrum(synth.timeseries(2 * n, sig, seed=seed), n)[0]


def plain(x, bank, thr):
    p = make_pipeline(x.size, log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A)
    nc = p.get_candidate_list_sz()
    loc, pwr = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A), p.last_error
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    fop = np.zeros(p.get_fop_sz(), np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    return rec, loc, pwr, fop


def batch_results(b, i):
    v = b.trial(i)
    rec, total, dropped = v.retrieve_candidate_list(FDAS.A)
    nc = v.get_candidate_list_sz()
    loc, pwr = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert v.retrieve_candidates(loc, pwr, FDAS.A)
    fop = np.zeros(v.get_fop_sz(), np.float32)
    assert v.retrieve_FOP(fop, FDAS.A)
    assert dropped == 0
    return rec, loc, pwr, fop


@pytest.fixture(scope="module")
def inputs():
    bank = template_bank()
    xs = [spectrum(n, 10 + i) for i, n in enumerate(N_BINS)]
    thr = O.chi2_thresholds(1e-6, 8)
    ref = [plain(x, bank, thr) for x in xs]
    return bank, xs, thr, ref


def test_batch_equals_plain_searches(inputs):
    bank, xs, thr, ref = inputs
    with Batch(bank, N_BINS, autotune=False) as b:
        b.set_tuning(2, 2, False)  # the plain path's configuration: bit-identical results
        b.set_inputs(xs)
        b.run(thr)
        for i in range(len(N_BINS)):
            rec, loc, pwr, fop = batch_results(b, i)
            r_rec, r_loc, r_pwr, r_fop = ref[i]
            assert np.array_equal(fop, r_fop), i
            assert np.array_equal(rec, r_rec), i
            assert np.array_equal(loc, r_loc) and np.array_equal(pwr, r_pwr), i
        # graph replay on new inputs (trials in reverse order of seeds) and back
        b.set_inputs([spectrum(n, 99 + i) for i, n in enumerate(N_BINS)])
        b.run(thr)
        b.set_inputs(xs)
        b.run(thr)
        for i in range(len(N_BINS)):
            assert np.array_equal(batch_results(b, i)[0], ref[i][0]), i


def test_batch_autotuned_same_candidates(inputs):
    bank, xs, thr, ref = inputs
    with Batch(bank, N_BINS, autotune=True) as b:
        b.set_inputs(xs)
        b.run(thr)
        info = b.info()
        assert info["tuned"] and len(info["tune_ms"]) == 8 and min(info["tune_ms"]) > 0
        assert info["ftc_launches"] in (1, 4, 16)
        for i in range(len(N_BINS)):
            rec, loc, pwr, fop = batch_results(b, i)
            r_rec = ref[i][0]
            # whatever FFT split was chosen: the same cells (the FP64 recheck
            # decides near-threshold cells), powers within the FOP tolerance
            key = lambda r: list(zip(r["harmonic"], r["template_num"], r["bin"]))
            assert key(rec) == key(r_rec), i
            np.testing.assert_allclose(rec["power"], r_rec["power"], rtol=1e-5, atol=1e-5 * 8)


@pytest.mark.parametrize("groups", [1, 4, 16])
def test_batch_groupings_equal_plain(groups):
    """Every grouping of the FT convolution (one launch over the whole
    (trial, tile, template) queue, or one launch per run of trials; each warp
    pair walks forward through the trial table of its launch) gives the plain
    searches' FOPs and candidate lists bit for bit, also when trials outnumber
    groups so that a launch spans several trials."""
    bank = template_bank()
    thr = O.chi2_thresholds(1e-6, 8)
    n_bins = [1628 * 3 + 17, 20000, 4096, 70001, 1628, 33333, 9000, 131072, 2048, 50000, 1, 12345]
    xs = [spectrum(n, 200 + i) if n > 1 else np.ones(1, np.complex64) for i, n in enumerate(n_bins)]
    ref = [plain(x, bank, thr) for x in xs]
    with Batch(bank, n_bins, autotune=False) as b:
        b.set_tuning(2, 2, False)
        b.set_groups(groups)
        assert b.info()["ftc_launches"] == groups
        b.set_inputs(xs)
        b.run(thr)
        for i in range(len(n_bins)):
            rec, loc, pwr, fop = batch_results(b, i)
            r_rec, r_loc, r_pwr, r_fop = ref[i]
            assert np.array_equal(fop, r_fop), (groups, i)
            assert np.array_equal(rec, r_rec), (groups, i)
            assert np.array_equal(loc, r_loc) and np.array_equal(pwr, r_pwr), (groups, i)
        with pytest.raises(RuntimeError):
            b.set_groups(17)
