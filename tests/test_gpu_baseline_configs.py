"""The three forms of the search at the sizes of their own workloads, against
the FP64 oracle (ft_conv.py:199-207 + hsum.py:95-151 in float64) and against
the plain path:

* precision form at 2^21 bins (the benchmark spectrum), split FP16 and split
  BF16 on tcgen05 (forward and inverse DFTs): candidate set equal to the FP64
  oracle's, FOP within bounds twice the measured errors;
* batched form over the 256-trial mix (2^17 .. 2^21 bins, log-uniform),
  autotuned: every trial's candidates equal to its own plain search, six
  trials (the shortest, the longest and four more) equal to the FP64 oracle;
* served form with a mix of 2^21-bin full-bank, 2^21-bin 16-plane, 2^21-bin
  half-bank and shorter requests: each result equal alone and in the mix, and
  the 2^21-bin requests equal to the FP64 oracle."""
import io

import numpy as np
import pytest

import full_oracle as F
from gpu_util import make_pipeline
from test_gpu_parity import fop_within, FOP_REL_TOL
from fdas_gb300 import synth
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

HALF = 42


def search(x, bank, thr, precision=0, n_templates=85, want_fop=False):
    p = make_pipeline(x.size, log=io.StringIO(), precision=precision, n_planes=thr.size, n_templates=n_templates,
                      max_template_len=bank.shape[1])
    assert p.upload_templates(bank, FDAS.A), p.last_error
    nc = p.get_candidate_list_sz()
    loc, pwr = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A), p.last_error
    rec, total, dropped = p.retrieve_candidate_list(FDAS.A)
    assert dropped == 0 and p.counters(FDAS.A)["status"] == 0
    fop = None
    if want_fop:
        fop = np.zeros(p.get_fop_sz(), np.float32)
        assert p.retrieve_FOP(fop, FDAS.A)
        fop = fop.reshape(n_templates, x.size)
    p.close()
    return rec, fop


@pytest.mark.parametrize("precision", [2, 1], ids=["split_fp16", "split_bf16"])
def test_precision_full_size_vs_fp64(precision):
    x, _, bank, fop64 = F.full_case()
    thr = O.chi2_thresholds(1e-6)
    rec, fop = search(x, bank, thr, precision=precision, want_fop=True)
    want, _ = F.full_case_candidates(8)
    got = F.record_keys(rec, HALF)
    print(f"precision {precision}: {got.size} candidates, oracle {want.size}")
    assert np.array_equal(got, want)
    mean = fop64.mean(axis=1, keepdims=True)
    err = np.abs(fop - fop64)
    weak = fop64 < 30 * mean
    print(f"FOP error: max |d| / plane mean {np.max(err / mean):.2e}, over cells below 30x the mean "
          f"{np.max((err / mean)[weak]):.2e}, max |d| / |FOP| over the others {np.max((err / fop64)[~weak]):.2e}, "
          f"within the FP32 path's tolerance: {fop_within(fop, fop64).mean():.9f} of the cells")
    # bounds of the split forms at this size, twice the measured errors (the
    # FP32 FFT meets 1e-5 x mean + 1e-6 x |FOP|, test_full_size_properties):
    # the tensor-core products carry the rounding of a tile's largest values
    # (the injected signals, ~10^4 x the mean) into the weak cells of the
    # same tile, in the forward and in the inverse DFT
    a, b = (1e-4, 4e-6) if precision == 2 else (2e-3, 6e-5)
    assert (err <= a * mean + b * np.abs(fop64)).all()


# ------------------------------------------------------------------ batched
def test_batched_mix_256_trials():
    from fdas_gb300.batch import Batch
    bank = template_bank()
    thr = O.chi2_thresholds(1e-6)
    n_bins, offs, d_all = synth.batch_mix(256)
    assert n_bins.min() >= 1 << 17 and n_bins.max() <= 1 << 21
    with Batch(bank, n_bins, autotune=True) as b:
        b.set_inputs_device(d_all.data_ptr())
        b.run(thr)
        b.run(thr)  # a graph replay gives the same results
        info = b.info()
        got = []
        for i in range(n_bins.size):
            rec, total, dropped = b.trial(i).retrieve_candidate_list(FDAS.A)
            assert dropped == 0 and total == rec.size
            got.append(rec)
    print("autotuned:", info)
    # every trial against its own plain search (one handle, reshaped per trial)
    p = make_pipeline(int(n_bins.max()), log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A)
    key = lambda r: F.record_keys(r, HALF)
    same_config = info["ftc_split"].startswith("warp pair") and info["ftc_ctas_per_sm"] == 2
    for i in range(n_bins.size):
        assert p.reshape(int(n_bins[i])), p.last_error
        assert p.enqueue_search_device(d_all.data_ptr() + 8 * int(offs[i]), thr, FDAS.AllAccelerations, FDAS.A)
        assert p.synchronize(FDAS.A), p.last_error
        rec, _, dropped = p.retrieve_candidate_list(FDAS.A)
        assert dropped == 0
        if same_config:  # the plain path's kernels and launch shape: bit-identical
            assert np.array_equal(got[i], rec), i
        else:  # another FFT split: the same cells (near-threshold cells go to the FP64 recheck)
            assert np.array_equal(key(got[i]), key(rec)), i
            np.testing.assert_allclose(got[i]["power"], rec["power"], rtol=1e-5, atol=1e-5 * 8)
    # six trials against the FP64 oracle
    rng = np.random.default_rng(1)
    pick = [int(np.argmin(n_bins)), int(np.argmax(n_bins))]
    pick += [int(i) for i in rng.choice(np.setdiff1d(np.arange(n_bins.size), pick), 4, replace=False)]
    host = d_all.cpu().numpy()
    for i in pick:
        x = host[2 * offs[i]:2 * offs[i + 1]].view(np.complex64)
        want, _ = F.candidate_keys(F.fop64(x, bank), thr, 8)
        print(f"trial {i}: {n_bins[i]} bins, {got[i].size} candidates")
        assert np.array_equal(key(got[i]), want), i


# ------------------------------------------------------------------ served
def served_spectrum(n, seed):
    rng = np.random.default_rng(seed)
    amp = 0.05 * np.sqrt((1 << 15) / n)
    sig = [dict(r0=float(rng.uniform(0.05, 0.45) * n), z=float(rng.uniform(-40, 40)), n_harm=int(rng.integers(1, 9)),
                amp=amp) for _ in range(2)]
    return synth.spectrum(synth.timeseries(2 * n, sig, seed=seed), n)[0]


def test_served_mix_full_size():
    from fdas_gb300.server import Server, HALF_BANK
    bank = template_bank()
    x_full = F.full_case()[0]
    specs = {"full8": x_full, "full16": x_full, "half8": served_spectrum(1 << 21, 31),
             "m20h16": served_spectrum(1 << 20, 32), "s17f4": served_spectrum(1 << 17, 33),
             "s18f8": served_spectrum(200_003, 34)}
    reqs = {"full8": (None, 8), "full16": (None, 16), "half8": (HALF_BANK, 8), "m20h16": (HALF_BANK, 16),
            "s17f4": (None, 4), "s18f8": (None, 8)}
    names = list(reqs)
    with Server(bank, max_bins=1 << 21, max_slots=6, max_planes=16, candidate_capacity=1 << 23) as srv:
        alone = {k: srv.result(srv.submit(specs[k], O.chi2_thresholds(1e-6, reqs[k][1]), reqs[k][0]),
                               timeout_ms=120_000) for k in names}
        ids = [(k, srv.submit(specs[k], O.chi2_thresholds(1e-6, reqs[k][1]), reqs[k][0])) for k in names + names]
        mixed = [(k, srv.result(rid, timeout_ms=120_000)) for k, rid in ids]
        st = srv.stats()
    assert st["peak_in_flight"] >= 2
    for k, (rec, total, dropped, _) in mixed:
        assert dropped == 0 and alone[k][2] == 0
        assert np.array_equal(rec, alone[k][0]), k
    # the 2^21-bin requests against the FP64 oracle
    for k, planes in (("full8", 8), ("full16", 16)):
        want, _ = F.full_case_candidates(planes)
        assert np.array_equal(F.record_keys(alone[k][0], HALF), want), k
    half_taps = np.ascontiguousarray(bank[HALF_BANK[0]:HALF_BANK[0] + HALF_BANK[1], :211])
    thr8 = O.chi2_thresholds(1e-6, 8)
    want, _ = F.candidate_keys(F.fop64(specs["half8"], half_taps), thr8, 8)
    assert np.array_equal(F.record_keys(alone["half8"][0], HALF_BANK[1] // 2), want)
