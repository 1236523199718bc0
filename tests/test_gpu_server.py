"""Served form: the request server (fdas_server_*) and fdas_reshape.

* a reshaped handle gives the same FOP and candidates as a handle initialised
  for that shape;
* requests of mixed lengths, banks (full / half) and plane counts submitted at
  once give exactly the results each gives alone, and the full-bank 8-plane
  request equals the plain fdas_launch path."""
import io

import numpy as np
import pytest

from gpu_util import make_pipeline
from fdas_gb300 import synth
from fdas_gb300.fdas import FDAS
from fdas_gb300.server import Server, HALF_BANK
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu


def spectrum(n, seed):
    """Unit-power spectrum of noise + two accelerated signals of moderate
    strength (peak power ~40x the mean whatever the length)."""
    rng = np.random.default_rng(seed)
    amp = 0.05 * np.sqrt((1 << 15) / n)
    sig = [dict(r0=float(rng.uniform(0.05, 0.45) * n), z=float(rng.uniform(-40, 40)), n_harm=int(rng.integers(1, 6)),
                amp=amp) for _ in range(2)]
    return synth.spectrum(synth.timeseries(2 * n, sig, seed=seed), n)[0]


def thresholds(n_planes):
    return O.chi2_thresholds(1e-6, n_planes)


def plain_search(x, bank, thr, n_templates=85, rows=None, tile_overlap=0):
    p = make_pipeline(x.size, log=io.StringIO(), n_planes=thr.size, n_templates=n_templates,
                      tile_overlap=tile_overlap)
    b = bank if rows is None else np.ascontiguousarray(bank[rows[0]:rows[0] + rows[1]])
    assert p.upload_templates(b, FDAS.A), p.last_error
    nc = p.get_candidate_list_sz()
    loc, pwr = np.zeros(nc, np.uint32), np.zeros(nc, np.float32)
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A), p.last_error
    rec, _, _ = p.retrieve_candidate_list(FDAS.A)
    return rec


def test_reshape_equals_fresh_handle():
    bank = template_bank()
    n0, n1 = 1 << 16, 40_000
    x = spectrum(n1, 3)
    thr = thresholds(4)
    p = make_pipeline(n0, log=io.StringIO(), n_planes=16)
    assert p.upload_templates(bank, FDAS.A)
    # half bank, 4 planes, fewer bins; overlap from the longest template of the range (211 taps -> 212)
    assert p.reshape(n1, HALF_BANK[0], HALF_BANK[1], 0, 4), p.last_error
    assert p.get_input_sz() == n1 and p.get_thresholds_sz() == 4
    assert p.perform_input_tiling(x, FDAS.A) and p.perform_ft_convolution(FDAS.AllAccelerations, FDAS.A)
    fop = np.zeros(p.get_fop_sz(), np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    assert p.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A), p.last_error
    rec, _, _ = p.retrieve_candidate_list(FDAS.A)
    # the half bank's taps are the first 211 of each row (left aligned)
    q = make_pipeline(n1, log=io.StringIO(), n_planes=4, n_templates=43, max_template_len=211)
    assert q.upload_templates(np.ascontiguousarray(bank[21:64, :211]), FDAS.A)
    assert q.perform_input_tiling(x, FDAS.A) and q.perform_ft_convolution(FDAS.AllAccelerations, FDAS.A)
    fop_q = np.zeros(q.get_fop_sz(), np.float32)
    assert q.retrieve_FOP(fop_q, FDAS.A)
    assert q.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A), q.last_error
    rec_q, _, _ = q.retrieve_candidate_list(FDAS.A)
    assert np.array_equal(fop, fop_q)
    assert rec.size > 0 and np.array_equal(rec, rec_q)
    # too large for the allocation
    assert not p.reshape(n0 + 1, 0, 85, 0, 8)


REQUESTS = [  # (bins, template rows or None = full bank, planes, seed)
    (1 << 15, None, 8, 1), (40_000, HALF_BANK, 4, 2), (1 << 16, None, 16, 3), (70_001, HALF_BANK, 8, 4),
    (1 << 17, None, 8, 5), (1 << 15, HALF_BANK, 16, 6), (50_000, None, 4, 7), (1 << 16, HALF_BANK, 8, 8),
]


def run_requests(srv, reqs, at_once):
    out = {}
    if at_once:
        specs = [spectrum(n, s) for n, rows, P, s in reqs]  # made first, then submitted back to back
        ids = [srv.submit(x, thresholds(P), rows) for x, (n, rows, P, s) in zip(specs, reqs)]
        for i, rid in enumerate(ids):
            out[i] = srv.result(rid, timeout_ms=60_000)
    else:
        for i, (n, rows, P, s) in enumerate(reqs):
            out[i] = srv.result(srv.submit(spectrum(n, s), thresholds(P), rows), timeout_ms=60_000)
    return out


def test_server_mix_equals_alone():
    bank = template_bank()
    with Server(bank, max_bins=1 << 17, max_slots=4) as srv:
        alone = run_requests(srv, REQUESTS, at_once=False)
    with Server(bank, max_bins=1 << 17, max_slots=4) as srv:
        run_requests(srv, REQUESTS, at_once=True)  # creates the slots
        mixed = run_requests(srv, REQUESTS + REQUESTS, at_once=True)
        st = srv.stats()
    assert st["completed"] == 3 * len(REQUESTS) and st["peak_in_flight"] >= 2
    for i in range(len(REQUESTS)):
        rec_a, n_a, d_a, _ = alone[i]
        for rec_m, n_m, d_m, _ in (mixed[i], mixed[i + len(REQUESTS)]):
            assert d_a == 0 and d_m == 0 and n_a == n_m
            assert np.array_equal(rec_a, rec_m), i
    # full bank, 8 planes: the plain launch path on its own handle
    n, rows, P, s = REQUESTS[4]
    rec_plain = plain_search(spectrum(n, s), bank, thresholds(P))
    assert np.array_equal(mixed[4][0], rec_plain)
    assert mixed[4][1] > 0


def test_server_rejects():
    bank = template_bank()
    with Server(bank, max_bins=1 << 15, max_slots=1) as srv:
        with pytest.raises(ValueError):
            srv.submit(spectrum(1 << 16, 1), thresholds(8))      # longer than max_bins
        with pytest.raises(ValueError):
            srv.submit(spectrum(1 << 15, 1), thresholds(8), (0, 84))  # even template count
        with pytest.raises(ValueError):
            srv.submit(spectrum(1 << 15, 1), np.ones(17, np.float32))  # more planes than max_planes
