"""Tracing lines with the reference's field layout, and the failure paths that
can be driven without faulting a GPU: a device wait that runs out (the kernels
stop, report FDAS_ERR_TIMEOUT and leave the handle usable) and a host-side
wait on the request server that expires.

Reference: FDAS.cpp:60-63 ("^^^" clock sync), 556-575 ("[INFO] Enqueueing",
"%%%" host enqueue times), 643-666 (print_stats "complete @ ... II ~ ..."),
668-686 (print_events "@@@" stage boundaries), 34-52 (errors are reported,
never fatal)."""
import io
import re
import time

import numpy as np
import pytest

from fdas_gb300 import _lib, synth
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from gpu_util import make_pipeline
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

INT = r"(-?\d+)"
RE_SYNC = re.compile(rf"^\^\^\^,{INT},{INT}$")
RE_ENQ = re.compile(r"^\[INFO\] Enqueueing: ([AB])\n(?:       \d+ms\n){4}       \d+ms$")
RE_HOST = re.compile(rf"^%%%,([AB]),{INT},{INT},{INT},{INT},{INT},$")
RE_DONE = re.compile(r"^\[INFO\] Launch  #(\d+)([AB]) complete @ ([\d.]+) ms II ~ ([\d.]+) ms$")
RE_DUR = re.compile(r"^\[INFO\]   (Preparation|FT convolution and IFFT|Harmonic summing|Total) duration: ([\d.]+) ms$")
RE_EV = re.compile(r"^@@@,([AB])" + rf",{INT}" * 10 + "$")


class Lines:
    """A log sink that keeps whole lines (a line may span several newlines)."""

    def __init__(self):
        self.lines = []

    def write(self, s):
        self.lines.append(s[:-1] if s.endswith("\n") else s)


def _case(n=8192, seed=11):
    samples, _ = synth.small_case(n, seed=seed)
    x, _ = synth.spectrum(samples)
    return x, O.chi2_thresholds(1e-6)


def test_trace_lines_reference_layout():
    x, thr = _case()
    log = Lines()
    t_init0, w_init0 = time.monotonic_ns(), time.time_ns()
    p = make_pipeline(x.size, log=log, trace_enqueue=True)
    t_init1, w_init1 = time.monotonic_ns(), time.time_ns()
    # "^^^,<system ns>,<steady ns>" comes first, from initialisation itself
    m = RE_SYNC.match(log.lines[0])
    assert m, log.lines[:2]
    assert w_init0 - 10**9 <= int(m.group(1)) <= w_init1 + 10**9
    assert t_init0 <= int(m.group(2)) <= t_init1  # std::chrono::steady_clock is CLOCK_MONOTONIC
    bank = template_bank()
    assert p.upload_templates(bank, FDAS.A) and p.upload_templates(bank, FDAS.B)
    n = p.get_candidate_list_sz()
    loc = np.zeros(n, np.uint32)
    pwr = np.zeros(n, np.float32)
    done_at = []
    windows = []
    for i in range(4):
        ab = FDAS.A if i % 2 == 0 else FDAS.B
        del log.lines[:]
        t0 = time.monotonic_ns()
        assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, ab), p.last_error
        assert p.wait(ab), p.last_error
        t1 = time.monotonic_ns()
        p.print_stats(ab, i == 0)
        p.print_events(ab)
        lines = log.lines
        enq = [ln for ln in lines if RE_ENQ.match(ln)]
        host = [RE_HOST.match(ln) for ln in lines if RE_HOST.match(ln)]
        assert len(enq) == 1 and len(host) == 1, lines
        h = [int(v) for v in host[0].groups()[1:]]
        assert host[0].group(1) == "AB"[ab]
        assert t0 <= h[0] <= h[1] <= h[2] <= h[3] <= h[4] <= t1
        done = [RE_DONE.match(ln) for ln in lines if RE_DONE.match(ln)]
        assert len(done) == 1 and int(done[0].group(1)) == i + 1 and done[0].group(2) == "AB"[ab]
        done_at.append((float(done[0].group(3)), float(done[0].group(4))))
        durs = {mm.group(1): float(mm.group(2)) for mm in map(RE_DUR.match, lines) if mm}
        assert set(durs) == {"Preparation", "FT convolution and IFFT", "Harmonic summing", "Total"}
        assert all(v >= 0 for v in durs.values())
        ev = [RE_EV.match(ln) for ln in lines if RE_EV.match(ln)]
        assert len(ev) == 1 and ev[0].group(1) == "AB"[ab]
        e = [int(v) for v in ev[0].groups()[1:]]
        # ten stage boundaries in order on the host's steady clock; a stage
        # starts where the one before it ends on the set's stream
        assert all(a <= b for a, b in zip(e, e[1:])), e
        assert e[1] == e[2] and e[3] == e[4] and e[5] == e[6] and e[7] == e[8]
        slack = 2_000_000  # the anchor maps device events onto the host clock to within microseconds
        assert h[0] - slack <= e[0] and e[9] <= t1 + slack
        windows.append((e[0], e[9]))
    # "complete @" grows along the series; II is its increase
    assert all(b[0] > a[0] for a, b in zip(done_at, done_at[1:]))
    for a, b in zip(done_at, done_at[1:]):
        assert abs((b[0] - a[0]) - b[1]) < 2e-3
    assert abs(done_at[0][0] - done_at[0][1]) < 1e-3  # first launch: II equals the time since the series start
    assert abs(done_at[-1][0] - (windows[-1][1] - windows[0][0]) * 1e-6) < 2e-3


def test_trace_off_by_default():
    x, thr = _case()
    log = Lines()
    p = make_pipeline(x.size, log=log)
    assert p.upload_templates(template_bank(), FDAS.A)
    n = p.get_candidate_list_sz()
    loc, pwr = np.zeros(n, np.uint32), np.zeros(n, np.float32)
    del log.lines[:]
    assert p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A)
    assert not any(RE_HOST.match(ln) or RE_ENQ.match(ln) for ln in log.lines)


def _search(p, x, thr):
    n = p.get_candidate_list_sz()
    loc, pwr = np.zeros(n, np.uint32), np.zeros(n, np.float32)
    ok = p.launch(x, thr, loc, pwr, FDAS.AllAccelerations, FDAS.A) and p.wait(FDAS.A)
    return ok, loc, pwr


@pytest.mark.parametrize("hook,bit,what", [(_lib.INJECT_FTC_STALL, 16, "FT convolution"),
                                           (_lib.INJECT_HSUM_STALL, 1, "harmonic summing")],
                         ids=["ft_convolution", "harmonic_summing"])
def test_device_wait_timeout_reported_and_recovered(hook, bit, what):
    """A device wait that runs out: a test hook announces copies on a barrier
    without issuing them (each warp pair's first template copy of the FT
    convolution, or the first staged item of every harmonic-summing CTA), so
    that wait can never complete.  After the (shortened) bound the kernel
    stops, the search reports FDAS_ERR_TIMEOUT with the stage's timeout bit,
    and once the hook is off the next searches on the same handle are exact
    again -- the context stays usable."""
    x, thr = _case(n=1 << 15, seed=5)
    bank = template_bank()
    ref = make_pipeline(x.size, log=io.StringIO())
    assert ref.upload_templates(bank, FDAS.A)
    ok, ref_loc, ref_pwr = _search(ref, x, thr)
    assert ok, ref.last_error
    ref_rec, _, _ = ref.retrieve_candidate_list(FDAS.A)

    p = make_pipeline(x.size, log=io.StringIO())
    assert p.upload_templates(bank, FDAS.A)
    assert p.set_wait_timeout(1_000_000)  # 1 ms
    assert p.set_fault_injection(hook)
    for _ in range(2):
        t0 = time.monotonic()
        ok, _, _ = _search(p, x, thr)
        assert not ok
        assert p.last_status == _lib.ERR_TIMEOUT, p.last_error
        assert what in p.last_error
        assert p.counters(FDAS.A)["status"] & bit
        assert time.monotonic() - t0 < 1.5  # the bound, not the 2 s default, ended the wait
    assert not p.set_fault_injection(4)  # unknown flags are refused
    assert p.set_fault_injection(0)
    assert p.set_wait_timeout(0)  # back to 2 s
    for _ in range(2):
        ok, loc, pwr = _search(p, x, thr)
        assert ok, p.last_error
        assert p.counters(FDAS.A)["status"] == 0
        assert np.array_equal(loc, ref_loc) and np.array_equal(pwr, ref_pwr)
        rec, _, _ = p.retrieve_candidate_list(FDAS.A)
        assert np.array_equal(rec, ref_rec)


def test_server_wait_expires_then_collects():
    """fdas_server_wait with a limit that runs out reports FDAS_ERR_TIMEOUT and
    keeps the request; a later wait collects the same result as a plain
    search; an unknown id is an argument error."""
    from fdas_gb300.server import Server
    bank = template_bank()
    n = 1 << 17
    x, _ = synth.spectrum(synth.timeseries(2 * n, [dict(r0=0.3 * n, z=12.0, n_harm=4, amp=0.004)], seed=3), n)
    thr = O.chi2_thresholds(1e-6)
    with Server(bank, max_bins=n, max_slots=2) as srv:
        rid = srv.submit(x, thr)
        with pytest.raises(TimeoutError):
            srv.result(rid, timeout_ms=0)  # the first request also creates its slot: not done in 0 ms
        rec, total, dropped, lat = srv.result(rid)
        assert dropped == 0 and lat > 0
        with pytest.raises(RuntimeError):
            srv.result(rid + 1000)
    p = make_pipeline(n, log=io.StringIO(), n_planes=8)
    assert p.upload_templates(bank, FDAS.A)
    ok, _, _ = _search(p, x, thr)
    assert ok, p.last_error
    want, want_total, _ = p.retrieve_candidate_list(FDAS.A)
    assert total == want_total and np.array_equal(rec, want)


def test_stream_priority_same_results():
    """fdas_config.stream_priority only orders work on the device: a handle
    on high-priority streams gives the same candidate lists."""
    x, thr = _case(n=1 << 15, seed=7)
    bank = template_bank()
    out = []
    for prio in (0, -5):
        p = make_pipeline(x.size, log=io.StringIO(), stream_priority=prio)
        assert p.upload_templates(bank, FDAS.A)
        ok, loc, pwr = _search(p, x, thr)
        assert ok, p.last_error
        rec, _, _ = p.retrieve_candidate_list(FDAS.A)
        out.append((loc, pwr, rec))
        p.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])
