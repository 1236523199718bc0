#!/usr/bin/env python3
"""Benchmark: FDAS searches/s at 2^21 bins x 85 templates x 8 harmonics on GB300.

One step = one full search of one spectrum: overlap-save tiling + forward FFT,
FT convolution of all 85 templates into the filter-output plane (FOP), 8-plane
harmonic summing with chi-square thresholds (FAR 1e-6), FP64 recheck and the
sorted candidate list.

* ``value``: searches/s with the spectrum already resident in HBM
  (fdas_enqueue_search_device), timed with CUDA events on the library's
  streams; the best of three issue forms (``mode``): one buffer set
  (sequential), searches alternating between sets A and B (alternating), and
  A/B with the overlap configuration (pipelined); all three are reported.
* ``e2e``: the same metric through the reference-facing call (fdas_launch /
  fdas_wait) with pinned HOST buffers: the 2^21-bin spectrum is copied in and
  the 4096-entry candidate list copied out inside every step.
* ``roofline``: the dominant kernel's algorithmic bytes / its average duration
  (CUDA events around each stage) against the measured HBM copy bandwidth.
* ``cpu_baseline``: the oracle port (NumPy/SciPy restatement of the reference's
  ft_conv.py + hsum.py) on a bounded sample, extrapolated to one search.

``--impl reference`` times the reference's own CPU path (the oracle port of
ft_conv.py / hsum.py: float32/complex64 like the reference) with all host cores.
Multi-GPU (torchrun, N > 1): independent replicas, one search stream per rank,
no collective on the data path; value = all ranks' searches / max time.
"""
import argparse
import json
import os
import pathlib
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_BINS = 1 << 21
N_TEMPLATES = 85
N_PLANES = 8
METRIC = "searches/s at 2^21 bins x 85 tmpl x 8 harm"
UNIT = "searches/s"
WORKLOAD = {"workload": "FDAS full single-trial search: 2^22-sample Gaussian series -> 2^21 complex64 bins, "
                        "3 injected accelerated signals (z -30/0/+35), 85 x 421-tap Fresnel template bank, "
                        "2048-point overlap-save tiles (overlap 420, 1289 tiles), 8 harmonic planes, "
                        "chi-square thresholds FAR 1e-6, all accelerations",
            "n_bins": N_BINS, "n_templates": N_TEMPLATES, "n_planes": N_PLANES, "tile": 2048, "overlap": 420,
            "l2": "inputs larger than L2: each search writes and reads a 713 MB FOP (L2 is 129 MB)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(v, device):
    """The largest ``v`` over the ranks (one rank: ``v``).  Timings are
    combined this way: the job ends when its slowest replica ends."""
    ws, _, _ = dist_env()
    if ws == 1:
        return float(v)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, seconds, ws):
    """Units all replicas processed per second of the slowest one."""
    return ws * units_per_rank / seconds


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_bf16_peak():
    """Dense BF16 tensor rate (TFLOP/s) for a kernel timed alone: the burst
    figure of MEASURED_PEAKS.json, else the fallback measurement."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


# tensor-core work of one (tile, template) item in the precision form: the
# inverse DFT as DFT-64 (M 128 x K 128 x N 32 per item) and DFT-32 (M 128 x
# K 64 x N 64 per two items) real GEMMs, each as three split products
# (hi*hi + hi*lo + lo*hi)
TC_FLOPS_PER_ITEM = 3 * (2 * 128 * 128 * 32 + 2 * 64 * 64 * 64)


# ------------------------------------------------------------------ CPU side
def cpu_search(x, bank, thr, ex, workers):
    """One whole CPU search of the reference's path at its own precision:
    the FOP of all 85 rows by direct linear convolution in complex64
    (ft_conv.py:199-205: scipy.signal.convolve with the non-zero taps) and
    harmonic summing of all bins, rows and planes in float32 with the
    reference's index math and strict '>' (hsum.py:95-151, vectorised).  FOP
    rows and harmonic-summing bin ranges are spread over the ``workers``
    threads of the pool ``ex`` (SciPy's FFTs and NumPy's loops release the
    GIL).  Returns (seconds, candidates)."""
    from oracle import fdas_oracle as O
    n = x.size
    fop = np.empty((N_TEMPLATES, n), dtype=np.float32)

    def rows(rs):
        fop[rs] = O.fop(x, bank, dtype=np.float32, rows=rs)

    def hsum(b):
        return O.detections_streaming(fop, thr, N_PLANES, dtype=np.float32, bins=b)[0]

    t0 = time.perf_counter()
    list(ex.map(rows, [list(c) for c in np.array_split(np.arange(N_TEMPLATES), workers) if len(c)]))
    edges = np.linspace(0, n, 4 * workers + 1).astype(np.int64)
    locs = list(ex.map(hsum, list(zip(edges[:-1], edges[1:]))))
    n_cand = int(sum(v.size for v in locs))
    return time.perf_counter() - t0, n_cand


CPU_SAMPLE = ("whole search, nothing sampled or extrapolated: FOP of all 85 rows x 2^21 bins by direct "
              "linear convolution in complex64 (scipy.signal.convolve, ft_conv.py:199-205) + harmonic summing "
              "of all 85 rows x 2^21 bins x 8 planes in float32 (hsum.py:95-151 vectorised), the reference's "
              "CPU path at its own precision, rows and bin ranges spread over {w} host threads; "
              "{c} candidates per search")


def fp32_pipe(ftc_ms, n_bins, clocks):
    import torch
    n_tiles = -(-n_bins // 1628)
    flops = n_tiles * N_TEMPLATES * (6 * 2048 + 5 * 2048 * 11 + 3 * 2048)
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    n_sm = torch.cuda.get_device_properties(0).multi_processor_count
    peak = n_sm * 128 * 2 * mhz * 1e6 / 1e12
    achieved = flops / (ftc_ms / 1e3) / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "algorithmic_flops_per_launch": flops, "peak_source": f"nominal: {n_sm} SMs x 128 FP32 lanes x 2 x "
                                                                 f"{mhz:.0f} MHz"}


def make_inputs(n_bins=N_BINS, noise_only=False):
    from fdas_gb300 import synth
    from fdas_gb300.templates import template_bank
    samples = synth.timeseries(1 << 22, (), seed=7) if noise_only else synth.full_case()[0]
    x, _ = synth.spectrum(samples[:2 * n_bins])
    bank = template_bank()
    from scipy.stats import gamma
    thr = np.array([gamma.isf(1e-6, k) for k in range(1, N_PLANES + 1)], dtype=np.float32)
    return x, bank, thr


# ------------------------------------------------------------------ arms
def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from concurrent.futures import ThreadPoolExecutor
    x, bank, thr = make_inputs()
    workers = os.cpu_count() or 1
    times = []
    with ThreadPoolExecutor(workers) as ex:
        for i in range(args.warmup + args.steps):
            t, n_cand = cpu_search(x, bank, thr, ex, workers)
            if i >= args.warmup:
                times.append(t)
    ms = 1e3 * float(np.mean(times))
    v = 1e3 / ms
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(WORKLOAD, parallelism="replicas1"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
                             "sample": "one step = one " + CPU_SAMPLE.format(w=workers, c=n_cand)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from fdas_gb300.fdas import FDAS, PinnedArray

    n_bins = args.bins
    x, bank, thr = make_inputs(n_bins, args.noise_only)
    log = open(os.devnull, "w")
    d_x = None

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def make_handle(overlap):
        h = FDAS(log)
        assert h.initialise_accelerator(n_bins, device=local, overlap=overlap), h.last_error
        assert h.upload_templates(bank, FDAS.A), h.last_error
        assert h.upload_templates(bank, FDAS.B), h.last_error
        return h

    def timed_device_loop(h, sets, steps, clocks=None):
        """K searches on the device-resident spectrum; sets alternate per step.
        CUDA events on the library streams (stream A brackets the region)."""
        streams = {ab: torch.cuda.ExternalStream(h.stream(ab), device=f"cuda:{local}") for ab in sets}
        for i in range(args.warmup):
            ab = sets[i % len(sets)]
            assert h.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, ab), h.last_error
        for ab in sets:
            assert h.synchronize(ab)
        sa = streams[sets[0]]
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        per = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)] if len(sets) == 1 else None
        barrier()
        torch.cuda.synchronize()
        ev0.record(sa)
        for ab in sets[1:]:
            streams[ab].wait_event(ev0)
        if per:
            per[0].record(sa)
        for i in range(steps):
            ab = sets[i % len(sets)]
            assert h.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, ab), h.last_error
            if per:
                per[i + 1].record(sa)
        for ab in sets[1:]:
            sa.wait_stream(streams[ab])
        ev1.record(sa)
        for ab in sets:
            assert h.synchronize(ab)
        torch.cuda.synchronize()
        barrier()
        total = ev0.elapsed_time(ev1)
        lat = np.array([per[i].elapsed_time(per[i + 1]) for i in range(steps)]) if per else None
        return total, lat

    def max_over_ranks(v):
        return reduce_max(v, f"cuda:{local}")

    d_x = torch.from_numpy(x.view(np.float32)).to(f"cuda:{local}")
    # sequential form: one buffer set, one stream; gives the per-search latency
    p = make_handle(False)
    with ClockSampler(local) as clocks_seq:
        seq_ms, per = timed_device_loop(p, [FDAS.A], args.steps)
    seq_ms = max_over_ranks(seq_ms)
    counters = p.counters(FDAS.A)
    n_cand = sum(counters["per_plane"])
    dropped = max(0, n_cand - counters["records"])
    # alternating form: the same handle, searches alternate between buffer
    # sets A and B on their own streams, so one search's kernels start on the
    # SMs the previous search's kernels release at their ends
    with ClockSampler(local) as clocks_alt:
        alt_ms, _ = timed_device_loop(p, [FDAS.A, FDAS.B], args.steps)
    alt_ms = max_over_ranks(alt_ms)
    # pipelined form: A/B as above with kernels sized so that the FT
    # convolution of one search and the harmonic summing of the previous share
    # every SM for their whole duration
    q = make_handle(True)
    with ClockSampler(local) as clocks:
        pipe_ms, _ = timed_device_loop(q, [FDAS.A, FDAS.B], args.steps)
    pipe_ms = max_over_ranks(pipe_ms)
    runs = {"sequential": (seq_ms, clocks_seq, p), "alternating": (alt_ms, clocks_alt, p),
            "pipelined": (pipe_ms, clocks, q)}
    mode = min(runs, key=lambda k: runs[k][0])
    total_ms = runs[mode][0]
    value = whole_job_rate(args.steps, total_ms / 1e3, ws)
    clk = runs[mode][1].summary()  # clocks of the reported loop
    mode_values = {f"value_{k}": whole_job_rate(args.steps, v[0] / 1e3, ws) for k, v in runs.items()}

    # ---- stage times (separate pass, so the per-launch host syncs do not
    # disturb the throughput number above)
    n_stage = min(args.steps, 50)
    st = []
    for i in range(n_stage):
        assert p.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, FDAS.A)
        st.append(p.stage_times(FDAS.A))
    st = np.array(st)
    names = ["input", "tiling", "ft_convolution", "harmonic_summing", "download", "total"]
    stage_ms = {n: float(np.mean(st[:, i])) for i, n in enumerate(names)}
    alg = {"tiling": 8 * n_bins, "ft_convolution": 4 * N_TEMPLATES * n_bins,
           "harmonic_summing": 4 * N_TEMPLATES * n_bins}
    dom = max(alg, key=lambda k: stage_ms[k])
    peak, peak_kind = measured_peaks()
    achieved = alg[dom] / (stage_ms[dom] / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(dom)

    # ---- e2e: pinned host buffers through fdas_launch / fdas_wait, A/B sets
    if args.no_e2e:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_bins": n_bins, "mode": mode,
                              **mode_values,
                              "stage_ms": stage_ms, "counters": counters, "profile_run": True}), flush=True)
        return
    hx = {ab: PinnedArray((n_bins,), np.complex64) for ab in (FDAS.A, FDAS.B)}
    for ab in hx:
        hx[ab].array[:] = x
    n_list = p.get_candidate_list_sz()
    hl = {ab: PinnedArray((n_list,), np.uint32) for ab in (FDAS.A, FDAS.B)}
    hp = {ab: PinnedArray((n_list,), np.float32) for ab in (FDAS.A, FDAS.B)}
    e2e_steps = args.steps
    ep = runs[mode][2]  # the faster configuration
    for i in range(args.warmup):
        ab = i & 1
        assert ep.launch(hx[ab].array, thr, hl[ab].array, hp[ab].array, FDAS.AllAccelerations, ab)
        assert ep.wait(ab)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        ab = i & 1
        assert ep.launch(hx[ab].array, thr, hl[ab].array, hp[ab].array, FDAS.AllAccelerations, ab), ep.last_error
        if i > 0:
            assert ep.wait(1 - ab), ep.last_error
    assert ep.wait((e2e_steps - 1) & 1)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_s = reduce_max(e2e_s, f"cuda:{local}")
    e2e = whole_job_rate(e2e_steps, e2e_s, ws)

    if rank != 0:
        return
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        from concurrent.futures import ThreadPoolExecutor
        workers = os.cpu_count() or 1
        with ThreadPoolExecutor(workers) as ex:
            t_cpu, n_cpu = cpu_search(x, bank, thr, ex, workers)
        cpu = {"value": 1.0 / t_cpu, "unit": UNIT, "cores": workers, "kind": "port",
               "sample": "one " + CPU_SAMPLE.format(w=workers, c=n_cpu)}
    # tiling, FT convolution, harmonic summing, FP64 recheck, 3 selection kernels
    launches_per_search = 7
    forms = None
    if ws == 1 and not args.no_forms:
        # the three forms of the search beside the plain path, short runs of
        # their own workloads (each reports the plain path it is compared with)
        p.close()
        q.close()
        forms = {"batched": batched_form(256, steps=3, warmup=3),
                 "served": [served_form(rate, 400, 8) for rate in (400.0, 2000.0)],
                 "precision": precision_form(N_BINS, steps=20, warmup=3)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "mode": mode, **mode_values,
        "dtype": "f32", "data": "synthetic", "config": dict(WORKLOAD, parallelism=f"replicas{ws}"),
        "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                       "note": "sequential searches one at a time, no load; under load: forms.served"},
        "stage_ms": stage_ms, "candidates": int(n_cand), "candidates_dropped": int(dropped),
        "recheck_cells": counters["recheck"], "device_status": counters["status"],
        "selected_per_plane": counters["selected"],
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg[dom], "traffic": traffic},
        # the FT convolution is bound by the FP32 pipe, not by HBM: its algorithmic
        # flops (per (tile, template): complex multiply 6 x 2048, inverse FFT
        # 5 x 2048 x 11, power 3 x 2048) against the FP32 FMA peak of the GPU
        # (SMs x 128 lanes x 2 flops x the sampled SM clock)
        "ft_convolution_fp32": fp32_pipe(stage_ms["ft_convolution"], n_bins, clk),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * n_bins,
                "d2h_bytes_per_step": 8 * n_list},
        "gpu_launches": launches_per_search * args.steps,
        "clocks": clk,
        "cpu_baseline": cpu,
        "forms": forms,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ served form
def served_spectrum(n, seed):
    """Seeded unit-power Gaussian trial of 2n samples with 0-2 accelerated
    signals (random z in [-42, 42], 1-8 harmonics)."""
    from fdas_gb300 import synth
    rng = np.random.default_rng(seed)
    amp = 0.05 * np.sqrt((1 << 15) / n)
    sig = [dict(r0=float(rng.uniform(0.05, 0.45) * n), z=float(rng.uniform(-42, 42)),
                n_harm=int(rng.integers(1, 9)), amp=amp) for _ in range(int(rng.integers(0, 3)))]
    return synth.spectrum(synth.timeseries(2 * n, sig, seed=seed), n)[0]


def served_form(rate, n_req, slots):
    """Open request loop: Poisson arrivals at ``rate`` searches/s; each request is
    a trial of 2^16..2^22 samples (2^15..2^21 bins), the 85-template bank or
    its z = -21..+21 half, 4, 8 or 16 planes, chi-square FAR 1e-6 thresholds.
    The request server (continuous batching, slots admitted by FOP bytes
    against free HBM) against the plain path per request (one search at a time
    through fdas_launch / fdas_wait, first come first served)."""
    import torch
    from scipy.stats import gamma
    from fdas_gb300.fdas import FDAS
    from fdas_gb300.server import Server, HALF_BANK
    from fdas_gb300.templates import template_bank
    torch.cuda.set_device(0)
    bank = template_bank()
    rng = np.random.default_rng(2025)
    sizes = [1 << k for k in range(15, 22)]
    args = argparse.Namespace(rate=rate, requests=n_req, slots=slots)
    pool = {n: [served_spectrum(n, 100 * k + i) for i in range(2)] for k, n in enumerate(sizes)}
    thr = {P: np.array([gamma.isf(1e-6, k) for k in range(1, P + 1)], dtype=np.float32) for P in (4, 8, 16)}
    n_req = args.requests
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, n_req))
    reqs = [(sizes[int(rng.integers(0, len(sizes)))], bool(rng.integers(0, 2)), int(rng.choice([4, 8, 16])),
             int(rng.integers(0, 2))) for _ in range(n_req)]

    def rows_of(half):
        return HALF_BANK if half else (0, 85)

    def stats(lat, wall):
        lat = np.asarray(lat)
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "mean_ms": float(lat.mean()), "searches_per_s": n_req / wall}

    # ---- served
    with Server(bank, max_bins=1 << 21, max_slots=args.slots) as srv:
        for n in sizes:  # warm-up: one request per length class creates the slots
            for half in (False, True):
                srv.result(srv.submit(pool[n][0], thr[8], rows_of(half)))
        ids, t_sub = [], []
        t0 = time.perf_counter()
        for (n, half, P, k), ta in zip(reqs, arrivals):
            dt = t0 + ta - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            t_sub.append(time.perf_counter())
            ids.append(srv.submit(pool[n][k], thr[P], rows_of(half)))
        lat_srv = [srv.result(rid)[3] for rid in ids]
        # the server measures from the entry of submit (the spectrum's copy
        # included); like the plain path below, each request's latency counts
        # from its scheduled arrival, so a submitting loop that falls behind
        # the arrivals is charged too
        lag = [(ts - (t0 + ta)) * 1e3 for ts, ta in zip(t_sub, arrivals)]
        lat = [g + l for g, l in zip(lag, lat_srv)]
        wall = max(t0 + ta + l * 1e-3 for ta, l in zip(arrivals, lat)) - t0
        served = stats(lat, wall)
        served["server_p50_ms"] = float(np.percentile(lat_srv, 50))
        served["submit_lag_p99_ms"] = float(np.percentile(lag, 99))
        served["peak_in_flight"] = srv.stats()["peak_in_flight"]

    # ---- plain path per request: one handle per length class, searches one at a time
    log = open(os.devnull, "w")
    handles = {}
    for n in sizes:
        h = FDAS(log)
        assert h.initialise_accelerator(n, n_planes=16), h.last_error
        assert h.upload_templates(bank, FDAS.A), h.last_error
        handles[n] = h
    loc = np.zeros(16 * 512, np.uint32)
    pwr = np.zeros(16 * 512, np.float32)

    def plain_one(n, half, P, k):
        h = handles[n]
        r0, nt = rows_of(half)
        assert h.reshape(n, r0, nt, 0, P), h.last_error
        assert h.launch(pool[n][k], thr[P], loc, pwr, FDAS.AllAccelerations, FDAS.A), h.last_error
        assert h.wait(FDAS.A), h.last_error
        h.retrieve_candidate_list(FDAS.A)

    for n in sizes:
        plain_one(n, False, 8, 0)
    lat = []
    t0 = time.perf_counter()
    for (n, half, P, k), ta in zip(reqs, arrivals):
        dt = t0 + ta - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        plain_one(n, half, P, k)
        lat.append((time.perf_counter() - (t0 + ta)) * 1e3)
    plain = stats(lat, time.perf_counter() - t0)
    for h in handles.values():
        h.close()
    return {"form": "served", "metric": "served searches: p50/p99 latency (submit to candidate list) and searches/s",
            "unit": "ms", "rate_per_s": args.rate, "requests": n_req, "slots": args.slots,
            "mix": "2^15..2^21 bins (uniform in log2), full 85 or half 43 template bank, 4/8/16 planes, "
                   "0-2 signals, chi-square FAR 1e-6", "served": served, "plain_per_request": plain,
            "data": "synthetic"}


# ------------------------------------------------------------------ batched form
def batched_form(n_tr=256, steps=5, warmup=3, autotune=True, profile_one=False):
    """256 dedispersed trials of uneven length (log-uniform 2^18..2^22 samples,
    i.e. 2^17..2^21 bins), 0-2 accelerated signals each (z in [-42, 42], 1-8
    harmonics), 85-template bank, 8 planes, chi-square FAR 1e-6: one batched
    pass (persistent FT-convolution launches over all trials' items, CUDA
    graph, autotuned) against the plain path searching the same trials one by
    one and on two alternating handles.  ``profile_one``: after the timed
    replays, one more replay between cudaProfilerStart and cudaProfilerStop,
    for ``ncu --profile-from-start off``."""
    import torch
    from scipy.stats import gamma
    from fdas_gb300.batch import Batch
    from fdas_gb300.fdas import FDAS
    from fdas_gb300.templates import template_bank
    torch.cuda.set_device(0)
    bank = template_bank()
    from fdas_gb300 import synth
    args = argparse.Namespace(steps=steps, warmup=warmup, no_autotune=not autotune)
    thr = np.array([gamma.isf(1e-6, k) for k in range(1, 9)], dtype=np.float32)
    n_bins, offs, d_all = synth.batch_mix(n_tr)  # synthetic spectra made on the GPU (not timed)
    torch.cuda.synchronize()
    total_bins = int(n_bins.sum())

    # ---- batched
    b = Batch(bank, n_bins, autotune=not args.no_autotune)
    b.set_inputs_device(d_all.data_ptr())
    t = time.perf_counter()
    b.run(thr)  # autotune + capture + first replay
    t_setup = time.perf_counter() - t
    for _ in range(args.warmup):
        b.run(thr)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        b.run(thr)
        times.append(time.perf_counter() - t)
    batched_s = float(np.median(times))
    if profile_one:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        b.run(thr)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    info = b.info()
    n_cand = sum(b.trial(i).retrieve_candidate_list(FDAS.A, capacity=0)[1] for i in range(n_tr))
    b.close()

    # ---- plain path: the same trials one at a time on one handle (reshaped per trial)
    log = open(os.devnull, "w")
    h = FDAS(log)
    assert h.initialise_accelerator(int(n_bins.max())), h.last_error
    assert h.upload_templates(bank, FDAS.A), h.last_error

    def plain_pass():
        for i in range(n_tr):
            assert h.reshape(int(n_bins[i])), h.last_error
            assert h.enqueue_search_device(d_all.data_ptr() + 8 * int(offs[i]), thr, FDAS.AllAccelerations,
                                           FDAS.A), h.last_error
        assert h.synchronize(FDAS.A)

    plain_pass()
    pt = []
    for _ in range(max(1, args.steps // 2)):
        t = time.perf_counter()
        plain_pass()
        pt.append(time.perf_counter() - t)
    plain_s = float(np.median(pt))

    # the plain path with two handles on their own streams, trials alternating
    # between them (the next trial's kernels start where the previous ones end)
    h2 = FDAS(log)
    assert h2.initialise_accelerator(int(n_bins.max())), h2.last_error
    assert h2.upload_templates(bank, FDAS.A), h2.last_error
    hs = (h, h2)

    def plain_alt_pass():
        for i in range(n_tr):
            hh = hs[i & 1]
            assert hh.reshape(int(n_bins[i])), hh.last_error
            assert hh.enqueue_search_device(d_all.data_ptr() + 8 * int(offs[i]), thr, FDAS.AllAccelerations,
                                            FDAS.A), hh.last_error
        for hh in hs:
            assert hh.synchronize(FDAS.A)

    plain_alt_pass()
    pa = []
    for _ in range(max(1, args.steps // 2)):
        t = time.perf_counter()
        plain_alt_pass()
        pa.append(time.perf_counter() - t)
    plain_alt_s = float(np.median(pa))
    h.close()
    h2.close()
    return {"form": "batched", "metric": "batched searches/s (trials of uneven length)", "unit": "searches/s",
            "value": n_tr / batched_s, "ms_per_batch": batched_s * 1e3, "trials": n_tr, "total_bins": total_bins,
            "fop_gb": 4 * 85 * total_bins / 1e9, "plain_value": n_tr / plain_s, "plain_ms_per_batch": plain_s * 1e3,
            "speedup_vs_plain": plain_s / batched_s, "plain_alternating_ms_per_batch": plain_alt_s * 1e3,
            "speedup_vs_plain_alternating": plain_alt_s / batched_s, "autotune": info, "setup_s": t_setup,
            "candidates": int(n_cand), "steps": args.steps, "warmup": args.warmup,
            "timing": "host clock around graph replays (each ~100 ms), median", "data": "synthetic (seeded, on GPU)"}


# ------------------------------------------------------------------ precision form
def precision_form(bins=N_BINS, steps=50, warmup=3, noise_only=False):
    """The 2^21-bin search with the forward DFT of the tiles and the inverse
    DFT of the FT convolution on the tensor cores (split BF16 / split FP16
    operands, tcgen05) beside the FP32 FFT path: searches/s, FT-convolution stage time and whether the candidate set
    equals the FP32 path's (errors against FP64 are measured by the tests)."""
    import torch
    from fdas_gb300.fdas import FDAS
    torch.cuda.set_device(0)
    args = argparse.Namespace(bins=bins, steps=steps, warmup=warmup)
    x, bank, thr = make_inputs(bins, noise_only)
    d_x = torch.from_numpy(x.view(np.float32)).cuda()
    log = open(os.devnull, "w")
    out = {}
    ref_keys = None
    for prec, name in ((0, "fp32_fft"), (1, "split_bf16_tcgen05"), (2, "split_fp16_tcgen05")):
        h = FDAS(log)
        assert h.initialise_accelerator(args.bins, precision=prec), h.last_error
        assert h.upload_templates(bank, FDAS.A), h.last_error
        for _ in range(args.warmup):
            assert h.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, FDAS.A), h.last_error
        assert h.synchronize(FDAS.A)
        s = torch.cuda.ExternalStream(h.stream(FDAS.A))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(args.steps):
            h.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, FDAS.A)
        e1.record(s)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        stages = []
        for _ in range(5):
            h.enqueue_search_device(d_x.data_ptr(), thr, FDAS.AllAccelerations, FDAS.A)
            h.synchronize(FDAS.A)
            stages.append(h.stage_times(FDAS.A))
        st = np.mean(np.array(stages), axis=0)
        rec, n_total, dropped = h.retrieve_candidate_list(FDAS.A)
        keys = set(zip(rec["harmonic"].tolist(), rec["template_num"].tolist(), rec["bin"].tolist()))
        if ref_keys is None:
            ref_keys = keys
        out[name] = {"searches_per_s": 1e3 / ms, "ms_per_search": ms, "ft_convolution_ms": float(st[2]),
                     "candidates": n_total, "same_candidates_as_fp32": keys == ref_keys}
        if prec:  # tensor-core rate of the FT convolution stage against the dense BF16 peak
            items = -(-args.bins // 1628) * N_TEMPLATES
            flops = TC_FLOPS_PER_ITEM * items
            peak, src = measured_bf16_peak()
            achieved = flops / (float(st[2]) * 1e-3) / 1e12
            out[name]["tensor"] = {"flops_per_search": flops, "achieved_tflops": achieved, "peak_tflops": peak,
                                   "frac": achieved / peak, "peak_source": src}
        h.close()
    return {"form": "precision", "metric": "searches/s at 2^21 bins x 85 tmpl x 8 harm by DFT precision",
            "unit": "searches/s", "n_bins": args.bins, "steps": args.steps, "warmup": args.warmup,
            "results": out, "data": "synthetic", "timing": "CUDA events on the library stream, sequential searches"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps; default 1500 searches for the GPU arm (a timed region above a "
                         "second, so the clock sampler sees it several times), 5 for the reference arm "
                         "and the batched form, 50 for the precision form")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--stage-times", action="store_true", help="per-step stage events inside the timed loop")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="device-resident leg only (profiling runs)")
    ap.add_argument("--no-forms", action="store_true",
                    help="leave out the short batched / served / precision runs of the default line")
    ap.add_argument("--noise-only", action="store_true",
                    help="Gaussian noise without the injected signals (profiling the no-candidate path)")
    ap.add_argument("--bins", type=int, default=N_BINS,
                    help="spectrum bins; the reported workload is 2^21, smaller values are for ncu captures")
    ap.add_argument("--trials", type=int, default=256, help="batched form: number of trials")
    ap.add_argument("--no-autotune", action="store_true", help="batched form: default tuning")
    ap.add_argument("--profile-one", action="store_true",
                    help="batched form: one extra replay inside cudaProfilerStart/Stop (ncu --profile-from-start off)")
    ap.add_argument("--form", default="plain", choices=["plain", "served", "batched", "precision"],
                    help="served: the request server under Poisson arrivals (prints its own JSON line)")
    ap.add_argument("--rate", type=float, default=200.0, help="served form: arrival rate (searches/s)")
    ap.add_argument("--requests", type=int, default=400, help="served form: number of requests")
    ap.add_argument("--slots", type=int, default=8, help="served form: searches in flight at most")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 5 if (args.impl == "reference" or args.form == "batched") else \
            50 if args.form == "precision" else 1500
    if args.warmup < 3:
        args.warmup = 3
    if args.form == "served":
        print(json.dumps(served_form(args.rate, args.requests, args.slots)), flush=True)
        return
    if args.form == "batched":
        print(json.dumps(batched_form(args.trials, args.steps, args.warmup, not args.no_autotune,
                                      args.profile_one)), flush=True)
        return
    if args.form == "precision":
        print(json.dumps(precision_form(args.bins, args.steps, args.warmup, args.noise_only)), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
