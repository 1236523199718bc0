#!/usr/bin/env python3
"""Benchmark: FDAS searches/s at 2^21 bins x 85 templates x 8 harmonics on GB300.

One step = one full search of one spectrum: overlap-save tiling + forward FFT,
FT convolution of all 85 templates into the filter-output plane (FOP), 8-plane
harmonic summing with chi-square thresholds (FAR 1e-6), FP64 recheck and the
sorted candidate list.

* ``value``: searches/s with the spectrum already resident in HBM
  (fdas_enqueue_search_device), timed with CUDA events on the library's stream.
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


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
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
                                          "--format=csv,noheader,nounits", "-lms", "200"],
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


# ------------------------------------------------------------------ CPU side
def cpu_fop_rows(args):
    """FOP rows by direct convolution (ft_conv.py:199-205 semantics)."""
    from oracle import fdas_oracle as O
    x, bank, rows, dtype = args
    return O.fop(x, bank, dtype=dtype, rows=rows)


def cpu_search_time(x, bank, thr, n_rows_sample, bin_frac, dtype, pool=None, workers=1):
    """Extrapolated time of one CPU search from a bounded sample.

    FOP: ``n_rows_sample`` of the 85 rows by direct linear convolution (scaled
    by 85 / n_rows_sample).  Harmonic summing: the vectorised restatement of
    hsum.py over the first ``bin_frac`` of the bins for all rows (scaled by
    1 / bin_frac).  Returns (seconds per search, description).
    """
    from oracle import fdas_oracle as O
    rows = np.linspace(0, N_TEMPLATES - 1, n_rows_sample).astype(int)
    t0 = time.perf_counter()
    if pool is not None:
        chunks = np.array_split(rows, workers)
        pool.map(cpu_fop_rows, [(x, bank, list(c), dtype) for c in chunks if len(c)])
    else:
        O.fop(x, bank, dtype=dtype, rows=rows)
    t_fop = (time.perf_counter() - t0) * N_TEMPLATES / n_rows_sample
    nb = int(x.size * bin_frac)
    rng = np.random.default_rng(0)
    plane = rng.exponential(size=(N_TEMPLATES, nb)).astype(dtype)
    t0 = time.perf_counter()
    O.detections_streaming(plane, thr, N_PLANES, dtype=dtype)
    t_hs = (time.perf_counter() - t0) / bin_frac
    desc = (f"FOP of {n_rows_sample}/85 rows at 2^21 bins (x{N_TEMPLATES / n_rows_sample:.1f}) + vectorised "
            f"harmonic summing over {nb} of 2^21 bins, 85 rows, 8 planes (x{1 / bin_frac:.0f}); "
            f"{np.dtype(dtype).name}")
    return t_fop + t_hs, desc


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
    x, bank, thr = make_inputs()
    workers = os.cpu_count() or 1
    times = []
    desc = ""
    import multiprocessing as mp
    # one row per worker and 1/64 of the bins per step keeps a step near half
    # a second on 16 cores, so --steps K --warmup W ends within minutes
    with mp.get_context("spawn").Pool(workers) as pool:
        for i in range(args.warmup + args.steps):
            t, desc = cpu_search_time(x, bank, thr, n_rows_sample=min(N_TEMPLATES, workers), bin_frac=1 / 64,
                                      dtype=np.float32, pool=pool, workers=workers)
            if i >= args.warmup:
                times.append(t)
    v = 1.0 / float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": WORKLOAD,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
                             "sample": "per step: " + desc + " (the reference's ft_conv.py + hsum.py path, "
                                       "restated in NumPy/SciPy at its own float32/complex64 precision)"},
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
        if ws > 1:
            import torch.distributed as dist
            t = torch.tensor([v], device=f"cuda:{local}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return v

    d_x = torch.from_numpy(x.view(np.float32)).to(f"cuda:{local}")
    # sequential form: one buffer set, one stream; gives the per-search latency
    p = make_handle(False)
    seq_ms, per = timed_device_loop(p, [FDAS.A], args.steps)
    seq_ms = max_over_ranks(seq_ms)
    counters = p.counters(FDAS.A)
    n_cand = sum(counters["per_plane"])
    dropped = max(0, n_cand - counters["records"])
    # pipelined form: searches alternate between buffer sets A and B on their
    # own streams; the kernels are sized so that the FT convolution of one
    # search and the harmonic summing of the previous share every SM
    q = make_handle(True)
    with ClockSampler(local) as clocks:
        pipe_ms, _ = timed_device_loop(q, [FDAS.A, FDAS.B], args.steps)
    pipe_ms = max_over_ranks(pipe_ms)
    total_ms = min(seq_ms, pipe_ms)
    value = ws * args.steps / (total_ms / 1e3)
    mode = "pipelined" if pipe_ms <= seq_ms else "sequential"

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
                              "value_sequential": ws * args.steps / (seq_ms / 1e3),
                              "value_pipelined": ws * args.steps / (pipe_ms / 1e3),
                              "stage_ms": stage_ms, "counters": counters, "profile_run": True}), flush=True)
        return
    hx = {ab: PinnedArray((n_bins,), np.complex64) for ab in (FDAS.A, FDAS.B)}
    for ab in hx:
        hx[ab].array[:] = x
    n_list = p.get_candidate_list_sz()
    hl = {ab: PinnedArray((n_list,), np.uint32) for ab in (FDAS.A, FDAS.B)}
    hp = {ab: PinnedArray((n_list,), np.float32) for ab in (FDAS.A, FDAS.B)}
    e2e_steps = args.steps
    ep = q if mode == "pipelined" else p  # the faster configuration
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
    if ws > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = ws * e2e_steps / e2e_s

    if rank != 0:
        return
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        t_cpu, desc = cpu_search_time(x, bank, thr, n_rows_sample=4, bin_frac=1 / 32, dtype=np.float32)
        cpu = {"value": 1.0 / t_cpu, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "one search extrapolated from: " + desc}
    # tiling, FT convolution, harmonic summing, FP64 recheck, 3 selection kernels
    launches_per_search = 7
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "mode": mode, "value_sequential": ws * args.steps / (seq_ms / 1e3),
        "value_pipelined": ws * args.steps / (pipe_ms / 1e3),
        "dtype": "f32", "data": "synthetic", "config": dict(WORKLOAD, parallelism=f"replicas{ws}"),
        "latency_ms": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99))},
        "stage_ms": stage_ms, "candidates": int(n_cand), "candidates_dropped": int(dropped),
        "recheck_cells": counters["recheck"], "device_status": counters["status"],
        "selected_per_plane": counters["selected"],
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg[dom], "traffic": traffic},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8 * n_bins,
                "d2h_bytes_per_step": 8 * n_list},
        "gpu_launches": launches_per_search * args.steps,
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--stage-times", action="store_true", help="per-step stage events inside the timed loop")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="device-resident leg only (profiling runs)")
    ap.add_argument("--noise-only", action="store_true",
                    help="Gaussian noise without the injected signals (profiling the no-candidate path)")
    ap.add_argument("--bins", type=int, default=N_BINS,
                    help="spectrum bins; the reported workload is 2^21, smaller values are for ncu captures")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
