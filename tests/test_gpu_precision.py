"""Precision form (fdas_config.precision): the forward DFT of the tiles and
the inverse DFT of the FT convolution as DFT-64 x DFT-32 factor products on
the tensor cores (tcgen05) with split (hi + lo) BF16 or FP16 operands, against
the FP64 oracle.

Per stage against FP64: the tiles (forward DFT) and the FOP (inverse DFT +
power).  Split FP16 (22 significant bits) meets the tile and FOP tolerances of
the FP32 path at these sizes; split BF16 (16 bits) is held to measured wider
bounds (tiles 3e-5 of the rms, FOP ten times the FP32 path's).  With the FP64
recheck both forms give the FP64 oracle's candidate set."""
import io

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import make_pipeline, candidates_as_arrays
from test_gpu_parity import fop_within, FOP_REL_TOL
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

NAMES = {0: "fp32 fft", 1: "split bf16 tcgen05", 2: "split fp16 tcgen05"}


def run(x, bank, precision, thr=None):
    p = make_pipeline(x.size, log=io.StringIO(), precision=precision)
    assert p.upload_templates(bank, FDAS.A), p.last_error
    assert p.perform_input_tiling(x, FDAS.A), p.last_error
    assert p.perform_ft_convolution(FDAS.AllAccelerations, FDAS.A), p.last_error
    tiles = np.zeros(p.get_tiles_sz(), np.complex64)
    assert p.retrieve_tiles(tiles, FDAS.A)
    fop = np.zeros(p.get_fop_sz(), np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    rec = None
    if thr is not None:
        assert p.perform_harmonic_summing(thr, FDAS.AllAccelerations, FDAS.A), p.last_error
        rec, _, dropped = p.retrieve_candidate_list(FDAS.A)
        assert dropped == 0
    return tiles.reshape(-1, 2048), fop.reshape(85, x.size), rec


def stage_errors(x, bank64, tiles, fop):
    t_ref = O.to_p4(O.tiles(x))
    t_rms = np.sqrt(np.mean(np.abs(t_ref) ** 2))
    ref = O.fop(x, bank64)
    mean = ref.mean(axis=1, keepdims=True)
    d = np.abs(fop - ref) / mean
    cell = (np.abs(fop - ref) / (mean + np.abs(ref))).max()
    print(f"    per cell: max |d| / (plane mean + |FOP|) {cell:.2e}")
    return np.abs(tiles - t_ref).max() / t_rms, d.max(), np.sqrt(np.mean(d ** 2)), ref


@pytest.mark.parametrize("name", ["n4096", "n32768"])
def test_precision_fop_per_stage(name):
    g = load_golden(name)
    bank64 = template_bank()
    x = g["input"]
    for precision in (0, 1, 2):
        tiles, fop, _ = run(x, bank64, precision)
        t_err, f_max, f_rms, ref = stage_errors(x, bank64, tiles, fop)
        print(f"{name} {NAMES[precision]}: tiles max |d| / rms {t_err:.2e}; "
              f"FOP |d| / plane mean: max {f_max:.2e}, rms {f_rms:.2e}")
        assert t_err < (3e-5 if precision == 1 else 1e-5)  # split BF16 forward DFT: 1.8e-5 measured
        if precision in (0, 2):
            assert fop_within(fop, ref, x, bank64).all()
        else:  # split BF16: ten times the FP32 path's bound (1e-4 of the plane mean + 1e-4 of the cell)
            mean = ref.mean(axis=1, keepdims=True)
            assert (np.abs(fop - ref) <= 10 * FOP_REL_TOL * mean + 1e-4 * np.abs(ref)).all()


@pytest.mark.parametrize("n", [1629, 3001])
def test_precision_ragged(n):
    rng = np.random.default_rng(n)
    x = ((rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)).astype(np.complex64)
    bank64 = template_bank()
    _, fop, _ = run(x, bank64, 2)
    assert fop_within(fop, O.fop(x, bank64), x, bank64).all()


@pytest.mark.parametrize("precision", [1, 2])
def test_precision_candidates_equal_fp64(precision):
    g = load_golden("n32768")
    bank64 = template_bank()
    x = g["input"]
    thr = g["thresholds_chi2"]
    _, _, rec = run(x, bank64, precision, thr)
    _, _, rec0 = run(x, bank64, 0, thr)
    key = lambda r: list(zip(r["harmonic"].tolist(), r["template_num"].tolist(), r["bin"].tolist()))
    assert len(rec) > 0 and key(rec) == key(rec0)
    loc, pwr = O.detections(O.harmonic_planes(O.fop(x, bank64), dtype=np.float64), thr)[:2]
    got, _ = candidates_as_arrays(rec)
    assert np.array_equal(got, loc)  # the same set of (plane, template, bin) as the FP64 oracle


def test_precision_rejected_value():
    from fdas_gb300 import _lib
    import ctypes
    lib = _lib.load()
    cfg = _lib.FdasConfig()
    lib.fdas_default_config(ctypes.byref(cfg), 4096)
    cfg.precision = 3
    h = ctypes.c_void_p()
    assert lib.fdas_initialise_accelerator(ctypes.byref(cfg), ctypes.byref(h)) == _lib.ERR_INVALID_ARG
