#!/usr/bin/env python3
"""Generate the golden fixtures in this directory from the reference's own scripts.

Runs the UNMODIFIED reference CPU path -- ``fdas/test/ft_conv.py`` and
``fdas/test/hsum.py`` of UOA-PARC-SKA/FDAS, read from a local checkout given by
``--reference`` -- on seeded synthetic headerless ``.tim`` files (the PSS
test-vector generator the reference uses is not available), with the shipped
template bank ``fdas/tmpl/fdas_templates_85_350.npy``.  Its outputs are stored
here as small ``.npz`` fixtures so that tests can pin the oracle restatement
without the reference being present.

Usage:  python tests/golden/make_golden.py --reference /path/to/FDAS
"""

import argparse
import json
import os
import pathlib
import subprocess
import sys
import tempfile

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from fdas_gb300 import synth  # noqa: E402

# name -> (n_freq, seed, signals, rows of the FOP to keep (None = all), tiles to keep (None = all))
CASES = {
    "n1000": dict(n_freq=1000, seed=11, n_signals=1, fop_rows=None, tiles=None),
    "n4096": dict(n_freq=4096, seed=5, n_signals=2, fop_rows=None, tiles=None),
    "n32768": dict(n_freq=32768, seed=42, n_signals=None, fop_rows=[0, 1, 21, 41, 42, 43, 63, 84],
                   tiles=[0, 1, 10, 20]),
}


def run(cmd, cwd):
    print("+", " ".join(map(str, cmd)), flush=True)
    subprocess.run(list(map(str, cmd)), cwd=cwd, check=True, stdout=subprocess.DEVNULL)


def make_case(name, spec, ref, out_dir, tmp):
    n_freq = spec["n_freq"]
    if spec["n_signals"] is None:
        samples, sig = synth.emulator_case(seed=spec["seed"])
    else:
        samples, sig = synth.small_case(n_freq, seed=spec["seed"], n_signals=spec["n_signals"])
    tim = tmp / f"{name}.tim"
    samples.astype(np.float32).tofile(tim)
    bank = ref / "fdas/tmpl/fdas_templates_85_350.npy"
    test_dir = ref / "fdas/test"
    run([sys.executable, test_dir / "ft_conv.py", "-H", "-t", bank, "-f", n_freq,
         "--tile-and-transform", "--fft-order", "-B", tmp, tim], cwd=tmp)
    od = tmp / name
    # mock-up thresholds (hsum.py default: ~64 candidates per plane)
    run([sys.executable, test_dir / "hsum.py", od / "fop_ref.npy"], cwd=tmp)
    fix = dict(
        samples=samples.astype(np.float32),
        input=np.load(od / "input.npy"),
        thresholds=np.load(od / "thresholds.npy"),
        det_loc_ref=np.load(od / "det_loc_ref.npy"),
        det_pwr_ref=np.load(od / "det_pwr_ref.npy"),
    )
    fop_ref = np.load(od / "fop_ref.npy")
    tiles_ref = np.load(od / "input_tiled_p4_ref.npy")
    rows = spec["fop_rows"]
    tiles = spec["tiles"]
    fix["fop_rows"] = np.arange(fop_ref.shape[0]) if rows is None else np.array(rows)
    fix["fop_ref"] = fop_ref[fix["fop_rows"]]
    fix["fop_row_sum"] = fop_ref.astype(np.float64).sum(axis=1)
    fix["fop_row_max"] = fop_ref.max(axis=1)
    fix["tile_idx"] = np.arange(tiles_ref.shape[0]) if tiles is None else np.array(tiles)
    fix["tiles_p4_ref"] = tiles_ref[fix["tile_idx"]]
    fix["n_tiles"] = np.array(tiles_ref.shape[0])
    # second harmonic-summing run with user thresholds (hsum.py --thresholds): the
    # chi-square FAR 1e-6 thresholds scaled to this spectrum's mean power
    mean_pwr = float(np.mean(np.abs(fix["input"].astype(np.complex128)) ** 2))
    from scipy.stats import gamma
    thr2 = np.array([gamma.isf(1e-6, k) * mean_pwr for k in range(1, 9)], dtype=np.float32)
    thr_file = tmp / f"{name}_thr.npy"
    np.save(thr_file, thr2)
    od2 = tmp / "chi2"
    run([sys.executable, test_dir / "hsum.py", "-B", od2, "--thresholds", f"@{thr_file}",
         od / "fop_ref.npy"], cwd=tmp)
    fix["thresholds_chi2"] = np.load(od2 / name / "thresholds.npy")
    fix["det_loc_ref_chi2"] = np.load(od2 / name / "det_loc_ref.npy")
    fix["det_pwr_ref_chi2"] = np.load(od2 / name / "det_pwr_ref.npy")
    np.savez_compressed(out_dir / f"{name}.npz", **fix)
    meta = dict(name=name, n_freq=n_freq, n_samp=2 * n_freq, seed=spec["seed"], signals=sig,
                normalisation="ft_conv.py: fft(samples)/n_samp, first n_freq bins",
                template_bank="fdas/tmpl/fdas_templates_85_350.npy (85 x 421 complex64)",
                tile_sz=2048, tile_overlap=420, n_planes=8,
                thresholds="hsum.py mock-up quantiles (64/plane); *_chi2: gamma.isf(1e-6,k)*mean power")
    (out_dir / f"{name}.json").write_text(json.dumps(meta, indent=1) + "\n")
    print(f"{name}: {len(fix['det_loc_ref'])} mock-threshold and {len(fix['det_loc_ref_chi2'])} "
          f"chi2 candidates")


def make_bank_fixture(ref, out_dir):
    """Checksums and a few rows of the shipped template banks."""
    bank = np.load(ref / "fdas/tmpl/fdas_templates_85_350.npy")
    ft = np.load(ref / "fdas/tmpl/fdas_templates_85_350_ft_p4.npy")
    rows = np.array([0, 20, 41, 42, 43, 64, 84])
    np.savez_compressed(out_dir / "template_bank.npz", rows=rows, bank_rows=bank[rows],
                        ft_p4_rows=ft[rows], bank_shape=np.array(bank.shape),
                        ft_shape=np.array(ft.shape),
                        bank_row_energy=np.sum(np.abs(bank.astype(np.complex128)) ** 2, axis=1),
                        bank_nnz=np.count_nonzero(bank, axis=1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, type=pathlib.Path)
    ap.add_argument("--cases", nargs="*", default=list(CASES))
    args = ap.parse_args()
    ref = args.reference.resolve()
    with tempfile.TemporaryDirectory() as td:
        tmp = pathlib.Path(td)
        for name in args.cases:
            make_case(name, CASES[name], ref, HERE, tmp)
    make_bank_fixture(ref, HERE)


if __name__ == "__main__":
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    main()
