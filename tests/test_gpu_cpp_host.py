"""The C++ host class (include/FDAS.hpp) driven like the reference's gtest."""
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from fdas_gb300 import build
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu


def test_cpp_driver_gtest_sequence(tmp_path):
    drv = build.build_driver()
    assert drv is not None and drv.exists()
    g = load_golden("n4096")
    bank_p4 = O.to_p4(np.fft.fft(template_bank().astype(np.complex128), 2048, axis=1)).astype(np.complex64)
    g["input"].astype(np.complex64).tofile(tmp_path / "input.bin")
    bank_p4.tofile(tmp_path / "templates_p4.bin")
    g["thresholds"].astype(np.float32).tofile(tmp_path / "thresholds.bin")
    g["tiles_p4_ref"].astype(np.complex64).tofile(tmp_path / "tiles_ref.bin")
    g["fop_ref"].astype(np.float32).tofile(tmp_path / "fop_ref.bin")
    g["det_loc_ref"].astype(np.uint32).tofile(tmp_path / "det_loc_ref.bin")
    g["det_pwr_ref"].astype(np.float32).tofile(tmp_path / "det_pwr_ref.bin")
    r = subprocess.run([str(drv), str(tmp_path), "4"], capture_output=True, text=True, timeout=600)
    print(r.stdout[-3000:])
    print(r.stderr[-3000:])
    assert r.returncode == 0
    assert "PASSED" in r.stdout
    for name in ["FT_Convolution", "Harmonic_Summing", "FDAS_steps", "FDAS_serial", "FDAS_pipelined"]:
        assert f"[ OK ] {name}" in r.stdout
