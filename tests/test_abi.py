"""CPU-side checks of the C ABI: the library builds, loads and exports every
symbol declared in include/fdas_gb300.h (no compute calls without a GPU)."""
import ctypes
import re

import pytest

from conftest import ROOT


def declared_symbols():
    text = (ROOT / "include" / "fdas_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(fdas_[a-z_0-9]+)\s*\(", text)) - {"fdas_log_fn"})


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__.build()
    from fdas_gb300 import _lib
    return _lib.load()


def test_header_symbols_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s


def test_python_binding_covers_header(lib):
    from fdas_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_no_device_is_reported_not_crashed(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fdas_gb300 import _lib
    cfg = _lib.FdasConfig()
    lib.fdas_default_config(ctypes.byref(cfg), 4096)
    assert cfg.n_templates == 85 and cfg.n_planes == 8 and cfg.max_template_len == 421
    h = ctypes.c_void_p()
    st = lib.fdas_initialise_accelerator(ctypes.byref(cfg), ctypes.byref(h))
    assert st in (_lib.ERR_NO_DEVICE, _lib.ERR_CUDA)
    assert not h.value
    assert lib.fdas_last_error(None)
    # null handles are rejected, not dereferenced
    assert lib.fdas_wait(None, 0) == _lib.ERR_INVALID_ARG
    assert lib.fdas_get_input_sz(None) == 0


def test_invalid_config_rejected_before_device(lib):
    from fdas_gb300 import _lib
    cfg = _lib.FdasConfig()
    lib.fdas_default_config(ctypes.byref(cfg), 4096)
    cfg.n_templates = 84
    h = ctypes.c_void_p()
    assert lib.fdas_initialise_accelerator(ctypes.byref(cfg), ctypes.byref(h)) == _lib.ERR_INVALID_ARG
    lib.fdas_default_config(ctypes.byref(cfg), 4096)
    cfg.tile_overlap = 100
    assert lib.fdas_initialise_accelerator(ctypes.byref(cfg), ctypes.byref(h)) == _lib.ERR_INVALID_ARG
