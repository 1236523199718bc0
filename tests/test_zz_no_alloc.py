"""fdas_ft_convolution_noalloc: the FT convolution that allocates nothing,
against the handle path (fdas_perform_input_tiling + fdas_perform_ft_convolution)
on the same inputs.

Both run the same kernels on the same scaled template spectra, so the FOPs are
compared with the FOP tolerance of the parity tests (1e-5 of the plane's power
+ 1e-6 of the cell's power); two calls in a row on different spectra show that
nothing left in the shared scratch by the first call leaks into the second.
Device buffers of the test are torch tensors; the entry point itself only
takes their pointers.  Named to be collected last, so it also runs after every
other GPU test in the same process.
"""
import io

import numpy as np
import pytest

from gpu_util import make_pipeline
from test_gpu_parity import fop_within
from fdas_gb300 import _lib, synth
from fdas_gb300.fdas import FDAS
from fdas_gb300.templates import template_bank
from oracle import fdas_oracle as O

pytestmark = pytest.mark.gpu

OVERLAP = 420  # 421-tap bank


@pytest.fixture(scope="module")
def bank_p4():
    b = template_bank()
    return np.ascontiguousarray(O.to_p4(np.fft.fft(b.astype(np.complex128), 2048, axis=1)).astype(np.complex64))


def spectrum(n, seed):
    """n complex64 bins of a seeded series with one accelerated signal."""
    sig = [dict(r0=0.3 * n, z=10.0 * seed, n_harm=3, amp=0.2)]
    return synth.spectrum(synth.timeseries(2 * n, sig, seed=seed), n)[0]


def handle_fop(x, bank_p4, part=FDAS.AllAccelerations):
    p = make_pipeline(x.size, log=io.StringIO())
    assert p.upload_templates(bank_p4, FDAS.A, layout=FDAS.TemplatesFFTP4), p.last_error
    assert p.perform_input_tiling(x, FDAS.A), p.last_error
    assert p.perform_ft_convolution(part, FDAS.A), p.last_error
    fop = np.zeros(p.get_fop_sz(), dtype=np.float32)
    assert p.retrieve_FOP(fop, FDAS.A)
    return fop.reshape(85, x.size)


def noalloc_call(lib, d_x, n, d_t, d_fop, stride, d_status, part=FDAS.AllAccelerations, n_templates=85,
                 layout=FDAS.TemplatesFFTP4, stream=0):
    return lib.fdas_ft_convolution_noalloc(d_x, n, d_t, int(layout), n_templates, OVERLAP, int(part), d_fop,
                                           stride, d_status, stream)


def test_noalloc_matches_handle_two_calls(bank_p4):
    import torch
    lib = _lib.load()
    n = 100_003  # ragged: the last tile is partly padding
    stride = n + 61
    d_t = torch.from_numpy(bank_p4.view(np.float32)).cuda()
    d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for seed in (1, 2):
        x = spectrum(n, seed)
        ref = handle_fop(x, bank_p4)
        d_x = torch.from_numpy(x.view(np.float32)).cuda()
        d_fop = torch.full((85, stride), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        st = noalloc_call(lib, d_x.data_ptr(), n, d_t.data_ptr(), d_fop.data_ptr(), stride, d_status.data_ptr(),
                          stream=stream)
        assert st == _lib.OK
        torch.cuda.synchronize()
        assert int(d_status.item()) == 0
        fop = d_fop.cpu().numpy()
        assert np.isnan(fop[:, n:]).all()  # columns beyond n_bins untouched
        assert fop_within(fop[:, :n], ref).all()


def test_noalloc_part_rows_only(bank_p4):
    import torch
    lib = _lib.load()
    n = 4096
    x = spectrum(n, 3)
    d_x = torch.from_numpy(x.view(np.float32)).cuda()
    d_t = torch.from_numpy(bank_p4.view(np.float32)).cuda()
    for part, rows in ((FDAS.NegativeAccelerations, np.arange(0, 43)),
                       (FDAS.PositiveAccelerations, np.arange(42, 85))):
        ref = handle_fop(x, bank_p4, part)
        d_fop = torch.full((85, n), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        assert noalloc_call(lib, d_x.data_ptr(), n, d_t.data_ptr(), d_fop.data_ptr(), n, None, part=part) == _lib.OK
        torch.cuda.synchronize()
        fop = d_fop.cpu().numpy()
        other = np.setdiff1d(np.arange(85), rows)
        assert fop_within(fop[rows], ref[rows]).all()
        assert np.isnan(fop[other]).all()


def test_noalloc_rejects_beyond_limits(bank_p4):
    """Sizes beyond the static scratch and bad arguments are refused before
    any work is enqueued."""
    import torch
    lib = _lib.load()
    d_x = torch.zeros(2 * 4096, dtype=torch.float32, device="cuda")
    d_t = torch.from_numpy(bank_p4.view(np.float32)).cuda()
    d_fop = torch.zeros((85, 4096), dtype=torch.float32, device="cuda")
    big = 1628 * 384 + 1  # one bin more than 384 tiles hold at overlap 420
    x, t, f = d_x.data_ptr(), d_t.data_ptr(), d_fop.data_ptr()
    assert noalloc_call(lib, x, big, t, f, big, None) == _lib.ERR_CAPACITY
    assert noalloc_call(lib, x, 4096, t, f, 4096, None, n_templates=129) == _lib.ERR_CAPACITY
    assert noalloc_call(lib, x, 4096, t, f, 4096, None, n_templates=84) == _lib.ERR_INVALID_ARG
    assert noalloc_call(lib, x, 4096, t, f, 4095, None) == _lib.ERR_INVALID_ARG
    assert noalloc_call(lib, x, 4096, t, f, 4096, None, layout=FDAS.TemplatesTimeDomain) == _lib.ERR_UNSUPPORTED
    assert noalloc_call(lib, None, 4096, t, f, 4096, None) == _lib.ERR_INVALID_ARG
    # the largest accepted size runs
    n = 1628 * 384
    d_x = torch.zeros(2 * n, dtype=torch.float32, device="cuda")
    d_fop = torch.zeros((85, n), dtype=torch.float32, device="cuda")
    assert noalloc_call(lib, d_x.data_ptr(), n, t, d_fop.data_ptr(), n, None) == _lib.OK
    torch.cuda.synchronize()
    assert float(d_fop.abs().max().item()) == 0.0


def test_noalloc_natural_order_layout(bank_p4):
    """Template spectra in natural bin order (FDAS_TEMPLATES_FFT_NATURAL) give
    the same FOP as the p4-order upload of the handle path."""
    import torch
    lib = _lib.load()
    n = 20_000
    x = spectrum(n, 4)
    ref = handle_fop(x, bank_p4)
    natural = np.ascontiguousarray(O.from_p4(bank_p4).astype(np.complex64))
    d_x = torch.from_numpy(x.view(np.float32)).cuda()
    d_t = torch.from_numpy(natural.view(np.float32)).cuda()
    d_fop = torch.full((85, n), float("nan"), dtype=torch.float32, device="cuda")
    d_status = torch.zeros(1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert noalloc_call(lib, d_x.data_ptr(), n, d_t.data_ptr(), d_fop.data_ptr(), n, d_status.data_ptr(),
                        layout=FDAS.TemplatesFFTNatural) == _lib.OK
    torch.cuda.synchronize()
    assert int(d_status.item()) == 0
    assert fop_within(d_fop.cpu().numpy(), ref).all()
