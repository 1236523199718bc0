"""Helpers shared by the GPU tests."""
import numpy as np

from fdas_gb300.fdas import FDAS
from oracle import fdas_oracle as O


def make_pipeline(n_bins, log=None, **kw):
    p = FDAS(log)
    assert p.initialise_accelerator(n_bins, **kw), p.last_error
    return p


def candidates_as_arrays(rec, half=42):
    """(location u32, power f32) sorted by location from candidate records."""
    loc = O.encode_location(rec["harmonic"], rec["template_num"], rec["bin"])
    return loc, rec["power"].astype(np.float32)


def validate_harmonic_summing(loc, pwr, loc_ref, pwr_ref, tol=1e-5):
    """main_gtest.cpp:192-228: strip invalid entries, require >= 1 candidate and
    every candidate in the reference list with |d power| < tol."""
    keep = loc != O.INVALID_LOCATION
    loc, pwr = loc[keep], pwr[keep]
    assert loc.size <= loc_ref.size
    assert loc.size >= 1
    idx = {int(l): i for i, l in enumerate(loc_ref.tolist())}
    bad = [int(l) for l in loc.tolist() if int(l) not in idx]
    assert not bad, f"{len(bad)} candidates not in the reference list, e.g. {O.decode_location(bad[:3])}"
    ref_p = pwr_ref[[idx[int(l)] for l in loc.tolist()]]
    assert np.all(np.abs(pwr - ref_p) < tol)
