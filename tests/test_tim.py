"""SIGPROC .tim reader (fdas_gb300.tim) against what the reference's own
reader (ft_conv.py:39-64) returned for the committed fixture files
(tests/golden/make_tim_golden.py), plus a write / read round trip."""
import json

import numpy as np
import pytest

from conftest import ROOT
from fdas_gb300 import tim

GOLD = ROOT / "tests" / "golden"


def cases():
    return json.loads((GOLD / "tim_golden.json").read_text())


@pytest.mark.parametrize("name", sorted(json.loads((ROOT / "tests/golden/tim_golden.json").read_text())))
def test_reader_matches_reference(name):
    g = cases()[name]
    path = GOLD / f"{name}.tim"
    if g["error"]:
        with pytest.raises(RuntimeError) as e:
            tim.read_tim(path, read_header=g["read_header"])
        assert str(e.value) == g["error"]
        return
    x, t = tim.read_tim(path, read_header=g["read_header"])
    assert x.dtype == np.float32 and x.size == g["n"]
    assert t == g["t_samp"]
    assert np.array_equal(x[:4], np.array(g["first"], dtype=np.float32))
    assert float(np.sum(x.astype(np.float64))) == g["sum"]


@pytest.mark.parametrize("header", [True, False])
def test_write_read_round_trip(tmp_path, header):
    x = np.random.default_rng(3).standard_normal(4099).astype(np.float32)
    p = tmp_path / "a.tim"
    tim.write_tim(p, x, t_samp=1.28e-4, header=header)
    y, t = tim.read_tim(p, read_header=header)
    assert np.array_equal(x, y)
    assert t == (1.28e-4 if header else None)
