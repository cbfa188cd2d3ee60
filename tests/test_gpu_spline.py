"""Mesh refinement and field transfer of the deal.II driver on the GPU:
scft_spline against the golden values of the reference's spline_chen
(spline_chen.c:13-106, compiled from the reference) and the oracle's
restatement; scft_refine_bisect; the refine_mesh transfer of the N=33 golden
field (scft.cc:132-166)."""
import json
import os

import numpy as np
import pytest

from scft_gb300 import ScftError, _lib, api

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def cases():
    return json.load(open(os.path.join(GOLD, "spline.json")))["cases"]


def test_spline_matches_reference_golden_values():
    for c in cases():
        if c["rc"] != 0:
            with pytest.raises(ScftError) as e:
                api.spline([(c["x"], c["y"], c["xp"])], m=c["m"])
            assert e.value.code == _lib.SCFT_EINVAL
            continue
        yp = api.spline([(c["x"], c["y"], c["xp"])], m=c["m"])[0]
        np.testing.assert_allclose(yp, c["yp"], rtol=1e-12, atol=1e-12 * np.abs(c["yp"]).max(), err_msg=c["name"])


def test_many_tables_in_one_call_match_the_oracle(oracle):
    rng = np.random.default_rng(3)
    tabs = []
    for k in range(300):
        nx = int(rng.integers(4, 200))
        x = np.sort(rng.uniform(0, 10, nx))
        tabs.append((x, np.sin(x) * k / 300 + 0.01 * rng.normal(size=nx), rng.uniform(-1, 11, int(rng.integers(0, 50)))))
    for m in (None, 0.0):
        got = api.spline(tabs, m=m)
        for (x, y, xp), g in zip(tabs, got):
            ref = oracle.spline(x, y, xp, m)[1]
            np.testing.assert_allclose(g, ref, rtol=1e-11, atol=1e-11 * max(1.0, np.abs(ref).max() if len(ref) else 1.0))


def test_refine_bisect_and_field_transfer_of_the_golden_field(oracle):
    g = json.load(open(os.path.join(GOLD, "dealii_N33.json")))
    x, w = np.array(g["x"]), np.array(g["w"])
    xn = api.refine_bisect(x)
    assert len(xn) == 65 and np.all(xn[0::2] == x) and np.allclose(xn[1::2], 0.5 * (x[:-1] + x[1:]))
    wn = api.transfer_field(x, w, xn)
    ref = next(c for c in json.load(open(os.path.join(GOLD, "spline.json")))["cases"] if c["name"].startswith("refine"))
    np.testing.assert_allclose(wn[1:-1], ref["yp"], rtol=1e-12, atol=1e-12)
    assert wn[0] == w[0] and wn[-1] == w[-1]
    np.testing.assert_allclose(wn[2:-1:2], w[1:-1], rtol=1e-12, atol=1e-12)  # old interior nodes keep their values
    with pytest.raises(ScftError):
        api.refine_bisect([0.0, 1.0, 1.0])
