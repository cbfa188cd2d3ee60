"""The scheme-general propagator on the GPU (FP64): the deal.II form of the
reference (consistent field term, 2-stage Gauss-Legendre IRK; drivescft.cc:130-207,
scft.cc:589-696) and the implicit-Euler / row-scaled forms, against the oracle's
restatement of each, and the deal.II golden field through the drop-in residual.
Bar: density within 1e-10 relative of the oracle (FP64), Q alike."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from scft_gb300 import (F64, RULE_ROMBERG, RULE_TRAPEZOID, SCHEME_IE, SCHEME_IRK2, W_CONSISTENT, W_ROWSCALED,
                        api, workloads as W)

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-10


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def fields(insts, seed):
    r = np.random.default_rng(seed)
    out = []
    for d in insts:
        x, L = d["x"], d["L"]
        w = -6.0 * (np.exp(-(x / 0.3) ** 2) + np.exp(-((L - x) / 0.3) ** 2)) + 0.05 * r.normal(size=len(x))
        w[0], w[-1] = r.uniform(-2, 2, 2)  # wall values: used by the consistent field term only
        out.append(w)
    return out


@pytest.mark.parametrize("scheme,wmode", [(SCHEME_IRK2, W_CONSISTENT), (SCHEME_IRK2, W_ROWSCALED),
                                          (SCHEME_IE, W_CONSISTENT), (SCHEME_IE, W_ROWSCALED)])
def test_schemes_match_oracle(oracle, scheme, wmode):
    insts = [W.instance(32, 3.7, 2048, 5, 0), W.instance(65, 5.0, 512, 5, 1, rule=RULE_TRAPEZOID),
             W.instance(200, 8.0, 1024, 5, 2), W.instance(96, 4.0, 256, 5, 3, graded=1.03)]
    ws = fields(insts, 11)
    with api.Batch(insts) as b:
        b.set_fields(ws)
        b.evaluate_scheme(scheme, wmode)
        _, phi, Q = b.get()
    for i, d in enumerate(insts):
        p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d["rule"], wmode=wmode, scheme=scheme,
                              wall_w=[ws[i][0], ws[i][-1]])
        phi_ref, q_ref = oracle.propagate(p, ws[i])
        assert rel(phi[i], phi_ref) <= TOL64, (i, rel(phi[i], phi_ref))
        assert abs(Q[i] - q_ref) <= TOL64 * abs(q_ref), (i, Q[i], q_ref)


def test_ie_rowscaled_scheme_matches_the_batched_propagator():
    """Implicit Euler with the row-scaled term is the batched propagator's own
    discretisation: both GPU paths agree."""
    insts = W.batch_mixed(12, seed=17, m_hi=300)
    with api.Batch(insts) as b:
        b.evaluate(F64)
        _, p1, q1 = b.get()
        b.evaluate_scheme(SCHEME_IE, W_ROWSCALED)
        _, p2, q2 = b.get()
    for a, c in zip(p1, p2):
        assert rel(c, a) <= TOL64
    np.testing.assert_allclose(q2, q1, rtol=TOL64)


def test_dealii_golden_field_through_the_drop_in(oracle):
    """N=33_for_read.txt (file: ERROR= 1.422819e-09) with the drop-in residual in
    the deal.II configuration (f0 - phi, Romberg, 2048 steps, IRK2, consistent
    W, the file's wall values): the oracle's residual to 1e-12."""
    g = json.load(open(os.path.join(GOLD, "dealii_N33.json")))
    x, w = np.array(g["x"]), np.array(g["w"])
    f0 = oracle.f0_tanh2_le(x, g["tau"])
    api.set_config(f0, x=x, nsteps=2048, ds=1.0 / 2048, rule=RULE_ROMBERG, sign=-1, precision=F64,
                   scheme=SCHEME_IRK2, wmode=W_CONSISTENT, w_wall=(w[0], w[-1]))
    out = api.fem_residual(w[1:-1])
    p = orc.OracleProblem(x, f0, 1.0 / 2048, 2048, rule=orc.RULE_ROMBERG, wmode=orc.W_CONSISTENT,
                          scheme=orc.SCHEME_IRK2, sign=-1, wall_w=[w[0], w[-1]])
    ref, _ = oracle.residual(p, w[1:-1])
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12)
    assert abs(np.abs(out).max() - g["file_error"]) < 5e-10
    phi, Q = api.density(w)
    phi_ref, q_ref = oracle.propagate(p, w)
    assert rel(phi, phi_ref) <= TOL64 and abs(Q - q_ref) <= TOL64 * abs(q_ref)
    api.set_config(f0, x=x)  # back to the default drop-in configuration


def test_one_thread_form_for_instances_beyond_shared_memory(oracle):
    """Instances too large for the block-parallel form (coefficients in one CTA's
    shared memory, about 2200 nodes) run the one-thread form; both match the
    oracle."""
    d = W.instance(2400, 6.0, 32, 5, 0)
    ws = fields([d], 13)
    with api.Batch([d]) as b:
        b.set_fields(ws)
        b.evaluate_scheme(SCHEME_IRK2, W_CONSISTENT)
        _, phi, Q = b.get()
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d["rule"], wmode=W_CONSISTENT,
                          scheme=SCHEME_IRK2, wall_w=[ws[0][0], ws[0][-1]])
    phi_ref, q_ref = oracle.propagate(p, ws[0])
    assert rel(phi[0], phi_ref) <= TOL64 and abs(Q[0] - q_ref) <= TOL64 * abs(q_ref)
