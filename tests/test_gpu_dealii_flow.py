"""One refinement level of the deal.II driver (drivescft.cc:258-321) on the GPU,
through the library's entry points: the N=33 field of N=33_for_read.txt
(converged to 1.4e-9 under IRK2 + consistent W, Romberg, 2048 steps, f0 - phi),
every cell bisected and the field carried over by the not-a-knot spline
(refine_mesh, scft.cc:132-166), then the driver's chain of adm_chen calls
(drivescft.cc:292-296) on the 65-node problem with the device residual.  The
converged field is checked with the oracle's deal.II propagator."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from scft_gb300 import F64, RULE_ROMBERG, SCHEME_IRK2, W_CONSISTENT, api

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def configure(oracle, x, w, tau):
    f0 = oracle.f0_tanh2_le(x, tau)
    api.set_config(f0, x=x, nsteps=2048, ds=1.0 / 2048, rule=RULE_ROMBERG, sign=-1, precision=F64,
                   scheme=SCHEME_IRK2, wmode=W_CONSISTENT, w_wall=(w[0], w[-1]))
    return f0


def test_refine_then_adm_chen_chain_converges(oracle):
    g = json.load(open(os.path.join(GOLD, "dealii_N33.json")))
    x, w = np.array(g["x"]), np.array(g["w"])
    configure(oracle, x, w, g["tau"])
    assert np.abs(api.fem_residual(w[1:-1])).max() < 2e-9       # the file's field is converged
    xn = api.refine_bisect(x)
    wn = api.transfer_field(x, w, xn)
    f0n = configure(oracle, xn, wn, g["tau"])
    e0 = np.abs(api.fem_residual(wn[1:-1])).max()
    v = wn[1:-1].copy()
    n = len(v)
    import time
    t = time.perf_counter()
    evals = 0
    for tol, maxit, lmd, nn, final in ((1e-1, 200, 0.99, 2, False), (1e-3, 300, 0.9, 3, False),
                                       (1e-7, 800, 0.9, 15, False), (1e-7, 1000, 0.9, 30, False),
                                       (1e-7, 10000, 0.1, 50, True)):
        rc, v = api.adm_chen(api.FEM_RESIDUAL0, v, tol, maxit, n, lmd, nn, final)
    print(f"adm_chen chain on 65 nodes (IRK2, consistent W): {time.perf_counter() - t:.2f} s")
    e1 = np.abs(api.fem_residual(v)).max()
    assert e1 < 1e-7 < e0, (e0, e1)
    p = orc.OracleProblem(xn, f0n, 1.0 / 2048, 2048, rule=orc.RULE_ROMBERG, wmode=orc.W_CONSISTENT,
                          scheme=orc.SCHEME_IRK2, sign=-1, wall_w=[wn[0], wn[-1]])
    ref, _ = oracle.residual(p, v)
    assert np.abs(ref).max() < 1e-7
    api.set_config(f0n, x=xn)  # back to the default drop-in configuration
