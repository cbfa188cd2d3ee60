"""GPU propagator parity: the sm_103a kernels through the C ABI against the oracle.

Bars: FP64 density within 1e-10 relative (of max |phi|) of the oracle; FP32
density within 1e-5 relative; Q alike."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc
from scft_gb300 import F32, F64, RULE_ROMBERG, RULE_TRAPEZOID, ST_CONVERGED, api, workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL64, TOL32 = 1e-10, 1e-5


def ref_phi(O, d, w=None):
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d.get("rule", RULE_ROMBERG))
    return O.propagate(p, d["w0"] if w is None else w)


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def gpu_eval(insts, prec):
    with api.Batch(insts) as b:
        b.evaluate(prec)
        _, phi, Q = b.get()
        st = b.status()
    return phi, Q, st


def field(d, amp=1.0, seed=0):
    """A wall-attracting field of converged shape (strongly negative near the walls)."""
    x, L = d["x"], d["L"]
    r = np.random.default_rng(seed)
    w = -amp * 8.0 * (np.exp(-(x / 0.3) ** 2) + np.exp(-((L - x) / 0.3) ** 2)) + 0.05 * r.normal(size=len(x))
    w[0] = w[-1] = 0.0
    return w


@pytest.mark.parametrize("m_elem,nsteps,rule", [
    (2, 16, RULE_ROMBERG), (3, 16, RULE_ROMBERG), (16, 64, RULE_ROMBERG), (32, 2048, RULE_ROMBERG),
    (33, 512, RULE_ROMBERG), (62, 128, RULE_ROMBERG), (65, 1024, RULE_ROMBERG), (128, 256, RULE_ROMBERG),
    (200, 512, RULE_ROMBERG), (255, 512, RULE_ROMBERG), (300, 1024, RULE_ROMBERG),
    (513, 512, RULE_ROMBERG), (1024, 2048, RULE_ROMBERG), (32, 2049, RULE_TRAPEZOID),
    (100, 777, RULE_TRAPEZOID),
])
def test_density_matches_oracle(oracle, m_elem, nsteps, rule):
    d = W.instance(m_elem, 4.0 + m_elem / 200.0, nsteps, seed=1, inst=m_elem, rule=rule)
    if rule == RULE_TRAPEZOID:
        d["ds"] = 1.0 / 2048 if nsteps == 2049 else 1.0 / nsteps
    for w in (d["w0"], field(d)):
        phi_ref, Q_ref = ref_phi(oracle, d, w)
        dd = dict(d, w0=w)
        for prec, tol in ((F64, TOL64), (F32, TOL32)):
            phi, Q, st = gpu_eval([dd], prec)
            assert rel(phi[0], phi_ref) <= tol, (prec, rel(phi[0], phi_ref))
            assert abs(Q[0] - Q_ref) <= tol * abs(Q_ref)
            assert st[0] == 0


def test_every_shape_gives_the_same_density(oracle):
    d = W.instance(200, 6.0, 256, seed=2, inst=0)
    w = field(d)
    phi_ref, _ = ref_phi(oracle, d, w)
    dd = dict(d, w0=w)
    shapes = [(C, NW) for C in (1, 2, 4, 8) for NW in (1, 2, 4, 8, 16, 32) if 32 * NW * C >= 199]
    for prec, tol in ((F64, TOL64), (F32, TOL32)):
        for C, NW in shapes:
            with api.Batch([dd]) as b:
                b.set_shape(prec, 0, C, NW)
                b.evaluate(prec)
                _, phi, _ = b.get()
            assert rel(phi[0], phi_ref) <= tol, (prec, C, NW, rel(phi[0], phi_ref))


def test_mixed_batch_matches_oracle(oracle):
    insts = W.batch_mixed(48, seed=9)
    refs = [ref_phi(oracle, d) for d in insts]
    for prec, tol in ((F64, TOL64), (F32, TOL32)):
        phi, Q, st = gpu_eval(insts, prec)
        for i, (pr, qr) in enumerate(refs):
            assert rel(phi[i], pr) <= tol, (prec, i)
            assert abs(Q[i] - qr) <= tol * abs(qr)
        assert not np.any(st)


def test_graded_mesh_matches_oracle(oracle):
    d = W.instance(512, 7.0, 512, seed=4, inst=0, graded=1.01)
    w = field(d)
    phi_ref, Q_ref = ref_phi(oracle, d, w)
    for prec, tol in ((F64, TOL64), (F32, TOL32)):
        phi, Q, _ = gpu_eval([dict(d, w0=w)], prec)
        assert rel(phi[0], phi_ref) <= tol, (prec, rel(phi[0], phi_ref))


def test_drop_in_residual_on_matlab_golden(oracle):
    """simple_FEM_1D_transient replacement on Matlab_files/inputFiles/solution_matlab_N=33."""
    g = json.load(open(os.path.join(GOLD, "matlab_N33.json")))
    x, w, f0 = map(np.array, (g["x"], g["w"], g["f0"]))
    api.set_config(f0, x=x, nsteps=2049, ds=1.0 / 2048, rule=RULE_TRAPEZOID, sign=-1)
    N = len(x) - 2
    win = np.concatenate([[0.0], w[1:-1]])
    out = np.zeros(N + 1)
    assert api.simple_FEM_1D_transient(N, win, out) == 0
    ref = np.array(g["f0"])[1:-1] - np.array(g["oracle_phi"])[1:-1]
    np.testing.assert_allclose(out[1:], ref, rtol=0, atol=1e-13)
    assert np.abs(out[1:]).max() < 3e-7
    phi, Q = api.density(w)
    np.testing.assert_allclose(phi, g["oracle_phi"], rtol=0, atol=1e-13)


def test_fp32_error_budget_large_mesh(oracle):
    """1024 elements, 2048 steps: FP32 density / Q / free-energy-type integral
    against the FP64 oracle."""
    d = W.single_large()
    w = field(d, amp=1.5)
    phi_ref, Q_ref = ref_phi(oracle, d, w)
    phi, Q, _ = gpu_eval([dict(d, w0=w)], F32)
    assert rel(phi[0], phi_ref) <= TOL32
    assert abs(Q[0] - Q_ref) / Q_ref <= TOL32
    x = d["x"]
    fe = lambda p: np.sum(0.5 * (p[1:] + p[:-1]) * np.diff(x) * 0.5 * (w[1:] + w[:-1]))  # noqa: E731
    assert abs(fe(phi[0]) - fe(phi_ref)) <= TOL32 * abs(fe(phi_ref))


def test_evaluation_is_deterministic():
    insts = W.batch_mixed(16, seed=12)
    a = gpu_eval(insts, F32)[0]
    b = gpu_eval(insts, F32)[0]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_lost_dominance_is_flagged():
    d = W.instance(40, 4.0, 64, seed=0, inst=0)
    w = np.full(41, -200.0)
    w[0] = w[-1] = 0
    _, _, st = gpu_eval([dict(d, w0=w)], F64)
    assert st[0] & 1


def test_free_energy_known_answer(oracle):
    """N=33_for_read.txt stores the mean-field free energy 0.001945037280931 of
    its field (scft.cc:404-450: Romberg over 2^18+1 samples of the tanh^2 target)."""
    g = json.load(open(os.path.join(GOLD, "dealii_N33.json")))
    x, w = np.array(g["x"]), np.array(g["w"])
    m = 2 ** 18
    xs = np.linspace(0.0, g["L"], m + 1)
    fs = oracle.f0_tanh2_le(xs, g["tau"])
    d = {"n_nodes": len(x), "x": x, "L": g["L"], "f0": np.array(g["f0"]), "w0": w, "nsteps": 2048,
         "ds": 1.0 / 2048}
    with api.Batch([d]) as b:
        F = b.free_energy(fs[None, :])
    assert abs(F[0] - g["file_free_energy"]) < 1e-13


def test_free_energy_matches_oracle(oracle):
    insts = W.batch_mixed(8, seed=21)
    m = 2 ** 12
    fs = np.stack([W.gauss_wall_f0(np.linspace(0.0, d["L"], m + 1), d["L"]) for d in insts])
    ws = [field(d) for d in insts]
    with api.Batch([dict(d, w0=w) for d, w in zip(insts, ws)]) as b:
        F = b.free_energy(fs)
    for i, d in enumerate(insts):
        ref = oracle.free_energy(d["x"], ws[i], fs[i])
        assert abs(F[i] - ref) <= 1e-12 * max(1.0, abs(ref)), (i, F[i], ref)


def test_fp32_solution_error_single_large(oracle):
    """1024 elements, 2048 steps, L = 4: the field converged by the batched
    solver with the FP32 propagator against the oracle's FP64 solve of the same
    instance (both to ||phi - f0||_inf <= 1e-6): density at the converged
    fields, Q and the mean-field free energy."""
    d = W.single_large()
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d.get("rule", RULE_ROMBERG))
    rc, w64, it64, err64 = oracle.anderson_solve(p, d["w0"], tol=1e-6)
    assert rc == 0
    phi64, Q64 = oracle.propagate(p, w64)
    with api.Batch([d]) as b:
        r = b.solve(api.solve_opts(precision=F32, tol=1e-6))
        assert r["status"][0] & ST_CONVERGED
        w32, phi32, Q32 = b.get()
    m = 2 ** 14
    xs = np.linspace(0.0, d["L"], m + 1)
    fs = W.gauss_wall_f0(xs, d["L"])
    fe64 = oracle.free_energy(d["x"], w64, fs)
    fe32 = oracle.free_energy(d["x"], w32[0], fs)
    e_phi = float(np.abs(phi32[0] - phi64).max())
    e_Q = abs(Q32[0] - Q64) / abs(Q64)
    e_F = abs(fe32 - fe64)
    print(f"fp32 solution error: phi {e_phi:.3e} Q(rel) {e_Q:.3e} F {e_F:.3e} (F64 {fe64:.15e})")
    assert e_phi <= 3e-6 and e_Q <= 1e-5 and e_F <= 1e-8
