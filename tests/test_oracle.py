"""The oracle pinned against the reference: golden fields, known answers and the
reference's own NR routines (compiled from source, or their committed outputs)."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


def test_matlab_golden_field_pins_the_method(oracle):
    """solution_matlab_N=33 is converged under row-scaled W, implicit Euler with
    2049 steps of 1/2048 and the trapezoid rule (simple_FEM_1D_transient.m)."""
    g = load("matlab_N33.json")
    x, w, f0 = map(np.array, (g["x"], g["w"], g["f0"]))
    p = orc.OracleProblem(x, f0, 1.0 / 2048, 2049, rule=orc.RULE_TRAPEZOID, sign=-1)
    out, _ = oracle.residual(p, w[1:-1])
    assert np.abs(out).max() < 3e-7
    # any other reading of the method leaves a residual thousands of times larger
    for ns, rule, wm in [(2048, orc.RULE_TRAPEZOID, orc.W_ROWSCALED),
                         (2048, orc.RULE_ROMBERG, orc.W_ROWSCALED),
                         (2049, orc.RULE_TRAPEZOID, orc.W_CONSISTENT)]:
        q = orc.OracleProblem(x, f0, 1.0 / 2048, ns, rule=rule, wmode=wm, sign=-1)
        o2, _ = oracle.residual(q, w[1:-1])
        assert np.abs(o2).max() > 1e-4


def test_dealii_golden_field_pins_irk(oracle):
    """N=33_for_read.txt (ERROR= 1.422819e-09) under consistent W, Gauss-Legendre
    IRK2, 2048 steps, Romberg (drivescft.cc:130-207, scft.cc:589-696)."""
    g = load("dealii_N33.json")
    x, w = np.array(g["x"]), np.array(g["w"])
    f0 = oracle.f0_tanh2_le(x, g["tau"])
    p = orc.OracleProblem(x, f0, 1.0 / 2048, 2048, rule=orc.RULE_ROMBERG, wmode=orc.W_CONSISTENT,
                          scheme=orc.SCHEME_IRK2, sign=-1, wall_w=[w[0], w[-1]])
    out, phi = oracle.residual(p, w[1:-1])
    err = np.abs(out).max()
    assert err < 2e-9
    assert abs(err - g["file_error"]) < 5e-10
    for scheme, wm in [(orc.SCHEME_IE, orc.W_CONSISTENT), (orc.SCHEME_IRK2, orc.W_ROWSCALED)]:
        q = orc.OracleProblem(x, f0, 1.0 / 2048, 2048, rule=orc.RULE_ROMBERG, wmode=wm, scheme=scheme,
                              sign=-1, wall_w=[w[0], w[-1]])
        assert np.abs(oracle.residual(q, w[1:-1])[0]).max() > 1e-5


def test_f0bar_known_answer(oracle):
    """scft.cc:368 / testFiBar.cc:50: f0bar = 0.892581217773656 (Romberg, 2^16+1 pts)."""
    n = 2 ** 16 + 1
    L, tau = 3.72374357332160, 5.30252230020752e-01
    x = oracle.mesh_uniform(n, L)
    f = oracle.f0_tanh2_le(x, tau)
    fbar = oracle.romint(f, n - 1, L / (n - 1)) / L
    assert abs(fbar - 0.892581217773656) < 2e-15
    assert abs(fbar - load("res_m32.json")["mphi"]) < 1e-11


def test_free_energy_known_answer(oracle):
    """N=33_for_read.txt stores the mean-field free energy 0.001945037280931 of its
    field (scft.cc:404-450: Romberg over 2^18+1 samples of the tanh^2 target)."""
    g = load("dealii_N33.json")
    m = 2 ** 18
    xs = np.linspace(0.0, g["L"], m + 1)
    fs = oracle.f0_tanh2_le(xs, g["tau"])
    F = oracle.free_energy(np.array(g["x"]), np.array(g["w"]), fs)
    assert abs(F - g["file_free_energy"]) < 1e-13


def test_res_phi_column_is_the_target(oracle):
    """Exp_m32_n2048_IE.res: its phi column equals the tanh^2 wall profile."""
    g = load("res_m32.json")
    x = np.array(g["x_over_l"]) * g["l"]
    f0 = oracle.f0_tanh2_le(x, g["t"])
    assert np.abs(f0 - np.array(g["phi"])).max() < 1e-10


def test_romint_matches_reference_outputs(oracle):
    for case in load("nr_routines.json")["romint"]:
        v = oracle.romint(np.array(case["f"]), case["m"], case["hh"])
        assert v == pytest.approx(case["ref"], rel=1e-13, abs=1e-15)


@pytest.mark.parametrize("m", [16, 32, 256, 2048])
def test_quadrature_weights_reproduce_romberg(oracle, m):
    rng = np.random.default_rng(m)
    f = rng.uniform(0.2, 1.0, m + 1)
    W = oracle.quad_weights(m, 1.0 / m, orc.RULE_ROMBERG)
    assert W @ f == pytest.approx(oracle.romint(f, m, 1.0 / m), rel=1e-13)
    assert W.sum() == pytest.approx(1.0, rel=1e-13)
    T = oracle.quad_weights(m + 1, 1.0 / m, orc.RULE_TRAPEZOID)
    assert T.sum() == pytest.approx((m + 1) / m, rel=1e-14)


def test_romberg_rejects_non_power_of_two(oracle):
    assert np.isnan(oracle.romint(np.ones(2050), 2049, 1 / 2048))
    with pytest.raises(ValueError):
        oracle.quad_weights(2049, 1 / 2048, orc.RULE_ROMBERG)


def test_gaussj_matches_reference_outputs(oracle):
    for case in load("nr_routines.json")["gaussj"]:
        a, b = np.array(case["a"]), np.array(case["b"])
        rc1, _, x1 = oracle.gaussj(a, b, singular_mode=1)
        assert rc1 == case["rc_dealii"]
        if case.get("singular"):
            continue
        rc0, _, x0 = oracle.gaussj(a, b, singular_mode=0)
        np.testing.assert_allclose(x0.ravel(), case["x_root"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(x1.ravel(), case["x_dealii"], rtol=1e-12, atol=1e-12)


def toy3(v):
    x, y, z = v
    return np.array([x * y * z - 12.0, x * x + y * y - 8.0, x + y + z - 511.0])


def test_adm_chen_toy_matches_reference(oracle):
    c = load("nr_routines.json")["adm_chen_toy"]
    rc, x, it, _ = oracle.adm_chen(toy3, c["x0"], c["tol"], c["maxit"], c["lmd"], c["nn"])
    assert rc == c["rc"] == 0
    np.testing.assert_allclose(x, c["x"], rtol=1e-9)
    assert it + 1 == c["calls"]


def test_adm_toy_matches_reference(oracle):
    c = load("nr_routines.json")["adm_toy"]
    myfun = lambda v: np.array([0.5 * v[0] - 2.0, 0.5 * v[1] + 3.0])  # noqa: E731
    rc, x, its = oracle.adm(myfun, c["x0"], 1e-10, 1000)
    assert rc == 0 and c["check"] == 0
    np.testing.assert_allclose(x, c["x"], rtol=1e-10)
    assert its == c["calls"]


def test_broydn_toy_matches_reference(oracle):
    c = load("nr_routines.json")["broydn_toy"]
    rc, x, its, nfev = oracle.broydn(toy3, c["x0"], c["tol"])
    np.testing.assert_allclose(x, c["x"], rtol=1e-7)
    assert nfev == c["calls"]


def test_adm_chen_scft_trajectory_matches_reference(oracle):
    """The restated adm_chen driving the restated propagator retraces the
    reference adm_chen's iterates on the MATLAB golden problem."""
    g, s = load("matlab_N33.json"), load("admchen_scft.json")
    p = orc.OracleProblem(np.array(g["x"]), np.array(g["f0"]), g["ds"], g["nsteps"],
                          rule=orc.RULE_TRAPEZOID, sign=-1)
    seen = []

    def f(v):
        seen.append(v.copy())
        return oracle.residual(p, v)[0]

    oracle.adm_chen(f, s["w0"], s["tol"], s["maxit"], s["lmd"], s["nn"])
    ref = np.array(s["trajectory"])
    got = np.array(seen[: len(ref)])
    assert len(got) == len(ref)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_broydn_scft_matches_reference(oracle):
    g, s = load("matlab_N33.json"), load("broydn_scft.json")
    p = orc.OracleProblem(np.array(g["x"]), np.array(g["f0"]), g["ds"], g["nsteps"],
                          rule=orc.RULE_TRAPEZOID, sign=-1)
    rc, x, its, nfev = oracle.broydn(p, s["w0"], s["tol"])
    assert rc == 0
    np.testing.assert_allclose(x, s["x"], rtol=1e-6, atol=1e-8)
    assert np.abs(oracle.residual(p, x)[0]).max() < s["tol"]


def test_half_store_weights_match_full_store(oracle):
    """The oracle's streaming form (quadrature weights over a half store) equals
    the per-node Romberg of the reference on the same slices."""
    x = oracle.mesh_uniform(41, 5.0)
    f0 = oracle.f0_gauss_wall(x, 5.0)
    w = np.concatenate([[0], np.sin(np.arange(39)), [0]]) * 0.3
    p = orc.OracleProblem(x, f0, 1 / 256, 256, rule=orc.RULE_ROMBERG)
    phi, Q, q = oracle.propagate(p, w, want_q=True)
    W = oracle.quad_weights(256, 1 / 256, orc.RULE_ROMBERG)
    phi_w = (W[:, None] * q * q[::-1]).sum(axis=0)
    np.testing.assert_allclose(phi_w, phi, rtol=1e-13, atol=1e-15)
    M = np.zeros(41)
    M[1:-1] = 0.5 * (x[2:] - x[:-2])
    assert Q == pytest.approx((M * q[-1]).sum() / 5.0, rel=1e-14)


def test_graded_mesh(oracle):
    x = oracle.mesh_graded(64, 1.05, 6.0)
    h = np.diff(x)
    assert x[0] == 0 and x[-1] == pytest.approx(6.0) and x[32] == pytest.approx(3.0)
    np.testing.assert_allclose(h[1:32] / h[:31], 1.05, rtol=1e-12)
    np.testing.assert_allclose(h, h[::-1], rtol=1e-12)


def test_live_reference_matches_restatement(oracle, reference):
    """Where the reference sources are present: the reference's own romint,
    gaussj and adm_chen against the restatement on fresh inputs."""
    rng = np.random.default_rng(11)
    for m in (16, 128, 1024):
        f = rng.uniform(size=m + 1)
        assert oracle.romint(f, m, 0.1) == pytest.approx(reference.romint(f, m, 0.1), rel=1e-13)
    a = rng.normal(size=(6, 6))
    b = rng.normal(size=(6, 1))
    np.testing.assert_allclose(oracle.gaussj(a, b, 1)[2], reference.gaussj(a, b)[2], rtol=1e-12)
    rc, x, _, _ = oracle.adm_chen(toy3, [1.0, 2.0, 3.0], 1e-12, 5000, 0.9, 5)
    rc2, x2, _ = reference.adm_chen(toy3, [1.0, 2.0, 3.0], 1e-12, 5000, 0.9, 5)
    assert rc == rc2
    np.testing.assert_allclose(x, x2, rtol=1e-9)


def test_spline_restatement_matches_reference_fixture(oracle):
    """spline_chen.c:13-106 restated (banded solve) against the reference's own
    routine: the refine_mesh transfer N=33 -> 65 and random tables with every
    end condition, extrapolation included; the 3-point not-a-knot call the
    reference exits on is refused."""
    for c in load("spline.json")["cases"]:
        rc, yp = oracle.spline(c["x"], c["y"], c["xp"], c["m"])
        if c["rc"] != 0:
            assert rc != 0, c["name"]
            continue
        assert rc == 0, c["name"]
        np.testing.assert_allclose(yp, c["yp"], rtol=1e-12, atol=1e-12 * np.abs(c["yp"]).max(), err_msg=c["name"])


def test_spline_restatement_matches_live_reference(oracle, reference):
    rng = np.random.default_rng(11)
    for nx in (4, 9, 64):
        x = np.sort(rng.uniform(-1, 3, nx))
        y = np.exp(-x * x) + 0.01 * rng.normal(size=nx)
        xp = np.linspace(x[0] - 0.2, x[-1] + 0.2, 33)
        for m in (None, 0.0, 0.7):
            a = oracle.spline(x, y, xp, m)[1]
            b = reference.spline(x, y, xp, m)[1]
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-13)
