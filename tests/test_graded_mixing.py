"""The graded-mesh step of the batched mixing (scft_solve_opts.graded_ratio /
precond_hfloor), on the oracle's restatement (CPU) and on the GPU.

On meshes graded toward the walls far below the contour diffusion scale
sqrt(ds), the preconditioner's curvature term at the smallest elements and one
wall node's bounded move would throttle the whole field update: the error stays
near 0.8.  Flooring the preconditioner's spacings at sqrt(0.1 ds) and clamping
each node's move instead of scaling the whole step lets these instances
converge; meshes with a spacing ratio below graded_ratio are unaffected."""
import numpy as np
import pytest

from oracle import oracle as orc
from scft_gb300 import F32, F64, ST_CONVERGED, api, workloads as W


def graded(k, L=None, m=512, ratio=1.032, nsteps=2048):
    return W.instance(m, 3.0 + 2.0 * k if L is None else L, nsteps, 5, k, graded=ratio)


def test_graded_step_converges_where_the_uniform_step_stalls(oracle):
    d = graded(0)
    h = np.diff(d["x"])
    assert h.max() / h.min() > 1000 and h.min() < 1e-3 * d["ds"] ** 0.5
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"])
    rc, w, it, err = oracle.anderson_solve(p, d["w0"], tol=1e-6, maxit=400)
    assert rc == 0 and err <= 1e-6 and it < 400, (rc, it, err)
    rc, w, it, err = oracle.anderson_solve(p, d["w0"], tol=1e-6, maxit=60, graded_ratio=0.0)
    assert rc == 1 and err > 0.5, (rc, it, err)  # the uniform step: stuck


def test_graded_step_leaves_uniform_meshes_alone(oracle):
    d = W.warmstart_eval(1, seed=57)[0]
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"])
    a = oracle.anderson_solve(p, d["w0"], tol=1e-6, maxit=30)
    b = oracle.anderson_solve(p, d["w0"], tol=1e-6, maxit=30, graded_ratio=0.0)
    assert a[2] == b[2]
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.gpu
@pytest.mark.parametrize("k", [1, 3])
def test_gpu_graded_iterates_match_oracle(oracle, k):
    """k FP64 iterations of the batched GPU solver on graded meshes against the
    oracle's restatement of the graded-mesh step."""
    insts = [graded(i) for i in range(3)]
    with api.Batch(insts) as b:
        b.solve(precision=F64, tol=1e-12, maxit=k)
        w, _, _ = b.get()
    for i, d in enumerate(insts):
        p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"])
        rc, wo, it, err = oracle.anderson_solve(p, d["w0"], tol=1e-12, maxit=k)
        assert it == k
        np.testing.assert_allclose(w[i], wo, rtol=0, atol=1e-8 * max(1.0, np.abs(wo).max()))


@pytest.mark.gpu
def test_gpu_graded_iterates_match_oracle_at_depth_16(oracle):
    """13 FP64 iterations with the mixing used for graded batches (Anderson depth
    16, preconditioner 0.2), so that the history holds more than the default 10
    entries, against the oracle with the same options.  From a cold start these
    iterations amplify rounding (clamped wall nodes, near-singular least
    squares): the oracle's own 13th iterate moves by up to 5e-5 of max|w| when
    its start moves by 1e-14.  The bound is 20 times that spread, measured here
    for each instance; the depth-10 iterate differs from the depth-16 one by more
    than 0.1 of max|w|, far outside it."""
    k, mix = 13, dict(depth=16, precond=0.2)
    insts = [graded(i) for i in range(3)]
    with api.Batch(insts) as b:
        b.solve(precision=F64, tol=1e-12, maxit=k, **mix)
        w, _, _ = b.get()
    for i, d in enumerate(insts):
        p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"])
        rc, wo, it, err = oracle.anderson_solve(p, d["w0"], tol=1e-12, maxit=k, **mix)
        assert it == k
        scale = max(1.0, np.abs(wo).max())
        spread = 0.0
        for e in (1e-14, -1e-14):
            w1 = d["w0"].copy()
            w1[1:-1] *= 1.0 + e
            spread = max(spread, np.abs(oracle.anderson_solve(p, w1, tol=1e-12, maxit=k, **mix)[1] - wo).max())
        bound = max(1e-8 * scale, 20.0 * spread)
        assert bound <= 1e-3 * scale, (i, spread / scale)
        np.testing.assert_allclose(w[i], wo, rtol=0, atol=bound)
        w10 = oracle.anderson_solve(p, d["w0"], tol=1e-12, maxit=k, depth=10, precond=0.2)[1]
        assert np.abs(w10 - wo).max() > 100.0 * bound, i


@pytest.mark.gpu
def test_gpu_graded_batch_converges():
    """A batch of graded instances converges in the fused FP32 solve, and every
    field passes the tolerance under the FP64 propagator.  These 512-element
    meshes leave a discretisation floor near 6e-7 on ||phi - f0|| (the FP64
    oracle stalls there too), so the tolerance is 2e-6."""
    insts = [graded(i, L=3.0 + 0.5 * i) for i in range(12)]  # L in [3, 8.5]
    with api.Batch(insts) as b:
        r = b.solve(api.solve_opts(precision=F32, tol=2e-6))
        b.evaluate(F64)
        _, phi64, _ = b.get()
    assert np.all(r["status"] & ST_CONVERGED), r
    for i, d in enumerate(insts):
        assert np.abs(phi64[i][1:-1] - d["f0"][1:-1]).max() <= 2e-6, i


def _staged_plan(insts, stride):
    """CPU restatement of the staged solve's plan (one mesh shape): sorted by
    film width, every stride-th and the widest solved first; the others start
    between their nearest first-stage neighbours.  Returns (first, {i: (a, b, t)})."""
    order = sorted(range(len(insts)), key=lambda i: insts[i]["L"])
    m = len(order)
    first = {order[r] for r in range(m) if r % stride == 0 or r == m - 1}
    plan = {}
    for r, i in enumerate(order):
        if i in first:
            continue
        a = max((order[q] for q in range(r) if order[q] in first), key=lambda j: insts[j]["L"], default=None)
        b = min((order[q] for q in range(r + 1, m) if order[q] in first), key=lambda j: insts[j]["L"], default=None)
        a = b if a is None else a
        b = a if b is None else b
        t = 0.0 if insts[b]["L"] == insts[a]["L"] else (insts[i]["L"] - insts[a]["L"]) / (insts[b]["L"] - insts[a]["L"])
        plan[i] = (a, b, t)
    return first, plan


@pytest.mark.gpu
def test_gpu_staged_transfer_starts_from_interpolated_neighbours():
    """transfer_stride: the second-stage instances of a staged solve start from
    the field interpolated in L between their converged first-stage neighbours.
    Each one's result is bit-identical to a plain solve started from that field
    computed on the host, every instance converges and passes the FP64 check, and
    the transferred starts need fewer iterations than the first stage."""
    insts = [graded(i, L=3.0 + 0.1 * i) for i in range(21)]
    stride = 4
    with api.Batch(insts) as b:
        r = b.solve(api.solve_opts(precision=F32, tol=2e-6, transfer_stride=stride))
        w, _, _ = b.get()
        b.evaluate(F64)
        _, phi64, _ = b.get()
    assert np.all(r["status"] & ST_CONVERGED), r["status"]
    for i, d in enumerate(insts):
        assert np.abs(phi64[i][1:-1] - d["f0"][1:-1]).max() <= 2e-6, i
    first, plan = _staged_plan(insts, stride)
    assert len(first) == 6 and len(plan) == 15
    second = sorted(plan)
    starts = []
    for i in second:
        a, b_, t = plan[i]
        s = insts[i]["w0"].copy()
        s[1:-1] = (1.0 - t) * w[a][1:-1] + t * w[b_][1:-1]
        starts.append(s)
    with api.Batch([insts[i] for i in second]) as b2:
        b2.set_fields(starts)
        r2 = b2.solve(api.solve_opts(precision=F32, tol=2e-6))
        w2, _, _ = b2.get()
    for k, i in enumerate(second):
        assert r2["iterations"][k] == r["iterations"][i], i
        np.testing.assert_array_equal(w2[k], w[i])
    it1 = np.mean([r["iterations"][i] for i in first])
    it2 = np.mean([r["iterations"][i] for i in second])
    assert it2 < it1, (it1, it2)


@pytest.mark.gpu
def test_gpu_graded_fp64_hand_off_matches_the_oracle(oracle):
    """Graded 1024-element meshes (the spacing range of the 8192-element workload
    at 1/8 of its nodes): FP32 solves with the FP64 hand-off (finish_stall)
    converge every instance the oracle's FP64 restatement converges, and each
    field passes the tolerance under the FP64 propagator."""
    insts = [W.instance(1024, L, 2048, 5, k, graded=1.0161) for k, L in enumerate((3.0, 4.5, 6.0, 8.0))]
    tol = 2e-6
    out, _, _ = orc.cpu_solve_batch(insts, workers=len(insts), tol=tol, maxit=600)
    ok = [rc == 0 for rc, _, _ in out]
    assert any(ok)
    with api.Batch(insts) as b:
        r = b.solve(api.solve_opts(precision=F32, tol=tol, maxit=600, finish_stall=10, finish_tol=1e-4))
        b.evaluate(F64)
        _, phi64, _ = b.get()
    for i, d in enumerate(insts):
        if ok[i]:
            assert r["status"][i] & ST_CONVERGED, (i, r["status"][i], r["iterations"][i])
        if r["status"][i] & ST_CONVERGED:
            assert np.abs(phi64[i][1:-1] - d["f0"][1:-1]).max() <= tol, i


@pytest.mark.gpu
def test_gpu_staged_solve_on_a_mixed_batch_converges_every_instance():
    """A staged solve of a uniform-mesh batch in which only some instances share
    a mesh shape (node count, contour steps, rule): shapes with fewer than three
    instances stay in the first stage, the rest transfer; every instance
    converges to the FP32 stopping tolerance and passes 1e-6 under FP64."""
    insts = [W.instance(m, 2.0 + 0.4 * k, ns, 7, k) for k, (m, ns) in
             enumerate([(128, 1024)] * 9 + [(200, 2048)] * 2 + [(96, 512)] * 5)]
    with api.Batch(insts) as b:
        r = b.solve(api.solve_opts(precision=F32, tol=1e-6, transfer_stride=3))
        st = b.status()
        b.evaluate(F64)
        _, phi64, _ = b.get()
    assert np.all(r["status"] & ST_CONVERGED), r["status"]
    np.testing.assert_array_equal(st, r["status"])
    for i, d in enumerate(insts):
        assert np.abs(phi64[i][1:-1] - d["f0"][1:-1]).max() <= 1e-6, i
