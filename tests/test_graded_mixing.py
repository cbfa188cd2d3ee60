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
