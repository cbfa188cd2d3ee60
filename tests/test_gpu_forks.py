"""Forked mixing paths of the fused FP32 solve (scft_solve_opts.forks): an
instance still running at update fork_at continues on further paths with other
mixing parameters; the instance's own path wins if it converges within
fork_grace further iterations, otherwise the path that converges in the fewest
iterations wins.

Properties checked on the GPU: the instance's own path is unchanged by the forks
(instances it wins are bit-identical to the unforked solve, and no instance needs
more iterations than without forks); the outcome does not depend on which thread
groups ran which path (two solves, synchronous and asynchronous, agree bit for
bit); forked winners meet the same tolerance, also under the FP64 propagator."""
import numpy as np
import pytest

from scft_gb300 import F32, F64, ST_CONVERGED, ST_FORKED, ScftError, api, workloads as W

pytestmark = pytest.mark.gpu


def opts(**kw):
    return api.solve_opts(precision=F32, tol=1e-6, **kw)


def test_forks_never_cost_iterations_and_keep_the_instances_own_wins():
    insts = W.batch_mixed(128, seed=95)
    with api.Batch(insts) as b:
        r0 = b.solve(opts(forks=0))
        w0, phi0, _ = b.get()
        b.reset()
        r1 = b.solve(opts(forks=3, fork_at=6))
        w1, phi1, _ = b.get()
        b.evaluate(F64)
        _, phi64, _ = b.get()
    assert np.all(r0["status"] & ST_CONVERGED) and np.all(r1["status"] & ST_CONVERGED)
    assert np.all(r1["iterations"] <= r0["iterations"])
    forked = (r1["status"] & ST_FORKED) != 0
    assert forked.sum() > 0, "no forked path won on a batch forked at update 6"
    assert np.all(r1["iterations"][forked] < r0["iterations"][forked])
    for i, d in enumerate(insts):
        if not forked[i]:
            assert r1["iterations"][i] == r0["iterations"][i]
            np.testing.assert_array_equal(w1[i], w0[i])
            np.testing.assert_array_equal(phi1[i], phi0[i])
        # the FP32 stopping tolerance on the density the winner reported, and the
        # full tolerance under the FP64 propagator at the winner's field
        assert np.abs(phi1[i][1:-1] - d["f0"][1:-1]).max() <= 1e-6 * api.solve_opts().tol32_factor * (1 + 1e-9), i
        assert np.abs(phi64[i][1:-1] - d["f0"][1:-1]).max() <= 1e-6, i


def test_forked_solve_does_not_depend_on_scheduling():
    """Synchronous solves with paths taken late or first, and an asynchronous
    solve next to another batch in flight (so different groups take the paths),
    give identical results."""
    insts = W.batch_mixed(96, seed=96)
    other = W.batch_mixed(64, seed=97)
    o = opts(forks=4, fork_at=5)
    runs = []
    with api.Batch(insts) as b, api.Batch(other) as c:
        for k in range(4):
            b.reset()
            if k < 2:
                r = b.solve(o)
            elif k == 3:
                r = b.solve(opts(forks=4, fork_at=5, fork_first=1))
            else:
                c.reset()
                c.solve_async(opts(forks=2, fork_at=3))
                b.solve_async(o)
                r = b.wait()
                rc = c.wait()
                assert np.all(rc["status"] & ST_CONVERGED)
            w, phi, Q = b.get()
            runs.append((r, w, phi, Q))
    r_ref, w_ref, phi_ref, q_ref = runs[0]
    assert np.all(r_ref["status"] & ST_CONVERGED)
    for r, w, phi, Q in runs[1:]:
        np.testing.assert_array_equal(r["iterations"], r_ref["iterations"])
        np.testing.assert_array_equal(r["status"], r_ref["status"])
        np.testing.assert_array_equal(r["err"], r_ref["err"])
        np.testing.assert_array_equal(Q, q_ref)
        for x, y in zip(w, w_ref):
            np.testing.assert_array_equal(x, y)
        for x, y in zip(phi, phi_ref):
            np.testing.assert_array_equal(x, y)


def test_fork_options_are_checked():
    insts = W.batch_mixed(4, seed=98)
    with api.Batch(insts) as b:
        for bad in (dict(forks=5), dict(forks=-1), dict(forks=2, fork_at=0),
                    dict(forks=2, fork_grace=-1), dict(forks=2, fork_err=0.0)):
            with pytest.raises(ScftError):
                b.solve(opts(**bad))
        o = opts(forks=1, beta=1.0)
        o.fork_scale[0] = 1.5  # mixing parameter 1.5 > 1
        with pytest.raises(ScftError):
            b.solve(o)
        r = b.solve(opts(forks=1, fork_at=1000))  # no instance reaches the fork: the plain solve
        assert np.all(r["status"] & ST_CONVERGED) and not np.any(r["status"] & ST_FORKED)
        b.reset()
        r = b.solve(opts(forks=2, fork_at=1, finish_stall=1, finish_tol=1.0))  # the FP64 hand-off: no forks
        assert np.all(r["status"] & ST_CONVERGED) and not np.any(r["status"] & ST_FORKED)


def test_spent_budget_ends_a_forked_solve_while_groups_wait_for_paths():
    """Groups with nothing left to claim wait for other groups' forks.  A time
    budget that runs out in the middle of a forked solve must end those waits
    too: the solve returns promptly, every instance is either converged or
    stopped with the watchdog bit, and the next solve of the batch is normal."""
    import time

    insts = W.batch_mixed(64, seed=96)
    with api.Batch(insts) as b:
        r0 = b.solve(opts(forks=0))
        assert np.all(r0["status"] & ST_CONVERGED)
        b.reset()
        t = time.perf_counter()
        r = b.solve(opts(forks=3, fork_at=2, fork_err=1.0, budget_ms=4.0))
        dt = time.perf_counter() - t
        st = r["status"]
        assert np.all((st & ST_CONVERGED) | (st & 32)), st
        assert np.any(st & 32), "the budget ran out after every instance had finished"
        assert dt < 20.0
        b.reset()
        r2 = b.solve(opts(forks=3, fork_at=2, fork_err=1.0))
        assert np.all(r2["status"] & ST_CONVERGED) and not np.any(r2["status"] & 32)
