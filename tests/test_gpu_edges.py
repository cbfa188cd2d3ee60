"""Edge cases of the batched path through the C ABI: the largest instance the
propagator shapes cover (32 warps x 32 lanes x 8 unknowns = 8192 interior
nodes) against the oracle, one node more rejected, empty and malformed batches
rejected with SCFT_EINVAL, a one-element mesh edge (one interior node), and
instances that differ only in their contour step counts (odd, even, powers of
two and not) in one batch."""
import numpy as np
import pytest

from oracle import oracle as orc
from scft_gb300 import F32, F64, RULE_ROMBERG, RULE_TRAPEZOID, ST_WATCHDOG, ScftError, _lib, api, workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_largest_instance_matches_oracle_and_one_more_node_is_rejected(oracle):
    d = W.instance(8193, 12.0, 64, 3, 0)   # 8194 nodes: 8192 interior unknowns
    assert d["n_nodes"] - 2 == 32 * 32 * 8
    p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"])
    phi_ref, q_ref = oracle.propagate(p, d["w0"])
    with api.Batch([d]) as b:
        for prec, tol in ((F64, 1e-10), (F32, 1e-5)):
            b.evaluate(prec)
            _, phi, Q = b.get()
            assert rel(phi[0], phi_ref) <= tol, (prec, rel(phi[0], phi_ref))
            assert abs(Q[0] - q_ref) <= tol * abs(q_ref)
            assert (b.status()[0] & ST_WATCHDOG) == 0
    big = W.instance(8194, 12.0, 64, 3, 0)
    with api.Batch([big]) as b:
        with pytest.raises(ScftError) as e:
            b.evaluate(F32)
        assert e.value.code == _lib.SCFT_EINVAL


def test_empty_and_malformed_batches_are_rejected():
    with pytest.raises(ScftError) as e:
        api.Batch([])
    assert e.value.code == _lib.SCFT_EINVAL
    good = W.instance(16, 4.0, 64, 1, 0)
    bad = [dict(good, nsteps=0), dict(good, ds=-1.0), dict(good, rule=7),
           dict(good, x=good["x"][::-1].copy()), dict(good, nsteps=48, rule=RULE_ROMBERG)]
    for d in bad:
        with pytest.raises(ScftError) as e:
            api.Batch([good, d])
        assert e.value.code == _lib.SCFT_EINVAL


def test_single_interior_node_and_ragged_step_counts(oracle):
    insts = [W.instance(2, 3.0, 16, 4, 0),                                # one interior node
             W.instance(40, 5.0, 777, 4, 1, rule=RULE_TRAPEZOID),        # odd step count
             W.instance(40, 5.0, 1000, 4, 2, rule=RULE_TRAPEZOID),       # even, not a power of two
             W.instance(40, 5.0, 4096, 4, 3),
             W.instance(41, 5.0, 16, 4, 4)]
    with api.Batch(insts) as b:
        for prec, tol in ((F64, 1e-10), (F32, 1e-5)):
            b.evaluate(prec)
            _, phi, Q = b.get()
            for i, d in enumerate(insts):
                p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d["rule"])
                phi_ref, q_ref = oracle.propagate(p, d["w0"])
                assert rel(phi[i], phi_ref) <= tol, (prec, i, rel(phi[i], phi_ref))
                assert abs(Q[i] - q_ref) <= tol * abs(q_ref), (prec, i)


def test_cluster_exchange_over_many_instances_per_cluster(oracle):
    """Shapes above 2048 interior unknowns run on thread-block clusters whose
    CTAs exchange each contour step's separator values by st.async stores that
    complete on mbarriers, the barriers' phases carried from one instance to
    the next.  200 such instances (more than the clusters resident at once, so
    each cluster takes several) with odd and even step counts, in FP32 and FP64,
    against the oracle; no exchange wait ran out.  A value that missed an
    exchange would be a step stale (an error of order ds); the FP64 bound is
    2e-10 because on these 3000-element meshes with about 60 steps the FP64
    propagator's rounding differs from the oracle's Thomas sweeps by up to
    1.05e-10 of max(phi)."""
    insts = [W.instance(3000 + 7 * (k % 5), 4.0 + 0.01 * k, 61 + (k % 4), 3, k, rule=RULE_TRAPEZOID)
             for k in range(200)]
    refs = []
    for d in insts:
        p = orc.OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d["rule"])
        refs.append(oracle.propagate(p, d["w0"]))
    with api.Batch(insts) as b:
        for prec, tol in ((F32, 1e-5), (F64, 2e-10)):
            b.evaluate(prec)
            _, phi, Q = b.get()
            assert not np.any(b.status() & ST_WATCHDOG), prec
            for i, (phi_ref, q_ref) in enumerate(refs):
                assert rel(phi[i], phi_ref) <= tol, (prec, i, rel(phi[i], phi_ref))
                assert abs(Q[i] - q_ref) <= tol * abs(q_ref), (prec, i)


def test_cluster_passes_are_bitwise_repeatable():
    """The cluster classes' per-step exchange (st.async into every CTA's shared
    memory, mbarrier completion, double-buffered by step parity) leaves no
    room for a race: repeated FP32 and FP64 passes over 48 graded
    8192-element instances (4-CTA clusters, more instances than one wave) give
    bitwise identical densities, and no exchange wait runs out."""
    insts = W.batch_graded(48)
    with api.Batch(insts) as b:
        for prec, reps in ((F32, 4), (F64, 2)):
            first = None
            for _ in range(reps):
                b.evaluate(prec)
                _, phi, Q = b.get()
                assert not np.any(b.status() & ST_WATCHDOG), prec
                cur = (np.concatenate(phi), np.asarray(Q))
                if first is None:
                    first = cur
                else:
                    np.testing.assert_array_equal(cur[0], first[0])
                    np.testing.assert_array_equal(cur[1], first[1])
