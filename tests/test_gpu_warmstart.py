"""Learned warm start: the CUDA forward/backward kernels against the FP64 numpy
gradient oracle, the device feature resampling, and what a trained network
gains over the cold start on held-out instances."""
import numpy as np
import pytest

from oracle import warmstart_oracle as WO
from scft_gb300 import F32, ST_CONVERGED, api, workloads as W
from scft_gb300.warmstart import WarmStart, batch_features, generate_and_train

pytestmark = pytest.mark.gpu


def rand_inputs(B, seed=0):
    r = np.random.default_rng(seed)
    f = r.uniform(-1, 1, (B, 5, 256)).astype(np.float32)
    t = r.normal(0, 0.5, (B, 256)).astype(np.float32)
    return f, t


def test_forward_and_gradient_match_fp64_oracle():
    ws = WarmStart(bf16=False, seed=3)
    p = ws.params()
    f, t = rand_inputs(8)
    out = ws.forward(f)
    ref_out, _ = WO.forward(p, f)
    assert np.max(np.abs(out - ref_out)) <= 1e-5 * max(1.0, np.max(np.abs(ref_out)))
    loss, g = ws.loss_grad(f, t)
    ref_loss, ref_g = WO.loss_grad(p, f, t)
    assert loss == pytest.approx(ref_loss, rel=1e-5)
    assert np.linalg.norm(g - ref_g) <= 1e-4 * np.linalg.norm(ref_g)
    # per layer block, so that no block hides behind a large one
    off = 0
    for ci, co, d, act in WO.LAYERS:
        for size in (co * ci * 5, co):
            gb, rb = g[off:off + size], ref_g[off:off + size]
            assert np.linalg.norm(gb - rb) <= 1e-4 * np.linalg.norm(rb) + 1e-12, (ci, co, size)
            off += size
    ws.close()


def test_bf16_activations_stay_close():
    ws = WarmStart(bf16=True, seed=3)
    p = ws.params()
    f, t = rand_inputs(8, seed=1)
    _, ref_g = WO.loss_grad(p, f, t)
    _, g = ws.loss_grad(f, t)
    assert np.linalg.norm(g - ref_g) <= 3e-2 * np.linalg.norm(ref_g)
    ws.close()


def test_device_features_match_oracle():
    insts = W.warmstart_eval(6, seed=77)
    with api.Batch(insts) as b:
        f, t = batch_features(b)
    for i, d in enumerate(insts):
        rf, rt = WO.features(d["x"], d["f0"], d["nsteps"], d["w0"])
        np.testing.assert_allclose(f[i], rf, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(t[i], rt, rtol=1e-5, atol=1e-6)


def test_training_reduces_loss_and_warm_start_saves_iterations():
    train = W.warmstart_train(512, seed=101)
    ws, losses, stats = generate_and_train(train, steps=600, batch=128, lr=2e-3, seed=0)
    assert stats["solved"] >= 0.95 * stats["total"]
    assert np.mean(losses[-50:]) < 0.25 * np.mean(losses[:10])
    held = W.warmstart_eval(128, seed=202)
    with api.Batch(held) as b:
        cold = b.solve(precision=F32, tol=1e-6)
        ws.predict(b)
        warm = b.solve(precision=F32, tol=1e-6)
    assert np.all(cold["status"] & ST_CONVERGED) and np.all(warm["status"] & ST_CONVERGED)
    assert warm["iterations"].mean() < 0.8 * cold["iterations"].mean(), (
        warm["iterations"].mean(), cold["iterations"].mean())
    ws.close()


def test_graded_meshes_keep_their_start():
    """The network is trained on uniform meshes: predicting over a batch leaves
    the field of an instance graded beyond a spacing ratio of 16 untouched and
    replaces the others."""
    import os
    insts = [W.instance(200, 5.0, 1024, 9, 0), W.instance(512, 5.0, 1024, 9, 1, graded=1.032)]
    ws = WarmStart(bf16=True)
    ws.load(os.path.join(os.path.dirname(__file__), "..", "scft_gb300", "weights", "warmstart_w0.npz"))
    with api.Batch(insts) as b:
        w_before = b.get()[0]
        ws.predict(b)
        w_after = b.get()[0]
    assert np.abs(w_after[0] - w_before[0]).max() > 1e-3
    np.testing.assert_array_equal(w_after[1], w_before[1])


def test_tensor_core_layers_match_the_cuda_core_layers_and_the_oracle():
    """With BF16 activations the two 64 -> 64 layers run as tcgen05 GEMMs (BF16
    operands, FP32 accumulation in tensor memory).  Their network output matches
    the CUDA-core layers and the FP64 oracle within the BF16 rounding of weights
    and activations, on two calls in a row, and no bounded wait ran out."""
    ws = WarmStart(bf16=True, seed=3)
    p = ws.params()
    f, _ = rand_inputs(64, seed=2)
    ref, _ = WO.forward(p, f)
    scale = max(1.0, float(np.max(np.abs(ref))))
    assert ws.set_tensor_cores(False)
    out_cc = ws.forward(f)
    assert not ws.set_tensor_cores(True)
    for _ in range(2):
        out_tc = ws.forward(f)
        e_ref = float(np.max(np.abs(out_tc - ref))) / scale
        e_cc = float(np.max(np.abs(out_tc - out_cc))) / scale
        e_cc_ref = float(np.max(np.abs(out_cc - ref))) / scale
        assert e_ref <= 2e-2 and e_cc <= 2e-2, (e_ref, e_cc, e_cc_ref)
    assert ws.tensor_core_status() == 0
    ws.close()
