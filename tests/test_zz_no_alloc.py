"""scft_density_noalloc, the entry point that allocates no device memory.

It exists for callers that may not allocate GPU memory -- applications whose
device memory belongs to another allocator with a fixed budget, and tight
per-iteration loops that cannot afford cudaMalloc/cudaFree, which can block on
or synchronize the whole device.  The caller hands in device buffers and the
propagator keeps its half-contour store in one fixed device array of the
library.  This test calls it through the C ABI twice in a row (two different
instances, so the second call runs over the first call's leftover scratch) and
checks each result against the allocating entry point, scft_batch_evaluate,
with the tolerances of the other parity tests: 1e-10 relative in FP64, 1e-5 in
FP32.  It also checks that the second call changes no device memory usage and
that an instance larger than the fixed scratch is refused with a clear error.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from scft_gb300 import F32, F64, RULE_ROMBERG, RULE_TRAPEZOID, _lib, api, workloads as W

pytestmark = pytest.mark.gpu

TOL = {F64: 1e-10, F32: 1e-5}


def _instances():
    a = W.instance(300, 6.0, 1024, seed=5, inst=0)
    b = W.instance(120, 3.5, 2049, seed=5, inst=1, rule=RULE_TRAPEZOID)
    b["ds"] = 1.0 / 2048
    return [a, b]


def _ptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def test_noalloc_matches_the_allocating_entry_point_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    insts = _instances()
    for prec in (F64, F32):
        with api.Batch(insts) as b:
            b.evaluate(prec)
            _, phi_ref, Q_ref = b.get()
        bufs = []
        for d in insts:
            n = d["n_nodes"]
            bufs.append((torch.tensor(d["x"], dtype=torch.float64, device="cuda"),
                         torch.tensor(d["w0"], dtype=torch.float64, device="cuda"),
                         torch.full((n,), float("nan"), dtype=torch.float64, device="cuda"),
                         torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")))
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        for call, (d, (x, w, phi, Q)) in enumerate(zip(insts, bufs)):
            free_before = torch.cuda.mem_get_info()[0]
            rc = lib.scft_density_noalloc(d["n_nodes"], _ptr(x), _ptr(w), d["nsteps"], d["ds"],
                                          d.get("rule", RULE_ROMBERG), prec, _ptr(phi), _ptr(Q), stream)
            assert rc == 0, lib.scft_last_error().decode()
            torch.cuda.synchronize()
            if call > 0:
                assert torch.cuda.mem_get_info()[0] == free_before
            got = phi.cpu().numpy()
            ref = phi_ref[call]
            assert np.max(np.abs(got - ref)) <= TOL[prec] * np.max(np.abs(ref)), (prec, call)
            assert abs(Q.cpu().item() - Q_ref[call]) <= TOL[prec] * abs(Q_ref[call])


def test_noalloc_refuses_an_instance_larger_than_its_scratch():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d = W.instance(8192, 7.0, 8192, seed=1, inst=0, graded=1.002)
    x = torch.tensor(d["x"], dtype=torch.float64, device="cuda")
    phi = torch.empty(d["n_nodes"], dtype=torch.float64, device="cuda")
    rc = lib.scft_density_noalloc(d["n_nodes"], _ptr(x), _ptr(x), d["nsteps"], d["ds"], RULE_ROMBERG, F64,
                                  _ptr(phi), None, None)
    assert rc == _lib.SCFT_EINVAL
    assert b"scratch" in lib.scft_last_error()
