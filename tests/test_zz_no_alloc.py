"""scft_density_noalloc, the entry point that allocates no device memory.

It exists for callers that may not allocate GPU memory -- applications whose
device memory belongs to another allocator with a fixed budget, and tight
per-iteration loops that cannot afford cudaMalloc/cudaFree, which can block on
or synchronize the whole device.  The caller hands in device buffers and the
propagator keeps its half-contour store in one fixed device array of the
library.  These tests call it through the C ABI:

* twice in a row per precision (two different instances, so the second call
  runs over the first call's leftover scratch), each result against the
  allocating entry point, scft_batch_evaluate, with the tolerances of the other
  parity tests (1e-10 relative in FP64, 1e-5 in FP32), the status word included;
  the library's own allocation counters must not move during either call;
* on shapes whose propagator runs as a thread-block cluster, in FP32 and FP64;
* on a field that breaks diagonal dominance: the status bit must come back;
* with an instance larger than the fixed scratch, and with host memory in place
  of a device buffer: both refused with SCFT_EINVAL before any launch.

This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from scft_gb300 import F32, F64, RULE_ROMBERG, RULE_TRAPEZOID, _lib, api, workloads as W

pytestmark = pytest.mark.gpu

TOL = {F64: 1e-10, F32: 1e-5}


def _ptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def _iptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_int))


def _counters(lib):
    req, cuda = C.c_longlong(), C.c_longlong()
    lib.scft_mem_counters(C.byref(req), C.byref(cuda))
    return req.value, cuda.value


def _reference(insts, prec):
    """Density, Q and status of the instances from the allocating entry point."""
    with api.Batch(insts) as b:
        b.evaluate(prec)
        _, phi, Q = b.get()
        st = b.status()
    return phi, Q, st


def _call(lib, torch, d, prec):
    """One scft_density_noalloc call on fresh device buffers (NaN-filled outputs);
    returns (rc, phi, Q, status, allocation counters before, after)."""
    n = d["n_nodes"]
    x = torch.tensor(d["x"], dtype=torch.float64, device="cuda")
    w = torch.tensor(d["w0"], dtype=torch.float64, device="cuda")
    phi = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    Q = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    before = _counters(lib)
    rc = lib.scft_density_noalloc(n, _ptr(x), _ptr(w), d["nsteps"], d["ds"], d.get("rule", RULE_ROMBERG), prec,
                                  _ptr(phi), _ptr(Q), _iptr(st), stream)
    torch.cuda.synchronize()
    after = _counters(lib)
    return rc, phi.cpu().numpy(), Q.cpu().item(), int(st.cpu().item()), before, after


def _check(lib, torch, insts, prec):
    phi_ref, Q_ref, st_ref = _reference(insts, prec)
    for call, d in enumerate(insts):
        rc, phi, Q, st, before, after = _call(lib, torch, d, prec)
        assert rc == 0, lib.scft_last_error().decode()
        assert after == before, f"call {call} allocated through the library"
        ref = phi_ref[call]
        assert np.max(np.abs(phi - ref)) <= TOL[prec] * np.max(np.abs(ref)), (prec, call)
        assert abs(Q - Q_ref[call]) <= TOL[prec] * abs(Q_ref[call]), (prec, call)
        assert st == (int(st_ref[call]) & 3), (prec, call, st, st_ref[call])


def test_noalloc_matches_the_allocating_entry_point_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    a = W.instance(300, 6.0, 1024, seed=5, inst=0)
    b = W.instance(120, 3.5, 2049, seed=5, inst=1, rule=RULE_TRAPEZOID)
    b["ds"] = 1.0 / 2048
    for prec in (F64, F32):
        _check(lib, torch, [a, b], prec)


def test_noalloc_cluster_shape():
    """Above 2048 interior unknowns in FP32 (1024 in FP64) the propagator of one
    instance spans a cluster of CTAs.  3000 nodes in FP32 (8 x 16 warps x 32)
    and 1800 nodes in FP64 (4 x 16 x 32), 2048 steps: each needs about 17 MB of
    the fixed scratch."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    for prec, m_elem in ((F32, 2999), (F64, 1799)):
        d = W.instance(m_elem, 8.0, 2048, seed=9, inst=0)
        _check(lib, torch, [d, d], prec)


def test_noalloc_reports_lost_dominance():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d = W.instance(40, 4.0, 64, seed=0, inst=0)
    w = np.full(41, -200.0)
    w[0] = w[-1] = 0.0
    d = dict(d, w0=w)
    for prec in (F64, F32):
        rc, _, _, st, _, _ = _call(lib, torch, d, prec)
        assert rc == 0, lib.scft_last_error().decode()
        assert st & _lib.ST_NOT_DOMINANT
        # the next call on a sound field starts from a cleared status
        rc, _, _, st, _, _ = _call(lib, torch, W.instance(40, 4.0, 64, seed=0, inst=0), prec)
        assert rc == 0 and st == 0


def test_noalloc_refuses_an_instance_larger_than_its_scratch():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d = W.instance(8192, 7.0, 8192, seed=1, inst=0, graded=1.002)
    x = torch.tensor(d["x"], dtype=torch.float64, device="cuda")
    phi = torch.empty(d["n_nodes"], dtype=torch.float64, device="cuda")
    rc = lib.scft_density_noalloc(d["n_nodes"], _ptr(x), _ptr(x), d["nsteps"], d["ds"], RULE_ROMBERG, F64,
                                  _ptr(phi), None, None, None)
    assert rc == _lib.SCFT_EINVAL
    assert b"scratch" in lib.scft_last_error()


def test_noalloc_refuses_host_memory():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    d = W.instance(64, 4.0, 256, seed=2, inst=0)
    x = torch.tensor(d["x"], dtype=torch.float64, device="cuda")
    w_host = np.ascontiguousarray(d["w0"])
    phi = torch.empty(d["n_nodes"], dtype=torch.float64, device="cuda")
    rc = lib.scft_density_noalloc(d["n_nodes"], _ptr(x), w_host.ctypes.data_as(C.POINTER(C.c_double)),
                                  d["nsteps"], d["ds"], RULE_ROMBERG, F64, _ptr(phi), None, None, None)
    assert rc == _lib.SCFT_EINVAL
    assert b"device memory" in lib.scft_last_error()
