"""The C ABI library: it loads, exports every entry point include/scft.h
declares, and the ctypes mirror has the compiler's struct layout.  No compute
call is made here (these run without a GPU)."""
import os
import re
import subprocess

import pytest

from scft_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "scft.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(scft_[a-z0-9_]+)\s*\(", src)
    return sorted(set(n for n in names if not n.startswith("scft_vecfunc")))


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_exports_are_plain_c(tmp_path):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True)
    exported = {ln.split()[-1] for ln in out.stdout.splitlines() if " T " in ln}
    for n in declared_functions():
        assert n in exported, n


def test_struct_layouts_match_ctypes(tmp_path):
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_layout.c"), "-o", str(exe)], check=True)
    got = dict(ln.rsplit(" ", 1) for ln in subprocess.run([str(exe)], capture_output=True,
                                                          text=True, check=True).stdout.splitlines())
    import ctypes as C
    for cname, ct in [("scft_config", _lib.ScftConfig), ("scft_instance", _lib.ScftInstance),
                      ("scft_solve_opts", _lib.ScftSolveOpts), ("scft_result", _lib.ScftResult)]:
        assert int(got[cname]) == C.sizeof(ct), cname
        for fname, _ in ct._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(ct, fname).offset, (cname, fname)


def test_strerror_and_defaults_without_device():
    lib = _lib.load()
    assert lib.scft_strerror(_lib.SCFT_ENODEV) == b"no CUDA device"
    from scft_gb300 import api
    o = api.solve_opts()
    assert o.depth == 10 and o.beta == pytest.approx(1.0) and o.fused == 1 and o.precision == _lib.F32
    # forked paths off by default, with the bench's settings ready; graded-mesh step above ratio 16
    assert o.forks == 0 and o.fork_at == 42 and o.fork_grace == 6 and o.fork_first == 1
    assert o.fork_err == pytest.approx(1e-5) and list(o.fork_scale)[:3] == pytest.approx([0.9, 0.8, 0.6])
    assert o.graded_ratio == pytest.approx(16.0) and o.precond_hfloor == pytest.approx(0.1)
    # FP32 iterations stop at 0.65 tol; the staged solve is off
    assert o.tol32_factor == pytest.approx(0.65) and o.transfer_stride == 0
    import ctypes as C
    c = _lib.ScftConfig()
    lib.scft_config_init(C.byref(c))
    assert c.nsteps == 2049 and c.ds == pytest.approx(1 / 2048) and c.rule == _lib.RULE_TRAPEZOID
