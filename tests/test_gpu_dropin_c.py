"""The drop-in boundary from C: tests/dropin_driver.c is compiled with gcc
against include/scft.h and linked with -lscft, the way the reference's own
1D_FEM.c driver would be (1D_FEM.c:289-370), and run on the MATLAB N=33 golden
problem (2049 implicit-Euler steps of 1/2048, trapezoid density, residual
f0 - phi).  Broyden through scft_broydn and through scft_nr_broydn (the exact
signature of broydn.c:44-46) must reach the reference broydn's converged field;
scft_nr_adm (the exact signature of adm.c:24-27) must lower the residual and
return its xnew vector, which the program frees as the reference frees its NR
vectors."""
import json
import os
import subprocess

import numpy as np
import pytest

from scft_gb300 import _lib

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")


def test_c_driver_runs_the_reference_solvers_through_libscft(tmp_path):
    lib_dir = os.path.dirname(_lib.LIB_PATH)
    exe = tmp_path / "dropin_driver"
    subprocess.run(["gcc", "-std=c11", "-O2", "-Wall", "-Werror", os.path.join(HERE, "dropin_driver.c"),
                    "-I", os.path.join(ROOT, "include"), "-L", lib_dir, "-lscft", f"-Wl,-rpath,{lib_dir}",
                    "-lm", "-o", str(exe)], check=True)
    g = json.load(open(os.path.join(GOLD, "matlab_N33.json")))
    s = json.load(open(os.path.join(GOLD, "broydn_scft.json")))
    n = len(g["x"])
    data = " ".join([str(n), repr(s["tol"])] + [repr(v) for v in g["x"]] + [repr(v) for v in g["f0"]]
                    + [repr(v) for v in s["w0"]])
    r = subprocess.run([str(exe)], input=data, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = {}
    for ln in r.stdout.splitlines():
        head, *vals = ln.split()
        kv = dict(t.split("=") for t in vals if "=" in t)
        rows[head] = (kv, np.array([float(t) for t in vals if "=" not in t]))
    w0 = np.array(s["w0"])
    for name in ("scft_broydn", "scft_nr_broydn"):
        kv, x = rows[name]
        assert kv["check"] == "0" and kv["rc"] == "0", (name, kv)
        assert float(kv["maxres"]) < s["tol"]
        np.testing.assert_allclose(x, s["x"], rtol=1e-6, atol=1e-8)
    kv, x = rows["scft_nr_adm"]
    assert kv["rc"] == "0"
    assert 0.0 <= float(kv["maxres"]) < float(rows["initial"][0]["maxres"])
    assert not np.allclose(x, w0)
    assert rows["scft_nr_adm_xnew"][0]["finite"] == "1"
