"""Generate the committed golden fixtures of tests/golden/ from the reference.

Run on a host that has the reference sources (where oracle/Makefile looks for
them: its REF, or ``SCFT_REFERENCE_DIR``) after ``make -C oracle ref``:

    python tests/golden/make_golden.py

It reads the reference's converged-field files as data and runs the reference's
own NR routines compiled from source (oracle/_ref) on small inputs, so that GPU
hosts without the reference can still check against reference outputs.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

REF = orc.reference_dir()
if REF is None:
    raise SystemExit("reference sources not found (set SCFT_REFERENCE_DIR)")


def dump(name, obj):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(obj, f, indent=1)
        f.write("\n")


def read_csv_field(path, skip):
    rows = []
    with open(path) as f:
        lines = f.read().splitlines()[skip:]
    for ln in lines:
        if "," in ln:
            parts = ln.split(",")
            rows.append((float(parts[1]), float(parts[2])))
    x = np.array([r[0] for r in rows])
    w = np.array([r[1] for r in rows])
    return x, w


def fixtures_fields(O):
    # 1. MATLAB prototype's converged field (row-scaled W, implicit Euler, 2049 steps
    #    of 1/2048, trapezoid; Matlab_files/simple_FEM_1D_transient.m)
    x, w = read_csv_field(os.path.join(REF, "Matlab_files/inputFiles/solution_matlab_N=33"), 1)
    tau, L = 0.5302, 3.72374
    f0 = O.f0_tanh2_ceil(x, tau, L)
    p = orc.OracleProblem(x, f0, 1.0 / 2048, 2049, rule=orc.RULE_TRAPEZOID, sign=-1)
    out, phi = O.residual(p, w[1:-1])
    dump("matlab_N33.json", {
        "source": "Matlab_files/inputFiles/solution_matlab_N=33 (x, w); f0 by set_f0_given.m",
        "tau": tau, "L": L, "nsteps": 2049, "ds": 1.0 / 2048, "rule": "trapezoid", "sign": -1,
        "x": x.tolist(), "w": w.tolist(), "f0": f0.tolist(),
        "oracle_phi": phi.tolist(), "oracle_max_residual": float(np.abs(out).max()),
    })
    # 2. deal.II converged field (consistent W, Gauss-Legendre IRK2, 2048 steps, Romberg)
    x, w = read_csv_field(os.path.join(REF, "DEALII_SCFT/inputFiles/N=33_for_read.txt"), 2)
    head = open(os.path.join(REF, "DEALII_SCFT/inputFiles/N=33_for_read.txt")).read().splitlines()[:2]
    tau, L = 5.30252230020752e-01, 3.72374357332160
    f0 = O.f0_tanh2_le(x, tau)
    p = orc.OracleProblem(x, f0, 1.0 / 2048, 2048, rule=orc.RULE_ROMBERG, wmode=orc.W_CONSISTENT,
                          scheme=orc.SCHEME_IRK2, sign=-1, wall_w=[w[0], w[-1]])
    out, phi = O.residual(p, w[1:-1])
    dump("dealii_N33.json", {
        "source": "DEALII_SCFT/inputFiles/N=33_for_read.txt",
        "header": head,
        "file_error": float(head[0].split("ERROR=")[1]),
        "file_free_energy": float(head[1].split(",")[1]),
        "tau": tau, "L": L, "nsteps": 2048, "ds": 1.0 / 2048,
        "x": x.tolist(), "w": w.tolist(), "f0": f0.tolist(),
        "oracle_phi": phi.tolist(), "oracle_max_residual": float(np.abs(out).max()),
    })
    # 3. Wang's .res: the phi column equals the tanh^2 target at its nodes
    lines = open(os.path.join(REF, "Exp_m32_n2048_IE.res")).read().splitlines()
    rows = [list(map(float, ln.split())) for ln in lines[9:] if ln.strip()]
    xl = np.array([r[0] for r in rows])
    phi_col = np.array([r[1] for r in rows])
    dump("res_m32.json", {
        "source": "Exp_m32_n2048_IE.res (x/l and phi columns, header l, t, mphi)",
        "l": 3.72374357332160, "t": 5.30252230020752e-01, "mphi": 8.92581217765433e-01,
        "x_over_l": xl.tolist(), "phi": phi_col.tolist(),
    })


def fixtures_routines(R):
    rng = np.random.default_rng(7)
    # romint (romint.c:21) on smooth and rough samples
    rom = []
    for m in (16, 64, 256):
        t = np.linspace(0.0, 1.0, m + 1)
        for f in (np.sin(3 * t) * np.exp(-t), rng.uniform(-1, 1, m + 1)):
            rom.append({"m": m, "hh": 1.0 / m, "f": f.tolist(), "ref": R.romint(f, m, 1.0 / m)})
    # gaussj, both variants (gaussj.c, DEALII_SCFT/src/gaussj.c)
    gj = []
    for n in (1, 3, 7, 10):
        a = rng.normal(size=(n, n))
        b = rng.normal(size=(n, 1))
        _, _, xr = R.gaussj(a, b, "root")
        rc, _, xd = R.gaussj(a, b, "dealii")
        gj.append({"a": a.tolist(), "b": b.ravel().tolist(), "x_root": xr.ravel().tolist(),
                   "x_dealii": xd.ravel().tolist(), "rc_dealii": rc})
    a = np.zeros((3, 3)); a[0, 0] = 1.0
    rc, _, _ = R.gaussj(a, np.ones((3, 1)), "dealii")
    gj.append({"a": a.tolist(), "b": [1.0, 1.0, 1.0], "rc_dealii": rc, "singular": True})

    # adm_chen on the 3-equation toy of Matlab_files/drive_adm_chen.m / DEALII_SCFT/test_ADM.c
    def toy3(v):
        x, y, z = v
        return np.array([x * y * z - 12.0, x * x + y * y - 8.0, x + y + z - 511.0])

    traj = []
    rc, xs, nc = R.adm_chen(toy3, [1.0, 2.0, 3.0], 1e-12, 50000, 0.99, 30, log=traj)
    admchen_toy = {"x0": [1.0, 2.0, 3.0], "tol": 1e-12, "maxit": 50000, "lmd": 0.99, "nn": 30,
                   "rc": rc, "x": xs.tolist(), "calls": nc,
                   "trajectory": [t.tolist() for t in traj[:40]]}

    # adm on the linear map of 1D_FEM.c:372-379 (fixed point (-4, 6))
    def myfun(v):
        return np.array([0.5 * v[0] - 2.0, 0.5 * v[1] + 3.0])

    traj = []
    rc, xa, nc, chk = R.adm(myfun, [0.3, -0.7], log=traj)
    adm_toy = {"x0": [0.3, -0.7], "rc": rc, "check": chk, "x": xa.tolist(), "calls": nc,
               "trajectory": [t.tolist() for t in traj]}

    # broydn on the 3-equation toy
    traj = []
    rc, xb, nc, chk = R.broydn(toy3, [1.0, 2.0, 3.0], 1e-10, log=traj)
    broydn_toy = {"x0": [1.0, 2.0, 3.0], "tol": 1e-10, "rc": rc, "check": chk, "x": xb.tolist(),
                  "calls": nc}
    dump("nr_routines.json", {"romint": rom, "gaussj": gj, "adm_chen_toy": admchen_toy,
                              "adm_toy": adm_toy, "broydn_toy": broydn_toy})


def fixtures_scft_mixing(O, R):
    """The reference adm_chen driving the oracle propagator on the MATLAB golden
    problem from a perturbed start: the first iterates of the reference solver."""
    g = json.load(open(os.path.join(HERE, "matlab_N33.json")))
    x, f0 = np.array(g["x"]), np.array(g["f0"])
    w = np.array(g["w"])
    p = orc.OracleProblem(x, f0, g["ds"], g["nsteps"], rule=orc.RULE_TRAPEZOID, sign=-1)
    w0 = w[1:-1] + 0.05 * np.sin(np.arange(1, len(w) - 1))
    traj, ys = [], []
    res_fn = lambda v: O.residual(p, v)[0]  # noqa: E731
    rc, xs, nc = R.adm_chen(res_fn, w0, 1e-7, 12, 0.9, 10, log=traj, ylog=ys)
    dump("admchen_scft.json", {
        "problem": "matlab_N33.json", "w0": w0.tolist(), "tol": 1e-7, "maxit": 12, "lmd": 0.9, "nn": 10,
        "rc": rc, "x_final": xs.tolist(), "trajectory": [t.tolist() for t in traj],
        "residuals": [y.tolist() for y in ys],
    })
    traj = []
    rc, xb, nc, chk = R.broydn(res_fn, w0, 1e-9, log=traj)
    dump("broydn_scft.json", {
        "problem": "matlab_N33.json", "w0": w0.tolist(), "tol": 1e-9, "rc": rc, "check": chk,
        "x": xb.tolist(), "calls": nc, "max_residual": float(np.abs(res_fn(xb)).max()),
    })


def fixtures_spline(R):
    """spline_chen (spline_chen.c:13-106) compiled from the reference: the field
    transfer of refine_mesh (scft.cc:162-163) on a bisected mesh, and random
    tables with every end condition, extrapolation included."""
    cases = []
    g = json.load(open(os.path.join(HERE, "dealii_N33.json")))
    x = np.array(g["x"]); w = np.array(g["w"])
    xn = np.empty(2 * len(x) - 1); xn[0::2] = x; xn[1::2] = 0.5 * (x[:-1] + x[1:])
    rc, yp = R.spline(x[1:-1], w[1:-1], xn[1:-1])
    cases.append({"name": "refine_mesh N=33 -> 65", "x": x[1:-1].tolist(), "y": w[1:-1].tolist(),
                  "xp": xn[1:-1].tolist(), "m": None, "rc": rc, "yp": yp.tolist()})
    rng = np.random.default_rng(7)
    for nx, m in ((4, None), (7, 0.0), (40, None), (40, -2.5), (129, None)):
        xs = np.sort(rng.uniform(0.0, 6.0, nx))
        ys = np.cos(xs) + 0.05 * rng.normal(size=nx)
        xp = np.concatenate([np.linspace(xs[0] - 0.5, xs[-1] + 0.5, 61), xs])
        rc, yp = R.spline(xs, ys, xp, m)
        cases.append({"name": f"random nx={nx} m={m}", "x": xs.tolist(), "y": ys.tolist(), "xp": xp.tolist(),
                      "m": m, "rc": rc, "yp": yp.tolist()})
    rc, _ = R.spline([0.0, 1.0, 2.0], [0.0, 1.0, 0.0], [0.5])
    cases.append({"name": "not-a-knot with 3 points", "x": [0.0, 1.0, 2.0], "y": [0.0, 1.0, 0.0], "xp": [0.5],
                  "m": None, "rc": rc, "yp": None})
    dump("spline.json", {"source": "DEALII_SCFT/src/spline_chen.c compiled from the reference", "cases": cases})


def main():
    orc.build(with_reference=True)
    O = orc.Oracle()
    R = orc.Reference()
    fixtures_fields(O)
    fixtures_routines(R)
    fixtures_scft_mixing(O, R)
    fixtures_spline(R)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
