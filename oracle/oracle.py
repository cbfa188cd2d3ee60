"""ctypes bridge to the checker libraries (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this module.
It loads

* ``_build/liboracle.so`` -- the C restatement of the reference's method
  (scft_oracle.c), and
* ``_ref/libscft_ref_{dealii,root}.so`` -- the reference's own NR routines
  compiled from source by the Makefile (present only where the reference
  sources were available at build time).

Nothing in the product package imports this file.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUILD_DIR = os.path.join(HERE, "_build")

RULE_ROMBERG, RULE_TRAPEZOID = 0, 1
W_ROWSCALED, W_CONSISTENT = 0, 1
SCHEME_IE, SCHEME_IRK2 = 0, 1

_dp = C.POINTER(C.c_double)
VECFUNC = C.CFUNCTYPE(None, C.c_int, _dp, _dp, C.c_void_p)
REF_VECFUNC = C.CFUNCTYPE(None, C.c_int, _dp, _dp)


def reference_dir() -> str | None:
    """Directory of the reference sources that the recipe (oracle/Makefile,
    variable REF; SCFT_REFERENCE_DIR overrides it) compiles, or None when that
    directory does not exist on this host."""
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                       capture_output=True, text=True)
    d = r.stdout.strip()
    return d if r.returncode == 0 and d and os.path.isdir(d) else None


def build(with_reference: bool | None = None) -> None:
    """Compile the restatement (always) and the reference routines (when the
    reference sources are present)."""
    targets = ["oracle"]
    if with_reference is None:
        with_reference = reference_dir() is not None
    if with_reference:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


class Problem(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("x", _dp),
        ("f0", _dp),
        ("ds", C.c_double),
        ("nsteps", C.c_int),
        ("rule", C.c_int),
        ("wmode", C.c_int),
        ("scheme", C.c_int),
        ("sign", C.c_int),
        ("wall_w", _dp),
    ]


class MixOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("beta", C.c_double), ("clip", C.c_double), ("grow", C.c_double),
                ("reg", C.c_double), ("precond", C.c_double), ("maxit", C.c_int), ("depth", C.c_int),
                ("mode", C.c_int), ("schedule", C.c_int), ("cap", C.c_double), ("floor", C.c_double),
                ("weighted", C.c_int), ("graded_ratio", C.c_double), ("hfloor", C.c_double)]


# the batched GPU solver's defaults (scft_solve_opts_init)
MIX_DEFAULTS = dict(tol=1e-6, beta=1.0, clip=1.0, grow=10.0, reg=1e-12, precond=0.6, maxit=2000,
                    depth=10, mode=1, schedule=0, cap=0.25, floor=0.5, weighted=1, graded_ratio=16.0, hfloor=0.1)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class OracleProblem:
    """One SCFT instance for the oracle: mesh, target and discretisation."""

    def __init__(self, x, f0, ds, nsteps, rule=RULE_ROMBERG, wmode=W_ROWSCALED,
                 scheme=SCHEME_IE, sign=1, wall_w=None):
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.f0 = np.ascontiguousarray(f0, dtype=np.float64)
        self.wall = None if wall_w is None else np.ascontiguousarray(wall_w, dtype=np.float64)
        self.c = Problem(len(self.x), _ptr(self.x), _ptr(self.f0), float(ds), int(nsteps),
                         int(rule), int(wmode), int(scheme), int(sign),
                         _ptr(self.wall) if self.wall is not None else None)

    @property
    def n(self):
        return len(self.x)


class Oracle:
    def __init__(self, path: str | None = None):
        path = path or os.path.join(BUILD_DIR, "liboracle.so")
        if not os.path.exists(path):
            build(with_reference=False)
        L = C.CDLL(path)
        self.L = L
        L.or_romint.restype = C.c_double
        L.or_romint.argtypes = [_dp, C.c_int, C.c_double]
        L.or_quad_weights.argtypes = [C.c_int, C.c_double, C.c_int, _dp]
        L.or_propagate.argtypes = [C.POINTER(Problem), _dp, _dp, _dp, _dp]
        L.or_residual.argtypes = [C.POINTER(Problem), _dp, _dp, _dp]
        L.or_gaussj.argtypes = [_dp, C.c_int, _dp, C.c_int, C.c_int]
        L.or_adm_chen.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_double, C.c_int, C.c_int,
                                  C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int), _dp]
        L.or_adm.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_int, C.c_double, C.c_int,
                             C.POINTER(C.c_int)]
        L.or_broydn.argtypes = [C.c_void_p, C.c_void_p, _dp, C.c_int, C.c_double,
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_mesh_graded.argtypes = [C.c_int, C.c_double, C.c_double, _dp]
        L.or_mesh_uniform.argtypes = [C.c_int, C.c_double, _dp]
        L.or_f0_tanh2_ceil.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        L.or_f0_tanh2_le.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.or_spline.argtypes = [_dp, _dp, C.c_int, _dp, _dp, C.c_int, _dp]
        L.or_f0_gauss_wall.argtypes = [C.c_int, _dp, C.c_double, C.c_double, _dp]
        L.or_anderson_solve.argtypes = [C.POINTER(Problem), _dp, C.POINTER(MixOpts),
                                        C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.or_anderson_solve_batch.argtypes = [C.POINTER(Problem), C.c_int, _dp, C.POINTER(MixOpts), C.c_int,
                                              C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]
        self.problem_vecfunc = C.cast(L.or_problem_vecfunc, C.c_void_p)

    # -- meshes / targets
    def mesh_uniform(self, n, L):
        x = np.empty(n)
        self.L.or_mesh_uniform(n, L, _ptr(x))
        return x

    def mesh_graded(self, m_elem, ratio, L):
        x = np.empty(m_elem + 1)
        if self.L.or_mesh_graded(m_elem, ratio, L, _ptr(x)):
            raise ValueError("graded mesh needs an even element count")
        return x

    def f0_tanh2_ceil(self, x, tau, L):
        f = np.empty(len(x)); x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.or_f0_tanh2_ceil(len(x), _ptr(x), tau, L, _ptr(f))
        return f

    def spline(self, x, y, xp, m=None):
        """spline_chen.c:13-106 restated: (rc, yp)."""
        x, y, xp = (np.ascontiguousarray(v, dtype=np.float64) for v in (x, y, xp))
        yp = np.empty(len(xp))
        mm = None if m is None else np.array([m], dtype=np.float64)
        rc = self.L.or_spline(_ptr(x), _ptr(y), len(x), _ptr(xp), _ptr(yp), len(xp), None if mm is None else _ptr(mm))
        return rc, yp

    def f0_tanh2_le(self, x, tau):
        f = np.empty(len(x)); x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.or_f0_tanh2_le(len(x), _ptr(x), tau, _ptr(f))
        return f

    def f0_gauss_wall(self, x, L, width=0.25):
        f = np.empty(len(x)); x = np.ascontiguousarray(x, dtype=np.float64)
        self.L.or_f0_gauss_wall(len(x), _ptr(x), L, width, _ptr(f))
        return f

    # -- quadrature
    def romint(self, f, m, hh):
        f = np.ascontiguousarray(f, dtype=np.float64)
        return self.L.or_romint(_ptr(f), m, hh)

    def free_energy(self, x, w, f0_samples):
        """Mean-field free energy reported by DEALII_SCFT/src/scft.cc:404-450:
        F = (<w f0> / <f0> + ln <f0>) / (-1000), <.> the Romberg average
        (romint.c:21-57) over m+1 uniform samples of [x_0, x_L], w the
        piecewise-linear field of the mesh."""
        x = np.asarray(x, dtype=np.float64)
        fs = np.ascontiguousarray(f0_samples, dtype=np.float64)
        m = len(fs) - 1
        xs = x[0] + ((x[-1] - x[0]) * np.arange(m + 1, dtype=np.float64)) / m
        wq = np.interp(xs, x, np.asarray(w, dtype=np.float64))
        a = self.romint(wq * fs, m, 1.0 / m)
        b = self.romint(fs, m, 1.0 / m)
        return (a / b + np.log(b)) / -1000.0

    def quad_weights(self, nsteps, ds, rule):
        W = np.empty(nsteps + 1)
        if self.L.or_quad_weights(nsteps, ds, rule, _ptr(W)):
            raise ValueError("Romberg needs a power-of-two step count >= 16")
        return W

    # -- propagator
    def propagate(self, prob: OracleProblem, w_full, want_q=False):
        w = np.ascontiguousarray(w_full, dtype=np.float64)
        phi = np.empty(prob.n)
        Q = C.c_double()
        q = np.empty((prob.c.nsteps + 1, prob.n)) if want_q else None
        rc = self.L.or_propagate(C.byref(prob.c), _ptr(w), _ptr(phi), C.byref(Q),
                                 _ptr(q) if want_q else None)
        if rc:
            raise RuntimeError(f"or_propagate failed: {rc}")
        return (phi, Q.value, q) if want_q else (phi, Q.value)

    def residual(self, prob: OracleProblem, w_int):
        w = np.ascontiguousarray(w_int, dtype=np.float64)
        out = np.empty(prob.n - 2)
        phi = np.empty(prob.n)
        rc = self.L.or_residual(C.byref(prob.c), _ptr(w), _ptr(out), _ptr(phi))
        if rc:
            raise RuntimeError(f"or_residual failed: {rc}")
        return out, phi

    # -- dense algebra / solvers
    def gaussj(self, a, b, singular_mode=0):
        a = np.array(a, dtype=np.float64, order="C")
        b = np.array(b, dtype=np.float64, order="C").reshape(a.shape[0], -1)
        rc = self.L.or_gaussj(_ptr(a), a.shape[0], _ptr(b), b.shape[1], singular_mode)
        return rc, a, b

    def _wrap(self, f):
        if isinstance(f, OracleProblem):
            return self.problem_vecfunc, C.cast(C.pointer(f.c), C.c_void_p), None

        def cb(n, xp, op, _ctx):
            x = np.ctypeslib.as_array(xp, shape=(n,)).copy()
            np.ctypeslib.as_array(op, shape=(n,))[:] = f(x)

        c = VECFUNC(cb)
        return C.cast(c, C.c_void_p), None, c

    def adm_chen(self, f, x0, tol, maxit, lmd, nn, final=False):
        fp, ctx, keep = self._wrap(f)
        x = np.array(x0, dtype=np.float64)
        it = C.c_int()
        trace = np.full(maxit + 2, np.nan)
        rc = self.L.or_adm_chen(fp, ctx, _ptr(x), tol, maxit, len(x), lmd, nn, int(final),
                                C.byref(it), _ptr(trace))
        del keep
        return rc, x, it.value, trace[: it.value + 1]

    def adm(self, g, x0, tol, maxit):
        fp, ctx, keep = self._wrap(g)
        x = np.array(x0, dtype=np.float64)
        it = C.c_int()
        rc = self.L.or_adm(fp, ctx, _ptr(x), len(x), tol, maxit, C.byref(it))
        del keep
        return rc, x, it.value

    def broydn(self, f, x0, tol):
        fp, ctx, keep = self._wrap(f)
        x = np.array(x0, dtype=np.float64)
        it, nfev = C.c_int(), C.c_int()
        rc = self.L.or_broydn(fp, ctx, _ptr(x), len(x), tol, C.byref(it), C.byref(nfev))
        del keep
        return rc, x, it.value, nfev.value


    def anderson_solve(self, prob: OracleProblem, w_full, **kw):
        """CPU restatement of the batched GPU solver (safeguarded Anderson)."""
        o = dict(MIX_DEFAULTS)
        o.update(kw)
        mo = MixOpts(**o)
        w = np.array(w_full, dtype=np.float64)
        it, err = C.c_int(), C.c_double()
        rc = self.L.or_anderson_solve(C.byref(prob.c), _ptr(w), C.byref(mo), C.byref(it), C.byref(err))
        return rc, w, it.value, err.value


def cpu_solve_batch(instances, workers=None, **kw):
    """Solve instances on the host cores with the oracle: or_anderson_solve on
    `workers` threads of the C batch driver (each takes the next unsolved
    instance).  Returns (list of (rc, iters, err), seconds, workers)."""
    import time

    workers = workers or os.cpu_count() or 1
    O = Oracle()
    probs = [OracleProblem(d["x"], d["f0"], d["ds"], d["nsteps"], rule=d.get("rule", RULE_ROMBERG))
             for d in instances]
    arr = (Problem * len(probs))(*[p.c for p in probs])
    w = np.ascontiguousarray(np.concatenate([np.asarray(d["w0"], dtype=np.float64) for d in instances]))
    o = dict(MIX_DEFAULTS)
    o.update(kw)
    mo = MixOpts(**o)
    k = len(instances)
    rc, it, err = (C.c_int * k)(), (C.c_int * k)(), (C.c_double * k)()
    t0 = time.perf_counter()
    if O.L.or_anderson_solve_batch(arr, k, _ptr(w), C.byref(mo), int(workers), rc, it, err) != 0:
        raise RuntimeError("or_anderson_solve_batch: could not start its threads")
    dt = time.perf_counter() - t0
    return [(rc[i], it[i], err[i]) for i in range(k)], dt, min(workers, k)


class Reference:
    """The reference's own NR routines compiled from source (oracle/_ref)."""

    def __init__(self):
        d = os.path.join(REF_DIR, "libscft_ref_dealii.so")
        r = os.path.join(REF_DIR, "libscft_ref_root.so")
        if not (os.path.exists(d) and os.path.exists(r)):
            raise FileNotFoundError("reference routines not built (oracle/_ref)")
        self.D = C.CDLL(d)
        self.R = C.CDLL(r)
        self.D.ref_romint.restype = C.c_double
        self.D.ref_romint.argtypes = [_dp, C.c_int, C.c_double]
        self.D.ref_adm_chen.argtypes = [REF_VECFUNC, _dp, C.c_double, C.c_int, C.c_int,
                                        C.c_double, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(C.c_int)]
        self.D.ref_broydn.argtypes = [REF_VECFUNC, _dp, C.c_int, C.c_double, C.c_int,
                                      C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self.D.ref_gaussj_dealii.argtypes = [_dp, C.c_int, _dp, C.c_int]
        self.R.ref_adm.argtypes = [REF_VECFUNC, _dp, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]
        self.R.ref_gaussj_root.argtypes = [_dp, C.c_int, _dp, C.c_int]
        self.D.ref_spline_chen.argtypes = [_dp, _dp, _dp, _dp, C.c_int, C.c_int, _dp]

    @staticmethod
    def available() -> bool:
        return os.path.exists(os.path.join(REF_DIR, "libscft_ref_dealii.so"))

    def romint(self, f, m, hh):
        f = np.ascontiguousarray(f, dtype=np.float64)
        return self.D.ref_romint(_ptr(f), m, hh)

    def spline(self, x, y, xp, m=None):
        """The reference's spline_chen itself: (rc, yp)."""
        x, y, xp = (np.array(v, dtype=np.float64) for v in (x, y, xp))
        yp = np.empty(len(xp))
        mm = None if m is None else np.array([m], dtype=np.float64)
        rc = self.D.ref_spline_chen(_ptr(x), _ptr(y), _ptr(xp), _ptr(yp), len(x), len(xp),
                                    None if mm is None else _ptr(mm))
        return rc, yp

    def gaussj(self, a, b, variant="dealii"):
        a = np.array(a, dtype=np.float64, order="C")
        b = np.array(b, dtype=np.float64, order="C").reshape(a.shape[0], -1)
        if variant == "dealii":
            rc = self.D.ref_gaussj_dealii(_ptr(a), a.shape[0], _ptr(b), b.shape[1])
        else:
            self.R.ref_gaussj_root(_ptr(a), a.shape[0], _ptr(b), b.shape[1])
            rc = 0
        return rc, a, b

    @staticmethod
    def _cb(f, base, log, ylog=None):
        """Reference callbacks get raw NR pointers; base is the first index."""

        def cb(n, xp, op):
            x = np.ctypeslib.as_array(xp, shape=(n + base,))[base:].copy()
            if log is not None:
                log.append(x.copy())
            y = np.asarray(f(x), dtype=np.float64)
            if ylog is not None:
                ylog.append(y.copy())
            np.ctypeslib.as_array(op, shape=(n + base,))[base:] = y

        return REF_VECFUNC(cb)

    def adm_chen(self, f, x0, tol, maxit, lmd, nn, final=False, max_calls=0, log=None, ylog=None):
        x = np.array(x0, dtype=np.float64)
        cb = self._cb(f, 0, log, ylog)
        nc = C.c_int()
        rc = self.D.ref_adm_chen(cb, _ptr(x), tol, maxit, len(x), lmd, nn, int(final),
                                 max_calls, C.byref(nc))
        return rc, x, nc.value

    def adm(self, g, x0, max_calls=0, log=None):
        x1 = np.concatenate([[0.0], np.asarray(x0, dtype=np.float64)])
        cb = self._cb(g, 1, log)
        nc, check = C.c_int(), C.c_int(1)
        rc = self.R.ref_adm(cb, _ptr(x1), len(x1) - 1, 1, max_calls, C.byref(nc), C.byref(check))
        return rc, x1[1:], nc.value, check.value

    def broydn(self, f, x0, tol, max_calls=0, log=None):
        x1 = np.concatenate([[0.0], np.asarray(x0, dtype=np.float64)])
        cb = self._cb(f, 1, log)
        nc, check = C.c_int(), C.c_int(1)
        rc = self.D.ref_broydn(cb, _ptr(x1), len(x1) - 1, tol, max_calls, C.byref(nc),
                               C.byref(check))
        return rc, x1[1:], nc.value, check.value
