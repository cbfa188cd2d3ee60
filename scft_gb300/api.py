"""Host-side mirror of the reference's SCFT interface, over the C ABI.

* ``simple_FEM_1D_transient(N, w, out)``  -- 1D_FEM.c:47 (1-based arrays)
* ``adm(x, n, f, flag)``                   -- adm.c:24
* ``adm_chen(f, x, tol, maxit, n, lmd, nn, final)`` -- ADM_chen_C.c:18
* ``broydn(x, n, f, tol)``                 -- broydn.c:44 (tolerance = the global err)
* ``Batch``                                -- thousands of instances per launch

The callbacks the solvers accept are either Python callables ``f(x) -> out``
(0-based numpy arrays) or one of the library's own evaluators
(``FEM_RESIDUAL``, ``FEM_RESIDUAL0``, ``FEM_FIXEDPOINT``), which keep every
evaluation on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import check


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Native:
    """Marker for the library's own C callbacks."""

    def __init__(self, name: str, base: int):
        self.name = name
        self.base = base

    def pointer(self):
        return C.cast(getattr(L.load(), self.name), C.c_void_p)


FEM_RESIDUAL = _Native("scft_fem_residual_vf", 1)     # 1-based, broydn / adm(flag=1) form
FEM_RESIDUAL0 = _Native("scft_fem_residual0_vf", 0)   # 0-based, adm_chen form
FEM_FIXEDPOINT = _Native("scft_fem_fixedpoint_vf", 1) # x + (phi - f0), adm form


def _callback(f, base: int):
    """Return (void* function pointer, keep-alive) for a solver callback."""
    if isinstance(f, _Native):
        return f.pointer(), None

    def cb(n, xp, op):
        x = np.ctypeslib.as_array(xp, shape=(n + base,))[base:].copy()
        np.ctypeslib.as_array(op, shape=(n + base,))[base:] = np.asarray(f(x), dtype=np.float64)

    c = L.VECFUNC(cb)
    return C.cast(c, C.c_void_p), c


# ---------------------------------------------------------------------------
# drop-in single instance
# ---------------------------------------------------------------------------
_config_keep: list = []


def set_config(f0, L_width=None, x=None, nsteps=2049, ds=1.0 / 2048, rule=L.RULE_TRAPEZOID, sign=1,
               precision=L.F64, scheme=L.SCHEME_IE, wmode=L.W_ROWSCALED, w_wall=(0.0, 0.0)):
    """Configure the problem that simple_FEM_1D_transient evaluates (the reference's
    globals f0_given, L and total_time_step).  scheme=SCHEME_IRK2 with
    wmode=W_CONSISTENT and the field's wall values selects the deal.II
    propagator (drivescft.cc:130-165, scft.cc:653-655)."""
    lib = L.load()
    f0 = np.ascontiguousarray(f0, dtype=np.float64)
    xa = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
    cfg = L.ScftConfig()
    lib.scft_config_init(C.byref(cfg))
    cfg.n_nodes = len(f0)
    cfg.x = _dp(xa)
    cfg.L = float(L_width if L_width is not None else (xa[-1] - xa[0]))
    cfg.f0 = _dp(f0)
    cfg.nsteps = int(nsteps)
    cfg.ds = float(ds)
    cfg.rule = int(rule)
    cfg.sign = int(sign)
    cfg.precision = int(precision)
    cfg.scheme = int(scheme)
    cfg.wmode = int(wmode)
    cfg.w_wall[0], cfg.w_wall[1] = float(w_wall[0]), float(w_wall[1])
    check(lib.scft_set_config(C.byref(cfg)), "scft_set_config")
    _config_keep[:] = [f0, xa]


def simple_FEM_1D_transient(N: int, w: np.ndarray, out: np.ndarray) -> int:
    """Drop-in for simple_FEM_1D_transient(int N, double* w, double* out)
    (1D_FEM.c:47-287): N interior nodes, w[1..N] read, out[1..N] written."""
    lib = L.load()
    if len(w) < N + 1 or len(out) < N + 1:
        raise ValueError("1-based arrays need N+1 entries")
    return check(lib.scft_fem_residual(int(N), _dp(w), _dp(out)), "simple_FEM_1D_transient")


def fem_residual(w_interior: np.ndarray) -> np.ndarray:
    """0-based convenience form of the drop-in residual."""
    w = np.concatenate([[0.0], np.asarray(w_interior, dtype=np.float64)])
    out = np.zeros_like(w)
    simple_FEM_1D_transient(len(w) - 1, w, out)
    return out[1:]


def density(w_nodes: np.ndarray):
    lib = L.load()
    w = np.ascontiguousarray(w_nodes, dtype=np.float64)
    phi = np.empty_like(w)
    Q = C.c_double()
    check(lib.scft_density(_dp(w), _dp(phi), C.byref(Q)), "scft_density")
    return phi, Q.value


# ---------------------------------------------------------------------------
# the reference's field files
# ---------------------------------------------------------------------------
def read_field(path: str, max_nodes: int = 1 << 20):
    """Field file of scft.cc:317-333 / read_yita_middle_1D (scft_util.cc:14-41),
    MATLAB inputs included.  Returns dict(x, w, err, free_energy); absent header
    values are NaN."""
    lib = L.load()
    n = C.c_int()
    err, F = C.c_double(), C.c_double()
    rc = lib.scft_field_read(path.encode(), 0, C.byref(n), None, None, None, None)
    if rc != 0 and n.value <= 0:
        check(rc, "scft_field_read")
    x = np.empty(n.value)
    w = np.empty(n.value)
    check(lib.scft_field_read(path.encode(), min(n.value, max_nodes), C.byref(n), _dp(x), _dp(w), C.byref(err),
                              C.byref(F)), "scft_field_read")
    return {"x": x, "w": w, "err": err.value, "free_energy": F.value}


def write_field(path: str, x, w, err: float, free_energy: float):
    """Write a field file read_yita_middle_1D reads back (scft.cc:317-333 formats)."""
    xa = np.ascontiguousarray(x, dtype=np.float64)
    wa = np.ascontiguousarray(w, dtype=np.float64)
    if xa.shape != wa.shape:
        raise ValueError("x and w differ in length")
    check(L.load().scft_field_write(path.encode(), len(xa), _dp(xa), _dp(wa), float(err), float(free_energy)),
          "scft_field_write")


def read_res(path: str, max_rows: int = 1 << 20):
    """.res table (the starting field of 1D_FEM.c:321-342): columns x/l, phi, eta,
    phie, phij for every node, and the header values."""
    lib = L.load()
    rows, m, ns = C.c_int(), C.c_int(), C.c_int()
    hdr = np.empty(6)
    table = np.empty((max_rows, 5))
    check(lib.scft_res_read(path.encode(), max_rows, C.byref(rows), _dp(table), C.byref(m), C.byref(ns), _dp(hdr)),
          "scft_res_read")
    t = table[:rows.value]
    out = {k: t[:, i].copy() for i, k in enumerate(("x_over_l", "phi", "eta", "phie", "phij"))}
    out.update(m=m.value, nsteps=ns.value, **dict(zip(("l", "mphi", "t", "Z", "f", "fmax"), hdr)))
    return out


# ---------------------------------------------------------------------------
# mesh refinement and field transfer (refine_mesh of the deal.II driver)
# ---------------------------------------------------------------------------
def refine_bisect(x):
    """Every element of the mesh cut in two (scft.cc:132-166)."""
    xa = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(2 * len(xa) - 1)
    check(L.load().scft_refine_bisect(len(xa), _dp(xa), _dp(out)), "scft_refine_bisect")
    return out


def spline(tables, m=None):
    """Cubic splines on the GPU: tables is a sequence of (x, y, xp); returns
    the list of yp (spline_chen.c:13-106; m None = not-a-knot ends)."""
    nx = (C.c_int * len(tables))(*[len(t[0]) for t in tables])
    npt = (C.c_int * len(tables))(*[len(t[2]) for t in tables])
    x = np.ascontiguousarray(np.concatenate([np.asarray(t[0], dtype=np.float64) for t in tables]))
    y = np.ascontiguousarray(np.concatenate([np.asarray(t[1], dtype=np.float64) for t in tables]))
    xp = np.ascontiguousarray(np.concatenate([np.asarray(t[2], dtype=np.float64) for t in tables]))
    yp = np.empty(len(xp))
    mm = None if m is None else np.array([m], dtype=np.float64)
    check(L.load().scft_spline(len(tables), nx, _dp(x), _dp(y), npt, _dp(xp), _dp(yp), _dp(mm)), "scft_spline")
    off = np.concatenate([[0], np.cumsum([len(t[2]) for t in tables])])
    return [yp[off[i]:off[i + 1]] for i in range(len(tables))]


def transfer_field(x, w, x_new):
    """refine_mesh's transfer of a nodal field to a new mesh: the interior values
    through the not-a-knot spline of the interior table, the wall values kept."""
    x, w, x_new = (np.asarray(v, dtype=np.float64) for v in (x, w, x_new))
    out = np.empty(len(x_new))
    out[1:-1] = spline([(x[1:-1], w[1:-1], x_new[1:-1])])[0]
    out[0], out[-1] = w[0], w[-1]
    return out


# ---------------------------------------------------------------------------
# solvers
# ---------------------------------------------------------------------------
def adm(x, n, f, flag=0, maxit=1000000):
    """adm.c:24: Anderson mixing for x = f(x).  Returns (x, check)."""
    lib = L.load()
    xx = np.ascontiguousarray(np.concatenate([[0.0] * flag, np.asarray(x, dtype=np.float64)]))
    fp, keep = _callback(f, flag)
    chk = C.c_int(1)
    lib.scft_adm_set_maxit(int(maxit))
    check(lib.scft_adm(_dp(xx), int(n), C.byref(chk), fp, int(flag)), "scft_adm")
    del keep
    return xx[flag:], chk.value


def adm_chen(f, x, tol, maxit, n, lmd, nn, final=False):
    """ADM_chen_C.c:18: Anderson mixing for F(x) = 0.  Returns (status, x)."""
    lib = L.load()
    xx = np.ascontiguousarray(np.asarray(x, dtype=np.float64).copy())
    fp, keep = _callback(f, 0)
    rc = check(lib.scft_adm_chen(fp, _dp(xx), float(tol), int(maxit), int(n), float(lmd), int(nn),
                                 int(bool(final))), "scft_adm_chen")
    del keep
    return rc, xx


def broydn(x, n, f, tol):
    """broydn.c:44 with the global err = tol.  Returns (x, check, err)."""
    lib = L.load()
    xx = np.ascontiguousarray(np.concatenate([[0.0], np.asarray(x, dtype=np.float64)]))
    fp, keep = _callback(f, 1)
    chk = C.c_int(1)
    lib.scft_broydn_set_tol(float(tol))
    check(lib.scft_broydn(_dp(xx), int(n), C.byref(chk), fp), "scft_broydn")
    del keep
    return xx[1:], chk.value, lib.scft_broydn_get_err()


# ---------------------------------------------------------------------------
# batched path
# ---------------------------------------------------------------------------
def solve_opts(**kw) -> L.ScftSolveOpts:
    o = L.ScftSolveOpts()
    L.load().scft_solve_opts_init(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def _results(res) -> dict:
    """The scft_result array as one numpy array per field (a structured view of
    the ctypes array, copied)."""
    a = np.ctypeslib.as_array(res)
    return {k: a[k].copy() for k in ("status", "iterations", "err", "Q")}


class Batch:
    """Independent SCFT instances solved together on the GPU.

    ``instances`` is a sequence of dicts with keys n_nodes, L, f0, nsteps, ds and
    optional x, w0, rule."""

    def __init__(self, instances=None, *, arrays=None):
        """From a sequence of instance dicts, or from `arrays` (the output of
        Batch.pack: node arrays already concatenated)."""
        self.lib = L.load()
        a = arrays if arrays is not None else Batch.pack(instances)
        self.count = len(a["n_nodes"])
        self.n_nodes = a["n_nodes"]
        self.offsets = np.concatenate([[0], np.cumsum(self.n_nodes)])
        self._bounds = list(zip(self.offsets[:-1].tolist(), self.offsets[1:].tolist()))
        desc = Batch._descriptors(a, self.offsets)
        self._keep = [a]
        h = C.c_void_p()
        check(self.lib.scft_batch_create(C.cast(desc.ctypes.data, C.POINTER(L.ScftInstance)), self.count,
                                         C.byref(h)), "scft_batch_create")
        self._keep = []
        self.h = h

    @classmethod
    def from_arrays(cls, arrays):
        return cls(arrays=arrays)

    @staticmethod
    def pack(instances):
        """Per-instance dicts -> dict of host arrays: n_nodes, L, nsteps, ds, rule
        (one entry per instance) and x, f0, w0 (node arrays concatenated; x and
        w0 may be None, then the library uses a uniform mesh on [0, L] and a zero
        field)."""
        n = np.array([int(d["n_nodes"]) for d in instances], dtype=np.int64)
        out = {"n_nodes": n,
               "L": np.array([float(d.get("L", 0.0)) for d in instances]),
               "nsteps": np.array([int(d["nsteps"]) for d in instances], dtype=np.int32),
               "ds": np.array([float(d["ds"]) for d in instances]),
               "rule": np.array([int(d.get("rule", L.RULE_ROMBERG)) for d in instances], dtype=np.int32)}
        for key in ("x", "f0", "w0"):
            have = [d.get(key) is not None for d in instances]
            if key == "f0" and not all(have):
                raise ValueError("every instance needs f0")
            if not any(have):
                out[key] = None
                continue
            if not all(have):
                raise ValueError(f"{key}: give it for every instance or for none")
            parts = [np.asarray(d[key], dtype=np.float64) for d in instances]
            if any(p.shape != (k,) for p, k in zip(parts, n)):
                raise ValueError(f"{key}: every array needs n_nodes entries")
            out[key] = np.ascontiguousarray(np.concatenate(parts))
        return out

    @staticmethod
    def _descriptors(a, offsets):
        """The scft_instance array as a numpy structured array with the C layout
        (field offsets of the ctypes mirror), pointing into the packed arrays."""
        st = L.ScftInstance
        names = [f for f, _ in st._fields_]
        fmt = {"n_nodes": np.int32, "x": np.uint64, "L": np.float64, "f0": np.uint64, "w0": np.uint64,
               "nsteps": np.int32, "ds": np.float64, "rule": np.int32}
        dt = np.dtype({"names": names, "formats": [fmt[f] for f in names],
                       "offsets": [getattr(st, f).offset for f in names], "itemsize": C.sizeof(st)})
        cnt = len(a["n_nodes"])
        desc = np.zeros(cnt, dtype=dt)
        for k in ("n_nodes", "L", "nsteps", "ds", "rule"):
            desc[k] = a[k]
        total = int(offsets[-1])
        for key in ("x", "f0", "w0"):
            arr = a[key]
            if arr is None:
                continue
            if arr.dtype != np.float64 or not arr.flags.c_contiguous or arr.size != total:
                raise ValueError(f"{key}: need {total} contiguous doubles")
            desc[key] = (arr.ctypes.data + 8 * offsets[:-1]).astype(np.uint64)
        return desc

    def split(self, flat):
        return [flat[a:z] for a, z in self._bounds]

    def set_fields(self, w_nodes_list):
        flat = np.ascontiguousarray(np.concatenate(w_nodes_list), dtype=np.float64)
        check(self.lib.scft_batch_set_fields(self.h, _dp(flat)), "scft_batch_set_fields")

    def evaluate(self, precision=L.F64):
        check(self.lib.scft_batch_evaluate(self.h, int(precision)), "scft_batch_evaluate")

    def evaluate_scheme(self, scheme=L.SCHEME_IRK2, wmode=L.W_CONSISTENT):
        """FP64 density of every instance with the given contour scheme and field
        term (IRK2 + consistent: the deal.II propagator)."""
        check(self.lib.scft_batch_evaluate_scheme(self.h, int(scheme), int(wmode)), "scft_batch_evaluate_scheme")

    def solve(self, opts: L.ScftSolveOpts | None = None, **kw):
        o = opts if opts is not None else solve_opts(**kw)
        res = (L.ScftResult * self.count)()
        check(self.lib.scft_batch_solve(self.h, C.byref(o), res), "scft_batch_solve")
        return _results(res)

    def solve_async(self, opts: L.ScftSolveOpts | None = None, **kw):
        """Enqueue the fused FP32 solve and return at once; wait() completes it.
        Batches solving at the same time share the GPU."""
        o = opts if opts is not None else solve_opts(**kw)
        check(self.lib.scft_batch_solve_async(self.h, C.byref(o)), "scft_batch_solve_async")

    def wait(self):
        res = (L.ScftResult * self.count)()
        check(self.lib.scft_batch_wait(self.h, res), "scft_batch_wait")
        return _results(res)

    def get(self):
        tot = int(self.offsets[-1])
        w = np.empty(tot)
        phi = np.empty(tot)
        Q = np.empty(self.count)
        check(self.lib.scft_batch_get(self.h, _dp(w), _dp(phi), _dp(Q)), "scft_batch_get")
        return self.split(w), self.split(phi), Q

    def status(self):
        st = (C.c_int * self.count)()
        check(self.lib.scft_batch_status(self.h, st), "scft_batch_status")
        return np.array(st[:])

    def reset(self):
        """Restore the creation-time fields on the device."""
        check(self.lib.scft_batch_reset(self.h), "scft_batch_reset")

    def last_ms(self) -> float:
        """Event-timed device duration of the last evaluate / solve / reset."""
        return float(self.lib.scft_batch_last_ms(self.h))

    def free_energy(self, f0_samples):
        """Free energy of each instance (scft.cc:404-450) from its target sampled
        at m+1 uniform points of [0, L] (array count x (m+1), m a power of two)."""
        fs = np.ascontiguousarray(f0_samples, dtype=np.float64)
        m = fs.shape[1] - 1
        F = np.empty(self.count)
        check(self.lib.scft_batch_free_energy(self.h, int(m), _dp(fs), _dp(F)), "scft_batch_free_energy")
        return F

    def trace(self, max_entries=100000):
        """(unfinished instances, ms since start) after each graph launch of the last solve."""
        a = (C.c_int * max_entries)()
        m = (C.c_double * max_entries)()
        k = check(self.lib.scft_batch_trace(self.h, max_entries, a, m), "scft_batch_trace")
        k = min(k, max_entries)
        return np.array(a[:k]), np.array(m[:k])

    def profile(self, precision=L.F32, max_classes=64):
        """Per shape class: (C, NW, items, algorithmic bytes, ms) of one pass alone."""
        n = max_classes
        Cs, NWs, its = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
        by, ms = (C.c_double * n)(), (C.c_double * n)()
        k = check(self.lib.scft_batch_profile(self.h, int(precision), n, Cs, NWs, its, by, ms),
                  "scft_batch_profile")
        return [dict(C=Cs[i], NW=NWs[i], items=its[i], bytes=by[i], ms=ms[i]) for i in range(min(k, n))]

    def live_stats(self, precision=L.F32, max_classes=64):
        """Per shape class, over the propagator launches of the last solve that
        evaluated anything: (C, NW, launches, algorithmic bytes, summed ms)."""
        n = max_classes
        Cs, NWs = (C.c_int * n)(), (C.c_int * n)()
        ln, by, ms = (C.c_longlong * n)(), (C.c_double * n)(), (C.c_double * n)()
        k = check(self.lib.scft_batch_live_stats(self.h, int(precision), n, Cs, NWs, ln, by, ms),
                  "scft_batch_live_stats")
        return [dict(C=Cs[i], NW=NWs[i], launches=ln[i], bytes=by[i], ms=ms[i]) for i in range(min(k, n))]

    def set_shape(self, precision, index, C_nodes, NW):
        check(self.lib.scft_batch_set_shape(self.h, int(precision), int(index), int(C_nodes), int(NW)),
              "scft_batch_set_shape")

    def autotune(self, precision=L.F32):
        check(self.lib.scft_batch_autotune(self.h, int(precision)), "scft_batch_autotune")

    def close(self):
        if getattr(self, "h", None):
            self.lib.scft_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launches() -> int:
    return int(L.load().scft_kernel_launches())
