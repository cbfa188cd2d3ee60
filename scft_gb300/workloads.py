"""Seeded synthetic SCFT workloads (no public dataset is involved).

Every random draw is a splitmix64 hash of (seed, instance, slot), so any host
regenerates identical instances.  The shapes follow the five workloads the
solver is measured on:

* ``single_small``  L=4, 32 uniform elements, 2048 steps, FP64, tol 1e-8
* ``single_large``  the same physics at 1024 elements
* ``batch_mixed``   4096 instances, elements log-uniform in [32, 1024],
                    L ~ U[2, 10], steps in {512, 1024, 2048, 4096}
* ``warmstart_train`` / ``warmstart_eval``  L ~ U[2, 10], elements in [64, 512]
* ``batch_graded``  512 instances of 8192 elements graded by 1.002 toward
                    both walls, 8192 steps, L ~ U[2, 12]

The target profile is the Gaussian wall f0 = (1-exp(-(x/0.25)^2))(1-exp(-((L-x)/0.25)^2))
and the initial field is U[-0.1, 0.1] per interior node.
"""
from __future__ import annotations

import numpy as np

from ._lib import RULE_ROMBERG

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(z: np.ndarray) -> np.ndarray:
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, inst, slot) -> np.ndarray:
    """U[0,1) draw keyed by (seed, instance, slot)."""
    inst = np.asarray(inst, dtype=np.uint64)
    slot = np.asarray(slot, dtype=np.uint64)
    with np.errstate(over="ignore"):
        k = splitmix64(np.uint64(seed) ^ splitmix64(inst * np.uint64(0x100000001B3) + slot))
    return (k >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def gauss_wall_f0(x: np.ndarray, L: float, width: float = 0.25) -> np.ndarray:
    a = x / width
    b = (L - x) / width
    return (1.0 - np.exp(-a * a)) * (1.0 - np.exp(-b * b))


def uniform_mesh(m_elem: int, L: float) -> np.ndarray:
    x = L * np.arange(m_elem + 1, dtype=np.float64) / m_elem
    x[-1] = L
    return x


def graded_mesh(m_elem: int, ratio: float, L: float) -> np.ndarray:
    """m_elem elements, element k from the nearer wall of length h0*ratio^k."""
    half = m_elem // 2
    h = ratio ** np.arange(half, dtype=np.float64)
    h *= 0.5 * L / h.sum()
    left = np.concatenate([[0.0], np.cumsum(h)])
    left[-1] = 0.5 * L
    x = np.concatenate([left, L - left[-2::-1]])
    return x


def initial_field(seed: int, inst: int, n_nodes: int) -> np.ndarray:
    w = -0.1 + 0.2 * uniform(seed, inst, 16 + np.arange(n_nodes))
    w[0] = w[-1] = 0.0
    return w


def instance(m_elem: int, L: float, nsteps: int, seed: int, inst: int, graded: float | None = None,
             rule: int = RULE_ROMBERG) -> dict:
    x = graded_mesh(m_elem, graded, L) if graded else uniform_mesh(m_elem, L)
    return {
        "n_nodes": m_elem + 1,
        "x": x,
        "L": L,
        "f0": gauss_wall_f0(x, L),
        "w0": initial_field(seed, inst, m_elem + 1),
        "nsteps": nsteps,
        "ds": 1.0 / nsteps,
        "rule": rule,
        "seed": seed,
        "index": inst,
    }


def single_small(seed: int = 0) -> dict:
    return instance(32, 4.0, 2048, seed, 0)


def single_large(seed: int = 0) -> dict:
    return instance(1024, 4.0, 2048, seed, 0)


NSTEPS_CHOICES = (512, 1024, 2048, 4096)


def batch_mixed(count: int = 4096, seed: int = 3, m_lo: int = 32, m_hi: int = 1024,
                L_lo: float = 2.0, L_hi: float = 10.0) -> list:
    idx = np.arange(count)
    m = np.rint(np.exp(np.log(m_lo) + uniform(seed, idx, 0) * (np.log(m_hi) - np.log(m_lo)))).astype(int)
    m = np.clip(m, m_lo, m_hi)
    Ls = L_lo + (L_hi - L_lo) * uniform(seed, idx, 1)
    ns = np.array(NSTEPS_CHOICES)[np.minimum((uniform(seed, idx, 2) * 4).astype(int), 3)]
    return [instance(int(m[i]), float(Ls[i]), int(ns[i]), seed, i) for i in range(count)]


def warmstart_train(count: int = 20000, seed: int = 41) -> list:
    return batch_mixed(count, seed, 64, 512)


def warmstart_eval(count: int = 4096, seed: int = 43) -> list:
    return batch_mixed(count, seed, 64, 512)


def batch_graded(count: int = 512, seed: int = 5, m_elem: int = 8192, nsteps: int = 8192) -> list:
    idx = np.arange(count)
    Ls = 2.0 + 10.0 * uniform(seed, idx, 1)
    return [instance(m_elem, float(Ls[i]), nsteps, seed, i, graded=1.002) for i in range(count)]
