"""Seeded synthetic point sets for the Voronoi workloads.

    uniform      n points i.i.d. uniform in the unit cube
    clustered    90% from 64 isotropic Gaussians (centres uniform in
                 [0.1, 0.9]^3, sigma 0.01, equal weights) + 10% uniform,
                 out-of-cube draws re-sampled
    batched      many diagrams, n_i log-uniform in [64, 65536], box sides
                 uniform in [0.5, 2], points uniform in each box
    lattice_sc   simple cubic m^3 lattice in the unit cube, jittered by
                 uniform noise of amplitude 1e-7 of the spacing
    lattice_bcc  body-centred cubic 2 m^3 lattice, same jitter

All generators are numpy PCG64 streams seeded per workload.
"""
from __future__ import annotations

import numpy as np


def uniform(n: int, seed: int = 0) -> np.ndarray:
    return np.random.default_rng(seed).random((n, 3))


def clustered(n: int, seed: int = 3, nclusters: int = 64, sigma: float = 0.01,
              background: float = 0.1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    nbg = int(round(background * n))
    ncl = n - nbg
    centres = 0.1 + 0.8 * rng.random((nclusters, 3))
    which = rng.integers(0, nclusters, ncl)
    pts = centres[which] + sigma * rng.standard_normal((ncl, 3))
    bad = np.any((pts < 0.0) | (pts >= 1.0), axis=1)
    while bad.any():
        k = int(bad.sum())
        pts[bad] = centres[which[bad]] + sigma * rng.standard_normal((k, 3))
        bad = np.any((pts < 0.0) | (pts >= 1.0), axis=1)
    out = np.concatenate([pts, rng.random((nbg, 3))])
    return out[rng.permutation(n)]


def batched(ndiag: int = 4096, seed: int = 4, nmin: int = 64, nmax: int = 65536):
    """Returns (points, offsets[ndiag+1], boxes[ndiag, 6])."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(nmin), np.log(nmax), ndiag))).astype(np.int64)
    sides = rng.uniform(0.5, 2.0, (ndiag, 3))
    offs = np.zeros(ndiag + 1, dtype=np.uint64)
    offs[1:] = np.cumsum(sizes)
    pts = rng.random((int(offs[-1]), 3))
    pts *= np.repeat(sides, sizes, axis=0)
    boxes = np.concatenate([np.zeros((ndiag, 3)), sides], axis=1)
    return pts, offs, boxes


def lattice_sc(m: int = 128, seed: int = 5, jitter: float = 1e-7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    h = 1.0 / m
    g = (np.arange(m) + 0.5) * h
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    return pts + (rng.random(pts.shape) - 0.5) * (jitter * h)


def lattice_bcc(m: int = 100, seed: int = 6, jitter: float = 1e-7) -> np.ndarray:
    rng = np.random.default_rng(seed)
    a = 1.0 / m
    g1 = (np.arange(m) + 0.25) * a
    g2 = (np.arange(m) + 0.75) * a
    parts = []
    for g in (g1, g2):
        x, y, z = np.meshgrid(g, g, g, indexing="ij")
        parts.append(np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1))
    pts = np.concatenate(parts)
    return pts + (rng.random(pts.shape) - 0.5) * (jitter * a)
