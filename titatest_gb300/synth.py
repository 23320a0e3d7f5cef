"""Seeded synthetic tomodirs with the shapes of the benchmark configurations.

No public data set is involved: meshes, resistivity models and electrode
configurations are generated from seeds.  The grids follow the conventions of
the reference's own grid files (tests/*/grid/elem.dat): counter-clockwise
quadrilaterals listed row by row from the surface, type-12 (no-flow) lines
along the surface from left to right, type-11 (mixed) lines clockwise down the
right side, along the bottom and up the left side, and the Cuthill-McKee
renumbering of cutmckee/cutmck.f applied last (titatest_gb300.cutmck).

Configurations (seed = 1000*cfg + i):
  1  60x20 quads of 1 m, 30 surface electrodes at 2 m, 10 ohm-m 6x4 block in a
     100 ohm-m half-space, zero phase, dipole-dipole a = 1 spacing, n = 1..8.
  2  200x60 quads (1 m x 0.5 m, cells growing 1.1x below 20 m), 3-sinusoid
     topography (<= 2 m) draped, 96 electrodes at 1 m, log10|rho| Gaussian
     random field (mean 2, sd 0.3, exponential variogram 10 m x 3 m), phase
     U(-5, -30) mrad from a second field of the same variogram, 2000
     dipole-dipole (a 1..4, n 1..8) + 2000 Wenner-Schlumberger.
  3  250x100 grid split into 50k triangles, interior nodes jittered by
     <= 0.2 cell, 64 electrodes, 2000 dipole-dipole, model as in 2.
  4  400x100 quads, 192 electrodes at 0.5 m, 20000 dipole-dipole
     (a 1..6, n 1..10) sub-sampled, model of 2 plus two elliptic anomalies.
  5  ensemble of 256 problems, 40x15 ... 300x80 quads (log-uniform), 24-128
     electrodes at 1 m, 200-6000 dipole-dipole each.

The generator itself is numpy only.  The Cuthill-McKee renumbering is the
library's (crgpu_cutmck) unless a `cutmck(grid, enr) -> (grid, enr)` callable
is passed: any implementation of cutmckee/cutmck.f gives the same integers.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import formats


@dataclasses.dataclass
class Synthetic:
    name: str
    grid: formats.Grid
    survey: formats.Survey
    sigma: np.ndarray
    nx: int = 0            # model cells per row (structured grids)
    nz: int = 0
    triangles: bool = False


# ---------------------------------------------------------------------------
# meshes
# ---------------------------------------------------------------------------
def _quad_grid(xs: np.ndarray, depths: np.ndarray, topo: Optional[np.ndarray] = None,
               triangles: bool = False, jitter: float = 0.0, rng=None):
    """Structured grid: node (i, j), i along x, j downwards from the surface.
    Returns (grid in natural numbering, surface node numbers)."""
    nx, nz = len(xs) - 1, len(depths) - 1
    X = np.repeat(xs[None, :], nz + 1, axis=0).astype(np.float64)
    top = np.zeros(nx + 1) if topo is None else topo
    Y = top[None, :] - depths[:, None]
    if jitter > 0.0 and rng is not None:
        dx = np.diff(xs)
        dz = np.diff(depths)
        hx = np.minimum(np.r_[dx[0], dx], np.r_[dx, dx[-1]])
        hz = np.minimum(np.r_[dz[0], dz], np.r_[dz, dz[-1]])
        jx = rng.uniform(-jitter, jitter, size=X.shape) * hx[None, :]
        jz = rng.uniform(-jitter, jitter, size=X.shape) * hz[:, None]
        inner = np.zeros(X.shape, bool)
        inner[1:-1, 1:-1] = True
        X = X + np.where(inner, jx, 0.0)
        Y = Y + np.where(inner, jz, 0.0)

    def node(i, j):
        return j * (nx + 1) + i + 1

    area = []
    rnr_of = {}
    for j in range(nz):
        for i in range(nx):
            bl, br, tr, tl = node(i, j + 1), node(i + 1, j + 1), node(i + 1, j), node(i, j)
            if triangles:
                area.append([bl, br, tr])   # holds edges (br,tr) and (bl,br)
                e1 = len(area)
                area.append([bl, tr, tl])   # holds edges (tr,tl) and (tl,bl)
                e2 = len(area)
                rnr_of[("top", i, j)] = e2
                rnr_of[("right", i, j)] = e1
                rnr_of[("bottom", i, j)] = e1
                rnr_of[("left", i, j)] = e2
            else:
                area.append([bl, br, tr, tl])
                e = len(area)
                for side in ("top", "right", "bottom", "left"):
                    rnr_of[(side, i, j)] = e
    top_b, mixed_b = [], []
    for i in range(nx):
        top_b.append(([node(i, 0), node(i + 1, 0)], rnr_of[("top", i, 0)]))
    for j in range(nz):
        mixed_b.append(([node(nx, j), node(nx, j + 1)], rnr_of[("right", nx - 1, j)]))
    for i in range(nx - 1, -1, -1):
        mixed_b.append(([node(i + 1, nz), node(i, nz)], rnr_of[("bottom", i, nz - 1)]))
    for j in range(nz - 1, -1, -1):
        mixed_b.append(([node(0, j + 1), node(0, j)], rnr_of[("left", 0, j)]))
    nk = 3 if triangles else 4
    ne = len(area) + len(top_b) + len(mixed_b)
    nrel = np.zeros((ne, 4), np.int32)
    nrel[: len(area), :nk] = np.array(area, np.int32)
    off = len(area)
    for q, (nodes, _) in enumerate(top_b + mixed_b):
        nrel[off + q, :2] = nodes
    rnr = np.array([r for _, r in top_b + mixed_b], np.int32)
    sanz = (nx + 1) * (nz + 1)
    grid = formats.Grid(
        sanz=sanz, mb=0,
        typ=np.array([3 if triangles else 8, 12, 11], np.int32),
        nelanz=np.array([len(area), len(top_b), len(mixed_b)], np.int32),
        selanz=np.array([nk, 2, 2], np.int32),
        snr=np.arange(1, sanz + 1, dtype=np.int32),
        sx=X.reshape(-1).copy(), sy=Y.reshape(-1).copy(),
        nrel=nrel if nk == 4 else nrel[:, :4], rnr=rnr)
    if nk == 3:
        grid.nrel = np.ascontiguousarray(grid.nrel[:, :3])
    surface = np.array([node(i, 0) for i in range(nx + 1)], np.int32)
    return grid, surface, X, Y


def _centroids(grid: formats.Grid):
    x, y = grid.node_xy()
    E = grid.elanz
    nk = grid.selanz[0]
    idx = grid.nrel[:E, :nk] - 1
    return x[idx].mean(1), y[idx].mean(1)


# ---------------------------------------------------------------------------
# Gaussian random field by circulant embedding (exponential covariance)
# ---------------------------------------------------------------------------
def grf(points_x, points_y, ax: float, az: float, rng, h: float = 0.25) -> np.ndarray:
    """Standard-normal field with covariance exp(-sqrt((dx/ax)^2 + (dz/az)^2)),
    sampled at the given points (nearest node of an auxiliary regular grid)."""
    x0, x1 = points_x.min() - h, points_x.max() + h
    z0, z1 = points_y.min() - h, points_y.max() + h
    nxg = int(math.ceil((x1 - x0) / h)) + 1
    nzg = int(math.ceil((z1 - z0) / h)) + 1
    mx, mz = 2 * nxg, 2 * nzg
    ix = np.arange(mx)
    iz = np.arange(mz)
    dx = np.minimum(ix, mx - ix) * h
    dz = np.minimum(iz, mz - iz) * h
    C = np.exp(-np.sqrt((dx[None, :] / ax) ** 2 + (dz[:, None] / az) ** 2))
    lam = np.fft.fft2(C).real
    lam = np.maximum(lam, 0.0)
    noise = rng.standard_normal((mz, mx)) + 1j * rng.standard_normal((mz, mx))
    field = np.fft.ifft2(np.sqrt(lam) * noise) * math.sqrt(mx * mz)
    f = field.real[:nzg, :nxg]
    f = (f - f.mean()) / (f.std() + 1e-300)
    gi = np.clip(np.rint((points_x - x0) / h).astype(int), 0, nxg - 1)
    gj = np.clip(np.rint((points_y - z0) / h).astype(int), 0, nzg - 1)
    return f[gj, gi]


def _normal_cdf(z):
    return 0.5 * (1.0 + np.vectorize(math.erf)(z / math.sqrt(2.0)))


def _sigma_from(mag, pha_mrad):
    pha = 1e-3 * pha_mrad
    return (np.cos(pha) - 1j * np.sin(pha)) / mag


def random_model(grid, rng, mean=2.0, sd=0.3, ax=10.0, az=3.0):
    cx, cy = _centroids(grid)
    z1 = grf(cx, cy, ax, az, rng)
    z2 = grf(cx, cy, ax, az, rng)
    mag = 10.0 ** (mean + sd * z1)
    pha = -5.0 - 25.0 * _normal_cdf(z2)
    return mag, pha


# ---------------------------------------------------------------------------
# electrode configurations (strnr = A*10000+B, vnr = M*10000+N)
# ---------------------------------------------------------------------------
def dipole_dipole(ne: int, a_list, n_list):
    out = []
    for a in a_list:
        for n in n_list:
            for A in range(1, ne + 1):
                B, M = A + a, A + a + n * a
                N = M + a
                if N > ne:
                    break
                out.append((A, B, M, N))
    return out


def wenner_schlumberger(ne: int, a_list, n_list):
    out = []
    for a in a_list:
        for n in n_list:
            for A in range(1, ne + 1):
                M = A + n * a
                N = M + a
                B = N + n * a
                if B > ne:
                    break
                out.append((A, B, M, N))
    return out


def _encode(quads):
    s = np.array([a * 10000 + b for a, b, _, _ in quads], np.int32)
    v = np.array([m * 10000 + n for _, _, m, n in quads], np.int32)
    return s, v


def _subsample(quads, k, rng):
    if len(quads) <= k:
        return quads
    idx = np.sort(rng.choice(len(quads), size=k, replace=False))
    return [quads[i] for i in idx]


def _finish(name, grid, surface, enodes, quads, mag, pha, nx, nz, triangles=False, cutmck=None):
    if cutmck is None:
        from .crmod import cutmck
    enr = surface[enodes]
    g2, enr2 = cutmck(grid, enr)
    s, v = _encode(quads)
    formats.check_config(s, v, len(enr2))
    survey = formats.Survey(enr=enr2, strnr=s, vnr=v, strom=np.ones(len(s)))
    return Synthetic(name=name, grid=g2, survey=survey, sigma=_sigma_from(mag, pha), nx=nx, nz=nz,
                     triangles=triangles)


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------
def config1(seed: int = 1000, cutmck=None) -> Synthetic:
    rng = np.random.default_rng(seed)
    nx, nz = 60, 20
    grid, surface, X, Y = _quad_grid(np.arange(nx + 1, dtype=float), np.arange(nz + 1, dtype=float))
    mag = np.full(nx * nz, 100.0)
    ci = int(rng.integers(3, nx - 3))          # block centre column
    cj = int(rng.integers(2, nz // 2 - 1))     # upper half
    for j in range(cj - 2, cj + 2):
        for i in range(ci - 3, ci + 3):
            mag[j * nx + i] = 10.0
    pha = np.zeros(nx * nz)
    enodes = np.arange(1, 60, 2)               # 30 electrodes at 2 m
    quads = dipole_dipole(30, [1], range(1, 9))
    return _finish("cfg1", grid, surface, enodes, quads, mag, pha, nx, nz, cutmck=cutmck)


def _cfg2_depths():
    d = [0.0]
    h = 0.5
    while d[-1] < 20.0 - 1e-9:
        d.append(d[-1] + h)
    while len(d) < 61:
        h *= 1.1
        d.append(d[-1] + h)
    return np.array(d)


def _topography(xs, rng, amp=2.0):
    L = xs[-1] - xs[0]
    t = np.zeros_like(xs)
    for _ in range(3):
        a = rng.uniform(0.2, 1.0)
        lam = rng.uniform(0.2, 1.0) * L
        ph = rng.uniform(0, 2 * math.pi)
        t += a * np.sin(2 * math.pi * xs / lam + ph)
    return amp * t / (np.abs(t).max() + 1e-300)


def config2(seed: int = 2000, cutmck=None) -> Synthetic:
    rng = np.random.default_rng(seed)
    nx = 200
    xs = np.arange(nx + 1, dtype=float) - 52.0   # electrodes at x = 0..95
    depths = _cfg2_depths()
    nz = len(depths) - 1
    topo = _topography(xs, rng)
    grid, surface, X, Y = _quad_grid(xs, depths, topo)
    mag, pha = random_model(grid, rng)
    enodes = np.arange(52, 52 + 96)
    dd = _subsample(dipole_dipole(96, range(1, 5), range(1, 9)), 2000, rng)
    ws = _subsample(wenner_schlumberger(96, range(1, 5), range(1, 9)), 2000, rng)
    return _finish("cfg2", grid, surface, enodes, dd + ws, mag, pha, nx, nz, cutmck=cutmck)


def config3(seed: int = 3000, cutmck=None) -> Synthetic:
    rng = np.random.default_rng(seed)
    nx, nz = 250, 100
    xs = np.arange(nx + 1, dtype=float) * 0.5 - 30.0
    depths = np.arange(nz + 1, dtype=float) * 0.5
    grid, surface, X, Y = _quad_grid(xs, depths, triangles=True, jitter=0.2, rng=rng)
    mag, pha = random_model(grid, rng)
    enodes = np.arange(60, 60 + 2 * 64, 2)   # 64 electrodes at 1 m
    dd = _subsample(dipole_dipole(64, range(1, 5), range(1, 9)), 2000, rng)
    return _finish("cfg3", grid, surface, enodes, dd, mag, pha, nx, nz, triangles=True, cutmck=cutmck)


def config4(seed: int = 4000, cutmck=None) -> Synthetic:
    rng = np.random.default_rng(seed)
    nx, nz = 400, 100
    xs = np.arange(nx + 1, dtype=float) * 0.5 - 52.0
    depths = np.arange(nz + 1, dtype=float) * 0.5
    grid, surface, X, Y = _quad_grid(xs, depths)
    mag, pha = random_model(grid, rng)
    cx, cy = _centroids(grid)
    for _ in range(2):
        ex, ey = rng.uniform(10, 80), -rng.uniform(3, 15)
        rx, ry = rng.uniform(4, 10), rng.uniform(1.5, 4)
        inside = ((cx - ex) / rx) ** 2 + ((cy - ey) / ry) ** 2 <= 1.0
        mag[inside] = 10.0
        pha[inside] = -50.0
    enodes = np.arange(104, 104 + 192)
    dd = _subsample(dipole_dipole(192, range(1, 7), range(1, 11)), 20000, rng)
    return _finish("cfg4", grid, surface, enodes, dd, mag, pha, nx, nz, cutmck=cutmck)


def _config5_shape(rng):
    f = rng.uniform(0, 1)
    nx = int(round(40 * (300 / 40) ** f))
    nz = int(round(15 * (80 / 15) ** f))
    return nx, nz


def config5_shapes(seed: int = 5000, count: int = 256) -> List[Tuple[int, int]]:
    """(nx, nz) quads of every ensemble problem, without building them."""
    return [_config5_shape(np.random.default_rng(seed + q)) for q in range(count)]


def config5(seed: int = 5000, count: int = 256, cutmck=None,
            indices: Optional[Sequence[int]] = None) -> List[Synthetic]:
    """The ensemble; `indices` builds only those problems (same seeds)."""
    out = []
    for q in (range(count) if indices is None else indices):
        rng = np.random.default_rng(seed + q)
        nx, nz = _config5_shape(rng)
        ne = int(rng.integers(24, min(128, nx - 4) + 1))
        first = (nx - ne) // 2
        xs = np.arange(nx + 1, dtype=float) - first
        depths = np.arange(nz + 1, dtype=float) * 0.5
        grid, surface, X, Y = _quad_grid(xs, depths)
        mag, pha = random_model(grid, rng)
        enodes = np.arange(first, first + ne)
        allq = dipole_dipole(ne, range(1, 7), range(1, 11))
        k = int(rng.integers(200, 6001))
        out.append(_finish(f"cfg5_{q}", grid, surface, enodes, _subsample(allq, k, rng), mag, pha, nx, nz,
                           cutmck=cutmck))
    return out


def make(cfg: int, seed: Optional[int] = None, cutmck=None):
    f = {1: config1, 2: config2, 3: config3, 4: config4, 5: config5}[cfg]
    return f(cutmck=cutmck) if seed is None else f(seed, cutmck=cutmck)
