"""Smoothness regularisation of the Gauss-Newton update (host side, set-up
once per grid, as in the reference):

* bnachbar  -- src/bnachbar.f90:7-93: for every area element and every edge
               (nodes k, k+1 mod nk) the element sharing that edge (the last
               one in element order), plus the neighbour count;
* bsmatmreg -- src/bsmatm_mod.f90:190-362 (ltri = 0): smatm(manz, 3) of the
               structured nx x nz grid (no discontinuities);
* bsmatmtri -- src/bsmatm_mod.f90:364-460 (ltri = 1, 2): smatm(manz, nk+1)
               over the neighbours (no decouplings).

Arrays are returned in the layout the C ABI takes: column-major
(manz, ncol) as an array of shape (ncol, manz).
"""
from __future__ import annotations

import numpy as np

from . import formats


def bnachbar(grid: formats.Grid) -> np.ndarray:
    E = grid.elanz
    nk = grid.maxnk
    nrel = grid.nrel[:E, :nk].astype(np.int64)
    nb = np.zeros((nk + 1, E), np.int32)
    edges = {}
    for e in range(E):
        for k in range(nk):
            a, b = nrel[e, k], nrel[e, (k + 1) % nk]
            key = (min(a, b), max(a, b))
            edges.setdefault(key, []).append((e, k))
    for lst in edges.values():
        for e, k in lst:
            others = [o for o, _ in lst if o != e]
            if others:
                # the reference records every matching (element, edge) pair;
                # the stored neighbour is the last element in order
                nb[k, e] = max(others) + 1
                nb[nk, e] += len(others)
    return nb


def _centroids(grid: formats.Grid):
    """Element centroids as src/relem.f90:107-118 computes espx/espy."""
    x, y = grid.node_xy()
    E = grid.elanz
    out_x = np.zeros(E)
    out_y = np.zeros(E)
    iel = 0
    for t, n, s in zip(grid.typ, grid.nelanz, grid.selanz):
        if t < 10:
            idx = grid.nrel[iel:iel + n, :s] - 1
            out_x[iel:iel + n] = x[idx].sum(1) / s
            out_y[iel:iel + n] = y[idx].sum(1) / s
        iel += n
    return out_x, out_y


def bsmatmreg(grid: formats.Grid, nx: int, nz: int, alfx: float = 1.0, alfz: float = 1.0) -> np.ndarray:
    x, y = grid.node_xy()
    manz = nx * nz
    nr = grid.nrel[:manz, :4] - 1
    X = x[nr]
    Y = y[nr]
    xmean = X.sum(1) / 4.0
    zmean = Y.sum(1) / 4.0
    dzleft = np.abs(Y[:, 3] - Y[:, 0])
    dzright = np.abs(Y[:, 2] - Y[:, 1])
    dxup = np.abs(X[:, 2] - X[:, 3])
    dxdown = np.abs(X[:, 1] - X[:, 0])
    sm = np.zeros((3, manz))
    e = np.arange(manz)
    i, j = e // nx, e % nx
    left = j > 0
    sm[0, left] = alfx * dzleft[left] / np.abs(xmean[left] - xmean[e[left] - 1])
    right = j < nx - 1
    dum = alfx * dzright[right] / np.abs(xmean[e[right] + 1] - xmean[right])
    sm[0, right] += dum
    sm[1, right] = -dum
    up = i > 0
    sm[0, up] += alfz * dxup[up] / np.abs(zmean[e[up] - nx] - zmean[up])
    down = i < nz - 1
    dum = alfz * dxdown[down] / np.abs(zmean[down] - zmean[e[down] + nx])
    sm[0, down] += dum
    sm[2, down] = -dum
    return sm


def bsmatmtri(grid: formats.Grid, nachbar: np.ndarray, alfx: float = 1.0, alfz: float = 1.0) -> np.ndarray:
    x, y = grid.node_xy()
    E = grid.elanz
    nk = grid.maxnk
    cx, cy = _centroids(grid)
    sm = np.zeros((nk + 1, E))
    nr = grid.nrel[:E, :nk] - 1
    for k in range(nk):
        a, b = nr[:, k], nr[:, (k + 1) % nk]
        edglen = np.sqrt((x[a] - x[b]) ** 2 + (y[a] - y[b]) ** 2)
        nbk = nachbar[k]
        has = nbk > 0
        o = nbk[has] - 1
        dx = cx[has] - cx[o]
        dy = cy[has] - cy[o]
        dist = np.sqrt(dx ** 2 + dy ** 2)
        ang = np.arctan2(dy, dx)
        alfgeo = np.sqrt((alfx * np.cos(ang)) ** 2 + (alfz * np.sin(ang)) ** 2)
        rs = edglen[has] / dist * alfgeo
        sm[k, has] = -rs
        sm[nk, has] += rs
    return sm
