"""Synthetic sparse SPD inputs for the CG path (host side, numpy).

These stand in for the SuiteSparse matrices the reference downloads
(conjugateGradient/data/filelist.txt), which are not available offline:

* ``laplacian_2d(n)`` — 5-point Laplacian on an n x n grid, Dirichlet
  boundary (diag 4, off-diagonals -1); n = 2048 gives N = 4,194,304 and
  nnz = 20,963,328.
* ``laplacian_3d(n)`` — 7-point Laplacian on n^3 (diag 6, off -1); n = 160
  gives N = 4,096,000 and nnz = 28,518,400.
* ``random_spd(n, seed)`` — symmetric pattern, row degrees power-law in
  [3, 60] with mean about 14, off-diagonals N(0,1), diagonal
  sum|offdiag| + U(0.1, 1) (strictly diagonally dominant, hence SPD).
* ``csr_to_dia`` — diagonal-major DIA (data[k][i] = A[i][i+offset[k]]).

CSR uses int32 row pointers and column indices, columns sorted within a row.
"""
from __future__ import annotations

import numpy as np


def _stencil_csr(shape, offsets, weights):
    """CSR of a constant-coefficient stencil operator on a grid with Dirichlet
    boundary: entry (i, i+off) exists when the neighbour lies inside."""
    dims = np.array(shape)
    n = int(np.prod(dims))
    idx = np.arange(n, dtype=np.int64)
    coords = np.unravel_index(idx, shape)
    cols, vals, valid = [], [], []
    for off, w in zip(offsets, weights):
        ok = np.ones(n, bool)
        lin = np.zeros(n, np.int64)
        stride = 1
        for ax in reversed(range(len(shape))):
            c = coords[ax] + off[ax]
            ok &= (c >= 0) & (c < shape[ax])
            lin += np.clip(c, 0, shape[ax] - 1) * stride
            stride *= shape[ax]
        cols.append(lin)
        vals.append(np.full(n, w, np.float64))
        valid.append(ok)
    order = np.argsort([sum(o[a] * int(np.prod(shape[a + 1:])) for a in range(len(shape))) for o in offsets])
    C = np.stack([cols[k] for k in order], axis=1)
    Vv = np.stack([vals[k] for k in order], axis=1)
    M = np.stack([valid[k] for k in order], axis=1)
    counts = M.sum(axis=1)
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    return row_ptr.astype(np.int32), C[M].astype(np.int32), Vv[M]


def laplacian_2d(n: int):
    offs = [(-1, 0), (0, -1), (0, 0), (0, 1), (1, 0)]
    return _stencil_csr((n, n), offs, [-1.0, -1.0, 4.0, -1.0, -1.0])


def laplacian_3d(n: int):
    offs = [(-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0)]
    return _stencil_csr((n, n, n), offs, [-1.0, -1.0, -1.0, 6.0, -1.0, -1.0, -1.0])


def _powerlaw_alpha(target_mean: float, lo: int, hi: int) -> float:
    d = np.arange(lo, hi + 1, dtype=np.float64)
    a_lo, a_hi = 0.0, 5.0
    for _ in range(60):
        a = 0.5 * (a_lo + a_hi)
        p = d ** -a
        m = (d * p).sum() / p.sum()
        if m > target_mean:
            a_lo = a
        else:
            a_hi = a
    return 0.5 * (a_lo + a_hi)


def random_spd(n: int, seed: int = 0, lo: int = 3, hi: int = 60, mean_degree: float = 14.0):
    """Random strictly diagonally dominant symmetric matrix in CSR (float64).

    Each row draws a target degree from a power law on [lo, hi]; half of it is
    spent on random partners, and symmetrisation supplies the other half, so
    the mean off-diagonal degree lands near `mean_degree`."""
    rng = np.random.default_rng(seed)
    d = np.arange(lo, hi + 1)
    alpha = _powerlaw_alpha(mean_degree, lo, hi)
    p = d.astype(np.float64) ** -alpha
    p /= p.sum()
    deg = rng.choice(d, size=n, p=p)
    out_deg = (deg + 1) // 2
    rows = np.repeat(np.arange(n, dtype=np.int64), out_deg)
    cols = rng.integers(0, n, size=rows.size, dtype=np.int64)
    keep = rows != cols
    rows, cols = rows[keep], cols[keep]
    a = np.minimum(rows, cols)
    b = np.maximum(rows, cols)
    key = np.unique(a * n + b)
    a, b = key // n, key % n
    w = rng.standard_normal(a.size)
    r = np.concatenate([a, b])
    c = np.concatenate([b, a])
    v = np.concatenate([w, w])
    # bincount adds the weights in array order, as np.add.at would
    diag = np.bincount(r, weights=np.abs(v), minlength=n)
    diag += rng.uniform(0.1, 1.0, n)
    r = np.concatenate([r, np.arange(n)])
    c = np.concatenate([c, np.arange(n)])
    v = np.concatenate([v, diag])
    order = np.argsort(r * n + c)  # (row, column) keys are unique: the row-major order
    r, c, v = r[order], c[order], v[order]
    row_ptr = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=row_ptr[1:])
    return row_ptr.astype(np.int32), c.astype(np.int32), v


def csr_to_dia(row_ptr, col, val, max_diags: int = 32):
    """Diagonal-major DIA: (offsets[int32], data[ndiag][n])."""
    n = len(row_ptr) - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
    off = col.astype(np.int64) - rows
    offsets = np.unique(off)
    if offsets.size > max_diags:
        raise ValueError(f"{offsets.size} diagonals (max {max_diags})")
    k = np.searchsorted(offsets, off)
    data = np.zeros((offsets.size, n), dtype=val.dtype)
    data[k, rows] = val
    return offsets.astype(np.int32), data


def shifted(row_ptr, col, val, shift: float):
    """A + shift*I (the batched workload's random diagonal shift)."""
    n = len(row_ptr) - 1
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    v = val.copy()
    v[rows == col] += shift
    return row_ptr, col, v


def read_mtx(path: str):
    """A MatrixMarket file as CSR (row_ptr int32, col int32, val float64),
    read by the library the way the reference's CooMatrix::InitMarket and
    CsrMatrix::Init read it (symmetric entries mirrored, rows and columns
    sorted, duplicates kept, pattern values 1.0). Host only."""
    import ctypes

    from . import _native as N
    L = N.lib()
    rows, cols, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
    b = str(path).encode()
    N.check(L.perks_mtx_size(b, ctypes.byref(rows), ctypes.byref(cols), ctypes.byref(nnz)))
    rp = np.zeros(rows.value + 1, np.int32)
    ci = np.zeros(max(nnz.value, 1), np.int32)
    val = np.zeros(max(nnz.value, 1), np.float64)
    got = ctypes.c_longlong()
    N.check(L.perks_mtx_read_csr(b, rows.value, nnz.value, rp.ctypes.data, ci.ctypes.data, val.ctypes.data,
                                 ctypes.byref(got)))
    return rp, ci[:got.value], val[:got.value]
