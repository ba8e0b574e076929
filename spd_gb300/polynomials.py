"""Setup-time 1D operators of the SD-ADER scheme (host, FP64, NumPy).

These build the small constant matrices the CUDA kernels apply: the
solution and flux points of a spectral-difference cell, Lagrange
interpolation and derivative matrices, the subcell-average matrix and the
ADER time matrix.  They follow the definitions in the reference's
src/polynomials.py (line numbers per function) with the same floating-point
operation sequence, so the matrices are the same bits on the same platform.
"""
from __future__ import annotations

import concurrent.futures
import os
from typing import Callable, Tuple

import numpy as np


def gauss_legendre_quadrature(x0: float, x1: float, p: int) -> Tuple[np.ndarray, np.ndarray]:
    """p Gauss-Legendre nodes and weights on [x0, x1] (src/polynomials.py:5-17)."""
    if p == 0:
        return np.ndarray(0), np.ndarray(0)
    x, w = np.polynomial.legendre.leggauss(p)
    return x0 + (x + 1.0) * (x1 - x0) / 2.0, w * (x1 - x0) / 2.0


def solution_points(x0: float, x1: float, p: int) -> np.ndarray:
    """p+1 Chebyshev-Gauss points on [x0, x1] (src/polynomials.py:19-31)."""
    i = np.arange(p + 1)
    return x0 + (1.0 - np.cos((2 * i + 1) / (2 * (p + 1)) * np.pi)) * (x1 - x0) / 2.0


def flux_points(x0: float, x1: float, p: int) -> np.ndarray:
    """The p Gauss-Legendre nodes plus both end points (src/polynomials.py:33-44)."""
    x, _ = gauss_legendre_quadrature(x0, x1, p)
    return np.hstack((x0, x, x1))


def lagrange_matrix(x_to: np.ndarray, x_from: np.ndarray) -> np.ndarray:
    """(len(x_to), len(x_from)) Lagrange interpolation matrix (src/polynomials.py:46-65)."""
    nt, nf = x_to.shape[0], x_from.shape[0]
    diff = np.broadcast_to(x_to[:, None, None] - x_from[None, None, :], (nt, nf, nf)).copy()
    diff[:, np.arange(nf), np.arange(nf)] = 1.0
    den = x_from[:, None] - x_from[None, :]
    np.fill_diagonal(den, 1.0)
    return diff.prod(axis=-1) / den.prod(axis=-1)[None, :]


def lagrangeprime_matrix(x_to: np.ndarray, x_from: np.ndarray) -> np.ndarray:
    """Derivatives of the Lagrange basis on x_from at x_to (src/polynomials.py:67-88)."""
    nt, nf = x_to.shape[0], x_from.shape[0]
    diff = np.broadcast_to(x_to[:, None, None, None] - x_from[None, None, None, :], (nt, nf, nf, nf)).copy()
    a = np.arange(nf)
    diff[:, a, :, a] = 1.0
    diff[:, :, a, a] = 1.0
    den = x_from[:, None] - x_from[None, :]
    np.fill_diagonal(den, 1.0)
    terms = diff.prod(axis=-1) / den.prod(axis=-1)[None, :, None]
    terms[:, a, a] = 0.0
    return terms.sum(axis=-1)


def intfromsol_matrix(x_sp: np.ndarray, x_fp: np.ndarray) -> np.ndarray:
    """Point values -> averages over the control volumes bounded by x_fp
    (src/polynomials.py:90-107)."""
    m = x_fp.shape[0] - x_sp.shape[0]
    n = x_sp.shape[0] - 1
    if n == 0:
        return np.ones((1, 1))
    x, w = gauss_legendre_quadrature(0.0, 1.0, n)
    xi = (x_fp[:-1, None] + np.diff(x_fp)[:, None] * x[None, :]).ravel()
    lm = lagrange_matrix(xi, x_sp).reshape(n + m, n, n + 1)
    return np.einsum("ijk,j->ik", lm, w)


def ader_matrix(x_time: np.ndarray, w_time: np.ndarray, dt: float) -> np.ndarray:
    """ADER time matrix on [0, dt] (src/polynomials.py:109-122)."""
    ltm = lagrange_matrix(np.array([dt]), x_time).ravel()
    lpm = lagrangeprime_matrix(x_time, x_time)
    return ltm[None, :] * ltm[:, None] - lpm.T * w_time[None, :]


def quadrature_points(mesh: np.ndarray, d: int, light: bool = True):
    """Tensor Gauss-Legendre points of every control volume of ``mesh`` and
    the 1D weights (src/polynomials.py:124-148).  The points do not depend
    on the variable, so a caller sampling several variables builds them
    once.  The returned point array is read-only."""
    nq = 2 if light else max(mesh.shape[-d:]) - 1
    x, w = gauss_legendre_quadrature(0.0, 1.0, nq)
    pts = mesh[(Ellipsis,) + (slice(-1),) * d + (np.newaxis,) * d]
    pts = np.broadcast_to(pts, pts.shape[:-d] + (nq,) * d).copy()
    for i in range(d):
        edges = mesh[(Ellipsis,) + (slice(-1),) * i + (slice(None),) + (slice(-1),) * (d - i - 1)]
        pts += (np.diff(edges, axis=(i - d))[(Ellipsis,) + (np.newaxis,) * d]
                * x[(np.newaxis,) * len(mesh.shape) + (np.newaxis,) * i + (slice(None),) + (np.newaxis,) * (d - i - 1)])
    pts.setflags(write=False)
    return pts, w


def quadrature_mean(mesh: np.ndarray, fct: Callable, d: int, v: int, light: bool = True,
                    points=None, workers: int = 1) -> np.ndarray:
    """Cell means of fct(x, v) over the control volumes of ``mesh`` with a
    tensor Gauss-Legendre rule (src/polynomials.py:124-148).  ``points`` is
    the result of quadrature_points(mesh, d, light) when already built.
    fct is called once on all points, as in the reference; with workers > 1
    the weighted sums run on thread slabs of cells (the same sum per cell)."""
    pts, w = points if points is not None else quadrature_points(mesh, d, light)
    vals = fct(pts, v)

    def mean(block):
        args = [block, (Ellipsis,) + tuple(range(d))]
        for i in range(d):
            args.extend([w, (i,)])
        return np.einsum(*args)

    return _on_slabs(mean, vals, workers)


def _on_slabs(fn, arr: np.ndarray, workers: int) -> np.ndarray:
    """fn(arr) computed as fn of slabs of the leading axis on host threads
    (NumPy releases the GIL in its loops); fn must act on each index of that
    axis on its own, so that the result is the same array, bit for bit."""
    n0 = arr.shape[0]
    if workers < 2 or n0 < 2:
        return fn(arr)
    bounds = np.linspace(0, n0, min(workers * 4, n0) + 1).astype(int)
    first = fn(arr[bounds[0]:bounds[1]])
    out = np.empty((n0,) + first.shape[1:], dtype=first.dtype)
    out[bounds[0]:bounds[1]] = first

    def one(k):
        out[bounds[k]:bounds[k + 1]] = fn(arr[bounds[k]:bounds[k + 1]])

    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(one, range(1, len(bounds) - 1)))
    return out


def quadrature_points_threaded(mesh: np.ndarray, d: int, light: bool = True, workers: int | None = None,
                               min_cells: int = 1 << 15):
    """quadrature_points on host thread slabs of the outermost cell axis
    (each point is formed from its own cell's edges only: the same bits)."""
    ncells = int(np.prod(mesh.shape[1:1 + d]))
    workers = workers or min(16, os.cpu_count() or 1)
    if ncells < min_cells or workers < 2:
        return quadrature_points(mesh, d, light)
    w = quadrature_points(mesh[:, :1], d, light)[1]
    moved = np.moveaxis(mesh, 1, 0)
    pts = _on_slabs(lambda m: np.moveaxis(quadrature_points(np.moveaxis(m, 0, 1), d, light)[0], 1, 0), moved,
                    workers)
    pts = np.ascontiguousarray(np.moveaxis(pts, 0, 1))
    pts.setflags(write=False)
    return pts, w


def transform_axis(B: np.ndarray, A: np.ndarray, idim: int, ndim: int, ader: bool = False) -> np.ndarray:
    """Apply the 1D operator A along the in-cell axis of direction idim of an
    SD-layout array (src/transforms.py:3-25)."""
    y = "y" if ndim > 1 else ""
    j = "j" if ndim > 1 else ""
    z = "z" if ndim > 2 else ""
    k = "k" if ndim > 2 else ""
    t = "t" if ader else ""
    u = f"u{t}{z}{y}x"
    if idim == 0:
        u += f"{k}{j}"
        return np.einsum(f"fs,{u}s->{u}f", A, B)
    if idim == 1 and ndim > 1:
        u += k
        return np.einsum(f"fs,{u}si->{u}fi", A, B)
    if idim == 2 and ndim > 2:
        return np.einsum(f"fs,{u}sji->{u}fji", A, B)
    raise TypeError("Wrong option for dim")


def transform_full(B: np.ndarray, A: np.ndarray, ndim: int) -> np.ndarray:
    """Apply A along every in-cell axis (src/transforms.py:27-45)."""
    if ndim == 3:
        return np.einsum("kn,jm,il,uzyxnml->uzyxkji", A, A, A, B)
    if ndim == 2:
        return np.einsum("jm,il,uyxml->uyxji", A, A, B)
    return np.einsum("il,uxl->uxi", A, B)


def transform_full_threaded(B: np.ndarray, A: np.ndarray, ndim: int, min_cells: int = 1 << 16,
                            workers: int | None = None) -> np.ndarray:
    """transform_full of a C-contiguous SD-layout array on several host
    threads: slabs of whole (variable, outermost cell row) blocks, each the
    same einsum on its slab (einsum releases the GIL).  Every output
    element is the same sum over its own cell's points as in one einsum of
    the whole array (bit-identical; checked in the CPU tests).  Arrays of
    fewer than ``min_cells`` cells take the single call."""
    ncells = int(np.prod(B.shape[1:1 + ndim]))
    workers = workers or min(16, os.cpu_count() or 1)
    if ncells < min_cells or workers < 2 or not B.flags.c_contiguous:
        return transform_full(B, A, ndim)
    flat = B.reshape((B.shape[0] * B.shape[1],) + B.shape[2:])
    out = np.empty_like(flat)
    bounds = np.linspace(0, flat.shape[0], min(workers * 4, flat.shape[0]) + 1).astype(int)

    def one(k):
        lo, hi = bounds[k], bounds[k + 1]
        if hi > lo:
            out[lo:hi] = transform_full(flat[lo:hi][:, None], A, ndim)[:, 0]

    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(one, range(len(bounds) - 1)))
    return out.reshape(B.shape)
