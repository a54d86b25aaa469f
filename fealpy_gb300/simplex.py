"""Lagrange basis on the reference simplex and the mesh-independent tables the
assembly kernels contract with per-cell factors.

Multi-indices follow FEALPy's ``multi_index_matrix`` ordering
(``fealpy/backend/numpy_backend.py:357-365``): all ``m`` with ``|m| = p``,
sorted descending lexicographically, so local dof ``k`` of a cell is the
interpolation point ``sum_v m_v x_v / p``.

The basis is the classical product form
``phi_m(lambda) = prod_v prod_{j<m_v} (p*lambda_v - j) / m_v!``; its gradient
with respect to the barycentric coordinates follows from the product rule.
"""
from functools import lru_cache
from math import factorial

import numpy as np

from .quadrature import simplex_quadrature

__all__ = ["multi_index_matrix", "shape_function", "grad_shape_function", "diffusion_tables",
           "mass_table", "metric_pairs", "local_face_of_multi_index"]


@lru_cache(maxsize=None)
def _multi_index(p: int, TD: int):
    out = []

    def rec(prefix, left, slots):
        if slots == 1:
            out.append(prefix + (left,))
            return
        for v in range(left, -1, -1):
            rec(prefix + (v,), left - v, slots - 1)

    rec((), p, TD + 1)
    return np.asarray(out, dtype=np.int32)


def multi_index_matrix(p: int, TD: int) -> np.ndarray:
    """All multi-indices of degree ``p`` in ``TD+1`` slots, FEALPy ordering."""
    return _multi_index(p, TD).copy()


def _factor_values(t: np.ndarray, p: int):
    """f_k(t) = prod_{j<k} (p t - j)/k! and f_k'(t) for k = 0..p; shapes (..., p+1)."""
    shape = t.shape + (p + 1,)
    f = np.ones(shape, dtype=np.float64)
    df = np.zeros(shape, dtype=np.float64)
    for k in range(1, p + 1):
        lin = p * t - (k - 1)
        # f_k = f_{k-1} * (p t - (k-1)) / k ; derivative by the product rule
        f[..., k] = f[..., k - 1] * lin / k
        df[..., k] = (df[..., k - 1] * lin + f[..., k - 1] * p) / k
    return f, df


def shape_function(bcs: np.ndarray, p: int) -> np.ndarray:
    """phi (NQ, ldof) at barycentric points ``bcs`` (NQ, TD+1)."""
    bcs = np.asarray(bcs, dtype=np.float64)
    TD = bcs.shape[-1] - 1
    mi = _multi_index(p, TD)
    f, _ = _factor_values(bcs, p)           # (NQ, TD+1, p+1)
    vals = np.ones((bcs.shape[0], mi.shape[0]))
    for v in range(TD + 1):
        vals *= f[:, v, mi[:, v]]
    return vals


def grad_shape_function(bcs: np.ndarray, p: int) -> np.ndarray:
    """d phi / d lambda (NQ, ldof, TD+1)."""
    bcs = np.asarray(bcs, dtype=np.float64)
    TD = bcs.shape[-1] - 1
    mi = _multi_index(p, TD)
    f, df = _factor_values(bcs, p)
    NQ, ldof = bcs.shape[0], mi.shape[0]
    out = np.empty((NQ, ldof, TD + 1))
    for v in range(TD + 1):
        g = df[:, v, mi[:, v]]
        for u in range(TD + 1):
            if u != v:
                g = g * f[:, u, mi[:, u]]
        out[:, :, v] = g
    return out


def metric_pairs(TD: int):
    """(k, l) pairs k <= l of the symmetric metric channels, in kernel channel order."""
    return [(k, l) for k in range(TD) for l in range(k, TD)]


@lru_cache(maxsize=None)
def _diffusion_tables(TD: int, p: int, q: int):
    bcs, ws = simplex_quadrature(TD, q)
    R = grad_shape_function(bcs, p)                 # (NQ, ldof, TD+1)
    Rr = R[:, :, 1:] - R[:, :, :1]                   # reduced: grad phi = sum_k Rr_k grad lambda_{k+1}
    S = np.einsum("q,qik,qjl->klij", ws, Rr, Rr)     # (TD, TD, ldof, ldof)
    tabs = []
    for k, l in metric_pairs(TD):
        tabs.append(S[k, k] if k == l else S[k, l] + S[l, k])
    T = np.stack(tabs, axis=0)
    return 0.5 * (T + T.transpose(0, 2, 1))   # exactly symmetric tables -> symmetric local matrices


@lru_cache(maxsize=None)
def _diffusion_tables_q(TD: int, p: int, q: int):
    bcs, ws = simplex_quadrature(TD, q)
    R = grad_shape_function(bcs, p)
    Rr = R[:, :, 1:] - R[:, :, :1]
    S = np.einsum("q,qik,qjl->qklij", ws, Rr, Rr)    # (NQ, TD, TD, ldof, ldof)
    tabs = []
    for iq in range(S.shape[0]):
        for k, l in metric_pairs(TD):
            tabs.append(S[iq, k, k] if k == l else S[iq, k, l] + S[iq, l, k])
    T = np.stack(tabs, axis=0)
    return 0.5 * (T + T.transpose(0, 2, 1))


def diffusion_tables_q(TD: int, p: int, q: int) -> np.ndarray:
    """Per-quadrature-point tables (NQ * n_metric, ldof, ldof), point-major:
    with a coefficient c_q given per point the diffusion local matrix is
    ``sum_q sum_t c_q G_t * T_{q,t}`` (``G_t`` as in :func:`diffusion_tables`)."""
    return _diffusion_tables_q(TD, p, q).copy()


@lru_cache(maxsize=None)
def _mass_tables_q(TD: int, p: int, q: int):
    bcs, ws = simplex_quadrature(TD, q)
    phi = shape_function(bcs, p)
    return np.einsum("q,qi,qj->qij", ws, phi, phi)


def mass_tables_q(TD: int, p: int, q: int) -> np.ndarray:
    """Per-quadrature-point mass tables (NQ, ldof, ldof): ``w_q phi_i phi_j``."""
    return _mass_tables_q(TD, p, q).copy()


def diffusion_tables(TD: int, p: int, q: int) -> np.ndarray:
    """Tables (n_metric, ldof, ldof) such that the diffusion local matrix is
    ``sum_t G_t * T_t`` with ``G_t = |T| kappa grad(l_{k+1}).grad(l_{l+1})``
    for the pairs of :func:`metric_pairs`.  Exactly the quadrature sum of
    ``fealpy/functional.py:bilinear_integral`` regrouped by metric entry."""
    return _diffusion_tables(TD, p, q).copy()


@lru_cache(maxsize=None)
def _mass_table(TD: int, p: int, q: int):
    bcs, ws = simplex_quadrature(TD, q)
    phi = shape_function(bcs, p)
    M = np.einsum("q,qi,qj->ij", ws, phi, phi)
    return (0.5 * (M + M.T))[None]


def mass_table(TD: int, p: int, q: int) -> np.ndarray:
    """Table (1, ldof, ldof): ``sum_q w_q phi_i phi_j`` (times |T| rho per cell)."""
    return _mass_table(TD, p, q).copy()


def local_face_of_multi_index(p: int, TD: int) -> np.ndarray:
    """Boolean (TD+1, ldof): local dof k lies on the facet opposite vertex v."""
    mi = _multi_index(p, TD)
    return (mi == 0).T.copy()


def simplex_ldof(p: int, TD: int) -> int:
    return factorial(p + TD) // (factorial(p) * factorial(TD))
