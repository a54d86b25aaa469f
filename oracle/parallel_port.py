"""The oracle's scalar pipeline (assembly + right-hand side + Dirichlet +
Jacobi-PCG) split over the host's cores, for timing the reference algorithm
on the full-size bench workload.

TEST INFRASTRUCTURE AND CPU TIMING ONLY: used by ``bench.py --impl reference``
(the reference arm) and by ``tests/``; the product never imports it.

The work is split by row ranges of the global matrix.  A process takes a range
[r0, r1), computes the local matrices of the cells that touch it
(``fem_oracle.diffusion_local`` / ``mass_local``, the restatement of
fealpy/fem/scalar_diffusion_integrator.py:54-63 and
fealpy/fem/scalar_mass_integrator.py:47-54), keeps the COO triplets whose row
lies in the range in the order FEALPy's ``_scalar_assembly`` lays them out
(fealpy/fem/bilinear_form.py:46-75: cell, then local row, then local column),
and coalesces them with the same stable lexsort + ``np.add.at``
(fealpy/sparse/coo_tensor.py:184-213).  The relative order of the triplets of
any (row, column) pair is the same as in the global sort, so every value is
summed in the same order as the sequential oracle: the concatenated ranges are
the sequential result bit for bit.  The right-hand side and the Dirichlet
elimination (fealpy/fem/dirichlet_bc.py:101-229) are done per range the same
way.  The CG loop (fealpy/solver/cg.py:76-123) runs in the parent with the
matrix-vector product computed by one thread per row block (scipy's CSR
product releases the GIL); each row is summed in CSR order as in a single
product, so the iterates equal the sequential oracle's.
"""
import os
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.sparse as sp

from oracle import fem_oracle as O

_CACHE = {}


def _problem(kind, n):
    """Set-up of one worker (cached): mesh, topology, dof map, boundary flags."""
    key = (kind, n)
    if key in _CACHE:
        return _CACHE[key]
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    if kind != "c2":
        raise ValueError(kind)
    node, cell, kappa = diffusion_mass_tet_box(n)
    topo = O.construct(cell)
    NN = node.shape[0]
    c2d = O.cell_to_dof(cell, topo, NN, 2)
    N = O.n_global_dofs(cell, topo, NN, 2)
    is_bd = O.boundary_dof_flag(cell, topo, c2d, 2, N)
    _CACHE.clear()
    _CACHE[key] = (node, cell, kappa, c2d, N, is_bd)
    return _CACHE[key]


def _coalesce_rows(I, J, V, r0, r1):
    """Stable lexsort + add.at of triplets whose rows lie in [r0, r1)."""
    order = np.lexsort((J, I))
    I, J, V = I[order], J[order], V[order]
    unique = np.concatenate([[True], (I[1:] != I[:-1]) | (J[1:] != J[:-1])]) if I.size else np.zeros(0, bool)
    idx = np.cumsum(unique) - 1
    vals = np.zeros(int(unique.sum()))
    np.add.at(vals, idx, V)
    rows, cols = I[unique], J[unique]
    crow = np.concatenate([[0], np.cumsum(np.bincount(rows - r0, minlength=r1 - r0))]).astype(np.int64)
    return crow, cols.astype(np.int32), vals


def range_pipeline(kind, n, r0, r1, q=4):
    """Rows [r0, r1) of the pre- and post-Dirichlet CSR and of the right-hand
    sides (f = 1, u = 0).  Returns a dict; ``setup_s`` is the time spent on the
    cached set-up (non-zero only on a worker's first call)."""
    t0 = time.perf_counter()
    node, cell, kappa, c2d, N, is_bd = _problem(kind, n)
    t1 = time.perf_counter()
    touch = np.nonzero(np.any((c2d >= r0) & (c2d < r1), axis=1))[0]
    sub = cell[touch]
    sc2d = c2d[touch]
    K = O.diffusion_local(node, sub, 2, q, kappa[touch]) + O.mass_local(node, sub, 2, q, 1.0)
    I = np.broadcast_to(sc2d[:, :, None], K.shape).ravel()
    J = np.broadcast_to(sc2d[:, None, :], K.shape).ravel()
    V = K.ravel()
    keep = (I >= r0) & (I < r1)
    crow, col, val = _coalesce_rows(I[keep], J[keep], V[keep], r0, r1)
    # right-hand side f = 1 (fealpy/fem/linear_form.py:36-86, scalar_source_integrator.py:51-58)
    bcs, ws = O._rule(3, 2, q)
    cm = O.simplex_measure(sub, node)
    phi = O.simplex_shape_function(bcs, 2)
    # the same contraction as fem_oracle.source_vector (same summation order)
    loc = np.einsum("c, q, qi, cq -> ci", cm, ws, phi, np.ones((sub.shape[0], bcs.shape[0])), optimize=True)
    F = np.zeros(r1 - r0)
    m = (sc2d >= r0) & (sc2d < r1)
    np.add.at(F, sc2d[m] - r0, loc[m])
    # Dirichlet u = 0: boundary rows and columns removed, unit diagonal on
    # boundary rows, f[bd] = 0 (f - A u = f for u = 0)
    rows = np.repeat(np.arange(r0, r1), np.diff(crow))
    k2 = (~is_bd[rows]) & (~is_bd[col])
    bd_rows = np.nonzero(is_bd[r0:r1])[0] + r0
    r2 = np.concatenate([rows[k2], bd_rows])
    c2 = np.concatenate([col[k2], bd_rows])
    v2 = np.concatenate([val[k2], np.ones(bd_rows.size)])
    o2 = np.lexsort((c2, r2))
    r2, c2, v2 = r2[o2], c2[o2], v2[o2]
    bcrow = np.concatenate([[0], np.cumsum(np.bincount(r2 - r0, minlength=r1 - r0))]).astype(np.int64)
    Fb = F.copy()
    Fb[is_bd[r0:r1]] = 0.0
    t2 = time.perf_counter()
    return {"r0": r0, "r1": r1, "crow": crow, "col": col, "val": val, "F": F, "bc_crow": bcrow,
            "bc_col": c2.astype(np.int32), "bc_val": v2, "bc_F": Fb, "N": N, "setup_s": t1 - t0,
            "work_s": t2 - t1}


def _task(args):
    return range_pipeline(*args)


def row_ranges(N, parts):
    b = np.linspace(0, N, parts + 1).astype(np.int64)
    return [(int(b[k]), int(b[k + 1])) for k in range(parts) if b[k + 1] > b[k]]


def assemble(pool, kind, n, N, parts, keep_pre=False):
    """All row ranges through ``pool`` (a process pool); returns the
    post-Dirichlet blocks, the right-hand side and per-stage seconds."""
    t0 = time.perf_counter()
    outs = pool.map(_task, [(kind, n, r0, r1) for r0, r1 in row_ranges(N, parts)], chunksize=1)
    t1 = time.perf_counter()
    blocks = [sp.csr_matrix((o["bc_val"], o["bc_col"], o["bc_crow"]), shape=(o["r1"] - o["r0"], N)) for o in outs]
    b = np.concatenate([o["bc_F"] for o in outs])
    res = {"blocks": blocks, "b": b, "bounds": [(o["r0"], o["r1"]) for o in outs], "assembly_s": t1 - t0,
           "setup_s": max(o["setup_s"] for o in outs)}
    if keep_pre:
        res["pre"] = outs
    return res


class BlockOperator:
    """y = A x by one thread per row block (row sums in CSR order, as scipy's
    single product)."""

    def __init__(self, blocks, bounds, threads):
        self.blocks, self.bounds = blocks, bounds
        self.ex = ThreadPoolExecutor(max(1, threads))
        self.n = bounds[-1][1]

    def __matmul__(self, x):
        y = np.empty(self.n)

        def run(k):
            r0, r1 = self.bounds[k]
            y[r0:r1] = self.blocks[k] @ x

        list(self.ex.map(run, range(len(self.blocks))))
        return y

    def diagonal(self):
        return np.concatenate([blk.diagonal(k=r0) for blk, (r0, _) in zip(self.blocks, self.bounds)])

    def close(self):
        self.ex.shutdown()


def jacobi_cg(A, b, atol=1e-30, rtol=1e-10, maxit=100000):
    """fealpy/solver/cg.py:76-123 with M = diag(A)^-1, the products through
    ``A @ x`` (a BlockOperator here), in the oracle's arithmetic."""
    d = A.diagonal()
    dinv = 1.0 / d
    info = {"residual": 0.0, "niter": 0}
    if np.linalg.norm(b) < 1e-15:
        return np.zeros_like(b), info
    x = np.zeros_like(b)
    r = b - A @ x
    z = dinv * r
    p = z
    b_norm = np.linalg.norm(b)
    rTr = np.sum(r * z)
    n_iter = 0
    while True:
        Ap = A @ p
        alpha = rTr / np.sum(p * Ap)
        x = x + alpha * p
        r_new = r - alpha * Ap
        z_new = dinv * r_new
        rTr_new = np.sum(r_new * z_new)
        r_norm_new = np.sqrt(rTr_new)
        n_iter += 1
        info["residual"] = r_norm_new
        info["niter"] = n_iter
        if r_norm_new < atol or r_norm_new < rtol * b_norm or (maxit is not None and n_iter >= maxit):
            break
        beta = rTr_new / rTr
        p = z_new + beta * p
        r, z, rTr = r_new, z_new, rTr_new
    return x, info


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1
