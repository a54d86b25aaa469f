"""CPU oracle for the FEALPy Lagrange assemble + Dirichlet + Jacobi-PCG path.

TEST INFRASTRUCTURE ONLY.  This module is a plain numpy/scipy restatement of
the reference algorithm, used as the checker by ``tests/``,
``__graft_entry__.smoke()`` and as the CPU baseline in ``bench.py``.  The
product (``fealpy_gb300``) never imports it.  Its own correctness is pinned
against fixtures produced by running the reference itself
(``tests/golden/make_golden.py``; see ``tests/test_oracle_golden.py``).

Every function follows the reference step by step, citing the file:line it
restates (paths inside the FEALPy checkout).  The quadrature tables are taken
from ``fealpy_gb300.quadrature`` (pure data, pinned against the reference's own
tables by the same tests).
"""
from itertools import combinations_with_replacement
from math import factorial

import numpy as np
import scipy.sparse as sp

from fealpy_gb300.quadrature import simplex_quadrature

TRI_LOCAL_EDGE = np.array([(1, 2), (2, 0), (0, 1)])
TET_LOCAL_EDGE = np.array([(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)])
TET_LOCAL_FACE = np.array([(1, 2, 3), (0, 3, 2), (0, 1, 3), (0, 2, 1)])


# --------------------------------------------------------------------------- meshes
def tri_from_box(box, nx, ny):
    """fealpy/mesh/triangle_mesh.py:1387-1435"""
    x = np.linspace(box[0], box[1], nx + 1)
    y = np.linspace(box[2], box[3], ny + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    node = np.concatenate((X.reshape(-1, 1), Y.reshape(-1, 1)), axis=1)
    idx = np.arange((nx + 1) * (ny + 1), dtype=np.int32).reshape(nx + 1, ny + 1)
    cell0 = np.concatenate((idx[1:, 0:-1].T.reshape(-1, 1), idx[1:, 1:].T.reshape(-1, 1),
                            idx[0:-1, 0:-1].T.reshape(-1, 1)), axis=1)
    cell1 = np.concatenate((idx[0:-1, 1:].T.reshape(-1, 1), idx[0:-1, 0:-1].T.reshape(-1, 1),
                            idx[1:, 1:].T.reshape(-1, 1)), axis=1)
    return node, np.concatenate((cell0, cell1), axis=0)


def tet_from_box(box, nx, ny, nz):
    """fealpy/mesh/tetrahedron_mesh.py:1017-1056 (6 Kuhn tetrahedra per cube)"""
    x = np.linspace(box[0], box[1], nx + 1)
    y = np.linspace(box[2], box[3], ny + 1)
    z = np.linspace(box[4], box[5], nz + 1)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    node = np.concatenate((X.reshape(-1, 1), Y.reshape(-1, 1), Z.reshape(-1, 1)), axis=1)
    NN = (nx + 1) * (ny + 1) * (nz + 1)
    idx = np.arange(NN, dtype=np.int32).reshape(nx + 1, ny + 1, nz + 1)
    nyz = (ny + 1) * (nz + 1)
    c0 = idx[:-1, :-1, :-1]
    c1 = c0 + nyz
    c2 = c1 + nz + 1
    c3 = c0 + nz + 1
    c4 = c0 + 1
    c5 = c4 + nyz
    c6 = c5 + nz + 1
    c7 = c4 + nz + 1
    cube = np.concatenate([c.reshape(-1, 1) for c in (c0, c1, c2, c3, c4, c5, c6, c7)], axis=1)
    local = np.array([[0, 1, 2, 6], [0, 5, 1, 6], [0, 4, 5, 6], [0, 7, 4, 6], [0, 3, 7, 6], [0, 2, 3, 6]])
    return node, cube[:, local].reshape(-1, 4)


def flocc(array):
    """fealpy/mesh/utils.py:81-110: first/last occurrence of unique rows."""
    indices = np.lexsort(tuple(reversed(array.T)), axis=0)
    sorted_array = array[indices]
    diff_flag = np.any(sorted_array[1:] != sorted_array[:-1], axis=1)
    diff_flag = np.concatenate([[True], diff_flag, [True]])
    group_index = np.cumsum(diff_flag[:-1]) - 1
    i0 = indices[diff_flag[:-1]]
    i1 = indices[diff_flag[1:]]
    j = np.empty_like(indices)
    j[indices] = np.arange(len(indices))
    return i0, i1, group_index[j]


def construct(cell):
    """fealpy/mesh/mesh_data_structure.py:428-464"""
    NC, NV = cell.shape
    local_face = TRI_LOCAL_EDGE if NV == 3 else TET_LOCAL_FACE
    NFC = local_face.shape[0]
    total_face = cell[:, local_face].reshape(-1, local_face.shape[1])
    i0, i1, j = flocc(np.sort(total_face, axis=1))
    topo = {"face": total_face[i0], "cell2face": j.reshape(NC, NFC),
            "face2cell": np.stack([i0 // NFC, i1 // NFC, i0 % NFC, i1 % NFC], axis=-1)}
    if NV == 4:
        total_edge = cell[:, TET_LOCAL_EDGE].reshape(-1, 2)
        i2, _, je = flocc(np.sort(total_edge, axis=1))
        topo["edge"] = total_edge[i2]
        topo["cell2edge"] = je.reshape(NC, 6)
    else:
        topo["edge"] = topo["face"]
        topo["cell2edge"] = topo["cell2face"]
    return topo


def multi_index_matrix(p, dim):
    """fealpy/backend/numpy_backend.py:357-365"""
    sep = np.flip(np.array(tuple(combinations_with_replacement(range(p + 1), dim)), dtype=np.int32), axis=0)
    raw = np.zeros((sep.shape[0], dim + 2), dtype=np.int32)
    raw[:, -1] = p
    raw[:, 1:-1] = sep
    return raw[:, 1:] - raw[:, :-1]


def edge_to_ipoint(edge, NN, p):
    """fealpy/mesh/mesh_base.py:188-210"""
    NE = edge.shape[0]
    idx = np.arange(NE)
    return np.concatenate([edge[:, :1], (p - 1) * idx[:, None] + np.arange(p - 1) + NN, edge[:, 1:]], axis=-1)


def tri_cell_to_ipoint(cell, topo, NN, p):
    """fealpy/mesh/triangle_mesh.py:218-270 (the face2cell flip logic)."""
    if p == 1:
        return cell.copy()
    mi = multi_index_matrix(p, 2)
    idx0 = np.nonzero(mi[:, 0] == 0)[0]
    idx1 = np.nonzero(mi[:, 1] == 0)[0]
    idx2 = np.nonzero(mi[:, 2] == 0)[0]
    f2c = topo["face2cell"]
    NE = topo["edge"].shape[0]
    NC = cell.shape[0]
    e2p = edge_to_ipoint(topo["edge"], NN, p)
    ldof = (p + 1) * (p + 2) // 2
    c2p = np.zeros((NC, ldof), dtype=np.int64)
    flag = f2c[:, 2] == 0
    c2p[f2c[flag, 0][:, None], idx0] = e2p[flag]
    flag = f2c[:, 2] == 1
    c2p[f2c[flag, 0][:, None], np.flip(idx1)] = e2p[flag]
    flag = f2c[:, 2] == 2
    c2p[f2c[flag, 0][:, None], idx2] = e2p[flag]
    iflag = f2c[:, 0] != f2c[:, 1]
    flag = iflag & (f2c[:, 3] == 0)
    c2p[f2c[flag, 1][:, None], np.flip(idx0)] = e2p[flag]
    flag = iflag & (f2c[:, 3] == 1)
    c2p[f2c[flag, 1][:, None], idx1] = e2p[flag]
    flag = iflag & (f2c[:, 3] == 2)
    c2p[f2c[flag, 1][:, None], np.flip(idx2)] = e2p[flag]
    cdof = (p - 1) * (p - 2) // 2
    flag = np.sum(mi > 0, axis=1) == 3
    c2p[:, flag] = NN + NE * (p - 1) + np.arange(NC * cdof).reshape(NC, cdof)
    return c2p


def tet_cell_to_ipoint(cell, topo, NN, p):
    """fealpy/mesh/tetrahedron_mesh.py:388-441 for p <= 2: vertices, then the
    edge midpoints NN + edge index."""
    if p == 1:
        return cell.copy()
    if p != 2:
        raise NotImplementedError
    mi = multi_index_matrix(2, 3)
    c2p = np.zeros((cell.shape[0], 10), dtype=np.int64)
    lookup = {tuple(e): k for k, e in enumerate(TET_LOCAL_EDGE.tolist())}
    for k, m in enumerate(mi):
        nz = np.nonzero(m)[0]
        if len(nz) == 1:
            c2p[:, k] = cell[:, nz[0]]
        else:
            c2p[:, k] = NN + topo["cell2edge"][:, lookup[(nz[0], nz[1])]]
    return c2p


def cell_to_dof(cell, topo, NN, p):
    return tri_cell_to_ipoint(cell, topo, NN, p) if cell.shape[1] == 3 else tet_cell_to_ipoint(cell, topo, NN, p)


def n_global_dofs(cell, topo, NN, p):
    NE = topo["edge"].shape[0]
    NC = cell.shape[0]
    if cell.shape[1] == 3:
        return NN + NE * (p - 1) + NC * (p - 1) * (p - 2) // 2
    NF = topo["face"].shape[0]
    return NN + NE * (p - 1) + NF * (p - 1) * (p - 2) // 2 + NC * (p - 1) * (p - 2) * (p - 3) // 6


# ------------------------------------------------------------------ basis/geometry
def simplex_shape_function(bc, p):
    """fealpy/backend/numpy_backend.py:424-440 (cumulative-product recipe)."""
    TD = bc.shape[-1] - 1
    mi = multi_index_matrix(p, TD)
    c = np.arange(1, p + 1)
    P = 1.0 / np.multiply.accumulate(c)
    t = np.arange(0, p)
    A = np.ones(bc.shape[:-1] + (p + 1, TD + 1))
    A[..., 1:, :] = p * bc[..., None, :] - t.reshape(-1, 1)
    A = np.cumprod(A, axis=-2)
    A[..., 1:, :] *= P.reshape(-1, 1)
    return np.prod(A[..., mi, np.arange(TD + 1)], axis=-1)


def simplex_grad_shape_function(bc, p):
    """fealpy/backend/numpy_backend.py:443-477 -> (NQ, ldof, TD+1)."""
    TD = bc.shape[-1] - 1
    mi = multi_index_matrix(p, TD)
    ldof = mi.shape[0]
    c = np.arange(1, p + 1)
    P = 1.0 / np.multiply.accumulate(c)
    t = np.arange(0, p)
    shape = bc.shape[:-1] + (p + 1, TD + 1)
    A = np.ones(shape)
    A[..., 1:, :] = p * bc[..., None, :] - t.reshape(-1, 1)
    FF = np.einsum("...jk, m->...kjm", A[..., 1:, :], np.ones(p))
    FF[..., range(p), range(p)] = p
    FF = np.cumprod(FF, axis=-2)
    F = np.zeros(shape)
    F[..., 1:, :] = np.sum(np.tril(FF), axis=-1).swapaxes(-1, -2)
    F[..., 1:, :] *= P.reshape(-1, 1)
    A = np.cumprod(A, axis=-2)
    A[..., 1:, :] *= P.reshape(-1, 1)
    Q = A[..., mi, range(TD + 1)]
    M = F[..., mi, range(TD + 1)]
    R = np.zeros(bc.shape[:-1] + (ldof, TD + 1))
    for i in range(TD + 1):
        idx = list(range(TD + 1))
        idx.remove(i)
        R[..., i] = M[..., i] * np.prod(Q[..., idx], axis=-1)
    return R


def simplex_measure(cell, node):
    """fealpy/backend/numpy_backend.py:414-421 (signed)."""
    pts = node[cell]
    TD = pts.shape[-2] - 1
    edges = pts[..., 1:, :] - pts[..., :-1, :]
    return np.linalg.det(edges) / factorial(TD)


def grad_lambda(cell, node):
    """fealpy/backend/numpy_backend.py:587-598 (triangles) and :620-629 (tetrahedra)."""
    if cell.shape[1] == 3:
        pts = node[cell]
        e0 = pts[..., 2, :] - pts[..., 1, :]
        e1 = pts[..., 0, :] - pts[..., 2, :]
        e2 = pts[..., 1, :] - pts[..., 0, :]
        nv = np.linalg.det(np.stack([e0, e1], axis=-2))
        res = np.stack([np.flip(e0, -1), np.flip(e1, -1), np.flip(e2, -1)], axis=-2)
        res[..., 0] *= -1
        return res / nv[..., None, None]
    NC = cell.shape[0]
    vol = simplex_measure(cell, node)
    D = np.zeros((NC, 4, 3))
    for i in range(4):
        j, k, m = TET_LOCAL_FACE[i]
        vjk = node[cell[:, k]] - node[cell[:, j]]
        vjm = node[cell[:, m]] - node[cell[:, j]]
        D[:, i, :] = np.cross(vjm, vjk) / (6 * vol.reshape(-1, 1))
    return D


def _rule(TD, p, q):
    return simplex_quadrature(TD, p + 3 if q is None else q)


def diffusion_local(node, cell, p, q=None, coef=None):
    """ScalarDiffusionIntegrator.assembly (fealpy/fem/scalar_diffusion_integrator.py:54-63)
    -> bilinear_integral (fealpy/functional.py:68-106)."""
    TD = cell.shape[1] - 1
    bcs, ws = _rule(TD, p, q)
    cm = simplex_measure(cell, node)
    R = simplex_grad_shape_function(bcs, p)
    gphi = np.einsum("...bm, qjb -> ...qjm", grad_lambda(cell, node), R, optimize=True)
    K = np.einsum("q, c, cqid, cqjd -> cij", ws, cm, gphi, gphi, optimize=True)
    if coef is None:
        return K
    coef = np.asarray(coef, dtype=np.float64)
    return K * (coef if coef.ndim == 0 else coef[:, None, None])


def mass_local(node, cell, p, q=None, coef=None):
    """ScalarMassIntegrator.assembly (fealpy/fem/scalar_mass_integrator.py:47-54)."""
    TD = cell.shape[1] - 1
    bcs, ws = _rule(TD, p, q)
    cm = simplex_measure(cell, node)
    phi = simplex_shape_function(bcs, p)[None, ...]
    K = np.einsum("q, c, cqi, cqj -> cij", ws, cm, np.broadcast_to(phi, (cell.shape[0],) + phi.shape[1:]),
                  np.broadcast_to(phi, (cell.shape[0],) + phi.shape[1:]), optimize=True)
    if coef is None:
        return K
    coef = np.asarray(coef, dtype=np.float64)
    return K * (coef if coef.ndim == 0 else coef[:, None, None])


def elasticity_local(node, cell, lam, mu, q=None):
    """LinearElasticityIntegrator.assembly, interleaved (dof_priority=False) 3-D
    branch with D01 = lam, D55 = mu per cell
    (fealpy/fem/linear_elasticity_integrator.py:60-181)."""
    bcs, ws = _rule(3, 1, q)
    cm = simplex_measure(cell, node)
    R = simplex_grad_shape_function(bcs, 1)
    gphi = np.einsum("...bm, qjb -> ...qjm", grad_lambda(cell, node), R, optimize=True)
    A = [[np.einsum("q, cqi, cqj, c -> cij", ws, gphi[..., a], gphi[..., b], cm, optimize=True) for b in range(3)]
         for a in range(3)]
    NC, ldof = cell.shape
    KK = np.zeros((NC, 3 * ldof, 3 * ldof))
    D01 = np.broadcast_to(np.asarray(lam, dtype=np.float64), (NC,))[:, None, None]
    D55 = np.broadcast_to(np.asarray(mu, dtype=np.float64), (NC,))[:, None, None]
    for a in range(3):
        others = [b for b in range(3) if b != a]
        KK[:, a::3, a::3] = (2 * D55 + D01) * A[a][a] + D55 * (A[others[0]][others[0]] + A[others[1]][others[1]])
        for b in range(3):
            if b != a:
                KK[:, a::3, b::3] = D01 * A[a][b] + D55 * A[b][a]
    return KK


# ------------------------------------------------------------------ global assembly
def coalesce_to_csr(c2d, K, n):
    """BilinearForm._scalar_assembly (fealpy/fem/bilinear_form.py:46-75) +
    COOTensor.coalesce (fealpy/sparse/coo_tensor.py:184-213) + tocsr (:137-157).
    Returns the canonical CSR (rows and columns ascending)."""
    NC, ldof = c2d.shape
    I = np.broadcast_to(c2d[:, :, None], K.shape).ravel()
    J = np.broadcast_to(c2d[:, None, :], K.shape).ravel()
    V = K.ravel()
    order = np.lexsort((J, I))
    I, J, V = I[order], J[order], V[order]
    unique = np.concatenate([[True], (I[1:] != I[:-1]) | (J[1:] != J[:-1])])
    add_index = np.cumsum(unique) - 1
    vals = np.zeros(int(unique.sum()))
    np.add.at(vals, add_index, V)
    rows, cols = I[unique], J[unique]
    crow = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int64)
    return crow, cols.astype(np.int32), vals


def vector_elasticity_dofs(cell):
    """TensorFunctionSpace(space, (-1, 3)).cell_to_dof (fealpy/functionspace/utils.py:44)."""
    return (cell[:, :, None] * 3 + np.arange(3)[None, None, :]).reshape(cell.shape[0], -1)


def source_vector(node, cell, c2d, p, n, fvals_at_q, q=None):
    """LinearForm + ScalarSourceIntegrator (fealpy/fem/linear_form.py:36-86,
    fealpy/functional.py:27-65): fvals_at_q is (NC, NQ)."""
    TD = cell.shape[1] - 1
    bcs, ws = _rule(TD, p, q)
    cm = simplex_measure(cell, node)
    phi = simplex_shape_function(bcs, p)
    loc = np.einsum("c, q, qi, cq -> ci", cm, ws, phi, fvals_at_q, optimize=True)
    F = np.zeros(n)
    np.add.at(F, c2d, loc)
    return F


def bc_to_point(node, cell, bcs):
    return np.einsum("cvd,qv->cqd", node[cell], bcs)


# ------------------------------------------------------------------ Dirichlet
def boundary_dof_flag(cell, topo, c2d, p, n, face_mask=None):
    """LinearMeshCFEDof.is_boundary_dof, method 'centroid' (fealpy/functionspace/dofs.py:23-55):
    every dof of every boundary face (face2cell[:,0] == face2cell[:,1])."""
    f2c = topo["face2cell"]
    bd = np.nonzero(f2c[:, 0] == f2c[:, 1])[0]
    if face_mask is not None:
        bd = bd[face_mask(bd)]
    TD = cell.shape[1] - 1
    mi = multi_index_matrix(p, TD)
    flag = np.zeros(n, dtype=bool)
    for f in bd:
        c, lf = f2c[f, 0], f2c[f, 2]
        flag[c2d[c, mi[:, lf] == 0]] = True
    return flag


def dirichlet_apply(crow, col, val, is_bd, f, uh):
    """DirichletBC.apply (fealpy/fem/dirichlet_bc.py:101-229): f - A uh with
    f[bd] = uh[bd]; boundary rows/columns removed (_mul) and a unit diagonal
    added on boundary rows; the result is returned in canonical order."""
    n = len(crow) - 1
    A = sp.csr_matrix((val, col, crow), shape=(n, n))
    f_new = f - A @ uh
    f_new[is_bd] = uh[is_bd]
    is_in = ~is_bd
    row = np.repeat(np.arange(n), np.diff(crow))
    keep = is_in[row] & is_in[col]
    r2 = np.concatenate([row[keep], np.nonzero(is_bd)[0]])
    c2 = np.concatenate([col[keep], np.nonzero(is_bd)[0]])
    v2 = np.concatenate([val[keep], np.ones(int(is_bd.sum()))])
    order = np.lexsort((c2, r2))
    r2, c2, v2 = r2[order], c2[order], v2[order]
    crow2 = np.concatenate([[0], np.cumsum(np.bincount(r2, minlength=n))]).astype(np.int64)
    return (crow2, c2.astype(np.int32), v2), f_new


# ------------------------------------------------------------------ CG
def jacobi_cg(crow, col, val, b, atol=1e-12, rtol=1e-8, maxit=10000, use_jacobi=True, x0=None):
    """fealpy/solver/cg.py:76-123 with M = JacobiPreconditioner.apply(A)
    (fealpy/solver/iterative_solver_manger.py:273-280); SpMV through scipy's
    csr_matvec as the numpy backend does (fealpy/backend/numpy_backend.py:181-199)."""
    n = len(crow) - 1
    A = sp.csr_matrix((val, col, crow), shape=(n, n))
    if use_jacobi:
        d = A.diagonal()
        M = sp.csr_matrix((1.0 / d, np.arange(n), np.arange(n + 1)), shape=(n, n))
    else:
        M = None
    info = {"residual": 0.0, "niter": 0}
    if np.linalg.norm(b) < 1e-15:
        return np.zeros_like(b), info
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - A @ x
    z = M @ r if M is not None else r
    p = z
    b_norm = np.linalg.norm(b)
    rTr = np.sum(r * z)
    n_iter = 0
    while True:
        Ap = A @ p
        alpha = rTr / np.sum(p * Ap)
        x = x + alpha * p
        r_new = r - alpha * Ap
        z_new = M @ r_new if M is not None else r_new
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


# ------------------------------------------------------------------ pipelines
def poisson_pipeline(node, cell, p, kappa=None, rho=None, q=None, f_at_q=None, gd_dofs=None, rtol=1e-10,
                     maxit=100000, f_vec=None):
    """Full reference pipeline: assembly (diffusion [+ mass]) -> RHS -> BC -> Jacobi-PCG.
    ``f_vec``: a right-hand-side vector given per dof (instead of the source
    integral of ``f_at_q``, default f = 1).
    Returns a dict of every intermediate (used by the parity tests and the CPU baseline)."""
    topo = construct(cell)
    NN = node.shape[0]
    c2d = cell_to_dof(cell, topo, NN, p)
    n = n_global_dofs(cell, topo, NN, p)
    K = diffusion_local(node, cell, p, q, kappa)
    if rho is not None:
        K = K + mass_local(node, cell, p, q, rho)
    crow, col, val = coalesce_to_csr(c2d, K, n)
    TD = cell.shape[1] - 1
    bcs, _ = _rule(TD, p, q)
    if f_vec is not None:
        F = np.asarray(f_vec, dtype=np.float64).copy()
    else:
        fq = np.ones((cell.shape[0], bcs.shape[0])) if f_at_q is None else f_at_q(bc_to_point(node, cell, bcs))
        F = source_vector(node, cell, c2d, p, n, fq, q)
    is_bd = boundary_dof_flag(cell, topo, c2d, p, n)
    uh = np.zeros(n)
    if gd_dofs is not None:
        uh[is_bd] = gd_dofs[is_bd]
    (bcrow, bcol, bval), Fb = dirichlet_apply(crow, col, val, is_bd, F, uh)
    x, info = jacobi_cg(bcrow, bcol, bval, Fb, atol=1e-30, rtol=rtol, maxit=maxit)
    return {"c2d": c2d, "n": n, "crow": crow, "col": col, "val": val, "F": F, "is_bd": is_bd,
            "bc_crow": bcrow, "bc_col": bcol, "bc_val": bval, "bc_F": Fb, "x": x, "info": info}


def elasticity_pipeline(node, cell, lam, mu, q=4, force=(0.0, 0.0, -1.0), clamp=None, rtol=1e-10, maxit=100000):
    """P1 vector elasticity on tetrahedra, interleaved dofs (3 node + comp):
    LinearElasticityIntegrator local matrices (elasticity_local), coalesce to
    CSR, a constant body force through VectorSourceIntegrator
    (fealpy/fem/vector_source_integrator.py; the cell vector is
    sum_q w_q |T| phi_i f_d), Dirichlet u = 0 on the boundary nodes where
    ``clamp(node)`` holds (TensorFunctionSpace.is_boundary_dof, method 'interp',
    fealpy/functionspace/tensor_space.py:156-185: boundary-face dofs filtered
    at their interpolation points, the nodes for P1), Jacobi-PCG."""
    NN = node.shape[0]
    n = 3 * NN
    topo = construct(cell)
    c2d = vector_elasticity_dofs(cell)
    KK = elasticity_local(node, cell, lam, mu, q)
    crow, col, val = coalesce_to_csr(c2d, KK, n)
    bcs, ws = _rule(3, 1, q)
    cm = simplex_measure(cell, node)
    phi = simplex_shape_function(bcs, 1)
    loc = np.einsum("c, q, qi, d -> cid", cm, ws, phi, np.asarray(force, dtype=np.float64), optimize=True)
    F = np.zeros(n)
    np.add.at(F, c2d, loc.reshape(cell.shape[0], -1))
    node_bd = boundary_dof_flag(cell, topo, cell, 1, NN)
    if clamp is not None:
        node_bd &= np.asarray(clamp(node), dtype=bool)
    is_bd = np.repeat(node_bd, 3)
    (bcrow, bcol, bval), Fb = dirichlet_apply(crow, col, val, is_bd, F, np.zeros(n))
    x, info = jacobi_cg(bcrow, bcol, bval, Fb, atol=1e-30, rtol=rtol, maxit=maxit)
    return {"c2d": c2d, "n": n, "crow": crow, "col": col, "val": val, "F": F, "is_bd": is_bd,
            "bc_crow": bcrow, "bc_col": bcol, "bc_val": bval, "bc_F": Fb, "x": x, "info": info}
