"""Host-side logic of the package on CPU tensors (no GPU): mesh topology, dof
numbering, boundary dofs and the factor x table decomposition the assembly
kernels evaluate, all checked against the reference's fixtures."""
import os

import numpy as np
import pytest
import torch

from fealpy_gb300 import simplex as sx
from fealpy_gb300.mesh import TriangleMesh, TetrahedronMesh
from fealpy_gb300.functionspace import LagrangeFESpace, TensorFunctionSpace


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def make_mesh(node, cell):
    node_t = torch.as_tensor(node)
    cell_t = torch.as_tensor(cell, dtype=torch.int32)
    return (TriangleMesh if cell.shape[1] == 3 else TetrahedronMesh)(node_t, cell_t)


def kernel_factors_numpy(node, cell):
    """What fgb_cell_factors computes: signed measure, grad(lambda_{1..TD})."""
    TD = cell.shape[1] - 1
    x = node[cell]
    J = np.stack([x[:, k + 1] - x[:, 0] for k in range(TD)], axis=-1)   # J[c, a, k]
    det = np.linalg.det(J)
    inv = np.linalg.inv(J)                                               # inv[c, k, a]
    measure = det / (2.0 if TD == 2 else 6.0)
    return measure, inv


@pytest.mark.parametrize("tag", ["tri_p1", "tri_p2", "tri_p3", "tet_p1", "tet_p2"])
def test_topology_dofs_and_boundary(golden_dir, tag):
    z = load(golden_dir, f"small_{tag}.npz")
    mesh = make_mesh(z["node"], z["cell"])
    p = int(z["p"])
    assert np.array_equal(mesh.edge.numpy(), z["edge"])
    assert np.array_equal(mesh.face2cell.numpy(), z["face2cell"])
    space = LagrangeFESpace(mesh, p)
    assert np.array_equal(space.cell_to_dof().numpy(), z["cell2dof"])
    assert space.number_of_global_dofs() == z["f"].shape[0]
    assert np.array_equal(space.is_boundary_dof().numpy(), z["is_bd"])
    assert np.allclose(space.interpolation_points().numpy(), z["ipoints"], atol=1e-15, rtol=0)


@pytest.mark.parametrize("tag", ["tri_p1", "tri_p2", "tri_p3", "tet_p1", "tet_p2"])
def test_factor_table_decomposition(golden_dir, tag):
    """sum_t factor_t * table_t reproduces the reference's quadrature local matrices."""
    z = load(golden_dir, f"small_{tag}.npz")
    node, cell, p = z["node"], z["cell"], int(z["p"])
    TD = cell.shape[1] - 1
    q = p + 3 if int(z["q"]) < 0 else int(z["q"])
    measure, inv = kernel_factors_numpy(node, cell)
    pairs = sx.metric_pairs(TD)
    G = np.stack([measure * np.einsum("ca,ca->c", inv[:, k], inv[:, l]) for k, l in pairs], axis=1)
    Kd = np.einsum("ct,tij->cij", G * z["kappa"][:, None], sx.diffusion_tables(TD, p, q))
    Km = np.einsum("c,tij->cij", measure, sx.mass_table(TD, p, q))
    scale = np.max(np.abs(z["K_diff"]))
    assert np.max(np.abs(Kd - z["K_diff"])) / scale < 1e-12
    assert np.max(np.abs(Km - z["K_mass"])) / np.max(np.abs(z["K_mass"])) < 1e-12


def test_elasticity_host_logic(golden_dir):
    z = load(golden_dir, "small_elasticity_tet_p1.npz")
    node, cell, s = z["node"], z["cell"], z["scale"]
    mesh = make_mesh(node, cell)
    ts = TensorFunctionSpace(LagrangeFESpace(mesh, 1), (-1, 3))
    assert np.array_equal(ts.cell_to_dof().numpy(), z["cell2dof"])
    clamp = lambda x: torch.abs(x[..., 0]) < 1e-12
    assert np.array_equal(ts.is_boundary_dof(threshold=clamp, method=None).numpy(), z["is_bd"])
    # the per-(row block, column block) formula of the elasticity kernel
    measure, inv = kernel_factors_numpy(node, cell)
    g = np.concatenate([-inv.sum(axis=1, keepdims=True), inv], axis=1)   # (NC, 4, 3) grad lambda
    _, ws = mesh.quadrature_formula(4).get_quadrature_points_and_weights()
    wsum = ws.sum()
    lam, mu = 1.0 * s * measure * wsum, 0.5 * s * measure * wsum
    d00 = 2 * mu + lam
    NC = cell.shape[0]
    KK = np.zeros((NC, 12, 12))
    for a in range(3):
        for b in range(3):
            gi, gj = g[:, :, None, :], g[:, None, :, :]
            if a == b:
                dot = np.einsum("cid,cjd->cij", g, g)
                blk = d00[:, None, None] * gi[..., a] * gj[..., a] + mu[:, None, None] * (dot - gi[..., a] * gj[..., a])
            else:
                blk = lam[:, None, None] * gi[..., a] * gj[..., b] + mu[:, None, None] * gi[..., b] * gj[..., a]
            KK[:, a::3, b::3] = blk
    assert np.max(np.abs(KK - z["KK"])) / np.max(np.abs(z["KK"])) < 1e-12


def test_c1_mesh_bitwise(golden_dir):
    z = load(golden_dir, "c1_poisson_tri_p1_64.npz")
    mesh = TriangleMesh.from_box([0, 1, 0, 1], 64, 64)
    assert np.array_equal(mesh.node.numpy(), z["node"])
    assert np.array_equal(mesh.cell.numpy(), z["cell"])
    space = LagrangeFESpace(mesh, 1)
    assert np.array_equal(space.is_boundary_dof().numpy(), z["is_bd"])


def test_tet_from_box_matches_oracle():
    from oracle import fem_oracle as O
    node, cell = O.tet_from_box([0, 1, 0, 1, 0, 1], 3, 2, 2)
    mesh = TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 3, 2, 2)
    assert np.array_equal(mesh.node.numpy(), node)
    assert np.array_equal(mesh.cell.numpy(), cell)
    topo = O.construct(cell)
    assert np.array_equal(mesh.edge.numpy(), topo["edge"])
    assert np.array_equal(mesh.face.numpy(), topo["face"])
    assert np.array_equal(mesh.cell_to_ipoint(2).numpy(), O.cell_to_dof(cell, topo, node.shape[0], 2))


@pytest.mark.parametrize("kind,p", [("tri", 1), ("tri", 2), ("tri", 3), ("tet", 1), ("tet", 2), ("tet", 3)])
def test_dof_blocks_partition_the_numbering(kind, p):
    """dof_blocks(): the contiguous vertex/edge/face/cell ranges of the global
    dof numbering, in order (the input of the block-merge renumbering of the
    delta-coded SELL copy); for vector spaces scaled or repeated by component."""
    mesh = TriangleMesh.from_box([0, 1, 0, 1], 3, 2) if kind == "tri" else \
        TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 2, 2, 1)
    space = LagrangeFESpace(mesh, p=p)
    blocks = space.dof_blocks()
    assert sum(blocks) == space.number_of_global_dofs() and all(b > 0 for b in blocks)
    assert blocks[0] == mesh.number_of_nodes()
    c2d = space.cell_to_dof().numpy()
    starts = np.cumsum([0] + blocks)
    # the first dofs of a cell (its vertices) lie in the vertex block, the
    # rest in the later blocks
    assert np.all(c2d[:, :mesh.cell.shape[1]] < starts[1]) if p == 1 else np.all(c2d.max(axis=1) >= starts[1])
    gd = mesh.geo_dimension()
    inter = TensorFunctionSpace(space, (-1, gd)).dof_blocks()
    major = TensorFunctionSpace(space, (gd, -1)).dof_blocks()
    assert inter == [gd * b for b in blocks] and major == blocks * gd


def test_bench_roofline_record():
    """The roofline block of the C2 record (dominant-kernel SpMV and whole
    iteration) from a profiling-solve summary: formulas and keys."""
    import importlib
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    bench = importlib.import_module("bench")
    mixed = {"nnz": 57_611_761, "sell_cols": "i32", "kernel_ms_avg": 0.0841, "ms_per_step": 131.6, "niter": 1127,
             "stages_ms": {"assembly (pattern + values)": 5.4, "rhs": 1.5, "dirichlet": 1.5,
                           "solver copy (SELL)": 0.4, "pcg": 143.6, "assembly/pattern": 2.3}}
    r = bench.spmv_roofline(mixed, 2_146_689, 64, 6685.8, "measured")
    assert r["algorithmic_bytes_per_launch"] == 57_611_761 * 8 + 2_146_689 * 16
    assert abs(r["frac"] - r["achieved"] / 6685.8) < 1e-12 and 0.8 < r["frac"] < 0.95
    it = r["iteration"]
    assert it["bytes_per_iteration"] == r["algorithmic_bytes_per_launch"] + 11 * 2_146_689 * 4
    assert abs(it["us_per_iteration"] - (131.6 - 8.8) / 1127 * 1e3) < 1e-6
    assert r["traffic"] is not None and r["bound"] == "hbm" and r["unit"] == "GB/s"


def test_no_cpu_fallback():
    """The product path computes only on the GPU: with CPU tensors every
    compute entry (assembly, Dirichlet, SpMV, both solvers) raises instead of
    computing on the host."""
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, DirichletBC
    from fealpy_gb300.sparse import CSRTensor
    mesh = TriangleMesh.from_box([0, 1, 0, 1], 4, 4)
    space = LagrangeFESpace(mesh, p=1)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=1.0, q=3))
    with pytest.raises((ValueError, RuntimeError)):
        bf.assembly()
    n = space.number_of_global_dofs()
    A = CSRTensor(torch.arange(n + 1, dtype=torch.int64), torch.arange(n, dtype=torch.int32),
                  torch.ones(n, dtype=torch.float64), (n, n))
    b = torch.ones(n, dtype=torch.float64)
    with pytest.raises((ValueError, RuntimeError)):
        A @ b
    with pytest.raises((ValueError, RuntimeError)):
        F.cg(A, b)
    with pytest.raises((ValueError, RuntimeError)):
        F.cg_mixed(A, b)
    with pytest.raises((ValueError, RuntimeError)):
        DirichletBC(space, gd=0.0).apply(A, b)


def test_coo_tensor_conversions():
    """COOTensor (``fealpy/sparse/coo_tensor.py``): coalescing sorts by
    (row, column) and sums duplicates; tocsr/tocoo round trip; to_dense adds
    repeated entries.  Pure index bookkeeping on CPU tensors, compared with
    scipy."""
    from scipy.sparse import coo_matrix
    from fealpy_gb300.sparse import COOTensor, CSRTensor
    g = torch.Generator().manual_seed(5)
    n, m, nnz = 13, 9, 60
    rows = torch.randint(0, n, (nnz,), generator=g)
    cols = torch.randint(0, m, (nnz,), generator=g)
    vals = torch.rand(nnz, generator=g, dtype=torch.float64)
    A = COOTensor(torch.stack([rows, cols]), vals, (n, m))
    S = coo_matrix((vals.numpy(), (rows.numpy(), cols.numpy())), shape=(n, m)).tocsr()
    S.sum_duplicates()
    C = A.tocsr()
    assert isinstance(C, CSRTensor) and C.shape == (n, m)
    assert np.array_equal(C.crow.numpy(), S.indptr)
    assert np.array_equal(C.col.numpy(), S.indices)
    assert np.allclose(C.values.numpy(), S.data, rtol=0, atol=1e-15)
    assert np.allclose(A.to_dense().numpy(), S.toarray(), rtol=0, atol=1e-15)
    B = C.tocoo()
    assert B.is_coalesced and B.nnz == S.nnz
    assert torch.equal(B.row, C.row) and torch.equal(B.col, C.col.long())
    assert B.tocsr().crow.equal(C.crow)
    # no values: coalescing counts each position's multiplicity
    P = COOTensor(torch.stack([rows, cols]), None, (n, m)).coalesce()
    ones = coo_matrix((np.ones(nnz), (rows.numpy(), cols.numpy())), shape=(n, m)).tocsr()
    ones.sum_duplicates()
    assert np.array_equal(P.values.numpy(), ones.data.astype(np.int64))
    # shape inferred from the largest index, as FEALPy does
    assert COOTensor(torch.tensor([[0, 4], [2, 1]]), None).shape == (5, 3)
    with pytest.raises(ValueError):
        COOTensor(torch.zeros(3, 2, dtype=torch.int64), None)


def test_coo_coalesce_reference_known_answers():
    """The reference's own coalesce cases (``test/sparse/test_coo_tensor.py:29-90``):
    duplicates summed in (row, column) order; without values the multiplicity
    (accumulate) or no values at all."""
    from fealpy_gb300.sparse import COOTensor
    idx = torch.tensor([[0, 0, 1, 2, 0, 1], [1, 2, 0, 0, 2, 0]])
    c = COOTensor(idx, torch.tensor([1, 2, 3, 4, 5, 6], dtype=torch.float64), torch.tensor([3, 3]),
                  is_coalesced=False).coalesce()
    assert c.is_coalesced
    assert torch.equal(c.indices, torch.tensor([[0, 0, 1, 2], [1, 2, 0, 0]]))
    assert torch.equal(c.values, torch.tensor([1, 7, 9, 4], dtype=torch.float64))
    c = COOTensor(torch.tensor([[0, 0, 1, 2, 0], [1, 2, 0, 0, 2]]), None, (3, 3), is_coalesced=False)
    a = c.coalesce(accumulate=True)
    assert torch.equal(a.indices, torch.tensor([[0, 0, 1, 2], [1, 2, 0, 0]]))
    assert torch.equal(a.values, torch.tensor([1, 2, 1, 1]))
    b = COOTensor(torch.tensor([[0, 0, 1, 2], [1, 2, 0, 0]]), None, (3, 3),
                  is_coalesced=False).coalesce(accumulate=False)
    assert b.is_coalesced and b.values is None


def test_csr_arithmetic_matches_scipy():
    """CSRTensor arithmetic of FEALPy's interface (``fealpy/sparse/csr_tensor.py:218-420``):
    sums of two patterns (union, duplicates added) and of one pattern
    (values added), scalar and dense operands, transpose, triangles, column
    sums, selection.  Index bookkeeping on CPU tensors, compared with scipy."""
    import scipy.sparse as sps
    from fealpy_gb300.sparse import CSRTensor
    a = sps.random(40, 30, density=0.15, random_state=3, format="csr")
    b = sps.random(40, 30, density=0.15, random_state=4, format="csr")
    a.sort_indices(); b.sort_indices()
    A, B = CSRTensor.from_scipy(a, device="cpu"), CSRTensor.from_scipy(b, device="cpu")

    def same(M, ref, exact_pattern=True):
        ref = sps.csr_matrix(ref)
        ref.sum_duplicates()
        ref.sort_indices()
        assert isinstance(M, CSRTensor) and tuple(M.shape) == ref.shape
        assert np.allclose(M.to_dense().numpy(), ref.toarray(), rtol=0, atol=1e-14)
        if exact_pattern:
            assert np.array_equal(M.crow.numpy(), ref.indptr) and np.array_equal(M.col.numpy(), ref.indices)

    same(A + B, a + b)
    same(A - B, a - b)
    same(A.add(B, alpha=2.5), a + 2.5 * b)
    C = A + A                       # one pattern: values added, the pattern shared
    assert C.crow is A.crow and C.col is A.col
    same(C, 2 * a)
    same(A * 3.0, 3.0 * a)
    same(A / 4.0, a / 4.0)
    same(A ** 2, a.power(2))
    D = torch.rand(40, 30, dtype=torch.float64, generator=torch.Generator().manual_seed(1))
    assert np.allclose((A + D).numpy(), a.toarray() + D.numpy(), rtol=0, atol=1e-14)
    same(A.mul(D), a.multiply(D.numpy()))
    rs = torch.arange(1, 41, dtype=torch.float64)
    same(A.div(rs), sps.diags(1.0 / rs.numpy()) @ a)
    same(A.T, a.T)
    same(A.tril(), sps.tril(a)); same(A.triu(1), sps.triu(a, 1))
    assert np.allclose(A.sum(axis=1).numpy(), np.asarray(a.sum(axis=0)).ravel(), rtol=0, atol=1e-14)
    mask = A.values > 0.5
    same(A.partial(mask), sps.csr_matrix((a.data * (a.data > 0.5), a.indices, a.indptr), shape=a.shape),
         exact_pattern=False)
    assert A.partial(mask).nnz == int(mask.sum())
    with pytest.raises(ValueError):
        A + CSRTensor.from_scipy(sps.random(30, 30, density=0.1, format="csr"), device="cpu")


def test_batched_sparse_bookkeeping():
    """Batched values (B, nnz) on one pattern (a form with batched
    coefficients): dense form, COO round trip, coalescing per member."""
    from fealpy_gb300.sparse import COOTensor, CSRTensor
    crow = torch.tensor([0, 2, 3, 5])
    col = torch.tensor([0, 2, 1, 0, 2], dtype=torch.int32)
    vals = torch.arange(10, dtype=torch.float64).reshape(2, 5)
    A = CSRTensor(crow, col, vals, (3, 3))
    assert A.is_batched and A.shape == (2, 3, 3) and A.sparse_shape == (3, 3)
    D = A.to_dense()
    for b in range(2):
        assert torch.equal(D[b], CSRTensor(crow, col, vals[b], (3, 3)).to_dense())
    C = A.tocoo()
    assert C.shape == (2, 3, 3) and torch.equal(C.to_dense(), D)
    R = C.tocsr()
    assert torch.equal(R.crow, crow) and torch.equal(R.values, vals)
    # duplicates summed member by member
    U = COOTensor(torch.tensor([[0, 0, 1], [1, 1, 0]]), torch.tensor([[1., 2., 3.], [4., 5., 6.]]), (2, 2))
    c = U.coalesce()
    assert torch.equal(c.values, torch.tensor([[3., 3.], [9., 6.]]))
    with pytest.raises(ValueError):
        A.diags()


def test_batched_csr_dense_operands():
    """Dense operands of a batched CSR (values (B, nnz)) act member by member."""
    from fealpy_gb300.sparse import CSRTensor
    crow = torch.tensor([0, 2, 3, 5])
    col = torch.tensor([0, 2, 1, 0, 2], dtype=torch.int32)
    vals = torch.arange(1, 11, dtype=torch.float64).reshape(2, 5)
    A = CSRTensor(crow, col, vals, (3, 3))
    D = torch.rand(2, 3, 3, dtype=torch.float64, generator=torch.Generator().manual_seed(2))
    dense = A.to_dense()
    assert torch.allclose(A + D, dense + D, rtol=0, atol=1e-15)
    assert torch.allclose(A.mul(D).to_dense(), dense * D * (dense != 0), rtol=0, atol=1e-15)
    for b in range(2):
        Ab = CSRTensor(crow, col, vals[b], (3, 3))
        assert torch.allclose(A.div(D).values[b], Ab.div(D[b]).values, rtol=0, atol=1e-15)
        assert torch.allclose((A ** D).values[b], (Ab ** D[b]).values, rtol=0, atol=1e-15)
