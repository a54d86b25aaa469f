"""GPU parity: the sm_103a path through the public API (and so through the C
ABI) against the reference fixtures and the CPU oracle.

Tolerances: CSR indptr/indices bit-exact (canonical order); values, right-hand
sides and boundary-modified vectors within 1e-12 relative (max-norm relative to
the array's max-norm); CG iteration counts within +-1 of the reference;
solutions within 1e-9 relative of the reference's solution."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def rel_err(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def same(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return a.shape == np.asarray(b).shape and np.array_equal(a, np.asarray(b))


def test_c1_poisson_full_path(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator,
                                  DirichletBC)
    z = load(golden_dir, "c1_poisson_tri_p1_64.npz")
    mesh = F.TriangleMesh.from_box([0, 1, 0, 1], 64, 64, device=dev)
    assert same(mesh.node, z["node"]) and same(mesh.cell, z["cell"])
    space = F.LagrangeFESpace(mesh, p=1)

    def solution(p):
        return torch.sin(np.pi * p[..., 0]) * torch.sin(np.pi * p[..., 1])
    solution.coordtype = "cartesian"

    def source(p):
        return 2 * np.pi ** 2 * solution(p)
    source.coordtype = "cartesian"

    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=1, q=3))
    A = bf.assembly()
    assert same(A.crow, z["crow"]) and same(A.col, z["col"])
    assert rel_err(A.values, z["val"]) < VAL_TOL
    # format="coo": the coalesced coordinate form of the same matrix
    Ac = bf.assembly(format="coo")
    assert isinstance(Ac, F.COOTensor) and Ac.is_coalesced and Ac.shape == A.shape
    assert torch.equal(Ac.row, A.row) and torch.equal(Ac.col, A.col.long())
    assert torch.equal(Ac.values, A.values)
    assert torch.equal(Ac.tocsr().crow, A.crow)
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(source, q=3))
    Fv = lf.assembly()
    assert rel_err(Fv, z["F"]) < VAL_TOL
    bc = DirichletBC(space, gd=solution)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(A, Fv)
    assert same(A2.crow, z["bc_crow"]) and same(A2.col, z["bc_col"])
    assert rel_err(A2.values, z["bc_val"]) < VAL_TOL
    assert rel_err(F2, z["bc_F"]) < VAL_TOL
    M = F.JacobiPreconditioner().apply(A2)
    uh, info = F.cg(A2, F2, M=M, atol=1e-30, rtol=1e-10, returninfo=True)
    assert abs(info["niter"] - int(z["niter"])) <= 1
    assert rel_err(uh, z["uh"]) < 1e-9


@pytest.mark.parametrize("tag", ["tri_p1", "tri_p2", "tri_p3", "tet_p1", "tet_p2"])
def test_small_cases(golden_dir, tag):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator, DirichletBC
    z = load(golden_dir, f"small_{tag}.npz")
    node = torch.as_tensor(z["node"], device=dev)
    cell = torch.as_tensor(z["cell"], dtype=torch.int32, device=dev)
    mesh = (F.TriangleMesh if z["cell"].shape[1] == 3 else F.TetrahedronMesh)(node, cell)
    p = int(z["p"])
    q = None if int(z["q"]) < 0 else int(z["q"])
    space = F.LagrangeFESpace(mesh, p)
    kappa = torch.as_tensor(z["kappa"], device=dev)
    # local matrices through the integrator API
    Kd = ScalarDiffusionIntegrator(coef=kappa, q=q).assembly(space)
    assert rel_err(Kd, z["K_diff"]) < VAL_TOL
    Km = ScalarMassIntegrator(coef=1.0, q=q).assembly(space)
    assert rel_err(Km, z["K_mass"]) < VAL_TOL
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q), ScalarMassIntegrator(coef=1.0, q=q))
    A = bf.assembly()
    assert same(A.crow, z["crow"]) and same(A.col, z["col"])
    assert rel_err(A.values, z["val"]) < VAL_TOL
    gd = torch.as_tensor(z["gd"], device=dev)
    bc = DirichletBC(space, gd=gd)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(A, torch.as_tensor(z["f"], device=dev))
    assert same(A2.crow, z["bc_crow"]) and same(A2.col, z["bc_col"])
    assert rel_err(A2.values, z["bc_val"]) < VAL_TOL
    assert rel_err(F2, z["bc_F"]) < VAL_TOL
    uh, info = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    assert abs(info["niter"] - int(z["niter"])) <= 1
    assert rel_err(uh, z["uh"]) < 1e-8


def test_elasticity_p1(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, LinearElasticityIntegrator, VectorSourceIntegrator, DirichletBC
    z = load(golden_dir, "small_elasticity_tet_p1.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    ts = F.TensorFunctionSpace(F.LagrangeFESpace(mesh, 1), (-1, 3))
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5,
                                  cell_scale=torch.as_tensor(z["scale"], device=dev))
    bf = BilinearForm(ts)
    bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
    A = bf.assembly()
    assert same(A.crow, z["crow"]) and same(A.col, z["col"])
    assert rel_err(A.values, z["val"]) < VAL_TOL
    # FEALPy's 'voigt' and 'fast' variants form the same matrix
    for method in ("voigt", "fast"):
        bv = BilinearForm(ts)
        bv.add_integrator(LinearElasticityIntegrator(mat, q=4, method=method))
        assert torch.equal(bv.assembly().values, A.values)
    lf = LinearForm(ts)
    lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
    Fv = lf.assembly()
    assert rel_err(Fv, z["F"]) < VAL_TOL
    clamp = lambda x: torch.abs(x[..., 0]) < 1e-12
    bc = DirichletBC(ts, gd=0.0, threshold=clamp)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(A, Fv)
    assert same(A2.crow, z["bc_crow"]) and same(A2.col, z["bc_col"])
    assert rel_err(A2.values, z["bc_val"]) < VAL_TOL
    assert rel_err(F2, z["bc_F"]) < VAL_TOL
    uh, info = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    assert abs(info["niter"] - int(z["niter"])) <= 1
    assert rel_err(uh, z["uh"]) < 1e-8


def test_spmv_all_lane_widths(golden_dir):
    dev = cuda()
    from fealpy_gb300 import kernels as K
    import scipy.sparse as sp
    z = load(golden_dir, "small_tet_p2.npz")
    crow, col, val = z["crow"], z["col"], z["val"]
    n = len(crow) - 1
    x = np.random.default_rng(0).normal(size=n)
    ref = sp.csr_matrix((val, col, crow), shape=(n, n)) @ x
    t = lambda a, dt=None: torch.as_tensor(a, device=dev, dtype=dt)
    for lanes in (0, 1, 2, 4, 8, 16, 32):
        y = K.csr_spmv(t(crow), t(col), t(val), t(x), lanes)
        assert rel_err(y, ref) < 1e-14
        y32 = K.csr_spmv(t(crow), t(col), t(val, torch.float32), t(x, torch.float32), lanes)
        assert rel_err(y32, ref) < 1e-5


def test_spmm_columns_in_one_pass(golden_dir):
    """A @ X for X (n, k) (the (n, batch) product of bm.csr_spmm): one pass
    over the matrix for all k columns, against scipy; each column the same
    sum as the one-lane-per-row SpMV; k = 1, 3, 64 and a rectangular
    matrix."""
    dev = cuda()
    import scipy.sparse as sp
    import fealpy_gb300 as F
    from fealpy_gb300 import kernels as K
    z = load(golden_dir, "cfg_c2_tet_p2_8.npz")
    crow, col, val = z["crow"], z["col"], z["val"]
    n = len(crow) - 1
    S = sp.csr_matrix((val, col, crow), shape=(n, n))
    A = F.CSRTensor(torch.as_tensor(crow, device=dev), torch.as_tensor(col, device=dev),
                    torch.as_tensor(val, device=dev), (n, n))
    rng = np.random.default_rng(3)
    for k in (1, 3, 64):
        X = rng.normal(size=(n, k))
        Y = A @ torch.as_tensor(X, device=dev)
        assert Y.shape == (n, k) and rel_err(Y, S @ X) < 1e-14
        y0 = K.csr_spmv(A.crow, A.col, A.values, torch.as_tensor(X[:, 0].copy(), device=dev), 1)
        assert torch.equal(Y[:, 0], y0)
    # wider than 64 columns: one product per column
    X = rng.normal(size=(n, 65))
    assert rel_err(A @ torch.as_tensor(X, device=dev), S @ X) < 1e-14
    # a rectangular matrix (the first 100 columns of A)
    R = S[:, :100].tocsr()
    R.sort_indices()
    Ar = F.CSRTensor(torch.as_tensor(R.indptr, dtype=torch.int64, device=dev),
                     torch.as_tensor(R.indices, dtype=torch.int32, device=dev),
                     torch.as_tensor(R.data, device=dev), R.shape)
    X = rng.normal(size=(100, 5))
    assert rel_err(Ar @ torch.as_tensor(X, device=dev), R @ X) < 1e-14


def test_determinism_bitwise(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    mesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 6, 5, 4, device=dev)
    space = F.LagrangeFESpace(mesh, 2)
    kappa = torch.rand(mesh.number_of_cells(), device=dev, dtype=torch.float64) + 0.5
    vals = []
    for _ in range(2):
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(q=4))
        vals.append(bf.assembly())
    assert torch.equal(vals[0].crow, vals[1].crow) and torch.equal(vals[0].col, vals[1].col)
    assert torch.equal(vals[0].values, vals[1].values)


def test_high_valence_rows_take_the_wide_path():
    """A fan of 300 triangles around one vertex: that row (301 entries) exceeds
    the first-pass capacity of the pattern and assembly kernels."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator
    from oracle import fem_oracle as O
    m = 300
    ang = np.linspace(0, 2 * np.pi, m, endpoint=False)
    node = np.concatenate([[[0.0, 0.0]], np.c_[np.cos(ang), np.sin(ang)]], axis=0)
    cell = np.array([[0, 1 + k, 1 + (k + 1) % m] for k in range(m)], dtype=np.int32)
    mesh = F.TriangleMesh(torch.as_tensor(node, device=dev), torch.as_tensor(cell, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(q=4))
    A = bf.assembly()
    topo = O.construct(cell)
    c2d = O.cell_to_dof(cell, topo, node.shape[0], 2)
    n = O.n_global_dofs(cell, topo, node.shape[0], 2)
    crow, col, val = O.coalesce_to_csr(c2d, O.diffusion_local(node, cell, 2, 4), n)
    assert same(A.crow, crow) and same(A.col, col)
    assert rel_err(A.values, val) < VAL_TOL
    # a form that reuses its pattern (slot map for rows up to 128 entries, the
    # column search for the wide row): the same values, bit for bit, twice
    rf = BilinearForm(space, reuse_pattern=True)
    rf.add_integrator(ScalarDiffusionIntegrator(q=4))
    for _ in range(2):
        R = rf.assembly()
        assert torch.equal(R.col, A.col) and torch.equal(R.values, A.values)


def test_mixed_precision_reaches_fp64_accuracy():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator, DirichletBC
    mesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 12, 12, 12, device=dev)
    space = F.LagrangeFESpace(mesh, 2)
    g = torch.Generator(device="cpu").manual_seed(0)
    kappa = torch.exp(torch.randn(mesh.number_of_cells(), generator=g, dtype=torch.float64)).to(dev)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
    A = bf.assembly(emit_f32=True)
    n = space.number_of_global_dofs()
    A2, F2 = DirichletBC(space, gd=0.0).apply(A, torch.ones(n, dtype=torch.float64, device=dev))
    x64, i64 = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-12, returninfo=True)
    xm, im = F.cg_mixed(A2, F2, rtol=1e-10, returninfo=True)
    r = F2 - A2 @ xm
    rel = float(torch.linalg.norm(r) / torch.linalg.norm(F2))
    assert rel <= 1e-10 * 1.0001, rel
    assert abs(rel - im["relres"]) <= 1e-3 * rel + 1e-16
    err = float(torch.max(torch.abs(xm - x64)) / torch.max(torch.abs(x64)))
    assert err < 1e-8, err
    assert im["n_updates"] >= 1


def test_fp32_assembly_refined_solve():
    """FP32 cell-local assembly + FP32 inner CG + FP64 refinement: the FP32
    matrix equals the FP64 one rounded (to FP32 accumulation accuracy), the
    refinement reaches 1e-10 on the FP32 operator (residual in FP64
    arithmetic), and the solution's error against the FP64-assembled solve is
    of the order of FP32 rounding (stated bound 1e-5 relative, max norm)."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator, DirichletBC
    mesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 12, 12, 12, device=dev)
    space = F.LagrangeFESpace(mesh, 2)
    g = torch.Generator(device="cpu").manual_seed(0)
    kappa = torch.exp(torch.randn(mesh.number_of_cells(), generator=g, dtype=torch.float64)).to(dev)
    mats = {}
    for dt in (torch.float64, torch.float32):
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
        mats[dt] = bf.assembly(dtype=dt)
    A64, A32 = mats[torch.float64], mats[torch.float32]
    assert A32.values.dtype == torch.float32
    assert torch.equal(A64.crow, A32.crow) and torch.equal(A64.col, A32.col)
    assert rel_err(A32.values.double(), A64.values.cpu().numpy()) < 1e-6
    n = space.number_of_global_dofs()
    bc = DirichletBC(space, gd=0.0)
    f = torch.ones(n, dtype=torch.float64, device=dev)
    B64, F64 = bc.apply(A64, f)
    B32, F32 = bc.apply(A32, f)
    x64 = F.cg(B64, F64, M=F.JacobiPreconditioner().apply(B64), atol=1e-30, rtol=1e-12)
    xm, im = F.cg_mixed(B32, F32, rtol=1e-10, returninfo=True)
    Bd = F.CSRTensor(B32.crow, B32.col, B32.values.double(), B32.shape)
    r = F32.double() - Bd @ xm
    rel = float(torch.linalg.norm(r) / torch.linalg.norm(F32.double()))
    assert rel <= 1e-10 * 1.0001, rel
    assert im["relres"] <= 1e-10 and im["graph"]
    err = float(torch.max(torch.abs(xm - x64)) / torch.max(torch.abs(x64)))
    assert err < 1e-5, err


def test_cg_edge_cases():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, DirichletBC
    mesh = F.TriangleMesh.from_box([0, 1, 0, 1], 8, 8, device=dev)
    space = F.LagrangeFESpace(mesh, 1)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator())
    A = bf.assembly()
    n = space.number_of_global_dofs()
    A2, F2 = DirichletBC(space, gd=0.0).apply(A, torch.ones(n, dtype=torch.float64, device=dev))
    # zero right-hand side: x = 0 and no iteration
    x, info = F.cg(A2, torch.zeros(n, dtype=torch.float64, device=dev), x0=torch.ones(n, dtype=torch.float64, device=dev),
                   returninfo=True)
    assert info["niter"] == 0 and float(torch.abs(x).max()) == 0.0
    # iteration limit
    x, info = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-30, maxit=5, returninfo=True)
    assert info["niter"] == 5
    # a negative definite matrix is reported, not silently iterated
    neg = A2.mul(-1.0)
    with pytest.raises(RuntimeError):
        F.cg(neg, F2, rtol=1e-10)


def test_full_size_properties():
    """Size-independent checks on a 32^3 P2 tetrahedral case: diffusion rows sum
    to zero, the mass matrix integrates 1 to |Omega| = 1, A is symmetric."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    mesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 32, 32, 32, device=dev)
    space = F.LagrangeFESpace(mesh, 2)
    n = space.number_of_global_dofs()
    one = torch.ones(n, dtype=torch.float64, device=dev)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(q=4))
    A = bf.assembly()
    scale = float(A.values.abs().max())
    assert float((A @ one).abs().max()) < 1e-12 * scale * 30
    bm = BilinearForm(space)
    bm.add_integrator(ScalarMassIntegrator(q=4))
    M = bm.assembly()
    assert abs(float(M.values.sum()) - 1.0) < 1e-12
    d = A.to_dense() if n < 20000 else None
    # symmetry via a random bilinear form: y^T A x == x^T A y
    g = torch.Generator(device="cpu").manual_seed(1)
    x = torch.randn(n, generator=g, dtype=torch.float64).to(dev)
    y = torch.randn(n, generator=g, dtype=torch.float64).to(dev)
    a = float(torch.dot(y, A @ x))
    b = float(torch.dot(x, A @ y))
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0) * 10


def test_sell_copy_spmv_and_solver_drivers(golden_dir):
    """The SELL-32 solver copy: SpMV against scipy; FP64 cg: the graph-driven
    loop against the host-polled loop (same kernels, bitwise-equal iterates);
    cg_mixed: the persistent kernel against the host-polled loop."""
    dev = cuda()
    import scipy.sparse as sp
    import fealpy_gb300 as F
    from fealpy_gb300 import kernels as K
    from fealpy_gb300.sparse import CSRTensor
    for name in ("small_tet_p2.npz", "small_tri_p3.npz", "c1_poisson_tri_p1_64.npz"):
        z = load(golden_dir, name)
        crow, col, val = z["crow"], z["col"], z["val"]
        n = len(crow) - 1
        t = lambda a, dt=None: torch.as_tensor(a, device=dev, dtype=dt)
        S = K.sell_build(t(crow), t(col), t(val), None, want64=True, want32=True)
        assert S.padded_nnz >= len(col)
        x = np.random.default_rng(1).normal(size=n)
        ref = sp.csr_matrix((val, col, crow), shape=(n, n)) @ x
        assert rel_err(K.sell_spmv(S, t(x), torch.float64), ref) < 1e-14
        assert rel_err(K.sell_spmv(S, t(x, torch.float32), torch.float32), ref) < 1e-5
    z = load(golden_dir, "c1_poisson_tri_p1_64.npz")
    A = CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                  torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
    b = torch.as_tensor(z["bc_F"], device=dev)
    M = F.JacobiPreconditioner().apply(A)
    xs = {}
    for fmt, graph in (("sell", True), ("sell", False), ("csr", False)):
        x, info = F.cg(A, b, M=M, atol=1e-30, rtol=1e-10, returninfo=True, solver_format=fmt, graph=graph)
        assert abs(info["niter"] - int(z["niter"])) <= 1, (fmt, graph, info["niter"])
        assert rel_err(x, z["uh"]) < 1e-9
        xs[(fmt, graph)] = x
    assert torch.equal(xs[("sell", True)], xs[("sell", False)])
    xm = {}
    for graph in (True, False):
        x, info = F.cg_mixed(A, b, rtol=1e-10, returninfo=True, graph=graph)
        assert info["relres"] <= 1e-10 and rel_err(x, z["uh"]) < 1e-8
        assert info["graph"] == graph, info
        xm[graph] = (x, info["niter"], info["persistent"])
    # the persistent kernel (one cooperative launch) forms its block partials
    # over another grid than the multi-kernel loop: the same iteration up to
    # FP32 rounding of the dot products, and deterministic run to run
    assert xm[True][2] and not xm[False][2]
    assert abs(xm[True][1] - xm[False][1]) <= 2
    assert rel_err(xm[True][0], xm[False][0].cpu().numpy()) < 1e-9
    x2, info2 = F.cg_mixed(A, b, rtol=1e-10, returninfo=True, graph=True)
    assert info2["niter"] == xm[True][1] and torch.equal(x2, xm[True][0])  # deterministic


def test_sell_launch_shapes_and_autotune(golden_dir):
    """Every launch shape of the slice kernels gives the same SpMV bit for bit
    (a lane owns its row whatever the grid) and a converged solve; the
    autotuner times all candidates and keeps the fastest."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300 import kernels as K
    from fealpy_gb300.sparse import CSRTensor
    z = load(golden_dir, "c1_poisson_tri_p1_64.npz")
    A = CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                  torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
    b = torch.as_tensor(z["bc_F"], device=dev)
    S = K.sell_build(A.crow, A.col, A.values, None, want64=True, want32=True)
    x = torch.as_tensor(np.random.default_rng(3).normal(size=A.shape[0]), device=dev)
    y0 = K.sell_spmv(S, x, torch.float64)
    for shape in K.SELL_LAUNCH_CANDIDATES + ((32, 1), (96, 7)):
        S.set_launch(*shape)
        assert torch.equal(K.sell_spmv(S, x, torch.float64), y0), shape
    with pytest.raises(ValueError):
        S.set_launch(100, 1)
    with pytest.raises(ValueError):
        S.set_launch(256, K.SELL_MAX_BLOCKS + 1)
    times = K.sell_autotune(S, torch.float32, reps=3)
    assert set(times) == set(K.SELL_LAUNCH_CANDIDATES) and S.launch == min(times, key=times.get)
    A._sell = S
    for shape in ((32, 1), S.launch):
        S.set_launch(*shape)
        xs, info = F.cg_mixed(A, b, rtol=1e-10, returninfo=True)
        assert info["relres"] <= 1e-10 and rel_err(xs, z["uh"]) < 1e-8, (shape, info)


def test_elasticity_fp32_assembly_and_refined_solve(golden_dir):
    """P1 elasticity assembled in FP32 (factors from FP64 geometry): the
    pattern equals the FP64 one bit for bit, values within FP32 rounding, and
    the FP32-refined solve of it meets 1e-10 on that operator."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, LinearElasticityIntegrator, VectorSourceIntegrator
    from fealpy_gb300.fem import DirichletBC
    z = load(golden_dir, "small_elasticity_tet_p1.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    ts = F.TensorFunctionSpace(F.LagrangeFESpace(mesh, 1), (-1, 3))
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5,
                                  cell_scale=torch.as_tensor(z["scale"], device=dev))
    out = {}
    for dt in (torch.float64, torch.float32):
        bf = BilinearForm(ts)
        bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
        out[dt] = bf.assembly(dtype=dt)
    A64, A32 = out[torch.float64], out[torch.float32]
    assert A32.values.dtype == torch.float32
    assert torch.equal(A64.crow, A32.crow) and torch.equal(A64.col, A32.col)
    assert rel_err(A32.values.double(), A64.values.cpu().numpy()) < 1e-6
    lf = LinearForm(ts)
    lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
    bc = DirichletBC(ts, gd=0.0, threshold=lambda x: torch.abs(x[..., 0]) < 1e-12)
    B, f = bc.apply(A32, lf.assembly())
    x, info = F.cg_mixed(B, f, rtol=1e-10, returninfo=True)
    Bd = F.CSRTensor(B.crow, B.col, B.values.double(), B.shape)
    rel = float(torch.linalg.norm(f.double() - Bd @ x) / torch.linalg.norm(f.double()))
    assert info["reason"] == 2 and rel <= 1e-10 * 1.0001, (info, rel)
    assert rel_err(x, z["uh"]) < 1e-4


def test_residual_norm_kernel_matches_numpy(golden_dir):
    """fgb_residual_norm (the true residual of the restart loops): ||b - A x||
    and ||b|| against numpy on a FEALPy matrix, deterministic across calls."""
    dev = cuda()
    import scipy.sparse as sp
    from fealpy_gb300 import kernels as K
    z = load(golden_dir, "cfg_c2_tet_p2_8.npz")
    n = len(z["bc_crow"]) - 1
    A = sp.csr_matrix((z["bc_val"], z["bc_col"], z["bc_crow"]), shape=(n, n))
    rng = np.random.default_rng(11)
    x, b = rng.normal(size=n), rng.normal(size=n)
    t = lambda a: torch.as_tensor(a, device=dev)
    r1, b1 = K.residual_norm(t(z["bc_crow"]), t(z["bc_col"]), t(z["bc_val"]), t(b), t(x))
    r2, b2 = K.residual_norm(t(z["bc_crow"]), t(z["bc_col"]), t(z["bc_val"]), t(b), t(x))
    assert (r1, b1) == (r2, b2)
    assert abs(r1 - np.linalg.norm(b - A @ x)) <= 1e-12 * np.linalg.norm(b - A @ x)
    assert abs(b1 - np.linalg.norm(b)) <= 1e-13 * np.linalg.norm(b)


def test_forms_assembled_apart_add_to_the_grouped_form(golden_dir):
    """K + M of two forms assembled on one space (one pattern: the values add)
    equals the reference's grouped diffusion+mass matrix; the row sums
    (``sum(axis=0)``, the GPU product with ones) and the transpose of the
    symmetric matrix agree as well."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = load(golden_dir, "small_tet_p2.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    q = None if int(z["q"]) < 0 else int(z["q"])
    space = F.LagrangeFESpace(mesh, int(z["p"]))
    kappa = torch.as_tensor(z["kappa"], device=dev)
    bk, bm_ = BilinearForm(space), BilinearForm(space)
    bk.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q))
    bm_.add_integrator(ScalarMassIntegrator(coef=1.0, q=q))
    K, M = bk.assembly(), bm_.assembly()
    S = K + M
    assert same(S.crow, z["crow"]) and same(S.col, z["col"])
    assert rel_err(S.values, z["val"]) < VAL_TOL
    n = S.shape[1]
    ref = np.zeros(n)
    np.add.at(ref, np.repeat(np.arange(n), np.diff(z["crow"])), z["val"])
    ones = torch.ones(n, dtype=torch.float64, device=dev)
    assert torch.equal(S.sum(axis=0), S @ ones)
    assert rel_err(S.sum(axis=0), ref) < VAL_TOL
    T = S.T
    assert same(T.crow, z["crow"]) and same(T.col, z["col"])
    assert rel_err(T.values, z["val"]) < VAL_TOL


def test_batched_form_against_reference(golden_dir):
    """A form with batched coefficients (``BilinearForm(space, batch_size=3)``,
    diffusion with a (B, NC) coefficient and mass with a (B,) coefficient,
    both ``batched=True``) against the reference's batched CSR (values
    (B, nnz)), batched local matrices and batched right-hand side; products
    per member (assembled and matrix free), COO output; the single-matrix
    paths refuse the batch."""
    dev = cuda()
    import scipy.sparse as sps
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator, DirichletBC
    z = load(golden_dir, "batched_tri_p2.npz")
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev),
                          torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    kappa = torch.as_tensor(z["kappa"], device=dev)
    rho = torch.as_tensor(z["rho"], device=dev)
    Kd = ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True).assembly(space)
    assert Kd.shape == z["K_diff"].shape and rel_err(Kd, z["K_diff"]) < VAL_TOL
    bf = BilinearForm(space, batch_size=3)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True))
    bf.add_integrator(ScalarMassIntegrator(coef=rho, q=4, batched=True))
    A = bf.assembly()
    n = space.number_of_global_dofs()
    assert A.is_batched and tuple(A.shape) == (3, n, n) and A.values.shape == z["val"].shape
    assert same(A.crow, z["crow"]) and same(A.col, z["col"])
    assert rel_err(A.values, z["val"]) < VAL_TOL
    # mixing a batched and an unbatched integrator in one group: the unbatched
    # one repeats over the batch
    bg = BilinearForm(space, batch_size=3)
    bg.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True), ScalarMassIntegrator(coef=1.0, q=4))
    Ag = bg.assembly()
    for b in range(3):
        bm_ = BilinearForm(space)
        bm_.add_integrator(ScalarDiffusionIntegrator(coef=kappa[b], q=4), ScalarMassIntegrator(coef=1.0, q=4))
        assert torch.equal(Ag.values[b], bm_.assembly().values)
    # products per member: one vector for all, one vector per member
    x = torch.as_tensor(np.random.default_rng(5).normal(size=(3, n)), device=dev)
    y1 = A @ x[0]
    yb = A @ x
    for b in range(3):
        Sb = sps.csr_matrix((z["val"][b], z["col"], z["crow"]), shape=(n, n))
        assert rel_err(y1[b], Sb @ x[0].cpu().numpy()) < VAL_TOL
        assert rel_err(yb[b], Sb @ x[b].cpu().numpy()) < VAL_TOL
    # matrix free before assembly (fealpy/fem/bilinear_form.py:126-158): (B, n)
    bu = BilinearForm(space, batch_size=3)
    bu.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4, batched=True))
    bu.add_integrator(ScalarMassIntegrator(coef=rho, q=4, batched=True))
    assert bu.shape == (3, n, n)
    m1, mb = bu @ x[0], bu @ x
    assert bu._M is None and m1.shape == (3, n) and mb.shape == (3, n)
    assert rel_err(m1, y1.cpu().numpy()) < VAL_TOL and rel_err(mb, yb.cpu().numpy()) < VAL_TOL
    C = bf.assembly(format="coo")
    assert C.shape == (3, n, n) and torch.equal(C.values, A.values)
    assert torch.equal(A.to_dense()[1], F.CSRTensor(A.crow, A.col, A.values[1], (n, n)).to_dense())
    # batched right-hand side (fealpy/fem/linear_form.py:36-60)
    from fealpy_gb300.fem import LinearForm, ScalarSourceIntegrator
    lf = LinearForm(space, batch_size=3)
    lf.add_integrator(ScalarSourceIntegrator(source=torch.as_tensor(z["source"], device=dev), q=4, batched=True))
    Fb = lf.assembly()
    assert Fb.shape == (3, n) and rel_err(Fb, z["F"]) < VAL_TOL
    with pytest.raises(ValueError):
        F.cg(A, x[0])
    with pytest.raises(ValueError):
        DirichletBC(space, gd=0.0).apply(A, x[0])


def test_elasticity_component_major_layout(golden_dir):
    """P1 elasticity with ``shape=(3, -1)`` (component-major dofs): dof map,
    local matrices and CSR against the reference in that layout; the solve
    with the x = 0 clamp equals the interleaved solve with its dofs permuted."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, LinearElasticityIntegrator, VectorSourceIntegrator, DirichletBC
    z0 = load(golden_dir, "small_elasticity_tet_p1.npz")
    z = load(golden_dir, "elasticity_component_major.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z0["node"], device=dev),
                             torch.as_tensor(z0["cell"], dtype=torch.int32, device=dev))
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5,
                                  cell_scale=torch.as_tensor(z0["scale"], device=dev))
    sols = {}
    for shape in ((3, -1), (-1, 3)):
        ts = F.TensorFunctionSpace(F.LagrangeFESpace(mesh, 1), shape)
        bf = BilinearForm(ts)
        bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
        A = bf.assembly()
        if shape == (3, -1):
            assert same(ts.cell_to_dof(), z["cell2dof"])
            assert rel_err(LinearElasticityIntegrator(mat, q=4).assembly(ts), z["KK"]) < VAL_TOL
            assert same(A.crow, z["crow"]) and same(A.col, z["col"])
            assert rel_err(A.values, z["val"]) < VAL_TOL
        lf = LinearForm(ts)
        lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
        bc = DirichletBC(ts, gd=0.0, threshold=lambda x: torch.abs(x[..., 0]) < 1e-12)
        A2, F2 = bc.apply(A, lf.assembly())
        sols[shape] = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-12)
    NN = mesh.number_of_nodes()
    inter = sols[(-1, 3)].reshape(NN, 3)
    assert rel_err(sols[(3, -1)], inter.T.reshape(-1).cpu().numpy()) < 1e-9
