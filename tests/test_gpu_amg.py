"""Aggregation AMG in cg's M slot (GAMGSolver; FEALPy's multigrid solver role,
fealpy/solver/gamg_solver.py): PCG with the V-cycle reaches the reference's
solution (the C2-law fixture the reference produced, the oracle on the bench
workload at 24^3) within 1e-8, in a fraction of the Jacobi iterations; the
hierarchy and the iterates are bit-for-bit reproducible; 'MG' iterations and
vector (elasticity) systems converge too."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _fixture_system(golden_dir, name, dev):
    import fealpy_gb300 as F
    z = np.load(os.path.join(golden_dir, name))
    A = F.CSRTensor(torch.as_tensor(z["bc_crow"], device=dev), torch.as_tensor(z["bc_col"], device=dev),
                    torch.as_tensor(z["bc_val"], device=dev), (len(z["bc_crow"]) - 1,) * 2)
    return A, torch.as_tensor(z["bc_F"], device=dev), z


def _hash31(i):
    """The aggregation's node priority (a 32-bit integer mix), restated."""
    m = np.uint64(0xffffffff)
    x = i.astype(np.uint64)
    x ^= x >> np.uint64(16)
    x = (x * np.uint64(0x7feb352d)) & m
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x846ca68b)) & m
    x ^= x >> np.uint64(16)
    return x & np.uint64(0x7fffffff)


def _mis_aggregates(A, theta=0.0):
    """numpy restatement of the set-up's aggregation: maximal independent set
    by rounds of (rank, priority, index) keys over the strong graph, roots
    numbered in index order, every other node joining its largest-keyed
    assigned neighbour (sweeps until none is left)."""
    import scipy.sparse as sp
    n = A.shape[0]
    d = A.diagonal()
    C = A.tocoo()
    off = (C.row != C.col) & (C.data != 0)
    if theta > 0:
        off &= np.abs(C.data) > theta * np.sqrt(np.abs(d[C.row] * d[C.col]))
    S = sp.csr_matrix((np.ones(off.sum()), (C.row[off], C.col[off])), shape=(n, n))
    rows = np.repeat(np.arange(n), np.diff(S.indptr))
    idx = np.arange(n).astype(np.uint64)
    pr = _hash31(np.arange(n))
    state = np.where(np.diff(S.indptr) == 0, -1, 1)
    U = np.uint64
    while (state == 1).any():
        rank = np.where(state == 2, 2, np.where(state == 1, 1, 0)).astype(U)
        key = np.where(state < 0, U(0), (rank << U(62)) | (pr << U(31)) | idx)
        m = np.zeros(n, dtype=U)
        np.maximum.at(m, rows, key[S.indices])
        und = state == 1
        root = und & (key > m)
        out = und & ((m >> U(62)) == 2) & ~root
        state[root] = 2
        state[out] = 0
    agg = np.full(n, -1, dtype=np.int64)
    roots = np.nonzero(state == 2)[0]
    agg[roots] = np.arange(len(roots))
    while True:
        cand = (agg[S.indices] >= 0)
        kk = np.where(cand, ((U(1) << U(62)) | (pr[S.indices] << U(31)) | idx[S.indices]), U(0))
        best = np.zeros(n, dtype=U)
        np.maximum.at(best, rows, kk)
        need = (agg < 0) & (state >= 0) & (best > 0)
        if not need.any():
            break
        agg[need] = agg[(best[need] & U(0x7fffffff)).astype(np.int64)]
    return agg, len(roots)


def test_amg_hierarchy_matches_restatement(golden_dir):
    """The aggregates equal the numpy restatement bit for bit, and the coarse
    matrix equals P^T A P (scipy) to rounding."""
    dev = cuda()
    import scipy.sparse as sp
    import fealpy_gb300 as F
    A, b, z = _fixture_system(golden_dir, "cfg_c2_tet_p2_8.npz", dev)
    Ah = sp.csr_matrix((z["bc_val"], z["bc_col"], z["bc_crow"]))
    M = F.GAMGSolver().setup(A)
    L0 = M.levels[0]
    agg_ref, nc_ref = _mis_aggregates(Ah)
    assert L0.n_coarse == nc_ref
    assert np.array_equal(L0.agg.cpu().numpy(), agg_ref)
    sizes = np.bincount(agg_ref[agg_ref >= 0])
    assert 4 <= sizes.mean() <= 30, sizes.mean()
    m = agg_ref >= 0
    P = sp.csr_matrix((np.ones(m.sum()), (np.nonzero(m)[0], agg_ref[m])), shape=(Ah.shape[0], nc_ref))
    Ac = (P.T @ Ah @ P).tocsr()
    Ac.sort_indices()
    L1 = M.levels[1]
    got = sp.csr_matrix((L1.values.cpu().numpy(), L1.indices.cpu().numpy(), L1.indptr.cpu().numpy()),
                        shape=(nc_ref, nc_ref))
    assert np.array_equal(got.indptr, Ac.indptr) and np.array_equal(got.indices, Ac.indices)
    assert np.max(np.abs(got.data - Ac.data)) <= 1e-12 * np.max(np.abs(Ac.data))
    assert torch.equal(L0.values32, L0.values.to(torch.float32))


def test_amg_pcg_c2_law_against_reference(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    A, b, z = _fixture_system(golden_dir, "cfg_c2_tet_p2_8.npz", dev)
    M = F.AMGPreconditioner().apply(A)
    assert len(M.levels) >= 2 and M.levels[1].n < M.levels[0].n / 4
    x, info = F.cg(A, b, M=M, atol=1e-30, rtol=1e-10, returninfo=True)
    assert info["reason"] == 2 and info["amg_levels"] == len(M.levels)
    assert info["niter"] < int(z["niter"]) / 2, (info["niter"], int(z["niter"]))
    assert rel(x, z["uh"]) < 1e-8
    r = float(torch.linalg.norm(b - A @ x) / torch.linalg.norm(b))
    assert r < 1e-9
    # reproducible: a second hierarchy and solve give the same bits
    M2 = F.AMGPreconditioner().apply(A)
    for L1, L2 in zip(M.levels, M2.levels):
        assert torch.equal(L1.values, L2.values) and torch.equal(L1.indices, L2.indices)
        if L1.agg is not None:
            assert torch.equal(L1.agg, L2.agg)
    x2 = F.cg(A, b, M=M2, atol=1e-30, rtol=1e-10)
    assert torch.equal(x, x2)


def test_amg_bench_workload_24_against_oracle():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                                  ScalarSourceIntegrator, DirichletBC)
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    from oracle import fem_oracle as O
    node, cell, kappa = diffusion_mass_tet_box(24)
    ref = O.poisson_pipeline(node, cell, 2, kappa=kappa, rho=1.0, q=4, rtol=1e-12)
    mesh = F.TetrahedronMesh(torch.as_tensor(node, device=dev), torch.as_tensor(cell, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=torch.as_tensor(kappa, device=dev), q=4),
                      ScalarMassIntegrator(coef=1.0, q=4))
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=4))
    A2, F2 = DirichletBC(space, gd=0.0).apply(bf.assembly(), lf.assembly())
    M = F.GAMGSolver().setup(A2)
    x, info = F.cg(A2, F2, M=M, atol=0.0, rtol=1e-10, returninfo=True, stop="residual")
    assert info["reason"] == 2 and info["niter"] < 120, info
    assert rel(x, ref["x"]) < 1e-8
    # level 0 (117649 rows) smooths on its SELL copy; the CSR sweeps give the
    # same V-cycle to FP32 rounding, and an FP64 V-cycle to FP32 accuracy
    assert M.levels[0].sell is not None
    z_sell = M.vcycle(F2)
    z_csr = F.GAMGSolver(sell_min_rows=1 << 40).setup(A2).vcycle(F2)
    z_64 = F.GAMGSolver(vcycle_f32=False).setup(A2).vcycle(F2)
    assert rel(z_sell, z_csr.cpu().numpy()) < 1e-4
    assert rel(z_sell, z_64.cpu().numpy()) < 1e-4
    # the reference's solver interface: setup + solve, CG and MG
    xs, inf = F.GAMGSolver(rtol=1e-10, atol=1e-30, maxit=500).setup(A2).solve(F2)
    assert inf["niter"] > 0 and rel(xs, ref["x"]) < 1e-8
    xm, infm = F.GAMGSolver(isolver="MG", rtol=1e-8, atol=1e-30, maxit=500).setup(A2).solve(F2)
    assert infm["niter"] < 500 and rel(xm, ref["x"]) < 1e-6, infm


def test_amg_elasticity_c5_law(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    A, b, z = _fixture_system(golden_dir, "cfg_c5_elasticity_8.npz", dev)
    x, info = F.cg(A, b, M=F.AMGPreconditioner().apply(A), atol=1e-30, rtol=1e-10, returninfo=True)
    assert info["reason"] == 2 and info["niter"] < int(z["niter"]), (info["niter"], int(z["niter"]))
    assert rel(x, z["uh"]) < 1e-8
    # aggregates of whole nodes (three interleaved components): every level
    # keeps the interleaved layout, and the solve reaches the same solution
    M3 = F.GAMGSolver(block_size=3).setup(A)
    for L in M3.levels[:-1]:
        agg = L.agg.cpu().numpy().reshape(-1, 3)
        ok = agg[:, 0] >= 0
        assert np.array_equal(agg[ok], (agg[ok, :1] // 3) * 3 + np.arange(3)) and np.all(agg[~ok] == -1)
    x3, info3 = F.cg(A, b, M=M3, atol=1e-30, rtol=1e-10, returninfo=True)
    assert info3["reason"] == 2 and rel(x3, z["uh"]) < 1e-8
