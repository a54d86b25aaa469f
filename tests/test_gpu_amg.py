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
