"""GPU parity at the benchmark configurations' scale: the sm_103a path through
the public API against fixtures the reference itself produced on mid-size cases
of each configuration's law (tests/golden/make_golden.py --configs), and
against the CPU oracle on the bench workload's own generator at 24^3.

Tolerances (as in test_gpu_parity): canonical CSR indptr/indices bit-exact
before and after Dirichlet; values, right-hand sides and boundary-modified
right-hand sides within 1e-12 relative (max-norm); Jacobi-PCG iteration counts
within +-1; FP64 solutions within 1e-9 relative; FP32-refined solutions of the
FP64 operator within 1e-8; FP32-refined solutions of the FP32-assembled
operator within 1e-5 (the FP32 assembly's rounding) with a true residual of
1e-10 on that operator, and below 1e-4 against the FP64 operator."""
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


def true_relres(A, b, x):
    import fealpy_gb300 as F
    Ad = F.CSRTensor(A.crow, A.col, A.values.to(torch.float64), A.shape)
    bd = b.to(torch.float64)
    return float(torch.linalg.norm(bd - Ad @ x) / torch.linalg.norm(bd))


def check_system(A, Fv, A2, F2, z, uh_tol=1e-9):
    """Pre- and post-Dirichlet CSR and right-hand sides against fixture ``z``."""
    assert same(A.crow, z["crow"]) and same(A.col, z["col"])
    assert rel_err(A.values, z["val"]) < VAL_TOL
    assert rel_err(Fv, z["F"]) < VAL_TOL
    assert same(A2.crow, z["bc_crow"]) and same(A2.col, z["bc_col"])
    assert rel_err(A2.values, z["bc_val"]) < VAL_TOL
    assert rel_err(F2, z["bc_F"]) < VAL_TOL


def solve_checks(A2, F2, z, fp32_operator=None):
    """FP64 Jacobi-PCG, FP32-refined on the FP64 operator and, when given, on
    the FP32-assembled operator ``fp32_operator = (B32, f32)``."""
    import fealpy_gb300 as F
    uh, info = F.cg(A2, F2, M=F.JacobiPreconditioner().apply(A2), atol=1e-30, rtol=1e-10, returninfo=True)
    assert abs(info["niter"] - int(z["niter"])) <= 1, (info["niter"], int(z["niter"]))
    assert rel_err(uh, z["uh"]) < 1e-9
    xm, im = F.cg_mixed(A2, F2, rtol=1e-10, returninfo=True)
    assert im["relres"] <= 1e-10 and true_relres(A2, F2, xm) <= 1e-10 * 1.0001, im
    assert rel_err(xm, z["uh"]) < 1e-8
    if fp32_operator is not None:
        B32, f32 = fp32_operator
        x32, i32 = F.cg_mixed(B32, f32, rtol=1e-10, returninfo=True)
        assert i32["relres"] <= 1e-10 and true_relres(B32, f32, x32) <= 1e-10 * 1.0001, i32
        assert rel_err(x32, z["uh"]) < 1e-5
        # the same iterate measured against the FP64 operator: the residual of
        # the FP32 assembly's rounding (2.5e-5 measured on the elasticity case)
        assert true_relres(A2, F2, x32) < 1e-4


def test_c2_law_p2_tet_8(golden_dir):
    """C2 law: P2 diffusion + mass, 8^3 jittered tet box, lognormal kappa, q = 4."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                                  ScalarSourceIntegrator, DirichletBC)
    z = load(golden_dir, "cfg_c2_tet_p2_8.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    assert same(space.cell_to_dof(), z["cell2dof"])
    kappa = torch.as_tensor(z["kappa"], device=dev)
    mats = {}
    for dt in (torch.float64, torch.float32):
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
        mats[dt] = bf.assembly(dtype=dt)
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=4))
    Fv = lf.assembly()
    bc = DirichletBC(space, gd=0.0)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(mats[torch.float64], Fv)
    check_system(mats[torch.float64], Fv, A2, F2, z)
    B32, f32 = bc.apply(mats[torch.float32], Fv)
    assert same(B32.crow, z["bc_crow"]) and same(B32.col, z["bc_col"])
    solve_checks(A2, F2, z, (B32, f32))


def test_c3_law_p3_tri_32(golden_dir):
    """C3 law: P3 diffusion on a jittered 32x32 triangle box, 4x4 checkerboard
    coefficient in [0.1, 10], q = p + 3."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator, DirichletBC
    z = load(golden_dir, "cfg_c3_tri_p3_32.npz")
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev),
                          torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 3)
    assert same(space.cell_to_dof(), z["cell2dof"])
    kappa = torch.as_tensor(z["kappa"], device=dev)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=6))
    A = bf.assembly()
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=6))
    Fv = lf.assembly()
    bc = DirichletBC(space, gd=0.0)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(A, Fv)
    check_system(A, Fv, A2, F2, z)
    solve_checks(A2, F2, z)


def test_c5_law_elasticity_8(golden_dir):
    """C5 law: P1 vector elasticity on the 8^3 tet box, lambda = 1, mu = 0.5
    scaled per cell by lognormal(0, 0.5), clamped at x = 0, body force -z."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, LinearForm, LinearElasticityIntegrator, VectorSourceIntegrator
    from fealpy_gb300.fem import DirichletBC
    z = load(golden_dir, "cfg_c5_elasticity_8.npz")
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    ts = F.TensorFunctionSpace(F.LagrangeFESpace(mesh, 1), (-1, 3))
    assert same(ts.cell_to_dof(), z["cell2dof"])
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5,
                                  cell_scale=torch.as_tensor(z["scale"], device=dev))
    mats = {}
    for dt in (torch.float64, torch.float32):
        bf = BilinearForm(ts)
        bf.add_integrator(LinearElasticityIntegrator(mat, q=4))
        mats[dt] = bf.assembly(dtype=dt)
    lf = LinearForm(ts)
    lf.add_integrator(VectorSourceIntegrator(source=[0.0, 0.0, -1.0], q=4))
    Fv = lf.assembly()
    bc = DirichletBC(ts, gd=0.0, threshold=lambda x: torch.abs(x[..., 0]) < 1e-12)
    assert same(bc.is_boundary_dof, z["is_bd"])
    A2, F2 = bc.apply(mats[torch.float64], Fv)
    check_system(mats[torch.float64], Fv, A2, F2, z)
    B32, f32 = bc.apply(mats[torch.float32], Fv)
    solve_checks(A2, F2, z, (B32, f32))


def test_bench_workload_24_against_oracle():
    """The bench's own C2 generator (jittered P2 tet box, lognormal kappa,
    reaction 1, f = 1, u = 0, q = 4) at 24^3 (117,649 dofs): the GPU pipeline
    against the CPU oracle's, stage by stage."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import (BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator,
                                  ScalarSourceIntegrator, DirichletBC)
    from fealpy_gb300.workloads import diffusion_mass_tet_box
    from oracle import fem_oracle as O
    node, cell, kappa = diffusion_mass_tet_box(24)
    ref = O.poisson_pipeline(node, cell, 2, kappa=kappa, rho=1.0, q=4, rtol=1e-10)
    mesh = F.TetrahedronMesh(torch.as_tensor(node, device=dev), torch.as_tensor(cell, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    assert same(space.cell_to_dof(), ref["c2d"])
    kap = torch.as_tensor(kappa, device=dev)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kap, q=4), ScalarMassIntegrator(coef=1.0, q=4))
    A = bf.assembly()
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(1.0, q=4))
    Fv = lf.assembly()
    bc = DirichletBC(space, gd=0.0)
    assert same(bc.is_boundary_dof, ref["is_bd"])
    A2, F2 = bc.apply(A, Fv)
    z = {"crow": ref["crow"], "col": ref["col"], "val": ref["val"], "F": ref["F"], "bc_crow": ref["bc_crow"],
         "bc_col": ref["bc_col"], "bc_val": ref["bc_val"], "bc_F": ref["bc_F"], "uh": ref["x"],
         "niter": ref["info"]["niter"]}
    check_system(A, Fv, A2, F2, z)
    bf32 = BilinearForm(space)
    bf32.add_integrator(ScalarDiffusionIntegrator(coef=kap, q=4), ScalarMassIntegrator(coef=1.0, q=4))
    B32, f32 = bc.apply(bf32.assembly(dtype=torch.float32), Fv)
    solve_checks(A2, F2, z, (B32, f32))
