"""Integration over a sub-region of cells (``region=`` of ScalarDiffusion /
ScalarSource, ``index=`` of ScalarMass / LinearElasticity;
``fealpy/fem/integrator.py:141-162``).

* Diffusion (region) + mass (index) on P2 triangles against the reference's
  CSR (``region_cases.npz``, made by ``make_golden.py --coef``): the pattern
  holds only the region's couplings, bit-exact; values 1e-12.  The region as
  indices, as a boolean mask and as a callable of the mesh give the same.
* The matrix-free product over the region equals the region CSR product.
* Integrator groups over two overlapping regions of one form against the
  reference's CSR (``multi_region_tri_p2.npz``, ``make_golden.py --regions``).
* Cases the reference itself cannot run (its source integrator ignores the
  region in its dof map; its elasticity integrator sizes local matrices by all
  cells) are checked for consistency: a region source equals the full source
  with the values outside the region set to zero; a region elasticity matrix
  acts as the full matrix of a material scaled by the region's indicator."""
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
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _kappa(p):
    return 1.0 + p[..., 0] ** 2 + p[..., 1]


_kappa.coordtype = "cartesian"


def test_region_against_reference(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = np.load(os.path.join(golden_dir, "region_cases.npz"))
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], device=dev))
    space = F.LagrangeFESpace(mesh, p=2)
    reg = torch.as_tensor(z["region"], device=dev)
    mask = torch.zeros(mesh.number_of_cells(), dtype=torch.bool, device=dev)
    mask[reg] = True
    for region in (reg, mask, lambda m: reg):
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=_kappa, q=4, region=region),
                          ScalarMassIntegrator(coef=2.0, q=4, index=region))
        A = bf.assembly()
        assert np.array_equal(A.crow.cpu().numpy(), z["crow"]) and np.array_equal(A.col.cpu().numpy(), z["col"])
        assert rel(A.values, z["val"]) < 1e-12
    # matrix free over the region
    bf2 = BilinearForm(space)
    bf2.add_integrator(ScalarDiffusionIntegrator(coef=_kappa, q=4, region=reg),
                       ScalarMassIntegrator(coef=2.0, q=4, index=reg))
    u = torch.rand(space.number_of_global_dofs(), dtype=torch.float64, device=dev)
    assert rel(bf2 @ u, A @ u) < 1e-12
    # local matrices of the region's cells
    K_all = ScalarDiffusionIntegrator(coef=_kappa, q=4).assembly(space)
    K_reg = ScalarDiffusionIntegrator(coef=_kappa, q=4, region=reg).assembly(space)
    assert K_reg.shape[0] == reg.numel() and rel(K_reg, K_all[reg]) < 1e-13


def test_region_source_and_elasticity_consistency(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import (BilinearForm, LinearForm, ScalarSourceIntegrator, LinearElasticityIntegrator)
    z = np.load(os.path.join(golden_dir, "region_cases.npz"))
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], device=dev))
    space = F.LagrangeFESpace(mesh, p=2)
    reg = torch.as_tensor(z["region"], device=dev)
    NC = mesh.number_of_cells()
    ind = torch.zeros(NC, dtype=torch.float64, device=dev)
    ind[reg] = 1.0

    def src(p):
        return torch.sin(3.0 * p[..., 0]) + p[..., 1]
    src.coordtype = "cartesian"
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(src, q=4, region=reg))
    Fr = lf.assembly()
    bcs, _ = mesh.quadrature_formula(4).get_quadrature_points_and_weights()
    fq = src(mesh.bc_to_point(bcs)) * ind[:, None]
    lf2 = LinearForm(space)
    lf2.add_integrator(ScalarSourceIntegrator(fq, q=4))
    assert rel(Fr, lf2.assembly()) < 1e-13
    # P1 elasticity on a tetrahedral box, region = cells with centroid x < 0.5
    tmesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 3, 3, 3, device=dev)
    cent = tmesh.node[tmesh.cell.long()].mean(dim=1)
    treg = torch.nonzero(cent[:, 0] < 0.5).reshape(-1)
    tind = torch.zeros(tmesh.number_of_cells(), dtype=torch.float64, device=dev)
    tind[treg] = 1.0
    ts = F.TensorFunctionSpace(F.LagrangeFESpace(tmesh, 1), (-1, 3))
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5)
    b1 = BilinearForm(ts)
    b1.add_integrator(LinearElasticityIntegrator(mat, q=4, index=treg))
    A1 = b1.assembly()
    mat0 = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5, cell_scale=tind)
    b2 = BilinearForm(ts)
    b2.add_integrator(LinearElasticityIntegrator(mat0, q=4))
    A2 = b2.assembly()
    assert A1.nnz < A2.nnz
    u = torch.rand(ts.number_of_global_dofs(), dtype=torch.float64, device=dev)
    assert rel(A1 @ u, A2 @ u) < 1e-13
    KK = LinearElasticityIntegrator(mat, q=4, index=treg).assembly(ts)
    KA = LinearElasticityIntegrator(mat, q=4).assembly(ts)
    assert KK.shape[0] == treg.numel() and rel(KK, KA[treg]) < 1e-13


def test_groups_over_different_regions_against_reference(golden_dir):
    """Integrator groups over different (overlapping) regions of one form
    (fealpy/fem/integrator.py:141-162): the pattern of the union of the
    regions, each group's values added into it, against the reference's CSR;
    the matrix-free product (the sum of the groups' products) against the
    assembled one."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = np.load(os.path.join(golden_dir, "multi_region_tri_p2.npz"))
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], device=dev))
    space = F.LagrangeFESpace(mesh, p=2)
    reg1 = torch.as_tensor(z["reg1"], device=dev)
    reg2 = torch.as_tensor(z["reg2"], device=dev)

    def form():
        bf = BilinearForm(space)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=_kappa, q=4), region=reg1)
        bf.add_integrator(ScalarDiffusionIntegrator(coef=3.0, q=4), region=reg2)
        bf.add_integrator(ScalarMassIntegrator(coef=2.0, q=4, index=reg2))
        return bf

    A = form().assembly()
    assert np.array_equal(A.crow.cpu().numpy(), z["crow"]) and np.array_equal(A.col.cpu().numpy(), z["col"])
    assert rel(A.values, z["val"]) < 1e-12
    bf = form()
    u = torch.rand(space.number_of_global_dofs(), dtype=torch.float64, device=dev)
    assert rel(bf @ u, (A @ u).cpu().numpy()) < 1e-12 and bf._M is None
    # the FP32 copy for the mixed-precision solver covers every row
    A2 = form().assembly(emit_f32=True)
    assert torch.equal(A2.values, A.values) and torch.equal(A2._f32, A.values.to(torch.float32))
