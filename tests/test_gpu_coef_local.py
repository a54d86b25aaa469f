"""Coefficients given per quadrature point and cell-local matrices on request.

* (NC, NQ) coefficients (``fealpy/utils/utils.py:21-53`` feeding
  ``bilinear_integral``): a cartesian diffusion function and an (NC, NQ) mass
  array on P2 triangles and P2 tetrahedra; local matrices and the assembled
  CSR against fixtures the reference produced (``make_golden.py --coef``).
  Their factor channels exceed one factor launch, so the CSR values come from
  several passes that add into the values.
* The matrix-free product with such a coefficient equals the CSR product.
* P1 elasticity local matrices (``LinearElasticityIntegrator.assembly``,
  ``fealpy/fem/linear_elasticity_integrator.py:61-181``) against the
  reference's ``KK``, in the interleaved and the component-major order.

Tolerances: CSR indptr/indices bit-exact; values 1e-12 relative."""
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-12


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _kappa(dim):
    def k(p):
        if dim == 2:
            return 1.0 + p[..., 0] ** 2 + p[..., 1]
        return 1.0 + p[..., 0] ** 2 + p[..., 1] * p[..., 2]
    k.coordtype = "cartesian"
    return k


@pytest.mark.parametrize("tag", ["tri_p2", "tet_p2"])
def test_quadrature_point_coefficients_against_reference(golden_dir, tag):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = np.load(os.path.join(golden_dir, f"coefq_{tag}.npz"))
    node = torch.as_tensor(z["node"], device=dev)
    cell = torch.as_tensor(z["cell"], device=dev)
    mesh = F.TriangleMesh(node, cell) if tag.startswith("tri") else F.TetrahedronMesh(node, cell)
    q = int(z["q"])
    space = F.LagrangeFESpace(mesh, p=int(z["p"]))
    kappa = _kappa(node.shape[1])
    rho = torch.as_tensor(z["rho"], device=dev)
    di = ScalarDiffusionIntegrator(coef=kappa, q=q)
    mi = ScalarMassIntegrator(coef=rho, q=q)
    plan = di.plan(space) + mi.plan(space)
    assert len(plan.passes()) > 1  # more channels than one factor launch
    assert rel(di.assembly(space), z["K_diff"]) < TOL
    assert rel(mi.assembly(space), z["K_mass"]) < TOL
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q), ScalarMassIntegrator(coef=rho, q=q))
    A = bf.assembly()
    assert np.array_equal(A.crow.cpu().numpy(), z["crow"]) and np.array_equal(A.col.cpu().numpy(), z["col"])
    assert rel(A.values, z["val"]) < TOL
    # the matrix-free product of the same form
    bf2 = BilinearForm(space)
    bf2.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=q), ScalarMassIntegrator(coef=rho, q=q))
    u = torch.rand(space.number_of_global_dofs(), dtype=torch.float64, device=dev)
    assert rel(bf2 @ u, (A @ u).cpu().numpy()) < 1e-12


def test_constant_along_points_stays_per_cell(golden_dir):
    """An (NC, NQ) array equal along the points is a per-cell coefficient: one
    pass, the same values as the (NC,) form."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator
    z = np.load(os.path.join(golden_dir, "coefq_tet_p2.npz"))
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], device=dev))
    space = F.LagrangeFESpace(mesh, p=2)
    k = torch.rand(mesh.number_of_cells(), dtype=torch.float64, device=dev) + 0.5
    NQ = z["rho"].shape[1]
    d1 = ScalarDiffusionIntegrator(coef=k, q=4)
    d2 = ScalarDiffusionIntegrator(coef=k[:, None].expand(-1, NQ).contiguous(), q=4)
    assert len(d2.plan(space).passes()) == 1
    b1, b2 = BilinearForm(space), BilinearForm(space)
    b1.add_integrator(d1)
    b2.add_integrator(d2)
    assert torch.equal(b1.assembly().values, b2.assembly().values)


def test_elasticity_local_matrices_against_reference(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import LinearElasticityIntegrator
    z = np.load(os.path.join(golden_dir, "small_elasticity_tet_p1.npz"))
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev), torch.as_tensor(z["cell"], device=dev))
    scale = torch.as_tensor(z["scale"], device=dev)
    mat = F.LinearElasticMaterial("m", lame_lambda=1.0, shear_modulus=0.5, cell_scale=scale)
    ss = F.LagrangeFESpace(mesh, p=1)
    ts = F.TensorFunctionSpace(ss, (-1, 3))
    KK = LinearElasticityIntegrator(mat, q=4).assembly(ts)
    assert KK.shape == z["KK"].shape
    assert rel(KK, z["KK"]) < TOL
    # component-major order: the same matrices with rows and columns permuted
    tp = F.TensorFunctionSpace(ss, (3, -1))
    KP = LinearElasticityIntegrator(mat, q=4).assembly(tp).cpu().numpy()
    perm = np.array([li * 3 + a for a in range(3) for li in range(4)])
    assert np.array_equal(KP, KK.cpu().numpy()[:, perm][:, :, perm])
