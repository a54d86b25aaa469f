"""Matrix-free BilinearForm products (``bform @ x`` before ``assembly()``),
as FEALPy forms them from cell-local matrices without a global matrix
(fealpy/fem/bilinear_form.py:126-158).  Mirrors the reference's own test
(test/fem/test_bilinear_form.py:19-44: the two small triangle meshes of
bilinear_form_data.py, p = 1..4, the matrix-free product equals the assembled
product to 1e-12 and leaves ``_M`` unset), and checks the kernels against the
reference's assembled matrices of the C2 (P2 tetrahedra, diffusion + mass)
and C3 (P3 triangles) laws: FP64 within 1e-12, FP32 within 1e-5, batched
inputs row by row."""
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
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


REF_MESHES = [
    (np.array([[0, 0], [1, 0], [0, 1]], dtype=np.float64), np.array([[0, 1, 2]], dtype=np.int32)),
    (np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.float64), np.array([[1, 2, 0], [3, 0, 2]], dtype=np.int32)),
]


@pytest.mark.parametrize("mesh_id", [0, 1])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_matmul_before_and_after_assembly(mesh_id, p):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator
    node, cell = REF_MESHES[mesh_id]
    mesh = F.TriangleMesh(torch.as_tensor(node, device=dev), torch.as_tensor(cell, device=dev))
    space = F.LagrangeFESpace(mesh, p)
    gdof = space.number_of_global_dofs()
    x = torch.rand(gdof, dtype=torch.float64, device=dev)
    bform = BilinearForm(space)
    bform.add_integrator(ScalarDiffusionIntegrator())
    y = bform @ x
    assert bform._M is None
    bform.assembly()
    assert bform._M is not None
    z = bform @ x
    assert float(torch.linalg.norm(y - z)) < 1e-12


def _fixture_product(z, x):
    import scipy.sparse as sp
    n = len(z["crow"]) - 1
    return sp.csr_matrix((z["val"], z["col"], z["crow"]), shape=(n, n)) @ x


def test_matfree_c2_law_against_reference_matrix(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = np.load(os.path.join(golden_dir, "cfg_c2_tet_p2_8.npz"))
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    kappa = torch.as_tensor(z["kappa"], device=dev)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
    n = space.number_of_global_dofs()
    xs = np.random.default_rng(0).normal(size=(2, n))
    ref = np.stack([_fixture_product(z, v) for v in xs])
    y = bf @ torch.as_tensor(xs[0], device=dev)
    assert bf._M is None and rel(y, ref[0]) < 1e-12
    yb = bf @ torch.as_tensor(xs, device=dev)
    assert yb.shape == (2, n) and rel(yb, ref) < 1e-12
    y32 = bf @ torch.as_tensor(xs[1], device=dev, dtype=torch.float32)
    assert y32.dtype == torch.float32 and rel(y32.double(), ref[1]) < 1e-5


def test_matfree_c3_law_p3_triangles(golden_dir):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator
    z = np.load(os.path.join(golden_dir, "cfg_c3_tri_p3_32.npz"))
    mesh = F.TriangleMesh(torch.as_tensor(z["node"], device=dev),
                          torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 3)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=torch.as_tensor(z["kappa"], device=dev), q=6))
    x = np.random.default_rng(1).normal(size=space.number_of_global_dofs())
    y = bf @ torch.as_tensor(x, device=dev)
    assert rel(y, _fixture_product(z, x)) < 1e-12


def test_cg_on_the_unassembled_form(golden_dir):
    """``cg`` takes any operator with ``@`` (fealpy/solver/cg.py:10-17): the
    C2-law form before assembly (diffusion + mass, no boundary condition: SPD)
    solved matrix free with Jacobi, against a direct solve of the reference's
    assembled matrix, and against cg on the assembled CSR (same recurrence:
    the same iteration count within one)."""
    dev = cuda()
    import scipy.sparse as sps
    from scipy.sparse.linalg import spsolve
    import fealpy_gb300 as F
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    z = np.load(os.path.join(golden_dir, "cfg_c2_tet_p2_8.npz"))
    mesh = F.TetrahedronMesh(torch.as_tensor(z["node"], device=dev),
                             torch.as_tensor(z["cell"], dtype=torch.int32, device=dev))
    space = F.LagrangeFESpace(mesh, 2)
    kappa = torch.as_tensor(z["kappa"], device=dev)
    ints = lambda: (ScalarDiffusionIntegrator(coef=kappa, q=4), ScalarMassIntegrator(coef=1.0, q=4))
    bf = BilinearForm(space)
    bf.add_integrator(*ints())
    n = space.number_of_global_dofs()
    b = np.random.default_rng(2).normal(size=n)
    A_ref = sps.csr_matrix((z["val"], z["col"], z["crow"]), shape=(n, n))
    u_ref = spsolve(A_ref.tocsc(), b)
    ba = BilinearForm(space)
    ba.add_integrator(*ints())
    A = ba.assembly()
    M = F.JacobiPreconditioner().apply(A)
    bt = torch.as_tensor(b, device=dev)
    u, info = F.cg(bf, bt, M=M, atol=1e-30, rtol=1e-11, returninfo=True)
    assert bf._M is None
    assert rel(u, u_ref) < 1e-9, rel(u, u_ref)
    ua, infoa = F.cg(A, bt, M=M, atol=1e-30, rtol=1e-11, returninfo=True)
    assert abs(info["niter"] - infoa["niter"]) <= 1, (info, infoa)
    assert rel(u, ua.cpu().numpy()) < 1e-9
    # a COO operator goes to its CSR form
    uc = F.cg(ba.assembly(format="coo"), bt, M=M, atol=1e-30, rtol=1e-11)
    assert torch.equal(uc, ua)
