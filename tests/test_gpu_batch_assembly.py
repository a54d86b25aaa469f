"""Batched assembly (fealpy_gb300.fem.batch_assembly.BatchAssembler): many
systems grouped by structure and assembled as one block-diagonal system per
group, then split.  Every system's matrix (pattern and values), right-hand
side and Dirichlet elimination equal, bit for bit, those of its own
BilinearForm.assembly + LinearForm.assembly + DirichletBC.apply; systems that
do not fit the grouped path (a callable source) go through their own forms."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch.device("cuda", 0)


def _forms(F, dev, nx, p, seed, source=1.0):
    from fealpy_gb300.fem import BilinearForm, LinearForm, ScalarDiffusionIntegrator, ScalarSourceIntegrator
    from fealpy_gb300.fem import DirichletBC
    mesh = F.TriangleMesh.from_box([0, 1, 0, 1], nx, nx + 1, device=dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    kappa = torch.exp(torch.randn(mesh.number_of_cells(), generator=g, dtype=torch.float64)).to(dev)
    space = F.LagrangeFESpace(mesh, p)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 3))
    lf = LinearForm(space)
    lf.add_integrator(ScalarSourceIntegrator(source, q=p + 3))
    return bf, lf, DirichletBC(space, gd=0.0)


def test_batched_assembly_equals_per_system():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.fem.batch_assembly import BatchAssembler

    def src(p):
        return 1.0 + p[..., 0]
    src.coordtype = "cartesian"
    specs = [(5, 1, 1.0), (9, 2, 2.0), (4, 3, 1.0), (12, 1, 0.5), (7, 2, 1.0), (3, 3, 3.0), (6, 2, src)]
    systems = [_forms(F, dev, nx, p, k, s) for k, (nx, p, s) in enumerate(specs)]
    asm = BatchAssembler(systems)
    assert len(asm.groups) == 3 and asm.fallback == [6]
    got = asm.assemble(torch.float64)
    for k, (bf, lf, bc) in enumerate(systems):
        A, b = bc.apply(bf.assembly(), lf.assembly())
        Ag, bg = got[k]
        assert Ag.shape == A.shape
        assert torch.equal(Ag.crow, A.crow) and torch.equal(Ag.col, A.col), k
        assert torch.equal(Ag.values, A.values), k
        assert torch.equal(bg, b), k
    # FP32 assembly: the same values as each form's FP32 assembly
    got32 = asm.assemble(torch.float32)
    for k, (bf, lf, bc) in enumerate(systems[:6]):
        A, _ = bc.apply(bf.assembly(dtype=torch.float32), lf.assembly())
        assert torch.equal(got32[k][0].values, A.values), k
