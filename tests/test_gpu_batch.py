"""Batched FP32-refined PCG (fealpy_gb300.batch): every system of a batch
reaches the true relative residual 1e-10, agrees with the single-system FP64
solve and with the CPU oracle's pipeline on the same inputs, and gives the same bits alone and inside any mix, whether it joins
at the start or while others are in flight (continuous batching)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch.device("cuda", 0)


def _poisson(F, mesh, p, seed, dtype=torch.float64, inputs=None):
    """Diffusion (lognormal kappa) + mass, quadrature p + 2, a random nodal
    right-hand side, u = 0 on the boundary.  ``inputs`` (a list) receives the
    host copies of the mesh, kappa and f for the oracle."""
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator, DirichletBC
    g = torch.Generator(device="cpu").manual_seed(seed)
    NC = mesh.number_of_cells()
    kappa = torch.exp(torch.randn(NC, generator=g, dtype=torch.float64)).to(mesh.node.device)
    space = F.LagrangeFESpace(mesh, p)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 2), ScalarMassIntegrator(coef=1.0, q=p + 2))
    A = bf.assembly(dtype=dtype)
    n = space.number_of_global_dofs()
    f = torch.rand(n, generator=g, dtype=torch.float64).to(mesh.node.device)
    if inputs is not None:
        inputs.append({"node": mesh.node.cpu().numpy(), "cell": mesh.cell.cpu().numpy(), "p": p,
                       "kappa": kappa.cpu().numpy(), "f": f.cpu().numpy()})
    return DirichletBC(space, gd=0.0).apply(A, f)


def _systems(dev, inputs=None):
    import fealpy_gb300 as F
    out = []
    for k, (nx, p) in enumerate([(8, 1), (20, 2), (13, 3), (40, 1), (6, 2)]):
        m = F.TriangleMesh.from_box([0, 1, 0, 1], nx, nx, device=dev)
        out.append(_poisson(F, m, p, k, inputs=inputs))
    m = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], 6, 5, 4, device=dev)
    out.append(_poisson(F, m, 1, 9, inputs=inputs))
    return out


def _oracle_solution(d):
    """The CPU oracle's pipeline (reference algorithm) on the same inputs."""
    from oracle import fem_oracle as O
    out = O.poisson_pipeline(d["node"], d["cell"], d["p"], kappa=d["kappa"], rho=1.0, q=d["p"] + 2,
                             f_vec=d["f"], rtol=1e-12)
    return out["x"]


def _residual(A, b, x):
    import fealpy_gb300 as F
    Ad = F.CSRTensor(A.crow, A.col, A.values.to(torch.float64), A.shape)
    bd = b.to(torch.float64)
    return float(torch.linalg.norm(bd - Ad @ x) / torch.linalg.norm(bd))


def test_batch_converges_and_matches_fp64():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.batch import BatchSolver
    inputs = []
    systems = _systems(dev, inputs)
    bs = BatchSolver(8, slices_per_tile=4, rows_per_tile=512)
    for k, (A, b) in enumerate(systems):
        bs.add(A, b, rtol=RTOL, key=k)
    res = bs.solve_all()
    assert sorted(res) == list(range(len(systems)))
    assert bs.used_graph
    for k, (A, b) in enumerate(systems):
        r = res[k]
        assert r.reason == 2, (k, r.info())
        rel = _residual(A, b, r.x)
        assert rel <= RTOL * 1.0001 and abs(rel - r.relres) <= 1e-3 * rel, (k, rel, r.relres)
        x64 = F.cg(A, b, M=F.JacobiPreconditioner().apply(A), atol=1e-30, rtol=1e-13)
        err = float((r.x - x64).abs().max() / x64.abs().max())
        assert err < 1e-8, (k, err)
        # against the CPU oracle's assembly + Dirichlet + PCG of the same inputs
        xo = _oracle_solution(inputs[k])
        erro = float(np.max(np.abs(r.x.cpu().numpy() - xo)) / np.max(np.abs(xo)))
        assert erro < 1e-8, (k, erro)


def test_batch_solo_equals_mix_and_late_admission():
    dev = cuda()
    from fealpy_gb300.batch import BatchSolver
    systems = _systems(dev)
    cfg = dict(slices_per_tile=4, rows_per_tile=512)
    solo = {}
    for k, (A, b) in enumerate(systems):
        bs = BatchSolver(2, **cfg)
        bs.add(A, b, rtol=RTOL, key=k)
        solo[k] = bs.solve_all()[k]
    # mix: half start together, the rest join while the first ones run
    bs = BatchSolver(4, **cfg)
    res, waiting = {}, list(range(len(systems)))
    for k in waiting[:3]:
        bs.add(*systems[k], rtol=RTOL, key=k)
    waiting = waiting[3:]
    while bs.active() or waiting:
        for r in bs.step(max_iterations=7):
            res[r.key] = r
        while waiting and bs.free_slots():
            k = waiting.pop(0)
            bs.add(*systems[k], rtol=RTOL, key=k)
    for k in solo:
        assert res[k].niter == solo[k].niter, (k, res[k].niter, solo[k].niter)
        assert torch.equal(res[k].x, solo[k].x), k
    # host-driven loop: same kernels, same bits
    bs = BatchSolver(8, **cfg)
    for k, (A, b) in enumerate(systems):
        bs.add(A, b, rtol=RTOL, key=k)
    polled = bs.solve_all(graph=False)
    for k in solo:
        assert torch.equal(polled[k].x, solo[k].x), k


def test_batch_fp32_operators_and_autotune():
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.batch import BatchSolver, autotune
    m = F.TriangleMesh.from_box([0, 1, 0, 1], 24, 24, device=dev)
    A32, b32 = _poisson(F, m, 2, 3, dtype=torch.float32)
    bs = BatchSolver(2)
    bs.add(A32, b32, rtol=RTOL, key="a")
    r = bs.solve_all()["a"]
    assert r.reason == 2 and _residual(A32, b32, r.x) <= RTOL * 1.0001
    times = autotune([(A32, b32)], candidates=((8, 128), (16, 256)))
    assert set(times) == {(8, 128), (16, 256)} and all(t > 0 for t in times.values())


def _laplace_1d(n, dev, dtype):
    """Tridiagonal 1-D Laplacian (condition number ~ 0.4 n^2), random b (a
    constant b would let CG end early by symmetry)."""
    import fealpy_gb300 as F
    rows, cols, vals = [], [], []
    for i in range(n):
        for j, v in ((i - 1, -1.0), (i, 2.0), (i + 1, -1.0)):
            if 0 <= j < n:
                rows.append(i)
                cols.append(j)
                vals.append(v)
    crow = torch.zeros(n + 1, dtype=torch.int64)
    crow[1:] = torch.cumsum(torch.bincount(torch.tensor(rows), minlength=n), 0)
    A = F.CSRTensor(crow.to(dev), torch.tensor(cols, dtype=torch.int32, device=dev),
                    torch.tensor(vals, dtype=dtype, device=dev), (n, n))
    g = torch.Generator(device="cpu").manual_seed(n)
    return A, torch.rand(n, generator=g, dtype=torch.float64).to(dev)


def test_batch_fp64_systems_and_stagnation_continuation():
    """An FP64 system of the batch follows plain FP64 PCG; an ill-conditioned
    FP32 system either converges or is continued in FP64 after stagnating,
    and always ends at the 1e-10 true residual."""
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300.batch import BatchSolver
    (A, b) = _systems(dev)[1]
    L, lb = _laplace_1d(3000, dev, torch.float32)
    bs = BatchSolver(4)
    bs.add(A, b, rtol=RTOL, key="fp64", fp64=True)
    bs.add(L, lb, rtol=RTOL, key="ill", maxit=200000)
    res = bs.solve_all()
    r = res["fp64"]
    assert r.reason == 2 and _residual(A, b, r.x) <= RTOL * 1.0001
    x64 = F.cg(A, b, M=F.JacobiPreconditioner().apply(A), atol=0.0, rtol=RTOL, stop="residual", returninfo=True)
    assert abs(r.niter - x64[1]["niter"]) <= 2, (r.niter, x64[1]["niter"])
    q = res["ill"]
    # the recomputed residual of this operator (|A||x| / |b| ~ 1e3) carries
    # summation-order differences of a few 1e-11
    assert q.reason == 2 and q.relres <= RTOL and _residual(L, lb, q.x) <= 2 * RTOL, (q.info(), bs.fallbacks)


def test_cg_mixed_continues_in_fp64_after_stagnation():
    """The single-system FP32-refined solver on an operator beyond FP32
    (condition number ~4e6) continues in FP64 when its FP32 iterations stall
    and ends at 1e-10 or at the attainable accuracy of this operator (its
    FP64 residual floor is about 1.2e-10: then reason 7, 'stagnated')."""
    dev = cuda()
    import fealpy_gb300 as F
    L, lb = _laplace_1d(3000, dev, torch.float32)
    x, info = F.cg_mixed(L, lb, rtol=RTOL, maxit=200000, returninfo=True)
    assert info["fp64_iterations"] > 0, info
    assert info["reason"] in (2, 7) and _residual(L, lb, x) <= 2 * RTOL, info


def test_batch_with_multigrid_lane():
    """The two largest systems by multigrid PCG beside the batch: every result
    at 1e-10 against the oracle's solution; a lane result equals the same
    system's multigrid solve alone (bit for bit)."""
    dev = cuda()
    from fealpy_gb300.batch import BatchSolver, solve_with_multigrid_lane
    from fealpy_gb300.amg import multigrid_solve
    inputs = []
    systems = _systems(dev, inputs)
    big = sorted(range(len(systems)), key=lambda k: systems[k][0].shape[0])[-2:]
    bs = BatchSolver(8, slices_per_tile=4, rows_per_tile=512)
    lane = []
    for k, (A, b) in enumerate(systems):
        if k in big:
            lane.append((k, A, b, RTOL, 100000))
        else:
            bs.add(A, b, rtol=RTOL, key=k)
    res = solve_with_multigrid_lane(bs, lane, workers=2)
    assert sorted(res) == list(range(len(systems)))
    for k, (A, b) in enumerate(systems):
        rel = _residual(A, b, res[k].x)
        assert rel <= RTOL * 1.0001, (k, rel)
        xo = _oracle_solution(inputs[k])
        erro = float(np.max(np.abs(res[k].x.cpu().numpy() - xo)) / np.max(np.abs(xo)))
        assert erro < 1e-8, (k, erro)
    for k in big:
        A, b = systems[k]
        x, niter, _, _ = multigrid_solve(A, b, RTOL, 100000)
        assert torch.equal(x, res[k].x) and niter == res[k].niter
