"""Numeric assembly with the pattern's slot map (``build_pattern(...,
positions=True)``, kept by forms that reuse their pattern): the recorded
within-row positions point at the right columns, and the values assembled
through them (with and without an accumulated second pass) are bitwise those
of the column-search path, which is the one pinned to the reference's
fixtures elsewhere: every entry is summed in the same order."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def cuda():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    return torch.device("cuda", 0)


def _case(F, dev, kind, n, p):
    from fealpy_gb300.fem import BilinearForm, ScalarDiffusionIntegrator, ScalarMassIntegrator
    g = torch.Generator(device="cpu").manual_seed(7)
    if kind == "tet":
        mesh = F.TetrahedronMesh.from_box([0, 1, 0, 1, 0, 1], n, n, n, device=dev)
    else:
        mesh = F.TriangleMesh.from_box([0, 1, 0, 1], n, n + 1, device=dev)
    NC = mesh.number_of_cells()
    kappa = torch.exp(torch.randn(NC, generator=g, dtype=torch.float64)).to(dev)
    space = F.LagrangeFESpace(mesh, p)
    bf = BilinearForm(space)
    bf.add_integrator(ScalarDiffusionIntegrator(coef=kappa, q=p + 2), ScalarMassIntegrator(coef=1.0, q=p + 2))
    return mesh, space, bf


@pytest.mark.parametrize("kind,n,p", [("tet", 9, 2), ("tet", 5, 1), ("tri", 24, 3), ("tri", 30, 2), ("tri", 40, 1)])
def test_slot_map_and_values(kind, n, p):
    dev = cuda()
    import fealpy_gb300 as F
    from fealpy_gb300 import kernels as K, _lib
    mesh, space, bf = _case(F, dev, kind, n, p)
    c2d = space.cell_to_dof()
    N = space.number_of_global_dofs()
    st = _lib.status_word(dev)
    adj_ptr, adj, _ = K.build_adjacency(c2d, N, st)
    indptr, indices, pos = K.build_pattern(adj_ptr, adj, c2d, N, st, positions=True)
    ip2, ix2 = K.build_pattern(adj_ptr, adj, c2d, N, st)
    assert torch.equal(indptr, ip2) and torch.equal(indices, ix2)
    # every recorded slot holds the column of its (cell, local dof)
    ldof = c2d.shape[1]
    rows = torch.repeat_interleave(torch.arange(N, device=dev), (adj_ptr[1:] - adj_ptr[:-1]))
    cells = (adj.long() // ldof)
    cols = c2d.long()[cells]                                   # (n_adj, ldof)
    slots = pos[: adj.numel() * ldof].long().view(-1, ldof)
    lens = (indptr[1:] - indptr[:-1])[rows]
    assert bool((slots < lens[:, None]).all())
    got = indices.long()[indptr[rows][:, None] + slots]
    assert torch.equal(got, cols)
    plan = bf._plan()
    (chans, tabs), = plan.passes()
    for dt in (torch.float64, torch.float32):
        fac = K.cell_factors(mesh, chans, plan.coef_matrix(), dt, st)
        tab = torch.as_tensor(tabs, dtype=dt, device=dev)
        v_s, _ = K.assemble_scalar(adj_ptr, adj, c2d, tab, fac, indptr, indices, status=st)
        v_m, _ = K.assemble_scalar(adj_ptr, adj, c2d, tab, fac, indptr, indices, status=st, positions=pos)
        assert torch.equal(v_s, v_m), dt
        # a second pass added into the first (split channels)
        w_s, w32_s = K.assemble_scalar(adj_ptr, adj, c2d, tab, fac, indptr, indices, status=st,
                                       accumulate_into=v_s.clone(), values_f32=True)
        w_m, w32_m = K.assemble_scalar(adj_ptr, adj, c2d, tab, fac, indptr, indices, status=st,
                                       accumulate_into=v_m.clone(), values_f32=True, positions=pos)
        assert torch.equal(w_s, w_m) and torch.equal(w32_s, w32_m), dt
    _lib.check_status_word("slot map", st)
    # a form that reuses its pattern keeps the slot map with it: its first and
    # repeated assemblies equal the search path
    from fealpy_gb300.fem import BilinearForm
    rf = BilinearForm(space, reuse_pattern=True)
    for it in bf.integrators.values():
        rf.add_integrator(it)
    fac = K.cell_factors(mesh, chans, plan.coef_matrix(), torch.float64, st)
    v_s, _ = K.assemble_scalar(adj_ptr, adj, c2d, torch.as_tensor(tabs, dtype=torch.float64, device=dev), fac,
                               indptr, indices, status=st)
    for _ in range(2):
        A = rf.assembly()
        assert torch.equal(A.values, v_s) and torch.equal(A.col, indices)
    assert any(k[0] == "symbolic" and k[2] for k in space._cache)
